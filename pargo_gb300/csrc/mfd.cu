// mfd.cu -- MFD-md flow partition weights and the MFD specific catchment area.
//
// Weights (MFDOperator::Operator, apps/hydrology/flowdirmfdmd/mfdOperator.cpp:36-123):
// per work cell, drops to strictly lower valid neighbours -- (z - zn) / (1.414 cs)
// on diagonals with contour length 0.354 cs, (z - zn) / cs with 0.5 cs on
// cardinals -- the exponent pe = (1 - e) min(max drop, 1) + e, and
// w_i = drop_i^pe l_i / sum.  All 8 weights are nodata on a nodata cell
// (|z - nd| <= 1e-6, the operator's test) and on the ring.  Computed in FP32
// (powf; about 1e-6 relative to the reference's FP64 pow): drops of float DEMs
// are exact float differences; for float64 DEMs (pit-removed levels, whose
// differences are of order the gap) the drop is taken in FP64 and rounded once.
// Layer i is the window position i (i < 4) or i + 1 (i >= 4).
//
// MFD SCA (the scamfdmd SCAOperator, apps/hydrology/scamfdmd/scaOperator.cpp:42-113):
// the reference makes ONE raster-order accumulation sweep, in which a cell
// adds sca(n) w(n -> cell) for each inflow n whose degree is 0 at that moment
// -- a source, or an earlier cell that pulled all its own inflows ("done").
// Here the same sums are evaluated in dependency order: the sweep can pull
// only sources (whose sum is 1 from the start) and earlier cells, so a cell
// needs only its NW, N, NE and W neighbours' sums and done flags -- nothing
// that follows it.  The band form below walks 32-row bands in step on that
// structure; the round form (frontier rounds over counters of those earlier
// inflows, a fallback where the band launch cannot be configured) processes
// a cell once they are processed.  Either then adds, in the reference's
// window order and in FP64 with separately rounded products and sums, the
// inflows the sweep pulls (source, or earlier in raster order and done), so
// with the same weights the result equals the reference's bit for bit.
// Inflows from cells that are never processed (the ring, nodata) are never
// pulled.

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

constexpr int kThreads = 256;
constexpr uint8_t kValid = 1, kSource = 2, kNeverDone = 4, kDone = 8;
// flag bits 4-7: the receivers at positions 5-8 (layers 4-7) that wait on the
// cell -- valid work cells its positive weights reach, when it is no source
constexpr int kReleaseShift = 4;

// window position of c seen from its neighbour at position k, and that
// neighbour's layer for it
__device__ __forceinline__ int layer_towards_centre(int k) {
    const int dir = 8 - k;
    return dir < 4 ? dir : dir - 1;
}
__device__ __forceinline__ int pos_of_layer(int i) { return i < 4 ? i : i + 1; }

// weight > 0 without an FP64 compare
__device__ __forceinline__ bool positive(const InView& v, int64_t r, int64_t c) {
    const char* row = v.base + r * v.pitch;
    if (v.dtype == PARGO_F64) {
        const long long b = reinterpret_cast<const long long*>(row)[c];
        return b > 0 && b <= 0x7FF0000000000000LL;  // positive, not NaN (+inf counts, as in the reference)
    }
    return reinterpret_cast<const float*>(row)[c] > 0.0f;
}

// ------------------------------------------------------------- weights --
__global__ void __launch_bounds__(kThreads) mfd_weights_kernel(const MfdParams p) {
    const int64_t n = p.rows * p.cols;
    const bool f64 = p.dem.dtype == PARGO_F64;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        bool nd_out = r < 1 || c < 1 || r > p.rows - 2 || c > p.cols - 2;
        float drop[9], len[9];
        float maxd = 0.0f;
        if (!nd_out) {
            const char* rowc = p.dem.base + r * p.dem.pitch;
            const float zf = f64 ? 0.0f : reinterpret_cast<const float*>(rowc)[c];
            const double zd = f64 ? reinterpret_cast<const double*>(rowc)[c] : 0.0;
            const long long kz = f64 ? dkey64(zd) : 0;
            nd_out = f64 ? (kz >= p.ndd_lo && kz <= p.ndd_hi) : p.ndf.has(zf);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                drop[k] = 0.0f;
                len[k] = 0.0f;
                if (k == 4 || nd_out) continue;
                const char* row = p.dem.base + (r + k / 3 - 1) * p.dem.pitch;
                const int64_t cc = c + k % 3 - 1;
                const bool diag = k == 0 || k == 2 || k == 6 || k == 8;
                float d;
                if (f64) {
                    const double zn = reinterpret_cast<const double*>(row)[cc];
                    const long long kn = dkey64(zn);
                    if ((kn >= p.ndd_lo && kn <= p.ndd_hi) || kz <= kn) continue;  // nodata or not lower
                    d = (float)__dsub_rn(zd, zn);
                } else {
                    const float zn = reinterpret_cast<const float*>(row)[cc];
                    if (p.ndf.has(zn) || zf <= zn) continue;
                    d = __fsub_rn(zf, zn);
                }
                drop[k] = __fdiv_rn(d, diag ? p.den_diag : p.den_card);
                len[k] = diag ? p.len_diag : p.len_card;
                maxd = fmaxf(maxd, drop[k]);
            }
        }
        if (nd_out) {
#pragma unroll
            for (int q = 0; q < 8; q++) put_value(p.w[q], r, c, p.w[q].nodata);
            continue;
        }
        if (maxd > 1.0f) maxd = 1.0f;
        const float pe = (1.0f - p.slp_exp) * maxd + p.slp_exp;
        float t[9], sum = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            t[k] = powf(drop[k], pe) * len[k];  // 0^pe * 0: 0, or NaN when pe < 0 (as the reference's pow)
            sum += t[k];
        }
        const bool any = sum > 0.0f;
#pragma unroll
        for (int q = 0; q < 8; q++) put_float(p.w[q], r, c, any ? __fdiv_rn(t[pos_of_layer(q)], sum) : 0.0f);
    }
}

// ------------------------------------------------------------------ SCA --
__device__ __forceinline__ bool w0_nodata(const ScaMfdParams& p, int64_t r, int64_t c) {
    // |w - nd| < 1e-6 (scaOperator.cpp:47), as a band of order-preserving keys
    const char* row = p.w[0].base + r * p.w[0].pitch;
    const long long k = p.w[0].dtype == PARGO_F64 ? dkey64(reinterpret_cast<const double*>(row)[c])
                                                  : fkey64(reinterpret_cast<const float*>(row)[c]);
    return k >= p.nd_lo && k <= p.nd_hi;
}

__global__ void __launch_bounds__(kThreads) sca_mfd_init_kernel(const ScaMfdParams p) {
    const int64_t n = p.rows * p.cols;
    unsigned long long nvalid = 0, bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        const bool work = r >= 1 && c >= 1 && r <= p.rows - 2 && c <= p.cols - 2;
        uint8_t f = 0;
        if (work) {
            const bool valid = !w0_nodata(p, r, c);
            int indeg = 0, cnt = 0;
            for (int k = 0; k < 9; k++) {
                if (k == 4) continue;
                const int64_t qr = r + k / 3 - 1, qc = c + k % 3 - 1;
                if (!positive(p.w[layer_towards_centre(k)], qr, qc)) continue;
                indeg++;
                const bool qwork = qr >= 1 && qc >= 1 && qr <= p.rows - 2 && qc <= p.cols - 2;
                if (qwork && !w0_nodata(p, qr, qc)) cnt++;
            }
            if (valid) {
                f = kValid | (indeg == 0 ? kSource : 0) | (indeg > cnt ? kNeverDone : 0);
                nvalid++;
            } else {
                bool out = false;
                for (int q = 0; q < 8; q++) out = out || positive(p.w[q], r, c);
                if (indeg > 0 || out) bad++;  // weights into or out of a nodata cell
            }
        }
        p.flags[i] = f;
    }
    if (nvalid) atomicAdd(&p.totals[0], nvalid);
    if (bad) atomicAdd(&p.totals[2], bad);
}

// What a cell waits for: the sweep pulls an inflow n into c only when n is a
// source (its sum is 1 from the start) or n precedes c in raster order and
// is done, so c's sum and flag depend on its inflows at window positions 0-3
// (NW, N, NE, W) that are valid work cells and not sources, and on nothing
// that follows it.  cnt = the number of those; cells with none form the first
// frontier (appended with one atomic per warp).
__global__ void __launch_bounds__(kThreads) sca_mfd_counts_kernel(const ScaMfdParams p) {
    const int64_t n = p.rows * p.cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        const uint8_t f = p.flags[i];
        int cnt = 0;
        if (f & kValid) {  // a valid work cell: its 8 neighbours are in the raster
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int64_t qr = r + k / 3 - 1, qc = c + k % 3 - 1;
                const uint8_t fq = p.flags[qr * p.cols + qc];  // 0 on the ring
                if ((fq & kValid) && !(fq & kSource) && positive(p.w[layer_towards_centre(k)], qr, qc)) cnt++;
            }
        }
        p.cnt[i] = cnt;
        if ((f & kValid) && !(f & kSource)) {
            unsigned rel = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int pos = pos_of_layer(4 + j);  // 5 .. 8: after the cell in raster order
                const uint8_t fd = p.flags[i + (int64_t)(pos / 3 - 1) * p.cols + (pos % 3 - 1)];  // 0 on the ring
                if ((fd & kValid) && positive(p.w[4 + j], r, c)) rel |= 1u << j;
            }
            // only this thread writes this byte; kValid and kSource, which others
            // read here, keep their values
            if (rel) p.flags[i] = (uint8_t)(f | (rel << kReleaseShift));
        }
        const bool first = (f & kValid) && cnt == 0;
        const unsigned act = __activemask();
        const unsigned m = __ballot_sync(act, first);
        if (m) {
            const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
            int32_t base = 0;
            if (lane == leader) base = atomicAdd(&p.counts[0], __popc(m));
            base = __shfl_sync(act, base, leader);
            if (first) p.list_a[base + __popc(m & ((1u << lane) - 1u))] = (int32_t)i;
        }
    }
}

// the cell of layer q's receiver
__device__ __forceinline__ int64_t receiver(const ScaMfdParams& p, int64_t i, int q) {
    const int pos = pos_of_layer(q);
    return i + (int64_t)(pos / 3 - 1) * p.cols + (pos % 3 - 1);
}

// A weight: whether it is > 0 (positive() above) and its value, from one load.
__device__ __forceinline__ double weight_at(const InView& v, int64_t r, int64_t c, bool& pos) {
    const char* row = v.base + r * v.pitch;
    if (v.dtype == PARGO_F64) {
        const long long b = reinterpret_cast<const long long*>(row)[c];
        pos = b > 0 && b <= 0x7FF0000000000000LL;
        return __longlong_as_double(b);
    }
    const float f = reinterpret_cast<const float*>(row)[c];
    pos = f > 0.0f;
    return (double)f;
}

// One cell of a frontier: its sum and done flag, then the counters of the
// cells it flows into; a counter reaching zero queues that cell in `next`.
// A frontier cell is a work cell, so its 8 neighbours are in the raster, and
// every cell it may pull from was finished in an earlier round: all its loads
// (the 8 inflow weights, flags and sums, then the 8 outflow weights and
// flags) are issued before the first is used, and the counter decrements go
// out together -- a level costs a few memory round trips, not one per
// neighbour.  The sum is still taken in the reference's window order.
// Returns the layers q whose receiving cell this call made ready (its last
// inflow): bit q.
__device__ __forceinline__ unsigned sca_mfd_process(const ScaMfdParams& p, int64_t i) {
    const int64_t r = i / p.cols, c = i % p.cols;
    double wq[8], sq[8];
    bool pq[8];
    uint8_t fq[8];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int k = t < 4 ? t : t + 1;  // window position
        const int64_t qr = r + k / 3 - 1, qc = c + k % 3 - 1;
        wq[t] = weight_at(p.w[layer_towards_centre(k)], qr, qc, pq[t]);
        const int64_t q = qr * p.cols + qc;
        fq[t] = p.flags[q];
        sq[t] = p.sca[q];
    }
    const uint8_t fi = p.flags[i];
    double sum = 1.0;
    bool done = !(fi & kNeverDone);
#pragma unroll
    for (int t = 0; t < 8; t++) {  // window order, as the reference sweeps it
        if (!pq[t]) continue;
        const int k = t < 4 ? t : t + 1;
        const int64_t q = i + (int64_t)(k / 3 - 1) * p.cols + (k % 3 - 1);
        const bool src = (fq[t] & kSource) != 0;
        const bool pulled = (fq[t] & kValid) && (src || (q < i && (fq[t] & kDone)));
        // a source's sum is 1 (it has no inflow), whether or not it has been processed yet
        if (pulled) sum = __dadd_rn(sum, __dmul_rn(src ? 1.0 : sq[t], wq[t]));
        else done = false;
    }
    p.sca[i] = sum;
    p.flags[i] = fi | (done ? kDone : 0);
    __threadfence();  // this cell's sum and flag before the counters that release its receivers
    // the receivers that counted this cell (set up front in its flags)
    const unsigned rel = fi >> kReleaseShift;
    int left[4];
#pragma unroll
    for (int j = 0; j < 4; j++) left[j] = (rel >> j) & 1u ? atomicSub(&p.cnt[receiver(p, i, 4 + j)], 1) : 0;
    unsigned ready = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) ready |= (left[j] == 1 ? 1u : 0u) << (4 + j);
    return ready;
}

__device__ __forceinline__ void sca_mfd_cell(const ScaMfdParams& p, int64_t i, int32_t* next, int32_t* next_count) {
    unsigned ready = sca_mfd_process(p, i);
    while (ready) {
        const int q = __ffs(ready) - 1;
        ready &= ready - 1;
        next[atomicAdd(next_count, 1)] = (int32_t)receiver(p, i, q);
    }
}

// One round: process the current frontier, queue the cells whose last inflow it was.
__global__ void __launch_bounds__(kThreads) sca_mfd_round_kernel(const ScaMfdParams p, int parity) {
    int32_t* cur = parity ? p.list_b : p.list_a;
    int32_t* next = parity ? p.list_a : p.list_b;
    int32_t* cur_count = &p.counts[parity];
    int32_t* next_count = &p.counts[parity ^ 1];
    const int32_t ncur = *((volatile int32_t*)cur_count);
    unsigned long long done_cells = 0;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < ncur;
         idx += (int64_t)gridDim.x * blockDim.x) {
        sca_mfd_cell(p, cur[idx], next, next_count);
        done_cells++;
    }
    if (done_cells) atomicAdd(&p.totals[1], done_cells);
    // the last block to finish empties the consumed list
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&p.counts[2], 1) == (int32_t)gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        *cur_count = 0;
        p.counts[2] = 0;
        __threadfence();
    }
}

// ---------------------------------------------------------- band form --
// Every dependency of the sweep points forward in raster order: a cell needs
// only its NW, N, NE and W neighbours' sums and done flags (the sources
// anywhere count as 1).  A warp takes a band of 32 rows; lane L walks row
// R0 + L, two columns behind lane L - 1 (at step s it is at column
// 1 + s - 2L), so the three upper neighbours of its cell are the results of
// lane L - 1's last three steps (shuffles) and the left one is its own last
// result.  Lane 0's upper row is the previous band's last row, read from
// global memory in chunks of 8 columns once that band has published them
// (bands are taken in order, so the band waited on is running or done; the
// wait sleeps 20 ns at a time, gives up after kBandPatience cycles without
// progress and sets the error flag).
// A cell's static data -- the 8 inflow weights and the valid / source /
// positive masks of its neighbours -- is gathered first into one record per
// cell (sca_mfd_records_kernel) and streamed by each lane a few steps ahead
// with asynchronous copies.

// rm bits: 0-3 the cell's own static flags; 8-15 positive inflow weight from
// neighbour t (window order t = 0..7: positions 0-3, 5-8); 16-23 that
// neighbour is a valid work cell; 24-31 it is a source.
template <typename WT>
__global__ void __launch_bounds__(kThreads) sca_mfd_records_kernel(const ScaMfdParams p, WT* rw, uint32_t* rm) {
    const int64_t n = p.rows * p.cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t fi = p.flags[i];
        uint32_t m = 0;
        if (fi & kValid) {  // a valid work cell: its 8 neighbours are in the raster
            const int64_t r = i / p.cols, c = i % p.cols;
            m = fi & 0x0Fu;
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int k = t < 4 ? t : t + 1;
                const int64_t qr = r + k / 3 - 1, qc = c + k % 3 - 1;
                bool pos;
                const double w = weight_at(p.w[layer_towards_centre(k)], qr, qc, pos);
                const uint8_t fq = p.flags[qr * p.cols + qc];
                rw[i * 8 + t] = pos ? (WT)w : (WT)0;  // exact: WT is the weights' own type
                m |= (pos ? 1u : 0u) << (8 + t);
                m |= ((fq & kValid) ? 1u : 0u) << (16 + t);
                m |= ((fq & kSource) ? 1u : 0u) << (24 + t);
            }
        }
        rm[i] = m;
    }
}

constexpr int kBandRows = 32;
constexpr int kBandPre = 8;    // record slots a lane has in flight (16 measured no faster)
constexpr int kBandWarps = 4;  // bands (warps) per block
constexpr int kBandChunk = 8;  // columns of the previous band's last row published and read at a time
constexpr long long kBandPatience = 4000000000LL;  // ~2 s of SM clocks without the previous band moving

template <typename WT>
struct BandSmem {
    WT w[kBandPre][8][32];              // [slot][t][lane]
    uint32_t m[kBandPre][32];
    double up[64];                      // the previous band's last row, a ring of 64 columns
    uint8_t upd[64];                    // its done flags
};

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}

// One warp per band; kBandWarps warps per block, each with its own smem.
template <typename WT>
__global__ void __launch_bounds__(kBandWarps * 32) sca_mfd_band_kernel(const ScaMfdParams p, const WT* rw, const uint32_t* rm,
                                                               int* band_next, int* prog, int nbands) {
    extern __shared__ __align__(16) unsigned char band_smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    BandSmem<WT>& S = reinterpret_cast<BandSmem<WT>*>(band_smem)[wid];
    const int64_t cols = p.cols, last_col = p.cols - 2;  // work columns 1 .. cols - 2
    const int64_t nsteps = last_col + 2 * (kBandRows - 1);
    unsigned long long processed = 0;
    bool failed = false;
    for (;;) {
        int b = 0;
        if (lane == 0) b = atomicAdd(band_next, 1);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= nbands || failed) break;
        const int64_t R0 = 1 + (int64_t)b * kBandRows, r = R0 + lane;
        const bool row_ok = r <= p.rows - 2;
        // the previous band's last row (row R0 - 1), chunk j = columns 8j .. 8j + 7
        auto load_chunk = [&](int64_t j) -> bool {
            const int64_t c_hi = min(kBandChunk * j + kBandChunk - 1, last_col);
            if (b > 0 && c_hi >= 1) {
                if (lane == 0) {
                    const long long t0 = clock64();
                    while (*((volatile int*)&prog[b - 1]) < c_hi) {
                        if (*((volatile int*)p.error_flag) != 0 || clock64() - t0 > kBandPatience) {
                            atomicExch(p.error_flag, 1);
                            failed = true;
                            break;
                        }
                        __nanosleep(20);  // the band above is a few steps ahead: short sleeps
                    }
                    __threadfence();
                }
                failed = __shfl_sync(0xffffffffu, failed, 0);
                __syncwarp();  // orders lane 0's observation before the other lanes' loads
            }
            const int64_t c = kBandChunk * j + lane;
            double v = 0.0;
            uint8_t d = 0;
            if (lane < kBandChunk && b > 0 && !failed && c >= 1 && c <= last_col) {
                const int64_t g = (R0 - 1) * cols + c;
                v = __ldcg(p.sca + g);
                d = (__ldcg(reinterpret_cast<const unsigned*>(p.flags + (g & ~3LL))) >> (8 * (g & 3))) & kDone;
            }
            if (lane < kBandChunk) {
                S.up[c & 63] = v;
                S.upd[c & 63] = d;
            }
            __syncwarp();
            return !failed;
        };
        // the record of this lane's cell at step s into slot s % kBandPre
        auto fetch = [&](int64_t s) {
            const int slot = (int)(s % kBandPre);
            const int64_t c = 1 + s - 2 * lane;
            if (row_ok && c >= 1 && c <= last_col) {
                const int64_t i = r * cols + c;
#pragma unroll
                for (int t = 0; t < 8; t++) {
                    if (sizeof(WT) == 8) cp_async8(&S.w[slot][t][lane], rw + i * 8 + t);
                    else cp_async4(&S.w[slot][t][lane], rw + i * 8 + t);
                }
                cp_async4(&S.m[slot][lane], rm + i);
            } else {
                S.m[slot][lane] = 0;  // no cell: nothing to process
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        };
        if (!load_chunk(0)) break;
        for (int64_t s = 0; s < kBandPre - 1; s++) fetch(s);
        double h0 = 0.0, h1 = 0.0, h2 = 0.0;  // this lane's results at steps s-1, s-2, s-3
        unsigned hd = 0;                        // their done flags: bit 0 = s-1, bit 1 = s-2, bit 2 = s-3
        for (int64_t s = 0; s < nsteps; s++) {
            if ((s % kBandChunk) == 0 && !load_chunk(s / kBandChunk + 1)) break;
            fetch(s + kBandPre - 1);
            asm volatile("cp.async.wait_group %0;\n" ::"n"(kBandPre - 1) : "memory");
            // upper neighbours at columns c-1, c, c+1: lane L-1's last three results
            double u0 = __shfl_up_sync(0xffffffffu, h2, 1), u1 = __shfl_up_sync(0xffffffffu, h1, 1),
                   u2 = __shfl_up_sync(0xffffffffu, h0, 1);
            unsigned ud = __shfl_up_sync(0xffffffffu, hd, 1);  // bit 2: c-1, bit 1: c, bit 0: c+1
            const int64_t c = 1 + s - 2 * lane;
            if (lane == 0) {  // the previous band's last row, columns s .. s + 2
                u0 = S.up[s & 63];
                u1 = S.up[(s + 1) & 63];
                u2 = S.up[(s + 2) & 63];
                ud = (S.upd[s & 63] ? 4u : 0u) | (S.upd[(s + 1) & 63] ? 2u : 0u) | (S.upd[(s + 2) & 63] ? 1u : 0u);
            }
            const int slot = (int)(s % kBandPre);
            const uint32_t m = S.m[slot][lane];
            double sum = 0.0;
            bool done = false;
            if (m & kValid) {
                sum = 1.0;
                // the inflows the sweep pulls: valid and a source, or one of the
                // earlier four (NW, N, NE, W) and done
                const unsigned pos = (m >> 8) & 0xFFu, val = (m >> 16) & 0xFFu, src = (m >> 24) & 0xFFu;
                const unsigned dn = ((ud >> 2) & 1u) | (((ud >> 1) & 1u) << 1) | ((ud & 1u) << 2) | ((hd & 1u) << 3);
                unsigned pulled = pos & val & (src | dn);
                done = !(m & kNeverDone) && pulled == pos;
                while (pulled) {  // in window order, as the reference sweeps it
                    const int t = __ffs(pulled) - 1;
                    pulled &= pulled - 1;
                    const double x = (src >> t) & 1u ? 1.0 : t == 0 ? u0 : t == 1 ? u1 : t == 2 ? u2 : h0;
                    sum = __dadd_rn(sum, __dmul_rn(x, (double)S.w[slot][t][lane]));
                }
                const int64_t g = r * cols + c;
                p.sca[g] = sum;
                p.flags[g] = (uint8_t)((m & 0x0Fu) | (done ? kDone : 0));
                processed++;
            }
            h2 = h1;
            h1 = h0;
            h0 = sum;
            hd = ((hd << 1) | (done ? 1u : 0u)) & 7u;
            // the last lane publishes its row's progress every kBandChunk columns
            if (lane == kBandRows - 1 && c >= 1 && c <= last_col &&
                ((c % kBandChunk) == kBandChunk - 1 || c == last_col)) {
                __threadfence();
                atomicExch(&prog[b], (int)c);
            }
            __syncwarp();
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        __syncwarp();
    }
    const unsigned long long tot = __reduce_add_sync(0xffffffffu, (unsigned)processed);
    if (lane == 0 && tot) atomicAdd(&p.totals[1], tot);
}

__global__ void __launch_bounds__(kThreads) sca_mfd_output_kernel(const ScaMfdParams p) {
    const int64_t n = p.rows * p.cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        put_value(p.out, r, c, (p.flags[i] & kValid) ? p.sca[i] : p.nodata);
    }
}

int64_t blocks_for(int64_t n, int num_sms) {
    int64_t b = (n + kThreads - 1) / kThreads;
    if (b > (int64_t)num_sms * 16) b = (int64_t)num_sms * 16;
    return b < 1 ? 1 : b;
}

}  // namespace

cudaError_t launch_mfd_weights(const MfdParams& p, int num_sms, cudaStream_t st) {
    if (p.rows * p.cols == 0) return cudaSuccess;
    mfd_weights_kernel<<<(unsigned)blocks_for(p.rows * p.cols, num_sms), kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_sca_mfd_init(const ScaMfdParams& p, int num_sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(p.counts, 0, 4 * sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(p.totals, 0, 4 * sizeof(unsigned long long), st)) != cudaSuccess) return e;
    sca_mfd_init_kernel<<<(unsigned)blocks_for(p.rows * p.cols, num_sms), kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_sca_mfd_counts(const ScaMfdParams& p, int num_sms, cudaStream_t st) {
    sca_mfd_counts_kernel<<<(unsigned)blocks_for(p.rows * p.cols, num_sms), kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_sca_mfd_round(const ScaMfdParams& p, int parity, int num_sms, cudaStream_t st) {
    // a grid sized for the frontier the image can hold at once; the kernel strides
    sca_mfd_round_kernel<<<(unsigned)num_sms * 4, kThreads, 0, st>>>(p, parity);
    return cudaGetLastError();
}


// The band form: records, then one launch of 32-row bands.  `words` holds the
// band cursor and one progress word per band.
size_t sca_mfd_band_bytes(int64_t rows, int64_t cols, bool f32) {
    return (size_t)(rows * cols) * ((f32 ? 4 : 8) * 8 + 4) + 256;
}

template <typename WT>
static cudaError_t launch_band(const ScaMfdParams& p, void* records, int* words, int num_sms, cudaStream_t st) {
    const int64_t n = p.rows * p.cols;
    WT* rw = reinterpret_cast<WT*>(((uintptr_t)records + 15) & ~(uintptr_t)15);
    uint32_t* rm = reinterpret_cast<uint32_t*>(rw + n * 8);
    const int nbands = (int)((p.rows - 2 + kBandRows - 1) / kBandRows);
    cudaError_t e = cudaMemsetAsync(words, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(words + 1, 0xFF, (size_t)nbands * sizeof(int), st)) != cudaSuccess) return e;
    sca_mfd_records_kernel<WT><<<(unsigned)blocks_for(n, num_sms), kThreads, 0, st>>>(p, rw, rm);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int smem = kBandWarps * (int)sizeof(BandSmem<WT>);
    if ((e = cudaFuncSetAttribute(sca_mfd_band_kernel<WT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) !=
        cudaSuccess)
        return e;
    // enough warps for every band at once (bands are taken in order, so none
    // waits on a band no warp has taken)
    int64_t blocks = (nbands + kBandWarps - 1) / kBandWarps;
    if (blocks < num_sms) blocks = num_sms;
    sca_mfd_band_kernel<WT><<<(unsigned)blocks, kBandWarps * 32, smem, st>>>(p, rw, rm, words, words + 1, nbands);
    return cudaGetLastError();
}

cudaError_t launch_sca_mfd_band(const ScaMfdParams& p, void* records, int* words, int num_sms, cudaStream_t st) {
    if (p.rows < 3 || p.cols < 3) return cudaSuccess;  // no work cell
    bool f32 = true;
    for (int q = 0; q < 8; q++) f32 = f32 && p.w[q].dtype == PARGO_F32;
    return f32 ? launch_band<float>(p, records, words, num_sms, st) : launch_band<double>(p, records, words, num_sms, st);
}

cudaError_t launch_sca_mfd_output(const ScaMfdParams& p, int num_sms, cudaStream_t st) {
    sca_mfd_output_kernel<<<(unsigned)blocks_for(p.rows * p.cols, num_sms), kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace pargo
