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
// is processed once its inflows that precede it in raster order and are valid
// work cells other than sources are processed (counters; the thread that
// releases a cell's last such inflow processes it next, see the walk form
// below) -- nothing that follows it, so the chains are the flow paths that
// keep going forward in raster order (2048^2 hydro: 632 levels, against 3264
// when every inflow was waited on).  It then adds, in the reference's window
// order and in FP64 with separately rounded products and sums, the inflows
// the sweep pulls (source, or earlier in raster order and done), so with the
// same weights the result equals the reference's bit for bit.  Inflows from
// cells that are never processed (the ring, nodata) are never pulled.

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

constexpr long long kWaitBudget = 4000000000LL;  // ~2 s of SM clocks without a queued cell arriving

// Walk form, one persistent launch with every block resident.  A thread takes
// a ready cell (the first frontier, then cells queued by other threads),
// processes it, and goes on at once with a receiver this made ready -- its
// last inflow is then final -- queuing any further ready receivers; a
// thread's walk follows the flow down the DAG, so no round waits on the
// slowest cell of a level.  Each cell is processed once, after all its
// inflows (their counters), so the sums are those of the rounds.
//   counts[0]  cells of the first frontier (list_a), from the init kernel
//   counts[3]  claimed from list_a
//   counts[1]  queued in list_b (each cell at most once: room for every cell)
//   counts[2]  claimed from list_b
//   barrier[0] pending: ready cells not yet finished, raised before a cell is
//              queued and lowered when a walk ends -- zero exactly when every
//              ready cell is done.
// list_b starts filled with -1; a claimed position is waited on until its
// cell is written (bounded: the error flag ends the launch).
__global__ void sca_mfd_walk_setup_kernel(const ScaMfdParams p) {
    p.barrier[0] = (unsigned int)p.counts[0];
    p.counts[1] = 0;
    p.counts[2] = 0;
    p.counts[3] = 0;
}

__device__ int64_t walk_claim(const ScaMfdParams& p, int64_t n) {
    const int32_t a = atomicAdd(&p.counts[3], 1);
    if (a < *((volatile int32_t*)&p.counts[0])) return p.list_a[a];
    const int32_t b = atomicAdd(&p.counts[2], 1);
    const long long t0 = clock64();
    unsigned ns = 32;
    for (;;) {
        if (b < n) {
            const int32_t v = *((volatile int32_t*)&p.list_b[b]);
            if (v >= 0) return v;
        }
        if (*((volatile unsigned int*)&p.barrier[0]) == 0) return -1;  // every ready cell done
        if (*((volatile int*)p.error_flag) != 0) return -1;
        if (clock64() - t0 > kWaitBudget) {
            atomicExch(p.error_flag, 1);
            return -1;
        }
        __nanosleep(ns);
        if (ns < 1024) ns *= 2;
    }
}

__global__ void __launch_bounds__(kThreads) sca_mfd_walk_kernel(const ScaMfdParams p) {
    const int64_t n = p.rows * p.cols;
    unsigned long long done_cells = 0;
    for (;;) {
        int64_t cell = walk_claim(p, n);
        if (cell < 0) break;
        while (cell >= 0) {
            __threadfence();  // the released inflows' sums and flags are visible
            unsigned ready = sca_mfd_process(p, cell);
            done_cells++;
            const int nr = __popc(ready);
            int64_t next = -1;
            if (nr) {
                const int q0 = __ffs(ready) - 1;
                next = receiver(p, cell, q0);
                ready &= ready - 1;
                if (nr > 1) {
                    __threadfence();  // what released these cells is visible to whoever takes them
                    atomicAdd(&p.barrier[0], (unsigned int)(nr - 1));  // raised before the cells are queued
                    const int32_t pos = atomicAdd(&p.counts[1], nr - 1);
                    int k = 0;
                    while (ready) {
                        const int q = __ffs(ready) - 1;
                        ready &= ready - 1;
                        if (pos + k < n) atomicExch(&p.list_b[pos + k], (int32_t)receiver(p, cell, q));
                        k++;
                    }
                }
            } else {
                atomicAdd(&p.barrier[0], 0xFFFFFFFFu);  // this walk ends: one pending cell fewer
            }
            cell = next;
        }
    }
    const unsigned dc = __reduce_add_sync(__activemask(), (unsigned)done_cells);
    if ((threadIdx.x & 31) == __ffs(__activemask()) - 1 && dc) atomicAdd(&p.totals[1], (unsigned long long)dc);
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
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_mfd_counts_kernel<<<(unsigned)blocks_for(p.rows * p.cols, num_sms), kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_sca_mfd_round(const ScaMfdParams& p, int parity, int num_sms, cudaStream_t st) {
    // a grid sized for the frontier the image can hold at once; the kernel strides
    sca_mfd_round_kernel<<<(unsigned)num_sms * 4, kThreads, 0, st>>>(p, parity);
    return cudaGetLastError();
}

cudaError_t launch_sca_mfd_persistent(const ScaMfdParams& p, int num_sms, cudaStream_t st) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sca_mfd_walk_kernel, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
    const int64_t n = p.rows * p.cols;
    if ((e = cudaMemsetAsync(p.list_b, 0xFF, (size_t)n * sizeof(int32_t), st)) != cudaSuccess) return e;
    sca_mfd_walk_setup_kernel<<<1, 1, 0, st>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // every block resident: a thread waiting for a queued cell never waits on
    // a block that has not started
    // one block per SM: more walkers than that only contend for the queue
    // (8192^2: 64 ms with one block per SM, 77 / 90 / 104 ms with 2 / 3 / 4;
    // half the SMs, 71 ms)
    sca_mfd_walk_kernel<<<(unsigned)num_sms, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_sca_mfd_output(const ScaMfdParams& p, int num_sms, cudaStream_t st) {
    sca_mfd_output_kernel<<<(unsigned)blocks_for(p.rows * p.cols, num_sms), kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace pargo
