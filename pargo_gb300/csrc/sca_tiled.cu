// sca_tiled.cu -- D8 specific catchment area as subtree sums over the flow
// forest, tiled so that the long serial chains stay in shared memory.
//
// Reference: SCAOperator::Operator (apps/hydrology/scad8/scaOperator.cpp:37-131).
// Flow forest: the parent of a valid work cell c is the cell its code names,
// when that cell is a valid work cell that does not name c back (a mutual
// pair is no inflow, :71).  Converged SCA = subtree size (counts are integers:
// exact in any summation order).  The shipped single raster-order sweep pulls
// the inflow p -> c when p is a source or p precedes c and p is "done"; p is
// done exactly when no cell u of p's subtree has a non-source inflow q that
// follows u in raster order ("bad" cells), so done is an OR over the subtree
// -- a second subtree reduction -- and shipped(c) = 1 + the pulled children's
// subtree sizes, gathered in the output pass.
//
// Phases (one launch each):
//  1. per 64 x 64 tile (codes with a 2-cell halo in shared memory): the in-tile
//     forest, its subtree sums by a shared-memory topological walk (in-degree
//     counters; the last contributor continues), and for every border cell the
//     exit its in-tile path reaches.  Exits (cells whose parent lies in another
//     tile) record their in-tile sum and the entry cell they feed.
//  2. the exit forest: exit x's parent is the exit reached from the entry x
//     feeds; its in-degrees.
//  3. subtree sums over the exit forest (its leaves marked first, then a
//     global-memory walk; chains are as long as the tiles a river crosses);
//     each exit adds its total to the inflow of the entry it feeds.
//  4. per tile again: the in-tile sums with the entries' inflows added -> the
//     final counts and flags.
//  5. output: converged counts, or the shipped sums; the reference's last-cell
//     quirk (a nodata last work cell accumulates what flows into it).
// Cycles (inside a tile or across tiles) and inflows from the raster's ring,
// which the reference never releases, leave cells or exits uncompleted; the
// host compares the completion counts.

#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

constexpr int kT = kScaTile;       // tile side
constexpr int kH = kT + 4;         // codes with a 2-cell halo
constexpr int kCells = kT * kT;
constexpr int8_t kNodata = -1, kNoFlow = -2;

__device__ __forceinline__ int8_t decode8(const ScaParams& p, int64_t r, int64_t c) {
    if (r < 0 || c < 0 || r >= p.rows || c >= p.cols) return kNodata;
    const char* row = p.d8.base + r * p.d8.pitch;
    double v;
    switch (p.d8.dtype) {
        case PARGO_F64: v = reinterpret_cast<const double*>(row)[c]; break;
        case PARGO_F32: v = (double)reinterpret_cast<const float*>(row)[c]; break;
        case PARGO_I8: v = (double)reinterpret_cast<const int8_t*>(row)[c]; break;
        case PARGO_I16: v = (double)reinterpret_cast<const int16_t*>(row)[c]; break;
        default: v = (double)reinterpret_cast<const int32_t*>(row)[c]; break;
    }
    const bool nd = (p.d8.dtype == PARGO_F64 || p.d8.dtype == PARGO_F32) ? fabs(v - p.nodata) < kEpsHydro
                                                                        : v == p.nodata;  // scaOperator.cpp:48
    if (nd) return kNodata;
    const int k = (int)v;
    return ((double)k == v && k >= 0 && k <= 8 && k != 4) ? (int8_t)k : kNoFlow;
}

__device__ __forceinline__ bool in_work(const ScaParams& p, int64_t r, int64_t c) {
    return r >= 1 && c >= 1 && r <= p.rows - 2 && c <= p.cols - 2;
}

// Border slot of tile-local (lr, lc) in a th x tw tile, or -1 inside.
__device__ __forceinline__ int slot_of(int lr, int lc, int th, int tw) {
    if (lr == 0) return lc;
    if (lr == th - 1) return tw + lc;
    if (lc == 0) return 2 * tw + (lr - 1);
    if (lc == tw - 1) return 2 * tw + (th - 2) + (lr - 1);
    return -1;
}

// Shared state of one tile.  The in-tile flow forest is summed by the Euler
// tour technique: every non-root cell v contributes two tour elements,
// down(v) = 2v (weight w(v)) and up(v) = 2v + 1 (weight 0); the tour of a
// tree visits down(v), the tours of v's children, up(v).  Suffix sums along
// the tours by pointer jumping (log2 of the tour length rounds, each a
// read phase and a write phase between barriers) give every subtree sum as
// R(down(v)) - R(up(v)), so no thread walks a chain: a filled lake makes
// in-tile flow paths thousands of cells long, and walking them one thread per
// chain made the tile passes latency bound.  A weight packs two counts:
// the cell's own count 1 + inflow (low field) and whether it is "bad" (high
// field), so one ranking gives the subtree sum and the subtree OR of "bad".
// Roots are found by pointer jumping on the parents (log2(cells) rounds); a
// cell whose chain reaches no root lies on or above a cycle and is not
// completed.
template <bool FINAL>
struct TileSmem {
    // packed tour weights: first pass 16 + 16 bits, final pass 48 + 16 bits
    using Val = typename std::conditional<FINAL, unsigned long long, unsigned int>::type;
    static constexpr int kBadShift = FINAL ? 48 : 16;
    int8_t cd[kH * kH];                  // codes, (a, b) = (r - r0 + 2, c - c0 + 2)
    uint8_t src[(kT + 2) * (kT + 2)];    // the tile and a one-cell ring: reference in-degree is zero
    uint8_t flags[kCells];               // 1 valid work cell, 2 bad, 4 completed, 16 an unpulled inflow from another tile
    int16_t lpar[kCells];                // in-tile parent, -1 none, -2 outside the tile
    int16_t root[kCells];                // pointer jumping towards the chain's last cell
    int16_t next[2 * kCells];            // tour successor, -1 at the end
    Val val[2 * kCells];                 // tour weights, then suffix sums
    unsigned long long cnt[3];           // valid, completed, ring inflows
};

constexpr int kTourThreads = 512;
constexpr int kCellsPerThread = kCells / kTourThreads;  // 8
constexpr int kElemsPerThread = 2 * kCellsPerThread;    // 16

// Whether the neighbour at (a, b) of the cell at codes position (ca, cb)
// flows into it: its code names the cell and the cell does not name it back.
template <class S_t>
__device__ __forceinline__ bool flows_in(const S_t& S, int ca, int cb, int a, int b) {
    const int k = (a + 1) * 3 + (b + 1);  // window index of the neighbour seen from the cell
    const int8_t q = S.cd[(ca + a) * kH + (cb + b)];
    return q == 8 - k && S.cd[ca * kH + cb] != k;
}

// First in-tile child of v after window position `after` (-1: from the
// start), or -1: the neighbours whose in-tile parent is v, in window order.
template <class S_t>
__device__ __forceinline__ int child_after(const S_t& S, int v, int after, int th, int tw) {
    const int vr = v / kT, vc = v % kT;
#pragma unroll 1
    for (int k = after + 1; k < 9; k++) {
        if (k == 4) continue;
        const int qr = vr + k / 3 - 1, qc = vc + k % 3 - 1;
        if (qr < 0 || qc < 0 || qr >= th || qc >= tw) continue;
        const int q = qr * kT + qc;
        if (S.lpar[q] == v) return q;
    }
    return -1;
}

template <bool FINAL>
__global__ void __launch_bounds__(kTourThreads, 2) sca_tile_kernel(const ScaParams p, ScaScratch s, ScaTiles T) {
    extern __shared__ __align__(16) unsigned char sca_smem[];
    using Smem = TileSmem<FINAL>;
    using Val = typename Smem::Val;
    Smem& S = *reinterpret_cast<Smem*>(sca_smem);
    const int tid = threadIdx.x;
    const int64_t ntiles = T.tiles_x * T.tiles_y;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t r0 = (t / T.tiles_x) * kT, c0 = (t % T.tiles_x) * kT;
        const int th = (int)min((int64_t)kT, p.rows - r0), tw = (int)min((int64_t)kT, p.cols - c0);
        if (tid < 3) S.cnt[tid] = 0;
        if (!FINAL && tid < kScaSlots) {  // every slot starts as "no exit"; the exit forest's accumulators empty
            const int64_t node = t * kScaSlots + tid;
            T.exit_of[node] = -1;
            T.yslot[node] = -1;
            T.xdeg[node] = 0;
            T.tin[node] = 0;
            T.tinb[node] = 0;
        }
        for (int i = tid; i < kH * kH; i += kTourThreads) S.cd[i] = decode8(p, r0 - 2 + i / kH, c0 - 2 + i % kH);
        __syncthreads();
        // Reference sources (in-degree zero) over the tile and a one-cell ring.
        for (int i = tid; i < (kT + 2) * (kT + 2); i += kTourThreads) {
            const int ca = i / (kT + 2) + 1, cb = i % (kT + 2) + 1;
            bool src = true;
#pragma unroll
            for (int a = -1; a <= 1; a++)
#pragma unroll
                for (int b = -1; b <= 1; b++)
                    if ((a || b) && flows_in(S, ca, cb, a, b)) src = false;
            S.src[i] = src ? 1 : 0;
        }
        // The in-tile forest: parents, flags.
        unsigned long long nvalid = 0, nring = 0;
        for (int i = tid; i < kCells; i += kTourThreads) {
            const int lr = i / kT, lc = i % kT;
            const int64_t r = r0 + lr, c = c0 + lc;
            const int ca = lr + 2, cb = lc + 2;
            int16_t lp = -1;
            uint8_t f = 0;
            if (lr < th && lc < tw && in_work(p, r, c) && S.cd[ca * kH + cb] != kNodata) {
                f = 1;
                nvalid++;
                const int8_t k = S.cd[ca * kH + cb];
                if (k >= 0) {
                    const int a = k / 3 - 1, b = k % 3 - 1;
                    const int8_t tk = S.cd[(ca + a) * kH + (cb + b)];
                    if (in_work(p, r + a, c + b) && tk != kNodata && tk != 8 - k) {
                        const int tr = lr + a, tc = lc + b;
                        lp = (tr >= 0 && tc >= 0 && tr < th && tc < tw) ? (int16_t)(tr * kT + tc) : (int16_t)-2;
                    }
                }
                // an inflow from the ring is never released; a non-source child
                // that follows the cell in raster order is not pulled by the
                // single sweep ("bad")
#pragma unroll
                for (int a = -1; a <= 1; a++)
#pragma unroll
                    for (int b = -1; b <= 1; b++) {
                        if (!(a || b) || !flows_in(S, ca, cb, a, b)) continue;
                        if (!in_work(p, r + a, c + b)) {
                            nring++;
                            continue;
                        }
                        if ((a > 0 || (a == 0 && b > 0)) && !S.src[(lr + 1 + a) * (kT + 2) + (lc + 1 + b)]) f |= 2;
                    }
                if (FINAL) {
                    const int sl = slot_of(lr, lc, th, tw);
                    if (sl >= 0 && T.tinb[t * kScaSlots + sl]) f |= 16;  // an inflow from another tile was not pulled
                }
            }
            S.lpar[i] = lp;
            S.root[i] = lp >= 0 ? lp : (int16_t)i;
            S.flags[i] = f;
        }
        atomicAdd(&S.cnt[0], nvalid);
        if (nring) atomicAdd(&S.cnt[2], nring);
        __syncthreads();
        // Tour successors and weights.
        for (int v = tid; v < kCells; v += kTourThreads) {
            const int lp = S.lpar[v];
            Val wd = 0;
            int16_t nd = -1, nu = -1;
            if (lp >= 0) {  // a non-root valid cell (only valid cells have parents)
                const unsigned f = S.flags[v];
                unsigned long long own = 1;
                if (FINAL) {
                    const int sl = slot_of(v / kT, v % kT, th, tw);
                    if (sl >= 0) own += T.tin[t * kScaSlots + sl];
                }
                wd = (Val)own | ((Val)((f & 18u) ? 1u : 0u) << Smem::kBadShift);
                const int fc = child_after(S, v, -1, th, tw);
                nd = fc >= 0 ? (int16_t)(2 * fc) : (int16_t)(2 * v + 1);
                const int kpos = ((v / kT) - (lp / kT) + 1) * 3 + ((v % kT) - (lp % kT) + 1);  // v in lp's window
                const int ns = child_after(S, lp, kpos, th, tw);
                nu = ns >= 0 ? (int16_t)(2 * ns) : (S.lpar[lp] >= 0 ? (int16_t)(2 * lp + 1) : (int16_t)-1);
            }
            S.val[2 * v] = wd;
            S.val[2 * v + 1] = 0;
            S.next[2 * v] = nd;
            S.next[2 * v + 1] = nu;
        }
        __syncthreads();
        // Suffix sums along the tours (Wyllie's pointer jumping).
#pragma unroll 1
        for (int round = 0; round < 14; round++) {
            Val nv[kElemsPerThread];
            int16_t nn[kElemsPerThread];
            bool more = false;
#pragma unroll
            for (int j = 0; j < kElemsPerThread; j++) {
                const int e = tid + j * kTourThreads;
                const int n = S.next[e];
                nv[j] = S.val[e];
                nn[j] = (int16_t)n;
                if (n >= 0) {
                    nv[j] += S.val[n];
                    nn[j] = S.next[n];
                    more = true;
                }
            }
            if (!__syncthreads_or(more)) break;
#pragma unroll
            for (int j = 0; j < kElemsPerThread; j++) {
                const int e = tid + j * kTourThreads;
                S.val[e] = nv[j];
                S.next[e] = nn[j];
            }
            __syncthreads();
        }
        // Roots: pointer jumping on the parents (a chain without a cycle
        // reaches its root within kCells - 1 steps: 12 doublings).
#pragma unroll 1
        for (int round = 0; round < 12; round++) {
            int16_t nr[kCellsPerThread];
#pragma unroll
            for (int j = 0; j < kCellsPerThread; j++) nr[j] = S.root[S.root[tid + j * kTourThreads]];
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kCellsPerThread; j++) S.root[tid + j * kTourThreads] = nr[j];
            __syncthreads();
        }
        // Subtree sums; completion; outputs of the pass.
        unsigned long long ndone = 0;
        for (int v = tid; v < kCells; v += kTourThreads) {
            const unsigned f = S.flags[v];
            if (!(f & 1u)) continue;
            const bool done = S.lpar[S.root[v]] < 0;  // its chain ends at a root
            Val tot;
            if (S.lpar[v] >= 0) {
                tot = S.val[2 * v] - S.val[2 * v + 1];
            } else {  // a root: its own weight and every down edge of its tree
                unsigned long long own = 1;
                if (FINAL) {
                    const int sl = slot_of(v / kT, v % kT, th, tw);
                    if (sl >= 0) own += T.tin[t * kScaSlots + sl];
                }
                tot = (Val)own | ((Val)((f & 18u) ? 1u : 0u) << Smem::kBadShift);
                const int fc = child_after(S, v, -1, th, tw);
                if (fc >= 0) tot += S.val[2 * fc];
            }
            const unsigned long long sum = (unsigned long long)(tot & (((Val)1 << Smem::kBadShift) - 1));
            const unsigned bad = (tot >> Smem::kBadShift) != 0 ? 1u : 0u;
            if (done) ndone++;
            if (FINAL) {
                const int64_t g = (r0 + v / kT) * p.cols + (c0 + v % kT);
                s.conv[g] = done ? sum : 0ULL;
                s.ship[g] = done ? (unsigned long long)bad : 0ULL;
            } else if (done) {
                const int lr = v / kT, lc = v % kT;
                const int sl = slot_of(lr, lc, th, tw);
                if (sl >= 0) {
                    // a border cell: the exit its path reaches; an exit: where its flow enters
                    const int64_t node = t * kScaSlots + sl;
                    const int rt = S.root[v];
                    if (S.lpar[rt] == -2) T.exit_of[node] = (int32_t)(t * kScaSlots + slot_of(rt / kT, rt % kT, th, tw));
                    if (S.lpar[v] == -2) {
                        const int8_t k = S.cd[(lr + 2) * kH + (lc + 2)];
                        const int64_t yr = r0 + lr + k / 3 - 1, yc = c0 + lc + k % 3 - 1;
                        const int64_t yt = (yr / kT) * T.tiles_x + (yc / kT);
                        const int yth = (int)min((int64_t)kT, p.rows - (yr / kT) * kT);
                        const int ytw = (int)min((int64_t)kT, p.cols - (yc / kT) * kT);
                        T.yslot[node] = (int32_t)(yt * kScaSlots + slot_of((int)(yr % kT), (int)(yc % kT), yth, ytw));
                        T.tot[node] = sum;
                        T.totb[node] = bad;
                    }
                }
            }
        }
        atomicAdd(&S.cnt[1], ndone);
        __syncthreads();
        if (tid == 0) {
            if (FINAL) {
                atomicAdd(&s.counters[1], S.cnt[0]);
                atomicAdd(&s.counters[0], S.cnt[1]);
            } else if (S.cnt[2]) {
                atomicAdd(&s.counters[6], S.cnt[2]);
            }
        }
        __syncthreads();
    }
}

// Exit forest: parents and in-degrees.
__global__ void sca_exit_links_kernel(ScaScratch s, ScaTiles T) {
    const int64_t n = T.tiles_x * T.tiles_y * kScaSlots;
    unsigned long long nexit = 0;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t y = T.yslot[x];
        int32_t px = -1;
        if (y >= 0) {
            nexit++;
            px = T.exit_of[y];
            if (px >= 0) atomicAdd(&T.xdeg[px], 1);
        }
        T.xpar[x] = px;
    }
    nexit = __reduce_add_sync(0xffffffffu, (unsigned)nexit);
    if ((threadIdx.x & 31) == 0 && nexit) atomicAdd(&s.counters[4], nexit);
}

// Exit forest: mark its leaves (bit 1 of totb) once every in-degree is known,
// so that the walk below starts from them only.
__global__ void sca_exit_leaves_kernel(ScaTiles T) {
    const int64_t n = T.tiles_x * T.tiles_y * kScaSlots;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x)
        if (T.yslot[x] >= 0 && T.xdeg[x] == 0) T.totb[x] |= 2u;
}

// Exit forest: totals by a topological walk from its leaves; each exit feeds
// its total into the entry it flows into.
__global__ void sca_exit_walk_kernel(ScaScratch s, ScaTiles T) {
    const int64_t n = T.tiles_x * T.tiles_y * kScaSlots;
    unsigned long long ndone = 0;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        if (T.yslot[x] < 0 || !(T.totb[x] & 2u)) continue;
        int64_t cur = x;
        for (;;) {
            const unsigned long long tot = atomicAdd(&T.tot[cur], 0ULL);
            const uint32_t bad = atomicOr(&T.totb[cur], 0u) & 1u;
            const int32_t y = T.yslot[cur];
            atomicAdd(&T.tin[y], tot);
            if (bad) atomicOr(&T.tinb[y], 1u);
            ndone++;
            const int32_t px = T.xpar[cur];
            if (px < 0) break;
            atomicAdd(&T.tot[px], tot);
            if (bad) atomicOr(&T.totb[px], 1u);
            __threadfence();
            if (atomicSub(&T.xdeg[px], 1) != 1) break;
            __threadfence();
            cur = px;
        }
    }
    ndone = __reduce_add_sync(0xffffffffu, (unsigned)ndone);
    if ((threadIdx.x & 31) == 0 && ndone) atomicAdd(&s.counters[5], ndone);
}

// Output: converged counts, or the shipped sweep's pulled sums.
__global__ void sca_output_kernel(const ScaParams p, ScaScratch s) {
    const int64_t n = p.rows * p.cols;
    const int64_t last = (p.rows - 2) * p.cols + (p.cols - 2);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        const bool work = in_work(p, r, c);
        const int8_t me = work ? decode8(p, r, c) : kNodata;
        const bool is_last = i == last && p.rows >= 3 && p.cols >= 3;
        double v = p.out.nodata;
        if (me != kNodata || is_last) {
            unsigned long long sum = 0;
            if (me != kNodata && !p.shipped) {
                sum = s.conv[i];
            } else {
                // children: neighbours whose code names this cell (and, for a
                // valid cell, that it does not name back)
                for (int a = -1; a <= 1; a++)
                    for (int b = -1; b <= 1; b++) {
                        if (!(a || b)) continue;
                        const int k = (a + 1) * 3 + (b + 1);
                        if (!in_work(p, r + a, c + b) || (me != kNodata && me == k)) continue;
                        if (decode8(p, r + a, c + b) != 8 - k) continue;
                        const int64_t q = i + a * p.cols + b;
                        const unsigned long long cq = s.conv[q];
                        const bool pulled = cq == 1 || (q < i && s.ship[q] == 0);
                        if (!p.shipped || pulled) sum += cq;
                    }
                if (me != kNodata) sum += 1;
            }
            v = me != kNodata ? (double)sum : p.out.nodata + (double)sum;
        }
        put_value(p.out, r, c, v);
    }
}

}  // namespace

size_t sca_tiles_bytes(int64_t rows, int64_t cols) {
    const int64_t nodes = ((rows + kT - 1) / kT) * ((cols + kT - 1) / kT) * kScaSlots;
    return (size_t)nodes * (4 * 4 + 2 * 8 + 2 * 4) + 256;
}

ScaTiles sca_tiles_layout(void* base, int64_t rows, int64_t cols) {
    ScaTiles T{};
    T.tiles_y = (rows + kT - 1) / kT;
    T.tiles_x = (cols + kT - 1) / kT;
    const int64_t nodes = T.tiles_x * T.tiles_y * kScaSlots;
    char* b = (char*)(((uintptr_t)base + 15) & ~(uintptr_t)15);
    T.tot = (unsigned long long*)b;
    b += nodes * 8;
    T.tin = (unsigned long long*)b;
    b += nodes * 8;
    T.exit_of = (int32_t*)b;
    b += nodes * 4;
    T.yslot = (int32_t*)b;
    b += nodes * 4;
    T.xpar = (int32_t*)b;
    b += nodes * 4;
    T.xdeg = (int32_t*)b;
    b += nodes * 4;
    T.totb = (uint32_t*)b;
    b += nodes * 4;
    T.tinb = (uint32_t*)b;
    return T;
}

cudaError_t sca_run_tiled(const ScaParams& p, const ScaScratch& s, const ScaTiles& T, cudaStream_t st) {
    const int64_t n = p.rows * p.cols;
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(s.counters, 0, 8 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const size_t smem0 = sizeof(TileSmem<false>), smem1 = sizeof(TileSmem<true>);
    if ((e = cudaFuncSetAttribute(sca_tile_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0)) !=
        cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(sca_tile_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1)) !=
        cudaSuccess)
        return e;
    int dev = 0, sms = 0, per0 = 0, per1 = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, sca_tile_kernel<false>, kTourThreads, smem0)) !=
        cudaSuccess)
        return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, sca_tile_kernel<true>, kTourThreads, smem1)) !=
        cudaSuccess)
        return e;
    const int64_t ntiles = T.tiles_x * T.tiles_y;
    int64_t grid0 = (int64_t)sms * (per0 > 0 ? per0 : 1), grid1 = (int64_t)sms * (per1 > 0 ? per1 : 1);
    if (grid0 > ntiles) grid0 = ntiles;
    if (grid1 > ntiles) grid1 = ntiles;
    sca_tile_kernel<false><<<(unsigned)grid0, kTourThreads, smem0, st>>>(p, s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int64_t nodes = ntiles * kScaSlots;
    int64_t nb = (nodes + 255) / 256;
    if (nb > 8192) nb = 8192;
    sca_exit_links_kernel<<<(unsigned)nb, 256, 0, st>>>(s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_exit_leaves_kernel<<<(unsigned)nb, 256, 0, st>>>(T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_exit_walk_kernel<<<(unsigned)nb, 256, 0, st>>>(s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_tile_kernel<true><<<(unsigned)grid1, kTourThreads, smem1, st>>>(p, s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    sca_output_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, s);
    return cudaGetLastError();
}

}  // namespace pargo
