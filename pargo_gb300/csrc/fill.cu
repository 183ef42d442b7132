// fill.cu -- Planchon-Darboux pit removal (epsilon filling) by tiled
// relaxation with worklists.
//
// Reference: PitRemoveOperator::Operator (apps/hydrology/pitremove/
// pitRemoveOperator.cpp:26-72) swept by RasterOperator::Work
// (gpro/rasterOperator.h:169-219) until a sweep changes nothing.  Per valid
// cell c with level W(c) > dem(c), one visit computes
//     W(c) <- dem(c)                      if some neighbour n has a nodata level
//                                         or dem(c) >= W(n) + gap,
//     W(c) <- min(W(c), min_n W(n) + gap) otherwise,
// with W(n) + gap rounded to double exactly as the reference adds it.  The
// update is monotone (levels only fall) so every visiting order -- the
// reference's raster-order Gauss-Seidel, Jacobi, or this chaotic tiled order --
// ends at the same fixpoint, bit for bit.
//
// GPU structure
//  * init: levels = +inf on the nodata ring and on nodata cells (standing for
//    the reference's nodata level), init_level on valid cells, and dem(c) at
//    once on valid cells next to a nodata level (their first visit does that).
//  * rounds: a worklist of 32 x 32 tiles.  A CTA claims a tile, loads its
//    levels plus a one-cell halo into shared memory, relaxes the tile until it
//    is stable against that halo, writes back the cells that changed and puts
//    the neighbour tiles whose halo changed on the next worklist.  Rounds run
//    until the worklist is empty (a device-side count the host reads after a
//    CUDA graph of rounds).
//  * levels are kept as double bit patterns in an order-preserving integer
//    key, so min/compare run on the integer pipes; W + gap is done on the bit
//    pattern with a per-binade step table (the exact double sum while the sum
//    stays in the binade) and with a real double add otherwise.

#include <math.h>

#include <map>
#include <mutex>

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

constexpr int kT = 32;            // tile side
constexpr int kH = kT + 2;        // with halo
constexpr int kThreads = 256;     // 4 cells per thread
constexpr int kLocalCap = 4096;   // relaxation sweeps per visit before the tile re-queues itself
constexpr int64_t kKeyInf = 0x7FF0000000000000LL;  // key of +inf

// Per biased exponent e: fl64(x + gap) - x in ulps of x's binade when that
// is the same for every x of the binade, else -1 (subnormals, inf/nan, a sum
// that can leave the binade, and the binade in which gap is an odd number of
// half-ulps, where the tie rounds by the parity of x): those use the double add.
__device__ int64_t g_step[2048];

__device__ __forceinline__ int64_t dkey(double x) {
    int64_t b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double dval(int64_t k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL)); }

// key of fl64(x + gap) for x = dval(k)
__device__ __forceinline__ int64_t add_gap(int64_t k, double gap) {
    if (k >= 0 && k < kKeyInf) {
        const int e = (int)(k >> 52);
        const int64_t st = g_step[e];
        if (st >= 0) {
            const int64_t y = k + st;
            if ((int)(y >> 52) == e) return y;
        }
    }
    return dkey(__dadd_rn(dval(k), gap));
}

// DEM value (float32 or float64 input) and its nodata test (Eps 1e-6).
__device__ __forceinline__ double dem_at(const FillParams& p, int64_t r, int64_t c) {
    const char* row = reinterpret_cast<const char*>(p.dem) + r * p.dem_pitch;
    return p.dem_f64 ? reinterpret_cast<const double*>(row)[c] : (double)reinterpret_cast<const float*>(row)[c];
}
__device__ __forceinline__ bool dem_nodata(const FillParams& p, double z) {
    return p.dem_f64 ? p.nd6d.has(z) : p.nd6f.has((float)z);
}

__global__ void fill_init_kernel(const FillParams p, FillScratch s) {
    const int64_t n = p.rows * p.cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        double w = INFINITY;
        const bool inner = r > 0 && c > 0 && r < p.rows - 1 && c < p.cols - 1;
        if (inner) {
            const double z = dem_at(p, r, c);
            if (!dem_nodata(p, z)) {
                w = p.init_level;
                if (p.init_level > z) {
                    bool outlet = false;
                    for (int a = -1; a <= 1; a++)
                        for (int b = -1; b <= 1; b++) {
                            const int64_t rr = r + a, cc = c + b;
                            const bool ring = rr <= 0 || cc <= 0 || rr >= p.rows - 1 || cc >= p.cols - 1;
                            if (ring || dem_nodata(p, dem_at(p, rr, cc))) outlet = true;
                        }
                    if (outlet) w = z;
                }
            }
        }
        p.w[r * p.w_stride + c] = w;
    }
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
        s.list_a[t] = (int32_t)t;
        s.queued[t] = 1;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s.counts[0] = (int32_t)ntiles;
        s.counts[1] = 0;
        s.counts[2] = 0;
        s.counts[3] = 0;
    }
}

__device__ __forceinline__ void enqueue(const FillScratch& s, int32_t* next, int32_t* next_count, int64_t ty, int64_t tx,
                                        const FillParams& p) {
    if (ty < 0 || tx < 0 || ty >= p.tiles_y || tx >= p.tiles_x) return;
    const int32_t t = (int32_t)(ty * p.tiles_x + tx);
    if (atomicExch(&s.queued[t], 1) == 0) next[atomicAdd(next_count, 1)] = t;
}

__global__ void __launch_bounds__(kThreads) fill_round_kernel(const FillParams p, FillScratch s, int parity) {
    __shared__ int64_t lv[kH][kH];
    __shared__ int32_t claim;
    __shared__ int edges;  // bit 0 top, 1 bottom, 2 left, 3 right, 4 tl, 5 tr, 6 bl, 7 br
    __shared__ bool last_block;
    int32_t* cur = parity ? s.list_b : s.list_a;
    int32_t* next = parity ? s.list_a : s.list_b;
    int32_t* cur_count = &s.counts[parity];
    int32_t* next_count = &s.counts[parity ^ 1];
    const int32_t ncur = *((volatile int32_t*)cur_count);
    const int tid = threadIdx.x;
    if (blockIdx.x == 0 && tid == 0 && ncur > 0) atomicAdd(s.active, 1ULL);
    const int lr = tid >> 3;            // local row 0..31
    const int lc0 = (tid & 7) * 4;      // local cols lc0..lc0+3

    for (;;) {
        if (tid == 0) {
            int32_t k = atomicAdd(&s.counts[2], 1);
            claim = k < ncur ? cur[k] : -1;
            edges = 0;
            if (claim >= 0) {
                atomicExch(&s.queued[claim], 0);
                __threadfence();
            }
        }
        __syncthreads();
        const int32_t t = claim;
        if (t < 0) break;
        const int64_t ty = t / p.tiles_x, tx = t % p.tiles_x;
        const int64_t y0 = ty * kT - 1, x0 = tx * kT - 1;  // global coords of lv[0][0]
        for (int i = tid; i < kH * kH; i += kThreads) {
            const int a = i / kH, b = i % kH;
            const int64_t r = y0 + a, c = x0 + b;
            int64_t k = kKeyInf;
            if (r >= 0 && c >= 0 && r < p.rows && c < p.cols) k = dkey(((volatile double*)p.w)[r * p.w_stride + c]);
            lv[a][b] = k;
        }
        __syncthreads();
        // This thread's cells: row lr, cols lc0..lc0+3 of the tile interior.
        int64_t zk[4], orig[4];
        bool act[4];
        const int64_t gr = y0 + 1 + lr;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int64_t gc = x0 + 1 + lc0 + j;
            orig[j] = lv[lr + 1][lc0 + 1 + j];
            act[j] = false;
            zk[j] = 0;
            if (gr < p.rows - 1 && gc < p.cols - 1 && gr > 0 && gc > 0) {
                zk[j] = dkey(dem_at(p, gr, gc));
                act[j] = orig[j] < kKeyInf && orig[j] > zk[j];
            }
        }
        int it = 0;
        for (;;) {
            int changed = 0;
#pragma unroll
            for (int jj = 0; jj < 4; jj++) {
                const int j = (it & 1) ? 3 - jj : jj;
                if (!act[j]) continue;
                const int a = lr + 1, b = lc0 + 1 + j;
                int64_t m = lv[a - 1][b - 1];
                m = min(m, lv[a - 1][b]);
                m = min(m, lv[a - 1][b + 1]);
                m = min(m, lv[a][b - 1]);
                m = min(m, lv[a][b + 1]);
                m = min(m, lv[a + 1][b - 1]);
                m = min(m, lv[a + 1][b]);
                m = min(m, lv[a + 1][b + 1]);
                const int64_t up = add_gap(m, p.gap);
                const int64_t cur_v = lv[a][b];
                int64_t nv = cur_v;
                if (up <= zk[j]) {
                    nv = zk[j];
                    act[j] = false;
                } else if (up < cur_v) {
                    nv = up;
                }
                if (nv != cur_v) {
                    lv[a][b] = nv;
                    changed = 1;
                }
            }
            it++;
            if (!__syncthreads_or(changed) || it >= kLocalCap) break;
        }
        // Write back and note which borders moved.
        int e = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int a = lr + 1, b = lc0 + 1 + j;
            const int64_t v = lv[a][b];
            if (v != orig[j]) {
                p.w[gr * p.w_stride + (x0 + b)] = dval(v);
                if (lr == 0) e |= 1;
                if (lr == kT - 1) e |= 2;
                if (b == 1) e |= 4;
                if (b == kT) e |= 8;
                if (lr == 0 && b == 1) e |= 16;
                if (lr == 0 && b == kT) e |= 32;
                if (lr == kT - 1 && b == 1) e |= 64;
                if (lr == kT - 1 && b == kT) e |= 128;
            }
        }
        const int any = __syncthreads_or(e != 0);
        if (e) atomicOr(&edges, e);
        __syncthreads();
        if (tid == 0) {
            if (it >= kLocalCap) enqueue(s, next, next_count, ty, tx, p);
            if (any) {
                __threadfence();
                const int ed = edges;
                if (ed & 1) enqueue(s, next, next_count, ty - 1, tx, p);
                if (ed & 2) enqueue(s, next, next_count, ty + 1, tx, p);
                if (ed & 4) enqueue(s, next, next_count, ty, tx - 1, p);
                if (ed & 8) enqueue(s, next, next_count, ty, tx + 1, p);
                if (ed & 16) enqueue(s, next, next_count, ty - 1, tx - 1, p);
                if (ed & 32) enqueue(s, next, next_count, ty - 1, tx + 1, p);
                if (ed & 64) enqueue(s, next, next_count, ty + 1, tx - 1, p);
                if (ed & 128) enqueue(s, next, next_count, ty + 1, tx + 1, p);
                atomicAdd(s.changed, 1ULL);
            }
            atomicAdd(s.visits, 1ULL);
            atomicAdd(s.iters, (unsigned long long)it);
        }
        __syncthreads();
    }
    // The last CTA to finish resets the consumed list and the claim cursor.
    if (tid == 0) {
        __threadfence();
        const int32_t done = atomicAdd(&s.counts[3], 1);
        last_block = done == (int32_t)gridDim.x - 1;
    }
    __syncthreads();
    if (last_block && tid == 0) {
        *cur_count = 0;
        s.counts[2] = 0;
        s.counts[3] = 0;
        __threadfence();
    }
}

__global__ void fill_finish_kernel(const FillParams p, const OutView out, unsigned long long* raised) {
    const int64_t n = p.rows * p.cols;
    unsigned long long cnt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        const double w = p.w[r * p.w_stride + c];
        const bool nd = isinf(w);
        if (!nd && w > dem_at(p, r, c)) cnt++;
        put_value(out, r, c, nd ? out.nodata : w);
    }
    cnt = __reduce_add_sync(0xffffffffu, (unsigned)cnt);
    if (raised && (threadIdx.x & 31) == 0 && cnt) atomicAdd(raised, cnt);
}

}  // namespace

int fill_tile_rows() { return kT; }
int fill_tile_cols() { return kT; }

// Host: per-binade step table for the gap, exact: for the binade starting at
// x = 2^(e-1023), (x + gap) - x is exact (both in the binade) and, divided by
// the binade's ulp, is the integer step that fl64(y + gap) adds to any y of the
// binade whose sum stays in it.
static cudaError_t upload_steps(double gap, cudaStream_t st) {
    // The table lives in each device's memory: remember the gap per device.
    static std::mutex mu;
    static std::map<int, double> uploaded;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    std::lock_guard<std::mutex> lock(mu);
    auto it = uploaded.find(dev);
    if (it != uploaded.end() && it->second == gap) return cudaSuccess;
    int64_t tab[2048];
    for (int e = 0; e < 2048; e++) {
        tab[e] = -1;
        if (e == 0 || e >= 2047 || !(gap >= 0.0)) continue;
        const double x = ldexp(1.0, e - 1023);
        const double ulp = ldexp(1.0, e - 1023 - 52);
        const volatile double s0 = x + gap;  // one IEEE double add, even x
        const volatile double x1 = x + ulp;
        const volatile double s1 = x1 + gap;  // odd x
        const int64_t d0 = (int64_t)((s0 - x) / ulp);
        const int64_t d1 = (int64_t)((s1 - x1) / ulp);
        // Same step for even and odd x: no tie in this binade.  A sum that
        // leaves the binade is caught on the device by the result's exponent.
        if (!(s0 < 2.0 * x) || d0 != d1) continue;
        tab[e] = d0;
    }
    // Pageable source: staged at once, copied in stream order.
    err = cudaMemcpyToSymbolAsync(g_step, tab, sizeof(tab), 0, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) uploaded[dev] = gap;
    return err;
}

cudaError_t fill_init(const FillParams& p, const FillScratch& s, cudaStream_t st) {
    cudaError_t e = upload_steps(p.gap, st);
    if (e != cudaSuccess) return e;
    const int64_t n = p.rows * p.cols;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    fill_init_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, s);
    return cudaGetLastError();
}

cudaError_t fill_round(const FillParams& p, const FillScratch& s, int parity, int num_sms, cudaStream_t st) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill_round_kernel, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    if (grid > ntiles) grid = ntiles;
    fill_round_kernel<<<(unsigned)grid, kThreads, 0, st>>>(p, s, parity);
    return cudaGetLastError();
}

cudaError_t fill_finish(const FillParams& p, const OutView& out, unsigned long long* raised, cudaStream_t st) {
    const int64_t n = p.rows * p.cols;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    fill_finish_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, out, raised);
    return cudaGetLastError();
}

}  // namespace pargo
