// focal.cu -- fused Horn slope + D8 over a 3x3 Moore window.
//
// Replaces the per-cell RasterOperator::Work loop (gpro/rasterOperator.h:169-219)
// running SlopeOperator::Operator (apps/morphology/slope/slopeOperator.cpp:51-139)
// and D8Operator::Operator (apps/hydrology/flowdird8/d8Operator.cpp:28-101).
//
// Hot path (float32 DEM, 16-byte aligned rows): a persistent kernel whose CTAs
// walk 32 x 128-cell tiles; each tile plus its one-cell halo (box 34 x 136,
// x starting 4 cells left so the TMA x coordinate stays 16-byte aligned) is
// loaded by TMA into a double-buffered shared-memory stage while the previous
// tile is computed.  A thread owns a 4 x 4 cell block: it reads its 6 x 6
// window rows as float4 from shared memory, the outer columns by warp shuffle,
// and writes slope as float4 and D8 codes as packed 4-byte words.
// Everything else (other pitches, float64 input, other output types) runs the
// generic one-cell-per-thread kernel below.

#include "common.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace pargo {

namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kTW = 128;        // tile cols: 32 lanes x 4
constexpr int kBoxW = kTW + 8;  // 4 halo columns each side keeps the TMA x 16-byte aligned

// Tile shape of one kernel variant: each warp walks ROWS rows, so a tile is
// 4 * ROWS rows; the TMA box adds one halo row above and below.
template <int ROWS>
struct Shape {
    static constexpr int kTH = kWarps * ROWS;
    static constexpr int kBoxH = kTH + 2;
    static constexpr int kStageBytes = kBoxW * kBoxH * 4;
    static constexpr int kStageStride = (kStageBytes + 1023) / 1024 * 1024;
};
constexpr long long kWaitBudget = 4000000000LL;  // ~2 s of SM clocks

struct CellOut {
    float slope;
    int code;
    int flags;  // bit0: slope nodata, bit1: D8 nodata, bit2: the D8 took the exact FP64 path
};

// The general per-cell path: exact nodata bands, any slope method, certified
// D8 with the FP64 fallback.  Values come by value so nothing is spilled.
template <typename T>
__device__ __noinline__ CellOut cell_general(T z0, T z1, T z2, T z3, T z4, T z5, T z6, T z7, T z8,
                                             const FocalParams* pp, bool ring) {
    const FocalParams& p = *pp;
    CellOut o{0.0f, 0, 0};
    if (ring) {
        o.flags = 3;
        return o;
    }
    const T z[9] = {z0, z1, z2, z3, z4, z5, z6, z7, z8};
    bool nd_slope = false, nd_d8 = false;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        if constexpr (sizeof(T) == 4) {
            nd_slope |= p.nd7f.has((float)z[q]);
            nd_d8 |= p.nd6f.has((float)z[q]);
        } else {
            nd_slope |= p.nd7d.has((double)z[q]);
            nd_d8 |= p.nd6d.has((double)z[q]);
        }
    }
    if (nd_slope) o.flags |= 1;
    if (nd_d8) o.flags |= 2;
    if (p.do_slope && !nd_slope) o.slope = slope_from_window(z, p.sk);
    if (p.do_d8 && !nd_d8) {
        int k = d8_certified(z, p.dir_type);
        if (k == kD8Unsure) {
            double d[9];
#pragma unroll
            for (int i = 0; i < 9; i++) d[i] = (double)z[i];
            k = d8_exact(d, p.dir_type);
            o.flags |= 4;
        }
        o.code = k;
    }
    return o;
}

__device__ __forceinline__ void count_fallbacks(int fell_back, unsigned long long* counter) {
    const unsigned total = __reduce_add_sync(0xffffffffu, (unsigned)fell_back);
    if (counter && total && (threadIdx.x & 31) == 0) atomicAdd(counter, (unsigned long long)total);
}

// Row `ty` (tile-local, -1 .. kTH) of the stage as this lane's 6 values:
// columns 4l-1 .. 4l+4.  Centre four by one float4, the outer two by shuffle.
__device__ __forceinline__ void load_row(const float* s, int ty, int lane, float v[6]) {
    const float* row = s + (ty + 1) * kBoxW;
    const float4 q = *reinterpret_cast<const float4*>(row + 4 * lane + 4);
    float left = __shfl_up_sync(0xffffffffu, q.w, 1);
    float right = __shfl_down_sync(0xffffffffu, q.x, 1);
    if (lane == 0) left = row[3];
    if (lane == 31) right = row[4 * 31 + 8];
    v[0] = left; v[1] = q.x; v[2] = q.y; v[3] = q.z; v[4] = q.w; v[5] = right;
}

// Whether some of the 6 values may lie in the wide (Eps 1e-6) nodata band.
// A band below zero (the usual negative nodata) needs only the row minimum.
__device__ __forceinline__ bool row_maybe_nodata(const float v[6], const Band<float>& b) {
    const float mn = fminf(fminf(fminf(v[0], v[1]), fminf(v[2], v[3])), fminf(v[4], v[5]));
    if (b.hi < 0.0f) return mn <= b.hi;
    const float mx = fmaxf(fmaxf(fmaxf(v[0], v[1]), fmaxf(v[2], v[3])), fmaxf(v[4], v[5]));
    return mn <= b.hi && mx >= b.lo;
}

// FP32 D8 fast path on the eight drops x (window order, x4 unused): returns
// the code when the maximum is single and certain, else kD8Unsure.
//   M vs 1e-6: |x_k - r_k| <= 2^-22 x_k;
//   single maximum: every other x_i <= m - (1e-6 + 2^-19 m) is certainly
//   outside the tie set (x_i >= 0: |x_i| <= m; x_i < 0: the gap exceeds m).
__device__ __forceinline__ int d8_fast(float x0, float x1, float x2, float x3, float x5, float x6, float x7, float x8,
                                       int dir_type) {
    const float m = fmaxf(fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)), fmaxf(fmaxf(x5, x6), fmaxf(x7, x8)));
    if (m <= 0.0f) return -1;
    const float em = m * k2m22;
    if (m + em < kTLo) return -1;
    if (!(m - em > kTHi)) return kD8Unsure;
    const float t = m - (kTHi + m * 1.9073486328125e-06f);  // 2^-19
    const unsigned mask = (x0 > t ? 1u : 0u) | (x1 > t ? 2u : 0u) | (x2 > t ? 4u : 0u) | (x3 > t ? 8u : 0u) |
                          (x5 > t ? 32u : 0u) | (x6 > t ? 64u : 0u) | (x7 > t ? 128u : 0u) | (x8 > t ? 256u : 0u);
    if (mask & (mask - 1)) return kD8Unsure;
    const int k = __ffs(mask) - 1;
    return dir_type == 8 ? k : d8_bit_code(k);
}

// One (4 ROWS) x 128 tile from its TMA stage `s` ((4 ROWS + 2) x 136 floats,
// origin at (y0 - 1, x0 - 4)).  Warp w owns tile rows ROWS w .. ROWS w + ROWS - 1,
// lane l columns 4l..4l+3.
// A rolling three-row register window walks down the rows; each neighbour
// difference is formed once and serves both cells it joins:
//   row differences   h[a]  = z(r, a+1) - z(r, a)           (W of a+1, -E of a)
//   column differences vS[j] = z(r, j) - z(r+1, j)           (S of row r, -N of row r+1)
//   diagonals e1[a] = (z(r, a) - z(r+1, a+1)) / sqrt 2        (SE of a-1, -NW of row r+1)
//             e2[a] = (z(r, a+1) - z(r+1, a)) / sqrt 2        (SW of a, -NE of row r+1)
// (negating an IEEE difference is exact, so each drop is bit-identical to
// z4 - z_i computed per cell).  Horn numerators come from two-apart
// differences sh (rows) and sv (columns).  Windows that may touch nodata, the
// ring, other slope methods and uncertain D8 decisions take cell_general.
template <int FAST_OUT, bool FD, int ROWS, int UNROLL>
__device__ __forceinline__ void compute_tile(const float* s, int64_t y0, int64_t x0, const FocalParams& p,
                                             int& fell_back) {
    constexpr int kRowsPerWarp = ROWS;
    const float kinv = 0.70710677f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = warp * kRowsPerWarp;
    const int64_t gx0 = x0 + 4 * lane, gy0 = y0 + r0;
    const bool interior = gy0 >= 1 && gy0 + kRowsPerWarp <= p.rows - 1 && gx0 >= 1 && gx0 + 4 <= p.cols - 1;
    float va[6], vb[6], vc[6];
    load_row(s, r0 - 1, lane, va);
    load_row(s, r0, lane, vb);
    bool nda = row_maybe_nodata(va, p.nd6f), ndb = row_maybe_nodata(vb, p.nd6f);
    float shA[4], shB[4], vN[4], nw[4], ne[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        shA[j] = va[j + 2] - va[j];
        shB[j] = vb[j + 2] - vb[j];
        vN[j] = vb[j + 1] - va[j + 1];
        nw[j] = (vb[j + 1] - va[j]) * kinv;
        ne[j] = (vb[j + 1] - va[j + 2]) * kinv;
    }
#pragma unroll UNROLL
    for (int i = 0; i < kRowsPerWarp; i++) {
        load_row(s, r0 + i + 1, lane, vc);
        const bool ndc = row_maybe_nodata(vc, p.nd6f);
        float shC[4], h[5], vS[4], e1[5], e2[5], sv[6];
#pragma unroll
        for (int a = 0; a < 5; a++) {
            h[a] = vb[a + 1] - vb[a];
            e1[a] = (vb[a] - vc[a + 1]) * kinv;
            e2[a] = (vb[a + 1] - vc[a]) * kinv;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            shC[j] = vc[j + 2] - vc[j];
            vS[j] = vb[j + 1] - vc[j + 1];
        }
#pragma unroll
        for (int a = 0; a < 6; a++) sv[a] = va[a] - vc[a];
        const bool slow_row = !FD || nda || ndb || ndc || !interior;
        const int64_t gy = gy0 + i;
        float sl[4];
        int cd[4];
        int fl[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int code = kD8Unsure;
            float slope = 0.0f;
            fl[j] = 0;
            if (!slow_row) {
                if (p.do_slope) {
                    const float nx = __fmaf_rn(2.0f, shB[j], __fadd_rn(shA[j], shC[j]));
                    const float ny = __fmaf_rn(2.0f, sv[j + 1], __fadd_rn(sv[j], sv[j + 2]));
                    slope = horn_slope(nx, ny, p.sk.k_fd);
                    if (p.sk.degrees) slope = atanf(slope) * 57.29577951308232f;
                }
                code = p.do_d8 ? d8_fast(nw[j], vN[j], ne[j], h[j], -h[j + 1], e2[j], vS[j], e1[j + 1], p.dir_type)
                               : 0;
            }
            if (code == kD8Unsure) {
                const int64_t gx = gx0 + j;
                const bool ring = gy <= 0 || gx <= 0 || gy >= p.rows - 1 || gx >= p.cols - 1;
                const CellOut o = cell_general<float>(va[j], va[j + 1], va[j + 2], vb[j], vb[j + 1], vb[j + 2],
                                                      vc[j], vc[j + 1], vc[j + 2], &p, ring);
                slope = o.slope;
                code = o.code;
                fl[j] = o.flags;
                fell_back += (o.flags >> 2) & 1;
            }
            sl[j] = (fl[j] & 1) ? (float)p.slope.nodata : slope;
            cd[j] = (fl[j] & 2) ? (int)(int8_t)p.d8.nodata : code;
        }
        if (gy < p.rows) {
            if (FAST_OUT && gx0 + 3 < p.cols) {
                if (p.do_slope) {
                    float4* o = reinterpret_cast<float4*>(p.slope.base + gy * p.slope.pitch) + (gx0 >> 2);
                    *o = make_float4(sl[0], sl[1], sl[2], sl[3]);
                }
                if (p.do_d8) {
                    const uint32_t w = (uint32_t)(uint8_t)cd[0] | ((uint32_t)(uint8_t)cd[1] << 8) |
                                       ((uint32_t)(uint8_t)cd[2] << 16) | ((uint32_t)(uint8_t)cd[3] << 24);
                    reinterpret_cast<uint32_t*>(p.d8.base + gy * p.d8.pitch)[gx0 >> 2] = w;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int64_t gx = gx0 + j;
                    if (gx >= p.cols) break;
                    if (p.do_slope) put_value(p.slope, gy, gx, (fl[j] & 1) ? p.slope.nodata : (double)sl[j]);
                    if (p.do_d8) put_value(p.d8, gy, gx, (fl[j] & 2) ? p.d8.nodata : (double)cd[j]);
                }
            }
        }
        // roll the window down one row
#pragma unroll
        for (int a = 0; a < 6; a++) {
            va[a] = vb[a];
            vb[a] = vc[a];
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            shA[j] = shB[j];
            shB[j] = shC[j];
            vN[j] = -vS[j];
            nw[j] = -e1[j];
            ne[j] = -e2[j + 1];
        }
        nda = ndb;
        ndb = ndc;
    }
}

template <int FAST_OUT, bool FD, int ROWS, int UNROLL, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) focal_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                                const __grid_constant__ FocalParams p, int64_t ntx,
                                                                int64_t ntiles) {
    using S = Shape<ROWS>;
    constexpr int kTH = S::kTH, kStageBytes = S::kStageBytes, kStageStride = S::kStageStride;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar[2];
    const int tid = threadIdx.x;

    if (tid == 0) {
        tma_prefetch_desc(&map);
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();

    int64_t t = blockIdx.x;
    if (tid == 0 && t < ntiles) {
        mbar_arrive_expect_tx(&bar[0], kStageBytes);
        tma_load_2d(smem, &map, (int32_t)((t % ntx) * kTW - 4), (int32_t)((t / ntx) * kTH - 1), &bar[0]);
    }
    int fell_back = 0;
    for (int k = 0; t < ntiles; t += gridDim.x, k++) {
        const int st = k & 1;
        const int64_t tn = t + gridDim.x;
        if (tid == 0 && tn < ntiles) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[st ^ 1], kStageBytes);
            tma_load_2d(smem + (st ^ 1) * kStageStride, &map, (int32_t)((tn % ntx) * kTW - 4),
                        (int32_t)((tn / ntx) * kTH - 1), &bar[st ^ 1]);
        }
        if (!mbar_wait_bounded(&bar[st], (uint32_t)((k >> 1) & 1), kWaitBudget)) {
            if (p.error_flag) atomicExch(p.error_flag, 1);
            return;
        }
        compute_tile<FAST_OUT, FD, ROWS, UNROLL>(reinterpret_cast<const float*>(smem + st * kStageStride),
                                                 (t / ntx) * kTH, (t % ntx) * kTW, p, fell_back);
        __syncthreads();  // every thread is done with stage st before it is refilled
    }
    count_fallbacks(fell_back, p.fallbacks);
}

template <typename T>
__global__ void __launch_bounds__(256) focal_generic_kernel(const InView dem, const __grid_constant__ FocalParams p) {
    const int64_t n = p.rows * p.cols;
    int fell_back = 0;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t y = idx / p.cols, x = idx % p.cols;
        const bool ring = y <= 0 || x <= 0 || y >= p.rows - 1 || x >= p.cols - 1;
        T z[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (!ring) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const T* row = reinterpret_cast<const T*>(dem.base + (y - 1 + a) * dem.pitch);
#pragma unroll
                for (int b = 0; b < 3; b++) z[a * 3 + b] = __ldg(row + x - 1 + b);
            }
        }
        const CellOut o = cell_general<T>(z[0], z[1], z[2], z[3], z[4], z[5], z[6], z[7], z[8], &p, ring);
        fell_back += (o.flags >> 2) & 1;
        if (p.do_slope) put_value(p.slope, y, x, (o.flags & 1) ? p.slope.nodata : (double)o.slope);
        if (p.do_d8) put_value(p.d8, y, x, (o.flags & 2) ? p.d8.nodata : (double)o.code);
    }
    count_fallbacks(fell_back, p.fallbacks);
}

// Batched form: one persistent launch over the tiles of many rasters.  Tiles
// are numbered raster by raster (tile_start = prefix sums, the host orders the
// rasters by decreasing estimated cost); CTAs claim tiles one at a time from a
// global counter, so uneven rasters balance dynamically.  Each raster has its
// own TMA descriptor in global memory; the next tile's load is in flight while
// the current one is computed.
constexpr int kBatchRows = 8;
template <int FAST_OUT, bool FD>
__global__ void __launch_bounds__(kThreads, 5) batch_tma_kernel(const CUtensorMap* maps, const FocalParams* params,
                                                             const int64_t* tile_start, const int64_t* ntx_of,
                                                             int count, int64_t total, unsigned long long* claim,
                                                             unsigned long long* fallbacks, int* error_flag) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int64_t slot_tile[2];
    __shared__ int slot_item[2];
    const int tid = threadIdx.x;
    using S = Shape<kBatchRows>;
    constexpr int kTH = S::kTH, kStageBytes = S::kStageBytes, kStageStride = S::kStageStride;

    auto claim_and_issue = [&](int st) {
        const int64_t t = (int64_t)atomicAdd(claim, 1ULL);
        slot_tile[st] = t;
        if (t >= total) return;
        int lo = 0, hi = count - 1;  // last item whose first tile <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tile_start[mid] <= t) lo = mid; else hi = mid - 1;
        }
        slot_item[st] = lo;
        const int64_t local = t - tile_start[lo], ntx = ntx_of[lo];
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[st], kStageBytes);
        tma_load_2d(smem + st * kStageStride, &maps[lo], (int32_t)((local % ntx) * kTW - 4),
                    (int32_t)((local / ntx) * kTH - 1), &bar[st]);
    };

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
        claim_and_issue(0);
    }
    __syncthreads();
    int fell_back = 0;
    for (int k = 0;; k++) {
        const int st = k & 1;
        const int64_t t = slot_tile[st];
        if (t >= total) break;
        const int item = slot_item[st];
        if (tid == 0) claim_and_issue(st ^ 1);
        if (!mbar_wait_bounded(&bar[st], (uint32_t)((k >> 1) & 1), kWaitBudget)) {
            if (error_flag) atomicExch(error_flag, 1);
            return;
        }
        const int64_t local = t - tile_start[item], ntx = ntx_of[item];
        compute_tile<FAST_OUT, FD, kBatchRows, 1>(reinterpret_cast<const float*>(smem + st * kStageStride),
                                                  (local / ntx) * kTH, (local % ntx) * kTW, params[item], fell_back);
        __syncthreads();
    }
    count_fallbacks(fell_back, fallbacks);
}

// Batched generic form (rasters TMA cannot address): one cell per thread over
// the concatenated cell index space.
__global__ void __launch_bounds__(256) batch_generic_kernel(const FocalParams* params, const InView* dems,
                                                            const int64_t* cell_start, int count, int64_t total,
                                                            unsigned long long* fallbacks) {
    int fell_back = 0;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (cell_start[mid] <= g) lo = mid; else hi = mid - 1;
        }
        const FocalParams& p = params[lo];
        const InView dem = dems[lo];
        const int64_t idx = g - cell_start[lo];
        const int64_t y = idx / p.cols, x = idx % p.cols;
        const bool ring = y <= 0 || x <= 0 || y >= p.rows - 1 || x >= p.cols - 1;
        float z[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (!ring) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float* row = reinterpret_cast<const float*>(dem.base + (y - 1 + a) * dem.pitch);
#pragma unroll
                for (int b = 0; b < 3; b++) z[a * 3 + b] = __ldg(row + x - 1 + b);
            }
        }
        const CellOut o = cell_general<float>(z[0], z[1], z[2], z[3], z[4], z[5], z[6], z[7], z[8], &p, ring);
        fell_back += (o.flags >> 2) & 1;
        if (p.do_slope) put_value(p.slope, y, x, (o.flags & 1) ? p.slope.nodata : (double)o.slope);
        if (p.do_d8) put_value(p.d8, y, x, (o.flags & 2) ? p.d8.nodata : (double)o.code);
    }
    count_fallbacks(fell_back, fallbacks);
}

}  // namespace

// Kernel variants the autotuner chooses among (tile rows = 4 x ROWS).
struct Variant {
    int rows, unroll, minb;
};
static const Variant kVariants[] = {{8, 1, 5}, {9, 3, 4}, {12, 3, 4}, {6, 3, 5}, {6, 1, 6}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

int focal_num_variants() { return kNumVariants; }
int focal_variant_rows(int v) { return kWarps * kVariants[(v >= 0 && v < kNumVariants) ? v : 0].rows; }
size_t focal_tma_smem_bytes() { return 2 * Shape<kBatchRows>::kStageStride; }
int focal_tma_tile_rows() { return Shape<kBatchRows>::kTH; }
int focal_tma_tile_cols() { return kTW; }
int focal_tma_box_cols() { return kBoxW; }
int focal_tma_box_rows() { return Shape<kBatchRows>::kBoxH; }

template <int FAST_OUT, bool FD, int ROWS, int UNROLL, int MINB>
static cudaError_t launch_variant(const CUtensorMap* map, const FocalParams& p, int num_sms, cudaStream_t s) {
    using S = Shape<ROWS>;
    const int64_t ntx = (p.cols + kTW - 1) / kTW, nty = (p.rows + S::kTH - 1) / S::kTH;
    const int64_t ntiles = ntx * nty;
    if (ntiles == 0) return cudaSuccess;
    const size_t smem = 2 * S::kStageStride;
    auto kern = focal_tma_kernel<FAST_OUT, FD, ROWS, UNROLL, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > ntiles) grid = ntiles;
    kern<<<(unsigned)grid, kThreads, smem, s>>>(*map, p, ntx, ntiles);
    return cudaGetLastError();
}

// The tensor map's box must be (kBoxW, focal_variant_rows(variant) + 2).
cudaError_t launch_focal_tma(const CUtensorMap* map, const FocalParams& p, int fast_out, int variant, int num_sms,
                             cudaStream_t s) {
    const bool fd = p.sk.method == PARGO_SLOPE_FD || !p.do_slope;
    if (fast_out && fd) {
        switch (variant) {
            case 1: return launch_variant<1, true, 9, 3, 4>(map, p, num_sms, s);
            case 2: return launch_variant<1, true, 12, 3, 4>(map, p, num_sms, s);
            case 3: return launch_variant<1, true, 6, 3, 5>(map, p, num_sms, s);
            case 4: return launch_variant<1, true, 6, 1, 6>(map, p, num_sms, s);
            default: return launch_variant<1, true, 8, 1, 5>(map, p, num_sms, s);
        }
    }
    if (fast_out) return launch_variant<1, false, 8, 1, 5>(map, p, num_sms, s);
    return fd ? launch_variant<0, true, 8, 1, 5>(map, p, num_sms, s)
              : launch_variant<0, false, 8, 1, 5>(map, p, num_sms, s);
}

cudaError_t launch_batch_tma(const CUtensorMap* maps, const FocalParams* params, const int64_t* tile_start,
                             const int64_t* ntx_of, int count, int64_t total_tiles, int fast_out, int fd,
                             unsigned long long* claim, unsigned long long* fallbacks, int* error_flag, int num_sms,
                             cudaStream_t s) {
    if (total_tiles == 0) return cudaSuccess;
    const size_t smem = focal_tma_smem_bytes();
    auto kern = fast_out ? (fd ? batch_tma_kernel<1, true> : batch_tma_kernel<1, false>)
                         : (fd ? batch_tma_kernel<0, true> : batch_tma_kernel<0, false>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > total_tiles) grid = total_tiles;
    e = cudaMemsetAsync(claim, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    kern<<<(unsigned)grid, kThreads, smem, s>>>(maps, params, tile_start, ntx_of, count, total_tiles, claim,
                                                fallbacks, error_flag);
    return cudaGetLastError();
}

cudaError_t launch_batch_generic(const FocalParams* params, const InView* dems, const int64_t* cell_start, int count,
                                 int64_t total_cells, unsigned long long* fallbacks, int num_sms, cudaStream_t s) {
    if (total_cells == 0) return cudaSuccess;
    int64_t blocks = (total_cells + 255) / 256;
    if (blocks > (int64_t)num_sms * 64) blocks = (int64_t)num_sms * 64;
    batch_generic_kernel<<<(unsigned)blocks, 256, 0, s>>>(params, dems, cell_start, count, total_cells, fallbacks);
    return cudaGetLastError();
}

cudaError_t launch_focal_generic(const InView& dem, const FocalParams& p, cudaStream_t s) {
    const int64_t n = p.rows * p.cols;
    if (n == 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 65535LL * 16) blocks = 65535LL * 16;
    if (dem.dtype == PARGO_F64)
        focal_generic_kernel<double><<<(unsigned)blocks, 256, 0, s>>>(dem, p);
    else
        focal_generic_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(dem, p);
    return cudaGetLastError();
}

}  // namespace pargo
