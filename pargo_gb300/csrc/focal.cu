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

constexpr int kTH = 32;              // tile rows
constexpr int kTW = 128;             // tile cols
constexpr int kBoxW = kTW + 8;       // 4 halo columns each side keeps x 16-byte aligned
constexpr int kBoxH = kTH + 2;
constexpr int kStageBytes = kBoxW * kBoxH * 4;            // 18496
constexpr int kStageStride = (kStageBytes + 1023) / 1024 * 1024;
constexpr int kThreads = 256;
constexpr long long kWaitBudget = 4000000000LL;          // ~2 s of SM clocks

// Nodata tests: float input carries exact float bands for |v - nodata| < Eps.
struct CellFlags {
    bool nd_slope, nd_d8;
};

// Compute slope / code of one window.  `nd_any` is true when some window value
// is inside the wide (1e-6) band, which contains the 1e-7 band.
template <typename T>
__device__ __forceinline__ void eval_cell(const T* z, bool nd_slope, bool nd_d8, const FocalParams& p, float& slope,
                                          int& code, int& fell_back) {
    if (p.do_slope) slope = nd_slope ? 0.0f : slope_from_window(z, p.sk);
    if (p.do_d8) {
        if (nd_d8) {
            code = kD8Unsure - 1;  // marker: nodata
        } else {
            float c[9];
#pragma unroll
            for (int i = 0; i < 9; i++) c[i] = (i == 4) ? 0.0f : zdiff(z, 4, i);
            int k = d8_certified(c, p.dir_type);
            if (k == kD8Unsure) {
                double d[9];
#pragma unroll
                for (int i = 0; i < 9; i++) d[i] = (double)z[i];
                k = d8_exact(d, p.dir_type);
                fell_back++;
            }
            code = k;
        }
    }
}

__device__ __forceinline__ void count_fallbacks(int fell_back, unsigned long long* counter) {
    const unsigned total = __reduce_add_sync(0xffffffffu, (unsigned)fell_back);
    if (counter && total && (threadIdx.x & 31) == 0) atomicAdd(counter, (unsigned long long)total);
}

// One 32 x 128 tile from its TMA stage `s` (34 x 136 floats, origin at
// (y0 - 1, x0 - 4)).  Thread (warp w, lane l) owns rows 4w..4w+3 and columns
// 4l..4l+3 of the tile.
template <int FAST_OUT>
__device__ __forceinline__ void compute_tile(const float* s, int64_t y0, int64_t x0, const FocalParams& p,
                                             int& fell_back) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // 6 x 6 window of this thread's 4 x 4 block: tile rows 4w-1..4w+4
    // (stage rows 4w..4w+5), tile cols 4l-1..4l+4 (stage cols 4l+3..4l+8).
    float v[6][6];
#pragma unroll
    for (int r = 0; r < 6; r++) {
        const float* row = s + (4 * warp + r) * kBoxW;
        float4 q = *reinterpret_cast<const float4*>(row + 4 * lane + 4);
        float left = __shfl_up_sync(0xffffffffu, q.w, 1);
        float right = __shfl_down_sync(0xffffffffu, q.x, 1);
        if (lane == 0) left = row[3];
        if (lane == 31) right = row[4 * 31 + 8];
        v[r][0] = left; v[r][1] = q.x; v[r][2] = q.y; v[r][3] = q.z; v[r][4] = q.w; v[r][5] = right;
    }
    // Wide-band (Eps 1e-6) nodata flags of the 36 values, as row bitmasks.
    unsigned ndw[6];
#pragma unroll
    for (int r = 0; r < 6; r++) {
        unsigned m = 0;
#pragma unroll
        for (int c = 0; c < 6; c++) m |= (p.nd6f.has(v[r][c]) ? 1u : 0u) << c;
        ndw[r] = m;
    }

#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int64_t gy = y0 + 4 * warp + i;
        float sl[4];
        int cd[4];
        bool snd[4], dnd[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int64_t gx = x0 + 4 * lane + j;
            float z[9];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) z[a * 3 + b] = v[i + a][j + b];
            const unsigned win = ((ndw[i] >> j) | (ndw[i + 1] >> j) | (ndw[i + 2] >> j)) & 7u;
            bool nd_d8 = win != 0, nd_slope = false;
            if (nd_d8) {
#pragma unroll
                for (int q = 0; q < 9; q++) nd_slope |= p.nd7f.has(z[q]);
            }
            const bool ring = gy <= 0 || gx <= 0 || gy >= p.rows - 1 || gx >= p.cols - 1;
            float slope = 0.0f;
            int code = 0;
            if (!ring) eval_cell(z, nd_slope, nd_d8, p, slope, code, fell_back);
            snd[j] = ring || nd_slope;
            dnd[j] = ring || nd_d8;
            sl[j] = snd[j] ? (float)p.slope.nodata : slope;
            cd[j] = dnd[j] ? (int)(int8_t)p.d8.nodata : code;
        }
        if (gy >= p.rows) continue;
        const int64_t gx0 = x0 + 4 * lane;
        if (FAST_OUT && gx0 + 3 < p.cols) {
            if (p.do_slope) {
                float4* o = reinterpret_cast<float4*>(p.slope.base + gy * p.slope.pitch) + (gx0 >> 2);
                *o = make_float4(sl[0], sl[1], sl[2], sl[3]);
            }
            if (p.do_d8) {
                uint32_t w = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) w |= (uint32_t)(uint8_t)cd[j] << (8 * j);
                reinterpret_cast<uint32_t*>(p.d8.base + gy * p.d8.pitch)[gx0 >> 2] = w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int64_t gx = gx0 + j;
                if (gx >= p.cols) break;
                if (p.do_slope) put_value(p.slope, gy, gx, snd[j] ? p.slope.nodata : (double)sl[j]);
                if (p.do_d8) put_value(p.d8, gy, gx, dnd[j] ? p.d8.nodata : (double)cd[j]);
            }
        }
    }
}

template <int FAST_OUT>
__global__ void __launch_bounds__(kThreads) focal_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                             const FocalParams p, int64_t ntx, int64_t ntiles) {
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
        compute_tile<FAST_OUT>(reinterpret_cast<const float*>(smem + st * kStageStride), (t / ntx) * kTH,
                               (t % ntx) * kTW, p, fell_back);
        __syncthreads();  // every thread is done with stage st before it is refilled
    }
    count_fallbacks(fell_back, p.fallbacks);
}

template <typename T>
__global__ void __launch_bounds__(256) focal_generic_kernel(const InView dem, const FocalParams p) {
    const int64_t n = p.rows * p.cols;
    int fell_back = 0;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const bool live = true;
        const int64_t y = idx / p.cols, x = idx % p.cols;
        const bool ring = y <= 0 || x <= 0 || y >= p.rows - 1 || x >= p.cols - 1;
        float slope = 0.0f;
        int code = 0;
        bool nd_slope = false, nd_d8 = false;
        if (live && !ring) {
            T z[9];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const T* row = reinterpret_cast<const T*>(dem.base + (y - 1 + a) * dem.pitch);
#pragma unroll
                for (int b = 0; b < 3; b++) z[a * 3 + b] = __ldg(row + x - 1 + b);
            }
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
            eval_cell(z, nd_slope, nd_d8, p, slope, code, fell_back);
        }
        if (live) {
            if (p.do_slope) put_value(p.slope, y, x, (ring || nd_slope) ? p.slope.nodata : (double)slope);
            if (p.do_d8) put_value(p.d8, y, x, (ring || nd_d8) ? p.d8.nodata : (double)code);
        }
    }
    count_fallbacks(fell_back, p.fallbacks);
}


// Batched form: one persistent launch over the tiles of many rasters.  Tiles
// are numbered raster by raster (tile_start = prefix sums, the host orders the
// rasters by decreasing estimated cost); CTAs claim tiles one at a time from a
// global counter, so uneven rasters balance dynamically.  Each raster has its
// own TMA descriptor in global memory; the next tile's load is in flight while
// the current one is computed.
template <int FAST_OUT>
__global__ void __launch_bounds__(kThreads) batch_tma_kernel(const CUtensorMap* maps, const FocalParams* params,
                                                             const int64_t* tile_start, const int64_t* ntx_of,
                                                             int count, int64_t total, unsigned long long* claim,
                                                             unsigned long long* fallbacks, int* error_flag) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int64_t slot_tile[2];
    __shared__ int slot_item[2];
    const int tid = threadIdx.x;

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
        compute_tile<FAST_OUT>(reinterpret_cast<const float*>(smem + st * kStageStride), (local / ntx) * kTH,
                               (local % ntx) * kTW, params[item], fell_back);
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
        float slope = 0.0f;
        int code = 0;
        bool nd_slope = false, nd_d8 = false;
        if (!ring) {
            float z[9];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float* row = reinterpret_cast<const float*>(dem.base + (y - 1 + a) * dem.pitch);
#pragma unroll
                for (int b = 0; b < 3; b++) z[a * 3 + b] = __ldg(row + x - 1 + b);
            }
#pragma unroll
            for (int q = 0; q < 9; q++) {
                nd_slope |= p.nd7f.has(z[q]);
                nd_d8 |= p.nd6f.has(z[q]);
            }
            eval_cell(z, nd_slope, nd_d8, p, slope, code, fell_back);
        }
        if (p.do_slope) put_value(p.slope, y, x, (ring || nd_slope) ? p.slope.nodata : (double)slope);
        if (p.do_d8) put_value(p.d8, y, x, (ring || nd_d8) ? p.d8.nodata : (double)code);
    }
    count_fallbacks(fell_back, fallbacks);
}

}  // namespace

size_t focal_tma_smem_bytes() { return 2 * kStageStride; }
int focal_tma_tile_rows() { return kTH; }
int focal_tma_tile_cols() { return kTW; }
int focal_tma_box_cols() { return kBoxW; }
int focal_tma_box_rows() { return kBoxH; }

cudaError_t launch_focal_tma(const CUtensorMap* map, const FocalParams& p, int fast_out, int num_sms,
                             cudaStream_t s) {
    const int64_t ntx = (p.cols + kTW - 1) / kTW, nty = (p.rows + kTH - 1) / kTH;
    const int64_t ntiles = ntx * nty;
    if (ntiles == 0) return cudaSuccess;
    const size_t smem = focal_tma_smem_bytes();
    auto kern = fast_out ? focal_tma_kernel<1> : focal_tma_kernel<0>;
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

cudaError_t launch_batch_tma(const CUtensorMap* maps, const FocalParams* params, const int64_t* tile_start,
                             const int64_t* ntx_of, int count, int64_t total_tiles, int fast_out,
                             unsigned long long* claim, unsigned long long* fallbacks, int* error_flag, int num_sms,
                             cudaStream_t s) {
    if (total_tiles == 0) return cudaSuccess;
    const size_t smem = focal_tma_smem_bytes();
    auto kern = fast_out ? batch_tma_kernel<1> : batch_tma_kernel<0>;
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
