// focal64.cu -- Horn slope + D8 over a float64 surface, TMA-tiled.
//
// The surface is the pit-removed levels of the hydrology chain: the reference
// D8 reads the Float64 output of pit removal (pPitRemove.cpp:129 writes it,
// pD8.cpp:113 reads it), so the codes must come from the float64 levels.
// Their differences are of order the gap (5e-4 m), so every neighbour
// difference is formed in FP64 -- once per row, shared by the two cells it
// joins -- and only then rounded to float for the certified D8 decision
// (common.cuh: the same bounds hold, r_i = fl64(d4 - d_i) is what the
// reference computes).  Horn numerators are combined in FP64 too.
//
// Layout: CTAs of 4 warps walk 32 x 64-cell tiles; the box (34 x 68 doubles,
// x starting 2 cells left so x * 8 bytes stays a multiple of 16) is TMA-loaded
// into a double-buffered stage.  A lane owns 2 columns and walks 8 rows with a
// rolling three-row window (values kept as doubles, drops as floats).  The
// kernel can also copy the levels out as the filled-DEM raster (float32 or
// float64, +inf levels written as that raster's nodata), so the chain reads
// the levels once.

#include <string.h>

#include "common.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace pargo {

namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kRows = 8;                 // rows per warp
constexpr int kTH = kWarps * kRows;      // 32
constexpr int kTW = 64;                  // 32 lanes x 2 columns
constexpr int kBoxW = kTW + 4;           // 2 halo columns each side (16 bytes)
constexpr int kBoxH = kTH + 2;
constexpr int kStageBytes = kBoxW * kBoxH * 8;
constexpr int kStageStride = (kStageBytes + 1023) / 1024 * 1024;
constexpr long long kWaitBudget = 4000000000LL;

struct CellOut {
    float slope;
    int code;
    int flags;  // bit0 slope nodata, bit1 D8 nodata, bit2 exact FP64 D8 path
};

__device__ __noinline__ CellOut cell_general64(double z0, double z1, double z2, double z3, double z4, double z5,
                                               double z6, double z7, double z8, const FocalParams* pp, bool ring) {
    const FocalParams& p = *pp;
    CellOut o{0.0f, 0, 0};
    if (ring) {
        o.flags = 3;
        return o;
    }
    const double z[9] = {z0, z1, z2, z3, z4, z5, z6, z7, z8};
    bool nd_slope = false, nd_d8 = false;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        nd_slope |= p.nd7d.has(z[q]);
        nd_d8 |= p.nd6d.has(z[q]);
    }
    if (nd_slope) o.flags |= 1;
    if (nd_d8) o.flags |= 2;
    if (p.do_slope && !nd_slope) o.slope = slope_from_window(z, p.sk);
    if (p.do_d8 && !nd_d8) {
        int k = d8_certified(z, p.dir_type);
        if (k == kD8Unsure) {
            double d[9];
#pragma unroll
            for (int i = 0; i < 9; i++) d[i] = z[i];
            k = d8_exact(d, p.dir_type);
            o.flags |= 4;
        }
        o.code = k;
    }
    return o;
}

// Conservative "some value may be nodata" test of a row.  Pipeline levels
// mark nodata with +inf: any inf/NaN high word.  Otherwise the high 32 bits of
// the order-preserving key against the band's.
__device__ __forceinline__ bool row_maybe_nodata64(const double v[4], const Focal64Params& p, int klo, int khi) {
    bool m = false;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int hi = __double2hiint(v[a]);
        if (p.nodata_is_inf) {
            m |= (hi & 0x7FFFFFFF) >= 0x7FF00000;
        } else {
            const int k = hi ^ ((hi >> 31) & 0x7FFFFFFF);
            m |= k >= klo && k <= khi;
        }
    }
    return m;
}

__device__ __forceinline__ void load_row64(const double* s, int ty, int lane, double v[4]) {
    const double* row = s + (ty + 1) * kBoxW;
    const double2 q = *reinterpret_cast<const double2*>(row + 2 * lane + 2);
    double left = __shfl_up_sync(0xffffffffu, q.y, 1);
    double right = __shfl_down_sync(0xffffffffu, q.x, 1);
    if (lane == 0) left = row[1];
    if (lane == 31) right = row[2 * 31 + 4];
    v[0] = left; v[1] = q.x; v[2] = q.y; v[3] = right;
}

__device__ __forceinline__ void put_copy(const OutView& o, int64_t r, int64_t c, double w) {
    put_value(o, r, c, isinf(w) ? o.nodata : w);
}

// same decision as focal.cu's d8_fast (see the bounds there)
__device__ __forceinline__ int d8_fast64(float x0, float x1, float x2, float x3, float x5, float x6, float x7,
                                         float x8, int dir_type) {
    const float m = fmaxf(fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)), fmaxf(fmaxf(x5, x6), fmaxf(x7, x8)));
    if (m <= 0.0f) return -1;
    const float em = m * k2m22;
    if (m + em < kTLo) return -1;
    if (!(m - em > kTHi)) return kD8Unsure;
    const float t = m - (kTHi + m * 1.9073486328125e-06f);
    const unsigned mask = (x0 > t ? 1u : 0u) | (x1 > t ? 2u : 0u) | (x2 > t ? 4u : 0u) | (x3 > t ? 8u : 0u) |
                          (x5 > t ? 32u : 0u) | (x6 > t ? 64u : 0u) | (x7 > t ? 128u : 0u) | (x8 > t ? 256u : 0u);
    if (mask & (mask - 1)) return kD8Unsure;
    const int k = __ffs(mask) - 1;
    return dir_type == 8 ? k : d8_bit_code(k);
}

__device__ __forceinline__ void compute_tile64(const double* s, int64_t y0, int64_t x0, const Focal64Params& P,
                                               int klo, int khi, int& fell_back, unsigned long long& raised) {
    const FocalParams& p = P.f;
    const float kinv = 0.70710677f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = warp * kRows;
    const int64_t gx0 = x0 + 2 * lane, gy0 = y0 + r0;
    const bool interior = gy0 >= 1 && gy0 + kRows <= p.rows - 1 && gx0 >= 1 && gx0 + 2 <= p.cols - 1;
    double va[4], vb[4], vc[4];
    load_row64(s, r0 - 1, lane, va);
    load_row64(s, r0, lane, vb);
    bool nda = row_maybe_nodata64(va, P, klo, khi), ndb = row_maybe_nodata64(vb, P, klo, khi);
    double shA[2], shB[2];
    float vN[2], nw[2], ne[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        shA[j] = va[j + 2] - va[j];
        shB[j] = vb[j + 2] - vb[j];
        vN[j] = (float)(vb[j + 1] - va[j + 1]);
        nw[j] = (float)(vb[j + 1] - va[j]) * kinv;
        ne[j] = (float)(vb[j + 1] - va[j + 2]) * kinv;
    }
#pragma unroll 1
    for (int i = 0; i < kRows; i++) {
        load_row64(s, r0 + i + 1, lane, vc);
        const bool ndc = row_maybe_nodata64(vc, P, klo, khi);
        float h[3], e1[3], e2[3], vS[2];
        double shC[2], sv[4];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            h[a] = (float)(vb[a + 1] - vb[a]);
            e1[a] = (float)(vb[a] - vc[a + 1]) * kinv;
            e2[a] = (float)(vb[a + 1] - vc[a]) * kinv;
        }
#pragma unroll
        for (int j = 0; j < 2; j++) {
            shC[j] = vc[j + 2] - vc[j];
            vS[j] = (float)(vb[j + 1] - vc[j + 1]);
        }
#pragma unroll
        for (int a = 0; a < 4; a++) sv[a] = va[a] - vc[a];
        const bool slow_row = p.sk.method != PARGO_SLOPE_FD || nda || ndb || ndc || !interior;
        const int64_t gy = gy0 + i;
        float sl[2];
        int cd[2], fl[2];
#pragma unroll
        for (int j = 0; j < 2; j++) {
            int code = kD8Unsure;
            float slope = 0.0f;
            fl[j] = 0;
            if (!slow_row) {
                if (p.do_slope) {
                    const double nx = (shA[j] + shC[j]) + 2.0 * shB[j];
                    const double ny = (sv[j] + sv[j + 2]) + 2.0 * sv[j + 1];
                    slope = horn_slope((float)nx, (float)ny, p.sk.k_fd);
                    if (p.sk.degrees) slope = atanf(slope) * 57.29577951308232f;
                }
                code = p.do_d8 ? d8_fast64(nw[j], vN[j], ne[j], h[j], -h[j + 1], e2[j], vS[j], e1[j + 1], p.dir_type)
                               : 0;
            }
            if (code == kD8Unsure) {
                const int64_t gx = gx0 + j;
                const bool ring = gy <= 0 || gx <= 0 || gy >= p.rows - 1 || gx >= p.cols - 1;
                const CellOut o = cell_general64(va[j], va[j + 1], va[j + 2], vb[j], vb[j + 1], vb[j + 2], vc[j],
                                                 vc[j + 1], vc[j + 2], &p, ring);
                slope = o.slope;
                code = o.code;
                fl[j] = o.flags;
                fell_back += (o.flags >> 2) & 1;
            }
            sl[j] = slope;
            cd[j] = code;
        }
        if (gy < p.rows) {
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const int64_t gx = gx0 + j;
                if (gx >= p.cols) break;
                if (p.do_slope) put_value(p.slope, gy, gx, (fl[j] & 1) ? p.slope.nodata : (double)sl[j]);
                if (p.do_d8) put_value(p.d8, gy, gx, (fl[j] & 2) ? p.d8.nodata : (double)cd[j]);
                if (P.do_copy) put_copy(P.copy, gy, gx, vb[j + 1]);
                if (P.raised) {
                    const char* row = reinterpret_cast<const char*>(P.dem) + gy * P.dem_pitch;
                    const double z = P.dem_f64 ? reinterpret_cast<const double*>(row)[gx]
                                               : (double)reinterpret_cast<const float*>(row)[gx];
                    raised += (!isinf(vb[j + 1]) && vb[j + 1] > z) ? 1 : 0;
                }
            }
        }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            va[a] = vb[a];
            vb[a] = vc[a];
        }
#pragma unroll
        for (int j = 0; j < 2; j++) {
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

__global__ void __launch_bounds__(kThreads, 4) focal64_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                                  const __grid_constant__ Focal64Params P,
                                                                  int64_t ntx, int64_t ntiles, int klo, int khi) {
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
        tma_load_2d(smem, &map, (int32_t)((t % ntx) * kTW - 2), (int32_t)((t / ntx) * kTH - 1), &bar[0]);
    }
    int fell_back = 0;
    unsigned long long raised = 0;
    for (int k = 0; t < ntiles; t += gridDim.x, k++) {
        const int st = k & 1;
        const int64_t tn = t + gridDim.x;
        if (tid == 0 && tn < ntiles) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[st ^ 1], kStageBytes);
            tma_load_2d(smem + (st ^ 1) * kStageStride, &map, (int32_t)((tn % ntx) * kTW - 2),
                        (int32_t)((tn / ntx) * kTH - 1), &bar[st ^ 1]);
        }
        if (!mbar_wait_bounded(&bar[st], (uint32_t)((k >> 1) & 1), kWaitBudget)) {
            if (P.f.error_flag) atomicExch(P.f.error_flag, 1);
            return;
        }
        compute_tile64(reinterpret_cast<const double*>(smem + st * kStageStride), (t / ntx) * kTH, (t % ntx) * kTW, P,
                       klo, khi, fell_back, raised);
        __syncthreads();
    }
    const unsigned fb = __reduce_add_sync(0xffffffffu, (unsigned)fell_back);
    if (P.f.fallbacks && fb && (tid & 31) == 0) atomicAdd(P.f.fallbacks, (unsigned long long)fb);
    if (P.raised) {
        const unsigned r = __reduce_add_sync(0xffffffffu, (unsigned)raised);
        if (r && (tid & 31) == 0) atomicAdd(P.raised, (unsigned long long)r);
    }
}

// high 32 bits of the order-preserving key of a double (host)
int key_hi(double x) {
    int64_t b;
    memcpy(&b, &x, 8);
    const int hi = (int)(b >> 32);
    return hi ^ ((hi >> 31) & 0x7FFFFFFF);
}

}  // namespace

int focal64_tile_rows() { return kTH; }
int focal64_box_cols() { return kBoxW; }

cudaError_t launch_focal64_tma(const CUtensorMap* map, const Focal64Params& p, int num_sms, cudaStream_t s) {
    const int64_t ntx = (p.f.cols + kTW - 1) / kTW, nty = (p.f.rows + kTH - 1) / kTH;
    const int64_t ntiles = ntx * nty;
    if (ntiles == 0) return cudaSuccess;
    const size_t smem = 2 * kStageStride;
    cudaError_t e = cudaFuncSetAttribute(focal64_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, focal64_tma_kernel, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > ntiles) grid = ntiles;
    // band of the levels' nodata as high-word keys (conservative superset)
    int klo = key_hi(p.f.nd6d.lo), khi = key_hi(p.f.nd6d.hi);
    if (!(p.f.nd6d.lo <= p.f.nd6d.hi)) {
        klo = 1;
        khi = 0;  // empty band
    }
    focal64_tma_kernel<<<(unsigned)grid, kThreads, smem, s>>>(*map, p, ntx, ntiles, klo, khi);
    return cudaGetLastError();
}

}  // namespace pargo
