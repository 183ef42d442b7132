// focal64.cu -- Horn slope + D8 over a float64 surface, TMA-tiled.
//
// The surface is the pit-removed levels of the hydrology chain: the reference
// D8 reads the Float64 output of pit removal (pPitRemove.cpp:129 writes it,
// pD8.cpp:113 reads it), so the codes must come from the float64 levels.
// Their differences are of order the gap (5e-4 m) and must be exact before
// rounding.  GB300's FP64 rate is a small fraction of its FP32 rate, so the
// differences are taken on integer keys instead: within one binade a key
// difference is the exact value difference in ulps.  Windows that span
// binades or touch nodata fall back to FP64 (cell_general64).

// Layout: CTAs of 4 warps walk 32 x 64-cell tiles; the box (34 x 68 doubles,
// x starting 2 cells left so x * 8 bytes stays a multiple of 16) is TMA-loaded
// into a double-buffered stage.  A lane owns 2 columns and walks 8 rows with a
// rolling three-row window of integer keys.  The
// kernel can also copy the levels out as the filled-DEM raster (float32 or
// float64, +inf levels written as that raster's nodata), so the chain reads
// the levels once.

#include <string.h>

#include <algorithm>

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
    // nodata bands as order-preserving integer keys (the same sets; no FP64 compares)
    const long long k7lo = dkey64(p.nd7d.lo), k7hi = dkey64(p.nd7d.hi);
    const long long k6lo = dkey64(p.nd6d.lo), k6hi = dkey64(p.nd6d.hi);
    const bool empty7 = !(p.nd7d.lo <= p.nd7d.hi), empty6 = !(p.nd6d.lo <= p.nd6d.hi);
    bool nd_slope = false, nd_d8 = false;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const long long k = dkey64(z[q]);
        const bool nan = (k & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL;
        nd_slope |= !empty7 && !nan && k >= k7lo && k <= k7hi;
        nd_d8 |= !empty6 && !nan && k >= k6lo && k <= k6hi;
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

constexpr int kNoBinade = -1000000;

// Keys of row `ty` (tile-local) for this lane's columns 2l-1 .. 2l+2, the
// common binade of each of its two cells' three columns (kNoBinade when they
// differ, when one may be nodata, or when the binade's ulp scale does not fit
// a normal float), and which columns hold +inf.  Within one binade (equal
// key >> 52: sign and exponent) key differences are the exact value
// differences in units of the binade's ulp, of either sign.
constexpr long long kInfKey = 0x7FF0000000000000LL;  // key of +inf: the pipeline levels' nodata

struct RowKeys {
    int t0, t1;    // the common binade of columns 0-2 (cell 0's window) and 1-3 (cell 1's), else kNoBinade
    unsigned inf;  // bit a: column a holds +inf (a nodata level of the pipeline)
};
__device__ __forceinline__ RowKeys load_keys(const double* s, int ty, int lane, long long k[4], const Focal64Params& P,
                                             int klo, int khi) {
    const double* row = s + (ty + 1) * kBoxW + 2 * lane + 1;  // column 2l-1 sits at box column 2l+1
    const double2 q = *reinterpret_cast<const double2*>(row + 1);
    k[0] = dkey64(row[0]);
    k[1] = dkey64(q.x);
    k[2] = dkey64(q.y);
    k[3] = dkey64(row[3]);
    RowKeys o;
    int t[4];
    bool ok[4];
    o.inf = 0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        t[a] = (int)(k[a] >> 52);
        const int e = t[a] >= 0 ? t[a] : -1 - t[a];  // biased exponent
        ok[a] = e >= 960 && e <= 1190;  // 2^(1075 - e) and 2^(e - 1075) are normal floats; no inf/NaN
        if (!P.nodata_is_inf) {
            const int hi = (int)(k[a] >> 32);
            ok[a] = ok[a] && !(hi >= klo && hi <= khi);
        }
        o.inf |= (k[a] == kInfKey ? 1u : 0u) << a;
    }
    o.t0 = ok[0] && ok[1] && ok[2] && t[1] == t[0] && t[2] == t[0] ? t[0] : kNoBinade;
    o.t1 = ok[1] && ok[2] && ok[3] && t[2] == t[1] && t[3] == t[1] ? t[1] : kNoBinade;
    return o;
}

// An exact int64 difference (|d| < 2^53) as a float without the 64-bit
// conversion (an FP64-pipe instruction): the magnitude's two 32-bit halves
// converted separately and joined by one fma.  Below 2^32 this is the single
// correct rounding; above, the error is at most 2^-23 |d| (the low half's
// rounding, 2^8, is below 2^-24 |d|), which keeps the certified D8 bound
// |x - r| <= 2^-22 |x| with the diagonal's extra roundings.
// The conversions run on the FP32 and integer pipes: an integer x < 2^23 is
// exactly the float 2^23 + x (x in the significand) minus 2^23, so the high
// half (< 2^22: |d| < 2^54) converts exactly, and the low half's two 16-bit
// halves convert exactly and are joined by one fma -- the single correct
// rounding of the low half, the same bits as __uint2float_rn gives.  The
// hardware conversion instructions ran on the FP64 pipe here (a narrow pipe
// on this part; 50% busy on the 2048^2 profile with ~5% of cells on FP64).
__device__ __forceinline__ float u23f(unsigned x) { return __int_as_float(0x4B000000u | x) - 8388608.0f; }
__device__ __forceinline__ float i64f(long long d) {
    const unsigned long long a = (unsigned long long)(d < 0 ? -d : d);
    const unsigned lo = (unsigned)a, hi = (unsigned)(a >> 32);
    const float lof = __fmaf_rn(u23f(lo >> 16), 65536.0f, u23f(lo & 0xFFFFu));
    const float f = __fmaf_rn(u23f(hi), 4294967296.0f, lof);
    return d < 0 ? -f : f;
}

__device__ __forceinline__ void put_copy(const OutView& o, int64_t r, int64_t c, double w) {
    const bool nd = (__double_as_longlong(w) & 0x7FFFFFFFFFFFFFFFLL) == 0x7FF0000000000000LL;  // +-inf, bit test
    if (o.dtype == PARGO_F32) reinterpret_cast<float*>(o.base + r * o.pitch)[c] = nd ? (float)o.nodata : dbl2flt_rn(w);
    else put_value(o, r, c, nd ? o.nodata : w);
}

// The FP32 fast decision of focal.cu (bounds there) on drops measured in
// units of the binade's ulp: the 1e-6 thresholds scale by inv_unit, an exact
// power of two.  Index of a certain single maximum, -1 when the maximum is
// certainly below 1e-6, else kD8Unsure.
__device__ __forceinline__ int d8_fast_scaled(float x0, float x1, float x2, float x3, float x5, float x6, float x7,
                                              float x8, float inv_unit) {
    const float m = fmaxf(fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)), fmaxf(fmaxf(x5, x6), fmaxf(x7, x8)));
    const float t = __fadd_rn(__fmaf_rn(m, -1.9073486328125e-06f, m), -kTHi * inv_unit);
    const unsigned mask = (x0 > t ? 1u : 0u) | (x1 > t ? 2u : 0u) | (x2 > t ? 4u : 0u) | (x3 > t ? 8u : 0u) |
                          (x5 > t ? 32u : 0u) | (x6 > t ? 64u : 0u) | (x7 > t ? 128u : 0u) | (x8 > t ? 256u : 0u);
    const int k = __ffs(mask) - 1;
    const bool single = (mask & (mask - 1)) == 0;
    return m < 0.99996924e-6f * inv_unit ? -1 : (m > 1.0000329e-6f * inv_unit && single) ? k : kD8Unsure;
}

// One 32 x 64 tile.  Lane l owns columns 2l, 2l+1 and walks 8 rows with a
// rolling three-row window of keys.  Rows whose 3 x 4 window shares one
// binade (and holds no nodata) take the integer path: every neighbour
// difference is an exact int64 key difference, formed once per row for the
// two cells it joins and rounded to float in ulp units; the Horn numerators
// are summed exactly in int64 before rounding.  No FP64 instruction runs on
// that path.  Other rows (binade crossings, nodata), the ring, other slope
// methods and uncertain D8 decisions are recomputed afterwards by
// cell_general64 from the staged doubles.
__device__ __forceinline__ void compute_tile64(const double* s, int64_t y0, int64_t x0, const Focal64Params& P,
                                               int klo, int khi, int& fell_back, unsigned long long& raised) {
    const FocalParams& p = P.f;
    const float kinv = 0.70710677f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = warp * kRows;
    const int64_t gx0 = x0 + 2 * lane, gy0 = y0 + r0;
    const bool interior = (p.sk.method == PARGO_SLOPE_FD || !p.do_slope) && gy0 >= 1 && gy0 + kRows <= p.rows - 1 &&
                          gx0 >= 1 && gx0 + 2 <= p.cols - 1;
    const float slope_nd = (float)p.slope.nodata;  // nodata outputs, converted once
    const int d8_nd = (int)p.d8.nodata;
    long long ka[4], kb[4], kc[4];
    RowKeys ra = load_keys(s, r0 - 1, lane, ka, P, klo, khi);
    RowKeys rb = load_keys(s, r0, lane, kb, P, klo, khi);
    // the previous row's downward drops seen from this row (negated): S, SE (e1), SW (e2) of row a
    float nS[2], e1p[3], e2p[3];
#pragma unroll
    for (int j = 0; j < 2; j++) nS[j] = i64f(ka[j + 1] - kb[j + 1]);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        e1p[a] = i64f(ka[a] - kb[a + 1]) * kinv;
        e2p[a] = i64f(ka[a + 1] - kb[a]) * kinv;
    }
    unsigned redo = 0;  // bit 2i + j: cell j of row i goes to the general path
#pragma unroll 1
    for (int i = 0; i < kRows; i++) {
        const RowKeys rc = load_keys(s, r0 + i + 1, lane, kc, P, klo, khi);
        const int64_t gy = gy0 + i;
        // drops of row b shared by the cells they join
        float h[3], e1[3], e2[3], vS[2];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            h[a] = i64f(kb[a + 1] - kb[a]);
            e1[a] = i64f(kb[a] - kc[a + 1]) * kinv;
            e2[a] = i64f(kb[a + 1] - kc[a]) * kinv;
        }
#pragma unroll
        for (int j = 0; j < 2; j++) vS[j] = i64f(kb[j + 1] - kc[j + 1]);
        const unsigned infs = ra.inf | rb.inf | rc.inf;
        float sl[2] = {0.0f, 0.0f};
        int cd[2] = {0, 0};
        bool nodata[2], gen[2];
#pragma unroll
        for (int j = 0; j < 2; j++) {
            // a +inf level in the cell's window makes both outputs nodata, as
            // the general path's nodata bands do; else the integer path when
            // the window lies in one binade
            nodata[j] = P.nodata_is_inf && ((infs >> j) & 7u) != 0;
            const int ta = j ? ra.t1 : ra.t0, tb = j ? rb.t1 : rb.t0, tc = j ? rc.t1 : rc.t0;
            const bool fast = !nodata[j] && interior && ta != kNoBinade && ta == tb && tb == tc;
            gen[j] = !nodata[j] && !fast;
            if (fast) {
                const int e = ta >= 0 ? ta : -1 - ta;
                const float unit = __int_as_float((127 + e - 1075) << 23);     // the binade's ulp
                const float inv_unit = __int_as_float((127 + 1075 - e) << 23);
                if (p.do_slope) {
                    const long long nx = ((ka[j + 2] - ka[j]) + (kc[j + 2] - kc[j])) + 2 * (kb[j + 2] - kb[j]);
                    const long long ny = ((ka[j] - kc[j]) + (ka[j + 2] - kc[j + 2])) + 2 * (ka[j + 1] - kc[j + 1]);
                    sl[j] = horn_slope(i64f(nx) * unit, i64f(ny) * unit, p.sk.k_fd);
                    if (p.sk.degrees) sl[j] = atanf(sl[j]) * 57.29577951308232f;
                }
                if (p.do_d8) {
                    cd[j] = d8_fast_scaled(-e1p[j], -nS[j], -e2p[j + 1], h[j], -h[j + 1], e2[j], vS[j], e1[j + 1],
                                           inv_unit);
                    if (cd[j] != kD8Unsure && p.dir_type != 8 && cd[j] >= 0) cd[j] = d8_bit_code(cd[j]);
                    gen[j] = cd[j] == kD8Unsure;
                }
            }
            redo |= (gen[j] ? 1u : 0u) << (2 * i + j);
        }
        if (gy < p.rows) {
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const int64_t gx = gx0 + j;
                if (gx >= p.cols) break;
                if (nodata[j]) {
                    if (p.do_slope) put_float(p.slope, gy, gx, slope_nd);
                    if (p.do_d8) put_int(p.d8, gy, gx, d8_nd);
                } else if (!gen[j]) {
                    if (p.do_slope) put_float(p.slope, gy, gx, sl[j]);
                    if (p.do_d8) put_int(p.d8, gy, gx, cd[j]);
                }
                const double w = s[(r0 + i + 1) * kBoxW + 2 * lane + j + 2];
                if (P.do_copy) put_copy(P.copy, gy, gx, w);
                if (P.raised) {  // level above the DEM, compared as order-preserving keys
                    const char* row = reinterpret_cast<const char*>(P.dem) + gy * P.dem_pitch;
                    const long long kz = P.dem_f64 ? dkey64(reinterpret_cast<const double*>(row)[gx])
                                                   : fkey64(reinterpret_cast<const float*>(row)[gx]);
                    const long long kw = kb[j + 1];
                    raised += (kw < 0x7FF0000000000000LL && kw > kz) ? 1 : 0;
                }
            }
        }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            ka[a] = kb[a];
            kb[a] = kc[a];
        }
#pragma unroll
        for (int j = 0; j < 2; j++) nS[j] = vS[j];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            e1p[a] = e1[a];
            e2p[a] = e2[a];
        }
        ra = rb;
        rb = rc;
    }
    // Rows the integer path did not finish: the general FP64 path on the
    // staged window.  Their cells are first gathered across the warp, so the
    // FP64 work (a slow pipe on this part) runs on full warps rather than on
    // the few lanes of each row that need it.
    __shared__ uint16_t redo_items[kWarps][kRows * 64];  // (row << 6) | tile column
    uint16_t* items = redo_items[warp];
    const unsigned lt = (1u << lane) - 1u;
    int n = 0;
#pragma unroll 1
    for (int i = 0; i < kRows; i++) {
        const unsigned rd = (redo >> (2 * i)) & 3u;  // this lane's cells of row i
        const unsigned b1 = __ballot_sync(0xFFFFFFFFu, rd & 1u), b2 = __ballot_sync(0xFFFFFFFFu, rd & 2u);
        int pos = n + __popc(b1 & lt) + __popc(b2 & lt);
        if (rd & 1u) items[pos++] = (uint16_t)((i << 6) | (2 * lane));
        if (rd & 2u) items[pos] = (uint16_t)((i << 6) | (2 * lane + 1));
        n += __popc(b1) + __popc(b2);
    }
    __syncwarp();
#pragma unroll 1
    for (int q = lane; q < n; q += 32) {
        const int i = items[q] >> 6, cc = items[q] & 63;
        const int64_t gy = gy0 + i, gx = x0 + cc;
        if (gy >= p.rows || gx >= p.cols) continue;
        const bool ring = gy <= 0 || gx <= 0 || gy >= p.rows - 1 || gx >= p.cols - 1;
        const double* w = s + (r0 + i) * kBoxW + cc + 1;  // window's top-left
        const CellOut o = cell_general64(w[0], w[1], w[2], w[kBoxW], w[kBoxW + 1], w[kBoxW + 2], w[2 * kBoxW],
                                         w[2 * kBoxW + 1], w[2 * kBoxW + 2], &p, ring);
        fell_back += (o.flags >> 2) & 1;
        if (p.do_slope) {
            if (o.flags & 1) put_value(p.slope, gy, gx, p.slope.nodata);
            else put_float(p.slope, gy, gx, o.slope);
        }
        if (p.do_d8) {
            if (o.flags & 2) put_value(p.d8, gy, gx, p.d8.nodata);
            else put_int(p.d8, gy, gx, o.code);
        }
    }
    __syncwarp();  // the list is rewritten by the next tile
}

__global__ void __launch_bounds__(kThreads, 4) focal64_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                                  const __grid_constant__ Focal64Params P,
                                                                  int64_t ntx, int64_t t_begin, int64_t ntiles,
                                                                  int klo, int khi) {
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
    int64_t t = t_begin + blockIdx.x;  // tiles t_begin .. ntiles-1
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

cudaError_t launch_focal64_tma(const CUtensorMap* map, const Focal64Params& p, int num_sms, cudaStream_t s,
                               int64_t row_begin, int64_t row_end) {
    const int64_t ntx = (p.f.cols + kTW - 1) / kTW, nty = (p.f.rows + kTH - 1) / kTH;
    // tile rows covering output rows [row_begin, row_end); row_begin is a multiple of kTH
    const int64_t ty0 = row_begin / kTH;
    const int64_t ty1 = row_end < 0 ? nty : std::min(nty, (row_end + kTH - 1) / kTH);
    const int64_t t_begin = ty0 * ntx, ntiles = ty1 * ntx;
    if (ntiles <= t_begin) return cudaSuccess;
    const size_t smem = 2 * kStageStride;
    cudaError_t e = cudaFuncSetAttribute(focal64_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, focal64_tma_kernel, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > ntiles - t_begin) grid = ntiles - t_begin;
    // band of the levels' nodata as high-word keys (conservative superset)
    int klo = key_hi(p.f.nd6d.lo), khi = key_hi(p.f.nd6d.hi);
    if (!(p.f.nd6d.lo <= p.f.nd6d.hi)) {
        klo = 1;
        khi = 0;  // empty band
    }
    focal64_tma_kernel<<<(unsigned)grid, kThreads, smem, s>>>(*map, p, ntx, t_begin, ntiles, klo, khi);
    return cudaGetLastError();
}

}  // namespace pargo
