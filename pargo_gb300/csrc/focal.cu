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

#include <type_traits>

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
    static constexpr int kStageStride = (kStageBytes + 127) / 128 * 128;  // TMA needs 128-byte aligned stages
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
// columns 4l-1 .. 4l+4 (box columns 4l+3 .. 4l+8): one 16-byte load and two
// scalar loads.
__device__ __forceinline__ void load_row(const float* s, int ty, int lane, float v[6]) {
    const float* row = s + (ty + 1) * kBoxW + 4 * lane + 3;
    const float4 q = *reinterpret_cast<const float4*>(row + 1);
    v[0] = row[0]; v[1] = q.x; v[2] = q.y; v[3] = q.z; v[4] = q.w; v[5] = row[5];
}

// Whether some of the 6 values may lie in the wide (Eps 1e-6) nodata band.
// A band below zero (the usual negative nodata) needs only the row minimum.
__device__ __forceinline__ bool row_maybe_nodata(const float v[6], const Band<float>& b) {
    const float mn = fminf(fminf(fminf(v[0], v[1]), fminf(v[2], v[3])), fminf(v[4], v[5]));
    if (b.hi < 0.0f) return mn <= b.hi;
    const float mx = fmaxf(fmaxf(fmaxf(v[0], v[1]), fmaxf(v[2], v[3])), fmaxf(v[4], v[5]));
    return mn <= b.hi && mx >= b.lo;
}

// Packed FP32 pairs (one f32x2 instruction for two IEEE operations, each
// rounded exactly as the scalar operation).
#ifndef PARGO_PACK
#define PARGO_PACK 0
#endif
#if PARGO_PACK == 0
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    return make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y));
}
#else
#if PARGO_PACK == 1
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
#else
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
#endif
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
#endif
__device__ __forceinline__ float2 pr(float a, float b) { return make_float2(a, b); }

// Byte permute in the sign-replicating form: a selector nibble with bit 3
// set yields the selected byte's top bit copied over all eight bits.
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
    return d;
}

// FP32 D8 fast path on the eight drops (window order; the centre is absent):
// the window index of a certain single maximum, -1 when the maximum is
// certainly below 1e-6, else kD8Unsure.
//   M vs 1e-6: |x_k - r_k| <= 2^-22 x_k, so x < kLowCut gives M < 1e-6 and
//   x > kHighCut gives M >= 1e-6 for certain;
//   single maximum: every other x_i <= m - (1e-6 + 2^-19 m) is certainly
//   outside the tie set (x_i >= 0: |x_i| <= m; x_i < 0: the gap exceeds m).
constexpr float kLowCut = 0.99996924e-6f;   // kTLo (1 - 2^-21), rounded down
constexpr float kHighCut = 1.0000329e-6f;   // kTHi (1 + 2^-21), rounded up
constexpr float k2m19 = 1.9073486328125e-06f;
#ifndef PARGO_D8MASK
#define PARGO_D8MASK 0
#endif
#if PARGO_D8MASK
__device__ __forceinline__ int d8_fast(float x0, float x1, float x2, float x3, float x5, float x6, float x7, float x8) {
    const float m = fmaxf(fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)), fmaxf(fmaxf(x5, x6), fmaxf(x7, x8)));
    const float t = __fadd_rn(__fmaf_rn(m, -k2m19, m), -kTHi);
    const unsigned mask = (x0 > t ? 1u : 0u) | (x1 > t ? 2u : 0u) | (x2 > t ? 4u : 0u) | (x3 > t ? 8u : 0u) |
                          (x5 > t ? 32u : 0u) | (x6 > t ? 64u : 0u) | (x7 > t ? 128u : 0u) | (x8 > t ? 256u : 0u);
    const int k = __ffs(mask) - 1;
    const bool single = (mask & (mask - 1)) == 0;
    return m < kLowCut ? -1 : (m > kHighCut && single) ? k : kD8Unsure;
}
#else
__device__ __forceinline__ int d8_fast(float x0, float x1, float x2, float x3, float x5, float x6, float x7, float x8) {
    const float m = fmaxf(fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)), fmaxf(fmaxf(x5, x6), fmaxf(x7, x8)));
    const float t = __fadd_rn(__fmaf_rn(m, -k2m19, m), -kTHi);
    // x_i > t  <=>  t - x_i < 0: gather the eight sign bits, each replicated
    // over one byte, for x0..x3 in `ua` and x5..x8 in `ub`; blend them into
    // one word (ua on even bits, ub on odd bits).  A single x_i above t sets
    // exactly four bits, and the highest of them gives i.
    const float2 tt = pr(t, t);
    const float2 d01 = sub2(tt, pr(x0, x1)), d23 = sub2(tt, pr(x2, x3));
    const float2 d56 = sub2(tt, pr(x5, x6)), d78 = sub2(tt, pr(x7, x8));
    const uint32_t ua = prmt(prmt(__float_as_uint(d01.x), __float_as_uint(d01.y), 0x00FB),
                             prmt(__float_as_uint(d23.x), __float_as_uint(d23.y), 0x00FB), 0x5410);
    const uint32_t ub = prmt(prmt(__float_as_uint(d56.x), __float_as_uint(d56.y), 0x00FB),
                             prmt(__float_as_uint(d78.x), __float_as_uint(d78.y), 0x00FB), 0x5410);
    const uint32_t w = (ua & 0x55555555u) | (ub & 0xAAAAAAAAu);
    uint32_t hb;
    asm("bfind.u32 %0, %1;" : "=r"(hb) : "r"(w));  // position of the highest set bit
    const int k = (int)((hb >> 3) + (hb & 1) * 5);  // byte b of ua -> window b, of ub -> window b + 5
    const bool sure = (m > kHighCut) & (__popc(w) == 4);  // no short-circuit branch
    return m < kLowCut ? -1 : sure ? k : kD8Unsure;
}
#endif

// ArcGIS weight of a window index (d8Operator.cpp:96-97): 1 << shift, the
// shifts packed as nibbles 0..8 = 5,6,7,4,-,0,3,2,1.
__device__ __forceinline__ int d8_weight(int k) {
    return (unsigned)k > 8u ? k : 1 << (int)((0x123004765ULL >> (4 * k)) & 15);  // -1 and kD8Unsure pass through
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
// differences sh (rows) and sv (columns).  Arithmetic runs on packed f32x2
// pairs.  The main loop has no per-cell branch: cells whose window may touch
// nodata or the raster's ring, any slope method but Horn, and D8 decisions the
// FP32 bounds cannot certify are marked in a bit set and recomputed from the
// stage by cell_general afterwards (overwriting what the loop stored).
template <int ROWS, int UNROLL, bool SLOPE, bool D8>
__device__ __forceinline__ void compute_tile(const float* s, int64_t y0, int64_t x0, const FocalParams& p,
                                             int& fell_back) {
    const float2 kinv2 = pr(0.70710677f, 0.70710677f);
    const float2 two2 = pr(2.0f, 2.0f);
    const float2 kfd2 = pr(p.sk.k_fd, p.sk.k_fd);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = warp * ROWS;
    const int64_t gx0 = x0 + 4 * lane, gy0 = y0 + r0;
    const bool interior = p.fd && gy0 >= 1 && gy0 + ROWS <= p.rows - 1 && gx0 >= 1 && gx0 + 4 <= p.cols - 1;
    const bool dir8 = p.dir_type == 8;
    unsigned redo = 0;  // bit i: row i's four cells go to the general path
    float va[6], vb[6], vc[6];
    load_row(s, r0 - 1, lane, va);
    load_row(s, r0, lane, vb);
    bool nda = row_maybe_nodata(va, p.nd6f), ndb = row_maybe_nodata(vb, p.nd6f);
    float shA[4], shB[4], nS[4], e1p[5], e2p[5];  // nS, e1p, e2p: the previous row's vS, e1, e2
    {
        const float2 a01 = sub2(pr(va[2], va[3]), pr(va[0], va[1])), a23 = sub2(pr(va[4], va[5]), pr(va[2], va[3]));
        const float2 b01 = sub2(pr(vb[2], vb[3]), pr(vb[0], vb[1])), b23 = sub2(pr(vb[4], vb[5]), pr(vb[2], vb[3]));
        shA[0] = a01.x; shA[1] = a01.y; shA[2] = a23.x; shA[3] = a23.y;
        shB[0] = b01.x; shB[1] = b01.y; shB[2] = b23.x; shB[3] = b23.y;
        // previous-row quantities seen from row b: vS = va[j+1] - vb[j+1],
        // e1[a] = (va[a] - vb[a+1]) / sqrt 2, e2[a] = (va[a+1] - vb[a]) / sqrt 2
        const float2 s01 = sub2(pr(va[1], va[2]), pr(vb[1], vb[2])), s23 = sub2(pr(va[3], va[4]), pr(vb[3], vb[4]));
        nS[0] = s01.x; nS[1] = s01.y; nS[2] = s23.x; nS[3] = s23.y;
        const float2 p01 = mul2(sub2(pr(va[0], va[1]), pr(vb[1], vb[2])), kinv2);
        const float2 p23 = mul2(sub2(pr(va[2], va[3]), pr(vb[3], vb[4])), kinv2);
        const float2 q01 = mul2(sub2(pr(va[1], va[2]), pr(vb[0], vb[1])), kinv2);
        const float2 q23 = mul2(sub2(pr(va[3], va[4]), pr(vb[2], vb[3])), kinv2);
        const float2 pq4 = mul2(sub2(pr(va[4], va[5]), pr(vb[5], vb[4])), kinv2);
        e1p[0] = p01.x; e1p[1] = p01.y; e1p[2] = p23.x; e1p[3] = p23.y; e1p[4] = pq4.x;
        e2p[0] = q01.x; e2p[1] = q01.y; e2p[2] = q23.x; e2p[3] = q23.y; e2p[4] = pq4.y;
    }
    char* srow = SLOPE ? p.slope.base + gy0 * p.slope.pitch : nullptr;
    char* drow = D8 ? p.d8.base + gy0 * p.d8.pitch : nullptr;
    const bool vec = p.fast_out && gx0 + 3 < p.cols;
#pragma unroll UNROLL
    for (int i = 0; i < ROWS; i++) {
        load_row(s, r0 + i + 1, lane, vc);
        const bool ndc = row_maybe_nodata(vc, p.nd6f);
        // row-b / row-c differences
        const float2 c01 = sub2(pr(vc[2], vc[3]), pr(vc[0], vc[1])), c23 = sub2(pr(vc[4], vc[5]), pr(vc[2], vc[3]));
        const float2 v01 = sub2(pr(va[0], va[1]), pr(vc[0], vc[1])), v23 = sub2(pr(va[2], va[3]), pr(vc[2], vc[3]));
        const float2 v45 = sub2(pr(va[4], va[5]), pr(vc[4], vc[5]));
        const float2 h01 = sub2(pr(vb[1], vb[2]), pr(vb[0], vb[1])), h23 = sub2(pr(vb[3], vb[4]), pr(vb[2], vb[3]));
        const float2 s01 = sub2(pr(vb[1], vb[2]), pr(vc[1], vc[2])), s23 = sub2(pr(vb[3], vb[4]), pr(vc[3], vc[4]));
        const float2 p01 = mul2(sub2(pr(vb[0], vb[1]), pr(vc[1], vc[2])), kinv2);
        const float2 p23 = mul2(sub2(pr(vb[2], vb[3]), pr(vc[3], vc[4])), kinv2);
        const float2 q01 = mul2(sub2(pr(vb[1], vb[2]), pr(vc[0], vc[1])), kinv2);
        const float2 q23 = mul2(sub2(pr(vb[3], vb[4]), pr(vc[2], vc[3])), kinv2);
        const float2 pq4 = mul2(sub2(pr(vb[4], vb[5]), pr(vc[5], vc[4])), kinv2);
        const float2 h4s = sub2(pr(vb[5], 0.0f), pr(vb[4], 0.0f));
        const float h[5] = {h01.x, h01.y, h23.x, h23.y, h4s.x};
        const float vS[4] = {s01.x, s01.y, s23.x, s23.y};
        const float e1[5] = {p01.x, p01.y, p23.x, p23.y, pq4.x};
        const float e2[5] = {q01.x, q01.y, q23.x, q23.y, pq4.y};
        const bool slow = !interior || nda || ndb || ndc;
        float sl[4];
        int cd[4];
        if (SLOPE) {
            const float2 nx01 = fma2(two2, pr(shB[0], shB[1]), add2(pr(shA[0], shA[1]), c01));
            const float2 nx23 = fma2(two2, pr(shB[2], shB[3]), add2(pr(shA[2], shA[3]), c23));
            const float2 ny01 = fma2(two2, pr(v01.y, v23.x), add2(v01, pr(v23.x, v23.y)));
            const float2 ny23 = fma2(two2, pr(v23.y, v45.x), add2(v23, v45));
            const float2 q01s = fma2(nx01, nx01, mul2(ny01, ny01));
            const float2 q23s = fma2(nx23, nx23, mul2(ny23, ny23));
            const float2 r01 = mul2(pr(sqrt_sfu(q01s.x), sqrt_sfu(q01s.y)), kfd2);
            const float2 r23 = mul2(pr(sqrt_sfu(q23s.x), sqrt_sfu(q23s.y)), kfd2);
            sl[0] = r01.x; sl[1] = r01.y; sl[2] = r23.x; sl[3] = r23.y;
            if (p.sk.degrees) {
#pragma unroll
                for (int j = 0; j < 4; j++) sl[j] = atanf(sl[j]) * 57.29577951308232f;
            }
        }
        if (D8) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                cd[j] = d8_fast(-e1p[j], -nS[j], -e2p[j + 1], h[j], -h[j + 1], e2[j], vS[j], e1[j + 1]);
        }
        bool rb = slow;
        if (D8) {
            rb = rb || cd[0] == kD8Unsure || cd[1] == kD8Unsure || cd[2] == kD8Unsure || cd[3] == kD8Unsure;
            if (!dir8) {
#pragma unroll
                for (int j = 0; j < 4; j++) cd[j] = d8_weight(cd[j]);
            }
        }
        redo |= (rb ? 1u : 0u) << i;
        const int64_t gy = gy0 + i;
        if (gy < p.rows) {
            if (vec) {
                if (SLOPE) *reinterpret_cast<float4*>(srow + 4 * gx0) = make_float4(sl[0], sl[1], sl[2], sl[3]);
                if (D8)
                    *reinterpret_cast<uint32_t*>(drow + gx0) = __byte_perm(
                        __byte_perm((uint32_t)cd[0], (uint32_t)cd[1], 0x0040), __byte_perm((uint32_t)cd[2], (uint32_t)cd[3], 0x0040),
                        0x5410);
            } else if (!rb) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int64_t gx = gx0 + j;
                    if (gx >= p.cols) break;
                    if (SLOPE) put_float(p.slope, gy, gx, sl[j]);
                    if (D8) put_int(p.d8, gy, gx, cd[j]);
                }
            }
        }
        if (SLOPE) srow += p.slope.pitch;
        if (D8) drow += p.d8.pitch;
        // roll the window down one row
#pragma unroll
        for (int a = 0; a < 6; a++) {
            va[a] = vb[a];
            vb[a] = vc[a];
        }
        shA[0] = shB[0]; shA[1] = shB[1]; shA[2] = shB[2]; shA[3] = shB[3];
        shB[0] = c01.x; shB[1] = c01.y; shB[2] = c23.x; shB[3] = c23.y;
#pragma unroll
        for (int j = 0; j < 4; j++) nS[j] = vS[j];
#pragma unroll
        for (int a = 0; a < 5; a++) {
            e1p[a] = e1[a];
            e2p[a] = e2[a];
        }
        nda = ndb;
        ndb = ndc;
    }
    // Cells the loop could not finish: the general path on the staged window.
    while (redo) {
        const int i = __ffs(redo) - 1;
        redo &= redo - 1;
        const int64_t gy = gy0 + i;
        if (gy >= p.rows) break;  // rows only grow from here
#pragma unroll 1
        for (int j = 0; j < 4; j++) {
            const int64_t gx = gx0 + j;
            if (gx >= p.cols) break;
            const bool ring = gy <= 0 || gx <= 0 || gy >= p.rows - 1 || gx >= p.cols - 1;
            const float* w = s + (r0 + i) * kBoxW + 4 * lane + j + 3;  // window's top-left: stage row r0+i, col 4l+j+3
            const CellOut o = cell_general<float>(w[0], w[1], w[2], w[kBoxW], w[kBoxW + 1], w[kBoxW + 2], w[2 * kBoxW],
                                                  w[2 * kBoxW + 1], w[2 * kBoxW + 2], &p, ring);
            fell_back += (o.flags >> 2) & 1;
            if (SLOPE) {
                if (o.flags & 1) put_value(p.slope, gy, gx, p.slope.nodata);
                else put_float(p.slope, gy, gx, o.slope);
            }
            if (D8) {
                if (o.flags & 2) put_value(p.d8, gy, gx, p.d8.nodata);
                else put_int(p.d8, gy, gx, o.code);
            }
        }
    }
}

template <int ROWS, int UNROLL, int MINB, bool SLOPE, bool D8>
__global__ void __launch_bounds__(kThreads, MINB) focal_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                                const __grid_constant__ FocalParams p, int64_t ntx,
                                                                int64_t ntiles) {
    using S = Shape<ROWS>;
    constexpr int kTH = S::kTH, kStageBytes = S::kStageBytes, kStageStride = S::kStageStride;
    extern __shared__ __align__(128) unsigned char smem[];
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
        compute_tile<ROWS, UNROLL, SLOPE, D8>(reinterpret_cast<const float*>(smem + st * kStageStride),
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
template <bool SLOPE, bool D8>
__global__ void __launch_bounds__(kThreads, 5) batch_tma_kernel(const CUtensorMap* maps, const FocalParams* params,
                                                             const int64_t* tile_start, const int64_t* ntx_of,
                                                             int count, int64_t total, unsigned long long* claim,
                                                             unsigned long long* fallbacks, int* error_flag) {
    extern __shared__ __align__(128) unsigned char smem[];
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
        compute_tile<kBatchRows, 1, SLOPE, D8>(reinterpret_cast<const float*>(smem + st * kStageStride),
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

// ------------------------------------------------------------ strip walk --
// Warp-independent form of the same computation.  Each warp walks a 128-cell
// wide column strip down a segment of kSegRows rows, keeping the three-row
// window and the per-row / per-row-pair differences in registers from one
// row to the next (no tile prologue, no re-read halo rows), with a private
// pipeline of TMA stages: a 2-row priming box per segment, then kSegStages
// boxes of kSR rows, double-buffered and waited on by mbarrier.  Segments
// are claimed from a device counter, so strips whose lanes fall back to the
// general path often (the raster's left and right edges) do not stretch the
// launch.  The row loop is unrolled by three with the registers' roles
// rotated (above / centre / below), so no register is copied from row to row.
// Strip geometry, a tuning parameter: SR rows per TMA stage (a multiple of 3:
// the row loop rotates three register roles; at most 32: one bit per row of
// a stage), STAGES stages per segment.
template <int SR_, int STAGES_>
struct StripGeom {
    static_assert(SR_ % 3 == 0 && SR_ <= 30 && STAGES_ >= 2, "strip geometry");
    static constexpr int kSR = SR_;                                   // rows per stage
    static constexpr int kStages = STAGES_;                           // stages per segment
    static constexpr int kSegRows = SR_ * STAGES_;                    // output rows per segment
    static constexpr int kStageBytes = kBoxW * SR_ * 4;
    static constexpr int kStageStride = (kStageBytes + 127) / 128 * 128;
    static constexpr int kPrimeBytes = kBoxW * 2 * 4;                 // 1088
    static constexpr int kPrimeStride = (kPrimeBytes + 127) / 128 * 128;
    static constexpr int kWarpBytes = 2 * kStageStride + 2 * kPrimeStride;
};
// The batched walk's geometry (and the single walk's default): 6-row stages,
// 8 stages, 48-row segments.
using StripDefault = StripGeom<6, 8>;
constexpr int kSR = StripDefault::kSR;
constexpr int kSegStages = StripDefault::kStages;
constexpr int kSegRows = StripDefault::kSegRows;
constexpr int kSStageBytes = StripDefault::kStageBytes;  // 3264
constexpr int kSStageStride = StripDefault::kStageStride;
constexpr int kSPrimeBytes = StripDefault::kPrimeBytes;
constexpr int kSPrimeStride = StripDefault::kPrimeStride;
constexpr int kSWarpBytes = StripDefault::kWarpBytes;
constexpr int kSWarps = 4;

__device__ __forceinline__ float fmax3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// d8_fast with the maximum taken by three-input max (the same value); the
// certification is returned as a flag (false: the general path decides).
// The four drops toward the row above and the east neighbour arrive negated
// (n0 = -x0, n1 = -x1, n2 = -x2, n5 = -x5): their maximum is minus a minimum.
__device__ __forceinline__ int d8_fast3(float n0, float n1, float n2, float x3, float n5, float x6, float x7, float x8,
                                        bool& sure) {
    const float m = fmax3f(fmax3f(x3, x6, x7), x8, -fmin3f(n0, n1, fminf(n2, n5)));
    const float x0 = -n0, x1 = -n1, x2 = -n2, x5 = -n5;
    const float t = __fadd_rn(__fmaf_rn(m, -k2m19, m), -kTHi);
    const uint32_t ua = prmt(prmt(__float_as_uint(__fsub_rn(t, x0)), __float_as_uint(__fsub_rn(t, x1)), 0x00FB),
                             prmt(__float_as_uint(__fsub_rn(t, x2)), __float_as_uint(__fsub_rn(t, x3)), 0x00FB), 0x5410);
    const uint32_t ub = prmt(prmt(__float_as_uint(__fsub_rn(t, x5)), __float_as_uint(__fsub_rn(t, x6)), 0x00FB),
                             prmt(__float_as_uint(__fsub_rn(t, x7)), __float_as_uint(__fsub_rn(t, x8)), 0x00FB), 0x5410);
    const uint32_t w = (ua & 0x55555555u) | (ub & 0xAAAAAAAAu);
    uint32_t hb;
    asm("bfind.u32 %0, %1;" : "=r"(hb) : "r"(w));  // position of the highest set bit
    const bool low = m < kLowCut;
    sure = low | ((m > kHighCut) & (__popc(w) == 4));  // no short-circuit branches
    return low ? -1 : (int)((hb >> 3) + (hb & 1) * 5);
}

__device__ __forceinline__ bool row6_maybe_nodata(const float v[6], const Band<float>& b) {
    const float mn = fminf(fmin3f(v[0], v[1], v[2]), fmin3f(v[3], v[4], v[5]));
    const float mx = fmaxf(fmax3f(v[0], v[1], v[2]), fmax3f(v[3], v[4], v[5]));
    return (mn <= b.hi) & (mx >= b.lo);
}

// One window row: this lane's six values (columns 4l-1 .. 4l+4 of the strip),
// its two-apart differences (Horn x numerator) and whether it may hold nodata.
struct SRow {
    float v[6];
    float sh[4];
    bool nd;
};
// Differences between a row (U) and the row below it (L), each serving the
// two cells it joins: vd[j] = U - L in column j (S of U, -N of L);
// e1[a] = (U[a] - L[a+1]) / sqrt 2 (SE of U[a], -NW of L[a+1]);
// e2[a] = (U[a+1] - L[a]) / sqrt 2 (SW of U[a+1], -NE of L[a]).
struct SPair {
    float vd[4];
    float e1[5];
    float e2[5];
};

// ND: the row's own nodata test; without it the caller knows the row's stage
// holds no value in the nodata band.
template <bool ND = true>
__device__ __forceinline__ void s_load_row(const float* row, int lane, SRow& r, const Band<float>& nd6) {
    const float* q = row + 4 * lane + 3;
    const float4 c = *reinterpret_cast<const float4*>(q + 1);
    r.v[0] = q[0]; r.v[1] = c.x; r.v[2] = c.y; r.v[3] = c.z; r.v[4] = c.w; r.v[5] = q[5];
#pragma unroll
    for (int j = 0; j < 4; j++) r.sh[j] = __fsub_rn(r.v[j + 2], r.v[j]);
    r.nd = ND ? row6_maybe_nodata(r.v, nd6) : false;
}

__device__ __forceinline__ void s_pair(const SRow& u, const SRow& l, SPair& p) {
    const float kinv = 0.70710677f;
#pragma unroll
    for (int j = 0; j < 4; j++) p.vd[j] = __fsub_rn(u.v[j + 1], l.v[j + 1]);
#pragma unroll
    for (int a = 0; a < 5; a++) {
        p.e1[a] = __fmul_rn(__fsub_rn(u.v[a], l.v[a + 1]), kinv);
        p.e2[a] = __fmul_rn(__fsub_rn(u.v[a + 1], l.v[a]), kinv);
    }
}

// Where the fast path cannot finish a lane's four cells of a row (the ring,
// windows that may touch nodata, uncertain D8, lanes at the raster's edge),
// the (row, lane) goes to a device list -- index y * lanes_per_row + gx0 / 4,
// collected as one bit per row through a stage and appended after it -- and
// strip_fixup_kernel recomputes those cells afterwards through the general
// path.
struct SlowList {
    uint32_t* items;
    unsigned long long* count;
    int64_t lanes_per_row;  // ceil(cols / 4)
};

// Output row y from the window rows A (y-1), B (y), C (y+1); C is loaded
// here from stage row `crow`, and the pair B/C is formed for the next row.
// `sp` / `dp` point to this lane's four slope / code cells of row y.  Only the
// plain configuration runs here (Horn, rise/run, dirType 8).
// CLEAN: the stage lies inside the raster's ring, holds no value in the
// nodata band and follows two rows without one, so the row needs none of the
// tests.
template <bool SLOPE, bool D8, bool CLEAN>
__device__ __forceinline__ void strip_step(const float* crow, SRow& A, SRow& B, SRow& C, const SPair& PAB, SPair& PBC,
                                           int y, int rows, int64_t gx0, bool lane_int, float k_fd, const Band<float>& nd6,
                                           char* sp, char* dp, uint32_t& pend, int64_t cols) {
    s_load_row<!CLEAN>(crow, threadIdx.x & 31, C, nd6);
    s_pair(B, C, PBC);
    float sl[4];
    int cd[4];
    if (SLOPE) {
        float sv[6];
#pragma unroll
        for (int a = 0; a < 6; a++) sv[a] = __fsub_rn(A.v[a], C.v[a]);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float nx = __fmaf_rn(2.0f, B.sh[j], __fadd_rn(A.sh[j], C.sh[j]));
            const float ny = __fmaf_rn(2.0f, sv[j + 1], __fadd_rn(sv[j], sv[j + 2]));
            sl[j] = horn_slope(nx, ny, k_fd);
        }
    }
    bool sure = true;
    if (D8) {
        float hd[5];
#pragma unroll
        for (int a = 0; a < 5; a++) hd[a] = __fsub_rn(B.v[a + 1], B.v[a]);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            bool ok;
            cd[j] = d8_fast3(PAB.e1[j], PAB.vd[j], PAB.e2[j + 1], hd[j], hd[j + 1], PBC.e2[j], PBC.vd[j],
                             PBC.e1[j + 1], ok);
            sure &= ok;
        }
    }
    const bool live = CLEAN || y < rows;
    const bool fast = CLEAN ? lane_int & sure
                            : lane_int & ((unsigned)(y - 1) < (unsigned)(rows - 2)) & !(A.nd | B.nd | C.nd) & sure;
    if (live & fast) {
        if (SLOPE) *reinterpret_cast<float4*>(sp) = make_float4(sl[0], sl[1], sl[2], sl[3]);
        if (D8)
            *reinterpret_cast<uint32_t*>(dp) = __byte_perm(__byte_perm((uint32_t)cd[0], (uint32_t)cd[1], 0x0040),
                                                          __byte_perm((uint32_t)cd[2], (uint32_t)cd[3], 0x0040), 0x5410);
    }
    // one bit per row of the stage, shifted in (the stage's first row ends
    // highest); lanes past the raster's last column are dropped at the flush
    pend = pend * 2u + (uint32_t)(live & !fast);
}

// Appends the (row, lane) items of a stage's rows the fast path left (bit b
// of `pend`: row y_last - b), one atomic per lane that has any.
__device__ __noinline__ void strip_flush(uint32_t pend, int y_last, int64_t gx0, const SlowList slow) {
    if ((gx0 >> 2) >= slow.lanes_per_row) return;  // past the raster's last column
    unsigned long long base = atomicAdd(slow.count, (unsigned long long)__popc(pend));
    while (pend) {
        const int b = __ffs(pend) - 1;
        pend &= pend - 1;
        slow.items[base++] = (uint32_t)((int64_t)(y_last - b) * slow.lanes_per_row + (gx0 >> 2));
    }
}

// Whether any value of a stage (kSR rows of the box) may lie in the nodata
// band: the warp's lanes scan it as float4 and vote.
// This lane's share of the stage scan: whether any of its quarter-rows may
// hold a value in the nodata band.  A band below zero (the usual negative
// nodata) needs only the minimum: a stage with values below the band is
// flagged too, which only sends it through the per-row tests.
template <int SR = kSR>
__device__ __forceinline__ bool stage_lane_maybe_nodata(const float* st, const Band<float>& b) {
    const float4* s4 = reinterpret_cast<const float4*>(st);
    constexpr int kQuads = SR * kBoxW / 4;
    float mn = INFINITY, mx = -INFINITY;
    if (b.hi < 0.0f) {
#pragma unroll
        for (int q = threadIdx.x & 31; q < kQuads; q += 32) {
            const float4 v = s4[q];
            mn = fmin3f(fmin3f(v.x, v.y, v.z), v.w, mn);
        }
        return mn <= b.hi;
    }
#pragma unroll
    for (int q = threadIdx.x & 31; q < kQuads; q += 32) {
        const float4 v = s4[q];
        mn = fmin3f(fmin3f(v.x, v.y, v.z), v.w, mn);
        mx = fmax3f(fmax3f(v.x, v.y, v.z), v.w, mx);
    }
    return (mn <= b.hi) & (mx >= b.lo);
}

// Warp-uniform bounded wait on an mbarrier phase.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity) {
    const bool ok = mbar_wait_bounded(bar, parity, kWaitBudget);
    return __all_sync(0xffffffffu, ok);
}

template <bool SLOPE, bool D8, int MINB, int SR, int STAGES>
__global__ void __launch_bounds__(kSWarps * 32, MINB) focal_strip_kernel(const __grid_constant__ CUtensorMap map_stage,
                                                                       const __grid_constant__ CUtensorMap map_prime,
                                                                       const __grid_constant__ FocalParams p,
                                                                       int64_t nstrips, int64_t nsegs,
                                                                       unsigned long long* claim, SlowList slow) {
    using G = StripGeom<SR, STAGES>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[kSWarps][4];  // stage 0, stage 1, prime 0, prime 1
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem + warp * G::kWarpBytes;
    auto stage = [&](int b) { return reinterpret_cast<float*>(wbase + b * G::kStageStride); };
    auto prime = [&](int b) { return reinterpret_cast<float*>(wbase + 2 * G::kStageStride + b * G::kPrimeStride); };
    uint64_t* bar = bars[warp];
    if (lane == 0) {
        tma_prefetch_desc(&map_stage);
        tma_prefetch_desc(&map_prime);
        for (int i = 0; i < 4; i++) mbar_init(&bar[i], 1);
        mbar_fence_init();
    }
    __syncwarp();
    const int64_t box_y_max = p.rows - 1;  // a box always starts inside the raster
    auto claim_seg = [&]() -> int64_t {
        unsigned long long v = 0;
        if (lane == 0) v = atomicAdd(claim, 1ULL);
        return (int64_t)__shfl_sync(0xffffffffu, v, 0);
    };
    // a segment's first column and first output row (segment ids fit 32 bits:
    // the launcher requires rows * ceil(cols / 4) < 2^32), computed once
    struct Origin {
        int x0, y0;
    };
    const uint32_t ns32 = (uint32_t)nstrips;
    auto origin = [&](int64_t seg) {
        const uint32_t sg = (uint32_t)seg;
        return Origin{(int)((sg % ns32) * kTW), (int)((sg / ns32) * G::kSegRows)};
    };
    auto issue_prime = [&](const Origin& o, int buf) {
        if (lane == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[2 + buf], G::kPrimeBytes);
            tma_load_2d(prime(buf), &map_prime, o.x0 - 4, o.y0 - 1, &bar[2 + buf]);
        }
    };
    auto issue_stage = [&](const Origin& o, int k, int buf) {
        if (lane == 0) {
            const int yb = min(o.y0 + 1 + k * G::kSR, (int)box_y_max);  // rows past the raster: never stored
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[buf], G::kStageBytes);
            tma_load_2d(stage(buf), &map_stage, o.x0 - 4, yb, &bar[buf]);
        }
    };

    int64_t cur = claim_seg();
    if (cur >= nsegs) return;
    Origin co = origin(cur);
    issue_prime(co, 0);
    issue_stage(co, 0, 0);
    issue_stage(co, 1, 1);
    uint32_t sphase = 0, pphase = 0;
    int pb = 0;
    SRow A, B, C;
    SPair PAB, PBC, PCA;
    const int rows = (int)p.rows;
    const float k_fd = p.sk.k_fd;
    // the fast path's configuration: Horn rise/run slope, dirType 8, vector stores
    const bool plain = p.fd && p.fast_out && !p.sk.degrees && (!D8 || p.dir_type == 8);
    while (true) {
        const int64_t x0 = co.x0, y0 = co.y0;
        const int64_t gx0 = x0 + 4 * lane;
        const bool lane_int = plain && gx0 >= 1 && gx0 + 4 <= p.cols - 1;
        char* sp = SLOPE ? p.slope.base + y0 * p.slope.pitch + 4 * gx0 : nullptr;
        char* dp = D8 ? p.d8.base + y0 * p.d8.pitch + gx0 : nullptr;
        int64_t nxt = nsegs;
        Origin no = co;
        if (!warp_wait(&bar[2 + pb], (pphase >> pb) & 1u)) {
            if (lane == 0 && p.error_flag) atomicExch(p.error_flag, 1);
            return;
        }
        pphase ^= 1u << pb;
        s_load_row(prime(pb), lane, A, p.nd6f);
        s_load_row(prime(pb) + kBoxW, lane, B, p.nd6f);
        s_pair(A, B, PAB);
#pragma unroll 1
        for (int k = 0; k < G::kStages; k++) {
            const int buf = k & 1;
            if (!warp_wait(&bar[buf], (sphase >> buf) & 1u)) {
                if (lane == 0 && p.error_flag) atomicExch(p.error_flag, 1);
                return;
            }
            sphase ^= 1u << buf;
            const int64_t spp = SLOPE ? p.slope.pitch : 0, dpp = D8 ? p.d8.pitch : 0;
            uint32_t pend = 0;
            const int ys = (int)y0 + k * G::kSR;
            const bool inside = (ys >= 1) & (ys + G::kSR - 1 <= rows - 2);
            // one vote: the stage's values and the two rows above it
            if (__any_sync(0xffffffffu, stage_lane_maybe_nodata<SR>(stage(buf), p.nd6f) | A.nd | B.nd) | !inside) {
#pragma unroll 1
                for (int t = 0; t < G::kSR; t += 3) {
                    const float* st = stage(buf) + t * kBoxW;
                    const int y = ys + t;
                    strip_step<SLOPE, D8, false>(st, A, B, C, PAB, PBC, y, rows, gx0, lane_int, k_fd, p.nd6f, sp, dp,
                                                pend, p.cols);
                    strip_step<SLOPE, D8, false>(st + kBoxW, B, C, A, PBC, PCA, y + 1, rows, gx0, lane_int, k_fd,
                                                p.nd6f, sp + spp, dp + dpp, pend, p.cols);
                    strip_step<SLOPE, D8, false>(st + 2 * kBoxW, C, A, B, PCA, PAB, y + 2, rows, gx0, lane_int, k_fd,
                                                p.nd6f, sp + 2 * spp, dp + 2 * dpp, pend, p.cols);
                    sp += 3 * spp;
                    dp += 3 * dpp;
                }
            } else {  // inside the ring, no nodata in any row it reads: the rows skip the tests
#pragma unroll 1
                for (int t = 0; t < G::kSR; t += 3) {
                    const float* st = stage(buf) + t * kBoxW;
                    const int y = ys + t;
                    strip_step<SLOPE, D8, true>(st, A, B, C, PAB, PBC, y, rows, gx0, lane_int, k_fd, p.nd6f, sp, dp,
                                                 pend, p.cols);
                    strip_step<SLOPE, D8, true>(st + kBoxW, B, C, A, PBC, PCA, y + 1, rows, gx0, lane_int, k_fd,
                                                 p.nd6f, sp + spp, dp + dpp, pend, p.cols);
                    strip_step<SLOPE, D8, true>(st + 2 * kBoxW, C, A, B, PCA, PAB, y + 2, rows, gx0, lane_int, k_fd,
                                                 p.nd6f, sp + 2 * spp, dp + 2 * dpp, pend, p.cols);
                    sp += 3 * spp;
                    dp += 3 * dpp;
                }
            }
            if (pend) strip_flush(pend, ys + G::kSR - 1, gx0, slow);
            __syncwarp();
            // refill this buffer with the item two ahead
            if (k + 2 < G::kStages) {
                issue_stage(co, k + 2, buf);
            } else {
                if (k + 2 == G::kStages) {
                    nxt = claim_seg();
                    if (nxt < nsegs) {
                        no = origin(nxt);
                        issue_prime(no, pb ^ 1);
                    }
                }
                if (nxt < nsegs) issue_stage(no, k + 2 - G::kStages, buf);
            }
        }
        if (nxt >= nsegs) break;
        cur = nxt;
        co = no;
        pb ^= 1;
    }
}

// Batched strip walk: one persistent launch walks the segments of many
// rasters.  Segments are numbered raster by raster (seg_start), claimed from
// a device counter, and each carries its raster's tensor maps (maps[2k]: the
// stage box, maps[2k+1]: the priming box) and parameters; the rows the fast
// path leaves go to one list of 64-bit items (raster << 40 | row * lanes +
// lane) for batch_strip_fixup_kernel.
struct BatchStripTables {
    const CUtensorMap* maps;
    const FocalParams* params;
    const InView* dems;
    const int64_t* seg_start;  // count + 1
    const int* nstrips;
    const uint64_t* order;     // queue position -> raster << 40 | segment of the raster; null: raster by raster
    int count;
    int64_t nsegs;
    unsigned long long* claim;
    unsigned long long* slow_count;
    uint64_t* slow_items;
    int* error_flag;
};

__device__ __noinline__ void batch_strip_flush(uint32_t pend, int y_last, int64_t gx0, int item, int64_t cols,
                                               const BatchStripTables t) {
    const int64_t lanes = (cols + 3) / 4;
    if ((gx0 >> 2) >= lanes) return;  // past the raster's last column
    unsigned long long base = atomicAdd(t.slow_count, (unsigned long long)__popc(pend));
    while (pend) {
        const int b = __ffs(pend) - 1;
        pend &= pend - 1;
        t.slow_items[base++] = ((uint64_t)item << 40) | (uint64_t)((int64_t)(y_last - b) * lanes + (gx0 >> 2));
    }
}

template <bool SLOPE, bool D8>
__global__ void __launch_bounds__(kSWarps * 32, 5) batch_strip_kernel(const BatchStripTables t) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[kSWarps][4];  // stage 0, stage 1, prime 0, prime 1
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem + warp * kSWarpBytes;
    auto stage = [&](int b) { return reinterpret_cast<float*>(wbase + b * kSStageStride); };
    auto prime = [&](int b) { return reinterpret_cast<float*>(wbase + 2 * kSStageStride + b * kSPrimeStride); };
    uint64_t* bar = bars[warp];
    if (lane == 0) {
        for (int i = 0; i < 4; i++) mbar_init(&bar[i], 1);
        mbar_fence_init();
    }
    __syncwarp();
    auto claim_seg = [&]() -> int64_t {
        unsigned long long v = 0;
        if (lane == 0) v = atomicAdd(t.claim, 1ULL);
        return (int64_t)__shfl_sync(0xffffffffu, v, 0);
    };
    struct Origin {
        int x0, y0, item, rows;
    };
    auto origin = [&](int64_t g) {
        int lo = 0;
        uint32_t local;
        if (t.order) {  // the queue ordered by the segments' compute intensity
            const uint64_t v = t.order[g];
            lo = (int)(v >> 40);
            local = (uint32_t)(v & ((1ULL << 40) - 1));
        } else {
            int hi = t.count - 1;  // the last raster whose first segment is <= g
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (t.seg_start[mid] <= g) lo = mid; else hi = mid - 1;
            }
            local = (uint32_t)(g - t.seg_start[lo]);
        }
        const uint32_t ns = (uint32_t)t.nstrips[lo];
        return Origin{(int)((local % ns) * kTW), (int)((local / ns) * kSegRows), lo, (int)t.params[lo].rows};
    };
    auto issue_prime = [&](const Origin& o, int buf) {
        if (lane == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[2 + buf], kSPrimeBytes);
            tma_load_2d(prime(buf), &t.maps[2 * o.item + 1], o.x0 - 4, o.y0 - 1, &bar[2 + buf]);
        }
    };
    auto issue_stage = [&](const Origin& o, int k, int buf) {
        if (lane == 0) {
            const int yb = min(o.y0 + 1 + k * kSR, o.rows - 1);  // rows past the raster: never stored
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bar[buf], kSStageBytes);
            tma_load_2d(stage(buf), &t.maps[2 * o.item], o.x0 - 4, yb, &bar[buf]);
        }
    };

    int64_t cur = claim_seg();
    if (cur >= t.nsegs) return;
    Origin co = origin(cur);
    issue_prime(co, 0);
    issue_stage(co, 0, 0);
    issue_stage(co, 1, 1);
    uint32_t sphase = 0, pphase = 0;
    int pb = 0;
    SRow A, B, C;
    SPair PAB, PBC, PCA;
    while (true) {
        const FocalParams& p = t.params[co.item];
        const int rows = co.rows;
        const int64_t cols = p.cols;
        const float k_fd = p.sk.k_fd;
        const Band<float> nd6 = p.nd6f;
        const bool plain = p.fd && p.fast_out && !p.sk.degrees && (!D8 || p.dir_type == 8);
        const int64_t x0 = co.x0, y0 = co.y0;
        const int64_t gx0 = x0 + 4 * lane;
        const bool lane_int = plain && gx0 >= 1 && gx0 + 4 <= cols - 1;
        const int64_t spp = SLOPE ? p.slope.pitch : 0, dpp = D8 ? p.d8.pitch : 0;
        char* sp = SLOPE ? p.slope.base + y0 * spp + 4 * gx0 : nullptr;
        char* dp = D8 ? p.d8.base + y0 * dpp + gx0 : nullptr;
        int64_t nxt = t.nsegs;
        Origin no = co;
        if (!warp_wait(&bar[2 + pb], (pphase >> pb) & 1u)) {
            if (lane == 0 && t.error_flag) atomicExch(t.error_flag, 1);
            return;
        }
        pphase ^= 1u << pb;
        s_load_row(prime(pb), lane, A, nd6);
        s_load_row(prime(pb) + kBoxW, lane, B, nd6);
        s_pair(A, B, PAB);
#pragma unroll 1
        for (int k = 0; k < kSegStages; k++) {
            const int buf = k & 1;
            if (!warp_wait(&bar[buf], (sphase >> buf) & 1u)) {
                if (lane == 0 && t.error_flag) atomicExch(t.error_flag, 1);
                return;
            }
            sphase ^= 1u << buf;
            uint32_t pend = 0;
            const int ys = (int)y0 + k * kSR;
            const bool inside = (ys >= 1) & (ys + kSR - 1 <= rows - 2);
            if (__any_sync(0xffffffffu, stage_lane_maybe_nodata(stage(buf), nd6) | A.nd | B.nd) | !inside) {
#pragma unroll 1
                for (int tt = 0; tt < kSR; tt += 3) {
                    const float* st = stage(buf) + tt * kBoxW;
                    const int y = ys + tt;
                    strip_step<SLOPE, D8, false>(st, A, B, C, PAB, PBC, y, rows, gx0, lane_int, k_fd, nd6, sp, dp,
                                                pend, cols);
                    strip_step<SLOPE, D8, false>(st + kBoxW, B, C, A, PBC, PCA, y + 1, rows, gx0, lane_int, k_fd, nd6,
                                                sp + spp, dp + dpp, pend, cols);
                    strip_step<SLOPE, D8, false>(st + 2 * kBoxW, C, A, B, PCA, PAB, y + 2, rows, gx0, lane_int, k_fd,
                                                nd6, sp + 2 * spp, dp + 2 * dpp, pend, cols);
                    sp += 3 * spp;
                    dp += 3 * dpp;
                }
            } else {
#pragma unroll 1
                for (int tt = 0; tt < kSR; tt += 3) {
                    const float* st = stage(buf) + tt * kBoxW;
                    const int y = ys + tt;
                    strip_step<SLOPE, D8, true>(st, A, B, C, PAB, PBC, y, rows, gx0, lane_int, k_fd, nd6, sp, dp,
                                                pend, cols);
                    strip_step<SLOPE, D8, true>(st + kBoxW, B, C, A, PBC, PCA, y + 1, rows, gx0, lane_int, k_fd, nd6,
                                                sp + spp, dp + dpp, pend, cols);
                    strip_step<SLOPE, D8, true>(st + 2 * kBoxW, C, A, B, PCA, PAB, y + 2, rows, gx0, lane_int, k_fd,
                                                nd6, sp + 2 * spp, dp + 2 * dpp, pend, cols);
                    sp += 3 * spp;
                    dp += 3 * dpp;
                }
            }
            if (pend) batch_strip_flush(pend, ys + kSR - 1, gx0, co.item, cols, t);
            __syncwarp();
            if (k + 2 < kSegStages) {
                issue_stage(co, k + 2, buf);
            } else {
                if (k + 2 == kSegStages) {
                    nxt = claim_seg();
                    if (nxt < t.nsegs) {
                        no = origin(nxt);
                        issue_prime(no, pb ^ 1);
                    }
                }
                if (nxt < t.nsegs) issue_stage(no, k + 2 - kSegStages, buf);
            }
        }
        if (nxt >= t.nsegs) break;
        cur = nxt;
        co = no;
        pb ^= 1;
    }
}

__global__ void __launch_bounds__(128) batch_strip_fixup_kernel(const BatchStripTables t,
                                                                unsigned long long* fallbacks) {
    const unsigned long long n = *((volatile unsigned long long*)t.slow_count) * 4;  // one thread per cell
    int fell_back = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t e = t.slow_items[i >> 2];
        const int item = (int)(e >> 40);
        const uint64_t local = e & ((1ULL << 40) - 1);
        const FocalParams& p = t.params[item];
        const InView& dem = t.dems[item];
        const uint64_t lanes = (uint64_t)((p.cols + 3) / 4);
        const int64_t y = (int64_t)(local / lanes), gx = (int64_t)(local % lanes) * 4 + (int64_t)(i & 3);
        if (gx >= p.cols) continue;
        const bool ring = y <= 0 || gx <= 0 || y >= p.rows - 1 || gx >= p.cols - 1;
        float z[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (!ring) {
#pragma unroll
            for (int q = 0; q < 9; q++)
                z[q] = reinterpret_cast<const float*>(dem.base + (y + q / 3 - 1) * dem.pitch)[gx + q % 3 - 1];
        }
        const CellOut o = cell_general<float>(z[0], z[1], z[2], z[3], z[4], z[5], z[6], z[7], z[8], &p, ring);
        fell_back += (o.flags >> 2) & 1;
        if (p.do_slope) {
            if (o.flags & 1) put_value(p.slope, y, gx, p.slope.nodata);
            else put_float(p.slope, y, gx, o.slope);
        }
        if (p.do_d8) {
            if (o.flags & 2) put_value(p.d8, y, gx, p.d8.nodata);
            else put_int(p.d8, y, gx, o.code);
        }
    }
    count_fallbacks(fell_back, fallbacks);
}

// The (row, lane) items the strip walk left: their cells, one thread each,
// through cell_general on the window read from the DEM.
__global__ void __launch_bounds__(128) strip_fixup_kernel(const InView dem, const __grid_constant__ FocalParams p,
                                                          const SlowList slow) {
    const unsigned long long n = *((volatile unsigned long long*)slow.count) * 4;  // one thread per cell
    int fell_back = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t e = slow.items[i >> 2];
        const int64_t y = (int64_t)(e / (uint64_t)slow.lanes_per_row);
        const int64_t gx0 = (int64_t)(e % (uint64_t)slow.lanes_per_row) * 4;
        {
            const int64_t gx = gx0 + (int64_t)(i & 3);
            if (gx >= p.cols) continue;
            const bool ring = y <= 0 || gx <= 0 || y >= p.rows - 1 || gx >= p.cols - 1;
            float z[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (!ring) {
#pragma unroll
                for (int q = 0; q < 9; q++)
                    z[q] = reinterpret_cast<const float*>(dem.base + (y + q / 3 - 1) * dem.pitch)[gx + q % 3 - 1];
            }
            const CellOut o = cell_general<float>(z[0], z[1], z[2], z[3], z[4], z[5], z[6], z[7], z[8], &p, ring);
            fell_back += (o.flags >> 2) & 1;
            if (p.do_slope) {
                if (o.flags & 1) put_value(p.slope, y, gx, p.slope.nodata);
                else put_float(p.slope, y, gx, o.slope);
            }
            if (p.do_d8) {
                if (o.flags & 2) put_value(p.d8, y, gx, p.d8.nodata);
                else put_int(p.d8, y, gx, o.code);
            }
        }
    }
    count_fallbacks(fell_back, p.fallbacks);
}

}  // namespace

// Kernel variants the autotuner searches.  Tiled kernel: tile rows (4 x
// ROWS; each thread computes ROWS rows of 4 cells, 4 x ROWS cells) and CTAs
// per SM.  Strip walk: rows per TMA stage, stages per segment (the segment
// height is their product) and CTAs per SM; the strip width is the warp's 32
// lanes x 4 cells (one float4 per lane and row).  Every variant computes the
// same bytes.  A variant is named for its parameters; the names key the
// persisted tuning cache, so a rebuilt table still resolves a cached choice.
struct Variant {
    char kind;       // 't' tiled, 's' strip walk
    int rows, stages, minb;
    const char* name;
};
static const Variant kVariants[] = {
    {'t', 8, 0, 5, "tile-r32-b5"},     {'t', 6, 0, 6, "tile-r24-b6"},     {'t', 6, 0, 7, "tile-r24-b7"},
    {'t', 4, 0, 8, "tile-r16-b8"},     {'t', 8, 0, 6, "tile-r32-b6"},     {'s', 6, 8, 5, "strip-s6x8-b5"},
    {'s', 6, 8, 6, "strip-s6x8-b6"},   {'s', 3, 16, 5, "strip-s3x16-b5"}, {'s', 6, 4, 5, "strip-s6x4-b5"},
    {'s', 6, 16, 5, "strip-s6x16-b5"}, {'s', 9, 6, 5, "strip-s9x6-b5"},   {'s', 12, 4, 4, "strip-s12x4-b4"},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
constexpr int kNumTiled = 5;          // variants 0 .. 4 are tiled
constexpr int kDefaultStrip = 5;      // strip-s6x8-b5

int focal_num_variants() { return kNumVariants; }
int focal_default_strip_variant() { return kDefaultStrip; }
bool focal_variant_is_strip(int v) { return v >= kNumTiled && v < kNumVariants; }
int focal_variant_rows(int v) { return kWarps * kVariants[(v >= 0 && v < kNumTiled) ? v : 0].rows; }
const char* focal_variant_name(int v) { return (v >= 0 && v < kNumVariants) ? kVariants[v].name : nullptr; }
// Stage rows of strip variant v for these outputs: the stage geometries other
// than the default are built for the fused slope + D8 (the tuned operation);
// single-output calls run them at the default geometry.
int focal_strip_stage_rows(int v, int do_slope, int do_d8) {
    if (!focal_variant_is_strip(v) || !(do_slope && do_d8)) return kSR;
    return kVariants[v].rows;
}
size_t focal_tma_smem_bytes() { return 2 * Shape<kBatchRows>::kStageStride; }
int focal_tma_tile_rows() { return Shape<kBatchRows>::kTH; }
int focal_tma_tile_cols() { return kTW; }
int focal_tma_box_cols() { return kBoxW; }
int focal_tma_box_rows() { return Shape<kBatchRows>::kBoxH; }

template <int ROWS, int UNROLL, int MINB, bool SLOPE, bool D8>
static cudaError_t launch_variant(const CUtensorMap* map, const FocalParams& p, int num_sms, cudaStream_t s) {
    using S = Shape<ROWS>;
    const int64_t ntx = (p.cols + kTW - 1) / kTW, nty = (p.rows + S::kTH - 1) / S::kTH;
    const int64_t ntiles = ntx * nty;
    if (ntiles == 0) return cudaSuccess;
    const size_t smem = 2 * S::kStageStride;
    auto kern = focal_tma_kernel<ROWS, UNROLL, MINB, SLOPE, D8>;
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

template <bool SLOPE, bool D8>
static cudaError_t launch_variants(const CUtensorMap* map, const FocalParams& p, int variant, int num_sms,
                                   cudaStream_t s) {
    switch (variant) {
        case 1: return launch_variant<6, 1, 6, SLOPE, D8>(map, p, num_sms, s);
        case 2: return launch_variant<6, 1, 7, SLOPE, D8>(map, p, num_sms, s);
        case 3: return launch_variant<4, 1, 8, SLOPE, D8>(map, p, num_sms, s);
        case 4: return launch_variant<8, 1, 6, SLOPE, D8>(map, p, num_sms, s);
        default: return launch_variant<8, 1, 5, SLOPE, D8>(map, p, num_sms, s);
    }
}

template <bool SLOPE, bool D8, int MINB, int SR = kSR, int STAGES = kSegStages>
static cudaError_t launch_strip(const CUtensorMap* map_stage, const CUtensorMap* map_prime, const InView& dem,
                                const FocalParams& p, unsigned long long* counters, uint32_t* slow_items, int num_sms,
                                cudaStream_t s) {
    using G = StripGeom<SR, STAGES>;
    const int64_t nstrips = (p.cols + kTW - 1) / kTW, nbands = (p.rows + G::kSegRows - 1) / G::kSegRows;
    const int64_t nsegs = nstrips * nbands;
    if (nsegs == 0) return cudaSuccess;
    const size_t smem = (size_t)kSWarps * G::kWarpBytes;
    auto kern = focal_strip_kernel<SLOPE, D8, MINB, SR, STAGES>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSWarps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    const int64_t need = (nsegs + kSWarps - 1) / kSWarps;
    if (grid > need) grid = need;
    if ((e = cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), s)) != cudaSuccess) return e;
    const SlowList slow{slow_items, counters + 1, (p.cols + 3) / 4};
    kern<<<(unsigned)grid, kSWarps * 32, smem, s>>>(*map_stage, *map_prime, p, nstrips, nsegs, counters, slow);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    strip_fixup_kernel<<<(unsigned)num_sms * 8, 128, 0, s>>>(dem, p, slow);
    return cudaGetLastError();
}

size_t focal_strip_slow_bytes(int64_t rows, int64_t cols) { return (size_t)(rows * ((cols + 3) / 4)) * 4; }

// Strip-walk form: `map_stage` has a (kBoxW, focal_strip_stage_rows(variant,
// ...)) box and
// `map_prime` a (kBoxW, 2) box over the same float32 DEM `dem`; `counters`
// points to two device counters (segment claims, slow items) and
// `slow_items` to focal_strip_slow_bytes() of scratch.
template <int MINB>
static cudaError_t launch_strip_minb(const CUtensorMap* map_stage, const CUtensorMap* map_prime, const InView& dem,
                                     const FocalParams& q, unsigned long long* counters, uint32_t* slow_items,
                                     int num_sms, cudaStream_t s) {
    if (q.do_slope && q.do_d8)
        return launch_strip<true, true, MINB>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
    if (q.do_slope)
        return launch_strip<true, false, MINB>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
    if (q.do_d8)
        return launch_strip<false, true, MINB>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
    return cudaSuccess;
}

cudaError_t launch_focal_strip(const CUtensorMap* map_stage, const CUtensorMap* map_prime, const InView& dem,
                               const FocalParams& p, int fast_out, int variant, unsigned long long* counters,
                               uint32_t* slow_items, int num_sms, cudaStream_t s) {
    FocalParams q = p;
    q.fast_out = fast_out;
    q.fd = p.sk.method == PARGO_SLOPE_FD || !p.do_slope;
    if (q.do_slope && q.do_d8) {
        switch (variant) {  // the stage geometries (map_stage's box: focal_strip_stage_rows())
            case 7: return launch_strip<true, true, 5, 3, 16>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
            case 8: return launch_strip<true, true, 5, 6, 4>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
            case 9: return launch_strip<true, true, 5, 6, 16>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
            case 10: return launch_strip<true, true, 5, 9, 6>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
            case 11: return launch_strip<true, true, 4, 12, 4>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
            default: break;
        }
    }
    if (variant == 6) return launch_strip_minb<6>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
    return launch_strip_minb<5>(map_stage, map_prime, dem, q, counters, slow_items, num_sms, s);
}

// The tensor map's box must be (kBoxW, focal_variant_rows(variant) + 2).
cudaError_t launch_focal_tma(const CUtensorMap* map, const FocalParams& p, int fast_out, int variant, int num_sms,
                             cudaStream_t s) {
    FocalParams q = p;
    q.fast_out = fast_out;
    q.fd = p.sk.method == PARGO_SLOPE_FD || !p.do_slope;
    if (q.do_slope && q.do_d8) return launch_variants<true, true>(map, q, variant, num_sms, s);
    if (q.do_slope) return launch_variants<true, false>(map, q, variant, num_sms, s);
    if (q.do_d8) return launch_variants<false, true>(map, q, variant, num_sms, s);
    return cudaSuccess;
}

cudaError_t launch_batch_tma(const CUtensorMap* maps, const FocalParams* params, const int64_t* tile_start,
                             const int64_t* ntx_of, int count, int64_t total_tiles, int do_slope, int do_d8,
                             unsigned long long* claim, unsigned long long* fallbacks, int* error_flag, int num_sms,
                             cudaStream_t s) {
    if (total_tiles == 0) return cudaSuccess;
    const size_t smem = focal_tma_smem_bytes();
    auto kern = do_slope ? (do_d8 ? batch_tma_kernel<true, true> : batch_tma_kernel<true, false>)
                         : batch_tma_kernel<false, true>;
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

// Compute intensity of the batch's strip segments (a kTW-column strip by
// kSegRows rows of one raster): the intensity-ratio estimate of the load
// estimator (gpro/transformation.h:155-197: valid_load per cell whose
// |v - nodata| > Eps, nodata_load per other cell), here counted per segment.
// One warp per segment, 4 columns per lane; out[g] = the valid cells of
// segment g (the host turns counts into loads and orders the queue).
__global__ void __launch_bounds__(256) batch_segment_valid_kernel(const SegLoadRaster* rs, int count, int64_t nsegs,
                                                                  uint32_t* out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t g = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); g < nsegs; g += warps) {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (rs[mid].seg_start <= g) lo = mid; else hi = mid - 1;
        }
        const SegLoadRaster r = rs[lo];
        const int64_t local = g - r.seg_start;
        const int64_t x0 = (local % r.nstrips) * kTW, y0 = (local / r.nstrips) * kSegRows;
        const int64_t y1 = min(y0 + kSegRows, r.rows);
        const int64_t xa = x0 + 4 * lane;
        uint32_t valid = 0;
        for (int64_t y = y0; y < y1; y++) {
            const float* row = reinterpret_cast<const float*>(r.dem.base + y * r.dem.pitch);
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (xa + j < r.cols) valid += r.nd.has(row[xa + j]) ? 0u : 1u;
        }
        valid = __reduce_add_sync(0xffffffffu, valid);
        if (lane == 0) out[g] = valid;
    }
}

cudaError_t launch_batch_segment_valid(const SegLoadRaster* rs, int count, int64_t nsegs, uint32_t* out, int num_sms,
                                       cudaStream_t s) {
    if (nsegs == 0) return cudaSuccess;
    int64_t blocks = (nsegs + 7) / 8;
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    batch_segment_valid_kernel<<<(unsigned)blocks, 256, 0, s>>>(rs, count, nsegs, out);
    return cudaGetLastError();
}

int batch_strip_segment_rows() { return kSegRows; }
int batch_strip_segment_cols() { return kTW; }

// Batched strip walk over `count` rasters: maps[2k] / maps[2k+1] are raster
// k's stage (kBoxW x focal_strip_stage_rows()) and priming (kBoxW x 2) tensor
// maps; seg_start[k] its first segment (batch_strip_segments() per raster);
// counters[0..1] the claim and slow-item counters; slow_items room for one
// 64-bit item per (row, 4-cell lane) of every raster.
int64_t batch_strip_segments(int64_t rows, int64_t cols, int* nstrips) {
    *nstrips = (int)((cols + kTW - 1) / kTW);
    return (int64_t)*nstrips * ((rows + kSegRows - 1) / kSegRows);
}

cudaError_t launch_batch_strip(const CUtensorMap* maps, const FocalParams* params, const InView* dems,
                               const int64_t* seg_start, const int* nstrips, const uint64_t* order, int count,
                               int64_t nsegs, int do_slope, int do_d8, unsigned long long* counters,
                               uint64_t* slow_items, unsigned long long* fallbacks, int* error_flag, int num_sms,
                               cudaStream_t s) {
    if (nsegs == 0) return cudaSuccess;
    const BatchStripTables t{maps, params, dems, seg_start, nstrips, order, count, nsegs, counters, counters + 1,
                             slow_items, error_flag};
    const size_t smem = (size_t)kSWarps * kSWarpBytes;
    auto kern = do_slope ? (do_d8 ? batch_strip_kernel<true, true> : batch_strip_kernel<true, false>)
                         : batch_strip_kernel<false, true>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSWarps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    const int64_t need = (nsegs + kSWarps - 1) / kSWarps;
    if (grid > need) grid = need;
    if ((e = cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), s)) != cudaSuccess) return e;
    kern<<<(unsigned)grid, kSWarps * 32, smem, s>>>(t);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    batch_strip_fixup_kernel<<<(unsigned)num_sms * 8, 128, 0, s>>>(t, fallbacks);
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
