// common.cuh -- shared device/host definitions of the focal raster kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pargo_gpu.h"

#define PARGO_HD __host__ __device__ __forceinline__

namespace pargo {

// Eps literals of the reference operators.
constexpr double kEpsSlope = 0.0000001;  // apps/morphology/slope/slopeOperator.h:13
constexpr double kEpsHydro = 0.000001;   // d8Operator.cpp:3, pitRemoveOperator.h:13, scaOperator.cpp:3

// Output view: base pointer, pitch, dtype, the nodata value it writes.
struct OutView {
    char* base;
    int64_t pitch;
    int32_t dtype;
    double nodata;
};

// Input view (read-only).
struct InView {
    const char* base;
    int64_t pitch;
    int32_t dtype;
};

PARGO_HD int elem_size(int dtype) {
    switch (dtype) {
        case PARGO_F32: return 4;
        case PARGO_F64: return 8;
        case PARGO_I8: return 1;
        case PARGO_I16: return 2;
        case PARGO_I32: return 4;
        default: return 0;
    }
}

__device__ __forceinline__ void put_value(const OutView& o, int64_t r, int64_t c, double v) {
    char* p = o.base + r * o.pitch;
    switch (o.dtype) {
        case PARGO_F32: reinterpret_cast<float*>(p)[c] = (float)v; break;
        case PARGO_F64: reinterpret_cast<double*>(p)[c] = v; break;
        case PARGO_I8: reinterpret_cast<int8_t*>(p)[c] = (int8_t)v; break;
        case PARGO_I16: reinterpret_cast<int16_t*>(p)[c] = (int16_t)v; break;
        case PARGO_I32: reinterpret_cast<int32_t*>(p)[c] = (int32_t)v; break;
        default: break;
    }
}

// Typed stores that keep float and integer values off the FP64 pipe (a
// conversion through double costs an FP64 instruction on each side).
__device__ __forceinline__ void put_float(const OutView& o, int64_t r, int64_t c, float v) {
    char* p = o.base + r * o.pitch;
    if (o.dtype == PARGO_F32) reinterpret_cast<float*>(p)[c] = v;
    else put_value(o, r, c, (double)v);
}
__device__ __forceinline__ void put_int(const OutView& o, int64_t r, int64_t c, int v) {
    char* p = o.base + r * o.pitch;
    switch (o.dtype) {
        case PARGO_I8: reinterpret_cast<int8_t*>(p)[c] = (int8_t)v; break;
        case PARGO_I16: reinterpret_cast<int16_t*>(p)[c] = (int16_t)v; break;
        case PARGO_I32: reinterpret_cast<int32_t*>(p)[c] = v; break;
        case PARGO_F32: reinterpret_cast<float*>(p)[c] = (float)v; break;
        default: put_value(o, r, c, (double)v); break;
    }
}

// Double -> float, round to nearest even, on the integer pipes for results
// in the normal float range (else the hardware conversion).
__device__ __forceinline__ float dbl2flt_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if (e < 1 || e > 253) return __double2float_rn(x);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFULL;
    const unsigned long long rem = m & 0x1FFFFFFFULL;  // the 29 dropped bits
    unsigned int f = (unsigned int)(b >> 63) << 31 | (unsigned int)e << 23 | (unsigned int)(m >> 29);
    f += (rem > 0x10000000ULL || (rem == 0x10000000ULL && (f & 1u))) ? 1u : 0u;  // a carry moves into the exponent
    return __uint_as_float(f);
}

// Order-preserving integer keys: a double's, and a float's as the same
// double's (exact: every float is a double), without a conversion.
__device__ __forceinline__ long long dkey64(double v) {
    const long long b = __double_as_longlong(v);
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ long long fkey64(float f) {
    const unsigned int u = __float_as_uint(f);
    const unsigned int ef = (u >> 23) & 0xFF;
    long long b;
    if (ef == 0 || ef == 0xFF) {
        b = __double_as_longlong((double)f);  // zero, subnormal, inf, NaN: the hardware conversion
    } else {
        b = (long long)(u >> 31) << 63 | (long long)(ef - 127 + 1023) << 52 | (long long)(u & 0x7FFFFF) << 29;
    }
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}

// The set { x : |x - nodata| < eps } as a closed interval of the input type.
// |(double)x - nodata| is monotone in x, so the set is an interval; the host
// finds its exact float/double end points (see host_nodata_band in abi.cu).
template <typename T>
struct Band {
    T lo, hi;
    PARGO_HD bool has(T v) const { return v >= lo && v <= hi; }
};

// Slope method constants (float, computed on the host from the float-rounded
// cell size the reference uses).
struct SlopeConsts {
    float k_fd;     // 1 / (8 cs)
    float k_ffd;    // 1 / (4 cs)
    float k_sd;     // 1 / cs
    float k_sfd;    // 1 / (2 cs)
    float k_tfd;    // 1 / (6 cs)
    float k_tfdw;   // 1 / ((4 + sqrt 8) cs)
    float sqrt2;    // sqrt(2) as float
    double sqrt2d;  // sqrt(2) as double
    float k_md;     // 1 / (cs * sqrt 2): MD divides by the last-visited (SE) distance
    int method;
    int degrees;
};

// ---------------------------------------------------------------- slope --
// z[0..8] = row-major 3x3 window.  Differences of neighbouring elevations are
// formed first -- exactly for nearby float elevations (Sterbenz), and in FP64
// for double input -- then combined in FP32, which keeps ~1e-7 relative
// accuracy against the reference's FP64 result.
__device__ __forceinline__ float zdiff(const float* z, int i, int j) { return z[i] - z[j]; }
__device__ __forceinline__ float zdiff(const double* z, int i, int j) { return (float)__dsub_rn(z[i], z[j]); }

// Numerators of each method in the input's precision: float input keeps
// them exact (sums of exact neighbour differences of nearby float elevations
// fit in 24 bits); double input (pit-removed levels, differences of order the
// gap) combines in FP64 so nothing cancels in float.
template <typename T>
__device__ __forceinline__ void slope_numerators(const T* z, int method, T& nx, T& ny) {
    switch (method) {
        case PARGO_SLOPE_FD:  // slopeOperator.cpp:84-86
            if constexpr (sizeof(T) == 4) {  // same rounding as the tiled kernel's shared differences
                nx = __fmaf_rn(2.0f, __fsub_rn(z[5], z[3]), __fadd_rn(__fsub_rn(z[2], z[0]), __fsub_rn(z[8], z[6])));
                ny = __fmaf_rn(2.0f, __fsub_rn(z[1], z[7]), __fadd_rn(__fsub_rn(z[0], z[6]), __fsub_rn(z[2], z[8])));
            } else {
                nx = ((z[2] - z[0]) + (z[8] - z[6])) + (T)2 * (z[5] - z[3]);
                ny = ((z[0] - z[6]) + (z[2] - z[8])) + (T)2 * (z[1] - z[7]);
            }
            break;
        case PARGO_SLOPE_FFD:  // :88-90
            nx = (z[8] - z[6]) + (z[2] - z[0]);
            ny = (z[0] - z[6]) + (z[2] - z[8]);
            break;
        case PARGO_SLOPE_MD: {  // :92-103 (max drop; divided by the last-visited SE distance below)
            T m = 0;
#pragma unroll
            for (int i = 0; i < 9; i++)
                if (i != 4 && z[4] - z[i] > m) m = z[4] - z[i];
            nx = m;
            ny = 0;
            break;
        }
        case PARGO_SLOPE_SD:  // :122-124
            nx = z[4] - z[3];
            ny = z[4] - z[7];
            break;
        case PARGO_SLOPE_SFD:  // :126-128
            nx = z[5] - z[3];
            ny = z[1] - z[7];
            break;
        case PARGO_SLOPE_TFD:  // :130-132; dy uses z[6] twice, as the reference does
            nx = (z[8] - z[0]) + (z[5] - z[3]) + (z[2] - z[6]);
            ny = (z[2] - z[6]) + (z[1] - z[7]) + (z[0] - z[6]);
            break;
        default:  // TFDW :134-136: sqrt(2) multiplies differences, not raw levels
            nx = (z[8] - z[6]) + (z[2] - z[0]);
            ny = (z[2] - z[6]) + (z[0] - z[8]);
            break;
    }
}

// Square root by the SFU's approximate instruction (relative error ~2^-23,
// far inside the 1e-5 slope tolerance); 0 stays 0.
__device__ __forceinline__ float sqrt_sfu(float q) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(q));
    return r;
}

// Horn slope from its two numerators: k sqrt(nx^2 + ny^2), with the rounding
// pinned (explicit fma / mul) so every kernel produces the same bits.
__device__ __forceinline__ float horn_slope(float nx, float ny, float k) {
    return __fmul_rn(sqrt_sfu(__fmaf_rn(nx, nx, __fmul_rn(ny, ny))), k);
}

template <typename T>
__device__ __forceinline__ float slope_from_window(const T* z, const SlopeConsts& k) {
    T nx, ny;
    slope_numerators(z, k.method, nx, ny);
    float s;
    switch (k.method) {
        case PARGO_SLOPE_FD:
            s = horn_slope((float)nx, (float)ny, k.k_fd);
            break;
        case PARGO_SLOPE_MD:
            s = (float)nx * k.k_md;
            break;
        case PARGO_SLOPE_TFDW: {
            const T s2 = (T)k.sqrt2d;
            const float fx = (float)(nx + s2 * (z[5] - z[3])) * k.k_tfdw;
            const float fy = (float)(ny + s2 * (z[1] - z[7])) * k.k_tfdw;
            s = sqrtf(fx * fx + fy * fy);
            break;
        }
        default: {
            const float kk = k.method == PARGO_SLOPE_FFD ? k.k_ffd
                           : k.method == PARGO_SLOPE_SD  ? k.k_sd
                           : k.method == PARGO_SLOPE_SFD ? k.k_sfd
                                                         : k.k_tfd;
            const float fx = (float)nx * kk, fy = (float)ny * kk;
            s = sqrtf(fx * fx + fy * fy);
            break;
        }
    }
    if (k.degrees) s = atanf(s) * 57.29577951308232f;
    return s;
}

// ------------------------------------------------------------------- D8 --
// Exact FP64 restatement of D8Operator::Operator (d8Operator.cpp:59-98) for
// one window, used when the FP32 decision below cannot be certified.
static __device__ __noinline__ int d8_exact(const double d[9], int dir_type) {
    const double s2 = __dsqrt_rn(2.0);
    double diff[9], mx = 0.0;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        diff[i] = __dsub_rn(d[4], d[i]);
        if (i == 0 || i == 2 || i == 6 || i == 8) diff[i] = __ddiv_rn(diff[i], s2);
        if (diff[i] > mx) mx = diff[i];
    }
    if (mx < kEpsHydro) return -1;
    unsigned mask = 0;
#pragma unroll
    for (int i = 0; i < 9; i++)
        if (fabs(__dsub_rn(diff[i], mx)) < kEpsHydro) mask |= 1u << i;
    if (dir_type == 8) {
        int n = __popc(mask) >> 1;
        for (int i = 0; i < 9; i++)
            if (mask & (1u << i)) {
                if (n == 0) return i;
                n--;
            }
        return -1;
    }
    return ((mask >> 5) & 1) * 1 + ((mask >> 8) & 1) * 2 + ((mask >> 7) & 1) * 4 + ((mask >> 6) & 1) * 8 +
           ((mask >> 3) & 1) * 16 + ((mask >> 0) & 1) * 32 + ((mask >> 1) & 1) * 64 + ((mask >> 2) & 1) * 128;
}

__device__ __forceinline__ int d8_code_from_mask(unsigned mask, int dir_type) {
    if (dir_type == 8) {
        int n = __popc(mask) >> 1;
        return __fns(mask, 0, n + 1);
    }
    return ((mask >> 5) & 1) * 1 + ((mask >> 8) & 1) * 2 + ((mask >> 7) & 1) * 4 + ((mask >> 6) & 1) * 8 +
           ((mask >> 3) & 1) * 16 + ((mask >> 0) & 1) * 32 + ((mask >> 1) & 1) * 64 + ((mask >> 2) & 1) * 128;
}

// Certified FP32 D8 decision, reproducing the reference's FP64 decisions.
//
// The reference (d8Operator.cpp:64-97) forms r_i = fl64(d4 - d_i), divides the
// diagonals by fl64(sqrt 2), takes M = max(0, r_i), returns -1 when M < 1e-6
// and otherwise the set T = { i : |r_i - M| < 1e-6 }.  Here
//   x_i = fl32(d4 - d_i), times fl32(1/sqrt 2) for diagonals,
// with |x_i - r_i| <= 2^-22 |x_i| (three float roundings of 2^-24 and the
// constant's; the double roundings are 2^-53).  Decisions are taken in FP32
// only where they are certain under those bounds:
//  * every x_i <= 0: all r_i <= 0 (rounding keeps signs), M = 0, code -1;
//  * M against 1e-6: |x_k - r_k| <= 2^-22 x_k for the argmax k;
//  * a clear single maximum (second largest further than 1e-6 plus both
//    error bounds below it): T = {k};
//  * otherwise the near ties are re-measured from direct differences (exact
//    for two cardinals or two diagonals, which is where exact ties occur) in
//    d8_certified_ties below.
// Anything still inside an error band returns kD8Unsure and the caller runs
// the exact FP64 restatement d8_exact.
constexpr int kD8Unsure = 0x7fff;
constexpr float kTLo = 0.99996948e-6f, kTHi = 1.0000305e-6f;  // 1e-6 widened by 2^-15 relative
constexpr float k2m22 = 2.384185791015625e-07f;                 // 2^-22
constexpr float k2m20 = 9.5367431640625e-07f;                   // 2^-20

PARGO_HD bool is_diag(int i) { return i == 0 || i == 2 || i == 6 || i == 8; }

__device__ __forceinline__ int d8_bit_code(int k) {
    // ArcGIS-style weight of window index k (d8Operator.cpp:96-97)
    const int w[9] = {32, 64, 128, 16, 0, 1, 8, 4, 2};
    return w[k];
}

// Near-tie resolution: k is the FP32 argmax (value m); T is built from
// g_i = r_k - r_i measured directly.  Same-type pairs: g = d_i - d_k (times
// 1/sqrt 2 for diagonals), error <= 2^-22 g + 2^-48 m (the reference's own
// roundings of r_i, r_k).  Mixed pairs: g = m - x_i, error <= 2^-21 (m + |x_i|).
template <typename T>
__device__ __noinline__ int d8_certified_ties(const T* z, const float* x, int k, float m, int dir_type) {
    const float kinv = 0.70710677f;
    const bool kd = is_diag(k);
    unsigned mask = 1u << k;
    for (int i = 0; i < 9; i++) {
        if (i == 4 || i == k) continue;
        float g, err;
        if (is_diag(i) == kd) {
            g = zdiff(z, i, k);
            if (kd) g *= kinv;
            err = fabsf(g) * k2m22 + m * 3.5527136788005009e-15f;  // 2^-48 m
            if (g < 0.0f || (g > 0.0f && g <= err)) return kD8Unsure;  // the reference max may be i
        } else {
            g = m - x[i];
            err = (m + fabsf(x[i])) * 4.76837158203125e-07f;  // 2^-21
            if (g <= err) return kD8Unsure;
        }
        if (g + err < kTLo) mask |= 1u << i;
        else if (!(g - err > kTHi)) return kD8Unsure;
    }
    return d8_code_from_mask(mask, dir_type);
}

template <typename T>
__device__ __forceinline__ int d8_certified(const T* z, int dir_type) {
    const float kinv = 0.70710677f;
    float x[9];
    float m = -3.0e38f, m2 = -3.0e38f;
    int k = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        if (i == 4) continue;
        const float c = zdiff(z, 4, i);
        x[i] = is_diag(i) ? c * kinv : c;
        if (x[i] > m) {
            m2 = m;
            m = x[i];
            k = i;
        } else {
            m2 = fmaxf(m2, x[i]);
        }
    }
    if (m <= 0.0f) return -1;
    const float em = m * k2m22;
    if (m + em < kTLo) return -1;
    if (!(m - em > kTHi)) return kD8Unsure;
    if (m - m2 > kTHi + (m + fabsf(m2)) * k2m20) return dir_type == 8 ? k : d8_bit_code(k);
    x[4] = 0.0f;
    return d8_certified_ties(z, x, k, m, dir_type);
}

}  // namespace pargo
