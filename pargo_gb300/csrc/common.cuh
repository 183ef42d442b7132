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

template <typename T>
__device__ __forceinline__ float slope_from_window(const T* z, const SlopeConsts& k) {
    float dx, dy, s;
    switch (k.method) {
        case PARGO_SLOPE_FD: {  // slopeOperator.cpp:84-86
            float nx = (zdiff(z, 2, 0) + zdiff(z, 8, 6)) + 2.0f * zdiff(z, 5, 3);
            float ny = (zdiff(z, 0, 6) + zdiff(z, 2, 8)) + 2.0f * zdiff(z, 1, 7);
            s = sqrtf(nx * nx + ny * ny) * k.k_fd;
            break;
        }
        case PARGO_SLOPE_FFD:  // :88-90
            dx = (zdiff(z, 8, 6) + zdiff(z, 2, 0)) * k.k_ffd;
            dy = (zdiff(z, 0, 6) + zdiff(z, 2, 8)) * k.k_ffd;
            s = sqrtf(dx * dx + dy * dy);
            break;
        case PARGO_SLOPE_MD: {  // :92-103, divided by the last-visited (SE) distance
            float m = 0.0f;
#pragma unroll
            for (int i = 0; i < 9; i++)
                if (i != 4) m = fmaxf(m, zdiff(z, 4, i));
            s = m * k.k_md;
            break;
        }
        case PARGO_SLOPE_SD:  // :122-124
            dx = zdiff(z, 4, 3) * k.k_sd;
            dy = zdiff(z, 4, 7) * k.k_sd;
            s = sqrtf(dx * dx + dy * dy);
            break;
        case PARGO_SLOPE_SFD:  // :126-128
            dx = zdiff(z, 5, 3) * k.k_sfd;
            dy = zdiff(z, 1, 7) * k.k_sfd;
            s = sqrtf(dx * dx + dy * dy);
            break;
        case PARGO_SLOPE_TFD:  // :130-132; dy uses z[6] twice, as the reference does
            dx = (zdiff(z, 8, 0) + zdiff(z, 5, 3) + zdiff(z, 2, 6)) * k.k_tfd;
            dy = (zdiff(z, 2, 6) + zdiff(z, 1, 7) + zdiff(z, 0, 6)) * k.k_tfd;
            s = sqrtf(dx * dx + dy * dy);
            break;
        default:  // TFDW :134-136
            dx = (zdiff(z, 8, 6) + zdiff(z, 2, 0) + k.sqrt2 * zdiff(z, 5, 3)) * k.k_tfdw;
            dy = (zdiff(z, 2, 6) + zdiff(z, 0, 8) + k.sqrt2 * zdiff(z, 1, 7)) * k.k_tfdw;
            s = sqrtf(dx * dx + dy * dy);
            break;
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

// Certified FP32 D8 decision.
//   c_i = fl32(z4 - z_i); diagonal x_i = fl32(c_i * fl32(1/sqrt 2)), cardinal x_i = c_i.
// Against the reference's double r_i = fl64(d4 - d_i) [/ fl64(sqrt 2)],
// |x_i - r_i| <= |x_i| 2^-22 (three float roundings of relative 2^-24 and the
// constant's error; the double roundings are 2^-53).  With E = 2^-21 max|x_i|
// (twice that bound), the reference max M_ref = max(0, r_i) is within E/2 of
// M = max(0, x_i), and each tie test |r_i - M_ref| < 1e-6 is decided exactly
// when u_i = x_i - (M - 1e-6) is further than 3E from zero (the float rounding
// of u and of M - 1e-6 is below E/2 because E >= 2^-21 M).  Returns the code,
// or kD8Unsure when some decision lies inside its error band.
constexpr int kD8Unsure = 0x7fff;
__device__ __forceinline__ int d8_certified(const float c[9], int dir_type) {
    const float kinv = 0.70710677f;
    // Threshold 1e-6 widened by 2^-15 relative on each side: covers the
    // distance between fl32(1e-6) and the double literal.
    const float t_lo = 0.99996948e-6f, t_hi = 1.0000305e-6f;
    float x[9];
    float m = 0.0f, a = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        if (i == 4) continue;
        x[i] = (i == 0 || i == 2 || i == 6 || i == 8) ? c[i] * kinv : c[i];
        m = fmaxf(m, x[i]);
        a = fmaxf(a, fabsf(x[i]));
    }
    const float e = a * 4.76837158203125e-07f;  // 2^-21
    if (m + e < t_lo) return -1;
    if (!(m - e > t_hi)) return kD8Unsure;
    const float thr = m - 1.0e-6f;
    const float err = 3.0f * e;
    unsigned mask = 0;
    float close = 3.0e38f;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        if (i == 4) continue;
        float u = x[i] - thr;
        close = fminf(close, fabsf(u));
        mask |= (u > 0.0f ? 1u : 0u) << i;
    }
    if (close <= err) return kD8Unsure;
    return d8_code_from_mask(mask, dir_type);
}

}  // namespace pargo
