// twi.cu -- topographic wetness index from a slope and an SCA raster.
//
// Reference: TWIOperator::Operator (apps/hydrology/twi/TWIOperator.cpp:42-69).
// On a work cell the result is nodata when any value of its 3x3 window, in
// the SCA or the slope raster, equals the SCA raster's nodata exactly
// (:51-55; the reference compares both layers against that one value);
// otherwise ln(sca / slope), slope raised to Eps = 1e-7 when below it
// (:61-65).  Ring cells get the output's nodata (the reference output starts
// as a copy of the slope layer's nodata, pTWI.cpp:66).
//
// The arithmetic is FP32 (quotient and logf: about 1e-6 relative against the
// reference's FP64); the equality tests keep the reference's double
// semantics without FP64 instructions: a float input equals the nodata
// double only if that double is exactly a float, a double input is compared
// by its bits (with +0 == -0).

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

struct TwiIn {
    const char* base;
    int64_t pitch;
    int f64;
};

__device__ __forceinline__ bool is_nd(const TwiIn& v, int64_t r, int64_t c, const TwiParams& p) {
    const char* row = v.base + r * v.pitch;
    if (v.f64) {
        const long long b = reinterpret_cast<const long long*>(row)[c];
        return b == p.nd_bits || (((b | p.nd_bits) << 1) == 0);  // bit equality, or +0 / -0
    }
    return p.nd_is_float && reinterpret_cast<const float*>(row)[c] == p.nd_f;
}

__device__ __forceinline__ float as_f(const TwiIn& v, int64_t r, int64_t c) {
    const char* row = v.base + r * v.pitch;
    return v.f64 ? dbl2flt_rn(reinterpret_cast<const double*>(row)[c]) : reinterpret_cast<const float*>(row)[c];
}

__global__ void __launch_bounds__(256) twi_kernel(const TwiParams p) {
    const TwiIn sl{p.slope.base, p.slope.pitch, p.slope.dtype == PARGO_F64};
    const TwiIn sa{p.sca.base, p.sca.pitch, p.sca.dtype == PARGO_F64};
    const int64_t n = p.rows * p.cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        if (r < 1 || c < 1 || r > p.rows - 2 || c > p.cols - 2) {
            if (p.out.dtype == PARGO_F64) put_value(p.out, r, c, p.out.nodata);
            else put_float(p.out, r, c, p.out_nd_f);
            continue;
        }
        bool nd = false;
#pragma unroll
        for (int a = -1; a <= 1; a++)
#pragma unroll
            for (int b = -1; b <= 1; b++) nd = nd || is_nd(sa, r + a, c + b, p) || is_nd(sl, r + a, c + b, p);
        if (nd) {
            if (p.out.dtype == PARGO_F64) put_value(p.out, r, c, p.sca_nodata);
            else put_float(p.out, r, c, p.sca_nd_f);
            continue;
        }
        float s = as_f(sl, r, c);
        // the reference raises slope < 1e-7 (a double compare) to 1e-7;
        // eps_cut is the least float >= 1e-7, so s < eps_cut decides the same
        if (s < p.eps_cut) s = 1.0e-7f;
        put_float(p.out, r, c, logf(__fdiv_rn(as_f(sa, r, c), s)));
    }
}

}  // namespace

cudaError_t launch_twi(const TwiParams& p, int num_sms, cudaStream_t st) {
    const int64_t n = p.rows * p.cols;
    if (n == 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    twi_kernel<<<(unsigned)blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace pargo
