// grad.cu -- hand-written adjoint of Horn (FD) slope, fused with the forward.
//
// Forward (slopeOperator.cpp:84-86, differences-first in FP32):
//   nx = (z2 - z0) + 2 (z5 - z3) + (z8 - z6),  ny = (z0 - z6) + 2 (z1 - z7) + (z2 - z8),
//   s  = k sqrt(nx^2 + ny^2),  k = 1 / (8 cs).
// Adjoint: with g(c) = dL/ds(c),
//   A(c) = g(c) k nx / |n|,  B(c) = g(c) k ny / |n|   (0 when |n| = 0: the
//   subgradient at zero slope is taken as 0),
//   dL/dz(q) = sum over the 9 cells c whose window holds q at position j of
//              A(c) a_j + B(c) b_j,  a = d nx / d z_j, b = d ny / d z_j.
// It is a gather (each output cell reads its 3x3 neighbours' A, B), so no
// atomics.  Cells whose window touches nodata (Eps 1e-7, the slope operator's)
// or lies on the ring have no slope and contribute nothing.
//
// mode 0: L = sum_c (s(c) - s_ref(c))^2 over cells where both slopes exist,
//         g(c) = 2 (s - s_ref); writes dL/dz and accumulates L.
// mode 1: g(c) = gslope(c) given (backward only).
//
// One CTA computes a 32 x 32 block of dL/dz: it stages z (and z_ref) with a
// two-cell halo in shared memory, forms A and B on the 34 x 34 cells around
// the block, then gathers.

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

constexpr int kB = 32;
constexpr int kZ = kB + 4;  // z with a two-cell halo
constexpr int kA = kB + 2;  // A, B with a one-cell halo

__constant__ float c_a[9] = {-1.f, 0.f, 1.f, -2.f, 0.f, 2.f, -1.f, 0.f, 1.f};
__constant__ float c_b[9] = {1.f, 2.f, 1.f, 0.f, 0.f, 0.f, -1.f, -2.f, -1.f};

__device__ __forceinline__ float load_f32(const InView& v, int64_t r, int64_t c) {
    return reinterpret_cast<const float*>(v.base + r * v.pitch)[c];
}

__global__ void __launch_bounds__(256) slope_grad_kernel(const GradParams p, int mode, int64_t nbx) {
    __shared__ float sz[kZ][kZ + 1];
    __shared__ float sr[kZ][kZ + 1];
    __shared__ float sa[kA][kA + 1];
    __shared__ float sb[kA][kA + 1];
    __shared__ double red[8];
    const int tid = threadIdx.x;
    const int64_t by = blockIdx.x / nbx, bx = blockIdx.x % nbx;
    const int64_t y0 = by * kB, x0 = bx * kB;
    const float NDV = 3.0e38f;  // marks nodata / outside in shared memory

    for (int i = tid; i < kZ * kZ; i += 256) {
        const int a = i / kZ, b = i % kZ;
        const int64_t r = y0 - 2 + a, c = x0 - 2 + b;
        float z = NDV, zr = NDV;
        if (r >= 0 && c >= 0 && r < p.rows && c < p.cols) {
            z = load_f32(p.z, r, c);
            if (p.nd7f.has(z)) z = NDV;
            if (mode == 0) {
                zr = load_f32(p.zref, r, c);
                if (p.nd7f.has(zr)) zr = NDV;
            }
        }
        sz[a][b] = z;
        sr[a][b] = zr;
    }
    __syncthreads();

    float lsum = 0.0f;
    for (int i = tid; i < kA * kA; i += 256) {
        const int a = i / kA, b = i % kA;  // cell (y0 - 1 + a, x0 - 1 + b); its window is sz[a..a+2][b..b+2]
        const int64_t r = y0 - 1 + a, c = x0 - 1 + b;
        float A = 0.0f, B = 0.0f;
        const bool inner = r >= 1 && c >= 1 && r <= p.rows - 2 && c <= p.cols - 2;
        if (inner) {
            float w[9];
            bool ok = true;
#pragma unroll
            for (int q = 0; q < 9; q++) {
                w[q] = sz[a + q / 3][b + q % 3];
                ok &= w[q] != NDV;
            }
            if (ok) {
                const float nx = ((w[2] - w[0]) + (w[8] - w[6])) + 2.0f * (w[5] - w[3]);
                const float ny = ((w[0] - w[6]) + (w[2] - w[8])) + 2.0f * (w[1] - w[7]);
                const float nn = sqrtf(nx * nx + ny * ny);
                const float s = nn * p.k_fd;
                float g = 0.0f;
                bool have = true;
                if (mode == 0) {
                    float v[9];
#pragma unroll
                    for (int q = 0; q < 9; q++) {
                        v[q] = sr[a + q / 3][b + q % 3];
                        have &= v[q] != NDV;
                    }
                    if (have) {
                        const float mx = ((v[2] - v[0]) + (v[8] - v[6])) + 2.0f * (v[5] - v[3]);
                        const float my = ((v[0] - v[6]) + (v[2] - v[8])) + 2.0f * (v[1] - v[7]);
                        const float sref = sqrtf(mx * mx + my * my) * p.k_fd;
                        const float d = s - sref;
                        g = 2.0f * d;
                        if (a >= 1 && b >= 1 && a <= kB && b <= kB) lsum += d * d;
                    }
                } else {
                    g = load_f32(p.gslope, r, c);
                }
                if (have && nn > 0.0f) {
                    const float f = g * p.k_fd / nn;
                    A = f * nx;
                    B = f * ny;
                }
            }
        }
        sa[a][b] = A;
        sb[a][b] = B;
    }
    __syncthreads();

    for (int i = tid; i < kB * kB; i += 256) {
        const int a = i / kB, b = i % kB;
        const int64_t r = y0 + a, c = x0 + b;
        if (r >= p.rows || c >= p.cols) continue;
        // q = (a+1, b+1) in the A frame; c_j = q - (j/3 - 1, j%3 - 1)
        float acc = 0.0f;
#pragma unroll
        for (int j = 0; j < 9; j++) {
            const int ca = a + 1 - (j / 3 - 1), cb = b + 1 - (j % 3 - 1);
            acc += sa[ca][cb] * c_a[j] + sb[ca][cb] * c_b[j];
        }
        reinterpret_cast<float*>(reinterpret_cast<char*>(p.gz) + r * p.gz_pitch)[c] = acc;
    }

    if (mode == 0 && p.loss) {
        float v = lsum;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) red[tid >> 5] = (double)v;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < 8; w++) t += red[w];
            if (t != 0.0) atomicAdd(p.loss, t);
        }
    }
}

}  // namespace

cudaError_t launch_slope_loss_grad(const GradParams& p, int mode, cudaStream_t st) {
    const int64_t nby = (p.rows + kB - 1) / kB, nbx = (p.cols + kB - 1) / kB;
    if (nby * nbx == 0) return cudaSuccess;
    slope_grad_kernel<<<(unsigned)(nby * nbx), 256, 0, st>>>(p, mode, nbx);
    return cudaGetLastError();
}

}  // namespace pargo
