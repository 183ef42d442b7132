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
// One CTA computes a 32 x 64 block of dL/dz: it stages z (and z_ref) with a
// two-cell halo in shared memory (nodata as NaN), forms A and B on the
// 34 x 66 cells around the block, then gathers with the stencil's constant
// coefficients.  The forward uses the slope kernels' pinned rounding
// (horn_slope), so the fused loss sees the same slopes as pargo_slope_fwd.

#include "common.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace pargo {

namespace {

constexpr int kBH = 32, kBW = 64;           // dL/dz block of one CTA
constexpr int kZH = kBH + 4, kZW = kBW + 4;  // z with a two-cell halo
constexpr int kAH = kBH + 2, kAW = kBW + 2;  // A, B with a one-cell halo
constexpr int kThreads = 256;

__device__ __forceinline__ float load_f32(const InView& v, int64_t r, int64_t c) {
    return reinterpret_cast<const float*>(v.base + r * v.pitch)[c];
}

// Horn numerators of the window whose top-left is w (row stride ld), in the
// forward's pinned rounding.  A NaN anywhere among the 8 neighbours (nodata,
// or outside the raster) makes nx or ny NaN: NaN survives every difference,
// even two equal markers, so validity is one test on the result.
__device__ __forceinline__ void numerators(const float* w, int ld, float& nx, float& ny) {
    const float z0 = w[0], z1 = w[1], z2 = w[2], z3 = w[ld], z5 = w[ld + 2];
    const float z6 = w[2 * ld], z7 = w[2 * ld + 1], z8 = w[2 * ld + 2];
    nx = __fmaf_rn(2.0f, __fsub_rn(z5, z3), __fadd_rn(__fsub_rn(z2, z0), __fsub_rn(z8, z6)));
    ny = __fmaf_rn(2.0f, __fsub_rn(z1, z7), __fadd_rn(__fsub_rn(z0, z6), __fsub_rn(z2, z8)));
}

__global__ void __launch_bounds__(kThreads) slope_grad_kernel(const GradParams p, int mode, int64_t nbx) {
    __shared__ float sz[kZH][kZW + 1];
    __shared__ float sr[kZH][kZW + 1];
    __shared__ float sa[kAH][kAW + 1];
    __shared__ float sb[kAH][kAW + 1];
    __shared__ double red[kThreads / 32];
    const int tid = threadIdx.x;
    const int64_t by = blockIdx.x / nbx, bx = blockIdx.x % nbx;
    const int64_t y0 = by * kBH, x0 = bx * kBW;
    const float kNaN = __int_as_float(0x7FC00000);

    // z (and z_ref) with the halo; nodata (Eps 1e-7) and outside as NaN.
    // All of a thread's loads are issued before the first is used.
    {
        constexpr int kPer = (kZH * kZW + kThreads - 1) / kThreads;  // 10
        float vz[kPer], vr[kPer];
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int i = tid + q * kThreads;
            const int a = i / kZW, b = i % kZW;
            const int64_t r = y0 - 2 + a, c = x0 - 2 + b;
            const bool in = i < kZH * kZW && r >= 0 && c >= 0 && r < p.rows && c < p.cols;
            vz[q] = in ? load_f32(p.z, r, c) : kNaN;
            vr[q] = (in && mode == 0) ? load_f32(p.zref, r, c) : kNaN;
        }
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int i = tid + q * kThreads;
            if (i < kZH * kZW) {
                sz[i / kZW][i % kZW] = p.nd7f.has(vz[q]) ? kNaN : vz[q];
                sr[i / kZW][i % kZW] = p.nd7f.has(vr[q]) ? kNaN : vr[q];
            }
        }
    }
    __syncthreads();

    // A = g k nx / |n|, B = g k ny / |n| on the block plus a one-cell ring
    float lsum = 0.0f;
    for (int i = tid; i < kAH * kAW; i += kThreads) {
        const int a = i / kAW, b = i % kAW;  // cell (y0 - 1 + a, x0 - 1 + b); its window is sz[a..a+2][b..b+2]
        const int64_t r = y0 - 1 + a, c = x0 - 1 + b;
        float A = 0.0f, B = 0.0f;
        const bool inner = r >= 1 && c >= 1 && r <= p.rows - 2 && c <= p.cols - 2;
        float nx, ny;
        numerators(&sz[a][b], kZW + 1, nx, ny);
        const float q = __fmaf_rn(nx, nx, __fmul_rn(ny, ny));
        if (inner && sz[a + 1][b + 1] == sz[a + 1][b + 1] && q == q) {  // centre and neighbours valid
            const float s = horn_slope(nx, ny, p.k_fd);
            float g = 0.0f;
            bool have = true;
            if (mode == 0) {
                float mx, my;
                numerators(&sr[a][b], kZW + 1, mx, my);
                const float sref = horn_slope(mx, my, p.k_fd);
                have = sr[a + 1][b + 1] == sr[a + 1][b + 1] && sref == sref;
                if (have) {
                    const float d = s - sref;
                    g = 2.0f * d;
                    if (a >= 1 && b >= 1 && a <= kBH && b <= kBW) lsum += d * d;
                }
            } else {
                g = load_f32(p.gslope, r, c);
            }
            if (have && q > 0.0f) {  // subgradient 0 at zero slope
                const float f = g * p.k_fd * rsqrtf(q);  // g k / |n|
                A = f * nx;
                B = f * ny;
            }
        }
        sa[a][b] = A;
        sb[a][b] = B;
    }
    __syncthreads();

    // dL/dz(q) = sum over the 3 x 3 cells c around q of A(c) a_j + B(c) b_j,
    // j = q's position in c's window (a = d nx / d z_j, b = d ny / d z_j).
    for (int i = tid; i < kBH * kBW; i += kThreads) {
        const int a = i / kBW, b = i % kBW;
        const int64_t r = y0 + a, c = x0 + b;
        if (r >= p.rows || c >= p.cols) continue;
        // cell c_j = q - (j/3 - 1, j%3 - 1); in the A frame q sits at (a+1, b+1)
        const float* A0 = &sa[a][b];  // A of the cell at q + (-1, -1)
        const float* B0 = &sb[a][b];
        constexpr int L = kAW + 1;
        // window position j of q in c_j: c_j = q + (1 - j/3, 1 - j%3)
        // a_j: -1 0 1 / -2 0 2 / -1 0 1 ; b_j: 1 2 1 / 0 0 0 / -1 -2 -1
        const float ga = (-A0[2 * L + 2] + A0[2 * L]) + 2.0f * (-A0[L + 2] + A0[L]) + (-A0[2] + A0[0]);
        const float gb = (B0[2 * L + 2] + 2.0f * B0[2 * L + 1] + B0[2 * L]) - (B0[2] + 2.0f * B0[1] + B0[0]);
        reinterpret_cast<float*>(reinterpret_cast<char*>(p.gz) + r * p.gz_pitch)[c] = ga + gb;
    }

    if (mode == 0 && p.loss) {
        float v = lsum;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) red[tid >> 5] = (double)v;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < kThreads / 32; w++) t += red[w];
            if (t != 0.0) atomicAdd(p.loss, t);
        }
    }
}

// TMA-staged form of the same computation, for 16-byte aligned float32
// inputs, on 32 x 60 blocks: one thread loads the block's z (and z_ref) with
// its two-cell halo as a 2-D box (68 x 36 floats from column x0 - 4: the
// box's x coordinate stays 16-byte aligned), the block turns nodata into NaN
// in place four values at a time, and each phase runs on column strips: a
// thread owns one column of 9 (A, B) rows or 8 output rows and walks down it
// with a rolling three-row window in registers, so a cell reads its three new
// values instead of its whole window and no index is divided.  The arithmetic
// of each cell is that of the form above, in the same order.  Cells outside
// the raster load as 0 instead of NaN: only ring cells and cells beyond the
// raster have them in their windows, and those have no slope.
constexpr int kGH = 32, kGW = 60;             // dL/dz block (60: x0 stays a multiple of 4)
constexpr int kGAH = kGH + 2, kGAW = kGW + 2;  // A, B with a one-cell halo: 34 x 62
constexpr int kTBW = kGW + 8;                 // box columns: x0-4 .. x0+63
constexpr int kTBH = kGH + 4;                 // box rows: y0-2 .. y0+33
constexpr int kBoxFloats = kTBW * kTBH;
constexpr int kBoxBytes = kBoxFloats * 4;     // 9792
// a TMA destination starts on a 128-byte boundary: z_ref's box follows z's
// at the next one
constexpr int kBoxStride = (kBoxBytes + 127) / 128 * 128;  // 9856
static_assert(kBoxStride % 128 == 0 && kBoxStride >= kBoxBytes, "box alignment");
constexpr int kSegA = 9, kSegO = 8;           // rows per thread: A/B (4 strips of 34), output (4 of 32)
constexpr long long kWaitBudget = 4000000000LL;
static_assert(kGAW * 4 <= kThreads && kGW * 4 <= kThreads, "one thread per column strip");

__global__ void __launch_bounds__(kThreads) slope_grad_tma_kernel(const __grid_constant__ CUtensorMap mz,
                                                                  const __grid_constant__ CUtensorMap mr,
                                                                  const GradParams p, int mode, int64_t nbx) {
    extern __shared__ __align__(1024) unsigned char grad_smem[];
    float* bz = reinterpret_cast<float*>(grad_smem);
    float* br = reinterpret_cast<float*>(grad_smem + kBoxStride);
    __shared__ float sa[kGAH][kGAW + 1];
    __shared__ float sb[kGAH][kGAW + 1];
    __shared__ double red[kThreads / 32];
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x;
    const int64_t by = blockIdx.x / nbx, bx = blockIdx.x % nbx;
    const int64_t y0 = by * kGH, x0 = bx * kGW;
    const float kNaN = __int_as_float(0x7FC00000);
    if (tid == 0) {
        tma_prefetch_desc(&mz);
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(&bar, mode == 0 ? 2 * kBoxBytes : kBoxBytes);
        tma_load_2d(bz, &mz, (int32_t)(x0 - 4), (int32_t)(y0 - 2), &bar);
        if (mode == 0) tma_load_2d(br, &mr, (int32_t)(x0 - 4), (int32_t)(y0 - 2), &bar);
    }
    if (!mbar_wait_bounded(&bar, 0, kWaitBudget)) {
        if (tid == 0 && p.error_flag) atomicExch(p.error_flag, 1);
        return;
    }
    // nodata (Eps 1e-7) as NaN, four values at a time
    for (int box = 0; box < (mode == 0 ? 2 : 1); box++) {
        float4* z4 = reinterpret_cast<float4*>(box ? br : bz);
        for (int i = tid; i < kBoxFloats / 4; i += kThreads) {
            float4 v = z4[i];
            v.x = p.nd7f.has(v.x) ? kNaN : v.x;
            v.y = p.nd7f.has(v.y) ? kNaN : v.y;
            v.z = p.nd7f.has(v.z) ? kNaN : v.z;
            v.w = p.nd7f.has(v.w) ? kNaN : v.w;
            z4[i] = v;
        }
    }
    __syncthreads();
    // A and B on the 34 x 62 cells around the block: cell (a, b) is raster
    // (y0 - 1 + a, x0 - 1 + b), its window the box's rows a .. a+2, columns
    // b+2 .. b+4.  Thread: column b = tid % 62, rows 9k .. 9k + 8.
    float lsum = 0.0f;
    if (tid < kGAW * 4) {
        const int b = tid % kGAW, a0 = (tid / kGAW) * kSegA, a1 = min(a0 + kSegA, kGAH);
        const int64_t c = x0 - 1 + b;
        const bool col_in = c >= 1 && c <= p.cols - 2;
        const float* wz = bz + a0 * kTBW + b + 2;
        const float* wr = br + a0 * kTBW + b + 2;
        float z0 = wz[0], z1 = wz[1], z2 = wz[2], z3 = wz[kTBW], z4 = wz[kTBW + 1], z5 = wz[kTBW + 2];
        float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, r3 = 0.0f, r4 = 0.0f, r5 = 0.0f;
        if (mode == 0) {
            r0 = wr[0], r1 = wr[1], r2 = wr[2], r3 = wr[kTBW], r4 = wr[kTBW + 1], r5 = wr[kTBW + 2];
        }
        for (int a = a0; a < a1; a++) {
            const float* nz = bz + (a + 2) * kTBW + b + 2;  // the window's third row
            const float z6 = nz[0], z7 = nz[1], z8 = nz[2];
            const int64_t r = y0 - 1 + a;
            float A = 0.0f, B = 0.0f;
            const bool inner = col_in && r >= 1 && r <= p.rows - 2;
            const float nx = __fmaf_rn(2.0f, __fsub_rn(z5, z3), __fadd_rn(__fsub_rn(z2, z0), __fsub_rn(z8, z6)));
            const float ny = __fmaf_rn(2.0f, __fsub_rn(z1, z7), __fadd_rn(__fsub_rn(z0, z6), __fsub_rn(z2, z8)));
            const float q = __fmaf_rn(nx, nx, __fmul_rn(ny, ny));
            float r6 = 0.0f, r7 = 0.0f, r8 = 0.0f;
            if (mode == 0) {
                const float* nr = br + (a + 2) * kTBW + b + 2;
                r6 = nr[0], r7 = nr[1], r8 = nr[2];
            }
            if (inner && z4 == z4 && q == q) {  // centre and neighbours valid
                const float s = horn_slope(nx, ny, p.k_fd);
                float g = 0.0f;
                bool have = true;
                if (mode == 0) {
                    const float mx = __fmaf_rn(2.0f, __fsub_rn(r5, r3), __fadd_rn(__fsub_rn(r2, r0), __fsub_rn(r8, r6)));
                    const float my = __fmaf_rn(2.0f, __fsub_rn(r1, r7), __fadd_rn(__fsub_rn(r0, r6), __fsub_rn(r2, r8)));
                    const float sref = horn_slope(mx, my, p.k_fd);
                    have = r4 == r4 && sref == sref;
                    if (have) {
                        const float d = s - sref;
                        g = 2.0f * d;
                        if (a >= 1 && b >= 1 && a <= kGH && b <= kGW) lsum += d * d;
                    }
                } else {
                    g = load_f32(p.gslope, r, c);
                }
                if (have && q > 0.0f) {  // subgradient 0 at zero slope
                    const float f = g * p.k_fd * rsqrtf(q);
                    A = f * nx;
                    B = f * ny;
                }
            }
            sa[a][b] = A;
            sb[a][b] = B;
            z0 = z3, z1 = z4, z2 = z5, z3 = z6, z4 = z7, z5 = z8;
            r0 = r3, r1 = r4, r2 = r5, r3 = r6, r4 = r7, r5 = r8;
        }
    }
    __syncthreads();
    // dL/dz of the 32 x 60 block: thread column b = tid % 60, rows 8k .. 8k + 7
    if (tid < kGW * 4) {
        const int b = tid % kGW, a0 = (tid / kGW) * kSegO;
        const int64_t c = x0 + b;
        // A's middle column has no weight in d nx / d z
        float A0 = sa[a0][b], A2 = sa[a0][b + 2], A3 = sa[a0 + 1][b], A5 = sa[a0 + 1][b + 2];
        float B0 = sb[a0][b], B1 = sb[a0][b + 1], B2 = sb[a0][b + 2];
        float B3 = sb[a0 + 1][b], B4 = sb[a0 + 1][b + 1], B5 = sb[a0 + 1][b + 2];
        for (int a = a0; a < a0 + kSegO; a++) {
            const float A6 = sa[a + 2][b], A8 = sa[a + 2][b + 2];
            const float B6 = sb[a + 2][b], B7 = sb[a + 2][b + 1], B8 = sb[a + 2][b + 2];
            const int64_t r = y0 + a;
            // the form above's sums, in its order
            const float ga = (-A8 + A6) + 2.0f * (-A5 + A3) + (-A2 + A0);
            const float gb = (B8 + 2.0f * B7 + B6) - (B2 + 2.0f * B1 + B0);
            if (r < p.rows && c < p.cols)
                reinterpret_cast<float*>(reinterpret_cast<char*>(p.gz) + r * p.gz_pitch)[c] = ga + gb;
            A0 = A3, A2 = A5, A3 = A6, A5 = A8;
            B0 = B3, B1 = B4, B2 = B5, B3 = B6, B4 = B7, B5 = B8;
        }
    }
    if (mode == 0 && p.loss) {
        float v = lsum;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) red[tid >> 5] = (double)v;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < kThreads / 32; w++) t += red[w];
            if (t != 0.0) atomicAdd(p.loss, t);
        }
    }
}

}  // namespace

cudaError_t launch_slope_loss_grad(const GradParams& p, int mode, cudaStream_t st) {
    const int64_t nby = (p.rows + kBH - 1) / kBH, nbx = (p.cols + kBW - 1) / kBW;
    if (nby * nbx == 0) return cudaSuccess;
    slope_grad_kernel<<<(unsigned)(nby * nbx), kThreads, 0, st>>>(p, mode, nbx);
    return cudaGetLastError();
}

}  // namespace pargo

namespace pargo {

int grad_box_rows() { return kTBH; }
int grad_box_cols() { return kTBW; }

cudaError_t launch_slope_loss_grad_tma(const CUtensorMap* mz, const CUtensorMap* mr, const GradParams& p, int mode,
                                       cudaStream_t st) {
    const int64_t nby = (p.rows + kGH - 1) / kGH, nbx = (p.cols + kGW - 1) / kGW;
    if (nby * nbx == 0) return cudaSuccess;
    const size_t smem = (size_t)kBoxStride + kBoxBytes;
    cudaError_t e = cudaFuncSetAttribute(slope_grad_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    slope_grad_tma_kernel<<<(unsigned)(nby * nbx), kThreads, smem, st>>>(*mz, mode == 0 ? *mr : *mz, p, mode, nbx);
    return cudaGetLastError();
}

}  // namespace pargo
