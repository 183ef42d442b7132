// sca.cu -- D8 specific catchment area by lock-free topological accumulation.
//
// Reference: SCAOperator::Operator (apps/hydrology/scad8/scaOperator.cpp:37-131).
// Phase 1 of the reference counts, for every valid cell c, the neighbours p
// whose code points at c while c does not point back at p (:65-84); phase 2
// pulls completed upstream totals into c in raster order (:86-128).  The
// shipped operator stops after ONE such sweep (:126); iterating the same rule
// until no in-degree remains gives the full upslope count.
//
// Both results come out of one topological pass:
//   conv(c)    = 1 + sum of conv(p) over the inflows p of c;
//   shipped(c) = 1 + sum of conv(p) over the inflows p that the single
//                raster-order sweep pulls: p is a source, or p precedes c in
//                raster order and p itself pulled all of its inflows ("done").
// The pass: every source cell starts a thread that walks downstream; at each
// receiver it adds its total (atomics on 64-bit integer counts, exact and
// order-free), then decrements the receiver's remaining in-degree; only the
// thread that brings it to zero continues, carrying the receiver's completed
// total.  No thread ever waits on another, so nothing can hang; cells whose
// in-degree never reaches zero (a cycle, or an inflow from the ring, which the
// reference never releases) are reported through the completed-cell count.
//
// Reference quirk kept: the last work cell (rows-2, cols-2) is visited in
// phase 2 even when its degree is not positive (:86), so when it is nodata it
// adds the inflows it pulls onto the nodata value (the SCA layer's nodata,
// which the reference copies from the D8 layer: here the output's nodata).

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

constexpr int kNoFlow = -2;  // valid cell whose code names no neighbour
constexpr uint8_t kSource = 1, kNotDone = 2, kValid = 4;

struct Decoded {
    bool nodata;
    int code;  // 0..8 (never 4) or kNoFlow
};

__device__ __forceinline__ Decoded decode(const ScaParams& p, int64_t r, int64_t c) {
    Decoded d{true, kNoFlow};
    const char* row = p.d8.base + r * p.d8.pitch;
    double v;
    switch (p.d8.dtype) {
        case PARGO_F64: v = reinterpret_cast<const double*>(row)[c]; break;
        case PARGO_F32: v = (double)reinterpret_cast<const float*>(row)[c]; break;
        case PARGO_I8: v = (double)reinterpret_cast<const int8_t*>(row)[c]; break;
        case PARGO_I16: v = (double)reinterpret_cast<const int16_t*>(row)[c]; break;
        default: v = (double)reinterpret_cast<const int32_t*>(row)[c]; break;
    }
    if (p.d8.dtype == PARGO_F64 || p.d8.dtype == PARGO_F32) {
        d.nodata = fabs(v - p.nodata) < kEpsHydro;  // scaOperator.cpp:48
    } else {
        d.nodata = v == p.nodata;
    }
    if (!d.nodata) {
        const int k = (int)v;
        d.code = ((double)k == v && k >= 0 && k <= 8 && k != 4) ? k : kNoFlow;
    }
    return d;
}

__device__ __forceinline__ bool in_work(const ScaParams& p, int64_t r, int64_t c) {
    return r >= 1 && c >= 1 && r <= p.rows - 2 && c <= p.cols - 2;
}

// Phase-1 rule: in-degree of c, sources, validity.
__global__ void sca_init_kernel(const ScaParams p, ScaScratch s) {
    const int64_t n = p.rows * p.cols;
    unsigned long long nvalid = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        s.conv[i] = 0;
        s.ship[i] = 0;
        uint8_t f = 0;
        int32_t deg = 0;
        if (in_work(p, r, c)) {
            const Decoded me = decode(p, r, c);
            if (!me.nodata) {
                f |= kValid;
                nvalid++;
                int dir = 8;  // code a neighbour at window position k needs to point at c
                for (int a = -1; a <= 1; a++)
                    for (int b = -1; b <= 1; b++, dir--) {
                        if (dir == 4) continue;
                        const Decoded nb = decode(p, r + a, c + b);
                        if (!nb.nodata && nb.code == dir && me.code != 8 - dir) deg++;
                    }
                if (deg == 0) f |= kSource;
            }
        }
        s.indeg[i] = deg;
        s.flags[i] = f;
    }
    nvalid = __reduce_add_sync(0xffffffffu, (unsigned)nvalid);
    if ((threadIdx.x & 31) == 0 && nvalid) atomicAdd(&s.counters[1], nvalid);
}

__global__ void sca_walk_kernel(const ScaParams p, ScaScratch s) {
    const int64_t n = p.rows * p.cols;
    const int64_t last = (p.rows - 2) * p.cols + (p.cols - 2);
    unsigned long long completed = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!(s.flags[i] & kSource)) continue;
        completed++;
        int64_t cur = i;
        unsigned long long total = 1;  // conv(cur)
        bool done = true;              // cur pulled all of its inflows (sources trivially)
        bool source = true;
        for (;;) {
            const int64_t r = cur / p.cols, c = cur % p.cols;
            const Decoded me = decode(p, r, c);
            if (me.code == kNoFlow) break;
            const int64_t tr = r + me.code / 3 - 1, tc = c + me.code % 3 - 1;
            if (!in_work(p, tr, tc)) break;
            const int64_t tgt = tr * p.cols + tc;
            const bool pulled = source || (cur < tgt && done);
            const Decoded td = decode(p, tr, tc);
            if (td.nodata) {
                if (tgt == last) {
                    atomicAdd(&s.counters[2], total);
                    if (pulled) atomicAdd(&s.counters[3], total);
                }
                break;
            }
            if (td.code == 8 - me.code) break;  // mutual pair: not an inflow (scaOperator.cpp:71)
            atomicAdd(&s.conv[tgt], total);
            if (pulled) atomicAdd(&s.ship[tgt], total);
            else atomicOr(reinterpret_cast<unsigned int*>(&s.flags[tgt & ~3LL]), (unsigned)kNotDone << (8 * (tgt & 3)));
            __threadfence();
            if (atomicSub(&s.indeg[tgt], 1) != 1) break;
            __threadfence();
            // Last contributor: tgt is complete.
            total = 1 + atomicAdd(&s.conv[tgt], 0ULL);
            const unsigned fw = atomicOr(reinterpret_cast<unsigned int*>(&s.flags[tgt & ~3LL]), 0u);
            done = !((fw >> (8 * (tgt & 3))) & kNotDone);
            source = false;
            cur = tgt;
            completed++;
        }
    }
    completed = __reduce_add_sync(0xffffffffu, (unsigned)completed);
    if ((threadIdx.x & 31) == 0 && completed) atomicAdd(&s.counters[0], completed);
}

__global__ void sca_finish_kernel(const ScaParams p, ScaScratch s) {
    const int64_t n = p.rows * p.cols;
    const int64_t last = (p.rows - 2) * p.cols + (p.cols - 2);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        double v = p.out.nodata;
        if (s.flags[i] & kValid) {
            v = 1.0 + (double)(p.shipped ? s.ship[i] : s.conv[i]);
        } else if (i == last && p.rows >= 3 && p.cols >= 3) {
            // nodata last work cell: the output's nodata value plus what it pulled
            v = p.out.nodata + (double)(p.shipped ? s.counters[3] : s.counters[2]);
        }
        put_value(p.out, r, c, v);
    }
}

}  // namespace

cudaError_t sca_run(const ScaParams& p, const ScaScratch& s, cudaStream_t st) {
    const int64_t n = p.rows * p.cols;
    if (n == 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    cudaError_t e = cudaMemsetAsync(s.counters, 0, 4 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    sca_init_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, s);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_walk_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, s);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_finish_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, s);
    return cudaGetLastError();
}

}  // namespace pargo
