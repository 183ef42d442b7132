// load.cu -- the load estimator: compute-intensity layer and the row loads
// its decomposition is cut from.
//
// Compute layer (ComputeLayer::_init, gpro/computeLayer.h:210-262, and the
// intensity-ratio Transformation::Operator, gpro/transformation.h:155-197):
// one compute cell per grain x grain block of the data's work rectangle; its
// value sums, layer by layer and data row by data row, valid_load for every
// valid data cell (|v - nodata| > 1e-7, the layer's own nodata) and
// nodata_load for the others,
// skipping data cells past the raster's last row or column.  The sums are
// sequential FP64 additions in that order, so the layer equals the
// reference's bit for bit.  Two kernels:
//  * integer loads whose sums stay below 2^53 and a grain dividing 32
//    (compute_load_count_kernel): every partial sum is exact, so the cells
//    are counted in any order -- a warp reads 32 consecutive data columns of
//    one compute row, coalesced, and the counts are scaled by the loads;
//  * any other grain or load (compute_load_kernel): one thread per compute
//    cell, counting (integer loads) or adding the loads in the reference's
//    order.
//
// Row loads (DeComposition::valRowDcmp, gpro/deComposition.h:320-335): per
// compute row, the left-to-right FP64 sum of the cells that are above -9999
// and above nodata by more than 1e-7; one warp per row.

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

// |v - nodata| <= 1e-7 against layer l's own nodata (transformation.h:187)
__device__ __forceinline__ bool load_nodata(const LoadParams& p, int l, int64_t r, int64_t c) {
    const InView& v = p.data[l];
    const char* row = v.base + r * v.pitch;
    if (v.dtype == PARGO_F64) {
        const long long k = dkey64(reinterpret_cast<const double*>(row)[c]);
        return k >= p.nd_lo[l] && k <= p.nd_hi[l];
    }
    return p.ndf[l].has(reinterpret_cast<const float*>(row)[c]);
}

__global__ void __launch_bounds__(256) compute_load_kernel(const LoadParams p) {
    const int64_t n = p.crows * p.ccols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t cr = i / p.ccols, cc = i % p.ccols;
        double acc = 0.0;
        const bool work = !p.compute_ring || (cr >= 1 && cc >= 1 && cr <= p.crows - 2 && cc <= p.ccols - 2);
        if (work) {
            const int64_t r_end = min((cr + 1) * p.grain + 1, p.rows), c_end = min((cc + 1) * p.grain + 1, p.cols);
            if (p.integral) {
                // integer loads: every partial sum is an integer below 2^53, so
                // the sequential sum is exact and equals counts times loads
                long long nd = 0, total = 0;
                for (int l = 0; l < p.count; l++)
                    for (int64_t r = cr * p.grain + 1; r < r_end; r++)
                        for (int64_t c = cc * p.grain + 1; c < c_end; c++) nd += load_nodata(p, l, r, c) ? 1 : 0;
                total = (long long)p.count * (r_end - (cr * p.grain + 1)) * (c_end - (cc * p.grain + 1));
                acc = __dadd_rn(__dmul_rn((double)(total - nd), p.valid_load), __dmul_rn((double)nd, p.nodata_load));
            } else {
                for (int l = 0; l < p.count; l++)
                    for (int64_t r = cr * p.grain + 1; r < r_end; r++)
                        for (int64_t c = cc * p.grain + 1; c < c_end; c++)
                            acc = __dadd_rn(acc, load_nodata(p, l, r, c) ? p.nodata_load : p.valid_load);
            }
        }
        put_value(p.load, cr, cc, acc);
    }
}

// Nodata count of data column c over rows r0 .. r0 + nrows - 1 of layer l:
// every row's load issued before the first test.
template <int G>
__device__ __forceinline__ int column_nodata(const LoadParams& p, int l, int64_t r0, int nrows, int64_t c) {
    const InView& v = p.data[l];
    const char* base = v.base + r0 * v.pitch;
    int nd = 0;
    if (v.dtype == PARGO_F64) {
        double x[G];
#pragma unroll
        for (int q = 0; q < G; q++) x[q] = q < nrows ? reinterpret_cast<const double*>(base + q * v.pitch)[c] : 0.0;
#pragma unroll
        for (int q = 0; q < G; q++) {
            const long long k = dkey64(x[q]);
            nd += (q < nrows && k >= p.nd_lo[l] && k <= p.nd_hi[l]) ? 1 : 0;
        }
    } else {
        float x[G];
#pragma unroll
        for (int q = 0; q < G; q++) x[q] = q < nrows ? reinterpret_cast<const float*>(base + q * v.pitch)[c] : 0.0f;
#pragma unroll
        for (int q = 0; q < G; q++) nd += (q < nrows && p.ndf[l].has(x[q])) ? 1 : 0;
    }
    return nd;
}

// Integer loads with a grain G that divides 32: the counts do not depend on
// the order of the cells, so a warp reads 32 consecutive data columns of one
// compute row (one column per lane, G rows, coalesced) and adds each compute
// cell's counts over its G lanes.  The 32-column chunks start at data column
// 1 + 32 j, a compute cell's first column, so no cell straddles two chunks.
template <int G>
__global__ void __launch_bounds__(256) compute_load_count_kernel(const LoadParams p) {
    const int lane = threadIdx.x & 31;
    const int64_t chunks = (p.ccols * G + 31) / 32;  // per compute row
    const int64_t tasks = p.crows * chunks;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < tasks; w += nwarps) {
        const int64_t cr = w / chunks, j = w % chunks;
        const int64_t cc = (32 * j + lane) / G;  // this lane's compute column
        const int64_t c = 1 + 32 * j + lane;     // and data column
        const bool work = cc < p.ccols &&
                          (!p.compute_ring || (cr >= 1 && cc >= 1 && cr <= p.crows - 2 && cc <= p.ccols - 2));
        const int64_t r0 = cr * G + 1;
        const int nrows = (int)(min(r0 + G, p.rows) - r0);
        int nd = 0;
        if (work && c < p.cols)
            for (int l = 0; l < p.count; l++) nd += column_nodata<G>(p, l, r0, nrows, c);
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1) nd += __shfl_xor_sync(0xffffffffu, nd, o);
        if (lane % G == 0 && cc < p.ccols) {
            double acc = 0.0;
            if (work) {
                const int64_t c_end = min((cc + 1) * G + 1, p.cols);
                const long long total = (long long)p.count * nrows * (c_end - (cc * G + 1));
                acc = __dadd_rn(__dmul_rn((double)(total - nd), p.valid_load), __dmul_rn((double)nd, p.nodata_load));
            }
            put_value(p.load, cr, cc, acc);
        }
    }
}

__device__ __forceinline__ double load_at(const InView& load, const char* row, int64_t c) {
    return load.dtype == PARGO_F64 ? reinterpret_cast<const double*>(row)[c]
                                   : (double)reinterpret_cast<const float*>(row)[c];
}
__device__ __forceinline__ bool row_counts(double v, double nodata) {
    return __dadd_rn(v, 9999.0) > 0.0000001 && __dsub_rn(v, nodata) > 0.0000001;
}

// One warp per compute row, lanes over its columns (coalesced).  When every
// value the row counts is an integer of magnitude below int_bound (2^53 over
// the row's length), every partial sum of the reference's left-to-right FP64
// sum is an integer below 2^53, exact, so that sum equals the integer sum
// the lanes form in any order; otherwise lane 0 adds the row in order.
__global__ void __launch_bounds__(256) row_load_kernel(const InView load, int64_t crows, int64_t ccols, double nodata,
                                                       double int_bound, double* row_load) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < crows; r += nwarps) {
        const char* row = load.base + r * load.pitch;
        long long isum = 0;
        bool exact = true;
        for (int64_t c = lane; c < ccols; c += 32) {
            const double v = load_at(load, row, c);
            if (!row_counts(v, nodata)) continue;
            if (v == floor(v) && fabs(v) < int_bound) isum += (long long)v;
            else exact = false;
        }
        exact = __all_sync(0xffffffffu, exact);
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) isum += __shfl_xor_sync(0xffffffffu, isum, o);
        if (lane == 0) {
            double acc = (double)isum;
            if (!exact) {
                acc = 0.0;
                for (int64_t c = 0; c < ccols; c++) {
                    const double v = load_at(load, row, c);
                    if (row_counts(v, nodata)) acc = __dadd_rn(acc, v);
                }
            }
            row_load[r] = acc;
        }
    }
}

}  // namespace

template <int G>
static cudaError_t launch_count(const LoadParams& p, int num_sms, cudaStream_t s) {
    const int64_t tasks = p.crows * ((p.ccols * G + 31) / 32);  // one warp each
    int64_t blocks = (tasks + 7) / 8;
    if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
    compute_load_count_kernel<G><<<(unsigned)blocks, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_compute_load(const LoadParams& p, int num_sms, cudaStream_t s) {
    const int64_t n = p.crows * p.ccols;
    if (n == 0) return cudaSuccess;
    if (p.integral) {
        switch (p.grain) {
            case 1: return launch_count<1>(p, num_sms, s);
            case 2: return launch_count<2>(p, num_sms, s);
            case 4: return launch_count<4>(p, num_sms, s);
            case 8: return launch_count<8>(p, num_sms, s);
            case 16: return launch_count<16>(p, num_sms, s);
            case 32: return launch_count<32>(p, num_sms, s);
            default: break;  // other grains: one thread per compute cell
        }
    }
    int64_t blocks = (n + 255) / 256;
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    compute_load_kernel<<<(unsigned)blocks, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_row_load(const InView& load, int64_t crows, int64_t ccols, double nodata, double* row_load,
                            int num_sms, cudaStream_t s) {
    if (crows == 0) return cudaSuccess;
    int64_t blocks = (crows + 7) / 8;  // a warp per compute row
    if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
    const double int_bound = 9007199254740992.0 / (double)(ccols > 0 ? ccols : 1);
    row_load_kernel<<<(unsigned)blocks, 256, 0, s>>>(load, crows, ccols, nodata, int_bound, row_load);
    return cudaGetLastError();
}

}  // namespace pargo
