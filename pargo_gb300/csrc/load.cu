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
// reference's bit for bit.  One thread per compute cell: a warp's 32 threads
// read 32 adjacent blocks, i.e. 32 * grain consecutive values of a data row.
//
// Row loads (DeComposition::valRowDcmp, gpro/deComposition.h:320-335): per
// compute row, the left-to-right FP64 sum of the cells that are above -9999
// and above nodata by more than 1e-7; one thread per row.

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

__global__ void __launch_bounds__(128) row_load_kernel(const InView load, int64_t crows, int64_t ccols, double nodata,
                                                       double* row_load) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < crows; r += (int64_t)gridDim.x * blockDim.x) {
        const char* row = load.base + r * load.pitch;
        double acc = 0.0;
        for (int64_t c = 0; c < ccols; c++) {
            const double v = load.dtype == PARGO_F64 ? reinterpret_cast<const double*>(row)[c]
                                                     : (double)reinterpret_cast<const float*>(row)[c];
            if (__dadd_rn(v, 9999.0) > 0.0000001 && __dsub_rn(v, nodata) > 0.0000001) acc = __dadd_rn(acc, v);
        }
        row_load[r] = acc;
    }
}

}  // namespace

cudaError_t launch_compute_load(const LoadParams& p, int num_sms, cudaStream_t s) {
    const int64_t n = p.crows * p.ccols;
    if (n == 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    compute_load_kernel<<<(unsigned)blocks, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_row_load(const InView& load, int64_t crows, int64_t ccols, double nodata, double* row_load,
                            int num_sms, cudaStream_t s) {
    if (crows == 0) return cudaSuccess;
    int64_t blocks = (crows + 127) / 128;
    if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
    row_load_kernel<<<(unsigned)blocks, 128, 0, s>>>(load, crows, ccols, nodata, row_load);
    return cudaGetLastError();
}

}  // namespace pargo
