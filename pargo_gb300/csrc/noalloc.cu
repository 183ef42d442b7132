// noalloc.cu -- SCA for callers that cannot allocate device memory.
//
// pargo_sca() takes its scratch (in-degrees, upstream totals, flags) from a
// context whose buffers grow with cudaMalloc.  Some callers of this library
// cannot allocate: a host application that runs under a strict device-memory
// budget owned by another component (a GIS runtime's own pool), a plugin that
// is handed device buffers and a stream and nothing else, code paths that must
// not take the allocator's locks or trigger its implicit synchronisation.
// pargo_sca_noalloc() serves them: its scratch is a fixed array in the
// library's own device image, so the call allocates nothing.
//
// Limits and sharing:
//  * rasters of at most PARGO_SCA_NOALLOC_MAX_CELLS cells (2^20, e.g. 1024 x 1024);
//    the array holds 21 bytes per cell (~22 MB) on every GPU that loads the
//    library, for as long as the process lives;
//  * every call, on every stream, uses the same array: two calls whose work
//    overlaps on the GPU race and corrupt each other -- serialise them;
//  * the array keeps the previous call's contents; every field a call reads is
//    rewritten by that call before it is read (the in-degree pass rewrites all
//    per-cell scratch, the counters are cleared with a memset).
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (once per device, with that device current).  The
// address is kept for the life of the process: after cudaDeviceReset (which
// unloads the library's device image) the cached address is stale, so calls
// after a reset are not supported.
//
// Every call is synchronous: it waits on `stream` for the completion count
// before it returns, so it cannot be called on a stream being captured.

#include <math.h>

#include <mutex>

#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int64_t kMaxCells = PARGO_SCA_NOALLOC_MAX_CELLS;
// per cell: int32 in-degree, 2 x uint64 totals, uint8 flags; then 4 uint64 counters
constexpr size_t kIndegOff = 0;
constexpr size_t kConvOff = kIndegOff + 4 * (size_t)kMaxCells;
constexpr size_t kShipOff = kConvOff + 8 * (size_t)kMaxCells;
constexpr size_t kFlagsOff = kShipOff + 8 * (size_t)kMaxCells;
constexpr size_t kCountersOff = (kFlagsOff + (size_t)kMaxCells + 255) / 256 * 256;
constexpr size_t kScratchBytes = kCountersOff + 8 * sizeof(unsigned long long);

static __device__ __align__(256) unsigned char g_sca_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once).
cudaError_t scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sca_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

int64_t pitch_or_dense(const pargo_raster* r) {
    return r->pitch ? r->pitch : r->cols * (int64_t)pargo::elem_size(r->dtype);
}

}  // namespace

extern "C" pargo_status pargo_sca_noalloc(const pargo_raster* d8, pargo_raster* sca, const pargo_nbr* nbr,
                                          int contract, void* stream) {
    using namespace pargo;
    if (!d8 || !sca) return PARGO_ERR_INVALID_ARG;
    if (d8->location != PARGO_DEVICE || sca->location != PARGO_DEVICE || !d8->data || !sca->data)
        return PARGO_ERR_INVALID_ARG;
    if (d8->rows < 3 || d8->cols < 3 || d8->rows != sca->rows || d8->cols != sca->cols)
        return PARGO_ERR_INVALID_ARG;
    if (d8->rows > INT32_MAX || d8->cols > INT32_MAX) return PARGO_ERR_INVALID_ARG;
    if (d8->rows > kMaxCells / d8->cols) return PARGO_ERR_INVALID_ARG;  // beyond the fixed scratch (no overflow)
    if (elem_size(d8->dtype) == 0 || (sca->dtype != PARGO_F64 && sca->dtype != PARGO_F32))
        return PARGO_ERR_INVALID_ARG;
    // The same layout rules as every other entry point: pitches cover a row and
    // are whole elements, and the data is aligned to its element size (a
    // misaligned load or store in a kernel would end the CUDA context).
    for (const pargo_raster* r : {(const pargo_raster*)d8, (const pargo_raster*)sca}) {
        const int64_t es = (int64_t)elem_size(r->dtype);
        if (r->pitch < 0 || (r->pitch != 0 && r->pitch < r->cols * es) || r->pitch % es != 0) return PARGO_ERR_INVALID_ARG;
        if ((uintptr_t)r->data % (uintptr_t)es != 0) return PARGO_ERR_INVALID_ARG;
    }
    if (contract != PARGO_SCA_CONVERGED && contract != PARGO_SCA_SHIPPED) return PARGO_ERR_INVALID_ARG;
    if (nbr) {
        const int half = ((int)sqrt((double)nbr->count)) / 2;
        if (half != 1 || nbr->min_row != -1 || nbr->min_col != -1 || nbr->max_row != 1 || nbr->max_col != 1)
            return PARGO_ERR_NBR_UNSUPPORTED;
    }
    unsigned char* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return PARGO_ERR_CUDA;
    ScaScratch s{};
    s.indeg = reinterpret_cast<int32_t*>(base + kIndegOff);
    s.conv = reinterpret_cast<unsigned long long*>(base + kConvOff);
    s.ship = reinterpret_cast<unsigned long long*>(base + kShipOff);
    s.flags = base + kFlagsOff;
    s.counters = reinterpret_cast<unsigned long long*>(base + kCountersOff);
    ScaParams p{};
    p.rows = d8->rows;
    p.cols = d8->cols;
    p.d8 = InView{static_cast<const char*>(d8->data), pitch_or_dense(d8), d8->dtype};
    p.nodata = d8->nodata;
    p.out = OutView{static_cast<char*>(sca->data), pitch_or_dense(sca), sca->dtype, sca->nodata};
    p.shipped = contract == PARGO_SCA_SHIPPED;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (sca_run(p, s, st) != cudaSuccess) return PARGO_ERR_CUDA;
    // completed vs valid cells, read into host stack memory (no allocation)
    unsigned long long c[2] = {0, 0};
    if (cudaMemcpyAsync(c, s.counters, sizeof(c), cudaMemcpyDeviceToHost, st) != cudaSuccess) return PARGO_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return PARGO_ERR_CUDA;
    return c[0] == c[1] ? PARGO_OK : PARGO_ERR_CYCLE;
}
