// abi.cu -- the extern "C" entry points declared in include/pargo_gpu.h.
//
// Host side of every operator: argument checks (mirroring the reference's own
// checks where it has them), host<->device staging for host buffers, exact
// nodata bands, TMA descriptors, kernel dispatch, CUDA-graph-captured fill
// rounds.  No CPU compute path exists: every result is produced by a kernel.

#include <cudaTypedefs.h>
#include <math.h>

#include <cmath>
#include <string.h>

#include <errno.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstdarg>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "tune_cache.h"

using namespace pargo;

struct pargo_ctx {
    int device = 0;
    int num_sms = 0;
    std::string err;
    cudaStream_t own = nullptr;  // stream for captured fill rounds
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;  // stream hand-off
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;  // timing of the fill rounds
    cudaEvent_t ev_band[8] = {nullptr};  // pipeline: row bands computed, their host copies may start
    // grow-only device scratch slots
    struct Slot {
        void* p = nullptr;
        size_t n = 0;
    };
    Slot slots[48];
    // pinned host scratch (counter read-back, table staging)
    void* pinned = nullptr;
    size_t pinned_n = 0;
    unsigned long long* d_counters = nullptr;  // [0] fallbacks [1] visits [2] changed [3] raised [4,5] strip walk
    int* d_error = nullptr;
    int64_t last_fallbacks = 0;
    // fill graph cache
    cudaGraphExec_t fill_graph = nullptr;
    std::string fill_graph_key;
    // batch table cache
    std::string batch_key;
    bool batch_ordered = false;  // the cached batch has an intensity-ordered queue (kSlotBatchOrder)
    // autotuned focal kernel variant per size class (log2 of the cell count); -1 = untuned
    int focal_variant[64];
    std::string device_sig;  // key of this device in the tuning cache
    pargo_ctx() {
        for (int& v : focal_variant) v = -1;
    }
};

enum SlotId {
    kSlotIn0 = 0, kSlotIn1, kSlotOut0, kSlotOut1, kSlotFillW, kSlotFillLists, kSlotFillQueued,
    kSlotScaIndeg, kSlotScaConv, kSlotScaShip, kSlotScaFlags, kSlotScaCounters, kSlotBatchMaps,
    kSlotBatchParams, kSlotBatchStart, kSlotBatchNtx, kSlotBatchDems, kSlotClaim, kSlotLoss, kSlotGradOut,
    kSlotPipeD8, kSlotPipeSca, kSlotPipeCodes, kSlotScaTiles, kSlotMfdLayer0,
    kSlotMfdCnt = kSlotMfdLayer0 + 8, kSlotMfdFlags, kSlotMfdSca, kSlotMfdLists, kSlotStripSlow, kSlotLoadRows,
    kSlotBatchStripMaps, kSlotBatchSegStart, kSlotBatchNstrips, kSlotBatchSlow, kSlotFillMosaic, kSlotFillItems,
    kSlotBatchSegLoad, kSlotBatchOrder, kSlotScaForest, kSlotMfdRecords, kSlotCount
};
static_assert(kSlotCount <= 48, "context slot table");

namespace {

pargo_status fail(pargo_ctx* ctx, pargo_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    return st;
}

pargo_status cuda_fail(pargo_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, PARGO_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return fail(ctx, PARGO_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
    return fail(ctx, PARGO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CU(ctx, call)                                          \
    do {                                                       \
        cudaError_t e__ = (call);                              \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, #call); \
    } while (0)

void* slot(pargo_ctx* ctx, int id, size_t bytes, cudaError_t* err) {
    auto& s = ctx->slots[id];
    *err = cudaSuccess;
    if (bytes == 0) bytes = 16;
    if (s.n >= bytes) return s.p;
    if (s.p) {
        cudaDeviceSynchronize();
        cudaFree(s.p);
        s.p = nullptr;
        s.n = 0;
    }
    size_t want = bytes + bytes / 8;
    *err = cudaMalloc(&s.p, want);
    if (*err != cudaSuccess) {
        s.p = nullptr;
        return nullptr;
    }
    s.n = want;
    return s.p;
}

void* pinned(pargo_ctx* ctx, size_t bytes, cudaError_t* err) {
    *err = cudaSuccess;
    if (ctx->pinned_n >= bytes) return ctx->pinned;
    if (ctx->pinned) {
        cudaDeviceSynchronize();
        cudaFreeHost(ctx->pinned);
    }
    ctx->pinned = nullptr;
    ctx->pinned_n = 0;
    *err = cudaMallocHost(&ctx->pinned, bytes);
    if (*err != cudaSuccess) return nullptr;
    ctx->pinned_n = bytes;
    return ctx->pinned;
}

int64_t row_bytes(const pargo_raster* r) { return r->cols * (int64_t)elem_size(r->dtype); }
int64_t pitch_of(const pargo_raster* r) { return r->pitch ? r->pitch : row_bytes(r); }

pargo_status check_raster(pargo_ctx* ctx, const pargo_raster* r, const char* name) {
    if (!r) return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: null raster", name);
    if (elem_size(r->dtype) == 0) return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: unknown dtype %d", name, r->dtype);
    if (r->location != PARGO_HOST && r->location != PARGO_DEVICE)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: unknown location %d", name, r->location);
    if (r->rows < 0 || r->cols < 0) return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: negative size", name);
    if (r->rows > 0 && r->cols > 0 && !r->data) return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: null data", name);
    if (r->pitch != 0 && r->pitch < row_bytes(r))
        return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: pitch %lld below row size %lld", name, (long long)r->pitch,
                    (long long)row_bytes(r));
    if (r->pitch % elem_size(r->dtype) != 0)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: pitch not a multiple of the element size", name);
    if ((uintptr_t)r->data % elem_size(r->dtype) != 0)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: data not aligned to its element size", name);
    return PARGO_OK;
}

// The neighbourhood the focal operators accept: iNeighborCells = int(sqrt(n))/2
// must be 1 (the operators read exactly d[0..8], slopeOperator.cpp:55-73) and
// the MBR must be the 3x3 square (the work rectangle, neighborhood.h:447-448).
pargo_status check_nbr(pargo_ctx* ctx, const pargo_nbr* nbr) {
    if (!nbr) return PARGO_OK;  // NULL = Moore
    const int half = ((int)sqrt((double)nbr->count)) / 2;
    if (half != 1 || nbr->min_row != -1 || nbr->min_col != -1 || nbr->max_row != 1 || nbr->max_col != 1)
        return fail(ctx, PARGO_ERR_NBR_UNSUPPORTED,
                    "neighbourhood of %d cells with MBR [%d,%d]x[%d,%d]: the focal operators need the 3x3 Moore "
                    "window (int(sqrt(n))/2 == 1)",
                    nbr->count, nbr->min_row, nbr->max_row, nbr->min_col, nbr->max_col);
    return PARGO_OK;
}

// Neighborhood::calcWorkBR rejects rasters smaller than the window
// (neighborhood.h:440-446).
pargo_status check_dims(pargo_ctx* ctx, const pargo_raster* r) {
    if (r->rows < 3 || r->cols < 3)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "raster %lldx%lld is smaller than the 3x3 neighbourhood",
                    (long long)r->rows, (long long)r->cols);
    if (r->rows > INT32_MAX || r->cols > INT32_MAX)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "raster dimensions above 2^31-1");
    return PARGO_OK;
}

pargo_status check_same(pargo_ctx* ctx, const pargo_raster* a, const pargo_raster* b, const char* name) {
    if (a->rows != b->rows || a->cols != b->cols)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: %lldx%lld does not match the input %lldx%lld", name,
                    (long long)b->rows, (long long)b->cols, (long long)a->rows, (long long)a->cols);
    return PARGO_OK;
}

// ---- exact nodata bands: { x : |(double)x - nodata| < eps } as [lo, hi] ----
uint32_t fkey(float x) {
    uint32_t b;
    memcpy(&b, &x, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
float fval(uint32_t k) {
    uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float x;
    memcpy(&x, &b, 4);
    return x;
}
uint64_t dkey_h(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
double dval_h(uint64_t k) {
    uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    double x;
    memcpy(&x, &b, 8);
    return x;
}

template <typename K, typename T, typename ToV>
void band_search(K kmin, K kmax, double nodata, double eps, ToV val, T* lo, T* hi, bool inclusive = false) {
    // f(k) = fl64((double)val(k) - nodata) is non-decreasing in k.  The band is
    // |f| < eps, or |f| <= eps when inclusive.
    auto f = [&](K k) { return (double)val(k) - nodata; };
    auto above = [&](K k) { return inclusive ? f(k) >= -eps : f(k) > -eps; };
    auto below = [&](K k) { return inclusive ? f(k) <= eps : f(k) < eps; };
    // smallest k above -eps
    K a = kmin, b = kmax;
    if (!above(b)) { *lo = (T)INFINITY; *hi = (T)-INFINITY; return; }
    while (a < b) {
        K m = a + (b - a) / 2;
        if (above(m)) b = m; else a = m + 1;
    }
    K l = a;
    // largest k below eps
    a = kmin; b = kmax;
    if (!below(a)) { *lo = (T)INFINITY; *hi = (T)-INFINITY; return; }
    while (a < b) {
        K m = a + (b - a + 1) / 2;
        if (below(m)) a = m; else b = m - 1;
    }
    K h = a;
    if (l > h) { *lo = (T)INFINITY; *hi = (T)-INFINITY; return; }
    *lo = val(l);
    *hi = val(h);
}

Band<float> float_band(double nodata, double eps) {
    Band<float> b;
    // keys of -inf .. +inf (NaNs excluded)
    band_search<uint32_t, float>(fkey(-INFINITY), fkey(INFINITY), nodata, eps, fval, &b.lo, &b.hi);
    return b;
}
Band<double> double_band(double nodata, double eps) {
    Band<double> b;
    band_search<uint64_t, double>(dkey_h(-INFINITY), dkey_h(INFINITY), nodata, eps, dval_h, &b.lo, &b.hi);
    return b;
}
Band<float> float_band_incl(double nodata, double eps) {
    Band<float> b;
    band_search<uint32_t, float>(fkey(-INFINITY), fkey(INFINITY), nodata, eps, fval, &b.lo, &b.hi, true);
    return b;
}
Band<double> double_band_incl(double nodata, double eps) {
    Band<double> b;
    band_search<uint64_t, double>(dkey_h(-INFINITY), dkey_h(INFINITY), nodata, eps, dval_h, &b.lo, &b.hi, true);
    return b;
}
// A band of doubles as signed order-preserving keys (the device's dkey64);
// an empty band gives lo > hi.
void band_keys(const Band<double>& b, long long* lo, long long* hi) {
    if (!(b.lo <= b.hi)) {
        *lo = 1;
        *hi = 0;
        return;
    }
    auto k = [](double x) {
        long long v;
        memcpy(&v, &x, 8);
        return v ^ ((v >> 63) & 0x7FFFFFFFFFFFFFFFLL);
    };
    *lo = k(b.lo);
    *hi = k(b.hi);
}

SlopeConsts slope_consts(double cellsize, int method, int units) {
    const double cs = (double)(float)cellsize;  // MetaData::cellSize is a float (gpro/metaData.h:56)
    SlopeConsts k;
    k.k_fd = (float)(1.0 / (8.0 * cs));
    k.k_ffd = (float)(1.0 / (4.0 * cs));
    k.k_sd = (float)(1.0 / cs);
    k.k_sfd = (float)(1.0 / (2.0 * cs));
    k.k_tfd = (float)(1.0 / (6.0 * cs));
    k.k_tfdw = (float)(1.0 / ((4.0 + sqrt(8.0)) * cs));
    k.sqrt2 = (float)sqrt(2.0);
    k.sqrt2d = sqrt(2.0);
    k.k_md = (float)(1.0 / (cs * sqrt(2.0)));
    k.method = method;
    k.degrees = units == PARGO_SLOPE_DEGREES;
    return k;
}

// ---- staging of host buffers ----
struct Staged {
    InView in;   // device view of an input
    OutView out; // device view of an output
    bool host = false;
    const pargo_raster* user = nullptr;
    int64_t dpitch = 0;
};

int64_t round16(int64_t x) { return (x + 15) / 16 * 16; }

pargo_status stage_in(pargo_ctx* ctx, const pargo_raster* r, int slot_id, cudaStream_t st, Staged* s) {
    s->user = r;
    s->host = r->location == PARGO_HOST;
    if (!s->host) {
        s->in = InView{(const char*)r->data, pitch_of(r), r->dtype};
        return PARGO_OK;
    }
    const int64_t dp = round16(row_bytes(r));
    cudaError_t e;
    char* d = (char*)slot(ctx, slot_id, (size_t)(dp * r->rows), &e);
    if (!d) return cuda_fail(ctx, e, "staging input");
    CU(ctx, cudaMemcpy2DAsync(d, dp, r->data, pitch_of(r), row_bytes(r), r->rows, cudaMemcpyHostToDevice, st));
    s->in = InView{d, dp, r->dtype};
    s->dpitch = dp;
    return PARGO_OK;
}

pargo_status stage_out(pargo_ctx* ctx, pargo_raster* r, int slot_id, Staged* s) {
    s->user = r;
    s->host = r->location == PARGO_HOST;
    if (!s->host) {
        s->out = OutView{(char*)r->data, pitch_of(r), r->dtype, r->nodata};
        return PARGO_OK;
    }
    const int64_t dp = round16(row_bytes(r));
    cudaError_t e;
    char* d = (char*)slot(ctx, slot_id, (size_t)(dp * r->rows), &e);
    if (!d) return cuda_fail(ctx, e, "staging output");
    s->out = OutView{d, dp, r->dtype, r->nodata};
    s->dpitch = dp;
    return PARGO_OK;
}

// Rows [r0, r1) of a staged host output back to the host.
pargo_status unstage_rows(pargo_ctx* ctx, const Staged& s, int64_t r0, int64_t r1, cudaStream_t st) {
    if (!s.host || r1 <= r0) return PARGO_OK;
    const pargo_raster* r = s.user;
    CU(ctx, cudaMemcpy2DAsync((char*)r->data + r0 * pitch_of(r), pitch_of(r), s.out.base + r0 * s.dpitch, s.dpitch,
                              row_bytes(r), r1 - r0, cudaMemcpyDeviceToHost, st));
    return PARGO_OK;
}

pargo_status unstage_out(pargo_ctx* ctx, const Staged& s, cudaStream_t st) {
    if (!s.host) return PARGO_OK;
    const pargo_raster* r = s.user;
    CU(ctx, cudaMemcpy2DAsync(r->data, pitch_of(r), s.out.base, s.dpitch, row_bytes(r), r->rows,
                              cudaMemcpyDeviceToHost, st));
    return PARGO_OK;
}

pargo_status make_tma_map(pargo_ctx* ctx, CUtensorMap* map, const void* base, int64_t rows, int64_t cols,
                          int64_t pitch, int box_rows, int box_cols = 0, bool f64 = false) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return fail(ctx, PARGO_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)pitch};
    cuuint32_t box[2] = {(cuuint32_t)(box_cols ? box_cols : focal_tma_box_cols()), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(ctx, PARGO_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return PARGO_OK;
}

bool tma_ok(const InView& v) {
    return v.dtype == PARGO_F32 && ((uintptr_t)v.base % 16 == 0) && (v.pitch % 16 == 0);
}

// Outputs the TMA kernel can store directly (float4 slope, packed int8 codes).
bool fast_out_ok(const FocalParams& p) {
    if (p.do_slope && !(p.slope.dtype == PARGO_F32 && (uintptr_t)p.slope.base % 16 == 0 && p.slope.pitch % 16 == 0))
        return false;
    if (p.do_d8 && !(p.d8.dtype == PARGO_I8 && (uintptr_t)p.d8.base % 4 == 0 && p.d8.pitch % 4 == 0)) return false;
    return true;
}

pargo_status check_d8_out(pargo_ctx* ctx, const pargo_raster* d8, int dir_type) {
    if (d8->dtype == PARGO_I8) {
        if (dir_type != 8)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "I8 D8 output holds dir_type 8 codes only (bit sums reach 255)");
        if (d8->nodata < -128 || d8->nodata > 127 || d8->nodata != floor(d8->nodata))
            return fail(ctx, PARGO_ERR_INVALID_ARG, "I8 D8 output: nodata %g is not an int8 value", d8->nodata);
        if (d8->nodata >= -1 && d8->nodata <= 8)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "I8 D8 output: nodata %g collides with a D8 code", d8->nodata);
    }
    if (d8->dtype == PARGO_I16 && (d8->nodata < -32768 || d8->nodata > 32767 || d8->nodata != floor(d8->nodata)))
        return fail(ctx, PARGO_ERR_INVALID_ARG, "I16 D8 output: nodata %g is not an int16 value", d8->nodata);
    return PARGO_OK;
}

pargo_status finish_call(pargo_ctx* ctx, cudaStream_t st, bool sync) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel launch");
    if (sync) {
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "stream synchronize");
        int flag = 0;
        e = cudaMemcpy(&flag, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "error flag read");
        if (flag) {
            cudaMemset(ctx->d_error, 0, sizeof(int));
            return fail(ctx, PARGO_ERR_DEVICE_TIMEOUT, "a device-side wait exceeded its bound");
        }
    }
    return PARGO_OK;
}

// ---- persisted tuning cache (the file's format and reader: tune_cache.h) --
std::string device_signature(int dev) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return std::string();
    char buf[320];
    snprintf(buf, sizeof(buf), "sm_%d%d %d %s", prop.major, prop.minor, prop.multiProcessorCount, prop.name);
    return std::string(buf);
}

int variant_by_name(const std::string& name) {
    for (int v = 0; v < focal_num_variants(); v++)
        if (name == focal_variant_name(v)) return v;
    return -1;
}

int size_class(int64_t cells) {
    int c = 0;
    while (c < 63 && ((int64_t)1 << (c + 1)) <= cells) c++;
    return c;
}

// Focal kernel variant for a raster of `cells` cells: the environment
// (PARGO_FOCAL_VARIANT) first, then the context's autotuned choice for the
// size class, else variant 0.
int pick_variant(pargo_ctx* ctx, int64_t cells) {
    const char* env = getenv("PARGO_FOCAL_VARIANT");
    if (env && *env) {
        const int v = atoi(env);
        if (v >= 0 && v < focal_num_variants()) return v;
    }
    const int v = ctx->focal_variant[size_class(cells)];
    if (v >= 0) return v;
    // untuned: the strip walk from 4096^2 cells up (2.03 ms against the tiled
    // kernel's 3.6 ms on 32768^2), the tiled kernel below
    return cells >= (1LL << 24) ? focal_default_strip_variant() : 0;
}

// Slope + D8 over a float32 DEM with TMA-compatible rows by kernel variant v
// (a tiled variant, or the strip walk with its fix-up pass).
pargo_status launch_focal_variant(pargo_ctx* ctx, const InView& dem, const FocalParams& p, int fast_out, int v,
                                  cudaStream_t s) {
    pargo_status st;
    // the strip walk's fast path covers Horn rise/run slope and dirType 8
    const bool plain = (p.sk.method == PARGO_SLOPE_FD || !p.do_slope) && !p.sk.degrees && (!p.do_d8 || p.dir_type == 8);
    const bool strip = focal_variant_is_strip(v) && plain && fast_out && p.rows * ((p.cols + 3) / 4) < (1LL << 32);
    if (strip) {
        CUtensorMap ms, mp;
        if ((st = make_tma_map(ctx, &ms, dem.base, p.rows, p.cols, dem.pitch,
                               focal_strip_stage_rows(v, p.do_slope, p.do_d8))) != PARGO_OK)
            return st;
        if ((st = make_tma_map(ctx, &mp, dem.base, p.rows, p.cols, dem.pitch, 2)) != PARGO_OK) return st;
        cudaError_t e;
        uint32_t* slow = (uint32_t*)slot(ctx, kSlotStripSlow, focal_strip_slow_bytes(p.rows, p.cols), &e);
        if (!slow) return cuda_fail(ctx, e, "strip walk scratch");
        CU(ctx, launch_focal_strip(&ms, &mp, dem, p, fast_out, v, &ctx->d_counters[4], slow, ctx->num_sms, s));
        return PARGO_OK;
    }
    if (focal_variant_is_strip(v)) v = 0;
    CUtensorMap map;
    if ((st = make_tma_map(ctx, &map, dem.base, p.rows, p.cols, dem.pitch, focal_variant_rows(v) + 2)) != PARGO_OK)
        return st;
    CU(ctx, launch_focal_tma(&map, p, fast_out, v, ctx->num_sms, s));
    return PARGO_OK;
}

pargo_status focal_impl(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* slope, pargo_raster* d8,
                        const pargo_nbr* nbr, int method, int units, int dir_type, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if ((st = check_raster(ctx, dem, "dem")) != PARGO_OK) return st;
    if (dem->dtype != PARGO_F32 && dem->dtype != PARGO_F64)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "dem must be F32 or F64");
    if ((st = check_dims(ctx, dem)) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    if (!slope && !d8) return fail(ctx, PARGO_ERR_INVALID_ARG, "no output requested");
    if (slope) {
        if ((st = check_raster(ctx, slope, "slope")) != PARGO_OK) return st;
        if ((st = check_same(ctx, dem, slope, "slope")) != PARGO_OK) return st;
        if (slope->dtype != PARGO_F32 && slope->dtype != PARGO_F64)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "slope must be F32 or F64");
        if (method < 0 || method > 6) return fail(ctx, PARGO_ERR_INVALID_ARG, "unknown slope method %d", method);
        if (units != PARGO_SLOPE_RATIO && units != PARGO_SLOPE_DEGREES)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "unknown slope units %d", units);
    }
    if (d8) {
        if ((st = check_raster(ctx, d8, "d8")) != PARGO_OK) return st;
        if ((st = check_same(ctx, dem, d8, "d8")) != PARGO_OK) return st;
        if ((st = check_d8_out(ctx, d8, dir_type)) != PARGO_OK) return st;
    }
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sdem, sslope, sd8;
    if ((st = stage_in(ctx, dem, kSlotIn0, s, &sdem)) != PARGO_OK) return st;
    if (slope && (st = stage_out(ctx, slope, kSlotOut0, &sslope)) != PARGO_OK) return st;
    if (d8 && (st = stage_out(ctx, d8, kSlotOut1, &sd8)) != PARGO_OK) return st;

    FocalParams p{};
    p.rows = dem->rows;
    p.cols = dem->cols;
    p.nd6f = float_band(dem->nodata, kEpsHydro);
    p.nd7f = float_band(dem->nodata, kEpsSlope);
    p.nd6d = double_band(dem->nodata, kEpsHydro);
    p.nd7d = double_band(dem->nodata, kEpsSlope);
    p.sk = slope_consts(dem->cellsize, method, units);
    p.do_slope = slope != nullptr;
    p.do_d8 = d8 != nullptr;
    p.dir_type = dir_type;
    if (slope) p.slope = sslope.out;
    if (d8) p.d8 = sd8.out;
    p.fallbacks = &ctx->d_counters[0];
    p.error_flag = ctx->d_error;
    CU(ctx, cudaMemsetAsync(&ctx->d_counters[0], 0, sizeof(unsigned long long), s));

    const bool f64_tma = sdem.in.dtype == PARGO_F64 && (uintptr_t)sdem.in.base % 16 == 0 && sdem.in.pitch % 16 == 0;
    if (f64_tma) {
        Focal64Params q{};
        q.f = p;
        q.wpitch = sdem.in.pitch;
        q.nodata_is_inf = 0;
        CUtensorMap map;
        if ((st = make_tma_map(ctx, &map, sdem.in.base, p.rows, p.cols, sdem.in.pitch, focal64_tile_rows() + 2,
                               focal64_box_cols(), true)) != PARGO_OK)
            return st;
        CU(ctx, launch_focal64_tma(&map, q, ctx->num_sms, s));
    } else if (tma_ok(sdem.in)) {
        const int v = pick_variant(ctx, p.rows * p.cols);
        if ((st = launch_focal_variant(ctx, sdem.in, p, fast_out_ok(p) ? 1 : 0, v, s)) != PARGO_OK) return st;
    } else {
        CU(ctx, launch_focal_generic(sdem.in, p, s));
    }
    const bool host_io = sdem.host || (slope && sslope.host) || (d8 && sd8.host);
    if (slope && (st = unstage_out(ctx, sslope, s)) != PARGO_OK) return st;
    if (d8 && (st = unstage_out(ctx, sd8, s)) != PARGO_OK) return st;
    if (host_io) {
        unsigned long long fb = 0;
        CU(ctx, cudaMemcpyAsync(&fb, &ctx->d_counters[0], sizeof(fb), cudaMemcpyDeviceToHost, s));
        if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
        ctx->last_fallbacks = (int64_t)fb;
        return PARGO_OK;
    }
    ctx->last_fallbacks = -1;  // not read back for asynchronous device calls
    return finish_call(ctx, s, false);
}

}  // namespace

extern "C" {

int pargo_abi_version(void) { return PARGO_ABI_VERSION; }

const char* pargo_last_error(const pargo_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int64_t pargo_last_d8_fallbacks(const pargo_ctx* ctx) { return ctx ? ctx->last_fallbacks : -1; }

pargo_status pargo_create(int device, pargo_ctx** out) {
    if (!out) return PARGO_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return PARGO_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return PARGO_ERR_INVALID_ARG;
    pargo_ctx* ctx = new pargo_ctx();
    ctx->device = device;
    if ((e = cudaSetDevice(device)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->ev_a, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->ev_b, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreate(&ctx->ev_t0)) != cudaSuccess || (e = cudaEventCreate(&ctx->ev_t1)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->d_counters, 8 * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMalloc(&ctx->d_error, sizeof(int))) != cudaSuccess ||
        (e = cudaMemset(ctx->d_counters, 0, 8 * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMemset(ctx->d_error, 0, sizeof(int))) != cudaSuccess) {
        pargo_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? PARGO_ERR_OUT_OF_MEMORY : PARGO_ERR_CUDA;
    }
    // the autotuner's persisted choices for this device
    ctx->device_sig = device_signature(device);
    for (const TuneEntry& t : read_tune_cache(tune_cache_path())) {
        if (t.op != "slope_d8" || t.device != ctx->device_sig) continue;
        const int v = variant_by_name(t.variant);
        if (v >= 0) ctx->focal_variant[t.size_class] = v;
    }
    *out = ctx;
    return PARGO_OK;
}

pargo_status pargo_destroy(pargo_ctx* ctx) {
    if (!ctx) return PARGO_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    if (ctx->fill_graph) cudaGraphExecDestroy(ctx->fill_graph);
    for (auto& s : ctx->slots)
        if (s.p) cudaFree(s.p);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->d_error) cudaFree(ctx->d_error);
    if (ctx->ev_a) cudaEventDestroy(ctx->ev_a);
    if (ctx->ev_b) cudaEventDestroy(ctx->ev_b);
    if (ctx->ev_t0) cudaEventDestroy(ctx->ev_t0);
    if (ctx->ev_t1) cudaEventDestroy(ctx->ev_t1);
    for (cudaEvent_t& ev : ctx->ev_band)
        if (ev) cudaEventDestroy(ev);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
    return PARGO_OK;
}

pargo_status pargo_nbr_parse(const char* text, pargo_nbr* out) {
    if (!text || !out) return PARGO_ERR_INVALID_ARG;
    std::istringstream is(text);
    int n = 0;
    if (!(is >> n) || n <= 0) return PARGO_ERR_INVALID_ARG;  // empty set (neighborhood.h:113-117)
    std::vector<std::pair<int, int>> v;
    if (n >= 100) {  // automatic sqrt(n) x sqrt(n) square (neighborhood.h:634-646)
        const int half = ((int)sqrt((double)n)) / 2;
        for (int i = -half; i <= half; i++)
            for (int j = -half; j <= half; j++) v.emplace_back(i, j);
    } else {
        for (int k = 0; k < n; k++) {
            int r, c;
            double w;
            if (!(is >> r >> c >> w)) return PARGO_ERR_INVALID_ARG;
            v.emplace_back(r, c);
        }
    }
    bool origin = false;
    for (size_t i = 0; i < v.size(); i++) {
        if (v[i].first == 0 && v[i].second == 0) origin = true;
        for (size_t j = 0; j < i; j++)
            if (v[j] == v[i]) return PARGO_ERR_INVALID_ARG;  // duplicate (neighborhood.h:131-137)
    }
    if (!origin) return PARGO_ERR_INVALID_ARG;  // must hold (0,0) (neighborhood.h:118-123)
    pargo_nbr r{(int32_t)v.size(), v[0].first, v[0].second, v[0].first, v[0].second};
    for (auto& p : v) {
        r.min_row = std::min(r.min_row, p.first);
        r.min_col = std::min(r.min_col, p.second);
        r.max_row = std::max(r.max_row, p.first);
        r.max_col = std::max(r.max_col, p.second);
    }
    *out = r;
    return PARGO_OK;
}

pargo_status pargo_slope(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* slope, const pargo_nbr* nbr,
                         int method, int units, void* stream) {
    if (!slope) return fail(ctx, PARGO_ERR_INVALID_ARG, "slope output is required");
    return focal_impl(ctx, dem, slope, nullptr, nbr, method, units, 8, stream);
}

pargo_status pargo_d8(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* d8, const pargo_nbr* nbr, int dir_type,
                      void* stream) {
    if (!d8) return fail(ctx, PARGO_ERR_INVALID_ARG, "d8 output is required");
    return focal_impl(ctx, dem, nullptr, d8, nbr, 0, 0, dir_type, stream);
}

pargo_status pargo_slope_d8(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* slope, pargo_raster* d8,
                            const pargo_nbr* nbr, int method, int units, int dir_type, void* stream) {
    return focal_impl(ctx, dem, slope, d8, nbr, method, units, dir_type, stream);
}

int pargo_focal_num_variants(void) { return focal_num_variants(); }

const char* pargo_focal_variant_name(int v) { return focal_variant_name(v); }

int pargo_focal_variant(const pargo_ctx* ctx, int64_t cells) {
    if (!ctx || cells < 0) return -1;
    return pick_variant(const_cast<pargo_ctx*>(ctx), cells);
}

pargo_status pargo_tune_focal(pargo_ctx* ctx, const pargo_raster* dem, int reps, int* best, float* times_ms,
                              int max_times) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if ((st = check_raster(ctx, dem, "dem")) != PARGO_OK) return st;
    if ((st = check_dims(ctx, dem)) != PARGO_OK) return st;
    if (dem->dtype != PARGO_F32 || dem->location != PARGO_DEVICE || (uintptr_t)dem->data % 16 || pitch_of(dem) % 16)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "tune: dem must be an F32 device raster with 16-byte aligned rows");
    if (reps < 1) reps = 1;
    CU(ctx, cudaSetDevice(ctx->device));
    const int64_t rows = dem->rows, cols = dem->cols;
    const int64_t sp = round16(cols * 4), cp = round16(cols);
    cudaError_t e;
    char* sbuf = (char*)slot(ctx, kSlotOut0, (size_t)(sp * rows), &e);
    char* cbuf = sbuf ? (char*)slot(ctx, kSlotOut1, (size_t)(cp * rows), &e) : nullptr;
    if (!sbuf || !cbuf) return cuda_fail(ctx, e, "tune outputs");
    FocalParams p{};
    p.rows = rows;
    p.cols = cols;
    p.nd6f = float_band(dem->nodata, kEpsHydro);
    p.nd7f = float_band(dem->nodata, kEpsSlope);
    p.sk = slope_consts(dem->cellsize, PARGO_SLOPE_FD, PARGO_SLOPE_RATIO);
    p.do_slope = 1;
    p.do_d8 = 1;
    p.dir_type = 8;
    p.slope = OutView{sbuf, sp, PARGO_F32, dem->nodata};
    p.d8 = OutView{cbuf, cp, PARGO_I8, -128.0};
    p.fallbacks = &ctx->d_counters[0];
    p.error_flag = ctx->d_error;
    float best_ms = 1e30f;
    int best_v = 0;
    const InView din{(const char*)dem->data, pitch_of(dem), PARGO_F32};
    for (int v = 0; v < focal_num_variants(); v++) {
        if ((st = launch_focal_variant(ctx, din, p, 1, v, ctx->own)) != PARGO_OK) return st;  // warm
        CU(ctx, cudaEventRecord(ctx->ev_t0, ctx->own));
        for (int r = 0; r < reps; r++)
            if ((st = launch_focal_variant(ctx, din, p, 1, v, ctx->own)) != PARGO_OK) return st;
        CU(ctx, cudaEventRecord(ctx->ev_t1, ctx->own));
        CU(ctx, cudaEventSynchronize(ctx->ev_t1));
        float ms = 0.0f;
        CU(ctx, cudaEventElapsedTime(&ms, ctx->ev_t0, ctx->ev_t1));
        ms /= (float)reps;
        if (times_ms && v < max_times) times_ms[v] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best_v = v;
        }
    }
    const int sc = size_class(rows * cols);
    ctx->focal_variant[sc] = best_v;
    if (best) *best = best_v;
    if ((st = finish_call(ctx, ctx->own, true)) != PARGO_OK) return st;
    // persist the choice (a cache that cannot be written only costs the next
    // context a re-tune: not an error)
    const std::string path = tune_cache_path();
    if (!path.empty() && !ctx->device_sig.empty()) {
        std::vector<TuneEntry> all = read_tune_cache(path);
        all.erase(std::remove_if(all.begin(), all.end(),
                                 [&](const TuneEntry& t) {
                                     return t.op == "slope_d8" && t.device == ctx->device_sig && t.size_class == sc;
                                 }),
                  all.end());
        TuneEntry t;
        t.op = "slope_d8";
        t.device = ctx->device_sig;
        t.size_class = sc;
        t.variant = focal_variant_name(best_v);
        t.ms = best_ms;
        all.push_back(t);
        write_tune_cache(path, all);
    }
    return PARGO_OK;
}

// ------------------------------------------------------------------ fill --
}  // extern "C"

namespace {

// Runs the pit removal of `dem` (F32, staged) into the context's level buffer
// (dense rows x cols doubles, +inf on nodata levels) and returns its params.
pargo_status fill_core(pargo_ctx* ctx, const Staged& sdem, const pargo_raster* dem, const pargo_fill_opts& o,
                       FillParams* out_p, pargo_fill_stats* stats, bool* converged, cudaStream_t s) {
    const int64_t rows = dem->rows, cols = dem->cols;
    const int T = fill_tile_rows();
    FillParams p{};
    p.rows = rows;
    p.cols = cols;
    p.dem = sdem.in.base;
    p.dem_pitch = sdem.in.pitch;
    p.dem_f64 = dem->dtype == PARGO_F64;
    p.nd6f = float_band(dem->nodata, kEpsHydro);
    p.nd6d = double_band(dem->nodata, kEpsHydro);
    p.gap = o.gap;
    p.init_level = o.init_level;
    p.tiles_y = (rows + T - 1) / T;
    p.tiles_x = (cols + T - 1) / T;
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    if (ntiles >= INT32_MAX) return fail(ctx, PARGO_ERR_INVALID_ARG, "fill: raster too large");
    cudaError_t e;
    p.w_stride = (cols + 1) / 2 * 2;  // 16-byte rows: the levels can be TMA-loaded
    p.w = (double*)slot(ctx, kSlotFillW, (size_t)(rows * p.w_stride) * sizeof(double), &e);
    if (!p.w) return cuda_fail(ctx, e, "fill levels");
    // two worklists (or one ring) of ntiles ids, 8 round counters, 8 queue words (u64)
    int32_t* lists = (int32_t*)slot(ctx, kSlotFillLists, (size_t)(2 * ntiles + 8) * sizeof(int32_t) + 8 * 8 + 8, &e);
    if (!lists) return cuda_fail(ctx, e, "fill worklists");
    // per tile: its state word, then 5 words of changed halo cells
    int32_t* queued = (int32_t*)slot(ctx, kSlotFillQueued, (size_t)ntiles * 6 * sizeof(int32_t), &e);
    if (!queued) return cuda_fail(ctx, e, "fill queue flags");
    FillScratch sc{};
    sc.list_a = lists;
    sc.list_b = lists + ntiles;
    sc.counts = lists + 2 * ntiles;
    sc.queued = queued;
    sc.visits = &ctx->d_counters[1];
    sc.changed = &ctx->d_counters[2];
    sc.active = &ctx->d_counters[4];
    sc.iters = &ctx->d_counters[5];
    sc.ring = lists;
    sc.ring_cap = 2 * ntiles;
    sc.halo_chg = (uint32_t*)(queued + ntiles);
    sc.q = (unsigned long long*)(((uintptr_t)(lists + 2 * ntiles + 8) + 7) & ~(uintptr_t)7);
    const char* force_rounds = getenv("PARGO_FILL_ROUNDS");
    const bool persistent = o.max_rounds <= 0 && !(force_rounds && force_rounds[0] == '1');
    CU(ctx, cudaMemsetAsync(ctx->d_counters, 0, 8 * sizeof(unsigned long long), s));
    {
        cudaError_t ee = fill_init(p, sc, s);
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "fill init");
    }
    if (persistent) {
        // One launch: tiles pop from and push to a device ring until the
        // pending count reaches zero.  Waits give up after ~2 s without progress.
        const long long patience = 4000000000LL;  // SM cycles
        unsigned long long* hp = (unsigned long long*)pinned(ctx, 128, &e);
        if (!hp) return cuda_fail(ctx, e, "pinned counters");
        CU(ctx, cudaEventRecord(ctx->ev_t0, s));
        {
            cudaError_t ee = fill_persistent(p, sc, patience, ctx->num_sms, s);
            if (ee != cudaSuccess) return cuda_fail(ctx, ee, "fill persistent launch");
        }
        CU(ctx, cudaEventRecord(ctx->ev_t1, s));
        CU(ctx, cudaMemcpyAsync(hp, sc.q, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        CU(ctx, cudaMemcpyAsync(hp + 8, ctx->d_counters, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        CU(ctx, cudaStreamSynchronize(s));
        if (hp[4] != 0)
            return fail(ctx, PARGO_ERR_DEVICE_TIMEOUT,
                        hp[4] == 1   ? "fill: a device wait for queued tiles made no progress"
                        : hp[4] == 2 ? "fill: a device wait for a free queue slot made no progress"
                                     : "fill: a tile state did not settle");
        *converged = hp[2] == 0;
        float ms = 0.0f;
        CU(ctx, cudaEventElapsedTime(&ms, ctx->ev_t0, ctx->ev_t1));
        if (stats) {
            stats->rounds = 1;
            stats->active_rounds = 1;
            stats->tile_visits = (int64_t)hp[8 + 1];
            stats->local_iterations = (int64_t)hp[8 + 5];
            stats->raised_cells = 0;
            stats->rounds_ms = ms;
        }
        *out_p = p;
        return PARGO_OK;
    }
    // Rounds run on the context's own stream, as CUDA-graph launches of
    // kRoundsPerGraph rounds (an even number, so list A is current again); a
    // round cap below 16 shortens the graph so the cap is honoured exactly
    // (rounded up to even).
    int kRoundsPerGraph = 16;
    if (o.max_rounds > 0 && o.max_rounds < 16) kRoundsPerGraph = (int)((o.max_rounds + 1) / 2 * 2);
    CU(ctx, cudaEventRecord(ctx->ev_a, s));
    CU(ctx, cudaStreamWaitEvent(ctx->own, ctx->ev_a, 0));
    char keybuf[256];
    snprintf(keybuf, sizeof(keybuf), "%p %p %p %p %lld %lld %a %a %a %a %a %a %lld %d %d", (void*)p.w, p.dem,
             (void*)lists, (void*)queued, (long long)rows, (long long)cols, p.gap, p.init_level, (double)p.nd6f.lo,
             (double)p.nd6f.hi, p.nd6d.lo, p.nd6d.hi, (long long)p.dem_pitch, p.dem_f64, kRoundsPerGraph);
    if (!ctx->fill_graph || ctx->fill_graph_key != keybuf) {
        if (ctx->fill_graph) {
            cudaGraphExecDestroy(ctx->fill_graph);
            ctx->fill_graph = nullptr;
        }
        cudaGraph_t g;
        CU(ctx, cudaStreamBeginCapture(ctx->own, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaSuccess;
        for (int r = 0; r < kRoundsPerGraph && ce == cudaSuccess; r++)
            ce = fill_round(p, sc, r & 1, ctx->num_sms, ctx->own);
        cudaError_t ee = cudaStreamEndCapture(ctx->own, &g);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "fill round capture");
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "fill graph capture");
        ee = cudaGraphInstantiate(&ctx->fill_graph, g, 0);
        cudaGraphDestroy(g);
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "fill graph instantiate");
        ctx->fill_graph_key = keybuf;
    }
    unsigned long long* hp = (unsigned long long*)pinned(ctx, 128, &e);
    if (!hp) return cuda_fail(ctx, e, "pinned counters");
    int32_t* hc = (int32_t*)(hp + 8);
    int64_t rounds = 0;
    *converged = false;
    CU(ctx, cudaEventRecord(ctx->ev_t0, ctx->own));
    for (;;) {
        CU(ctx, cudaGraphLaunch(ctx->fill_graph, ctx->own));
        rounds += kRoundsPerGraph;
        CU(ctx, cudaMemcpyAsync(hc, sc.counts, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->own));
        CU(ctx, cudaStreamSynchronize(ctx->own));
        if (hc[0] == 0 && hc[1] == 0) {
            *converged = true;
            break;
        }
        if (o.max_rounds > 0 && rounds >= o.max_rounds) break;
    }
    CU(ctx, cudaEventRecord(ctx->ev_t1, ctx->own));
    CU(ctx, cudaEventRecord(ctx->ev_b, ctx->own));
    CU(ctx, cudaStreamWaitEvent(s, ctx->ev_b, 0));
    CU(ctx, cudaEventSynchronize(ctx->ev_t1));
    float ms = 0.0f;
    CU(ctx, cudaEventElapsedTime(&ms, ctx->ev_t0, ctx->ev_t1));
    CU(ctx, cudaMemcpy(hp, ctx->d_counters, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    if (stats) {
        stats->rounds = rounds;
        stats->active_rounds = (int64_t)hp[4];
        stats->tile_visits = (int64_t)hp[1];
        stats->local_iterations = (int64_t)hp[5];
        stats->raised_cells = 0;
        stats->rounds_ms = ms;
    }
    *out_p = p;
    return PARGO_OK;
}

pargo_status check_fill_args(pargo_ctx* ctx, const pargo_raster* dem, const pargo_nbr* nbr,
                             const pargo_fill_opts* opts, pargo_fill_opts* o) {
    pargo_status st;
    if ((st = check_raster(ctx, dem, "dem")) != PARGO_OK) return st;
    if (dem->dtype != PARGO_F32 && dem->dtype != PARGO_F64)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "fill: dem must be F32 or F64");
    if ((st = check_dims(ctx, dem)) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    *o = pargo_fill_opts{0.0005, 10000.0, 0};
    if (opts) *o = *opts;
    if (!(o->gap > 0.0) || !isfinite(o->gap) || !isfinite(o->init_level))
        return fail(ctx, PARGO_ERR_INVALID_ARG, "fill: gap must be positive and finite");
    return PARGO_OK;
}

}  // namespace

extern "C" {

pargo_status pargo_fill(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* wdem, const pargo_nbr* nbr,
                        const pargo_fill_opts* opts, pargo_fill_stats* stats, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    pargo_fill_opts o;
    if ((st = check_fill_args(ctx, dem, nbr, opts, &o)) != PARGO_OK) return st;
    if ((st = check_raster(ctx, wdem, "wdem")) != PARGO_OK) return st;
    if ((st = check_same(ctx, dem, wdem, "wdem")) != PARGO_OK) return st;
    if (wdem->dtype != PARGO_F64 && wdem->dtype != PARGO_F32)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "fill: wdem must be F64 or F32");
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sdem, sw;
    if ((st = stage_in(ctx, dem, kSlotIn0, s, &sdem)) != PARGO_OK) return st;
    if ((st = stage_out(ctx, wdem, kSlotOut0, &sw)) != PARGO_OK) return st;
    FillParams p;
    bool converged = false;
    pargo_fill_stats local{};
    if ((st = fill_core(ctx, sdem, dem, o, &p, &local, &converged, s)) != PARGO_OK) return st;
    {
        cudaError_t ee = fill_finish(p, sw.out, &ctx->d_counters[3], s);
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "fill finish");
    }
    if ((st = unstage_out(ctx, sw, s)) != PARGO_OK) return st;
    cudaError_t e;
    unsigned long long* hp = (unsigned long long*)pinned(ctx, 128, &e);
    if (!hp) return cuda_fail(ctx, e, "pinned counters");
    CU(ctx, cudaMemcpyAsync(hp, &ctx->d_counters[3], sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
    local.raised_cells = (int64_t)hp[0];
    if (stats) *stats = local;
    if (!converged)
        return fail(ctx, PARGO_ERR_NOT_CONVERGED, "fill: worklist not empty after %lld rounds",
                    (long long)local.rounds);
    return PARGO_OK;
}

// ------------------------------------------------------------ batch fill --
// Pit removal of many rasters in one persistent relaxation: the rasters are
// shelf-packed into one mosaic DEM (each raster's ring and nodata cells, and
// the mosaic cells outside the rasters, become nodata -- two neighbouring
// rasters meet at two rows or columns of nodata levels, so they never see
// each other), the mosaic is filled by the single-raster machinery, and each
// raster's rectangle of levels goes to its own output.  Rasters whose nodata
// differ from the first one's (a common nodata is what the mosaic needs) are
// filled one by one instead.
static pargo_status batch_fill_one_by_one(pargo_ctx* ctx, int count, const pargo_raster* dems, pargo_raster* wdems,
                                   const pargo_nbr* nbr, const pargo_fill_opts* opts, pargo_fill_stats* stats,
                                   void* stream) {
    pargo_fill_stats total{};
    for (int i = 0; i < count; i++) {
        pargo_fill_stats one{};
        pargo_status st = pargo_fill(ctx, &dems[i], &wdems[i], nbr, opts, &one, stream);
        if (st != PARGO_OK) return st;
        total.rounds += one.rounds;
        total.active_rounds += one.active_rounds;
        total.tile_visits += one.tile_visits;
        total.local_iterations += one.local_iterations;
        total.raised_cells += one.raised_cells;
        total.rounds_ms += one.rounds_ms;
    }
    if (stats) *stats = total;
    return PARGO_OK;
}

pargo_status pargo_batch_fill(pargo_ctx* ctx, int count, const pargo_raster* dems, pargo_raster* wdems,
                                         const pargo_nbr* nbr, const pargo_fill_opts* opts, pargo_fill_stats* stats,
                                         void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (count < 0 || (count > 0 && (!dems || !wdems)))
        return fail(ctx, PARGO_ERR_INVALID_ARG, "batch fill: bad count, dems or wdems");
    if (stats) *stats = pargo_fill_stats{};
    if (count == 0) return PARGO_OK;
    pargo_status st;
    pargo_fill_opts o;
    bool mosaic = true;
    for (int i = 0; i < count; i++) {
        if ((st = check_fill_args(ctx, &dems[i], nbr, opts, &o)) != PARGO_OK) return st;
        if ((st = check_raster(ctx, &wdems[i], "batch wdem")) != PARGO_OK) return st;
        if ((st = check_same(ctx, &dems[i], &wdems[i], "batch wdem")) != PARGO_OK) return st;
        if (wdems[i].dtype != PARGO_F64 && wdems[i].dtype != PARGO_F32)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "batch fill: wdem %d must be F64 or F32", i);
        if (dems[i].location != PARGO_DEVICE || wdems[i].location != PARGO_DEVICE)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "batch fill: raster %d must be on the device", i);
        if (dems[i].dtype != dems[0].dtype || !(dems[i].nodata == dems[0].nodata)) mosaic = false;
    }
    const bool f64 = dems[0].dtype == PARGO_F64;
    const Band<float> bf = float_band(dems[0].nodata, kEpsHydro);
    const Band<double> bd = double_band(dems[0].nodata, kEpsHydro);
    if (!f64 && !(bf.lo <= bf.hi)) mosaic = false;  // no float value stands for this nodata
    if (!(bd.lo <= bd.hi)) mosaic = false;
    if (!mosaic) return batch_fill_one_by_one(ctx, count, dems, wdems, nbr, opts, stats, stream);
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    // Shelf packing: tallest rasters first, left to right on shelves of the
    // mosaic's width (at least the widest raster, about square overall).
    std::vector<int> order(count);
    int64_t total = 0, max_cols = 0, max_cells = 0;
    for (int i = 0; i < count; i++) {
        order[i] = i;
        total += dems[i].rows * dems[i].cols;
        max_cols = std::max(max_cols, dems[i].cols);
        max_cells = std::max(max_cells, dems[i].rows * dems[i].cols);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return dems[a].rows > dems[b].rows; });
    const int64_t width = std::max(max_cols, (int64_t)ceil(sqrt((double)total * 1.15)));
    std::vector<FillBatchItem> items(count);
    int64_t x = 0, y = 0, shelf = 0;
    for (int k = 0; k < count; k++) {
        const int i = order[k];
        if (x + dems[i].cols > width) {
            y += shelf;
            x = 0;
            shelf = 0;
        }
        FillBatchItem& it = items[k];
        it.dem = dems[i].data;
        it.pitch = pitch_of(&dems[i]);
        it.rows = dems[i].rows;
        it.cols = dems[i].cols;
        it.oy = y;
        it.ox = x;
        it.nd6f = bf;
        it.nd6d = bd;
        it.out = OutView{(char*)wdems[i].data, pitch_of(&wdems[i]), wdems[i].dtype, wdems[i].nodata};
        x += dems[i].cols;
        shelf = std::max(shelf, dems[i].rows);
    }
    const int64_t mrows = std::max<int64_t>(y + shelf, 3), mcols = std::max<int64_t>(width, 3);
    if (mrows > INT32_MAX || mcols > INT32_MAX) return fail(ctx, PARGO_ERR_INVALID_ARG, "batch fill: batch too large");
    const int64_t es = f64 ? 8 : 4;
    const int64_t mstride = (mcols * es + 15) / 16 * 16 / es;
    cudaError_t e;
    void* md = slot(ctx, kSlotFillMosaic, (size_t)(mrows * mstride * es), &e);
    if (!md) return cuda_fail(ctx, e, "batch fill mosaic");
    FillBatchItem* ditems = (FillBatchItem*)slot(ctx, kSlotFillItems, (size_t)count * sizeof(FillBatchItem), &e);
    if (!ditems) return cuda_fail(ctx, e, "batch fill table");
    CU(ctx, cudaMemcpyAsync(ditems, items.data(), (size_t)count * sizeof(FillBatchItem), cudaMemcpyHostToDevice, s));
    // the stored nodata: a value of the batch's own nodata band
    const double nd_store = f64 ? dems[0].nodata : (double)bf.lo;
    {
        cudaError_t ee = fill_mosaic_pack(ditems, count, max_cells, md, mrows, mstride, f64 ? 1 : 0, nd_store, s);
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "batch fill pack");
    }
    pargo_raster mr{};
    mr.data = md;
    mr.dtype = dems[0].dtype;
    mr.location = PARGO_DEVICE;
    mr.rows = mrows;
    mr.cols = mcols;
    mr.pitch = mstride * es;
    mr.nodata = dems[0].nodata;
    mr.cellsize = dems[0].cellsize;
    Staged sm;
    sm.in = InView{(const char*)md, mstride * es, mr.dtype};
    FillParams p;
    bool converged = false;
    pargo_fill_stats local{};
    if ((st = fill_core(ctx, sm, &mr, o, &p, &local, &converged, s)) != PARGO_OK) return st;
    {
        cudaError_t ee = fill_mosaic_finish(p, ditems, count, max_cells, &ctx->d_counters[3], s);
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "batch fill finish");
    }
    unsigned long long* hp = (unsigned long long*)pinned(ctx, 128, &e);
    if (!hp) return cuda_fail(ctx, e, "pinned counters");
    CU(ctx, cudaMemcpyAsync(hp, &ctx->d_counters[3], sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
    local.raised_cells = (int64_t)hp[0];
    if (stats) *stats = local;
    if (!converged)
        return fail(ctx, PARGO_ERR_NOT_CONVERGED, "batch fill: worklist not empty after %lld rounds",
                    (long long)local.rounds);
    return PARGO_OK;
}

// SCA by tiled subtree sums: scratch, launches (stream-ordered), and the
// check of the completion counts once the stream has been synchronised.
pargo_status sca_launch(pargo_ctx* ctx, const ScaParams& q, cudaStream_t s, const char* what) {
    const int64_t n = q.rows * q.cols;
    const int64_t nodes = ((q.rows + kScaTile - 1) / kScaTile) * ((q.cols + kScaTile - 1) / kScaTile) * kScaSlots;
    if (nodes >= INT32_MAX) return fail(ctx, PARGO_ERR_INVALID_ARG, "%s: raster too large", what);
    cudaError_t e;
    ScaScratch sc{};
    sc.conv = (unsigned long long*)slot(ctx, kSlotScaConv, (size_t)n * 8, &e);
    if (!sc.conv) return cuda_fail(ctx, e, "sca totals");
    sc.ship = (unsigned long long*)slot(ctx, kSlotScaShip, (size_t)n * 8, &e);
    if (!sc.ship) return cuda_fail(ctx, e, "sca flags");
    sc.counters = (unsigned long long*)slot(ctx, kSlotScaCounters, 8 * sizeof(unsigned long long), &e);
    if (!sc.counters) return cuda_fail(ctx, e, "sca counters");
    sc.forest = (uint32_t*)slot(ctx, kSlotScaForest, (size_t)n * 4, &e);
    if (!sc.forest) return cuda_fail(ctx, e, "sca tile forests");
    void* tb = slot(ctx, kSlotScaTiles, sca_tiles_bytes(q.rows, q.cols), &e);
    if (!tb) return cuda_fail(ctx, e, "sca tile forest");
    const ScaTiles T = sca_tiles_layout(tb, q.rows, q.cols);
    cudaError_t ee = sca_run_tiled(q, sc, T, s);
    if (ee != cudaSuccess) return cuda_fail(ctx, ee, what);
    return PARGO_OK;
}

// hp: the 8 SCA counters copied to the host after the stream finished.
pargo_status sca_check(pargo_ctx* ctx, const unsigned long long* hp, const char* what) {
    if (hp[6] != 0)
        return fail(ctx, PARGO_ERR_CYCLE, "%s: %llu inflows from the raster's ring (never released)", what, hp[6]);
    if (hp[0] != hp[1] || hp[4] != hp[5])
        return fail(ctx, PARGO_ERR_CYCLE, "%s: %llu of %llu valid cells and %llu of %llu tile exits completed (cycle)",
                    what, hp[0], hp[1], hp[5], hp[4]);
    return PARGO_OK;
}

pargo_status pargo_hydro_pipeline(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* wdem, pargo_raster* slope,
                                  pargo_raster* d8, pargo_raster* sca, const pargo_nbr* nbr,
                                  const pargo_fill_opts* opts, int slope_method, int slope_units, int sca_contract,
                                  pargo_fill_stats* stats, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    pargo_fill_opts o;
    if ((st = check_fill_args(ctx, dem, nbr, opts, &o)) != PARGO_OK) return st;
    if (!wdem && !slope && !d8 && !sca) return fail(ctx, PARGO_ERR_INVALID_ARG, "pipeline: no output requested");
    if (wdem) {
        if ((st = check_raster(ctx, wdem, "wdem")) != PARGO_OK) return st;
        if ((st = check_same(ctx, dem, wdem, "wdem")) != PARGO_OK) return st;
        if (wdem->dtype != PARGO_F64 && wdem->dtype != PARGO_F32)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "pipeline: wdem must be F64 or F32");
    }
    if (slope) {
        if ((st = check_raster(ctx, slope, "slope")) != PARGO_OK) return st;
        if ((st = check_same(ctx, dem, slope, "slope")) != PARGO_OK) return st;
        if (slope->dtype != PARGO_F32 && slope->dtype != PARGO_F64)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "pipeline: slope must be F32 or F64");
        if (slope_method < 0 || slope_method > 6)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "unknown slope method %d", slope_method);
        if (slope_units != PARGO_SLOPE_RATIO && slope_units != PARGO_SLOPE_DEGREES)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "unknown slope units %d", slope_units);
    }
    if (d8) {
        if ((st = check_raster(ctx, d8, "d8")) != PARGO_OK) return st;
        if ((st = check_same(ctx, dem, d8, "d8")) != PARGO_OK) return st;
        if ((st = check_d8_out(ctx, d8, 8)) != PARGO_OK) return st;
    }
    if (sca) {
        if ((st = check_raster(ctx, sca, "sca")) != PARGO_OK) return st;
        if ((st = check_same(ctx, dem, sca, "sca")) != PARGO_OK) return st;
        if (sca->dtype != PARGO_F64 && sca->dtype != PARGO_F32)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "pipeline: sca must be F64 or F32");
        if (sca_contract != PARGO_SCA_CONVERGED && sca_contract != PARGO_SCA_SHIPPED)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "unknown SCA contract %d", sca_contract);
    }
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sdem, sw, ss, sd, sa;
    if ((st = stage_in(ctx, dem, kSlotIn0, s, &sdem)) != PARGO_OK) return st;
    if (wdem && (st = stage_out(ctx, wdem, kSlotOut0, &sw)) != PARGO_OK) return st;
    if (slope && (st = stage_out(ctx, slope, kSlotOut1, &ss)) != PARGO_OK) return st;
    if (d8 && (st = stage_out(ctx, d8, kSlotPipeD8, &sd)) != PARGO_OK) return st;
    if (sca && (st = stage_out(ctx, sca, kSlotPipeSca, &sa)) != PARGO_OK) return st;
    FillParams p;
    bool converged = false;
    pargo_fill_stats local{};
    if ((st = fill_core(ctx, sdem, dem, o, &p, &local, &converged, s)) != PARGO_OK) return st;
    if (!converged)
        return fail(ctx, PARGO_ERR_NOT_CONVERGED, "pipeline fill: worklist not empty after %lld rounds",
                    (long long)local.rounds);
    const bool focal = slope || d8 || sca;
    if (wdem && !focal) {
        cudaError_t ee = fill_finish(p, sw.out, &ctx->d_counters[3], s);
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "fill finish");
    }
    // slope + D8 on the float64 levels (+inf marks their nodata cells); the
    // same pass copies the levels out as the filled DEM
    OutView codes{};
    if (d8) {
        codes = sd.out;
    } else if (sca) {
        cudaError_t e;
        char* buf = (char*)slot(ctx, kSlotPipeCodes, (size_t)(p.rows * p.cols), &e);
        if (!buf) return cuda_fail(ctx, e, "pipeline codes");
        codes = OutView{buf, p.cols, PARGO_I8, -128.0};
    }
    if (slope || d8 || sca) {
        FocalParams f{};
        f.rows = p.rows;
        f.cols = p.cols;
        f.nd6f = Band<float>{INFINITY, INFINITY};
        f.nd7f = f.nd6f;
        f.nd6d = Band<double>{INFINITY, INFINITY};  // the levels' nodata is +inf
        f.nd7d = f.nd6d;
        f.sk = slope_consts(dem->cellsize, slope_method, slope_units);
        f.do_slope = slope != nullptr;
        f.do_d8 = d8 != nullptr || sca != nullptr;
        f.dir_type = 8;
        if (slope) f.slope = ss.out;
        if (f.do_d8) f.d8 = codes;
        f.fallbacks = &ctx->d_counters[0];
        f.error_flag = ctx->d_error;
        Focal64Params q{};
        q.f = f;
        q.wpitch = p.w_stride * 8;
        q.nodata_is_inf = 1;
        q.do_copy = wdem != nullptr;
        if (wdem) q.copy = sw.out;
        q.raised = &ctx->d_counters[3];
        q.dem = p.dem;
        q.dem_pitch = p.dem_pitch;
        q.dem_f64 = p.dem_f64;
        CUtensorMap map;
        if ((st = make_tma_map(ctx, &map, p.w, p.rows, p.cols, q.wpitch, focal64_tile_rows() + 2, focal64_box_cols(),
                               true)) != PARGO_OK)
            return st;
        if (!sca && (sw.host || ss.host || sd.host)) {
            // Host outputs: the raster in row bands, each band's copies to the
            // host on the context's own stream as soon as the band is written,
            // so they overlap the following bands' kernel.
            constexpr int kBands = 8;
            const int64_t tr = focal64_tile_rows();
            const int64_t band = ((p.rows + kBands - 1) / kBands + tr - 1) / tr * tr;
            int b = 0;
            for (int64_t r0 = 0; r0 < p.rows; r0 += band, b++) {
                const int64_t r1 = std::min(p.rows, r0 + band);
                CU(ctx, launch_focal64_tma(&map, q, ctx->num_sms, s, r0, r1));
                if (!ctx->ev_band[b]) CU(ctx, cudaEventCreateWithFlags(&ctx->ev_band[b], cudaEventDisableTiming));
                CU(ctx, cudaEventRecord(ctx->ev_band[b], s));
                CU(ctx, cudaStreamWaitEvent(ctx->own, ctx->ev_band[b], 0));
                if (wdem && (st = unstage_rows(ctx, sw, r0, r1, ctx->own)) != PARGO_OK) return st;
                if (slope && (st = unstage_rows(ctx, ss, r0, r1, ctx->own)) != PARGO_OK) return st;
                if (d8 && (st = unstage_rows(ctx, sd, r0, r1, ctx->own)) != PARGO_OK) return st;
            }
            CU(ctx, cudaEventRecord(ctx->ev_b, ctx->own));
            CU(ctx, cudaStreamWaitEvent(s, ctx->ev_b, 0));
            sw.host = ss.host = sd.host = false;  // copied back already
        } else {
            CU(ctx, launch_focal64_tma(&map, q, ctx->num_sms, s));
        }
    }
    if (sca) {
        ScaParams q{};
        q.rows = p.rows;
        q.cols = p.cols;
        q.d8 = InView{codes.base, codes.pitch, codes.dtype};
        q.nodata = codes.nodata;
        q.out = sa.out;
        q.shipped = sca_contract == PARGO_SCA_SHIPPED;
        if ((st = sca_launch(ctx, q, s, "pipeline sca")) != PARGO_OK) return st;
    }
    if (wdem && (st = unstage_out(ctx, sw, s)) != PARGO_OK) return st;
    if (slope && (st = unstage_out(ctx, ss, s)) != PARGO_OK) return st;
    if (d8 && (st = unstage_out(ctx, sd, s)) != PARGO_OK) return st;
    if (sca && (st = unstage_out(ctx, sa, s)) != PARGO_OK) return st;
    cudaError_t e;
    unsigned long long* hp = (unsigned long long*)pinned(ctx, 128, &e);
    if (!hp) return cuda_fail(ctx, e, "pinned counters");
    CU(ctx, cudaMemcpyAsync(hp, &ctx->d_counters[3], sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    if (sca) {
        unsigned long long* sc = (unsigned long long*)ctx->slots[kSlotScaCounters].p;
        CU(ctx, cudaMemcpyAsync(hp + 1, sc, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    }
    if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
    local.raised_cells = wdem ? (int64_t)hp[0] : -1;
    if (stats) *stats = local;
    if (sca) return sca_check(ctx, hp + 1, "pipeline sca");
    return PARGO_OK;
}

// ---------------------------------------------------------------- MFD-md --
pargo_status pargo_mfd(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* weights, const pargo_nbr* nbr,
                       double slp_exp, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if (!weights) return fail(ctx, PARGO_ERR_INVALID_ARG, "mfd: weights must point to 8 rasters");
    if ((st = check_raster(ctx, dem, "dem")) != PARGO_OK) return st;
    if (dem->dtype != PARGO_F32 && dem->dtype != PARGO_F64)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "mfd: dem must be F32 or F64");
    if ((st = check_dims(ctx, dem)) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    for (int q = 0; q < 8; q++) {
        if ((st = check_raster(ctx, &weights[q], "weight")) != PARGO_OK) return st;
        if ((st = check_same(ctx, dem, &weights[q], "weight")) != PARGO_OK) return st;
        if (weights[q].dtype != PARGO_F32 && weights[q].dtype != PARGO_F64)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "mfd: weights must be F32 or F64");
    }
    if (!std::isfinite(slp_exp)) return fail(ctx, PARGO_ERR_INVALID_ARG, "mfd: slope exponent must be finite");
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sd, sw[8];
    if ((st = stage_in(ctx, dem, kSlotIn0, s, &sd)) != PARGO_OK) return st;
    for (int q = 0; q < 8; q++)
        if ((st = stage_out(ctx, &weights[q], kSlotMfdLayer0 + q, &sw[q])) != PARGO_OK) return st;
    MfdParams p{};
    p.rows = dem->rows;
    p.cols = dem->cols;
    p.dem = sd.in;
    p.ndf = float_band_incl(dem->nodata, kEpsHydro);  // flowdirmfdmd/mfdOperator.cpp:55,77 test <= 1e-6
    long long klo, khi;
    band_keys(double_band_incl(dem->nodata, kEpsHydro), &klo, &khi);
    p.ndd_lo = klo;
    p.ndd_hi = khi;
    const double cs = (double)(float)dem->cellsize;  // MetaData::cellSize is a float
    p.den_card = (float)cs;
    p.den_diag = (float)(1.414 * cs);
    p.len_card = (float)(0.5 * cs);
    p.len_diag = (float)(0.354 * cs);
    p.slp_exp = (float)slp_exp;
    bool any_host = false;
    for (int q = 0; q < 8; q++) {
        p.w[q] = sw[q].out;
        any_host = any_host || sw[q].host;
    }
    CU(ctx, launch_mfd_weights(p, ctx->num_sms, s));
    for (int q = 0; q < 8; q++)
        if ((st = unstage_out(ctx, sw[q], s)) != PARGO_OK) return st;
    return finish_call(ctx, s, any_host);
}

pargo_status pargo_sca_mfd(pargo_ctx* ctx, const pargo_raster* weights, pargo_raster* sca, const pargo_nbr* nbr,
                           void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if (!weights) return fail(ctx, PARGO_ERR_INVALID_ARG, "sca_mfd: weights must point to 8 rasters");
    for (int q = 0; q < 8; q++) {
        if ((st = check_raster(ctx, &weights[q], "weight")) != PARGO_OK) return st;
        if (q && (st = check_same(ctx, &weights[0], &weights[q], "weight")) != PARGO_OK) return st;
        if (weights[q].dtype != PARGO_F32 && weights[q].dtype != PARGO_F64)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "sca_mfd: weights must be F32 or F64");
    }
    if ((st = check_dims(ctx, &weights[0])) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    if ((st = check_raster(ctx, sca, "sca")) != PARGO_OK) return st;
    if ((st = check_same(ctx, &weights[0], sca, "sca")) != PARGO_OK) return st;
    if (sca->dtype != PARGO_F32 && sca->dtype != PARGO_F64)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "sca_mfd: sca must be F32 or F64");
    const int64_t n = weights[0].rows * weights[0].cols;
    if (n >= INT32_MAX) return fail(ctx, PARGO_ERR_INVALID_ARG, "sca_mfd: raster too large");
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sw[8], so;
    for (int q = 0; q < 8; q++)
        if ((st = stage_in(ctx, &weights[q], kSlotMfdLayer0 + q, s, &sw[q])) != PARGO_OK) return st;
    if ((st = stage_out(ctx, sca, kSlotOut0, &so)) != PARGO_OK) return st;
    cudaError_t e;
    ScaMfdParams p{};
    p.rows = weights[0].rows;
    p.cols = weights[0].cols;
    for (int q = 0; q < 8; q++) p.w[q] = sw[q].in;
    long long klo, khi;
    band_keys(double_band(weights[0].nodata, kEpsHydro), &klo, &khi);  // scamfdmd/scaOperator.cpp:50 tests < 1e-6
    p.nd_lo = klo;
    p.nd_hi = khi;
    p.nodata = weights[0].nodata;  // the reference's SCA layer copies weight layer 0's nodata
    p.out = so.out;
    p.cnt = (int32_t*)slot(ctx, kSlotMfdCnt, (size_t)n * 4, &e);
    p.flags = (uint8_t*)slot(ctx, kSlotMfdFlags, (size_t)n, &e);
    p.sca = (double*)slot(ctx, kSlotMfdSca, (size_t)n * 8, &e);
    int32_t* lists = (int32_t*)slot(ctx, kSlotMfdLists, (size_t)(3 * n + 16) * 4 + 64, &e);
    if (!p.cnt || !p.flags || !p.sca || !lists) return cuda_fail(ctx, e, "sca_mfd scratch");
    p.list_a = lists;
    p.list_b = lists + n;
    p.counts = lists + 3 * n;
    p.totals = (unsigned long long*)(((uintptr_t)(lists + 3 * n + 8) + 7) & ~(uintptr_t)7);
    p.error_flag = ctx->d_error;
    bool f32 = true;
    for (int q = 0; q < 8; q++) f32 = f32 && p.w[q].dtype == PARGO_F32;
    void* records = slot(ctx, kSlotMfdRecords, sca_mfd_band_bytes(p.rows, p.cols, f32), &e);
    if (!records) return cuda_fail(ctx, e, "sca_mfd records");
    CU(ctx, launch_sca_mfd_init(p, ctx->num_sms, s));
    int32_t* hc = (int32_t*)pinned(ctx, 128, &e);
    if (!hc) return cuda_fail(ctx, e, "pinned counters");
    // Warps walk 32-row bands in step (every dependency of the reference's
    // sweep points forward in raster order); the band cursor and the bands'
    // progress words live in the list scratch, which this form does not use.
    if (launch_sca_mfd_band(p, records, lists, ctx->num_sms, s) == cudaSuccess) {
        CU(ctx, launch_sca_mfd_output(p, ctx->num_sms, s));
        if ((st = unstage_out(ctx, so, s)) != PARGO_OK) return st;
        unsigned long long* ht = (unsigned long long*)(hc + 8);
        CU(ctx, cudaMemcpyAsync(ht, p.totals, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
        if (ht[2] != 0)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "sca_mfd: %llu nodata cells carry positive weights", ht[2]);
        if (ht[0] != ht[1])
            return fail(ctx, PARGO_ERR_CYCLE, "sca_mfd: only %llu of %llu valid cells processed",
                        ht[1], ht[0]);
        return PARGO_OK;
    }
    cudaGetLastError();  // clear the refused launch
    // Frontier rounds, 32 per CUDA graph (an even number: list A is current
    // again after each graph), until both lists are empty.
    CU(ctx, launch_sca_mfd_counts(p, ctx->num_sms, s));
    constexpr int kRounds = 32;
    CU(ctx, cudaEventRecord(ctx->ev_a, s));
    CU(ctx, cudaStreamWaitEvent(ctx->own, ctx->ev_a, 0));
    cudaGraph_t g;
    cudaGraphExec_t ge = nullptr;
    CU(ctx, cudaStreamBeginCapture(ctx->own, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    for (int r = 0; r < kRounds && ce == cudaSuccess; r++) ce = launch_sca_mfd_round(p, r & 1, ctx->num_sms, ctx->own);
    cudaError_t ee = cudaStreamEndCapture(ctx->own, &g);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "sca_mfd round capture");
    if (ee != cudaSuccess) return cuda_fail(ctx, ee, "sca_mfd graph capture");
    ee = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ee != cudaSuccess) return cuda_fail(ctx, ee, "sca_mfd graph instantiate");
    pargo_status rs = PARGO_OK;
    for (int64_t launched = 0;; launched += kRounds) {
        if ((e = cudaGraphLaunch(ge, ctx->own)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hc, p.counts, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->own)) != cudaSuccess ||
            (e = cudaStreamSynchronize(ctx->own)) != cudaSuccess) {
            rs = cuda_fail(ctx, e, "sca_mfd rounds");
            break;
        }
        if (hc[0] == 0 && hc[1] == 0) break;
        if (launched > n + kRounds) {  // more rounds than cells: cannot happen on a DAG
            rs = fail(ctx, PARGO_ERR_CYCLE, "sca_mfd: frontier did not drain");
            break;
        }
    }
    cudaGraphExecDestroy(ge);
    if (rs != PARGO_OK) return rs;
    CU(ctx, cudaEventRecord(ctx->ev_b, ctx->own));
    CU(ctx, cudaStreamWaitEvent(s, ctx->ev_b, 0));
    CU(ctx, launch_sca_mfd_output(p, ctx->num_sms, s));
    if ((st = unstage_out(ctx, so, s)) != PARGO_OK) return st;
    unsigned long long* ht = (unsigned long long*)(hc + 8);
    CU(ctx, cudaMemcpyAsync(ht, p.totals, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
    if (ht[2] != 0)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "sca_mfd: %llu nodata cells carry positive weights", ht[2]);
    if (ht[0] != ht[1])
        return fail(ctx, PARGO_ERR_CYCLE, "sca_mfd: only %llu of %llu valid cells processed",
                        ht[1], ht[0]);
    return PARGO_OK;
}

// ------------------------------------------------------------------ load --
pargo_status pargo_compute_load_dims(int64_t rows, int64_t cols, int grain, int64_t* crows, int64_t* ccols) {
    if (rows < 3 || cols < 3 || grain < 1 || !crows || !ccols) return PARGO_ERR_INVALID_ARG;
    *crows = (rows - 2 + grain - 1) / grain;  // ComputeLayer::_init over the 3x3 work rectangle
    *ccols = (cols - 2 + grain - 1) / grain;
    return PARGO_OK;
}

pargo_status pargo_compute_load(pargo_ctx* ctx, int count, const pargo_raster* data, const pargo_nbr* nbr, int grain,
                                int compute_ring, double nodata_load, double valid_load, pargo_raster* load,
                                void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if (count < 1 || count > kMaxLoadLayers || !data)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "compute_load: 1 to %d data rasters", kMaxLoadLayers);
    if (grain < 1) return fail(ctx, PARGO_ERR_INVALID_ARG, "compute_load: grain must be >= 1");
    if (nodata_load < 0 || valid_load < 0)  // transformation.h:169-172
        return fail(ctx, PARGO_ERR_INVALID_ARG, "compute_load: the loads cannot be negative");
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    for (int l = 0; l < count; l++) {
        if ((st = check_raster(ctx, &data[l], "data")) != PARGO_OK) return st;
        if (data[l].dtype != PARGO_F32 && data[l].dtype != PARGO_F64)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "compute_load: data must be F32 or F64");
        if (l && (data[l].rows != data[0].rows || data[l].cols != data[0].cols))
            return fail(ctx, PARGO_ERR_INVALID_ARG, "compute_load: data rasters differ in shape");
    }
    if ((st = check_dims(ctx, &data[0])) != PARGO_OK) return st;
    int64_t crows, ccols;
    pargo_compute_load_dims(data[0].rows, data[0].cols, grain, &crows, &ccols);
    if ((st = check_raster(ctx, load, "load")) != PARGO_OK) return st;
    if (load->rows != crows || load->cols != ccols)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "compute_load: load must be %lld x %lld", (long long)crows,
                    (long long)ccols);
    if (load->dtype != PARGO_F64 && load->dtype != PARGO_F32)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "compute_load: load must be F64 or F32");
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    LoadParams p{};
    p.rows = data[0].rows;
    p.cols = data[0].cols;
    p.count = count;
    Staged sd[kMaxLoadLayers], so;
    bool host = false;
    for (int l = 0; l < count; l++) {
        if ((st = stage_in(ctx, &data[l], kSlotMfdLayer0 + l, s, &sd[l])) != PARGO_OK) return st;
        p.data[l] = sd[l].in;
        host = host || sd[l].host;
    }
    if ((st = stage_out(ctx, load, kSlotOut0, &so)) != PARGO_OK) return st;
    for (int l = 0; l < count; l++) {  // each layer's own nodata; |v - nd| <= 1e-7 is nodata
        p.ndf[l] = float_band_incl(data[l].nodata, 0.0000001);
        long long klo, khi;
        band_keys(double_band_incl(data[l].nodata, 0.0000001), &klo, &khi);
        p.nd_lo[l] = klo;
        p.nd_hi[l] = khi;
    }
    p.grain = grain;
    p.compute_ring = compute_ring ? 1 : 0;
    p.nodata_load = nodata_load;
    p.valid_load = valid_load;
    {
        // sums of integer loads below 2^53 are exact in any order
        const double mx = std::max(nodata_load, valid_load);
        const double cells = (double)count * grain * grain;
        p.integral = nodata_load == std::floor(nodata_load) && valid_load == std::floor(valid_load) &&
                     mx * cells < 9007199254740992.0;
    }
    p.crows = crows;
    p.ccols = ccols;
    p.load = so.out;
    CU(ctx, launch_compute_load(p, ctx->num_sms, s));
    if ((st = unstage_out(ctx, so, s)) != PARGO_OK) return st;
    return finish_call(ctx, s, host || so.host);
}

pargo_status pargo_load_decompose(pargo_ctx* ctx, const pargo_raster* load, int compute_ring, int64_t data_rows,
                                  int64_t data_cols, const pargo_nbr* nbr, int nparts, int64_t* comp_rows,
                                  int64_t* bounds, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if ((st = check_raster(ctx, load, "load")) != PARGO_OK) return st;
    if (load->dtype != PARGO_F64 && load->dtype != PARGO_F32)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "load_decompose: load must be F64 or F32");
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    if (data_rows < 3 || data_cols < 3 || data_rows > INT32_MAX || data_cols > INT32_MAX)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "load_decompose: bad data dimensions");
    if (!bounds) return fail(ctx, PARGO_ERR_INVALID_ARG, "load_decompose: bounds is required");
    const int64_t crows = load->rows, ccols = load->cols;
    const int64_t work_rows = compute_ring ? crows - 2 : crows;
    if (nparts < 1 || nparts > work_rows)  // deComposition.h:314-320
        return fail(ctx, PARGO_ERR_INVALID_ARG, "load_decompose: %d parts for %lld compute rows", nparts,
                    (long long)work_rows);
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sl;
    if ((st = stage_in(ctx, load, kSlotIn0, s, &sl)) != PARGO_OK) return st;
    cudaError_t e;
    double* drow = (double*)slot(ctx, kSlotLoadRows, (size_t)crows * sizeof(double), &e);
    if (!drow) return cuda_fail(ctx, e, "row loads");
    CU(ctx, launch_row_load(sl.in, crows, ccols, load->nodata, drow, ctx->num_sms, s));
    std::vector<double> row_load((size_t)crows);
    CU(ctx, cudaMemcpyAsync(row_load.data(), drow, (size_t)crows * sizeof(double), cudaMemcpyDeviceToHost, s));
    if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
    // DeComposition::valRowDcmp (gpro/deComposition.h:337-385): nparts-1 greedy
    // cuts, each where the running load first passes the average of what is
    // left, moved one row back when that is nearer the average.
    double total = 0.0;
    for (double v : row_load) total += v;
    std::vector<int64_t> cb((size_t)nparts), ce((size_t)nparts);
    double aver = total / nparts, accu = 0.0;
    int64_t begin = 0;
    int k = 0;
    for (int i = 0; i < nparts - 1; i++) {
        double sub = 0.0, min_diff = 0.0;
        bool cut = false;
        for (int64_t r = begin; r < crows; r++) {
            sub += row_load[(size_t)r];
            accu += row_load[(size_t)r];
            const bool room = crows - 1 - r > nparts - 1 - i;  // rows left for the remaining parts
            if (sub <= aver && room) {
                if (fabs(min_diff) < 0.0000001 || (aver - sub) < min_diff) min_diff = aver - sub;
                continue;
            }
            if (fabs(min_diff) < 0.0000001 || (sub - aver) <= min_diff || crows - 1 - r == nparts - 1 - i) {
                cb[(size_t)k] = begin;
                ce[(size_t)k++] = r;
                begin = r + 1;
            } else {  // the row before is nearer the average: this row opens the next part
                accu -= row_load[(size_t)r];
                cb[(size_t)k] = begin;
                ce[(size_t)k++] = r - 1;
                begin = r;
            }
            aver = (total - accu) / (nparts - i - 1);
            cut = true;
            break;
        }
        if (!cut) return fail(ctx, PARGO_ERR_INVALID_ARG, "load_decompose: the cuts ran out of rows");
    }
    cb[(size_t)k] = begin;
    ce[(size_t)k] = crows - 1;
    // ComputeLayer::getCompuLoad (gpro/computeLayer.h:402-430): compute rows to
    // data rows of the data work rectangle, scaled by data rows / compute rows
    // and truncated.
    const double convert = (double)data_rows / (double)crows;
    const int64_t wr0 = 1, wr1 = data_rows - 2, wc0 = 1, wc1 = data_cols - 2;
    int64_t sub_end = wr0 - 1;
    for (int i = 0; i < nparts; i++) {
        if (comp_rows) {
            comp_rows[2 * i] = cb[(size_t)i];
            comp_rows[2 * i + 1] = ce[(size_t)i];
        }
        int64_t b0, b1;
        if (i < nparts - 1) {
            b0 = (int64_t)(int)((double)cb[(size_t)i] * convert + (double)wr0);
            b1 = (int64_t)(int)((double)cb[(size_t)i + 1] * convert + (double)wr0 - 1.0);
            sub_end = b1;
        } else {
            b0 = sub_end + 1;
            b1 = wr1;
        }
        bounds[4 * i] = b0;
        bounds[4 * i + 1] = wc0;
        bounds[4 * i + 2] = b1;
        bounds[4 * i + 3] = wc1;
    }
    return PARGO_OK;
}

// ------------------------------------------------------------------- TWI --
pargo_status pargo_twi(pargo_ctx* ctx, const pargo_raster* slope, const pargo_raster* sca, pargo_raster* twi,
                       const pargo_nbr* nbr, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if ((st = check_raster(ctx, slope, "slope")) != PARGO_OK) return st;
    if ((st = check_raster(ctx, sca, "sca")) != PARGO_OK) return st;
    if ((st = check_raster(ctx, twi, "twi")) != PARGO_OK) return st;
    if ((st = check_dims(ctx, slope)) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    if ((st = check_same(ctx, slope, sca, "sca")) != PARGO_OK) return st;
    if ((st = check_same(ctx, slope, twi, "twi")) != PARGO_OK) return st;
    for (const pargo_raster* r : {slope, sca, (const pargo_raster*)twi})
        if (r->dtype != PARGO_F32 && r->dtype != PARGO_F64)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "twi: slope, sca and twi must be F32 or F64");
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged ss, sa, so;
    if ((st = stage_in(ctx, slope, kSlotIn0, s, &ss)) != PARGO_OK) return st;
    if ((st = stage_in(ctx, sca, kSlotIn1, s, &sa)) != PARGO_OK) return st;
    if ((st = stage_out(ctx, twi, kSlotOut0, &so)) != PARGO_OK) return st;
    TwiParams p{};
    p.rows = slope->rows;
    p.cols = slope->cols;
    p.slope = ss.in;
    p.sca = sa.in;
    p.out = so.out;
    p.sca_nodata = sca->nodata;
    memcpy(&p.nd_bits, &sca->nodata, 8);
    p.nd_f = (float)sca->nodata;
    p.nd_is_float = (double)p.nd_f == sca->nodata;
    p.sca_nd_f = (float)sca->nodata;
    p.out_nd_f = (float)twi->nodata;
    float eps = 1.0e-7f;
    if ((double)eps < 1.0e-7) eps = nextafterf(eps, INFINITY);
    p.eps_cut = eps;
    CU(ctx, launch_twi(p, ctx->num_sms, s));
    if ((st = unstage_out(ctx, so, s)) != PARGO_OK) return st;
    return finish_call(ctx, s, so.host);
}

// ------------------------------------------------------------------- SCA --
pargo_status pargo_sca(pargo_ctx* ctx, const pargo_raster* d8, pargo_raster* sca, const pargo_nbr* nbr, int contract,
                       void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if ((st = check_raster(ctx, d8, "d8")) != PARGO_OK) return st;
    if ((st = check_dims(ctx, d8)) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    if ((st = check_raster(ctx, sca, "sca")) != PARGO_OK) return st;
    if ((st = check_same(ctx, d8, sca, "sca")) != PARGO_OK) return st;
    if (sca->dtype != PARGO_F64 && sca->dtype != PARGO_F32)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "sca must be F64 or F32");
    if (contract != PARGO_SCA_CONVERGED && contract != PARGO_SCA_SHIPPED)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "unknown SCA contract %d", contract);
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sd8, so;
    if ((st = stage_in(ctx, d8, kSlotIn0, s, &sd8)) != PARGO_OK) return st;
    if ((st = stage_out(ctx, sca, kSlotOut0, &so)) != PARGO_OK) return st;
    cudaError_t e;
    ScaParams p{};
    p.rows = d8->rows;
    p.cols = d8->cols;
    p.d8 = sd8.in;
    p.nodata = d8->nodata;
    p.out = so.out;
    p.shipped = contract == PARGO_SCA_SHIPPED;
    if ((st = sca_launch(ctx, p, s, "sca")) != PARGO_OK) return st;
    if ((st = unstage_out(ctx, so, s)) != PARGO_OK) return st;
    unsigned long long* hp = (unsigned long long*)pinned(ctx, 64, &e);
    if (!hp) return cuda_fail(ctx, e, "pinned counters");
    CU(ctx, cudaMemcpyAsync(hp, ctx->slots[kSlotScaCounters].p, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            s));
    if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
    return sca_check(ctx, hp, "sca");
}

// ------------------------------------------------------------------ batch --
// Defaults of the batched queue: ordered by compute intensity with the
// reference's example loads (a nodata cell 0, a valid cell 1: the
// "-nodataLoad 0 -validLoad 1" of apps/spatial/reclassify/pRelclassify.cpp:22).
static pargo_batch_opts batch_defaults(const pargo_batch_opts* opts) {
    pargo_batch_opts o{0.0, 1.0, PARGO_BATCH_BY_INTENSITY, 0};
    if (opts) o = *opts;
    return o;
}

static pargo_status check_batch_opts(pargo_ctx* ctx, const pargo_batch_opts& o) {
    if (o.order != PARGO_BATCH_BY_INTENSITY && o.order != PARGO_BATCH_BY_SIZE)
        return fail(ctx, PARGO_ERR_INVALID_ARG, "batch: unknown queue order %d", o.order);
    if (!(o.nodata_load >= 0.0) || !(o.valid_load >= 0.0) || !std::isfinite(o.nodata_load) ||
        !std::isfinite(o.valid_load))  // transformation.h:168-171 rejects negative loads
        return fail(ctx, PARGO_ERR_INVALID_ARG, "batch: loads must be finite and not negative");
    return PARGO_OK;
}

// The strip-walk queue of a batch ordered by compute intensity: every
// segment's load (valid_load per valid cell, nodata_load per nodata cell,
// counted on the device), summed per raster, and the rasters queued heaviest
// first (ties keep the order by size), each raster's segments together in
// raster order.  Keeping a raster's segments together keeps the rows that
// neighbouring segments share in L2: sorting the segments themselves by load
// (a raster's full segments first, every raster's partial edge segments
// last) measured 2.62 ms against 2.31 ms on the 512-raster batch.
// `korder[k]` is the caller's index of the k-th raster by size; seg_start /
// nstrips follow k.  Returns queue position -> (k << 40 | segment of raster
// k) and each queued segment's load.
static pargo_status batch_intensity_queue(pargo_ctx* ctx, int count, const pargo_raster* dems,
                                          const std::vector<int>& korder, const std::vector<int64_t>& seg_start,
                                          const std::vector<int>& nstrips, int64_t nsegs, const pargo_batch_opts& o,
                                          cudaStream_t s, std::vector<uint64_t>* queue, std::vector<double>* loads) {
    std::vector<SegLoadRaster> rs(count);
    for (int k = 0; k < count; k++) {
        const pargo_raster* d = &dems[korder[k]];
        rs[k].dem = InView{(const char*)d->data, pitch_of(d), d->dtype};
        rs[k].rows = d->rows;
        rs[k].cols = d->cols;
        rs[k].nd = float_band_incl(d->nodata, 0.0000001);  // transformation.h:187: |v - noData| > Eps is valid
        rs[k].seg_start = seg_start[k];
        rs[k].nstrips = nstrips[k];
    }
    const size_t tb = ((size_t)count * sizeof(SegLoadRaster) + 255) / 256 * 256;
    cudaError_t e;
    char* buf = (char*)slot(ctx, kSlotBatchSegLoad, tb + (size_t)nsegs * 4, &e);
    if (!buf) return cuda_fail(ctx, e, "batch intensity table");
    CU(ctx, cudaMemcpyAsync(buf, rs.data(), (size_t)count * sizeof(SegLoadRaster), cudaMemcpyHostToDevice, s));
    uint32_t* dvalid = (uint32_t*)(buf + tb);
    CU(ctx, launch_batch_segment_valid((const SegLoadRaster*)buf, count, nsegs, dvalid, ctx->num_sms, s));
    std::vector<uint32_t> valid((size_t)nsegs);
    CU(ctx, cudaMemcpyAsync(valid.data(), dvalid, (size_t)nsegs * 4, cudaMemcpyDeviceToHost, s));
    CU(ctx, cudaStreamSynchronize(s));
    const int SR = batch_strip_segment_rows(), SC = batch_strip_segment_cols();
    loads->assign((size_t)nsegs, 0.0);
    std::vector<uint64_t> ids((size_t)nsegs);
    for (int k = 0; k < count; k++) {
        const int64_t rows = rs[k].rows, cols = rs[k].cols;
        for (int64_t l = 0; l < seg_start[k + 1] - seg_start[k]; l++) {
            const int64_t g = seg_start[k] + l;
            const int64_t x0 = (l % nstrips[k]) * SC, y0 = (l / nstrips[k]) * SR;
            const int64_t cells = (std::min<int64_t>(y0 + SR, rows) - y0) * (std::min<int64_t>(x0 + SC, cols) - x0);
            (*loads)[g] = (double)valid[g] * o.valid_load + (double)(cells - (int64_t)valid[g]) * o.nodata_load;
            ids[g] = ((uint64_t)k << 40) | (uint64_t)l;
        }
    }
    std::vector<double> rload(count, 0.0);
    for (int k = 0; k < count; k++)
        for (int64_t g = seg_start[k]; g < seg_start[k + 1]; g++) rload[k] += (*loads)[g];
    std::vector<int> ks(count);
    for (int k = 0; k < count; k++) ks[k] = k;
    std::stable_sort(ks.begin(), ks.end(), [&](int a, int b) { return rload[a] > rload[b]; });
    queue->clear();
    queue->reserve((size_t)nsegs);
    std::vector<double> sorted;
    sorted.reserve((size_t)nsegs);
    for (int k : ks)
        for (int64_t g = seg_start[k]; g < seg_start[k + 1]; g++) {
            queue->push_back(ids[g]);
            sorted.push_back((*loads)[g]);
        }
    loads->swap(sorted);
    return PARGO_OK;
}

pargo_status pargo_batch_slope_d8(pargo_ctx* ctx, int count, const pargo_raster* dems, pargo_raster* slopes,
                                  pargo_raster* d8s, const pargo_nbr* nbr, int method, int units, int dir_type,
                                  void* stream) {
    return pargo_batch_slope_d8_ex(ctx, count, dems, slopes, d8s, nbr, method, units, dir_type, nullptr, stream);
}

pargo_status pargo_batch_queue(pargo_ctx* ctx, int count, const pargo_raster* dems, const pargo_batch_opts* opts,
                               int64_t cap, int64_t* n_out, int32_t* raster, int64_t* segment, double* load,
                               void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (count < 0 || (count > 0 && !dems) || cap < 0) return fail(ctx, PARGO_ERR_INVALID_ARG, "batch queue: bad args");
    const pargo_batch_opts o = batch_defaults(opts);
    pargo_status st;
    if ((st = check_batch_opts(ctx, o)) != PARGO_OK) return st;
    for (int i = 0; i < count; i++) {
        if ((st = check_raster(ctx, &dems[i], "batch dem")) != PARGO_OK) return st;
        if ((st = check_dims(ctx, &dems[i])) != PARGO_OK) return st;
        if (dems[i].dtype != PARGO_F32 || dems[i].location != PARGO_DEVICE)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "batch dem %d: must be F32 on the device", i);
    }
    std::vector<int> korder(count);
    for (int i = 0; i < count; i++) korder[i] = i;
    std::stable_sort(korder.begin(), korder.end(), [&](int a, int b) {
        return dems[a].rows * dems[a].cols > dems[b].rows * dems[b].cols;
    });
    std::vector<int64_t> seg_start(count + 1);
    std::vector<int> nstrips(count);
    int64_t nsegs = 0;
    for (int k = 0; k < count; k++) {
        seg_start[k] = nsegs;
        nsegs += batch_strip_segments(dems[korder[k]].rows, dems[korder[k]].cols, &nstrips[k]);
    }
    seg_start[count] = nsegs;
    if (n_out) *n_out = nsegs;
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    std::vector<uint64_t> q;
    std::vector<double> ld;
    if (o.order == PARGO_BATCH_BY_INTENSITY && count > 0) {
        if ((st = batch_intensity_queue(ctx, count, dems, korder, seg_start, nstrips, nsegs, o, s, &q, &ld)) !=
            PARGO_OK)
            return st;
    } else {
        for (int k = 0; k < count; k++)
            for (int64_t l = 0; l < seg_start[k + 1] - seg_start[k]; l++) q.push_back(((uint64_t)k << 40) | l);
        ld.assign(q.size(), 0.0);
    }
    for (int64_t i = 0; i < std::min<int64_t>(cap, nsegs); i++) {
        const int k = (int)(q[i] >> 40);
        if (raster) raster[i] = korder[k];
        if (segment) segment[i] = (int64_t)(q[i] & ((1ULL << 40) - 1));
        if (load) load[i] = ld[i];
    }
    return PARGO_OK;
}

pargo_status pargo_batch_slope_d8_ex(pargo_ctx* ctx, int count, const pargo_raster* dems, pargo_raster* slopes,
                                     pargo_raster* d8s, const pargo_nbr* nbr, int method, int units, int dir_type,
                                     const pargo_batch_opts* opts, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (count < 0 || (count > 0 && !dems)) return fail(ctx, PARGO_ERR_INVALID_ARG, "batch: bad count or dems");
    if (!slopes && !d8s) return fail(ctx, PARGO_ERR_INVALID_ARG, "batch: no output requested");
    if (count == 0) return PARGO_OK;
    pargo_status st;
    const pargo_batch_opts bo = batch_defaults(opts);
    if ((st = check_batch_opts(ctx, bo)) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    if (slopes && (method < 0 || method > 6)) return fail(ctx, PARGO_ERR_INVALID_ARG, "unknown slope method %d", method);
    bool all_tma = true;
    for (int i = 0; i < count; i++) {
        const pargo_raster* d = &dems[i];
        if ((st = check_raster(ctx, d, "batch dem")) != PARGO_OK) return st;
        if ((st = check_dims(ctx, d)) != PARGO_OK) return st;
        if (d->dtype != PARGO_F32 || d->location != PARGO_DEVICE)
            return fail(ctx, PARGO_ERR_INVALID_ARG, "batch dem %d: must be F32 on the device", i);
        if (slopes) {
            if ((st = check_raster(ctx, &slopes[i], "batch slope")) != PARGO_OK) return st;
            if ((st = check_same(ctx, d, &slopes[i], "batch slope")) != PARGO_OK) return st;
            if (slopes[i].location != PARGO_DEVICE || (slopes[i].dtype != PARGO_F32 && slopes[i].dtype != PARGO_F64))
                return fail(ctx, PARGO_ERR_INVALID_ARG, "batch slope %d: must be F32/F64 on the device", i);
        }
        if (d8s) {
            if ((st = check_raster(ctx, &d8s[i], "batch d8")) != PARGO_OK) return st;
            if ((st = check_same(ctx, d, &d8s[i], "batch d8")) != PARGO_OK) return st;
            if (d8s[i].location != PARGO_DEVICE)
                return fail(ctx, PARGO_ERR_INVALID_ARG, "batch d8 %d: must be on the device", i);
            if ((st = check_d8_out(ctx, &d8s[i], dir_type)) != PARGO_OK) return st;
        }
        InView v{(const char*)d->data, pitch_of(d), d->dtype};
        if (!tma_ok(v)) all_tma = false;
    }
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    // Order: largest rasters first (their tiles are claimed first).
    std::vector<int> order(count);
    for (int i = 0; i < count; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return dems[a].rows * dems[a].cols > dems[b].rows * dems[b].cols;
    });
    const int TH = focal_tma_tile_rows(), TW = focal_tma_tile_cols();
    std::vector<FocalParams> params(count);
    std::vector<int64_t> start(count + 1), ntx(count);
    std::vector<InView> views(count);
    int64_t total = 0;
    for (int k = 0; k < count; k++) {
        const int i = order[k];
        const pargo_raster* d = &dems[i];
        FocalParams& p = params[k];
        p = FocalParams{};
        p.rows = d->rows;
        p.cols = d->cols;
        p.nd6f = float_band(d->nodata, kEpsHydro);
        p.nd7f = float_band(d->nodata, kEpsSlope);
        p.sk = slope_consts(d->cellsize, method, units);
        p.do_slope = slopes != nullptr;
        p.do_d8 = d8s != nullptr;
        p.dir_type = dir_type;
        if (slopes) p.slope = OutView{(char*)slopes[i].data, pitch_of(&slopes[i]), slopes[i].dtype, slopes[i].nodata};
        if (d8s) p.d8 = OutView{(char*)d8s[i].data, pitch_of(&d8s[i]), d8s[i].dtype, d8s[i].nodata};
        p.fallbacks = &ctx->d_counters[0];
        p.error_flag = ctx->d_error;
        p.fast_out = fast_out_ok(p) ? 1 : 0;
        p.fd = method == PARGO_SLOPE_FD || !slopes;
        views[k] = InView{(const char*)d->data, pitch_of(d), d->dtype};
        start[k] = total;
        if (all_tma) {
            ntx[k] = (d->cols + TW - 1) / TW;
            total += ntx[k] * ((d->rows + TH - 1) / TH);
        } else {
            ntx[k] = 0;
            total += d->rows * d->cols;
        }
    }
    start[count] = total;
    // The strip walk covers the plain configuration (Horn rise/run slope,
    // dirType 8, float32 slope / int8 codes with vector-store alignment).
    bool strip = all_tma && (method == PARGO_SLOPE_FD || !slopes) && units == PARGO_SLOPE_RATIO &&
                 (dir_type == 8 || !d8s) && count > 0;
    std::vector<int64_t> seg_start(count + 1);
    std::vector<int> nstrips(count);
    int64_t nsegs = 0, slow_cap = 0;
    for (int k = 0; k < count && strip; k++) {
        strip = params[k].fast_out != 0;
        seg_start[k] = nsegs;
        nsegs += batch_strip_segments(params[k].rows, params[k].cols, &nstrips[k]);
        slow_cap += params[k].rows * ((params[k].cols + 3) / 4);
        if (params[k].rows * ((params[k].cols + 3) / 4) >= (1LL << 40)) strip = false;
    }
    seg_start[count] = nsegs;
    // Device tables (cached while the batch description is unchanged).
    std::string key((const char*)params.data(), params.size() * sizeof(FocalParams));
    key.append((const char*)dems, (size_t)count * sizeof(pargo_raster));
    key.append((const char*)&bo, sizeof(bo));
    cudaError_t e;
    CUtensorMap* dmaps = (CUtensorMap*)slot(ctx, kSlotBatchMaps, (size_t)count * sizeof(CUtensorMap), &e);
    FocalParams* dparams = (FocalParams*)slot(ctx, kSlotBatchParams, (size_t)count * sizeof(FocalParams), &e);
    int64_t* dstart = (int64_t*)slot(ctx, kSlotBatchStart, (size_t)(count + 1) * 8, &e);
    int64_t* dntx = (int64_t*)slot(ctx, kSlotBatchNtx, (size_t)count * 8, &e);
    InView* ddems = (InView*)slot(ctx, kSlotBatchDems, (size_t)count * sizeof(InView), &e);
    unsigned long long* claim = (unsigned long long*)slot(ctx, kSlotClaim, 64, &e);
    if (!dmaps || !dparams || !dstart || !dntx || !ddems || !claim) return cuda_fail(ctx, e, "batch tables");
    CUtensorMap* dsmaps = nullptr;
    int64_t* dseg = nullptr;
    int* dns = nullptr;
    uint64_t* dslow = nullptr;
    if (strip) {
        dsmaps = (CUtensorMap*)slot(ctx, kSlotBatchStripMaps, (size_t)2 * count * sizeof(CUtensorMap), &e);
        dseg = (int64_t*)slot(ctx, kSlotBatchSegStart, (size_t)(count + 1) * 8, &e);
        dns = (int*)slot(ctx, kSlotBatchNstrips, (size_t)count * sizeof(int), &e);
        dslow = (uint64_t*)slot(ctx, kSlotBatchSlow, (size_t)slow_cap * 8, &e);
        if (!dsmaps || !dseg || !dns || !dslow) return cuda_fail(ctx, e, "batch strip tables");
    }
    if (ctx->batch_key != key) {
        if (strip) {
            std::vector<CUtensorMap> smaps(2 * (size_t)count);
            for (int k = 0; k < count; k++) {
                if ((st = make_tma_map(ctx, &smaps[2 * k], views[k].base, params[k].rows, params[k].cols,
                                       views[k].pitch, focal_strip_stage_rows(-1, 1, 1))) != PARGO_OK)
                    return st;
                if ((st = make_tma_map(ctx, &smaps[2 * k + 1], views[k].base, params[k].rows, params[k].cols,
                                       views[k].pitch, 2)) != PARGO_OK)
                    return st;
            }
            CU(ctx, cudaStreamSynchronize(s));
            CU(ctx, cudaMemcpy(dsmaps, smaps.data(), smaps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
            CU(ctx, cudaMemcpy(dseg, seg_start.data(), (count + 1) * 8, cudaMemcpyHostToDevice));
            CU(ctx, cudaMemcpy(dns, nstrips.data(), count * sizeof(int), cudaMemcpyHostToDevice));
            // The queue: segments by compute intensity, heaviest first.  The
            // estimate is taken when a batch description is first seen and is
            // kept with the other tables; it orders the work only, so the
            // outputs never depend on it.
            ctx->batch_ordered = false;
            if (bo.order == PARGO_BATCH_BY_INTENSITY) {
                std::vector<uint64_t> q;
                std::vector<double> ld;
                if ((st = batch_intensity_queue(ctx, count, dems, order, seg_start, nstrips, nsegs, bo, s, &q, &ld)) !=
                    PARGO_OK)
                    return st;
                uint64_t* dq = (uint64_t*)slot(ctx, kSlotBatchOrder, (size_t)nsegs * 8, &e);
                if (!dq) return cuda_fail(ctx, e, "batch queue");
                CU(ctx, cudaMemcpy(dq, q.data(), (size_t)nsegs * 8, cudaMemcpyHostToDevice));
                ctx->batch_ordered = true;
            }
        }
        std::vector<CUtensorMap> maps(all_tma ? count : 0);
        if (all_tma)
            for (int k = 0; k < count; k++)
                if ((st = make_tma_map(ctx, &maps[k], views[k].base, params[k].rows, params[k].cols, views[k].pitch,
                                       focal_tma_box_rows())) != PARGO_OK)
                    return st;
        CU(ctx, cudaStreamSynchronize(s));
        if (all_tma) CU(ctx, cudaMemcpy(dmaps, maps.data(), count * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
        CU(ctx, cudaMemcpy(dparams, params.data(), count * sizeof(FocalParams), cudaMemcpyHostToDevice));
        CU(ctx, cudaMemcpy(dstart, start.data(), (count + 1) * 8, cudaMemcpyHostToDevice));
        CU(ctx, cudaMemcpy(dntx, ntx.data(), count * 8, cudaMemcpyHostToDevice));
        CU(ctx, cudaMemcpy(ddems, views.data(), count * sizeof(InView), cudaMemcpyHostToDevice));
        ctx->batch_key = key;
    }
    CU(ctx, cudaMemsetAsync(&ctx->d_counters[0], 0, sizeof(unsigned long long), s));
    if (strip)
        CU(ctx, launch_batch_strip(dsmaps, dparams, ddems, dseg, dns,
                                   ctx->batch_ordered ? (const uint64_t*)ctx->slots[kSlotBatchOrder].p : nullptr,
                                   count, nsegs, slopes ? 1 : 0, d8s ? 1 : 0,
                                   &ctx->d_counters[4], dslow, &ctx->d_counters[0], ctx->d_error, ctx->num_sms, s));
    else if (all_tma)
        CU(ctx, launch_batch_tma(dmaps, dparams, dstart, dntx, count, total, slopes ? 1 : 0, d8s ? 1 : 0, claim,
                                 &ctx->d_counters[0],
                                 ctx->d_error, ctx->num_sms, s));
    else
        CU(ctx, launch_batch_generic(dparams, ddems, dstart, count, total, &ctx->d_counters[0], ctx->num_sms, s));
    ctx->last_fallbacks = -1;
    return finish_call(ctx, s, false);
}

// ------------------------------------------------------------- gradients --
static pargo_status grad_impl(pargo_ctx* ctx, const pargo_raster* z, const pargo_raster* zref,
                              const pargo_raster* gslope, pargo_raster* gz, double* loss, const pargo_nbr* nbr,
                              int mode, void* stream) {
    if (!ctx) return PARGO_ERR_INVALID_ARG;
    ctx->err.clear();
    pargo_status st;
    if ((st = check_raster(ctx, z, "z")) != PARGO_OK) return st;
    if (z->dtype != PARGO_F32) return fail(ctx, PARGO_ERR_INVALID_ARG, "z must be F32");
    if ((st = check_dims(ctx, z)) != PARGO_OK) return st;
    if ((st = check_nbr(ctx, nbr)) != PARGO_OK) return st;
    const pargo_raster* other = mode == 0 ? zref : gslope;
    if ((st = check_raster(ctx, other, mode == 0 ? "z_ref" : "gslope")) != PARGO_OK) return st;
    if (other->dtype != PARGO_F32) return fail(ctx, PARGO_ERR_INVALID_ARG, "z_ref / gslope must be F32");
    if ((st = check_same(ctx, z, other, "z_ref / gslope")) != PARGO_OK) return st;
    if ((st = check_raster(ctx, gz, "gz")) != PARGO_OK) return st;
    if (gz->dtype != PARGO_F32) return fail(ctx, PARGO_ERR_INVALID_ARG, "gz must be F32");
    if ((st = check_same(ctx, z, gz, "gz")) != PARGO_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    CU(ctx, cudaSetDevice(ctx->device));
    Staged sz, so, sg;
    if ((st = stage_in(ctx, z, kSlotIn0, s, &sz)) != PARGO_OK) return st;
    if ((st = stage_in(ctx, other, kSlotIn1, s, &so)) != PARGO_OK) return st;
    if ((st = stage_out(ctx, gz, kSlotGradOut, &sg)) != PARGO_OK) return st;
    cudaError_t e;
    double* dloss = (double*)slot(ctx, kSlotLoss, 16, &e);
    if (!dloss) return cuda_fail(ctx, e, "loss accumulator");
    CU(ctx, cudaMemsetAsync(dloss, 0, sizeof(double), s));
    GradParams p{};
    p.rows = z->rows;
    p.cols = z->cols;
    p.z = sz.in;
    if (mode == 0) p.zref = so.in; else p.gslope = so.in;
    p.nd7f = float_band(z->nodata, kEpsSlope);
    p.k_fd = (float)(1.0 / (8.0 * (double)(float)z->cellsize));
    p.gz = (float*)sg.out.base;
    p.gz_pitch = sg.out.pitch;
    p.loss = dloss;
    p.error_flag = ctx->d_error;
    if (tma_ok(p.z) && (mode != 0 || tma_ok(p.zref))) {
        CUtensorMap mz, mr;
        if ((st = make_tma_map(ctx, &mz, p.z.base, p.rows, p.cols, p.z.pitch, grad_box_rows(), grad_box_cols())) !=
            PARGO_OK)
            return st;
        if (mode == 0 && (st = make_tma_map(ctx, &mr, p.zref.base, p.rows, p.cols, p.zref.pitch, grad_box_rows(),
                                            grad_box_cols())) != PARGO_OK)
            return st;
        CU(ctx, launch_slope_loss_grad_tma(&mz, &mr, p, mode, s));
    } else {
        CU(ctx, launch_slope_loss_grad(p, mode, s));
    }
    if ((st = unstage_out(ctx, sg, s)) != PARGO_OK) return st;
    const bool sync = sz.host || so.host || sg.host || loss;
    if (loss) {
        double* hp = (double*)pinned(ctx, 64, &e);
        if (!hp) return cuda_fail(ctx, e, "pinned loss");
        CU(ctx, cudaMemcpyAsync(hp, dloss, sizeof(double), cudaMemcpyDeviceToHost, s));
        if ((st = finish_call(ctx, s, true)) != PARGO_OK) return st;
        *loss = hp[0];
        return PARGO_OK;
    }
    return finish_call(ctx, s, sync);
}

pargo_status pargo_slope_fwd(pargo_ctx* ctx, const pargo_raster* z, pargo_raster* slope, const pargo_nbr* nbr,
                             void* stream) {
    return focal_impl(ctx, z, slope, nullptr, nbr, PARGO_SLOPE_FD, PARGO_SLOPE_RATIO, 8, stream);
}

pargo_status pargo_slope_bwd(pargo_ctx* ctx, const pargo_raster* z, const pargo_raster* gslope, pargo_raster* gz,
                             const pargo_nbr* nbr, void* stream) {
    return grad_impl(ctx, z, nullptr, gslope, gz, nullptr, nbr, 1, stream);
}

pargo_status pargo_slope_loss_grad(pargo_ctx* ctx, const pargo_raster* z, const pargo_raster* z_ref, pargo_raster* gz,
                                   double* loss, const pargo_nbr* nbr, void* stream) {
    return grad_impl(ctx, z, z_ref, nullptr, gz, loss, nbr, 0, stream);
}

}  // extern "C"
