/*
 * pargo_gpu.h -- C ABI of the GB300 focal raster operators (libpargo_gpu.so).
 *
 * The PaRGO reference runs its focal operators through
 * RasterOperator<double>::Run() -> Work() (gpro/rasterOperator.h:148-362), a
 * per-cell virtual Operator() sweep over a CellSpace with halos.  Each entry
 * point below replaces one such Run() for one operator:
 *
 *   pargo_slope / pargo_slope_d8  SlopeOperator::Run   apps/morphology/slope/slopeOperator.cpp:51-139
 *   pargo_d8 / pargo_slope_d8     D8Operator::Run      apps/hydrology/flowdird8/d8Operator.cpp:28-101
 *   pargo_fill                    PitRemoveOperator::Run apps/hydrology/pitremove/pitRemoveOperator.cpp:26-72
 *   pargo_sca                     SCAOperator::Run     apps/hydrology/scad8/scaOperator.cpp:37-131
 *   pargo_nbr_parse               operator>>(istream&, Neighborhood&) gpro/neighborhood.h:626-662
 *                                 + Neighborhood::_initCoords checks :110-194
 *
 * and additions with no reference counterpart: batched slope+D8 and batched
 * pit removal over many rasters in one launch, and the forward/backward
 * (adjoint) pair of Horn slope.
 *
 * Conventions
 *  - Plain C: pointers, sizes, enums.  `stream` is a cudaStream_t passed as
 *    void* (NULL = the legacy default stream).
 *  - A raster is row-major with a row pitch in bytes, like CellSpace::_matrix
 *    (gpro/cellSpace.h:230) but with an explicit pitch.  Every raster carries
 *    its own nodata value: inputs use it to detect nodata (|v - nodata| < Eps
 *    with the reference's Eps), outputs write it into nodata cells.
 *  - Buffers may live on the device or on the host.  Host buffers are copied
 *    through the context's device staging and the call returns after the
 *    results are back (synchronous); all-device calls are stream-ordered and
 *    return without waiting.
 *  - The caller owns every buffer.  The library owns only the scratch of a
 *    context (staging, work queues, counters); it grows on demand and is reused.
 *  - Errors are status codes; pargo_last_error() gives the message.  There is
 *    no CPU fallback: without a usable GPU every compute call fails with
 *    PARGO_ERR_NO_DEVICE or PARGO_ERR_CUDA.
 *  - One host thread per context at a time.
 */
#ifndef PARGO_GPU_H
#define PARGO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PARGO_ABI_VERSION 1

typedef enum pargo_status {
    PARGO_OK = 0,
    PARGO_ERR_INVALID_ARG = 1,     /* bad pointer, size, dtype, pitch or option */
    PARGO_ERR_NBR_UNSUPPORTED = 2, /* the operator needs a 3x3 Moore neighbourhood */
    PARGO_ERR_NOT_CONVERGED = 3,   /* fill hit its round cap before the fixpoint */
    PARGO_ERR_CYCLE = 4,           /* SCA: some in-degree is never consumed */
    PARGO_ERR_CUDA = 5,            /* a CUDA runtime or launch error */
    PARGO_ERR_NO_DEVICE = 6,       /* no CUDA device */
    PARGO_ERR_OUT_OF_MEMORY = 7,
    PARGO_ERR_DEVICE_TIMEOUT = 8   /* a bounded device-side wait gave up */
} pargo_status;

typedef enum pargo_dtype {
    PARGO_F32 = 0,
    PARGO_F64 = 1,
    PARGO_I8 = 2,
    PARGO_I16 = 3,
    PARGO_I32 = 4
} pargo_dtype;

typedef enum pargo_location { PARGO_HOST = 0, PARGO_DEVICE = 1 } pargo_location;

typedef struct pargo_raster {
    void* data;       /* cell (0, 0) */
    int32_t dtype;    /* pargo_dtype */
    int32_t location; /* pargo_location */
    int64_t rows;
    int64_t cols;
    int64_t pitch;    /* bytes from one row to the next; 0 = cols * element size */
    double nodata;    /* MetaData::noData (gpro/metaData.h:55) */
    double cellsize;  /* MetaData::cellSize; the reference stores it as float
                         (gpro/metaData.h:56) and the operators use that float
                         value, so it is rounded to float before use */
} pargo_raster;

/* A parsed .nbr neighbourhood: the cell count and the MBR of the offsets.
 * The focal operators use only int(sqrt(count))/2 (slopeOperator.cpp:55) and
 * the work rectangle the MBR implies (gpro/neighborhood.h:423-467). */
typedef struct pargo_nbr {
    int32_t count;
    int32_t min_row, min_col, max_row, max_col;
} pargo_nbr;

/* SlopeAlgor, apps/morphology/slope/slopeOperator.h:18-26 */
typedef enum pargo_slope_method {
    PARGO_SLOPE_FD = 0, PARGO_SLOPE_FFD = 1, PARGO_SLOPE_MD = 2, PARGO_SLOPE_SD = 3,
    PARGO_SLOPE_SFD = 4, PARGO_SLOPE_TFD = 5, PARGO_SLOPE_TFDW = 6
} pargo_slope_method;

typedef enum pargo_slope_units {
    PARGO_SLOPE_RATIO = 0,  /* rise/run, as the reference writes it (slopeOperator.cpp:86) */
    PARGO_SLOPE_DEGREES = 1 /* atan(rise/run) in degrees */
} pargo_slope_units;

typedef enum pargo_sca_contract {
    PARGO_SCA_CONVERGED = 0, /* the reference rule iterated until every in-degree is consumed */
    PARGO_SCA_SHIPPED = 1    /* what the shipped operator's single accumulation sweep leaves (scaOperator.cpp:126) */
} pargo_sca_contract;

typedef struct pargo_fill_opts {
    double gap;         /* reference: 0.0005 (pitRemoveOperator.cpp:36) */
    double init_level;  /* reference: 10000.0 (pitRemoveOperator.cpp:41) */
    int64_t max_rounds; /* <= 0: no cap, one persistent launch over a device work queue;
                           > 0: worklist rounds (CUDA graphs of round launches), at most this many */
} pargo_fill_opts;

typedef struct pargo_fill_stats {
    int64_t rounds;        /* worklist rounds launched (1 for the persistent launch) */
    int64_t active_rounds; /* rounds whose worklist was not empty (1 for the persistent launch) */
    int64_t tile_visits;   /* tiles relaxed, summed over rounds */
    int64_t local_iterations; /* relaxation iterations inside tiles, summed over visits */
    int64_t raised_cells;  /* cells whose filled level is above the DEM */
    double rounds_ms;      /* device time of the relaxation (CUDA events on the library's stream) */
} pargo_fill_stats;

typedef struct pargo_ctx pargo_ctx;

/* Context on CUDA device `device`. */
pargo_status pargo_create(int device, pargo_ctx** out);
pargo_status pargo_destroy(pargo_ctx* ctx);
const char* pargo_last_error(const pargo_ctx* ctx);
int pargo_abi_version(void);

/* Parse .nbr text: a count N, then N lines "dRow dCol weight"; N >= 100 means
 * an automatic sqrt(N) x sqrt(N) square (neighborhood.h:626-662).  Rejects an
 * empty set, a set without (0, 0) and duplicates (neighborhood.h:110-140). */
pargo_status pargo_nbr_parse(const char* text, pargo_nbr* out);

/* Slope of `dem` into `slope` (F32 or F64).  dem: F32 or F64. */
pargo_status pargo_slope(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* slope, const pargo_nbr* nbr,
                         int method, int units, void* stream);

/* D8 codes of `dem` into `d8`.  dir_type 8: receiver index 0..8 of the 3x3
 * window, -1 flat/pit (d8Operator.cpp:78-88); any other dir_type: the
 * ArcGIS-style bit sum (:89-97).  d8: I8 (dir_type 8 only), I16, I32, F32 or F64. */
pargo_status pargo_d8(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* d8, const pargo_nbr* nbr,
                      int dir_type, void* stream);

/* Fused slope + D8: one read of the DEM, either output may be NULL. */
pargo_status pargo_slope_d8(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* slope, pargo_raster* d8,
                            const pargo_nbr* nbr, int method, int units, int dir_type, void* stream);

/* Autotuner of the fused slope+D8 kernel (no reference counterpart).  It times
 * each kernel variant `reps` times on `dem` (an F32 device raster with
 * 16-byte aligned rows) and keeps the fastest for rasters of the same size
 * class (power of two of the cell count).  The variants span the tiled
 * kernel's tile rows (cells per thread) and CTAs per SM, and the strip
 * walk's rows per TMA stage, stages per segment (segment height) and CTAs
 * per SM; the halo every variant loads is the stencil's MBR
 * (gpro/neighborhood.h:423-467: one cell for the 3x3 window).  *best gets the
 * chosen variant and times_ms[0 .. max_times-1] the per-variant milliseconds
 * (either may be NULL).  The choice is kept in the context and persisted in a
 * JSON cache keyed by (operation, device, size class) that pargo_create
 * reads, so later contexts -- an application's main, say -- run the tuned
 * kernel: the file is $PARGO_TUNE_CACHE (set but empty: no cache), else
 * $XDG_CACHE_HOME/pargo_gb300/tune.json, else ~/.cache/pargo_gb300/tune.json.
 * PARGO_FOCAL_VARIANT in the environment overrides every choice.  Every
 * variant computes the same bytes. */
pargo_status pargo_tune_focal(pargo_ctx* ctx, const pargo_raster* dem, int reps, int* best, float* times_ms,
                              int max_times);

/* The focal kernel variants: their number, the name of variant v ("tile-r32-b5":
 * 32-row tiles at 5 CTAs per SM; "strip-s6x8-b5": 6-row stages, 8 stages per
 * segment, 5 CTAs per SM; NULL when v is out of range), and the variant a
 * context runs for a fused slope + D8 of `cells` cells (PARGO_FOCAL_VARIANT,
 * else the tuned or cached choice for the size class, else the size default). */
int pargo_focal_num_variants(void);
const char* pargo_focal_variant_name(int v);
int pargo_focal_variant(const pargo_ctx* ctx, int64_t cells);

/* Planchon-Darboux pit removal: the fixpoint the reference's Gauss-Seidel
 * sweeps reach (any visiting order reaches the same one).  dem: F32 or F64;
 * wdem: F64 (the reference's values) or F32 (those values rounded to float).
 * opts may be NULL (reference constants); stats may be NULL.  Without a round
 * cap the relaxation is one persistent launch whose tiles queue their
 * neighbours on the device; PARGO_FILL_ROUNDS=1 in the environment selects the
 * round form instead.  PARGO_ERR_DEVICE_TIMEOUT: a device-side wait found no
 * progress for about two seconds. */
pargo_status pargo_fill(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* wdem, const pargo_nbr* nbr,
                        const pargo_fill_opts* opts, pargo_fill_stats* stats, void* stream);

/* Batched pit removal: `count` independent rasters (all on the device) in one
 * persistent relaxation.  The rasters are packed side by side into one mosaic
 * whose nodata separates them -- each raster's ring is a nodata level in the
 * reference (PitRemoveOperator's wdem is initialised from copyLayerInfo), so
 * no level of one raster is a neighbour of a level of another -- and every
 * output holds exactly what pargo_fill gives for its raster.  dems: all F32 or
 * all F64 with one nodata value (otherwise the rasters are filled one by one,
 * with the same results); wdems: F64 or F32.  stats (may be NULL) covers the
 * whole batch.  No reference counterpart: the reference removes pits raster by
 * raster (pPitRemove.cpp).  Synchronous. */
pargo_status pargo_batch_fill(pargo_ctx* ctx, int count, const pargo_raster* dems, pargo_raster* wdems,
                              const pargo_nbr* nbr, const pargo_fill_opts* opts, pargo_fill_stats* stats,
                              void* stream);

/* Device-resident hydrology chain, as the reference runs it through files
 * (pPitRemove.cpp:129 -> pD8.cpp:113 -> pSCA.cpp:59): pit removal, then slope
 * and D8 on the float64 levels (what the reference D8 reads from the Float64
 * pit-remove output), then SCA on those codes.  Every output may be NULL
 * except that at least one must be given; wdem F64/F32, slope F32/F64,
 * d8 I8/I16/I32/F32/F64 (dir_type 8), sca F64/F32.  Synchronous. */
pargo_status pargo_hydro_pipeline(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* wdem, pargo_raster* slope,
                                  pargo_raster* d8, pargo_raster* sca, const pargo_nbr* nbr,
                                  const pargo_fill_opts* opts, int slope_method, int slope_units, int sca_contract,
                                  pargo_fill_stats* stats, void* stream);

/* D8 specific catchment area (upslope cell count, as the reference computes
 * it).  d8: F64 codes as the reference writes them, or I8/I16/I32 codes with
 * the raster's nodata as sentinel; sca: F64 or F32. */
pargo_status pargo_sca(pargo_ctx* ctx, const pargo_raster* d8, pargo_raster* sca, const pargo_nbr* nbr,
                       int contract, void* stream);

/* Topographic wetness index ln(sca / slope), replacing TWIOperator::Run()
 * (apps/hydrology/twi/TWIOperator.cpp:42-69): a work cell is nodata (the SCA
 * raster's nodata) when any value of its 3x3 window, in either input, equals
 * the SCA raster's nodata; slope below 1e-7 counts as 1e-7; ring cells get the
 * output's nodata.  slope, sca, twi: F32 or F64; computed in FP32 (about 1e-6
 * relative to the reference's FP64). */
pargo_status pargo_twi(pargo_ctx* ctx, const pargo_raster* slope, const pargo_raster* sca, pargo_raster* twi,
                       const pargo_nbr* nbr, void* stream);

/* MFD-md flow partition weights, replacing MFDOperator::Operator()
 * (apps/hydrology/flowdirmfdmd/mfdOperator.cpp:39-125) run over the raster: `weights` points to
 * 8 rasters, layer i holding the share of the cell's flow sent to window
 * position i (positions in row-major order, the centre skipped).  A cell's
 * weights are drop_i^pe * l_i / sum over its strictly lower valid neighbours,
 * pe = (1 - e) * min(max drop, 1) + e with e = slp_exp; a nodata cell (|z -
 * nodata| <= 1e-6) and the ring get the DEM's nodata in every layer.  dem: F32
 * or F64; weights: F32 or F64, computed in FP32 (about 1e-6 relative). */
pargo_status pargo_mfd(pargo_ctx* ctx, const pargo_raster* dem, pargo_raster* weights, const pargo_nbr* nbr,
                       double slp_exp, void* stream);

/* MFD specific catchment area, replacing the scamfdmd SCAOperator
 * (apps/hydrology/scamfdmd/scaOperator.cpp:43-113) as its single raster-order
 * sweep leaves it: a valid cell takes 1 + the sum, in window order, of
 * sca(q) * w(q -> cell) over the neighbours q that have finished before it in
 * that sweep.  Sums are FP64 with the reference's operation order, so the
 * output is bit-identical given the same weights.  weights: 8 rasters (F32 or
 * F64), nodata = |w0 - nodata| < 1e-6; sca: F32 or F64 with weight layer 0's
 * nodata.  A cell waits only on the cells before it in raster order, so
 * weights that form a cycle are evaluated as the sweep evaluates them (a
 * cycle's cells never pull each other's later inflows) rather than refused;
 * PARGO_ERR_CYCLE would report a valid cell left unprocessed. */
pargo_status pargo_sca_mfd(pargo_ctx* ctx, const pargo_raster* weights, pargo_raster* sca, const pargo_nbr* nbr,
                           void* stream);

/* Load estimator, intensity-ratio mode: the compute layer of `count` data
 * rasters (same shape, F32 or F64), replacing ComputeLayer::init +
 * Transformation::run (gpro/computeLayer.h:210-262,
 * gpro/transformation.h:155-229).  Compute cell (r, c) covers the data rows
 * r*grain+1 .. (r+1)*grain and columns c*grain+1 .. (c+1)*grain of the 3x3
 * work rectangle (clipped to the raster) and holds the sum, layer by layer and
 * row by row, of valid_load per valid cell (|v - nodata| > 1e-7, each
 * layer's own nodata) and nodata_load per other cell; the FP64 sums are the
 * reference's bit for bit.  compute_ring != 0 gives the compute layer a 3x3
 * neighbourhood of its own: its ring cells stay 0.  load: F64 or F32 of
 * pargo_compute_load_dims.  An application's own estimate function (the
 * reference's Transformation subclasses) writes its compute layer by other
 * means and goes straight to pargo_load_decompose. */
pargo_status pargo_compute_load_dims(int64_t rows, int64_t cols, int grain, int64_t* crows, int64_t* ccols);
pargo_status pargo_compute_load(pargo_ctx* ctx, int count, const pargo_raster* data, const pargo_nbr* nbr, int grain,
                                int compute_ring, double nodata_load, double valid_load, pargo_raster* load,
                                void* stream);

/* Row-wise decomposition of a compute layer into nparts by load, replacing
 * DeComposition::valRowDcmp (gpro/deComposition.h:305-393) and the mapping to
 * data rows of ComputeLayer::getCompuLoad (gpro/computeLayer.h:380-443): row
 * loads (cells above -9999 and above the load raster's nodata by more than
 * 1e-7) on the device, the greedy cuts on the host.  comp_rows (may be NULL)
 * receives each part's compute rows {begin, end}; bounds each part's data
 * rectangle {minRow, minCol, maxRow, maxCol} in a data_rows x data_cols
 * raster with a 3x3 neighbourhood.  Synchronous. */
pargo_status pargo_load_decompose(pargo_ctx* ctx, const pargo_raster* load, int compute_ring, int64_t data_rows,
                                  int64_t data_cols, const pargo_nbr* nbr, int nparts, int64_t* comp_rows,
                                  int64_t* bounds, void* stream);

/* Batched fused slope + D8 over `count` independent rasters in one persistent
 * launch; slopes / d8s may be NULL (no such output) and all rasters must be on
 * the device.  The launch's warps claim work items -- 128-column by 48-row
 * segments of every raster -- from one device queue.  The queue holds the
 * rasters heaviest first by the load estimator's intensity-ratio estimate
 * (Transformation::Operator, gpro/transformation.h:155-197: valid_load per
 * cell with |v - nodata| > 1e-7, nodata_load per other cell), each raster's
 * segments together; the estimate is counted per segment on the device the
 * first time a batch description (buffers, shapes, options) is seen and kept
 * with the batch's other device tables.  The order balances the work only and
 * never changes an output.  pargo_batch_slope_d8
 * uses the defaults: by intensity, nodata_load 0, valid_load 1 (the
 * reference's "-nodataLoad 0 -validLoad 1", apps/spatial/reclassify/
 * pRelclassify.cpp:22).  Configurations outside the strip walk (slope methods
 * other than Horn, degrees, dirType 256, unaligned rows) run a tiled launch
 * whose queue is ordered by raster size. */
typedef enum pargo_batch_order {
    PARGO_BATCH_BY_INTENSITY = 0, /* rasters by estimated load, heaviest first */
    PARGO_BATCH_BY_SIZE = 1       /* raster by raster, largest raster first */
} pargo_batch_order;

typedef struct pargo_batch_opts {
    double nodata_load;  /* Transformation::_nodataLoad (gpro/transformation.h:67), >= 0 */
    double valid_load;   /* Transformation::_validLoad (gpro/transformation.h:68), >= 0 */
    int32_t order;       /* pargo_batch_order */
    int32_t reserved;    /* 0 */
} pargo_batch_opts;

pargo_status pargo_batch_slope_d8(pargo_ctx* ctx, int count, const pargo_raster* dems, pargo_raster* slopes,
                                  pargo_raster* d8s, const pargo_nbr* nbr, int method, int units, int dir_type,
                                  void* stream);
pargo_status pargo_batch_slope_d8_ex(pargo_ctx* ctx, int count, const pargo_raster* dems, pargo_raster* slopes,
                                     pargo_raster* d8s, const pargo_nbr* nbr, int method, int units, int dir_type,
                                     const pargo_batch_opts* opts, void* stream);

/* The work queue the batched strip walk uses for these rasters and options:
 * *n_out = the number of segments; for the first `cap` queue positions i,
 * raster[i] (the caller's index), segment[i] (within its raster: strip
 * segment % strips, band segment / strips, strips = ceil(cols / 128)) and
 * load[i] (its estimated load); any output pointer may be NULL.  dems: F32 on
 * the device.  Synchronous.  No reference counterpart (the reference splits
 * rows among MPI ranks by the same estimate, deComposition.h:305-393). */
pargo_status pargo_batch_queue(pargo_ctx* ctx, int count, const pargo_raster* dems, const pargo_batch_opts* opts,
                               int64_t cap, int64_t* n_out, int32_t* raster, int64_t* segment, double* load,
                               void* stream);

/* Differentiable Horn (FD) slope.  Forward: slope of z into `slope`.
 * Backward: given dL/dslope per cell (`gslope`, F32), accumulate dL/dz into
 * `gz` (F32, overwritten).  Subgradient convention: at zero slope the
 * derivative is taken as 0; windows touching nodata contribute nothing. */
pargo_status pargo_slope_fwd(pargo_ctx* ctx, const pargo_raster* z, pargo_raster* slope, const pargo_nbr* nbr,
                             void* stream);
pargo_status pargo_slope_bwd(pargo_ctx* ctx, const pargo_raster* z, const pargo_raster* gslope, pargo_raster* gz,
                             const pargo_nbr* nbr, void* stream);

/* Fused forward + backward of L = sum over cells of (slope(z) - slope(z_ref))^2:
 * writes dL/dz into `gz` (F32) and L into *loss (may be NULL). */
pargo_status pargo_slope_loss_grad(pargo_ctx* ctx, const pargo_raster* z, const pargo_raster* z_ref,
                                   pargo_raster* gz, double* loss, const pargo_nbr* nbr, void* stream);

/* SCA without any device allocation, for callers that cannot allocate (a
 * plugin handed only device buffers and a stream, a host runtime that owns the
 * whole device-memory budget, code that must not take the allocator's locks).
 * No counterpart in the reference: same results as pargo_sca, but the scratch
 * is a fixed array inside the library's device image instead of a context, so
 * there is no context argument.  Rasters must be on the device and hold at
 * most PARGO_SCA_NOALLOC_MAX_CELLS cells (larger ones: PARGO_ERR_INVALID_ARG);
 * the array (21 bytes per cell, ~22 MB) stays allocated on every GPU that loads
 * the library until the process exits.  All calls share that array: calls that
 * overlap on the GPU race, so serialise them.  The first call on a device looks
 * up the array's address (once per device) and keeps it until the process
 * exits, so calls after cudaDeviceReset are not supported.  Layout rules as
 * elsewhere (pitch a whole number of elements covering a row, data aligned to
 * its element size; otherwise PARGO_ERR_INVALID_ARG).  Synchronous: returns
 * after the result and the completion count are known, so it must not be
 * called on a stream that is being captured. */
#define PARGO_SCA_NOALLOC_MAX_CELLS (1LL << 20)
pargo_status pargo_sca_noalloc(const pargo_raster* d8, pargo_raster* sca, const pargo_nbr* nbr, int contract,
                               void* stream);

/* Number of D8 cells of the last slope+D8/D8 call that took the exact FP64
 * path (the FP32 decision was not certified), for diagnostics. */
int64_t pargo_last_d8_fallbacks(const pargo_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* PARGO_GPU_H */
