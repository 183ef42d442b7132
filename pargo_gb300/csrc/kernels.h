// kernels.h -- host-side launch interface between the C ABI (abi.cu) and the
// kernel translation units.  Everything here takes device pointers only.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace pargo {

// One raster as the kernels see it (device memory).
struct DevRaster {
    const char* base;  // input rasters
    char* out;         // output rasters (same pointer, writable)
    int64_t rows, cols, pitch;
    int32_t dtype;
    double nodata;
};

struct FocalParams {
    int64_t rows, cols;
    Band<float> nd6f, nd7f;   // nodata bands for float input (Eps 1e-6 D8/fill, 1e-7 slope)
    Band<double> nd6d, nd7d;  // the same for double input
    SlopeConsts sk;
    int do_slope, do_d8, dir_type;
    int fast_out;  // slope F32 / D8 I8 with 16- / 4-byte aligned rows: vector stores
    int fd;        // Horn (FD) slope or no slope: the tiled fast path applies
    OutView slope, d8;
    unsigned long long* fallbacks;  // device counter of exact-path D8 cells (may be null)
    int* error_flag;                // device flag: a bounded wait gave up
};

// load.cu: the load estimator (compute-intensity layer, row loads).
constexpr int kMaxLoadLayers = 8;
struct LoadParams {
    int64_t rows, cols;            // data rasters
    int count;                     // data layers summed
    InView data[kMaxLoadLayers];
    Band<float> ndf[kMaxLoadLayers];               // per layer: |v - nodata| <= 1e-7 for float data
    long long nd_lo[kMaxLoadLayers], nd_hi[kMaxLoadLayers];  // the same bands as keys for double data
    int grain, compute_ring;
    double nodata_load, valid_load;
    int integral;                  // integer loads whose sums stay below 2^53: count, then scale
    int64_t crows, ccols;
    OutView load;
};
cudaError_t launch_compute_load(const LoadParams& p, int num_sms, cudaStream_t s);
cudaError_t launch_row_load(const InView& load, int64_t crows, int64_t ccols, double nodata, double* row_load,
                            int num_sms, cudaStream_t s);

// focal.cu
cudaError_t launch_focal_tma(const CUtensorMap* map, const FocalParams& p, int fast_out, int variant, int num_sms,
                             cudaStream_t s);
int focal_num_variants();
int focal_variant_rows(int v);  // tile rows of variant v (its TMA box is that + 2)
bool focal_variant_is_strip(int v);
cudaError_t launch_focal_generic(const InView& dem, const FocalParams& p, cudaStream_t s);
size_t focal_tma_smem_bytes();
int focal_tma_tile_rows();
int focal_tma_tile_cols();
int focal_tma_box_cols();
int focal_tma_box_rows();
// Strip-walk form of the same kernel (warp-private TMA pipelines down 128-cell
// column strips, segments claimed from `claim`).
cudaError_t launch_focal_strip(const CUtensorMap* map_stage, const CUtensorMap* map_prime, const InView& dem,
                               const FocalParams& p, int fast_out, int variant, unsigned long long* counters,
                               uint32_t* slow_items, int num_sms, cudaStream_t s);
int focal_strip_stage_rows(int variant, int do_slope, int do_d8);
int focal_default_strip_variant();
const char* focal_variant_name(int variant);
size_t focal_strip_slow_bytes(int64_t rows, int64_t cols);

// Batched slope+D8 (focal.cu): device tables of per-raster descriptors/params.
cudaError_t launch_batch_tma(const CUtensorMap* maps, const FocalParams* params, const int64_t* tile_start,
                             const int64_t* ntx_of, int count, int64_t total_tiles, int do_slope, int do_d8,
                             unsigned long long* claim, unsigned long long* fallbacks, int* error_flag, int num_sms,
                             cudaStream_t s);
int64_t batch_strip_segments(int64_t rows, int64_t cols, int* nstrips);
int batch_strip_segment_rows();
int batch_strip_segment_cols();
cudaError_t launch_batch_strip(const CUtensorMap* maps, const FocalParams* params, const InView* dems,
                               const int64_t* seg_start, const int* nstrips, const uint64_t* order, int count,
                               int64_t nsegs, int do_slope, int do_d8, unsigned long long* counters,
                               uint64_t* slow_items, unsigned long long* fallbacks, int* error_flag, int num_sms,
                               cudaStream_t s);
// One raster of a batch, for the segments' compute-intensity count.
struct SegLoadRaster {
    InView dem;             // float32
    int64_t rows, cols;
    Band<float> nd;         // |v - nodata| <= Eps 1e-7: a nodata cell of the intensity estimate
    int64_t seg_start;      // its first segment
    int nstrips;
};
cudaError_t launch_batch_segment_valid(const SegLoadRaster* rs, int count, int64_t nsegs, uint32_t* out, int num_sms,
                                       cudaStream_t s);
cudaError_t launch_batch_generic(const FocalParams* params, const InView* dems, const int64_t* cell_start, int count,
                                 int64_t total_cells, unsigned long long* fallbacks, int num_sms, cudaStream_t s);

// focal64.cu: slope + D8 over a float64 surface (the pit-removed levels),
// TMA-tiled; optionally copies the levels to `copy` (the filled-DEM output).
struct Focal64Params {
    FocalParams f;          // rows, cols, outputs, slope constants, dir_type
    int64_t wpitch;         // bytes per row of the levels
    int nodata_is_inf;      // the levels mark nodata with +inf (the pipeline) instead of a band
    int do_copy;
    OutView copy;           // filled-DEM output (+inf written as copy.nodata)
    unsigned long long* raised;  // cells whose level is above the DEM (needs dem), may be null
    const void* dem;
    int64_t dem_pitch;
    int dem_f64;
};
// Output rows [row_begin, row_end) (row_end < 0: to the last row); row_begin
// must be a multiple of focal64_tile_rows().
cudaError_t launch_focal64_tma(const CUtensorMap* map, const Focal64Params& p, int num_sms, cudaStream_t s,
                               int64_t row_begin = 0, int64_t row_end = -1);
int focal64_tile_rows();
int focal64_box_cols();

// fill.cu
struct FillParams {
    int64_t rows, cols;
    const void* dem;        // float32 or float64 (dem_f64)
    int64_t dem_pitch;      // bytes
    int dem_f64;
    Band<float> nd6f;       // nodata band of the DEM (Eps 1e-6), float input
    Band<double> nd6d;      // the same for float64 input
    double gap, init_level;
    double* w;              // working levels, rows x w_stride doubles, +inf marks nodata levels
    int64_t w_stride;       // elements per row of w (a multiple of 2: 16-byte rows for TMA)
    int64_t tiles_y, tiles_x;
};
struct FillScratch {
    int32_t* list_a;        // tile worklists (capacity tiles_y * tiles_x)
    int32_t* list_b;
    int32_t* counts;        // [0] = length of list_a, [1] = length of list_b, [2] = claim cursor
    int32_t* queued;        // per-tile flag: already in the next worklist
    unsigned long long* visits;
    unsigned long long* changed;
    unsigned long long* active;  // rounds that found a non-empty worklist
    unsigned long long* iters;   // local relaxation iterations, summed over tile visits
    // persistent form: list_a and list_b, contiguous, are one ring of ring_cap
    // = 2 * tiles slots; q = [head, tail, pending, progress, error]
    int32_t* ring;
    int64_t ring_cap;
    unsigned long long* q;
    // per tile, 5 words: the halo cells that changed since its last visit --
    // [0] top row, [1] bottom row, [2] left column, [3] right column (bit =
    // tile column or row), [4] corners (bit 0 TL, 1 TR, 2 BL, 3 BR; bit 31:
    // relax every cell, set for first visits)
    uint32_t* halo_chg;
};
cudaError_t fill_init(const FillParams& p, const FillScratch& s, cudaStream_t st);
cudaError_t fill_round(const FillParams& p, const FillScratch& s, int parity, int num_sms, cudaStream_t st);
cudaError_t fill_persistent(const FillParams& p, const FillScratch& s, long long patience, int num_sms, cudaStream_t st);
cudaError_t fill_finish(const FillParams& p, const OutView& out, unsigned long long* raised, cudaStream_t st);
// Batched fill: each raster's place in one mosaic DEM, and its output.
struct FillBatchItem {
    const void* dem;        // the raster's DEM (float32, or float64 for a float64 batch)
    int64_t pitch;          // bytes
    int64_t rows, cols;
    int64_t oy, ox;         // its cell (0, 0) in the mosaic
    Band<float> nd6f;       // its own nodata band (Eps 1e-6)
    Band<double> nd6d;
    OutView out;            // its filled output
};
cudaError_t fill_mosaic_pack(const FillBatchItem* items, int count, int64_t max_cells, void* mosaic, int64_t mrows,
                             int64_t mstride, int f64, double nd, cudaStream_t st);
cudaError_t fill_mosaic_finish(const FillParams& p, const FillBatchItem* items, int count, int64_t max_cells,
                               unsigned long long* raised, cudaStream_t st);
int fill_tile_rows();
int fill_tile_cols();

// sca.cu
struct ScaParams {
    int64_t rows, cols;
    InView d8;
    double nodata;          // nodata of the D8 input
    OutView out;
    int shipped;            // 0 converged, 1 shipped single sweep
};
struct ScaScratch {
    int32_t* indeg;         // remaining in-degree per cell
    unsigned long long* conv;  // accumulated converged upstream counts
    unsigned long long* ship;  // accumulated pulled counts (shipped contract)
    uint8_t* flags;         // bit0 source, bit1 not-done, bit2 valid, bit3 completed
    unsigned long long* counters;  // [0] completed cells, [1] valid cells, [2] last-cell conv, [3] last-cell ship
    uint32_t* forest;       // tiled SCA: per cell, the in-tile forest of the first pass for the final one
};
cudaError_t sca_run(const ScaParams& p, const ScaScratch& s, cudaStream_t st);

// Tiled SCA (sca_tiled.cu): per 64 x 64 tile, tree sums in shared memory;
// across tiles, a forest of tile exits.  Node = tile * 256 + border slot.
struct ScaTiles {
    int64_t tiles_x, tiles_y;
    int32_t* exit_of;   // border cell -> exit node its in-tile path reaches (-1: ends in the tile)
    int32_t* yslot;     // exit node -> entry node its flow enters (-1: not an exit)
    int32_t* xpar;      // exit node -> exit-forest parent (-1: root)
    unsigned long long* tot;   // exit: packed count of feeding exits, bad count, and sum (sca_tiled.cu)
    unsigned long long* tin;   // entry: external inflow total
    uint32_t* tinb;     // bit 0, entry: some inflow was not pulled (shipped contract); bit 1, exit: a leaf
};
constexpr int kScaTile = 64;
constexpr int kScaSlots = 256;
size_t sca_tiles_bytes(int64_t rows, int64_t cols);  // node arrays for a raster
ScaTiles sca_tiles_layout(void* base, int64_t rows, int64_t cols);
// conv[c] = upslope count incl. c; ship[c] = 1 if some cell of c's subtree has
// an inflow the single raster-order sweep does not pull, else 0.
// counters: [0] completed cells, [1] valid cells, [2] last-cell conv, [3]
// last-cell ship, [4] exits, [5] exits completed, [6] inflows from the ring.
cudaError_t sca_run_tiled(const ScaParams& p, const ScaScratch& s, const ScaTiles& t, cudaStream_t st);

// twi.cu
struct TwiParams {
    int64_t rows, cols;
    InView slope, sca;
    OutView out;
    double sca_nodata;     // the value both inputs are tested against (the SCA raster's nodata)
    long long nd_bits;     // its bit pattern, for double inputs
    int nd_is_float;       // it is exactly a float (else no float input can equal it)
    float nd_f;            // and that float
    float sca_nd_f;        // the nodata written on nodata windows, as float
    float out_nd_f;        // the output's nodata (ring), as float
    float eps_cut;         // the least float >= 1e-7
};
cudaError_t launch_twi(const TwiParams& p, int num_sms, cudaStream_t st);

// mfd.cu
struct MfdParams {
    int64_t rows, cols;
    InView dem;                    // F32 or F64
    Band<float> ndf;               // DEM nodata, |z - nd| <= 1e-6, float input
    long long ndd_lo, ndd_hi;      // the same band as order-preserving keys, double input
    float den_card, den_diag;      // cs, 1.414 cs
    float len_card, len_diag;      // 0.5 cs, 0.354 cs
    float slp_exp;
    OutView w[8];                  // layer i: window position i (i < 4) or i + 1
};
cudaError_t launch_mfd_weights(const MfdParams& p, int num_sms, cudaStream_t st);

struct ScaMfdParams {
    int64_t rows, cols;
    InView w[8];
    long long nd_lo, nd_hi;        // weight layer 0 nodata band (|w - nd| < 1e-6) as keys
    double nodata;                 // written on nodata cells and the ring
    OutView out;
    int32_t* cnt;                  // round form: earlier non-source inflows not yet processed
    uint8_t* flags;                // valid, source, never done, done; bits 4-7 the round form's release mask
    double* sca;
    int32_t* list_a;
    int32_t* list_b;
    int32_t* counts;               // round form: [0] length of list_a, [1] of list_b, [2] finished blocks
    unsigned long long* totals;    // [0] valid cells, [1] processed cells, [2] nodata cells with weights
    int* error_flag;               // a bounded wait of the band form gave up
};
cudaError_t launch_sca_mfd_init(const ScaMfdParams& p, int num_sms, cudaStream_t st);
// The round form's counters and first frontier (after the init).
cudaError_t launch_sca_mfd_counts(const ScaMfdParams& p, int num_sms, cudaStream_t st);
cudaError_t launch_sca_mfd_round(const ScaMfdParams& p, int parity, int num_sms, cudaStream_t st);
cudaError_t launch_sca_mfd_output(const ScaMfdParams& p, int num_sms, cudaStream_t st);
// The band form (every dependency of the sweep points forward in raster
// order): per-cell records, then warps walking 32-row bands in step.
// `records`: sca_mfd_band_bytes(rows, cols, all weights F32) bytes; `words`:
// 1 + ceil((rows - 2) / 32) ints.
size_t sca_mfd_band_bytes(int64_t rows, int64_t cols, bool f32);
cudaError_t launch_sca_mfd_band(const ScaMfdParams& p, void* records, int* words, int num_sms, cudaStream_t st);

// grad.cu
struct GradParams {
    int64_t rows, cols;
    InView z, zref, gslope;
    Band<float> nd7f;
    float k_fd;             // 1 / (8 cs)
    float* gz;
    int64_t gz_pitch;
    OutView slope;
    double* loss;           // device accumulator (may be null)
    int* error_flag;        // a bounded wait for the staged boxes gave up (TMA form)
};
cudaError_t launch_slope_loss_grad(const GradParams& p, int mode, cudaStream_t st);
// TMA form: mz (and, for mode 0, mr) are tensor maps of z (z_ref) with a
// grad_box_cols() x grad_box_rows() box; inputs float32, 16-byte aligned rows.
int grad_box_rows();
int grad_box_cols();
cudaError_t launch_slope_loss_grad_tma(const CUtensorMap* mz, const CUtensorMap* mr, const GradParams& p, int mode,
                                       cudaStream_t st);

}  // namespace pargo
