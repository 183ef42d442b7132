/*
 * Oracle driver around the UNMODIFIED PaRGO reference operators (test
 * infrastructure only; built into oracle/_ref/ by oracle/Makefile.ref from
 * the reference sources where they lie, never shipped).
 *
 * Each entry point mirrors what the reference mains do
 * (apps/morphology/slope/pSlope.cpp:129-150, apps/hydrology/flowdird8/pD8.cpp:104-135,
 * apps/hydrology/pitremove/pPitRemove.cpp:104-129, apps/hydrology/scad8/pSCA.cpp:39-78):
 * Application::START, RasterLayer::readNeighborhood + readFile, copyLayerInfo,
 * operator setters, Run().  Two deliberate differences, both forced by the
 * reference itself:
 *   - every layer is read with ROWWISE_DCMP: with the shipped NON_DCMP default
 *     writeFile() returns false (gpro/rasterLayer.h:1011-1013), and one rank's
 *     row band is the whole raster, so the result matrix is read directly;
 *   - the program type is MPI_Type (serial) for fill and SCA, whose OpenMP path
 *     races on the phase flag (pitRemoveOperator.cpp:39-50); slope and D8 may
 *     use MPI_OpenMP_Type (their Operator is stateless).
 * ref_sca_converged subclasses the reference SCAOperator and re-arms the sweep
 * while any in-degree is still positive; the shipped operator stops after one
 * accumulation sweep (scaOperator.cpp:126).
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <omp.h>
#include "mpi.h"
#include "gdal_priv.h"
#include "application.h"
#include "rasterLayer.h"

#include "slopeOperator.h"
#undef Eps
#include "d8Operator.h"
#undef Eps
#include "pitRemoveOperator.h"
#undef Eps
#include "scaOperator.h"
#undef Eps
#include "TWIOperator.h"
#undef Eps
#include "computeLayer.h"  // defines Eps 1e-7, which transformation.h uses
#include "transformation.h"
#include "deComposition.h"
#undef Eps

using namespace GPRO;

namespace {

void start(ProgramType t) {
    static char prog[] = "pargo_ref";
    static char* argv_storage[] = {prog, nullptr};
    char** argv = argv_storage;
    Application::START(t, 1, argv);
}

void copy_out(RasterLayer<double>& layer, double* out, int rows, int cols) {
    const double* m = layer.cellSpace()->_matrix;
    memcpy(out, m, sizeof(double) * (size_t)rows * cols);
}

/* Counts the sweeps of the reference Work() loop: one call per sweep lands on
 * the last workBR cell.  Behaviour is otherwise the reference operator's. */
class CountingPitRemove : public PitRemoveOperator {
public:
    int sweeps = 0;
    bool Operator(const CellCoord& c, bool f) override {
        bool r = PitRemoveOperator::Operator(c, f);
        if (c.iRow() == _xSize - 2 && c.iCol() == _ySize - 2) sweeps++;
        return r;
    }
};

/* Reference SCA rule iterated until every in-degree is consumed. */
class ConvergedSCA : public SCAOperator {
public:
    int sweeps = 0;
    bool Operator(const CellCoord& c, bool f) override {
        bool r = SCAOperator::Operator(c, f);
        if (c.iRow() == _maxRow && c.iCol() == _maxCol) {
            sweeps++;
            if (num == 2 && Termination == 1) {
                const CoordBR& br = _pD8Layer->_pMetaData->_localworkBR;
                CellSpace<double>& deg = *(_degreeLayer.cellSpace());
                bool left = false;
                for (int i = br.minIRow(); i <= br.maxIRow() && !left; ++i)
                    for (int j = br.minICol(); j <= br.maxICol(); ++j)
                        if (deg[i][j] > 0) { left = true; break; }
                if (left) Termination = 0;
            }
        }
        return r;
    }
};

}  // namespace

extern "C" {

/* Slope by the reference SlopeOperator; method = SlopeAlgor (0=FD Horn .. 6=TFDW).
 * threads > 0 selects MPI_OpenMP_Type with that many OpenMP threads. */
int ref_slope(const char* nbr, const float* dem, int rows, int cols, double nodata, double cellsize,
              int method, int threads, double* out) {
    start(threads > 0 ? MPI_OpenMP_Type : MPI_Type);
    if (threads > 0) omp_set_num_threads(threads);
    pargo_shim_register("ref://dem", dem, GDT_Float32, rows, cols, nodata, cellsize);
    RasterLayer<double> demLayer("demLayer");
    demLayer.readNeighborhood(nbr);
    if (!demLayer.readFile("ref://dem", ROWWISE_DCMP)) return 1;
    RasterLayer<double> slopeLayer("slopeLayer");
    slopeLayer.copyLayerInfo(demLayer);
    SlopeOperator op;
    op.demLayer(demLayer);
    op.slopeLayer(slopeLayer);
    op.calcAlgorithm(static_cast<SlopeAlgor>(method));
    if (!op.Run()) return 2;
    copy_out(slopeLayer, out, rows, cols);
    return 0;
}

/* D8 by the reference D8Operator on a float32 DEM (dem_is_f64 = 0) or on a
 * float64 surface such as the reference pit-remove output (dem_is_f64 = 1). */
int ref_d8(const char* nbr, const void* dem, int dem_is_f64, int rows, int cols, double nodata,
           double cellsize, int dir_type, int threads, double* out) {
    start(threads > 0 ? MPI_OpenMP_Type : MPI_Type);
    if (threads > 0) omp_set_num_threads(threads);
    pargo_shim_register("ref://d8dem", dem, dem_is_f64 ? GDT_Float64 : GDT_Float32, rows, cols, nodata, cellsize);
    RasterLayer<double> demLayer("demLayer");
    demLayer.readNeighborhood(nbr);
    if (!demLayer.readFile("ref://d8dem", ROWWISE_DCMP)) return 1;
    RasterLayer<double> d8Layer("d8Layer");
    d8Layer.copyLayerInfo(demLayer);
    D8Operator op(dir_type);
    op.demLayer(demLayer);
    op.d8Layer(d8Layer);
    if (!op.Run()) return 2;
    copy_out(d8Layer, out, rows, cols);
    return 0;
}

/* Pit removal by the reference PitRemoveOperator (serial Gauss-Seidel sweeps). */
int ref_fill(const char* nbr, const float* dem, int rows, int cols, double nodata, double cellsize,
             double* out, int* sweeps) {
    start(MPI_Type);
    pargo_shim_register("ref://filldem", dem, GDT_Float32, rows, cols, nodata, cellsize);
    RasterLayer<double> demLayer("demLayer");
    demLayer.readNeighborhood(nbr);
    if (!demLayer.readFile("ref://filldem", ROWWISE_DCMP)) return 1;
    RasterLayer<double> wdemLayer("wdemLayer");
    wdemLayer.readNeighborhood(nbr);
    wdemLayer.copyLayerInfo(demLayer);
    CountingPitRemove op;
    op.demLayer(demLayer);
    op.wdemLayer(wdemLayer);
    if (!op.Run()) return 2;
    copy_out(wdemLayer, out, rows, cols);
    if (sweeps) *sweeps = op.sweeps;
    return 0;
}

/* SCA by the reference SCAOperator: converged = 0 is the shipped operator
 * (one accumulation sweep), converged = 1 iterates the same rule to the end. */
int ref_sca(const char* nbr, const double* d8, int rows, int cols, double nodata, double cellsize,
            int converged, double* out, int* sweeps) {
    start(MPI_Type);
    pargo_shim_register("ref://d8", d8, GDT_Float64, rows, cols, nodata, cellsize);
    RasterLayer<double> d8Layer("d8Layer");
    d8Layer.readNeighborhood(nbr);
    if (!d8Layer.readFile("ref://d8", ROWWISE_DCMP)) return 1;
    RasterLayer<double> scaLayer("scaLayer");
    scaLayer.copyLayerInfo(d8Layer);
    if (converged) {
        ConvergedSCA op;
        op.d8Layer(d8Layer);
        op.scaLayer(scaLayer);
        if (!op.Run()) return 2;
        if (sweeps) *sweeps = op.sweeps;
    } else {
        SCAOperator op;
        op.d8Layer(d8Layer);
        op.scaLayer(scaLayer);
        if (!op.Run()) return 2;
        if (sweeps) *sweeps = 3;
    }
    copy_out(scaLayer, out, rows, cols);
    return 0;
}

/* TWI by the reference TWIOperator from a slope and an SCA raster (both
 * double, one nodata value), as pTWI.cpp:57-81 runs it. */
int ref_twi(const char* nbr, const double* slope, const double* sca, int rows, int cols, double nodata,
            double cellsize, double* out) {
    start(MPI_Type);
    pargo_shim_register("ref://slope", slope, GDT_Float64, rows, cols, nodata, cellsize);
    pargo_shim_register("ref://sca", sca, GDT_Float64, rows, cols, nodata, cellsize);
    RasterLayer<double> slopeLayer("slopeLayer");
    slopeLayer.readNeighborhood(nbr);
    if (!slopeLayer.readFile("ref://slope", ROWWISE_DCMP)) return 1;
    RasterLayer<double> scaLayer("scaLayer");
    scaLayer.readNeighborhood(nbr);
    if (!scaLayer.readFile("ref://sca", ROWWISE_DCMP)) return 1;
    RasterLayer<double> twiLayer("twiLayer");
    twiLayer.copyLayerInfo(slopeLayer);
    TWIOperator op;
    op.SCALayer(scaLayer);
    op.slopeLayer(slopeLayer);
    op.twiLayer(twiLayer);
    if (!op.Run()) return 2;
    copy_out(twiLayer, out, rows, cols);
    return 0;
}

/* Load estimation and row decomposition by the reference gpro classes, as
 * apps/spatial/reclassify/pRelclassify.cpp:164-178 drives them (intensity-ratio
 * mode): ComputeLayer::init(dataLayer, compute nbr, grain), Transformation(
 * nodataLoad, validLoad).run(), then DeComposition::valRowDcmp on the compute
 * layer and ComputeLayer::getCompuLoad(ROWWISE_DCMP) for rank 0's data rows.
 * `load` receives the compute layer (crows x ccols); comp_rows the compute
 * row range [begin, end] of every part; rank0 the data bounding rectangle
 * {minRow, minCol, maxRow, maxCol} getCompuLoad returns to rank 0. */
int ref_compute_load(const char* nbr, const float* data, int rows, int cols, double nodata, double cellsize,
                     int grain, double nodata_load, double valid_load, int compute_nbr, int nparts, double* load,
                     int* crows, int* ccols, int* comp_rows, int* rank0) {
    start(MPI_Type);
    pargo_shim_register("ref://load_data", data, GDT_Float32, rows, cols, nodata, cellsize);
    RasterLayer<double> dataLayer("dataLayer");
    dataLayer.readNeighborhood(nbr);
    if (!dataLayer.readFile("ref://load_data", ROWWISE_DCMP)) return 1;
    ComputeLayer<double> comptLayer("computLayer");
    if (!comptLayer.init(&dataLayer, compute_nbr ? nbr : nullptr, grain)) return 2;
    Transformation<double> trans(nodata_load, valid_load, &comptLayer);
    if (!trans.run()) return 3;
    const SpaceDims& cd = comptLayer._pMetaData->_glbDims;
    *crows = cd.nRows();
    *ccols = cd.nCols();
    memcpy(load, comptLayer.cellSpace()->_matrix, sizeof(double) * (size_t)cd.nRows() * cd.nCols());
    if (nparts < 1) return 0;
    DeComposition<double> deComp(cd, *(comptLayer.nbrhood()));
    vector<CoordBR> parts;
    if (!deComp.valRowDcmp(parts, comptLayer, nparts)) return 4;
    if ((int)parts.size() != nparts) return 5;
    for (int i = 0; i < nparts; i++) {
        comp_rows[2 * i] = parts[i].minIRow();
        comp_rows[2 * i + 1] = parts[i].maxIRow();
    }
    CoordBR sub;
    if (!comptLayer.getCompuLoad(ROWWISE_DCMP, nparts, sub)) return 6;
    rank0[0] = sub.minIRow();
    rank0[1] = sub.minICol();
    rank0[2] = sub.maxIRow();
    rank0[3] = sub.maxICol();
    return 0;
}

}  // extern "C"
