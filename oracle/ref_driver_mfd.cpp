/* ref_driver_mfd.cpp -- C entry points that run the reference's MFD-md
 * operators, compiled from their sources where they lie (see build.py), in a
 * library of their own: the scamfdmd operator is also named SCAOperator, like
 * the D8 one in ref_driver.cpp.
 *
 * ref_mfd follows apps/hydrology/flowdirmfdmd/pMFDmd.cpp:119-152 (weight
 * layers as copies of the DEM layer, MFDOperator(slpExp)); ref_sca_mfd follows
 * apps/hydrology/scamfdmd/pSCA.cpp:44-75 (8 weight layers in, SCA layer as a
 * copy of weight layer 0).  Serial MPI_Type, ROWWISE_DCMP. */
#include <cstring>
#include <string>
#include <vector>
#include "mpi.h"
#include "gdal_priv.h"
#include "application.h"
#include "rasterLayer.h"

#include "mfdOperator.h"
#undef Eps
#include "scaOperator.h"
#undef Eps

using namespace GPRO;

namespace {

void start_serial() {
    static char prog[] = "pargo_ref_mfd";
    static char* argv_storage[] = {prog, nullptr};
    char** argv = argv_storage;
    Application::START(MPI_Type, 1, argv);
}

}  // namespace

extern "C" {

/* 8 weight layers (layer-major, rows*cols each) from a float32 DEM. */
int ref_mfd(const char* nbr, const float* dem, int rows, int cols, double nodata, double cellsize, double slp_exp,
            double* out) {
    start_serial();
    pargo_shim_register("ref://mfd_dem", dem, GDT_Float32, rows, cols, nodata, cellsize);
    RasterLayer<double> demLayer("demLayer");
    demLayer.readNeighborhood(nbr);
    if (!demLayer.readFile("ref://mfd_dem", ROWWISE_DCMP)) return 1;
    std::vector<RasterLayer<double>*> wl;
    for (int i = 0; i < 8; i++) {
        wl.push_back(new RasterLayer<double>("weightLayer"));
        wl[i]->copyLayerInfo(demLayer);
    }
    MFDOperator op(slp_exp);
    op.demLayer(demLayer);
    op.weightLayers(wl);
    const bool ok = op.Run();
    const size_t n = (size_t)rows * cols;
    for (int i = 0; i < 8; i++) {
        if (ok) memcpy(out + i * n, wl[i]->cellSpace()->_matrix, n * sizeof(double));
        delete wl[i];
    }
    return ok ? 0 : 2;
}

/* MFD SCA from 8 double weight layers (layer-major). */
int ref_sca_mfd(const char* nbr, const double* w, int rows, int cols, double nodata, double cellsize, double* out) {
    start_serial();
    const size_t n = (size_t)rows * cols;
    std::vector<RasterLayer<double>*> wl;
    std::vector<std::string> names;
    for (int i = 0; i < 8; i++) names.push_back("ref://mfd_w" + std::to_string(i));
    for (int i = 0; i < 8; i++) {
        pargo_shim_register(names[i].c_str(), w + i * n, GDT_Float64, rows, cols, nodata, cellsize);
        wl.push_back(new RasterLayer<double>("unnamed"));
        wl[i]->readNeighborhood(nbr);
        if (!wl[i]->readFile(names[i].c_str(), ROWWISE_DCMP)) return 1;
    }
    RasterLayer<double> scaLayer("scaLayer");
    scaLayer.copyLayerInfo(*wl[0]);
    SCAOperator op;
    op.mfdLayer(wl);
    op.scaLayer(scaLayer);
    const bool ok = op.Run();
    if (ok) memcpy(out, scaLayer.cellSpace()->_matrix, n * sizeof(double));
    for (int i = 0; i < 8; i++) delete wl[i];
    return ok ? 0 : 2;
}

}  // extern "C"
