// pargo_slope -- slope of a DEM on the GPU, with the command line of the
// reference's slope application (apps/morphology/slope/pSlope.cpp):
//   pargo_slope -elev dem.tif -nbr moore.nbr -slp slope.tif [-mtd FD|FFD|MD|SD|SFD|TFD|TFDW]
//   pargo_slope dem.tif moore.nbr slope.tif [method]
#include "args.h"
#include "application.h"
#include "mpi.h"
#include "rasterLayer.h"
#include "slopeOperator.h"

using namespace GPRO;

int main(int argc, char** argv) {
    AppArgs a;
    std::string err;
    if (!parse_app_args(argc, argv, "-slp", "-mtd", &a, &err)) {
        cerr << "FAILURE: " << err << endl
             << "usage: pargo_slope -elev <dem> -nbr <nbr> -slp <out> [-mtd <method>]" << endl;
        return 1;
    }
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    RasterLayer<double> demLayer("demLayer");
    if (!demLayer.readNeighborhood(a.nbr) || !demLayer.readFile(a.elev, ROWWISE_DCMP)) return 1;
    RasterLayer<double> slopeLayer("slopeLayer");
    slopeLayer.copyLayerInfo(demLayer);
    const double t0 = MPI_Wtime();
    SlopeOperator op;
    op.demLayer(demLayer);
    op.slopeLayer(slopeLayer);
    op.calcAlgorithm(a.extra ? GetSlopeAlgorithm(a.extra) : FD);
    if (!op.Run()) return 1;
    cout << "run time is " << MPI_Wtime() - t0 << endl;
    if (!slopeLayer.writeFile(a.out)) return 1;
    Application::END();
    return 0;
}
