// pargo_pitremove -- pit removal on the GPU, with the command line of the
// reference's pitremove application (apps/hydrology/pitremove/pPitRemove.cpp):
//   pargo_pitremove -elev dem.tif -nbr moore.nbr -out filled.tif
//   pargo_pitremove dem.tif moore.nbr filled.tif
#include "args.h"
#include "application.h"
#include "mpi.h"
#include "pitRemoveOperator.h"
#include "rasterLayer.h"

using namespace GPRO;

int main(int argc, char** argv) {
    AppArgs a;
    std::string err;
    if (!parse_app_args(argc, argv, "-out", nullptr, &a, &err)) {
        cerr << "FAILURE: " << err << endl << "usage: pargo_pitremove -elev <dem> -nbr <nbr> -out <out>" << endl;
        return 1;
    }
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    RasterLayer<double> demLayer("demLayer");
    if (!demLayer.readNeighborhood(a.nbr) || !demLayer.readFile(a.elev, ROWWISE_DCMP)) return 1;
    RasterLayer<double> wdemLayer("wdemLayer");
    wdemLayer.readNeighborhood(a.nbr);
    wdemLayer.copyLayerInfo(demLayer);
    const double t0 = MPI_Wtime();
    PitRemoveOperator op;
    op.demLayer(demLayer);
    op.wdemLayer(wdemLayer);
    if (!op.Run()) return 1;
    cout << "run time is " << MPI_Wtime() - t0 << endl;
    if (!wdemLayer.writeFile(a.out)) return 1;
    Application::END();
    return 0;
}
