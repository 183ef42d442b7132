// pargo_sca -- D8 specific catchment area on the GPU, with the command line
// of the reference's scad8 application (apps/hydrology/scad8/pSCA.cpp):
//   pargo_sca d8.tif moore.nbr sca.tif [shipped|converged]
// The default reproduces the reference operator (one accumulation sweep);
// "converged" (or PARGO_SCA_CONTRACT=converged) gives the full upslope count.
#include "args.h"
#include "application.h"
#include "mpi.h"
#include "rasterLayer.h"
#include "scaOperator.h"
#include "utility.h"

using namespace GPRO;

int main(int argc, char** argv) {
    AppArgs a;
    std::string err;
    if (!parse_app_args(argc, argv, "-out", "-contract", &a, &err)) {
        cerr << "FAILURE: " << err << endl << "usage: pargo_sca <d8> <nbr> <out> [shipped|converged]" << endl;
        return 1;
    }
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    RasterLayer<double> d8Layer("d8Layer");
    if (!d8Layer.readNeighborhood(a.nbr) || !d8Layer.readFile(a.elev)) return 1;
    RasterLayer<double> scaLayer("scaLayer");
    scaLayer.copyLayerInfo(d8Layer);
    const double t0 = MPI_Wtime();
    SCAOperator op;
    op.d8Layer(d8Layer);
    op.scaLayer(scaLayer);
    if (a.extra) op.contract(StringMatch(a.extra, "converged") ? PARGO_SCA_CONVERGED : PARGO_SCA_SHIPPED);
    if (!op.Run()) return 1;
    cout << "run time is " << MPI_Wtime() - t0 << endl;
    if (!scaLayer.writeFile(a.out)) return 1;
    Application::END();
    return 0;
}
