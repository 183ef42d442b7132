// pargo_d8 -- D8 flow directions on the GPU, with the command line of the
// reference's flowdird8 application (apps/hydrology/flowdird8/pD8.cpp):
//   pargo_d8 -elev dem.tif -nbr moore.nbr -out d8.tif [-dirtype 8|256]
//   pargo_d8 dem.tif moore.nbr d8.tif 8|256
#include "args.h"
#include "application.h"
#include "d8Operator.h"
#include "mpi.h"
#include "rasterLayer.h"

using namespace GPRO;

int main(int argc, char** argv) {
    AppArgs a;
    std::string err;
    if (!parse_app_args(argc, argv, "-out", "-dirtype", &a, &err)) {
        cerr << "FAILURE: " << err << endl << "usage: pargo_d8 -elev <dem> -nbr <nbr> -out <out> [-dirtype 8|256]" << endl;
        return 1;
    }
    const int dirType = a.extra ? atoi(a.extra) : 8;
    if (!(dirType == 8 || dirType == 256)) {  // pD8.cpp:106-109
        cerr << "please input right parameter." << endl;
        return 1;
    }
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    RasterLayer<double> demLayer("demLayer");
    if (!demLayer.readNeighborhood(a.nbr) || !demLayer.readFile(a.elev)) return 1;
    RasterLayer<double> d8Layer("d8Layer");
    d8Layer.copyLayerInfo(demLayer);
    const double t0 = MPI_Wtime();
    D8Operator op(dirType);
    op.demLayer(demLayer);
    op.d8Layer(d8Layer);
    if (!op.Run()) return 1;
    cout << "run time is " << MPI_Wtime() - t0 << endl;
    if (!d8Layer.writeFile(a.out)) return 1;
    Application::END();
    return 0;
}
