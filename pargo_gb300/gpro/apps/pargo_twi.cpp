// pargo_twi -- topographic wetness index on the GPU, with the command line of
// the reference's twi application (apps/hydrology/twi/pTWI.cpp):
//   pargo_twi slope.tif sca.tif moore.nbr twi.tif
//   pargo_twi -slp slope.tif -sca sca.tif -nbr moore.nbr -out twi.tif
#include <cstring>

#include "application.h"
#include "mpi.h"
#include "rasterLayer.h"
#include "TWIOperator.h"

using namespace GPRO;

int main(int argc, char** argv) {
    const char *slope = nullptr, *sca = nullptr, *nbr = nullptr, *out = nullptr;
    if (argc == 5 && argv[1][0] != '-') {
        slope = argv[1];
        sca = argv[2];
        nbr = argv[3];
        out = argv[4];
    } else {
        for (int i = 1; i + 1 < argc; i += 2) {
            if (!strcmp(argv[i], "-slp")) slope = argv[i + 1];
            else if (!strcmp(argv[i], "-sca")) sca = argv[i + 1];
            else if (!strcmp(argv[i], "-nbr")) nbr = argv[i + 1];
            else if (!strcmp(argv[i], "-out")) out = argv[i + 1];
        }
    }
    if (!slope || !sca || !nbr || !out) {
        cerr << "usage: pargo_twi <slope> <sca> <nbr> <out>" << endl;
        return 1;
    }
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    RasterLayer<double> slopeLayer("slopeLayer");
    if (!slopeLayer.readNeighborhood(nbr) || !slopeLayer.readFile(slope)) return 1;
    RasterLayer<double> scaLayer("scaLayer");
    if (!scaLayer.readNeighborhood(nbr) || !scaLayer.readFile(sca)) return 1;
    RasterLayer<double> twiLayer("twiLayer");
    twiLayer.copyLayerInfo(slopeLayer);
    const double t0 = MPI_Wtime();
    TWIOperator op;
    op.SCALayer(scaLayer);
    op.slopeLayer(slopeLayer);
    op.twiLayer(twiLayer);
    if (!op.Run()) return 1;
    cout << "run time is " << MPI_Wtime() - t0 << endl;
    if (!twiLayer.writeFile(out)) return 1;
    Application::END();
    return 0;
}
