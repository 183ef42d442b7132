// pargo_sca_mfd -- MFD specific catchment area on the GPU, with the command
// line of the reference's scamfdmd application (apps/hydrology/scamfdmd/pSCA.cpp):
//   pargo_sca_mfd w0.tif,w1.tif,...,w8.tif moore.nbr sca.tif
// (the 8 weight layers comma-separated, in layer order).
#include <string>
#include <vector>

#include "application.h"
#include "mpi.h"
#include "rasterLayer.h"
#include "scaOperator.h"
#include "utility.h"

using namespace GPRO;

int main(int argc, char** argv) {
    if (argc != 4) {
        cerr << "usage: pargo_sca_mfd <w0,w1,...,w7> <nbr> <out>" << endl;
        return 1;
    }
    std::vector<std::string> files = SplitString(argv[1], ',');
    if (files.size() != 8) {
        cerr << "pargo_sca_mfd: 8 comma-separated weight files are required, got " << files.size() << endl;
        return 1;
    }
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    std::vector<RasterLayer<double>*> layers;
    for (int i = 0; i < 8; i++) {
        layers.push_back(new RasterLayer<double>("weightLayer"));
        if (!layers[i]->readNeighborhood(argv[2]) || !layers[i]->readFile(files[i].c_str())) return 1;
    }
    RasterLayer<double> scaLayer("scaLayer");
    scaLayer.copyLayerInfo(*layers[0]);
    const double t0 = MPI_Wtime();
    SCAOperator op;
    op.mfdLayer(layers);
    op.scaLayer(scaLayer);
    if (!op.Run()) return 1;
    cout << "run time is " << MPI_Wtime() - t0 << endl;
    if (!scaLayer.writeFile(argv[3])) return 1;
    for (RasterLayer<double>* l : layers) delete l;
    Application::END();
    return 0;
}
