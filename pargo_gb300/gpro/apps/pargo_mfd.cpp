// pargo_mfd -- MFD-md flow partition weights on the GPU, with the command line
// of the reference's flowdirmfdmd application (apps/hydrology/flowdirmfdmd/pMFDmd.cpp):
//   pargo_mfd dem.tif moore.nbr out [exp]
//   pargo_mfd -elev dem.tif -nbr moore.nbr -out out [-exp e]
// writes out + "weightLayer{0,1,2,3,5,6,7,8}.tif", one file per window position
// (pMFDmd.cpp:128-137).  The exponent defaults to -1 as in pMFDmd.cpp:57; after
// -exp the value that follows is read (pMFDmd.cpp:96 reads argv[4] instead).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "application.h"
#include "args.h"
#include "mfdOperator.h"
#include "mpi.h"
#include "rasterLayer.h"

using namespace GPRO;

int main(int argc, char** argv) {
    AppArgs a;
    std::string err;
    if (!parse_app_args(argc, argv, "-out", "-exp", &a, &err)) {
        cerr << "pargo_mfd: " << err << endl
             << "usage: pargo_mfd -elev <dem> -nbr <nbr> -out <prefix> [-exp <slope exponent>]" << endl;
        return 1;
    }
    double slp_exp = -1.0;
    if (a.extra) {
        char* end = nullptr;
        slp_exp = strtod(a.extra, &end);
        if (end == a.extra || *end) {
            cerr << "pargo_mfd: bad slope exponent " << a.extra << endl;
            return 1;
        }
    }
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    RasterLayer<double> demLayer("demLayer");
    if (!demLayer.readNeighborhood(a.nbr) || !demLayer.readFile(a.elev)) return 1;
    std::vector<RasterLayer<double>*> layers;
    std::vector<std::string> names;
    for (int i = 0; i < 8; i++) {
        char tmp[32];
        snprintf(tmp, sizeof tmp, "weightLayer%d.tif", i < 4 ? i : i + 1);
        names.push_back(std::string(a.out) + tmp);
        layers.push_back(new RasterLayer<double>(names.back()));
        layers.back()->copyLayerInfo(demLayer);
    }
    const double t0 = MPI_Wtime();
    MFDOperator op(slp_exp);
    op.demLayer(demLayer);
    op.weightLayers(layers);
    if (!op.Run()) return 1;
    cout << "run time is " << MPI_Wtime() - t0 << endl;
    for (int i = 0; i < 8; i++)
        if (!layers[i]->writeFile(names[i].c_str())) return 1;
    for (RasterLayer<double>* l : layers) delete l;
    Application::END();
    return 0;
}
