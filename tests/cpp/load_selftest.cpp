// The gpro load estimator as the reference's mains drive it
// (apps/spatial/reclassify/pRelclassify.cpp:164-178): a compute layer over a
// DEM, the intensity-ratio Transformation on the GPU, getCompuLoad for rank
// 0, every part's rows; then an estimate-function subclass (as
// apps/spatial/idw/idwTransformation.cpp) filling the layer on the host.
//   load_selftest dem.tif moore.nbr grain nparts
#include <cstdio>
#include <cstdlib>

#include "application.h"
#include "computeLayer.h"
#include "rasterLayer.h"
#include "transformation.h"

using namespace GPRO;

class ModEstimate : public Transformation<double> {
public:
    explicit ModEstimate(ComputeLayer<double>* l) : Transformation<double>(l) {}
    bool Operator(const CellCoord& c) override {
        CellSpace<double>& m = *_pComptLayer->cellSpace();
        m[c.iRow()][c.iCol()] = (double)(((long long)c.iRow() * m.nCols() + c.iCol()) % 7);
        return true;
    }
};

static void print_parts(const char* name, const vector<CoordBR>& parts) {
    printf("%s", name);
    for (const CoordBR& b : parts) printf(" %d %d %d %d", b.minIRow(), b.minICol(), b.maxIRow(), b.maxICol());
    printf("\n");
}

int main(int argc, char** argv) {
    if (argc != 5) return 2;
    const int grain = atoi(argv[3]), nparts = atoi(argv[4]);
    if (!Application::START(CUDA_Type, argc, argv)) return 1;
    RasterLayer<double> dem("dem");
    if (!dem.readNeighborhood(argv[2]) || !dem.readFile(argv[1])) return 1;
    ComputeLayer<double> comptLayer("computLayer");
    if (!comptLayer.init(&dem, nullptr, grain)) return 1;
    Transformation<double> trans(0.0, 1.0, &comptLayer);
    if (!trans.run()) return 1;
    double sum = 0.0;
    const CellSpace<double>& m = *comptLayer.cellSpace();
    for (int r = 0; r < m.nRows(); r++)
        for (int c = 0; c < m.nCols(); c++) sum += m[r][c];
    printf("sum %.17g\n", sum);
    CoordBR sub;
    if (!comptLayer.getCompuLoad(ROWWISE_DCMP, nparts, sub)) return 1;
    printf("rank0 %d %d %d %d\n", sub.minIRow(), sub.minICol(), sub.maxIRow(), sub.maxICol());
    vector<CoordBR> parts;
    if (!comptLayer.decompose(nparts, parts)) return 1;
    print_parts("parts", parts);
    ModEstimate est(&comptLayer);
    if (!est.run()) return 1;
    if (!comptLayer.decompose(nparts, parts)) return 1;
    print_parts("estimate_parts", parts);
    Application::END();
    return 0;
}
