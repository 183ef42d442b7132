// Host-only self test of the gpro-compatible layer: GeoTIFF round trip,
// neighbourhood parsing and work rectangle, copyLayerInfo semantics.
// Prints "ok" and exits 0, or names the failed check and exits 1.
#include <cstdio>
#include <fstream>

#include "gpro/gpro.h"
#include "gpro/operators.h"
#include "utility.h"

using namespace GPRO;

#define CHECK(c)                                          \
    do {                                                  \
        if (!(c)) {                                       \
            fprintf(stderr, "FAILED: %s (line %d)\n", #c, __LINE__); \
            return 1;                                     \
        }                                                 \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    // GeoTIFF round trip, float64 and float32
    GeoRaster g;
    g.rows = 7;
    g.cols = 11;
    g.nodata = -9999.0;
    g.has_nodata = true;
    const double t[6] = {100.0, 30.0, 0.0, 500.0, 0.0, -30.0};
    memcpy(g.transform, t, sizeof(t));
    std::vector<double> v(77);
    for (int i = 0; i < 77; i++) v[i] = 0.1 * i - 3.0;
    v[5] = -9999.0;
    std::string err;
    CHECK(write_geotiff((dir + "/a64.tif").c_str(), g, v.data(), PARGO_F64, &err));
    GeoRaster r;
    CHECK(read_geotiff((dir + "/a64.tif").c_str(), &r, &err));
    CHECK(r.rows == 7 && r.cols == 11 && r.dtype == PARGO_F64 && r.has_nodata && r.nodata == -9999.0);
    for (int i = 0; i < 77; i++) CHECK(r.values[i] == v[i]);
    for (int k = 0; k < 6; k++) CHECK(r.transform[k] == t[k]);
    CHECK(write_geotiff((dir + "/a32.tif").c_str(), g, v.data(), PARGO_F32, &err));
    CHECK(read_geotiff((dir + "/a32.tif").c_str(), &r, &err));
    for (int i = 0; i < 77; i++) CHECK(r.values[i] == (double)(float)v[i]);
    // neighbourhood files like the reference's neighbor/*.nbr
    {
        std::ofstream f(dir + "/moore.nbr");
        f << "9\n0 0 1.0\n-1 -1 1.0\n-1 0 1.0\n-1 1 1.0\n0 -1 1.0\n0 1 1.0\n1 -1 1.0\n1 0 1.0\n1 1 1.0\n";
    }
    RasterLayer<double> dem("demLayer");
    CHECK(dem.readNeighborhood((dir + "/moore.nbr").c_str()));
    CHECK(dem.nbrhood()->size() == 9 && dem.nbrhood()->minIRow() == -1 && dem.nbrhood()->maxICol() == 1);
    CHECK(dem.readFile((dir + "/a64.tif").c_str(), ROWWISE_DCMP));
    MetaData& m = *dem.metaData();
    CHECK(m.cellSize == 30.0f && m.noData == -9999.0);
    CHECK(m._localworkBR.minIRow() == 1 && m._localworkBR.maxIRow() == 5 && m._localworkBR.maxICol() == 9);
    CHECK((*dem.cellSpace())[2][3] == v[2 * 11 + 3]);
    RasterLayer<double> out("out");
    CHECK(out.copyLayerInfo(dem));
    CHECK((*out.cellSpace())[3][3] == -9999.0);  // copyLayerInfo fills with nodata (rasterLayer.h:739-745)
    CHECK(out.writeFile((dir + "/out.tif").c_str()));
    // a neighbourhood without (0,0) is rejected, as in neighborhood.h:118-123
    {
        std::ofstream f(dir + "/bad.nbr");
        f << "2\n1 0 1\n0 1 1\n";
    }
    RasterLayer<double> bad("bad");
    CHECK(!bad.readNeighborhood((dir + "/bad.nbr").c_str()));
    CHECK(GetSlopeAlgorithm("tfdw") == TFDW && GetSlopeAlgorithm("xx") == FD);
    CHECK(StringMatch("Converged", "converged"));
    printf("ok\n");
    return 0;
}
