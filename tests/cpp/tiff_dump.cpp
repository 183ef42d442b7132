// Reads a GeoTIFF with the gpro codec (pargo_gb300/gpro/src/geotiff.cpp) and
// dumps what it read, for tests/test_tiff_read_cpu.py:
//   int64 rows, int64 cols, int64 dtype, int64 has_nodata, double nodata,
//   double transform[6], then rows * cols doubles (row-major).
// Usage: tiff_dump <in.tif> <out.bin>.  Exit 1 with the error on stdout when
// the reader refuses the file.
// tiff_dump --write <out.tif> <rows> <cols> <dtype> <bigtiff>: writes the
// raster v(i, j) = i * cols + j - 7.25 (nodata -9999, cell size 30) with
// write_geotiff, BigTIFF when <bigtiff> is 1.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "gpro/gpro.h"

int main(int argc, char** argv) {
    if (argc >= 7 && std::strcmp(argv[1], "--write") == 0) {
        GPRO::GeoRaster g;
        g.rows = std::atoi(argv[3]);
        g.cols = std::atoi(argv[4]);
        g.nodata = -9999.0;
        g.has_nodata = true;
        const double t[6] = {500.0, 30.0, 0.0, 9000.0, 0.0, -30.0};
        std::memcpy(g.transform, t, sizeof(t));
        g.geoascii = "WGS 84|";
        std::vector<double> v((size_t)g.rows * g.cols);
        for (size_t k = 0; k < v.size(); k++) v[k] = (double)k - 7.25;
        std::string err;
        if (!GPRO::write_geotiff(argv[2], g, v.data(), std::atoi(argv[5]), &err, std::atoi(argv[6]) != 0)) {
            std::printf("%s\n", err.c_str());
            return 1;
        }
        return 0;
    }
    if (argc < 3) return 2;
    GPRO::GeoRaster g;
    std::string err;
    if (!GPRO::read_geotiff(argv[1], &g, &err)) {
        std::printf("%s\n", err.c_str());
        return 1;
    }
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    const long long head[4] = {g.rows, g.cols, g.dtype, g.has_nodata ? 1 : 0};
    std::fwrite(head, sizeof(head), 1, f);
    std::fwrite(&g.nodata, sizeof(double), 1, f);
    std::fwrite(g.transform, sizeof(double), 6, f);
    std::fwrite(g.values.data(), sizeof(double), g.values.size(), f);
    std::fclose(f);
    return 0;
}
