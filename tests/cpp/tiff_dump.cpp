// Reads a GeoTIFF with the gpro codec (pargo_gb300/gpro/src/geotiff.cpp) and
// dumps what it read, for tests/test_tiff_read_cpu.py:
//   int64 rows, int64 cols, int64 dtype, int64 has_nodata, double nodata,
//   double transform[6], then rows * cols doubles (row-major).
// Usage: tiff_dump <in.tif> <out.bin>.  Exit 1 with the error on stdout when
// the reader refuses the file.
#include <cstdio>
#include <string>

#include "gpro/gpro.h"

int main(int argc, char** argv) {
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
