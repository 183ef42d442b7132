/*
 * In-memory stand-in for <gdal_priv.h>, used ONLY to compile the unmodified
 * PaRGO reference sources into the test oracle under oracle/_ref/.  It is
 * test infrastructure: nothing in the product links it.
 *
 * GDALOpen(name) looks the name up in a process-wide registry of in-memory
 * single-band rasters that the oracle driver fills before calling the
 * reference (pargo_shim_register) and reads back afterwards.  RasterIO
 * converts between the stored band type and the caller's buffer type the
 * way GDAL does for the types the reference uses (float32 -> float64
 * widening is exact).  Driver::Create makes a new registry entry, so the
 * reference's writeFile() path also works.
 */
#ifndef PARGO_ORACLE_GDAL_SHIM_H
#define PARGO_ORACLE_GDAL_SHIM_H

#include <map>
#include <string>
#include <vector>
#include <cstring>
#include <cstdint>
#include <cstdlib>

#ifndef FALSE
#define FALSE 0
#endif
#ifndef TRUE
#define TRUE 1
#endif

typedef enum {
    GDT_Unknown = 0, GDT_Byte = 1, GDT_UInt16 = 2, GDT_Int16 = 3, GDT_UInt32 = 4,
    GDT_Int32 = 5, GDT_Float32 = 6, GDT_Float64 = 7
} GDALDataType;
typedef enum { GA_ReadOnly = 0, GA_Update = 1 } GDALAccess;
typedef enum { GF_Read = 0, GF_Write = 1 } GDALRWFlag;
typedef int CPLErr;
#define CE_None 0
#define CE_Failure 3
#define GDAL_DCAP_CREATE "DCAP_CREATE"
#define GDAL_DCAP_CREATECOPY "DCAP_CREATECOPY"

static inline size_t pargo_shim_gdal_size(GDALDataType t) {
    switch (t) {
        case GDT_Byte: return 1;
        case GDT_UInt16: case GDT_Int16: return 2;
        case GDT_UInt32: case GDT_Int32: case GDT_Float32: return 4;
        case GDT_Float64: return 8;
        default: return 0;
    }
}
static inline double pargo_shim_gdal_get(const void* p, GDALDataType t, size_t i) {
    switch (t) {
        case GDT_Byte: return ((const uint8_t*)p)[i];
        case GDT_UInt16: return ((const uint16_t*)p)[i];
        case GDT_Int16: return ((const int16_t*)p)[i];
        case GDT_UInt32: return ((const uint32_t*)p)[i];
        case GDT_Int32: return ((const int32_t*)p)[i];
        case GDT_Float32: return ((const float*)p)[i];
        case GDT_Float64: return ((const double*)p)[i];
        default: return 0.0;
    }
}
static inline void pargo_shim_gdal_put(void* p, GDALDataType t, size_t i, double v) {
    switch (t) {
        case GDT_Byte: ((uint8_t*)p)[i] = (uint8_t)v; break;
        case GDT_UInt16: ((uint16_t*)p)[i] = (uint16_t)v; break;
        case GDT_Int16: ((int16_t*)p)[i] = (int16_t)v; break;
        case GDT_UInt32: ((uint32_t*)p)[i] = (uint32_t)v; break;
        case GDT_Int32: ((int32_t*)p)[i] = (int32_t)v; break;
        case GDT_Float32: ((float*)p)[i] = (float)v; break;
        case GDT_Float64: ((double*)p)[i] = v; break;
        default: break;
    }
}

/* One in-memory raster: a single band stored row-major in its own type. */
struct PargoShimRaster {
    int rows = 0, cols = 0;
    GDALDataType type = GDT_Float32;
    double nodata = -9999.0;
    double transform[6] = {0, 1, 0, 0, 0, -1};
    std::string projection;
    std::vector<unsigned char> bytes;
};

inline std::map<std::string, PargoShimRaster>& pargo_shim_registry() {
    static std::map<std::string, PargoShimRaster> reg;
    return reg;
}

class GDALRasterBand {
public:
    explicit GDALRasterBand(PargoShimRaster* r) : _r(r) {}
    double GetNoDataValue(int* ok = nullptr) { if (ok) *ok = 1; return _r->nodata; }
    CPLErr SetNoDataValue(double v) { _r->nodata = v; return CE_None; }
    int GetXSize() { return _r->cols; }
    int GetYSize() { return _r->rows; }
    CPLErr RasterIO(GDALRWFlag flag, int xoff, int yoff, int xsize, int ysize, void* buf,
                    int bufx, int bufy, GDALDataType buftype, int pixspace, int linespace) {
        (void)pixspace; (void)linespace;
        if (xsize != bufx || ysize != bufy || xoff < 0 || yoff < 0 ||
            xoff + xsize > _r->cols || yoff + ysize > _r->rows) return CE_Failure;
        for (int i = 0; i < ysize; i++) {
            for (int j = 0; j < xsize; j++) {
                size_t src = (size_t)(yoff + i) * _r->cols + (xoff + j);
                size_t dst = (size_t)i * bufx + j;
                if (flag == GF_Read)
                    pargo_shim_gdal_put(buf, buftype, dst, pargo_shim_gdal_get(_r->bytes.data(), _r->type, src));
                else
                    pargo_shim_gdal_put(_r->bytes.data(), _r->type, src, pargo_shim_gdal_get(buf, buftype, dst));
            }
        }
        return CE_None;
    }
private:
    PargoShimRaster* _r;
};

class GDALDataset {
public:
    explicit GDALDataset(PargoShimRaster* r) : _r(r), _band(r) {}
    CPLErr GetGeoTransform(double* t) { memcpy(t, _r->transform, sizeof(_r->transform)); return CE_None; }
    CPLErr SetGeoTransform(double* t) { memcpy(_r->transform, t, sizeof(_r->transform)); return CE_None; }
    const char* GetProjectionRef() { return _r->projection.c_str(); }
    CPLErr SetProjection(const char* p) { _r->projection = p ? p : ""; return CE_None; }
    GDALRasterBand* GetRasterBand(int i) { return i == 1 ? &_band : nullptr; }
private:
    PargoShimRaster* _r;
    GDALRasterBand _band;
};
typedef void* GDALDatasetH;

class GDALDriver {
public:
    GDALDataset* Create(const char* name, int cols, int rows, int bands, GDALDataType type, char** opts) {
        (void)opts;
        if (bands != 1) return nullptr;
        PargoShimRaster& r = pargo_shim_registry()[name];
        r.rows = rows; r.cols = cols; r.type = type;
        r.bytes.assign((size_t)rows * cols * pargo_shim_gdal_size(type), 0);
        return new GDALDataset(&r);
    }
};
class GDALDriverManager {
public:
    GDALDriver* GetDriverByName(const char*) { static GDALDriver d; return &d; }
};
inline GDALDriverManager* GetGDALDriverManager() { static GDALDriverManager m; return &m; }
inline void GDALAllRegister() {}
inline GDALDatasetH GDALOpen(const char* name, GDALAccess) {
    auto& reg = pargo_shim_registry();
    auto it = reg.find(name);
    if (it == reg.end()) return nullptr;
    return new GDALDataset(&it->second);
}
inline void GDALClose(GDALDatasetH h) { delete static_cast<GDALDataset*>(h); }
inline char** CSLSetNameValue(char** list, const char*, const char*) { return list; }
inline int CSLFetchBoolean(char**, const char*, int dflt) { return dflt; }

/* gpro/rasterLayer.h:1292-1315 call min(double, int), which only resolves with
 * the min(a,b) macro of the Windows headers the reference was written
 * against; this overload gives the same value (a double, truncated on return
 * to int).  It is here because this header is included before rasterLayer.h. */
inline double min(double a, int b) { return a < b ? a : (double)b; }

/* Register a float32 raster under `name` (oracle driver side). */
inline void pargo_shim_register(const char* name, const void* data, GDALDataType type, int rows, int cols,
                                double nodata, double cellsize) {
    PargoShimRaster& r = pargo_shim_registry()[name];
    r.rows = rows; r.cols = cols; r.type = type; r.nodata = nodata;
    double t[6] = {0.0, cellsize, 0.0, 0.0, 0.0, -cellsize};
    memcpy(r.transform, t, sizeof(t));
    size_t n = (size_t)rows * cols * pargo_shim_gdal_size(type);
    r.bytes.assign((const unsigned char*)data, (const unsigned char*)data + n);
}

#endif
