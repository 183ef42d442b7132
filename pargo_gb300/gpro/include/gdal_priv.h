// gdal_priv.h -- include name some application mains name (e.g. the twi main)
// without calling GDAL: raster I/O here goes through the layer's own GeoTIFF
// reader and writer (gpro/gpro.h), so nothing is declared.
#ifndef PARGO_GPRO_GDAL_PRIV_H
#define PARGO_GPRO_GDAL_PRIV_H
#endif
