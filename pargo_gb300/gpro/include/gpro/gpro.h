// gpro.h -- the gpro programming interface of PaRGO, with the focal operators
// running on the GPU through the C ABI of include/pargo_gpu.h.
//
// Same class and method names as the reference framework (gpro/*.h) so that
// application code written against it -- Application::START, RasterLayer,
// Neighborhood, CellSpace, MetaData and the SlopeOperator / D8Operator /
// PitRemoveOperator / SCAOperator setters followed by Run() -- compiles and
// runs unchanged, on one GPU, in one process, without MPI or GDAL:
//   - Application::START(any ProgramType) opens the GPU context (device from
//     the PARGO_DEVICE environment variable, default 0);
//   - RasterLayer reads and writes GeoTIFF itself (classic or BigTIFF,
//     uncompressed strips or tiles; float/int samples), keeping the
//     georeferencing tags;
//   - a single process owns the whole raster, so every decomposition type
//     reads the full raster and writeFile writes it (the reference's writeFile
//     returns false for NON_DCMP, gpro/rasterLayer.h:1011-1013, which is why its
//     D8 and SCA mains wrote no output);
//   - each operator's Run() is one call of the C ABI on the layers' buffers;
//     an operator without a GPU implementation fails its Run() (no CPU path).
#ifndef PARGO_GPRO_H
#define PARGO_GPRO_H

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "pargo_gpu.h"

// The reference headers open namespace std globally and its application mains
// rely on that (string, cout unqualified); kept for source compatibility.
using namespace std;

namespace GPRO {

enum ProgramType { MPI_Type = 0, MPI_OpenMP_Type, CUDA_Type, Serial_Type };  // gpro/basicTypes.h:88-93
enum DomDcmpType { NON_DCMP = 0, ROWWISE_DCMP, COLWISE_DCMP, BLOCK_DCMP };    // gpro/basicTypes.h:51-56

class CellCoord {
public:
    CellCoord(int r = 0, int c = 0) : _iRow(r), _iCol(c) {}
    int iRow() const { return _iRow; }
    int iCol() const { return _iCol; }
    void iRow(int r) { _iRow = r; }
    void iCol(int c) { _iCol = c; }
    bool operator==(const CellCoord& o) const { return _iRow == o._iRow && _iCol == o._iCol; }
    bool operator!=(const CellCoord& o) const { return !(*this == o); }

private:
    int _iRow, _iCol;
};

class SpaceDims {
public:
    SpaceDims(int r = 0, int c = 0) : _nRows(r), _nCols(c) {}
    int nRows() const { return _nRows; }
    int nCols() const { return _nCols; }
    int64_t size() const { return (int64_t)_nRows * _nCols; }
    bool isNone() const { return _nRows <= 0 || _nCols <= 0; }

private:
    int _nRows, _nCols;
};

class CoordBR {
public:
    CoordBR() {}
    CoordBR(const CellCoord& nw, const CellCoord& se) : _nw(nw), _se(se) {}
    const CellCoord& nwCorner() const { return _nw; }
    const CellCoord& seCorner() const { return _se; }
    void nwCorner(const CellCoord& c) { _nw = c; }
    void seCorner(const CellCoord& c) { _se = c; }
    void nwCorner(int r, int c) { _nw = CellCoord(r, c); }
    void seCorner(int r, int c) { _se = CellCoord(r, c); }
    int minIRow() const { return _nw.iRow(); }
    int minICol() const { return _nw.iCol(); }
    int maxIRow() const { return _se.iRow(); }
    int maxICol() const { return _se.iCol(); }
    int nRows() const { return _se.iRow() - _nw.iRow() + 1; }
    int nCols() const { return _se.iCol() - _nw.iCol() + 1; }
    bool valid(const SpaceDims& d) const {
        return minIRow() >= 0 && minICol() >= 0 && maxIRow() < d.nRows() && maxICol() < d.nCols() &&
               minIRow() <= maxIRow() && minICol() <= maxICol();
    }

private:
    CellCoord _nw, _se;
};

// The MPI rank (gpro/utility.h:227): always 0 in the one-process GPU build.
int GetRank();

// Process-wide GPU context (gpro/application.h).
class Application {
public:
    static bool START(ProgramType programType, int argc, char* argv[]);
    static bool END();
    static pargo_ctx* context();  // opened by START, or lazily on first use
    static ProgramType _programType;
};

// GeoTIFF codec (src/geotiff.cpp).
struct GeoRaster {
    int rows = 0, cols = 0;
    int dtype = PARGO_F64;        // sample type in the file (pargo_dtype)
    double nodata = -9999.0;
    bool has_nodata = false;
    double transform[6] = {0, 1, 0, 0, 0, -1};
    std::vector<unsigned char> geokeys;      // tag 34735 (raw SHORTs)
    std::vector<unsigned char> geodoubles;   // tag 34736
    std::string geoascii;                    // tag 34737
    std::vector<double> values;              // row-major, converted to double
};
bool read_geotiff(const char* path, GeoRaster* out, std::string* err);
// Writes `values` (rows x cols doubles) as samples of `dtype` (F32 or F64):
// classic TIFF while the samples fit in it (below 4 GB), else BigTIFF, or
// BigTIFF always when `force_bigtiff`.
bool write_geotiff(const char* path, const GeoRaster& meta, const double* values, int dtype, std::string* err,
                   bool force_bigtiff = false);

class MetaData {
public:
    MetaData() { pTransform = new double[6]{0, 1, 0, 0, 0, -1}; }
    MetaData(const MetaData& o) : MetaData() { *this = o; }
    MetaData& operator=(const MetaData& o) {
        if (this != &o) {
            format = o.format;
            projection = o.projection;
            std::memcpy(pTransform, o.pTransform, 6 * sizeof(double));
            noData = o.noData;
            cellSize = o.cellSize;
            row = o.row;
            column = o.column;
            myrank = o.myrank;
            processor_number = o.processor_number;
            dataType = o.dataType;
            _domDcmpType = o._domDcmpType;
            _glbDims = o._glbDims;
            _MBR = o._MBR;
            _localdims = o._localdims;
            _localworkBR = o._localworkBR;
            geo = o.geo;
        }
        return *this;
    }
    ~MetaData() { delete[] pTransform; }
    int LoctoGloRow(int i) { return _MBR.minIRow() + i; }
    int LoctoGloCol(int j) { return _MBR.minICol() + j; }

    string format = "GTiff";
    string projection;
    double* pTransform;
    double noData = -9999.0;
    float cellSize = 1.0f;  // a float, as the reference stores it (gpro/metaData.h:56)
    int row = 0, column = 0;
    int myrank = 0, processor_number = 1;
    int dataType = PARGO_F64;
    DomDcmpType _domDcmpType = NON_DCMP;
    SpaceDims _glbDims, _localdims;
    CoordBR _MBR, _localworkBR;
    GeoRaster geo;  // georeferencing tags carried from the input file (values unused)
};

template <class elemType>
class CellSpace {
public:
    CellSpace() {}
    CellSpace(const SpaceDims& d, elemType init) { initMem(d, init); }
    bool initMem(const SpaceDims& d, elemType init) {
        _dims = d;
        _data.assign((size_t)d.size(), init);
        _matrix = _data.empty() ? nullptr : _data.data();
        return true;
    }
    void initVals(elemType v) { std::fill(_data.begin(), _data.end(), v); }
    elemType* operator[](int iRow) { return _matrix + (int64_t)iRow * _dims.nCols(); }
    const elemType* operator[](int iRow) const { return _matrix + (int64_t)iRow * _dims.nCols(); }
    int nRows() const { return _dims.nRows(); }
    int nCols() const { return _dims.nCols(); }
    int64_t size() const { return _dims.size(); }
    bool empty() const { return _data.empty(); }
    const SpaceDims& dims() const { return _dims; }

    elemType* _matrix = nullptr;  // row-major (gpro/cellSpace.h:230)

private:
    SpaceDims _dims;
    std::vector<elemType> _data;
};

// .nbr neighbourhood (gpro/neighborhood.h): offsets, MBR, work rectangle.
template <class elemType>
class Neighborhood {
public:
    int size() const { return (int)_coords.size(); }
    bool empty() const { return _coords.empty(); }
    int minIRow() const { return _nbr.min_row; }
    int minICol() const { return _nbr.min_col; }
    int maxIRow() const { return _nbr.max_row; }
    int maxICol() const { return _nbr.max_col; }
    int nRows() const { return maxIRow() - minIRow() + 1; }
    int nCols() const { return maxICol() - minICol() + 1; }
    const pargo_nbr& abi() const { return _nbr; }

    // Parse the .nbr text; same rules as the reference's operator>> and
    // _initCoords (through pargo_nbr_parse).
    bool parse(const std::string& text) {
        pargo_nbr n;
        if (pargo_nbr_parse(text.c_str(), &n) != PARGO_OK) {
            cerr << "Neighborhood: invalid neighbourhood definition" << endl;
            _coords.clear();
            return false;
        }
        _nbr = n;
        _coords.clear();
        std::istringstream is(text);
        int count = 0;
        is >> count;
        if (count >= 100) {
            const int half = ((int)std::sqrt((double)count)) / 2;
            for (int i = -half; i <= half; i++)
                for (int j = -half; j <= half; j++) _coords.push_back(CellCoord(i, j));
        } else {
            for (int k = 0; k < count; k++) {
                int r, c;
                double w;
                is >> r >> c >> w;
                _coords.push_back(CellCoord(r, c));
            }
        }
        return true;
    }

    // gpro/neighborhood.h:423-467: workBR = dims minus the MBR ring.
    bool calcWorkBR(CoordBR& workBR, const SpaceDims& dims) const {
        if (empty() || dims.isNone() || dims.nRows() < nRows() || dims.nCols() < nCols()) {
            cerr << "Neighborhood::calcWorkBR: raster smaller than the neighbourhood" << endl;
            return false;
        }
        workBR.nwCorner(-minIRow(), -minICol());
        workBR.seCorner(dims.nRows() - maxIRow() - 1, dims.nCols() - maxICol() - 1);
        return workBR.valid(dims);
    }

private:
    std::vector<CellCoord> _coords;
    pargo_nbr _nbr{0, 0, 0, 0, 0};
};

template <class elemType>
istream& operator>>(istream& is, Neighborhood<elemType>& n) {
    std::stringstream ss;
    ss << is.rdbuf();
    n.parse(ss.str());
    return is;
}

template <class elemType>
class RasterLayer {
public:
    explicit RasterLayer(const string& name = "Untitled") : _name(name) {}
    RasterLayer(const RasterLayer&) = delete;
    RasterLayer& operator=(const RasterLayer&) = delete;
    ~RasterLayer() {
        delete _pMetaData;
        delete _pCellSpace;
        delete _pNbrhood;
    }

    CellSpace<elemType>* cellSpace() { return _pCellSpace; }
    const CellSpace<elemType>* cellSpace() const { return _pCellSpace; }
    Neighborhood<elemType>* nbrhood() { return _pNbrhood; }
    const Neighborhood<elemType>* nbrhood() const { return _pNbrhood; }
    MetaData* metaData() { return _pMetaData; }
    const string& name() const { return _name; }

    bool newNbrhood() {
        delete _pNbrhood;
        _pNbrhood = new Neighborhood<elemType>();
        return true;
    }

    // gpro/rasterLayer.h:660-669
    bool readNeighborhood(const char* neighborfile) {
        std::ifstream f(neighborfile);
        if (!f) {
            cerr << "RasterLayer::readNeighborhood: cannot open " << neighborfile << endl;
            return false;
        }
        std::stringstream ss;
        ss << f.rdbuf();
        newNbrhood();
        return _pNbrhood->parse(ss.str());
    }

    // gpro/rasterLayer.h:882-903: metadata, work rectangle, whole-raster read.
    bool readFile(const char* inputfile, DomDcmpType dcmpType = NON_DCMP) {
        GeoRaster g;
        std::string err;
        if (!read_geotiff(inputfile, &g, &err)) {
            cerr << "[ERROR] " << err << endl;
            return false;
        }
        if (!_pNbrhood) {
            cerr << "RasterLayer::readFile: read the neighbourhood first" << endl;
            return false;
        }
        delete _pMetaData;
        _pMetaData = new MetaData();
        MetaData& m = *_pMetaData;
        std::memcpy(m.pTransform, g.transform, 6 * sizeof(double));
        m.noData = g.has_nodata ? g.nodata : -9999.0;
        m.row = g.rows;
        m.column = g.cols;
        m.cellSize = (float)g.transform[1];  // gpro/rasterLayer.h:770
        m.dataType = dtype_of();
        m._domDcmpType = dcmpType;
        m._glbDims = SpaceDims(g.rows, g.cols);
        m._localdims = m._glbDims;
        m._MBR = CoordBR(CellCoord(0, 0), CellCoord(g.rows - 1, g.cols - 1));
        if (!_pNbrhood->calcWorkBR(m._localworkBR, m._glbDims)) return false;
        m.geo = g;
        m.geo.values.clear();
        delete _pCellSpace;
        _pCellSpace = new CellSpace<elemType>(m._localdims, (elemType)0);
        for (int64_t i = 0; i < m._localdims.size(); i++) _pCellSpace->_matrix[i] = (elemType)g.values[i];
        return true;
    }

    // gpro/rasterLayer.h: a neighbourhood of the cell itself (no halo).
    bool newLocalNbrhood() {
        newNbrhood();
        return _pNbrhood->parse("1\n0 0 1.0\n");
    }
    // A new cell space of the metadata's local dims, every cell `init`.
    bool newCellSpace(const SpaceDims& dims, elemType init) {
        delete _pCellSpace;
        _pCellSpace = new CellSpace<elemType>(dims, init);
        return true;
    }

    // gpro/rasterLayer.h:739-745: same metadata and neighbourhood, cells = nodata.
    bool copyLayerInfo(const RasterLayer<elemType>& rhs) {
        if (!rhs._pMetaData) return false;
        delete _pMetaData;
        _pMetaData = new MetaData(*rhs._pMetaData);
        _pMetaData->dataType = dtype_of();
        if (rhs._pNbrhood) {
            newNbrhood();
            *_pNbrhood = *rhs._pNbrhood;
        }
        delete _pCellSpace;
        _pCellSpace = new CellSpace<elemType>(_pMetaData->_localdims, (elemType)rhs._pMetaData->noData);
        return true;
    }

    bool writeFile(const char* outputfile) {
        if (!_pMetaData || !_pCellSpace) return false;
        std::vector<double> v((size_t)_pCellSpace->size());
        for (size_t i = 0; i < v.size(); i++) v[i] = (double)_pCellSpace->_matrix[i];
        GeoRaster g = _pMetaData->geo;
        g.rows = _pMetaData->_glbDims.nRows();
        g.cols = _pMetaData->_glbDims.nCols();
        g.nodata = _pMetaData->noData;
        g.has_nodata = true;
        std::memcpy(g.transform, _pMetaData->pTransform, 6 * sizeof(double));
        std::string err;
        if (!write_geotiff(outputfile, g, v.data(), _pMetaData->dataType == PARGO_F32 ? PARGO_F32 : PARGO_F64,
                           &err)) {
            cerr << "[ERROR] " << err << endl;
            return false;
        }
        return true;
    }

    // The layer as a C-ABI raster over its host buffer.
    pargo_raster abi_raster() {
        pargo_raster r{};
        r.data = _pCellSpace ? _pCellSpace->_matrix : nullptr;
        r.dtype = dtype_of();
        r.location = PARGO_HOST;
        r.rows = _pMetaData ? _pMetaData->_localdims.nRows() : 0;
        r.cols = _pMetaData ? _pMetaData->_localdims.nCols() : 0;
        r.pitch = 0;
        r.nodata = _pMetaData ? _pMetaData->noData : -9999.0;
        r.cellsize = _pMetaData ? (double)_pMetaData->cellSize : 1.0;
        return r;
    }

    MetaData* _pMetaData = nullptr;

private:
    static int dtype_of() { return sizeof(elemType) == 4 ? PARGO_F32 : PARGO_F64; }
    string _name;
    CellSpace<elemType>* _pCellSpace = nullptr;
    Neighborhood<elemType>* _pNbrhood = nullptr;
};

// gpro/rasterOperator.h: the base of every operator.  Run() is virtual here;
// the four focal operators implement it on the GPU.
template <class elemType>
class RasterOperator {
public:
    RasterOperator() : _pWorkBR(nullptr), commFlag(false), Termination(1) {}
    virtual ~RasterOperator() {}
    virtual bool Operator(const CellCoord&, bool operFlag) { return operFlag; }
    virtual bool isTermination() { return false; }
    bool Configure(RasterLayer<elemType>* pLayer, bool isCommunication) {
        _pWorkBR = &pLayer->_pMetaData->_localworkBR;
        if (isCommunication) {
            CommVec.push_back(pLayer);
            commFlag = true;
        }
        return true;
    }
    virtual bool Run() {
        cerr << "RasterOperator::Run: this operator has no GPU implementation" << endl;
        return false;
    }

    vector<RasterLayer<elemType>*> CommVec;
    CoordBR* _pWorkBR;
    bool commFlag;
    int Termination;
};

bool report_status(pargo_status st, const char* what);  // cerr + false on failure, like the reference

}  // namespace GPRO

#endif
