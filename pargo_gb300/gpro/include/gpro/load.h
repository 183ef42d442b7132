// load.h -- the load estimator of PaRGO's load balancing with the reference's
// API (gpro/computeLayer.h, gpro/transformation.h, gpro/deComposition.h):
// ComputeLayer (a coarse raster of compute loads over data layers),
// Transformation (fills it: intensity ratio on the GPU, or an application's
// own estimate function on the host) and the load-weighted row decomposition.
#ifndef PARGO_GPRO_LOAD_H
#define PARGO_GPRO_LOAD_H

#include <typeinfo>

#include "gpro/gpro.h"

namespace GPRO {

template <class elemType>
class ComputeLayer : public RasterLayer<elemType> {
public:
    ComputeLayer() : RasterLayer<elemType>("Untitled") {}
    explicit ComputeLayer(const string& name) : RasterLayer<elemType>(name) {}
    ComputeLayer(RasterLayer<elemType>* dataLayer, int grain, const string& name)
        : RasterLayer<elemType>(name), _comptGrain(grain) {
        _vDataLayers.push_back(dataLayer);
    }
    ComputeLayer(vector<RasterLayer<elemType>*> dataLayers, int grain, const string& name)
        : RasterLayer<elemType>(name), _vDataLayers(dataLayers), _comptGrain(grain) {}

    double getComputeGrain() { return _comptGrain; }
    void setComputGrain(int comptGrain) { _comptGrain = comptGrain; }
    vector<RasterLayer<elemType>*>* dataLayers() { return &_vDataLayers; }
    void addRasterLayer(RasterLayer<elemType>* dataLayer) { _vDataLayers.push_back(dataLayer); }
    void addRasterLayers(vector<RasterLayer<elemType>*> dataLayers) { _vDataLayers = dataLayers; }
    // Whether the compute layer has a neighbourhood file of its own (its ring
    // is then outside its work rectangle and keeps load 0).
    bool hasRing() const { return _ring; }

    // gpro/computeLayer.h:359-378
    bool init(RasterLayer<elemType>* dataLayer, const char* neighborFile, int comptGrain = 1) {
        if (!dataLayer) return false;
        return init(vector<RasterLayer<elemType>*>(1, dataLayer), neighborFile, comptGrain);
    }
    bool init(vector<RasterLayer<elemType>*> dataLayers, const char* neighborFile, int comptGrain = 1) {
        if (dataLayers.empty()) return false;
        _vDataLayers = dataLayers;
        return init(neighborFile, comptGrain);
    }
    // gpro/computeLayer.h:210-262: ceil(work rows / grain) x ceil(work cols /
    // grain) cells of the first data layer's work rectangle, all 0.
    bool init(const char* neighborFile, int comptGrain = 1) {
        if (_vDataLayers.empty() || !_vDataLayers[0]->_pMetaData || comptGrain < 1) return false;
        if (neighborFile) {
            if (!this->readNeighborhood(neighborFile)) return false;
        } else if (!this->newLocalNbrhood()) {
            return false;
        }
        _ring = neighborFile != nullptr;
        const MetaData& rhs = *_vDataLayers[0]->_pMetaData;
        int64_t crows, ccols;
        if (pargo_compute_load_dims(rhs._glbDims.nRows(), rhs._glbDims.nCols(), comptGrain, &crows, &ccols) !=
            PARGO_OK)
            return false;
        _comptGrain = comptGrain;
        delete this->_pMetaData;
        this->_pMetaData = new MetaData(rhs);
        MetaData& m = *this->_pMetaData;
        m.cellSize = rhs.cellSize * comptGrain;
        m.row = (int)crows;
        m.column = (int)ccols;
        m.dataType = sizeof(elemType) == 4 ? PARGO_F32 : PARGO_F64;
        m._domDcmpType = NON_DCMP;
        m._glbDims = SpaceDims((int)crows, (int)ccols);
        m._localdims = m._glbDims;
        m._MBR = CoordBR(CellCoord(0, 0), CellCoord((int)crows - 1, (int)ccols - 1));
        if (!this->nbrhood()->calcWorkBR(m._localworkBR, m._glbDims)) return false;
        m.pTransform[0] += rhs._localworkBR.minICol() * rhs.cellSize;
        m.pTransform[3] -= rhs._localworkBR.minIRow() * rhs.cellSize;
        m.pTransform[1] *= comptGrain;
        m.pTransform[5] *= comptGrain;
        return this->newCellSpace(m._localdims, (elemType)0);
    }

    // Every part's data rectangle of a load-weighted row decomposition of the
    // first data layer (DeComposition::valRowDcmp + the mapping of
    // getCompuLoad); an addition -- the reference hands each rank its own.
    bool decompose(int nSubSpcs, vector<CoordBR>& parts) {
        parts.clear();
        if (_vDataLayers.empty() || !this->_pMetaData) return false;
        pargo_ctx* ctx = Application::context();
        if (!ctx) return false;
        const MetaData& d = *_vDataLayers[0]->_pMetaData;
        pargo_raster load = this->abi_raster();
        std::vector<int64_t> bounds(4 * (size_t)(nSubSpcs > 0 ? nSubSpcs : 1));
        if (!report_status(pargo_load_decompose(ctx, &load, _ring ? 1 : 0, d._glbDims.nRows(), d._glbDims.nCols(),
                                                &_vDataLayers[0]->nbrhood()->abi(), nSubSpcs, nullptr,
                                                bounds.data(), nullptr),
                           "ComputeLayer::decompose"))
            return false;
        for (int i = 0; i < nSubSpcs; i++)
            parts.push_back(CoordBR(CellCoord((int)bounds[4 * i], (int)bounds[4 * i + 1]),
                                    CellCoord((int)bounds[4 * i + 2], (int)bounds[4 * i + 3])));
        return true;
    }

    // gpro/computeLayer.h:380-443: this rank's data rows of the decomposition.
    bool getCompuLoad(DomDcmpType dcmpType, int nSubSpcs, CoordBR& subWorkBR) {
        if (dcmpType != ROWWISE_DCMP) {
            cerr << "compute layer decomposition: " << dcmpType << " not support until now." << endl;
            return false;
        }
        vector<CoordBR> parts;
        if (!decompose(nSubSpcs, parts)) return false;
        subWorkBR = parts[(size_t)GetRank()];
        return true;
    }

    // gpro/computeLayer.h:447-466
    bool readComputeLoadFile(const char* loadFile) {
        if (!this->nbrhood() && !this->newLocalNbrhood()) return false;
        return this->readFile(loadFile);
    }
    bool writeComputeIntensityFile(const char* outputfile) { return this->writeFile(outputfile); }

    vector<RasterLayer<elemType>*> _vDataLayers;  // gpro/computeLayer.h:121

private:
    double _comptGrain = 0;
    bool _ring = false;
};

// gpro/transformation.h:29-82.  run() fills the compute layer: the
// intensity-ratio Transformation itself runs on the GPU (pargo_compute_load);
// a subclass is an application's own estimate function (as the reference's
// IdwTransformation or KrigingTransformation) and its Operator runs on the
// host over the compute layer's work rectangle, as the reference runs it.
template <class elemType>
class Transformation {
public:
    Transformation() {}
    explicit Transformation(ComputeLayer<elemType>* pLayer) : _pComptLayer(pLayer) { Configure(pLayer, false); }
    Transformation(elemType nodataLoad, elemType validLoad, ComputeLayer<elemType>* pLayer)
        : _nodataLoad(nodataLoad), _validLoad(validLoad), _pComptLayer(pLayer) {
        Configure(pLayer, false);
    }
    virtual ~Transformation() {}

    bool Configure(ComputeLayer<elemType>* pLayer, bool) {
        if (!_pWorkBR && pLayer && pLayer->_pMetaData) _pWorkBR = &pLayer->_pMetaData->_localworkBR;
        return true;
    }
    bool paramInit() {
        if (!_pComptLayer || _pComptLayer->_vDataLayers.empty()) {
            cerr << "Datalayers used for calculating compute layer should not be null." << endl;
            return false;
        }
        _noData = _pComptLayer->_vDataLayers[0]->_pMetaData->noData;
        _computGrain = _pComptLayer->getComputeGrain();
        _dataMBR = _pComptLayer->_vDataLayers[0]->_pMetaData->_MBR;
        _dataWorkBR = _pComptLayer->_vDataLayers[0]->_pMetaData->_localworkBR;
        return true;
    }
    // The estimate of one compute cell; subclasses override it.  The base
    // class's intensity ratio is computed by run() on the GPU instead.
    virtual bool Operator(const CellCoord&) { return true; }
    virtual bool isTermination() { return true; }

    bool run() {
        if (!_pComptLayer || !_pWorkBR) return false;
        if (typeid(*this) == typeid(Transformation<elemType>)) return runIntensity();
        if (!paramInit()) return false;
        do {  // gpro/transformation.h:199-229: serial sweeps of the subclass's Operator
            Termination = 1;
            for (int r = _pWorkBR->minIRow(); r <= _pWorkBR->maxIRow(); r++)
                for (int c = _pWorkBR->minICol(); c <= _pWorkBR->maxICol(); c++)
                    if (!Operator(CellCoord(r, c))) {
                        cout << "Operator is not successes!" << endl;
                        return false;
                    }
        } while (!Termination);
        return true;
    }

protected:
    bool runIntensity() {
        if (_nodataLoad < 0 || _validLoad < 0) {
            cerr << "The load specified cannot be negative." << endl;
            return false;
        }
        vector<RasterLayer<elemType>*>& dl = _pComptLayer->_vDataLayers;
        if (dl.empty()) {
            cerr << "Datalayers used for calculating compute layer should not be null." << endl;
            return false;
        }
        pargo_ctx* ctx = Application::context();
        if (!ctx) return false;
        std::vector<pargo_raster> data;
        for (RasterLayer<elemType>* l : dl) data.push_back(l->abi_raster());
        pargo_raster load = _pComptLayer->abi_raster();
        return report_status(pargo_compute_load(ctx, (int)data.size(), data.data(), &dl[0]->nbrhood()->abi(),
                                                (int)_pComptLayer->getComputeGrain(), _pComptLayer->hasRing() ? 1 : 0,
                                                (double)_nodataLoad, (double)_validLoad, &load, nullptr),
                             "Transformation::run");
    }

    elemType _nodataLoad = 0, _validLoad = 0;
    double _noData = 0, _computGrain = 0;
    CoordBR _dataMBR, _dataWorkBR;
    ComputeLayer<elemType>* _pComptLayer = nullptr;
    CoordBR* _pWorkBR = nullptr;
    int _myRank = 0;

public:
    int Termination = 1;
};

// gpro/deComposition.h:31-80: the load-weighted row split of a compute layer
// (valRowDcmp), in compute rows.
template <class elemType>
class DeComposition {
public:
    DeComposition() {}
    DeComposition(const SpaceDims& cellSpaceDims, const Neighborhood<elemType>& nbrhood)
        : _glbDims(cellSpaceDims), _pNbrhood(&nbrhood) {}

    bool valRowDcmp(vector<CoordBR>& vDcmpBR, ComputeLayer<elemType>& layer, int nSubSpcs) const {
        pargo_ctx* ctx = Application::context();
        if (!ctx || layer._vDataLayers.empty()) return false;
        const MetaData& d = *layer._vDataLayers[0]->_pMetaData;
        pargo_raster load = layer.abi_raster();
        std::vector<int64_t> comp(2 * (size_t)(nSubSpcs > 0 ? nSubSpcs : 1)), bounds(4 * comp.size() / 2);
        if (!report_status(pargo_load_decompose(ctx, &load, layer.hasRing() ? 1 : 0, d._glbDims.nRows(),
                                                d._glbDims.nCols(), &layer._vDataLayers[0]->nbrhood()->abi(),
                                                nSubSpcs, comp.data(), bounds.data(), nullptr),
                           "DeComposition::valRowDcmp"))
            return false;
        const int maxCol = layer._pMetaData->_MBR.maxICol();
        for (int i = 0; i < nSubSpcs; i++)
            vDcmpBR.push_back(CoordBR(CellCoord((int)comp[2 * i], 0), CellCoord((int)comp[2 * i + 1], maxCol)));
        return true;
    }

private:
    SpaceDims _glbDims;
    const Neighborhood<elemType>* _pNbrhood = nullptr;
};

}  // namespace GPRO

#endif
