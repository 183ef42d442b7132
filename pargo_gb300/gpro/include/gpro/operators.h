// operators.h -- the four focal operators of PaRGO with the reference's setter
// API (apps/morphology/slope/slopeOperator.h, apps/hydrology/flowdird8/d8Operator.h,
// apps/hydrology/pitremove/pitRemoveOperator.h, apps/hydrology/scad8/scaOperator.h),
// TWI (apps/hydrology/twi/TWIOperator.h) and MFD-md (apps/hydrology/flowdirmfdmd/mfdOperator.h,
// apps/hydrology/scamfdmd/scaOperator.h);
// Run() is one call of the GPU C ABI on the layers' host buffers.
#ifndef PARGO_GPRO_OPERATORS_H
#define PARGO_GPRO_OPERATORS_H

#include "gpro/gpro.h"

namespace GPRO {

// apps/morphology/slope/slopeOperator.h:18-26
enum SlopeAlgor { FD, FFD, MD, SD, SFD, TFD, TFDW };
SlopeAlgor GetSlopeAlgorithm(const string& arg);

class SlopeOperator : public RasterOperator<double> {
public:
    void demLayer(RasterLayer<double>& layerD) {
        _pDEMLayer = &layerD;
        Configure(_pDEMLayer, false);
    }
    void slopeLayer(RasterLayer<double>& layerD) {
        _pSlopeLayer = &layerD;
        Configure(_pSlopeLayer, false);
    }
    void calcAlgorithm(SlopeAlgor algor) { calcAlgor = algor; }
    // slope in degrees instead of the reference's rise/run (an addition)
    void degrees(bool on) { _degrees = on; }
    bool Run() override;

protected:
    SlopeAlgor calcAlgor = FD;
    bool _degrees = false;
    RasterLayer<double>* _pDEMLayer = nullptr;
    RasterLayer<double>* _pSlopeLayer = nullptr;
};

class D8Operator : public RasterOperator<double> {
public:
    D8Operator() : dirType(0) {}
    explicit D8Operator(int type) : dirType(type) {}
    void demLayer(RasterLayer<double>& layerD) {
        _pDEMLayer = &layerD;
        Configure(_pDEMLayer, false);
    }
    void d8Layer(RasterLayer<double>& layerD) {
        _pD8Layer = &layerD;
        Configure(_pD8Layer, false);
    }
    bool Run() override;

protected:
    int dirType;
    RasterLayer<double>* _pDEMLayer = nullptr;
    RasterLayer<double>* _pD8Layer = nullptr;
};

class PitRemoveOperator : public RasterOperator<double> {
public:
    void demLayer(RasterLayer<double>& layerD) {
        _pDEMLayer = &layerD;
        Configure(_pDEMLayer, false);
    }
    void wdemLayer(RasterLayer<double>& layerD) {
        _pwDEMLayer = &layerD;
        Configure(_pwDEMLayer, true);
    }
    // the reference hard-codes gap 0.0005 and level 10000.0 (pitRemoveOperator.cpp:36,41)
    void gap(double g) { _gap = g; }
    bool Run() override;
    pargo_fill_stats stats{};

protected:
    double _gap = 0.0005;
    RasterLayer<double>* _pDEMLayer = nullptr;
    RasterLayer<double>* _pwDEMLayer = nullptr;
};

// Topographic wetness index ln(sca / slope) (apps/hydrology/twi/TWIOperator.h:10-31).
class TWIOperator : public RasterOperator<double> {
public:
    void SCALayer(RasterLayer<double>& layerD) {
        _pSCALayer = &layerD;
        Configure(_pSCALayer, false);
    }
    void slopeLayer(RasterLayer<double>& layerD) {
        _pSlopeLayer = &layerD;
        Configure(_pSlopeLayer, false);
    }
    void twiLayer(RasterLayer<double>& layerD) {
        _pTWILayer = &layerD;
        Configure(_pTWILayer, false);
    }
    bool Run() override;

protected:
    RasterLayer<double>* _pSCALayer = nullptr;
    RasterLayer<double>* _pSlopeLayer = nullptr;
    RasterLayer<double>* _pTWILayer = nullptr;
};

class SCAOperator : public RasterOperator<double> {
public:
    void d8Layer(RasterLayer<double>& layerD) {
        _pD8Layer = &layerD;
        Configure(_pD8Layer, false);
    }
    void scaLayer(RasterLayer<double>& layerD) {
        _pSCALayer = &layerD;
        Configure(_pSCALayer, true);
    }
    // PARGO_SCA_SHIPPED (default: what the reference operator outputs, one
    // accumulation sweep) or PARGO_SCA_CONVERGED (the full upslope count);
    // the environment variable PARGO_SCA_CONTRACT=converged selects the latter.
    void contract(int c) { _contract = c; }
    // The scamfdmd operator's input (apps/hydrology/scamfdmd/scaOperator.h:24):
    // 8 MFD weight layers instead of a D8 layer; Run() then computes the MFD SCA.
    void mfdLayer(vector<RasterLayer<double>*>& layerV) {
        _weightLayers.assign(layerV.begin(), layerV.end());
        for (RasterLayer<double>* l : _weightLayers) Configure(l, false);
    }
    bool Run() override;

protected:
    int _contract = -1;
    RasterLayer<double>* _pD8Layer = nullptr;
    RasterLayer<double>* _pSCALayer = nullptr;
    vector<RasterLayer<double>*> _weightLayers;
};

// MFD-md flow partition (apps/hydrology/flowdirmfdmd/mfdOperator.h:13-40): 8
// weight layers, layer i for window position i (i < 4) or i + 1.
class MFDOperator : public RasterOperator<double> {
public:
    MFDOperator() : slpExp(0.0) {}
    explicit MFDOperator(double pExp) : slpExp(pExp) {}
    void demLayer(RasterLayer<double>& layerD) {
        _pDEMLayer = &layerD;
        Configure(_pDEMLayer, false);
    }
    void weightLayers(vector<RasterLayer<double>*>& layers) {
        _weightLayers.assign(layers.begin(), layers.end());
        for (RasterLayer<double>* l : _weightLayers) Configure(l, false);
    }
    bool Run() override;

protected:
    double slpExp;
    RasterLayer<double>* _pDEMLayer = nullptr;
    vector<RasterLayer<double>*> _weightLayers;
};

}  // namespace GPRO

#endif
