// gpro.cpp -- Application, the single-rank MPI calls, utilities and the GPU
// Run() of the four focal operators.
#include <strings.h>
#include <sys/stat.h>
#include <time.h>

#include "gpro/gpro.h"
#include "gpro/operators.h"
#include "mpi.h"
#include "utility.h"

namespace GPRO {

ProgramType Application::_programType = Serial_Type;

namespace {
pargo_ctx* g_ctx = nullptr;
}

pargo_ctx* Application::context() {
    if (!g_ctx) {
        const char* env = getenv("PARGO_DEVICE");
        const int dev = env ? atoi(env) : 0;
        const pargo_status st = pargo_create(dev, &g_ctx);
        if (st != PARGO_OK) {
            cerr << "Application: no usable CUDA device " << dev << " (status " << (int)st << ")" << endl;
            g_ctx = nullptr;
        }
    }
    return g_ctx;
}

// application.cpp:6-18: every program type runs on the GPU here.
bool Application::START(ProgramType programType, int, char*[]) {
    _programType = programType;
    return context() != nullptr;
}

bool Application::END() {
    if (g_ctx) pargo_destroy(g_ctx);
    g_ctx = nullptr;
    return true;
}

bool report_status(pargo_status st, const char* what) {
    if (st == PARGO_OK) return true;
    cerr << what << " failed: " << pargo_last_error(g_ctx) << " (status " << (int)st << ")" << endl;
    return false;
}

// apps/morphology/slope/slopeOperator.cpp:3-25
SlopeAlgor GetSlopeAlgorithm(const string& arg) {
    if (StringMatch(arg, "FFD")) return FFD;
    if (StringMatch(arg, "MD")) return MD;
    if (StringMatch(arg, "SD")) return SD;
    if (StringMatch(arg, "SFD")) return SFD;
    if (StringMatch(arg, "TFD")) return TFD;
    if (StringMatch(arg, "TFDW")) return TFDW;
    return FD;
}

bool SlopeOperator::Run() {
    if (!_pDEMLayer || !_pSlopeLayer) {
        cerr << "SlopeOperator::Run: demLayer and slopeLayer must be set" << endl;
        return false;
    }
    pargo_ctx* ctx = Application::context();
    if (!ctx) return false;
    pargo_raster dem = _pDEMLayer->abi_raster(), out = _pSlopeLayer->abi_raster();
    return report_status(pargo_slope(ctx, &dem, &out, &_pDEMLayer->nbrhood()->abi(), (int)calcAlgor,
                                     _degrees ? PARGO_SLOPE_DEGREES : PARGO_SLOPE_RATIO, nullptr),
                         "SlopeOperator::Run");
}

bool D8Operator::Run() {
    if (!_pDEMLayer || !_pD8Layer) {
        cerr << "D8Operator::Run: demLayer and d8Layer must be set" << endl;
        return false;
    }
    pargo_ctx* ctx = Application::context();
    if (!ctx) return false;
    pargo_raster dem = _pDEMLayer->abi_raster(), out = _pD8Layer->abi_raster();
    return report_status(pargo_d8(ctx, &dem, &out, &_pDEMLayer->nbrhood()->abi(), dirType, nullptr),
                         "D8Operator::Run");
}

bool PitRemoveOperator::Run() {
    if (!_pDEMLayer || !_pwDEMLayer) {
        cerr << "PitRemoveOperator::Run: demLayer and wdemLayer must be set" << endl;
        return false;
    }
    pargo_ctx* ctx = Application::context();
    if (!ctx) return false;
    pargo_raster dem = _pDEMLayer->abi_raster(), out = _pwDEMLayer->abi_raster();
    pargo_fill_opts opts{_gap, 10000.0, 0};
    return report_status(pargo_fill(ctx, &dem, &out, &_pDEMLayer->nbrhood()->abi(), &opts, &stats, nullptr),
                         "PitRemoveOperator::Run");
}

bool SCAOperator::Run() {
    if (!_weightLayers.empty()) {  // the scamfdmd operator
        if (_weightLayers.size() != 8 || !_pSCALayer) {
            cerr << "SCAOperator::Run: 8 mfdLayer weight layers and scaLayer must be set" << endl;
            return false;
        }
        pargo_ctx* ctx = Application::context();
        if (!ctx) return false;
        pargo_raster w[8], out = _pSCALayer->abi_raster();
        for (int i = 0; i < 8; i++) w[i] = _weightLayers[i]->abi_raster();
        return report_status(pargo_sca_mfd(ctx, w, &out, &_weightLayers[0]->nbrhood()->abi(), nullptr),
                             "SCAOperator::Run");
    }
    if (!_pD8Layer || !_pSCALayer) {
        cerr << "SCAOperator::Run: d8Layer and scaLayer must be set" << endl;
        return false;
    }
    pargo_ctx* ctx = Application::context();
    if (!ctx) return false;
    int c = _contract;
    if (c < 0) {
        const char* env = getenv("PARGO_SCA_CONTRACT");
        c = (env && StringMatch(env, "converged")) ? PARGO_SCA_CONVERGED : PARGO_SCA_SHIPPED;
    }
    pargo_raster d8 = _pD8Layer->abi_raster(), out = _pSCALayer->abi_raster();
    return report_status(pargo_sca(ctx, &d8, &out, &_pD8Layer->nbrhood()->abi(), c, nullptr), "SCAOperator::Run");
}

bool MFDOperator::Run() {
    if (!_pDEMLayer || _weightLayers.size() != 8) {
        cerr << "MFDOperator::Run: demLayer and 8 weightLayers must be set" << endl;
        return false;
    }
    pargo_ctx* ctx = Application::context();
    if (!ctx) return false;
    pargo_raster dem = _pDEMLayer->abi_raster(), w[8];
    for (int i = 0; i < 8; i++) w[i] = _weightLayers[i]->abi_raster();
    return report_status(pargo_mfd(ctx, &dem, w, &_pDEMLayer->nbrhood()->abi(), slpExp, nullptr), "MFDOperator::Run");
}

bool TWIOperator::Run() {
    if (!_pSCALayer || !_pSlopeLayer || !_pTWILayer) {
        cerr << "TWIOperator::Run: SCALayer, slopeLayer and twiLayer must be set" << endl;
        return false;
    }
    pargo_ctx* ctx = Application::context();
    if (!ctx) return false;
    pargo_raster sl = _pSlopeLayer->abi_raster(), sa = _pSCALayer->abi_raster(), out = _pTWILayer->abi_raster();
    return report_status(pargo_twi(ctx, &sl, &sa, &out, &_pSCALayer->nbrhood()->abi(), nullptr), "TWIOperator::Run");
}

int GetRank() { return 0; }

}  // namespace GPRO

bool StringMatch(const char* a, const char* b) { return strcasecmp(a, b) == 0; }
bool StringMatch(const string& a, const string& b) { return strcasecmp(a.c_str(), b.c_str()) == 0; }
vector<string> SplitString(const string& item, char delimiter) {
    vector<string> out;
    size_t start = 0;
    while (start < item.size()) {  // fields as getline() yields them: no trailing empty field
        size_t end = item.find(delimiter, start);
        if (end == string::npos) end = item.size();
        out.push_back(item.substr(start, end - start));
        start = end + 1;
    }
    return out;
}
bool FileExists(string const& filename) {
    struct stat st;
    return stat(filename.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

extern "C" {
int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) {
    *rank = 0;
    return MPI_SUCCESS;
}
int MPI_Comm_size(MPI_Comm, int* size) {
    *size = 1;
    return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    const size_t sz = t == MPI_DOUBLE ? 8 : 4;
    if (s != r) memcpy(r, s, sz * (size_t)n);
    return MPI_SUCCESS;
}
int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int, MPI_Comm c) {
    return MPI_Allreduce(s, r, n, t, op, c);
}
}
