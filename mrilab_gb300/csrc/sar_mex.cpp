// Thin mex layer of the SAR engine: DoCalSARAtGPU on top of mrl_sar.
//
// The reference's SAR engine DoCalSARAtCPU (Lib/src/engine/CPUEngine/
// DoCalSARAtCPU.cpp:85) ignores its arguments and works on the MATLAB
// globals VObj (MassDen, ECon), VCoi (TxE1x/y/z, TxCoilNum), VCtl (TRNum),
// VSeq, VVar (cursor, SAR, SARi) and VSig (SAR, Muts, tSample, tRealSample)
// in place (:117-163); this wrapper binds the same fields and calls
// mrl_sar.  The SAR watcher (Src/Main/DoSARWatchExec.m:105) calls it by
// name in place of DoCalSARAtCPU.  Errors are raised with mexErrMsgIdAndTxt.
#include <cstring>

#include "../../include/mrl_sar.h"
#include "mex.h"

namespace {

const mxArray *field(const char *global, const char *name) {
    const mxArray *st = mexGetVariablePtr("global", global);
    if (!st) return nullptr;
    return mxGetField(st, 0, name);
}

template <typename T>
T *ptr(const char *global, const char *name) {
    const mxArray *f = field(global, name);
    return f ? static_cast<T *>(mxGetData(f)) : nullptr;
}

int count(const char *global, const char *name) {
    const mxArray *f = field(global, name);
    return f ? (int)mxGetNumberOfElements(f) : 0;
}

bool bind(mrl_sar_args &a) {
    std::memset(&a, 0, sizeof(a));
    a.abi_version = MRL_ABI_VERSION;
    const mxArray *md = field("VObj", "MassDen");
    if (!md) return false;
    const int nd = (int)mxGetNumberOfDimensions(md);
    const mwSize *dims = mxGetDimensions(md);
    a.ny = dims[0];
    a.nx = nd > 1 ? dims[1] : 1;
    a.nz = nd > 2 ? dims[2] : 1;
    a.econ = ptr<float>("VObj", "ECon");
    const int *txn = ptr<int>("VCoi", "TxCoilNum");
    if (!txn) return false;
    a.tx_num = *txn;
    a.tx_e1x = ptr<float>("VCoi", "TxE1x");
    a.tx_e1y = ptr<float>("VCoi", "TxE1y");
    a.tx_e1z = ptr<float>("VCoi", "TxE1z");
    const int *trn = ptr<int>("VCtl", "TRNum");
    const int *gpu = ptr<int>("VCtl", "GPUIndex");
    a.tr_num = trn ? *trn : 0;
    a.gpu_index = gpu ? *gpu : 0;
    const double *num = ptr<double>("VCtl", "Numerics");
    a.numerics = num ? (int)*num : MRL_NUMERICS_ACCURATE;
    mrl_sequence &q = a.seq;
    q.uts = ptr<double>("VSeq", "utsLine");
    q.ts = ptr<double>("VSeq", "tsLine");
    q.rf_amp = ptr<double>("VSeq", "rfAmpLine");
    q.rf_phase = ptr<double>("VSeq", "rfPhaseLine");
    q.rf_freq = ptr<double>("VSeq", "rfFreqLine");
    q.rf_coil = ptr<double>("VSeq", "rfCoilLine");
    q.ext = ptr<double>("VSeq", "ExtLine");
    q.flags = ptr<double>("VSeq", "flagsLine");
    q.n_uts = count("VSeq", "utsLine");
    q.n_ts = count("VSeq", "tsLine");
    q.n_rf = count("VSeq", "rfAmpLine");
    q.n_ext = count("VSeq", "ExtLine");
    mrl_state &v = a.var;
    v.t = ptr<double>("VVar", "t");
    v.dt = ptr<double>("VVar", "dt");
    v.rf_amp = ptr<double>("VVar", "rfAmp");
    v.rf_phase = ptr<double>("VVar", "rfPhase");
    v.rf_freq = ptr<double>("VVar", "rfFreq");
    v.rf_coil = ptr<double>("VVar", "rfCoil");
    v.ext = ptr<double>("VVar", "Ext");
    v.utsi = ptr<int>("VVar", "utsi");
    v.rfi = ptr<int>("VVar", "rfi");
    v.exti = ptr<int>("VVar", "Exti");
    v.tr_count = ptr<int>("VVar", "TRCount");
    a.sar_acc = ptr<float>("VVar", "SAR");
    a.sari = ptr<int>("VVar", "SARi");
    a.sar = ptr<float>("VSig", "SAR");
    a.muts = ptr<double>("VSig", "Muts");
    a.t_sample = ptr<double>("VSig", "tSample");
    a.t_real_sample = ptr<double>("VSig", "tRealSample");
    a.n_sample = count("VSig", "tSample");
    return true;
}

}  // namespace

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    (void)nlhs;
    (void)plhs;
    (void)nrhs;
    (void)prhs;
    mrl_sar_args a;
    if (!bind(a)) {
        mexErrMsgIdAndTxt("MRiLab:sar", "missing or malformed SAR globals (VObj/VCoi/VCtl/VSeq/VVar/VSig)");
        return;
    }
    const int rc = mrl_sar(&a);
    if (rc != MRL_OK) mexErrMsgIdAndTxt("MRiLab:sar", "%s: %s", mrl_status_string(rc), mrl_last_error());
}
