// Thin mex layer: the reference's mex entry points on top of mrl_scan.
//
// Built once per reference engine with MRL_WRAP_MODEL set, e.g.
//   -DMRL_WRAP_MODEL=MRL_MODEL_NORMAL -> DoScanAtGPU      (DoScanAtGPU.cu:76)
//   -DMRL_WRAP_MODEL=MRL_MODEL_ME     -> DoMEScanAtGPU
//   -DMRL_WRAP_MODEL=MRL_MODEL_MT     -> DoMTScanAtGPU
//   -DMRL_WRAP_MODEL=MRL_MODEL_CEST   -> DoCESTScanAtGPU
//   -DMRL_WRAP_MODEL=MRL_MODEL_GM     -> DoGMScanAtGPU
// Like the reference, mexFunction ignores its arguments and works on the
// MATLAB globals VObj, VMag, VCoi, VCtl, VSeq, VVar and VSig in place
// (DoScanAtGPU.cu:117-214); Ext events call back into MATLAB with
// mexEvalString("DoGPUFetch") and mexEvalString("DoExtPlugin") and re-read
// every pointer afterwards (:565-660).  Errors are raised with
// mexErrMsgIdAndTxt instead of being printed and ignored.
#include <cstring>

#include "../../include/mrl_scan.h"
#include "mex.h"

#ifndef MRL_WRAP_MODEL
#define MRL_WRAP_MODEL MRL_MODEL_NORMAL
#endif

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

// Bind every global the engine reads or writes (DoScanAtGPU.cu:124-214).
bool bind(mrl_scan_args &a) {
    std::memset(&a, 0, sizeof(a));
    a.abi_version = MRL_ABI_VERSION;
    a.model = MRL_WRAP_MODEL;
    const mxArray *mz = field("VObj", "Mz");
    if (!mz) return false;
    const int nd = (int)mxGetNumberOfDimensions(mz);
    const mwSize *dims = mxGetDimensions(mz);
    a.obj.ny = dims[0];
    a.obj.nx = dims[1];
    a.obj.nz = nd > 2 ? dims[2] : 1;
    const int *sn = ptr<int>("VObj", "SpinNum");
    const int *tn = ptr<int>("VObj", "TypeNum");
    const double *gy = ptr<double>("VObj", "Gyro");
    if (!sn || !tn || !gy) return false;
    a.obj.spin_num = *sn;
    a.obj.type_num = *tn;
    a.obj.gyro = *gy;
    a.obj.rho = ptr<float>("VObj", "Rho");
    a.obj.t1 = ptr<float>("VObj", "T1");
    a.obj.t2 = ptr<float>("VObj", "T2");
    a.obj.mx = ptr<float>("VObj", "Mx");
    a.obj.my = ptr<float>("VObj", "My");
    a.obj.mz = ptr<float>("VObj", "Mz");
    const long long V = (long long)a.obj.ny * a.obj.nx * a.obj.nz;
    if (MRL_WRAP_MODEL != MRL_MODEL_NORMAL) {
        a.obj.k = ptr<float>("VObj", "K");
        a.obj.k_channels = V > 0 ? (int)(count("VObj", "K") / V) : 0;
    }
    if (MRL_WRAP_MODEL == MRL_MODEL_GM) a.obj.type_flag = ptr<double>("VObj", "TypeFlag");

    a.mag.db0 = ptr<float>("VMag", "dB0");
    a.mag.dwrnd = ptr<float>("VMag", "dWRnd");
    a.mag.gzgrid = ptr<float>("VMag", "Gzgrid");
    a.mag.gygrid = ptr<float>("VMag", "Gygrid");
    a.mag.gxgrid = ptr<float>("VMag", "Gxgrid");

    const int *txn = ptr<int>("VCoi", "TxCoilNum");
    const int *rxn = ptr<int>("VCoi", "RxCoilNum");
    const double *txd = ptr<double>("VCoi", "TxCoilDefault");
    const double *rxd = ptr<double>("VCoi", "RxCoilDefault");
    if (!txn || !rxn || !txd || !rxd) return false;
    a.coil.tx_num = *txn;
    a.coil.rx_num = *rxn;
    a.coil.tx_default = *txd;
    a.coil.rx_default = *rxd;
    a.coil.tx_mg = ptr<float>("VCoi", "TxCoilmg");
    a.coil.tx_pe = ptr<float>("VCoi", "TxCoilpe");
    a.coil.rx_x = ptr<float>("VCoi", "RxCoilx");
    a.coil.rx_y = ptr<float>("VCoi", "RxCoily");

    a.ctl.cs = ptr<double>("VCtl", "CS");
    const int *trn = ptr<int>("VCtl", "TRNum");
    const int *gpu = ptr<int>("VCtl", "GPUIndex");
    a.ctl.tr_num = trn ? *trn : 0;
    a.ctl.gpu_index = gpu ? *gpu : 0;
    if (MRL_WRAP_MODEL != MRL_MODEL_NORMAL) {
        const int *rm = ptr<int>("VCtl", "RunMode");
        a.ctl.run_mode = rm ? *rm : 0;
    }
    // optional: VCtl.Numerics selects the integrator (0 accurate, 1 reference order, 2 exact propagator)
    const double *num = ptr<double>("VCtl", "Numerics");
    a.ctl.numerics = num ? (int)*num : MRL_NUMERICS_ACCURATE;

    mrl_sequence &q = a.seq;
    q.uts = ptr<double>("VSeq", "utsLine");
    q.ts = ptr<double>("VSeq", "tsLine");
    q.rf_amp = ptr<double>("VSeq", "rfAmpLine");
    q.rf_phase = ptr<double>("VSeq", "rfPhaseLine");
    q.rf_freq = ptr<double>("VSeq", "rfFreqLine");
    q.rf_coil = ptr<double>("VSeq", "rfCoilLine");
    q.gz = ptr<double>("VSeq", "GzAmpLine");
    q.gy = ptr<double>("VSeq", "GyAmpLine");
    q.gx = ptr<double>("VSeq", "GxAmpLine");
    q.adc = ptr<double>("VSeq", "ADCLine");
    q.ext = ptr<double>("VSeq", "ExtLine");
    q.flags = ptr<double>("VSeq", "flagsLine");
    q.n_uts = count("VSeq", "utsLine");
    q.n_ts = count("VSeq", "tsLine");
    q.n_rf = count("VSeq", "rfAmpLine");
    q.n_gz = count("VSeq", "GzAmpLine");
    q.n_gy = count("VSeq", "GyAmpLine");
    q.n_gx = count("VSeq", "GxAmpLine");
    q.n_adc = count("VSeq", "ADCLine");
    q.n_ext = count("VSeq", "ExtLine");

    mrl_state &v = a.var;
    v.t = ptr<double>("VVar", "t");
    v.dt = ptr<double>("VVar", "dt");
    v.rf_amp = ptr<double>("VVar", "rfAmp");
    v.rf_phase = ptr<double>("VVar", "rfPhase");
    v.rf_freq = ptr<double>("VVar", "rfFreq");
    v.rf_coil = ptr<double>("VVar", "rfCoil");
    v.rf_ref = ptr<double>("VVar", "rfRef");
    v.gz = ptr<double>("VVar", "GzAmp");
    v.gy = ptr<double>("VVar", "GyAmp");
    v.gx = ptr<double>("VVar", "GxAmp");
    v.adc = ptr<double>("VVar", "ADC");
    v.ext = ptr<double>("VVar", "Ext");
    v.kz = ptr<double>("VVar", "Kz");
    v.ky = ptr<double>("VVar", "Ky");
    v.kx = ptr<double>("VVar", "Kx");
    v.gpu_fetch = ptr<double>("VVar", "gpuFetch");
    v.utsi = ptr<int>("VVar", "utsi");
    v.rfi = ptr<int>("VVar", "rfi");
    v.gzi = ptr<int>("VVar", "Gzi");
    v.gyi = ptr<int>("VVar", "Gyi");
    v.gxi = ptr<int>("VVar", "Gxi");
    v.adci = ptr<int>("VVar", "ADCi");
    v.exti = ptr<int>("VVar", "Exti");
    v.tr_count = ptr<int>("VVar", "TRCount");

    mrl_signal &s = a.sig;
    s.sx = ptr<double>("VSig", "Sx");
    s.sy = ptr<double>("VSig", "Sy");
    s.kz = ptr<double>("VSig", "Kz");
    s.ky = ptr<double>("VSig", "Ky");
    s.kx = ptr<double>("VSig", "Kx");
    const int *sn2 = ptr<int>("VSig", "SignalNum");
    s.signal_num = sn2 ? *sn2 : 0;
    if (a.ctl.run_mode == 1) {  // history arrays (DoGMScanAtGPU.cu:218-221)
        s.mxs = ptr<float>("VSig", "Mx");
        s.mys = ptr<float>("VSig", "My");
        s.mzs = ptr<float>("VSig", "Mz");
        s.muts = ptr<double>("VSig", "Muts");
    }
    return true;
}

// Ext callback: DoGPUFetch, then DoExtPlugin, re-binding pointers after
// each call into MATLAB (DoScanAtGPU.cu:565-660).
int ext_callback(void *, mrl_scan_args *a, int what) {
    if (what == MRL_EXT_FETCH) {
        if (mexEvalString("DoGPUFetch") != 0) return 0;
        const double *f = ptr<double>("VVar", "gpuFetch");
        return f && *f != 0;
    }
    if (mexEvalString("DoExtPlugin") != 0) return 1;
    const int model = a->model;
    const int numerics = a->ctl.numerics;
    if (!bind(*a)) return 1;
    a->model = model;
    a->ctl.numerics = numerics;
    double *f = ptr<double>("VVar", "gpuFetch");
    if (f) *f = 0;
    return 0;
}

}  // namespace

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    (void)nlhs;
    (void)plhs;
    (void)nrhs;
    (void)prhs;
    mrl_scan_args a;
    if (!bind(a)) {
        mexErrMsgIdAndTxt("MRiLab:scan", "missing or malformed scan globals (VObj/VMag/VCoi/VCtl/VSeq/VVar/VSig)");
        return;
    }
    const int rc = mrl_scan(&a, ext_callback, nullptr);
    if (rc != MRL_OK) mexErrMsgIdAndTxt("MRiLab:scan", "%s: %s", mrl_status_string(rc), mrl_last_error());
}
