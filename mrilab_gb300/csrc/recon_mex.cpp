// Thin mex layer of the reconstruction: built once per entry point.
//
//   -DMRL_WRAP_GRID -> DoGridding: [Sx2, Sy2] = DoGridding(Kx, Ky, Sx, Sy,
//       DCF, Ker, GridSize, HalfWidth), the reference's gridding mex
//       (Lib/src/recon/DoGridding/DoGridding.cpp:14-66), on mrl_grid2d;
//   -DMRL_WRAP_CART -> DoCartReconGPU: [Real, Imag, Mag, Phase] =
//       DoCartReconGPU(Sx, Sy, [ResFreq Lines SliceNum RxCoilNum TypeNum
//       Echoes EPI_ETL ZF_Kx ZF_Ky ZF_Kz ReadoutFirst]), the transform part of
//       Src/Recon/Default/DoCartRecon.m / DoEPIRecon.m on mrl_recon_cart (the
//       MATLAB side keeps building VImg from the four arrays).
#include <cstring>

#include "../../include/mrl_recon.h"
#include "mex.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
#if defined(MRL_WRAP_GRID)
    if (nrhs < 8 || nlhs > 2) {
        mexErrMsgIdAndTxt("MRiLab:grid", "usage: [Sx2, Sy2] = DoGridding(Kx, Ky, Sx, Sy, DCF, Ker, GridSize, HalfWidth)");
        return;
    }
    const int n = (int)(mxGetM(prhs[0]) * mxGetN(prhs[0]));
    const int nk = (int)(mxGetM(prhs[5]) * mxGetN(prhs[5]));
    const int G = (int)*mxGetPr(prhs[6]);
    const double hw = *mxGetPr(prhs[7]);
    plhs[0] = mxCreateDoubleMatrix(G, G, mxREAL);
    plhs[1] = mxCreateDoubleMatrix(G, G, mxREAL);
    const int rc = mrl_grid2d(mxGetPr(prhs[0]), mxGetPr(prhs[1]), mxGetPr(prhs[2]), mxGetPr(prhs[3]),
                              mxGetPr(prhs[4]), n, mxGetPr(prhs[5]), nk, G, hw, mxGetPr(plhs[0]), mxGetPr(plhs[1]), 0);
    if (rc != MRL_OK) mexErrMsgIdAndTxt("MRiLab:grid", "%s: %s", mrl_status_string(rc), mrl_last_error());
#elif defined(MRL_WRAP_CART)
    if (nrhs < 3 || mxGetM(prhs[2]) * mxGetN(prhs[2]) < 11) {
        mexErrMsgIdAndTxt("MRiLab:recon", "usage: [Real, Imag, Mag, Phase] = DoCartReconGPU(Sx, Sy, dims(11))");
        return;
    }
    const double *d = mxGetPr(prhs[2]);
    mrl_recon_args a;
    std::memset(&a, 0, sizeof(a));
    a.abi_version = MRL_ABI_VERSION;
    a.sx = mxGetPr(prhs[0]);
    a.sy = mxGetPr(prhs[1]);
    a.res_freq = (int)d[0];
    a.lines = (int)d[1];
    a.slices = (int)d[2];
    a.rx = (int)d[3];
    a.pools = (int)d[4];
    a.echoes = (int)d[5];
    a.epi_etl = (int)d[6];
    a.zf_kx = (int)d[7];
    a.zf_ky = (int)d[8];
    a.zf_kz = (int)d[9];
    a.readout_first = (int)d[10];
    // output sizes as mrl_recon_cart computes them
    const int F = a.res_freq - 1, L = a.epi_etl > 0 ? a.epi_etl * a.lines : a.lines;
    const bool zf = a.zf_kx > 0 || a.zf_ky > 0 || a.zf_kz > 0;
    const int fx = zf ? a.zf_kx : F, fy = zf ? a.zf_ky : L, fz = zf ? a.zf_kz * a.slices : a.slices;
    const mwSize dims[5] = {a.readout_first ? fx : fy, a.readout_first ? fy : fx, fz, a.rx, a.echoes};
    double **outs[4] = {&a.img_real, &a.img_imag, &a.img_mag, &a.img_phase};
    const int nout = nlhs < 1 ? 1 : (nlhs > 4 ? 4 : nlhs);
    for (int k = 0; k < 4; ++k) {
        if (k < nout) {
            plhs[k] = mxCreateNumericArray(5, dims, mxDOUBLE_CLASS, mxREAL);
            *outs[k] = mxGetPr(plhs[k]);
        } else {
            *outs[k] = nullptr;
        }
    }
    const int rc = mrl_recon_cart(&a);
    if (rc != MRL_OK) mexErrMsgIdAndTxt("MRiLab:recon", "%s: %s", mrl_status_string(rc), mrl_last_error());
#else
#error "define MRL_WRAP_GRID or MRL_WRAP_CART"
#endif
}
