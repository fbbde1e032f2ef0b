/*
 * mex.h -- a small stand-in for MATLAB's MEX API, enough to build and drive
 * MRiLab-style scan engines (which read MATLAB *global* structs in place) in
 * a process that has no MATLAB.
 *
 * The real MATLAB header is used when the wrappers are built inside MATLAB
 * (`mex ...`); this one is used by the test harness, which fills the globals
 * (VObj, VMag, VCoi, VCtl, VSeq, VVar, VSig) from Python through the
 * fm_* functions below and then calls the engine's mexFunction.
 *
 * The calls implemented are exactly the ones the MRiLab engines use:
 * mexGetVariablePtr, mxGetField, mxGetData, mxGetNumberOfElements,
 * mxGetNumberOfDimensions, mxGetDimensions, mxCalloc, mxUnshareArray,
 * mexPrintf, mexEvalString, mexErrMsgTxt
 * (Lib/src/engine/CPUEngine/DoScanAtCPU.cpp:118-210,356-409).
 */
#ifndef MRL_FAKE_MEX_H
#define MRL_FAKE_MEX_H

#include <stddef.h>
#include "matrix.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Engines define this; declaring it here gives it C linkage, as MATLAB's
 * own mex.h does, so the harness can find it with dlsym. */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

const mxArray *mexGetVariablePtr(const char *workspace, const char *name);
int mexPrintf(const char *fmt, ...);
int mexEvalString(const char *command);
void mexErrMsgTxt(const char *msg);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);

#ifdef __cplusplus
}
#endif

#endif
