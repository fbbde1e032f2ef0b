/*
 * matrix.h -- mxArray part of the MATLAB stand-in (see mex.h).
 *
 * mwSize / mwIndex are 32-bit, as in MRiLab's own build, which compiles
 * with -DMX_COMPAT_32 (Lib/src/engine/CMakeLists.txt:11): the engines cast
 * int32 struct fields such as VObj.SpinNum to (mwSize*).
 */
#ifndef MRL_FAKE_MATRIX_H
#define MRL_FAKE_MATRIX_H

#include <stddef.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int mwSize;
typedef int mwIndex;

typedef enum {
    mxUNKNOWN_CLASS = 0,
    mxSTRUCT_CLASS = 2,
    mxDOUBLE_CLASS = 6,
    mxSINGLE_CLASS = 7,
    mxINT32_CLASS = 12,
} mxClassID;

typedef struct mxArray_tag mxArray;

mxArray *mxGetField(const mxArray *pm, mwIndex index, const char *fieldname);
void *mxGetData(const mxArray *pm);
size_t mxGetNumberOfElements(const mxArray *pm);
mwSize mxGetNumberOfDimensions(const mxArray *pm);
const mwSize *mxGetDimensions(const mxArray *pm);
void *mxCalloc(size_t n, size_t size);
bool mxUnshareArray(mxArray *pm, bool noDeepCopy);
/* argument-passing mex functions (DoGridding.cpp:51-66) */
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
double *mxGetPr(const mxArray *pm);
size_t mxGetM(const mxArray *pm);
size_t mxGetN(const mxArray *pm);
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity flag);
mxArray *mxCreateNumericArray(size_t ndim, const mwSize *dims, mxClassID classid, mxComplexity flag);

/* ---- harness side (not part of MATLAB's API) ---------------------------- */

/* Create a numeric array with the given class and dimensions (column-major,
 * zero-filled).  Returns the array; fm_data() gives its storage. */
mxArray *fm_new_numeric(int class_id, int ndims, const int *dims);
/* Create an empty 1x1 struct. */
mxArray *fm_new_struct(void);
/* Attach (or replace) a field of a struct; the struct takes ownership. */
int fm_set_field(mxArray *st, const char *name, mxArray *value);
/* Bind a struct as a global variable (replaces and frees an old binding). */
int fm_set_global(const char *name, mxArray *value);
/* Drop every global. */
void fm_clear_globals(void);
void *fm_data(const mxArray *pm);
/* Handler for mexEvalString: returns 0 on success, nonzero on error. */
typedef int (*fm_eval_fn)(const char *command);
void fm_set_eval_handler(fm_eval_fn fn);
/* Call an engine's mexFunction; returns 0, or 1 if it raised mexErrMsgTxt
 * (the message is then available from fm_last_error()). */
typedef void (*fm_mex_fn)(int, mxArray **, int, const mxArray **);
int fm_call(fm_mex_fn fn);
/* Call a mexFunction with arguments; plhs receives the outputs it creates
 * (free them with fm_free_array). */
int fm_call_args(fm_mex_fn fn, int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs);
void fm_free_array(mxArray *pm);
const char *fm_last_error(void);
void fm_set_verbose(int verbose);

#ifdef __cplusplus
}
#endif

#endif
