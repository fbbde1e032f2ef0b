/*
 * fakemex.c -- the MATLAB stand-in behind mex.h / matrix.h.
 *
 * Holds a table of global variables (name -> mxArray), numeric arrays in
 * MATLAB's column-major layout, 1x1 structs with named fields, and a
 * mexEvalString hook so that the Ext-plugin callbacks an engine makes
 * (mexEvalString("DoExtPlugin"), "DoGPUFetch") reach the test harness.
 * mexErrMsgTxt unwinds to fm_call() with longjmp, as MATLAB's does.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "matrix.h"
#include "mex.h"

struct mxArray_tag {
    int class_id;
    int ndims;
    mwSize dims[8];
    size_t numel;
    size_t elsize;
    void *data;
    /* struct fields */
    int nfields;
    char **names;
    mxArray **values;
};

#define FM_MAX_GLOBALS 64
static char *g_names[FM_MAX_GLOBALS];
static mxArray *g_values[FM_MAX_GLOBALS];
static int g_count = 0;
static fm_eval_fn g_eval = NULL;
static jmp_buf *g_jmp = NULL;
static char g_err[1024];
static int g_verbose = 0;

static size_t class_size(int c) {
    switch (c) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxINT32_CLASS: return 4;
    default: return 0;
    }
}

static void fm_free(mxArray *a) {
    if (!a) return;
    if (a->class_id == mxSTRUCT_CLASS) {
        for (int i = 0; i < a->nfields; ++i) {
            free(a->names[i]);
            fm_free(a->values[i]);
        }
        free(a->names);
        free(a->values);
    }
    free(a->data);
    free(a);
}

mxArray *fm_new_numeric(int class_id, int ndims, const int *dims) {
    size_t es = class_size(class_id);
    if (es == 0 || ndims < 1 || ndims > 8) return NULL;
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->class_id = class_id;
    /* MATLAB arrays have at least two dimensions */
    a->ndims = ndims < 2 ? 2 : ndims;
    a->dims[0] = dims[0];
    a->dims[1] = ndims >= 2 ? dims[1] : 1;
    for (int i = 2; i < ndims; ++i) a->dims[i] = dims[i];
    /* MATLAB drops trailing singleton dimensions beyond the second */
    while (a->ndims > 2 && a->dims[a->ndims - 1] == 1) a->ndims--;
    a->numel = 1;
    for (int i = 0; i < a->ndims; ++i) a->numel *= (size_t)a->dims[i];
    a->elsize = es;
    a->data = calloc(a->numel ? a->numel : 1, es);
    return a;
}

mxArray *fm_new_struct(void) {
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->class_id = mxSTRUCT_CLASS;
    a->ndims = 2;
    a->dims[0] = a->dims[1] = 1;
    a->numel = 1;
    return a;
}

int fm_set_field(mxArray *st, const char *name, mxArray *value) {
    if (!st || st->class_id != mxSTRUCT_CLASS) return -1;
    for (int i = 0; i < st->nfields; ++i) {
        if (strcmp(st->names[i], name) == 0) {
            fm_free(st->values[i]);
            st->values[i] = value;
            return 0;
        }
    }
    st->names = (char **)realloc(st->names, sizeof(char *) * (st->nfields + 1));
    st->values = (mxArray **)realloc(st->values, sizeof(mxArray *) * (st->nfields + 1));
    st->names[st->nfields] = strdup(name);
    st->values[st->nfields] = value;
    st->nfields++;
    return 0;
}

int fm_set_global(const char *name, mxArray *value) {
    for (int i = 0; i < g_count; ++i) {
        if (strcmp(g_names[i], name) == 0) {
            if (g_values[i] != value) fm_free(g_values[i]);
            g_values[i] = value;
            return 0;
        }
    }
    if (g_count >= FM_MAX_GLOBALS) return -1;
    g_names[g_count] = strdup(name);
    g_values[g_count] = value;
    g_count++;
    return 0;
}

void fm_clear_globals(void) {
    for (int i = 0; i < g_count; ++i) {
        free(g_names[i]);
        fm_free(g_values[i]);
    }
    g_count = 0;
}

void *fm_data(const mxArray *pm) { return pm ? pm->data : NULL; }
void fm_set_eval_handler(fm_eval_fn fn) { g_eval = fn; }
void fm_set_verbose(int v) { g_verbose = v; }
const char *fm_last_error(void) { return g_err; }

int fm_call(fm_mex_fn fn) {
    jmp_buf env;
    jmp_buf *prev = g_jmp;
    g_err[0] = 0;
    g_jmp = &env;
    if (setjmp(env) != 0) {
        g_jmp = prev;
        return 1;
    }
    fn(0, NULL, 0, NULL);
    g_jmp = prev;
    return 0;
}

int fm_call_args(fm_mex_fn fn, int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs) {
    jmp_buf env;
    jmp_buf *prev = g_jmp;
    g_err[0] = 0;
    g_jmp = &env;
    if (setjmp(env) != 0) {
        g_jmp = prev;
        return 1;
    }
    fn(nlhs, plhs, nrhs, prhs);
    g_jmp = prev;
    return 0;
}

void fm_free_array(mxArray *pm) { fm_free(pm); }

/* ---- MATLAB API --------------------------------------------------------- */

double *mxGetPr(const mxArray *pm) { return pm && pm->class_id == mxDOUBLE_CLASS ? (double *)pm->data : NULL; }
size_t mxGetM(const mxArray *pm) { return pm ? (size_t)pm->dims[0] : 0; }
size_t mxGetN(const mxArray *pm) {
    if (!pm) return 0;
    size_t n = 1;
    for (int i = 1; i < pm->ndims; ++i) n *= (size_t)pm->dims[i];
    return n;
}
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity flag) {
    (void)flag;
    int dims[2] = {(int)m, (int)n};
    return fm_new_numeric(mxDOUBLE_CLASS, 2, dims);
}
mxArray *mxCreateNumericArray(size_t ndim, const mwSize *dims, mxClassID classid, mxComplexity flag) {
    (void)flag;
    int d[8];
    for (size_t i = 0; i < ndim && i < 8; ++i) d[i] = dims[i];
    return fm_new_numeric(classid, (int)(ndim < 8 ? ndim : 8), d);
}

const mxArray *mexGetVariablePtr(const char *workspace, const char *name) {
    (void)workspace;
    for (int i = 0; i < g_count; ++i)
        if (strcmp(g_names[i], name) == 0) return g_values[i];
    return NULL;
}

mxArray *mxGetField(const mxArray *pm, mwIndex index, const char *fieldname) {
    if (!pm || pm->class_id != mxSTRUCT_CLASS || index != 0) return NULL;
    for (int i = 0; i < pm->nfields; ++i)
        if (strcmp(pm->names[i], fieldname) == 0) return pm->values[i];
    if (g_verbose) fprintf(stderr, "fakemex: missing field %s\n", fieldname);
    return NULL;
}

void *mxGetData(const mxArray *pm) { return pm ? pm->data : NULL; }
size_t mxGetNumberOfElements(const mxArray *pm) { return pm ? pm->numel : 0; }
mwSize mxGetNumberOfDimensions(const mxArray *pm) { return pm ? pm->ndims : 0; }
const mwSize *mxGetDimensions(const mxArray *pm) { return pm ? pm->dims : NULL; }
void *mxCalloc(size_t n, size_t size) { return calloc(n ? n : 1, size ? size : 1); }
bool mxUnshareArray(mxArray *pm, bool noDeepCopy) {
    (void)pm;
    (void)noDeepCopy;
    return true;
}

int mexPrintf(const char *fmt, ...) {
    if (!g_verbose) return 0;
    va_list ap;
    va_start(ap, fmt);
    int n = vfprintf(stderr, fmt, ap);
    va_end(ap);
    return n;
}

int mexEvalString(const char *command) {
    if (g_eval) return g_eval(command);
    return 0;
}

void mexErrMsgTxt(const char *msg) {
    snprintf(g_err, sizeof(g_err), "%s", msg ? msg : "");
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "mexErrMsgTxt outside fm_call: %s\n", g_err);
    abort();
}

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
    char buf[900];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    snprintf(g_err, sizeof(g_err), "%s: %s", id ? id : "", buf);
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "mexErrMsgIdAndTxt outside fm_call: %s\n", g_err);
    abort();
}
