/*
 * ipp.h -- project-written stand-in for the ~30 Intel IPP signal functions
 * that MRiLab's CPU engine calls (list: Lib/src/engine/CPUEngine/
 * DoScanAtCPU.cpp:27-55; call sites BlochKernel.h:19-395 and
 * DoScanAtCPU.cpp:238-242,412-414,453-489).  Test infrastructure only: it
 * lets the reference engine source compile unmodified into oracle/_ref so
 * that the oracle port can be checked against it.
 *
 * Every function is a plain element loop over libm single-precision
 * functions.  IPP's own A24 ("24 correct bits") functions are not
 * bit-identical to libm; results from the engine built on this shim are
 * labelled "reference engine on project IPP shim".  ippsSum_32f with
 * ippAlgHintFast is modelled as 16 interleaved float partial sums (the shape
 * of a SIMD float accumulation), then combined pairwise.
 *
 * Argument order follows IPP's conventions, e.g. ippsDiv_32f(a, b, dst, n)
 * computes dst = b / a, and ippsThreshold_LT_32f_I clamps values below the
 * level up to the level.
 */
#ifndef MRL_ORACLE_IPP_SHIM_H
#define MRL_ORACLE_IPP_SHIM_H

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef float Ipp32f;
typedef double Ipp64f;
typedef int IppStatus;
typedef enum { ippAlgHintNone = 0, ippAlgHintFast = 1, ippAlgHintAccurate = 2 } IppHintAlgorithm;

static inline Ipp32f *ippsMalloc_32f(int n) { return (Ipp32f *)malloc(sizeof(Ipp32f) * (size_t)(n > 0 ? n : 1)); }
static inline void ippsFree(void *p) { free(p); }
static inline IppStatus ippsZero_32f(Ipp32f *p, int n) { memset(p, 0, sizeof(Ipp32f) * (size_t)n); return 0; }
static inline IppStatus ippsZero_64f(Ipp64f *p, int n) { for (int i = 0; i < n; ++i) p[i] = 0.0; return 0; }
static inline IppStatus ippsCopy_32f(const Ipp32f *s, Ipp32f *d, int n) { memmove(d, s, sizeof(Ipp32f) * (size_t)n); return 0; }

static inline IppStatus ippsSum_32f(const Ipp32f *s, int n, Ipp32f *sum, IppHintAlgorithm hint) {
    (void)hint;
    Ipp32f lane[16] = {0};
    int i = 0;
    for (; i + 16 <= n; i += 16)
        for (int l = 0; l < 16; ++l) lane[l] += s[i + l];
    for (int l = 0; i < n; ++i, ++l) lane[l] += s[i];
    for (int w = 8; w >= 1; w >>= 1)
        for (int l = 0; l < w; ++l) lane[l] += lane[l + w];
    *sum = lane[0];
    return 0;
}

static inline IppStatus ippsAddC_32f(const Ipp32f *s, Ipp32f v, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = s[i] + v; return 0; }
static inline IppStatus ippsAddC_32f_I(Ipp32f v, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] += v; return 0; }
static inline IppStatus ippsAdd_32f(const Ipp32f *a, const Ipp32f *b, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = a[i] + b[i]; return 0; }
static inline IppStatus ippsAdd_32f_I(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] += s[i]; return 0; }
static inline IppStatus ippsMulC_32f(const Ipp32f *s, Ipp32f v, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = s[i] * v; return 0; }
static inline IppStatus ippsMulC_32f_I(Ipp32f v, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] *= v; return 0; }
static inline IppStatus ippsMul_32f(const Ipp32f *a, const Ipp32f *b, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = a[i] * b[i]; return 0; }
static inline IppStatus ippsMul_32f_I(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] *= s[i]; return 0; }
/* IPP: pDst = pSrc2 / pSrc1 */
static inline IppStatus ippsDiv_32f(const Ipp32f *a, const Ipp32f *b, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = b[i] / a[i]; return 0; }
static inline IppStatus ippsDivC_32f(const Ipp32f *s, Ipp32f v, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = s[i] / v; return 0; }
static inline IppStatus ippsInv_32f_A24(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = 1.0f / s[i]; return 0; }
static inline IppStatus ippsThreshold_LT_32f_I(Ipp32f *d, int n, Ipp32f level) { for (int i = 0; i < n; ++i) if (d[i] < level) d[i] = level; return 0; }
static inline IppStatus ippsExp_32f_I(Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = expf(d[i]); return 0; }
static inline IppStatus ippsArctan_32f(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = atanf(s[i]); return 0; }
static inline IppStatus ippsSqr_32f(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = s[i] * s[i]; return 0; }
static inline IppStatus ippsSqr_32f_I(Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = d[i] * d[i]; return 0; }
static inline IppStatus ippsSqrt_32f(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = sqrtf(s[i]); return 0; }
static inline IppStatus ippsSqrt_32f_I(Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = sqrtf(d[i]); return 0; }
static inline IppStatus ippsSin_32f_A24(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = sinf(s[i]); return 0; }
static inline IppStatus ippsCos_32f_A24(const Ipp32f *s, Ipp32f *d, int n) { for (int i = 0; i < n; ++i) d[i] = cosf(s[i]); return 0; }
static inline IppStatus ippsPolarToCart_32f(const Ipp32f *mag, const Ipp32f *ph, Ipp32f *re, Ipp32f *im, int n) {
    for (int i = 0; i < n; ++i) { re[i] = mag[i] * cosf(ph[i]); im[i] = mag[i] * sinf(ph[i]); }
    return 0;
}
static inline IppStatus ippsCartToPolar_32f(const Ipp32f *re, const Ipp32f *im, Ipp32f *mag, Ipp32f *ph, int n) {
    for (int i = 0; i < n; ++i) { mag[i] = sqrtf(re[i] * re[i] + im[i] * im[i]); ph[i] = atan2f(im[i], re[i]); }
    return 0;
}

#endif
