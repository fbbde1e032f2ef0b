/*
 * mrl_port.c -- CPU oracle for the MRiLab scan engine (TEST INFRASTRUCTURE;
 * see mrl_port.h for what it restates and who may call it).
 */
#include "mrl_port.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* the reference's constant (DoScanAtCPU.cpp:63, DoScanAtGPU.cu:68) */
#define PI 3.14159265359
#define MRL_PORT_MAX_TX 16
#define MRL_PORT_MAX_POOL 16

/* exp(A) - I and phi1(A) = sum_k A^k / (k+1)! of a small n x n matrix
 * (row-major): Taylor series of the matrix scaled by 2^-s to norm <= 1/4,
 * then s squarings by e^{2B} - I = F^2 + 2F, phi1(2B) = phi1(B)(F + 2I)/2. */
static void port_expm1_phi1(int n, const double *A, double *F, double *X) {
    double norm = 0, B[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL], T[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL],
           U[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL];
    for (int i = 0; i < n; ++i) {
        double r = 0;
        for (int j = 0; j < n; ++j) r += fabs(A[i * n + j]);
        if (r > norm) norm = r;
    }
    int s = 0;
    while (norm > 0.25 && s < 60) {
        norm *= 0.5;
        ++s;
    }
    const double scale = ldexp(1.0, -s);
    for (int i = 0; i < n * n; ++i) {
        B[i] = A[i] * scale;
        T[i] = (i % (n + 1) == 0) ? 1.0 : 0.0; /* B^0 / 0! */
        F[i] = 0.0;
        X[i] = T[i];
    }
    for (int k = 1; k <= 24; ++k) { /* T = B^k / k! */
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double acc = 0;
                for (int m = 0; m < n; ++m) acc += T[i * n + m] * B[m * n + j];
                U[i * n + j] = acc / k;
            }
        for (int i = 0; i < n * n; ++i) {
            T[i] = U[i];
            F[i] += T[i];
            X[i] += T[i] / (k + 1);
        }
    }
    for (int q = 0; q < s; ++q) {
        for (int i = 0; i < n; ++i) /* U = X (F + 2I) / 2 */
            for (int j = 0; j < n; ++j) {
                double acc = 0;
                for (int m = 0; m < n; ++m) acc += X[i * n + m] * (F[m * n + j] + (m == j ? 2.0 : 0.0));
                U[i * n + j] = 0.5 * acc;
            }
        for (int i = 0; i < n; ++i) /* T = F F + 2 F */
            for (int j = 0; j < n; ++j) {
                double acc = 0;
                for (int m = 0; m < n; ++m) acc += F[i * n + m] * F[m * n + j];
                T[i * n + j] = acc + 2.0 * F[i * n + j];
            }
        for (int i = 0; i < n * n; ++i) {
            X[i] = U[i];
            F[i] = T[i];
        }
    }
}

#define REAL float
#define RSIN sinf
#define RCOS cosf
#define REXP expf
#define RSQRT sqrtf
#define RATAN atanf
#define RATAN2 atan2f
#define PORT_T(x) f32_##x
#define PORT_FN mrl_port_scan_f32
#include "mrl_port_impl.h"
#undef REAL
#undef RSIN
#undef RCOS
#undef REXP
#undef RSQRT
#undef RATAN
#undef RATAN2
#undef PORT_T
#undef PORT_FN

#define REAL double
#define RSIN sin
#define RCOS cos
#define REXP exp
#define RSQRT sqrt
#define RATAN atan
#define RATAN2 atan2
#define PORT_T(x) f64_##x
#define PORT_FN mrl_port_scan_f64
#include "mrl_port_impl.h"
#undef REAL
#undef PORT_T
#undef PORT_FN
