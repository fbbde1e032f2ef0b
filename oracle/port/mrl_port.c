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
