/*
 * cuh_prelude.h -- lets MRiLab's CUDA kernel headers
 * (Lib/src/engine/GPUEngine/BlochKernel{,ME,MT,CEST,GM}.cuh) compile
 * unmodified as host C (gcc -std=c2x), so their arithmetic can serve as a
 * CPU oracle for the multi-pool models.  Test infrastructure only.
 *
 * - __global__/__shared__ expand to nothing; the kernels' shared-memory
 *   sequence buffer is never used because the driver passes SBufferLen = 0,
 *   which makes each kernel read the step records from global memory.
 * - blockIdx/threadIdx/blockDim are thread-local, so the driver can run one
 *   "CUDA thread" (one x-y column) per OpenMP iteration without races; the
 *   kernels only write per-column slots of their output and scratch arrays.
 * - C promotes the float arguments of sin/cos/exp/pow to double, so this
 *   build evaluates each math call in double precision (the GPU build used
 *   -use_fast_math single-precision intrinsics).
 */
#ifndef MRL_CUH_PRELUDE_H
#define MRL_CUH_PRELUDE_H

#include <math.h>

#define PI 3.14159265359
#define __global__
#define __shared__

typedef struct {
    unsigned x, y, z;
} mrl_dim3_t;

static _Thread_local mrl_dim3_t blockIdx;
static _Thread_local mrl_dim3_t threadIdx;
static _Thread_local mrl_dim3_t blockDim;
static float s_d_Sig[1];

static inline void __syncthreads(void) {}

#endif
