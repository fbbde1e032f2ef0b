/*
 * mrl_sar.h -- C ABI of the GB300 local-SAR engine (libmrl_scan.so).
 *
 * Replaces the reference's SAR engine DoCalSARAtCPU
 * (Lib/src/engine/CPUEngine/DoCalSARAtCPU.cpp:85-357, power kernel
 * SARKernel.h:7-65), which the SAR watcher calls as a bare MATLAB command
 * (Src/Main/DoSARWatchExec.m:105) and which reads and mutates the globals
 * VObj, VCoi, VCtl, VSeq, VVar and VSig in place.  Here the same arrays are
 * passed explicitly as plain pointers in MATLAB's column-major layout.
 *
 * What it computes (per voxel v of the E-field maps, per component
 * x, y, z): at every decoded step with dt > 0 and rf on,
 *     acc_xyz(v) += dt * (sum_c rfAmp_c TxE1xyz_c(v))^2
 * (the rf amplitudes as held by the decoder, signed, summed over the Tx
 * coils), and at every sample time tSample[k] reached,
 *     SAR[k](v) += acc_x ECon_x + acc_y ECon_y + acc_z ECon_z,
 *     tRealSample[k] = the time reached.
 * The run stops once every sample is taken, as the reference does.
 *
 * Layouts (V = ny*nx*nz voxels, Tx coils, n_sample samples):
 *   econ                [3][V]           VObj.ECon
 *   tx_e1x/y/z          [Tx][V]          VCoi.TxE1x/y/z
 *   sar_acc             [3][V]           VVar.SAR, updated in place
 *   sar                 [n_sample][V]    VSig.SAR, accumulated (+=)
 *   muts                [n_uts]          VSig.Muts, written
 *   t_sample            [n_sample]       VSig.tSample
 *   t_real_sample       [n_sample]       VSig.tRealSample, written
 */
#ifndef MRL_SAR_H
#define MRL_SAR_H

#include "mrl_scan.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int abi_version;            /* MRL_ABI_VERSION */
    int ny, nx, nz;             /* dimensions of VObj.MassDen */
    const float *econ;          /* [3][V] */
    int tx_num;                 /* VCoi.TxCoilNum (<= 8) */
    const float *tx_e1x, *tx_e1y, *tx_e1z; /* [Tx][V] */
    int tr_num;                 /* VCtl.TRNum */
    int gpu_index;              /* device */
    /* MRL_NUMERICS_ACCURATE: the steps between two samples are folded into
     *   one Tx x Tx matrix of sum dt a_c a_c' in FP64, applied per voxel in
     *   FP64 (the per-voxel sum of squares is a quadratic form of the E maps);
     * MRL_NUMERICS_REFERENCE: the reference's single-precision operation
     *   order, step by step (SARKernel.h:17-56), for bit-level parity. */
    int numerics;
    mrl_sequence seq;           /* VSeq: uts, ts, rf lines, ext, flags (gradient / ADC lines unused) */
    mrl_state var;              /* VVar cursor: t, dt, rf_amp/phase/freq/coil, ext, utsi, rfi, exti, tr_count */
    float *sar_acc;             /* VVar.SAR [3][V] */
    int *sari;                  /* VVar.SARi */
    float *sar;                 /* VSig.SAR [n_sample][V] */
    double *muts;               /* VSig.Muts [n_uts] */
    const double *t_sample;     /* VSig.tSample [n_sample] */
    double *t_real_sample;      /* VSig.tRealSample [n_sample] */
    int n_sample;
} mrl_sar_args;

/* Run the SAR accumulation.  Replaces the body of DoCalSARAtCPU's
 * `void mexFunction(int, mxArray*[], int, const mxArray*[])`
 * (DoCalSARAtCPU.cpp:85).  Returns an mrl_status; mrl_last_timing gives
 * [0] the whole call, [1] the device time of the SAR kernel (ms),
 * [5] kernel launches, [6] / [7] bytes copied to / from the device. */
int mrl_sar(mrl_sar_args *args);

#ifdef __cplusplus
}
#endif
#endif
