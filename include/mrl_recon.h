/*
 * mrl_recon.h -- C ABI of the GB300 image reconstruction (libmrl_scan.so):
 * the step after the scan engine in MRiLab's pipeline.
 *
 * mrl_recon_cart replaces the default Cartesian and EPI reconstructions
 * (Src/Recon/Default/DoCartRecon.m:10-88, DoEPIRecon.m:10-95): the signal
 * of the scan (VSig.Sx/Sy, [ResFreq * E][Lines][Slices][Rx][Pools] column-
 * major) is summed over the pools, split into its E echoes (Cartesian) or
 * sorted into lines with every second echo of the train reversed (EPI),
 * the most positive readout point is dropped, the k-space is optionally
 * zero filled, laid out readout-first or phase-first (the orientation
 * permutes of DoCartRecon.m:45-72), and each coil's volume is transformed
 * by fftshift(ifftn(fftshift(S))) (MATLAB semantics: 1/N normalised;
 * fftshift rolls each dimension by floor(n / 2)).
 *
 * mrl_grid2d replaces the gridding mex DoGridding
 * (Lib/src/recon/DoGridding/DoGridding.cpp:14-124) used by the non-Cartesian
 * reconstruction (Src/Recon/Default/DoNonCartRecon.m): every sample is
 * spread onto a GridSize x GridSize grid with a radial kernel looked up with
 * linear interpolation, weighted by its density compensation factor.
 */
#ifndef MRL_RECON_H
#define MRL_RECON_H

#include "mrl_scan.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int abi_version;           /* MRL_ABI_VERSION */
    const double *sx, *sy;     /* VSig.Sx / VSig.Sy */
    int res_freq;              /* VCtl.ResFreq: readout points per echo (the last is dropped) */
    int lines;                 /* Cartesian: VCtl.ResPhase; EPI: VCtl.EPI_ShotNum */
    int slices;                /* VCtl.SliceNum */
    int rx;                    /* VCoi.RxCoilNum */
    int pools;                 /* VObj.TypeNum */
    int echoes;                /* Cartesian: VCtl.TEPerTR (one image per echo); EPI: 1 */
    int epi_etl;               /* 0: Cartesian; > 0: EPI, VCtl.EPI_ETL echoes per shot */
    int zf_kx, zf_ky, zf_kz;   /* zero filling (VCtl.ZF_Kx, ZF_Ky, the factor of ZF_Kz); 0 0 0: none */
    int readout_first;         /* 1: image dims (readout, phase, slice); 0: (phase, readout, slice) */
    int gpu_index;
    /* outputs, [N0][N1][N2][Rx][E] column-major (N the image dims); any may be NULL */
    double *img_real, *img_imag, *img_mag, *img_phase;
    int out_dims[3];           /* written: N0, N1, N2 */
} mrl_recon_args;

/* Returns an mrl_status.  Needs the zero-filled sizes to be at least the
 * sampled ones, and (as MATLAB's colon ranges need) ZF_Kx - (ResFreq - 1)
 * and ZF_Ky - lines to be even. */
int mrl_recon_cart(mrl_recon_args *a);

/* Gridding (DoGridding.cpp:54-124): kx, ky in [-0.5, 0.5]; sx, sy, dcf per
 * sample; kernel[n_kernel] the lookup table over [0, half_width];
 * half_width in grid samples (VCtl.KernelWidth / 2), normalised by
 * grid_size - 1 as the reference does; gx, gy [grid_size][grid_size]
 * (column-major) receive the gridded data (overwritten).  Host pointers. */
int mrl_grid2d(const double *kx, const double *ky, const double *sx, const double *sy, const double *dcf,
               int n_sample, const double *kernel, int n_kernel, int grid_size, double half_width, double *gx,
               double *gy, int gpu_index);

#ifdef __cplusplus
}
#endif
#endif
