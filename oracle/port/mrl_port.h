/*
 * mrl_port.h -- CPU oracle for the MRiLab scan engine (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference's scan algorithm, used only by the
 * tests, __graft_entry__.smoke() and bench.py's cpu_baseline/reference arm
 * as the reference results and as the timed CPU baseline.  It is never part of the
 * product path.  Each step follows the reference file it cites:
 *
 *   sequence decode          Lib/src/engine/CPUEngine/DoScanAtCPU.cpp:246-420
 *   single pool (normal)     CPUEngine/BlochKernel.h:38-368,
 *                            GPUEngine/BlochKernel.cuh:143-276
 *   multi-pool exchange (me) GPUEngine/BlochKernelME.cuh:154-343
 *   two-pool MT (mt)         GPUEngine/BlochKernelMT.cuh:180-411
 *   CEST (cest)              GPUEngine/BlochKernelCEST.cuh:280-606
 *   generalized model (gm)   GPUEngine/BlochKernelGM.cuh:159-471
 *   receive                  DoScanAtCPU.cpp:445-491
 *
 * It is compiled twice: mrl_port_scan_f32 keeps the reference's single
 * precision state and arithmetic, mrl_port_scan_f64 does everything in
 * double precision (the "all-FP64 oracle").  Signal sums are accumulated in
 * double in both builds.
 */
#ifndef MRL_PORT_H
#define MRL_PORT_H

#ifdef __cplusplus
extern "C" {
#endif

enum { MRL_PORT_NORMAL = 0, MRL_PORT_ME = 1, MRL_PORT_MT = 2, MRL_PORT_CEST = 3, MRL_PORT_GM = 4 };

typedef struct mrl_port_args {
    int model;
    /* spin matrix: rows (y) x cols (x) x slices (z), column-major */
    int ny, nx, nz, spin_num, type_num, tx_num, rx_num;
    double gyro;
    const float *rho, *t1, *t2;     /* [P][V] */
    const float *k;                 /* model-specific exchange channels [nK][V] */
    const double *type_flag;        /* [P], gm only */
    float *mx, *my, *mz;            /* in/out [P][S][V] */
    const float *db0, *gzgrid, *gygrid, *gxgrid; /* [V] */
    const float *dwrnd;             /* [P][S][V] */
    const float *tx_mg, *tx_pe;     /* [Tx][V] */
    const float *rx_x, *rx_y;       /* [Rx][V] */
    double tx_default, rx_default;
    const double *cs;               /* [P] Hz */
    double rf_ref;
    /* VSeq lines */
    const double *uts, *ts, *rf_amp, *rf_phase, *rf_freq, *rf_coil, *gz, *gy, *gx, *adc, *ext, *flags;
    int n_uts, n_ts, n_rf, n_gz, n_gy, n_gx, n_adc, n_ext;
    /* outputs */
    double *sx, *sy;                /* [P][Rx][A], accumulated (+=) */
    double *kx, *ky, *kz;           /* [A], accumulated (+=) */
    int signal_num;
    int threads;                    /* OpenMP threads, <= 0: library default */
    /* stop after this many dt > 0 steps (< 0: whole sequence); used to time
     * a bounded sample of a long scan */
    long long max_steps;
    /* optional Ext callback: called with the state written back to mx/my/mz */
    int (*ext_cb)(void *user, double ext_value);
    void *ext_user;
    /* RunMode 1 (DoScanAtCPU.cpp:431-436,544-552): after every dt > 0 step
     * and at every TR boundary the state is copied into slot utsi of
     * mxs/mys/mzs [len(uts)][P][S][V] and muts[utsi] advances by dt (held
     * at a TR boundary); slot 0 is the caller's */
    int run_mode;
    float *mxs, *mys, *mzs;
    double *muts;
    /* exact relaxation-exchange propagator (ME, and GM with free and bound
     * pools): each step rotates every free pool and saturates every bound
     * one (exp(-W dt) on its z), then applies x' = E_T x, y' = E_T y,
     * z' = E_L z + dt phi1(A_L dt) b with E = exp(A dt) of the relaxation-
     * exchange generator (Bloch-McConnell equations without the rotation);
     * not in the reference, which splits the exchange (first order) */
    int exact;
    /* optional decoded-step capture (the FP64 adjoint's step list): for
     * every dt > 0 step, 10 + 3 (Tx - 1) doubles -- dt, Gz, Gy, Gx, Tx-0
     * amplitude and phase after the negative-amplitude fold, Tx-0
     * frequency, rf_sum, ADC flag, signal index, then amplitude, phase and
     * frequency of every further Tx coil -- up to steps_cap records */
    double *steps_out;
    long long steps_cap;
} mrl_port_args;

/* Returns 0 on success, < 0 on bad arguments.  *steps_done (optional)
 * receives the number of dt > 0 steps integrated. */
int mrl_port_scan_f32(const mrl_port_args *a, long long *steps_done);
int mrl_port_scan_f64(const mrl_port_args *a, long long *steps_done);

#ifdef __cplusplus
}
#endif
#endif
