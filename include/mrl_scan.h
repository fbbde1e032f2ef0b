/*
 * mrl_scan.h -- C ABI of the GB300 MRiLab scan engine (libmrl_scan.so).
 *
 * The engine replaces the discrete Bloch integration behind MRiLab's mex
 * engines.  Those engines take no arguments and read/mutate the MATLAB
 * globals VObj, VMag, VCoi, VCtl, VSeq, VVar and VSig in place
 * (Lib/src/engine/GPUEngine/DoScanAtGPU.cu:76-214); this ABI passes the same
 * arrays explicitly, as plain pointers in MATLAB's column-major layout, so a
 * thin mex layer (mrilab_gb300/csrc/mex_wrappers.cpp) or any FFI can bind it.
 * No type here depends on MATLAB, CUDA or PyTorch.
 *
 * Layouts (V = ny*nx*nz voxels, S spins, P pools, Tx/Rx coils, A samples):
 *   per-voxel maps            [V]           dB0, Gzgrid, Gygrid, Gxgrid
 *   per-pool maps             [P][V]        Rho, T1, T2
 *   isochromat maps           [P][S][V]     Mx, My, Mz, dWRnd
 *   exchange channels         [nK][V]       K (layout depends on the model)
 *   coil maps                 [Tx|Rx][V]    TxCoilmg/pe, RxCoilx/y
 *   signal                    [P][Rx][A]    Sx, Sy (double)
 * with the voxel index v = y + ny*(x + nx*z).
 */
#ifndef MRL_SCAN_H
#define MRL_SCAN_H

#ifdef __cplusplus
extern "C" {
#endif

#define MRL_ABI_VERSION 1

/* Tissue models: one per reference engine. */
typedef enum {
    MRL_MODEL_NORMAL = 0, /* DoScanAtGPU      (BlochKernel.cuh): independent pools */
    MRL_MODEL_ME = 1,     /* DoMEScanAtGPU    (BlochKernelME.cuh): exchanging free pools,
                             K channel t*P+p = rate t->p */
    MRL_MODEL_MT = 2,     /* DoMTScanAtGPU    (BlochKernelMT.cuh): free + bound pool,
                             K channel 1 = K12 (free->bound), 2 = K21 */
    MRL_MODEL_CEST = 3,   /* DoCESTScanAtGPU  (BlochKernelCEST.cuh): free, MT-bound, CEST
                             pools; channel t-1 = free->t, t+P-2 = t->free,
                             0 = free->MT, P-1 = MT->free */
    MRL_MODEL_GM = 4      /* DoGMScanAtGPU    (BlochKernelGM.cuh): TypeFlag 0 free / 1 bound,
                             K channel p*P+t = rate t->p */
} mrl_model;

/* Arithmetic of the integrator. */
typedef enum {
    /* FP32 state and arithmetic; gradient/off-resonance phase carried in
     * FP64 so long trains do not drift; compared with the all-FP64 oracle. */
    MRL_NUMERICS_ACCURATE = 0,
    /* The reference engine's own single-precision operation order
     * (BlochKernel.h for one pool, BlochKernel*.cuh otherwise), evaluated
     * without fused multiply-add and with correctly rounded FP32 math, for
     * bit-level parity studies against the reference CPU engine. */
    MRL_NUMERICS_REFERENCE = 1,
    /* The accurate integrator with the exact relaxation-exchange propagator
     * in place of the reference's first-order split exchange: after each
     * step's rotation, x' = E_T x, y' = E_T y, z' = E_L z + dt phi1(A_L dt) b,
     * E = exp(A dt) of the relaxation-exchange generator, computed in FP64 per
     * voxel and distinct dt.  ME, and GM with free and bound pools (a bound
     * pool is saturated on rf steps before the propagator and has no
     * transverse generator), TypeNum <= 3; MT and CEST (pool 1 bound, the
     * models' K channels and transverse map: no transverse outflow to the
     * bound pool; only pool 0 sampled), CEST with TypeNum <= 5; the normal
     * model runs as MRL_NUMERICS_ACCURATE (its relaxation is exact
     * already).  No reference counterpart. */
    MRL_NUMERICS_EXACT = 2
} mrl_numerics;

typedef enum {
    MRL_OK = 0,
    MRL_ERR_ARG = -1,         /* inconsistent sizes, NULL pointers, bad model */
    MRL_ERR_CUDA = -2,        /* a CUDA call failed (see mrl_last_error) */
    MRL_ERR_NOMEM = -3,       /* device or host allocation failed */
    MRL_ERR_EXT = -4,         /* an Ext plugin callback reported an error */
    MRL_ERR_TIMEOUT = -5,     /* a bounded device wait gave up */
    MRL_ERR_UNSUPPORTED = -6, /* a size the build does not support */
    MRL_ERR_NO_DEVICE = -7    /* no usable CUDA device */
} mrl_status;

/* VObj (Src/Main/DoDataTypeConv.m:34-64) */
typedef struct {
    int ny, nx, nz;      /* spin-matrix rows, columns, slices */
    int spin_num;        /* SpinNum */
    int type_num;        /* TypeNum (pools) */
    double gyro;         /* Gyro, rad/s/T */
    const float *rho, *t1, *t2; /* [P][V] */
    const float *k;      /* [k_channels][V], NULL for MRL_MODEL_NORMAL */
    int k_channels;
    const double *type_flag; /* [P], MRL_MODEL_GM only */
    float *mx, *my, *mz; /* [P][S][V], updated in place */
} mrl_object;

/* VMag */
typedef struct {
    const float *db0;    /* [V], tesla */
    const float *dwrnd;  /* [P][S][V], rad/s */
    const float *gzgrid, *gygrid, *gxgrid; /* [V], metres */
} mrl_field;

/* VCoi */
typedef struct {
    int tx_num, rx_num;
    double tx_default, rx_default; /* nonzero: uniform coil, maps ignored */
    const float *tx_mg, *tx_pe;    /* [Tx][V] */
    const float *rx_x, *rx_y;      /* [Rx][V] */
} mrl_coils;

/* VCtl */
typedef struct {
    const double *cs;    /* [P] chemical shift, Hz */
    int tr_num;
    int run_mode;        /* 0 scan; 1 = per-step history (requires sig.mxs..) */
    int gpu_index;       /* cudaSetDevice index */
    int numerics;        /* mrl_numerics */
} mrl_control;

/* VSeq lines (Src/Main/DoPulseGen.m:43-111) */
typedef struct {
    const double *uts, *ts, *rf_amp, *rf_phase, *rf_freq, *rf_coil;
    const double *gz, *gy, *gx, *adc, *ext;
    const double *flags; /* [len(ts)][6] */
    int n_uts, n_ts, n_rf, n_gz, n_gy, n_gx, n_adc, n_ext;
} mrl_sequence;

/* VVar: the pulse-packet cursor, read at entry and written back at exit
 * and around every Ext callback (DoScanAtGPU.cu:378-477).  Any pointer may
 * be NULL, in which case the engine keeps that field internally. */
typedef struct {
    double *t, *dt, *rf_amp, *rf_phase, *rf_freq, *rf_coil, *rf_ref;
    double *gz, *gy, *gx, *adc, *ext, *kz, *ky, *kx, *gpu_fetch;
    int *utsi, *rfi, *gzi, *gyi, *gxi, *adci, *exti, *tr_count;
} mrl_state;

/* VSig */
typedef struct {
    double *sx, *sy;         /* [P][Rx][A]; each acquired sample is assigned */
    double *kz, *ky, *kx;    /* [A]; accumulated (+=) like the reference */
    int signal_num;          /* A */
    float *mxs, *mys, *mzs;  /* RunMode 1 history [len(uts)][P][S][V], may be NULL */
    double *muts;            /* RunMode 1 step times [len(uts)], may be NULL */
} mrl_signal;

typedef struct {
    int abi_version;         /* MRL_ABI_VERSION */
    int model;               /* mrl_model */
    mrl_object obj;
    mrl_field mag;
    mrl_coils coil;
    mrl_control ctl;
    mrl_sequence seq;
    mrl_state var;
    mrl_signal sig;
} mrl_scan_args;

/* Ext events.  At every Ext sample whose value is nonzero the engine
 * finishes the steps before it, makes Sx/Sy and the VVar cursor current on
 * the host and calls the callback twice, mirroring DoScanAtGPU.cu:565-660:
 *   what = MRL_EXT_FETCH : return nonzero to have the magnetisation
 *                          (obj.mx/my/mz) written back to the host before
 *                          the plugin runs and read again after it;
 *   what = MRL_EXT_PLUGIN: run the plugin; return 0 on success.
 * The callback may replace any pointer in *args (MATLAB may reallocate);
 * the engine re-reads them after each call. */
enum { MRL_EXT_FETCH = 1, MRL_EXT_PLUGIN = 2 };
typedef int (*mrl_ext_fn)(void *user, mrl_scan_args *args, int what);

/* Run a scan.  Replaces the integration behind the mex entry points
 * DoScanAtGPU / DoMEScanAtGPU / DoMTScanAtGPU / DoCESTScanAtGPU /
 * DoGMScanAtGPU (each `void mexFunction(int, mxArray*[], int, const
 * mxArray*[])`, e.g. Lib/src/engine/GPUEngine/DoScanAtGPU.cu:76), with the
 * model selected by args->model.  Returns an mrl_status. */
int mrl_scan(mrl_scan_args *args, mrl_ext_fn ext, void *user);

/* Prepared scans.  A plan uploads the active voxels, decodes the whole
 * sequence and sizes every device buffer once; mrl_plan_execute then
 * re-runs the scan from the initial magnetisation entirely on the device
 * (asynchronously on `stream`, a cudaStream_t or NULL for the legacy
 * stream), and mrl_plan_download writes Sx/Sy and the final Mx/My/Mz into
 * the host arrays named by `args`.  Sequences with Ext events need the
 * callback path of mrl_scan and are rejected (MRL_ERR_UNSUPPORTED).  No
 * counterpart in the reference, which re-uploads everything per call
 * (DoScanAtGPU.cu:257-334). */
typedef struct mrl_plan mrl_plan;
int mrl_plan_create(const mrl_scan_args *args, mrl_plan **out);
int mrl_plan_execute(mrl_plan *plan, void *stream);
int mrl_plan_download(mrl_plan *plan, mrl_scan_args *args);
/* Work of one execution: isochromat-pool-steps (active isochromats x pools
 * x dt>0 steps), dt>0 steps, of which rf-on steps, acquired samples, kernel
 * launches. */
int mrl_plan_work(const mrl_plan *plan, long long out[5]);
void mrl_plan_destroy(mrl_plan *plan);

/* Batched scans: many independent scans (phantoms, sequences, coils of any
 * size) prepared together and run together on one GPU.  MRiLab's batch
 * mode calls the engine once per instance (Src/Main/BatchSim.m:160); here
 * the instances' tiles of 128 voxel-threads share one persistent launch
 * per kernel instantiation (tissue model, pools, spins per thread),
 * ordered longest first, and the receive sums of every instance are
 * reduced by one kernel.
 *
 * mrl_batch_create takes n scan descriptions (MRL_NUMERICS_ACCURATE,
 * RunMode 0, no Ext events; host pointers as for mrl_scan), uploads them
 * and decodes every sequence once.  mrl_batch_execute runs every scan from
 * its initial magnetisation, asynchronously on `stream`:
 *   MRL_BATCH_PERSISTENT  the batched form; captured into a CUDA graph on
 *                         its first use and replayed afterwards;
 *   MRL_BATCH_PLAIN       one launch (and one reduction) per instance, in
 *                         turn -- the per-instance form, for comparison.
 * mrl_batch_tune times candidate spins-per-thread and resident-blocks-per-SM
 * settings of every instantiation on a prefix of the steps and keeps the
 * fastest (it changes no result beyond float rounding).
 * mrl_batch_download writes Sx/Sy, Kx/Ky/Kz and the final Mx/My/Mz of
 * instance i into the host arrays named by args[i].
 * mrl_batch_work: [0] isochromat-pool-steps, [1] dt>0 steps, [2] acquired
 * samples, summed over the instances, [3] kernel launches of one batched
 * execution, [4] of one plain execution.
 * mrl_scan_batched: create, execute (batched), download, destroy. */
enum { MRL_BATCH_PERSISTENT = 0, MRL_BATCH_PLAIN = 1 };
typedef struct mrl_batch mrl_batch;
int mrl_batch_create(mrl_scan_args *const *args, int n, mrl_batch **out);
int mrl_batch_tune(mrl_batch *batch, void *stream);
int mrl_batch_execute(mrl_batch *batch, int mode, void *stream);
int mrl_batch_download(mrl_batch *batch, mrl_scan_args *const *args, int n);
int mrl_batch_work(const mrl_batch *batch, long long out[5]);
void mrl_batch_destroy(mrl_batch *batch);
int mrl_scan_batched(mrl_scan_args *const *args, int n);

/* Adjoint scan: the gradient of a loss L of the signal with respect to the
 * tissue parameters, the initial magnetisation and the rf waveform, given
 * dL/dSx and dL/dSy (for example 2 (S - target) for an L2 loss).  The
 * reference has no gradients; this runs the discrete map the integrator
 * applies (rotation, relaxation, split exchange) backwards, with the state
 * checkpointed every few steps and recomputed in between.
 * Scope: the normal, ME, GM, MT and CEST models (GM pools free or bound,
 * MT / CEST pool 1 bound: a bound pool's saturation is differentiated
 * through its lineshape, so g_t2 of a bound pool is dL/dT2b and g_db0
 * includes the lineshape's shift; g_k in each model's own channels), up to
 * 4 Tx coils (one with bound pools), RunMode 0, no Ext events,
 * TypeNum <= 3, up to 32 Rx coils.
 * Host arrays (NULL: not wanted), V voxels, layouts as in mrl_scan_args:
 *   grad_sx, grad_sy  [P][Rx][A]   inputs
 *   g_t1, g_t2, g_rho [P][V]       dL/dT1, dL/dT2, dL/dRho (the recovery
 *                                  term; the initial state's share is in g_mz0)
 *   g_db0             [V]          dL/d dB0
 *   g_k               [nK][V]      dL/dK, the model's exchange channels
 *   g_mx0, g_my0, g_mz0 [P][S][V]  dL/d(initial Mx, My, Mz)
 *   g_rf              [rf_capacity][Tx][2] dL/dRe A, dL/dIm A of every
 *                                  rf-on step in sequence order, per Tx coil
 *                                  (A = rfAmp e^{i rfPhase} of that coil;
 *                                  zero for a coil that is off at the step:
 *                                  it is not part of that step's field)
 *   rf_a              [rf_capacity][Tx][2] Re A, Im A of each of those steps
 *   rf_step_uts       [rf_capacity] the uts index of each of those steps
 *   g_rf_amp_line, g_rf_phase_line [n_rf of the sequence] dL/d VSeq.rfAmpLine
 *                                  and dL/d VSeq.rfPhaseLine: each step holds
 *                                  the smaller-magnitude end of its rf
 *                                  interval (separately for amplitude and
 *                                  phase), so each step's share goes to the
 *                                  entry it held (entries at a tie of
 *                                  magnitudes have a one-sided derivative);
 *                                  each coil's share to its own entries
 * n_rf_steps receives the number of rf-on steps (g_rf, rf_a and rf_step_uts
 * are filled only if they fit rf_capacity). */
typedef struct {
    const double *grad_sx, *grad_sy;
    float *g_t1, *g_t2, *g_rho, *g_db0, *g_k;
    float *g_mx0, *g_my0, *g_mz0;
    double *g_rf, *rf_a;
    int *rf_step_uts;
    int rf_capacity;
    int n_rf_steps;
    double *g_rf_amp_line, *g_rf_phase_line;
} mrl_adjoint_args;
int mrl_adjoint(mrl_scan_args *args, mrl_adjoint_args *adj);

/* Adjoint plans, for fitting loops: the forward scan (the accurate
 * integrator, which writes a lab-frame checkpoint of every isochromat every
 * 16 steps into device memory) and the adjoint kernel's inputs stay on the
 * device between iterations.  mrl_adjoint is create, forward, backward,
 * gradients, destroy.  args must outlive the plan (its host arrays are
 * read at create and written by download).
 *   create     decodes the sequence once, uploads the object and sizes the
 *              checkpoints: one every 16 steps while they fit in half the
 *              free device memory, else one every 16 M steps (M the
 *              smallest power of two that fits) from which backward
 *              rebuilds each segment's 16-step checkpoints (about one more
 *              forward pass of work); environment MRL_ADJ_SEGMENT=M forces
 *              M.  MRL_ERR_NOMEM if even that does not fit; same scope as
 *              mrl_adjoint
 *   forward    runs the scan from the initial magnetisation on `stream`
 *              (NULL: the default stream), writing the checkpoints
 *   download   signal and final magnetisation of the last forward pass
 *              into args' host arrays, like mrl_plan_download
 *   backward   dL/dSx, dL/dSy (host, [P][Rx][A]) of the last forward pass:
 *              enqueues the adjoint kernel on `stream`
 *   gradients  waits for the device and fills adj's outputs (its grad_sx,
 *              grad_sy are not read)
 *   work       out[0..4] as mrl_plan_work, out[5] = rf-on steps
 *   checkpoints out[0] = steps between stored checkpoints, out[1] = steps
 *              between the checkpoints backward walks from (16), out[2] =
 *              device bytes of both */
typedef struct mrl_adjoint_plan mrl_adjoint_plan;
int mrl_adjoint_plan_create(const mrl_scan_args *args, mrl_adjoint_plan **out);
int mrl_adjoint_plan_forward(mrl_adjoint_plan *plan, void *stream);
int mrl_adjoint_plan_download(mrl_adjoint_plan *plan, mrl_scan_args *args);
int mrl_adjoint_plan_backward(mrl_adjoint_plan *plan, const double *grad_sx, const double *grad_sy, void *stream);
int mrl_adjoint_plan_gradients(mrl_adjoint_plan *plan, mrl_adjoint_args *adj);
int mrl_adjoint_plan_work(const mrl_adjoint_plan *plan, long long out[6]);
int mrl_adjoint_plan_checkpoints(const mrl_adjoint_plan *plan, long long out[3]);
void mrl_adjoint_plan_destroy(mrl_adjoint_plan *plan);

/* Scan without allocating device memory.
 *
 * For callers that cannot call cudaMalloc themselves: code running inside a
 * host application or framework that owns the whole device heap and hands
 * out only its own buffers (a MATLAB session passing gpuArray storage, a
 * serving process with a fixed, pre-reserved memory pool), where an
 * allocation behind the host's back would fail or break its accounting.
 * This variant of the accurate scan kernel works entirely in buffers the
 * caller already owns.  It has no counterpart in the reference, whose
 * engines allocate and free every device array per call
 * (DoScanAtGPU.cu:257-334,765-784).
 *
 * Pointers in `args`: obj.rho/t1/t2/k/mx/my/mz, mag.*, coil.tx_mg/tx_pe/
 * rx_x/rx_y and sig.sx/sy are DEVICE pointers in the layouts above
 * (uncompacted); seq.*, ctl.cs, obj.type_flag, var.* and sig.kx/ky/kz are
 * host pointers.  Mx/My/Mz are updated in place and every acquired sample
 * of Sx/Sy is assigned.  `d_steps` is a 16-byte aligned device buffer of
 * `step_bytes` bytes for the decoded step records (16 floats per step;
 * len(uts) * 64 bytes always suffices); MRL_ERR_ARG if it is misaligned or
 * too small.  Work is queued on `stream` (a cudaStream_t, NULL for the
 * legacy stream) and the call returns when it has finished.
 *
 * Its only scratch is one statically allocated device array of 32 MiB
 * (held by every GPU that loads the library until the process exits): a
 * status word, the ADC map of one launch and the receive partial sums of
 * (thread blocks x Rx x pools) per sample.  Objects for which a single
 * sample does not fit are rejected with MRL_ERR_UNSUPPORTED; when all the
 * samples of the scan do not fit at once, the scan runs as several kernel
 * launches that reuse the scratch in turn (mrl_last_timing's [5] gives the
 * count).  The scratch
 * is shared by every call: calls that overlap on the GPU (different
 * streams or threads) race and must be serialised by the caller.  The
 * first call on a device looks up the scratch's device address on that
 * device (cudaGetSymbolAddress); make that first call before any stream
 * capture.  Limits: MRL_NUMERICS_ACCURATE, one Tx coil, no Ext events. */
int mrl_scan_noalloc(mrl_scan_args *args, float *d_steps, size_t step_bytes, void *stream);

/* The decoded step list of args' sequence, host only (no device needed):
 * the dt > 0 steps the integrator takes, in order, 5 + 3 Tx doubles each --
 * dt, Gz, Gy, Gx, ADC sample index (-1: none), then amplitude, phase and
 * frequency of every Tx coil as held by the decoder (DoScanAtGPU.cu:339-477
 * rules).  Ext stops are decoded through without running a plugin; the
 * caller's VVar and VSig are not written.  *n_steps receives the count;
 * MRL_ERR_ARG (with the count) if it exceeds cap. */
int mrl_decode(const mrl_scan_args *args, double *steps, long long cap, long long *n_steps);

/* Human-readable text for a status code (reference: errors were printed
 * with mexPrintf or raised with mexErrMsgTxt, DoScanAtGPU.cu:231-242,566). */
const char *mrl_status_string(int status);

/* Detail of the last failure on the calling thread ("" if none). */
const char *mrl_last_error(void);

/* Timing of the last mrl_scan (or mrl_scan_noalloc: [0] and [5] only) on
 * the calling thread: [0] whole call (ms),
 * [1] device time of the scan kernels (ms), [2] device time of the receive
 * reduction (ms), [3] host-to-device copies (ms), [4] device-to-host copies
 * (ms), [5] kernel launches, [6] bytes copied host-to-device, [7] bytes
 * copied device-to-host.  New in this engine; the reference has no
 * counterpart. */
int mrl_last_timing(double out[8]);

#ifdef __cplusplus
}
#endif
#endif
