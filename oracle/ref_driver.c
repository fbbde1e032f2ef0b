/*
 * ref_driver.c -- drives MRiLab's own CUDA kernels, compiled as host C, on
 * the CPU (TEST INFRASTRUCTURE: builds only where the reference tree is
 * mounted; used to pin the oracle port's multi-pool models).
 *
 * Compiled once per model with -DMRL_REF_MODEL_{normal,me,mt,cest,gm}; the
 * Makefile force-includes shim/cuh_prelude.h and points -I at the
 * reference's GPUEngine directory.  The host loop below restates the
 * reference GPU engines' host code (Lib/src/engine/GPUEngine/
 * DoScanAtGPU.cu:339-477,662-763 for the single-pool engine,
 * DoGMScanAtGPU.cu:420-531 for the multi-pool ones): decode the sequence
 * lines, push one record [dt, (amp, phase, freq) x Tx, Gz, Gy, Gx, ADC] per
 * step, and at every TR boundary run the kernel over all x-y columns and
 * sum the per-column partial signals.  Ext plugins are not supported here.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "port/mrl_port.h"

#if defined(MRL_REF_MODEL_normal)
#include "BlochKernel.cuh"
#define MULTIPOOL 0
#define ENTRY mrl_refkern_run_normal
#elif defined(MRL_REF_MODEL_me)
#include "BlochKernelME.cuh"
#define MULTIPOOL 1
#define ENTRY mrl_refkern_run_me
#elif defined(MRL_REF_MODEL_mt)
#include "BlochKernelMT.cuh"
#define MULTIPOOL 1
#define ENTRY mrl_refkern_run_mt
#elif defined(MRL_REF_MODEL_cest)
#include "BlochKernelCEST.cuh"
#define MULTIPOOL 1
#define ENTRY mrl_refkern_run_cest
#elif defined(MRL_REF_MODEL_gm)
#include "BlochKernelGM.cuh"
#define MULTIPOOL 1
#define ENTRY mrl_refkern_run_gm
#else
#error "define MRL_REF_MODEL_<model>"
#endif

typedef struct {
    float *v;
    long n, cap;
} fvec;

static void push(fvec *f, float x) {
    if (f->n == f->cap) {
        f->cap = f->cap ? 2 * f->cap : 4096;
        f->v = (float *)realloc(f->v, sizeof(float) * f->cap);
    }
    f->v[f->n++] = x;
}

/* Run the reference kernel over every column for the pushed steps, then
 * sum the per-column signal partials into Sx/Sy (DoScanAtGPU.cu:528-563). */
static void flush(const mrl_port_args *a, fvec *sig, int signal_len, int signali, float *dSx, float *dSy,
                  float *buffer, double *typeflag, float *bmx) {
    const int XY = a->ny * a->nx;
    const int P = a->type_num, RX = a->rx_num, TX = a->tx_num;
    const int rec = 5 + 3 * TX;
    const int seqlen = (int)(sig->n / rec);
    if (seqlen == 0) return;
    memset(dSx, 0, sizeof(float) * (size_t)XY * (signal_len > 0 ? signal_len : 1) * P * RX);
    memset(dSy, 0, sizeof(float) * (size_t)XY * (signal_len > 0 ? signal_len : 1) * P * RX);
    (void)typeflag;
    (void)buffer;
    (void)bmx;
#pragma omp parallel for schedule(static)
    for (int tid = 0; tid < XY; ++tid) {
        blockIdx.x = (unsigned)tid;
        blockDim.y = 1;
        threadIdx.y = 0;
#if defined(MRL_REF_MODEL_normal)
        BlochKernelNormalGPU((float)a->gyro, (double *)a->cs, (float *)a->rho, (float *)a->t1, (float *)a->t2, a->mz, a->my,
                             a->mx, (float *)a->db0, (float *)a->dwrnd, (float *)a->gzgrid, (float *)a->gygrid,
                             (float *)a->gxgrid, (float *)a->tx_mg, (float *)a->tx_pe, (float *)a->rx_x, (float *)a->rx_y,
                             sig->v, (float)a->rx_default, (float)a->tx_default, dSx, dSy, (float)a->rf_ref, signal_len,
                             0, a->nx, a->ny, a->nz, a->spin_num, P, TX, RX, seqlen);
#elif defined(MRL_REF_MODEL_me)
        BlochKernelMEGPU((float)a->gyro, (double *)a->cs, (float *)a->rho, (float *)a->t1, (float *)a->t2, (float *)a->k,
                         a->mz, a->my, a->mx, buffer, (float *)a->db0, (float *)a->dwrnd, (float *)a->gzgrid,
                         (float *)a->gygrid, (float *)a->gxgrid, (float *)a->tx_mg, (float *)a->tx_pe, (float *)a->rx_x,
                         (float *)a->rx_y, sig->v, (float)a->rx_default, (float)a->tx_default, dSx, dSy,
                         (float)a->rf_ref, signal_len, 0, 0, 0, bmx, bmx, bmx, a->nx, a->ny, a->nz, a->spin_num, P, TX,
                         RX, seqlen);
#elif defined(MRL_REF_MODEL_mt)
        BlochKernelMTGPU((float)a->gyro, (double *)a->cs, (float *)a->rho, (float *)a->t1, (float *)a->t2, (float *)a->k,
                         a->mz, a->my, a->mx, (float *)a->db0, (float *)a->dwrnd, (float *)a->gzgrid, (float *)a->gygrid,
                         (float *)a->gxgrid, (float *)a->tx_mg, (float *)a->tx_pe, (float *)a->rx_x, (float *)a->rx_y,
                         sig->v, (float)a->rx_default, (float)a->tx_default, dSx, dSy, (float)a->rf_ref, signal_len, 0,
                         0, 0, bmx, bmx, bmx, a->nx, a->ny, a->nz, a->spin_num, P, TX, RX, seqlen);
#elif defined(MRL_REF_MODEL_cest)
        BlochKernelCESTGPU((float)a->gyro, (double *)a->cs, (float *)a->rho, (float *)a->t1, (float *)a->t2,
                           (float *)a->k, a->mz, a->my, a->mx, buffer, (float *)a->db0, (float *)a->dwrnd,
                           (float *)a->gzgrid, (float *)a->gygrid, (float *)a->gxgrid, (float *)a->tx_mg,
                           (float *)a->tx_pe, (float *)a->rx_x, (float *)a->rx_y, sig->v, (float)a->rx_default,
                           (float)a->tx_default, dSx, dSy, (float)a->rf_ref, signal_len, 0, 0, 0, bmx, bmx, bmx, a->nx,
                           a->ny, a->nz, a->spin_num, P, TX, RX, seqlen);
#elif defined(MRL_REF_MODEL_gm)
        BlochKernelGMGPU((float)a->gyro, (double *)a->cs, typeflag, (float *)a->rho, (float *)a->t1, (float *)a->t2,
                         (float *)a->k, a->mz, a->my, a->mx, buffer, (float *)a->db0, (float *)a->dwrnd,
                         (float *)a->gzgrid, (float *)a->gygrid, (float *)a->gxgrid, (float *)a->tx_mg, (float *)a->tx_pe,
                         (float *)a->rx_x, (float *)a->rx_y, sig->v, (float)a->rx_default, (float)a->tx_default, dSx,
                         dSy, (float)a->rf_ref, signal_len, 0, 0, 0, bmx, bmx, bmx, a->nx, a->ny, a->nz, a->spin_num,
                         P, TX, RX, seqlen);
#endif
    }
    const int A = a->signal_num;
    for (int t = 0; t < P; ++t)
        for (int c = 0; c < RX; ++c)
            for (int j = 0; j < signal_len; ++j) {
                const int s = signali - signal_len + j;
                if (s < 0 || s >= A) continue;
                double sx = 0, sy = 0;
                const float *px = dSx + (size_t)t * XY * signal_len * RX + (size_t)c * XY * signal_len + (size_t)j * XY;
                const float *py = dSy + (size_t)t * XY * signal_len * RX + (size_t)c * XY * signal_len + (size_t)j * XY;
                for (int v = 0; v < XY; ++v) {
                    sx += px[v];
                    sy += py[v];
                }
                a->sx[(long)t * RX * A + (long)c * A + s] = sx;
                a->sy[(long)t * RX * A + (long)c * A + s] = sy;
            }
    sig->n = 0;
}

static double hold(const double *line, int n, int idx) {
    int nxt = idx + 1 < n - 1 ? idx + 1 : n - 1;
    if (fabs(line[idx]) <= fabs(line[nxt])) return line[idx];
    return line[idx + 1 < n ? idx + 1 : n - 1];
}

int ENTRY(const mrl_port_args *a) {
    const int TX = a->tx_num, P = a->type_num, RX = a->rx_num;
    const int XY = a->ny * a->nx;
    if (TX > 16) return -1;
    /* the kernels write at most one TR of per-column partials */
    int max_adc_tr = 0;
    {
        int cnt = 0;
        for (int u = 0; u + 1 < a->n_uts; ++u) {
            (void)u;
        }
        for (int i = 0; i < a->n_adc; ++i) cnt += a->adc[i] == 1;
        max_adc_tr = cnt > 0 ? cnt : 1;
    }
    float *dSx = (float *)calloc((size_t)XY * max_adc_tr * P * RX, sizeof(float));
    float *dSy = (float *)calloc((size_t)XY * max_adc_tr * P * RX, sizeof(float));
    float *buffer = (float *)calloc((size_t)XY * P * 6, sizeof(float));
    float bmx[1] = {0};
    double *typeflag = (double *)a->type_flag;
    fvec sig = {0, 0, 0};
    double rfAmp[16] = {0}, rfPhase[16] = {0}, rfFreq[16] = {0};
    double GzAmp = 0, GyAmp = 0, GxAmp = 0, ADC = 0;
    int utsi = 0, rfi = 0, Gzi = 0, Gyi = 0, Gxi = 0, ADCi = 0, signali = 0, signalptr = 0;
    const int MaxStep = a->n_ts;
    int i = 0;
    while (i < MaxStep) {
        double flag[6] = {0};
        if (i + 1 >= MaxStep || a->ts[i] != a->ts[i + 1]) {
            for (int f = 0; f < 6; ++f) flag[f] += a->flags[(long)i * 6 + f];
            i++;
        } else {
            for (int f = 0; f < 6; ++f) flag[f] += a->flags[(long)i * 6 + f];
            while (i + 1 < MaxStep && a->ts[i] == a->ts[i + 1]) {
                for (int f = 0; f < 6; ++f) flag[f] += a->flags[(long)(i + 1) * 6 + f];
                i++;
                if (i == MaxStep - 1) break;
            }
            i++;
        }
        const int cur = utsi < a->n_uts ? utsi : a->n_uts - 1;
        const int nxt = cur + 1 < a->n_uts - 1 ? cur + 1 : a->n_uts - 1;
        const double dt = a->uts[nxt] - a->uts[cur];
        utsi = MULTIPOOL ? utsi + 1 : nxt;
        const int keep = MULTIPOOL || dt > 0;
        if (keep) push(&sig, (float)dt);
        if (flag[0] >= 1) {
            for (int j = 0; j < flag[0]; ++j) {
                double coil = a->rf_coil[rfi];
                int txi = (int)coil;
                for (int s = rfi + 1; s < a->n_rf; ++s) {
                    if (coil == a->rf_coil[s]) {
                        if (txi >= 1 && txi <= TX) {
                            rfAmp[txi - 1] = fabs(a->rf_amp[rfi]) <= fabs(a->rf_amp[s]) ? a->rf_amp[rfi] : a->rf_amp[s];
                            rfPhase[txi - 1] = fabs(a->rf_phase[rfi]) <= fabs(a->rf_phase[s]) ? a->rf_phase[rfi] : a->rf_phase[s];
                            rfFreq[txi - 1] = fabs(a->rf_freq[rfi]) <= fabs(a->rf_freq[s]) ? a->rf_freq[rfi] : a->rf_freq[s];
                        }
                        break;
                    }
                }
                rfi++;
            }
            for (int c = 0; c < TX; ++c)
                if (rfAmp[c] < 0) {
                    rfAmp[c] = fabs(rfAmp[c]);
                    rfPhase[c] = rfPhase[c] + PI;
                }
        }
        if (keep)
            for (int c = 0; c < TX; ++c) {
                push(&sig, (float)rfAmp[c]);
                push(&sig, (float)rfPhase[c]);
                push(&sig, (float)rfFreq[c]);
            }
        if (flag[1] == 1) GzAmp = hold(a->gz, a->n_gz, Gzi++);
        if (keep) push(&sig, (float)GzAmp);
        if (flag[2] == 1) GyAmp = hold(a->gy, a->n_gy, Gyi++);
        if (keep) push(&sig, (float)GyAmp);
        if (flag[3] == 1) GxAmp = hold(a->gx, a->n_gx, Gxi++);
        if (keep) push(&sig, (float)GxAmp);
        ADC = 0;
        if (flag[4] == 1) ADC = a->adc[ADCi++];
        if (keep) push(&sig, (float)ADC);
        if (ADC == 1) signali++;
        if (flag[0] + flag[1] + flag[2] + flag[3] + flag[4] + flag[5] == 0) {
            for (int c = 0; c < TX; ++c) rfAmp[c] = rfPhase[c] = rfFreq[c] = 0;
            GzAmp = GyAmp = GxAmp = 0;
            ADC = 0;
        }
        if (dt <= 0 || i >= MaxStep) {
            flush(a, &sig, signali - signalptr, signali, dSx, dSy, buffer, typeflag, bmx);
            signalptr = signali;
        }
    }
    free(sig.v);
    free(dSx);
    free(dSy);
    free(buffer);
    return 0;
}
