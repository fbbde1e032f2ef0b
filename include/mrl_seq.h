/*
 * mrl_seq.h -- C ABI of the native sequence compiler (libmrl_scan.so): the
 * step that turns a pulse sequence's elements into the VSeq lines the scan
 * engine decodes.
 *
 * Replaces, in MRiLab:
 *   - the per-TR merge that every compiled PSD function ends with
 *     (Src/Main/DoWriteXML2m.m:219-333): clip each channel's samples to the
 *     TR's element span, put the span's two end points and every rf, Gz, Gy,
 *     Gx, ADC and Ext sample time on one stably sorted time line with a
 *     6-row flag column per entry (which channel it belongs to), the unique
 *     times, each channel's values sorted by their own times, and the first
 *     and last value of every channel except rfCoil set to zero;
 *   - the concatenation over TRs (Src/Main/DoPulseGen.m:20-111) with dummy
 *     TRs (VCtl.DP_Flag / DP_Num: their gradients and ADC zeroed), rfCoil
 *     forced to 1 without multi-transmit (:118-123);
 *   - the checks after it: DoMultiTransmitChk.m (coil ids), DoGradChk.m
 *     (gradient amplitude and slew rate, 0.5 % tolerance) and
 *     DoUpdRateChk.m (minimum update rate of every rf coil and gradient
 *     line, 1 % tolerance).
 * The output feeds mrl_scan_args.seq / mrl_decode directly.
 */
#ifndef MRL_SEQ_H
#define MRL_SEQ_H

#include "mrl_scan.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One TR's sequence-element samples, times in seconds (any origin): the
 * elements' span [t_start, t_end] (min and max of the elements' start / end
 * times, SEtAll), and per channel its sample times and values.  Samples
 * outside the span are dropped (the PSD's clip); every channel needs at
 * least one sample inside it. */
typedef struct {
    double t_start, t_end;
    int n_rf;
    const double *rf_t, *rf_amp, *rf_phase, *rf_freq, *rf_coil;
    int n_gz, n_gy, n_gx;
    const double *gz_t, *gz, *gy_t, *gy, *gx_t, *gx;
    int n_adc, n_ext;
    const double *adc_t, *adc, *ext_t, *ext;
} mrl_seq_tr;

typedef struct {
    int multi_transmit;     /* VCtl.MultiTransmit 'on': keep rfCoil and check it */
    int tx_coil_num;        /* VCoi.TxCoilNum (multi-transmit check; 0: no check) */
    int master_tx_coil;     /* VCtl.MasterTxCoil (multi-transmit check) */
    int dummy_trs;          /* VCtl.DP_Num with DP_Flag 'on', else 0: the first TRs are dummies */
    double max_grad;        /* VCtl.MaxGrad (T/m), 0: no check */
    double max_slew;        /* VCtl.MaxSlewRate (T/m/s), 0: no check */
    double min_upd_rate;    /* VCtl.MinUpdRate (s), 0: no check */
} mrl_seq_opts;

/* The VSeq lines.  Counts are written; each array is filled when its
 * capacity (in elements, flags in columns of 6) holds the count.  Returns
 * MRL_OK, MRL_ERR_ARG with the counts when a capacity is too small (call
 * again), or MRL_ERR_ARG when a channel is empty or a check fails
 * (mrl_last_error names it, as the reference's error dialogs do). */
typedef struct {
    double *rf_amp, *rf_phase, *rf_freq, *rf_coil; /* rfAmpLine .. rfCoilLine */
    double *gz, *gy, *gx, *adc, *ext;              /* GzAmpLine .. ExtLine */
    double *uts, *ts;                              /* utsLine, tsLine */
    double *flags;                                 /* flagsLine [n_ts][6] */
    long long cap_rf, cap_gz, cap_gy, cap_gx, cap_adc, cap_ext, cap_uts, cap_ts;
    long long n_rf, n_gz, n_gy, n_gx, n_adc, n_ext, n_uts, n_ts;
} mrl_seq_lines;

int mrl_seq_compile(const mrl_seq_tr *trs, int n_tr, const mrl_seq_opts *opts, mrl_seq_lines *out);

#ifdef __cplusplus
}
#endif
#endif
