// Sequence decoder: turns VSeq lines into per-step records for the device.
//
// Restates the host loop of the reference GPU engines
// (Lib/src/engine/GPUEngine/DoScanAtGPU.cu:339-477): entries of tsLine that
// share one time are merged by OR-ing (summing) their channel flags; at each
// unique time the rf / gradient values are updated by sample-and-hold of the
// smaller-magnitude end of the interval; a time point with no flag resets
// the pulse packet to zero; steps with dt > 0 are emitted; dt < 0 marks a TR
// boundary.  The decoder stops at every Ext sample with a nonzero value so
// the engine can run the plugin and then resume with the (possibly edited)
// VVar cursor.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/mrl_scan.h"

namespace mrl {

constexpr int kMaxTx = 8;

// Device step record: float4 {dt, Gz, Gy, Gx}, float4 {amp0, phase0, freq0,
// adc}, then one float4 {amp, phase, freq, 0} per extra Tx coil.
inline int record_stride_f4(int tx_num) { return 2 + (tx_num - 1); }

struct DecodeState {
    // VVar
    double t = 0, dt = 0, rf_coil = 0, rf_ref = 0;
    double rf_amp[kMaxTx] = {0}, rf_phase[kMaxTx] = {0}, rf_freq[kMaxTx] = {0};
    double gz = 0, gy = 0, gx = 0, adc = 0, ext = 0, kz = 0, ky = 0, kx = 0, gpu_fetch = 0;
    // the rfAmpLine / rfPhaseLine entries the held rf values came from (-1:
    // none, the value is a reset or was loaded from VVar)
    int rf_amp_src[kMaxTx] = {-1, -1, -1, -1, -1, -1, -1, -1};
    int rf_phase_src[kMaxTx] = {-1, -1, -1, -1, -1, -1, -1, -1};
    int utsi = 0, rfi = 0, gzi = 0, gyi = 0, gxi = 0, adci = 0, exti = 0, tr_count = 0;
    // decoder position
    int i = 0;        // tsLine cursor
    int signali = 0;  // next ADC sample index
    bool done = false;
    // second half of a time point interrupted by an Ext stop
    bool pend_active = false, pend_ext = false;
    double pend_flag_sum = 0, pend_dt = 0;
};

// One dt > 0 step in double precision, as decoded.
struct StepInfo {
    double dt, gz, gy, gx;
    double amp[kMaxTx], phase[kMaxTx], freq[kMaxTx];
    int adc;  // ADC sample index, or -1
    // per Tx coil: the rfAmpLine / rfPhaseLine entries held (-1: none)
    int amp_src[kMaxTx], phase_src[kMaxTx];
};

struct DecodeChunk {
    std::vector<StepInfo> steps;     // dt > 0 steps
    std::vector<float> records;      // n_steps * stride floats
    std::vector<int> step_adc;       // per step: ADC sample index, or -1
    int64_t n_steps = 0;
    int adc_begin = 0, adc_end = 0;  // sample indices acquired in this chunk
    int n_rf_steps = 0;              // steps with rf on
    bool stopped_at_ext = false;     // true: an Ext callback is due now
    // every time point decoded (RunMode 1 history): its uts index, the
    // number of dt > 0 steps of this chunk before it (the state at that
    // time is the state after those steps) and its dt
    std::vector<int> point_uts, point_step;
    std::vector<double> point_dt;
};

void load_state(DecodeState &s, const mrl_state &v, int tx_num);
void store_state(const DecodeState &s, mrl_state &v, int tx_num);

// Moments of the frame phase, accumulated over steps without rf (the rf
// steps rotate the magnetisation explicitly): elapsed time and gradient
// areas, in double precision, carried across chunks.
struct FrameMoments {
    double t = 0, kx = 0, ky = 0, kz = 0;
    // the previous step's dt and gradients as the kernels see them (float):
    // consecutive dt of a uniform raster differ in the last bits of their
    // double differences, so the change flags compare the float values
    float last_dt = -1.f, last_gx = 0.f, last_gy = 0.f, last_gz = 0.f;
    int since_anchor = 1 << 30;  // free steps since the last anchor
    bool last_rf = false;
};

// Step record of the MRL_NUMERICS_ACCURATE integrator (16 floats + 4 per
// extra Tx coil):
//   {dt, Gz, Gy, Gx}
//   {Re A0, Im A0, 2*pi*sum of rf frequencies of the active coils, flags}
//   {T hi, T lo, Kx hi, Kx lo}      moments at the start of the step
//   {Ky hi, Ky lo, Kz hi, Kz lo}
//   {Re Ac, Im Ac, freq c, |Ac|} for every coil c >= 1
// with Ac = amp_c * exp(i phase_c) the complex rf amplitude, and flag bits
// kFlagAdc, kFlagRf, kFlagAnchor (recompute the frame phasors exactly),
// kFlagState (dt or gradient changed), kFlagDt (dt changed), kFlagCkpt
// (write the lab-frame state before this step to its checkpoint slot).
enum : int { kFlagAdc = 1, kFlagRf = 2, kFlagAnchor = 4, kFlagState = 8, kFlagDt = 16, kFlagCkpt = 32 };
constexpr int kAnchorEvery = 16;
constexpr int kAdjWin = 16;  // steps between adjoint checkpoints (recomputed into shared memory)
inline int fast_stride_f4(int tx_num) { return 4 + (tx_num - 1); }
// ckpt_every > 0 flags every ckpt_every-th step of the chunk with kFlagCkpt
void pack_fast_records(const DecodeChunk &ch, int tx_num, FrameMoments &fm, std::vector<float> &out,
                       int ckpt_every = 0);

// Decode until the next nonzero Ext sample or the end of the sequence.
// K-space positions of acquired samples are accumulated into sig.kx/ky/kz.
void decode_until_ext(DecodeState &s, const mrl_sequence &q, int tx_num, double gyro, mrl_signal &sig,
                      DecodeChunk &out);

}  // namespace mrl
