// Sequence decoder (see decode.h).  Restates DoScanAtGPU.cu:339-477 and the
// Ext/TR-boundary bookkeeping around it (:478-481,662-763).
#include "decode.h"

#include <cmath>
#include <cstring>
#include <cstdlib>
#include <algorithm>

namespace mrl {

namespace {
constexpr double kPi = 3.14159265359;  // the reference's constant (DoScanAtGPU.cu:68)

// Smaller-magnitude end of the interval starting at line[idx]
// (DoScanAtGPU.cu:429-455).
inline double hold(const double *line, int n, int idx) {
    int nxt = idx + 1 < n - 1 ? idx + 1 : n - 1;
    if (std::fabs(line[idx]) <= std::fabs(line[nxt])) return line[idx];
    return line[idx + 1 < n ? idx + 1 : n - 1];
}
}  // namespace

void load_state(DecodeState &s, const mrl_state &v, int tx) {
#define LD(f) \
    if (v.f) s.f = *v.f;
    LD(t) LD(dt) LD(rf_coil) LD(rf_ref) LD(gz) LD(gy) LD(gx) LD(adc) LD(ext) LD(kz) LD(ky) LD(kx) LD(gpu_fetch)
    LD(utsi) LD(rfi) LD(gzi) LD(gyi) LD(gxi) LD(adci) LD(exti) LD(tr_count)
#undef LD
    for (int c = 0; c < tx; ++c) {
        if (v.rf_amp) s.rf_amp[c] = v.rf_amp[c];
        if (v.rf_phase) s.rf_phase[c] = v.rf_phase[c];
        if (v.rf_freq) s.rf_freq[c] = v.rf_freq[c];
        s.rf_amp_src[c] = s.rf_phase_src[c] = -1;
    }
}

void store_state(const DecodeState &s, mrl_state &v, int tx) {
#define ST(f) \
    if (v.f) *v.f = s.f;
    ST(t) ST(dt) ST(rf_coil) ST(gz) ST(gy) ST(gx) ST(adc) ST(ext) ST(kz) ST(ky) ST(kx)
    ST(utsi) ST(rfi) ST(gzi) ST(gyi) ST(gxi) ST(adci) ST(exti) ST(tr_count)
#undef ST
    for (int c = 0; c < tx; ++c) {
        if (v.rf_amp) v.rf_amp[c] = s.rf_amp[c];
        if (v.rf_phase) v.rf_phase[c] = s.rf_phase[c];
        if (v.rf_freq) v.rf_freq[c] = s.rf_freq[c];
    }
}

namespace {
// Second half of a time point: Ext cursor, packet reset, TR count.
void finish_time_point(DecodeState &s, int tx, bool ext_flag, double flag_sum, double dt) {
    if (ext_flag) s.exti++;
    if (flag_sum == 0) {  // no channel fired: reset the pulse packet (:463-472)
        for (int c = 0; c < tx; ++c) {
            s.rf_amp[c] = s.rf_phase[c] = s.rf_freq[c] = 0;
            s.rf_amp_src[c] = s.rf_phase_src[c] = -1;
        }
        s.gz = s.gy = s.gx = 0;
        s.adc = 0;
        s.ext = 0;
    }
    if (dt < 0) s.tr_count++;  // TR boundary (:759-762)
}
}  // namespace

void decode_until_ext(DecodeState &s, const mrl_sequence &q, int tx, double gyro, mrl_signal &sig,
                      DecodeChunk &out) {
    const int stride = record_stride_f4(tx) * 4;
    out.records.clear();
    out.steps.clear();
    out.step_adc.clear();
    out.n_steps = 0;
    out.n_rf_steps = 0;
    out.adc_begin = s.signali;
    out.stopped_at_ext = false;
    out.point_uts.clear();
    out.point_step.clear();
    out.point_dt.clear();
    {  // at most one step and one time point per remaining sequence entry:
       // reserving avoids regrowing (and copying) the step list many times
        const size_t left = (size_t)std::max(0, q.n_ts - s.i) + 1;
        out.records.reserve(left * (size_t)stride);
        out.steps.reserve(left);
        out.step_adc.reserve(left);
        out.point_uts.reserve(left);
        out.point_step.reserve(left);
        out.point_dt.reserve(left);
    }
    if (s.pend_active) {
        finish_time_point(s, tx, s.pend_ext, s.pend_flag_sum, s.pend_dt);
        s.pend_active = false;
    }
    const int max_step = q.n_ts;
    while (!s.done) {
        if (s.i >= max_step) {
            s.done = true;
            break;
        }
        double flag[6] = {0, 0, 0, 0, 0, 0};
        auto add_flags = [&](int k) {
            for (int f = 0; f < 6; ++f) flag[f] += q.flags[(long)k * 6 + f];
        };
        // entries with equal times merge (:346-376); the reference reads
        // tsLine[i+1] one past the end at i = MaxStep-1: treated as different
        if (s.i + 1 >= max_step || q.ts[s.i] != q.ts[s.i + 1]) {
            add_flags(s.i);
            s.i++;
        } else {
            add_flags(s.i);
            while (s.i + 1 < max_step && q.ts[s.i] == q.ts[s.i + 1]) {
                add_flags(s.i + 1);
                s.i++;
                if (s.i == max_step - 1) break;
            }
            s.i++;
        }
        const int nu = q.n_uts;
        const int cur = s.utsi < nu ? s.utsi : nu - 1;
        const int nxt = cur + 1 < nu - 1 ? cur + 1 : nu - 1;
        s.t = q.uts[cur];
        s.dt = q.uts[nxt] - q.uts[cur];
        s.utsi = nxt;
        const double dt = s.dt;
        out.point_uts.push_back(cur);
        out.point_step.push_back((int)out.n_steps);
        out.point_dt.push_back(dt);

        if (flag[0] >= 1) {  // rf: one update per merged rf entry (:385-419)
            for (int j = 0; j < flag[0]; ++j) {
                if (s.rfi >= q.n_rf) break;
                s.rf_coil = q.rf_coil[s.rfi];
                int txi = (int)s.rf_coil;
                for (int k = s.rfi + 1; k < q.n_rf; ++k) {
                    if (s.rf_coil == q.rf_coil[k]) {
                        if (txi >= 1 && txi <= tx) {
                            const int a = s.rfi;
                            const int ja = std::fabs(q.rf_amp[a]) <= std::fabs(q.rf_amp[k]) ? a : k;
                            const int jp = std::fabs(q.rf_phase[a]) <= std::fabs(q.rf_phase[k]) ? a : k;
                            s.rf_amp[txi - 1] = q.rf_amp[ja];
                            s.rf_phase[txi - 1] = q.rf_phase[jp];
                            s.rf_amp_src[txi - 1] = ja;
                            s.rf_phase_src[txi - 1] = jp;
                            s.rf_freq[txi - 1] = std::fabs(q.rf_freq[a]) <= std::fabs(q.rf_freq[k]) ? q.rf_freq[a] : q.rf_freq[k];
                        }
                        break;
                    }
                }
                s.rfi++;
            }
            // a negative amplitude becomes a phase shift of pi (:413-418)
            for (int c = 0; c < tx; ++c) {
                if (s.rf_amp[c] < 0) {
                    s.rf_amp[c] = std::fabs(s.rf_amp[c]);
                    s.rf_phase[c] = s.rf_phase[c] + kPi;
                }
            }
        }
        if (flag[1] == 1 && s.gzi < q.n_gz) s.gz = hold(q.gz, q.n_gz, s.gzi++);
        if (flag[2] == 1 && s.gyi < q.n_gy) s.gy = hold(q.gy, q.n_gy, s.gyi++);
        if (flag[3] == 1 && s.gxi < q.n_gx) s.gx = hold(q.gx, q.n_gx, s.gxi++);
        s.adc = 0;
        if (flag[4] == 1 && s.adci < q.n_adc) s.adc = q.adc[s.adci++];

        if (dt > 0) {
            const size_t base = out.records.size();
            out.records.resize(base + stride, 0.f);
            float *r = &out.records[base];
            r[0] = (float)dt;
            r[1] = (float)s.gz;
            r[2] = (float)s.gy;
            r[3] = (float)s.gx;
            r[4] = (float)s.rf_amp[0];
            r[5] = (float)s.rf_phase[0];
            r[6] = (float)s.rf_freq[0];
            r[7] = (float)s.adc;
            for (int c = 1; c < tx; ++c) {
                r[4 + 4 * c + 0] = (float)s.rf_amp[c];
                r[4 + 4 * c + 1] = (float)s.rf_phase[c];
                r[4 + 4 * c + 2] = (float)s.rf_freq[c];
            }
            StepInfo si;
            si.dt = dt;
            si.gz = s.gz;
            si.gy = s.gy;
            si.gx = s.gx;
            for (int c = 0; c < kMaxTx; ++c) {
                si.amp[c] = c < tx ? s.rf_amp[c] : 0.0;
                si.phase[c] = c < tx ? s.rf_phase[c] : 0.0;
                si.freq[c] = c < tx ? s.rf_freq[c] : 0.0;
            }
            si.adc = s.adc == 1 ? s.signali : -1;
            for (int c = 0; c < kMaxTx; ++c) {
                si.amp_src[c] = c < tx ? s.rf_amp_src[c] : -1;
                si.phase_src[c] = c < tx ? s.rf_phase_src[c] : -1;
            }
            out.steps.push_back(si);
            bool rf_on = false;
            for (int c = 0; c < tx; ++c) rf_on |= (float)s.rf_amp[c] != 0.f;
            out.n_rf_steps += rf_on;
            out.step_adc.push_back(s.adc == 1 ? s.signali : -1);
            out.n_steps++;
        }
        if (s.adc == 1) {  // k-space position of the sample (:466-472)
            if (s.signali < sig.signal_num) {
                if (sig.kz) sig.kz[s.signali] += s.kz;
                if (sig.ky) sig.ky[s.signali] += s.ky;
                if (sig.kx) sig.kx[s.signali] += s.kx;
            }
            s.signali++;
        }
        s.kz += s.gz * dt * (gyro / (2 * kPi));
        s.ky += s.gy * dt * (gyro / (2 * kPi));
        s.kx += s.gx * dt * (gyro / (2 * kPi));

        const bool ext_flag = flag[5] == 1;
        const double flag_sum = flag[0] + flag[1] + flag[2] + flag[3] + flag[4] + flag[5];
        if (ext_flag && s.exti < q.n_ext) {
            s.ext = q.ext[s.exti];
            if (s.ext != 0) {  // stop: the engine flushes, then runs the plugin
                s.pend_active = true;
                s.pend_ext = ext_flag;
                s.pend_flag_sum = flag_sum;
                s.pend_dt = dt;
                out.stopped_at_ext = true;
                break;
            }
        }
        finish_time_point(s, tx, ext_flag, flag_sum, dt);
    }
    out.adc_end = s.signali;
}

namespace {
inline void split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}
}  // namespace

void pack_fast_records(const DecodeChunk &ch, int tx, FrameMoments &fm, std::vector<float> &out, int ckpt_every) {
    const int stride = fast_stride_f4(tx) * 4;
    int every = kAnchorEvery;
    if (const char *e = std::getenv("MRL_ANCHOR_EVERY")) every = std::max(1, std::atoi(e));
    out.assign((size_t)ch.n_steps * stride, 0.f);
    for (int64_t q = 0; q < ch.n_steps; ++q) {
        const StepInfo &si = ch.steps[q];
        float *r = &out[(size_t)q * stride];
        bool rf = false;
        double dw_rf = 0;
        for (int c = 0; c < tx; ++c) {
            if ((float)si.amp[c] != 0.f) {
                rf = true;
                dw_rf += 2 * kPi * si.freq[c];
            }
        }
        int flags = 0;
        if (si.adc >= 0) flags |= kFlagAdc;
        if (rf) flags |= kFlagRf;
        const float fdt = (float)si.dt, fgx = (float)si.gx, fgy = (float)si.gy, fgz = (float)si.gz;
        const bool new_dt = fdt != fm.last_dt;
        const bool new_state = new_dt || fgx != fm.last_gx || fgy != fm.last_gy || fgz != fm.last_gz;
        if (new_dt) flags |= kFlagDt;
        if (new_state) flags |= kFlagState;
        if (ckpt_every > 0 && q % ckpt_every == 0) flags |= kFlagCkpt;
        // anchor the frames at every change of (dt, G), at the first step of
        // an rf block and after `every` free steps; within an rf block the
        // frames hold still, so their phasors stay exact without anchors
        if (new_state || (rf && !fm.last_rf) || (!rf && fm.since_anchor >= every)) {
            flags |= kFlagAnchor;
            fm.since_anchor = 0;
        }
        if (!rf) fm.since_anchor++;
        fm.last_rf = rf;
        fm.last_dt = fdt;
        fm.last_gx = fgx;
        fm.last_gy = fgy;
        fm.last_gz = fgz;
        r[0] = (float)si.dt;
        r[1] = (float)si.gz;
        r[2] = (float)si.gy;
        r[3] = (float)si.gx;
        // (steps without rf: no cosine or sine; the kernels read A only on rf steps)
        r[4] = si.amp[0] != 0 ? (float)(si.amp[0] * std::cos(si.phase[0])) : 0.f;
        r[5] = si.amp[0] != 0 ? (float)(si.amp[0] * std::sin(si.phase[0])) : 0.f;
        r[6] = (float)dw_rf;
        std::memcpy(&r[7], &flags, sizeof(int));
        split(fm.t, r[8], r[9]);
        split(fm.kx, r[10], r[11]);
        split(fm.ky, r[12], r[13]);
        split(fm.kz, r[14], r[15]);
        for (int c = 1; c < tx; ++c) {
            r[16 + 4 * (c - 1) + 0] = (float)(si.amp[c] * std::cos(si.phase[c]));
            r[16 + 4 * (c - 1) + 1] = (float)(si.amp[c] * std::sin(si.phase[c]));
            r[16 + 4 * (c - 1) + 2] = (float)si.freq[c];
            r[16 + 4 * (c - 1) + 3] = (float)std::fabs(si.amp[c]);
        }
        if (!rf) {  // the frame advances over steps without rf
            fm.t += si.dt;
            fm.kx += si.gx * si.dt;
            fm.ky += si.gy * si.dt;
            fm.kz += si.gz * si.dt;
        }
    }
}

}  // namespace mrl
