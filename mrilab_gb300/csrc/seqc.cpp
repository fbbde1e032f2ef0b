// Native sequence compiler: mrl_seq_compile (include/mrl_seq.h).
//
// Host code: the merge is a sort of a few thousand events per TR.  It
// restates the per-TR merge of MRiLab's compiled PSD functions
// (Src/Main/DoWriteXML2m.m:219-333), the TR concatenation with dummy TRs of
// DoPulseGen.m:20-123 and the checks DoMultiTransmitChk.m,
// DoGradChk.m:3-85 and DoUpdRateChk.m:3-56, with MATLAB's semantics where
// results depend on them: sort is stable, unique compares doubles exactly.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/mrl_seq.h"

namespace mrl {
void record_error(const char *msg);

namespace {

struct Lines {
    std::vector<double> rf_amp, rf_phase, rf_freq, rf_coil, gz, gy, gx, adc, ext, uts, ts, flags;
};

// one channel's samples inside the span, sorted by time (stable), times
// taken relative to the span's start
struct Chan {
    std::vector<double> t;
    std::vector<std::vector<double>> v;
};

Chan take(int n, const double *t, std::initializer_list<const double *> vals, double t0, double t1) {
    Chan c;
    c.v.resize(vals.size());
    std::vector<int> keep;
    for (int i = 0; i < n; ++i) {
        const double rel = t[i] - t0;
        if (rel < 0 || rel > t1 - t0) continue;  // DoWriteXML2m.m:219-233
        keep.push_back(i);
    }
    std::vector<double> tt(keep.size());
    for (size_t k = 0; k < keep.size(); ++k) tt[k] = t[keep[k]] - t0;
    std::vector<size_t> ord(keep.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return tt[a] < tt[b]; });
    c.t.resize(ord.size());
    for (size_t k = 0; k < ord.size(); ++k) c.t[k] = tt[ord[k]];
    size_t j = 0;
    for (const double *src : vals) {
        c.v[j].resize(ord.size());
        for (size_t k = 0; k < ord.size(); ++k) c.v[j][k] = src ? src[keep[ord[k]]] : 0.0;
        ++j;
    }
    return c;
}

void append(std::vector<double> &dst, const std::vector<double> &src) { dst.insert(dst.end(), src.begin(), src.end()); }

// the merge of one TR (DoWriteXML2m.m:263-333); false with an error text
bool merge_tr(const mrl_seq_tr &r, Lines &L, std::string &err) {
    const double t0 = r.t_start, t1 = r.t_end;
    Chan rf = take(r.n_rf, r.rf_t, {r.rf_amp, r.rf_phase, r.rf_freq, r.rf_coil}, t0, t1);
    Chan gz = take(r.n_gz, r.gz_t, {r.gz}, t0, t1);
    Chan gy = take(r.n_gy, r.gy_t, {r.gy}, t0, t1);
    Chan gx = take(r.n_gx, r.gx_t, {r.gx}, t0, t1);
    Chan ad = take(r.n_adc, r.adc_t, {r.adc}, t0, t1);
    Chan ex = take(r.n_ext, r.ext_t, {r.ext}, t0, t1);
    const char *names[6] = {"rf", "GzSS", "GyPE", "GxR", "ADC", "Ext"};
    Chan *ch[6] = {&rf, &gz, &gy, &gx, &ad, &ex};
    for (int k = 0; k < 6; ++k)
        if (ch[k]->t.empty()) {
            err = std::string(names[k]) + " sequence line can not be empty!";
            return false;
        }
    // the time line: the span's ends, then every channel's times in channel
    // order, stably sorted; the flag column of each entry follows it
    std::vector<double> ts{0.0, t1 - t0};
    std::vector<int> row{-1, -1};
    for (int k = 0; k < 6; ++k)
        for (double t : ch[k]->t) ts.push_back(t), row.push_back(k);
    std::vector<size_t> ord(ts.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return ts[a] < ts[b]; });
    std::vector<double> uts;
    for (size_t k = 0; k < ord.size(); ++k) {
        const double t = ts[ord[k]];
        L.ts.push_back(t);
        for (int f = 0; f < 6; ++f) L.flags.push_back(row[ord[k]] == f ? 1.0 : 0.0);
        if (uts.empty() || t != uts.back()) uts.push_back(t);
    }
    append(L.uts, uts);
    // first and last value of every channel but rfCoil are zero (:313-333)
    auto ends0 = [](std::vector<double> &v) {
        v.front() = 0.0;
        v.back() = 0.0;
    };
    for (int j = 0; j < 3; ++j) ends0(rf.v[j]);
    for (Chan *c : {&gz, &gy, &gx, &ad, &ex}) ends0(c->v[0]);
    append(L.rf_amp, rf.v[0]);
    append(L.rf_phase, rf.v[1]);
    append(L.rf_freq, rf.v[2]);
    append(L.rf_coil, rf.v[3]);
    append(L.gz, gz.v[0]);
    append(L.gy, gy.v[0]);
    append(L.gx, gx.v[0]);
    append(L.adc, ad.v[0]);
    append(L.ext, ex.v[0]);
    return true;
}

// times of the entries of flag row `row` (tsLine(flagsLine(row, :) ~= 0))
std::vector<double> row_times(const Lines &L, int row) {
    std::vector<double> t;
    for (size_t k = 0; k < L.ts.size(); ++k)
        if (L.flags[k * 6 + row] != 0) t.push_back(L.ts[k]);
    return t;
}

// DoGradChk.m: slew rate diff(G) ./ diff(t) and amplitude, tolerance 0.5 %
bool grad_check(const Lines &L, const mrl_seq_opts &o, std::string &err) {
    const char *names[3] = {"GzSS", "GyP", "GxR"};
    const std::vector<double> *g[3] = {&L.gz, &L.gy, &L.gx};
    for (int a = 0; a < 3; ++a) {
        const std::vector<double> t = row_times(L, 1 + a);
        const std::vector<double> &G = *g[a];
        if (o.max_slew > 0) {
            const double tol = std::fabs(o.max_slew * 0.005);
            for (size_t k = 0; k + 1 < G.size() && k + 1 < t.size(); ++k) {
                const double sr = (G[k + 1] - G[k]) / (t[k + 1] - t[k]);
                if (std::fabs(sr) - o.max_slew > tol) {  // a NaN (0/0) compares false, as in MATLAB
                    err = std::string(names[a]) + " exceeds maximum allowed gradient slew rate!";
                    return false;
                }
            }
        }
        if (o.max_grad > 0) {
            const double tol = std::fabs(o.max_grad * 0.005);
            for (double x : G)
                if (std::fabs(x) - o.max_grad > tol) {
                    err = std::string(names[a]) + " exceeds maximum allowed gradient amplitude!";
                    return false;
                }
        }
    }
    return true;
}

// DoUpdRateChk.m: steps between a line's samples below the minimum update
// rate (tolerance 1 %), steps below half of eps dropped (unique's ties)
bool upd_check(const Lines &L, const mrl_seq_opts &o, std::string &err) {
    const double tol = -std::fabs(o.min_upd_rate * 0.01);
    const double half_eps = 0.5 * 2.220446049250313e-16;
    auto bad = [&](const std::vector<double> &t) {
        for (size_t k = 0; k + 1 < t.size(); ++k) {
            const double dt = t[k + 1] - t[k];
            if (dt < half_eps) continue;
            if (std::fabs(dt) - o.min_upd_rate < tol) return true;
        }
        return false;
    };
    std::vector<double> ids = L.rf_coil;
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    const std::vector<double> trf = row_times(L, 0);
    for (double id : ids) {
        std::vector<double> t;
        for (size_t k = 0; k < trf.size() && k < L.rf_coil.size(); ++k)
            if (L.rf_coil[k] == id) t.push_back(trf[k]);
        if (bad(t)) {
            char buf[96];
            snprintf(buf, sizeof(buf), "rf%g sequence line exceeds minimum update rate!", id);
            err = buf;
            return false;
        }
    }
    const char *names[3] = {"GzSS", "GyP", "GxR"};
    for (int a = 0; a < 3; ++a)
        if (bad(row_times(L, 1 + a))) {
            err = std::string(names[a]) + " sequence line exceeds minimum update rate!";
            return false;
        }
    return true;
}

}  // namespace
}  // namespace mrl

extern "C" int mrl_seq_compile(const mrl_seq_tr *trs, int n_tr, const mrl_seq_opts *opts, mrl_seq_lines *out) {
    using namespace mrl;
    record_error("");
    if (!trs || n_tr < 1 || !out) {
        record_error("NULL argument or no TR");
        return MRL_ERR_ARG;
    }
    const mrl_seq_opts o = opts ? *opts : mrl_seq_opts{};
    Lines L;
    std::string err;
    for (int i = 0; i < n_tr; ++i) {
        if (!merge_tr(trs[i], L, err)) {
            record_error(err.c_str());
            return MRL_ERR_ARG;
        }
        // dummy TRs: every gradient and ADC value so far is zeroed after each
        // of them is appended (DoPulseGen.m:71-87)
        if (i < o.dummy_trs) {
            std::fill(L.gz.begin(), L.gz.end(), 0.0);
            std::fill(L.gy.begin(), L.gy.end(), 0.0);
            std::fill(L.gx.begin(), L.gx.end(), 0.0);
            std::fill(L.adc.begin(), L.adc.end(), 0.0);
        }
    }
    if (!o.multi_transmit) {
        std::fill(L.rf_coil.begin(), L.rf_coil.end(), 1.0);  // DoPulseGen.m:118-123
    } else if (o.tx_coil_num > 0) {
        // DoMultiTransmitChk.m
        double mx = 0;
        bool master = false;
        for (double c : L.rf_coil) mx = std::max(mx, c), master = master || c == (double)o.master_tx_coil;
        if (o.tx_coil_num < mx) {
            record_error("Selected sequence uses more coil elements than current Tx coil can provide.");
            return MRL_ERR_ARG;
        }
        if (!master) {
            record_error("Master Tx coil element must be used.");
            return MRL_ERR_ARG;
        }
    }
    if ((o.max_grad > 0 || o.max_slew > 0) && !grad_check(L, o, err)) {
        record_error(err.c_str());
        return MRL_ERR_ARG;
    }
    if (o.min_upd_rate > 0 && !upd_check(L, o, err)) {
        record_error(err.c_str());
        return MRL_ERR_ARG;
    }
    out->n_rf = (long long)L.rf_amp.size();
    out->n_gz = (long long)L.gz.size();
    out->n_gy = (long long)L.gy.size();
    out->n_gx = (long long)L.gx.size();
    out->n_adc = (long long)L.adc.size();
    out->n_ext = (long long)L.ext.size();
    out->n_uts = (long long)L.uts.size();
    out->n_ts = (long long)L.ts.size();
    const bool fits = out->cap_rf >= out->n_rf && out->cap_gz >= out->n_gz && out->cap_gy >= out->n_gy &&
                      out->cap_gx >= out->n_gx && out->cap_adc >= out->n_adc && out->cap_ext >= out->n_ext &&
                      out->cap_uts >= out->n_uts && out->cap_ts >= out->n_ts;
    if (!fits) {
        record_error("output capacity too small (counts written)");
        return MRL_ERR_ARG;
    }
    auto put = [](double *dst, const std::vector<double> &v) {
        if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(double));
    };
    put(out->rf_amp, L.rf_amp);
    put(out->rf_phase, L.rf_phase);
    put(out->rf_freq, L.rf_freq);
    put(out->rf_coil, L.rf_coil);
    put(out->gz, L.gz);
    put(out->gy, L.gy);
    put(out->gx, L.gx);
    put(out->adc, L.adc);
    put(out->ext, L.ext);
    put(out->uts, L.uts);
    put(out->ts, L.ts);
    put(out->flags, L.flags);
    return MRL_OK;
}
