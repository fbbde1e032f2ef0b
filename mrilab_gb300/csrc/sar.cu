// Local SAR engine: mrl_sar (include/mrl_sar.h).
//
// The reference (Lib/src/engine/CPUEngine/DoCalSARAtCPU.cpp:185-353) walks
// the sequence on the host -- the same equal-time flag merge and rf
// sample-and-hold as the scan engines, TR boundaries at dt < 0, the elapsed
// time written into VSig.Muts -- and at every step with dt > 0 and rf on
// adds, per voxel and E-field component, dt * (sum_c a_c E_c)^2 into
// VVar.SAR with about ten IPP passes over the voxels (SARKernel.h:7-65); at
// every sample time it adds VVar.SAR . ECon into VSig.SAR.
//
// Here the walk stays on the host (it is a scalar loop over the sequence)
// and produces an operation list; the per-voxel work runs in one kernel
// launch, one thread per voxel with its E-field maps in registers:
//   * accurate numerics: the steps between two samples are folded into one
//     symmetric Tx x Tx matrix W = sum_steps dt a a^T (FP64, host), so each
//     segment costs a voxel one quadratic form E^T W E per component,
//     accumulated in FP64; the kernel streams its maps once (HBM bound);
//   * reference numerics: the steps one by one in the reference's single-
//     precision operation order (products rounded, coils summed in order,
//     square, times dt, added), compiled without fused multiply-add.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/mrl_sar.h"

namespace mrl {
void record_error(const char *msg);
void record_timing(const double t[8]);

namespace {

constexpr int kSarMaxTx = 8;
constexpr int kSarBlock = 256;

// Operation list of one call.  Accurate: segment k = W[k] (Tx x Tx, row-
// major) then sample seg_sample[k] (-1: none).  Reference: ops[i] >= 0 is
// the rf step ops[i] (steps[(1 + Tx) * i] = dt, then the Tx amplitudes as
// floats), ops[i] < 0 takes sample -ops[i] - 1.
struct SarOps {
    std::vector<double> W;
    std::vector<int> seg_sample;
    std::vector<float> steps;
    std::vector<int> ops;
    long long rf_steps = 0;
};

// Host walk of the sequence, restating DoCalSARAtCPU.cpp:185-353: the flag
// merge of equal tsLine entries, the sample check before and after every
// step, the time-point update, the rf hold (the smaller-magnitude end of
// the interval of the next entry on the same coil), the packet reset when
// no flag fires, TR boundaries, and the early return once every sample is
// taken.  Writes the VVar cursor, Muts and tRealSample.
void sar_walk(mrl_sar_args &a, SarOps &o) {
    const mrl_sequence &q = a.seq;
    mrl_state &v = a.var;
    const int tx = a.tx_num;
    const int n_ts = q.n_ts, n_uts = q.n_uts, n_rf = q.n_rf;
    int utsi = v.utsi ? *v.utsi : 0, rfi = v.rfi ? *v.rfi : 0, trc = v.tr_count ? *v.tr_count : 0;
    int sari = a.sari ? *a.sari : 0;
    double t = v.t ? *v.t : 0, dt = v.dt ? *v.dt : 0, rf_coil = v.rf_coil ? *v.rf_coil : 0, ext = v.ext ? *v.ext : 0;
    double amp[kSarMaxTx] = {0}, ph[kSarMaxTx] = {0}, fr[kSarMaxTx] = {0};
    for (int c = 0; c < tx; ++c) {
        if (v.rf_amp) amp[c] = v.rf_amp[c];
        if (v.rf_phase) ph[c] = v.rf_phase[c];
        if (v.rf_freq) fr[c] = v.rf_freq[c];
    }
    const bool accurate = a.numerics != MRL_NUMERICS_REFERENCE;
    std::vector<double> w(tx * tx, 0.0);
    bool w_dirty = false;
    auto take_sample = [&]() -> bool {  // false: every sample taken, stop
        if (sari < a.n_sample) {
            if (a.muts[utsi] >= a.t_sample[sari]) {
                if (accurate) {
                    o.W.insert(o.W.end(), w.begin(), w.end());
                    o.seg_sample.push_back(sari);
                    std::fill(w.begin(), w.end(), 0.0);
                    w_dirty = false;
                } else {
                    o.ops.push_back(-sari - 1);
                }
                if (a.t_real_sample) a.t_real_sample[sari] = a.muts[utsi];
                ++sari;
            }
            if (sari == a.n_sample) return false;
        }
        return true;
    };
    int i = 0;
    bool stopped = false;
    while (i < n_ts - 1) {
        double flag[6] = {0, 0, 0, 0, 0, 0};
        auto add = [&](int k) {
            for (int f = 0; f < 6; ++f) flag[f] += q.flags[(long long)k * 6 + f];
        };
        if (q.ts[i] != q.ts[i + 1]) {
            add(i);
            ++i;
        } else {
            add(i);
            while (q.ts[i] == q.ts[i + 1]) {
                add(i + 1);
                ++i;
                if (i == n_ts - 1) break;
            }
            ++i;
        }
        if (!take_sample()) {
            stopped = true;
            break;
        }
        t = q.uts[utsi];
        const int nxt = std::min(utsi + 1, n_uts - 1);
        dt = q.uts[nxt] - q.uts[utsi];
        utsi = nxt;
        if (flag[0] >= 1) {
            for (int j = 0; j < flag[0]; ++j) {
                if (rfi >= n_rf) break;
                rf_coil = q.rf_coil[rfi];
                const int txi = (int)rf_coil;
                for (int s = rfi + 1; s < n_rf; ++s) {
                    if (rf_coil == q.rf_coil[s]) {
                        if (txi >= 1 && txi <= tx) {
                            amp[txi - 1] = std::fabs(q.rf_amp[rfi]) <= std::fabs(q.rf_amp[s]) ? q.rf_amp[rfi] : q.rf_amp[s];
                            ph[txi - 1] = std::fabs(q.rf_phase[rfi]) <= std::fabs(q.rf_phase[s]) ? q.rf_phase[rfi]
                                                                                                : q.rf_phase[s];
                            fr[txi - 1] = std::fabs(q.rf_freq[rfi]) <= std::fabs(q.rf_freq[s]) ? q.rf_freq[rfi] : q.rf_freq[s];
                        }
                        break;
                    }
                }
                ++rfi;
            }
        }
        if (flag[0] + flag[1] + flag[2] + flag[3] + flag[4] + flag[5] == 0) {
            for (int c = 0; c < tx; ++c) amp[c] = ph[c] = fr[c] = 0;
            ext = 0;
        }
        if (dt == 0) continue;
        if (dt < 0) {
            ++trc;
            a.muts[utsi] = a.muts[utsi - 1];
            continue;
        }
        // the power kernel runs only when sum |(float) a_c| != 0 (SARKernel.h:17-23)
        float asum = 0.f;
        for (int c = 0; c < tx; ++c) asum += std::fabs((float)amp[c]);
        if (asum != 0.f) {
            ++o.rf_steps;
            if (accurate) {
                for (int c = 0; c < tx; ++c)
                    for (int d = 0; d < tx; ++d) w[c * tx + d] += dt * amp[c] * amp[d];
                w_dirty = true;
            } else {
                o.ops.push_back((int)(o.steps.size() / (1 + tx)));
                o.steps.push_back((float)dt);
                for (int c = 0; c < tx; ++c) o.steps.push_back((float)amp[c]);
            }
        }
        a.muts[utsi] = a.muts[utsi - 1] + dt;
        if (!take_sample()) {
            stopped = true;
            break;
        }
    }
    (void)stopped;
    if (accurate && w_dirty) {  // steps after the last sample still reach VVar.SAR
        o.W.insert(o.W.end(), w.begin(), w.end());
        o.seg_sample.push_back(-1);
    }
    if (v.t) *v.t = t;
    if (v.dt) *v.dt = dt;
    if (v.rf_coil) *v.rf_coil = rf_coil;
    if (v.ext) *v.ext = ext;
    if (v.utsi) *v.utsi = utsi;
    if (v.rfi) *v.rfi = rfi;
    if (v.tr_count) *v.tr_count = trc;
    if (a.sari) *a.sari = sari;
    for (int c = 0; c < tx; ++c) {
        if (v.rf_amp) v.rf_amp[c] = amp[c];
        if (v.rf_phase) v.rf_phase[c] = ph[c];
        if (v.rf_freq) v.rf_freq[c] = fr[c];
    }
}

// VSig.SAR[s] += acc . ECon, in the reference's order: three rounded
// products, each added with one rounding (DoCalSARAtCPU.cpp:229-237).
__device__ __forceinline__ void sar_sample(float *sar, long long V, long long v, int s, const float acc[3],
                                           const float ec[3]) {
    float o = sar[(long long)s * V + v];
    o = __fadd_rn(o, __fmul_rn(acc[0], ec[0]));
    o = __fadd_rn(o, __fmul_rn(acc[1], ec[1]));
    o = __fadd_rn(o, __fmul_rn(acc[2], ec[2]));
    sar[(long long)s * V + v] = o;
}

// Accurate numerics: per segment acc += E^T W E per component (FP64).
template <int TX>
__global__ void __launch_bounds__(kSarBlock) sar_accurate_kernel(long long V, const float *__restrict__ ex,
                                                                 const float *__restrict__ ey,
                                                                 const float *__restrict__ ez,
                                                                 const float *__restrict__ econ, float *acc_io,
                                                                 float *sar, const double *__restrict__ W,
                                                                 const int *__restrict__ seg_sample, int nseg) {
    const long long v = (long long)blockIdx.x * kSarBlock + threadIdx.x;
    if (v >= V) return;
    float E[3][TX];
#pragma unroll
    for (int c = 0; c < TX; ++c) {
        E[0][c] = ex[(long long)c * V + v];
        E[1][c] = ey[(long long)c * V + v];
        E[2][c] = ez[(long long)c * V + v];
    }
    double acc[3];
    float ec[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        acc[k] = acc_io[(long long)k * V + v];
        ec[k] = econ[(long long)k * V + v];
    }
    for (int g = 0; g < nseg; ++g) {
        const double *w = W + (long long)g * TX * TX;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double q = 0.0;
#pragma unroll
            for (int c = 0; c < TX; ++c) {
                double u = 0.0;
#pragma unroll
                for (int d = 0; d < TX; ++d) u = fma(__ldg(w + c * TX + d), (double)E[k][d], u);
                q = fma((double)E[k][c], u, q);
            }
            acc[k] += q;
        }
        const int s = __ldg(seg_sample + g);
        if (s >= 0) {
            const float af[3] = {(float)acc[0], (float)acc[1], (float)acc[2]};
            sar_sample(sar, V, v, s, af, ec);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) acc_io[(long long)k * V + v] = (float)acc[k];
}

// Reference numerics: the steps one by one (SARKernel.h:32-56) in FP32 with
// every operation rounded separately.
template <int TX>
__global__ void __launch_bounds__(kSarBlock) sar_reference_kernel(long long V, const float *__restrict__ ex,
                                                                  const float *__restrict__ ey,
                                                                  const float *__restrict__ ez,
                                                                  const float *__restrict__ econ, float *acc_io,
                                                                  float *sar, const float *__restrict__ steps,
                                                                  const int *__restrict__ ops, int nops) {
    const long long v = (long long)blockIdx.x * kSarBlock + threadIdx.x;
    if (v >= V) return;
    float E[3][TX];
#pragma unroll
    for (int c = 0; c < TX; ++c) {
        E[0][c] = ex[(long long)c * V + v];
        E[1][c] = ey[(long long)c * V + v];
        E[2][c] = ez[(long long)c * V + v];
    }
    float acc[3], ec[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        acc[k] = acc_io[(long long)k * V + v];
        ec[k] = econ[(long long)k * V + v];
    }
    for (int i = 0; i < nops; ++i) {
        const int op = __ldg(ops + i);
        if (op < 0) {
            sar_sample(sar, V, v, -op - 1, acc, ec);
            continue;
        }
        const float *st = steps + (long long)op * (1 + TX);
        const float dt = __ldg(st);
        float a[TX];
#pragma unroll
        for (int c = 0; c < TX; ++c) a[c] = __ldg(st + 1 + c);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float b = 0.f;
#pragma unroll
            for (int c = 0; c < TX; ++c)
                if (a[c] != 0.f) b = __fadd_rn(b, __fmul_rn(E[k][c], a[c]));
            acc[k] = __fadd_rn(acc[k], __fmul_rn(__fmul_rn(b, b), dt));
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) acc_io[(long long)k * V + v] = acc[k];
}

template <int TX>
cudaError_t launch_sar(bool accurate, long long V, const float *ex, const float *ey, const float *ez,
                       const float *econ, float *acc, float *sar, const double *W, const int *seg, int nseg,
                       const float *steps, const int *ops, int nops, cudaStream_t st) {
    const unsigned grid = (unsigned)((V + kSarBlock - 1) / kSarBlock);
    if (accurate)
        sar_accurate_kernel<TX><<<grid, kSarBlock, 0, st>>>(V, ex, ey, ez, econ, acc, sar, W, seg, nseg);
    else
        sar_reference_kernel<TX><<<grid, kSarBlock, 0, st>>>(V, ex, ey, ez, econ, acc, sar, steps, ops, nops);
    return cudaGetLastError();
}

using SarLaunch = cudaError_t (*)(bool, long long, const float *, const float *, const float *, const float *, float *,
                                  float *, const double *, const int *, int, const float *, const int *, int,
                                  cudaStream_t);
SarLaunch pick_sar(int tx) {
    switch (tx) {
        case 1: return launch_sar<1>;
        case 2: return launch_sar<2>;
        case 3: return launch_sar<3>;
        case 4: return launch_sar<4>;
        case 5: return launch_sar<5>;
        case 6: return launch_sar<6>;
        case 7: return launch_sar<7>;
        case 8: return launch_sar<8>;
        default: return nullptr;
    }
}

int fail(const char *fmt, const char *what, int rc) {
    char buf[512];
    snprintf(buf, sizeof(buf), fmt, what);
    record_error(buf);
    return rc;
}

}  // namespace
}  // namespace mrl

extern "C" int mrl_sar(mrl_sar_args *a) {
    using namespace mrl;
    const auto t0 = std::chrono::steady_clock::now();
    double tim[8] = {0};
    record_timing(tim);
    record_error("");
    if (!a) return fail("%s", "NULL argument", MRL_ERR_ARG);
    if (a->abi_version != MRL_ABI_VERSION) return fail("%s", "ABI version mismatch", MRL_ERR_ARG);
    const long long V = (long long)a->ny * a->nx * a->nz;
    const int tx = a->tx_num;
    if (a->ny <= 0 || a->nx <= 0 || a->nz <= 0 || tx < 1) return fail("%s", "bad sizes", MRL_ERR_ARG);
    if (tx > kSarMaxTx) return fail("%s", "TxCoilNum > 8 is not supported", MRL_ERR_UNSUPPORTED);
    if (!a->econ || !a->tx_e1x || !a->tx_e1y || !a->tx_e1z || !a->sar_acc || !a->muts || !a->seq.uts ||
        !a->seq.ts || !a->seq.flags || (a->n_sample > 0 && (!a->sar || !a->t_sample)))
        return fail("%s", "missing input array", MRL_ERR_ARG);
    if (a->seq.n_ts < 1 || a->seq.n_uts < 1) return fail("%s", "empty sequence", MRL_ERR_ARG);
    if (a->seq.n_rf > 0 && (!a->seq.rf_amp || !a->seq.rf_phase || !a->seq.rf_freq || !a->seq.rf_coil))
        return fail("%s", "missing rf lines", MRL_ERR_ARG);
    const bool accurate = a->numerics != MRL_NUMERICS_REFERENCE;

    SarOps ops;
    sar_walk(*a, ops);
    const int nseg = (int)ops.seg_sample.size();
    const int nops = (int)ops.ops.size();
    if ((accurate && nseg == 0) || (!accurate && nops == 0)) {  // nothing for the device
        tim[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        record_timing(tim);
        return MRL_OK;
    }

    cudaError_t e = cudaSetDevice(a->gpu_index);
    if (e != cudaSuccess) return fail("cudaSetDevice: %s", cudaGetErrorString(e), MRL_ERR_NO_DEVICE);
    // device buffers: maps, accumulators, the samples this call writes, the op list
    int s_lo = a->n_sample, s_hi = -1;
    if (accurate) {
        for (int s : ops.seg_sample)
            if (s >= 0) s_lo = std::min(s_lo, s), s_hi = std::max(s_hi, s);
    } else {
        for (int o : ops.ops)
            if (o < 0) s_lo = std::min(s_lo, -o - 1), s_hi = std::max(s_hi, -o - 1);
    }
    const int ns = s_hi >= s_lo ? s_hi - s_lo + 1 : 0;
    const size_t map_b = (size_t)V * 4;
    size_t bytes = map_b * (3 * (size_t)tx + 3 + 3 + ns);
    size_t opb = accurate ? ops.W.size() * 8 + (size_t)nseg * 4 : ops.steps.size() * 4 + (size_t)nops * 4;
    unsigned char *dbuf = nullptr;
    if ((e = cudaMalloc(&dbuf, bytes + opb + 256)) != cudaSuccess)
        return fail("cudaMalloc: %s", cudaGetErrorString(e), MRL_ERR_NOMEM);
    float *d_ex = reinterpret_cast<float *>(dbuf), *d_ey = d_ex + (size_t)tx * V, *d_ez = d_ey + (size_t)tx * V;
    float *d_ec = d_ez + (size_t)tx * V, *d_acc = d_ec + 3 * V, *d_sar = d_acc + 3 * V;
    unsigned char *d_op = dbuf + (bytes + 255) / 256 * 256;
    cudaStream_t st = nullptr;
    cudaEvent_t k0 = nullptr, k1 = nullptr;
    int rc = MRL_OK;
    auto h2d = [&](void *d, const void *h, size_t n) {
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(d, h, n, cudaMemcpyHostToDevice, st);
        tim[6] += (double)n;
    };
    // the samples this call writes are accumulated (+=) into VSig.SAR; a row
    // that repeats (an earlier call's sample) is uploaded too
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&k0);
    if (e == cudaSuccess) e = cudaEventCreate(&k1);
    h2d(d_ex, a->tx_e1x, (size_t)tx * map_b);
    h2d(d_ey, a->tx_e1y, (size_t)tx * map_b);
    h2d(d_ez, a->tx_e1z, (size_t)tx * map_b);
    h2d(d_ec, a->econ, 3 * map_b);
    h2d(d_acc, a->sar_acc, 3 * map_b);
    if (ns) h2d(d_sar, a->sar + (size_t)s_lo * V, (size_t)ns * map_b);
    // sample indices relative to the uploaded rows
    if (accurate) {
        for (int &s : ops.seg_sample)
            if (s >= 0) s -= s_lo;
        h2d(d_op, ops.W.data(), ops.W.size() * 8);
        h2d(d_op + ops.W.size() * 8, ops.seg_sample.data(), (size_t)nseg * 4);
    } else {
        for (int &o : ops.ops)
            if (o < 0) o = -((-o - 1) - s_lo) - 1;
        h2d(d_op, ops.steps.data(), ops.steps.size() * 4);
        h2d(d_op + ops.steps.size() * 4, ops.ops.data(), (size_t)nops * 4);
    }
    if (e == cudaSuccess) e = cudaEventRecord(k0, st);
    if (e == cudaSuccess) {
        const double *W = reinterpret_cast<const double *>(d_op);
        const int *seg = reinterpret_cast<const int *>(d_op + ops.W.size() * 8);
        const float *stp = reinterpret_cast<const float *>(d_op);
        const int *opl = reinterpret_cast<const int *>(d_op + ops.steps.size() * 4);
        e = pick_sar(tx)(accurate, V, d_ex, d_ey, d_ez, d_ec, d_acc, d_sar, W, seg, nseg, stp, opl, nops, st);
        tim[5] = 1;
    }
    if (e == cudaSuccess) e = cudaEventRecord(k1, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a->sar_acc, d_acc, 3 * map_b, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && ns)
        e = cudaMemcpyAsync(a->sar + (size_t)s_lo * V, d_sar, (size_t)ns * map_b, cudaMemcpyDeviceToHost, st);
    tim[7] = (double)(3 + ns) * map_b;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, k0, k1);
        tim[1] = ms;
    } else {
        rc = fail("SAR engine: %s", cudaGetErrorString(e), MRL_ERR_CUDA);
    }
    if (k0) cudaEventDestroy(k0);
    if (k1) cudaEventDestroy(k1);
    if (st) cudaStreamDestroy(st);
    cudaFree(dbuf);
    tim[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    record_timing(tim);
    return rc;
}
