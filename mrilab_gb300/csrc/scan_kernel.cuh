// The scan kernel: discrete Bloch integration of every active isochromat
// over a range of sequence steps, with the receive sum.
//
// Layout and mapping
//   * voxels are compacted to the active ones (n_act); per-voxel data is
//     structure-of-arrays [field][n_act], isochromat state [P][S][n_act];
//   * one thread owns one voxel and NS of its S spins (tpv = S / NS threads
//     per voxel), keeping Mx/My/Mz of all P pools of those spins in
//     registers for the whole launch;
//   * the step records of the launch are staged into shared memory in
//     chunks of kChunk steps by a bulk TMA copy (cp.async.bulk + mbarrier),
//     double-buffered so the copy of chunk k+1 overlaps the work on chunk k;
//   * receive: at an ADC step each thread writes the transverse
//     magnetisation of its spins (summed per sampled pool) to a shared tile
//     of kAdcTile samples; when the tile is full the block contracts it
//     with the coil sensitivities of its voxels (coil x voxel x sample) and
//     writes one partial per (block, sample, pool, coil).  reduce_partials
//     sums the partials over blocks in FP64.
//
// Numerics (this file is the MRL_NUMERICS_REFERENCE integrator, compiled
// without FMA contraction): the reference's single-precision operation
// order -- CPU kernel order for one free pool (BlochKernel.h:38-368), GPU
// kernel formulas for the multi-pool models (BlochKernelME.cuh:225-343,
// BlochKernelMT.cuh:240-411, BlochKernelCEST.cuh:278-606,
// BlochKernelGM.cuh:240-471) -- with sin/cos/exp/atan rounded from double
// so every transcendental is correctly rounded to single precision.
#pragma once

#include "device_util.cuh"

namespace mrl {

constexpr int kBlock = 128;
constexpr int kChunk = 256;
constexpr int kFastChunk = 32;  // steps per staged chunk of the accurate kernel
constexpr int kAdcTile = 16;
constexpr int kMaxPool = 8;
constexpr int kMaxPairs = 64 * kMaxPool;

enum KModel : int { KM_NORMAL = 0, KM_EXCH = 1, KM_MT = 2, KM_CEST = 3 };

struct ScanLaunch {
    int n_act, S, tx, rx, nsamp, npairs, tpv;
    float gyro;
    int rx_default;
    int exch_gm;  // KM_EXCH: 1 = GM channel layout, no self-exchange
    const float *gxg, *gyg, *gzg, *db0;  // [n_act]
    const float *txmg, *txpe;            // [tx][n_act]
    const float2 *rxc;                   // [rx][n_act]
    const float *rho, *t1, *t2;          // [P][n_act]
    const float *kch;                    // [nk][n_act]
    const float *dwrnd;                  // [P][S][n_act]
    float *mx, *my, *mz;                 // [P][S][n_act]
    const float4 *rec;
    int stride4;
    long long s0, s1;
    float2 *partial;  // [(block * a_launch + a) * npairs + pair]
    int a_launch;
    // direct receive (accurate kernel): instead of partials, each block adds
    // its sums, rotated by (cr, sr) = exp(-i rfRef), into the FP64 signal
    // [P][rx][A] at the sample amap[launch-local sample] with atomics
    double *dsx, *dsy;
    const int *amap;
    int A;
    double cr, sr;
    // exact propagator (MRL_NUMERICS_EXACT): per distinct dt (index in the
    // step flags' bits 8 and up) and voxel, xnf coefficients [dt][xnf][n_act]
    const float *xtab;
    int xnf;
    int *err;
    float *hist;            // RunMode 1: [step][Mx|My|Mz][P][S][n_act] from the launch's first step, or null
    long long hist_stride;  // P * S * n_act
    // adjoint checkpoints: at steps flagged kFlagCkpt (every ckpt_every-th
    // step of the scan, a multiple of kAdjWin), the lab-frame state before
    // the step into slot (step / ckpt_every) of
    // [slot][3P: Mx, My, Mz of pool t at 3t + 0, 1, 2][S][n_act];
    // ckpt_step0 = the scan step index of the launch's first step
    float *ckpt;
    long long ckpt_step0;
    int ckpt_every;
    float cs2pi[kMaxPool];  // (float)(2*pi*(float)CS[t])
    int kind[kMaxPool];     // KM_EXCH: 0 free, 1 bound, other values: pool left untouched
};

// ---- correctly rounded single-precision transcendentals ------------------
__device__ __forceinline__ float rsin(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float rcos(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float rexp(float x) { return (float)exp((double)x); }
__device__ __forceinline__ float ratan(float x) { return (float)atan((double)x); }
__device__ __forceinline__ float ratan2(float y, float x) { return (float)atan2((double)y, (double)x); }

constexpr double kPiRef = 3.14159265359;  // the reference's constant

struct StepRF {
    float amp[4], phase[4], freq[4];
};

// RF rotation in the CPU engine's operation order (BlochKernel.h:57-310).
__device__ __forceinline__ void rotate_cpu(float &Mx, float &My, float &Mz, float dW, float dt, int tx,
                                           const StepRF &rf, float gyro, const float *mg, const float *pe) {
    float b1, b2;
    if (tx == 1) {
        b1 = mg[0] * rf.amp[0];
        b2 = pe[0] + rf.phase[0];
        dW = dW + (float)((double)(rf.freq[0] * 2.f) * kPiRef);
        b1 = b1 * gyro;
        b2 = b2 * -1.f;
    } else {
        float b5 = 0.f, b6 = 0.f;
        for (int c = 0; c < tx; ++c) {
            if (rf.amp[c] != 0.f) {
                float a1 = mg[c] * rf.amp[c];
                float a2 = pe[c] + rf.phase[c];
                b5 = b5 + a1 * rcos(a2);
                b6 = b6 + a1 * rsin(a2);
                dW = dW + (float)((double)(rf.freq[c] * 2.f) * kPiRef);
            }
        }
        b1 = __fsqrt_rn(b5 * b5 + b6 * b6);
        b2 = ratan2(b6, b5);
        b1 = b1 * gyro;
        b2 = b2 * -1.f;
    }
    const float beta = ratan(__fdiv_rn(dW, b1));
    float q = dW * dW;
    b1 = b1 * b1;
    q = q + b1;
    q = __fsqrt_rn(q);
    const float alpha = q * dt;
    const float SA = rsin(alpha), SB = rsin(beta), CA = rcos(alpha), CB = rcos(beta);
    const float SP = rsin(b2), mSP = SP * -1.f, CP = rcos(b2), mCP = CP * -1.f;
    float x1, x2, x3, x4, buf;
    x1 = SB * CA; x1 = x1 * mCP; x3 = SA * SP; x1 = x1 + x3; x1 = x1 * SB; x1 = x1 * -1.f;
    x3 = CB * CB; x3 = x3 * CP; x1 = x1 + x3; x3 = x1;
    x1 = x1 * CP; x3 = x3 * SP;
    x2 = SA * SB; x2 = x2 * CP; x4 = CA * SP; x2 = x2 + x4; x4 = x2;
    x2 = x2 * SP; x4 = x4 * mCP;
    x2 = x2 + x1; x2 = x2 * Mx;
    x4 = x4 + x3; x4 = x4 * My; x4 = x4 * -1.f;
    buf = x2 + x4;
    x1 = SB * CB; x1 = x1 * CP;
    x2 = SB * CA; x2 = x2 * mCP;
    x3 = SA * SP;
    x2 = x2 + x3; x2 = x2 * CB;
    x1 = x1 + x2; x1 = x1 * Mz;
    const float nx = buf + x1;
    x1 = CA * SB; x1 = x1 * SP; x3 = SA * CP; x1 = x1 + x3; x1 = x1 * SB;
    x3 = CB * CB; x3 = x3 * SP; x1 = x1 + x3; x3 = x1;
    x1 = x1 * SP; x3 = x3 * CP;
    x2 = SA * SB; x2 = x2 * mSP; x4 = CA * CP; x2 = x2 + x4; x4 = x2;
    x2 = x2 * CP; x4 = x4 * mSP;
    x2 = x2 + x1; x2 = x2 * My;
    x4 = x4 + x3; x4 = x4 * Mx; x4 = x4 * -1.f;
    buf = x2 + x4;
    x1 = CB * SB; x1 = x1 * mSP;
    x2 = CA * SB; x2 = x2 * SP;
    x3 = SA * CP;
    x2 = x2 + x3; x2 = x2 * CB;
    x1 = x1 + x2; x1 = x1 * Mz;
    const float ny = buf + x1;
    x1 = CA * CB; x1 = x1 * SB; x1 = x1 * -1.f;
    x3 = CB * SB; x1 = x1 + x3; x3 = x1;
    x1 = x1 * CP; x3 = x3 * SP;
    x2 = CB * SA; x2 = x2 * mSP;
    x4 = CB * SA; x4 = x4 * CP;
    x2 = x2 + x1; x2 = x2 * Mx;
    x4 = x4 + x3; x4 = x4 * My; x4 = x4 * -1.f;
    buf = x2 + x4;
    x1 = SB * SB;
    x2 = CB * CB; x2 = x2 * CA;
    x1 = x1 + x2; x1 = x1 * Mz;
    const float nz = buf + x1;
    Mx = nx;
    My = ny;
    Mz = nz;
}

// RF rotation / free precession with the GPU kernels' formulas
// (BlochKernel.cuh:189-265).
__device__ __forceinline__ void rotate_gpu(float &Mx, float &My, float &Mz, float dW, float dt, bool rf_on, int tx,
                                           const StepRF &rf, float gyro, const float *mg, const float *pe) {
    if (rf_on) {
        float b1, ph;
        if (tx == 1) {
            dW = dW + (float)(2 * kPiRef * (double)rf.freq[0]);
            b1 = mg[0] * rf.amp[0];
            ph = pe[0] + rf.phase[0];
        } else {
            float re = 0.f, im = 0.f;
            for (int c = 0; c < tx; ++c) {
                if (rf.amp[c] != 0.f) {
                    dW = dW + (float)(2 * kPiRef * (double)rf.freq[c]);
                    float a = mg[c] * rf.amp[c];
                    float p = pe[c] + rf.phase[c];
                    re = re + a * rcos(p);
                    im = im + a * rsin(p);
                }
            }
            b1 = __fsqrt_rn(re * re + im * im);
            ph = ratan2(im, re);
        }
        const float g1 = b1 * gyro;
        const float alpha = __fsqrt_rn(dW * dW + g1 * g1) * dt;
        const float beta = ratan(__fdiv_rn(dW, g1));
        const float sa = rsin(alpha), ca = rcos(alpha);
        const float sb = rsin(beta), cb = rcos(beta);
        const float cp = rcos(-ph), sp = rsin(-ph);
        const float b1x = cb * cb * cp - sb * (sa * sp - ca * cp * sb);
        const float b2x = sp * cb * cb + sb * (cp * sa + ca * sb * sp);
        const float nx = Mx * (cp * b1x + sp * (ca * sp + cp * sa * sb)) - My * (sp * b1x - cp * (ca * sp + cp * sa * sb)) +
                         Mz * (cb * (sa * sp - ca * cp * sb) + cb * cp * sb);
        const float ny = My * (sp * b2x + cp * (ca * cp - sa * sb * sp)) - Mx * (cp * b2x - sp * (ca * cp - sa * sb * sp)) +
                         Mz * (cb * (cp * sa + ca * sb * sp) - cb * sb * sp);
        const float nz = Mx * (cp * (cb * sb - ca * cb * sb) - cb * sa * sp) -
                         My * (sp * (cb * sb - ca * cb * sb) + cb * cp * sa) + Mz * (ca * cb * cb + sb * sb);
        Mx = nx;
        My = ny;
        Mz = nz;
    } else {
        const float a = dW * dt;
        const float s = rsin(a), c = rcos(a);
        const float nx = Mx * c + My * s;
        const float ny = My * c - Mx * s;
        Mx = nx;
        My = ny;
    }
}

// Super-Lorentzian lineshape by the reference's 1000-point rectangle rule
// (BlochKernelMT.cuh:348-358), u advancing in single precision.
static __device__ __noinline__ float lineshape(float rf_freq, float db0, float gyro, float t2b) {
    float u = 0.f, g = 0.f;
    for (int p = 0; p < 1000; ++p) {
        const float den = (float)(3 * (double)u * (double)u - 1);
        const float x = (float)(((2 * kPiRef * (double)rf_freq + (double)(db0 * gyro)) * (double)t2b) / (double)den);
        g = (float)((double)g + sqrt(2 / kPiRef) * (double)__fdiv_rn(t2b, fabsf(den)) * (double)rexp(-2.f * x * x) * 0.001);
        u = (float)((double)u + 0.001);
    }
    return g;
}

// Saturation rate W of a bound pool (BlochKernelMT.cuh:336-399), with the
// lineshape cached per thread while (rf frequency, T2b) stay the same.
struct LineshapeCache {
    float freq = 0.f, t2b = -1.f, g = 0.f;
};

__device__ __forceinline__ float bound_w(LineshapeCache &lc, int tx, const StepRF &rf, const float *mg, float db0,
                                         float gyro, float t2b) {
    if (tx == 1) {
        const float b1 = mg[0] * fabsf(rf.amp[0]);
        if (lc.t2b != t2b || lc.freq != rf.freq[0]) {
            lc.freq = rf.freq[0];
            lc.t2b = t2b;
            lc.g = lineshape(rf.freq[0], db0, gyro, t2b);
        }
        return (float)(kPiRef * (double)((b1 * gyro) * (b1 * gyro)) * (double)lc.g);
    }
    float w = 0.f, n = 0.f;
    for (int c = 0; c < tx; ++c) {
        if (rf.amp[c] != 0.f) {
            const float b1 = mg[c] * fabsf(rf.amp[c]);
            const float g = lineshape(rf.freq[c], db0, gyro, t2b);
            w = w + (float)(kPiRef * (double)((b1 * gyro) * (b1 * gyro)) * (double)g);
            n = n + 1.f;
        }
    }
    return __fdiv_rn(w, n);
}

__device__ __forceinline__ float relax_exp_clamped(float dt, float t) {
    float e = -(dt * __fdiv_rn(1.f, t));
    if (e < -200.f) e = -200.f;
    return rexp(e);
}

template <int MODEL, int P, int NS>
__global__ void __launch_bounds__(kBlock) scan_ref_kernel(ScanLaunch L) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float4 *rbuf = reinterpret_cast<float4 *>(smem + 128);
    const int rstride = L.stride4;
    float2 *mbuf = reinterpret_cast<float2 *>(rbuf + 2 * kChunk * rstride);
    constexpr int kRow = kBlock + 1;  // padded tile row

    const int tid = threadIdx.x;
    const long long gt = (long long)blockIdx.x * kBlock + tid;
    const int v = (int)(gt / L.tpv);
    const int sg = (int)(gt % L.tpv);
    const bool active = v < L.n_act;
    const int n = L.n_act;

    // ---- per-thread constants and state --------------------------------
    float X[NS][P], Y[NS][P], Z[NS][P], dwr[NS][P];
    float rho[P], t1[P], t2[P], rhoS[P];
    unsigned act = 0;
    float gxg = 0.f, gyg = 0.f, gzg = 0.f, db0 = 0.f;
    float mg0[4] = {0.f, 0.f, 0.f, 0.f}, pe0[4] = {0.f, 0.f, 0.f, 0.f};
    constexpr int kNK = MODEL == KM_EXCH ? P * P : (MODEL == KM_MT ? 2 : (MODEL == KM_CEST ? 2 * (P - 1) : 1));
    float kc[kNK];
#pragma unroll
    for (int i = 0; i < kNK; ++i) kc[i] = 0.f;
    if (active) {
        gxg = L.gxg[v];
        gyg = L.gyg[v];
        gzg = L.gzg[v];
        db0 = L.db0[v];
        for (int c = 0; c < L.tx && c < 4; ++c) {
            mg0[c] = L.txmg[(long long)c * n + v];
            pe0[c] = L.txpe[(long long)c * n + v];
        }
#pragma unroll
        for (int t = 0; t < P; ++t) {
            rho[t] = L.rho[(long long)t * n + v];
            t1[t] = L.t1[(long long)t * n + v];
            t2[t] = L.t2[(long long)t * n + v];
            rhoS[t] = __fdiv_rn(rho[t], (float)L.S);
            if (t1[t] != 0.f && t2[t] != 0.f && rho[t] != 0.f) act |= 1u << t;
        }
        if (MODEL == KM_EXCH) {
#pragma unroll
            for (int i = 0; i < kNK; ++i) kc[i] = L.kch[(long long)i * n + v];
        } else if (MODEL == KM_MT) {
            kc[0] = L.kch[1LL * n + v];
            kc[1] = L.kch[2LL * n + v];
        } else if (MODEL == KM_CEST) {
#pragma unroll
            for (int i = 0; i < kNK; ++i) kc[i] = L.kch[(long long)i * n + v];
        }
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const int sp = sg * NS + s;
#pragma unroll
            for (int t = 0; t < P; ++t) {
                const long long i = ((long long)t * L.S + sp) * n + v;
                X[s][t] = L.mx[i];
                Y[s][t] = L.my[i];
                Z[s][t] = L.mz[i];
                dwr[s][t] = L.dwrnd[i];
            }
        }
    } else {
#pragma unroll
        for (int t = 0; t < P; ++t) {
            rho[t] = t1[t] = t2[t] = rhoS[t] = 0.f;
#pragma unroll
            for (int s = 0; s < NS; ++s) X[s][t] = Y[s][t] = Z[s][t] = dwr[s][t] = 0.f;
        }
    }
    const float gyro = L.gyro;
    const float db0g = db0 * gyro;

    // exponentials cached while dt stays the same
    float prev_dt = -1.f;
    float e1[P], e2[P], m0[P], kout[P], fin[P][P];
    float mt_e1k = 0.f, mt_m0 = 0.f, mt_ek = 0.f, mt_e1b = 0.f, mt_m0b = 0.f, mt_ekb = 0.f;
    LineshapeCache lc;

    // ---- staging ---------------------------------------------------------
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nsteps = L.s1 - L.s0;
    const int nchunks = (int)((nsteps + kChunk - 1) / kChunk);
    auto issue = [&](int k) {
        const long long first = L.s0 + (long long)k * kChunk;
        const long long cnt = min((long long)kChunk, L.s1 - first);
        const uint32_t bytes = (uint32_t)(cnt * rstride * 16);
        float4 *dst = rbuf + (k & 1) * kChunk * rstride;
        mbar_expect_tx(&bar[k & 1], bytes);
        bulk_g2s(dst, L.rec + first * rstride, bytes, &bar[k & 1]);
    };
    if (tid == 0 && nchunks > 0) issue(0);

    int a_fill = 0;   // samples in the receive tile
    int a_base = 0;   // launch-relative index of tile row 0
    auto flush = [&]() {
        __syncthreads();
        const int nout = L.npairs * a_fill;
        for (int o = tid; o < nout; o += kBlock) {
            const int pair = o / a_fill;
            const int a = o - pair * a_fill;
            const int t = pair / L.rx;
            const int c = pair - t * L.rx;
            float sx = 0.f, sy = 0.f;
            const float2 *row = mbuf + (a * L.nsamp + t) * kRow;
            const long long vb = (long long)blockIdx.x * kBlock;
            for (int j = 0; j < kBlock; ++j) {
                const long long vj = (vb + j) / L.tpv;
                if (vj >= n) break;
                const float2 m = row[j];
                if (L.rx_default) {
                    sx = sx + m.x;
                    sy = sy + m.y;
                } else {
                    const float2 r = L.rxc[(long long)c * n + vj];
                    sx = sx + (m.x * r.x + m.y * r.y);
                    sy = sy + (-m.x * r.y + m.y * r.x);
                }
            }
            L.partial[((long long)blockIdx.x * L.a_launch + a_base + a) * L.npairs + pair] = make_float2(sx, sy);
        }
        a_base += a_fill;
        a_fill = 0;
        __syncthreads();
    };

    bool ok = true;
    for (int k = 0; k < nchunks && ok; ++k) {
        if (tid == 0 && k + 1 < nchunks) issue(k + 1);
        ok = mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, L.err);
        ok = __syncthreads_and(ok) != 0;  // block-uniform outcome
        if (!ok) {
            // a copy may still be in flight into this block's shared memory:
            // give it another bounded wait before the block exits
            if (tid == 0) mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, L.err);
            break;
        }
        const float4 *cb = rbuf + (k & 1) * kChunk * rstride;
        const int cnt = (int)min((long long)kChunk, nsteps - (long long)k * kChunk);
        for (int q = 0; q < cnt; ++q) {
            const float4 r0 = cb[q * rstride];
            const float4 r1 = cb[q * rstride + 1];
            const float dt = r0.x;
            StepRF rf;
            rf.amp[0] = r1.x;
            rf.phase[0] = r1.y;
            rf.freq[0] = r1.z;
            float rf_sum = fabsf(r1.x);
            for (int c = 1; c < L.tx && c < 4; ++c) {
                const float4 rc = cb[q * rstride + 1 + c];
                rf.amp[c] = rc.x;
                rf.phase[c] = rc.y;
                rf.freq[c] = rc.z;
                rf_sum = rf_sum + fabsf(rc.x);
            }
            const bool rf_on = rf_sum != 0.f;

            if (r1.w == 1.f) {  // receive before the step's rotation
                float2 *tile = mbuf + a_fill * L.nsamp * kRow;
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    if (t >= L.nsamp) break;
                    float sx = 0.f, sy = 0.f;
                    const bool sampled = (MODEL != KM_EXCH) || (L.kind[t] == 0);
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        sx = sx + X[s][t];
                        sy = sy + Y[s][t];
                    }
                    tile[t * kRow + tid] = (active && sampled) ? make_float2(sx, sy) : make_float2(0.f, 0.f);
                }
                if (++a_fill == kAdcTile) flush();
            }
            if (!active) continue;

            const float gzt = r0.y * gyro, gyt = r0.z * gyro, gxt = r0.w * gyro;
            const bool new_dt = dt != prev_dt;
            prev_dt = dt;

            if (MODEL == KM_NORMAL) {
                if (new_dt) {
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        e2[t] = relax_exp_clamped(dt, t2[t]);
                        e1[t] = relax_exp_clamped(dt, t1[t]);
                    }
                }
#pragma unroll
                for (int s = 0; s < NS; ++s) {
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        if (!(act >> t & 1u)) continue;
                        float dW = db0g + dwr[s][t];
                        dW = dW + L.cs2pi[t];
                        dW = dW + gzg * gzt;
                        dW = dW + gyg * gyt;
                        dW = dW + gxg * gxt;
                        float x = X[s][t], y = Y[s][t], z = Z[s][t];
                        if (rf_on)
                            rotate_cpu(x, y, z, dW, dt, L.tx, rf, gyro, mg0, pe0);
                        else
                            rotate_gpu(x, y, z, dW, dt, false, L.tx, rf, gyro, mg0, pe0);
                        X[s][t] = x * e2[t];
                        Y[s][t] = y * e2[t];
                        Z[s][t] = z * e1[t] + (1.f - e1[t]) * rhoS[t];
                    }
                }
            } else if (MODEL == KM_EXCH) {
                if (new_dt) {
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        e1[t] = rexp(__fdiv_rn(-dt, t1[t]));
                        e2[t] = rexp(__fdiv_rn(-dt, t2[t]));
                        m0[t] = __fdiv_rn(rho[t] * (1.f - e1[t]), (float)L.S);
                        float ko = 1.f;
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            fin[t][p] = 0.f;
                            if (L.exch_gm && p == t) continue;
                            const float kgo = L.exch_gm ? kc[p * P + t] : kc[t * P + p];
                            const float kin = L.exch_gm ? kc[t * P + p] : kc[p * P + t];
                            if (kgo != 0.f) ko = ko * rexp(-dt * kgo);
                            if (kin != 0.f) fin[t][p] = 1.f - rexp(-dt * kin);
                        }
                        kout[t] = ko;
                    }
                }
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    float px[P], py[P], pz[P];
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        px[t] = X[s][t];
                        py[t] = Y[s][t];
                        pz[t] = Z[s][t];
                    }
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        if (!(act >> t & 1u)) continue;
                        const int kind = L.kind[t];
                        if (kind != 0 && kind != 1) continue;
                        const bool bound = kind == 1;
                        float x = px[t], y = py[t], z = pz[t];
                        if (!bound) {
                            float dW = db0g + dwr[s][t];
                            dW = dW + L.cs2pi[t];
                            dW = dW + gzg * gzt;
                            dW = dW + gyg * gyt;
                            dW = dW + gxg * gxt;
                            rotate_gpu(x, y, z, dW, dt, rf_on, L.tx, rf, gyro, mg0, pe0);
                        } else if (rf_on) {
                            const float w = bound_w(lc, L.tx, rf, mg0, db0, gyro, t2[t]);
                            z = z * rexp(-w * dt);
                        }
                        float kx = 0.f, ky = 0.f, kz = 0.f;
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            if (fin[t][p] != 0.f) {
                                if (!bound) {
                                    kx = kx + fin[t][p] * px[p];
                                    ky = ky + fin[t][p] * py[p];
                                }
                                kz = kz + fin[t][p] * pz[p];
                            }
                        }
                        if (!bound) {
                            x = x * e2[t];
                            y = y * e2[t];
                            X[s][t] = x * kout[t] + kx;
                            Y[s][t] = y * kout[t] + ky;
                        }
                        z = z * e1[t];
                        Z[s][t] = z * kout[t] + kz + m0[t];
                    }
                }
            } else {  // KM_MT / KM_CEST: pool 0 free water, pool 1 bound
                const float K12 = kc[0];
                const float K21 = MODEL == KM_MT ? kc[1] : kc[P - 1];
                if (new_dt) {
                    e2[0] = rexp(__fdiv_rn(-dt, t2[0]));
                    mt_e1k = rexp(__fdiv_rn(-dt, t1[0]) - dt * K12);
                    mt_m0 = __fdiv_rn(rho[0] * (1.f - rexp(__fdiv_rn(-dt, t1[0]))), (float)L.S);
                    mt_ek = 1.f - rexp(-dt * K21);
                    mt_e1b = rexp(__fdiv_rn(-dt, t1[1]) - dt * K21);
                    mt_m0b = __fdiv_rn(rho[1] * (1.f - rexp(__fdiv_rn(-dt, t1[1]))), (float)L.S);
                    mt_ekb = 1.f - rexp(-dt * K12);
                    if (MODEL == KM_CEST) {
                        float ko = 1.f;
#pragma unroll
                        for (int t = 2; t < P; ++t) {
                            const float kgo = kc[t - 1], kin = kc[t + P - 2];
                            if (kgo != 0.f) ko = ko * rexp(-dt * kgo);
                            fin[0][t] = kin != 0.f ? 1.f - rexp(-dt * kin) : 0.f;
                            // CEST pool t: out to free water, in from free water
                            e2[t] = rexp(__fdiv_rn(-dt, t2[t]));
                            e1[t] = rexp(__fdiv_rn(-dt, t1[t]));
                            m0[t] = __fdiv_rn(rho[t] * (1.f - e1[t]), (float)L.S);
                            kout[t] = kin != 0.f ? rexp(-dt * kin) : 1.f;
                            fin[t][0] = kgo != 0.f ? 1.f - rexp(-dt * kgo) : 0.f;
                        }
                        kout[0] = ko;
                    }
                }
                float w = 0.f;
                if (rf_on) w = bound_w(lc, L.tx, rf, mg0, db0, gyro, t2[1]);
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    float x = X[s][0], y = Y[s][0], z = Z[s][0];
                    const float x0 = x, y0 = y, z0 = z, zb0 = Z[s][1];
                    float dW = db0g + dwr[s][0];
                    dW = dW + L.cs2pi[0];
                    dW = dW + gzg * gzt;
                    dW = dW + gyg * gyt;
                    dW = dW + gxg * gxt;
                    rotate_gpu(x, y, z, dW, dt, rf_on, L.tx, rf, gyro, mg0, pe0);
                    if (MODEL == KM_MT) {
                        x = x * e2[0];
                        y = y * e2[0];
                        z = z * mt_e1k + mt_m0 + zb0 * mt_ek;
                    } else {
                        float kx = 0.f, ky = 0.f, kz = 0.f;
#pragma unroll
                        for (int t = 2; t < P; ++t) {
                            if (fin[0][t] != 0.f) {
                                kx = kx + fin[0][t] * X[s][t];
                                ky = ky + fin[0][t] * Y[s][t];
                                kz = kz + fin[0][t] * Z[s][t];
                            }
                        }
                        x = x * e2[0] * kout[0] + kx;
                        y = y * e2[0] * kout[0] + ky;
                        z = z * mt_e1k * kout[0] + kz + zb0 * mt_ek + mt_m0;
#pragma unroll
                        for (int t = 2; t < P; ++t) {
                            float cx = X[s][t], cy = Y[s][t], cz = Z[s][t];
                            float dWc = db0g + dwr[s][t];
                            dWc = dWc + L.cs2pi[t];
                            dWc = dWc + gzg * gzt;
                            dWc = dWc + gyg * gyt;
                            dWc = dWc + gxg * gxt;
                            rotate_gpu(cx, cy, cz, dWc, dt, rf_on, L.tx, rf, gyro, mg0, pe0);
                            cx = cx * e2[t];
                            cy = cy * e2[t];
                            cz = cz * e1[t];
                            X[s][t] = cx * kout[t] + fin[t][0] * x0;
                            Y[s][t] = cy * kout[t] + fin[t][0] * y0;
                            Z[s][t] = cz * kout[t] + fin[t][0] * z0 + m0[t];
                        }
                    }
                    const float bz = rf_on ? zb0 * rexp(-w * dt) : zb0;
                    Z[s][1] = bz * mt_e1b + mt_m0b + z0 * mt_ekb;
                    X[s][0] = x;
                    Y[s][0] = y;
                    Z[s][0] = z;
                }
            }
        }
        __syncthreads();  // every thread is done with this buffer before it is refilled
    }
    if (a_fill > 0) flush();

    if (active) {
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const int sp = sg * NS + s;
#pragma unroll
            for (int t = 0; t < P; ++t) {
                const long long i = ((long long)t * L.S + sp) * n + v;
                L.mx[i] = X[s][t];
                L.my[i] = Y[s][t];
                L.mz[i] = Z[s][t];
            }
        }
    }
}

}  // namespace mrl
