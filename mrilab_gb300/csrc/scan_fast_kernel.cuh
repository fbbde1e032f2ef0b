// The MRL_NUMERICS_ACCURATE scan kernel: the same sequence model and tissue
// models as scan_ref_kernel (BlochKernel{,ME,MT,CEST,GM}.cuh), integrated
// in single precision in a rotating frame so that it is both faster and
// closer to the exact (FP64) solution than the reference's own FP32 code.
//
// Frame.  Each isochromat-pool keeps its magnetisation in a frame rotating
// with its free precession: m_lab = m_frame * P, P = exp(-i Phi), with
//   Phi = gamma (dB0 T + x Kx + y Ky + z Kz) + w_res T,
// T and K the elapsed time and gradient areas over the steps without rf
// (moments carried on the host in FP64 and passed as hi/lo float pairs),
// and w_res = dWRnd + 2 pi CS the isochromat's residual frequency (hi/lo).
// Free precession therefore never rotates m: only the phasor P advances,
// by a factor (1 + d) with d = exp(-i theta) - 1 evaluated once per change
// of (dt, G); P is recomputed exactly from the moments (double-float
// arithmetic, Cody-Waite reduction) at every change of (dt, G), every rf
// step and at least every kAnchorEvery steps, so its error never
// accumulates.  An rf step rotates m_frame about the effective field with
// the rf azimuth shifted by -Phi (exact identity of the reference's closed
// form, BlochKernel.cuh:241-254).
//
// Coefficients close to 1 are applied in "1 - y" form: relaxation
// exp(-dt/T) = 1 - y with y = -expm1(-dt/T), exchange exp(-k dt) likewise,
// so repeated multiplication does not accumulate the rounding of a stored
// factor.  The receive sum rotates each frame back to the lab with P.
#pragma once

#include "decode.h"
#include "scan_kernel.cuh"

namespace mrl {

struct FastLaunch {
    ScanLaunch b;             // shared fields; b.rec points at fast records
    const float2 *omega;      // [4][n_act] (hi, lo) of gamma*dB0, gamma*x, gamma*y, gamma*z
    const float2 *wres;       // [P][S][n_act] (hi, lo) residual frequency, rad/s
    const float2 *txc;        // [tx][n_act] TxCoilmg * exp(i TxCoilpe)
    // Direct layout (mrl_scan_noalloc): the arrays of ScanLaunch are the
    // caller's uncompacted MATLAB arrays (n = every voxel), and the three
    // derived fields above are computed here instead of being read.
    int direct;
    int all_free;             // KM_EXCH: every pool is free (ME, or GM without bound pools): selects
                              // the FREE instantiation
    const float *rx_x, *rx_y; // [rx][n]
    float gam_hi, gam_lo;     // gyromagnetic ratio split
    float cs_hi[kMaxPool], cs_lo[kMaxPool];  // 2 pi CS[t] split
};

// ---- double-float helpers ------------------------------------------------
struct df {
    float hi, lo;
};

__device__ __forceinline__ df two_prod(float a, float b) {
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

// (a_hi + a_lo) * (b_hi + b_lo), unnormalised
__device__ __forceinline__ df df_mul(float ah, float al, float bh, float bl) {
    df p = two_prod(ah, bh);
    p.lo = fmaf(ah, bl, fmaf(al, bh, p.lo));
    return p;
}

__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return s;
}

// exp(-i phi) for a double-float phase, reduced modulo 2 pi.
__device__ __forceinline__ float2 phasor(df phi) {
    constexpr float kInv2Pi = 0.15915494309189535f;
    constexpr float kC1 = 6.28318548202514648f;     // float(2 pi)
    constexpr float kC2 = -1.7484555314695172e-07f; // 2 pi - kC1
    const float k = rintf(phi.hi * kInv2Pi);
    float r = fmaf(-k, kC1, phi.hi);
    r = fmaf(-k, kC2, r);
    r += phi.lo;
    // |r| <= pi: the MUFU approximation's absolute error (~4e-7) is reset at
    // every anchor, so it does not accumulate
    float s, c;
    __sincosf(r, &s, &c);
    return make_float2(c, -s);
}

// sin and cos of x: Cody-Waite reduction (Cody and Waite, Software Manual
// for the Elementary Functions, 1980) x = k pi/2 + r with pi/2 split in
// three floats and fused multiply-adds, |r| <= pi/4, then the Taylor series
// of sin (to r^11) and cos (to r^12) by Horner's rule; truncation error
// below 1e-11 on |r| <= pi/4.  Small arguments (k = 0) keep full relative
// accuracy.  Meant for |x| well below 2^22 (rotation angles of one step).
__device__ __forceinline__ void sincos_cw(float x, float &sn, float &cs) {
    constexpr float kTwoOverPi = 0.636619746685028076f;
    constexpr float kC1 = 1.57079637050628662f;       // float(pi / 2)
    constexpr float kC2 = -4.37113882867379300e-08f;  // float(pi / 2 - kC1)
    constexpr float kC3 = -1.77635683940025046e-15f;  // pi / 2 - kC1 - kC2
    const float k = rintf(x * kTwoOverPi);
    float r = fmaf(-k, kC1, x);
    r = fmaf(-k, kC2, r);
    r = fmaf(-k, kC3, r);
    const float r2 = r * r;
    float ps = -1.f / 39916800.f;
    ps = fmaf(ps, r2, 1.f / 362880.f);
    ps = fmaf(ps, r2, -1.f / 5040.f);
    ps = fmaf(ps, r2, 1.f / 120.f);
    ps = fmaf(ps, r2, -1.f / 6.f);
    const float sr = fmaf(ps * r2, r, r);
    float pc = 1.f / 479001600.f;
    pc = fmaf(pc, r2, -1.f / 3628800.f);
    pc = fmaf(pc, r2, 1.f / 40320.f);
    pc = fmaf(pc, r2, -1.f / 720.f);
    pc = fmaf(pc, r2, 1.f / 24.f);
    pc = fmaf(pc, r2, -0.5f);
    const float cr = fmaf(pc, r2, 1.f);
    const int q = (int)k & 3;
    const float a = (q & 1) ? cr : sr, b = (q & 1) ? sr : cr;
    sn = (q & 2) ? -a : a;
    cs = ((q + 1) & 2) ? -b : b;
}

// exp(-i theta) - 1, accurate for small theta.
__device__ __forceinline__ float2 phase_step(float theta) {
    float s, c;
    sincos_cw(0.5f * theta, s, c);
    return make_float2(-2.f * s * s, -2.f * s * c);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float2 cmul_conj(float2 a, float2 b) {  // a * conj(b)
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}

// ---- receive contraction on the tensor cores --------------------------------
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// D += A (16x8, row) * B (8x8, col), TF32 inputs, FP32 accumulate
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// (x, y) as TF32 (big, small) parts: x = big + small to ~2^-22 relative,
// for the three-term TF32 product big*big + big*small + small*big
__device__ __forceinline__ uint4 tf32_split2(float x, float y) {
    const uint32_t xb = to_tf32(x), yb = to_tf32(y);
    return make_uint4(xb, to_tf32(x - __uint_as_float(xb)), yb, to_tf32(y - __uint_as_float(yb)));
}

// y = 1 - exp(-x)
__device__ __forceinline__ float one_minus_exp(float x) { return -expm1f(-x); }

// Rotation of the frame magnetisation by an rf step: angle alpha about
// n = (cb cos PHI, -cb sin PHI, sb) in the sense of the reference's closed
// form (verified identity: R = cos a I - sin a [n]x + (1 - cos a) n n^T).
__device__ __forceinline__ void rf_rotate(float &x, float &y, float &z, float dW, float b, float2 uphi, float dt) {
    const float q = fmaf(dW, dW, b * b);
    if (q == 0.f) return;
    const float rn = rsqrtf(q);
    const float Bm = q * rn;
    const float cb = fabsf(b) * rn;
    const float sb = copysignf(1.f, b) * dW * rn;
    float sh, ch;
    sincos_cw(0.5f * Bm * dt, sh, ch);
    const float sa = 2.f * sh * ch;
    const float omc = 2.f * sh * sh;  // 1 - cos(alpha)
    const float ca = 1.f - omc;
    const float nx = cb * uphi.x, ny = -cb * uphi.y, nz = sb;
    const float cx = ny * z - nz * y, cy = nz * x - nx * z, cz = nx * y - ny * x;
    const float k = fmaf(nx, x, fmaf(ny, y, nz * z));
    // increment form R M = M + (1 - cos a)((n.M) n - M) - sin a (n x M): the
    // small increment is added to M with a single rounding
    (void)ca;
    const float x2 = x + fmaf(omc, fmaf(k, nx, -x), -sa * cx);
    const float y2 = y + fmaf(omc, fmaf(k, ny, -y), -sa * cy);
    const float z2 = z + fmaf(omc, fmaf(k, nz, -z), -sa * cz);
    x = x2;
    y = y2;
    z = z2;
}

// FREE (KM_EXCH only): every pool is a free pool (ME, or GM without bound
// pools); the instantiation then has only the straight-line update path.
template <int MODEL, int P, int NS, bool FREE>
__global__ void __launch_bounds__(kBlock) scan_fast_kernel(FastLaunch F) {
    const ScanLaunch &L = F.b;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float4 *rbuf = reinterpret_cast<float4 *>(smem + 128);
    const int rstride = L.stride4;
    // receive tile: one row per (sample, sampled pool), one column per thread
    // holding its lab-frame transverse magnetisation as TF32 (big, small)
    // parts (x big, x small, y big, y small); the coil sensitivities of the
    // threads' voxels split the same way (x big, x small, y big, y small);
    // per-warp sums of the contraction
    constexpr int kNSampP = (MODEL == KM_MT || MODEL == KM_CEST) ? 1 : P;
    constexpr int kTile = (16 / kNSampP) < 1 ? 1 : 16 / kNSampP;  // samples per flush
    constexpr int kTRow = kBlock + 2;                             // padded row (uint4)
    const int C4 = (L.rx + 3) & ~3;
    uint4 *mtile = reinterpret_cast<uint4 *>(rbuf + 2 * kFastChunk * rstride);  // [16][kTRow]
    uint4 *rsm = mtile + 16 * kTRow;                                             // [C4][kTRow]
    float *red = reinterpret_cast<float *>(rsm + C4 * kTRow);                    // [warp][16][2*C4]
    constexpr int kWarps = kBlock / 32;
    constexpr bool kFreeAll = MODEL == KM_NORMAL || MODEL == KM_EXCH;

    const int tid = threadIdx.x;
    const long long gt = (long long)blockIdx.x * kBlock + tid;
    const int v = (int)(gt / L.tpv);
    const int sg = (int)(gt % L.tpv);
    bool active = v < L.n_act;
    const int n = L.n_act;

    float X[NS][P], Y[NS][P], Z[NS][P];
    float2 Ph[NS][P], D[NS][P];
    float Wh[NS][P], Wl[NS][P];
    float rhoS[P], it1[P], it2[P], t2v[P], y1[P], y2[P];
    unsigned act = 0;
    float2 om[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    float2 tx0 = make_float2(0.f, 0.f);
    float db0 = 0.f;
    constexpr int kNK = MODEL == KM_EXCH ? P * P : (MODEL == KM_MT ? 2 : (MODEL == KM_CEST ? 2 * (P - 1) : 1));
    float kc[kNK];
#pragma unroll
    for (int i = 0; i < kNK; ++i) kc[i] = 0.f;
#pragma unroll
    for (int t = 0; t < P; ++t) {
        rhoS[t] = it1[t] = it2[t] = t2v[t] = y1[t] = y2[t] = 0.f;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            X[s][t] = Y[s][t] = Z[s][t] = Wh[s][t] = Wl[s][t] = 0.f;
            Ph[s][t] = make_float2(1.f, 0.f);
            D[s][t] = make_float2(0.f, 0.f);
        }
    }
    if (active) {
        db0 = L.db0[v];
        if (F.direct) {
            const float g[4] = {db0, L.gxg[v], L.gyg[v], L.gzg[v]};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const df p = df_mul(F.gam_hi, F.gam_lo, g[i], 0.f);
                om[i] = make_float2(p.hi, p.lo);
            }
            float sp, cp;
            sincos_cw(L.txpe[v], sp, cp);
            tx0 = make_float2(L.txmg[v] * cp, L.txmg[v] * sp);
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) om[i] = F.omega[(long long)i * n + v];
            tx0 = F.txc[v];
        }
#pragma unroll
        for (int t = 0; t < P; ++t) {
            const float r = L.rho[(long long)t * n + v], T1 = L.t1[(long long)t * n + v],
                        T2 = L.t2[(long long)t * n + v];
            rhoS[t] = r / (float)L.S;
            it1[t] = T1 != 0.f ? 1.f / T1 : 0.f;
            it2[t] = T2 != 0.f ? 1.f / T2 : 0.f;
            t2v[t] = T2;
            if (T1 != 0.f && T2 != 0.f && r != 0.f) act |= 1u << t;
        }
        if (MODEL == KM_MT) {
            kc[0] = L.kch[1LL * n + v];
            kc[1] = L.kch[2LL * n + v];
        } else if (MODEL != KM_NORMAL) {
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
                if (F.direct) {
                    const df w = two_sum(L.dwrnd[i], F.cs_hi[t]);
                    Wh[s][t] = w.hi;
                    Wl[s][t] = w.lo + F.cs_lo[t];
                } else {
                    const float2 w = F.wres[i];
                    Wh[s][t] = w.x;
                    Wl[s][t] = w.y;
                }
            }
        }
    }
    if (F.direct) {
        const bool any = (MODEL == KM_MT || MODEL == KM_CEST) ? (act & 1u) != 0 : act != 0;
        if (!any) active = false;
    }
    // stage this thread's voxel's coil sensitivities (zero beyond the coil count)
    for (int c = 0; c < C4; ++c) {
        float2 r = make_float2(0.f, 0.f);
        if (active && c < L.rx) {
            if (L.rx_default)
                r = make_float2(1.f, 0.f);
            else if (F.direct)
                r = make_float2(F.rx_x[(long long)c * n + v], F.rx_y[(long long)c * n + v]);
            else
                r = L.rxc[(long long)c * n + v];
        }
        rsm[c * kTRow + tid] = tf32_split2(r.x, r.y);
    }
    // the isochromats enter the frame at the start of the launch: m_frame = m_lab / P
    bool entered = false;
    // exchange / MT coefficients, cached per dt
    float yo[P], fin[P][P];
#pragma unroll
    for (int t = 0; t < P; ++t) {
        yo[t] = 0.f;
#pragma unroll
        for (int p = 0; p < P; ++p) fin[t][p] = 0.f;
    }
    float mt_y1k = 0.f, mt_y21 = 0.f, mt_y1bk = 0.f, mt_y1b = 0.f, mt_y12 = 0.f;
    LineshapeCache lc;
    const float gyro = L.gyro;

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nsteps = L.s1 - L.s0;
    const int nchunks = (int)((nsteps + kFastChunk - 1) / kFastChunk);
    auto issue = [&](int k) {
        const long long first = L.s0 + (long long)k * kFastChunk;
        const long long cnt = min((long long)kFastChunk, L.s1 - first);
        const uint32_t bytes = (uint32_t)(cnt * rstride * 16);
        mbar_expect_tx(&bar[k & 1], bytes);
        bulk_g2s(rbuf + (k & 1) * kFastChunk * rstride, L.rec + first * rstride, bytes, &bar[k & 1]);
    };
    if (tid == 0 && nchunks > 0) issue(0);

    int a_fill = 0, a_base = 0;
    const int lane = tid & 31, warp = tid >> 5;
    // flush: S[row][2c + {x,y}] = sum over threads of m(row) conj(R_c): a
    // (16 x 2*128) x (2*128 x 2*C4) real GEMM, split by warps along the
    // thread (voxel) dimension, on the tensor cores in the three-term TF32
    // split (big*big + big*small + small*big, each term its own accumulator
    // chain); then the warp slices are added and one
    // partial per (block, sample, pool, coil) is written.
    //   A[row][2j + ri] = (x, y)[ri] of thread j;  B[2j + ri][2c + cmp]:
    //   (x,x) = rx, (y,x) = ry, (x,y) = -ry, (y,y) = rx.
    auto flush = [&]() {
        __syncthreads();
        const int g = lane >> 2, tig = lane & 3, ri = tig & 1, cmp = g & 1;
        const bool same = ri == cmp;                              // rx, else ry
        const uint32_t sgn = (cmp && !ri) ? 0x80000000u : 0u;     // -ry
        const uint2 *mt2 = reinterpret_cast<const uint2 *>(mtile);  // (big, small) pairs
        const int nt_all = C4 / 4;
        float *rw = red + warp * 16 * (2 * C4);
        for (int nt = 0; nt < nt_all; ++nt) {
            float acc[3][4];
#pragma unroll
            for (int u = 0; u < 3; ++u)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[u][i] = 0.f;
            const int c = nt * 4 + (g >> 1);
#pragma unroll
            for (int ks = 0; ks < 8; ++ks) {
                const int j0 = warp * 32 + ks * 4 + (tig >> 1), j1 = j0 + 2;
                const uint2 a00 = mt2[(g * kTRow + j0) * 2 + ri], a10 = mt2[((g + 8) * kTRow + j0) * 2 + ri];
                const uint2 a01 = mt2[(g * kTRow + j1) * 2 + ri], a11 = mt2[((g + 8) * kTRow + j1) * 2 + ri];
                const uint32_t ab[4] = {a00.x, a10.x, a01.x, a11.x};
                const uint32_t as[4] = {a00.y, a10.y, a01.y, a11.y};
                const uint4 q0 = rsm[c * kTRow + j0], q1 = rsm[c * kTRow + j1];
                const uint32_t bb[2] = {(same ? q0.x : q0.z) ^ sgn, (same ? q1.x : q1.z) ^ sgn};
                const uint32_t bs[2] = {(same ? q0.y : q0.w) ^ sgn, (same ? q1.y : q1.w) ^ sgn};
                mma_tf32(acc[0], as, bb);
                mma_tf32(acc[1], ab, bs);
                mma_tf32(acc[2], ab, bb);
            }
            float d[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) d[i] = (acc[0][i] + acc[1][i]) + acc[2][i];
            const int col = nt * 8 + 2 * tig;
            rw[g * (2 * C4) + col] = d[0];
            rw[g * (2 * C4) + col + 1] = d[1];
            rw[(g + 8) * (2 * C4) + col] = d[2];
            rw[(g + 8) * (2 * C4) + col + 1] = d[3];
        }
        __syncthreads();
        const int nout = a_fill * kNSampP * L.rx;
        for (int o = tid; o < nout; o += kBlock) {
            const int row = o / L.rx;  // = a * kNSampP + t
            const int c = o - row * L.rx;
            const int a = row / kNSampP, t = row - a * kNSampP;
            float sx = 0.f, sy = 0.f;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                sx += red[(w * 16 + row) * (2 * C4) + 2 * c];
                sy += red[(w * 16 + row) * (2 * C4) + 2 * c + 1];
            }
            L.partial[((long long)blockIdx.x * L.a_launch + a_base + a) * L.npairs + t * L.rx + c] = make_float2(sx, sy);
        }
        a_base += a_fill;
        a_fill = 0;
        __syncthreads();
    };

    bool ok = true;
    for (int k = 0; k < nchunks && ok; ++k) {
        if (tid == 0 && k + 1 < nchunks) issue(k + 1);
        ok = mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, L.err);
        ok = __syncthreads_and(ok) != 0;
        if (!ok) {
            if (tid == 0) mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, L.err);
            break;
        }
        const float4 *cb = rbuf + (k & 1) * kFastChunk * rstride;
        const int cnt = (int)min((long long)kFastChunk, nsteps - (long long)k * kFastChunk);
        for (int q = 0; q < cnt; ++q) {
            const float4 r0 = cb[q * rstride];
            const float4 r1 = cb[q * rstride + 1];
            int flags = __float_as_int(r1.w);
            if (k == 0 && q == 0) flags |= kFlagState | kFlagDt;  // a launch may start inside a run
            const float dt = r0.x;

            // ---- frame phasors ---------------------------------------------
            if (active && ((flags & kFlagAnchor) || !entered)) {
                const float4 r2 = cb[q * rstride + 2];
                const float4 r3 = cb[q * rstride + 3];
                df phc = df_mul(om[0].x, om[0].y, r2.x, r2.y);
                phc = df_add(phc, df_mul(om[1].x, om[1].y, r2.z, r2.w));
                phc = df_add(phc, df_mul(om[2].x, om[2].y, r3.x, r3.y));
                phc = df_add(phc, df_mul(om[3].x, om[3].y, r3.z, r3.w));
#pragma unroll
                for (int s = 0; s < NS; ++s)
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        const float2 pn = phasor(df_add(phc, df_mul(Wh[s][t], Wl[s][t], r2.x, r2.y)));
                        if (!entered) {  // m_frame = m_lab * conj(P)
                            const float2 m = cmul_conj(make_float2(X[s][t], Y[s][t]), pn);
                            X[s][t] = m.x;
                            Y[s][t] = m.y;
                        }
                        Ph[s][t] = pn;
                    }
                entered = true;
            }
            const float gzt = r0.y, gyt = r0.z, gxt = r0.w;
            // instantaneous common off-resonance (rad/s)
            const float wc = fmaf(om[3].x, gzt, fmaf(om[2].x, gyt, fmaf(om[1].x, gxt, om[0].x)));
            if (active && (flags & kFlagState)) {
#pragma unroll
                for (int s = 0; s < NS; ++s)
#pragma unroll
                    for (int t = 0; t < P; ++t)
                        D[s][t] = (MODEL == KM_MT || MODEL == KM_CEST || (act >> t & 1u))
                                      ? phase_step((wc + Wh[s][t]) * dt)
                                      : make_float2(0.f, 0.f);
            }
            if (active && (flags & kFlagDt)) {
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    y1[t] = one_minus_exp(dt * it1[t]);
                    y2[t] = one_minus_exp(dt * it2[t]);
                }
                if (MODEL == KM_EXCH) {
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        float ko = 0.f;  // exp(-sum k_out dt) = 1 - ko
                        float ksum = 0.f;
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            fin[t][p] = 0.f;
                            if (L.exch_gm && p == t) continue;
                            const float kgo = L.exch_gm ? kc[p * P + t] : kc[t * P + p];
                            const float kin = L.exch_gm ? kc[t * P + p] : kc[p * P + t];
                            ksum += kgo;
                            if (kin != 0.f) fin[t][p] = one_minus_exp(dt * kin);
                        }
                        ko = one_minus_exp(dt * ksum);
                        yo[t] = ko;
                    }
                } else if (MODEL == KM_MT || MODEL == KM_CEST) {
                    const float K12 = kc[0];
                    const float K21 = MODEL == KM_MT ? kc[1] : kc[P - 1];
                    mt_y1k = one_minus_exp(dt * (it1[0] + K12));
                    mt_y21 = one_minus_exp(dt * K21);
                    mt_y1bk = one_minus_exp(dt * (it1[1] + K21));
                    mt_y1b = one_minus_exp(dt * it1[1]);
                    mt_y12 = one_minus_exp(dt * K12);
                    if (MODEL == KM_CEST) {
                        float ksum = 0.f;
#pragma unroll
                        for (int t = 2; t < P; ++t) {
                            const float kgo = kc[t - 1], kin = kc[t + P - 2];
                            ksum += kgo;
                            fin[0][t] = kin != 0.f ? one_minus_exp(dt * kin) : 0.f;
                            yo[t] = kin != 0.f ? one_minus_exp(dt * kin) : 0.f;
                            fin[t][0] = kgo != 0.f ? one_minus_exp(dt * kgo) : 0.f;
                        }
                        yo[0] = one_minus_exp(dt * ksum);
                    }
                }
            }

            if (active && (flags & kFlagDt) && MODEL != KM_MT && MODEL != KM_CEST) {
                // an empty pool keeps its magnetisation: neutral coefficients
                // instead of branches keep the per-pool updates straight-line
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    if (act >> t & 1u) continue;
                    y1[t] = y2[t] = yo[t] = 0.f;
#pragma unroll
                    for (int p = 0; p < P; ++p) fin[t][p] = 0.f;
                }
            }

            // ---- receive, before the step's rotation ------------------------
            if (flags & kFlagAdc) {
#pragma unroll
                for (int t = 0; t < kNSampP; ++t) {
                    float mx = 0.f, my = 0.f;
                    const bool sampled = (MODEL != KM_EXCH) || FREE || (L.kind[t] == 0);
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        const float2 m = cmul(make_float2(X[s][t], Y[s][t]), Ph[s][t]);
                        mx += m.x;
                        my += m.y;
                    }
                    if (!(active && sampled)) mx = my = 0.f;
                    mtile[(a_fill * kNSampP + t) * kTRow + tid] = tf32_split2(mx, my);
                }
                if (++a_fill == kTile) flush();
            }
            if (!active) continue;

            const bool rf = (flags & kFlagRf) != 0;
            float b = 0.f;
            float2 u0 = make_float2(1.f, 0.f);  // exp(i PHI) before the frame shift
            float w_sat[P];                       // bound-pool saturation rates
#pragma unroll
            for (int t = 0; t < P; ++t) w_sat[t] = 0.f;
            if (rf) {
                // complex B1 = sum_c TxCoilmg_c exp(i pe_c) * amp_c exp(i phase_c)
                float2 B = cmul(tx0, make_float2(r1.x, r1.y));
                for (int c = 1; c < L.tx && c < 4; ++c) {
                    const float4 rc = cb[q * rstride + 3 + c];
                    const float2 t2 = cmul(F.txc[(long long)c * n + v], make_float2(rc.x, rc.y));
                    B.x += t2.x;
                    B.y += t2.y;
                }
                const float Bm = sqrtf(fmaf(B.x, B.x, B.y * B.y));
                b = Bm * gyro;
                if (Bm > 0.f) u0 = make_float2(B.x / Bm, -B.y / Bm);  // conj(B)/|B|
                if (MODEL != KM_NORMAL) {
                    // bound pools: W = pi (gamma TxCoilmg |amp|)^2 G(rf offset, T2b) with the
                    // reference's lineshape rule (single transmit coil)
                    const float b1 = sqrtf(fmaf(r1.x, r1.x, r1.y * r1.y)) * sqrtf(fmaf(tx0.x, tx0.x, tx0.y * tx0.y));
                    const float freq = r1.z * 0.15915494309189535f;
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        const bool bound = (MODEL == KM_EXCH) ? (!FREE && L.kind[t] == 1) : (t == 1);
                        if (!bound) continue;
                        if (lc.t2b != t2v[t] || lc.freq != freq) {
                            lc.freq = freq;
                            lc.t2b = t2v[t];
                            lc.g = lineshape(freq, db0, gyro, t2v[t]);
                        }
                        w_sat[t] = (float)(kPiRef * (double)((b1 * gyro) * (b1 * gyro)) * (double)lc.g);
                    }
                }
            }
            const float wrf = r1.z;  // 2 pi sum of active rf frequencies

#pragma unroll
            for (int s = 0; s < NS; ++s) {
                float2 Pprev[P];
#pragma unroll
                for (int t = 0; t < P; ++t) Pprev[t] = Ph[s][t];
                float px[P], py[P], pz[P];
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    px[t] = X[s][t];
                    py[t] = Y[s][t];
                    pz[t] = Z[s][t];
                }
                if (MODEL == KM_NORMAL || (MODEL == KM_EXCH && FREE)) {
                    // every pool free: straight-line updates of all pools
                    if (rf) {
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            float x = X[s][t], y = Y[s][t], z = Z[s][t];
                            rf_rotate(x, y, z, wc + Wh[s][t] + wrf, b, cmul(u0, Ph[s][t]), dt);
                            const bool on = act >> t & 1u;
                            X[s][t] = on ? x : X[s][t];
                            Y[s][t] = on ? y : Y[s][t];
                            Z[s][t] = on ? z : Z[s][t];
                        }
                    } else {
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            const float2 p = Ph[s][t], d = D[s][t];
                            Ph[s][t] = make_float2(fmaf(p.x, d.x, fmaf(-p.y, d.y, p.x)), fmaf(p.x, d.y, fmaf(p.y, d.x, p.y)));
                        }
                    }
                    if (MODEL == KM_NORMAL) {
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            X[s][t] = fmaf(-y2[t], X[s][t], X[s][t]);
                            Y[s][t] = fmaf(-y2[t], Y[s][t], Y[s][t]);
                            Z[s][t] = fmaf(y1[t], rhoS[t] - Z[s][t], Z[s][t]);
                        }
                    } else {
                        // inflow uses every pool's magnetisation before the step, in the lab
                        // frame, carried into the receiving pool's frame after the step
                        float2 ml[P];
#pragma unroll
                        for (int p = 0; p < P; ++p) ml[p] = cmul(make_float2(px[p], py[p]), Pprev[p]);
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            float ix = 0.f, iy = 0.f, iz = 0.f;
#pragma unroll
                            for (int p = 0; p < P; ++p) {
                                ix = fmaf(fin[t][p], ml[p].x, ix);
                                iy = fmaf(fin[t][p], ml[p].y, iy);
                                iz = fmaf(fin[t][p], pz[p], iz);
                            }
                            const float2 in = cmul_conj(make_float2(ix, iy), Ph[s][t]);
                            float x = fmaf(-y2[t], X[s][t], X[s][t]);
                            float y = fmaf(-y2[t], Y[s][t], Y[s][t]);
                            float z = fmaf(-y1[t], Z[s][t], Z[s][t]);
                            X[s][t] = fmaf(-yo[t], x, x) + in.x;
                            Y[s][t] = fmaf(-yo[t], y, y) + in.y;
                            Z[s][t] = fmaf(-yo[t], z, z) + iz + rhoS[t] * y1[t];
                        }
                    }
                    continue;
                }
                // rotation (rf) or frame advance (free precession)
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    const bool free_pool =
                        kFreeAll ? (MODEL == KM_NORMAL || L.kind[t] == 0) : (t == 0 || (MODEL == KM_CEST && t >= 2));
                    if (!free_pool) continue;
                    if (MODEL != KM_MT && MODEL != KM_CEST && !(act >> t & 1u)) continue;
                    if (rf) {
                        const float dW = wc + Wh[s][t] + wrf;
                        const float2 uphi = cmul(u0, Ph[s][t]);
                        rf_rotate(X[s][t], Y[s][t], Z[s][t], dW, b, uphi, dt);
                    } else {
                        const float2 p = Ph[s][t];
                        const float2 d = D[s][t];
                        Ph[s][t] = make_float2(fmaf(p.x, d.x, fmaf(-p.y, d.y, p.x)), fmaf(p.x, d.y, fmaf(p.y, d.x, p.y)));
                    }
                }
                // relaxation and exchange
                if (MODEL == KM_NORMAL) {
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        if (!(act >> t & 1u)) continue;
                        X[s][t] = fmaf(-y2[t], X[s][t], X[s][t]);
                        Y[s][t] = fmaf(-y2[t], Y[s][t], Y[s][t]);
                        Z[s][t] = fmaf(y1[t], rhoS[t] - Z[s][t], Z[s][t]);
                    }
                } else if (MODEL == KM_EXCH) {
                    float nx[P], ny[P], nz[P];
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        nx[t] = X[s][t];
                        ny[t] = Y[s][t];
                        nz[t] = Z[s][t];
                    }
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        if (!(act >> t & 1u)) continue;
                        const int kind = L.kind[t];
                        if (kind != 0 && kind != 1) continue;
                        const bool bound = kind == 1;
                        float x = nx[t], y = ny[t], z = nz[t];
                        float ix = 0.f, iy = 0.f, iz = 0.f;
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            const float f = fin[t][p];
                            if (f == 0.f) continue;
                            iz = fmaf(f, pz[p], iz);
                            if (!bound && L.kind[p] == 0) {
                                // m_p(prev) carried into t's frame after the step
                                const float2 rel = cmul_conj(Pprev[p], Ph[s][t]);
                                const float2 m = cmul(make_float2(px[p], py[p]), rel);
                                ix = fmaf(f, m.x, ix);
                                iy = fmaf(f, m.y, iy);
                            }
                        }
                        if (bound) {
                            if (rf) z = fmaf(-one_minus_exp(w_sat[t] * dt), z, z);
                        } else {
                            x = fmaf(-y2[t], x, x);
                            y = fmaf(-y2[t], y, y);
                            x = fmaf(-yo[t], x, x) + ix;
                            y = fmaf(-yo[t], y, y) + iy;
                            X[s][t] = x;
                            Y[s][t] = y;
                        }
                        z = fmaf(-y1[t], z, z);
                        Z[s][t] = fmaf(-yo[t], z, z) + iz + rhoS[t] * y1[t];
                    }
                } else {  // MT / CEST
                    float x = X[s][0], y = Y[s][0], z = Z[s][0];
                    const float zb0 = pz[1], z0 = pz[0];
                    x = fmaf(-y2[0], x, x);
                    y = fmaf(-y2[0], y, y);
                    if (MODEL == KM_MT) {
                        z = fmaf(-mt_y1k, z, z) + rhoS[0] * y1[0] + zb0 * mt_y21;
                    } else {
                        float ix = 0.f, iy = 0.f, iz = 0.f;
#pragma unroll
                        for (int t = 2; t < P; ++t) {
                            const float f = fin[0][t];
                            const float2 rel = cmul_conj(Pprev[t], Ph[s][0]);
                            const float2 m = cmul(make_float2(px[t], py[t]), rel);
                            ix = fmaf(f, m.x, ix);
                            iy = fmaf(f, m.y, iy);
                            iz = fmaf(f, pz[t], iz);
                        }
                        x = fmaf(-yo[0], x, x) + ix;
                        y = fmaf(-yo[0], y, y) + iy;
                        z = fmaf(-mt_y1k, z, z);
                        z = fmaf(-yo[0], z, z) + iz + zb0 * mt_y21 + rhoS[0] * y1[0];
#pragma unroll
                        for (int t = 2; t < P; ++t) {
                            float cx = X[s][t], cy = Y[s][t], cz = Z[s][t];
                            cx = fmaf(-y2[t], cx, cx);
                            cy = fmaf(-y2[t], cy, cy);
                            cz = fmaf(-y1[t], cz, cz);
                            const float f = fin[t][0];
                            const float2 rel = cmul_conj(Pprev[0], Ph[s][t]);
                            const float2 m = cmul(make_float2(px[0], py[0]), rel);
                            X[s][t] = fmaf(-yo[t], cx, cx) + f * m.x;
                            Y[s][t] = fmaf(-yo[t], cy, cy) + f * m.y;
                            Z[s][t] = fmaf(-yo[t], cz, cz) + f * z0 + rhoS[t] * y1[t];
                        }
                    }
                    float bz = zb0;
                    if (rf) bz = fmaf(-one_minus_exp(w_sat[1] * dt), bz, bz);
                    Z[s][1] = fmaf(-mt_y1bk, bz, bz) + rhoS[1] * mt_y1b + z0 * mt_y12;
                    X[s][0] = x;
                    Y[s][0] = y;
                    Z[s][0] = z;
                }
            }
        }
        __syncthreads();
    }
    if (a_fill > 0) flush();

    if (active) {
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const int sp = sg * NS + s;
#pragma unroll
            for (int t = 0; t < P; ++t) {
                // back to the lab frame: m_lab = m_frame * P
                const float2 m = entered ? cmul(make_float2(X[s][t], Y[s][t]), Ph[s][t]) : make_float2(X[s][t], Y[s][t]);
                const long long i = ((long long)t * L.S + sp) * n + v;
                L.mx[i] = m.x;
                L.my[i] = m.y;
                L.mz[i] = Z[s][t];
            }
        }
    }
}

}  // namespace mrl
