// Adjoint of the scan: gradients of a loss of the signal with respect to the
// tissue parameters, the initial magnetisation and the rf waveform.
//
// The map differentiated is the integrator's discrete step (free-pool
// models: the normal model and exchange among free pools, as
// BlochKernel.cuh:241-276 and BlochKernelME.cuh:225-343 define it), for
// isochromat-pool t of one spin:
//   rotation   m_r = exp([v]x) m,  v = -dt (gamma Bx, gamma By, w_t)
//              (B = TxCoil * A the complex rf field, w_t the off-resonance
//              gamma (dB0 + G.r) + dWRnd + 2 pi CS_t + 2 pi f_rf)
//   relaxation and split exchange, with the inflow taken from the
//              magnetisation before the step:
//              x' = d2_t x_r + sum_p f_tp x_p,  y' likewise,
//              z' = d1_t z_r + sum_p f_tp z_p + c_t,
//              d2 = (1 - yo)(1 - y2), d1 = (1 - yo)(1 - y1), c = rho / S y1,
//              y1,2 = 1 - exp(-dt / T1,2), yo = 1 - exp(-dt sum_p k_tp),
//              f_tp = 1 - exp(-dt k_pt)
// and the receive sums S_{t,c,a} = sum over isochromats of (x + i y)_t
// conj(R_c) at ADC steps, before the step.  Given G = dL/dSx + i dL/dSy the
// adjoint lambda_j = dL/dm_j runs backwards:
//   lambda_j = F_j^T lambda_{j+1} + sum_c G_{t,c,a} R_c  (ADC step j),
// and every step adds lambda_{j+1}^T dF_j/dtheta to the gradient of each
// parameter theta.  The rotation's derivative uses the left Jacobian of
// SO(3) exponential coordinates: lambda^T d(exp([v]x) m) = dv . J_l(v)^T
// (m_r x lambda_r), J_l(v)^T u = u - c1 v x u + c2 v x (v x u),
// c1 = (1 - cos a) / a^2, c2 = (a - sin a) / a^3, a = |v|.
//
// Bound pools of the general model (TypeFlag 1, BlochKernelGM.cuh; the
// CPU engine's rule as the oracle restates it) take no rotation and keep
// their transverse magnetisation; an rf step first saturates their
// longitudinal magnetisation, z_r = q z with q = exp(-W dt),
// W = pi (gamma |TxCoil| |A|)^2 G(a), G the super-Lorentzian lineshape at
// a = (2 pi f_rf + gamma dB0) T2b, then relaxation and exchange act on
// z alone.  Its gradients: dL/dW = -dt d1 lambda_z z_r, and through W the
// rf amplitude (dW/dA = 2 pi (gamma |TxCoil|)^2 G A), dB0 (dG/da gamma T2b)
// and T2b (dG/dT2b = (G + a dG/da) / T2b).
//
// One thread owns one isochromat (a voxel's spin, all its pools).  The
// forward scan (the accurate integrator, whose frames are anchored to FP64
// phase moments) stores the lab-frame state every seg * kAdjWin steps
// (checkpoints, in HBM); this kernel takes the windows of kAdjWin steps
// last to first, recomputes each window's states from its starting state
// into shared memory with the map above and walks them in reverse.  With
// seg > 1, entering a segment it first runs the segment forward from its
// checkpoint and keeps every window's starting state in ck2.  The rf
// gradient of a step is summed over the block (warp shuffles, then the
// warps) and added to its FP64 slot.  The receive term reads the thread's
// coil sensitivities from shared memory (staged once) and the step's dL/dS
// from a per-warp shared buffer that cp.async filled during the step
// before.
#include "scan_launch.h"

namespace mrl {

namespace {

// Super-Lorentzian lineshape of a bound pool and its slope, by the forward
// kernel's rule (BlochKernelMT.cuh:348-358: u = p / 1000, p < 1000):
//   G = c T2b sum_u |1/d| exp(-2 a^2 / d^2),  d = 3u^2 - 1,  c = sqrt(2 / pi) / 1000,
//   dG/da = -4 a c T2b sum_u |1/d|^3 exp(-2 a^2 / d^2),
// a = (2 pi f + gamma dB0) T2b.  Four interleaved partial sums (the value
// compensated, as in the forward scan); returns (G, dG/da).
static __device__ __noinline__ float2 lineshape_slope(float a, float t2b) {
    float g[4] = {0.f, 0.f, 0.f, 0.f}, comp[4] = {0.f, 0.f, 0.f, 0.f}, h[4] = {0.f, 0.f, 0.f, 0.f};
    for (int p0 = 0; p0 < 1000; p0 += 4) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float u = (float)(p0 + j) * 0.001f;
            const float inv = 1.f / fmaf(3.f * u, u, -1.f);
            const float x = a * inv;
            const float e = fabsf(inv) * __expf(-2.f * x * x);
            const float term = e - comp[j];
            const float sum = g[j] + term;
            comp[j] = (sum - g[j]) - term;
            g[j] = sum;
            h[j] = fmaf(e, inv * inv, h[j]);
        }
    }
    const float s0 = ((g[0] - comp[0]) + (g[1] - comp[1])) + ((g[2] - comp[2]) + (g[3] - comp[3]));
    const float s2 = (h[0] + h[1]) + (h[2] + h[3]);
    const float c = 0.79788456080286536f * 0.001f * t2b;
    return make_float2(s0 * c, -4.f * a * s2 * c);
}

__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }

struct Rot {  // exp([v]x) of one step for one pool: s = (sin a / a, (1 - cos a) / a^2)
    float3 v;
    float2 s;
};

__device__ __forceinline__ Rot make_rot(float3 v) {
    Rot r;
    r.v = v;
    r.s = rot_coeffs(dot3(v, v));
    return r;
}

__device__ __forceinline__ float3 rot_apply(const Rot &r, float3 m) {
    rot_exp(m.x, m.y, m.z, r.v.x, r.v.y, r.v.z, r.s);
    return m;
}
__device__ __forceinline__ float3 rot_apply_t(const Rot &r, float3 m) {  // exp(-[v]x) m
    rot_exp(m.x, m.y, m.z, -r.v.x, -r.v.y, -r.v.z, r.s);
    return m;
}
// (a - sin a) / a^3 = (1 - s1) / a^2: Taylor series in a^2 through a^6 below
// a = 0.25 (truncation below 1e-12), the quotient above
__device__ __forceinline__ float jl_c2(float a2, float s1) {
    if (a2 < 0.0625f)
        return fmaf(fmaf(fmaf(a2, -1.f / 362880.f, 1.f / 5040.f), a2, -1.f / 120.f), a2, 1.f / 6.f);
    return (1.f - s1) / a2;
}
// J_l(v)^T u = u - c1 v x u + c2 v x (v x u), c1 = (1 - cos a) / a^2
__device__ __forceinline__ float3 jl_t(const Rot &r, float3 u) {
    const float c2 = jl_c2(dot3(r.v, r.v), r.s.x);
    const float3 vu = cross3(r.v, u);
    const float3 vvu = cross3(r.v, vu);
    return make_float3(u.x - r.s.y * vu.x + c2 * vvu.x, u.y - r.s.y * vu.y + c2 * vvu.y,
                       u.z - r.s.y * vu.z + c2 * vvu.z);
}

// Two pools of one isochromat as the lanes of f32x2 values (the packed
// two-pool path of the kernel): a 3-vector per pool, lane t = pool t.
struct V2 {
    float2 x, y, z;
};
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// a x b per lane
__device__ __forceinline__ V2 cross2(const V2 &a, const V2 &b) {
    return {fma2(a.y, b.z, neg2(mul2(a.z, b.y))), fma2(a.z, b.x, neg2(mul2(a.x, b.z))),
            fma2(a.x, b.y, neg2(mul2(a.y, b.x)))};
}
__device__ __forceinline__ float2 dot2(const V2 &a, const V2 &b) { return fma2(a.x, b.x, fma2(a.y, b.y, mul2(a.z, b.z))); }
// (sin a / a, (1 - cos a) / a^2) per lane: the Taylor series of rot_coeffs
// on both lanes at once when both angles are below 0.25
__device__ __forceinline__ void rot_coeffs2(float2 a2, float2 &s1, float2 &s2) {
    if (a2.x < 0.0625f && a2.y < 0.0625f) {
        s1 = fma2(fma2(fma2(a2, bc(-1.f / 5040.f), bc(1.f / 120.f)), a2, bc(-1.f / 6.f)), a2, bc(1.f));
        s2 = fma2(fma2(fma2(a2, bc(-1.f / 40320.f), bc(1.f / 720.f)), a2, bc(-1.f / 24.f)), a2, bc(0.5f));
    } else {
        const float2 c0 = rot_coeffs(a2.x), c1 = rot_coeffs(a2.y);
        s1 = make_float2(c0.x, c1.x);
        s2 = make_float2(c0.y, c1.y);
    }
}
// exp([v]x) m per lane (Rodrigues' formula, m + s1 c + s2 e as two fused
// steps: the window recompute restarts from a checkpoint every 16 steps)
__device__ __forceinline__ V2 rot2(const V2 &v, float2 s1, float2 s2, const V2 &m) {
    const V2 c = cross2(v, m), e = cross2(v, c);
    return {fma2(s2, e.x, fma2(s1, c.x, m.x)), fma2(s2, e.y, fma2(s1, c.y, m.y)),
            fma2(s2, e.z, fma2(s1, c.z, m.z))};
}
// J_l(v)^T u per lane (jl_t)
__device__ __forceinline__ V2 jlt2(const V2 &v, float2 a2, float2 s1, float2 s2, const V2 &u) {
    float2 c2;
    if (a2.x < 0.0625f && a2.y < 0.0625f)
        c2 = fma2(fma2(fma2(a2, bc(-1.f / 362880.f), bc(1.f / 5040.f)), a2, bc(-1.f / 120.f)), a2, bc(1.f / 6.f));
    else
        c2 = make_float2(jl_c2(a2.x, s1.x), jl_c2(a2.y, s1.y));
    const V2 vu = cross2(v, u), vvu = cross2(v, vu);
    const float2 ns2 = neg2(s2);
    return {fma2(c2, vvu.x, fma2(ns2, vu.x, u.x)), fma2(c2, vvu.y, fma2(ns2, vu.y, u.y)),
            fma2(c2, vvu.z, fma2(ns2, vu.z, u.z))};
}

// compensated running sum (window sums added to a float total)
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// MTX: several Tx coils (L.tx of them); without, one (the instantiations of
// the common case carry no per-coil loops: they cost registers and spills)
template <int P, bool GM, bool BOUND, bool MTX>
__global__ void __launch_bounds__(kAdjBlock, P <= 2 ? (BOUND ? 3 : 4) : 2) adjoint_kernel(AdjLaunch L) {
    extern __shared__ __align__(16) float adj_sm[];
    constexpr int kWarps = kAdjBlock / 32;
    const int TXN = MTX ? L.tx : 1, RS = adjoint_record_f4(TXN);    // Tx coils, float4 per step record
    float *win = adj_sm;                                            // [kAdjWin][3P][kAdjBlock]
    float *rfp = adj_sm + kAdjWin * 3 * P * kAdjBlock;              // [kAdjWin][warp][tx][2]
    float4 *wrec = reinterpret_cast<float4 *>(rfp + kAdjWin * kWarps * 2 * TXN);  // [kAdjWin][RS]
    float2 *rxs = reinterpret_cast<float2 *>(wrec + kAdjWin * RS);                // [rx][kAdjBlock]
    const int PR = P * L.rx;                                        // dL/dS values of one sample
    float2 *gbuf = rxs + L.rx * kAdjBlock;                          // [warp][2][PR]
    float2 *txs = gbuf + kWarps * 2 * PR;                           // [tx-1][kAdjBlock] TxCoil of coils >= 1
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // lanes of a voxel that split its receive term (8 coils or more): the
    // largest power of two dividing the spin count, at most a warp (groups
    // never straddle a warp); with fewer coils the split costs more than it
    // saves.  Not in the packed two-pool instantiation (its registers are
    // at the launch bound)
    constexpr bool kGroup = !(P == 2 && !BOUND);
    const int GS = kGroup && L.rx >= 8 ? min(L.S & -L.S, 32) : 1, gl = tid & (GS - 1);
    // with groups the threads take the isochromats spin-minor (a voxel's
    // spins on adjacent lanes), else voxel-minor (coalesced checkpoint
    // reads); iso indexes the [spin][voxel] arrays (checkpoints, gradients)
    const long long ithr = (long long)blockIdx.x * kAdjBlock + tid;
    const bool active = ithr < L.n_iso;
    const int n = L.n_act;
    const int v = active ? (int)(GS > 1 ? ithr / L.S : ithr % n) : 0;
    const int s = active ? (int)(GS > 1 ? ithr % L.S : ithr / n) : 0;
    const long long iso = GS > 1 ? (long long)s * n + v : ithr;  // (voxel-minor: the thread index itself)
    // exchange channel of the rate from pool a to pool b (ME: a*P+b, GM: b*P+a)
    auto ch = [](int a, int b) { return GM ? b * P + a : a * P + b; };

    // ---- per-isochromat constants ------------------------------------------
    float om[4] = {0.f, 0.f, 0.f, 0.f}, wres[P], rhoS[P], t1[P], t2[P];
    float kc[P * P];
    float2 txc = make_float2(0.f, 0.f);
    float3 m[P];
#pragma unroll
    for (int i = 0; i < P * P; ++i) kc[i] = 0.f;
#pragma unroll
    for (int t = 0; t < P; ++t) {
        wres[t] = rhoS[t] = t1[t] = t2[t] = 0.f;
        m[t] = make_float3(0.f, 0.f, 0.f);
    }
    if (active) {
        om[0] = L.gyro * L.db0[v];
        om[1] = L.gyro * L.gxg[v];
        om[2] = L.gyro * L.gyg[v];
        om[3] = L.gyro * L.gzg[v];
        txc = L.txc[v];
#pragma unroll
        for (int t = 0; t < P; ++t) {
            const long long i = ((long long)t * L.S + s) * n + v;
            wres[t] = L.dwrnd[i] + L.cs2pi[t];
            rhoS[t] = L.rho[(long long)t * n + v] / (float)L.S;
            t1[t] = L.t1[(long long)t * n + v];
            t2[t] = L.t2[(long long)t * n + v];
        }
        if (L.kch)
#pragma unroll
            for (int i = 0; i < P * P; ++i) kc[i] = L.kch[(long long)i * n + v];
    }
    // this warp's asynchronous copy of sample a's dL/dS into its buffer b
    auto prefetch_g = [&](int a, int b) {
        float2 *dst = gbuf + (warp * 2 + b) * PR;
        const float2 *src = L.gsig + (long long)a * PR;
        for (int i = lane; i < PR; i += 32) cp_async8(dst + i, src + i);
        cp_async_commit();
    };
    // this thread's receive sensitivities, read once: every ADC step uses them
    for (int c = 0; c < L.rx; ++c)
        rxs[c * kAdjBlock + tid] = (active && L.rxc) ? L.rxc[(long long)c * n + v] : make_float2(1.f, 0.f);
    // and the further transmit coils' TxCoilmg exp(i TxCoilpe) (rf steps)
    for (int c = 1; c < TXN; ++c)
        txs[(c - 1) * kAdjBlock + tid] = active ? L.txc[(long long)c * n + v] : make_float2(0.f, 0.f);
    // a pool with T1, T2 or Rho zero is left alone (BlochKernel.cuh:103)
    bool on[P], bnd[P];
#pragma unroll
    for (int t = 0; t < P; ++t) {
        on[t] = active && t1[t] != 0.f && t2[t] != 0.f && rhoS[t] != 0.f;
        bnd[t] = BOUND && (L.bound >> t & 1u);
    }
    bool anyoff = false;
#pragma unroll
    for (int t = 0; t < P; ++t) anyoff = anyoff || !on[t];
    // bound pools: (gamma |TxCoil|)^2, and the lineshape G, its slope dG/da
    // and a at the rf frequency lsw (2 pi f) of the last rf step
    const float gtx2 = L.gyro * L.gyro * fmaf(txc.x, txc.x, txc.y * txc.y);
    float lsG[P], lsD[P], lsA[P];
#pragma unroll
    for (int t = 0; t < P; ++t) lsG[t] = lsD[t] = lsA[t] = 0.f;
    float lsw = 0.f;
    bool lsok = false;
    auto lineshapes = [&](float wrf) {
        if (lsok && wrf == lsw) return;
        const float freq = wrf * 0.15915494309189535f;
#pragma unroll
        for (int t = 0; t < P; ++t) {
            if (!bnd[t] || !on[t]) continue;
            const float a = fmaf((float)(2 * kPiRef), freq, om[0]) * t2[t];
            const float2 gs = lineshape_slope(a, t2[t]);
            lsG[t] = gs.x;
            lsD[t] = gs.y;
            lsA[t] = a;
        }
        lsw = wrf;
        lsok = true;
    };
    // saturation W / G = pi (gamma |TxCoil| |A|)^2 of an rf step (the forward
    // scan's arithmetic: b1 = |A| |TxCoil|)
    auto sat_wg = [&](float4 r1) {
        const float b1 = sqrtf(fmaf(r1.x, r1.x, r1.y * r1.y)) * sqrtf(fmaf(txc.x, txc.x, txc.y * txc.y));
        const float bg = b1 * L.gyro;
        return (float)kPiRef * bg * bg;
    };

    // ---- per-dt coefficients ------------------------------------------------
    // map: d2, d1, cc, fin; gradient: hT1 (of l.z mr.z), hR (of l.z), hT2 (of
    // l.xy mr.xy), e2, e1 (outflow rates, of l.xy mr.xy and l.z mr.z), ffin.
    // Without bound pools T1, T2 and K enter only here (dt changes are rare):
    // read again from global memory, they hold no registers in the step loop
    constexpr bool kLazy = !BOUND;
    auto par_t1 = [&](int t) { return kLazy ? (active ? __ldg(L.t1 + (long long)t * n + v) : 0.f) : t1[t]; };
    auto par_t2 = [&](int t) { return kLazy ? (active ? __ldg(L.t2 + (long long)t * n + v) : 0.f) : t2[t]; };
    auto par_k = [&](int i) { return kLazy ? ((active && L.kch) ? __ldg(L.kch + (long long)i * n + v) : 0.f) : kc[i]; };
    float d1[P], d2[P], y1[P], fin[P][P], hT1[P], hR[P], hT2[P], e1[P], e2[P];
    // one Tx coil, no bound pools: the coil's sensitivity scaled by -dt gamma
    // (dv_xy / dA of an rf step), set with dt
    constexpr bool kTcs = !MTX && !BOUND;
    float2 tcs = make_float2(0.f, 0.f);
    // packed two-pool path: (1 - f_tp) dt of each inflow, zero for a pool that is off
    constexpr bool kPk = P == 2 && !BOUND;
    float gin[kPk ? P : 1][kPk ? P : 1];
    bool selfx = false;  // (packed path) some pool of the voxel exchanges with itself
    float dtc = 0.f;  // dt of these coefficients
    auto set_dt = [&](float dt) {
#pragma unroll
        for (int t = 0; t < P; ++t) {
            const float t1t = par_t1(t), t2t = par_t2(t);
            const float y1t = on[t] ? one_minus_exp(dt / t1t) : 0.f;
            const float y2t = on[t] ? one_minus_exp(dt / t2t) : 0.f;
            float ksum = 0.f, ksum_t = 0.f;  // outflow: all partners, transverse partners
#pragma unroll
            for (int p = 0; p < P; ++p) {
                fin[t][p] = 0.f;
                if (GM && p == t) continue;
                const float kgo = par_k(ch(t, p)), kin = par_k(ch(p, t));
                ksum += kgo;
                if (!(L.mtc && bnd[p])) ksum_t += kgo;
                if (on[t] && kin != 0.f) fin[t][p] = one_minus_exp(dt * kin);
            }
            const float yot = on[t] ? one_minus_exp(dt * ksum) : 0.f;
            // MT / CEST: the transverse outflow leaves out the bound pool
            const float yot_t = L.mtc ? (on[t] ? one_minus_exp(dt * ksum_t) : 0.f) : yot;
            y1[t] = y1t;
            d1[t] = (1.f - yot) * (1.f - y1t);
            d2[t] = (1.f - yot_t) * (1.f - y2t);
            // dy1/dT1 = -(1 - y1) dt / T1^2, dyo/dk = (1 - yo) dt
            const float fT1 = on[t] ? -(1.f - y1t) * dt / (t1t * t1t) : 0.f;
            const float fT2 = on[t] ? -(1.f - y2t) * dt / (t2t * t2t) : 0.f;
            const float fyo = (1.f - yot) * dt;
            hT1[t] = -(1.f - yot) * fT1;
            hR[t] = rhoS[t] * fT1;
            hT2[t] = -(1.f - yot_t) * fT2;
            e2[t] = -(1.f - y2t) * (1.f - yot_t) * dt;
            e1[t] = -(1.f - y1t) * fyo;
            if (!on[t]) d1[t] = d2[t] = e1[t] = e2[t] = 0.f;  // (an off pool is left alone)
            if constexpr (kPk) {
#pragma unroll
                for (int p = 0; p < P; ++p) gin[t][p] = on[t] && !(GM && p == t) ? (1.f - fin[t][p]) * dt : 0.f;
            }
        }
        if constexpr (kPk) selfx = !GM && (fin[0][0] != 0.f || fin[1][1] != 0.f);
        if constexpr (kTcs) {
            const float2 tc = active ? __ldg(L.txc + v) : make_float2(0.f, 0.f);
            const float sc = -dt * L.gyro;
            tcs = make_float2(sc * tc.x, sc * tc.y);
        }
        dtc = dt;
    };
    // ---- per-state rotation of free steps -----------------------------------
    float cth[P], sth[P];
    // off-resonance of the step's gradients, gamma (dB0 + G.r), set with them
    // (dB0 and r stay in registers: reading them again at every gradient
    // change stalled the loop more than the registers cost)
    float wcc = 0.f;
    auto set_state = [&](float dt, float4 r0) {
        const float wc = fmaf(om[3], r0.y, fmaf(om[2], r0.z, fmaf(om[1], r0.w, om[0])));
        wcc = wc;
#pragma unroll
        for (int t = 0; t < P; ++t) sincos_cw((wc + wres[t]) * dt, sth[t], cth[t]);
    };
    // rotation vector of an rf step (step j of the window): -dt (gamma Bx,
    // gamma By, w_t), B = sum over the Tx coils of TxCoil_c A_c (a coil that
    // is off has A_c = 0)
    auto rf_vxy = [&](float dt, float4 r1, int j) {
        if constexpr (kTcs)
            return make_float2(fmaf(tcs.x, r1.x, -tcs.y * r1.y), fmaf(tcs.x, r1.y, tcs.y * r1.x));
        const float sc = -dt * L.gyro;
        float bx = fmaf(txc.x, r1.x, -txc.y * r1.y), by = fmaf(txc.x, r1.y, txc.y * r1.x);
        for (int c = 1; c < TXN; ++c) {
            const float2 tc = txs[(c - 1) * kAdjBlock + tid];
            const float4 ra = wrec[RS * j + 3 + (c - 1)];
            bx = fmaf(tc.x, ra.x, fmaf(-tc.y, ra.y, bx));
            by = fmaf(tc.x, ra.y, fmaf(tc.y, ra.x, by));
        }
        return make_float2(sc * bx, sc * by);
    };
    // one forward step, m -> F(m) (step j of the window)
    auto fwd = [&](float dt, float4 r0, float4 r1, bool rf, int j) {
        if constexpr (kPk) {  // both pools at once (lanes = pools)
            const V2 mm = {make_float2(m[0].x, m[1].x), make_float2(m[0].y, m[1].y), make_float2(m[0].z, m[1].z)};
            V2 mr;
            if (rf) {
                const float2 vxy = rf_vxy(dt, r1, j);
                const float wz = wcc + r1.z;
                const V2 v = {bc(vxy.x), bc(vxy.y), make_float2(-dt * (wz + wres[0]), -dt * (wz + wres[1]))};
                const float2 a2 = fma2(v.z, v.z, bc(fmaf(vxy.x, vxy.x, vxy.y * vxy.y)));
                float2 s1, s2;
                rot_coeffs2(a2, s1, s2);
                mr = rot2(v, s1, s2, mm);
            } else {
                const float2 c = make_float2(cth[0], cth[1]), sn = make_float2(sth[0], sth[1]);
                mr = {fma2(mm.x, c, mul2(mm.y, sn)), fma2(neg2(mm.x), sn, mul2(mm.y, c)), mm.z};
            }
            const float2 D2 = make_float2(d2[0], d2[1]), D1 = make_float2(d1[0], d1[1]);
            const float2 fd = make_float2(fin[0][0], fin[1][1]);
            const float2 cz = make_float2(rhoS[0] * y1[0], rhoS[1] * y1[1]);
            // the partner's inflow f_tp m_p per lane as scalar fused multiply-adds
            // (a packed operand with its lanes swapped costs two moves)
            auto inflow = [&](float2 a, float2 mp) {
                return make_float2(fmaf(fin[0][1], mp.y, a.x), fmaf(fin[1][0], mp.x, a.y));
            };
            float2 ax = inflow(mul2(D2, mr.x), mm.x);
            float2 ay = inflow(mul2(D2, mr.y), mm.y);
            float2 az = inflow(fma2(D1, mr.z, cz), mm.z);
            if (selfx) {  // a pool's inflow from itself (a nonzero K diagonal)
                ax = fma2(fd, mm.x, ax);
                ay = fma2(fd, mm.y, ay);
                az = fma2(fd, mm.z, az);
            }
            if (on[0]) m[0] = make_float3(ax.x, ay.x, az.x);
            if (on[1]) m[1] = make_float3(ax.y, ay.y, az.y);
            return;
        }
        float3 mr[P];
        if (rf) {
            const float2 vxy = rf_vxy(dt, r1, j);
            const float wz = wcc + r1.z;
            float wg = 0.f;
            if (BOUND) {
                lineshapes(r1.z);
                wg = sat_wg(r1);
            }
#pragma unroll
            for (int t = 0; t < P; ++t) {
                if (bnd[t]) {
                    const float q = 1.f - one_minus_exp(wg * lsG[t] * dt);
                    mr[t] = make_float3(m[t].x, m[t].y, q * m[t].z);
                } else {
                    mr[t] = rot_apply(make_rot(make_float3(vxy.x, vxy.y, -dt * (wz + wres[t]))), m[t]);
                }
            }
        } else {
#pragma unroll
            for (int t = 0; t < P; ++t)
                mr[t] = bnd[t] ? m[t]
                               : make_float3(fmaf(m[t].x, cth[t], m[t].y * sth[t]),
                                             fmaf(-m[t].x, sth[t], m[t].y * cth[t]), m[t].z);
        }
        float3 nm[P];
#pragma unroll
        for (int t = 0; t < P; ++t) {
            float3 a = make_float3(d2[t] * mr[t].x, d2[t] * mr[t].y, fmaf(d1[t], mr[t].z, rhoS[t] * y1[t]));
            if (bnd[t]) a = make_float3(m[t].x, m[t].y, a.z);  // transverse held
#pragma unroll
            for (int p = 0; p < P; ++p) {
                // (MT / CEST: no transverse inflow from the bound pool)
                if (!bnd[t] && !(L.mtc && bnd[p])) {
                    a.x = fmaf(fin[t][p], m[p].x, a.x);
                    a.y = fmaf(fin[t][p], m[p].y, a.y);
                }
                a.z = fmaf(fin[t][p], m[p].z, a.z);
            }
            nm[t] = on[t] ? a : m[t];
        }
#pragma unroll
        for (int t = 0; t < P; ++t) m[t] = nm[t];
    };

    const long long N = L.n_steps;
    const long long nwin = (N + kAdjWin - 1) / kAdjWin;
    const long long cs = (long long)3 * P;  // checkpoint components
    // (dt, Gz, Gy, Gx) of the coefficients in registers
    float4 cur = make_float4(-1.f, 0.f, 0.f, 0.f);
    // the nk steps of the window in wrec from the state m: with `states`,
    // the state before each step into shared memory and the last step not
    // taken (the backward walk starts from it); without, every step taken
    auto recompute = [&](int nk, float *states) {
        for (int j = 0; j < nk; ++j) {
            const float4 r0 = wrec[RS * j], r1 = wrec[RS * j + 1];
            const int flags = __float_as_int(r1.w);
            const float dt = r0.x;
            if (states && kPk) {  // packed: (pool 0, pool 1) of a component as one float2
                float2 *ws = reinterpret_cast<float2 *>(states + j * 3 * P * kAdjBlock) + tid;
                ws[0] = make_float2(m[0].x, m[1].x);
                ws[kAdjBlock] = make_float2(m[0].y, m[1].y);
                ws[2 * kAdjBlock] = make_float2(m[0].z, m[1].z);
            } else if (states) {
                float *ws = states + j * 3 * P * kAdjBlock + tid;
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    ws[(3 * t + 0) * kAdjBlock] = m[t].x;
                    ws[(3 * t + 1) * kAdjBlock] = m[t].y;
                    ws[(3 * t + 2) * kAdjBlock] = m[t].z;
                }
            }
            if (j == 0) {  // the coefficients of the window's first step, if not in registers
                if (dt != cur.x) set_dt(dt);
                if (dt != cur.x || r0.y != cur.y || r0.z != cur.z || r0.w != cur.w) set_state(dt, r0);
                cur = r0;
            } else if (flags & (kFlagDt | kFlagState)) {
                if (flags & kFlagDt) set_dt(dt);
                if (flags & kFlagState) set_state(dt, r0);
                cur = r0;
            }
            if (!states || j + 1 < nk) fwd(dt, r0, r1, (flags & kFlagRf) != 0, j);
        }
    };

    // ---- backward sweep -----------------------------------------------------
    float3 lam[P];
#pragma unroll
    for (int t = 0; t < P; ++t) lam[t] = make_float3(0.f, 0.f, 0.f);
    KSum gT1[P], gT2[P], grho[P], gw[P], gk[P * P];
    for (long long w = nwin - 1; w >= 0; --w) {
        const long long k0 = w * kAdjWin;
        const int nk = (int)min((long long)kAdjWin, N - k0);
        // two-level checkpoints (seg > 1): entering a segment (its last
        // window first), rebuild the states at its windows' starts from the
        // segment's stored checkpoint into ck2
        const long long wseg = w / L.seg * L.seg;  // the segment's first window
        if (L.seg > 1) {
            float *c2 = L.ck2 + iso;
            if (w == nwin - 1 || w % L.seg == L.seg - 1) {
                if (active) {
                    const float *cp = L.ckpt + (w / L.seg) * cs * L.n_iso + iso;
#pragma unroll
                    for (int t = 0; t < P; ++t)
                        m[t] = make_float3(cp[(3 * t + 0) * L.n_iso], cp[(3 * t + 1) * L.n_iso],
                                           cp[(3 * t + 2) * L.n_iso]);
                }
                for (long long u = wseg; u <= w; ++u) {
                    if (active) {
                        float *o = c2 + (u - wseg) * cs * L.n_iso;
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            o[(3 * t + 0) * L.n_iso] = m[t].x;
                            o[(3 * t + 1) * L.n_iso] = m[t].y;
                            o[(3 * t + 2) * L.n_iso] = m[t].z;
                        }
                    }
                    if (u == w) break;
                    // window u's records, then all its steps (full windows: u < w)
                    __syncthreads();
                    if (tid < RS * kAdjWin) wrec[tid] = __ldg(L.rec + u * kAdjWin * RS + tid);
                    __syncthreads();
                    recompute(kAdjWin, nullptr);
                }
                __syncthreads();
            }
        }
        // this window's starting state
        const float *wck = L.seg > 1 ? L.ck2 + (w - wseg) * cs * L.n_iso + iso : L.ckpt + w * cs * L.n_iso + iso;
        // the window's step records, staged in shared memory
        if (tid < RS * nk) wrec[tid] = __ldg(L.rec + k0 * RS + tid);
        __syncthreads();
        // dL/dS of the window's last step (the first one the backward walk
        // takes), fetched while the states are recomputed
        if (__float_as_int(wrec[RS * (nk - 1) + 2].x) >= 0)
            prefetch_g(__float_as_int(wrec[RS * (nk - 1) + 2].x), (nk - 1) & 1);
        // recompute the window's states (before each step) into shared memory
        if (active) {
#pragma unroll
            for (int t = 0; t < P; ++t)
                m[t] = make_float3(wck[(3 * t + 0) * L.n_iso], wck[(3 * t + 1) * L.n_iso], wck[(3 * t + 2) * L.n_iso]);
        }
        recompute(nk, win);
        // window partial sums of the parameter gradients
        float wT1[P], wT2[P], wrho[P], ww[P], wk[P * P];
#pragma unroll
        for (int t = 0; t < P; ++t) wT1[t] = wT2[t] = wrho[t] = ww[t] = 0.f;
#pragma unroll
        for (int i = 0; i < P * P; ++i) wk[i] = 0.f;
        // the coefficients in registers are those of the window's last step
        int fnext = 0;  // flags of step j + 1 (the step before in this walk)
        for (int j = nk - 1; j >= 0; --j) {
            const float4 r0 = wrec[RS * j], r1 = wrec[RS * j + 1], r2 = wrec[RS * j + 2];
            const int flags = __float_as_int(r1.w);
            const float dt = r0.x;
            if (j < nk - 1) {  // coefficients of step j, if step j + 1 changed them
                const int fn = fnext;
                if (fn & kFlagDt) set_dt(dt);
                if (fn & kFlagState) set_state(dt, r0);
                if (fn & (kFlagDt | kFlagState)) cur = r0;
            }
            fnext = flags;
            // dL/dS of step j - 1 (the next step back), if it samples: into the
            // buffer step j + 1 read, once every lane of the warp is done with it
            bool pend = false;
            if (j >= 1) {
                const int an = __float_as_int(wrec[RS * (j - 1) + 2].x);
                if (an >= 0) {
                    __syncwarp();
                    prefetch_g(an, (j - 1) & 1);
                    pend = true;
                }
            }
            const bool rf = (flags & kFlagRf) != 0;
            float3 mk[P];
            V2 Mk{};  // packed path: the state before the step, lanes = pools
            if constexpr (kPk) {
                const float2 *ws = reinterpret_cast<const float2 *>(win + j * 3 * P * kAdjBlock) + tid;
                Mk = {ws[0], ws[kAdjBlock], ws[2 * kAdjBlock]};
            } else {
                const float *ws = win + j * 3 * P * kAdjBlock + tid;
#pragma unroll
                for (int t = 0; t < P; ++t)
                    mk[t] = make_float3(ws[(3 * t + 0) * kAdjBlock], ws[(3 * t + 1) * kAdjBlock],
                                        ws[(3 * t + 2) * kAdjBlock]);
            }
            float2 vxy = make_float2(0.f, 0.f);
            float wz = 0.f, wg = 0.f;
            if (rf) {
                vxy = rf_vxy(dt, r1, j);
                wz = wcc + r1.z;
                if (BOUND) {
                    lineshapes(r1.z);
                    wg = sat_wg(r1);
                }
            }
            float3 nl[P];
#pragma unroll
            for (int t = 0; t < P; ++t) nl[t] = make_float3(0.f, 0.f, 0.f);
            float2 gv = make_float2(0.f, 0.f);  // dL/d(vx, vy) of the step, summed over the pools
            float2 gs = make_float2(0.f, 0.f);  // dL/dA through the bound pools' saturation
            if constexpr (kPk) {
                // both pools at once (lanes = pools); a pool that is off has zero
                // relaxation, exchange and gradient coefficients (set_dt) and
                // passes its adjoint through
                const V2 M = Mk;
                const V2 l = {make_float2(lam[0].x, lam[1].x), make_float2(lam[0].y, lam[1].y),
                              make_float2(lam[0].z, lam[1].z)};
                V2 v{}, mr;
                float2 a2 = bc(0.f), s1 = bc(0.f), s2 = bc(0.f);
                const float2 c = make_float2(cth[0], cth[1]), sn = make_float2(sth[0], sth[1]);
                if (rf) {
                    v = {bc(vxy.x), bc(vxy.y), make_float2(-dt * (wz + wres[0]), -dt * (wz + wres[1]))};
                    a2 = fma2(v.z, v.z, bc(fmaf(vxy.x, vxy.x, vxy.y * vxy.y)));
                    rot_coeffs2(a2, s1, s2);
                    mr = rot2(v, s1, s2, M);
                } else {
                    mr = {fma2(M.x, c, mul2(M.y, sn)), fma2(neg2(M.x), sn, mul2(M.y, c)), M.z};
                }
                // relaxation / recovery parameters
                const float2 gd2 = fma2(l.x, mr.x, mul2(l.y, mr.y)), gd1 = mul2(l.z, mr.z);
                const float2 t1w = fma2(gd1, make_float2(hT1[0], hT1[1]),
                                        fma2(l.z, make_float2(hR[0], hR[1]), make_float2(wT1[0], wT1[1])));
                const float2 t2w = fma2(gd2, make_float2(hT2[0], hT2[1]), make_float2(wT2[0], wT2[1]));
                const float2 rw = fma2(l.z, make_float2(y1[0], y1[1]), make_float2(wrho[0], wrho[1]));
                wT1[0] = t1w.x, wT1[1] = t1w.y, wT2[0] = t2w.x, wT2[1] = t2w.y, wrho[0] = rw.x, wrho[1] = rw.y;
                // exchange rates: the outflow of each pool (every channel out of it)
                // and the inflow to it from the magnetisation before the step
                const float2 go = fma2(gd1, make_float2(e1[0], e1[1]), mul2(gd2, make_float2(e2[0], e2[1])));
                // l_t . m_other per lane (scalar: no swapped operands)
                const float2 lx = make_float2(fmaf(l.x.x, M.x.y, fmaf(l.y.x, M.y.y, l.z.x * M.z.y)),
                                              fmaf(l.x.y, M.x.x, fmaf(l.y.y, M.y.x, l.z.y * M.z.x)));
                if (!GM) {
                    // the diagonal channels: the outflow, and the inflow from itself
                    // (its derivative (1 - f) dt is nonzero at a zero rate too)
                    const float2 ls = dot2(l, M);
                    wk[ch(0, 0)] += fmaf(ls.x, gin[0][0], go.x);
                    wk[ch(1, 1)] += fmaf(ls.y, gin[1][1], go.y);
                }
                wk[ch(0, 1)] += fmaf(lx.y, gin[1][0], go.x);
                wk[ch(1, 0)] += fmaf(lx.x, gin[0][1], go.y);
                const float2 fd = make_float2(fin[0][0], fin[1][1]);
                // the partner's inflow adjoint: lane t takes f_pt lambda_p
                V2 n2 = {make_float2(fin[1][0] * l.x.y, fin[0][1] * l.x.x),
                         make_float2(fin[1][0] * l.y.y, fin[0][1] * l.y.x),
                         make_float2(fin[1][0] * l.z.y, fin[0][1] * l.z.x)};
                if (selfx) n2 = {fma2(fd, l.x, n2.x), fma2(fd, l.y, n2.y), fma2(fd, l.z, n2.z)};
                // adjoint with respect to the rotated magnetisation
                const float2 D2 = make_float2(d2[0], d2[1]), D1 = make_float2(d1[0], d1[1]);
                const V2 lr = {mul2(D2, l.x), mul2(D2, l.y), mul2(D1, l.z)};
                const V2 u = cross2(mr, lr);
                float2 wwv = make_float2(ww[0], ww[1]);
                if (rf) {
                    const V2 g = jlt2(v, a2, s1, s2, u);
                    wwv = fma2(bc(-dt), g.z, wwv);
                    gv.x += g.x.x + g.x.y;
                    gv.y += g.y.x + g.y.y;
                    const V2 b = rot2(V2{neg2(v.x), neg2(v.y), neg2(v.z)}, s1, s2, lr);
                    n2 = {add2(n2.x, b.x), add2(n2.y, b.y), add2(n2.z, b.z)};
                } else {
                    wwv = fma2(bc(-dt), u.z, wwv);
                    n2.x = add2(n2.x, fma2(c, lr.x, neg2(mul2(sn, lr.y))));
                    n2.y = add2(n2.y, fma2(sn, lr.x, mul2(c, lr.y)));
                    n2.z = add2(n2.z, lr.z);
                }
                ww[0] = wwv.x, ww[1] = wwv.y;
                if (anyoff) {  // a pool that is off passes its adjoint through
                    const float2 off = make_float2(on[0] ? 0.f : 1.f, on[1] ? 0.f : 1.f);
                    n2 = {fma2(off, l.x, n2.x), fma2(off, l.y, n2.y), fma2(off, l.z, n2.z)};
                }
                nl[0] = make_float3(n2.x.x, n2.y.x, n2.z.x);
                nl[1] = make_float3(n2.x.y, n2.y.y, n2.z.y);
            }
#pragma unroll
            for (int t = 0; t < (kPk ? 0 : P); ++t) {
                if (!on[t]) {
                    nl[t].x += lam[t].x;
                    nl[t].y += lam[t].y;
                    nl[t].z += lam[t].z;
                    continue;
                }
                if (bnd[t]) {
                    // bound pool: transverse held, z saturated (rf) then relaxed and exchanged
                    const float q = rf ? 1.f - one_minus_exp(wg * lsG[t] * dt) : 1.f;
                    const float3 l = lam[t];
                    const float mrz = q * mk[t].z;
                    const float gd1 = l.z * mrz;
                    wT1[t] = fmaf(gd1, hT1[t], fmaf(l.z, hR[t], wT1[t]));
                    wrho[t] = fmaf(l.z, y1[t], wrho[t]);
                    const float go_g = gd1 * e1[t];
#pragma unroll
                    for (int p = 0; p < P; ++p) {
                        if (GM && p == t) continue;
                        wk[ch(t, p)] += go_g;
                        wk[ch(p, t)] = fmaf(l.z * mk[p].z, (1.f - fin[t][p]) * dtc, wk[ch(p, t)]);
                        nl[p].z = fmaf(fin[t][p], l.z, nl[p].z);
                    }
                    const float lz = d1[t] * l.z;
                    nl[t].x += l.x;
                    nl[t].y += l.y;
                    nl[t].z = fmaf(q, lz, nl[t].z);
                    if (rf) {
                        // dL/dW = dL/dq dq/dW, dq/dW = -dt q
                        const float dw = -dt * lz * mrz;
                        const float cA = 2.f * (float)kPiRef * gtx2 * lsG[t] * dw;
                        gs.x = fmaf(cA, r1.x, gs.x);
                        gs.y = fmaf(cA, r1.y, gs.y);
                        const float dwg = dw * wg;  // dL/dG
                        ww[t] = fmaf(dwg * lsD[t], t2[t], ww[t]);
                        wT2[t] = fmaf(dwg, fmaf(lsA[t], lsD[t], lsG[t]) / t2[t], wT2[t]);
                    }
                    continue;
                }
                // rotation of this step
                Rot R;
                float3 mr;
                if (rf) {
                    R = make_rot(make_float3(vxy.x, vxy.y, -dt * (wz + wres[t])));
                    mr = rot_apply(R, mk[t]);
                } else {
                    mr = make_float3(fmaf(mk[t].x, cth[t], mk[t].y * sth[t]), fmaf(-mk[t].x, sth[t], mk[t].y * cth[t]),
                                     mk[t].z);
                }
                const float3 l = lam[t];
                // relaxation / recovery parameters
                const float gd2 = fmaf(l.x, mr.x, l.y * mr.y), gd1 = l.z * mr.z;
                wT1[t] = fmaf(gd1, hT1[t], fmaf(l.z, hR[t], wT1[t]));
                wT2[t] = fmaf(gd2, hT2[t], wT2[t]);
                wrho[t] = fmaf(l.z, y1[t], wrho[t]);
                // exchange rates: the outflow of t (yo_t) and the inflow to t (f_tp)
                const float go_l = gd1 * e1[t], go_t = gd2 * e2[t];
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    if (GM && p == t) continue;
                    wk[ch(t, p)] += (L.mtc && bnd[p]) ? go_l : go_l + go_t;
                    // inflow to t from p's magnetisation before the step (MT /
                    // CEST: the bound pool's longitudinal part only)
                    const bool xy = !(L.mtc && bnd[p]);
                    // df_tp/dk_pt = (1 - f_tp) dt
                    const float lm = xy ? dot3(l, mk[p]) : l.z * mk[p].z;
                    wk[ch(p, t)] = fmaf(lm, (1.f - fin[t][p]) * dtc, wk[ch(p, t)]);
                    if (xy) {
                        nl[p].x = fmaf(fin[t][p], l.x, nl[p].x);
                        nl[p].y = fmaf(fin[t][p], l.y, nl[p].y);
                    }
                    nl[p].z = fmaf(fin[t][p], l.z, nl[p].z);
                }
                // adjoint with respect to the rotated magnetisation
                const float3 lr = make_float3(d2[t] * l.x, d2[t] * l.y, d1[t] * l.z);
                const float3 u = cross3(mr, lr);
                if (rf) {
                    const float3 g = jl_t(R, u);
                    ww[t] = fmaf(-dt, g.z, ww[t]);
                    gv.x += g.x;
                    gv.y += g.y;
                    const float3 b = rot_apply_t(R, lr);
                    nl[t].x += b.x;
                    nl[t].y += b.y;
                    nl[t].z += b.z;
                } else {
                    ww[t] = fmaf(-dt, u.z, ww[t]);
                    nl[t].x += fmaf(cth[t], lr.x, -sth[t] * lr.y);
                    nl[t].y += fmaf(sth[t], lr.x, cth[t] * lr.y);
                    nl[t].z += lr.z;
                }
            }
            // receive before the step: lambda += sum_c G R_c
            const int a = __float_as_int(r2.x);
            if (a >= 0) {  // this step's dL/dS copy complete and visible to the warp
                if (pend)
                    cp_async_wait<1>();
                else
                    cp_async_wait<0>();
                __syncwarp();
            }
            if (!kGroup && a >= 0 && active) {  // (bound pools are not received)
                // per pool: sum_c G R_c as four independent partial sums
                // (re and im of the even and of the odd coils)
                const float2 *ga = gbuf + (warp * 2 + (j & 1)) * PR;
                float4 src[P];
#pragma unroll
                for (int t = 0; t < P; ++t) src[t] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
                for (int c0 = 0; c0 < L.rx; c0 += 8) {
#pragma unroll
                    for (int c = c0; c < c0 + 8; ++c) {
                        if (c >= L.rx) break;
                        const float2 rc = rxs[c * kAdjBlock + tid];
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            if (bnd[t] || (L.mtc && t != 0)) continue;  // MT / CEST receive pool 0
                            const float2 g = ga[t * L.rx + c];
                            if (c & 1) {
                                src[t].z = fmaf(g.x, rc.x, fmaf(-g.y, rc.y, src[t].z));
                                src[t].w = fmaf(g.x, rc.y, fmaf(g.y, rc.x, src[t].w));
                            } else {
                                src[t].x = fmaf(g.x, rc.x, fmaf(-g.y, rc.y, src[t].x));
                                src[t].y = fmaf(g.x, rc.y, fmaf(g.y, rc.x, src[t].y));
                            }
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    nl[t].x += src[t].x + src[t].z;
                    nl[t].y += src[t].y + src[t].w;
                }
            }
            if (kGroup && a >= 0) {  // (bound pools are not received)
                // per pool sum_c G R_c: it depends on the voxel and the sample,
                // not on the spin, so lane gl of a voxel's group of GS lanes
                // sums coils gl, gl + GS, ... (two independent partial sums,
                // re and im) and the group adds its partial sums with shuffles
                const float2 *ga = gbuf + (warp * 2 + (j & 1)) * PR;
                const int rxn = L.rx;
                float4 src[P];
#pragma unroll
                for (int t = 0; t < P; ++t) src[t] = make_float4(0.f, 0.f, 0.f, 0.f);
                auto coil = [&](int c, bool second) {
                    const float2 rc = rxs[c * kAdjBlock + tid];
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        if (bnd[t] || (L.mtc && t != 0)) continue;  // MT / CEST receive pool 0
                        const float2 g = ga[t * rxn + c];
                        if (second) {
                            src[t].z = fmaf(g.x, rc.x, fmaf(-g.y, rc.y, src[t].z));
                            src[t].w = fmaf(g.x, rc.y, fmaf(g.y, rc.x, src[t].w));
                        } else {
                            src[t].x = fmaf(g.x, rc.x, fmaf(-g.y, rc.y, src[t].x));
                            src[t].y = fmaf(g.x, rc.y, fmaf(g.y, rc.x, src[t].y));
                        }
                    }
                };
                if (active) {
#pragma unroll 1
                    for (int c0 = gl; c0 < rxn; c0 += 8 * GS) {
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const int c = c0 + k * GS;
                            if (c >= rxn) break;
                            coil(c, (k & 1) != 0);
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    if (bnd[t] || (L.mtc && t != 0)) continue;
                    float sx = src[t].x + src[t].z, sy = src[t].y + src[t].w;
                    for (int o = 1; o < GS; o <<= 1) {  // (block-uniform: every lane of the warp takes part)
                        sx += __shfl_xor_sync(0xffffffffu, sx, o);
                        sy += __shfl_xor_sync(0xffffffffu, sy, o);
                    }
                    if (active) {
                        nl[t].x += sx;
                        nl[t].y += sy;
                    }
                }
            }
            // (an inactive thread's adjoint stays zero: its pools are off, its
            // state and coefficients zero, and it takes no receive term)
#pragma unroll
            for (int t = 0; t < P; ++t) lam[t] = nl[t];
            // rf gradient of this step: dB/dA = TxCoil, dv/dB = -dt gamma, so
            // dL/dA = -dt gamma conj(TxCoil) (gvx + i gvy) + the saturation's
            // share, summed over the warp
            if (rf) {
                const float sc = -dt * L.gyro;
                for (int c = 0; c < TXN; ++c) {  // dB/dA_c = TxCoil_c
                    const float2 tc = c == 0 ? txc : txs[(c - 1) * kAdjBlock + tid];
                    float2 gA = kTcs ? make_float2(fmaf(tcs.x, gv.x, tcs.y * gv.y), fmaf(tcs.x, gv.y, -tcs.y * gv.x))
                                     : make_float2(sc * fmaf(tc.x, gv.x, tc.y * gv.y), sc * fmaf(tc.x, gv.y, -tc.y * gv.x));
                    if (BOUND && c == 0) gA = make_float2(gA.x + gs.x, gA.y + gs.y);
                    // both components in one reduction: the first exchange leaves
                    // lanes 0-15 with partial sums of x and lanes 16-31 with those
                    // of y, four more exchanges finish each half (lane 0: x, 16: y)
                    const bool hi = (lane & 16) != 0;
                    float part = hi ? gA.y : gA.x;
                    part += __shfl_xor_sync(0xffffffffu, hi ? gA.x : gA.y, 16);
#pragma unroll
                    for (int o = 8; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                    if ((lane & 15) == 0) rfp[((j * kWarps + warp) * TXN + c) * 2 + (hi ? 1 : 0)] = part;
                }
            }
        }
#pragma unroll
        for (int t = 0; t < P; ++t) {
            gT1[t].add(wT1[t]);
            gT2[t].add(wT2[t]);
            grho[t].add(wrho[t]);
            gw[t].add(ww[t]);
        }
#pragma unroll
        for (int i = 0; i < P * P; ++i) gk[i].add(wk[i]);
        // the window's rf gradients, summed over the block, into their FP64 slots
        __syncthreads();
        if (tid < nk) {
            const int ri = __float_as_int(wrec[RS * tid + 2].y);
            if (ri >= 0 && (__float_as_int(wrec[RS * tid + 1].w) & kFlagRf)) {
                for (int c = 0; c < TXN; ++c) {  // slots [rf step][coil][re, im]
                    float gx = 0.f, gy = 0.f;
#pragma unroll
                    for (int q = 0; q < kWarps; ++q) {
                        gx += rfp[((tid * kWarps + q) * TXN + c) * 2 + 0];
                        gy += rfp[((tid * kWarps + q) * TXN + c) * 2 + 1];
                    }
                    atomicAdd(&L.grf[2 * ((long long)ri * TXN + c)], (double)gx);
                    atomicAdd(&L.grf[2 * ((long long)ri * TXN + c) + 1], (double)gy);
                }
            }
        }
        __syncthreads();
    }

    cp_async_wait<0>();

    // ---- per-isochromat outputs -------------------------------------------
    if (!active) return;
    float *g = L.giso + iso;
    const long long st = L.n_iso;
    int f = 0;
#pragma unroll
    for (int t = 0; t < P; ++t) g[(f + t) * st] = gT1[t].s;
    f += P;
#pragma unroll
    for (int t = 0; t < P; ++t) g[(f + t) * st] = gT2[t].s;
    f += P;
#pragma unroll
    for (int t = 0; t < P; ++t) g[(f + t) * st] = grho[t].s / (float)L.S;  // dc/dRho = y1 / S
    f += P;
    float gdb0 = 0.f;
#pragma unroll
    for (int t = 0; t < P; ++t) gdb0 = fmaf(L.gyro, gw[t].s, gdb0);
    g[f * st] = gdb0;
    f += 1;
#pragma unroll
    for (int i = 0; i < P * P; ++i) g[(f + i) * st] = gk[i].s;
    f += P * P;
#pragma unroll
    for (int t = 0; t < P; ++t) {  // dL/d(initial Mx, My, Mz)
        g[(f + t) * st] = lam[t].x;
        g[(f + P + t) * st] = lam[t].y;
        g[(f + 2 * P + t) * st] = lam[t].z;
    }
}

template <int P, bool GM, bool BOUND = false>
cudaError_t go(const AdjLaunch &L, cudaStream_t st) {
    const size_t smem = adjoint_smem_bytes(P, L.rx, L.tx);
    // (bound pools run with one Tx coil only: the plan refuses more)
    auto k = (!BOUND && L.tx > 1) ? adjoint_kernel<P, GM, BOUND, !BOUND> : adjoint_kernel<P, GM, BOUND, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long blocks = (L.n_iso + kAdjBlock - 1) / kAdjBlock;
    k<<<(unsigned)blocks, kAdjBlock, smem, st>>>(L);
    return cudaGetLastError();
}

}  // namespace

namespace {
// MT (layout 2: channel 1 = K12 (0 -> 1), 2 = K21 (1 -> 0)) and CEST
// (layout 3: 0 = 0 -> MT, P-1 = MT -> 0, t-1 = 0 -> t, t+P-2 = t -> 0)
// exchange channels into the general model's layout (p*P+t = rate t -> p)
__global__ void remap_k_mtc(int P, int layout, const float *__restrict__ src, float *dst, int n_act) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_act) return;
    for (int t = 0; t < P; ++t)
        for (int p = 0; p < P; ++p) {
            int c = -1;
            if (layout == 2) c = (t == 0 && p == 1) ? 1 : ((t == 1 && p == 0) ? 2 : -1);
            else if (t == 0 && p != 0) c = p == 1 ? 0 : p - 1;
            else if (p == 0 && t != 0) c = t == 1 ? P - 1 : t + P - 2;
            dst[(long long)(p * P + t) * n_act + v] = c < 0 ? 0.f : src[(long long)c * n_act + v];
        }
}
}  // namespace

cudaError_t launch_remap_k_mtc(int P, int layout, const float *k_src, float *k_gm, int n_act, cudaStream_t st) {
    if (n_act <= 0) return cudaSuccess;
    remap_k_mtc<<<(n_act + 127) / 128, 128, 0, st>>>(P, layout, k_src, k_gm, n_act);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(int P, const AdjLaunch &L, cudaStream_t st) {
    const bool gm = L.exch_gm != 0, bound = gm && L.bound != 0;
    switch (P) {
    case 1: return go<1, false>(L, st);
    case 2: return bound ? go<2, true, true>(L, st) : gm ? go<2, true>(L, st) : go<2, false>(L, st);
    case 3: return bound ? go<3, true, true>(L, st) : gm ? go<3, true>(L, st) : go<3, false>(L, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace mrl
