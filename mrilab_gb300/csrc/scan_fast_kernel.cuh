// The MRL_NUMERICS_ACCURATE scan kernel: the same sequence model and tissue
// models as scan_ref_kernel (BlochKernel{,ME,MT,CEST,GM}.cuh), integrated
// in single precision in rotating frames so that it is both faster and
// closer to the exact (FP64) solution than the reference's own FP32 code.
//
// Frames.  Pool t of a voxel has one frame, shared by the voxel's spins:
// m_lab = m_frame * P_t, P_t = exp(-i Phi_t), with
//   Phi_t = gamma (dB0 T + x Kx + y Ky + z Kz) + 2 pi CS_t T,
// T and K the elapsed time and gradient areas over the steps without rf
// (moments carried on the host in FP64 and passed as hi/lo float pairs).
// Between anchors P_t advances by a factor (1 + d_t), d_t = exp(-i theta) - 1
// evaluated once per change of (dt, G); P_t is recomputed exactly from the
// moments (double-float arithmetic, Cody-Waite reduction) at every change
// of (dt, G), the first step of every rf block (the frames hold still
// during rf) and at least every kAnchorEvery free steps, so the large
// gradient and off-resonance phases never accumulate rounding.  In
// its pool's frame an isochromat only sees its own small residual
// frequency dWRnd, relaxation and exchange: a free step is the increment
//   m += dm m + sum_p f_tp (P_p,before / P_t,after) m_p,
// dm = (1 - a) exp(-i dWRnd dt) - 1 in "1 - y" form (a the transverse decay
// of the step), f_tp the exchange inflow.  An rf step rotates the frame
// magnetisation about the effective field with the rf azimuth shifted by
// -Phi_t (exact identity of the reference's closed form,
// BlochKernel.cuh:241-254) while the frame holds still.
//
// Coefficients close to 1 are applied in "1 - y" form: relaxation
// exp(-dt/T) = 1 - y with y = -expm1(-dt/T), exchange exp(-k dt) likewise,
// so repeated multiplication does not accumulate the rounding of a stored
// factor.  The receive sums a pool's spins in the frame and rotates the
// sum back to the lab with P_t.
#pragma once

#include "decode.h"
#include "scan_kernel.cuh"
#include "tc_util.cuh"

namespace mrl {

struct FastLaunch {
    ScanLaunch b;             // shared fields; b.rec points at fast records
    const float2 *omega;      // [4][n_act] (hi, lo) of gamma*dB0, gamma*x, gamma*y, gamma*z
    const float2 *txc;        // [tx][n_act] TxCoilmg * exp(i TxCoilpe)
    // Direct layout (mrl_scan_noalloc): the arrays of ScanLaunch are the
    // caller's uncompacted MATLAB arrays (n = every voxel), and the two
    // derived fields above are computed here instead of being read.
    int direct;
    int all_free;             // KM_EXCH: every pool is free (ME, or GM without bound pools): selects
                              // the FREE instantiation
    const float *rx_x, *rx_y; // [rx][n]
    float gam_hi, gam_lo;     // gyromagnetic ratio split
    float cs_hi[kMaxPool], cs_lo[kMaxPool];  // 2 pi CS[t] split
    // KM_EXCH with bound pools: the sampled (free) pools get the receive
    // tile's rows, n_samp per sample; samp_rank[t] = the row of pool t within
    // a sample, or -1 for a bound pool (its signal is zero)
    int n_samp;
    int samp_rank[kMaxPool];
    // receive contraction on the fifth-generation tensor cores (tcgen05,
    // tc_receive_ok): 17 to 32 coils, 1, 2 or 4 threads per voxel; launched
    // with the instantiations built for it (select_fast_tc)
    int tc;
};
static_assert(sizeof(FastLaunch) % 4 == 0, "FastLaunch is copied to shared memory as 32-bit words");

// tcgen05 receive: the coil operand has 128 rows -- Re R_c (TF32 big part),
// Im R_c (big), Re R_c (small part), Im R_c (small) for 32 coil slots -- and
// K = the block's voxels; the magnetisation operand has 64 rows, 16 (sample
// x sampled pool) in each of four parts: Re m (big), Im m (big), Re m
// (small), Im m (small).  Both K-major with the 128-byte swizzle
// (tc_util.cuh).  One MMA per K step (M = 128, N = 64: an MMA's cost barely
// depends on N) into 64 tensor-memory columns, one per magnetisation row.
constexpr int kTcRows = 128, kTcN = 16, kTcBRows = 4 * kTcN, kTcCoils = 32, kTcCols = 64;
__host__ __device__ constexpr bool tc_receive_ok(int c4, int tpv) {
    return c4 > 16 && c4 <= kTcCoils && (tpv == 1 || tpv == 2 || tpv == 4);
}
// voxels of a block (the contraction's K) and the byte sizes of the
// operands: coil operand, one magnetisation part, the magnetisation region
// (also the epilogue's per-warp sums, [warp][16][32] float2)
__host__ __device__ constexpr int tc_kv(int tpv) { return kBlock / tpv; }
__host__ __device__ constexpr int tc_a_bytes(int tpv) { return kTcRows * tc_kv(tpv) * 4; }
__host__ __device__ constexpr int tc_b_bytes(int tpv) {
    return kTcBRows * tc_kv(tpv) * 4 > (kBlock / 32) * kTcN * kTcCoils * 8 ? kTcBRows * tc_kv(tpv) * 4
                                                                          : (kBlock / 32) * kTcN * kTcCoils * 8;
}

// Coil sensitivities in shared memory: up to 16 coils (C4 <= 16) already
// split into TF32 (big, small) pairs for the receive contraction; beyond,
// as plain float2 split in the flush, which halves their footprint (32
// coils: 33 KB instead of 66 KB, three blocks per SM instead of two).
__host__ __device__ constexpr bool coil_presplit(int c4) { return c4 <= 16; }

template <bool B>
struct BoolTag {
    static constexpr bool value = B;
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

// a - b on a spin pair (sub.rn.f32x2, sm_100 and later): the difference of two
// products without a separate negation
__device__ __forceinline__ float2 fsub2_rn(float2 a, float2 b) {
    float2 r;
    asm("{.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float2 cmul_conj(float2 a, float2 b) {  // a * conj(b)
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}

// ---- receive contraction on the tensor cores --------------------------------
// The hardware conversion, kept as the check of tf32_rn.
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// x rounded to TF32 (10-bit mantissa), to nearest with ties away from zero:
// the bits cvt.rna.tf32.f32 gives for finite x, in two integer operations.
__device__ __forceinline__ uint32_t tf32_rn(float x) { return (__float_as_uint(x) + 0x1000u) & 0xffffe000u; }

// D += A (16x8, row) * B (8x8, col), TF32 inputs, FP32 accumulate
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Super-Lorentzian lineshape of a bound pool by the reference's rule
// (BlochKernelMT.cuh:348-358): G = sum over u = p / 1000, p < 1000, of
// sqrt(2 / pi) T2b / |3u^2 - 1| exp(-2 x^2) / 1000, x = w T2b / (3u^2 - 1),
// w = 2 pi rf_freq + gamma dB0.  In single precision with an exact u and a
// compensated (Kahan) sum: the reference-order kernel keeps the
// reference's double-precision arithmetic, which on this GPU's FP64 pipe
// costs more than the rf steps it feeds.
static __device__ __noinline__ float lineshape_f32(float rf_freq, float db0, float gyro, float t2b) {
    const float a = fmaf((float)(2 * kPiRef), rf_freq, db0 * gyro) * t2b;
    // four interleaved compensated partial sums (u = p / 1000 for p = 4i + j):
    // independent chains, so the loop is not one serial dependency
    float g[4] = {0.f, 0.f, 0.f, 0.f}, comp[4] = {0.f, 0.f, 0.f, 0.f};
    for (int p0 = 0; p0 < 1000; p0 += 4) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float u = (float)(p0 + j) * 0.001f;
            const float den = fmaf(3.f * u, u, -1.f);
            const float inv = 1.f / den;
            const float x = a * inv;
            const float term = fabsf(inv) * __expf(-2.f * x * x) - comp[j];
            const float sum = g[j] + term;
            comp[j] = (sum - g[j]) - term;
            g[j] = sum;
        }
    }
    const float total = ((g[0] - comp[0]) + (g[1] - comp[1])) + ((g[2] - comp[2]) + (g[3] - comp[3]));
    return total * (0.79788456080286536f * 0.001f) * t2b;  // sqrt(2 / pi) / 1000
}

// y = 1 - exp(-x).  Relaxation and exchange arguments (dt / T, k dt) are
// almost always below 1/16: there the Taylor series x - x^2/2 + ... + x^7/7!
// in Horner form (truncation below 1e-13 relative, FP32 rounding a few ulp,
// GPU-tested against expm1f); otherwise CUDA's expm1f.
__device__ __forceinline__ float one_minus_exp(float x) {
    if (fabsf(x) < 0.0625f) {
        float r = fmaf(x, 1.f / 5040.f, -1.f / 720.f);
        r = fmaf(r, x, 1.f / 120.f);
        r = fmaf(r, x, -1.f / 24.f);
        r = fmaf(r, x, 1.f / 6.f);
        r = fmaf(r, x, -0.5f);
        r = fmaf(r, x, 1.f);
        return r * x;
    }
    return -expm1f(-x);
}

// Rotation of the magnetisation by an rf step, written with its rotation
// vector v (angle a = |v|): exp([v]x) m = m + s1 (v x m) + s2 (v x (v x m)),
// s1 = sin a / a, s2 = (1 - cos a) / a^2 (Rodrigues' formula), the
// increment added to m with one rounding.  An rf step of the reference's
// closed form (angle alpha = dt sqrt(b^2 + dW^2) about n = (cb cos PHI,
// -cb sin PHI, sb), R = cos a I - sin a [n]x + (1 - cos a) n n^T) is
// v = -alpha n = -dt (gamma Re(conj(B) P), -gamma Im(conj(B) P), dW) with B
// the complex rf field and P the frame phasor: no normalisation needed.
// Below a = 0.25 (rf steps of practical sequences turn by a few mrad) s1
// and s2 are their Taylor series in a^2 through a^6, truncated below 1e-10;
// larger angles take sin and cos.
static __device__ __noinline__ float2 rot_coeffs_large(float a2) {
    const float a = sqrtf(a2);
    float sh, ch;
    sincos_cw(0.5f * a, sh, ch);
    return make_float2(2.f * sh * ch / a, 2.f * sh * sh / a2);
}
__device__ __forceinline__ float2 rot_coeffs(float a2) {
    if (a2 < 0.0625f)
        return make_float2(fmaf(fmaf(fmaf(a2, -1.f / 5040.f, 1.f / 120.f), a2, -1.f / 6.f), a2, 1.f),
                           fmaf(fmaf(fmaf(a2, -1.f / 40320.f, 1.f / 720.f), a2, -1.f / 24.f), a2, 0.5f));
    return rot_coeffs_large(a2);
}
__device__ __forceinline__ void rot_exp(float &x, float &y, float &z, float vx, float vy, float vz, float2 s) {
    const float cx = fmaf(vy, z, -vz * y), cy = fmaf(vz, x, -vx * z), cz = fmaf(vx, y, -vy * x);
    const float dx = fmaf(vy, cz, -vz * cy), dy = fmaf(vz, cx, -vx * cz), dz = fmaf(vx, cy, -vy * cx);
    x += fmaf(s.x, cx, s.y * dx);
    y += fmaf(s.x, cy, s.y * dy);
    z += fmaf(s.x, cz, s.y * dz);
}

// Direct receive: the block's sum of launch-local sample `a`, pool t, coil
// c, rotated by exp(-i rfRef), added into the FP64 signal (out of line: the
// partial-sum path is the usual one)
static __device__ __noinline__ void direct_add(const ScanLaunch &L, int a, int t, int c, float sx, float sy) {
    const int sig = L.amap[a];
    if (sig < 0 || sig >= L.A) return;
    const long long idx = ((long long)t * L.rx + c) * L.A + sig;
    atomicAdd(L.dsx + idx, L.cr * sx - L.sr * sy);
    atomicAdd(L.dsy + idx, L.sr * sx + L.cr * sy);
}

// Pools with a frame: every pool but the bound pool (pool 1) of MT / CEST,
// which has no transverse magnetisation.
template <int MODEL>
__device__ __forceinline__ constexpr bool has_frame(int t) {
    return !((MODEL == KM_MT || MODEL == KM_CEST) && t == 1);
}

// FREE (KM_EXCH only): every pool is a free pool (ME, or GM without bound
// pools); the instantiation then carries no pool-kind tests.
// Resident blocks per SM the register allocation aims at: four (16 warps)
// while a thread's isochromat state is small.
template <int P, int NS>
__host__ __device__ constexpr int fast_min_blocks() {
    return (P <= 2 && P * NS <= 8) ? 4 : (((P <= 3 && P * NS <= 6) || P * NS <= 5) ? 3 : 2);
}

// One work item: tile `tile` (kBlock consecutive voxel-threads) of the scan
// described by F, over F's step range.  kbase counts the record chunks this
// block has staged before (it picks the buffer and mbarrier phase).
// Returns false, block-uniformly, when a wait ran out (status word raised).
// TC (F.tc): the receive contraction runs on tcgen05 into the tensor memory
// whose address the kernel keeps at smem + 24 (32 columns held by the
// block); the 32-bit word at smem + 28 counts the block's contractions (the
// phase of their completion mbarrier bar[2]) and the one at smem + 32 is
// raised when a contraction's wait ran out.  (Kept in shared memory, not in
// registers: the step loop's instantiations sit at their register limit.)
// Coefficient source CO of the relaxation / exchange step: 0 computed in the
// kernel at each dt change; 1 the same split-exchange coefficients from a
// table per (dt, voxel) computed in FP64 (fewer live registers: no rates or
// relaxation rates held); 2 the exact propagator's table (EXACT).
template <int MODEL, int P, int NS, bool FREE, int CO = 0, bool TC = false>
__device__ __forceinline__ bool scan_item(const FastLaunch &F, int tile, unsigned char *smem, uint32_t &kbase) {
    constexpr bool EXACT = CO == 2;
    static_assert(CO == 0 || (MODEL == KM_EXCH && (FREE || CO == 2)),
                  "tabulated coefficients: free pools exchanging (split), general-model pools (exact)");
    const ScanLaunch &L = F.b;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float4 *rbuf = reinterpret_cast<float4 *>(smem + 128);
    const int rstride = L.stride4;
    constexpr int chunk = kFastChunk;  // a runtime length costs registers (spills at P=2, 4 spins)
    constexpr bool kMTC = MODEL == KM_MT || MODEL == KM_CEST;
    // receive tile: one row per (sample, sampled pool), one column per thread
    // holding its lab-frame transverse magnetisation; the coil sensitivities
    // of the threads' voxels; per-warp sums of the contraction; then
    // per-thread values read only at anchors, state changes and rf steps:
    // the isochromats' dWRnd and the low parts of gamma * (dB0, x, y, z)
    constexpr int kNSampP = kMTC ? 1 : P;
    constexpr int NQ = (NS + 1) / 2;  // spin pairs of a thread
    // tile rows per sample and samples per flush (bound pools of KM_EXCH take no row)
    constexpr bool kRank = MODEL == KM_EXCH && !FREE;
    const int nsp = kRank ? max(1, F.n_samp) : kNSampP;
    const int ktile = 16 / nsp;
    constexpr int kTRow = kBlock + 2;                             // padded row (float2)
    constexpr int kWarps = kBlock / 32;
    const int C4 = (L.rx + 3) & ~3;
    float2 *mtile = reinterpret_cast<float2 *>(rbuf + 2 * chunk * rstride);  // [16][kTRow]
    // coil sensitivities: TF32 (big, small) pairs [C4][kTRow][rx, ry], or
    // float2 [C4][kTRow] beyond 16 coils (coil_presplit)
    const bool presplit = coil_presplit(C4);
    uint2 *rsq = reinterpret_cast<uint2 *>(mtile + 16 * kTRow);
    float2 *rsf = reinterpret_cast<float2 *>(rsq);
    float *wstage = reinterpret_cast<float *>(rsq + (presplit ? 2 : 1) * C4 * kTRow);  // [warp][16][2*C4]
    // tcgen05 receive instead (F.tc): the coil and magnetisation operands
    // from the first 1024-byte boundary after the records
    // a compile-time choice: the instantiations without it keep their step
    // loop as small as before (the headline's is bound by instruction fetch)
    constexpr bool tcr = TC;
#define TPV (L.tpv)
    // the coil operand at the first 1024-byte boundary after the records
    // (the magnetisation operand follows it)
#define TCA (reinterpret_cast<unsigned char *>(mtile) + ((1024u - (smem_u32(mtile) & 1023u)) & 1023u))
#define TCB (TCA + tc_a_bytes(TPV))
    volatile uint32_t *tc_word = reinterpret_cast<volatile uint32_t *>(smem + 24);  // [0] tmem, [1] kmma, [2] fail
    float2 *dwsm = tcr ? reinterpret_cast<float2 *>(TCB + tc_b_bytes(TPV))
                       : reinterpret_cast<float2 *>(wstage + kWarps * 16 * 2 * C4);  // [NQ][P][kBlock] spin pairs
    float *omlo = reinterpret_cast<float *>(dwsm + NQ * P * kBlock);              // [4][kBlock]

    const int tid = threadIdx.x;
    const long long gt = (long long)tile * kBlock + tid;
    const int v = (int)(gt / L.tpv);
    const int sg = (int)(gt % L.tpv);
    // tcgen05 receive: the magnetisation operand's base and this thread's
    // column in it (its voxel), fixed for the item -- derived from the
    // launch's threads per voxel once, not at every sample
    const int tpv_r = tcr ? L.tpv : 1;
    unsigned char *const tcb_base = tcr ? TCB : nullptr;
    const int tc_col = tcr ? tid / tpv_r : 0;
    bool active = v < L.n_act;
    const int n = L.n_act;

    // isochromat state, and the free-step increment of the frame
    // magnetisation dm = (dmX, dmY) per spin; the packed paths read and write
    // spins 2q and 2q + 1 as the two lanes of an f32x2 value (PAIR / UNPAIR)
    float Xs[NS][P], Ys[NS][P], Zs[NS][P];
    float dmXs[NS][P], dmYs[NS][P];
#define XS(s, t) Xs[s][t]
#define YS(s, t) Ys[s][t]
#define ZS(s, t) Zs[s][t]
#define DMX(s, t) dmXs[s][t]
#define DMY(s, t) dmYs[s][t]
#define PAIR(A, q, t) make_float2(A[2 * (q)][t], A[2 * (q) + 1][t])
#define UNPAIR(A, q, t, v) (A[2 * (q)][t] = (v).x, A[2 * (q) + 1][t] = (v).y)
#define DWS(s, t) (((s) & 1) ? dwsm[((s) >> 1) * P * kBlock + (t) * kBlock + tid].y \
                             : dwsm[((s) >> 1) * P * kBlock + (t) * kBlock + tid].x)
    float2 Pc[P], Dc[P];  // frame phasor of each pool and its free-step increment
    float rhoS[P], it1[P], it2[P], t2v[P], y1[P], y2[P];
    unsigned act = 0;
    float om[4] = {0.f, 0.f, 0.f, 0.f};  // high parts of gamma * (dB0, x, y, z)
    float2 tx0 = make_float2(0.f, 0.f);
    float db0 = 0.f;
    constexpr int kNK = MODEL == KM_EXCH ? P * P : (MODEL == KM_MT ? 2 : (MODEL == KM_CEST ? 2 * (P - 1) : 1));
    float kc[kNK];
#pragma unroll
    for (int i = 0; i < kNK; ++i) kc[i] = 0.f;
#pragma unroll
    for (int t = 0; t < P; ++t) {
        rhoS[t] = it1[t] = it2[t] = t2v[t] = y1[t] = y2[t] = 0.f;
        Pc[t] = make_float2(1.f, 0.f);
        Dc[t] = make_float2(0.f, 0.f);
#pragma unroll
        for (int s = 0; s < NS; ++s) Xs[s][t] = Ys[s][t] = Zs[s][t] = dmXs[s][t] = dmYs[s][t] = 0.f;
    }
    if (active) {
        db0 = L.db0[v];
        if (F.direct) {
            const float g[4] = {db0, L.gxg[v], L.gyg[v], L.gzg[v]};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const df p = df_mul(F.gam_hi, F.gam_lo, g[i], 0.f);
                om[i] = p.hi;
                omlo[i * kBlock + tid] = p.lo;
            }
            float sp, cp;
            sincos_cw(L.txpe[v], sp, cp);
            tx0 = make_float2(L.txmg[v] * cp, L.txmg[v] * sp);
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float2 o = F.omega[(long long)i * n + v];
                om[i] = o.x;
                omlo[i * kBlock + tid] = o.y;
            }
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
                XS(s, t) = L.mx[i];
                YS(s, t) = L.my[i];
                ZS(s, t) = L.mz[i];
                DWS(s, t) = L.dwrnd[i];
            }
        }
    }
    if (F.direct) {
        const bool any = kMTC ? (act & 1u) != 0 : act != 0;
        if (!any) active = false;
    }
    // pools whose magnetisation the step integrates; the others keep their
    // lab-frame magnetisation (the reference skips them)
    unsigned evo = 0;
#pragma unroll
    for (int t = 0; t < P; ++t) {
        bool e;
        if (kMTC)
            e = true;
        else if (MODEL == KM_NORMAL || FREE)
            e = (act >> t & 1u) != 0;
        else
            e = (act >> t & 1u) && (L.kind[t] == 0 || L.kind[t] == 1);
        if (e) evo |= 1u << t;
    }
    // transverse pools among them (GM: free pools only)
    unsigned tvo = evo;
    if (MODEL == KM_EXCH && !FREE) {
#pragma unroll
        for (int t = 0; t < P; ++t)
            if (L.kind[t] != 0) tvo &= ~(1u << t);
    }
    // stage this thread's voxel's coil sensitivities (zero beyond the coil count)
    if constexpr (tcr) {
        // one thread per voxel writes its column of the coil operand (all
        // 32 coil slots: the 128 rows of the MMA)
        if (sg == 0) {
            const int kv = tid / TPV;
            for (int c = 0; c < kTcCoils; ++c) {
                float2 r = make_float2(0.f, 0.f);
                if (active && c < L.rx) {
                    if (L.rx_default)
                        r = make_float2(1.f, 0.f);
                    else if (F.direct)
                        r = make_float2(F.rx_x[(long long)c * n + v], F.rx_y[(long long)c * n + v]);
                    else
                        r = L.rxc[(long long)c * n + v];
                }
                const float bx = __uint_as_float(tf32_rn(r.x)), by = __uint_as_float(tf32_rn(r.y));
                const float q[4] = {bx, by, __uint_as_float(tf32_rn(r.x - bx)), __uint_as_float(tf32_rn(r.y - by))};
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    *reinterpret_cast<float *>(TCA + tc::sw128_offset(i * kTcCoils + c, kv, kTcRows)) = q[i];
            }
        }
        tc::fence_async_smem();
    }
    for (int c = 0; c < (tcr ? 0 : C4); ++c) {
        float2 r = make_float2(0.f, 0.f);
        if (active && c < L.rx) {
            if (L.rx_default)
                r = make_float2(1.f, 0.f);
            else if (F.direct)
                r = make_float2(F.rx_x[(long long)c * n + v], F.rx_y[(long long)c * n + v]);
            else
                r = L.rxc[(long long)c * n + v];
        }
        if (presplit) {
            const uint32_t bx = tf32_rn(r.x), by = tf32_rn(r.y);
            rsq[2 * (c * kTRow + tid) + 0] = make_uint2(bx, tf32_rn(r.x - __uint_as_float(bx)));
            rsq[2 * (c * kTRow + tid) + 1] = make_uint2(by, tf32_rn(r.y - __uint_as_float(by)));
        } else {
            rsf[c * kTRow + tid] = r;
        }
    }
    // the isochromats enter their frames at the first step: m_frame = m_lab / P_t
    bool entered = false;
    // exchange / MT coefficients, cached per dt
    float yo[P], fin[P][P];
    // exact propagator (EXACT): longitudinal off-diagonal terms and recovery
    constexpr int kXP = EXACT ? P : 1;
    float fL[kXP][kXP], cL[kXP];
#pragma unroll
    for (int t = 0; t < P; ++t) {
        yo[t] = 0.f;
#pragma unroll
        for (int p = 0; p < P; ++p) fin[t][p] = 0.f;
    }
    // packed free steps (two spins per f32x2 operation): the exchange model
    // with the split scheme and an even spin count per thread.  With bound
    // pools (FREE false) the free step is the same arithmetic: a bound pool's
    // increment is its frame's step back (held in the lab), the transverse
    // inflow from a bound pool is zero in fr, and saturation acts on rf steps
    // only
    constexpr bool kPack = MODEL == KM_EXCH && !EXACT && NS % 2 == 0;
    // rf steps packed too while a thread's state is small (beyond 8
    // isochromat-pools, or 6 with bound pools, the packed rf step's
    // temporaries spill); a bound pool takes its saturation instead of the
    // rotation there
    constexpr bool kPackRf = kPack && NS * P <= (FREE ? 8 : 6);
    bool selfx = false;  // some pool of this voxel exchanges with itself (a nonzero K diagonal)
    float mt_y1k = 0.f, mt_y21 = 0.f, mt_y1bk = 0.f, mt_y1b = 0.f, mt_y12 = 0.f;
    LineshapeCache lc;
    float4 satk = make_float4(0.f, 0.f, 0.f, -1.f);  // (Re A, Im A, 2 pi f, dt) of satv
    float satv = 0.f;
    const float gyro = L.gyro;

    __syncthreads();  // the staged coil maps
    const long long nsteps = L.s1 - L.s0;
    const int nchunks = (int)((nsteps + chunk - 1) / chunk);
    // chunk k of this item uses buffer and mbarrier (kbase + k) & 1, phase ((kbase + k) >> 1) & 1
    auto issue = [&](int k) {
        const long long first = L.s0 + (long long)k * chunk;
        const long long cnt = min((long long)chunk, L.s1 - first);
        const uint32_t bytes = (uint32_t)(cnt * rstride * 16);
        const uint32_t b = (kbase + k) & 1;
        mbar_expect_tx(&bar[b], bytes);
        bulk_g2s(rbuf + b * chunk * rstride, L.rec + first * rstride, bytes, &bar[b]);
    };
    if (tid == 0 && nchunks > 0) issue(0);

    int a_fill = 0, a_base = 0;
    const int lane = tid & 31, warp = tid >> 5;
    // flush: S[row][2c + {x,y}] = sum over threads of m(row) conj(R_c): a
    // (16 x 2*128) x (2*128 x 2*C4) real GEMM, split by warps along the
    // thread (voxel) dimension, on the tensor cores in the three-term TF32
    // split (big*big + big*small + small*big, each term its own accumulator
    // chain); then the warp slices are added and one partial per (block,
    // sample, pool, coil) is written.
    //   A[row][2j + ri] = (x, y)[ri] of thread j;  B[2j + ri][2c + cmp]:
    //   (x,x) = rx, (y,x) = ry, (x,y) = -ry, (y,y) = rx.
    // the flush in two compiled forms, one per coil-map layout (a branch
    // inside its loops cost the 8-coil scan 4 %)
    auto flush_form = [&](auto pre_tag) {
        constexpr bool pre = decltype(pre_tag)::value;
        // a warp's tile columns are its own threads' (k = the warp's voxels): the
        // tile needs no block barrier before the contraction
        __syncwarp();
        const int g = lane >> 2, tig = lane & 3, ri = tig & 1, cmp = g & 1;
        const int bcomp = (ri == cmp) ? 0 : 1;                 // rx, else ry
        const uint32_t sgn = (cmp && !ri) ? 0x80000000u : 0u;  // -ry
        const float *mt1 = reinterpret_cast<const float *>(mtile) + ri;
        const uint2 *rs1 = rsq + bcomp;
        const float *rf1 = reinterpret_cast<const float *>(rsf) + bcomp;
        const int nt_all = C4 / 4;
        float *rw = wstage + warp * 16 * (2 * C4);
        // n-tiles (4 coils each) in groups of kNG: the magnetisation operand
        // is loaded and split once per k-step for the whole group; per n-tile
        // two accumulator chains, big*big and the two correction products
        constexpr int kNG = 2;
        for (int nt0 = 0; nt0 < nt_all; nt0 += kNG) {
            float accb[kNG][4], accs[kNG][4];
#pragma unroll
            for (int u = 0; u < kNG; ++u)
#pragma unroll
                for (int i = 0; i < 4; ++i) accb[u][i] = accs[u][i] = 0.f;
#pragma unroll
            for (int ks = 0; ks < 8; ++ks) {
                const int j0 = warp * 32 + ks * 4 + (tig >> 1), j1 = j0 + 2;
                const float a[4] = {mt1[2 * (g * kTRow + j0)], mt1[2 * ((g + 8) * kTRow + j0)],
                                    mt1[2 * (g * kTRow + j1)], mt1[2 * ((g + 8) * kTRow + j1)]};
                uint32_t ab[4], as[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    ab[i] = tf32_rn(a[i]);
                    as[i] = tf32_rn(a[i] - __uint_as_float(ab[i]));
                }
#pragma unroll
                for (int u = 0; u < kNG; ++u) {
                    if (nt0 + u >= nt_all) break;
                    const int c = (nt0 + u) * 4 + (g >> 1);
                    // the coil operand (split once per launch up to 16 coils, here
                    // beyond); -ry flips the signs of both parts
                    uint32_t bb[2], bs[2];
                    if (pre) {
                        const uint2 q0 = rs1[2 * (c * kTRow + j0)], q1 = rs1[2 * (c * kTRow + j1)];
                        bb[0] = q0.x ^ sgn, bb[1] = q1.x ^ sgn, bs[0] = q0.y ^ sgn, bs[1] = q1.y ^ sgn;
                    } else {
                        const float b0 = rf1[2 * (c * kTRow + j0)], b1 = rf1[2 * (c * kTRow + j1)];
                        const uint32_t h0 = tf32_rn(b0), h1 = tf32_rn(b1);
                        bb[0] = h0 ^ sgn, bb[1] = h1 ^ sgn;
                        bs[0] = tf32_rn(b0 - __uint_as_float(h0)) ^ sgn, bs[1] = tf32_rn(b1 - __uint_as_float(h1)) ^ sgn;
                    }
                    mma_tf32(accs[u], as, bb);
                    mma_tf32(accs[u], ab, bs);
                    mma_tf32(accb[u], ab, bb);
                }
            }
#pragma unroll
            for (int u = 0; u < kNG; ++u) {
                if (nt0 + u >= nt_all) break;
                const int col = (nt0 + u) * 8 + 2 * tig;
                rw[g * (2 * C4) + col] = accs[u][0] + accb[u][0];
                rw[g * (2 * C4) + col + 1] = accs[u][1] + accb[u][1];
                rw[(g + 8) * (2 * C4) + col] = accs[u][2] + accb[u][2];
                rw[(g + 8) * (2 * C4) + col + 1] = accs[u][3] + accb[u][3];
            }
        }
        __syncthreads();
        const float *red = wstage;
        const int rxn = L.rx;
        const int nout = a_fill * kNSampP * rxn;
        // output o = pr * rx + c, pr = a * kNSampP + t: (pr, c) advanced by
        // kBlock outputs per pass (two divisions per flush, not one per output)
        const int dpr = kBlock / rxn, dc = kBlock - dpr * rxn;
        // the launch's fields in registers (the stores below go through a
        // generic pointer: the compiler would reload them from shared memory
        // for every output)
        const bool direct = L.dsx != nullptr;
        const int npairs = L.npairs;
        float2 *const pbase = direct ? nullptr : L.partial + ((long long)tile * L.a_launch + a_base) * npairs;
        int pr = tid / rxn, c = tid - pr * rxn;
        for (int o = tid; o < nout; o += kBlock, pr += dpr, c += dc) {
            if (c >= rxn) {
                c -= rxn;
                ++pr;
            }
            const int a = pr / kNSampP, t = pr - a * kNSampP;
            const int rank = kRank ? F.samp_rank[t] : t;
            float sx = 0.f, sy = 0.f;
            if (rank >= 0) {
                const int row = a * nsp + rank;
#pragma unroll
                for (int w = 0; w < kWarps; ++w) {
                    sx += red[(w * 16 + row) * (2 * C4) + 2 * c];
                    sy += red[(w * 16 + row) * (2 * C4) + 2 * c + 1];
                }
            }
            if (direct) {
                direct_add(L, a_base + a, t, c, sx, sy);
            } else {
                pbase[(long long)a * npairs + t * rxn + c] = make_float2(sx, sy);
            }
        }
        a_base += a_fill;
        a_fill = 0;
        __syncthreads();
    };
    // the flush on tcgen05 (F.tc): D = R x m^T, R the 128-row coil operand
    // and m the 16-row sample tile, K = the block's voxels; the products of
    // Re m go to tensor-memory columns 0..15, of Im m to 16..31.  Each of the
    // two sums adds the big and the small part of m (R's rows carry R's big
    // and small parts), so the row sums give R m with FP32-level accuracy
    // (big*big + big*small + small*big + small*small).  One thread issues the
    // MMAs; the block waits (bounded) for their completion, and each warp
    // reads its 32 tensor-memory lanes: warp 0 Re R big, 1 Im R big, 2 Re R
    // small, 3 Im R small, one lane per coil slot.
    auto flush_tc = [&]() {
        tc::fence_async_smem();  // this thread's tile writes, for the tensor core
        tc::fence_before_sync();
        __syncthreads();
        const int kv = tc_kv(TPV);
        const uint32_t tmem = tc_word[0], kmma = tc_word[1];
        __syncthreads();  // every thread has read the counter
        if (tid == 0) {
            tc_word[1] = kmma + 1u;
            tc::fence_after_sync();
            // descriptors of the operands' bases; a K step adds its byte offset / 16
            // to the start-address field (shared addresses stay below 2^18)
            const uint64_t da = tc::sw128_desc(smem_u32(TCA)), db = tc::sw128_desc(smem_u32(TCB));
            constexpr uint32_t idesc = tc::idesc_tf32(kTcRows, kTcBRows);
#pragma unroll 4
            for (int ks = 0; ks < kv / 8; ++ks) {
                const uint32_t ao = (uint32_t)((ks >> 2) * kTcRows * 128 + (ks & 3) * 32) >> 4;
                const uint32_t bo = (uint32_t)((ks >> 2) * kTcBRows * 128 + (ks & 3) * 32) >> 4;
                tc::mma_tf32(tmem, da + ao, db + bo, idesc, ks > 0);
            }
            tc::mma_commit(&bar[2]);
        }
        if (!mbar_wait_bounded(&bar[2], kmma & 1u, L.err)) {
            // a second bounded wait for the MMAs still in flight before the
            // block gives up (the tensor memory is freed at kernel exit)
            mbar_wait_bounded(&bar[2], kmma & 1u, L.err);
            tc_word[2] = 1u;
        }
        tc::fence_after_sync();
        // per warp (S_x, S_y) of each (row, coil slot), S = m conj(R), over the
        // consumed tile ([warp][16][32] float2): Re R rows give (Re m, Im m)
        // products to (x, y), Im R rows (Im m, -Re m); read 8 columns of the big
        // parts and their 8 small-part columns (32 further) at a time
        float2 *stg = reinterpret_cast<float2 *>(TCB);
        float *stw = reinterpret_cast<float *>(stg + warp * kTcN * kTcCoils + lane);
        const bool imr = (warp & 1) != 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float d[8], e[8];
            tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(8 * q), d);
            tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(2 * kTcN + 8 * q), e);
#pragma unroll
            for (int j = 0; j < 8; ++j) d[j] += e[j];
            const bool im_m = q >= 2;  // columns 16..31: Im m products
            const int comp = (im_m != imr) ? 1 : 0;
            const float sgn = (imr && !im_m) ? -1.f : 1.f;
#pragma unroll
            for (int j = 0; j < 8; ++j) stw[((q & 1) * 8 + j) * kTcCoils * 2 + comp] = sgn * d[j];
        }
        __syncthreads();
        const int rxn = L.rx;
        const int nout = a_fill * kNSampP * rxn;
        // output o = pr * rx + c, pr = a * kNSampP + t: (pr, c) advanced by
        // kBlock outputs per pass (two divisions per flush, not one per output)
        const int dpr = kBlock / rxn, dc = kBlock - dpr * rxn;
        // the launch's fields in registers (the stores below go through a
        // generic pointer: the compiler would reload them from shared memory
        // for every output)
        const bool direct = L.dsx != nullptr;
        const int npairs = L.npairs;
        float2 *const pbase = direct ? nullptr : L.partial + ((long long)tile * L.a_launch + a_base) * npairs;
        int pr = tid / rxn, c = tid - pr * rxn;
        for (int o = tid; o < nout; o += kBlock, pr += dpr, c += dc) {
            if (c >= rxn) {
                c -= rxn;
                ++pr;
            }
            const int a = pr / kNSampP, t = pr - a * kNSampP;
            const int rank = kRank ? F.samp_rank[t] : t;
            float sx = 0.f, sy = 0.f;
            if (rank >= 0) {
                const int row = a * nsp + rank;
#pragma unroll
                for (int w = 0; w < kWarps; ++w) {
                    const float2 q = stg[(w * kTcN + row) * kTcCoils + c];
                    sx += q.x;
                    sy += q.y;
                }
            }
            if (direct) {
                direct_add(L, a_base + a, t, c, sx, sy);
            } else {
                pbase[(long long)a * npairs + t * rxn + c] = make_float2(sx, sy);
            }
        }
        a_base += a_fill;
        a_fill = 0;
        tc::fence_before_sync();
        __syncthreads();
    };
    auto flush = [&]() {
        if constexpr (tcr)
            flush_tc();
        else if (presplit)
            flush_form(BoolTag<true>{});
        else
            flush_form(BoolTag<false>{});
    };

    for (int k = 0; k < nchunks; ++k) {
        if (tid == 0 && k + 1 < nchunks) issue(k + 1);
        const uint32_t kk = kbase + k;
        bool ok = mbar_wait_bounded(&bar[kk & 1], (kk >> 1) & 1, L.err) && (!TC || tc_word[2] == 0u);
        ok = __syncthreads_and(ok) != 0;
        if (!ok) {
            // wait (bounded) for the copies still in flight: this chunk and the next
            if (tid == 0) {
                mbar_wait_bounded(&bar[kk & 1], (kk >> 1) & 1, L.err);
                if (k + 1 < nchunks) mbar_wait_bounded(&bar[(kk + 1) & 1], ((kk + 1) >> 1) & 1, L.err);
            }
            __syncthreads();
            return false;
        }
        const float4 *cb = rbuf + (kk & 1) * chunk * rstride;
        const int cnt = (int)min((long long)chunk, nsteps - (long long)k * chunk);
        for (int q = 0; q < cnt; ++q) {
            const float4 r0 = cb[q * rstride];
            const float4 r1 = cb[q * rstride + 1];
            int flags = __float_as_int(r1.w);
            if (k == 0 && q == 0) flags |= kFlagState | kFlagDt;  // a launch may start inside a run
            const float dt = r0.x;

            // ---- frame phasors, exact from the moments ----------------------
            if (active && ((flags & kFlagAnchor) || !entered)) {
                const float4 r2 = cb[q * rstride + 2];
                const float4 r3 = cb[q * rstride + 3];
                df phc = df_mul(om[0], omlo[0 * kBlock + tid], r2.x, r2.y);
                phc = df_add(phc, df_mul(om[1], omlo[1 * kBlock + tid], r2.z, r2.w));
                phc = df_add(phc, df_mul(om[2], omlo[2 * kBlock + tid], r3.x, r3.y));
                phc = df_add(phc, df_mul(om[3], omlo[3 * kBlock + tid], r3.z, r3.w));
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    if (!has_frame<MODEL>(t)) continue;
                    const float2 pn = phasor(df_add(phc, df_mul(F.cs_hi[t], F.cs_lo[t], r2.x, r2.y)));
                    if (!entered) {
#pragma unroll
                        for (int s = 0; s < NS; ++s) {  // m_frame = m_lab * conj(P)
                            const float2 m = cmul_conj(make_float2(XS(s, t), YS(s, t)), pn);
                            XS(s, t) = m.x;
                            YS(s, t) = m.y;
                        }
                    }
                    Pc[t] = pn;
                }
                entered = true;
            }
            const float gzt = r0.y, gyt = r0.z, gxt = r0.w;
            // instantaneous common off-resonance (rad/s)
            const float wc = fmaf(om[3], gzt, fmaf(om[2], gyt, fmaf(om[1], gxt, om[0])));
            if (active && (flags & kFlagDt) && EXACT) {
                // the exact relaxation-exchange propagator of this dt, from the
                // table [dt][field][n_act]: diag(E_T) - 1, E_T off-diagonal,
                // diag(E_L) - 1, E_L off-diagonal, recovery (as y2, fin, y1, fL, cL)
                const float *xt = L.xtab + (long long)(flags >> 8) * L.xnf * n + v;
                int f = 0;
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    y2[t] = -xt[(long long)(f++) * n];
                    yo[t] = 0.f;
                }
#pragma unroll
                for (int t = 0; t < P; ++t)
#pragma unroll
                    for (int p = 0; p < P; ++p) fin[t][p] = p == t ? 0.f : xt[(long long)(f++) * n];
#pragma unroll
                for (int t = 0; t < P; ++t) y1[t] = -xt[(long long)(f++) * n];
#pragma unroll
                for (int t = 0; t < kXP; ++t)
#pragma unroll
                    for (int p = 0; p < kXP; ++p) fL[t][p] = p == t ? 0.f : xt[(long long)(f++) * n];
#pragma unroll
                for (int t = 0; t < kXP; ++t) cL[t] = xt[(long long)(f++) * n];
            } else if (active && (flags & kFlagDt) && CO == 1) {
                // the split scheme's coefficients of this dt from the table
                // [dt][field][n_act]: y1[P], y2[P], yo[P], fin[P][P]
                const float *xt = L.xtab + (long long)(flags >> 8) * L.xnf * n + v;
                int f = 0;
#pragma unroll
                for (int t = 0; t < P; ++t) y1[t] = xt[(long long)(f++) * n];
#pragma unroll
                for (int t = 0; t < P; ++t) y2[t] = xt[(long long)(f++) * n];
#pragma unroll
                for (int t = 0; t < P; ++t) yo[t] = xt[(long long)(f++) * n];
#pragma unroll
                for (int t = 0; t < P; ++t)
#pragma unroll
                    for (int p = 0; p < P; ++p) fin[t][p] = xt[(long long)(f++) * n];
            } else if (active && (flags & kFlagDt)) {
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    y1[t] = one_minus_exp(dt * it1[t]);
                    y2[t] = one_minus_exp(dt * it2[t]);
                }
                if (MODEL == KM_EXCH) {
#pragma unroll
                    for (int t = 0; t < P; ++t) {
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
                        yo[t] = one_minus_exp(dt * ksum);
                    }
                } else if (kMTC) {
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
                if (!kMTC) {
                    // a pool the step leaves alone gets neutral coefficients
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        if (evo >> t & 1u) continue;
                        y1[t] = y2[t] = yo[t] = 0.f;
#pragma unroll
                        for (int p = 0; p < P; ++p) fin[t][p] = 0.f;
                    }
                }
            }
            if (kPack && active && (flags & kFlagDt)) {
                selfx = false;
#pragma unroll
                for (int t = 0; t < P; ++t) selfx |= fin[t][t] != 0.f;
            }
            if (active && (flags & kFlagState)) {
                const bool new_dt = (flags & kFlagDt) != 0;  // kFlagDt implies kFlagState
#pragma unroll
                for (int t = 0; t < P; ++t)
                    if (has_frame<MODEL>(t)) Dc[t] = phase_step((wc + F.cs_hi[t]) * dt);
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    if (!has_frame<MODEL>(t)) continue;
                    // transverse decay of a free step: (1 - a) = (1 - y2)(1 - yo)
                    // (EXACT: the increment is the pure rotation; decay and exchange follow)
                    const float a = EXACT ? 0.f
                                          : (MODEL == KM_NORMAL || MODEL == KM_MT) ? y2[t]
                                                                                   : y2[t] + yo[t] - y2[t] * yo[t];
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        if (tvo >> t & 1u) {
                            // the isochromat's own step in its pool's frame: a function of dt alone
                            if (new_dt) {
                                const float2 p = phase_step(DWS(s, t) * dt);
                                DMX(s, t) = fmaf(p.x, 1.f - a, -a);
                                DMY(s, t) = p.y * (1.f - a);
                            }
                        } else {
                            // constant in the lab: m_frame turns back by the frame's step
                            DMX(s, t) = Dc[t].x;
                            DMY(s, t) = -Dc[t].y;
                        }
                    }
                }
            }

            // ---- receive, before the step's rotation ------------------------
            if (flags & kFlagAdc) {
#pragma unroll
                for (int t = 0; t < kNSampP; ++t) {
                    const int rank = kRank ? F.samp_rank[t] : t;
                    if (kRank && rank < 0) continue;  // a pool with no tile row (block-uniform)
                    float sx = 0.f, sy = 0.f;
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        sx += XS(s, t);
                        sy += YS(s, t);
                    }
                    float2 m = cmul(make_float2(sx, sy), Pc[t]);
                    if (!active) m = make_float2(0.f, 0.f);
                    if constexpr (tcr) {
                        // the voxel's sum over its threads, written by its first
                        // thread as the TF32 big and small parts of Re and Im
                        for (int o = 1; o < tpv_r; o <<= 1) {
                            m.x += __shfl_xor_sync(0xffffffffu, m.x, o);
                            m.y += __shfl_xor_sync(0xffffffffu, m.y, o);
                        }
                        if (rank >= 0 && sg == 0) {
                            const float bx = __uint_as_float(tf32_rn(m.x)), by = __uint_as_float(tf32_rn(m.y));
                            // rows r, 16 + r, 32 + r, 48 + r: Re and Im, big then small
                            // (16 rows = two 1024-byte atoms further, the same swizzle)
                            const int r = a_fill * nsp + rank;
                            float *tb = reinterpret_cast<float *>(tcb_base + tc::sw128_offset(r, tc_col, kTcBRows));
                            constexpr int kPartF = kTcN / 8 * 1024 / 4;  // floats between parts
                            tb[0] = bx;
                            tb[kPartF] = by;
                            tb[2 * kPartF] = __uint_as_float(tf32_rn(m.x - bx));
                            tb[3 * kPartF] = __uint_as_float(tf32_rn(m.y - by));
                        }
                    } else if (rank >= 0) {
                        mtile[(a_fill * nsp + rank) * kTRow + tid] = m;
                    }
                }
                if (++a_fill == ktile) flush();
            }
            if (!active) continue;
            if (flags & kFlagCkpt) {  // adjoint checkpoint: the state at the start of the step, lab frame
                const long long g = L.ckpt_step0 + (long long)k * chunk + q;
                const long long niso = (long long)L.S * n;
                float *c = L.ckpt + (g / L.ckpt_every) * 3 * P * niso;
#pragma unroll
                for (int s = 0; s < NS; ++s)
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        float2 m = make_float2(XS(s, t), YS(s, t));
                        if (has_frame<MODEL>(t)) m = cmul(m, Pc[t]);
                        const long long i = (long long)(sg * NS + s) * n + v;
                        c[(3 * t + 0) * niso + i] = m.x;
                        c[(3 * t + 1) * niso + i] = m.y;
                        c[(3 * t + 2) * niso + i] = ZS(s, t);
                    }
            }
            if (L.hist != nullptr) {  // RunMode 1: the state at the start of the step, lab frame
                float *h = L.hist + ((long long)k * chunk + q) * 3 * L.hist_stride;
#pragma unroll
                for (int s = 0; s < NS; ++s)
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        float2 m = make_float2(XS(s, t), YS(s, t));
                        if (has_frame<MODEL>(t)) m = cmul(m, Pc[t]);
                        const long long i = ((long long)t * L.S + sg * NS + s) * n + v;
                        h[i] = m.x;
                        h[L.hist_stride + i] = m.y;
                        h[2 * L.hist_stride + i] = ZS(s, t);
                    }
            }

            const bool rf = (flags & kFlagRf) != 0;
            float2 Pprev[P];
#pragma unroll
            for (int t = 0; t < P; ++t) Pprev[t] = Pc[t];
            if (!rf) {
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    if (!has_frame<MODEL>(t)) continue;
                    const float2 p = Pc[t], d = Dc[t];
                    Pc[t] = make_float2(fmaf(p.x, d.x, fmaf(-p.y, d.y, p.x)), fmaf(p.x, d.y, fmaf(p.y, d.x, p.y)));
                }
            }
            // exchange inflow of transverse magnetisation between frames:
            // fr[t][p] = f_tp P_p(before the step) conj(P_t(after))
            float2 fr[P][P];
            if (MODEL == KM_EXCH) {
#pragma unroll
                for (int t = 0; t < P; ++t)
#pragma unroll
                    for (int p = 0; p < P; ++p) {
                        if (kPack && p == t && !selfx) {  // fin[t][t] = 0: no self-exchange
                            fr[t][p] = make_float2(0.f, 0.f);
                            continue;
                        }
                        // no transverse exchange with or of a bound pool, and none of a
                        // general-model pool with itself (block-uniform tests)
                        if (!FREE && !EXACT && (L.kind[p] != 0 || L.kind[t] != 0 || (L.exch_gm && p == t))) {
                            fr[t][p] = make_float2(0.f, 0.f);
                            continue;
                        }
                        // (EXACT: the partner after its rotation, in its frame after the step)
                        const float2 r = cmul_conj(EXACT ? Pc[p] : Pprev[p], Pc[t]);
                        const float f = (FREE || ((tvo >> t & 1u) && L.kind[p] == 0)) ? fin[t][p] : 0.f;
                        fr[t][p] = make_float2(f * r.x, f * r.y);
                    }
            } else if (MODEL == KM_CEST) {
#pragma unroll
                for (int t = 2; t < P; ++t) {
                    const float2 r0t = cmul_conj(Pprev[t], Pc[0]);
                    const float2 rt0 = cmul_conj(Pprev[0], Pc[t]);
                    fr[0][t] = make_float2(fin[0][t] * r0t.x, fin[0][t] * r0t.y);
                    fr[t][0] = make_float2(fin[t][0] * rt0.x, fin[t][0] * rt0.y);
                }
            }

            float sat[P];                        // bound-pool saturation of the rf step
#pragma unroll
            for (int t = 0; t < P; ++t) sat[t] = 0.f;
            float2 vt[P];
            if (rf) {
                // complex B1 = sum_c TxCoilmg_c exp(i pe_c) * amp_c exp(i phase_c)
                float2 B = cmul(tx0, make_float2(r1.x, r1.y));
                for (int c = 1; c < L.tx && c < 4; ++c) {
                    const float4 rc = cb[q * rstride + 3 + c];
                    const float2 t2 = cmul(F.txc[(long long)c * n + v], make_float2(rc.x, rc.y));
                    B.x += t2.x;
                    B.y += t2.y;
                }
                // transverse part of the rotation vector, per pool (the frames hold still)
                const float sc = -dt * gyro;
#pragma unroll
                for (int t = 0; t < P; ++t) {
                    const float wx = fmaf(B.x, Pc[t].x, B.y * Pc[t].y), wy = fmaf(B.x, Pc[t].y, -B.y * Pc[t].x);
                    vt[t] = make_float2(sc * wx, -sc * wy);
                }
                if (MODEL == KM_MT || MODEL == KM_CEST) {
                    // the bound pool (pool 1): saturation 1 - exp(-W dt), W = pi (gamma
                    // TxCoilmg |amp|)^2 G(rf offset, T2b) with the reference's lineshape rule
                    // (single transmit coil); kept while the step's (A, f, dt) repeat, as
                    // they do through a continuous-wave saturation
                    if (r1.x != satk.x || r1.y != satk.y || r1.z != satk.z || dt != satk.w) {
                        const float b1 = sqrtf(fmaf(r1.x, r1.x, r1.y * r1.y)) * sqrtf(fmaf(tx0.x, tx0.x, tx0.y * tx0.y));
                        const float freq = r1.z * 0.15915494309189535f;
                        if (lc.t2b != t2v[1] || lc.freq != freq) {
                            lc.freq = freq;
                            lc.t2b = t2v[1];
                            lc.g = lineshape_f32(freq, db0, gyro, t2v[1]);
                        }
                        const float bg = b1 * gyro;
                        satv = one_minus_exp((float)kPiRef * bg * bg * lc.g * dt);
                        satk = make_float4(r1.x, r1.y, r1.z, dt);
                    }
                    sat[1] = satv;
                } else if (MODEL == KM_EXCH && !FREE) {
                    // bound pools: W = pi (gamma TxCoilmg |amp|)^2 G(rf offset, T2b) with the
                    // reference's lineshape rule (single transmit coil)
                    const float b1 = sqrtf(fmaf(r1.x, r1.x, r1.y * r1.y)) * sqrtf(fmaf(tx0.x, tx0.x, tx0.y * tx0.y));
                    const float freq = r1.z * 0.15915494309189535f;
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        const bool bound = (evo >> t & 1u) && L.kind[t] == 1;
                        if (!bound) continue;
                        if (lc.t2b != t2v[t] || lc.freq != freq) {
                            lc.freq = freq;
                            lc.t2b = t2v[t];
                            lc.g = lineshape_f32(freq, db0, gyro, t2v[t]);
                        }
                        const float bg = b1 * gyro;
                        const float w = (float)kPiRef * bg * bg * lc.g;
                        sat[t] = one_minus_exp(w * dt);
                    }
                }
            }
            const float wrf = r1.z;  // 2 pi sum of active rf frequencies

            if constexpr (kPack) {
                if (!rf) {
                    // the free step of the loop below for spins 2q and 2q + 1 at
                    // once: m_t += dm_t m_t + sum_p fr[t][p] m_p (transverse, in the
                    // frames), z_t = (1 - yo)(1 - y1) z_t + sum_p fin[t][p] z_p +
                    // rho_t y1 / S, every partner taken before the step
                    auto step = [&](auto self_tag) {
                        constexpr bool kSelf = decltype(self_tag)::value;
#pragma unroll
                        for (int qq = 0; qq < NQ; ++qq) {
                            float2 nx[P], ny[P], nz[P];
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                const float2 px = PAIR(Xs, qq, t), py = PAIR(Ys, qq, t);
                                const float2 dx = PAIR(dmXs, qq, t), dy = PAIR(dmYs, qq, t);
                                float2 ax = __fmul2_rn(dx, px);  // real part: ax - bx
                                float2 bx = __fmul2_rn(dy, py);
                                float2 iy = __ffma2_rn(dx, py, __fmul2_rn(dy, px));
#pragma unroll
                                for (int p = 0; p < P; ++p) {
                                    if (p == t && !kSelf) continue;
                                    if (!FREE && (L.kind[p] != 0 || L.kind[t] != 0)) continue;  // fr is zero
                                    const float2 f1 = make_float2(fr[t][p].x, fr[t][p].x);
                                    const float2 f2 = make_float2(fr[t][p].y, fr[t][p].y);
                                    ax = __ffma2_rn(f1, PAIR(Xs, qq, p), ax);
                                    bx = __ffma2_rn(f2, PAIR(Ys, qq, p), bx);
                                    iy = __ffma2_rn(f1, PAIR(Ys, qq, p), iy);
                                    iy = __ffma2_rn(f2, PAIR(Xs, qq, p), iy);
                                }
                                nx[t] = __fadd2_rn(px, fsub2_rn(ax, bx));
                                ny[t] = __fadd2_rn(py, iy);
                                // longitudinal, in increment form with one rounding of the
                                // state: z + (inflow + recovery - yd z), yd = 1 - (1 - y1)(1 - yo)
                                // (three roundings of z per step walked to 2.4e-5 over the
                                // 220,416 steps of the long multi-echo train)
                                const float c = rhoS[t] * y1[t];
                                const float yd = fmaf(-y1[t], yo[t], y1[t] + yo[t]);
                                float2 iz = make_float2(c, c);
#pragma unroll
                                for (int p = 0; p < P; ++p) {
                                    if (p == t && !kSelf) continue;
                                    iz = __ffma2_rn(make_float2(fin[t][p], fin[t][p]), PAIR(Zs, qq, p), iz);
                                }
                                const float2 zt = PAIR(Zs, qq, t);
                                nz[t] = __fadd2_rn(zt, __ffma2_rn(make_float2(-yd, -yd), zt, iz));
                            }
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                UNPAIR(Xs, qq, t, nx[t]);
                                UNPAIR(Ys, qq, t, ny[t]);
                                UNPAIR(Zs, qq, t, nz[t]);
                            }
                        }
                    };
                    if (selfx)
                        step(BoolTag<true>{});
                    else
                        step(BoolTag<false>{});
                    continue;
                }
                if constexpr (kPackRf) {
                    // the rf step of the loop below for spins 2q and 2q + 1 at once:
                    // rotation exp([v]x) with v = (vt, -dt dW), dW per spin, then
                    // relaxation and inflow (partners taken before the step)
                    auto rfstep = [&](auto self_tag) {
                        constexpr bool kSelf = decltype(self_tag)::value;
#pragma unroll
                        for (int qq = 0; qq < NQ; ++qq) {
                            float2 rx[P], ry[P], rz[P];
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                const float2 x = PAIR(Xs, qq, t), y = PAIR(Ys, qq, t), z = PAIR(Zs, qq, t);
                                if (!FREE && L.kind[t] != 0) {
                                    // a bound pool (block-uniform): no rotation; its
                                    // longitudinal magnetisation saturated
                                    rx[t] = x;
                                    ry[t] = y;
                                    rz[t] = __ffma2_rn(make_float2(-sat[t], -sat[t]), z, z);
                                    continue;
                                }
                                const float w0 = wc + F.cs_hi[t] + wrf;
                                const float2 dwp = dwsm[qq * P * kBlock + t * kBlock + tid];
                                // nvz = -v_z = dt dW per spin
                                const float2 nvz =
                                    __fmul2_rn(make_float2(dt, dt), __fadd2_rn(dwp, make_float2(w0, w0)));
                                const float2 vz = make_float2(-nvz.x, -nvz.y);
                                const float vx = vt[t].x, vy = vt[t].y;
                                const float vv = fmaf(vx, vx, vy * vy);
                                const float2 a2 = __ffma2_rn(nvz, nvz, make_float2(vv, vv));
                                float2 s1, s2;
                                if (a2.x < 0.0625f && a2.y < 0.0625f) {
                                    s1 = __ffma2_rn(
                                        __ffma2_rn(__ffma2_rn(a2, make_float2(-1.f / 5040.f, -1.f / 5040.f),
                                                              make_float2(1.f / 120.f, 1.f / 120.f)),
                                                   a2, make_float2(-1.f / 6.f, -1.f / 6.f)),
                                        a2, make_float2(1.f, 1.f));
                                    s2 = __ffma2_rn(
                                        __ffma2_rn(__ffma2_rn(a2, make_float2(-1.f / 40320.f, -1.f / 40320.f),
                                                              make_float2(1.f / 720.f, 1.f / 720.f)),
                                                   a2, make_float2(-1.f / 24.f, -1.f / 24.f)),
                                        a2, make_float2(0.5f, 0.5f));
                                } else {
                                    const float2 c0 = rot_coeffs(a2.x), c1 = rot_coeffs(a2.y);
                                    s1 = make_float2(c0.x, c1.x);
                                    s2 = make_float2(c0.y, c1.y);
                                }
                                const float2 bvx = make_float2(vx, vx), bvy = make_float2(vy, vy);
                                const float2 bnvx = make_float2(-vx, -vx), bnvy = make_float2(-vy, -vy);
                                // c = v x m, e = v x c
                                const float2 cx = __ffma2_rn(bvy, z, __fmul2_rn(nvz, y));
                                const float2 cy = __ffma2_rn(vz, x, __fmul2_rn(bnvx, z));
                                const float2 cz = __ffma2_rn(bvx, y, __fmul2_rn(bnvy, x));
                                const float2 ex = __ffma2_rn(bvy, cz, __fmul2_rn(nvz, cy));
                                const float2 ey = __ffma2_rn(vz, cx, __fmul2_rn(bnvx, cz));
                                const float2 ez = __ffma2_rn(bvx, cy, __fmul2_rn(bnvy, cx));
                                const bool on = tvo >> t & 1u;
                                rx[t] = on ? __fadd2_rn(x, __ffma2_rn(s1, cx, __fmul2_rn(s2, ex))) : x;
                                ry[t] = on ? __fadd2_rn(y, __ffma2_rn(s1, cy, __fmul2_rn(s2, ey))) : y;
                                rz[t] = on ? __fadd2_rn(z, __ffma2_rn(s1, cz, __fmul2_rn(s2, ez))) : z;
                            }
                            float2 nx[P], ny[P], nz[P];
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                float2 ax = make_float2(0.f, 0.f), bx = ax, iy = ax;
#pragma unroll
                                for (int p = 0; p < P; ++p) {
                                    if (p == t && !kSelf) continue;
                                    if (!FREE && (L.kind[p] != 0 || L.kind[t] != 0)) continue;  // fr is zero
                                    const float2 f1 = make_float2(fr[t][p].x, fr[t][p].x);
                                    const float2 f2 = make_float2(fr[t][p].y, fr[t][p].y);
                                    ax = __ffma2_rn(f1, PAIR(Xs, qq, p), ax);
                                    bx = __ffma2_rn(f2, PAIR(Ys, qq, p), bx);
                                    iy = __ffma2_rn(f1, PAIR(Ys, qq, p), iy);
                                    iy = __ffma2_rn(f2, PAIR(Xs, qq, p), iy);
                                }
                                // relaxation in increment form, one rounding of the state:
                                // m + (inflow - y m), y = 1 - (1 - y2)(1 - yo) transverse,
                                // 1 - (1 - y1)(1 - yo) longitudinal
                                const float ya = fmaf(-y2[t], yo[t], y2[t] + yo[t]);
                                const float yd = fmaf(-y1[t], yo[t], y1[t] + yo[t]);
                                const float2 nya = make_float2(-ya, -ya), nyd = make_float2(-yd, -yd);
                                nx[t] = __fadd2_rn(rx[t], __ffma2_rn(nya, rx[t], fsub2_rn(ax, bx)));
                                ny[t] = __fadd2_rn(ry[t], __ffma2_rn(nya, ry[t], iy));
                                const float c = rhoS[t] * y1[t];
                                float2 iz = make_float2(c, c);
#pragma unroll
                                for (int p = 0; p < P; ++p) {
                                    if (p == t && !kSelf) continue;
                                    iz = __ffma2_rn(make_float2(fin[t][p], fin[t][p]), PAIR(Zs, qq, p), iz);
                                }
                                nz[t] = __fadd2_rn(rz[t], __ffma2_rn(nyd, rz[t], iz));
                            }
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                UNPAIR(Xs, qq, t, nx[t]);
                                UNPAIR(Ys, qq, t, ny[t]);
                                UNPAIR(Zs, qq, t, nz[t]);
                            }
                        }
                    };
                    if (selfx)
                        rfstep(BoolTag<true>{});
                    else
                        rfstep(BoolTag<false>{});
                    continue;
                }
            }

            // (the unpacked step: the packed paths above take every step when
            // both the free and the rf step are packed)
            if constexpr (!(kPack && kPackRf)) {
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    float px[P], py[P], pz[P];
#pragma unroll
                    for (int t = 0; t < P; ++t) {
                        px[t] = XS(s, t);
                        py[t] = YS(s, t);
                        pz[t] = ZS(s, t);
                    }
                    // ---- transverse ----------------------------------------------
                    if (rf) {
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            if (!has_frame<MODEL>(t)) continue;
                            float x = px[t], y = py[t], z = pz[t];
                            const float dW = wc + DWS(s, t) + F.cs_hi[t] + wrf;
                            const float vz = -dt * dW;
                            rot_exp(x, y, z, vt[t].x, vt[t].y, vz, rot_coeffs(fmaf(vz, vz, fmaf(vt[t].x, vt[t].x, vt[t].y * vt[t].y))));
                            const bool on = tvo >> t & 1u;
                            XS(s, t) = on ? x : px[t];
                            YS(s, t) = on ? y : py[t];
                            ZS(s, t) = on ? z : pz[t];
                        }
                        // relaxation and inflow after the rotation (the frames hold still);
                        // the exact propagator takes the partners after their rotation,
                        // and bound pools after their saturation (sat is zero for the others)
                        if constexpr (EXACT) {
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                if constexpr (!FREE) ZS(s, t) = fmaf(-sat[t], ZS(s, t), ZS(s, t));
                                px[t] = XS(s, t);
                                py[t] = YS(s, t);
                                pz[t] = ZS(s, t);
                            }
                        }
                        if constexpr (MODEL == KM_NORMAL || MODEL == KM_MT) {
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                if (!has_frame<MODEL>(t)) continue;
                                XS(s, t) = fmaf(-y2[t], XS(s, t), XS(s, t));
                                YS(s, t) = fmaf(-y2[t], YS(s, t), YS(s, t));
                            }
                        } else {
#pragma unroll
                            for (int t = 0; t < P; ++t) {
                                if (!has_frame<MODEL>(t)) continue;
                                float ix = 0.f, iy = 0.f;
#pragma unroll
                                for (int p = 0; p < P; ++p) {
                                    if (MODEL == KM_CEST && !((t == 0 && p >= 2) || (t >= 2 && p == 0))) continue;
                                    const float2 f = fr[t][p];
                                    ix = fmaf(f.x, px[p], fmaf(-f.y, py[p], ix));
                                    iy = fmaf(f.x, py[p], fmaf(f.y, px[p], iy));
                                }
                                const float x = fmaf(-y2[t], XS(s, t), XS(s, t));
                                const float y = fmaf(-y2[t], YS(s, t), YS(s, t));
                                XS(s, t) = fmaf(-yo[t], x, x) + ix;
                                YS(s, t) = fmaf(-yo[t], y, y) + iy;
                            }
                        }
                    } else if constexpr (EXACT) {
                        // every pool turns by its own step, then the exact propagator
                        float wx[P], wy[P];
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            const float2 d = make_float2(DMX(s, t), DMY(s, t));
                            wx[t] = px[t] + fmaf(d.x, px[t], -d.y * py[t]);
                            wy[t] = py[t] + fmaf(d.x, py[t], d.y * px[t]);
                        }
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            float ix = 0.f, iy = 0.f;
#pragma unroll
                            for (int p = 0; p < P; ++p) {
                                if (p == t) continue;
                                const float2 f = fr[t][p];
                                ix = fmaf(f.x, wx[p], fmaf(-f.y, wy[p], ix));
                                iy = fmaf(f.x, wy[p], fmaf(f.y, wx[p], iy));
                            }
                            XS(s, t) = fmaf(-y2[t], wx[t], wx[t]) + ix;
                            YS(s, t) = fmaf(-y2[t], wy[t], wy[t]) + iy;
                        }
                    } else {
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            if (!has_frame<MODEL>(t)) continue;
                            float2 d = make_float2(DMX(s, t), DMY(s, t));
                            if (MODEL == KM_EXCH) {  // self exchange (a nonzero K diagonal)
                                d.x += fr[t][t].x;
                                d.y += fr[t][t].y;
                            }
                            float ix = fmaf(d.x, px[t], -d.y * py[t]);
                            float iy = fmaf(d.x, py[t], d.y * px[t]);
#pragma unroll
                            for (int p = 0; p < P; ++p) {
                                if (p == t || !has_frame<MODEL>(p)) continue;
                                if (MODEL == KM_NORMAL || MODEL == KM_MT) continue;
                                if (MODEL == KM_CEST && !((t == 0 && p >= 2) || (t >= 2 && p == 0))) continue;
                                const float2 f = fr[t][p];
                                ix = fmaf(f.x, px[p], fmaf(-f.y, py[p], ix));
                                iy = fmaf(f.x, py[p], fmaf(f.y, px[p], iy));
                            }
                            XS(s, t) = px[t] + ix;
                            YS(s, t) = py[t] + iy;
                        }
                    }
                    // ---- longitudinal (and the bound pools) -----------------------
                    if (MODEL == KM_NORMAL) {
#pragma unroll
                        for (int t = 0; t < P; ++t) ZS(s, t) = fmaf(y1[t], rhoS[t] - ZS(s, t), ZS(s, t));
                    } else if (MODEL == KM_EXCH && EXACT) {
#pragma unroll
                        for (int t = 0; t < kXP; ++t) {
                            float iz = 0.f;
#pragma unroll
                            for (int p = 0; p < kXP; ++p) iz = fmaf(fL[t][p], pz[p], iz);
                            const float z = ZS(s, t);
                            ZS(s, t) = fmaf(-y1[t], z, z) + iz + cL[t];
                        }
                    } else if (MODEL == KM_EXCH) {
#pragma unroll
                        for (int t = 0; t < P; ++t) {
                            float iz = 0.f;
#pragma unroll
                            for (int p = 0; p < P; ++p) iz = fmaf(fin[t][p], pz[p], iz);
                            float z = ZS(s, t);
                            if (!FREE && rf) z = fmaf(-sat[t], z, z);
                            // one rounding of the state (as the packed free step)
                            const float yd = fmaf(-y1[t], yo[t], y1[t] + yo[t]);
                            ZS(s, t) = z + fmaf(-yd, z, fmaf(rhoS[t], y1[t], iz));
                        }
                    } else {  // MT / CEST
                        const float zb0 = pz[1], z0 = pz[0];
                        float z = ZS(s, 0);
                        if (MODEL == KM_MT) {
                            z = fmaf(-mt_y1k, z, z) + rhoS[0] * y1[0] + zb0 * mt_y21;
                        } else {
                            float iz = 0.f;
#pragma unroll
                            for (int t = 2; t < P; ++t) iz = fmaf(fin[0][t], pz[t], iz);
                            z = fmaf(-mt_y1k, z, z);
                            z = fmaf(-yo[0], z, z) + iz + zb0 * mt_y21 + rhoS[0] * y1[0];
#pragma unroll
                            for (int t = 2; t < P; ++t) {
                                const float cz = fmaf(-y1[t], ZS(s, t), ZS(s, t));
                                ZS(s, t) = fmaf(-yo[t], cz, cz) + fin[t][0] * z0 + rhoS[t] * y1[t];
                            }
                        }
                        float bz = zb0;
                        if (rf) bz = fmaf(-sat[1], bz, bz);
                        ZS(s, 1) = fmaf(-mt_y1bk, bz, bz) + rhoS[1] * mt_y1b + z0 * mt_y12;
                        ZS(s, 0) = z;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (a_fill > 0) flush();
    if (TC && __syncthreads_or(tc_word[2] != 0u)) return false;

    if (active) {
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const int sp = sg * NS + s;
#pragma unroll
            for (int t = 0; t < P; ++t) {
                // back to the lab frame: m_lab = m_frame * P
                float2 m = make_float2(XS(s, t), YS(s, t));
                if (entered && has_frame<MODEL>(t)) m = cmul(m, Pc[t]);
                const long long i = ((long long)t * L.S + sp) * n + v;
                L.mx[i] = m.x;
                L.my[i] = m.y;
                L.mz[i] = ZS(s, t);
            }
        }
    }
    kbase += (uint32_t)nchunks;
    return true;
#undef TCA
#undef TCB
#undef TPV
#undef XS
#undef YS
#undef ZS
#undef DMX
#undef DMY
#undef DWS
#undef PAIR
#undef UNPAIR
}

// The accurate scan kernel.  A block works through items (instance, tile):
// with counter == nullptr it runs item blockIdx.x alone (one scan, one
// block per tile); otherwise it is persistent and, after item blockIdx.x,
// takes items gridDim.x, gridDim.x + 1, ... from *counter (the batched
// form: the tiles of many scans, ordered longest first).  Each item's
// descriptor is copied from descs into shared memory.  A block whose items
// contract the receive on tcgen05 allocates 32 tensor-memory columns at its
// first such item and frees them before it exits.
template <int MODEL, int P, int NS, bool FREE, int CO = 0, bool TC = false>
__global__ void __launch_bounds__(kBlock, fast_min_blocks<P, NS>())
    scan_fast_kernel(const FastLaunch *__restrict__ descs, const int2 *__restrict__ items, int n_items, int *counter) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ FastLaunch fs;
    __shared__ int next_item;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);  // [0], [1] record chunks, [2] receive MMAs
    uint32_t *tc_word = reinterpret_cast<uint32_t *>(smem + 24);  // tensor memory, contractions, failure
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        fence_mbar_init();
        tc_word[1] = tc_word[2] = 0u;
    }
    uint32_t kbase = 0;
    bool tmem_held = false;
    for (int it = blockIdx.x; it < n_items;) {
        const int2 item = items ? items[it] : make_int2(0, it);
        const int *src = reinterpret_cast<const int *>(descs + item.x);
        int *dst = reinterpret_cast<int *>(&fs);
        for (int w = threadIdx.x; w < (int)(sizeof(FastLaunch) / 4); w += blockDim.x) dst[w] = src[w];
        __syncthreads();
        if (TC && !tmem_held) {
            if (threadIdx.x < 32) tc::tmem_alloc(&tc_word[0], kTcCols);
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            tmem_held = true;
        }
        if (!scan_item<MODEL, P, NS, FREE, CO, TC>(fs, item.y, smem, kbase)) break;
        if (counter == nullptr) break;
        __syncthreads();  // every thread is done with fs and the item's shared memory
        if (threadIdx.x == 0) next_item = atomicAdd(counter, 1) + (int)gridDim.x;
        __syncthreads();
        it = next_item;
    }
    if (TC && tmem_held) {
        tc::fence_before_sync();
        __syncthreads();
        if (threadIdx.x < 32) tc::tmem_dealloc(tc_word[0], kTcCols);
    }
}

}  // namespace mrl
