// Host-side launchers of the scan kernels, one per tissue model (each
// model's instantiations live in their own translation unit so they build
// in parallel).
#pragma once

#include <cuda_runtime.h>

#include "scan_fast_kernel.cuh"
#include "scan_kernel.cuh"

namespace mrl {

// Spins handled per thread for a given SpinNum: all of them when S <= 4 and
// S is 1, 2 or 4; otherwise one spin per thread.
// Spins of one voxel a thread integrates: as many as divide S while a
// thread holds at most 8 isochromat-pools (register budget).
inline int spins_per_thread(int S, int P) {
    for (int ns = 4; ns > 1; ns /= 2)
        if (S % ns == 0 && ns * P <= 8) return ns;
    return 1;
}

// Dynamic shared memory of one block.
inline size_t scan_smem_bytes(int stride4, int nsamp) {
    return 128 + (size_t)2 * kChunk * stride4 * 16 + (size_t)kAdcTile * nsamp * (kBlock + 1) * 8;
}
// ... of the accurate kernel: staged records, coil sensitivities of the
// block's voxels and the per-warp receive tile.
// Receive partial sums per block and sample (both kernels reduce their
// warps' sums in shared memory).
inline int partial_slices(bool fast) {
    (void)fast;
    return 1;
}

// tc_tpv > 0: the receive contraction on tcgen05 (FastLaunch::tc) with
// tc_tpv threads per voxel -- the coil and magnetisation operands from a
// 1024-byte boundary instead of the tile, coil maps and per-warp sums.
inline size_t scan_fast_smem_bytes(int stride4, int rx, int P, int NS, int tc_tpv = 0) {
    const size_t c4 = (size_t)((rx + 3) & ~3);
    const size_t row = kBlock + 2;
    const size_t recv = tc_tpv > 0 ? 1024 + (size_t)tc_a_bytes(tc_tpv) + (size_t)tc_b_bytes(tc_tpv)
                                   : 16 * row * 8 + c4 * row * (coil_presplit((int)c4) ? 16 : 8)  // tile, coil maps
                                         + (kBlock / 32) * 16 * 2 * c4 * 4;  // per-warp receive sums
    return 128 + (size_t)2 * kFastChunk * stride4 * 16  // staged step records
           + recv + ((size_t)2 * ((NS + 1) / 2) * P + 4) * kBlock * 4;  // dWRnd (spin pairs), low parts of omega
}

// One launch of the accurate kernel: n_items work items (instance, tile)
// of the scans described by descs (device memory).  items == nullptr: a
// single scan, item i = tile i, one block per item.  counter != nullptr
// (device int, zero at launch): a persistent grid that takes further items
// from the counter.
struct FastGrid {
    const FastLaunch *descs;
    const int2 *items;
    int n_items;
    int *counter;
};

cudaError_t launch_scan_ref_normal(int P, int NS, dim3 grid, size_t smem, cudaStream_t st, const ScanLaunch &L);
cudaError_t launch_scan_ref_exch(int P, int NS, dim3 grid, size_t smem, cudaStream_t st, const ScanLaunch &L);
cudaError_t launch_scan_ref_mt(int P, int NS, dim3 grid, size_t smem, cudaStream_t st, const ScanLaunch &L);
cudaError_t launch_scan_ref_cest(int P, int NS, dim3 grid, size_t smem, cudaStream_t st, const ScanLaunch &L);

cudaError_t launch_scan_fast_normal(int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                                    const FastGrid &g);
cudaError_t launch_scan_fast_exch(int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                                  const FastGrid &g);
cudaError_t launch_scan_fast_mt(int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                                const FastGrid &g);
cudaError_t launch_scan_fast_cest(int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                                  const FastGrid &g);
// ---- tabulated coefficients and the exact propagator (scan_fast_exact.cu) ------
// Split scheme: free pools exchanging (ME, GM without bound pools); exact
// propagator: ME and GM pools free or bound (a bound pool has no transverse
// generator: identity rows and no inflow); TypeNum <= 3.  Fields of the
// exact table per (dt, voxel): diag(E_T) - 1 [P], E_T off the diagonal
// [P][P] row-major without the diagonal, diag(E_L) - 1 [P], E_L off the
// diagonal, recovery dt phi1(A_L dt) b [P].
__host__ __device__ inline int exact_fields(int P) { return 2 * P * P + P; }
// The split scheme's table (coefficient source 1): y1 [P], y2 [P], yo [P], fin [P][P].
__host__ __device__ inline int split_fields(int P) { return 3 * P + P * P; }
// The instantiations reading a table: co = 1 split scheme, 2 exact propagator
// (all_free false: general-model pools with bound ones, co = 2 only).
cudaError_t launch_scan_fast_tab(int co, int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                                 const FastGrid &g);
int occupancy_scan_fast_tab(int co, int P, int NS, bool all_free, size_t smem);
using FastKernel = void (*)(const FastLaunch *, const int2 *, int, int *);
FastKernel select_exact_bound(int P, int NS);  // scan_fast_exact_bound.cu
// the instantiations with the tcgen05 receive contraction (scan_fast_tc.cu),
// nullptr where none is built: km, coefficient source co (0 or 1), P, NS
FastKernel select_fast_tc(int km, int co, int P, int NS, bool all_free);
cudaError_t launch_split_table(int P, const float *dts, int n_dt, int n_act, int gm, const float *rho,
                               const float *t1, const float *t2, const float *kch, float *tab, cudaStream_t st);
// tab[(d * exact_fields(P) + f) * n_act + v] for the n_dt values dts[]
// (bound: one bit per bound pool; layout of the exchange channels: 0 ME,
// 1 GM, 2 MT, 3 CEST)
cudaError_t launch_exact_table(int P, const float *dts, int n_dt, int n_act, int S, int layout, unsigned bound,
                               const float *rho, const float *t1, const float *t2, const float *kch, float *tab,
                               cudaStream_t st);
// ---- adjoint (adjoint.cu) ----------------------------------------------------
constexpr int kAdjBlock = 128;  // threads (isochromats) per block

// Step record of the adjoint: {dt, Gz, Gy, Gx}, {Re A_0, Im A_0, 2 pi times
// the sum of the active Tx coils' rf frequencies, flags (kFlagRf, kFlagState,
// kFlagDt)}, {ADC sample (int bits) or -1, rf step index (int bits) or -1,
// 0, 0}, then {Re A_c, Im A_c, 0, 0} for every further Tx coil c.
struct AdjLaunch {
    int n_act, S, rx, A, exch_gm;
    int tx;  // Tx coils (txc: [tx][n_act]; records adjoint_record_f4(tx) float4; grf [n_rf][tx][2])
    unsigned bound;  // GM bound pools (TypeFlag 1), one bit per pool
    // MT / CEST (pool 1 bound, kch remapped to the GM layout): a free pool's
    // transverse magnetisation does not flow out to the bound pool, and only
    // pool 0 is received
    int mtc;
    long long n_iso;  // n_act * S; isochromat i = spin (i / n_act) of voxel (i % n_act)
    float gyro;
    const float *gxg, *gyg, *gzg, *db0;  // [n_act]
    const float *rho, *t1, *t2;          // [P][n_act]
    const float *kch;                    // [P*P][n_act] exchange channels, or null
    const float *dwrnd;                  // [P][S][n_act]
    const float2 *rxc;                   // [rx][n_act], null: the default coil
    const float2 *txc;                   // [tx][n_act] TxCoilmg exp(i TxCoilpe)
    float cs2pi[kMaxPool];
    const float4 *rec;                   // [n_steps][adjoint_record_f4(tx)]
    long long n_steps;
    const float *ckpt;                   // [slot][3P][n_iso], every seg windows, written by the forward scan
    int seg;                             // windows (of kAdjWin steps) per stored checkpoint
    float *ck2;                          // seg > 1: [seg][3P][n_iso] the current segment's window checkpoints
    const float2 *gsig;                  // [A][P][rx] dL/dSx + i dL/dSy, one sample's values together
    float *giso;                         // [fields][n_iso]: T1[P] T2[P] Rho[P] dB0 K[P*P] Mx0[P] My0[P] Mz0[P]
    double *grf;                         // [n_rf][tx][2]
};
// float4 of an adjoint step record: the three above, then {Re A_c, Im A_c,
// 0, 0} for every further Tx coil c
__host__ __device__ inline int adjoint_record_f4(int tx) { return 2 + tx; }
// window states, rf partials (per Tx coil), window records, the block's
// receive sensitivities, per warp two buffers of one sample's dL/dS, and the
// further Tx coils' sensitivities
inline size_t adjoint_smem_bytes(int P, int rx, int tx) {
    return (size_t)kAdjWin * 3 * P * kAdjBlock * 4 + (size_t)kAdjWin * (kAdjBlock / 32) * 2 * tx * 4 +
           (size_t)kAdjWin * adjoint_record_f4(tx) * 16 + (size_t)rx * kAdjBlock * 8 +
           (size_t)(kAdjBlock / 32) * 2 * P * rx * 8 + (size_t)(tx - 1) * kAdjBlock * 8;
}
inline int adjoint_fields(int P) { return 3 * P + 1 + P * P + 3 * P; }
cudaError_t launch_adjoint(int P, const AdjLaunch &L, cudaStream_t st);
// MT / CEST exchange channels [nk][n_act] (model layout, see exch_rate) into
// the general model's layout [P*P][n_act] (channel p*P+t = rate t -> p)
cudaError_t launch_remap_k_mtc(int P, int layout, const float *k_src, float *k_gm, int n_act, cudaStream_t st);

// resident blocks per SM of an instantiation at `smem` bytes (0 if none)
int occupancy_scan_fast_normal(int P, int NS, bool all_free, size_t smem);
int occupancy_scan_fast_exch(int P, int NS, bool all_free, size_t smem);
int occupancy_scan_fast_mt(int P, int NS, bool all_free, size_t smem);
int occupancy_scan_fast_cest(int P, int NS, bool all_free, size_t smem);

}  // namespace mrl
