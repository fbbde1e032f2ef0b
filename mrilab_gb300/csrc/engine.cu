// mrl_scan: host side of the GB300 scan engine.
//
// One call replaces the body of a reference GPU mex engine
// (Lib/src/engine/GPUEngine/DoScanAtGPU.cu:215-787 and its ME/MT/CEST/GM
// variants): bind inputs, upload the active voxels once, decode the
// sequence, integrate on the device, sum the receive signal, service Ext
// callbacks, and write the results back in place.
//
// Differences in structure from the reference (results are the same):
//   * voxels whose pools are all empty (T1, T2 or Rho zero) are compacted
//     away instead of being skipped inside the kernel: the caller's arrays
//     are uploaded as they are and gathered on the device, and the final
//     magnetisation is scattered back on the device and downloaded whole;
//   * the magnetisation stays on the device for the whole scan: kernels are
//     launched per block of steps, not per TR, and only Ext events bring
//     data back to the host;
//   * the receive sum is reduced on the device in FP64 instead of
//     downloading per-column partial signals every TR.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <thread>
#include <memory>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/mrl_scan.h"
#include "decode.h"
#include "scan_launch.h"

namespace mrl {

namespace {

thread_local std::string g_err;
thread_local double g_timing[8];

void set_err(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
}

}  // namespace

// Error text and timing of the calling thread, for the other engines of the
// library (mrl_sar): read back through mrl_last_error / mrl_last_timing.
void record_error(const char *msg) { g_err = msg ? msg : ""; }
void record_timing(const double t[8]) {
    for (int i = 0; i < 8; ++i) g_timing[i] = t[i];
}

namespace {

// Receive reduction: Sx/Sy[pool][coil][signal] = sum over blocks of the
// per-block partial sums, then demodulated by rfRef (BlochKernel.cuh:160-170
// applies the same rotation per isochromat).  A block takes 32 consecutive
// (sample, pool, coil) outputs; its 8 warps split the scan blocks (warp w
// sums blocks w, w + 8, ...; 256-byte loads) and their sums are added in a
// fixed order, so results are reproducible.  A lane sums in double-float
// arithmetic (a float sum and the float sum of its exact rounding errors,
// Knuth's two-sum: FP64-level accuracy on the FP32 pipe -- this GPU's FP64
// rate made plain double adds the bound of the reduction), four independent
// chains per component; the warps' sums and the rotation are in FP64.
constexpr int kRedWarps = 8;

// a + b = s + e exactly (Knuth's two-sum; additions only, so nothing is
// contracted into a fused multiply-add)
struct DFSum {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float b) {
        const float s = hi + b;
        const float bb = s - hi;
        lo += (hi - (s - bb)) + (b - bb);
        hi = s;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ void reduce_block(int bx, const float2 *__restrict__ partial, int nblk, int a_launch,
                                             int npairs, int rx, const int *__restrict__ amap, int A, double *sx,
                                             double *sy, double cr, double sr) {
    __shared__ double2 red[kRedWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int o = bx * 32 + lane;
    const int tot = a_launch * npairs;
    double x = 0.0, y = 0.0;
    if (o < tot) {
        const size_t stride = (size_t)a_launch * npairs;
        const float2 *p = partial + o;
        DFSum sx4[4], sy4[4];
        int b = w;
        for (; b + 3 * kRedWarps < nblk; b += 4 * kRedWarps) {
            float2 q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) q[u] = p[(size_t)(b + u * kRedWarps) * stride];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                sx4[u].add(q[u].x);
                sy4[u].add(q[u].y);
            }
        }
        for (; b < nblk; b += kRedWarps) {
            const float2 q = p[(size_t)b * stride];
            sx4[0].add(q.x);
            sy4[0].add(q.y);
        }
        x = (sx4[0].value() + sx4[1].value()) + (sx4[2].value() + sx4[3].value());
        y = (sy4[0].value() + sy4[1].value()) + (sy4[2].value() + sy4[3].value());
    }
    red[w][lane] = make_double2(x, y);
    __syncthreads();
    if (w != 0 || o >= tot) return;
    x = 0.0;
    y = 0.0;
    for (int k = 0; k < kRedWarps; ++k) {
        x += red[k][lane].x;
        y += red[k][lane].y;
    }
    const int a = o / npairs;
    const int pair = o - a * npairs;
    const int sig = amap[a];
    if (sig < 0 || sig >= A) return;
    const int t = pair / rx;
    const int c = pair - t * rx;
    const long long idx = ((long long)t * rx + c) * A + sig;
    sx[idx] = cr * x - sr * y;
    sy[idx] = sr * x + cr * y;
}

__global__ void __launch_bounds__(32 * kRedWarps)
    reduce_partials(const float2 *__restrict__ partial, int nblk, int a_launch, int npairs, int rx,
                    const int *__restrict__ amap, int A, double *sx, double *sy, double cr, double sr) {
    reduce_block(blockIdx.x, partial, nblk, a_launch, npairs, rx, amap, A, sx, sy, cr, sr);
}

// The receive reduction of many scans in one launch: blockIdx.y picks the
// scan, blockIdx.x its block of 32 outputs.
struct RedDesc {
    const float2 *partial;
    const int *amap;
    double *sx, *sy;
    double cr, sr;
    int nblk, a_launch, npairs, rx, A;
};

__global__ void __launch_bounds__(32 * kRedWarps) reduce_partials_batched(const RedDesc *__restrict__ descs) {
    const RedDesc &d = descs[blockIdx.y];
    if ((int)blockIdx.x * 32 >= d.a_launch * d.npairs) return;  // block-uniform
    reduce_block(blockIdx.x, d.partial, d.nblk, d.a_launch, d.npairs, d.rx, d.amap, d.A, d.sx, d.sy, d.cr, d.sr);
}

// ---- object staging on the device -------------------------------------------
// The caller's column-major arrays are uploaded unchanged into one raw
// buffer; gather_object builds the compacted structure-of-arrays the scan
// kernels read (active voxels only, index i -> voxel act[i]) and, for the
// accurate integrator, the frame coefficients in FP64 split into (hi, lo)
// float pairs.  scatter_state writes the compacted magnetisation back into
// the raw arrays, which are then downloaded into the caller's arrays whole.
struct RawObject {
    const float *gx, *gy, *gz, *db0;  // [V]
    const float *txmg, *txpe;         // [Tx][V]
    const float *rho, *t1, *t2;       // [P][V]
    const float *k;                   // [nk][V]
    const float *dwr;                 // [P][S][V]
    float *mx, *my, *mz;              // [P][S][V]
    const float *rxx, *rxy;           // [Rx][V], null for the default coil
};

struct GatherArgs {
    RawObject r;
    const int *act;
    int n_act, n, P, S, TX, RX, nk;
    long long V;
    float *f;  // d_f base
    size_t o_gx, o_gy, o_gz, o_db0, o_txmg, o_txpe, o_rho, o_t1, o_t2, o_k, o_dwr;
    float *m;       // d_m: mx | my | mz, [P][S][n] each
    float2 *rxc;    // [Rx][n]
    float2 *f2;     // frame coefficients, null for reference numerics
    size_t o_om, o_txc;
    double gyro;
};

__device__ __forceinline__ float2 split_df(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}

__global__ void gather_object(GatherArgs G) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= G.n_act) return;
    const long long v = G.act[i];
    const long long V = G.V;
    const size_t n = (size_t)G.n;
    const RawObject &r = G.r;
    float *f = G.f;
    const float gx = r.gx[v], gy = r.gy[v], gz = r.gz[v], db0 = r.db0[v];
    f[G.o_gx + i] = gx;
    f[G.o_gy + i] = gy;
    f[G.o_gz + i] = gz;
    f[G.o_db0 + i] = db0;
    for (int c = 0; c < G.TX; ++c) {
        const float mg = r.txmg[c * V + v], pe = r.txpe[c * V + v];
        f[G.o_txmg + c * n + i] = mg;
        f[G.o_txpe + c * n + i] = pe;
        if (G.f2) {
            double sp, cp;
            sincos((double)pe, &sp, &cp);
            G.f2[G.o_txc + c * n + i] = make_float2((float)((double)mg * cp), (float)((double)mg * sp));
        }
    }
    const size_t ns = n * G.P * G.S;
    for (int t = 0; t < G.P; ++t) {
        f[G.o_rho + t * n + i] = r.rho[t * V + v];
        f[G.o_t1 + t * n + i] = r.t1[t * V + v];
        f[G.o_t2 + t * n + i] = r.t2[t * V + v];
        for (int s = 0; s < G.S; ++s) {
            const long long src = ((long long)t * G.S + s) * V + v;
            const size_t dst = ((size_t)t * G.S + s) * n + i;
            const float w = r.dwr[src];
            f[G.o_dwr + dst] = w;
            G.m[dst] = r.mx[src];
            G.m[ns + dst] = r.my[src];
            G.m[2 * ns + dst] = r.mz[src];
        }
    }
    for (int k = 0; k < G.nk; ++k) f[G.o_k + k * n + i] = r.k[k * V + v];
    if (r.rxx)
        for (int c = 0; c < G.RX; ++c) G.rxc[c * n + i] = make_float2(r.rxx[c * V + v], r.rxy[c * V + v]);
    if (G.f2) {
        G.f2[G.o_om + 0 * n + i] = split_df(G.gyro * (double)db0);
        G.f2[G.o_om + 1 * n + i] = split_df(G.gyro * (double)gx);
        G.f2[G.o_om + 2 * n + i] = split_df(G.gyro * (double)gy);
        G.f2[G.o_om + 3 * n + i] = split_df(G.gyro * (double)gz);
    }
}

__global__ void scatter_state(const float *__restrict__ m, const int *__restrict__ act, int n_act, int n, int PS,
                              long long V, float *mx, float *my, float *mz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_act) return;
    const long long v = act[i];
    const size_t ns = (size_t)n * PS;
    for (int ts = 0; ts < PS; ++ts) {
        const size_t src = (size_t)ts * n + i;
        const long long dst = (long long)ts * V + v;
        mx[dst] = m[src];
        my[dst] = m[ns + src];
        mz[dst] = m[2 * ns + src];
    }
}

// RunMode 1: out[c][j][ts][v] = component c of the state of isochromat-pool
// ts of voxel v at time point j: snapshot snap[j] for an active voxel (inv
// maps a voxel to its compact index), the voxel's unchanging state otherwise.
__global__ void expand_history(const float *__restrict__ hist, long long stride, int n_act,
                               const long long *__restrict__ snap, int npts, const int *__restrict__ inv,
                               long long V, int PS, const float *rx, const float *ry, const float *rz,
                               float *__restrict__ out) {
    const long long total = (long long)npts * PS * V;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long v = e % V;
        const long long r = e / V;
        const int ts = (int)(r % PS);
        const int j = (int)(r / PS);
        const int iv = inv[v];
        float x, y, z;
        if (iv >= 0) {
            const float *h = hist + snap[j] * 3 * stride + (long long)ts * n_act + iv;
            x = h[0];
            y = h[stride];
            z = h[2 * stride];
        } else {
            x = rx[(long long)ts * V + v];
            y = ry[(long long)ts * V + v];
            z = rz[(long long)ts * V + v];
        }
        out[e] = x;
        out[total + e] = y;
        out[2 * total + e] = z;
    }
}

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = std::max<size_t>(count, 1);
        return e;
    }
};

// Coefficient source of the accurate integrator (scan_item): the split
// scheme's table for free pools exchanging with at most three pools, else
// computed in the kernel.
inline int split_source(int km, int P, bool all_free) { return km == KM_EXCH && all_free && P <= 3 ? 1 : 0; }

cudaError_t launch_fast(int km, int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                        const FastGrid &g, int co = 0, bool tc = false) {
    if (tc) {  // the instantiations with the tcgen05 receive
        FastKernel k = select_fast_tc(km, co, P, NS, all_free);
        if (!k) return cudaErrorInvalidValue;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, kBlock, smem, st>>>(g.descs, g.items, g.n_items, g.counter);
        return cudaGetLastError();
    }
    if (co) return launch_scan_fast_tab(co, P, NS, all_free, grid, smem, st, g);
    switch (km) {
    case KM_NORMAL: return launch_scan_fast_normal(P, NS, all_free, grid, smem, st, g);
    case KM_EXCH: return launch_scan_fast_exch(P, NS, all_free, grid, smem, st, g);
    case KM_MT: return launch_scan_fast_mt(P, NS, all_free, grid, smem, st, g);
    default: return launch_scan_fast_cest(P, NS, all_free, grid, smem, st, g);
    }
}

int occupancy_fast(int km, int P, int NS, bool all_free, size_t smem, int co = 0, bool tc = false) {
    if (tc) {
        FastKernel k = select_fast_tc(km, co, P, NS, all_free);
        int n = 0;
        if (!k || cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kBlock, smem) != cudaSuccess)
            return 0;
        return n;
    }
    if (co) return occupancy_scan_fast_tab(co, P, NS, all_free, smem);
    switch (km) {
    case KM_NORMAL: return occupancy_scan_fast_normal(P, NS, all_free, smem);
    case KM_EXCH: return occupancy_scan_fast_exch(P, NS, all_free, smem);
    case KM_MT: return occupancy_scan_fast_mt(P, NS, all_free, smem);
    default: return occupancy_scan_fast_cest(P, NS, all_free, smem);
    }
}

// Receive-tile rows of the accurate kernel's general-model instantiations
// with bound pools: one per sampled (free) pool, in pool order.
void set_sampling(FastLaunch &F, const ScanLaunch &L, int P) {
    F.n_samp = 0;
    for (int t = 0; t < kMaxPool; ++t) F.samp_rank[t] = (t < P && L.kind[t] == 0) ? F.n_samp++ : -1;
}

struct ModelInfo {
    int km;        // KModel
    int nsamp;     // pools with a receive signal slot that can be nonzero
    int nk;        // exchange channels read
    bool gm;
};

// Active-voxel rule of each model: the reference kernels skip a pool (or,
// for MT/CEST, the whole voxel) whose T1, T2 or Rho is zero
// (BlochKernel.cuh:103, BlochKernelGM.cuh:176, BlochKernelMT.cuh:123).
bool voxel_active(const mrl_scan_args &a, int km, long long v, long long V) {
    const int P = a.obj.type_num;
    auto pool = [&](int t) {
        return a.obj.t1[t * V + v] != 0.f && a.obj.t2[t * V + v] != 0.f && a.obj.rho[t * V + v] != 0.f;
    };
    if (km == KM_MT || km == KM_CEST) return pool(0);
    for (int t = 0; t < P; ++t)
        if (pool(t)) return true;
    return false;
}

// ---- host staging of large copies --------------------------------------------
// The caller's arrays are pageable memory (MATLAB's, numpy's); copies of the
// object and of the results go through a pinned buffer of the calling
// thread instead: its host side is copied by several threads at once and
// the DMA runs from pinned memory (pageable copies of the 150 MB object and
// 100 MB of results took 20-30 ms each way).  Below stage_min() bytes (8 MB,
// or MRL_STAGE_MIN_MB) a copy goes directly.
size_t stage_min() {
    const char *e = getenv("MRL_STAGE_MIN_MB");
    return e ? (size_t)(std::max(0.0, atof(e)) * 1048576.0) : (size_t)(8u << 20);
}
struct HostCopy {
    void *dst;
    const void *src;
    size_t bytes;
};
// the host copies of `jobs`, split into pieces of about equal size over up to
// eight threads
void parallel_copy(const std::vector<HostCopy> &jobs) {
    size_t total = 0;
    for (const HostCopy &j : jobs) total += j.bytes;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nth = (int)std::min<size_t>(std::min(8u, hw), std::max<size_t>(1, total / (4u << 20)));
    if (nth <= 1) {
        for (const HostCopy &j : jobs) memcpy(j.dst, j.src, j.bytes);
        return;
    }
    const size_t share = (total + nth - 1) / nth;
    auto run = [&](int t) {  // bytes [t * share, (t + 1) * share) of the concatenated jobs
        size_t lo = (size_t)t * share, hi = std::min(total, lo + share), base = 0;
        for (const HostCopy &j : jobs) {
            const size_t a = std::max(lo, base), b = std::min(hi, base + j.bytes);
            if (a < b)
                memcpy(static_cast<char *>(j.dst) + (a - base), static_cast<const char *>(j.src) + (a - base), b - a);
            base += j.bytes;
        }
    };
    std::vector<std::thread> pool;
    int started = 1;
    try {  // (no exception crosses the C ABI: threads that cannot start are run here)
        for (; started < nth; ++started) pool.emplace_back(run, started);
    } catch (...) {
    }
    for (int t = started; t < nth; ++t) run(t);
    run(0);
    for (std::thread &t : pool) t.join();
}
// the calling thread's pinned staging buffer, grown to `bytes` (null if
// pinned memory cannot be had: the copies then go directly)
struct PinnedStage {
    void *p = nullptr;
    size_t cap = 0;
    ~PinnedStage() {
        if (p) cudaFreeHost(p);
    }
    void *get(size_t bytes) {
        if (p) {  // a device reset frees pinned allocations: then forget this one
            cudaPointerAttributes at{};
            if (cudaPointerGetAttributes(&at, p) != cudaSuccess || at.type != cudaMemoryTypeHost) {
                cudaGetLastError();
                p = nullptr;
                cap = 0;
            }
        }
        if (bytes <= cap) return p;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
            cudaGetLastError();  // clear the error; fall back to direct copies
            p = nullptr;
            return nullptr;
        }
        cap = bytes;
        return p;
    }
};
thread_local PinnedStage t_stage;

struct Scanner {
    mrl_scan_args *args;
    mrl_ext_fn ext;
    void *user;
    ModelInfo mi{};
    int P = 0, S = 0, TX = 0, RX = 0, A = 0, NS = 1, tpv = 1, stride4 = 2;
    long long V = 0;
    int n_act = 0;
    std::vector<int> act;        // compact index -> voxel
    cudaStream_t st = nullptr;
    DevBuf<float> d_f;           // all per-voxel float fields, packed
    DevBuf<float> d_m;           // mx | my | mz
    DevBuf<float2> d_rx;
    DevBuf<float4> d_rec;
    DevBuf<float2> d_part;
    DevBuf<int> d_amap;
    DevBuf<double> d_sx, d_sy;
    DevBuf<int> d_err;
    // accurate integrator: frame coefficients and moments
    bool fast = false;
    FrameMoments fmom;
    DevBuf<float2> d_f2;  // omega [4][n] | txc [Tx][n]
    DevBuf<float> d_raw;  // the caller's arrays as uploaded (RawObject)
    DevBuf<int> d_act;    // compact index -> voxel, on the device
    RawObject raw{};
    size_t o_om = 0, o_txc = 0;
    std::vector<float> frec;
    bool frec_ready = false;  // frec packed ahead (batches pack on host threads)
    // offsets into d_f
    size_t o_gx = 0, o_gy = 0, o_gz = 0, o_db0 = 0, o_txmg = 0, o_txpe = 0, o_rho = 0, o_t1 = 0, o_t2 = 0, o_k = 0,
           o_dwr = 0;
    // RunMode 1 history: snapshots of the state before every dt > 0 step
    bool hist_on = false;
    // adjoint checkpoints (single-chunk scans): every ckpt_every-th step's
    // lab-frame state into ckpt (kFlagCkpt), 0 = off
    float *ckpt = nullptr;
    int ckpt_every = 0;
    DevBuf<float> d_hist;        // [step][Mx|My|Mz][P][S][n_act], then the final state
    long long hist_steps = 0;    // steps of the chunks run so far
    long long hist_cap = 0;      // dt > 0 steps the buffer holds
    std::vector<int> pts_uts;    // every decoded time point: uts index
    std::vector<long long> pts_snap;  // ... and the snapshot holding its state
    std::vector<double> pts_dt;
    // accurate kernel: launch descriptors in device memory, one per launch
    // of the current chunk, uploaded when they change
    std::vector<FastLaunch> h_desc;
    DevBuf<FastLaunch> d_desc;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_scan, ev_red;
    int launches = 0;
    double h2d_ms = 0, d2h_ms = 0, h2d_bytes = 0, d2h_bytes = 0;
    bool own_st = true;          // false: st belongs to the caller (batched scans)
    double partial_budget = 0;   // bytes of receive partials per launch; 0: MRL_PARTIAL_MB or 16 GiB
    // direct receive (accurate numerics, MRL_RECEIVE=direct): blocks add into
    // the FP64 signal with atomics, no partials, one launch per chunk -- for
    // objects whose partials do not fit the device; otherwise partials are
    // faster (atomics: 631 ms, partials: 580 ms on a 128x128x32 32-coil EPI)
    bool direct_rx = false, no_direct = false;
    // exact relaxation-exchange propagator: its coefficient table per
    // (distinct float dt, voxel) and the dt values so far (index = position)
    bool exact = false;
    // MT / CEST under the exact propagator: integrated as the general model
    // with pool 1 bound (the kernel's bound-pool exact instantiation), the
    // model's own K layout read by the table kernel, only pool 0 sampled;
    // km_obj keeps the object's model for the active-voxel rule
    bool mtc_exact = false;
    int km_obj = 0;
    int coef = 0;  // coefficient source: 0 in the kernel, 1 split-scheme table, 2 exact table
    std::map<uint32_t, int> xdt_index;
    std::vector<float> xdts;
    DevBuf<float> d_xdts, d_xtab;

    ~Scanner() {
        for (auto &e : ev_scan) cudaEventDestroy(e.first), cudaEventDestroy(e.second);
        for (auto &e : ev_red) cudaEventDestroy(e.first), cudaEventDestroy(e.second);
        if (st && own_st) cudaStreamDestroy(st);
    }

    // the general model's bound pools (TypeFlag 1), one bit per pool
    // kind of pool t for the exchange kernels: 0 free, 1 bound (GM TypeFlag;
    // pool 1 of MT / CEST under the exact propagator)
    int pool_kind(int t) const {
        if (mtc_exact) return t == 1 ? 1 : 0;
        return (mi.gm && t < P) ? (int)args->obj.type_flag[t] : 0;
    }
    unsigned bound_mask() const {
        unsigned m = 0;
        for (int t = 0; mi.km == KM_EXCH && (mi.gm || mtc_exact) && t < P; ++t)
            if (pool_kind(t) == 1) m |= 1u << t;
        return m;
    }
    // layout of the exchange channels for the table kernels: 0 ME, 1 GM, 2 MT, 3 CEST
    int k_layout() const { return mtc_exact ? (km_obj == KM_MT ? 2 : 3) : (mi.gm ? 1 : 0); }

    // the accurate kernel contracts the receive on tcgen05: 17 to 32 coils,
    // 2 or 4 threads per voxel (64 or 32 voxels per block: the MMAs' K), and
    // an instantiation built for it.  With one thread per voxel (K = 128) the
    // warp-level TF32 form measured faster (MT EPI, 32 coils, 1 spin: 103 ms
    // against 132 ms) and stays the default.  MRL_RECEIVE_TC=1 takes tcgen05
    // wherever it can run (also with one thread per voxel), 0 never.
    bool tc_receive() const {
        const char *e = getenv("MRL_RECEIVE_TC");
        if (e && strcmp(e, "0") == 0) return false;
        const bool force = e && strcmp(e, "1") == 0;
        if (!force && tpv < 2) return false;
        return fast && tc_receive_ok((RX + 3) & ~3, tpv) &&
               select_fast_tc(mi.km, coef, P, NS, all_free() != 0) != nullptr;
    }
    // dynamic shared memory of an accurate-kernel launch of this scan
    size_t fast_smem() const { return scan_fast_smem_bytes(stride4, RX, P, NS, tc_receive() ? tpv : 0); }

    // every pool of an exchange model is a free pool (ME, or GM without bound pools)
    int all_free() const {
        if (mi.km != KM_EXCH) return 0;
        if (mtc_exact) return 0;
        if (!mi.gm) return 1;
        for (int t = 0; t < P; ++t)
            if ((int)args->obj.type_flag[t] != 0) return 0;
        return 1;
    }

    // MRL_DEBUG: host phase times on stderr
    const bool dbg = getenv("MRL_DEBUG") != nullptr;
    std::chrono::steady_clock::time_point t_phase = std::chrono::steady_clock::now();
    void phase(const char *name) {
        if (!dbg) return;
        const auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "mrl: %-16s %9.3f ms\n", name, std::chrono::duration<double, std::milli>(now - t_phase).count());
        t_phase = now;
    }

    int fail_cuda(cudaError_t e, const char *what) {
        set_err("%s: %s", what, cudaGetErrorString(e));
        return MRL_ERR_CUDA;
    }

    int validate() {
        const mrl_scan_args &a = *args;
        if (a.abi_version != MRL_ABI_VERSION) return set_err("abi_version %d, expected %d", a.abi_version, MRL_ABI_VERSION), MRL_ERR_ARG;
        P = a.obj.type_num;
        S = a.obj.spin_num;
        TX = a.coil.tx_num;
        RX = a.coil.rx_num;
        A = a.sig.signal_num;
        V = (long long)a.obj.ny * a.obj.nx * a.obj.nz;
        if (V <= 0 || P < 1 || S < 1 || TX < 1 || RX < 1 || A < 0)
            return set_err("bad sizes V=%lld P=%d S=%d Tx=%d Rx=%d A=%d", V, P, S, TX, RX, A), MRL_ERR_ARG;
        if (V > (1LL << 31) / std::max(1, P * S)) return set_err("spin matrix too large"), MRL_ERR_UNSUPPORTED;
        if (!a.obj.rho || !a.obj.t1 || !a.obj.t2 || !a.obj.mx || !a.obj.my || !a.obj.mz || !a.mag.db0 ||
            !a.mag.dwrnd || !a.mag.gzgrid || !a.mag.gygrid || !a.mag.gxgrid || !a.coil.tx_mg || !a.coil.tx_pe ||
            !a.obj.gyro)
            return set_err("missing input array"), MRL_ERR_ARG;
        if (a.coil.rx_default == 0 && (!a.coil.rx_x || !a.coil.rx_y)) return set_err("missing Rx coil maps"), MRL_ERR_ARG;
        if (A > 0 && (!a.sig.sx || !a.sig.sy)) return set_err("missing signal arrays"), MRL_ERR_ARG;
        if (!a.seq.uts || !a.seq.ts || !a.seq.flags || a.seq.n_ts < 1 || a.seq.n_uts < 1)
            return set_err("empty sequence"), MRL_ERR_ARG;
        if (TX > 4) return set_err("TxCoilNum %d > 4 not supported", TX), MRL_ERR_UNSUPPORTED;
        if (P > kMaxPool) return set_err("TypeNum %d > %d not supported", P, kMaxPool), MRL_ERR_UNSUPPORTED;
        switch (a.model) {
        case MRL_MODEL_NORMAL:
            if (P > 3) return set_err("normal model supports TypeNum <= 3"), MRL_ERR_UNSUPPORTED;
            mi = {KM_NORMAL, P, 0, false};
            break;
        case MRL_MODEL_ME:
        case MRL_MODEL_GM:
            if (P > 5) return set_err("exchange models support TypeNum <= 5"), MRL_ERR_UNSUPPORTED;
            mi = {KM_EXCH, P, P * P, a.model == MRL_MODEL_GM};
            if (mi.gm && !a.obj.type_flag) return set_err("GM model needs TypeFlag"), MRL_ERR_ARG;
            break;
        case MRL_MODEL_MT:
            if (P != 2) return set_err("MT model needs TypeNum == 2"), MRL_ERR_ARG;
            mi = {KM_MT, 1, 4, false};
            break;
        case MRL_MODEL_CEST:
            if (P < 2 || P > 6) return set_err("CEST model supports 2 <= TypeNum <= 6"), MRL_ERR_UNSUPPORTED;
            mi = {KM_CEST, 1, 2 * (P - 1), false};
            break;
        default:
            return set_err("unknown model %d", a.model), MRL_ERR_ARG;
        }
        if (mi.nk > 0 && (!a.obj.k || a.obj.k_channels < mi.nk))
            return set_err("K needs %d channels, got %d", mi.nk, a.obj.k ? a.obj.k_channels : 0), MRL_ERR_ARG;
        fast = a.ctl.numerics == MRL_NUMERICS_ACCURATE || a.ctl.numerics == MRL_NUMERICS_EXACT;
        if (a.ctl.numerics != MRL_NUMERICS_ACCURATE && a.ctl.numerics != MRL_NUMERICS_REFERENCE &&
            a.ctl.numerics != MRL_NUMERICS_EXACT)
            return set_err("unknown numerics %d", a.ctl.numerics), MRL_ERR_ARG;
        exact = a.ctl.numerics == MRL_NUMERICS_EXACT && mi.km != KM_NORMAL;
        km_obj = mi.km;
        if (exact && (mi.km == KM_MT || mi.km == KM_CEST)) {
            if (P > 5) return set_err("MRL_NUMERICS_EXACT supports CEST with TypeNum <= 5"), MRL_ERR_UNSUPPORTED;
            mtc_exact = true;
            // every pool has a signal slot in the exchange kernels' receive
            // layout; only pool 0 is sampled (set_sampling below)
            mi = {KM_EXCH, P, mi.nk, false};
        } else if (exact) {
            // ME, or GM pools free (TypeFlag 0) or bound (1) with a free one
            bool ok = mi.km == KM_EXCH, any_free = !mi.gm;
            for (int t = 0; ok && mi.gm && t < P; ++t) {
                const int k = (int)a.obj.type_flag[t];
                ok = k == 0 || k == 1;
                any_free = any_free || k == 0;
            }
            if (!ok || !any_free)
                return set_err("MRL_NUMERICS_EXACT covers the ME model and GM pools of TypeFlag 0 and 1 "
                               "(with a free pool)"),
                       MRL_ERR_UNSUPPORTED;
            if (P > 3) return set_err("MRL_NUMERICS_EXACT supports TypeNum <= 3"), MRL_ERR_UNSUPPORTED;
        }
        coef = exact ? 2 : (fast ? split_source(mi.km, P, all_free() != 0) : 0);
        hist_on = a.ctl.run_mode == 1;  // other values scan normally, as in the reference's switch
        if (hist_on && !fast)
            return set_err("RunMode 1 (per-step history) needs MRL_NUMERICS_ACCURATE"), MRL_ERR_UNSUPPORTED;
        if (hist_on && (!a.sig.mxs || !a.sig.mys || !a.sig.mzs))
            return set_err("RunMode 1 needs the history arrays VSig.Mx/My/Mz"), MRL_ERR_ARG;
        if (fast && TX > 1) {
            bool bound = mi.km == KM_MT || mi.km == KM_CEST || mtc_exact;
            if (mi.gm)
                for (int t = 0; t < P; ++t) bound |= (int)a.obj.type_flag[t] == 1;
            if (bound)
                return set_err("bound-pool saturation with several Tx coils needs MRL_NUMERICS_REFERENCE"),
                       MRL_ERR_UNSUPPORTED;
        }
        NS = spins_per_thread(S, P);
        if (const char *e = getenv("MRL_SPINS_PER_THREAD")) {
            const int ns = atoi(e);
            if ((ns == 1 || ns == 2 || ns == 4) && S % ns == 0) NS = ns;
        }
        // the exact propagator's bound-pool instantiations hold one spin per
        // thread from four pools up (their tables fill the registers)
        if (exact && !all_free() && P >= 4) NS = 1;
        tpv = S / NS;
        stride4 = fast ? fast_stride_f4(TX) : record_stride_f4(TX);
        return MRL_OK;
    }

    // Upload the caller's arrays unchanged and gather the active voxels into
    // structure-of-arrays form on the device (gather_object).
    int upload_object() {
        const mrl_scan_args &a = *args;
        act.clear();
        for (long long v = 0; v < V; ++v)
            if (voxel_active(a, km_obj, v, V)) act.push_back((int)v);
        n_act = (int)act.size();
        const size_t n = std::max(1, n_act);
        size_t off = 0;
        auto take = [&](size_t cnt) {
            size_t o = off;
            off += cnt;
            return o;
        };
        o_gx = take(n), o_gy = take(n), o_gz = take(n), o_db0 = take(n);
        o_txmg = take(n * TX), o_txpe = take(n * TX);
        o_rho = take(n * P), o_t1 = take(n * P), o_t2 = take(n * P);
        o_k = take(n * std::max(1, mi.nk));
        o_dwr = take(n * P * S);
        if (fast) {
            o_om = 0;
            o_txc = 4 * n;
        }
        phase("active voxels");
        const bool rxmap = a.coil.rx_default == 0;
        // raw buffer: the caller's arrays back to back, in the order below
        const size_t Vs = (size_t)V, PSV = (size_t)P * S * Vs;
        struct Piece {
            const float *host;
            size_t count;
        };
        const Piece pieces[] = {{a.mag.gxgrid, Vs},
                                {a.mag.gygrid, Vs},
                                {a.mag.gzgrid, Vs},
                                {a.mag.db0, Vs},
                                {a.coil.tx_mg, (size_t)TX * Vs},
                                {a.coil.tx_pe, (size_t)TX * Vs},
                                {a.obj.rho, (size_t)P * Vs},
                                {a.obj.t1, (size_t)P * Vs},
                                {a.obj.t2, (size_t)P * Vs},
                                {mi.nk > 0 ? a.obj.k : nullptr, (size_t)mi.nk * Vs},
                                {a.mag.dwrnd, PSV},
                                {a.obj.mx, PSV},
                                {a.obj.my, PSV},
                                {a.obj.mz, PSV},
                                {rxmap ? a.coil.rx_x : nullptr, rxmap ? (size_t)RX * Vs : 0},
                                {rxmap ? a.coil.rx_y : nullptr, rxmap ? (size_t)RX * Vs : 0}};
        constexpr int kPieces = sizeof(pieces) / sizeof(pieces[0]);
        size_t roff[kPieces], rtot = 0;
        for (int q = 0; q < kPieces; ++q) {
            roff[q] = rtot;
            rtot += (pieces[q].count + 63) & ~size_t(63);  // 256-byte aligned pieces
        }
        cudaError_t e;
        if ((e = d_raw.ensure(rtot)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(raw object)");
        if ((e = d_act.ensure(n)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(voxel map)");
        if ((e = d_f.ensure(off)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(object)");
        if ((e = d_m.ensure(3 * n * P * S)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(state)");
        if ((e = d_rx.ensure(rxmap ? n * RX : 1)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(coils)");
        if (fast && (e = d_f2.ensure(o_txc + (size_t)TX * n)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(frame)");
        auto t0 = std::chrono::steady_clock::now();
        // large objects: the pieces copied into the pinned stage in place (one
        // DMA of the whole raw buffer; the stage is free again after the
        // synchronisation below)
        float *stage = rtot * sizeof(float) >= stage_min() ? static_cast<float *>(t_stage.get(rtot * sizeof(float)))
                                                         : nullptr;
        if (stage) {
            std::vector<HostCopy> jobs;
            for (int q = 0; q < kPieces; ++q)
                if (pieces[q].host && pieces[q].count > 0)
                    jobs.push_back({stage + roff[q], pieces[q].host, pieces[q].count * sizeof(float)});
            parallel_copy(jobs);
            if ((e = cudaMemcpyAsync(d_raw.p, stage, rtot * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
                return fail_cuda(e, "upload object");
        }
        for (int q = 0; q < kPieces; ++q) {
            if (!pieces[q].host || pieces[q].count == 0) continue;
            if (!stage && (e = cudaMemcpyAsync(d_raw.p + roff[q], pieces[q].host, pieces[q].count * sizeof(float),
                                               cudaMemcpyHostToDevice, st)) != cudaSuccess)
                return fail_cuda(e, "upload object");
            h2d_bytes += (double)pieces[q].count * sizeof(float);
        }
        if (n_act > 0) {
            if ((e = cudaMemcpyAsync(d_act.p, act.data(), (size_t)n_act * sizeof(int), cudaMemcpyHostToDevice, st)) !=
                cudaSuccess)
                return fail_cuda(e, "upload voxel map");
            h2d_bytes += (double)n_act * sizeof(int);
        }
        raw.gx = d_raw.p + roff[0];
        raw.gy = d_raw.p + roff[1];
        raw.gz = d_raw.p + roff[2];
        raw.db0 = d_raw.p + roff[3];
        raw.txmg = d_raw.p + roff[4];
        raw.txpe = d_raw.p + roff[5];
        raw.rho = d_raw.p + roff[6];
        raw.t1 = d_raw.p + roff[7];
        raw.t2 = d_raw.p + roff[8];
        raw.k = d_raw.p + roff[9];
        raw.dwr = d_raw.p + roff[10];
        raw.mx = d_raw.p + roff[11];
        raw.my = d_raw.p + roff[12];
        raw.mz = d_raw.p + roff[13];
        raw.rxx = rxmap ? d_raw.p + roff[14] : nullptr;
        raw.rxy = rxmap ? d_raw.p + roff[15] : nullptr;
        if (n_act > 0) {
            GatherArgs G{};
            G.r = raw;
            G.act = d_act.p;
            G.n_act = n_act;
            G.n = (int)n;
            G.P = P;
            G.S = S;
            G.TX = TX;
            G.RX = RX;
            G.nk = mi.nk;
            G.V = V;
            G.f = d_f.p;
            G.o_gx = o_gx, G.o_gy = o_gy, G.o_gz = o_gz, G.o_db0 = o_db0, G.o_txmg = o_txmg, G.o_txpe = o_txpe;
            G.o_rho = o_rho, G.o_t1 = o_t1, G.o_t2 = o_t2, G.o_k = o_k, G.o_dwr = o_dwr;
            G.m = d_m.p;
            G.rxc = d_rx.p;
            G.f2 = fast ? d_f2.p : nullptr;
            G.o_om = o_om, G.o_txc = o_txc;
            G.gyro = a.obj.gyro;
            gather_object<<<(n_act + 255) / 256, 256, 0, st>>>(G);
            if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "gather launch");
        }
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "upload sync");
        h2d_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        phase("upload object");
        if (dbg) fprintf(stderr, "mrl: upload_object n_act=%d of %lld voxels\n", n_act, V);
        return MRL_OK;
    }

    // Copy the device magnetisation back into the caller's arrays.
    int download_state() {
        mrl_scan_args &a = *args;
        if (n_act == 0) return MRL_OK;  // nothing was integrated
        const size_t n = std::max(1, n_act);
        const size_t PSV = (size_t)P * S * V;
        auto t0 = std::chrono::steady_clock::now();
        scatter_state<<<(n_act + 255) / 256, 256, 0, st>>>(d_m.p, d_act.p, n_act, (int)n, P * S, V, raw.mx, raw.my,
                                                          raw.mz);
        cudaError_t e = cudaGetLastError();
        // large states: the three (padded, consecutive) raw arrays in one DMA
        // into the pinned stage, then copied out on several threads
        const size_t span = (size_t)(raw.mz + PSV - raw.mx);
        float *stage = 3 * PSV * sizeof(float) >= stage_min() ? static_cast<float *>(t_stage.get(span * sizeof(float)))
                                                            : nullptr;
        if (stage) {
            if (e == cudaSuccess) e = cudaMemcpyAsync(stage, raw.mx, span * sizeof(float), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e == cudaSuccess)
                parallel_copy({{a.obj.mx, stage, PSV * sizeof(float)},
                               {a.obj.my, stage + (raw.my - raw.mx), PSV * sizeof(float)},
                               {a.obj.mz, stage + (raw.mz - raw.mx), PSV * sizeof(float)}});
        } else {
            if (e == cudaSuccess) e = cudaMemcpyAsync(a.obj.mx, raw.mx, PSV * sizeof(float), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(a.obj.my, raw.my, PSV * sizeof(float), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(a.obj.mz, raw.mz, PSV * sizeof(float), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        }
        d2h_bytes += 3.0 * PSV * sizeof(float);
        if (e != cudaSuccess) return fail_cuda(e, "download state");
        d2h_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return MRL_OK;
    }

    // Copy acquired samples [a0, a1) of every (pool, coil) row to the host.
    int download_signal(int a0, int a1) {
        if (a1 <= a0 || A == 0) return MRL_OK;
        a1 = std::min(a1, A);
        if (a1 <= a0) return MRL_OK;
        mrl_scan_args &a = *args;
        const size_t pitch = (size_t)A * sizeof(double);
        d2h_bytes += 2.0 * (a1 - a0) * sizeof(double) * P * RX;
        auto t0 = std::chrono::steady_clock::now();
        const size_t rows = (size_t)P * RX, wb = (size_t)(a1 - a0) * sizeof(double);
        // large signals: both into the pinned stage ([Sx rows][Sy rows], packed),
        // then copied out on several threads
        char *stage = 2 * rows * wb >= stage_min() ? static_cast<char *>(t_stage.get(2 * rows * wb)) : nullptr;
        cudaError_t e;
        if (stage) {
            e = cudaMemcpy2DAsync(stage, wb, d_sx.p + a0, pitch, wb, rows, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaMemcpy2DAsync(stage + rows * wb, wb, d_sy.p + a0, pitch, wb, rows, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e == cudaSuccess) {
                std::vector<HostCopy> jobs;
                for (size_t r = 0; r < rows; ++r) {
                    jobs.push_back({a.sig.sx + r * A + a0, stage + r * wb, wb});
                    jobs.push_back({a.sig.sy + r * A + a0, stage + (rows + r) * wb, wb});
                }
                parallel_copy(jobs);
            }
        } else {
            e = cudaMemcpy2DAsync(a.sig.sx + a0, pitch, d_sx.p + a0, pitch, wb, rows, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaMemcpy2DAsync(a.sig.sy + a0, pitch, d_sy.p + a0, pitch, wb, rows, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        }
        if (e != cudaSuccess) return fail_cuda(e, "download signal");
        d2h_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return MRL_OK;
    }

    ScanLaunch make_launch(double rf_ref) {
        const mrl_scan_args &a = *args;
        const size_t n = std::max(1, n_act);
        ScanLaunch L{};
        L.n_act = n_act;
        L.S = S;
        L.tx = TX;
        L.rx = RX;
        L.nsamp = mi.nsamp;
        L.npairs = mi.nsamp * RX;
        L.tpv = tpv;
        L.gyro = (float)a.obj.gyro;
        L.rx_default = a.coil.rx_default != 0;
        L.exch_gm = mi.gm ? 1 : 0;
        L.gxg = d_f.p + o_gx;
        L.gyg = d_f.p + o_gy;
        L.gzg = d_f.p + o_gz;
        L.db0 = d_f.p + o_db0;
        L.txmg = d_f.p + o_txmg;
        L.txpe = d_f.p + o_txpe;
        L.rxc = d_rx.p;
        L.rho = d_f.p + o_rho;
        L.t1 = d_f.p + o_t1;
        L.t2 = d_f.p + o_t2;
        L.kch = d_f.p + o_k;
        L.dwrnd = d_f.p + o_dwr;
        L.mx = d_m.p;
        L.my = d_m.p + n * P * S;
        L.mz = d_m.p + 2 * n * P * S;
        L.stride4 = stride4;
        L.err = d_err.p;
        for (int t = 0; t < kMaxPool; ++t) {
            L.cs2pi[t] = t < P && a.ctl.cs ? (float)(2 * kPiRef * (double)(float)a.ctl.cs[t]) : 0.f;
            L.kind[t] = t < P ? pool_kind(t) : 0;
        }
        (void)rf_ref;
        return L;
    }

    struct LaunchDesc {
        long long s0, s1;
        int a_off, a_count;
    };
    std::vector<LaunchDesc> plan_launches;
    std::vector<int> amap_host;
    long long n_steps_total = 0, n_rf_total = 0;
    int n_adc_total = 0;

    long long n_blocks() const {
        const long long nthreads = (long long)n_act * tpv;
        return std::max(1LL, (nthreads + kBlock - 1) / kBlock);
    }
    // receive partial sums of one sample: one per block (reference order)
    // or per warp (accurate kernel)
    long long n_slices() const { return n_blocks() * partial_slices(fast); }

    // Split a decoded chunk into launches whose receive partials fit the
    // budget (MRL_PARTIAL_MB, default 16 GiB or a quarter of the free memory), upload its step records and
    // ADC map, and size the partial buffer.
    // Exact propagator: the index of every step's float dt in its flags (bits
    // 8 and up), and the coefficient table of every dt value so far (FP64
    // exponentials, one thread per (dt, voxel)).
    int tab_coefficients(std::vector<float> &rec) {
        const int stride = fast_stride_f4(TX) * 4;
        const size_t n_before = xdts.size();
        for (size_t q = 0; q < rec.size() / stride; ++q) {
            float *r = &rec[q * stride];
            uint32_t key;
            std::memcpy(&key, &r[0], sizeof(key));
            auto it = xdt_index.find(key);
            int idx;
            if (it == xdt_index.end()) {
                idx = (int)xdts.size();
                if (idx >= (1 << 22)) return set_err("more than 2^22 distinct step lengths"), MRL_ERR_UNSUPPORTED;
                xdt_index.emplace(key, idx);
                xdts.push_back(r[0]);
            } else {
                idx = it->second;
            }
            int flags;
            std::memcpy(&flags, &r[7], sizeof(int));
            flags |= idx << 8;
            std::memcpy(&r[7], &flags, sizeof(int));
        }
        if (n_act == 0 || (xdts.size() == n_before && d_xtab.p)) return MRL_OK;
        cudaError_t e = d_xdts.ensure(xdts.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_xdts.p, xdts.data(), xdts.size() * sizeof(float), cudaMemcpyHostToDevice, st);
        const int nf = coef == 2 ? exact_fields(P) : split_fields(P);
        if (e == cudaSuccess) e = d_xtab.ensure(xdts.size() * (size_t)nf * n_act);
        const float *kch = mi.nk > 0 ? d_f.p + o_k : nullptr;
        if (e == cudaSuccess)
            e = coef == 2 ? launch_exact_table(P, d_xdts.p, (int)xdts.size(), n_act, S, k_layout(),
                                               bound_mask(), d_f.p + o_rho, d_f.p + o_t1, d_f.p + o_t2, kch,
                                               d_xtab.p, st)
                          : launch_split_table(P, d_xdts.p, (int)xdts.size(), n_act, mi.gm ? 1 : 0,
                                               d_f.p + o_rho, d_f.p + o_t1, d_f.p + o_t2, kch, d_xtab.p, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail_cuda(e, "coefficient table");
        return MRL_OK;
    }

    int prepare_chunk(const DecodeChunk &ch, std::vector<LaunchDesc> &out) {
        out.clear();
        amap_host.clear();
        if (ch.n_steps == 0) return MRL_OK;
        const int npairs = mi.nsamp * RX;
        const char *env = getenv("MRL_PARTIAL_MB");
        double budget = partial_budget;
        if (budget <= 0 && env) budget = atof(env) * 1048576.0;
        if (budget <= 0) {  // 16 GiB, at most a quarter of the free device memory
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            budget = std::max(256.0 * 1048576.0, std::min(16.0 * 1073741824.0, 0.25 * (double)free_b));
        }
        long long a_max = std::max(1LL, (long long)(budget / ((double)n_slices() * npairs * sizeof(float2))));
        {
            long long n_adc = 0;
            for (long long q = 0; q < ch.n_steps; ++q) n_adc += ch.step_adc[q] >= 0;
            const char *mode = getenv("MRL_RECEIVE");
            direct_rx = fast && !no_direct && mode && strcmp(mode, "direct") == 0;
            if (direct_rx) a_max = std::max(1LL, n_adc);
        }
        long long s0 = 0;
        int a_off = 0, a_cnt = 0, a_peak = 0;
        for (long long q = 0; q < ch.n_steps; ++q) {
            if (ch.step_adc[q] < 0) continue;
            if (a_cnt == a_max) {
                out.push_back({s0, q, a_off, a_cnt});
                a_peak = std::max(a_peak, a_cnt);
                s0 = q;
                a_off += a_cnt;
                a_cnt = 0;
            }
            amap_host.push_back(ch.step_adc[q]);
            a_cnt++;
        }
        out.push_back({s0, ch.n_steps, a_off, a_cnt});
        a_peak = std::max(a_peak, a_cnt);
        const std::vector<float> *recs = &ch.records;
        if (fast) {
            if (!frec_ready) pack_fast_records(ch, TX, fmom, frec, ckpt_every);
            frec_ready = false;
            recs = &frec;
            if (coef) {
                const int rc = tab_coefficients(frec);
                if (rc) return rc;
            }
        }
        phase("pack records");
        cudaError_t e;
        if ((e = d_rec.ensure(recs->size() / 4)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(steps)");
        if ((e = d_amap.ensure(std::max<size_t>(1, amap_host.size()))) != cudaSuccess)
            return fail_cuda(e, "cudaMalloc(amap)");
        if ((e = d_part.ensure(direct_rx ? 1 : (size_t)n_slices() * std::max(1, a_peak) * npairs)) != cudaSuccess)
            return fail_cuda(e, "cudaMalloc(partials)");
        auto t0 = std::chrono::steady_clock::now();
        if ((e = cudaMemcpyAsync(d_rec.p, recs->data(), recs->size() * sizeof(float), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            return fail_cuda(e, "upload steps");
        h2d_bytes += (double)recs->size() * sizeof(float) + amap_host.size() * sizeof(int);
        if (!amap_host.empty() &&
            (e = cudaMemcpyAsync(d_amap.p, amap_host.data(), amap_host.size() * sizeof(int), cudaMemcpyHostToDevice,
                                 st)) != cudaSuccess)
            return fail_cuda(e, "upload amap");
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "upload steps");
        h2d_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        phase("upload steps");
        return MRL_OK;
    }

    // Enqueue the launches of a prepared chunk on `stream` (no host sync).
    // Descriptor of the accurate kernel for launch fields L.
    FastLaunch fast_launch(const ScanLaunch &L) const {
        FastLaunch F{};
        F.b = L;
        F.omega = d_f2.p + o_om;
        F.txc = d_f2.p + o_txc;
        F.all_free = all_free();
        F.tc = tc_receive() ? 1 : 0;
        set_sampling(F, L, P);
        if (mtc_exact) {  // MT / CEST sample pool 0 only (BlochKernelMT.cuh:230)
            F.n_samp = 1;
            for (int t = 0; t < kMaxPool; ++t) F.samp_rank[t] = t == 0 ? 0 : -1;
        }
        for (int t = 0; t < kMaxPool; ++t) {  // 2 pi CS[t] as a (hi, lo) pair
            const double w = (t < P && args->ctl.cs) ? 2 * kPiRef * args->ctl.cs[t] : 0.0;
            F.cs_hi[t] = (float)w;
            F.cs_lo[t] = (float)(w - (double)F.cs_hi[t]);
        }
        return F;
    }

    // Launch fields of launch d of the current chunk.
    ScanLaunch launch_fields(const LaunchDesc &d, double rf_ref) {
        ScanLaunch L = make_launch(rf_ref);
        L.rec = d_rec.p;
        L.partial = d_part.p;
        L.s0 = d.s0;
        L.s1 = d.s1;
        L.a_launch = d.a_count;
        L.hist_stride = (long long)P * S * std::max(1, n_act);
        L.hist = hist_on ? d_hist.p + (hist_steps + d.s0) * 3 * L.hist_stride : nullptr;
        L.ckpt = ckpt;
        L.ckpt_step0 = d.s0;
        L.ckpt_every = std::max(1, ckpt_every);
        L.xtab = coef ? d_xtab.p : nullptr;
        L.xnf = coef == 2 ? exact_fields(P) : split_fields(P);
        if (direct_rx) {
            L.dsx = d_sx.p;
            L.dsy = d_sy.p;
            L.amap = d_amap.p + d.a_off;
            L.A = A;
            L.cr = std::cos(-rf_ref);
            L.sr = std::sin(-rf_ref);
        }
        return L;
    }

    // Upload the accurate kernel's descriptors of launches ls (if changed).
    int upload_descs(const std::vector<LaunchDesc> &ls, double rf_ref, cudaStream_t stream) {
        std::vector<FastLaunch> h;
        h.reserve(ls.size());
        for (const LaunchDesc &d : ls) h.push_back(fast_launch(launch_fields(d, rf_ref)));
        if (h.size() == h_desc.size() && std::memcmp(h.data(), h_desc.data(), h.size() * sizeof(FastLaunch)) == 0)
            return MRL_OK;
        cudaError_t e = d_desc.ensure(h.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_desc.p, h.data(), h.size() * sizeof(FastLaunch), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return fail_cuda(e, "upload launch descriptors");
        h_desc.swap(h);
        return MRL_OK;
    }

    int enqueue(const std::vector<LaunchDesc> &ls, double rf_ref, cudaStream_t stream, bool timed) {
        if (ls.empty()) return MRL_OK;
        const int nblk = (int)n_blocks();
        const size_t smem =
            fast ? fast_smem() : scan_smem_bytes(stride4, mi.nsamp);
        const double cr = std::cos(-rf_ref), sr = std::sin(-rf_ref);
        cudaError_t e;
        int rc;
        if (fast && n_act > 0 && (rc = upload_descs(ls, rf_ref, stream))) return rc;
        for (size_t li = 0; li < ls.size(); ++li) {
            const LaunchDesc &d = ls[li];
            ScanLaunch L = launch_fields(d, rf_ref);
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (timed) {
                cudaEventCreate(&e0);
                cudaEventCreate(&e1);
                ev_scan.push_back({e0, e1});
                cudaEventRecord(e0, stream);
            }
            if (n_act > 0) {
                dim3 grid(nblk);
                if (fast) {
                    const FastGrid g{d_desc.p + li, nullptr, nblk, nullptr};
                    e = launch_fast(mi.km, P, NS, all_free() != 0, grid, smem, stream, g, coef, tc_receive());
                } else {
                    switch (mi.km) {
                    case KM_NORMAL: e = launch_scan_ref_normal(P, NS, grid, smem, stream, L); break;
                    case KM_EXCH: e = launch_scan_ref_exch(P, NS, grid, smem, stream, L); break;
                    case KM_MT: e = launch_scan_ref_mt(P, NS, grid, smem, stream, L); break;
                    default: e = launch_scan_ref_cest(P, NS, grid, smem, stream, L); break;
                    }
                }
                if (e != cudaSuccess) return fail_cuda(e, "scan kernel launch");
                launches++;
            }
            if (timed) cudaEventRecord(e1, stream);
            if (d.a_count > 0 && n_act > 0 && !direct_rx) {
                cudaEvent_t r0 = nullptr, r1 = nullptr;
                if (timed) {
                    cudaEventCreate(&r0);
                    cudaEventCreate(&r1);
                    ev_red.push_back({r0, r1});
                    cudaEventRecord(r0, stream);
                }
                const int tot = d.a_count * L.npairs;
                reduce_partials<<<(tot + 31) / 32, 32 * kRedWarps, 0, stream>>>(d_part.p, (int)n_slices(), d.a_count,
                                                                                  L.npairs, RX,
                                                                       d_amap.p + d.a_off, A, d_sx.p, d_sy.p, cr, sr);
                if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "reduce launch");
                launches++;
                if (timed) cudaEventRecord(r1, stream);
            }
        }
        return MRL_OK;
    }

    int run_chunk(const DecodeChunk &ch, double rf_ref) {
        std::vector<LaunchDesc> ls;
        int rc = prepare_chunk(ch, ls);
        if (rc) return rc;
        if (hist_on && hist_steps + ch.n_steps > hist_cap) return set_err("history buffer overrun"), MRL_ERR_ARG;
        if ((rc = enqueue(ls, rf_ref, st, true))) return rc;
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail_cuda(e, "scan kernels");
        phase("scan kernels");
        if (hist_on) {
            for (size_t j = 0; j < ch.point_uts.size(); ++j) {
                pts_uts.push_back(ch.point_uts[j]);
                pts_snap.push_back(hist_steps + ch.point_step[j]);
                pts_dt.push_back(ch.point_dt[j]);
            }
            hist_steps += ch.n_steps;
        }
        return MRL_OK;
    }

    int setup() {
        int rc = validate();
        if (rc) return rc;
        phase("validate");
        cudaError_t e;
        int dev = args->ctl.gpu_index;
        if ((e = cudaSetDevice(dev)) != cudaSuccess) {
            set_err("cudaSetDevice(%d): %s", dev, cudaGetErrorString(e));
            return e == cudaErrorNoDevice || e == cudaErrorInvalidDevice ? MRL_ERR_NO_DEVICE : MRL_ERR_CUDA;
        }
        if (!st && (e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess)
            return fail_cuda(e, "cudaStreamCreate");
        if ((e = d_err.ensure(1)) != cudaSuccess) return fail_cuda(e, "cudaMalloc(err)");
        cudaMemsetAsync(d_err.p, 0, sizeof(int), st);
        const size_t nsig = (size_t)P * RX * std::max(A, 1);
        if ((e = d_sx.ensure(nsig)) != cudaSuccess || (e = d_sy.ensure(nsig)) != cudaSuccess)
            return fail_cuda(e, "cudaMalloc(signal)");
        cudaMemsetAsync(d_sx.p, 0, nsig * sizeof(double), st);
        cudaMemsetAsync(d_sy.p, 0, nsig * sizeof(double), st);
        phase("device setup");
        if ((rc = upload_object())) return rc;
        return hist_on ? setup_history() : MRL_OK;
    }

    // RunMode 1: room for a snapshot before every dt > 0 step still to run
    // and one for the final state.
    int setup_history() {
        const mrl_sequence &q = args->seq;
        const int u0 = args->var.utsi ? *args->var.utsi : 0;
        hist_cap = 0;
        for (int i = std::max(0, u0); i + 1 < q.n_uts; ++i) hist_cap += q.uts[i + 1] - q.uts[i] > 0;
        const double stride = (double)P * S * std::max(1, n_act);
        const double bytes = (double)(hist_cap + 1) * 3 * stride * sizeof(float) +
                             (double)std::max(0, q.n_uts - u0) * 3 * P * S * (double)V * sizeof(float);
        if (bytes > 32.0 * (1ull << 30))
            return set_err("RunMode 1 history needs %.1f GiB of device memory (limit 32 GiB)", bytes / (1ull << 30)),
                   MRL_ERR_NOMEM;
        cudaError_t e = d_hist.ensure((size_t)((hist_cap + 1) * 3 * (long long)stride));
        if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(history)");
        hist_steps = 0;
        pts_uts.clear();
        pts_snap.clear();
        pts_dt.clear();
        return MRL_OK;
    }

    // RunMode 1 output: VSig.Mx/My/Mz[slot] = state at uts[slot] for every
    // decoded time point (the GPU engines' d_b_M* copies,
    // DoGMScanAtGPU.cu:347-358,831-840), VSig.Muts accumulated like
    // DoGMScanAtGPU.cu:437-446.
    int write_history() {
        mrl_scan_args &a = *args;
        const size_t npts = pts_uts.size();
        if (npts == 0) return MRL_OK;
        for (size_t j = 1; j < npts; ++j)
            if (pts_uts[j] != pts_uts[0] + (int)j) return set_err("history time points not contiguous"), MRL_ERR_ARG;
        const long long stride = (long long)P * S * std::max(1, n_act);
        cudaError_t e = cudaMemcpyAsync(d_hist.p + hist_steps * 3 * stride, d_m.p, 3 * stride * sizeof(float),
                                        cudaMemcpyDeviceToDevice, st);  // the final state
        std::vector<int> inv((size_t)V, -1);
        for (int j = 0; j < n_act; ++j) inv[act[j]] = j;
        DevBuf<int> d_inv;
        DevBuf<long long> d_snap;
        DevBuf<float> d_out;
        const long long PSV = (long long)P * S * V;
        if (e == cudaSuccess) e = d_inv.ensure(inv.size());
        if (e == cudaSuccess) e = d_snap.ensure(npts);
        if (e == cudaSuccess) e = d_out.ensure((size_t)(3 * (long long)npts * PSV));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_inv.p, inv.data(), inv.size() * sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_snap.p, pts_snap.data(), npts * sizeof(long long), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return fail_cuda(e, "history setup");
        const long long total = (long long)npts * PSV;
        const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 32);
        expand_history<<<blocks, 256, 0, st>>>(d_hist.p, stride, std::max(1, n_act), d_snap.p, (int)npts, d_inv.p, V,
                                               P * S, raw.mx, raw.my, raw.mz, d_out.p);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "history launch");
        launches++;
        float *dst[3] = {a.sig.mxs, a.sig.mys, a.sig.mzs};
        for (int c = 0; c < 3 && e == cudaSuccess; ++c)
            e = cudaMemcpyAsync(dst[c] + (long long)pts_uts[0] * PSV, d_out.p + c * total, total * sizeof(float),
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail_cuda(e, "history download");
        d2h_bytes += 3.0 * total * sizeof(float);
        if (a.sig.muts) {
            const int nu = a.seq.n_uts;
            for (size_t j = 0; j < npts; ++j) {
                const int cur = pts_uts[j], nxt = cur + 1 < nu - 1 ? cur + 1 : nu - 1;
                if (pts_dt[j] > 0)
                    a.sig.muts[nxt] = a.sig.muts[cur] + pts_dt[j];
                else if (pts_dt[j] < 0)
                    a.sig.muts[nxt] = a.sig.muts[cur];
            }
        }
        return MRL_OK;
    }

    // Active isochromat-pools (the work of one step).
    long long iso_pools() const {
        const mrl_scan_args &a = *args;
        long long n = 0;
        for (int i = 0; i < n_act; ++i) {
            const long long v = act[i];
            if (mi.km == KM_MT || mi.km == KM_CEST) {
                n += P;
            } else {
                for (int t = 0; t < P; ++t)
                    n += a.obj.t1[t * V + v] != 0.f && a.obj.t2[t * V + v] != 0.f && a.obj.rho[t * V + v] != 0.f;
            }
        }
        return n * S;
    }

    int check_device_status() {
        int herr = 0;
        cudaError_t e = cudaMemcpy(&herr, d_err.p, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail_cuda(e, "read status");
        if (herr) {
            set_err("a device wait timed out (status bits %d)", herr);
            return MRL_ERR_TIMEOUT;
        }
        return MRL_OK;
    }

    int run() {
        int rc = setup();
        if (rc) return rc;
        cudaError_t e;

        DecodeState ds;
        load_state(ds, args->var, TX);
        ds.i = 0;
        ds.signali = 0;
        DecodeChunk ch;
        int signal_synced = 0;
        for (;;) {
            decode_until_ext(ds, args->seq, TX, args->obj.gyro, args->sig, ch);
            phase("decode");
            const double rf_ref = args->var.rf_ref ? *args->var.rf_ref : 0.0;
            if ((rc = run_chunk(ch, rf_ref))) return rc;
            if (!ch.stopped_at_ext) break;
            // Ext event: make the signal and the cursor current, then run
            // DoGPUFetch / DoExtPlugin (DoScanAtGPU.cu:565-660)
            if ((rc = download_signal(signal_synced, ds.signali))) return rc;
            signal_synced = ds.signali;
            store_state(ds, args->var, TX);
            if (ext) {
                const int fetch = ext(user, args, MRL_EXT_FETCH);
                if (getenv("MRL_DEBUG")) fprintf(stderr, "mrl: Ext value %g, fetch %d\n", ds.ext, fetch);
                if (fetch && (rc = download_state())) return rc;
                if (ext(user, args, MRL_EXT_PLUGIN) != 0) {
                    set_err("Ext plugin returned an error");
                    return MRL_ERR_EXT;
                }
                load_state(ds, args->var, TX);
                if (fetch) {
                    const std::vector<int> act_before = act;
                    if ((rc = upload_object())) return rc;
                    if (hist_on && act != act_before)
                        return set_err("RunMode 1: an Ext plugin changed which voxels are active"),
                               MRL_ERR_UNSUPPORTED;
                }
            }
        }
        if ((rc = download_signal(signal_synced, ds.signali))) return rc;
        phase("download signal");
        if ((rc = download_state())) return rc;
        phase("download state");
        if (hist_on && (rc = write_history())) return rc;
        store_state(ds, args->var, TX);
        if ((rc = check_device_status())) return rc;
        (void)e;
        double scan_ms = 0, red_ms = 0;
        for (auto &p : ev_scan) {
            float ms = 0;
            cudaEventElapsedTime(&ms, p.first, p.second);
            scan_ms += ms;
        }
        for (auto &p : ev_red) {
            float ms = 0;
            cudaEventElapsedTime(&ms, p.first, p.second);
            red_ms += ms;
        }
        g_timing[1] = scan_ms;
        g_timing[2] = red_ms;
        g_timing[3] = h2d_ms;
        g_timing[4] = d2h_ms;
        g_timing[5] = launches;
        g_timing[6] = h2d_bytes;
        g_timing[7] = d2h_bytes;
        return MRL_OK;
    }
};

// ---- allocation-free scans (mrl_scan_noalloc) -------------------------------
// Scratch of mrl_scan_noalloc: [status word, padded to 256 B][kernel
// launch descriptor, padded to 256 B][ADC map of one launch (int)][receive
// partial sums (float2)].  One array per process per device, shared by
// every call.
constexpr size_t kNoAllocDescBytes = (sizeof(FastLaunch) + 255) / 256 * 256;
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};

// Device address of the scratch array on the current device.  Host code
// only sees a host-side stand-in named g_noalloc_scratch; the device address
// comes from cudaGetSymbolAddress, fetched once per device.
cudaError_t noalloc_scratch(int dev, unsigned char **out) {
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_noalloc_ptr[dev]);
    return cudaSuccess;
}

// TF32 rounding of the receive contraction: integer form and the
// hardware conversion side by side (hook of their equality test).
__global__ void tf32_probe(const float *x, uint32_t *rn, uint32_t *cvt, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        rn[i] = tf32_rn(x[i]);
        cvt[i] = to_tf32(x[i]);
    }
}

// Device sine/cosine of the accurate kernel on caller-given arguments: the
// hook of its accuracy test (not part of the scan interface).
__global__ void sincos_probe(const float *x, float *sn, float *cs, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float a, b;
        sincos_cw(x[i], a, b);
        sn[i] = a;
        cs[i] = b;
    }
}

// 1 - exp(-x) of the accurate kernel and CUDA's -expm1f(-x) on caller-given
// arguments: the hook of its accuracy test.
__global__ void one_minus_exp_probe(const float *x, float *ours, float *lib, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        ours[i] = one_minus_exp(x[i]);
        lib[i] = -expm1f(-x[i]);
    }
}

}  // namespace
}  // namespace mrl

struct mrl_plan {
    mrl::Scanner sc;
    mrl_scan_args args{};
    mrl::DevBuf<float> d_m0;
    std::vector<mrl::Scanner::LaunchDesc> ls;
    std::vector<double> kx, ky, kz;
    double rf_ref = 0;
    long long work[5] = {0, 0, 0, 0, 0};
};

// Batched scans: one Scanner per instance (sharing the batch's stream), the
// instances grouped by kernel instantiation, one persistent launch per group.
struct mrl_batch {
    struct Inst {
        std::unique_ptr<mrl::Scanner> sc;
        mrl_scan_args args{};
        mrl::DevBuf<float> d_m0;                     // initial magnetisation
        std::vector<mrl::Scanner::LaunchDesc> ls;    // exactly one launch
        std::vector<double> kx, ky, kz;
        double rf_ref = 0;
        long long steps = 0, rf_steps = 0, units = 0, samples = 0;
        int group = -1, slot = -1;                   // group and descriptor slot in it
    };
    struct Group {
        int km = 0, P = 0, NS = 1;
        bool free = false;
        bool tc = false;                             // the tcgen05 receive instantiation
        int cap = 0;                                 // resident blocks per SM (0: occupancy)
        std::vector<int> inst;
        size_t smem = 0;
        int grid = 0, n_items = 0;
        mrl::DevBuf<mrl::FastLaunch> descs;
        mrl::DevBuf<int2> items;
        mrl::DevBuf<int> counter;
        cudaStream_t st = nullptr;
        cudaEvent_t done = nullptr;
    };
    std::vector<Inst> in;
    std::vector<Group> groups;
    mrl::DevBuf<int> d_err;
    mrl::DevBuf<mrl::RedDesc> d_red;
    int red_x = 0, device = 0, sms = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    void drop_groups() {
        for (Group &g : groups) {
            if (g.st) cudaStreamDestroy(g.st);
            if (g.done) cudaEventDestroy(g.done);
        }
        groups.clear();
    }
    ~mrl_batch() {
        drop_graph();
        drop_groups();
        in.clear();  // Scanners before the stream they use
        if (fork) cudaEventDestroy(fork);
        if (st) cudaStreamDestroy(st);
    }
};

namespace mrl {
namespace {

// Descriptor of instance `it` for a run over at most `max_steps` steps.
FastLaunch batch_desc(mrl_batch &b, mrl_batch::Inst &it, long long max_steps) {
    Scanner &sc = *it.sc;
    ScanLaunch L = sc.launch_fields(it.ls[0], it.rf_ref);
    if (max_steps >= 0) L.s1 = std::min(L.s1, L.s0 + max_steps);
    L.err = b.d_err.p;
    return sc.fast_launch(L);
}

// (Re)build the groups from every instance's current spins per thread:
// descriptors, the item list ordered longest first, the persistent grid.
int batch_build(mrl_batch &b, long long max_steps) {
    std::vector<int> caps;
    for (auto &g : b.groups) caps.push_back(g.cap);
    std::vector<std::tuple<int, int, int, bool, bool, int>> keys;
    for (auto &g : b.groups) keys.emplace_back(g.km, g.P, g.NS, g.free, g.tc, g.cap);
    b.drop_groups();
    for (size_t i = 0; i < b.in.size(); ++i) {
        Scanner &sc = *b.in[i].sc;
        const bool fr = sc.all_free() != 0;
        const bool tc = sc.tc_receive();
        int gi = -1;
        for (size_t k = 0; k < b.groups.size(); ++k) {
            const auto &g = b.groups[k];
            if (g.km == sc.mi.km && g.P == sc.P && g.NS == sc.NS && g.free == fr && g.tc == tc) gi = (int)k;
        }
        if (gi < 0) {
            mrl_batch::Group g;
            g.km = sc.mi.km;
            g.P = sc.P;
            g.NS = sc.NS;
            g.free = fr;
            g.tc = tc;
            for (auto &k : keys)  // keep a tuned resident-block cap
                if (std::get<0>(k) == g.km && std::get<1>(k) == g.P && std::get<2>(k) == g.NS &&
                    std::get<3>(k) == g.free && std::get<4>(k) == g.tc)
                    g.cap = std::get<5>(k);
            b.groups.push_back(std::move(g));
            gi = (int)b.groups.size() - 1;
        }
        b.in[i].group = gi;
        b.in[i].slot = (int)b.groups[gi].inst.size();
        b.groups[gi].inst.push_back((int)i);
    }
    for (auto &g : b.groups) {
        std::vector<FastLaunch> h;
        std::vector<std::pair<long long, int2>> items;  // (cost, item)
        g.smem = 0;
        for (int i : g.inst) {
            mrl_batch::Inst &it = b.in[i];
            Scanner &sc = *it.sc;
            h.push_back(batch_desc(b, it, max_steps));
            g.smem = std::max(g.smem, sc.fast_smem());
            const long long steps = max_steps >= 0 ? std::min(it.steps, max_steps) : it.steps;
            const long long cost = steps + 3 * std::min(it.rf_steps, steps);  // an rf step costs ~4 free steps
            const int nblk = sc.n_act > 0 ? (int)sc.n_blocks() : 0;
            for (int t = 0; t < nblk; ++t) items.push_back({cost, make_int2(it.slot, t)});
        }
        std::stable_sort(items.begin(), items.end(),
                         [](const std::pair<long long, int2> &x, const std::pair<long long, int2> &y) {
                             return x.first > y.first;
                         });
        std::vector<int2> hi;
        for (auto &x : items) hi.push_back(x.second);
        g.n_items = (int)hi.size();
        cudaError_t e = g.descs.ensure(h.size());
        if (e == cudaSuccess) e = g.items.ensure(std::max<size_t>(1, hi.size()));
        if (e == cudaSuccess) e = g.counter.ensure(1);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(g.descs.p, h.data(), h.size() * sizeof(FastLaunch), cudaMemcpyHostToDevice, b.st);
        if (e == cudaSuccess && !hi.empty())
            e = cudaMemcpyAsync(g.items.p, hi.data(), hi.size() * sizeof(int2), cudaMemcpyHostToDevice, b.st);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b.st);
        if (e != cudaSuccess) return set_err("batch setup: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
        const int occ = occupancy_fast(g.km, g.P, g.NS, g.free, g.smem, split_source(g.km, g.P, g.free), g.tc);
        if (occ < 1) return set_err("batch: kernel does not fit (%zu bytes of shared memory)", g.smem), MRL_ERR_UNSUPPORTED;
        const int per_sm = g.cap > 0 ? std::min(g.cap, occ) : occ;
        g.grid = std::max(1, std::min(g.n_items, per_sm * b.sms));
    }
    // receive reduction of every instance (block counts follow the spins per thread)
    std::vector<RedDesc> rd;
    b.red_x = 0;
    for (auto &it : b.in) {
        Scanner &sc = *it.sc;
        const Scanner::LaunchDesc &d = it.ls[0];
        RedDesc r{};
        r.partial = sc.d_part.p;
        r.amap = sc.d_amap.p + d.a_off;
        r.sx = sc.d_sx.p;
        r.sy = sc.d_sy.p;
        r.cr = std::cos(-it.rf_ref);
        r.sr = std::sin(-it.rf_ref);
        r.nblk = (int)sc.n_slices();
        r.a_launch = sc.n_act > 0 ? d.a_count : 0;
        r.npairs = sc.mi.nsamp * sc.RX;
        r.rx = sc.RX;
        r.A = sc.A;
        rd.push_back(r);
        b.red_x = std::max(b.red_x, (r.a_launch * r.npairs + 31) / 32);
    }
    cudaError_t e = b.d_red.ensure(rd.size());
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b.d_red.p, rd.data(), rd.size() * sizeof(RedDesc), cudaMemcpyHostToDevice, b.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b.st);
    if (e != cudaSuccess) return set_err("batch setup: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    return MRL_OK;
}

// Enqueue one batched execution on s: reset, one persistent launch per
// group on the groups' streams (forked from and joined back into s), then
// the receive reduction of every instance.
int batch_record(mrl_batch &b, cudaStream_t s, bool reduce) {
    cudaError_t e = cudaMemsetAsync(b.d_err.p, 0, sizeof(int), s);
    for (auto &it : b.in)
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(it.sc->d_m.p, it.d_m0.p, it.d_m0.n * sizeof(float), cudaMemcpyDeviceToDevice, s);
    for (auto &g : b.groups)
        if (e == cudaSuccess) e = cudaMemsetAsync(g.counter.p, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaEventRecord(b.fork, s);
    for (auto &g : b.groups) {
        if (e != cudaSuccess) break;
        e = cudaStreamWaitEvent(g.st, b.fork, 0);
        if (e == cudaSuccess && g.n_items > 0)
            e = launch_fast(g.km, g.P, g.NS, g.free, dim3(g.grid), g.smem, g.st,
                            FastGrid{g.descs.p, g.items.p, g.n_items, g.counter.p}, split_source(g.km, g.P, g.free),
                            g.tc);
        if (e == cudaSuccess) e = cudaEventRecord(g.done, g.st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g.done, 0);
    }
    if (e == cudaSuccess && reduce && b.red_x > 0) {
        reduce_partials_batched<<<dim3(b.red_x, (unsigned)b.in.size()), 32 * kRedWarps, 0, s>>>(b.d_red.p);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return set_err("batch launch: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    return MRL_OK;
}

}  // namespace
}  // namespace mrl

extern "C" {

int mrl_scan(mrl_scan_args *args, mrl_ext_fn ext, void *user) {
    mrl::g_err.clear();
    for (double &t : mrl::g_timing) t = 0;
    if (!args) {
        mrl::set_err("args is NULL");
        return MRL_ERR_ARG;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    auto t0 = std::chrono::steady_clock::now();
    int rc;
    {
        mrl::Scanner sc;
        sc.args = args;
        sc.ext = ext;
        sc.user = user;
        rc = sc.run();
    }
    mrl::g_timing[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    cudaSetDevice(prev);
    return rc;
}

}  // extern "C"

namespace {
// Windows of kAdjWin steps per checkpoint segment of an adjoint plan: 1 (a
// stored checkpoint every kAdjWin steps) while those fit in half the free
// device memory, else the smallest power of two M for which the stored
// checkpoints (one every M windows) and one segment's rebuilt window
// checkpoints (M) fit.  MRL_ADJ_SEGMENT=M overrides the choice.
int adjoint_segment(long long n_steps, long long n_iso, int P) {
    if (const char *e = std::getenv("MRL_ADJ_SEGMENT")) {
        const int m = std::atoi(e);
        if (m >= 1) return m;
    }
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const double one = 3.0 * P * (double)std::max(1LL, n_iso) * sizeof(float);
    const long long nwin = std::max(1LL, (n_steps + mrl::kAdjWin - 1) / mrl::kAdjWin);
    long long M = 1;
    for (; M < nwin; M *= 2)
        if (one * (double)((nwin + M - 1) / M + (M > 1 ? M : 0)) <= 0.5 * (double)fr) break;
    return (int)std::min<long long>(M, 1 << 20);
}

// A prepared scan.  ckpt_every > 0 flags every ckpt_every-th step for an
// adjoint checkpoint (< 0: kAdjWin times adjoint_segment's choice); `keep`
// (optional) receives the decoded sequence.
int plan_create_impl(const mrl_scan_args *args, mrl_plan **out, int ckpt_every, mrl::DecodeChunk *keep) {
    mrl::g_err.clear();
    if (!args || !out) {
        mrl::set_err("NULL argument");
        return MRL_ERR_ARG;
    }
    *out = nullptr;
    if (args->ctl.run_mode == 1) {
        mrl::set_err("plans do not record RunMode 1 history; use mrl_scan");
        return MRL_ERR_UNSUPPORTED;
    }
    mrl_plan *p = new mrl_plan();
    p->args = *args;
    mrl::Scanner &sc = p->sc;
    sc.args = &p->args;
    sc.ext = nullptr;
    sc.user = nullptr;
    int rc = sc.setup();
    if (rc) {
        delete p;
        return rc;
    }
    const int A = sc.A;
    p->kx.assign(std::max(A, 1), 0.0);
    p->ky.assign(std::max(A, 1), 0.0);
    p->kz.assign(std::max(A, 1), 0.0);
    mrl_signal sig = p->args.sig;
    sig.kx = p->kx.data();
    sig.ky = p->ky.data();
    sig.kz = p->kz.data();
    mrl::DecodeState ds;
    mrl_state none{};
    mrl::load_state(ds, none, sc.TX);
    ds.tr_count = 0;
    mrl::DecodeChunk ch;
    mrl::decode_until_ext(ds, p->args.seq, sc.TX, p->args.obj.gyro, sig, ch);
    if (ch.stopped_at_ext) {
        mrl::set_err("the sequence has Ext events: use mrl_scan with a callback");
        delete p;
        return MRL_ERR_UNSUPPORTED;
    }
    if (ckpt_every < 0) ckpt_every = mrl::kAdjWin * adjoint_segment(ch.n_steps, (long long)sc.n_act * sc.S, sc.P);
    sc.ckpt_every = ckpt_every;
    if ((rc = sc.prepare_chunk(ch, p->ls))) {
        delete p;
        return rc;
    }
    p->rf_ref = args->var.rf_ref ? *args->var.rf_ref : 0.0;
    cudaError_t e = p->d_m0.ensure(sc.d_m.n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_m0.p, sc.d_m.p, sc.d_m.n * sizeof(float), cudaMemcpyDeviceToDevice, sc.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sc.st);
    if (e != cudaSuccess) {
        sc.fail_cuda(e, "plan state copy");
        delete p;
        return MRL_ERR_CUDA;
    }
    long long launches = 0;
    for (auto &d : p->ls) launches += 1 + (d.a_count > 0 ? 1 : 0);
    p->work[0] = sc.iso_pools() * ch.n_steps;  // active isochromat-pools x dt>0 steps
    p->work[1] = ch.n_steps;
    p->work[2] = ch.n_rf_steps;
    p->work[3] = ch.adc_end - ch.adc_begin;
    p->work[4] = launches;
    if (keep) *keep = std::move(ch);
    *out = p;
    return MRL_OK;
}
}  // namespace

extern "C" {

int mrl_plan_create(const mrl_scan_args *args, mrl_plan **out) { return plan_create_impl(args, out, 0, nullptr); }

int mrl_plan_execute(mrl_plan *p, void *stream) {
    if (!p) return MRL_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(p->sc.d_m.p, p->d_m0.p, p->sc.d_m.n * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && p->sc.direct_rx) {  // the direct receive accumulates into the signal
        e = cudaMemsetAsync(p->sc.d_sx.p, 0, p->sc.d_sx.n * sizeof(double), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(p->sc.d_sy.p, 0, p->sc.d_sy.n * sizeof(double), s);
    }
    if (e != cudaSuccess) return p->sc.fail_cuda(e, "plan reset");
    return p->sc.enqueue(p->ls, p->rf_ref, s, false);
}

int mrl_plan_download(mrl_plan *p, mrl_scan_args *args) {
    if (!p || !args) return MRL_ERR_ARG;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return p->sc.fail_cuda(e, "plan sync");
    int rc = p->sc.check_device_status();
    if (rc) return rc;
    mrl_scan_args *keep = p->sc.args;
    p->sc.args = args;
    rc = p->sc.download_signal(0, p->sc.A);
    if (!rc) rc = p->sc.download_state();
    p->sc.args = keep;
    for (int i = 0; i < p->sc.A; ++i) {
        if (args->sig.kx) args->sig.kx[i] = p->kx[i];
        if (args->sig.ky) args->sig.ky[i] = p->ky[i];
        if (args->sig.kz) args->sig.kz[i] = p->kz[i];
    }
    return rc;
}

int mrl_plan_work(const mrl_plan *p, long long out[5]) {
    if (!p || !out) return MRL_ERR_ARG;
    for (int i = 0; i < 5; ++i) out[i] = p->work[i];
    return MRL_OK;
}

void mrl_plan_destroy(mrl_plan *p) { delete p; }

int mrl_batch_create(mrl_scan_args *const *args, int n, mrl_batch **out) {
    using namespace mrl;
    g_err.clear();
    if (!args || n < 1 || !out) {
        set_err("mrl_batch_create: NULL argument or n < 1");
        return MRL_ERR_ARG;
    }
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!args[i]) return set_err("instance %d: NULL", i), MRL_ERR_ARG;
        if (args[i]->ctl.gpu_index != args[0]->ctl.gpu_index)
            return set_err("instance %d: every instance of a batch runs on one GPU", i), MRL_ERR_ARG;
        if (args[i]->ctl.run_mode == 1)
            return set_err("instance %d: batches do not record RunMode 1 history", i), MRL_ERR_UNSUPPORTED;
        if (args[i]->ctl.numerics != MRL_NUMERICS_ACCURATE)
            return set_err("instance %d: batches run MRL_NUMERICS_ACCURATE", i), MRL_ERR_UNSUPPORTED;
    }
    std::unique_ptr<mrl_batch> b(new mrl_batch());
    b->device = args[0]->ctl.gpu_index;
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) {
        set_err("cudaSetDevice(%d): %s", b->device, cudaGetErrorString(e));
        return e == cudaErrorNoDevice || e == cudaErrorInvalidDevice ? MRL_ERR_NO_DEVICE : MRL_ERR_CUDA;
    }
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = b->d_err.ensure(1);
    if (e != cudaSuccess) return set_err("batch setup: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    b->in.resize(n);
    for (int i = 0; i < n; ++i) {
        mrl_batch::Inst &it = b->in[i];
        it.args = *args[i];
        it.sc.reset(new Scanner());
        Scanner &sc = *it.sc;
        sc.args = &it.args;
        sc.st = b->st;
        sc.own_st = false;
        sc.partial_budget = 1e18;  // one launch per instance
        sc.no_direct = true;       // the batch reduces every instance's partials in one kernel
        const int rc = sc.validate();
        if (rc) {
            const std::string why = g_err;
            set_err("instance %d: %s", i, why.c_str());
            return rc;
        }
    }
    // the instances' sequences decoded and their records packed on host threads
    // (independent per instance; the host's share of a batch of long trains)
    std::vector<DecodeChunk> chunks(n);
    {
        std::atomic<int> next{0};
        auto work = [&]() {
            for (int i; (i = next.fetch_add(1)) < n;) {
                mrl_batch::Inst &it = b->in[i];
                Scanner &sc = *it.sc;
                it.kx.assign(std::max(sc.A, 1), 0.0);
                it.ky.assign(std::max(sc.A, 1), 0.0);
                it.kz.assign(std::max(sc.A, 1), 0.0);
                mrl_signal sig = it.args.sig;
                sig.kx = it.kx.data();
                sig.ky = it.ky.data();
                sig.kz = it.kz.data();
                DecodeState ds;
                mrl_state none{};
                load_state(ds, none, sc.TX);
                decode_until_ext(ds, it.args.seq, sc.TX, it.args.obj.gyro, sig, chunks[i]);
                if (!chunks[i].stopped_at_ext && sc.fast) {
                    pack_fast_records(chunks[i], sc.TX, sc.fmom, sc.frec, sc.ckpt_every);
                    sc.frec_ready = true;
                }
            }
        };
        const int nth = (int)std::max(1u, std::min<unsigned>((unsigned)n, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int t = 1; t < nth; ++t) pool.emplace_back(work);
        work();
        for (std::thread &t : pool) t.join();
    }
    for (int i = 0; i < n; ++i) {
        mrl_batch::Inst &it = b->in[i];
        Scanner &sc = *it.sc;
        int rc = sc.setup();
        if (rc) {
            const std::string why = g_err;
            set_err("instance %d: %s", i, why.c_str());
            return rc;
        }
        const DecodeChunk &ch = chunks[i];
        if (ch.stopped_at_ext) return set_err("instance %d: the sequence has Ext events", i), MRL_ERR_UNSUPPORTED;
        if ((rc = sc.prepare_chunk(ch, it.ls))) return rc;
        if (it.ls.size() != 1) return set_err("instance %d: receive partials do not fit one launch", i), MRL_ERR_NOMEM;
        // room for the partials of one spin per thread, the most blocks the tuner may pick
        const long long nblk1 = std::max(1LL, ((long long)sc.n_act * sc.S + kBlock - 1) / kBlock);
        if ((e = sc.d_part.ensure((size_t)nblk1 * std::max(1, it.ls[0].a_count) * sc.mi.nsamp * sc.RX)) !=
            cudaSuccess)
            return sc.fail_cuda(e, "cudaMalloc(partials)");
        it.rf_ref = it.args.var.rf_ref ? *it.args.var.rf_ref : 0.0;
        if ((e = it.d_m0.ensure(sc.d_m.n)) == cudaSuccess)
            e = cudaMemcpyAsync(it.d_m0.p, sc.d_m.p, sc.d_m.n * sizeof(float), cudaMemcpyDeviceToDevice, b->st);
        if (e != cudaSuccess) return sc.fail_cuda(e, "batch state copy");
        it.steps = ch.n_steps;
        it.rf_steps = ch.n_rf_steps;
        it.units = sc.iso_pools() * ch.n_steps;
        it.samples = ch.adc_end - ch.adc_begin;
    }
    int rc = batch_build(*b, -1);
    if (rc) return rc;
    *out = b.release();
    return MRL_OK;
}

int mrl_batch_execute(mrl_batch *b, int mode, void *stream) {
    using namespace mrl;
    if (!b || (mode != MRL_BATCH_PERSISTENT && mode != MRL_BATCH_PLAIN)) return MRL_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return set_err("cudaSetDevice: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    if (mode == MRL_BATCH_PERSISTENT) {
        if (!b->exec) {  // capture once, replay after
            if ((e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                return set_err("graph capture: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
            const int rc = batch_record(*b, b->st, true);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(b->st, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
            b->graph = g;
            if (e != cudaSuccess) {
                b->drop_graph();
                return set_err("graph instantiate: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
            }
        }
        if ((e = cudaGraphLaunch(b->exec, s)) != cudaSuccess)
            return set_err("graph launch: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
        return MRL_OK;
    }
    // plain: each instance in turn, its own launch and reduction
    e = cudaMemsetAsync(b->d_err.p, 0, sizeof(int), s);
    for (auto &it : b->in) {
        Scanner &sc = *it.sc;
        const mrl_batch::Group &g = b->groups[it.group];
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sc.d_m.p, it.d_m0.p, it.d_m0.n * sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess || sc.n_act == 0) continue;
        const int nblk = (int)sc.n_blocks();
        e = launch_fast(g.km, g.P, g.NS, g.free, dim3(nblk), sc.fast_smem(), s,
                        FastGrid{g.descs.p + it.slot, nullptr, nblk, nullptr}, split_source(g.km, g.P, g.free),
                        g.tc);
        const mrl::Scanner::LaunchDesc &d = it.ls[0];
        if (e == cudaSuccess && d.a_count > 0) {
            const int npairs = sc.mi.nsamp * sc.RX;
            const int tot = d.a_count * npairs;
            reduce_partials<<<(tot + 31) / 32, 32 * kRedWarps, 0, s>>>(
                sc.d_part.p, (int)sc.n_slices(), d.a_count, npairs, sc.RX, sc.d_amap.p + d.a_off, sc.A, sc.d_sx.p,
                sc.d_sy.p, std::cos(-it.rf_ref), std::sin(-it.rf_ref));
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) return set_err("batch launch: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    return MRL_OK;
}

int mrl_batch_tune(mrl_batch *b, void *stream) {
    using namespace mrl;
    if (!b) return MRL_ERR_ARG;
    (void)stream;  // trials run on the batch's own stream
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return set_err("cudaSetDevice: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    constexpr long long kTrialSteps = 256;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = MRL_OK;
    const std::vector<std::vector<int>> sets = [&] {
        std::vector<std::vector<int>> v;
        for (auto &g : b->groups) v.push_back(g.inst);
        return v;
    }();
    for (const std::vector<int> &set : sets) {
        if (rc) break;
        double best = 1e300;
        int best_ns = b->in[set[0]].sc->NS, best_cap = 0;
        long long units = 0;
        for (int i : set) units += b->in[i].units / std::max(1LL, b->in[i].steps) * std::min(b->in[i].steps, kTrialSteps);
        for (int ns : {1, 2, 4}) {
            bool ok = true;
            for (int i : set) ok &= b->in[i].sc->S % ns == 0 && b->in[i].sc->P * ns <= 8;
            if (!ok) continue;
            for (int i : set) {
                b->in[i].sc->NS = ns;
                b->in[i].sc->tpv = b->in[i].sc->S / ns;
            }
            if ((rc = batch_build(*b, kTrialSteps))) break;
            mrl_batch::Group &g = b->groups[b->in[set[0]].group];
            const int occ = occupancy_fast(g.km, g.P, g.NS, g.free, g.smem, split_source(g.km, g.P, g.free), g.tc);
            for (int cap : {occ, occ - 1}) {
                if (cap < 1 || g.n_items == 0) continue;
                const int grid = std::max(1, std::min(g.n_items, cap * b->sms));
                float ms = 0, run_best = 1e30f;
                for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
                    for (int i : set)
                        if (e == cudaSuccess)
                            e = cudaMemcpyAsync(b->in[i].sc->d_m.p, b->in[i].d_m0.p, b->in[i].d_m0.n * sizeof(float),
                                                cudaMemcpyDeviceToDevice, b->st);
                    if (e == cudaSuccess) e = cudaMemsetAsync(g.counter.p, 0, sizeof(int), b->st);
                    if (e == cudaSuccess) e = cudaEventRecord(e0, b->st);
                    if (e == cudaSuccess)
                        e = launch_fast(g.km, g.P, g.NS, g.free, dim3(grid), g.smem, b->st,
                                        FastGrid{g.descs.p, g.items.p, g.n_items, g.counter.p}, split_source(g.km, g.P, g.free),
                            g.tc);
                    if (e == cudaSuccess) e = cudaEventRecord(e1, b->st);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) run_best = std::min(run_best, ms);  // the first run warms up
                }
                if (e != cudaSuccess) break;
                const double per_unit = run_best / std::max(1LL, units);
                if (per_unit < best) {
                    best = per_unit;
                    best_ns = ns;
                    best_cap = cap;
                }
            }
            if (e != cudaSuccess) break;
        }
        if (e != cudaSuccess) {
            rc = MRL_ERR_CUDA;
            set_err("batch tune: %s", cudaGetErrorString(e));
            break;
        }
        for (int i : set) {
            b->in[i].sc->NS = best_ns;
            b->in[i].sc->tpv = b->in[i].sc->S / best_ns;
        }
        if ((rc = batch_build(*b, -1))) break;
        b->groups[b->in[set[0]].group].cap = best_cap;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc) rc = batch_build(*b, -1);  // final grids with the chosen caps
    if (!rc) {
        for (auto &it : b->in)
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(it.sc->d_m.p, it.d_m0.p, it.d_m0.n * sizeof(float), cudaMemcpyDeviceToDevice, b->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
        if (e != cudaSuccess) rc = MRL_ERR_CUDA;
    }
    b->drop_graph();  // the next persistent execution captures the tuned launches
    return rc;
}

int mrl_batch_download(mrl_batch *b, mrl_scan_args *const *args, int n) {
    using namespace mrl;
    if (!b || !args || n != (int)b->in.size()) return MRL_ERR_ARG;
    cudaError_t e = cudaSetDevice(b->device);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return set_err("batch sync: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    int herr = 0;
    if ((e = cudaMemcpy(&herr, b->d_err.p, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return set_err("batch status: %s", cudaGetErrorString(e)), MRL_ERR_CUDA;
    if (herr) return set_err("a device wait timed out (status bits %d)", herr), MRL_ERR_TIMEOUT;
    for (int i = 0; i < n; ++i) {
        if (!args[i]) return MRL_ERR_ARG;
        mrl_batch::Inst &it = b->in[i];
        Scanner &sc = *it.sc;
        mrl_scan_args *keep = sc.args;
        sc.args = args[i];
        int rc = sc.download_signal(0, sc.A);
        if (!rc) rc = sc.download_state();
        sc.args = keep;
        if (rc) return rc;
        for (int a = 0; a < sc.A; ++a) {
            if (args[i]->sig.kx) args[i]->sig.kx[a] = it.kx[a];
            if (args[i]->sig.ky) args[i]->sig.ky[a] = it.ky[a];
            if (args[i]->sig.kz) args[i]->sig.kz[a] = it.kz[a];
        }
    }
    return MRL_OK;
}

int mrl_batch_work(const mrl_batch *b, long long out[5]) {
    if (!b || !out) return MRL_ERR_ARG;
    for (int k = 0; k < 5; ++k) out[k] = 0;
    for (const auto &it : b->in) {
        out[0] += it.units;
        out[1] += it.steps;
        out[2] += it.samples;
        out[4] += (it.sc->n_act > 0) + (it.ls[0].a_count > 0);
    }
    for (const auto &g : b->groups) out[3] += g.n_items > 0;
    out[3] += b->red_x > 0;
    return MRL_OK;
}

void mrl_batch_destroy(mrl_batch *b) { delete b; }

int mrl_scan_batched(mrl_scan_args *const *args, int n) {
    mrl_batch *b = nullptr;
    int rc = mrl_batch_create(args, n, &b);
    if (!rc) rc = mrl_batch_execute(b, MRL_BATCH_PERSISTENT, nullptr);
    if (!rc) rc = mrl_batch_download(b, args, n);
    mrl_batch_destroy(b);
    return rc;
}

}  // extern "C"

// An adjoint plan: the forward scan, prepared with a checkpoint every
// kAdjWin steps, and the adjoint kernel's inputs and outputs, resident.
struct mrl_adjoint_plan {
    mrl_plan *fwd = nullptr;
    mrl::DevBuf<float4> d_rec;
    mrl::DevBuf<float> d_ck, d_ck2, d_g, d_kgm;  // d_kgm: MT / CEST channels in the general layout
    mrl::DevBuf<float2> d_gs;
    mrl::DevBuf<double> d_rf;
    mrl::AdjLaunch L{};
    // per rf step: uts index; per rf step and Tx coil: the rfAmpLine and
    // rfPhaseLine entries held (-1: none or the coil is off), Re A and Im A,
    // whether the coil is on
    std::vector<int> rf_uts, rf_src, rf_on;
    std::vector<double> rf_a;
    int P = 0, S = 0, RX = 0, A = 0, TX = 1, n_rf = 0, ck_every = 0;
    long long V = 0, n_iso = 0, N = 0, ck_bytes = 0;
    double rf_ref = 0;
    bool forward_done = false, backward_done = false;
    ~mrl_adjoint_plan() {
        if (fwd) mrl_plan_destroy(fwd);
    }
};

extern "C" {

int mrl_adjoint_plan_create(const mrl_scan_args *args, mrl_adjoint_plan **out) {
    using namespace mrl;
    g_err.clear();
    if (!args || !out) return set_err("NULL argument"), MRL_ERR_ARG;
    *out = nullptr;
    if (args->ctl.run_mode == 1) return set_err("the adjoint runs RunMode 0 scans"), MRL_ERR_UNSUPPORTED;
    std::unique_ptr<mrl_adjoint_plan> p(new mrl_adjoint_plan());
    mrl_scan_args a = *args;
    a.ctl.numerics = MRL_NUMERICS_ACCURATE;  // the checkpoints come from the accurate integrator
    DecodeChunk ch;
    int rc = plan_create_impl(&a, &p->fwd, -1, &ch);
    if (rc) return rc;
    Scanner &sc = p->fwd->sc;
    // MT and CEST run as the general model with pool 1 bound (their K
    // channels remapped), their transverse map and pool-0 receive
    const bool mtc = sc.mi.km == KM_MT || sc.mi.km == KM_CEST;
    if (!(sc.mi.km == KM_NORMAL || sc.mi.km == KM_EXCH || mtc))
        return set_err("unknown model for the adjoint"), MRL_ERR_UNSUPPORTED;
    if (sc.TX > 4) return set_err("the adjoint supports up to 4 Tx coils"), MRL_ERR_UNSUPPORTED;
    if (sc.P > 3) return set_err("the adjoint supports TypeNum <= 3"), MRL_ERR_UNSUPPORTED;
    if (mtc && sc.P < 2) return set_err("the MT / CEST adjoint needs the bound pool"), MRL_ERR_UNSUPPORTED;
    if (sc.RX > 32) return set_err("the adjoint supports up to 32 Rx coils"), MRL_ERR_UNSUPPORTED;
    // GM pools: free (TypeFlag 0) or bound (1); a bound pool needs a free one
    unsigned bound = 0;
    if (sc.mi.km == KM_EXCH && sc.mi.gm) {
        for (int t = 0; t < sc.P; ++t) {
            const double k = args->obj.type_flag[t];
            if (k != 0 && k != 1) return set_err("the adjoint covers GM pools of TypeFlag 0 and 1"), MRL_ERR_UNSUPPORTED;
            if (k == 1) bound |= 1u << t;
        }
        if (bound == (1u << sc.P) - 1) return set_err("the adjoint needs a free pool"), MRL_ERR_UNSUPPORTED;
    }
    if (mtc) bound = 1u << 1;
    if (bound && sc.TX > 1)
        return set_err("the adjoint with bound pools supports one Tx coil"), MRL_ERR_UNSUPPORTED;
    const int P = sc.P, S = sc.S, RX = sc.RX, A = sc.A, TX = sc.TX;
    p->TX = TX;
    p->P = P, p->S = S, p->RX = RX, p->A = A, p->V = sc.V;
    p->rf_ref = args->var.rf_ref ? *args->var.rf_ref : 0.0;
    // step records of the adjoint
    const long long N = ch.n_steps;
    p->N = N;
    const int RS = adjoint_record_f4(TX);
    std::vector<float4> rec((size_t)std::max<long long>(1, N) * RS);
    std::vector<int> step_uts((size_t)std::max<long long>(1, N), -1);
    for (size_t j = 0; j < ch.point_uts.size(); ++j)
        if (ch.point_dt[j] > 0) step_uts[ch.point_step[j]] = ch.point_uts[j];
    // change flags on the float values the kernel uses (see FrameMoments)
    float last_dt = -1.f, lgx = 0.f, lgy = 0.f, lgz = 0.f;
    for (long long q = 0; q < N; ++q) {
        const StepInfo &si = ch.steps[q];
        // an rf step: some Tx coil on; its frequency term sums the coils that are on
        bool rf = false;
        double wrf = 0;
        for (int c = 0; c < TX; ++c)
            if ((float)si.amp[c] != 0.f) {
                rf = true;
                wrf += 2 * kPiRef * si.freq[c];
            }
        int flags = rf ? kFlagRf : 0;
        const float fdt = (float)si.dt, fgx = (float)si.gx, fgy = (float)si.gy, fgz = (float)si.gz;
        if (fdt != last_dt) flags |= kFlagDt;
        if (fdt != last_dt || fgx != lgx || fgy != lgy || fgz != lgz) flags |= kFlagState;
        last_dt = fdt, lgx = fgx, lgy = fgy, lgz = fgz;
        float4 r1;
        r1.x = (float)(si.amp[0] * std::cos(si.phase[0]));
        r1.y = (float)(si.amp[0] * std::sin(si.phase[0]));
        r1.z = (float)wrf;
        std::memcpy(&r1.w, &flags, sizeof(int));
        const int ri = rf ? p->n_rf++ : -1;
        if (rf) {  // per coil: A, and the line entries it came from (-1: the coil is off)
            p->rf_uts.push_back(step_uts[q]);
            for (int c = 0; c < TX; ++c) {
                const bool on = (float)si.amp[c] != 0.f;
                p->rf_a.push_back(si.amp[c] * std::cos(si.phase[c]));
                p->rf_a.push_back(si.amp[c] * std::sin(si.phase[c]));
                p->rf_src.push_back(on ? si.amp_src[c] : -1);
                p->rf_src.push_back(on ? si.phase_src[c] : -1);
                p->rf_on.push_back(on ? 1 : 0);
            }
        }
        float4 r2 = make_float4(0.f, 0.f, 0.f, 0.f);
        std::memcpy(&r2.x, &si.adc, sizeof(int));
        std::memcpy(&r2.y, &ri, sizeof(int));
        rec[q * RS + 0] = make_float4((float)si.dt, (float)si.gz, (float)si.gy, (float)si.gx);
        rec[q * RS + 1] = r1;
        rec[q * RS + 2] = r2;
        for (int c = 1; c < TX; ++c)
            rec[q * RS + 2 + c] = make_float4((float)(si.amp[c] * std::cos(si.phase[c])),
                                              (float)(si.amp[c] * std::sin(si.phase[c])), 0.f, 0.f);
    }
    const int n = std::max(1, sc.n_act);
    const long long n_iso = (long long)sc.n_act * S;
    p->n_iso = n_iso;
    // stored checkpoints every ckpt_every steps; with M > 1 windows per
    // segment the adjoint rebuilds a segment's window checkpoints into d_ck2
    const int M = std::max(1, sc.ckpt_every / kAdjWin);
    const long long nck = (N + sc.ckpt_every - 1) / sc.ckpt_every;
    const double ck_bytes = (double)(nck + (M > 1 ? M : 0)) * 3 * P * std::max(1LL, n_iso) * sizeof(float);
    p->ck_every = sc.ckpt_every;
    p->ck_bytes = (long long)ck_bytes;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    if (ck_bytes > 0.85 * (double)free_b)
        return set_err("adjoint checkpoints need %.1f GiB, %.1f GiB free", ck_bytes / (1ull << 30),
                       (double)free_b / (1ull << 30)),
               MRL_ERR_NOMEM;
    const int nf = adjoint_fields(P);
    cudaError_t e = p->d_rec.ensure(rec.size());
    if (e == cudaSuccess) e = p->d_ck.ensure((size_t)std::max(1LL, nck * 3 * P * n_iso));
    if (e == cudaSuccess) e = p->d_ck2.ensure((size_t)std::max(1LL, (M > 1 ? M : 0) * 3 * P * n_iso));
    if (e == cudaSuccess) e = p->d_g.ensure((size_t)nf * std::max(1LL, n_iso));
    if (e == cudaSuccess) e = p->d_gs.ensure((size_t)P * RX * std::max(A, 1));
    if (e == cudaSuccess) e = p->d_rf.ensure((size_t)2 * TX * std::max(1, p->n_rf));
    if (e == cudaSuccess && mtc) {
        e = p->d_kgm.ensure((size_t)P * P * std::max(1, sc.n_act));
        if (e == cudaSuccess)
            e = launch_remap_k_mtc(P, sc.mi.km == KM_MT ? 2 : 3, sc.d_f.p + sc.o_k, p->d_kgm.p, sc.n_act, sc.st);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_rec.p, rec.data(), rec.size() * sizeof(float4), cudaMemcpyHostToDevice, sc.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sc.st);
    if (e != cudaSuccess) return sc.fail_cuda(e, "adjoint buffers");
    sc.ckpt = p->d_ck.p;
    AdjLaunch &L = p->L;
    L.n_act = sc.n_act;
    L.S = S;
    L.rx = RX;
    L.tx = TX;
    L.A = std::max(A, 1);
    L.exch_gm = (sc.mi.gm || mtc) ? 1 : 0;
    L.bound = bound;
    L.mtc = mtc ? 1 : 0;
    L.n_iso = n_iso;
    L.gyro = (float)args->obj.gyro;
    L.gxg = sc.d_f.p + sc.o_gx;
    L.gyg = sc.d_f.p + sc.o_gy;
    L.gzg = sc.d_f.p + sc.o_gz;
    L.db0 = sc.d_f.p + sc.o_db0;
    L.rho = sc.d_f.p + sc.o_rho;
    L.t1 = sc.d_f.p + sc.o_t1;
    L.t2 = sc.d_f.p + sc.o_t2;
    L.kch = mtc ? p->d_kgm.p : (sc.mi.nk > 0 ? sc.d_f.p + sc.o_k : nullptr);
    L.dwrnd = sc.d_f.p + sc.o_dwr;
    L.rxc = args->coil.rx_default == 0 ? sc.d_rx.p : nullptr;
    L.txc = sc.d_f2.p + sc.o_txc;
    for (int t = 0; t < kMaxPool; ++t)
        L.cs2pi[t] = (t < P && args->ctl.cs) ? (float)(2 * kPiRef * args->ctl.cs[t]) : 0.f;
    L.rec = p->d_rec.p;
    L.n_steps = N;
    L.ckpt = p->d_ck.p;
    L.seg = M;
    L.ck2 = M > 1 ? p->d_ck2.p : nullptr;
    L.gsig = p->d_gs.p;
    L.giso = p->d_g.p;
    L.grf = p->d_rf.p;
    (void)n;
    *out = p.release();
    return MRL_OK;
}

int mrl_adjoint_plan_forward(mrl_adjoint_plan *p, void *stream) {
    if (!p) return MRL_ERR_ARG;
    int rc = mrl_plan_execute(p->fwd, stream);
    p->forward_done = rc == MRL_OK;
    return rc;
}

int mrl_adjoint_plan_download(mrl_adjoint_plan *p, mrl_scan_args *args) {
    if (!p || !args) return MRL_ERR_ARG;
    return mrl_plan_download(p->fwd, args);
}

int mrl_adjoint_plan_backward(mrl_adjoint_plan *p, const double *grad_sx, const double *grad_sy, void *stream) {
    using namespace mrl;
    g_err.clear();
    if (!p) return set_err("NULL plan"), MRL_ERR_ARG;
    if (!p->forward_done) return set_err("mrl_adjoint_plan_backward needs a forward pass first"), MRL_ERR_ARG;
    Scanner &sc = p->fwd->sc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the signal is the receive sum rotated by exp(-i rfRef): dL/dS before
    // the rotation = exp(+i rfRef) dL/dS after it
    const double cr = std::cos(p->rf_ref), sr = std::sin(p->rf_ref);
    // [P][Rx][A] (the signal's layout) -> [A][P][Rx] (one sample's values together)
    std::vector<float2> gs((size_t)p->P * p->RX * std::max(p->A, 1), make_float2(0.f, 0.f));
    for (int t = 0; t < p->P; ++t)
        for (int c = 0; c < p->RX; ++c)
            for (int a = 0; a < p->A; ++a) {
                const size_t i = ((size_t)t * p->RX + c) * p->A + a;
                const double gx = grad_sx ? grad_sx[i] : 0.0, gy = grad_sy ? grad_sy[i] : 0.0;
                gs[((size_t)a * p->P + t) * p->RX + c] =
                    make_float2((float)(gx * cr - gy * sr), (float)(gx * sr + gy * cr));
            }
    cudaError_t e = cudaMemcpyAsync(p->d_gs.p, gs.data(), gs.size() * sizeof(float2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->d_rf.p, 0, p->d_rf.n * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->d_g.p, 0, p->d_g.n * sizeof(float), st);
    if (e == cudaSuccess && p->n_iso > 0 && p->N > 0) e = launch_adjoint(p->P, p->L, st);
    if (e != cudaSuccess) return sc.fail_cuda(e, "adjoint launch");
    p->backward_done = true;
    return MRL_OK;
}

int mrl_adjoint_plan_gradients(mrl_adjoint_plan *p, mrl_adjoint_args *adj) {
    using namespace mrl;
    g_err.clear();
    if (!p || !adj) return set_err("NULL argument"), MRL_ERR_ARG;
    if (!p->backward_done) return set_err("mrl_adjoint_plan_gradients needs a backward pass first"), MRL_ERR_ARG;
    Scanner &sc = p->fwd->sc;
    const mrl_scan_args *args = &p->fwd->args;
    const int P = p->P, S = p->S;
    const long long V = p->V, n_iso = p->n_iso;
    const int n_rf = p->n_rf;
    cudaError_t e = cudaDeviceSynchronize();
    std::vector<float> g(p->d_g.n);
    std::vector<double> grf(p->d_rf.n);
    if (e == cudaSuccess) e = cudaMemcpy(g.data(), p->d_g.p, g.size() * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(grf.data(), p->d_rf.p, grf.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return sc.fail_cuda(e, "adjoint download");
    adj->n_rf_steps = n_rf;
    // per voxel: sums over the voxel's spins; per isochromat: the initial state
    auto field = [&](int f, int s2, int j) { return g[(size_t)f * n_iso + (size_t)s2 * sc.n_act + j]; };
    const int F_T1 = 0, F_T2 = P, F_RHO = 2 * P, F_DB0 = 3 * P, F_K = 3 * P + 1, F_M0 = 3 * P + 1 + P * P;
    for (float *o : {adj->g_t1, adj->g_t2, adj->g_rho})
        if (o) std::fill(o, o + (size_t)P * V, 0.f);
    if (adj->g_db0) std::fill(adj->g_db0, adj->g_db0 + V, 0.f);
    if (adj->g_k && sc.mi.nk > 0) std::fill(adj->g_k, adj->g_k + (size_t)args->obj.k_channels * V, 0.f);
    for (float *o : {adj->g_mx0, adj->g_my0, adj->g_mz0})
        if (o) std::fill(o, o + (size_t)P * S * V, 0.f);
    for (int j = 0; j < sc.n_act; ++j) {
        const long long v = sc.act[j];
        for (int s2 = 0; s2 < S; ++s2) {
            for (int t = 0; t < P; ++t) {
                if (adj->g_t1) adj->g_t1[t * V + v] += field(F_T1 + t, s2, j);
                if (adj->g_t2) adj->g_t2[t * V + v] += field(F_T2 + t, s2, j);
                if (adj->g_rho) adj->g_rho[t * V + v] += field(F_RHO + t, s2, j);
                const long long i = ((long long)t * S + s2) * V + v;
                if (adj->g_mx0) adj->g_mx0[i] = field(F_M0 + t, s2, j);
                if (adj->g_my0) adj->g_my0[i] = field(F_M0 + P + t, s2, j);
                if (adj->g_mz0) adj->g_mz0[i] = field(F_M0 + 2 * P + t, s2, j);
            }
            if (adj->g_db0) adj->g_db0[v] += field(F_DB0, s2, j);
            if (adj->g_k && sc.mi.nk > 0) {
                if (sc.mi.km == KM_MT) {  // K12 = rate 0 -> 1 (GM channel 1*P+0), K21 = rate 1 -> 0 (0*P+1)
                    adj->g_k[1 * V + v] += field(F_K + 1 * P + 0, s2, j);
                    adj->g_k[2 * V + v] += field(F_K + 0 * P + 1, s2, j);
                } else if (sc.mi.km == KM_CEST) {  // channel c <-> rate a -> b, GM channel b*P+a
                    for (int c = 0; c < 2 * (P - 1); ++c) {
                        int ra, rb;
                        if (c == 0) ra = 0, rb = 1;
                        else if (c == P - 1) ra = 1, rb = 0;
                        else if (c < P - 1) ra = 0, rb = c + 1;
                        else ra = c - P + 2, rb = 0;
                        adj->g_k[(long long)c * V + v] += field(F_K + rb * P + ra, s2, j);
                    }
                } else {
                    for (int k = 0; k < P * P; ++k) adj->g_k[k * V + v] += field(F_K + k, s2, j);
                }
            }
        }
    }
    // a coil that is off at an rf step is not part of its field: no gradient
    const int TX = p->TX;
    for (int i = 0; i < n_rf * TX; ++i)
        if (!p->rf_on[i]) grf[2 * i] = grf[2 * i + 1] = 0.0;
    if (n_rf <= adj->rf_capacity) {
        if (adj->g_rf) std::copy(grf.begin(), grf.begin() + 2 * (size_t)n_rf * TX, adj->g_rf);
        if (adj->rf_step_uts) std::copy(p->rf_uts.begin(), p->rf_uts.end(), adj->rf_step_uts);
        if (adj->rf_a) std::copy(p->rf_a.begin(), p->rf_a.end(), adj->rf_a);
    }
    // onto the waveform lines: A = a e^{i phi} with a = rfAmpLine[ja] (a
    // negative a is the same A as |a| at phi + pi), phi = rfPhaseLine[jp];
    // each coil's entries are its own (rfCoilLine)
    const int n_line = args->seq.n_rf;
    if (adj->g_rf_amp_line) std::fill(adj->g_rf_amp_line, adj->g_rf_amp_line + n_line, 0.0);
    if (adj->g_rf_phase_line) std::fill(adj->g_rf_phase_line, adj->g_rf_phase_line + n_line, 0.0);
    for (int i = 0; i < n_rf * TX; ++i) {
        const double gx = grf[2 * i], gy = grf[2 * i + 1], ax = p->rf_a[2 * i], ay = p->rf_a[2 * i + 1];
        const int ja = p->rf_src[2 * i], jp = p->rf_src[2 * i + 1];
        if (adj->g_rf_amp_line && ja >= 0 && ja < n_line) {
            const double a = args->seq.rf_amp[ja];
            if (a != 0) adj->g_rf_amp_line[ja] += (gx * ax + gy * ay) / a;
        }
        if (adj->g_rf_phase_line && jp >= 0 && jp < n_line) adj->g_rf_phase_line[jp] += gy * ax - gx * ay;
    }
    return sc.check_device_status();
}

int mrl_adjoint_plan_work(const mrl_adjoint_plan *p, long long out[6]) {
    if (!p || !out) return MRL_ERR_ARG;
    for (int i = 0; i < 5; ++i) out[i] = p->fwd->work[i];
    out[5] = p->n_rf;
    return MRL_OK;
}

int mrl_adjoint_plan_checkpoints(const mrl_adjoint_plan *p, long long out[3]) {
    if (!p || !out) return MRL_ERR_ARG;
    out[0] = p->ck_every;
    out[1] = mrl::kAdjWin;
    out[2] = p->ck_bytes;
    return MRL_OK;
}

void mrl_adjoint_plan_destroy(mrl_adjoint_plan *p) { delete p; }

int mrl_adjoint(mrl_scan_args *args, mrl_adjoint_args *adj) {
    using namespace mrl;
    if (!args || !adj) return g_err.clear(), set_err("NULL argument"), MRL_ERR_ARG;
    const auto t_start = std::chrono::steady_clock::now();
    for (double &x : g_timing) x = 0;
    mrl_adjoint_plan *p = nullptr;
    int rc = mrl_adjoint_plan_create(args, &p);
    if (rc) return rc;
    std::unique_ptr<mrl_adjoint_plan> keep(p);
    cudaStream_t st = p->fwd->sc.st;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    rc = mrl_adjoint_plan_forward(p, st);
    if (!rc) cudaEventRecord(ev0, st);
    if (!rc) rc = mrl_adjoint_plan_backward(p, adj->grad_sx, adj->grad_sy, st);
    if (!rc) cudaEventRecord(ev1, st);
    float ms = 0.f;
    if (!rc && cudaEventSynchronize(ev1) == cudaSuccess) cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (!rc) rc = mrl_adjoint_plan_gradients(p, adj);
    g_timing[1] = ms;  // the adjoint kernel (after the forward scan that writes the checkpoints)
    g_timing[5] = (double)p->fwd->work[4] + 1;
    g_timing[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    return rc;
}

int mrl_scan_noalloc(mrl_scan_args *args, float *d_steps, size_t step_bytes, void *stream) {
    using namespace mrl;
    g_err.clear();
    for (double &x : g_timing) x = 0;
    const auto t_start = std::chrono::steady_clock::now();
    if (!args || !d_steps) {
        set_err("NULL argument");
        return MRL_ERR_ARG;
    }
    // the kernel stages step records with bulk copies, which need a 16-byte
    // aligned global source
    if ((reinterpret_cast<uintptr_t>(d_steps) & 15) != 0) {
        set_err("d_steps must be 16-byte aligned");
        return MRL_ERR_ARG;
    }
    Scanner sc;  // validation only: nothing of it is allocated
    sc.args = args;
    int rc = sc.validate();
    if (rc) return rc;
    if (!sc.fast || sc.exact) {
        set_err("mrl_scan_noalloc runs the MRL_NUMERICS_ACCURATE integrator only");
        return MRL_ERR_UNSUPPORTED;
    }
    if (sc.hist_on) {
        set_err("mrl_scan_noalloc does not record RunMode 1 history");
        return MRL_ERR_UNSUPPORTED;
    }
    if (sc.TX != 1) {
        set_err("mrl_scan_noalloc supports one Tx coil");
        return MRL_ERR_UNSUPPORTED;
    }
    if (sc.V * sc.tpv > (long long)INT32_MAX) {
        set_err("spin matrix too large");
        return MRL_ERR_UNSUPPORTED;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSetDevice(args->ctl.gpu_index);
    if (e != cudaSuccess) {
        set_err("cudaSetDevice(%d): %s", args->ctl.gpu_index, cudaGetErrorString(e));
        return MRL_ERR_NO_DEVICE;
    }
    unsigned char *scratch = nullptr;
    if ((e = noalloc_scratch(args->ctl.gpu_index, &scratch)) != cudaSuccess)
        return sc.fail_cuda(e, "cudaGetSymbolAddress(scratch)");
    int *d_status = reinterpret_cast<int *>(scratch);
    // decode the whole sequence on the host
    DecodeState ds;
    load_state(ds, args->var, sc.TX);
    DecodeChunk ch;
    decode_until_ext(ds, args->seq, sc.TX, args->obj.gyro, args->sig, ch);
    if (ch.stopped_at_ext) {
        set_err("the sequence has Ext events: use mrl_scan with a callback");
        return MRL_ERR_UNSUPPORTED;
    }
    store_state(ds, args->var, sc.TX);
    FrameMoments fm;
    std::vector<float> rec;
    pack_fast_records(ch, sc.TX, fm, rec);
    if (rec.size() * sizeof(float) > step_bytes) {
        set_err("step buffer holds %zu bytes, %zu needed", step_bytes, rec.size() * sizeof(float));
        return MRL_ERR_ARG;
    }
    // launches sized so that one launch's ADC map and partials fit the scratch
    const int n = (int)sc.V;
    const long long nblk = std::max(1LL, ((long long)n * sc.tpv + kBlock - 1) / kBlock);
    const int npairs = sc.mi.nsamp * sc.RX;
    const long long nslices = nblk * partial_slices(true);
    // layout: [status 256 B][descriptor][ADC map, rounded up to 256 B][partials];
    // the ADC map's rounding adds at most 252 B, reserved up front
    const unsigned long long per_sample = sizeof(int) + (unsigned long long)nslices * npairs * sizeof(float2);
    const unsigned long long room = kNoAllocScratchBytes - 2 * 256 - kNoAllocDescBytes;
    const long long a_cap = (long long)std::min<unsigned long long>(room / per_sample, (unsigned long long)INT32_MAX);
    if (a_cap < 1) {
        set_err("object too large for the %zu-byte scratch: one ADC sample needs %llu bytes", kNoAllocScratchBytes,
                per_sample);
        return MRL_ERR_UNSUPPORTED;
    }
    const size_t amap_bytes = ((size_t)a_cap * sizeof(int) + 255) / 256 * 256;
    const size_t part_off = 256 + kNoAllocDescBytes + amap_bytes;
    if (part_off + (size_t)a_cap * nslices * npairs * sizeof(float2) > kNoAllocScratchBytes) {
        set_err("internal: scratch layout exceeds %zu bytes", kNoAllocScratchBytes);
        return MRL_ERR_UNSUPPORTED;
    }
    FastLaunch *d_desc = reinterpret_cast<FastLaunch *>(scratch + 256);
    int *d_amap = reinterpret_cast<int *>(scratch + 256 + kNoAllocDescBytes);
    float2 *d_part = reinterpret_cast<float2 *>(scratch + part_off);
    if ((e = cudaMemsetAsync(d_status, 0, sizeof(int), st)) != cudaSuccess) return sc.fail_cuda(e, "status reset");
    if ((e = cudaMemcpyAsync(d_steps, rec.data(), rec.size() * sizeof(float), cudaMemcpyHostToDevice, st)) !=
        cudaSuccess)
        return sc.fail_cuda(e, "upload steps");
    ScanLaunch L{};
    L.n_act = n;
    L.S = sc.S;
    L.tx = sc.TX;
    L.rx = sc.RX;
    L.nsamp = sc.mi.nsamp;
    L.npairs = npairs;
    L.tpv = sc.tpv;
    L.gyro = (float)args->obj.gyro;
    L.rx_default = args->coil.rx_default != 0;
    L.exch_gm = sc.mi.gm ? 1 : 0;
    L.gxg = args->mag.gxgrid;
    L.gyg = args->mag.gygrid;
    L.gzg = args->mag.gzgrid;
    L.db0 = args->mag.db0;
    L.txmg = args->coil.tx_mg;
    L.txpe = args->coil.tx_pe;
    L.rho = args->obj.rho;
    L.t1 = args->obj.t1;
    L.t2 = args->obj.t2;
    L.kch = args->obj.k;
    L.dwrnd = args->mag.dwrnd;
    L.mx = args->obj.mx;
    L.my = args->obj.my;
    L.mz = args->obj.mz;
    L.rec = reinterpret_cast<const float4 *>(d_steps);
    L.stride4 = sc.stride4;
    L.err = d_status;
    L.partial = d_part;
    for (int t = 0; t < kMaxPool; ++t) {
        L.cs2pi[t] = t < sc.P && args->ctl.cs ? (float)(2 * kPiRef * (double)(float)args->ctl.cs[t]) : 0.f;
        L.kind[t] = (sc.mi.gm && t < sc.P) ? (int)args->obj.type_flag[t] : 0;
    }
    FastLaunch F{};
    F.b = L;
    F.direct = 1;
    F.all_free = sc.all_free();
    set_sampling(F, L, sc.P);
    F.rx_x = args->coil.rx_x;
    F.rx_y = args->coil.rx_y;
    F.gam_hi = (float)args->obj.gyro;
    F.gam_lo = (float)(args->obj.gyro - (double)F.gam_hi);
    for (int t = 0; t < kMaxPool; ++t) {
        const double w = (t < sc.P && args->ctl.cs) ? 2 * kPiRef * args->ctl.cs[t] : 0.0;
        F.cs_hi[t] = (float)w;
        F.cs_lo[t] = (float)(w - (double)F.cs_hi[t]);
    }
    const size_t smem = scan_fast_smem_bytes(sc.stride4, sc.RX, sc.P, sc.NS);
    const double rf_ref = args->var.rf_ref ? *args->var.rf_ref : 0.0;
    const double cr = std::cos(-rf_ref), sr = std::sin(-rf_ref);
    // walk the steps, one launch per a_cap samples
    long long s0 = 0;
    std::vector<int> amap;
    int n_launch = 0;
    auto launch = [&](long long s1) -> int {
        ++n_launch;
        F.b.s0 = s0;
        F.b.s1 = s1;
        F.b.a_launch = (int)amap.size();
        cudaError_t le;
        if (!amap.empty() &&
            (le = cudaMemcpyAsync(d_amap, amap.data(), amap.size() * sizeof(int), cudaMemcpyHostToDevice, st)) !=
                cudaSuccess)
            return sc.fail_cuda(le, "upload ADC map");
        if ((le = cudaMemcpyAsync(d_desc, &F, sizeof(F), cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return sc.fail_cuda(le, "upload launch descriptor");
        const FastGrid g{d_desc, nullptr, (int)nblk, nullptr};
        le = launch_fast(sc.mi.km, sc.P, sc.NS, F.all_free != 0, dim3((unsigned)nblk), smem, st, g);
        if (le != cudaSuccess) return sc.fail_cuda(le, "scan kernel launch");
        if (!amap.empty()) {
            const int tot = (int)amap.size() * npairs;
            reduce_partials<<<(tot + 31) / 32, 32 * kRedWarps, 0, st>>>(d_part, (int)nslices, (int)amap.size(), npairs,
                                                                        sc.RX,
                                                               d_amap, sc.A, args->sig.sx, args->sig.sy, cr, sr);
            if ((le = cudaGetLastError()) != cudaSuccess) return sc.fail_cuda(le, "reduce launch");
        }
        return MRL_OK;
    };
    for (long long q = 0; q < ch.n_steps; ++q) {
        if (ch.step_adc[q] < 0) continue;
        if ((long long)amap.size() == a_cap) {
            if ((rc = launch(q))) return rc;
            s0 = q;
            amap.clear();
        }
        amap.push_back(ch.step_adc[q]);
    }
    if (ch.n_steps > 0 && (rc = launch(ch.n_steps))) return rc;
    int status = 0;
    if ((e = cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return sc.fail_cuda(e, "scan");
    if (status) {
        set_err("a device wait timed out (status bits %d)", status);
        return MRL_ERR_TIMEOUT;
    }
    g_timing[5] = n_launch;
    g_timing[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    return MRL_OK;
}

int mrl_decode(const mrl_scan_args *args, double *steps, long long cap, long long *n_steps) {
    using namespace mrl;
    g_err.clear();
    if (!args || !n_steps || (cap > 0 && !steps)) return set_err("NULL argument"), MRL_ERR_ARG;
    *n_steps = 0;
    if (args->abi_version != MRL_ABI_VERSION)
        return set_err("abi_version %d, expected %d", args->abi_version, MRL_ABI_VERSION), MRL_ERR_ARG;
    const int TX = args->coil.tx_num;
    if (TX < 1 || TX > kMaxTx) return set_err("TxCoilNum %d outside 1..%d", TX, kMaxTx), MRL_ERR_UNSUPPORTED;
    const mrl_sequence &q = args->seq;
    if (!q.uts || !q.ts || !q.flags || q.n_uts < 1 || q.n_ts < 1) return set_err("VSeq lines missing"), MRL_ERR_ARG;
    // k-space goes to scratch: the caller's arrays are not touched
    const size_t A = (size_t)std::max(1, args->sig.signal_num);
    std::vector<double> kx(A, 0.0), ky(A, 0.0), kz(A, 0.0);
    mrl_signal sig = args->sig;
    sig.kx = kx.data(), sig.ky = ky.data(), sig.kz = kz.data();
    DecodeState ds;
    load_state(ds, args->var, TX);
    ds.i = 0;
    ds.signali = 0;
    const int stride = 5 + 3 * TX;
    long long n = 0;
    // Ext stops: decoding resumes where it stopped (no plugin runs); each
    // stop consumes at least one tsLine entry
    for (long long guard = 0; guard <= (long long)q.n_ts + 1; ++guard) {
        DecodeChunk ch;
        decode_until_ext(ds, q, TX, args->obj.gyro, sig, ch);
        for (const StepInfo &si : ch.steps) {
            if (n < cap) {
                double *r = steps + n * stride;
                r[0] = si.dt, r[1] = si.gz, r[2] = si.gy, r[3] = si.gx, r[4] = si.adc;
                for (int c = 0; c < TX; ++c)
                    r[5 + 3 * c] = si.amp[c], r[6 + 3 * c] = si.phase[c], r[7 + 3 * c] = si.freq[c];
            }
            ++n;
        }
        if (!ch.stopped_at_ext) break;
    }
    *n_steps = n;
    if (n > cap) return set_err("%lld steps, room for %lld", n, cap), MRL_ERR_ARG;
    return MRL_OK;
}

// Test hook (not declared in mrl_scan.h): the accurate integrator's step
// records of args' sequence (one Tx coil, no Ext events), host only: 16
// floats per step as pack_fast_records writes them.
int mrl_selftest_pack(const mrl_scan_args *args, int ckpt_every, float *out, long long cap, long long *n_steps) {
    using namespace mrl;
    if (!args || !n_steps || (cap > 0 && !out) || args->coil.tx_num != 1) return MRL_ERR_ARG;
    const size_t A = (size_t)std::max(1, args->sig.signal_num);
    std::vector<double> kx(A, 0.0), ky(A, 0.0), kz(A, 0.0);
    mrl_signal sig = args->sig;
    sig.kx = kx.data(), sig.ky = ky.data(), sig.kz = kz.data();
    DecodeState ds;
    load_state(ds, args->var, 1);
    ds.i = 0;
    ds.signali = 0;
    DecodeChunk ch;
    decode_until_ext(ds, args->seq, 1, args->obj.gyro, sig, ch);
    if (ch.stopped_at_ext) return MRL_ERR_UNSUPPORTED;
    FrameMoments fm;
    std::vector<float> rec;
    pack_fast_records(ch, 1, fm, rec, ckpt_every);
    *n_steps = ch.n_steps;
    if (ch.n_steps > cap) return MRL_ERR_ARG;
    std::copy(rec.begin(), rec.end(), out);
    return MRL_OK;
}

const char *mrl_status_string(int status) {
    switch (status) {
    case MRL_OK: return "ok";
    case MRL_ERR_ARG: return "invalid argument";
    case MRL_ERR_CUDA: return "CUDA error";
    case MRL_ERR_NOMEM: return "out of memory";
    case MRL_ERR_EXT: return "Ext plugin error";
    case MRL_ERR_TIMEOUT: return "device wait timed out";
    case MRL_ERR_UNSUPPORTED: return "unsupported configuration";
    case MRL_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

const char *mrl_last_error(void) { return mrl::g_err.c_str(); }

// Test hook (not declared in mrl_scan.h): sin and cos of n host floats as
// the accurate kernel computes them, on the current device.
int mrl_selftest_sincos(const float *x, float *sn, float *cs, int n) {
    using namespace mrl;
    if (!x || !sn || !cs || n < 0) return MRL_ERR_ARG;
    if (n == 0) return MRL_OK;
    DevBuf<float> d;
    cudaError_t e = d.ensure((size_t)3 * n);
    if (e == cudaSuccess) e = cudaMemcpy(d.p, x, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        sincos_probe<<<(n + 255) / 256, 256>>>(d.p, d.p + n, d.p + 2 * n, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(sn, d.p + n, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(cs, d.p + 2 * n, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_err("selftest sincos: %s", cudaGetErrorString(e));
        return MRL_ERR_CUDA;
    }
    return MRL_OK;
}

// Test hook (not declared in mrl_scan.h): 1 - exp(-x) of n host floats as
// the accurate kernel computes it, and as CUDA's expm1f does.
int mrl_selftest_one_minus_exp(const float *x, float *ours, float *lib, int n) {
    using namespace mrl;
    if (!x || !ours || !lib || n < 0) return MRL_ERR_ARG;
    if (n == 0) return MRL_OK;
    DevBuf<float> d;
    cudaError_t e = d.ensure((size_t)3 * n);
    if (e == cudaSuccess) e = cudaMemcpy(d.p, x, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        one_minus_exp_probe<<<(n + 255) / 256, 256>>>(d.p, d.p + n, d.p + 2 * n, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(ours, d.p + n, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(lib, d.p + 2 * n, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_err("selftest one_minus_exp: %s", cudaGetErrorString(e));
        return MRL_ERR_CUDA;
    }
    return MRL_OK;
}

// Test hook (not declared in mrl_scan.h): the accurate kernel's TF32
// rounding and the hardware conversion of n host floats.
int mrl_selftest_tf32(const float *x, uint32_t *rn, uint32_t *cvt, int n) {
    using namespace mrl;
    if (!x || !rn || !cvt || n < 0) return MRL_ERR_ARG;
    if (n == 0) return MRL_OK;
    DevBuf<uint32_t> d;
    cudaError_t e = d.ensure((size_t)3 * n);
    if (e == cudaSuccess) e = cudaMemcpy(d.p, x, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        tf32_probe<<<(n + 255) / 256, 256>>>(reinterpret_cast<const float *>(d.p), d.p + n, d.p + 2 * n, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(rn, d.p + n, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(cvt, d.p + 2 * n, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_err("selftest tf32: %s", cudaGetErrorString(e));
        return MRL_ERR_CUDA;
    }
    return MRL_OK;
}

int mrl_last_timing(double out[8]) {
    if (!out) return MRL_ERR_ARG;
    for (int i = 0; i < 8; ++i) out[i] = mrl::g_timing[i];
    return MRL_OK;
}

}  // extern "C"
