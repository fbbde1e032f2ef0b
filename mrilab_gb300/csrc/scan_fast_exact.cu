// Tabulated coefficients for free pools exchanging: the accurate scan
// kernel's instantiations that read their relaxation / exchange step from a
// table per (distinct dt, voxel) -- the reference's split exchange
// (MRL_NUMERICS_ACCURATE, coefficient source 1) and the exact propagator
// (MRL_NUMERICS_EXACT, source 2) -- and the FP64 kernels that fill the tables.
//
// Per step every pool is rotated exactly (rf or free precession, as in the
// accurate mode), then the Bloch-McConnell equations without the rotation
// are solved exactly over dt: x' = E_T x, y' = E_T y, z' = E_L z + c with
// E = exp(A dt), A_T = -diag(1/T2) + K, A_L = -diag(1/T1) + K (K the
// exchange generator: -sum of the outgoing rates on the diagonal, the
// incoming rate p -> t at (t, p)), c = dt phi1(A_L dt) b, b = rho / (S T1).
// The reference splits the exchange to first order instead
// (BlochKernelME.cuh:320-343), which departs from the equations when k dt
// is not small.
#include "scan_launch.h"

namespace mrl {

namespace {
using Kernel = FastKernel;

template <int P, int NS>
Kernel pick(int co) {
    return co == 2 ? scan_fast_kernel<KM_EXCH, P, NS, true, 2> : scan_fast_kernel<KM_EXCH, P, NS, true, 1>;
}

Kernel select(int co, int P, int NS, bool all_free) {
    if (co != 1 && co != 2) return nullptr;
    if (!all_free) return co == 2 ? select_exact_bound(P, NS) : nullptr;
    if (P == 1 && NS == 1) return pick<1, 1>(co);
    if (P == 1 && NS == 2) return pick<1, 2>(co);
    if (P == 1 && NS == 4) return pick<1, 4>(co);
    if (P == 2 && NS == 1) return pick<2, 1>(co);
    if (P == 2 && NS == 2) return pick<2, 2>(co);
    if (P == 2 && NS == 4) return pick<2, 4>(co);
    if (P == 3 && NS == 1) return pick<3, 1>(co);
    if (P == 3 && NS == 2) return pick<3, 2>(co);
    return nullptr;
}

// exp(A) - I and phi1(A) = sum_k A^k / (k+1)! (row-major P x P): Taylor
// series of A scaled by 2^-s to norm <= 1/4 (24 terms, far below FP64
// rounding), then s squarings: e^{2B} - I = F^2 + 2F, phi1(2B) = phi1(B)(F + 2I)/2
template <int P>
__device__ void expm1_phi1(const double (&A)[P][P], double (&F)[P][P], double (&X)[P][P]) {
    double norm = 0.0;
#pragma unroll
    for (int i = 0; i < P; ++i) {
        double r = 0.0;
#pragma unroll
        for (int j = 0; j < P; ++j) r += fabs(A[i][j]);
        norm = fmax(norm, r);
    }
    int s = 0;
    while (norm > 0.25 && s < 60) {
        norm *= 0.5;
        ++s;
    }
    const double scale = ldexp(1.0, -s);
    double B[P][P], T[P][P], U[P][P];
#pragma unroll
    for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j < P; ++j) {
            B[i][j] = A[i][j] * scale;
            T[i][j] = i == j ? 1.0 : 0.0;
            F[i][j] = 0.0;
            X[i][j] = T[i][j];
        }
    for (int k = 1; k <= 24; ++k) {
        const double ik = 1.0 / k, ik1 = 1.0 / (k + 1);
#pragma unroll
        for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P; ++j) {
                double acc = 0.0;
#pragma unroll
                for (int m = 0; m < P; ++m) acc = fma(T[i][m], B[m][j], acc);
                U[i][j] = acc * ik;
            }
#pragma unroll
        for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P; ++j) {
                T[i][j] = U[i][j];
                F[i][j] += T[i][j];
                X[i][j] = fma(T[i][j], ik1, X[i][j]);
            }
    }
    for (int q = 0; q < s; ++q) {
#pragma unroll
        for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P; ++j) {
                double a = 0.0, b = 0.0;
#pragma unroll
                for (int m = 0; m < P; ++m) {
                    a = fma(X[i][m], F[m][j] + (m == j ? 2.0 : 0.0), a);
                    b = fma(F[i][m], F[m][j], b);
                }
                U[i][j] = 0.5 * a;
                T[i][j] = b + 2.0 * F[i][j];
            }
#pragma unroll
        for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P; ++j) {
                X[i][j] = U[i][j];
                F[i][j] = T[i][j];
            }
    }
}

// Exchange rate from pool t to pool p of voxel v in each model's K layout
// (layout 0 ME: channel t*P+p; 1 GM: p*P+t; 2 MT: channel 1 = K12 (0 -> 1),
// 2 = K21 (1 -> 0); 3 CEST: 0 = 0 -> MT, P-1 = MT -> 0, t-1 = 0 -> t,
// t+P-2 = t -> 0), 0 where the model has no such rate.
template <int P>
__device__ __forceinline__ double exch_rate(const float *kch, int n_act, int v, int layout, int t, int p) {
    int ch = -1;
    if (layout == 0) ch = t * P + p;
    else if (layout == 1) ch = p * P + t;
    else if (layout == 2) ch = (t == 0 && p == 1) ? 1 : ((t == 1 && p == 0) ? 2 : -1);
    else if (t == 0) ch = p == 1 ? 0 : p - 1;
    else if (p == 0) ch = t == 1 ? P - 1 : t + P - 2;
    return ch < 0 ? 0.0 : (double)kch[(long long)ch * n_act + v];
}

// layout as exch_rate.  MT and CEST (layout 2, 3) keep their models'
// transverse map: a free pool's transverse magnetisation does not flow out
// to the bound pool (BlochKernelMT.cuh:324-333, BlochKernelCEST.cuh:364-395).
template <int P>
__global__ void exact_table_kernel(const float *__restrict__ dts, int n_dt, int n_act, int S, int layout,
                                   unsigned bound, const float *__restrict__ rho, const float *__restrict__ t1,
                                   const float *__restrict__ t2, const float *__restrict__ kch, float *tab) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n_dt * n_act) return;
    const int d = (int)(i / n_act), v = (int)(i % n_act);
    const double dt = dts[d];
    double At[P][P], Al[P][P], b[P];
#pragma unroll
    for (int t = 0; t < P; ++t) {
        b[t] = 0.0;
#pragma unroll
        for (int p = 0; p < P; ++p) At[t][p] = Al[t][p] = 0.0;
    }
#pragma unroll
    for (int t = 0; t < P; ++t) {
        const double T1 = t1[(long long)t * n_act + v], T2 = t2[(long long)t * n_act + v],
                     r = rho[(long long)t * n_act + v];
        const bool mtc = layout >= 2;
        if (T1 == 0.0 || T2 == 0.0 || r == 0.0) continue;  // a pool left alone: identity row
        // a bound pool: no transverse generator (identity row), and no free
        // pool takes transverse inflow from it
        const bool bt = bound >> t & 1u;
        if (!bt) At[t][t] = -1.0 / T2;
        Al[t][t] = -1.0 / T1;
        b[t] = r / (S * T1);
#pragma unroll
        for (int p = 0; p < P; ++p) {
            if (p == t || !kch) continue;  // a self rate moves nothing
            const double kgo = exch_rate<P>(kch, n_act, v, layout, t, p);
            const double kin = exch_rate<P>(kch, n_act, v, layout, p, t);
            if (!bt && !(mtc && (bound >> p & 1u))) At[t][t] -= kgo;
            Al[t][t] -= kgo;
            if (!bt && !(bound >> p & 1u)) At[t][p] += kin;
            Al[t][p] += kin;
        }
    }
#pragma unroll
    for (int t = 0; t < P; ++t)
#pragma unroll
        for (int p = 0; p < P; ++p) {
            At[t][p] *= dt;
            Al[t][p] *= dt;
        }
    double Ft[P][P], Xt[P][P], Fl[P][P], Xl[P][P];
    expm1_phi1<P>(At, Ft, Xt);
    expm1_phi1<P>(Al, Fl, Xl);
    float *o = tab + (long long)d * exact_fields(P) * n_act + v;
    int f = 0;
#pragma unroll
    for (int t = 0; t < P; ++t) o[(long long)(f++) * n_act] = (float)Ft[t][t];
#pragma unroll
    for (int t = 0; t < P; ++t)
#pragma unroll
        for (int p = 0; p < P; ++p)
            if (p != t) o[(long long)(f++) * n_act] = (float)Ft[t][p];
#pragma unroll
    for (int t = 0; t < P; ++t) o[(long long)(f++) * n_act] = (float)Fl[t][t];
#pragma unroll
    for (int t = 0; t < P; ++t)
#pragma unroll
        for (int p = 0; p < P; ++p)
            if (p != t) o[(long long)(f++) * n_act] = (float)Fl[t][p];
#pragma unroll
    for (int t = 0; t < P; ++t) {
        double c = 0.0;
#pragma unroll
        for (int p = 0; p < P; ++p) c = fma(Xl[t][p], b[p], c);
        o[(long long)(f++) * n_act] = (float)(dt * c);
    }
}
// The split scheme's coefficients (BlochKernelME.cuh:320-343, as the
// accurate kernel computes them at a dt change) in FP64 per (dt, voxel):
// y1 = 1 - e^{-dt/T1}, y2 = 1 - e^{-dt/T2}, yo = 1 - e^{-dt sum of the
// outgoing rates}, fin[t][p] = 1 - e^{-dt k(p -> t)}; zero for a pool left
// alone (T1, T2 or Rho zero).
template <int P>
__global__ void split_table_kernel(const float *__restrict__ dts, int n_dt, int n_act, int gm,
                                   const float *__restrict__ rho, const float *__restrict__ t1,
                                   const float *__restrict__ t2, const float *__restrict__ kch, float *tab) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n_dt * n_act) return;
    const int d = (int)(i / n_act), v = (int)(i % n_act);
    const double dt = dts[d];
    double y1[P], y2[P], yo[P], fin[P][P];
#pragma unroll
    for (int t = 0; t < P; ++t) {
        y1[t] = y2[t] = yo[t] = 0.0;
#pragma unroll
        for (int p = 0; p < P; ++p) fin[t][p] = 0.0;
        const double T1 = t1[(long long)t * n_act + v], T2 = t2[(long long)t * n_act + v],
                     r = rho[(long long)t * n_act + v];
        if (T1 == 0.0 || T2 == 0.0 || r == 0.0) continue;
        y1[t] = -expm1(-dt / T1);
        y2[t] = -expm1(-dt / T2);
        double ksum = 0.0;
#pragma unroll
        for (int p = 0; p < P; ++p) {
            if ((gm && p == t) || !kch) continue;
            // ME: channel a*P+b is the rate a -> b; GM: channel b*P+a
            const double kgo = kch[(long long)(gm ? p * P + t : t * P + p) * n_act + v];
            const double kin = kch[(long long)(gm ? t * P + p : p * P + t) * n_act + v];
            ksum += kgo;
            if (kin != 0.0) fin[t][p] = -expm1(-dt * kin);
        }
        yo[t] = -expm1(-dt * ksum);
    }
    float *o = tab + (long long)d * split_fields(P) * n_act + v;
    int f = 0;
#pragma unroll
    for (int t = 0; t < P; ++t) o[(long long)(f++) * n_act] = (float)y1[t];
#pragma unroll
    for (int t = 0; t < P; ++t) o[(long long)(f++) * n_act] = (float)y2[t];
#pragma unroll
    for (int t = 0; t < P; ++t) o[(long long)(f++) * n_act] = (float)yo[t];
#pragma unroll
    for (int t = 0; t < P; ++t)
#pragma unroll
        for (int p = 0; p < P; ++p) o[(long long)(f++) * n_act] = (float)fin[t][p];
}
}  // namespace

cudaError_t launch_split_table(int P, const float *dts, int n_dt, int n_act, int gm, const float *rho,
                               const float *t1, const float *t2, const float *kch, float *tab, cudaStream_t st) {
    const long long n = (long long)n_dt * n_act;
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n + 127) / 128);
    switch (P) {
    case 1: split_table_kernel<1><<<blocks, 128, 0, st>>>(dts, n_dt, n_act, gm, rho, t1, t2, kch, tab); break;
    case 2: split_table_kernel<2><<<blocks, 128, 0, st>>>(dts, n_dt, n_act, gm, rho, t1, t2, kch, tab); break;
    case 3: split_table_kernel<3><<<blocks, 128, 0, st>>>(dts, n_dt, n_act, gm, rho, t1, t2, kch, tab); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_scan_fast_tab(int co, int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                                 const FastGrid &g) {
    Kernel k = select(co, P, NS, all_free);
    if (!k) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kBlock, smem, st>>>(g.descs, g.items, g.n_items, g.counter);
    return cudaGetLastError();
}

int occupancy_scan_fast_tab(int co, int P, int NS, bool all_free, size_t smem) {
    Kernel k = select(co, P, NS, all_free);
    int n = 0;
    if (!k || cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kBlock, smem) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_exact_table(int P, const float *dts, int n_dt, int n_act, int S, int layout, unsigned bound,
                               const float *rho, const float *t1, const float *t2, const float *kch, float *tab,
                               cudaStream_t st) {
    const long long n = (long long)n_dt * n_act;
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n + 127) / 128);
#define MRL_XTAB(PP) \
    exact_table_kernel<PP><<<blocks, 128, 0, st>>>(dts, n_dt, n_act, S, layout, bound, rho, t1, t2, kch, tab)
    switch (P) {
    case 1: MRL_XTAB(1); break;
    case 2: MRL_XTAB(2); break;
    case 3: MRL_XTAB(3); break;
    case 4: MRL_XTAB(4); break;
    case 5: MRL_XTAB(5); break;
    default: return cudaErrorInvalidValue;
    }
#undef MRL_XTAB
    return cudaGetLastError();
}

}  // namespace mrl
