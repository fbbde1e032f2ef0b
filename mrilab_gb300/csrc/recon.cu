// Image reconstruction after the scan: mrl_recon_cart and mrl_grid2d
// (include/mrl_recon.h).
//
// Cartesian / EPI (DoCartRecon.m, DoEPIRecon.m): one gather kernel builds
// every (coil, echo) k-space volume in its final layout -- pools summed,
// echoes split or EPI lines sorted and reversed, the last readout point
// dropped, zero filling, orientation -- already rolled by floor(n / 2) in
// each dimension (the inner fftshift); cuFFT runs the batched inverse 3D
// transform in FP64; a second kernel applies the outer fftshift, the 1/N
// normalisation of ifftn and writes real, imaginary, magnitude and phase.
//
// Gridding (DoGridding.cpp): one thread per sample walks the sample's
// kernel window with the reference's index arithmetic and adds its weighted
// value into the grid with FP64 atomics (the order of the additions to one
// grid point is not fixed; each point takes a few terms).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>

#include "../../include/mrl_recon.h"

namespace mrl {
void record_error(const char *msg);
void record_timing(const double t[8]);

namespace {

struct ReconGeom {
    int F;           // readout points kept (res_freq - 1)
    int L;           // phase lines (Cartesian lines, EPI etl * shots)
    int Z;           // slices
    int fx, fy, fz;  // zero-filled sizes along readout, phase, slice
    int ox, oy, oz;  // offsets of the sampled block inside them
    int n[3];        // image dims (N0, N1, N2)
    int readout_first;
    int res_freq, lines_raw, rx, pools, echoes, etl;
};

// Value of zero-filled, oriented k-space point (i0, i1, i2) of coil c, echo
// e: the pools' sum of the signal sample it comes from, or 0.
__device__ __forceinline__ double2 ksample(const ReconGeom &g, const double *sx, const double *sy, int i0, int i1,
                                           int i2, int c, int e) {
    const int ir = g.readout_first ? i0 : i1;  // zero-filled readout index
    const int ip = g.readout_first ? i1 : i0;  // zero-filled phase index
    const int f = ir - g.ox, l = ip - g.oy, z = i2 - g.oz;
    if (f < 0 || f >= g.F || l < 0 || l >= g.L || z < 0 || z >= g.Z) return make_double2(0.0, 0.0);
    // row and column of the raw signal [res_freq * echoes][lines][slices][rx][pools]
    long long row, col;
    if (g.etl > 0) {  // EPI: line l = (echo of the train) * shots + shot; every second train echo reversed
        const int te = l / g.lines_raw, shot = l - te * g.lines_raw;
        const int fr = (te & 1) ? (g.res_freq - 1 - f) : f;
        row = (long long)te * g.res_freq + fr;
        col = shot;
    } else {
        row = (long long)e * g.res_freq + f;
        col = l;
    }
    const long long rows = (long long)g.res_freq * (g.etl > 0 ? g.etl : g.echoes);
    const long long per_pool = rows * g.lines_raw * g.Z * g.rx;
    const long long base = row + rows * (col + (long long)g.lines_raw * (z + (long long)g.Z * c));
    double x = 0.0, y = 0.0;
    for (int p = 0; p < g.pools; ++p) {  // sum(SX, 5) in pool order
        x += sx[base + p * per_pool];
        y += sy[base + p * per_pool];
    }
    return make_double2(x, y);
}

__device__ __forceinline__ void unshift(const ReconGeom &g, long long r, int &j0, int &j1, int &j2) {
    const int k0 = (int)(r % g.n[0]);
    const int k1 = (int)((r / g.n[0]) % g.n[1]);
    const int k2 = (int)(r / ((long long)g.n[0] * g.n[1]));
    j0 = (k0 - g.n[0] / 2 + g.n[0]) % g.n[0];
    j1 = (k1 - g.n[1] / 2 + g.n[1]) % g.n[1];
    j2 = (k2 - g.n[2] / 2 + g.n[2]) % g.n[2];
}

// buffer[k] = S[(k - floor(n/2)) mod n] per dimension (fftshift before the
// transform); cuFFT's layout of a column-major (N0, N1, N2) volume is its
// row-major (N2, N1, N0).
__global__ void recon_gather(ReconGeom g, const double *sx, const double *sy, cufftDoubleComplex *buf) {
    const long long vol = (long long)g.n[0] * g.n[1] * g.n[2];
    const long long total = vol * g.rx * g.echoes;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long b = i / vol, r = i - b * vol;
        int j0, j1, j2;
        unshift(g, r, j0, j1, j2);
        const double2 v = ksample(g, sx, sy, j0, j1, j2, (int)(b % g.rx), (int)(b / g.rx));
        buf[i] = make_cuDoubleComplex(v.x, v.y);
    }
}

// y[k] = X[(k - floor(n/2)) mod n] / N per dimension (fftshift after the
// transform, ifftn's normalisation); outputs [N0][N1][N2][Rx][E].
__global__ void recon_finish(ReconGeom g, const cufftDoubleComplex *buf, double *re, double *im, double *mag,
                             double *ph) {
    const long long vol = (long long)g.n[0] * g.n[1] * g.n[2];
    const long long total = vol * g.rx * g.echoes;
    const double scale = 1.0 / (double)vol;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long b = i / vol, r = i - b * vol;
        int j0, j1, j2;
        unshift(g, r, j0, j1, j2);
        const cufftDoubleComplex v = buf[b * vol + j0 + (long long)g.n[0] * (j1 + (long long)g.n[1] * j2)];
        const double x = v.x * scale, y = v.y * scale;
        if (re) re[i] = x;
        if (im) im[i] = y;
        if (mag) mag[i] = hypot(x, y);
        if (ph) ph[i] = atan2(y, x);
    }
}

// DoGridding.cpp:73-118, one thread per sample
__global__ void grid2d_kernel(const double *kx, const double *ky, const double *sx, const double *sy,
                              const double *dcf, int n, const double *kern, int nk, int G, double width, double *gx,
                              double *gy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = kx[i], y = ky[i];
    const double center = (G - 1) / 2.0;
    double kxmin = x - width, kxmax = x + width, kymin = y - width, kymax = y + width;
    if (kxmin < -0.5) kxmin = -0.5;
    if (kxmax > 0.5) kxmax = 0.5;
    if (kymin < -0.5) kymin = -0.5;
    if (kymax > 0.5) kymax = 0.5;
    const int ixmin = (int)((kxmin + 0.5) * (G - 1)), ixmax = (int)((kxmax + 0.5) * (G - 1));
    const int iymin = (int)((kymin + 0.5) * (G - 1)), iymax = (int)((kymax + 0.5) * (G - 1));
    for (int ix = ixmin; ix <= ixmax; ++ix) {
        const double dkx = ((double)ix - center) / (G - 1) - x;
        for (int iy = iymin; iy <= iymax; ++iy) {
            const double dky = ((double)iy - center) / (G - 1) - y;
            const double dk = sqrt(dkx * dkx + dky * dky);
            if (dk <= width) {
                const double fi = (dk / width) * (double)(nk - 1);
                const int ki = (int)fi;
                const double fr = fi - (double)ki;
                // the reference reads kern[ki + 1] at dk == width (one past the
                // table); that point gets the table's last value here
                const double k1 = ki + 1 < nk ? kern[ki + 1] : kern[nk - 1];
                const double kv = kern[ki] * (1 - fr) + k1 * fr;
                const long long o = (long long)ix * G + iy;
                atomicAdd(gx + o, kv * sx[i] * dcf[i]);
                atomicAdd(gy + o, kv * sy[i] * dcf[i]);
            }
        }
    }
}

int fail(const char *what, cudaError_t e, int rc) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    record_error(buf);
    return rc;
}

int fail_msg(const char *msg, int rc) {
    record_error(msg);
    return rc;
}

}  // namespace
}  // namespace mrl

extern "C" int mrl_recon_cart(mrl_recon_args *a) {
    using namespace mrl;
    const auto t0 = std::chrono::steady_clock::now();
    double tim[8] = {0};
    record_timing(tim);
    record_error("");
    if (!a || !a->sx || !a->sy) return fail_msg("NULL argument", MRL_ERR_ARG);
    if (a->abi_version != MRL_ABI_VERSION) return fail_msg("ABI version mismatch", MRL_ERR_ARG);
    if (a->res_freq < 2 || a->lines < 1 || a->slices < 1 || a->rx < 1 || a->pools < 1 || a->echoes < 1 ||
        a->epi_etl < 0 || (a->epi_etl > 0 && a->echoes != 1))
        return fail_msg("bad sizes", MRL_ERR_ARG);
    ReconGeom g{};
    g.res_freq = a->res_freq;
    g.lines_raw = a->lines;
    g.rx = a->rx;
    g.pools = a->pools;
    g.echoes = a->echoes;
    g.etl = a->epi_etl;
    g.F = a->res_freq - 1;
    g.L = a->epi_etl > 0 ? a->epi_etl * a->lines : a->lines;
    g.Z = a->slices;
    const bool zf = a->zf_kx > 0 || a->zf_ky > 0 || a->zf_kz > 0;
    if (zf) {
        if (a->zf_kx < g.F || a->zf_ky < g.L || a->zf_kz < 1)
            return fail_msg("zero filling below the sampled size", MRL_ERR_ARG);
        // DoCartRecon.m:27-36: the sampled block starts at ZF/2 - size/2 + 1
        // (1-based) in kx and ky and at ZFz floor(Z/2) - floor(Z/2) + 1 in z
        if ((a->zf_kx - g.F) % 2 || (a->zf_ky - g.L) % 2)
            return fail_msg("zero filling: the sampled block cannot be centred on whole samples", MRL_ERR_ARG);
        g.fx = a->zf_kx;
        g.fy = a->zf_ky;
        g.fz = a->zf_kz * g.Z;
        g.ox = a->zf_kx / 2 - g.F / 2;
        g.oy = a->zf_ky / 2 - g.L / 2;
        g.oz = a->zf_kz * (g.Z / 2) - g.Z / 2;
    } else {
        g.fx = g.F;
        g.fy = g.L;
        g.fz = g.Z;
    }
    g.readout_first = a->readout_first != 0;
    g.n[0] = g.readout_first ? g.fx : g.fy;
    g.n[1] = g.readout_first ? g.fy : g.fx;
    g.n[2] = g.fz;
    for (int d = 0; d < 3; ++d) a->out_dims[d] = g.n[d];
    const long long vol = (long long)g.n[0] * g.n[1] * g.n[2];
    const long long nb = (long long)g.rx * g.echoes;
    const long long raw =
        (long long)a->res_freq * (g.etl > 0 ? g.etl : g.echoes) * a->lines * g.Z * g.rx * g.pools;
    if (vol * nb > (1LL << 31)) return fail_msg("image too large", MRL_ERR_UNSUPPORTED);

    cudaError_t e = cudaSetDevice(a->gpu_index);
    if (e != cudaSuccess) return fail("cudaSetDevice", e, MRL_ERR_NO_DEVICE);
    double *d_raw = nullptr, *d_out = nullptr;
    cufftDoubleComplex *d_buf = nullptr;
    cufftHandle plan = 0;
    bool have_plan = false;
    int rc = MRL_OK;
    cudaStream_t st = nullptr;
    const size_t out_b = (size_t)vol * nb * sizeof(double);
    do {
        if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) break;
        if ((e = cudaMalloc(&d_raw, 2 * raw * sizeof(double))) != cudaSuccess) break;
        if ((e = cudaMalloc(&d_buf, vol * nb * sizeof(cufftDoubleComplex))) != cudaSuccess) break;
        if ((e = cudaMalloc(&d_out, 4 * out_b)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(d_raw, a->sx, raw * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess)
            break;
        if ((e = cudaMemcpyAsync(d_raw + raw, a->sy, raw * sizeof(double), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            break;
        const int threads = 256;
        const int blocks = (int)std::min<long long>((vol * nb + threads - 1) / threads, 152LL * 32);
        recon_gather<<<blocks, threads, 0, st>>>(g, d_raw, d_raw + raw, d_buf);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        // column-major (N0, N1, N2) = row-major (N2, N1, N0)
        int dims[3] = {g.n[2], g.n[1], g.n[0]};
        if (cufftPlanMany(&plan, 3, dims, nullptr, 1, (int)vol, nullptr, 1, (int)vol, CUFFT_Z2Z, (int)nb) !=
            CUFFT_SUCCESS) {
            rc = fail_msg("cufftPlanMany failed", MRL_ERR_CUDA);
            break;
        }
        have_plan = true;
        if (cufftSetStream(plan, st) != CUFFT_SUCCESS ||
            cufftExecZ2Z(plan, d_buf, d_buf, CUFFT_INVERSE) != CUFFT_SUCCESS) {
            rc = fail_msg("cufftExecZ2Z failed", MRL_ERR_CUDA);
            break;
        }
        double *o_re = d_out, *o_im = d_out + vol * nb, *o_mag = d_out + 2 * vol * nb, *o_ph = d_out + 3 * vol * nb;
        recon_finish<<<blocks, threads, 0, st>>>(g, d_buf, a->img_real ? o_re : nullptr,
                                                 a->img_imag ? o_im : nullptr, a->img_mag ? o_mag : nullptr,
                                                 a->img_phase ? o_ph : nullptr);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        double *hs[4] = {a->img_real, a->img_imag, a->img_mag, a->img_phase};
        double *ds[4] = {o_re, o_im, o_mag, o_ph};
        for (int k = 0; k < 4 && e == cudaSuccess; ++k)
            if (hs[k]) e = cudaMemcpyAsync(hs[k], ds[k], out_b, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) break;
        e = cudaStreamSynchronize(st);
        tim[5] = 3;
        tim[6] = 2.0 * raw * sizeof(double);
    } while (false);
    if (rc == MRL_OK && e != cudaSuccess)
        rc = fail("recon", e, e == cudaErrorMemoryAllocation ? MRL_ERR_NOMEM : MRL_ERR_CUDA);
    if (have_plan) cufftDestroy(plan);
    cudaFree(d_raw);
    cudaFree(d_buf);
    cudaFree(d_out);
    if (st) cudaStreamDestroy(st);
    tim[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    record_timing(tim);
    return rc;
}

extern "C" int mrl_grid2d(const double *kx, const double *ky, const double *sx, const double *sy, const double *dcf,
                          int n, const double *kernel, int nk, int G, double half_width, double *gx, double *gy,
                          int gpu_index) {
    using namespace mrl;
    double tim[8] = {0};
    record_timing(tim);
    record_error("");
    if (!kx || !ky || !sx || !sy || !dcf || !kernel || !gx || !gy) return fail_msg("NULL argument", MRL_ERR_ARG);
    if (n < 0 || nk < 2 || G < 2) return fail_msg("bad sizes", MRL_ERR_ARG);
    cudaError_t e = cudaSetDevice(gpu_index);
    if (e != cudaSuccess) return fail("cudaSetDevice", e, MRL_ERR_NO_DEVICE);
    const double width = half_width / (G - 1);  // DoGridding.cpp:58
    const size_t grid_b = (size_t)G * G * sizeof(double);
    const size_t in_b = (size_t)n * sizeof(double);
    double *d = nullptr;
    if ((e = cudaMalloc(&d, 5 * in_b + nk * sizeof(double) + 2 * grid_b)) != cudaSuccess)
        return fail("cudaMalloc", e, MRL_ERR_NOMEM);
    double *d_k = d + 5 * (size_t)n, *d_gx = d_k + nk, *d_gy = d_gx + (size_t)G * G;
    const double *src[5] = {kx, ky, sx, sy, dcf};
    for (int k = 0; k < 5 && e == cudaSuccess; ++k)
        e = cudaMemcpy(d + (size_t)k * n, src[k], in_b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_k, kernel, nk * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_gx, 0, 2 * grid_b);
    if (e == cudaSuccess && n > 0) {
        grid2d_kernel<<<(n + 127) / 128, 128>>>(d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n, d + 4 * (size_t)n, n,
                                                 d_k, nk, G, width, d_gx, d_gy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(gx, d_gx, grid_b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(gy, d_gy, grid_b, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail("gridding", e, MRL_ERR_CUDA);
    tim[5] = 1;
    record_timing(tim);
    return MRL_OK;
}
