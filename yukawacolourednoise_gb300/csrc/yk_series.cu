// yk_series.cu -- error analysis of a Monte Carlo time series on the device.
//
// The reference analyses its traces.csv offline (analysis/functions.py) with
// the Gamma-method of its FFTW-based AutoCorrelation library
// (analysis/AutoCorrelation/ac.cpp:73-181, called at functions.py:102-113):
//   <sigma>, <|sigma|>                 ComputeStatistics of the series (:42-49)
//   chi    = V <(s - <s>)^2>           ComputeStatistics((s - <s>)^2) x V (:54-57)
//   binder = 1 - <s^4> / (3 <s^2>^2)   (:73-78)
// Here the same estimators run on the GPU over a series of per-configuration
// <sigma> values.  Errors follow U. Wolff, "Monte Carlo errors with less
// errors", Comput. Phys. Commun. 156 (2004) 143: the autocorrelation function
// Gamma(t) of each observable's fluctuation series is summed on the device
// (one block per lag, fixed-order block reductions), the automatic window and
// the errors on the host (gamma_window).  The Binder cumulant, a function of
// two means, takes Wolff's derived-quantity error: its fluctuation series is
// the gradient-weighted sum f_1 (s^4 - <s^4>) + f_2 (s^2 - <s^2>).  (The
// reference's helper propagate_division_relative, functions.py:219, inverts
// the ratios dx/x; it is not restated.)
#include <algorithm>
#include <cstring>
#include <vector>

#include "yk_common.cuh"
#include "yk_host.h"
#include "yk_kernels.h"

namespace yk {

namespace {

constexpr int kSeriesBlock = 256;
constexpr int64_t kMaxLag = 8192;   // Gamma(t) is summed for t <= min(n / 2, kMaxLag)

// mom = {sum s, sum |s|, sum s^2, sum s^4} in one block (fixed order)
__global__ void __launch_bounds__(kSeriesBlock) series_moments_kernel(const double* __restrict__ x, int64_t n,
                                                                     double* __restrict__ mom)
{
    __shared__ double red[64];
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = x[i], v2 = v * v;
        a += v;
        b += fabs(v);
        c += v2;
        d += v2 * v2;
    }
    const double2 ab = block_sum2(a, b, red);
    const double2 cd = block_sum2(c, d, red);
    if (threadIdx.x == 0) {
        mom[0] = ab.x;
        mom[1] = ab.y;
        mom[2] = cd.x;
        mom[3] = cd.y;
    }
}

// The fluctuation series of the four observables, f[k * n + i]:
// 0: s - <s>; 1: |s| - <|s|>; 2: z - <z> with z = (s - <s>)^2; 3: the Binder
// projection.  zsum: sum z (one block, fixed order).
__global__ void __launch_bounds__(kSeriesBlock) series_fluct_kernel(const double* __restrict__ x, int64_t n,
                                                                   const double* __restrict__ mom,
                                                                   double* __restrict__ f, double* zsum)
{
    __shared__ double red[64];
    const double inv = 1.0 / (double)n;
    const double m1 = mom[0] * inv, ma = mom[1] * inv, m2 = mom[2] * inv, m4 = mom[3] * inv;
    const double g1 = -1.0 / (3.0 * m2 * m2), g2 = 2.0 * m4 / (3.0 * m2 * m2 * m2);
    double zs = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = x[i], v2 = v * v, dv = v - m1;
        f[i] = dv;
        f[n + i] = fabs(v) - ma;
        f[2 * n + i] = dv * dv;   // centred below
        f[3 * n + i] = g1 * (v2 * v2 - m4) + g2 * (v2 - m2);
        zs += dv * dv;
    }
    const double zt = block_sum(zs, red);
    if (threadIdx.x == 0) *zsum = zt;
}

__global__ void __launch_bounds__(kSeriesBlock) series_center_kernel(double* __restrict__ z, int64_t n,
                                                                    const double* zsum)
{
    const double mz = *zsum / (double)n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] -= mz;
}

// gam[k * (T + 1) + t] = sum_{i < n - t} f_k[i] f_k[i + t] / (n - t): block
// (t, k), fixed-order block reduction.
__global__ void __launch_bounds__(kSeriesBlock) series_gamma_kernel(const double* __restrict__ f, int64_t n,
                                                                   int64_t T, double* __restrict__ gam)
{
    __shared__ double red[64];
    const int64_t t = blockIdx.x;
    const int k = blockIdx.y;
    const double* fk = f + (size_t)k * n;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i + t < n; i += blockDim.x) s += fk[i] * fk[i + t];
    const double r = block_sum(s, red);
    if (threadIdx.x == 0) gam[(size_t)k * (T + 1) + t] = r / (double)(n - t);
}

}  // namespace

int series_analyse(const double* d_x, int64_t n, int64_t volume, double stau, yk_series_stats* out,
                   cudaStream_t s)
{
    std::memset(out, 0, sizeof(*out));
    out->n = n;
    if (n < 2) {
        set_error("series analysis: %lld measurements (need >= 2)", (long long)n);
        return YK_EINVAL;
    }
    const int64_t T = std::min(n / 2, kMaxLag);
    double* buf = nullptr;
    const size_t nbuf = 4 + 1 + 4 * (size_t)n + 4 * (size_t)(T + 1);
    if (cudaMalloc(&buf, sizeof(double) * nbuf) != cudaSuccess) {
        cudaGetLastError();
        set_error("series analysis: allocation of %zu bytes failed", sizeof(double) * nbuf);
        return YK_ENOMEM;
    }
    double *mom = buf, *zsum = buf + 4, *f = buf + 5, *gam = f + 4 * (size_t)n;
    cudaError_t e;
    series_moments_kernel<<<1, kSeriesBlock, 0, s>>>(d_x, n, mom);
    series_fluct_kernel<<<1, kSeriesBlock, 0, s>>>(d_x, n, mom, f, zsum);
    const int cgrid = (int)std::min<int64_t>((n + kSeriesBlock - 1) / kSeriesBlock, 1024);
    series_center_kernel<<<cgrid, kSeriesBlock, 0, s>>>(f + 2 * (size_t)n, n, zsum);
    series_gamma_kernel<<<dim3((unsigned)(T + 1), 4), kSeriesBlock, 0, s>>>(f, n, T, gam);
    e = cudaGetLastError();
    std::vector<double> hm(5), hg(4 * (size_t)(T + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), mom, sizeof(double) * 5, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hg.data(), gam, sizeof(double) * hg.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    if (e != cudaSuccess) {
        set_error("series analysis: %s", cudaGetErrorString(e));
        return YK_ECUDA;
    }
    const double inv = 1.0 / (double)n;
    const double m1 = hm[0] * inv, ma = hm[1] * inv, m2 = hm[2] * inv, m4 = hm[3] * inv, mz = hm[4] * inv;
    double* dst[4] = {out->sigma, out->abs_sigma, out->chi, out->binder};
    for (int k = 0; k < 4; ++k) gamma_window(hg.data() + (size_t)k * (T + 1), T, n, stau, dst[k]);
    out->sigma[0] = m1;
    out->abs_sigma[0] = ma;
    // chi: V times the mean and the error of z (functions.py:54-57)
    out->chi[0] = (double)volume * mz;
    out->chi[1] *= (double)volume;
    out->chi[2] *= (double)volume;
    out->binder[0] = 1.0 - m4 / (3.0 * m2 * m2);
    return YK_OK;
}

}  // namespace yk

using namespace yk;

extern "C" int yk_series_analyse_host(const double* series, int64_t n, int64_t volume, double stau,
                                      yk_series_stats* out)
{
    if (!series || !out || n < 2 || volume < 1 || !(stau > 0.0)) {
        set_error("yk_series_analyse_host: bad arguments");
        return YK_EINVAL;
    }
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * (size_t)n) != cudaSuccess) {
        cudaGetLastError();
        set_error("yk_series_analyse_host: allocation failed");
        return YK_ENOMEM;
    }
    cudaError_t e = cudaMemcpy(d, series, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    int rc = (e == cudaSuccess) ? series_analyse(d, n, volume, stau, out, nullptr) : YK_ECUDA;
    if (e != cudaSuccess) set_error("yk_series_analyse_host: %s", cudaGetErrorString(e));
    cudaFree(d);
    return rc;
}
