// yk_noise.cu -- coloured noise xi = Z2D(mask * D2Z(w)) / V of
// code/src/colouredNoise.cpp:155-178, rebuilt as three shared-memory FFT
// passes instead of RNG kernel + cuFFT D2Z + mask kernel + cuFFT Z2D:
//   1. rows:    Philox Gaussian white noise generated in registers, written
//               to shared memory, forward FFT along x, spectrum rows stored;
//               two real rows go through one complex FFT (w_t + i w_{t+1})
//               and are separated by the symmetry of real transforms;
//   2. columns: a strip of columns loaded once, forward FFT along t, sharp
//               momentum cutoff (and the 1/V normalisation of the reference's
//               mask), inverse FFT along t, stored back -- only strips that
//               hold a kept mode: a column kx keeps some mode exactly when it
//               keeps (0, kx), and the other columns come out zero;
//   3. rows:    inverse FFT along x of two rows at once (Y_t + i Y_{t+1}:
//               both results are real), written as xi.
// The real field is transformed as a complex one; since the cutoff is even
// in k, this equals the reference's r2c/c2r pair.
// When the cutoff keeps every mode (cutFraction >= 1) the filter is the
// identity and a single generation pass writes xi = w.
// Every chain of a context is handled by the same launches through
// block -> (chain, row / column strip) tables.
#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

// In-place FFT of `nseq` sequences of length N in shared memory; element j of
// sequence c is buf[j * sj + c * sc].  Radix-2 for powers of two, direct DFT
// (through tmp) otherwise.  tw[k] = exp(-2 pi i k / N), k < N.
__device__ void smem_fft(double2* buf, double2* tmp, int N, int nseq, int sj, int sc,
                         const double2* __restrict__ tw, bool inverse)
{
    const int nt = blockDim.x;
    if ((N & (N - 1)) == 0) {
        int lg = 0;
        while ((1 << lg) < N) ++lg;
        for (int idx = threadIdx.x; idx < N * nseq; idx += nt) {
            const int c = idx >> lg, j = idx & (N - 1);
            const int rj = (int)(__brev((unsigned)j) >> (32 - lg));
            if (lg > 0 && j < rj) {
                double2* a = buf + j * sj + c * sc;
                double2* b = buf + rj * sj + c * sc;
                const double2 t = *a;
                *a = *b;
                *b = t;
            }
        }
        __syncthreads();
        for (int s = 1; s <= lg; ++s) {
            const int h = 1 << (s - 1);   // butterfly span; twiddle stride N / 2^s
            for (int idx = threadIdx.x; idx < (N >> 1) * nseq; idx += nt) {
                const int c = idx >> (lg - 1), bidx = idx & ((N >> 1) - 1);
                const int grp = bidx >> (s - 1), k = bidx & (h - 1);
                const int i0 = (grp << s) + k, i1 = i0 + h;
                double2 w = tw[k << (lg - s)];
                if (inverse) w.y = -w.y;
                double2* pa = buf + i0 * sj + c * sc;
                double2* pb = buf + i1 * sj + c * sc;
                const double2 u = *pa, v0 = *pb;
                const double2 v = make_double2(v0.x * w.x - v0.y * w.y, v0.x * w.y + v0.y * w.x);
                *pa = make_double2(u.x + v.x, u.y + v.y);
                *pb = make_double2(u.x - v.x, u.y - v.y);
            }
            __syncthreads();
        }
    } else {
        for (int idx = threadIdx.x; idx < N * nseq; idx += nt) {
            const int c = idx / N, k = idx - c * N;
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < N; ++j) {
                double2 w = tw[(int)(((long long)j * k) % N)];
                if (inverse) w.y = -w.y;
                const double2 x = buf[j * sj + c * sc];
                sr += x.x * w.x - x.y * w.y;
                si += x.x * w.y + x.y * w.x;
            }
            tmp[k * sj + c * sc] = make_double2(sr, si);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < N * nseq; idx += nt) {
            const int c = idx / N, j = idx - c * N;
            buf[j * sj + c * sc] = tmp[j * sj + c * sc];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ double white_at(const ChainDev& C, const double* given, int n)
{
    if (given) return given[n];
    const RngStream rs = rng_stream(C.seed, C.chain_id, (uint64_t)C.step, 1u, 0u);
    return normal_at(rs, (uint32_t)n);
}

// rows t and t + 1 (when t + 1 < Nt) of the white noise, transformed along x
// as one complex sequence w_t + i w_{t+1}; with Z its transform,
// W_t[k] = (Z[k] + conj Z[-k]) / 2 and W_{t+1}[k] = (Z[k] - conj Z[-k]) / 2i.
// Only the columns that keep a mode are stored.
__global__ void __launch_bounds__(kBlock) noise_rows_fwd(ChainDev* chains, const int2* rows, int nrows,
                                                         const double* given)
{
    extern __shared__ double2 sm[];
    for (int item = blockIdx.x; item < nrows; item += gridDim.x) {
    if (item != (int)blockIdx.x) __syncthreads();   // the previous item's reads of sm are done
    const int2 ct = rows[item];
    const ChainDev& C = chains[ct.x];
    const int Nx = C.Nx, t = ct.y;
    const bool two = t + 1 < C.Nt;
    double2* buf = sm;
    double2* tmp = sm + Nx;
    const int base = t * Nx;
    if (!given && (Nx & 3) == 0) {
        // four normals of each row per counter
        const RngStream rs = rng_stream(C.seed, C.chain_id, (uint64_t)C.step, 1u, 0u);
        for (int x4 = threadIdx.x; x4 < Nx / 4; x4 += blockDim.x) {
            const float4 z = normal4(rs, (uint32_t)((base >> 2) + x4));
            const float4 y = two ? normal4(rs, (uint32_t)(((base + Nx) >> 2) + x4)) : make_float4(0.f, 0.f, 0.f, 0.f);
            buf[4 * x4] = make_double2(z.x, y.x);
            buf[4 * x4 + 1] = make_double2(z.y, y.y);
            buf[4 * x4 + 2] = make_double2(z.z, y.z);
            buf[4 * x4 + 3] = make_double2(z.w, y.w);
        }
    } else {
        for (int x = threadIdx.x; x < Nx; x += blockDim.x)
            buf[x] = make_double2(white_at(C, given, base + x), two ? white_at(C, given, base + Nx + x) : 0.0);
    }
    __syncthreads();
    smem_fft(buf, tmp, Nx, 1, 1, 0, C.tw_x, false);
    for (int k = threadIdx.x; k < Nx; k += blockDim.x) {
        if (!C.keep[k]) continue;   // the column keeps no mode
        const double2 zk = buf[k], zm = buf[k == 0 ? 0 : Nx - k];
        C.spec[base + k] = make_double2(0.5 * (zk.x + zm.x), 0.5 * (zk.y - zm.y));
        if (two) C.spec[base + Nx + k] = make_double2(0.5 * (zk.y + zm.y), 0.5 * (zm.x - zk.x));
    }
    }
}

__global__ void __launch_bounds__(kBlock) noise_cols(ChainDev* chains, const int2* cols, int ncols)
{
    extern __shared__ double2 sm[];
    for (int item = blockIdx.x; item < ncols; item += gridDim.x) {
    if (item != (int)blockIdx.x) __syncthreads();
    const int2 cc = cols[item];
    const ChainDev& C = chains[cc.x];
    const int Nt = C.Nt, Nx = C.Nx, x0 = cc.y;
    int cw = noise_strip(Nt);
    if (cw > Nx - x0) cw = Nx - x0;
    double2* buf = sm;
    double2* tmp = sm + Nt * cw;
    for (int idx = threadIdx.x; idx < Nt * cw; idx += blockDim.x) {
        const int t = idx / cw, c = idx - t * cw;
        buf[idx] = C.keep[x0 + c] ? C.spec[t * Nx + x0 + c] : make_double2(0.0, 0.0);   // unwritten otherwise
    }
    __syncthreads();
    smem_fft(buf, tmp, Nt, cw, cw, 1, C.tw_t, false);
    const double inv = 1.0 / (double)C.V;
    for (int idx = threadIdx.x; idx < Nt * cw; idx += blockDim.x) {
        const int t = idx / cw, c = idx - t * cw;
        const double m = C.keep[t * Nx + x0 + c] ? inv : 0.0;
        buf[idx].x *= m;
        buf[idx].y *= m;
    }
    __syncthreads();
    smem_fft(buf, tmp, Nt, cw, cw, 1, C.tw_t, true);
    for (int idx = threadIdx.x; idx < Nt * cw; idx += blockDim.x) {
        const int t = idx / cw, c = idx - t * cw;
        C.spec[t * Nx + x0 + c] = buf[idx];
    }
    }
}

// rows t and t + 1 of the filtered spectrum, inverse-transformed along x as
// one sequence Y_t + i Y_{t+1}: both results are real, so they come out as
// the real and imaginary parts.  Columns that keep no mode are zero.
__global__ void __launch_bounds__(kBlock) noise_rows_inv(ChainDev* chains, const int2* rows, int nrows)
{
    extern __shared__ double2 sm[];
    for (int item = blockIdx.x; item < nrows; item += gridDim.x) {
    if (item != (int)blockIdx.x) __syncthreads();
    const int2 ct = rows[item];
    const ChainDev& C = chains[ct.x];
    const int Nx = C.Nx, t = ct.y;
    const bool two = t + 1 < C.Nt;
    double2* buf = sm;
    double2* tmp = sm + Nx;
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        double2 v = make_double2(0.0, 0.0);
        if (C.keep[x]) {
            const double2 a = C.spec[t * Nx + x];
            const double2 b = two ? C.spec[(t + 1) * Nx + x] : make_double2(0.0, 0.0);
            v = make_double2(a.x - b.y, a.y + b.x);
        }
        buf[x] = v;
    }
    __syncthreads();
    smem_fft(buf, tmp, Nx, 1, 1, 0, C.tw_x, true);
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        C.xi[t * Nx + x] = buf[x].x;
        if (two) C.xi[(t + 1) * Nx + x] = buf[x].y;
    }
    }
}

__global__ void __launch_bounds__(kBlock) noise_white(ChainDev* chains, const int2* tiles, const double* given)
{
    const int2 ct = tiles[blockIdx.x];
    const ChainDev& C = chains[ct.x];
    const int n = ct.y + threadIdx.x;
    if (n < C.V) C.xi[n] = white_at(C, given, n);
}

void noise_init_attributes()
{
    static bool attr_set = false;
    if (!attr_set) {
        const int big = (int)(2 * sizeof(double2) * kMaxFFT);
        cudaFuncSetAttribute(noise_rows_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(noise_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        cudaFuncSetAttribute(noise_rows_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        attr_set = true;
    }
}

cudaError_t launch_noise_tables(ChainDev* d_chains, const NoiseTables& tb, int max_nx, int max_cols_elems,
                                const double* given, cudaStream_t stream, int max_blocks)
{
    noise_init_attributes();
    auto grid = [&](int n) { return (max_blocks > 0 && n > max_blocks) ? max_blocks : n; };
    if (tb.nwhite > 0) noise_white<<<tb.nwhite, kTile, 0, stream>>>(d_chains, tb.white, given);
    if (tb.nrows > 0) {
        const size_t rs = 2 * sizeof(double2) * (size_t)max_nx;
        const size_t cs = 2 * sizeof(double2) * (size_t)max_cols_elems;
        noise_rows_fwd<<<grid(tb.nrows), kBlock, rs, stream>>>(d_chains, tb.rows, tb.nrows, given);
        if (tb.ncols > 0) noise_cols<<<grid(tb.ncols), kBlock, cs, stream>>>(d_chains, tb.cols, tb.ncols);
        noise_rows_inv<<<grid(tb.nrows), kBlock, rs, stream>>>(d_chains, tb.rows, tb.nrows);
    }
    return cudaGetLastError();
}

}  // namespace yk
