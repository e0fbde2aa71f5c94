// yk_learned.cu -- the learned preconditioner: a small convolutional network
// z = M(r) on the lattice, its training on the GPU (own forward and backward
// kernels, Adam), and a flexible GCR solver that uses it inside FP64
// iterative refinement.  No reference counterpart: the reference solves with
// plain CG (code/src/CGsolver.cu:72-170); a learned solve is accepted only
// when its FP64 true residual meets the same tolerance.
//
// Network (one real plane; D has real coefficients, so a complex field is
// two independent real planes): M(r) = skip r + N^T N r, symmetric positive
// definite by construction (so A M has a positive real spectrum and a
// Krylov method cannot stall on it), with N:
//   features X0 = F r = (r, sigma r): 8 channels, adapted to sigma;
//   layers Y[o, n] = sum_k sum_i W[k][i][o] s_k(n) X[i, nb_k(n)] over the 3x3
//   taps k = (dt + 1) * 3 + (dx + 1), s_k(n) = -1 when t + dt wraps
//   (antiperiodic time, as the fermion fields); no activation;
//   channels 8 -> 8 -> ... -> 8 -> 4;
// and N^T the same layers transposed in reverse order, then F^T (a, b) =
// a + sigma b.  Each weight serves twice (in N and in N^T).
// Activations are channel-major float arrays [C][V]; the residual and the
// output are site-major (4 floats per site, the layout of the CG vectors).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

namespace {

constexpr int kNetThreads = 256;
constexpr int kPcgMaxConv = 16;   // the persistent PCG's convolutions per iteration (2L)
constexpr int kNetC = 8;          // feature and hidden channels
constexpr int kNetOut = 4;        // output channels (spinor components)
constexpr int kWTile = 64;        // sites per shared-memory tile of the weight gradient

struct TapSite {
    int m;      // neighbour site
    float s;    // boundary sign
};

// the site at tap k of n = t * Nx + x, with its antiperiodic sign
__device__ __forceinline__ TapSite tap_site(int t, int x, int k, int Nt, int Nx)
{
    const int dt = k / 3 - 1, dx = k % 3 - 1;
    int tt = t + dt;
    float s = 1.f;
    if (tt < 0) {
        tt += Nt;
        s = -1.f;
    } else if (tt >= Nt) {
        tt -= Nt;
        s = -1.f;
    }
    int xx = x + dx;
    if (xx < 0) xx += Nx;
    else if (xx >= Nx) xx -= Nx;
    return TapSite{tt * Nx + xx, s};
}

__global__ void __launch_bounds__(kNetThreads) net_features_kernel(const float* __restrict__ r,
                                                                   const double* __restrict__ sigma,
                                                                   float* __restrict__ X, int V)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const float4 v = reinterpret_cast<const float4*>(r)[n];
        const float sg = (float)sigma[n];
        X[0 * V + n] = v.x;
        X[1 * V + n] = v.y;
        X[2 * V + n] = v.z;
        X[3 * V + n] = v.w;
        X[4 * V + n] = sg * v.x;
        X[5 * V + n] = sg * v.y;
        X[6 * V + n] = sg * v.z;
        X[7 * V + n] = sg * v.w;
    }
}

// X (8 channels) = F g = (g, sigma g) for a channel-major 4-channel g
__global__ void __launch_bounds__(kNetThreads) net_feat_cm_kernel(const float* __restrict__ g,
                                                                  const double* __restrict__ sigma,
                                                                  float* __restrict__ X, int V)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const float sg = (float)sigma[n];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float v = g[c * V + n];
            X[c * V + n] = v;
            X[(4 + c) * V + n] = sg * v;
        }
    }
}

// z (site-major) = F^T a + skip r = a[0..3] + sigma a[4..7] + skip r
__global__ void __launch_bounds__(kNetThreads) net_featT_kernel(const float* __restrict__ a,
                                                                const double* __restrict__ sigma,
                                                                const float* __restrict__ r, float skip,
                                                                float* __restrict__ z, int V)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const float sg = (float)sigma[n];
        const float4 rv = reinterpret_cast<const float4*>(r)[n];
        float4 o;
        o.x = fmaf(sg, a[4 * V + n], a[0 * V + n]) + skip * rv.x;
        o.y = fmaf(sg, a[5 * V + n], a[1 * V + n]) + skip * rv.y;
        o.z = fmaf(sg, a[6 * V + n], a[2 * V + n]) + skip * rv.z;
        o.w = fmaf(sg, a[7 * V + n], a[3 * V + n]) + skip * rv.w;
        reinterpret_cast<float4*>(z)[n] = o;
    }
}

// Y[COUT][V] = conv(X[8][V]); the last layer (COUT = 4) may write site-major.
template <int COUT, bool SITE_OUT>
__global__ void __launch_bounds__(kNetThreads) net_conv_fwd_kernel(const float* __restrict__ X, float* __restrict__ Y,
                                                                   const float* __restrict__ Wl, int Nt, int Nx)
{
    __shared__ float w[9 * kNetC * COUT];
    for (int i = threadIdx.x; i < 9 * kNetC * COUT; i += blockDim.x) w[i] = Wl[i];
    __syncthreads();
    const int V = Nt * Nx;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const int t = n / Nx, x = n - t * Nx;
        float acc[COUT];
#pragma unroll
        for (int o = 0; o < COUT; ++o) acc[o] = 0.f;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const TapSite q = tap_site(t, x, k, Nt, Nx);
#pragma unroll
            for (int i = 0; i < kNetC; ++i) {
                const float xv = q.s * X[i * V + q.m];
#pragma unroll
                for (int o = 0; o < COUT; ++o) acc[o] = fmaf(w[(k * kNetC + i) * COUT + o], xv, acc[o]);
            }
        }
        if constexpr (SITE_OUT) {
            reinterpret_cast<float4*>(Y)[n] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        } else {
#pragma unroll
            for (int o = 0; o < COUT; ++o) Y[o * V + n] = acc[o];
        }
    }
}

// gX[8][V] = conv^T(gY[COUT][V]): the transpose of a tap is the opposite tap
// with the same sign (a wrap from n to m by +d is a wrap from m to n by -d).
template <int COUT>
__global__ void __launch_bounds__(kNetThreads) net_conv_bwd_in_kernel(const float* __restrict__ gY,
                                                                      float* __restrict__ gX,
                                                                      const float* __restrict__ Wl, int Nt, int Nx)
{
    __shared__ float w[9 * kNetC * COUT];
    for (int i = threadIdx.x; i < 9 * kNetC * COUT; i += blockDim.x) w[i] = Wl[i];
    __syncthreads();
    const int V = Nt * Nx;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < V; m += gridDim.x * blockDim.x) {
        const int t = m / Nx, x = m - t * Nx;
        float acc[kNetC];
#pragma unroll
        for (int i = 0; i < kNetC; ++i) acc[i] = 0.f;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const TapSite q = tap_site(t, x, 8 - k, Nt, Nx);   // the opposite tap
            float g[COUT];
#pragma unroll
            for (int o = 0; o < COUT; ++o) g[o] = q.s * gY[o * V + q.m];
#pragma unroll
            for (int i = 0; i < kNetC; ++i)
#pragma unroll
                for (int o = 0; o < COUT; ++o) acc[i] = fmaf(w[(k * kNetC + i) * COUT + o], g[o], acc[i]);
        }
#pragma unroll
        for (int i = 0; i < kNetC; ++i) gX[i * V + m] = acc[i];
    }
}

// Per-block partial weight gradients of one layer:
// gW[k][i][o] = sum_n s_k(n) X[i, nb_k(n)] gY[o, n], a [72 x V] x [V x COUT]
// product staged through shared memory tiles of kWTile sites.  gY may be
// site-major (the output layer's gradient).
template <int COUT, bool SITE_GY>
__global__ void __launch_bounds__(kNetThreads) net_conv_bwd_w_kernel(const float* __restrict__ X,
                                                                     const float* __restrict__ gY,
                                                                     float* __restrict__ part, int Nt, int Nx)
{
    constexpr int NW = 9 * kNetC * COUT;
    constexpr int PER = (NW + kNetThreads - 1) / kNetThreads;
    __shared__ float nb[kWTile][9 * kNetC + 1];
    __shared__ float gy[kWTile][COUT];
    const int V = Nt * Nx;
    float acc[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) acc[j] = 0.f;
    for (int base = blockIdx.x * kWTile; base < V; base += gridDim.x * kWTile) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < kWTile * 9; idx += blockDim.x) {
            const int ts = idx / 9, k = idx - ts * 9, n = base + ts;
            if (n < V) {
                const int t = n / Nx, x = n - t * Nx;
                const TapSite q = tap_site(t, x, k, Nt, Nx);
#pragma unroll
                for (int i = 0; i < kNetC; ++i) nb[ts][k * kNetC + i] = q.s * X[i * V + q.m];
            } else {
#pragma unroll
                for (int i = 0; i < kNetC; ++i) nb[ts][k * kNetC + i] = 0.f;
            }
        }
        for (int idx = threadIdx.x; idx < kWTile * COUT; idx += blockDim.x) {
            const int ts = idx / COUT, o = idx - ts * COUT, n = base + ts;
            gy[ts][o] = n < V ? (SITE_GY ? gY[(size_t)n * COUT + o] : gY[o * V + n]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int wi = threadIdx.x + j * kNetThreads;
            if (wi < NW) {
                const int kk = wi / COUT, o = wi - kk * COUT;
                float a = acc[j];
                for (int ts = 0; ts < kWTile; ++ts) a = fmaf(nb[ts][kk], gy[ts][o], a);
                acc[j] = a;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int wi = threadIdx.x + j * kNetThreads;
        if (wi < NW) part[(size_t)blockIdx.x * NW + wi] = acc[j];
    }
}

// g[i] += sum over blocks of part[b][i], in block order (deterministic)
__global__ void net_reduce_w_kernel(const float* __restrict__ part, int nblocks, int nw, float* __restrict__ g)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * nw + i];
        g[i] += s;
    }
}

// d = z - e (site-major)
__global__ void net_diff_kernel(const float* __restrict__ z, const float* __restrict__ e, float* __restrict__ d, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = z[i] - e[i];
}

// gZ (channel-major [4][V]) = 2 u (site-major)
__global__ void net_gz_kernel(const float* __restrict__ u, float* __restrict__ gz, int V)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * V; i += gridDim.x * blockDim.x)
        gz[(i & 3) * V + (i >> 2)] = 2.f * u[i];
}

__global__ void net_adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int nw, float lr, float c1, float c2, float gscale)
{
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) {
        const float gi = g[i] * gscale;
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// ---- vectors of the flexible solver (4V floats or doubles, site-major) ----

// per-block partial sums of a . b (products in FP32, sums in FP64)
__global__ void __launch_bounds__(kNetThreads) fvec_dot_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                                               double* __restrict__ part, int n)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s = fma((double)a[i], (double)b[i], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kNetThreads) dvec_dot_kernel(const double* __restrict__ a,
                                                               const double* __restrict__ b,
                                                               double* __restrict__ part, int n)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s = fma(a[i], b[i], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// y += a x
__global__ void fvec_axpy_kernel(float* __restrict__ y, const float* __restrict__ x, float a, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = fmaf(a, x[i], y[i]);
}

// r = b - t (FP64) and its float copy
__global__ void dvec_residual_kernel(const double* __restrict__ b, const double* __restrict__ t, double* __restrict__ r,
                                     float* __restrict__ rf, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = b[i] - t[i];
        r[i] = v;
        rf[i] = (float)v;
    }
}

// out = (float) a
__global__ void dvec_to_f_kernel(const double* __restrict__ a, float* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = (float)a[i];
}

// x += d (FP64 from FP32)
__global__ void dvec_add_f_kernel(double* __restrict__ x, const float* __restrict__ d, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += (double)d[i];
}

// ---- tensor-core convolutions of the solvers' preconditioner ----
//
// The solvers apply M through BF16 activations, site-major: the 8 channels
// of a site are 16 bytes (uint4).  Two 3x3 taps of an 8 -> 8 layer are one
// [16 sites x 16] x [16 x 8 out] product, one mma.sync m16n8k16 with BF16
// inputs and FP32 accumulation (K = tap A's 8 channels, then tap B's), so a
// layer is 5 of them per 16 sites (the fifth pairs tap 8 with zeros).  A
// block stages its R x W tile with a one-site halo in shared memory by 16-byte
// asynchronous copies; lane (g = lane / 4, c = lane % 4) then gathers the
// 32-bit word c (channels 2c, 2c + 1) of the tap neighbours of sites g and
// g + 8 (the A fragment: 8 sites x 4 words = 32 distinct banks) and holds the
// weights as B fragments in registers.  The 4-channel activations (the output
// of N, the input of N^T) keep 8 channels, 4 of them zero.  BF16 keeps 8
// mantissa bits: M(r) is then a slightly perturbed operator, which the
// flexible CG's Polak-Ribiere beta absorbs.  Training and yk_net_apply use the
// exact FP32 kernels above.

constexpr int kTcMaxR = 8, kTcMaxW = 64;
constexpr int kTcSW = kTcMaxW + 2;   // staged sites per tile row

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Programmatic dependent launch: the kernels of a PCG iteration are launched
// with programmatic stream serialisation, so a kernel's launch and its
// independent prologue overlap the previous kernel's tail.  pdl_wait() comes
// before the first access to memory an earlier kernel of the chain reads or
// writes (it returns once that kernel has completed and its writes are
// visible; without a programmatic dependency it returns at once);
// pdl_trigger() after a block's main work lets the next kernel launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ float2 unpack_bf2(uint32_t w)
{
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// FP32 copy of the field (the preconditioner's features)
__global__ void f_of_d_kernel(const double* __restrict__ a, float* __restrict__ out, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = (float)a[i];
}

// the 8 BF16 channels (r, sigma r) of a site
__device__ __forceinline__ uint4 features_bf(float4 v, float sg)
{
    return make_uint4(pack_bf2(v.x, v.y), pack_bf2(v.z, v.w), pack_bf2(sg * v.x, sg * v.y), pack_bf2(sg * v.z, sg * v.w));
}

// X = F r (BF16, site-major)
__global__ void __launch_bounds__(kNetThreads) net_feat_bf_kernel(const float* __restrict__ r,
                                                                  const float* __restrict__ sigma,
                                                                  uint4* __restrict__ X, int V)
{
    pdl_wait();
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x)
        X[n] = features_bf(reinterpret_cast<const float4*>(r)[n], sigma[n]);
    pdl_trigger();
}

// F^T a + skip r for the BF16 site-major a
__device__ __forceinline__ float4 featT_bf(uint4 a, float sg, float4 rv, float skip)
{
    const float2 a01 = unpack_bf2(a.x), a23 = unpack_bf2(a.y), a45 = unpack_bf2(a.z), a67 = unpack_bf2(a.w);
    return make_float4(fmaf(sg, a45.x, a01.x) + skip * rv.x, fmaf(sg, a45.y, a01.y) + skip * rv.y,
                       fmaf(sg, a67.x, a23.x) + skip * rv.z, fmaf(sg, a67.y, a23.y) + skip * rv.w);
}

__global__ void __launch_bounds__(kNetThreads) net_featT_bf_kernel(const uint4* __restrict__ a,
                                                                   const float* __restrict__ sigma,
                                                                   const float* __restrict__ r, float skip,
                                                                   float* __restrict__ z, int V)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x)
        reinterpret_cast<float4*>(z)[n] = featT_bf(a[n], sigma[n], reinterpret_cast<const float4*>(r)[n], skip);
}

// TRANS = false: Y = conv(X) (a layer of N, 8 -> COUT channels);
// TRANS = true: Y = conv^T(X) (its transpose in N^T, COUT -> 8: the opposite
// tap, the same sign, W[k] transposed).  X, Y: BF16 site-major, 8 channels.
// The layer on the tiles blockIdx.x, blockIdx.x + gridDim.x, ... (PDL: the
// kernel form, one tile per block, with its programmatic-launch wait and
// trigger; else the persistent PCG's form, tiles in turn).
template <int COUT, bool TRANS, bool PDL>
__device__ __forceinline__ void conv_bf_tiles(const uint4* __restrict__ X, uint4* __restrict__ Y,
                                              const float* __restrict__ Wl, int Nt, int Nx, int R, int W, uint4* sm)
{
    constexpr int SW = kTcSW;   // sm: (kTcMaxR + 2) x kTcSW staged sites
    const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
    const int tiles_x = (Nx + W - 1) / W;
    const int ntiles = ((Nt + R - 1) / R) * tiles_x;
    // B fragments of the tap pairs (2p, 2p + 1): K = the pair's 16 inputs, N = 8 outputs
    uint32_t b0[5], b1[5];
#pragma unroll
    for (int p = 0; p < 5; ++p) {
        float w[4] = {0.f, 0.f, 0.f, 0.f};   // B[2c][g], B[2c + 1][g], B[2c + 8][g], B[2c + 9][g]
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * p + h;
            if (k > 8) continue;
            if (!TRANS) {   // B[i][o] = W[k][i][o]
                if (g < COUT) {
                    w[2 * h] = Wl[(k * kNetC + 2 * c) * COUT + g];
                    w[2 * h + 1] = Wl[(k * kNetC + 2 * c + 1) * COUT + g];
                }
            } else {        // B[o][i] = W[k][i][o]
                if (2 * c + 1 < COUT) {
                    w[2 * h] = Wl[(k * kNetC + g) * COUT + 2 * c];
                    w[2 * h + 1] = Wl[(k * kNetC + g) * COUT + 2 * c + 1];
                }
            }
        }
        b0[p] = pack_bf2(w[0], w[1]);
        b1[p] = pack_bf2(w[2], w[3]);
    }
    if (PDL) pdl_wait();   // the weights above are constant during a solve; X is the previous layer's
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (tile != (int)blockIdx.x) __syncthreads();   // the previous tile's reads of sm are done
    const int t0 = (tile / tiles_x) * R, x0 = (tile % tiles_x) * W;
    const int Rt = min(R, Nt - t0), Wt = min(W, Nx - x0);
    // stage the tile and its halo: warp w takes the staged rows w, w + 8
    for (int lr = threadIdx.x >> 5; lr < Rt + 2; lr += kNetThreads / 32) {
        int t = t0 - 1 + lr;
        if (t < 0) t += Nt;
        else if (t >= Nt) t -= Nt;
        const uint4* src = X + (size_t)t * Nx;
        for (int lc = lane; lc < Wt + 2; lc += 32) {
            int x = x0 - 1 + lc;
            if (x < 0) x += Nx;
            else if (x >= Nx) x -= Nx;
            cp_async16(&sm[lr * SW + lc], src + x);
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // the antiperiodic sign of halo rows that wrapped in time (BF16 sign bits)
    const bool top = t0 == 0, bottom = t0 + Rt == Nt;
    if (top || bottom) {
        uint32_t* w32 = reinterpret_cast<uint32_t*>(sm);
        for (int idx = threadIdx.x; idx < 2 * (Wt + 2) * 4; idx += blockDim.x) {
            const int which = idx / ((Wt + 2) * 4), rem = idx - which * (Wt + 2) * 4;
            if (which == 0 ? top : bottom) w32[((which == 0 ? 0 : Rt + 1) * SW) * 4 + rem] ^= 0x80008000u;
        }
        __syncthreads();
    }
    const uint32_t* smw = reinterpret_cast<const uint32_t*>(sm);
    uint32_t* Yw = reinterpret_cast<uint32_t*>(Y);
    const int S = Rt * Wt;
    for (int base = (threadIdx.x >> 5) * 16; base < S; base += (blockDim.x >> 5) * 16) {
        const int i0 = base + g, i1 = base + g + 8;
        const bool in0 = i0 < S, in1 = i1 < S;
        const int r0 = in0 ? i0 / Wt : 0, c0 = in0 ? i0 - r0 * Wt : 0;
        const int r1 = in1 ? i1 / Wt : 0, c1 = in1 ? i1 - r1 * Wt : 0;
        // word c of the sites' centres in the staged tile
        const uint32_t* q0 = smw + ((r0 + 1) * SW + c0 + 1) * 4 + c;
        const uint32_t* q1 = smw + ((r1 + 1) * SW + c1 + 1) * 4 + c;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int p = 0; p < 5; ++p) {
            const int kA = TRANS ? 8 - 2 * p : 2 * p;   // gathered taps
            const int kB = TRANS ? 7 - 2 * p : 2 * p + 1;
            const int offA = ((kA / 3 - 1) * SW + (kA % 3 - 1)) * 4;
            const int offB = ((kB / 3 - 1) * SW + (kB % 3 - 1)) * 4;
            uint32_t a[4];
            a[0] = q0[offA];
            a[1] = q1[offA];
            a[2] = p < 4 ? q0[offB] : 0u;
            a[3] = p < 4 ? q1[offB] : 0u;
            mma_bf16(acc, a, b0[p], b1[p]);
        }
        // D fragment: rows g, g + 8 (sites), columns 2c, 2c + 1 (output channels)
        const int n0 = (t0 + r0) * Nx + x0 + c0, n1 = (t0 + r1) * Nx + x0 + c1;
        if (in0) Yw[(size_t)n0 * 4 + c] = pack_bf2(acc[0], acc[1]);
        if (in1) Yw[(size_t)n1 * 4 + c] = pack_bf2(acc[2], acc[3]);
    }
    }
    if (PDL) pdl_trigger();
}

template <int COUT, bool TRANS>
__global__ void __launch_bounds__(kNetThreads) net_conv_bf_kernel(const uint4* __restrict__ X, uint4* __restrict__ Y,
                                                                  const float* __restrict__ Wl, int Nt, int Nx,
                                                                  int R, int W)
{
    __shared__ __align__(16) uint4 sm[(kTcMaxR + 2) * kTcSW];
    conv_bf_tiles<COUT, TRANS, true>(X, Y, Wl, Nt, Nx, R, W, sm);
}

// Several layers in one launch.  A block stages its R x W tile with a halo
// of H sites (H = the layers it runs) and computes layer j on the tile
// widened by H - 1 - j sites, in shared memory, so that only the last layer
// writes to global memory.  Time is treated as the antiperiodically extended
// field: a staged row at virtual time t_v takes the sign (-1)^floor(t_v / Nt)
// and every tap after that is a plain shift (a convolution commutes with the
// extension), so rows that wrap more than once are right too.  Each layer's
// taps, weights and channel counts follow net_conv_bf_kernel.
constexpr int kFuseMax = 8;   // layers of one fused launch
constexpr size_t kFusedMaxSmem = 160 * 1024;   // its shared memory (two regions of the widened tile)
struct FusedLayers {
    const float* w[kFuseMax];   // weights of each layer
    int cout[kFuseMax];         // its output channels (8 or 4) in the forward direction
    int trans[kFuseMax];        // 1: the transposed layer
    int n;                      // layers in this launch (= the halo H)
};

__host__ __device__ inline int fused_region(int R, int W, int H) { return (R + 2 * H) * (W + 2 * H); }

__global__ void __launch_bounds__(kNetThreads) net_conv_fused_kernel(const uint4* __restrict__ X,
                                                                     uint4* __restrict__ Y, FusedLayers L, int Nt,
                                                                     int Nx, int R, int W)
{
    extern __shared__ __align__(16) uint4 fsm[];
    pdl_wait();
    const int H = L.n;
    const int cap = fused_region(R, W, H);
    uint4* bufA = fsm;
    uint4* bufB = fsm + cap;
    const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
    const int tiles_x = (Nx + W - 1) / W;
    const int t0 = (blockIdx.x / tiles_x) * R, x0 = (blockIdx.x % tiles_x) * W;
    const int Rt = min(R, Nt - t0), Wt = min(W, Nx - x0);
    // stage the tile with its halo of H sites (virtual rows carry the
    // antiperiodic sign; columns wrap periodically)
    {
        const int SR = Rt + 2 * H, SC = Wt + 2 * H;
        for (int lr = threadIdx.x >> 5; lr < SR; lr += kNetThreads / 32) {
            const int tv = t0 - H + lr;
            const int k = tv >= 0 ? tv / Nt : -((-tv + Nt - 1) / Nt);   // floor(tv / Nt)
            const int t = tv - k * Nt;
            const uint4* src = X + (size_t)t * Nx;
            for (int lc = lane; lc < SC; lc += 32) {
                int x = (x0 - H + lc) % Nx;
                if (x < 0) x += Nx;
                cp_async16(&bufA[lr * SC + lc], src + x);
            }
        }
        cp_async_wait_all();
        __syncthreads();
        uint32_t* w32 = reinterpret_cast<uint32_t*>(bufA);
        for (int idx = threadIdx.x; idx < SR * SC * 4; idx += blockDim.x) {
            const int tv = t0 - H + idx / (SC * 4);
            const int k = tv >= 0 ? tv / Nt : -((-tv + Nt - 1) / Nt);
            if (k & 1) w32[idx] ^= 0x80008000u;
        }
        __syncthreads();
    }
    uint4* in = bufA;
    uint4* out = bufB;
    for (int j = 0; j < H; ++j) {
        const int hin = H - j, hout = H - 1 - j;   // halo of this layer's input and output regions
        const int SWi = Wt + 2 * hin;              // input row stride (sites)
        const int RO = Rt + 2 * hout, WO = Wt + 2 * hout;
        const bool tr = L.trans[j] != 0;
        const int co = L.cout[j];
        const float* Wl = L.w[j];
        uint32_t b0[5], b1[5];
#pragma unroll
        for (int p = 0; p < 5; ++p) {
            float w[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = 2 * p + h;
                if (k > 8) continue;
                if (!tr) {
                    if (g < co) {
                        w[2 * h] = Wl[(k * kNetC + 2 * c) * co + g];
                        w[2 * h + 1] = Wl[(k * kNetC + 2 * c + 1) * co + g];
                    }
                } else if (2 * c + 1 < co) {
                    w[2 * h] = Wl[(k * kNetC + g) * co + 2 * c];
                    w[2 * h + 1] = Wl[(k * kNetC + g) * co + 2 * c + 1];
                }
            }
            b0[p] = pack_bf2(w[0], w[1]);
            b1[p] = pack_bf2(w[2], w[3]);
        }
        // tap word offsets in the input region, in the order of the products
        int offA[5], offB[5];
#pragma unroll
        for (int p = 0; p < 5; ++p) {
            const int kA = tr ? 8 - 2 * p : 2 * p, kB = tr ? 7 - 2 * p : 2 * p + 1;
            offA[p] = ((kA / 3 - 1) * SWi + (kA % 3 - 1)) * 4;
            offB[p] = p < 4 ? ((kB / 3 - 1) * SWi + (kB % 3 - 1)) * 4 : 0;
        }
        const uint32_t* inw = reinterpret_cast<const uint32_t*>(in);
        const bool last = j == H - 1;
        uint32_t* ow = last ? reinterpret_cast<uint32_t*>(Y) : reinterpret_cast<uint32_t*>(out);
        const int S = RO * WO;
        for (int base = (threadIdx.x >> 5) * 16; base < S; base += (blockDim.x >> 5) * 16) {
            const int i0 = base + g, i1 = base + g + 8;
            const bool in0 = i0 < S, in1 = i1 < S;
            const int r0 = in0 ? i0 / WO : 0, c0 = in0 ? i0 - r0 * WO : 0;
            const int r1 = in1 ? i1 / WO : 0, c1 = in1 ? i1 - r1 * WO : 0;
            const uint32_t* q0 = inw + ((r0 + 1) * SWi + c0 + 1) * 4 + c;
            const uint32_t* q1 = inw + ((r1 + 1) * SWi + c1 + 1) * 4 + c;
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int p = 0; p < 5; ++p) {
                uint32_t a[4];
                a[0] = q0[offA[p]];
                a[1] = q1[offA[p]];
                a[2] = p < 4 ? q0[offB[p]] : 0u;
                a[3] = p < 4 ? q1[offB[p]] : 0u;
                mma_bf16(acc, a, b0[p], b1[p]);
            }
            if (last) {
                const int n0 = (t0 + r0) * Nx + x0 + c0, n1 = (t0 + r1) * Nx + x0 + c1;
                if (in0) ow[(size_t)n0 * 4 + c] = pack_bf2(acc[0], acc[1]);
                if (in1) ow[(size_t)n1 * 4 + c] = pack_bf2(acc[2], acc[3]);
            } else {
                if (in0) ow[(r0 * WO + c0) * 4 + c] = pack_bf2(acc[0], acc[1]);
                if (in1) ow[(r1 * WO + c1) * 4 + c] = pack_bf2(acc[2], acc[3]);
            }
        }
        __syncthreads();
        uint4* tmp = in;
        in = out;
        out = tmp;
    }
}


}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct PcgGraph;
void pcg_graph_destroy(PcgGraph* g);

// the inner tolerance of the preconditioned CG under trial: solves counted,
// milliseconds of the trial solves, the choice (-1: still trying)
struct InnerChoice {
    int tried = 0;
    double ms[2] = {0.0, 0.0};
    int chosen = -1;
};

struct LearnedNet {
    int Nt = 0, Nx = 0, V = 0, layers = 0, nw = 0, nblk = 0, grid = 0;
    int tc_R = 8, tc_W = 64;          // tile of the tensor-core convolutions (rows x columns)
    int tc_G = 1;                     // layers per launch (1: one launch per layer)
    bool tc_tuned = false;            // tile chosen by timing (first solve) or by YK_NET_TILE
    InnerChoice inner[2];             // the PCG's inner tolerance (identity, network), chosen by timing
    float* sig32 = nullptr;           // FP32 copy of the field of the current solve
    float* diag32 = nullptr;          // FP32 diagonal 2 r + m0 + g sigma of the current solve
    uint4* h16[2] = {nullptr, nullptr};   // BF16 site-major activations of the solvers' M (ping-pong)
    std::vector<int> woff;            // each layer's first weight
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    float* act = nullptr;             // layers x [8][V]: the input of each layer of N
    float* dec = nullptr;             // (layers + 1) x [8][V]: dec[L] = N r, dec[l] = L_l^T dec[l + 1]
    float* gbuf[2] = {nullptr, nullptr};   // [8][V] input gradients (ping-pong)
    float* gz = nullptr;              // [4][V] output gradient
    float* z = nullptr;               // 4V site-major output
    float* part = nullptr;            // nblk x 576 weight-gradient partials
    double* dpart = nullptr;          // grid doubles of dot partials
    double* hpart = nullptr;          // pinned host copy of dpart
    size_t hpart_cap = 0;             // doubles in dpart and hpart
    int adam_t = 0;
    float skip = 0.f;                 // M(r) = skip r + N(r)
    // training pairs: npairs x (r, e), 4V floats each, scaled to |e| = 1
    float* pairs = nullptr;
    int npairs = 0, pair_cap = 0;
    // FP64 and FP32 scratch of the pair builder and of the solver
    double *d0 = nullptr, *d1 = nullptr, *d2 = nullptr;
    float *f0 = nullptr, *f1 = nullptr, *f2 = nullptr, *f3 = nullptr;
    float* Zs = nullptr;              // restart x 4V: preconditioned directions
    float* Ws = nullptr;              // restart x 4V: their images under A
    int restart = 0;
    PcgGraph* pcg = nullptr;          // its captured chunk of iterations
    bool pcg_no_graph = false;        // capture failed once (e.g. the legacy stream)
    bool persistent = false;          // chunks of iterations as one cooperative launch (grid <= co-resident)
    unsigned* pbar = nullptr;         // its barrier counter and error word
};

namespace {

int pcg_chunk_max_grid();

int cout_of(const LearnedNet* n, int l) { return l == n->layers - 1 ? kNetOut : kNetC; }

cudaError_t alloc_f(float** p, size_t n) { return cudaMalloc(p, sizeof(float) * (n ? n : 1)); }
cudaError_t alloc_d(double** p, size_t n) { return cudaMalloc(p, sizeof(double) * (n ? n : 1)); }

// sum of the dot partials of the last dot launch (in block order)
cudaError_t host_sum(LearnedNet* n, cudaStream_t s, double* out)
{
    cudaError_t e = cudaMemcpyAsync(n->hpart, n->dpart, sizeof(double) * n->grid, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    double t = 0.0;
    for (int i = 0; i < n->grid; ++i) t += n->hpart[i];
    *out = t;
    return e;
}

}  // namespace

namespace {

using DiracArgs = NetOp;

// out = D^dag D in (K = 1), FP64 or FP32 (tmp: scratch of the same type)
cudaError_t apply_A(const DiracArgs& d, const void* in, void* tmp, void* out, int prec, cudaStream_t s)
{
    cudaError_t e = launch_dirac(in, tmp, d.sigma, d.Nt, d.Nx, d.m0, d.g, d.r, 0, prec, 1, s);
    if (e == cudaSuccess) e = launch_dirac(tmp, out, d.sigma, d.Nt, d.Nx, d.m0, d.g, d.r, 1, prec, 1, s);
    return e;
}

cudaError_t ensure_scratch(LearnedNet* n, int restart)
{
    const size_t V4 = 4 * (size_t)n->V;
    cudaError_t e = cudaSuccess;
    if (!n->d0) e = alloc_d(&n->d0, V4);
    if (e == cudaSuccess && !n->d1) e = alloc_d(&n->d1, V4);
    if (e == cudaSuccess && !n->d2) e = alloc_d(&n->d2, V4);
    if (e == cudaSuccess && !n->f0) e = alloc_f(&n->f0, V4);
    if (e == cudaSuccess && !n->f1) e = alloc_f(&n->f1, V4);
    if (e == cudaSuccess && !n->f2) e = alloc_f(&n->f2, V4);
    if (e == cudaSuccess && !n->f3) e = alloc_f(&n->f3, V4);
    if (e == cudaSuccess && restart > n->restart) {
        if (n->Zs) cudaFree(n->Zs);
        if (n->Ws) cudaFree(n->Ws);
        n->Zs = n->Ws = nullptr;
        e = alloc_f(&n->Zs, (size_t)restart * V4);
        if (e == cudaSuccess) e = alloc_f(&n->Ws, (size_t)restart * V4);
        n->restart = e == cudaSuccess ? restart : 0;
    }
    return e;
}

cudaError_t dot_f(LearnedNet* n, const float* a, const float* b, cudaStream_t s, double* out)
{
    fvec_dot_kernel<<<n->grid, kNetThreads, 0, s>>>(a, b, n->dpart, 4 * n->V);
    return host_sum(n, s, out);
}

cudaError_t dot_d(LearnedNet* n, const double* a, const double* b, cudaStream_t s, double* out)
{
    dvec_dot_kernel<<<n->grid, kNetThreads, 0, s>>>(a, b, n->dpart, 4 * n->V);
    return host_sum(n, s, out);
}

}  // namespace

void net_destroy(LearnedNet* n)
{
    if (!n) return;
    float* fs[] = {n->w, n->g, n->m, n->v, n->act, n->dec, n->gbuf[0], n->gbuf[1], n->gz, n->z, n->part, n->pairs,
                   n->f0, n->f1, n->f2, n->f3, n->Zs, n->Ws, n->sig32, n->diag32};
    for (float* p : fs)
        if (p) cudaFree(p);
    double* ds[] = {n->dpart, n->d0, n->d1, n->d2};
    for (double* p : ds)
        if (p) cudaFree(p);
    if (n->hpart) cudaFreeHost(n->hpart);
    if (n->pbar) cudaFree(n->pbar);
    pcg_graph_destroy(n->pcg);
    for (uint4* h : n->h16)
        if (h) cudaFree(h);
    delete n;
}

int net_size(const LearnedNet* n) { return n->nw; }

void net_tile(const LearnedNet* n, int* rows, int* cols, int* per_launch)
{
    *rows = n->tc_tuned ? n->tc_R : 0;
    *cols = n->tc_tuned ? n->tc_W : 0;
    *per_launch = n->tc_tuned ? n->tc_G : 0;
}

bool net_tile_from_env(LearnedNet* n);

void net_set_skip(LearnedNet* n, float skip) { n->skip = skip; }

LearnedNet* net_create(int Nt, int Nx, int layers, cudaError_t* err)
{
    LearnedNet* n = new LearnedNet();
    n->Nt = Nt;
    n->Nx = Nx;
    n->V = Nt * Nx;
    n->layers = layers;
    for (int l = 0; l < layers; ++l) {
        n->woff.push_back(n->nw);
        n->nw += 9 * kNetC * cout_of(n, l);
    }
    const size_t V = (size_t)n->V;
    n->grid = (int)std::min<size_t>((V + kNetThreads - 1) / kNetThreads, 4096);
    // YK_PCG_PERSISTENT=k (opt-in): the PCG chunk as one cooperative launch
    // of at most k blocks per SM, grid barriers between its phases.  Off by
    // default: at 512 x 512 its barriers cost more than the PDL launch
    // boundaries they replace (2-layer network 151 against 178 steps/s).
    const char* pe = getenv("YK_PCG_PERSISTENT");
    const int pk = pe ? atoi(pe) : 0;
    int pg = pk > 0 ? pcg_chunk_max_grid() : 0;
    if (pg > 0 && 2 * layers <= kPcgMaxConv) {
        int dev0 = 0, nsm0 = 0;
        cudaGetDevice(&dev0);
        cudaDeviceGetAttribute(&nsm0, cudaDevAttrMultiProcessorCount, dev0);
        pg = std::min(pg, pk * nsm0);
        n->grid = std::min(n->grid, pg);
        n->persistent = true;
    }
    n->nblk = (int)std::min<size_t>((V + kWTile - 1) / kWTile, 512);
    // convolution tiles: 64 columns (or the whole row), rows halved from 8
    // while there are fewer than two tiles per SM
    int dev = 0, n_sm = 148;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    n->tc_W = std::min(Nx, kTcMaxW);
    n->tc_R = kTcMaxR;
    cudaFuncSetAttribute((const void*)net_conv_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kFusedMaxSmem);
    while (n->tc_R > 2 && (int64_t)((Nt + n->tc_R - 1) / n->tc_R) * ((Nx + n->tc_W - 1) / n->tc_W) < 2 * n_sm)
        n->tc_R /= 2;
    cudaError_t e = alloc_f(&n->w, n->nw);
    if (e == cudaSuccess) e = alloc_f(&n->g, n->nw);
    if (e == cudaSuccess) e = alloc_f(&n->m, n->nw);
    if (e == cudaSuccess) e = alloc_f(&n->v, n->nw);
    if (e == cudaSuccess) e = alloc_f(&n->act, (size_t)layers * kNetC * V);
    if (e == cudaSuccess) e = alloc_f(&n->dec, (size_t)(layers + 1) * kNetC * V);
    if (e == cudaSuccess) e = alloc_f(&n->gbuf[0], kNetC * V);
    if (e == cudaSuccess) e = alloc_f(&n->gbuf[1], kNetC * V);
    if (e == cudaSuccess) e = alloc_f(&n->gz, kNetOut * V);
    if (e == cudaSuccess) e = alloc_f(&n->z, 4 * V);
    if (e == cudaSuccess) e = alloc_f(&n->part, (size_t)n->nblk * 9 * kNetC * kNetC);
    if (e == cudaSuccess) e = alloc_d(&n->dpart, n->grid);
    if (e == cudaSuccess) e = alloc_f(&n->sig32, V);
    if (e == cudaSuccess) e = alloc_f(&n->diag32, V);
    if (e == cudaSuccess) e = cudaMalloc(&n->h16[0], sizeof(uint4) * V);
    if (e == cudaSuccess) e = cudaMalloc(&n->h16[1], sizeof(uint4) * V);
    if (e == cudaSuccess) e = cudaMallocHost(&n->hpart, sizeof(double) * n->grid);
    if (e == cudaSuccess) e = cudaMalloc(&n->pbar, 2 * sizeof(unsigned));
    if (e == cudaSuccess) n->hpart_cap = (size_t)n->grid;
    if (e == cudaSuccess) e = cudaMemset(n->m, 0, sizeof(float) * n->nw);
    if (e == cudaSuccess) e = cudaMemset(n->v, 0, sizeof(float) * n->nw);
    if (e == cudaSuccess) e = cudaMemset(n->g, 0, sizeof(float) * n->nw);
    if (e != cudaSuccess) {
        net_destroy(n);
        n = nullptr;
    } else {
        net_tile_from_env(n);
    }
    *err = e;
    return n;
}

cudaError_t net_weights(LearnedNet* n, float* host, bool set)
{
    if (set) {
        n->inner[1] = InnerChoice();
        n->adam_t = 0;
        cudaError_t e = cudaMemset(n->m, 0, sizeof(float) * n->nw);
        if (e == cudaSuccess) e = cudaMemset(n->v, 0, sizeof(float) * n->nw);
        if (e == cudaSuccess) e = cudaMemcpy(n->w, host, sizeof(float) * n->nw, cudaMemcpyHostToDevice);
        return e;
    }
    return cudaMemcpy(host, n->w, sizeof(float) * n->nw, cudaMemcpyDeviceToHost);
}

// z = M(r): r, z 4V floats site-major; sigma the chain's field
namespace {

// conv of layer l (8 -> cout_l channels)
void conv_fwd(LearnedNet* n, int l, const float* X, float* Y, cudaStream_t s)
{
    if (cout_of(n, l) == kNetOut)
        net_conv_fwd_kernel<kNetOut, false><<<n->grid, kNetThreads, 0, s>>>(X, Y, n->w + n->woff[l], n->Nt, n->Nx);
    else
        net_conv_fwd_kernel<kNetC, false><<<n->grid, kNetThreads, 0, s>>>(X, Y, n->w + n->woff[l], n->Nt, n->Nx);
}

// transposed conv of layer l (cout_l -> 8 channels)
void conv_T(LearnedNet* n, int l, const float* Y, float* X, cudaStream_t s)
{
    if (cout_of(n, l) == kNetOut)
        net_conv_bwd_in_kernel<kNetOut><<<n->grid, kNetThreads, 0, s>>>(Y, X, n->w + n->woff[l], n->Nt, n->Nx);
    else
        net_conv_bwd_in_kernel<kNetC><<<n->grid, kNetThreads, 0, s>>>(Y, X, n->w + n->woff[l], n->Nt, n->Nx);
}

// g[layer l] += sum_n s_k(n) X[i, nb_k(n)] Y[o, n]  (X 8 channels, Y cout_l)
void conv_wgrad(LearnedNet* n, int l, const float* X, const float* Y, cudaStream_t s)
{
    const int co = cout_of(n, l);
    if (co == kNetOut)
        net_conv_bwd_w_kernel<kNetOut, false><<<n->nblk, kNetThreads, 0, s>>>(X, Y, n->part, n->Nt, n->Nx);
    else
        net_conv_bwd_w_kernel<kNetC, false><<<n->nblk, kNetThreads, 0, s>>>(X, Y, n->part, n->Nt, n->Nx);
    const int nwl = 9 * kNetC * co;
    net_reduce_w_kernel<<<(nwl + 255) / 256, 256, 0, s>>>(n->part, n->nblk, nwl, n->g + n->woff[l]);
}

float* act_of(LearnedNet* n, int l) { return n->act + (size_t)l * kNetC * n->V; }
float* dec_of(LearnedNet* n, int l) { return n->dec + (size_t)l * kNetC * n->V; }

// N then N^T on the BF16 features in h16[0] (tensor-core convolutions,
// one block per tile); returns the buffer that holds F^T's input
size_t fused_smem(int R, int W, int G) { return 2 * sizeof(uint4) * (size_t)fused_region(R, W, G); }

// Launch with programmatic stream serialisation (the kernel calls pdl_wait()
// before touching its inputs); YK_PDL=0 in the environment: plain launches.
bool pdl_enabled()
{
    static const bool on = [] {
        const char* e = getenv("YK_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

template <typename... K, typename... A>
void launch_pdl(void (*kern)(K...), int grid, size_t smem, cudaStream_t s, A... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kNetThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kern, static_cast<K>(args)...);
}

uint4* net_convs_fast(LearnedNet* n, cudaStream_t s)
{
    const int L = n->layers, Nt = n->Nt, Nx = n->Nx, R = n->tc_R, W = n->tc_W;
    const int grid = ((Nt + R - 1) / R) * ((Nx + W - 1) / W);
    if (n->tc_G > 1) {   // the 2L layers in launches of tc_G
        FusedLayers seq = {};
        int cur = 0;
        auto flush = [&]() {
            if (!seq.n) return;
            launch_pdl(net_conv_fused_kernel, grid, fused_smem(R, W, seq.n), s, (const uint4*)n->h16[cur],
                       n->h16[cur ^ 1], seq, Nt, Nx, R, W);
            cur ^= 1;
            seq.n = 0;
        };
        for (int q = 0; q < 2 * L; ++q) {
            const int l = q < L ? q : 2 * L - 1 - q;
            seq.w[seq.n] = n->w + n->woff[l];
            seq.cout[seq.n] = cout_of(n, l);
            seq.trans[seq.n] = q >= L ? 1 : 0;
            if (++seq.n == n->tc_G) flush();
        }
        flush();
        return n->h16[cur];
    }
    int cur = 0;
    for (int l = 0; l < L; ++l, cur ^= 1) {
        const float* w = n->w + n->woff[l];
        launch_pdl(cout_of(n, l) == kNetOut ? net_conv_bf_kernel<kNetOut, false> : net_conv_bf_kernel<kNetC, false>,
                   grid, 0, s, (const uint4*)n->h16[cur], n->h16[cur ^ 1], w, Nt, Nx, R, W);
    }
    for (int l = L - 1; l >= 0; --l, cur ^= 1) {
        const float* w = n->w + n->woff[l];
        launch_pdl(cout_of(n, l) == kNetOut ? net_conv_bf_kernel<kNetOut, true> : net_conv_bf_kernel<kNetC, true>,
                   grid, 0, s, (const uint4*)n->h16[cur], n->h16[cur ^ 1], w, Nt, Nx, R, W);
    }
    return n->h16[cur];
}

}  // namespace

// z = M(r) = skip r + N^T N r (r, z site-major)
cudaError_t net_forward(LearnedNet* n, const float* r, const double* sigma, float* z, cudaStream_t s)
{
    const int V = n->V, L = n->layers;
    net_features_kernel<<<n->grid, kNetThreads, 0, s>>>(r, sigma, n->act, V);
    for (int l = 0; l < L - 1; ++l) conv_fwd(n, l, act_of(n, l), act_of(n, l + 1), s);
    conv_fwd(n, L - 1, act_of(n, L - 1), dec_of(n, L), s);
    for (int l = L - 1; l >= 0; --l) conv_T(n, l, dec_of(n, l + 1), dec_of(n, l), s);
    net_featT_kernel<<<n->grid, kNetThreads, 0, s>>>(n->dec, sigma, r, n->skip, z, V);
    return cudaGetLastError();
}

// The convolution tile, chosen by timing the network's layers (one warm-up,
// three timed passes on zeroed activations) at each candidate of 16, 32 or 64
// columns (at most Nx) and 2, 4 or 8 rows; the default (8 x 64, rows halved
// while there are fewer than two tiles per SM) is a candidate.
// YK_NET_TILE=RxW or RxWxG in the environment fixes the tile (R in 1..8,
// W in 1..64) and the layers per launch (G in 1..8): true if it did
bool net_tile_from_env(LearnedNet* n)
{
    const char* env = getenv("YK_NET_TILE");
    if (!env) return false;
    int R = 0, W = 0, G = 1;
    const int k = sscanf(env, "%dx%dx%d", &R, &W, &G);
    if (k < 2 || R < 1 || R > kTcMaxR || W < 1 || W > kTcMaxW || G < 1 || G > kFuseMax) return false;
    if (G > 1 && fused_smem(R, std::min(W, n->Nx), G) > kFusedMaxSmem) return false;
    n->tc_R = R;
    n->tc_W = std::min(W, n->Nx);
    n->tc_G = G;
    n->tc_tuned = true;
    return true;
}

// The convolution tile and the layers per launch, chosen by timing the
// network's layers (one warm-up, three timed passes on zeroed activations)
// at each candidate: 16, 32 or 64 columns (at most Nx), 2, 4 or 8 rows, and
// one launch per layer, per half of the network (N, N^T) or for all 2L
// layers (when its shared memory fits).
cudaError_t net_tune_tile(LearnedNet* n, cudaStream_t s)
{
    if (net_tile_from_env(n)) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(n->h16[0], 0, sizeof(uint4) * n->V, s);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    int bestR = n->tc_R, bestW = n->tc_W, bestG = 1;
    float best = -1.f;
    const int Gs[3] = {1, n->layers, 2 * n->layers};
    for (int gi = 0; gi < 3; ++gi) {
        const int G = Gs[gi];
        if (G > kFuseMax || (gi > 0 && Gs[gi] == Gs[gi - 1])) continue;
        for (int W : {64, 32, 16}) {
            if (W > n->Nx && W != 64) continue;
            for (int R : {8, 4, 2}) {
                if (e != cudaSuccess) break;
                const int Wc = std::min(W, n->Nx);
                if (G > 1 && fused_smem(R, Wc, G) > kFusedMaxSmem) continue;
                n->tc_R = R;
                n->tc_W = Wc;
                n->tc_G = G;
                net_convs_fast(n, s);
                e = cudaEventRecord(e0, s);
                for (int rep = 0; rep < 3; ++rep) net_convs_fast(n, s);
                if (e == cudaSuccess) e = cudaEventRecord(e1, s);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e == cudaSuccess && (best < 0.f || ms < best)) {
                    best = ms;
                    bestR = n->tc_R;
                    bestW = n->tc_W;
                    bestG = n->tc_G;
                }
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    n->tc_R = bestR;
    n->tc_W = bestW;
    n->tc_G = bestG;
    n->tc_tuned = e == cudaSuccess;
    return e == cudaSuccess ? cudaGetLastError() : e;
}

// z = M(r) with the tensor-core convolutions (the solvers' preconditioner)
cudaError_t net_forward_fast(LearnedNet* n, const float* r, const double* sigma, float* z, cudaStream_t s)
{
    const int V = n->V;
    f_of_d_kernel<<<n->grid, kNetThreads, 0, s>>>(sigma, n->sig32, V);
    net_feat_bf_kernel<<<n->grid, kNetThreads, 0, s>>>(r, n->sig32, n->h16[0], V);
    const uint4* a = net_convs_fast(n, s);
    net_featT_bf_kernel<<<n->grid, kNetThreads, 0, s>>>(a, n->sig32, r, n->skip, z, V);
    return cudaGetLastError();
}

// The loss of a pair (r, e): the energy norm of the error left by the
// correction M(r), L = (M r - e)^T A (M r - e) = |D (M r - e)|^2 (A = D^dag D;
// the pairs are scaled to e^T A e = 1).  The plain norm |M r - e|^2 would be
// dominated by the smooth, low modes of e and train a network whose output
// never corrects the high modes that dominate the residual.  Leaves
// d = M r - e in f0, D d in f1 and the loss partials in dpart.
cudaError_t net_loss_terms(LearnedNet* n, const float* r, const float* e, const DiracArgs& op, cudaStream_t s)
{
    cudaError_t err = ensure_scratch(n, 0);
    if (err == cudaSuccess) err = net_forward(n, r, op.sigma, n->z, s);
    if (err != cudaSuccess) return err;
    const int V4 = 4 * n->V;
    net_diff_kernel<<<n->grid, kNetThreads, 0, s>>>(n->z, e, n->f0, V4);
    err = launch_dirac(n->f0, n->f1, op.sigma, op.Nt, op.Nx, op.m0, op.g, op.r, 0, YK_FP32, 1, s);
    if (err == cudaSuccess) fvec_dot_kernel<<<n->grid, kNetThreads, 0, s>>>(n->f1, n->f1, n->dpart, V4);
    return err == cudaSuccess ? cudaGetLastError() : err;
}

// accumulates into n->g the weight gradient of the pair's loss; *loss (if
// given) receives its value
cudaError_t net_accumulate_grad(LearnedNet* n, const float* r, const float* e, const DiracArgs& op, cudaStream_t s,
                                double* loss)
{
    const int V = n->V, L = n->layers;
    cudaError_t err = net_loss_terms(n, r, e, op, s);
    if (err != cudaSuccess) return err;
    // dL/dz = 2 A d = 2 D^dag (D d)
    err = launch_dirac(n->f1, n->f2, op.sigma, op.Nt, op.Nx, op.m0, op.g, op.r, 1, YK_FP32, 1, s);
    if (err != cudaSuccess) return err;
    net_gz_kernel<<<n->grid, kNetThreads, 0, s>>>(n->f2, n->gz, V);
    // through F^T and the transposed layers (dec[l] = L_l^T dec[l + 1]):
    // the weight gradient of a transposed conv has the conv's form with the
    // roles of input and output swapped, and the gradient flows on by the conv
    net_feat_cm_kernel<<<n->grid, kNetThreads, 0, s>>>(n->gz, op.sigma, n->gbuf[0], V);
    int cur = 0;
    for (int l = 0; l < L; ++l) {
        conv_wgrad(n, l, n->gbuf[cur], dec_of(n, l + 1), s);
        if (l < L - 1) {
            conv_fwd(n, l, n->gbuf[cur], n->gbuf[cur ^ 1], s);
            cur ^= 1;
        } else {
            conv_fwd(n, l, n->gbuf[cur], n->gz, s);   // the gradient of N r
        }
    }
    // through N
    const float* gy = n->gz;
    for (int l = L - 1; l >= 0; --l) {
        conv_wgrad(n, l, act_of(n, l), gy, s);
        if (l > 0) {
            float* gx = n->gbuf[l & 1];
            conv_T(n, l, gy, gx, s);
            gy = gx;
        }
    }
    err = cudaGetLastError();
    if (err == cudaSuccess && loss) {
        // the loss partials were written by net_loss_terms into dpart
        err = host_sum(n, s, loss);
    }
    return err;
}

cudaError_t net_zero_grad(LearnedNet* n, cudaStream_t s) { return cudaMemsetAsync(n->g, 0, sizeof(float) * n->nw, s); }

cudaError_t net_grad_to_host(LearnedNet* n, float* host, cudaStream_t s)
{
    cudaError_t e = cudaMemcpyAsync(host, n->g, sizeof(float) * n->nw, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

// one Adam step on the accumulated gradient of `batch` pairs
cudaError_t net_adam_step(LearnedNet* n, float lr, int batch, cudaStream_t s)
{
    n->inner[1] = InnerChoice();   // new weights: the inner tolerance is chosen again
    n->adam_t += 1;
    const float c1 = 1.f / (1.f - powf(0.9f, (float)n->adam_t)), c2 = 1.f / (1.f - powf(0.999f, (float)n->adam_t));
    net_adam_kernel<<<(n->nw + 255) / 256, 256, 0, s>>>(n->w, n->g, n->m, n->v, n->nw, lr, c1, c2, 1.f / batch);
    return cudaGetLastError();
}

namespace {

__global__ void dvec_sub_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) c[i] = a[i] - b[i];
}

// one training pair, scaled: r = (b - A xk) * sc, e = (x* - xk) * sc (= e_in * sc)
__global__ void pair_make_kernel(const double* __restrict__ b, const double* __restrict__ Axk,
                                 const double* __restrict__ e, double sc, float* __restrict__ pr,
                                 float* __restrict__ pe, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        pr[i] = (float)((b[i] - Axk[i]) * sc);
        pe[i] = (float)(e[i] * sc);
    }
}

}  // namespace

// Adds the training pair (b - A xk, x* - xk), scaled to e^T A e = 1, to the
// network's pair store (capacity cap pairs).  Returns cudaErrorInvalidValue
// when the error vanishes (x* = xk).
cudaError_t net_add_pair(LearnedNet* n, int cap, const double* sigma, double m0, double g, double r, const double* b,
                         const double* xstar, const double* xk, cudaStream_t s)
{
    const size_t V4 = 4 * (size_t)n->V;
    cudaError_t e = ensure_scratch(n, 0);
    if (e != cudaSuccess) return e;
    if (!n->pairs || cap != n->pair_cap) {
        if (n->pairs) cudaFree(n->pairs);
        n->pairs = nullptr;
        n->npairs = 0;
        e = alloc_f(&n->pairs, (size_t)cap * 2 * V4);
        if (e != cudaSuccess) return e;
        n->pair_cap = cap;
    }
    if (n->npairs >= n->pair_cap) return cudaSuccess;   // full: ignore
    const DiracArgs d = {sigma, n->Nt, n->Nx, m0, g, r};
    e = apply_A(d, xk, n->d0, n->d1, YK_FP64, s);
    if (e != cudaSuccess) return e;
    dvec_sub_kernel<<<n->grid, kNetThreads, 0, s>>>(xstar, xk, n->d2, (int)V4);
    dvec_sub_kernel<<<n->grid, kNetThreads, 0, s>>>(b, n->d1, n->d0, (int)V4);
    // e^T A e through A e = b - A xk (x* solves to the tolerance)
    double ee = 0.0;
    e = dot_d(n, n->d2, n->d0, s, &ee);
    if (e != cudaSuccess) return e;
    if (!(ee > 0.0)) return cudaErrorInvalidValue;
    float* pr = n->pairs + (size_t)n->npairs * 2 * V4;
    pair_make_kernel<<<n->grid, kNetThreads, 0, s>>>(b, n->d1, n->d2, 1.0 / std::sqrt(ee), pr, pr + V4, (int)V4);
    e = cudaGetLastError();
    if (e == cudaSuccess) n->npairs += 1;
    return e;
}

int net_pairs(const LearnedNet* n) { return n->npairs; }

// mean of |M(r) - e|^2 over the stored pairs
cudaError_t net_mean_loss(LearnedNet* n, const DiracArgs& op, cudaStream_t s, double* out)
{
    const size_t V4 = 4 * (size_t)n->V;
    double sum = 0.0;
    for (int p = 0; p < n->npairs; ++p) {
        const float* pr = n->pairs + (size_t)p * 2 * V4;
        cudaError_t e = net_loss_terms(n, pr, pr + V4, op, s);
        if (e != cudaSuccess) return e;
        double l = 0.0;
        e = host_sum(n, s, &l);
        if (e != cudaSuccess) return e;
        sum += l;
    }
    *out = n->npairs ? sum / n->npairs : 0.0;
    return cudaSuccess;
}

// `steps` Adam steps on mini-batches of `batch` stored pairs drawn by a
// xorshift generator from `seed`
cudaError_t net_train(LearnedNet* n, const DiracArgs& op, int steps, int batch, float lr, uint64_t seed,
                      cudaStream_t s)
{
    if (n->npairs == 0) return cudaErrorInvalidValue;
    const size_t V4 = 4 * (size_t)n->V;
    uint64_t st = seed ? seed : 0x9E3779B97F4A7C15ull;
    for (int it = 0; it < steps; ++it) {
        cudaError_t e = net_zero_grad(n, s);
        for (int b = 0; b < batch && e == cudaSuccess; ++b) {
            st ^= st << 13;
            st ^= st >> 7;
            st ^= st << 17;
            const float* pr = n->pairs + (size_t)(st % (uint64_t)n->npairs) * 2 * V4;
            e = net_accumulate_grad(n, pr, pr + V4, op, s, nullptr);
        }
        if (e == cudaSuccess) e = net_adam_step(n, lr, batch, s);
        if (e != cudaSuccess) return e;
    }
    return cudaStreamSynchronize(s);
}

namespace {

// part[i * gridDim.x + block] = partial of <Ws[i], w>, i < cnt (Ws contiguous, n floats each)
__global__ void __launch_bounds__(kNetThreads) fvec_multidot_kernel(const float* __restrict__ Ws, int cnt,
                                                                    const float* __restrict__ w,
                                                                    double* __restrict__ part, int n)
{
    __shared__ double red[32];
    for (int i = 0; i < cnt; ++i) {
        const float* a = Ws + (size_t)i * n;
        double s = 0.0;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
            s = fma((double)a[j], (double)w[j], s);
        s = block_sum(s, red);
        if (threadIdx.x == 0) part[(size_t)i * gridDim.x + blockIdx.x] = s;
        __syncthreads();
    }
}

// part[0][block] = partial <w, w>, part[1][block] = partial <w, r>
__global__ void __launch_bounds__(kNetThreads) fvec_dot2_kernel(const float* __restrict__ w, const float* __restrict__ r,
                                                                double* __restrict__ part, int n)
{
    __shared__ double red[64];
    double s0 = 0.0, s1 = 0.0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const double wj = (double)w[j];
        s0 = fma(wj, wj, s0);
        s1 = fma(wj, (double)r[j], s1);
    }
    const double2 t = block_sum2(s0, s1, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = t.x;
        part[gridDim.x + blockIdx.x] = t.y;
    }
}

// y -= sum_i c[i] Xs[i] (c in constant-size argument arrays)
constexpr int kMaxRestart = 32;
struct Coefs {
    float c[kMaxRestart];
};

__global__ void fvec_multi_axpy_kernel(float* __restrict__ y, const float* __restrict__ Xs, int cnt, Coefs c, int n)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        float v = y[j];
        for (int i = 0; i < cnt; ++i) v = fmaf(-c.c[i], Xs[(size_t)i * n + j], v);
        y[j] = v;
    }
}

cudaError_t ensure_parts(LearnedNet* n, int segs)
{
    const size_t need = (size_t)segs * n->grid;
    if (n->hpart_cap >= need) return cudaSuccess;
    if (n->dpart) cudaFree(n->dpart);
    if (n->hpart) cudaFreeHost(n->hpart);
    n->dpart = nullptr;
    n->hpart = nullptr;
    cudaError_t e = alloc_d(&n->dpart, need);
    if (e == cudaSuccess) e = cudaMallocHost(&n->hpart, sizeof(double) * need);
    n->hpart_cap = e == cudaSuccess ? need : 0;
    return e;
}

// sums of `segs` consecutive partial segments (block order)
cudaError_t host_sums(LearnedNet* n, int segs, cudaStream_t s, double* out)
{
    cudaError_t e =
        cudaMemcpyAsync(n->hpart, n->dpart, sizeof(double) * segs * n->grid, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int k = 0; k < segs; ++k) {
        double t = 0.0;
        for (int i = 0; i < n->grid; ++i) t += n->hpart[(size_t)k * n->grid + i];
        out[k] = t;
    }
    return e;
}

}  // namespace

// Restarted flexible GCR (FP32) with z = M(r) (the network) or z = r as the
// preconditioner, inside FP64 iterative refinement: x = 0; repeat
// r = b - A x (FP64); solve A d = r to relative `inner_tol` by FGCR (at most
// `restart` directions); x += d; until |r|^2 <= stop2 or max_iter FGCR
// iterations.  A = D^dag D (K = 1); b, x: 4V doubles (device).  Classical
// Gram-Schmidt of A z against the stored directions, all its dots in one
// launch: two host synchronisations per iteration.
cudaError_t fgcr_solve(LearnedNet* n, bool use_net, const double* sigma, double m0, double g, double r,
                       const double* b, double* x, double tol, int tol_mode, int max_iter, int restart,
                       double inner_tol, cudaStream_t s, FgcrResult* res)
{
    if (restart < 1) restart = 1;
    if (restart > kMaxRestart) restart = kMaxRestart;
    const int V4 = 4 * n->V;
    const DiracArgs d = {sigma, n->Nt, n->Nx, m0, g, r};
    cudaError_t e = ensure_scratch(n, restart);
    if (e == cudaSuccess) e = ensure_parts(n, restart + 2);
    if (e != cudaSuccess) return e;
    double* Ax = n->d1;
    double* r64 = n->d2;
    float* rf = n->f0;
    float* dd = n->f1;
    float* rin = n->f2;
    float* tmp = n->f3;
    e = cudaMemsetAsync(x, 0, sizeof(double) * V4, s);
    double bb = 0.0;
    if (e == cudaSuccess) e = dot_d(n, b, b, s, &bb);
    if (e != cudaSuccess) return e;
    const double stop2 = tol_mode == YK_TOL_REL ? tol * tol * bb : tol * tol;
    double rr = bb, ww[kMaxRestart], sums[kMaxRestart + 2];
    int iters = 0, outer = 0;
    e = cudaMemcpyAsync(r64, b, sizeof(double) * V4, cudaMemcpyDeviceToDevice, s);   // r = b (x = 0)
    while (e == cudaSuccess && rr > stop2 && iters < max_iter) {
        ++outer;
        // the FP32 copy of the residual, the correction and the inner residual
        dvec_to_f_kernel<<<n->grid, kNetThreads, 0, s>>>(r64, rf, V4);
        e = cudaMemsetAsync(dd, 0, sizeof(float) * V4, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(rin, rf, sizeof(float) * V4, cudaMemcpyDeviceToDevice, s);
        double rin2 = 0.0;
        if (e == cudaSuccess) e = dot_f(n, rin, rin, s, &rin2);
        const double rin2_0 = rin2;
        for (int j = 0; j < restart && e == cudaSuccess && iters < max_iter; ++j) {
            float* Zj = n->Zs + (size_t)j * V4;
            float* Wj = n->Ws + (size_t)j * V4;
            if (use_net)
                e = net_forward_fast(n, rin, sigma, Zj, s);
            else
                e = cudaMemcpyAsync(Zj, rin, sizeof(float) * V4, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = apply_A(d, Zj, tmp, Wj, YK_FP32, s);
            if (e == cudaSuccess && j > 0) {
                fvec_multidot_kernel<<<n->grid, kNetThreads, 0, s>>>(n->Ws, j, Wj, n->dpart, V4);
                e = host_sums(n, j, s, sums);
                Coefs c = {};
                for (int i = 0; i < j; ++i) c.c[i] = (float)(sums[i] / ww[i]);
                fvec_multi_axpy_kernel<<<n->grid, kNetThreads, 0, s>>>(Wj, n->Ws, j, c, V4);
                fvec_multi_axpy_kernel<<<n->grid, kNetThreads, 0, s>>>(Zj, n->Zs, j, c, V4);
            }
            if (e != cudaSuccess) break;
            fvec_dot2_kernel<<<n->grid, kNetThreads, 0, s>>>(Wj, rin, n->dpart, V4);
            e = host_sums(n, 2, s, sums);
            if (e != cudaSuccess) break;
            ww[j] = sums[0];
            if (!(ww[j] > 0.0)) break;
            const double alpha = sums[1] / ww[j];
            fvec_axpy_kernel<<<n->grid, kNetThreads, 0, s>>>(dd, Zj, (float)alpha, V4);
            fvec_axpy_kernel<<<n->grid, kNetThreads, 0, s>>>(rin, Wj, (float)-alpha, V4);
            rin2 -= sums[1] * sums[1] / ww[j];
            ++iters;
            if (rin2 <= inner_tol * inner_tol * rin2_0) break;
        }
        if (e != cudaSuccess) break;
        // x += d; r = b - A x in FP64
        dvec_add_f_kernel<<<n->grid, kNetThreads, 0, s>>>(x, dd, V4);
        e = apply_A(d, x, n->d0, Ax, YK_FP64, s);
        if (e == cudaSuccess) dvec_residual_kernel<<<n->grid, kNetThreads, 0, s>>>(b, Ax, r64, rf, V4);
        if (e == cudaSuccess) e = dot_d(n, r64, r64, s, &rr);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    res->iterations = iters;
    res->outer = outer;
    res->rr = rr;
    res->rr0 = bb;
    res->converged = rr <= stop2 ? 1 : 0;
    return e;
}

}  // namespace yk
// ---------------------------------------------------------------------------
// Flexible preconditioned CG with the network or the identity: FP32 vectors,
// FP64 scalars kept on the device, inside FP64 iterative refinement.  The
// host reads |r|^2 every kPcgChunk iterations; a chunk of iterations is one
// captured CUDA graph (launched again for every chunk and every solve while
// the operator, the field and the network's skip are unchanged).
//
// beta is the Polak-Ribiere form, beta = <z', r' - r> / <z, r> =
// -alpha <z', q> / <z, r> (r' - r = -alpha q): equal to the classical
// <z', r'> / <z, r> for a fixed symmetric positive definite M, and the form
// that stays robust when M(r) carries rounding (flexible CG).
// ---------------------------------------------------------------------------
namespace yk {

namespace {

constexpr int kPcgChunk = 8;

// Block sums of NV FP32 values: FP32 within a warp (32 terms), FP64 across
// warps (GB300's FP64 pipe is narrow: per-site FP64 work would bound these
// kernels); the results are valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum_f(float (&v)[NV], double (&out)[NV], double* red)
{
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NV; ++j) red[j * 32 + w] = (double)v[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        double r = 0.0;
        if (w == 0) {
            r = lane < nw ? red[j * 32 + lane] : 0.0;
            r = warp_sum(r);
        }
        out[j] = r;
    }
}

// The totals of two arrays of nb per-block FP32 partials, in every thread
// of the block: FP32 sums in a fixed order (so every block computes the same
// scalar bits; the FP64 pipe is kept out of the iteration), the loads of a
// chunk of 8 per thread issued together.
__device__ __forceinline__ float2 block_totals(const float* a, const float* b, int nb)
{
    __shared__ float2 wsum[32];
    __shared__ float2 tot;
    float sa = 0.f, sb = 0.f;
    for (int base = 0; base < nb; base += 8 * blockDim.x) {
        float wa[8], wb[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int i = base + threadIdx.x + j * blockDim.x;
            wa[j] = i < nb ? __ldcg(a + i) : 0.f;
            wb[j] = i < nb ? __ldcg(b + i) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            sa += wa[j];
            sb += wb[j];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sa += __shfl_xor_sync(0xffffffffu, sa, o);
        sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) wsum[w] = make_float2(sa, sb);
    __syncthreads();
    if (threadIdx.x == 0) {
        float2 t = make_float2(0.f, 0.f);
        for (int i = 0; i < nw; ++i) {
            t.x += wsum[i].x;
            t.y += wsum[i].y;
        }
        tot = t;
    }
    __syncthreads();
    return tot;
}

// x += alpha p, r -= alpha q; with X != null also the network's BF16
// features (r, sigma r) of the new r
// alpha = <r, z> / <p, q> from the z kernel's and the q kernel's partials
template <bool PDL>
__device__ __forceinline__ void pcg_xr_body(float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p,
                                            const float* __restrict__ q, const float* __restrict__ part_rz,
                                            const float* __restrict__ part_pq, int nb, const float* __restrict__ sigma,
                                            uint4* __restrict__ X, int V)
{
    if (PDL) pdl_wait();
    const float2 t = block_totals(part_rz, part_pq, nb);
    const float a = t.y != 0.f ? t.x / t.y : 0.f;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        float4 xv = reinterpret_cast<float4*>(x)[n], rv = reinterpret_cast<float4*>(r)[n];
        const float4 pv = reinterpret_cast<const float4*>(p)[n], qv = reinterpret_cast<const float4*>(q)[n];
        xv.x = fmaf(a, pv.x, xv.x);
        xv.y = fmaf(a, pv.y, xv.y);
        xv.z = fmaf(a, pv.z, xv.z);
        xv.w = fmaf(a, pv.w, xv.w);
        rv.x = fmaf(-a, qv.x, rv.x);
        rv.y = fmaf(-a, qv.y, rv.y);
        rv.z = fmaf(-a, qv.z, rv.z);
        rv.w = fmaf(-a, qv.w, rv.w);
        reinterpret_cast<float4*>(x)[n] = xv;
        reinterpret_cast<float4*>(r)[n] = rv;
        if (X) X[n] = features_bf(rv, sigma[n]);
    }
    if (PDL) pdl_trigger();
}

__global__ void __launch_bounds__(kNetThreads) pcg_xr_kernel(float* __restrict__ x, float* __restrict__ r,
                                                             const float* __restrict__ p, const float* __restrict__ q,
                                                             const float* __restrict__ part_rz,
                                                             const float* __restrict__ part_pq, int nb,
                                                             const float* __restrict__ sigma, uint4* __restrict__ X,
                                                             int V)
{
    pcg_xr_body<true>(x, r, p, q, part_rz, part_pq, nb, sigma, X, V);
}

// z = F^T a + skip r (a != null: the network's last transposed layer) or
// z = r (a == null), with the per-block partials of <r, z>, <r, r> and
// <z, q> (q null: 0) in part[0..nb), part[nb..2nb), part[2nb..3nb) (FP32
// products of a site, FP64 across warps, stored in FP32).
template <bool PDL>
__device__ __forceinline__ void pcg_z_body(const uint4* __restrict__ a, const float* __restrict__ sigma,
                                           const float* __restrict__ r, float skip, float* __restrict__ z,
                                           const float* __restrict__ q, float* __restrict__ part, int V)
{
    __shared__ double red[96];
    if (PDL) pdl_wait();
    float acc[3] = {0.f, 0.f, 0.f};
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const float4 rv = reinterpret_cast<const float4*>(r)[n];
        const float4 o = a ? featT_bf(a[n], sigma[n], rv, skip) : rv;
        reinterpret_cast<float4*>(z)[n] = o;
        acc[0] += fmaf(rv.x, o.x, fmaf(rv.y, o.y, fmaf(rv.z, o.z, rv.w * o.w)));
        acc[1] += fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, fmaf(rv.z, rv.z, rv.w * rv.w)));
        if (q) {
            const float4 qv = reinterpret_cast<const float4*>(q)[n];
            acc[2] += fmaf(o.x, qv.x, fmaf(o.y, qv.y, fmaf(o.z, qv.z, o.w * qv.w)));
        }
    }
    if (PDL) pdl_trigger();
    double tot[3];
    block_sum_f<3>(acc, tot, red);
    const int nb = gridDim.x;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = (float)tot[0];
        part[nb + blockIdx.x] = (float)tot[1];
        part[2 * nb + blockIdx.x] = (float)tot[2];
    }
}

__global__ void __launch_bounds__(kNetThreads) pcg_z_kernel(const uint4* __restrict__ a,
                                                            const float* __restrict__ sigma,
                                                            const float* __restrict__ r, float skip,
                                                            float* __restrict__ z, const float* __restrict__ q,
                                                            float* __restrict__ part, int V)
{
    pcg_z_body<true>(a, sigma, r, skip, z, q, part, V);
}

// diag32[n] = 2 r + m0 + g sigma[n] in FP32 (the stencils below run on the
// FP32 pipes only)
__global__ void diag_f_kernel(const double* __restrict__ sigma, float* __restrict__ out, double m0, double g,
                              double r, int V)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x)
        out[n] = (float)(2.0 * r + m0 + g * sigma[n]);
}

// p' = z + beta p (written at the own site), and t = D p' with the
// neighbours' p' formed on the fly from z and p (p' goes to the other
// buffer: a neighbour may still read p)
// beta = -<z', q> / <p, q> (the Polak-Ribiere beta, -alpha <z', q> / <r, z>
// with alpha = <r, z> / <p, q>) from the partials; 0 when <p, q> = 0 (the
// round's first direction: the q partials are zeroed)
template <bool PDL>
__device__ __forceinline__ void pcg_dp_body(const float* __restrict__ z, const float* __restrict__ p,
                                            float* __restrict__ p_new, float* __restrict__ t,
                                            const float* __restrict__ diag, const float* __restrict__ part_zq,
                                            const float* __restrict__ part_pq, int nb, int Nt, int Nx, float rw)
{
    if (PDL) pdl_wait();
    const float2 tt = block_totals(part_zq, part_pq, nb);
    const float b = tt.y != 0.f ? -tt.x / tt.y : 0.f;
    const int V = Nt * Nx;
    auto pn = [&](int m) {
        const Site<float, 1> zz = load_site<float, 1>(z, m), pp = load_site<float, 1>(p, m);
        Site<float, 1> o;
#pragma unroll
        for (int q = 0; q < 4; ++q) o.v[q] = fmaf(b, pp.v[q], zz.v[q]);
        return o;
    };
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const Nbr nb = neighbours(n, Nt, Nx);
        const Site<float, 1> c = pn(n), tu = pn(nb.tu), td = pn(nb.td), xu = pn(nb.xu), xd = pn(nb.xd);
        store_site<float, 1>(p_new, n, c);
        store_site<float, 1>(t, n, dirac_combine<float, 1, false>(c, tu, td, xu, xd, diag[n], rw, (float)nb.sp,
                                                                  (float)nb.sm));
    }
    if (PDL) pdl_trigger();
}

__global__ void __launch_bounds__(kNetThreads) pcg_dp_kernel(const float* __restrict__ z,
                                                             const float* __restrict__ p, float* __restrict__ p_new,
                                                             float* __restrict__ t, const float* __restrict__ diag,
                                                             const float* __restrict__ part_zq,
                                                             const float* __restrict__ part_pq, int nb, int Nt,
                                                             int Nx, float rw)
{
    pcg_dp_body<true>(z, p, p_new, t, diag, part_zq, part_pq, nb, Nt, Nx, rw);
}

// q = D^dag t and the per-block partials of <p, q> (FP32 per site, FP64
// across warps)
template <bool PDL>
__device__ __forceinline__ void pcg_dq_body(const float* __restrict__ t, const float* __restrict__ p,
                                            float* __restrict__ q, const float* __restrict__ diag,
                                            float* __restrict__ part, int Nt, int Nx, float rw)
{
    __shared__ double red[32];
    const int V = Nt * Nx;
    if (PDL) pdl_wait();
    float acc[1] = {0.f};
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const Nbr nb = neighbours(n, Nt, Nx);
        const Site<float, 1> o = dirac_combine<float, 1, true>(
            load_site<float, 1>(t, n), load_site<float, 1>(t, nb.tu), load_site<float, 1>(t, nb.td),
            load_site<float, 1>(t, nb.xu), load_site<float, 1>(t, nb.xd), diag[n], rw, (float)nb.sp, (float)nb.sm);
        store_site<float, 1>(q, n, o);
        const Site<float, 1> pv = load_site<float, 1>(p, n);
        acc[0] += fmaf(pv.v[0], o.v[0], fmaf(pv.v[1], o.v[1], fmaf(pv.v[2], o.v[2], pv.v[3] * o.v[3])));
    }
    if (PDL) pdl_trigger();
    double tot[1];
    block_sum_f<1>(acc, tot, red);
    if (threadIdx.x == 0) part[blockIdx.x] = (float)tot[0];
}

__global__ void __launch_bounds__(kNetThreads) pcg_dq_kernel(const float* __restrict__ t,
                                                             const float* __restrict__ p, float* __restrict__ q,
                                                             const float* __restrict__ diag,
                                                             float* __restrict__ part, int Nt, int Nx, float rw)
{
    pcg_dq_body<true>(t, p, q, diag, part, Nt, Nx, rw);
}

struct PcgBufs {
    float *r, *x, *z, *p[2], *q, *tmp;
    float* part_z;    // 3 x grid FP32 partials of the z kernel: <r, z>, <r, r>, <z, q>
    float* part_pq;   // grid FP32 partials of <p, q>
};

// ---------------------------------------------------------------------------
// The persistent form of a chunk of PCG iterations: one cooperative launch
// runs the 4 + 2L phases of every iteration (p' and D p', D^dag, x and r with
// the features, the network's 2L convolutions, z = M r) with a grid barrier
// between phases instead of a kernel boundary.  The phases are the kernels'
// own bodies; the partials stay per block (nb = the launch's blocks, the
// solver's grid), so every value is the launched kernels' bit for bit.
// ---------------------------------------------------------------------------
struct PcgChunk {
    float *z, *p[2], *tmp, *q, *x, *r;
    const float *diag, *sig32;
    float *part_z, *part_pq;
    uint4* h16[2];
    const float* w[kPcgMaxConv];   // the convolutions in order: N's layers, then N^T's
    int cout[kPcgMaxConv];
    int nconv;
    int Nt, Nx, V, R, W;
    float rw, skip;
    int use_net, count, parity;
    unsigned* bar;   // arrival counter (zeroed before the launch), then the error word
};

// Grid barrier of the persistent PCG: release-arrival, acquiring poll,
// bounded (the error word set and every block leaving when it gives up).
__device__ bool pcg_sync(unsigned* bar, unsigned& gen)
{
    __syncthreads();
    int bad = 0;
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
        const unsigned target = gridDim.x * (gen + 1u);
        const long long t0 = clock64();
        for (;;) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
            if ((int)(v - target) >= 0) break;
            if (*(volatile unsigned*)(bar + 1) != 0u) {
                bad = 1;
                break;
            }
            if (clock64() - t0 > 4000000000LL) {   // about 2 s
                atomicExch(bar + 1, 1u);
                bad = 1;
                break;
            }
        }
    }
    ++gen;
    return __syncthreads_or(bad) == 0;
}

__global__ void __launch_bounds__(kNetThreads) pcg_chunk_kernel(PcgChunk P)
{
    __shared__ __align__(16) uint4 sm[(kTcMaxR + 2) * kTcSW];
    unsigned gen = 0;
    const int nb = gridDim.x;
    int parity = P.parity;
    for (int it = 0; it < P.count; ++it, parity ^= 1) {
        const float* p = P.p[parity];
        float* pn = P.p[parity ^ 1];
        pcg_dp_body<false>(P.z, p, pn, P.tmp, P.diag, P.part_z + 2 * nb, P.part_pq, nb, P.Nt, P.Nx, P.rw);
        if (!pcg_sync(P.bar, gen)) return;
        pcg_dq_body<false>(P.tmp, pn, P.q, P.diag, P.part_pq, P.Nt, P.Nx, P.rw);
        if (!pcg_sync(P.bar, gen)) return;
        pcg_xr_body<false>(P.x, P.r, pn, P.q, P.part_z, P.part_pq, nb, P.sig32, P.use_net ? P.h16[0] : nullptr,
                           P.V);
        if (!pcg_sync(P.bar, gen)) return;
        const uint4* a = nullptr;
        if (P.use_net) {
            int cur = 0;
            for (int l = 0; l < P.nconv; ++l, cur ^= 1) {
                const uint4* X = P.h16[cur];
                uint4* Y = P.h16[cur ^ 1];
                const bool trans = l >= P.nconv / 2, out4 = P.cout[l] == kNetOut;
                if (!trans) {
                    if (out4) conv_bf_tiles<kNetOut, false, false>(X, Y, P.w[l], P.Nt, P.Nx, P.R, P.W, sm);
                    else conv_bf_tiles<kNetC, false, false>(X, Y, P.w[l], P.Nt, P.Nx, P.R, P.W, sm);
                } else {
                    if (out4) conv_bf_tiles<kNetOut, true, false>(X, Y, P.w[l], P.Nt, P.Nx, P.R, P.W, sm);
                    else conv_bf_tiles<kNetC, true, false>(X, Y, P.w[l], P.Nt, P.Nx, P.R, P.W, sm);
                }
                if (!pcg_sync(P.bar, gen)) return;
            }
            a = P.h16[cur];
        }
        pcg_z_body<false>(a, P.sig32, P.r, P.skip, P.z, P.q, P.part_z, P.V);
        if (!pcg_sync(P.bar, gen)) return;
    }
}

// Blocks of pcg_chunk_kernel that fit on the device at once (0: none).
int pcg_chunk_max_grid()
{
    static int maxg = -1;
    if (maxg < 0) {
        int dev = 0, nsm = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)pcg_chunk_kernel, kNetThreads, 0) !=
            cudaSuccess) {
            cudaGetLastError();
            per = 0;
        }
        maxg = per * nsm;
    }
    return maxg;
}

// z = M r, its partials and the scalars; X: the features (already written
// by pcg_xr_kernel, or written here on the first round)
void pcg_precond(LearnedNet* n, bool use_net, const DiracArgs& d, const PcgBufs& b, bool first, cudaStream_t s)
{
    const int V = n->V, nb = n->grid;
    const uint4* a = nullptr;
    if (use_net) {
        if (first) launch_pdl(net_feat_bf_kernel, nb, 0, s, (const float*)b.r, (const float*)n->sig32, n->h16[0], V);
        a = net_convs_fast(n, s);
    }
    launch_pdl(pcg_z_kernel, nb, 0, s, a, (const float*)n->sig32, (const float*)b.r, n->skip, b.z,
               (const float*)(first ? nullptr : b.q), b.part_z, V);
}

// `count` iterations from the direction buffer `parity`: p' = z + beta p and
// t = D p', q = D^dag t with alpha, x and r (and the features of r),
// z = M r with beta.  Returns the parity after them.
int pcg_iterations(LearnedNet* n, bool use_net, const DiracArgs& d, const PcgBufs& b, int count, int parity,
                   cudaStream_t s)
{
    const int V = n->V, nb = n->grid;
    const float rw = (float)d.r;
    if (n->persistent && count > 0 && (!use_net || n->tc_G == 1)) {
        PcgChunk P = {};
        P.z = b.z;
        P.p[0] = b.p[0];
        P.p[1] = b.p[1];
        P.tmp = b.tmp;
        P.q = b.q;
        P.x = b.x;
        P.r = b.r;
        P.diag = n->diag32;
        P.sig32 = n->sig32;
        P.part_z = b.part_z;
        P.part_pq = b.part_pq;
        P.h16[0] = n->h16[0];
        P.h16[1] = n->h16[1];
        const int L = n->layers;
        P.nconv = use_net ? 2 * L : 0;
        for (int q = 0; q < P.nconv; ++q) {
            const int l = q < L ? q : 2 * L - 1 - q;   // N's layers, then N^T's in reverse
            P.w[q] = n->w + n->woff[l];
            P.cout[q] = cout_of(n, l);
        }
        P.Nt = d.Nt;
        P.Nx = d.Nx;
        P.V = V;
        P.R = n->tc_R;
        P.W = n->tc_W;
        P.rw = rw;
        P.skip = n->skip;
        P.use_net = use_net ? 1 : 0;
        P.count = count;
        P.parity = parity;
        P.bar = n->pbar;
        cudaMemsetAsync(n->pbar, 0, 2 * sizeof(unsigned), s);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(nb);
        cfg.blockDim = dim3(kNetThreads);
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        void* args[] = {&P};
        cudaLaunchKernelExC(&cfg, (const void*)pcg_chunk_kernel, args);
        return parity ^ (count & 1);
    }
    for (int it = 0; it < count; ++it, parity ^= 1) {
        float* p = b.p[parity];
        float* pn = b.p[parity ^ 1];
        launch_pdl(pcg_dp_kernel, nb, 0, s, (const float*)b.z, (const float*)p, pn, b.tmp, (const float*)n->diag32,
                   (const float*)(b.part_z + 2 * nb), (const float*)b.part_pq, nb, d.Nt, d.Nx, rw);
        launch_pdl(pcg_dq_kernel, nb, 0, s, (const float*)b.tmp, (const float*)pn, b.q, (const float*)n->diag32,
                   b.part_pq, d.Nt, d.Nx, rw);
        launch_pdl(pcg_xr_kernel, nb, 0, s, b.x, b.r, (const float*)pn, (const float*)b.q, (const float*)b.part_z,
                   (const float*)b.part_pq, nb, (const float*)n->sig32, use_net ? n->h16[0] : nullptr, V);
        pcg_precond(n, use_net, d, b, false, s);
    }
    return parity;
}

}  // namespace

// the captured chunk of a learned net (see pcg_solve)
struct PcgGraph {
    cudaGraphExec_t exec = nullptr;
    PcgBufs buf = {};
    const double* dpart = nullptr;
    bool use_net = false;
    const double* sigma = nullptr;
    double m0 = 0, g = 0, r = 0;
    float skip = 0;
};

void pcg_graph_destroy(PcgGraph* g)
{
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    delete g;
}

static cudaError_t pcg_solve_once(LearnedNet* n, bool use_net, const double* sigma, double m0, double g, double r,
                                  const double* b, double* x, double tol, int tol_mode, int max_iter,
                                  double inner_tol, cudaStream_t s, FgcrResult* res)
{
    const int V4 = 4 * n->V;
    const DiracArgs d = {sigma, n->Nt, n->Nx, m0, g, r};
    cudaError_t e = ensure_scratch(n, 2);   // Zs, Ws: two 4V float vectors each
    if (e == cudaSuccess) e = ensure_parts(n, 4);
    if (e != cudaSuccess) return e;
    double* Ax = n->d1;
    double* r64 = n->d2;
    float* fpart = reinterpret_cast<float*>(n->dpart);   // 4 x grid floats in the partials' space
    const PcgBufs B = {n->f0, n->f1, n->f2, {n->Zs, n->Zs + (size_t)V4}, n->Ws, n->f3, fpart,
                       fpart + 3 * (size_t)n->grid};
    // |r|^2 of the inner solve from the z kernel's partials (host sum)
    auto inner_rr = [&](double* out) -> cudaError_t {
        float* hf = reinterpret_cast<float*>(n->hpart);
        unsigned* hbad = reinterpret_cast<unsigned*>(hf + n->grid);   // the persistent chunk's error word
        *hbad = 0u;
        cudaError_t ce = cudaMemcpyAsync(hf, B.part_z + n->grid, sizeof(float) * n->grid, cudaMemcpyDeviceToHost, s);
        if (ce == cudaSuccess && n->persistent)
            ce = cudaMemcpyAsync(hbad, n->pbar + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
        if (ce == cudaSuccess && *hbad) ce = cudaErrorLaunchTimeout;   // a barrier wait gave up
        double t = 0.0;
        for (int i = 0; i < n->grid; ++i) t += hf[i];
        *out = t;
        return ce;
    };
    f_of_d_kernel<<<n->grid, kNetThreads, 0, s>>>(sigma, n->sig32, n->V);
    diag_f_kernel<<<n->grid, kNetThreads, 0, s>>>(sigma, n->diag32, m0, g, r, n->V);
    const int nb = n->grid;
    if (use_net && !n->tc_tuned) {
        e = net_tune_tile(n, s);
        if (e != cudaSuccess) return e;
        if (n->pcg) {   // captured with the previous tile
            pcg_graph_destroy(n->pcg);
            n->pcg = nullptr;
        }
    }
    // the chunk graph, captured again when the operator or the network changed
    PcgGraph*& G = n->pcg;
    if (G && (G->use_net != use_net || G->sigma != sigma || G->m0 != m0 || G->g != g || G->r != r ||
              G->skip != n->skip || G->dpart != n->dpart || std::memcmp(&G->buf, &B, sizeof(B)) != 0)) {
        pcg_graph_destroy(G);
        G = nullptr;
    }
    if (!G && !n->pcg_no_graph) {
        G = new PcgGraph();
        G->buf = B;
        G->dpart = n->dpart;
        G->use_net = use_net;
        G->sigma = sigma;
        G->m0 = m0;
        G->g = g;
        G->r = r;
        G->skip = n->skip;
        cudaGraph_t graph = nullptr;
        bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            pcg_iterations(n, use_net, d, B, kPcgChunk, 0, s);   // an even count: parity 0 -> 0
            const cudaError_t ce = cudaGetLastError();
            ok = cudaStreamEndCapture(s, &graph) == cudaSuccess && ce == cudaSuccess && graph;
        }
        if (ok) ok = cudaGraphInstantiate(&G->exec, graph, 0) == cudaSuccess;
        if (graph) cudaGraphDestroy(graph);
        if (!ok) {   // e.g. the legacy stream, which cannot be captured: run uncaptured
            cudaGetLastError();
            pcg_graph_destroy(G);
            G = nullptr;
            n->pcg_no_graph = true;
        }
    }
    e = cudaMemsetAsync(x, 0, sizeof(double) * V4, s);
    double bb = 0.0;
    if (e == cudaSuccess) e = dot_d(n, b, b, s, &bb);
    if (e != cudaSuccess) return e;
    const double stop2 = tol_mode == YK_TOL_REL ? tol * tol * bb : tol * tol;
    double rr64 = bb;
    int iters = 0, outer = 0;
    e = cudaMemcpyAsync(r64, b, sizeof(double) * V4, cudaMemcpyDeviceToDevice, s);
    while (e == cudaSuccess && rr64 > stop2 && iters < max_iter) {
        ++outer;
        dvec_to_f_kernel<<<nb, kNetThreads, 0, s>>>(r64, B.r, V4);
        e = cudaMemsetAsync(B.x, 0, sizeof(float) * V4, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(B.p[0], 0, sizeof(float) * V4, s);
        // zero <p, q> partials: the first direction takes beta = 0, p' = z
        if (e == cudaSuccess) e = cudaMemsetAsync(B.part_pq, 0, sizeof(float) * nb, s);
        if (e != cudaSuccess) break;
        pcg_precond(n, use_net, d, B, true, s);   // z = M r
        int parity = 0;
        double rr0 = 0.0;
        e = inner_rr(&rr0);
        double rrc = rr0;
        // Past the looser 1e-4 reduction a round also ends when a chunk
        // reduces |r|^2 by less than a third of the round's average (in
        // logarithm): the FP32 recurrence, with the BF16 preconditioner's
        // rounding, has stagnated and an FP64 restart is cheaper.
        const double loose2 = 1e-8 * rr0;
        int chunks = 0;
        while (e == cudaSuccess && iters < max_iter && rrc > inner_tol * inner_tol * rr0) {
            const double rr_before = rrc;
            const int cnt = std::min(kPcgChunk, max_iter - iters);
            if (G && cnt == kPcgChunk && parity == 0) {
                e = cudaGraphLaunch(G->exec, s);
            } else {
                parity = pcg_iterations(n, use_net, d, B, cnt, parity, s);
                e = cudaGetLastError();
            }
            iters += cnt;
            if (e == cudaSuccess) e = inner_rr(&rrc);
            if (!(rrc == rrc)) break;   // NaN: the FP64 check below decides
            ++chunks;
            if (rrc < loose2 && rrc > 0.0 && rr_before > 0.0) {
                const double avg = std::log(rr0 / rrc) / chunks, last = std::log(rr_before / rrc);
                if (last < avg / 3.0) break;
            }
        }
        if (e != cudaSuccess) break;
        dvec_add_f_kernel<<<nb, kNetThreads, 0, s>>>(x, B.x, V4);
        e = apply_A(d, x, n->d0, Ax, YK_FP64, s);
        if (e == cudaSuccess) dvec_residual_kernel<<<nb, kNetThreads, 0, s>>>(b, Ax, r64, B.r, V4);
        if (e == cudaSuccess) e = dot_d(n, r64, r64, s, &rr64);
        if (!(rr64 == rr64)) break;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    res->iterations = iters;
    res->outer = outer;
    res->rr = rr64;
    res->rr0 = bb;
    res->converged = rr64 <= stop2 ? 1 : 0;
    return e;
}

// inner_tol > 0: that tolerance.  inner_tol <= 0: chosen by measurement per
// network and mode (with or without M): after one warm-up solve, solves
// alternate between 1e-4 (three FP64 rounds to 1e-10) and 1e-5 (two rounds),
// kInnerTrials of each (consecutive right-hand sides differ: one solve each
// would be noise), and later solves take the one with the smaller total.  The better one depends on the
// problem: a hard system (1024^2, m0 = 0.01) converges more slowly in FP32
// below 1e-4 than a restart costs, an easier one (512^2, m0 = 0.02) the
// other way round.  New weights start the choice again.
cudaError_t pcg_solve(LearnedNet* n, bool use_net, const double* sigma, double m0, double g, double r,
                      const double* b, double* x, double tol, int tol_mode, int max_iter, double inner_tol,
                      cudaStream_t s, FgcrResult* res)
{
    if (inner_tol > 0.0) return pcg_solve_once(n, use_net, sigma, m0, g, r, b, x, tol, tol_mode, max_iter, inner_tol, s, res);
    static const double kTols[2] = {1e-4, 1e-5};
    constexpr int kInnerTrials = 3;
    InnerChoice& ic = n->inner[use_net ? 1 : 0];
    const int k = ic.chosen >= 0 ? ic.chosen : ic.tried == 0 ? 1 : (ic.tried - 1) % 2;   // warm-up: 1e-5
    const auto t0 = std::chrono::steady_clock::now();
    const cudaError_t e = pcg_solve_once(n, use_net, sigma, m0, g, r, b, x, tol, tol_mode, max_iter, kTols[k], s, res);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (ic.chosen < 0 && e == cudaSuccess) {
        if (ic.tried >= 1) ic.ms[k] += ms;   // the first solve warms up (tile tuning, graph capture)
        if (++ic.tried == 1 + 2 * kInnerTrials) ic.chosen = ic.ms[0] <= ic.ms[1] ? 0 : 1;
    }
    return e;
}

double pcg_inner_choice(const LearnedNet* n)
{
    const InnerChoice& ic = n->inner[1];
    return ic.chosen < 0 ? 0.0 : ic.chosen == 0 ? 1e-4 : 1e-5;
}

}  // namespace yk
