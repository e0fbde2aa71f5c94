// yk_common.cuh -- device-side building blocks shared by the sm_103a kernels:
// spinor site vectors, the Wilson-Dirac site stencil, Philox4x32-10 normals
// and deterministic block reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "yk_internal.h"

namespace yk {

// ---------------------------------------------------------------------------
// Spinor sites.  A site holds 4 entries [f1s1, f1s2, f2s1, f2s2]
// (code/src/Spinor.cuh:7-16); each entry has K real planes: K = 1 for the
// real sigma-only Langevin path (imaginary parts are exactly zero there,
// code/src/FermionicDrift.cu:107), K = 2 for interleaved complex buffers.
// ---------------------------------------------------------------------------
template <typename R, int K>
struct Site {
    R v[4 * K];
};

template <typename R, int K>
__device__ __forceinline__ Site<R, K> load_site(const R* base, int64_t n)
{
    Site<R, K> s;
    const R* p = base + n * (4 * K);
    if constexpr (sizeof(R) * 4 * K == 16) {
        const float4 a = *reinterpret_cast<const float4*>(p);
        s.v[0] = reinterpret_cast<const R*>(&a)[0];
        s.v[1] = reinterpret_cast<const R*>(&a)[1];
        s.v[2] = reinterpret_cast<const R*>(&a)[2];
        s.v[3] = reinterpret_cast<const R*>(&a)[3];
    } else {
        constexpr int NV = (int)(sizeof(R) * 4 * K / 16);
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const float4 a = reinterpret_cast<const float4*>(p)[i];
            constexpr int PER = (int)(16 / sizeof(R));
#pragma unroll
            for (int j = 0; j < PER; ++j) s.v[i * PER + j] = reinterpret_cast<const R*>(&a)[j];
        }
    }
    return s;
}

// Coherent 16-byte load of data that other blocks of the same launch wrote
// before the last grid barrier.  A volatile access: the compiler neither
// caches nor speculates it (the __ldcg/__ldg intrinsics are plain inline asm
// that it may hoist, merge or issue ahead of a bounds test).
__device__ __forceinline__ double2 ld_volatile2(const double2* p)
{
    const volatile double* q = reinterpret_cast<const volatile double*>(p);
    return make_double2(q[0], q[1]);
}

__device__ __forceinline__ double ld_volatile(const double* p) { return *reinterpret_cast<const volatile double*>(p); }

template <typename R, int K>
__device__ __forceinline__ void store_site(R* base, int64_t n, const Site<R, K>& s)
{
    float4* p = reinterpret_cast<float4*>(base + n * (4 * K));
    constexpr int NV = (int)(sizeof(R) * 4 * K / 16);
    constexpr int PER = (int)(16 / sizeof(R));
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        float4 a;
#pragma unroll
        for (int j = 0; j < PER; ++j) reinterpret_cast<R*>(&a)[j] = s.v[i * PER + j];
        p[i] = a;
    }
}

// ---------------------------------------------------------------------------
// Lattice geometry of one site: neighbours and antiperiodic-time signs.
// Site n = t*Nx + x (code/src/Lattice.cu:16-30); tables IUP/IDN of
// code/src/Dirac.cu:10-21 are replaced by index arithmetic.
// ---------------------------------------------------------------------------
struct Nbr {
    int64_t tu, td, xu, xd;
    float sp, sm;   // sign of the hop to n+t (t == Nt-1 -> -1) and to n-t (t == 0 -> -1)
};

__device__ __forceinline__ Nbr neighbours(int n, int Nt, int Nx)
{
    const int t = n / Nx;
    const int x = n - t * Nx;
    Nbr b;
    b.tu = (t + 1 == Nt) ? x : n + Nx;
    b.td = (t == 0) ? (int64_t)(Nt - 1) * Nx + x : n - Nx;
    b.xu = (x + 1 == Nx) ? n - x : n + 1;
    b.xd = (x == 0) ? n + Nx - 1 : n - 1;
    b.sp = (t + 1 == Nt) ? -1.f : 1.f;
    b.sm = (t == 0) ? -1.f : 1.f;
    return b;
}

// Wilson-Dirac operator at one site (code/src/Dirac.cu:49-70 and :144-190):
//  (D psi)(n)   = diag psi(n) - 1/2 sum_mu [ s+ (r - g_mu) psi(n+mu) + s- (r + g_mu) psi(n-mu) ]
//  (D^+ psi)(n) = diag psi(n) - 1/2 sum_mu [ s+ (r + g_mu) psi(n+mu) + s- (r - g_mu) psi(n-mu) ]
// with g_t = diag(1,-1), g_x = sigma_1, diag = 2r + m0 + g sigma(n).
// Both flavours and every real plane see the same real coefficients.
template <typename R, int K, bool DAG>
__device__ __forceinline__ Site<R, K> dirac_combine(const Site<R, K>& c, const Site<R, K>& tu,
                                                    const Site<R, K>& td, const Site<R, K>& xu,
                                                    const Site<R, K>& xd, R diag, R r, R sp, R sm)
{
    Site<R, K> o;
    const R h = R(0.5);
    // time hops: coefficient on the upper (u) and lower (d) spin component
    const R cu_up = DAG ? -sp * h * (r + R(1)) : -sp * h * (r - R(1));
    const R cd_up = DAG ? -sp * h * (r - R(1)) : -sp * h * (r + R(1));
    const R cu_dn = DAG ? -sm * h * (r - R(1)) : -sm * h * (r + R(1));
    const R cd_dn = DAG ? -sm * h * (r + R(1)) : -sm * h * (r - R(1));
    // space hops: up-neighbour uses (r - s1) for D and (r + s1) for D^+
    const R sx_up = DAG ? R(1) : R(-1);
    const R sx_dn = -sx_up;
#pragma unroll
    for (int f = 0; f < 2; ++f) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int iu = (2 * f) * K + k, id = (2 * f + 1) * K + k;
            R ou = diag * c.v[iu];
            R od = diag * c.v[id];
            ou += cu_up * tu.v[iu] + cu_dn * td.v[iu];
            od += cd_up * tu.v[id] + cd_dn * td.v[id];
            // -1/2 (r u +- d), -1/2 (r d +- u)
            ou -= h * (r * xu.v[iu] + sx_up * xu.v[id]) + h * (r * xd.v[iu] + sx_dn * xd.v[id]);
            od -= h * (r * xu.v[id] + sx_up * xu.v[iu]) + h * (r * xd.v[id] + sx_dn * xd.v[iu]);
            o.v[iu] = ou;
            o.v[id] = od;
        }
    }
    return o;
}

// Pion term of the Yukawa coupling (no reference counterpart: the reference is
// sigma-only, code/src/params.h:25, Dirac.cu:57-69).  With the pions the site
// term is g (sigma + i gamma5 tau.pi), gamma5 = -i gamma_t gamma_x = sigma_2,
// so i gamma5 = [[0, 1], [-1, 0]] on spin and tau.s = [[s3, s1 - i s2],
// [s1 + i s2, -s3]] on flavour:  o += (i gamma5 tau.s) c  for s = +-g pi(n)
// (D: +g, D^dag: -g).  Complex sites (K = 2) only: tau_2 makes D complex.
template <typename R>
__device__ __forceinline__ void pion_add(Site<R, 2>& o, const Site<R, 2>& c, R s1, R s2, R s3)
{
#pragma unroll
    for (int sp = 0; sp < 2; ++sp) {
        // w_f = i sigma_2 c_f: (w_f)_0 = c_{f,1}, (w_f)_1 = -c_{f,0}
        const int src = sp == 0 ? 1 : 0;
        const R sgn = sp == 0 ? R(1) : R(-1);
        const R ar = sgn * c.v[(0 + src) * 2], ai = sgn * c.v[(0 + src) * 2 + 1];   // w_1 (flavour 1)
        const R br = sgn * c.v[(2 + src) * 2], bi = sgn * c.v[(2 + src) * 2 + 1];   // w_2 (flavour 2)
        o.v[(0 + sp) * 2] += s3 * ar + (s1 * br + s2 * bi);
        o.v[(0 + sp) * 2 + 1] += s3 * ai + (s1 * bi - s2 * br);
        o.v[(2 + sp) * 2] += (s1 * ar - s2 * ai) - s3 * br;
        o.v[(2 + sp) * 2 + 1] += (s1 * ai + s2 * ar) - s3 * bi;
    }
}

// The pion term at site n of a V-site lattice with pions pi[a * V + n] (a < 3);
// no-op for real sites or without pions.
template <typename R, int K>
__device__ __forceinline__ void pion_term(Site<R, K>& o, const Site<R, K>& c, const double* __restrict__ pi, int n,
                                          int V, double g, bool dag)
{
    if constexpr (K == 2) {
        if (pi) {
            const double sg = dag ? -g : g;
            pion_add<R>(o, c, (R)(sg * pi[n]), (R)(sg * pi[V + n]), (R)(sg * pi[2 * V + n]));
        }
    }
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (J. Salmon et al., "Parallel random numbers: as easy as
// 1, 2, 3", SC'11) with the framework's counter scheme:
//   key = (seed_lo, seed_hi ^ chain), ctr = (pair index, step_lo, step_hi, kind<<24 | rhs)
// Each counter yields two 52-bit uniforms and, by Box-Muller, two normals.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        if (i > 0) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x;
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

__device__ __forceinline__ double u52(uint32_t hi, uint32_t lo)
{
    const uint64_t m = ((uint64_t)hi << 20) | (lo >> 12);
    return ((double)m + 0.5) * 0x1p-52;
}

struct RngStream {
    uint2 key;
    uint32_t c1, c2, c3;
};

__device__ __forceinline__ RngStream rng_stream(uint64_t seed, uint32_t chain, uint64_t step,
                                                uint32_t kind, uint32_t rhs)
{
    RngStream s;
    s.key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32) ^ chain);
    s.c1 = (uint32_t)step;
    s.c2 = (uint32_t)(step >> 32);
    s.c3 = (kind << 24) | (rhs & 0xFFFFFFu);
    return s;
}

// Normals 2e and 2e+1 of the stream.
__device__ __forceinline__ double2 normal_pair(const RngStream& s, uint32_t e)
{
    const uint4 o = philox4x32_10(make_uint4(e, s.c1, s.c2, s.c3), s.key);
    const double u1 = u52(o.x, o.y), u2 = u52(o.z, o.w);
    const double R = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    return make_double2(R * cs, R * sn);
}

// Fermion noise eta of one CG system at site n: real Gaussian entries from the
// Philox stream (seed, chain; step, kind, rhs), imaginary parts zero
// (FermionicDrift.cu:102-110).
template <int K>
__device__ __forceinline__ Site<double, K> eta_site_at(const SysDev& S, int n, int kind, int64_t step)
{
    const RngStream rs = rng_stream(S.seed, (uint32_t)S.chain, (uint64_t)step, (uint32_t)kind, (uint32_t)S.rhs);
    const double2 a = normal_pair(rs, (uint32_t)(2 * n));
    const double2 b = normal_pair(rs, (uint32_t)(2 * n + 1));
    Site<double, K> s;
    const double e[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        s.v[i * K] = e[i];
        if constexpr (K == 2) s.v[i * K + 1] = 0.0;
    }
    return s;
}

template <int K>
__device__ __forceinline__ Site<double, K> eta_site(const SysDev& S, int n, int kind)
{
    return eta_site_at<K>(S, n, kind, *S.step);
}

// eta of the step at site n (kind 2: the Langevin step's sources): from the
// buffer generated one step ahead when it holds this step, else generated
// here.  Both give the same bits (the same Philox stream and arithmetic).
template <int K>
__device__ __forceinline__ Site<double, K> eta_of_step(const SysDev& S, int n, int kind)
{
    const int64_t st = *S.step;
    if (kind == 2 && S.eta_tag && S.eta_tag[st & 1] == st) return load_site<double, K>(S.eta_ahead[st & 1], n);
    return eta_site_at<K>(S, n, kind, st);
}

// ---------------------------------------------------------------------------
// Reductions (fixed order => deterministic for a given block size).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block sum; result valid in thread 0.  scratch: >= 32 doubles.
__device__ __forceinline__ double block_sum(double a, double* scratch)
{
    a = warp_sum(a);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[w] = a;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = lane < nw ? scratch[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// Block sum of two values; result valid in thread 0.  scratch: >= 2*32 doubles.
__device__ __forceinline__ double2 block_sum2(double a, double b, double* scratch)
{
    a = warp_sum(a);
    b = warp_sum(b);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
        scratch[2 * w] = a;
        scratch[2 * w + 1] = b;
    }
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double x = lane < nw ? scratch[2 * lane] : 0.0;
        double y = lane < nw ? scratch[2 * lane + 1] : 0.0;
        x = warp_sum(x);
        y = warp_sum(y);
        r = make_double2(x, y);
    }
    return r;
}

__device__ __forceinline__ double block_max(double a, double* scratch)
{
    a = warp_max(a);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[w] = a;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = lane < nw ? scratch[lane] : 0.0;
        r = warp_max(r);
    }
    return r;
}

// Block max of non-negative IEEE bit patterns into *word (one atomic per block).
__device__ __forceinline__ void block_max_bits(unsigned long long b, unsigned long long* word)
{
    __shared__ unsigned long long s_max;
    if (threadIdx.x == 0) s_max = 0ull;
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned mh = __reduce_max_sync(full, hi);
    const unsigned ml = __reduce_max_sync(full, hi == mh ? lo : 0u);
    if ((threadIdx.x & 31) == 0) atomicMax(&s_max, ((unsigned long long)mh << 32) | ml);
    __syncthreads();
    if (threadIdx.x == 0 && s_max) atomicMax(word, s_max);
}

}  // namespace yk
