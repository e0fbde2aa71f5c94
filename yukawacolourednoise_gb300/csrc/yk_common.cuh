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
// Both flavours and every real plane see the same real coefficients.  The
// space hops are gathered before their coefficients: the up and down
// neighbours share r / 2 on the same component and take -+1/2 on the other
// (sigma_1), so each output component costs one multiply, four FMAs and two
// adds (GB300's FP64 rate is 1/64 of its FP32 rate: the FP64 applications of
// the reliable updates and the force pay per operation).
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
    // space hops: -1/2 [(r -+ s1) psi(n+x) + (r +- s1) psi(n-x)] (D: upper sign)
    //   = -r/2 (psi(n+x) + psi(n-x)) + sx/2 s1 (psi(n+x) - psi(n-x)),  sx = +1 for D
    const R a = -h * r;
    const R bx = DAG ? -h : h;
#pragma unroll
    for (int f = 0; f < 2; ++f) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int iu = (2 * f) * K + k, id = (2 * f + 1) * K + k;
            R ou = diag * c.v[iu];
            R od = diag * c.v[id];
            ou = fma(cu_up, tu.v[iu], ou);
            od = fma(cd_up, tu.v[id], od);
            ou = fma(cu_dn, td.v[iu], ou);
            od = fma(cd_dn, td.v[id], od);
            ou = fma(bx, xu.v[id] - xd.v[id], ou);
            od = fma(bx, xu.v[iu] - xd.v[iu], od);
            ou = fma(a, xu.v[iu] + xd.v[iu], ou);
            od = fma(a, xu.v[id] + xd.v[id], od);
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
//   key = (seed_lo, seed_hi ^ chain), ctr = (index, step_lo, step_hi, kind<<24 | rhs)
// Each counter yields two 52-bit uniforms (the initial fields) or four
// normals (the noise and the sources).
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

// ---------------------------------------------------------------------------
// Gaussian normals: Box-Muller in FP32 arithmetic, every operation an IEEE
// round-to-nearest intrinsic (no contraction), so that the oracle's C
// restatement (fmaf, -ffp-contract=off) gives the same bits.  GB300 runs FP64
// at 1/64 of its FP32 rate, and an FP64 log + sincospi per pair made the
// sources and the white noise a sizeable part of a step.
// Normals 4e .. 4e+3 of a stream come from counter e: pair 0 from words
// (x, y), pair 1 from (z, w); a pair (a, b) is
//   R = sqrt(2 E), E = -ln u, u = (a + 1/2) 2^-32;   angle 2 pi (b + 1/2) 2^-32;
//   (R cos, R sin).
// ln: u < 1/2 is split into 2^e m (m in [sqrt 1/2, sqrt 2)); u >= 1/2 goes
// through w = 1 - u = (~a + 1/2) 2^-32, exact from the complemented word, so
// that small radii keep their resolution.  ln(1 + f) = 2 atanh(f / (2 + f))
// by its Taylor series to s^9 (|s| <= 0.1716: truncation below 2e-9).
// sin and cos of 2 pi y, |y| <= 1/8 turn, by their Taylor series (to y^9 and
// y^10, truncation below 3e-9), the quadrant from the word's top bits.
// Accuracy: a few FP32 ulps against the exact transform of the same words;
// the largest |normal| is 6.76 (u = 2^-33).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float nm_log1p_core(float f)   // ln(1 + f), f in [-0.293, 0.415]
{
    const float s = __fdiv_rn(f, __fadd_rn(2.0f, f));
    const float t = __fmul_rn(2.0f, s);
    const float z = __fmul_rn(s, s);
    float p = __fmaf_rn(z, 0x1.c71c72p-4f, 0x1.24924ap-3f);   // 1/9, 1/7
    p = __fmaf_rn(z, p, 0x1.99999ap-3f);                       // 1/5
    p = __fmaf_rn(z, p, 0x1.555556p-2f);                       // 1/3
    return __fmaf_rn(__fmul_rn(t, z), p, t);
}

__device__ __forceinline__ float nm_neglog(uint32_t a)   // -ln((a + 1/2) 2^-32)
{
    constexpr float kLn2Hi = 0x1.62e4p-1f, kLn2Lo = 0x1.7f7d1cp-20f;   // ln 2 = hi + lo
    if (a < 0x80000000u) {
        const float u = __fmul_rn(__uint2float_rn(2u * a + 1u), 0x1p-33f);
        uint32_t bits = __float_as_uint(u);
        int e = (int)(bits >> 23) - 127;
        float m = __uint_as_float((bits & 0x007FFFFFu) | 0x3F800000u);
        if (m > 0x1.6a09e6p+0f) {
            m = __fmul_rn(m, 0.5f);
            e += 1;
        }
        const float L = nm_log1p_core(__fsub_rn(m, 1.0f));
        const float fe = __int2float_rn(e);
        return -__fmaf_rn(fe, kLn2Hi, __fmaf_rn(fe, kLn2Lo, L));
    }
    const float w = __fmul_rn(__uint2float_rn(2u * ~a + 1u), 0x1p-33f);   // 1 - u
    if (w <= 0x1.2bec34p-2f) return -nm_log1p_core(-w);                  // w <= 1 - sqrt 1/2
    return __fadd_rn(__fsub_rn(kLn2Hi, nm_log1p_core(__fsub_rn(1.0f, __fmul_rn(2.0f, w)))), kLn2Lo);
}

__device__ __forceinline__ float2 nm_pair(uint32_t a, uint32_t b)
{
    const float R = __fsqrt_rn(__fmul_rn(2.0f, nm_neglog(a)));
    const uint32_t j = (b + 0x20000000u) >> 30;            // nearest quarter turn
    const int d = (int)(b - (j << 30));                    // in [-2^29, 2^29)
    const float y = __fmul_rn(__int2float_rn(2 * d + 1), 0x1p-33f);
    const float y2 = __fmul_rn(y, y);
    // (2 pi)^k / k! with alternating signs
    float sp = __fmaf_rn(y2, 0x1.507834p+5f, -0x1.32d2ccp+6f);
    sp = __fmaf_rn(y2, sp, 0x1.466bc6p+6f);
    sp = __fmaf_rn(y2, sp, -0x1.4abbcep+5f);
    sp = __fmaf_rn(y2, sp, 0x1.921fb6p+2f);
    const float sn = __fmul_rn(y, sp);
    float cp = __fmaf_rn(y2, -0x1.a6d1f2p+4f, 0x1.e1f506p+5f);
    cp = __fmaf_rn(y2, cp, -0x1.55d3c8p+6f);
    cp = __fmaf_rn(y2, cp, 0x1.03c1f0p+6f);
    cp = __fmaf_rn(y2, cp, -0x1.3bd3ccp+4f);
    const float cs = __fmaf_rn(y2, cp, 1.0f);
    float c, s;
    if (j == 0) {
        c = cs;
        s = sn;
    } else if (j == 1) {
        c = -sn;
        s = cs;
    } else if (j == 2) {
        c = -cs;
        s = -sn;
    } else {
        c = sn;
        s = -cs;
    }
    return make_float2(__fmul_rn(R, c), __fmul_rn(R, s));
}

// Normals 4e .. 4e+3 of the stream.
__device__ __forceinline__ float4 normal4(const RngStream& s, uint32_t e)
{
    const uint4 o = philox4x32_10(make_uint4(e, s.c1, s.c2, s.c3), s.key);
    const float2 p = nm_pair(o.x, o.y), q = nm_pair(o.z, o.w);
    return make_float4(p.x, p.y, q.x, q.y);
}

// Normal i of the stream.
__device__ __forceinline__ double normal_at(const RngStream& s, uint32_t i)
{
    const float4 z = normal4(s, i >> 2);
    const int c = (int)(i & 3u);
    return (double)(c == 0 ? z.x : c == 1 ? z.y : c == 2 ? z.z : z.w);
}

// Fermion noise eta of one CG system at site n: real Gaussian entries from the
// Philox stream (seed, chain; step, kind, rhs), imaginary parts zero
// (FermionicDrift.cu:102-110).
template <int K>
__device__ __forceinline__ Site<double, K> eta_site_at(const SysDev& S, int n, int kind, int64_t step)
{
    const RngStream rs = rng_stream(S.seed, (uint32_t)S.chain, (uint64_t)step, (uint32_t)kind, (uint32_t)S.rhs);
    const float4 z = normal4(rs, (uint32_t)n);   // normals 4n .. 4n + 3
    Site<double, K> s;
    const double e[4] = {z.x, z.y, z.z, z.w};
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

// The step's drift at site n of chain C given the fermion force F: F plus
// the bosonic drift phi (m^2 + lambda/6 phi^2) - Lap phi of
// langevin_gpu_v2.cu:9-27, the Laplacian summed over its five columns in
// ascending site order (the reference's CSR rows).
__device__ __forceinline__ void cswap(int& a, int& b)
{
    const int lo = min(a, b), hi = max(a, b);
    a = lo;
    b = hi;
}

__device__ __forceinline__ double step_drift(const ChainDev& C, int n, double F)
{
    const Nbr nb = neighbours(n, C.Nt, C.Nx);
    const double v = C.phi[n];
    double d = F;
    d += v * (C.m2 + C.lambda6 * (v * v));
    int col[5] = {n, (int)nb.tu, (int)nb.td, (int)nb.xu, (int)nb.xd};
    // 5-input sorting network (9 comparators)
    cswap(col[0], col[1]); cswap(col[3], col[4]); cswap(col[2], col[4]);
    cswap(col[2], col[3]); cswap(col[0], col[3]); cswap(col[0], col[2]);
    cswap(col[1], col[4]); cswap(col[1], col[3]); cswap(col[1], col[2]);
    double lap = 0.0;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const double f = C.phi[col[q]];
        lap += col[q] != n ? f : -4.0 * f;   // the CSR row's weights 1 and -4 (the product by 1 is exact)
    }
    return d - lap;
}

}  // namespace yk
