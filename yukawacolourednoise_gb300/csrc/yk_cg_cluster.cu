// yk_cg_cluster.cu -- the mixed-precision CG of one system inside one
// thread-block cluster (16 CTAs on 16 SMs of a GPC), for lattices whose
// search direction, D p and A p fit the cluster's shared memory (Nt / 16
// rounded up, times Nx, at most 4096 sites per CTA: 256 x 256 and smaller).
//
// The algorithm is the Hestenes-Stiefel CG of code/src/CGsolver.cu:72-170
// with the mixed-precision scheme of yk_cg.cu (FP32 vectors and stencils,
// float-float sums, |r_{k+1}|^2 from the expansion of |r_k - alpha A p_k|^2,
// FP64 reliable updates with re-orthogonalisation; convergence only on an
// FP64 residual).  What differs is where the data lives and how the parts
// synchronise:
//  * CTA c owns lattice rows [c R, c R + R), R = ceil(Nt / 16); its threads
//    hold r and the FP32 solution increment of their sites in registers, and
//    p, t = D_first p, A p and the FP32 diagonal in shared memory;
//  * the stencil reads the two neighbouring rows of the other CTAs through
//    distributed shared memory;
//  * phases are separated by the hardware cluster barrier (~600 cycles on
//    GB300, against ~1500-2000 for one round trip through L2), three per
//    iteration; no grid-wide synchronisation at all;
//  * every CTA reads the 16 CTA partial sums through distributed shared
//    memory, adds them in the same order and runs the same scalar recurrence,
//    so all CTAs take the same decisions without a broadcast.
// Systems of a batched launch are independent clusters (one per system).
//
// The right-hand side b = eta is drawn by a separate kernel spread over the
// whole GPU (its FP64 Box-Muller transform costs 1/64-rate instructions);
// the FP64 solution x, b and the FP64 scratch of the reliable updates live in
// global memory.
#include <cooperative_groups.h>

#include "yk_common.cuh"
#include "yk_kernels.h"

namespace cg = cooperative_groups;

#ifdef YK_CG_TIMING
#include <cstdio>
// Timing build: CTA 0 of the first cluster accumulates the clock cycles of
// each part of an iteration and prints the averages when the solve ends.
#define YK_CMARK(i)                                                       \
    do {                                                                  \
        if (blockIdx.x == 0 && threadIdx.x == 0) {                        \
            const long long t_ = clock64();                               \
            tacc[i] += t_ - tlast;                                        \
            tlast = t_;                                                   \
        }                                                                 \
    } while (0)
#else
#define YK_CMARK(i) \
    do {            \
    } while (0)
#endif

namespace yk {

namespace {

constexpr int kCC = 16;             // CTAs per cluster
constexpr int kCThreads = 512;      // threads per CTA
constexpr int kCSpt = 8;            // sites per thread
constexpr int kCMaxSites = kCThreads * kCSpt;   // sites per CTA (4096)

enum CMode { kCStep = 1, kCRu = 2, kCRedo = 3 };

// Scalar state of the system, identical in every CTA (thread 0 computes it).
struct CState {
    double rr, rr0, rr_prev, stop2, rmax2;
    float alpha, beta, c;
    int mode, iters, n_ru, status, converged, done;
};

// Per-CTA shared memory: the vectors, then the reduction scratch.
struct CShared {
    float4* p;
    float4* t;
    float4* ap;
    float* diag;
    float* wsum;    // 16 warps x 4 values
    float2* cpart;  // this CTA's four partial sums (float-float)
};

struct FFc {
    float hi, lo;
};

__device__ __forceinline__ FFc ffc_add(FFc a, FFc b)
{
    const float s = a.hi + b.hi;
    const float bp = s - a.hi;
    float e = (a.hi - (s - bp)) + (b.hi - bp);
    e += a.lo + b.lo;
    const float hi = s + e;
    return FFc{hi, e - (hi - s)};
}

__device__ __forceinline__ FFc ffc_of(double x)
{
    const float hi = (float)x;
    return FFc{hi, (float)(x - (double)hi)};
}

__device__ __forceinline__ FFc ffc_shfl(FFc a, int o)
{
    return FFc{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}

__device__ __forceinline__ Site<float, 1> s4(const float4& v)
{
    Site<float, 1> s;
    s.v[0] = v.x;
    s.v[1] = v.y;
    s.v[2] = v.z;
    s.v[3] = v.w;
    return s;
}

__device__ __forceinline__ float4 f4(const Site<float, 1>& s) { return make_float4(s.v[0], s.v[1], s.v[2], s.v[3]); }

// Lattice geometry of the system as seen by one CTA.
struct CGeo {
    int Nt, Nx, R;      // rows per CTA
    int row0, rows;     // this CTA's rows
    int L;              // this CTA's sites
    unsigned rank;
};

// The rows just above and below this CTA's rows, in the CTAs that own them
// (row 0 follows row Nt - 1): element 0 of each, as generic pointers into
// distributed shared memory, for one CTA-distributed buffer.
struct Halo {
    const float4* up;
    const float4* dn;
};

__device__ __forceinline__ Halo halo_of(const float4* buf, const CGeo& g, cg::cluster_group& cl)
{
    Halo h = {nullptr, nullptr};
    if (g.rows == 0) return h;
    const unsigned q_up = (g.row0 + g.rows == g.Nt) ? 0u : g.rank + 1;   // its local row 0
    const unsigned q_dn = (g.row0 == 0) ? (unsigned)((g.Nt - 1) / g.R) : g.rank - 1;
    const int dn_row = (g.row0 == 0) ? (g.Nt - 1) - (int)q_dn * g.R : g.R - 1;
    h.up = cl.map_shared_rank(buf, q_up);
    h.dn = cl.map_shared_rank(buf, q_dn) + dn_row * g.Nx;
    return h;
}

// FP32 stencil of a CTA-distributed buffer at local site l = (local row lr,
// column x); rows outside the CTA come from the halo pointers.
template <bool DAG>
__device__ __forceinline__ float4 stencil32(const float4* buf, const Halo& h, int l, int lr, int x, const CGeo& g,
                                            float diag, float r)
{
    const int t = g.row0 + lr;
    const float4 c = buf[l];
    const float4 xu = buf[l + (x + 1 == g.Nx ? 1 - g.Nx : 1)];
    const float4 xd = buf[l + (x == 0 ? g.Nx - 1 : -1)];
    float4 vu, vd;
    if (lr + 1 < g.rows)
        vu = buf[l + g.Nx];
    else
        vu = h.up[x];
    if (lr > 0)
        vd = buf[l - g.Nx];
    else
        vd = h.dn[x];
    const float sp = (t + 1 == g.Nt) ? -1.f : 1.f, sm = (t == 0) ? -1.f : 1.f;
    return f4(dirac_combine<float, 1, DAG>(s4(c), s4(vu), s4(vd), s4(xu), s4(xd), diag, r, sp, sm));
}

// FP64 site of a global buffer that other CTAs of the cluster wrote before the
// last cluster barrier (relaxed loads at gpu scope: served by L2).
__device__ __forceinline__ Site<double, 1> ld_site64(const double* p, int64_t n)
{
    Site<double, 1> s;
    const double2* q = reinterpret_cast<const double2*>(p + 4 * n);
    double2 a, b;
    asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(a.x), "=d"(a.y) : "l"(q) : "memory");
    asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(b.x), "=d"(b.y) : "l"(q + 1) : "memory");
    s.v[0] = a.x;
    s.v[1] = a.y;
    s.v[2] = b.x;
    s.v[3] = b.y;
    return s;
}

// FP64 stencil of a global buffer (reliable updates) at global site n.
template <bool DAG>
__device__ __forceinline__ Site<double, 1> stencil64(const double* buf, int n, const SysDev& S)
{
    const Nbr nb = neighbours(n, S.Nt, S.Nx);
    const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
    return dirac_combine<double, 1, DAG>(ld_site64(buf, n), ld_site64(buf, nb.tu), ld_site64(buf, nb.td),
                                         ld_site64(buf, nb.xu), ld_site64(buf, nb.xd), diag, S.r, (double)nb.sp,
                                         (double)nb.sm);
}

// CTA sums of four per-thread values -> this CTA's float-float partials:
// FP32 warp butterflies, the warps' sums added in float-float by warp 0.
__device__ void cta_partials(float v0, float v1, float v2, float v3, const CShared& sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float v[4] = {v0, v1, v2, v3};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 4; ++c) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < 4; ++c) sh.wsum[w * 4 + c] = v[c];
    __syncthreads();
    if (w == 0) {
        FFc f[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) f[c] = FFc{lane < nw ? sh.wsum[lane * 4 + c] : 0.f, 0.f};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < 4; ++c) f[c] = ffc_add(f[c], ffc_shfl(f[c], o));
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 4; ++c) sh.cpart[c] = make_float2(f[c].hi, f[c].lo);
    }
}

// FP64 per-thread values of a reliable update -> this CTA's partials
// (|r|^2 in slot 0, <r, p> in slot 2).
__device__ void cta_partials64(double v0, double v2, const CShared& sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    FFc f[2] = {ffc_of(v0), ffc_of(v2)};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 2; ++c) f[c] = ffc_add(f[c], ffc_shfl(f[c], o));
    float2* ws = reinterpret_cast<float2*>(sh.wsum);
    if (lane == 0) {
        ws[w * 2] = make_float2(f[0].hi, f[0].lo);
        ws[w * 2 + 1] = make_float2(f[1].hi, f[1].lo);
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int c = 0; c < 2; ++c) f[c] = lane < nw ? FFc{ws[lane * 2 + c].x, ws[lane * 2 + c].y} : FFc{0.f, 0.f};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < 2; ++c) f[c] = ffc_add(f[c], ffc_shfl(f[c], o));
        if (lane == 0) {
            sh.cpart[0] = make_float2(f[0].hi, f[0].lo);
            sh.cpart[1] = make_float2(0.f, 0.f);
            sh.cpart[2] = make_float2(f[1].hi, f[1].lo);
            sh.cpart[3] = make_float2(0.f, 0.f);
        }
    }
}

// After a cluster barrier: warp 0 of every CTA reads the 16 CTA partials
// through distributed shared memory and adds them in rank order (float-float
// butterfly, the same bits in every CTA); thread 0 runs the scalar recurrence.
__device__ void cluster_step(const CGArgs& a, const CShared& sh, cg::cluster_group& cl, CState& st, int k,
                             bool ru_round)
{
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        FFc f[4];
        if (lane < kCC) {
            const float2* rp = cl.map_shared_rank(sh.cpart, (unsigned)lane);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float2 q = rp[c];
                f[c] = FFc{q.x, q.y};
            }
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) f[c] = FFc{0.f, 0.f};
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < 4; ++c) f[c] = ffc_add(f[c], ffc_shfl(f[c], o));
        if (lane == 0) {
            double s[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) s[c] = (double)f[c].hi + (double)f[c].lo;
            const double rr = s[0];
            st.rr = rr;
            st.iters = k;
            if (ru_round) {
                // s[0] = |b - A x|^2 (FP64 residual), s[2] = <r, p_{k-1}>
                st.n_ru += 1;
                if (!isfinite(rr)) {
                    st.status = YK_ENAN;
                    st.done = 1;
                } else if (!(rr > st.stop2)) {
                    st.converged = 1;
                    st.done = 1;
                } else if (k >= a.max_iter) {
                    st.status = YK_ENOCONV;
                    st.done = 1;
                } else {
                    // p_k = r + beta (p_{k-1} - gamma r), gamma = <r, p_{k-1}> / |r|^2
                    const double beta = rr / st.rr_prev;
                    st.beta = (float)beta;
                    st.c = (float)(1.0 - beta * (s[2] / rr));
                    st.mode = kCRedo;
                    st.rmax2 = rr;
                }
            } else {
                // s: |r|^2, |Ap|^2, <p, Ap>, <r, Ap>
                if (k == 0) {
                    st.stop2 = (a.tol_mode == YK_TOL_ABS) ? a.tol * a.tol : a.tol * a.tol * rr;
                    st.rmax2 = rr;
                    st.rr0 = rr;
                }
                const float alpha = (float)rr / (float)s[2];
                if (!isfinite(rr)) {
                    st.status = YK_ENAN;
                    st.done = 1;
                } else if (k == 0 && !(rr > st.stop2)) {
                    st.converged = 1;   // x = 0 is exact
                    st.done = 1;
                } else if (k >= a.max_iter) {
                    st.status = YK_ENOCONV;
                    st.done = 1;
                } else if (!isfinite(alpha)) {
                    st.status = YK_ENAN;
                    st.done = 1;
                } else {
                    // |r - alpha q|^2 = |r|^2 - 2 alpha <r, q> + alpha^2 |q|^2
                    const double al = (double)alpha;
                    double est = rr - 2.0 * al * s[3] + al * al * s[1];
                    if (!(est > 0.0)) est = 0.0;
                    st.alpha = alpha;
                    st.beta = (float)est / (float)rr;
                    st.c = 1.f;
                    st.rr_prev = rr;
                    st.rmax2 = fmax(st.rmax2, rr);
                    const bool cand = !(rr > st.stop2) || !(est > st.stop2);
                    const bool drop = est < a.reliable_delta * a.reliable_delta * st.rmax2;
                    const bool due = a.reliable_every > 0 && (k + 1) % a.reliable_every == 0;
                    const bool cap = k + 1 >= a.max_iter;
                    st.mode = (cand || drop || due || cap) ? kCRu : kCStep;
                }
            }
        }
    }
    __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(kCThreads, 1) cg_cluster_kernel(CGArgs a)
{
    extern __shared__ __align__(16) unsigned char cg_smem[];
    __shared__ CState st;
    cg::cluster_group cl = cg::this_cluster();
    const int sys = a.sys_first + (int)(blockIdx.x / kCC);
    const SysDev& S = a.sys[sys];
    CGeo g;
    g.Nt = S.Nt;
    g.Nx = S.Nx;
    g.R = (S.Nt + kCC - 1) / kCC;
    g.rank = cl.block_rank();
    g.row0 = (int)g.rank * g.R;
    g.rows = max(0, min(g.R, g.Nt - g.row0));
    g.L = g.rows * g.Nx;
    CShared sh;
    {
        const int Lmax = g.R * g.Nx;   // the same in every CTA of the system
        float4* v = reinterpret_cast<float4*>(cg_smem);
        sh.p = v;
        sh.t = v + Lmax;
        sh.ap = v + 2 * Lmax;
        sh.diag = reinterpret_cast<float*>(v + 3 * Lmax);
        sh.wsum = sh.diag + ((Lmax + 3) & ~3);
        sh.cpart = reinterpret_cast<float2*>(sh.wsum + 64);
    }
    const bool first_dag = (a.mtype == YK_NORMAL);   // Normal: A = D D^dag, apply D^dag first
    const float rW = (float)S.r;
    const int n0 = g.row0 * g.Nx;   // first global site of the CTA

    // per-thread state: r and the FP32 solution increment of its sites
    // l = threadIdx.x + j * kCThreads (row l >> lgx, column l & (Nx - 1))
    float4 r[kCSpt], xs[kCSpt];
    const int lgx = __ffs(g.Nx) - 1;   // Nx is a power of two (cg_cluster_fits)
    const Halo hp = halo_of(sh.p, g, cl), ht = halo_of(sh.t, g, cl);

    // ---------------- round 0: r = p = b, x = 0
    if (threadIdx.x == 0) {
        st.rr = st.rr0 = st.rr_prev = st.stop2 = st.rmax2 = 0.0;
        st.alpha = st.beta = 0.f;
        st.c = 1.f;
        st.mode = kCStep;
        st.iters = st.n_ru = st.status = st.converged = st.done = 0;
    }
#pragma unroll
    for (int j = 0; j < kCSpt; ++j) {
        const int l = threadIdx.x + j * kCThreads;
        r[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        xs[j] = r[j];
        if (l < g.L) {
            const int n = n0 + l;
            const Site<double, 1> b = ld_site64(S.b, n);
            r[j] = make_float4((float)b.v[0], (float)b.v[1], (float)b.v[2], (float)b.v[3]);
            sh.p[l] = r[j];
            sh.diag[l] = (float)(2.0 * S.r + S.m0 + S.g * S.sigma[n]);
            double* x = S.x + 4 * (int64_t)n;
            x[0] = x[1] = x[2] = x[3] = 0.0;
        }
    }
    int k = 0;
#ifdef YK_CG_TIMING
    long long tacc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, tlast = clock64();
    int nit = 0;
#endif
    for (;;) {
        // ---------------- t = D_first p
        YK_CMARK(0);   // A pass / reliable update
        cl.sync();
        YK_CMARK(1);   // barrier
#pragma unroll 2
        for (int j = 0; j < kCSpt; ++j) {
            const int l = threadIdx.x + j * kCThreads;
            if (l < g.L)
                sh.t[l] = first_dag ? stencil32<true>(sh.p, hp, l, l >> lgx, l & (g.Nx - 1), g, sh.diag[l], rW)
                                    : stencil32<false>(sh.p, hp, l, l >> lgx, l & (g.Nx - 1), g, sh.diag[l], rW);
        }
        YK_CMARK(2);   // T pass
        cl.sync();
        YK_CMARK(1);
        // ---------------- A p = D_second t; |r|^2, |Ap|^2, <p,Ap>, <r,Ap>
        float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f;
#pragma unroll
        for (int j = 0; j < kCSpt; ++j) {
            const int l = threadIdx.x + j * kCThreads;
            if (l < g.L) {
                const float4 ap = first_dag
                    ? stencil32<false>(sh.t, ht, l, l >> lgx, l & (g.Nx - 1), g, sh.diag[l], rW)
                    : stencil32<true>(sh.t, ht, l, l >> lgx, l & (g.Nx - 1), g, sh.diag[l], rW);
                sh.ap[l] = ap;
                const float4 p = sh.p[l], rr = r[j];
                v0 = fmaf(rr.x, rr.x, fmaf(rr.y, rr.y, fmaf(rr.z, rr.z, fmaf(rr.w, rr.w, v0))));
                v1 = fmaf(ap.x, ap.x, fmaf(ap.y, ap.y, fmaf(ap.z, ap.z, fmaf(ap.w, ap.w, v1))));
                v2 = fmaf(p.x, ap.x, fmaf(p.y, ap.y, fmaf(p.z, ap.z, fmaf(p.w, ap.w, v2))));
                v3 = fmaf(rr.x, ap.x, fmaf(rr.y, ap.y, fmaf(rr.z, ap.z, fmaf(rr.w, ap.w, v3))));
            }
        }
        YK_CMARK(3);   // B pass
        cta_partials(v0, v1, v2, v3, sh);
        YK_CMARK(4);   // CTA partials
        cl.sync();
        YK_CMARK(1);
        cluster_step(a, sh, cl, st, k, false);
        YK_CMARK(5);   // cluster sums + scalars
#ifdef YK_CG_TIMING
        ++nit;
#endif
        if (st.done) break;
        ++k;
        if (st.mode == kCRu) {
            // ---------------- reliable update: x = x + xs + alpha p (FP64), xs = 0
            const double al = (double)st.alpha;
#pragma unroll
            for (int j = 0; j < kCSpt; ++j) {
                const int l = threadIdx.x + j * kCThreads;
                if (l < g.L) {
                    double* x = S.x + 4 * (int64_t)(n0 + l);
                    const float4 p = sh.p[l];
                    x[0] += (double)xs[j].x + al * (double)p.x;
                    x[1] += (double)xs[j].y + al * (double)p.y;
                    x[2] += (double)xs[j].z + al * (double)p.z;
                    x[3] += (double)xs[j].w + al * (double)p.w;
                    xs[j] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            cl.sync();
            // t64 = D_first x
#pragma unroll
            for (int j = 0; j < kCSpt; ++j) {
                const int l = threadIdx.x + j * kCThreads;
                if (l < g.L) {
                    const int n = n0 + l;
                    const Site<double, 1> t = first_dag ? stencil64<true>(S.x, n, S) : stencil64<false>(S.x, n, S);
                    double* o = S.t64 + 4 * (int64_t)n;
                    o[0] = t.v[0];
                    o[1] = t.v[1];
                    o[2] = t.v[2];
                    o[3] = t.v[3];
                }
            }
            cl.sync();
            // r = b - D_second t64 (FP64); |r|^2, <r, p_{k-1}>
            double w0 = 0.0, w2 = 0.0;
#pragma unroll
            for (int j = 0; j < kCSpt; ++j) {
                const int l = threadIdx.x + j * kCThreads;
                if (l < g.L) {
                    const int n = n0 + l;
                    const Site<double, 1> ax = first_dag ? stencil64<false>(S.t64, n, S) : stencil64<true>(S.t64, n, S);
                    const Site<double, 1> b = ld_site64(S.b, n);
                    const float4 p = sh.p[l];
                    const double e0 = b.v[0] - ax.v[0], e1 = b.v[1] - ax.v[1], e2 = b.v[2] - ax.v[2],
                                 e3 = b.v[3] - ax.v[3];
                    w0 += e0 * e0 + e1 * e1 + e2 * e2 + e3 * e3;
                    w2 += e0 * (double)p.x + e1 * (double)p.y + e2 * (double)p.z + e3 * (double)p.w;
                    r[j] = make_float4((float)e0, (float)e1, (float)e2, (float)e3);
                }
            }
            cta_partials64(w0, w2, sh);
            cl.sync();
            cluster_step(a, sh, cl, st, k, true);
            if (st.done) break;
            // p = c r + beta p  (st.mode == kCRedo)
            const float be = st.beta, c = st.c;
#pragma unroll
            for (int j = 0; j < kCSpt; ++j) {
                const int l = threadIdx.x + j * kCThreads;
                if (l < g.L) {
                    const float4 p = sh.p[l];
                    sh.p[l] = make_float4(fmaf(be, p.x, c * r[j].x), fmaf(be, p.y, c * r[j].y),
                                          fmaf(be, p.z, c * r[j].z), fmaf(be, p.w, c * r[j].w));
                }
            }
            YK_CMARK(6);   // reliable update
        } else {
            // ---------------- r -= alpha Ap, xs += alpha p, p = r + beta p
            const float al = st.alpha, be = st.beta;
#pragma unroll
            for (int j = 0; j < kCSpt; ++j) {
                const int l = threadIdx.x + j * kCThreads;
                if (l < g.L) {
                    const float4 ap = sh.ap[l], p = sh.p[l];
                    float4 rr = r[j];
                    rr.x = fmaf(-al, ap.x, rr.x);
                    rr.y = fmaf(-al, ap.y, rr.y);
                    rr.z = fmaf(-al, ap.z, rr.z);
                    rr.w = fmaf(-al, ap.w, rr.w);
                    r[j] = rr;
                    xs[j].x = fmaf(al, p.x, xs[j].x);
                    xs[j].y = fmaf(al, p.y, xs[j].y);
                    xs[j].z = fmaf(al, p.z, xs[j].z);
                    xs[j].w = fmaf(al, p.w, xs[j].w);
                    sh.p[l] = make_float4(fmaf(be, p.x, rr.x), fmaf(be, p.y, rr.y), fmaf(be, p.z, rr.z),
                                          fmaf(be, p.w, rr.w));
                }
            }
        }
    }
#ifdef YK_CG_TIMING
    if (blockIdx.x == 0 && threadIdx.x == 0 && nit > 0)
        printf("cluster cg timing (cycles per iteration over %d): A %lld  barriers %lld  T %lld  B %lld  "
               "partials %lld  step %lld | reliable updates %d, %lld cycles each\n", nit, tacc[0] / nit,
               tacc[1] / nit, tacc[2] / nit, tacc[3] / nit, tacc[4] / nit, tacc[5] / nit, st.n_ru,
               st.n_ru ? tacc[6] / st.n_ru : 0ll);
#endif
    // x is complete: convergence is declared only after a reliable update
    // folded the increment (or at k = 0, where x = 0 is exact)
    if (g.rank == 0 && threadIdx.x == 0) {
        CGState& o = a.st[sys];
        o.rr = st.rr;
        o.rr0 = st.rr0;
        o.rr_prev = st.rr_prev;
        o.stop2 = st.stop2;
        o.rmax2 = st.rmax2;
        o.active = 0;
        o.iters = st.iters;
        o.converged = st.converged;
        o.status = st.status;
        o.n_ru = st.n_ru;
        o.mode = 0;
        o.chi_ready = 0;   // its reliable updates keep D x in shared memory
    }
    cl.sync();   // no CTA leaves while others may still read its shared memory
}

// b = eta (Philox stream `kind`) for every site of the systems of the tiles.
__global__ void __launch_bounds__(kTile) eta_kernel(const SysDev* __restrict__ sys, const int2* __restrict__ tiles,
                                                    int kind)
{
    const int2 tl = tiles[blockIdx.x];
    const SysDev& S = sys[tl.x];
    const int n = tl.y + threadIdx.x;
    if (n >= S.V) return;
    store_site<double, 1>(S.b, n, eta_site<1>(S, n, kind));
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static size_t cluster_smem(int max_sites)
{
    // p, t, Ap (float4) + diag (float, padded to 4) + 64 warp sums + 4 float2
    return (size_t)max_sites * 3 * sizeof(float4) + (size_t)((max_sites + 3) & ~3) * sizeof(float) +
           64 * sizeof(float) + 4 * sizeof(float2);
}

bool cg_cluster_fits(int Nt, int Nx)
{
    const int R = (Nt + kCC - 1) / kCC;
    return Nx >= 1 && (Nx & (Nx - 1)) == 0 && (int64_t)R * Nx <= kCMaxSites;
}

// Opt in to 16-CTA clusters and the shared memory of the largest case, and
// check that at least one such cluster can be resident (call before capture).
bool cg_cluster_init()
{
    static int ok = -1;
    if (ok >= 0) return ok == 1;
    ok = 0;
    const size_t smem = cluster_smem(kCMaxSites);
    if (cudaFuncSetAttribute(cg_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(cg_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCC);
    cfg.blockDim = dim3(kCThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kCC;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, cg_cluster_kernel, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ok = n >= 1 ? 1 : 0;
    return ok == 1;
}

cudaError_t launch_eta(const SysDev* sys, const int2* tiles, int ntiles, int kind, cudaStream_t stream)
{
    if (ntiles <= 0) return cudaSuccess;
    eta_kernel<<<ntiles, kTile, 0, stream>>>(sys, tiles, kind);
    return cudaGetLastError();
}

// One cluster per system of [sys_first, sys_first + sys_count); max_sites =
// the largest CTA share (rows per CTA x Nx) over those systems.
cudaError_t launch_cg_cluster(const CGArgs& a, int max_sites, cudaStream_t stream)
{
    if (a.sys_count <= 0) return cudaSuccess;
    if (max_sites > kCMaxSites || max_sites < 1) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCC * a.sys_count);
    cfg.blockDim = dim3(kCThreads);
    cfg.dynamicSmemBytes = cluster_smem(max_sites);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kCC;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, cg_cluster_kernel, a);
}

}  // namespace yk
