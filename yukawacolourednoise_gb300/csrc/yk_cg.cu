// yk_cg.cu -- batched CG on D^dag D (or D D^dag) as one persistent
// cooperative kernel per solve.
//
// Follows the algorithm of code/src/CGsolver.cu:72-170 (x0 = 0, r = p = b,
// alpha = |r|^2 / <p, A p>, x += alpha p, r -= alpha A p, beta = |r'|^2/|r|^2,
// p = r + beta p; stop when sqrt(|r|^2) <= tol), restructured for GB300:
//   * one launch solves every (chain, rhs) system of a context; sites are cut
//     into tiles and a bounded grid barrier separates the three phases of an
//     iteration (the reference pays 15 grid syncs per iteration);
//   * p_{k+1} = r + beta p_k is never a separate pass: the D apply of the next
//     iteration forms it on the fly (double-buffered p);
//   * dot products are deterministic: per-tile partials are summed in tile
//     order by the last tile to finish (no floating-point atomics);
//   * MIXED: FP32 vectors and stencil, FP64 partial sums, and every
//     `reliable_every` iterations (or when the FP32 residual claims
//     convergence) an FP64 reliable update x += xs, r = b - A x.  Convergence
//     is only declared on the FP64 true residual.
#include <type_traits>

#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

namespace {

enum Phase { PH_INIT = 0, PH_ALPHA = 1, PH_BETA = 2, PH_RU = 3 };

__device__ __forceinline__ void deactivate(const CGArgs& a, volatile CGState& s, int converged, int status)
{
    s.active = 0;
    s.converged = converged;
    if (status) s.status = status;
    atomicSub(a.n_active, 1);
}

// Runs in one thread: turns the summed partials of system `s` into the
// scalars the next phase needs.
template <bool MIXED>
__device__ void finalize(const CGArgs& a, int sys, int ph, double x, double y)
{
    // volatile: other SMs finalised this system in earlier phases
    volatile CGState& s = a.st[sys];
    if (ph == PH_INIT) {
        s.rr = x;
        s.rr0 = x;
        s.rr_prev = x;
        s.stop = (a.tol_mode == YK_TOL_ABS) ? a.tol : a.tol * sqrt(x);
        s.iters = 0;
        s.n_ru = 0;
        s.ru = 0;
        s.last = 0;
        s.status = 0;
        s.beta = 0.0;
        s.active = 1;
        s.converged = 0;
        if (!isfinite(x)) deactivate(a, s, 0, YK_ENAN);
        else if (!(sqrt(x) > s.stop)) deactivate(a, s, 1, 0);
        else if (a.max_iter <= 0) deactivate(a, s, 0, YK_ENOCONV);
    } else if (ph == PH_ALPHA) {
        // alpha = rr / (x + i y), Smith's complex division
        const double c = x, d = y, num = s.rr;
        double ar, ai;
        if (fabs(c) >= fabs(d)) {
            const double q = d / c, den = c + d * q;
            ar = num / den;
            ai = (-num * q) / den;
        } else {
            const double q = c / d, den = c * q + d;
            ar = (num * q) / den;
            ai = -num / den;
        }
        s.alpha_re = ar;
        s.alpha_im = ai;
        if (!isfinite(ar) || !isfinite(ai)) deactivate(a, s, 0, YK_ENAN);
    } else if (ph == PH_BETA) {
        const double rr = x;
        s.iters += 1;
        s.beta = rr / s.rr;
        s.rr_prev = s.rr;
        s.rr = rr;
        if (!isfinite(rr)) {
            deactivate(a, s, 0, YK_ENAN);
        } else if (!MIXED) {
            if (!(sqrt(rr) > s.stop)) deactivate(a, s, 1, 0);
            else if (s.iters >= a.max_iter) deactivate(a, s, 0, YK_ENOCONV);
        } else {
            const bool cand = !(sqrt(rr) > s.stop);
            const bool due = a.reliable_every > 0 && (s.iters % a.reliable_every) == 0;
            const bool cap = s.iters >= a.max_iter;
            if (cand || due || cap) {
                s.ru = 1;
                s.last = cap ? 1 : 0;
                atomicOr(a.any_ru, 1);
            }
        }
    } else {  // PH_RU: x holds |b - A x|^2 in FP64
        const double rt = x;
        s.n_ru += 1;
        s.ru = 0;
        if (!isfinite(rt)) {
            deactivate(a, s, 0, YK_ENAN);
        } else if (!(sqrt(rt) > s.stop)) {
            s.rr = rt;
            deactivate(a, s, 1, 0);
        } else if (s.last) {
            s.rr = rt;
            deactivate(a, s, 0, YK_ENOCONV);
        } else {
            s.beta = rt / s.rr_prev;
            s.rr = rt;
        }
    }
    __threadfence();
}

// Publishes the block's partial of `tile`; the last tile of the system sums
// all partials of the system in tile order and finalises.
template <bool MIXED>
__device__ __forceinline__ void tile_reduce(const CGArgs& a, int tile, int sys, const SysDev& S,
                                            double2 v, int ph, volatile int* s_last)
{
    if (threadIdx.x == 0) {
        a.partial[tile] = v;
        __threadfence();
        const unsigned prev = atomicAdd(&a.st[sys].counter, 1u);
        *s_last = (prev == (unsigned)S.ntiles - 1) ? 1 : 0;
    }
    __syncthreads();
    if (*s_last) {
        if (threadIdx.x < 32) {
            __threadfence();
            const int lane = threadIdx.x;
            double x = 0.0, y = 0.0;
            for (int i = lane; i < S.ntiles; i += 32) {
                const double2 p = __ldcg(a.partial + S.tile0 + i);
                x += p.x;
                y += p.y;
            }
            x = warp_sum(x);
            y = warp_sum(y);
            if (lane == 0) {
                *(volatile unsigned*)&a.st[sys].counter = 0;
                finalize<MIXED>(a, sys, ph, x, y);
            }
        }
    }
    __syncthreads();
}

__device__ __forceinline__ int st_active(const CGArgs& a, int sys)
{
    return *(volatile int*)&a.st[sys].active;
}

__device__ __forceinline__ double st_load(const double* p) { return *(volatile const double*)p; }

// p_k at site m: p_0 = b (already stored), p_k = r + beta p_{k-1}.
template <typename W, int K>
__device__ __forceinline__ Site<W, K> p_at(const W* r, const W* pold, int64_t m, W beta, bool fresh)
{
    Site<W, K> po = load_site_cg<W, K>(pold, m);
    if (fresh) return po;
    const Site<W, K> rv = load_site_cg<W, K>(r, m);
#pragma unroll
    for (int i = 0; i < 4 * K; ++i) po.v[i] = fma(beta, po.v[i], rv.v[i]);
    return po;
}

template <typename W, int K, bool DAG>
__device__ __forceinline__ Site<W, K> apply_site(const Site<W, K>& c, const Site<W, K>& tu,
                                                 const Site<W, K>& td, const Site<W, K>& xu,
                                                 const Site<W, K>& xd, W diag, W r, const Nbr& nb)
{
    return dirac_combine<W, K, DAG>(c, tu, td, xu, xd, diag, r, (W)nb.sp, (W)nb.sm);
}

template <typename W, int K>
__device__ __forceinline__ Site<W, K> apply_d(const W* in, int n, const SysDev& S, bool dag,
                                              bool cg_loads)
{
    const Nbr nb = neighbours(n, S.Nt, S.Nx);
    Site<W, K> c, tu, td, xu, xd;
    if (cg_loads) {
        c = load_site_cg<W, K>(in, n);
        tu = load_site_cg<W, K>(in, nb.tu);
        td = load_site_cg<W, K>(in, nb.td);
        xu = load_site_cg<W, K>(in, nb.xu);
        xd = load_site_cg<W, K>(in, nb.xd);
    } else {
        c = load_site<W, K>(in, n);
        tu = load_site<W, K>(in, nb.tu);
        td = load_site<W, K>(in, nb.td);
        xu = load_site<W, K>(in, nb.xu);
        xd = load_site<W, K>(in, nb.xd);
    }
    const W diag = (W)(2.0 * S.r + S.m0 + S.g * S.sigma[n]);
    const W r = (W)S.r;
    return dag ? apply_site<W, K, true>(c, tu, td, xu, xd, diag, r, nb)
               : apply_site<W, K, false>(c, tu, td, xu, xd, diag, r, nb);
}

// Re and Im of sum conj(a) b over one site.
template <typename W, int K>
__device__ __forceinline__ double2 site_dot(const Site<W, K>& a, const Site<W, K>& b)
{
    W re = 0, im = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if constexpr (K == 1) {
            re = fma(a.v[e], b.v[e], re);
        } else {
            const W ar = a.v[2 * e], ai = a.v[2 * e + 1], br = b.v[2 * e], bi = b.v[2 * e + 1];
            re = fma(ar, br, fma(ai, bi, re));
            im = fma(ar, bi, fma(-ai, br, im));
        }
    }
    return make_double2((double)re, (double)im);
}

// y += (ar + i ai) * v
template <typename W, int K>
__device__ __forceinline__ void site_axpy(Site<W, K>& y, W ar, W ai, const Site<W, K>& v)
{
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if constexpr (K == 1) {
            y.v[e] = fma(ar, v.v[e], y.v[e]);
        } else {
            const W vr = v.v[2 * e], vi = v.v[2 * e + 1];
            y.v[2 * e] = fma(ar, vr, fma(-ai, vi, y.v[2 * e]));
            y.v[2 * e + 1] = fma(ar, vi, fma(ai, vr, y.v[2 * e + 1]));
        }
    }
}

template <int K>
__device__ __forceinline__ Site<double, K> eta_site(const SysDev& S, int n, int kind)
{
    // real Gaussian entries, imaginary parts zero (FermionicDrift.cu:102-110)
    const RngStream rs = rng_stream(S.seed, (uint32_t)S.chain, (uint64_t)(*S.step), (uint32_t)kind,
                                    (uint32_t)S.rhs);
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

}  // namespace

template <int K, bool MIXED>
__global__ void __launch_bounds__(kBlock) cg_kernel(CGArgs a)
{
    using W = typename std::conditional<MIXED, float, double>::type;
    __shared__ double red[64];
    __shared__ int s_last;
    const unsigned nb = gridDim.x;
    const bool first_dag = (a.mtype == YK_NORMAL);   // Normal: A = D D^dag, apply D^dag first

    // ---------------- init: x = 0, r = p_0 = b, |b|^2
    for (int tile = a.tile_begin + blockIdx.x; tile < a.tile_end; tile += nb) {
        const int2 td = a.tiles[tile];
        const SysDev& S = a.sys[td.x];
        const int n = td.y + threadIdx.x;
        double pr = 0.0;
        if (n < S.V) {
            Site<double, K> bv = S.gen_eta ? eta_site<K>(S, n, a.eta_kind) : load_site<double, K>(S.b, n);
            if (S.gen_eta) store_site<double, K>(S.b, n, bv);
            Site<double, K> z;
#pragma unroll
            for (int i = 0; i < 4 * K; ++i) {
                z.v[i] = 0.0;
                pr = fma(bv.v[i], bv.v[i], pr);
            }
            store_site<double, K>(S.x, n, z);
            if constexpr (MIXED) {
                Site<float, K> bf, zf;
#pragma unroll
                for (int i = 0; i < 4 * K; ++i) {
                    bf.v[i] = (float)bv.v[i];
                    zf.v[i] = 0.f;
                }
                store_site<float, K>(S.r32, n, bf);
                store_site<float, K>(S.p32[0], n, bf);
                store_site<float, K>(S.xs32, n, zf);
            } else {
                store_site<double, K>(S.r64, n, bv);
                store_site<double, K>(S.p64[0], n, bv);
            }
        }
        const double2 v = block_sum2(pr, 0.0, red);
        tile_reduce<MIXED>(a, tile, td.x, S, v, PH_INIT, &s_last);
    }
    if (!grid_sync(a.bar, nb, a.err)) return;

    for (int k = 0; k <= a.max_iter + 1; ++k) {
        if (*(volatile int*)a.n_active == 0) break;
        const bool fresh = (k == 0);
        const int cur = k & 1, prv = (k + 1) & 1;

        // ---------------- phase 1: p_k (on the fly) and t = D_first p_k
        for (int tile = a.tile_begin + blockIdx.x; tile < a.tile_end; tile += nb) {
            const int2 td = a.tiles[tile];
            if (!st_active(a, td.x)) continue;
            const SysDev& S = a.sys[td.x];
            const int n = td.y + threadIdx.x;
            if (n >= S.V) continue;
            const W beta = (W)st_load(&a.st[td.x].beta);
            const W* rv;
            const W* pold;
            W* pnew;
            W* tv;
            if constexpr (MIXED) {
                rv = S.r32; pold = S.p32[fresh ? 0 : prv]; pnew = S.p32[cur]; tv = S.t32;
            } else {
                rv = S.r64; pold = S.p64[fresh ? 0 : prv]; pnew = S.p64[cur]; tv = S.t64;
            }
            const Nbr nbr = neighbours(n, S.Nt, S.Nx);
            const Site<W, K> c = p_at<W, K>(rv, pold, n, beta, fresh);
            const Site<W, K> tu = p_at<W, K>(rv, pold, nbr.tu, beta, fresh);
            const Site<W, K> tdn = p_at<W, K>(rv, pold, nbr.td, beta, fresh);
            const Site<W, K> xu = p_at<W, K>(rv, pold, nbr.xu, beta, fresh);
            const Site<W, K> xd = p_at<W, K>(rv, pold, nbr.xd, beta, fresh);
            const W diag = (W)(2.0 * S.r + S.m0 + S.g * S.sigma[n]);
            const Site<W, K> o = first_dag
                ? apply_site<W, K, true>(c, tu, tdn, xu, xd, diag, (W)S.r, nbr)
                : apply_site<W, K, false>(c, tu, tdn, xu, xd, diag, (W)S.r, nbr);
            store_site<W, K>(tv, n, o);
            if (!fresh) store_site<W, K>(pnew, n, c);
        }
        if (!grid_sync(a.bar, nb, a.err)) return;

        // ---------------- phase 2: Ap = D_second t, <p, Ap>
        for (int tile = a.tile_begin + blockIdx.x; tile < a.tile_end; tile += nb) {
            const int2 td = a.tiles[tile];
            if (!st_active(a, td.x)) continue;
            const SysDev& S = a.sys[td.x];
            const int n = td.y + threadIdx.x;
            double2 d = make_double2(0.0, 0.0);
            if (n < S.V) {
                const W* tv;
                const W* pk;
                W* apv;
                if constexpr (MIXED) { tv = S.t32; pk = S.p32[cur]; apv = S.Ap32; }
                else { tv = S.t64; pk = S.p64[cur]; apv = S.Ap64; }
                const Site<W, K> ap = apply_d<W, K>(tv, n, S, !first_dag, true);
                store_site<W, K>(apv, n, ap);
                const Site<W, K> pv = load_site_cg<W, K>(pk, n);
                d = site_dot<W, K>(pv, ap);
            }
            const double2 v = block_sum2(d.x, d.y, red);
            tile_reduce<MIXED>(a, tile, td.x, S, v, PH_ALPHA, &s_last);
        }
        if (!grid_sync(a.bar, nb, a.err)) return;

        // ---------------- phase 3: x += alpha p, r -= alpha Ap, |r|^2
        for (int tile = a.tile_begin + blockIdx.x; tile < a.tile_end; tile += nb) {
            const int2 td = a.tiles[tile];
            if (!st_active(a, td.x)) continue;
            const SysDev& S = a.sys[td.x];
            const int n = td.y + threadIdx.x;
            double rr = 0.0;
            if (n < S.V) {
                const W ar = (W)st_load(&a.st[td.x].alpha_re);
                const W ai = (W)st_load(&a.st[td.x].alpha_im);
                const W* pk;
                const W* apv;
                W* xv;
                W* rv;
                if constexpr (MIXED) { pk = S.p32[cur]; apv = S.Ap32; xv = S.xs32; rv = S.r32; }
                else { pk = S.p64[cur]; apv = S.Ap64; xv = S.x; rv = S.r64; }
                const Site<W, K> pv = load_site_cg<W, K>(pk, n);
                const Site<W, K> ap = load_site_cg<W, K>(apv, n);
                Site<W, K> xs = load_site_cg<W, K>(xv, n);
                Site<W, K> rs = load_site_cg<W, K>(rv, n);
                site_axpy<W, K>(xs, ar, ai, pv);
                site_axpy<W, K>(rs, -ar, -ai, ap);
                store_site<W, K>(xv, n, xs);
                store_site<W, K>(rv, n, rs);
                W acc = 0;
#pragma unroll
                for (int i = 0; i < 4 * K; ++i) acc = fma(rs.v[i], rs.v[i], acc);
                rr = (double)acc;
            }
            const double2 v = block_sum2(rr, 0.0, red);
            tile_reduce<MIXED>(a, tile, td.x, S, v, PH_BETA, &s_last);
        }
        if (!grid_sync(a.bar, nb, a.err)) return;

        if constexpr (MIXED) {
            if (*(volatile int*)a.any_ru) {
                // RU1: x += xs, xs = 0
                for (int tile = a.tile_begin + blockIdx.x; tile < a.tile_end; tile += nb) {
                    const int2 td = a.tiles[tile];
                    if (!*(volatile int*)&a.st[td.x].ru) continue;
                    const SysDev& S = a.sys[td.x];
                    const int n = td.y + threadIdx.x;
                    if (n >= S.V) continue;
                    Site<double, K> xv = load_site_cg<double, K>(S.x, n);
                    const Site<float, K> xs = load_site_cg<float, K>(S.xs32, n);
                    Site<float, K> z;
#pragma unroll
                    for (int i = 0; i < 4 * K; ++i) {
                        xv.v[i] += (double)xs.v[i];
                        z.v[i] = 0.f;
                    }
                    store_site<double, K>(S.x, n, xv);
                    store_site<float, K>(S.xs32, n, z);
                }
                if (!grid_sync(a.bar, nb, a.err)) return;
                if (blockIdx.x == 0 && threadIdx.x == 0) *a.any_ru = 0;
                // RU2: t = D_first x  (FP64)
                for (int tile = a.tile_begin + blockIdx.x; tile < a.tile_end; tile += nb) {
                    const int2 td = a.tiles[tile];
                    if (!*(volatile int*)&a.st[td.x].ru) continue;
                    const SysDev& S = a.sys[td.x];
                    const int n = td.y + threadIdx.x;
                    if (n >= S.V) continue;
                    const Site<double, K> t = apply_d<double, K>(S.x, n, S, first_dag, true);
                    store_site<double, K>(S.t64, n, t);
                }
                if (!grid_sync(a.bar, nb, a.err)) return;
                // RU3: r = b - D_second t  (FP64), r32 = r, |r|^2
                for (int tile = a.tile_begin + blockIdx.x; tile < a.tile_end; tile += nb) {
                    const int2 td = a.tiles[tile];
                    if (!*(volatile int*)&a.st[td.x].ru) continue;
                    const SysDev& S = a.sys[td.x];
                    const int n = td.y + threadIdx.x;
                    double rr = 0.0;
                    if (n < S.V) {
                        const Site<double, K> ax = apply_d<double, K>(S.t64, n, S, !first_dag, true);
                        const Site<double, K> bv = load_site_cg<double, K>(S.b, n);
                        Site<float, K> rf;
#pragma unroll
                        for (int i = 0; i < 4 * K; ++i) {
                            const double rv = bv.v[i] - ax.v[i];
                            rr = fma(rv, rv, rr);
                            rf.v[i] = (float)rv;
                        }
                        store_site<float, K>(S.r32, n, rf);
                    }
                    const double2 v = block_sum2(rr, 0.0, red);
                    tile_reduce<MIXED>(a, tile, td.x, S, v, PH_RU, &s_last);
                }
                if (!grid_sync(a.bar, nb, a.err)) return;
            }
        }
    }
}

// Resets the barrier, counters and activity flags before a solve.
__global__ void cg_prepare_kernel(CGArgs a)
{
    for (int i = a.sys_first + threadIdx.x; i < a.sys_first + a.sys_count; i += blockDim.x) {
        a.st[i].counter = 0;
        a.st[i].active = 0;
        a.st[i].iters = 0;
        a.st[i].converged = 0;
        a.st[i].status = 0;
        a.st[i].n_ru = 0;
    }
    if (threadIdx.x == 0) {
        *a.n_active = a.sys_count;
        *a.any_ru = 0;
        a.bar->count = 0;
        *a.err = 0;
    }
}

static int max_coresident(const void* fn, int block)
{
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0);
    return per * nsm;
}

template <int K, bool MIXED>
static int max_grid_t()
{
    static int maxg = -1;
    if (maxg < 0) maxg = max_coresident((const void*)cg_kernel<K, MIXED>, kBlock);
    return maxg;
}

int cg_max_grid(int K, bool mixed)
{
    if (K == 1) return mixed ? max_grid_t<1, true>() : max_grid_t<1, false>();
    return mixed ? max_grid_t<2, true>() : max_grid_t<2, false>();
}

template <int K, bool MIXED>
static cudaError_t launch_cg_t(const CGArgs& a, cudaStream_t stream, int* grid_out)
{
    const int maxg = max_grid_t<K, MIXED>();
    const int nt = a.tile_end - a.tile_begin;
    int grid = nt < maxg ? nt : maxg;
    if (grid < 1) grid = 1;
    if (grid_out) *grid_out = grid;
    cg_prepare_kernel<<<1, 256, 0, stream>>>(a);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, cg_kernel<K, MIXED>, a);
}

cudaError_t launch_cg(const CGArgs& a, int K, bool mixed, cudaStream_t stream, int* grid_out)
{
    if (K == 1) return mixed ? launch_cg_t<1, true>(a, stream, grid_out) : launch_cg_t<1, false>(a, stream, grid_out);
    return mixed ? launch_cg_t<2, true>(a, stream, grid_out) : launch_cg_t<2, false>(a, stream, grid_out);
}

}  // namespace yk
