// yk_cg.cu -- batched CG on D^dag D (or D D^dag) as one persistent
// cooperative kernel per solve: the algorithm of code/src/CGsolver.cu:72-170
// -- x0 = 0, r = p = b, alpha = |r|^2 / <p, A p>, x += alpha p,
// r -= alpha A p, beta = |r'|^2 / |r|^2, p = r + beta p, stop when
// sqrt(|r|^2) <= tol -- in three phases per iteration (the reference pays 15
// grid syncs): p is formed on the fly inside the first D apply
// (double-buffered), the second D apply carries <p, Ap>, the axpys carry |r|^2.
//
// FP64: every vector and scalar in FP64.  MIXED: FP32 vectors and stencils,
// FP64 partial sums and scalars, FP64 reliable updates (the solution is kept
// as an FP64 x plus an FP32 increment; r = b - A x is recomputed in FP64
// when the FP32 residual claims convergence, every `reliable_every`
// iterations and at the cap; convergence is only declared on that residual).
//
// One launch solves every (chain, rhs) system; each block owns a contiguous
// range of 256-site tiles; a bounded sense-reversing grid barrier separates
// phases; reductions are deterministic (per-tile partials, summed in tile
// order by every block that needs them, right after the barrier).
#include <cstdio>
#include <type_traits>

#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

#ifdef YK_CG_CHECKED
// Self-checking build: every site access of the CG kernels is checked
// against the system's volume and for null buffers; the first bad access is
// printed with its source line and skipped.
__device__ int g_cg_bad;

template <typename R, int K>
__device__ Site<R, K> chk_ld(const R* p, int64_t n, int V, int line)
{
    if (p == nullptr || n < 0 || n >= V) {
        if (atomicCAS(&g_cg_bad, 0, line) == 0)
            printf("cg check: bad load line %d ptr %p n %lld V %d block %d\n", line, p, (long long)n, V, blockIdx.x);
        Site<R, K> z;
#pragma unroll
        for (int i = 0; i < 4 * K; ++i) z.v[i] = R(0);
        return z;
    }
    return load_site<R, K>(p, n);
}

template <typename R, int K>
__device__ void chk_st(R* p, int64_t n, const Site<R, K>& v, int V, int line)
{
    if (p == nullptr || n < 0 || n >= V) {
        if (atomicCAS(&g_cg_bad, 0, line) == 0)
            printf("cg check: bad store line %d ptr %p n %lld V %d block %d\n", line, p, (long long)n, V, blockIdx.x);
        return;
    }
    store_site<R, K>(p, n, v);
}
#define YK_LD(R, K, p, n) chk_ld<R, K>((p), (n), S.V, __LINE__)
#define YK_ST(R, K, p, n, v) chk_st<R, K>((p), (n), (v), S.V, __LINE__)
#else
#define YK_LD(R, K, p, n) load_site<R, K>((p), (n))
#define YK_ST(R, K, p, n, v) store_site<R, K>((p), (n), (v))
#endif

namespace {

constexpr int kMaxSysPerBlock = 48;

// Per-block view of one system whose tiles fall in the block's range.
struct SysLocal {
    int sys;
    int owner;       // this block holds the system's first tile: writes CGState
    int active;
    int iters;
    int ru;          // reliable update pending (mixed)
    int ru_done;     // the last reduction came from a reliable update
    int go;          // phase 1 forms p and t for this system in this pass
    int status;
    double rr, rr0, stop, alpha, alpha_im, beta;
    double cre, cim;         // p = beta p + c r (c = 1 except after a reliable update)
    double rmax;             // largest |r| since the last reliable update (mixed)
    double sx, sy, sz, sw;   // reduction results of the current phase
};

// Sense-reversing grid barrier (one counter word; block 0 adds 2^31 - (n-1),
// the others 1, so bit 31 flips once every block has arrived).  Bounded:
// after kBarrierCycles it records YK_ETIMEOUT and every caller leaves.
__device__ __forceinline__ bool gsync(GridBarrier* b, int* err)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned inc = (blockIdx.x == 0) ? (0x80000000u - (gridDim.x - 1)) : 1u;
        __threadfence();
        const unsigned old = atomicAdd(&b->count, inc);
        volatile unsigned* vc = &b->count;
        const long long t0 = clock64();
        while (((*vc ^ old) & 0x80000000u) == 0) {
            if (clock64() - t0 > kBarrierCycles) {
                atomicCAS(err, 0, YK_ETIMEOUT);
                break;
            }
            __nanosleep(20);
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)err == 0;
}

// Builds the block's system table from its tile range [tb, te).
__device__ void build_table(const CGArgs& a, int tb, int te, SysLocal* sl, int* nsl, int* tile_slot)
{
    if (threadIdx.x == 0) {
        int n = 0, last = -1;
        for (int t = tb; t < te; ++t) {
            const int s = a.tiles[t].x;
            if (s != last) {
                if (n == kMaxSysPerBlock) {
                    atomicCAS(a.err, 0, YK_EINVAL);
                    break;
                }
                SysLocal& L = sl[n];
                L.sys = s;
                L.owner = (a.sys[s].tile0 >= tb && a.sys[s].tile0 < te) ? 1 : 0;
                L.active = 1;
                L.iters = 0;
                L.ru = 0;
                L.ru_done = 0;
                L.go = 0;
                L.status = 0;
                L.rr = L.rr0 = L.stop = L.alpha = L.alpha_im = L.beta = 0.0;
                L.cre = 1.0;
                L.cim = 0.0;
                L.rmax = 0.0;
                L.sx = L.sy = L.sz = L.sw = 0.0;
                ++n;
                last = s;
            }
            tile_slot[t - tb] = n - 1;
        }
        *nsl = n;
    }
    __syncthreads();
}

// Sums the (x, y) partials -- and (z, w) when NV = 2 -- of every active
// system of the block: one warp per system; lane l adds tiles l, l+32,
// l+64, ... in order, then a fixed butterfly -- the same bits in every block
// that reduces the system.  Eight tiles per lane are loaded before they are
// added, so a 256-tile system costs one L2 round trip.
template <int NV>
__device__ void reduce_systems(const CGArgs& a, SysLocal* sl, int nsl)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    constexpr int U = 8;
    for (int j = w; j < nsl; j += nw) {
        if (!sl[j].active) continue;
        const SysDev& S = a.sys[sl[j].sys];
        double acc[2 * NV];
#pragma unroll
        for (int c = 0; c < 2 * NV; ++c) acc[c] = 0.0;
        for (int base = lane; base < S.ntiles; base += 32 * U) {
            double2 v[U][NV];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                // the load address is clamped into the system's tiles, so a load the
                // compiler issues ahead of the range test never leaves the array
                const int i = base + 32 * u;
                const int ii = i < S.ntiles ? i : S.ntiles - 1;
                const double2* q = reinterpret_cast<const double2*>(a.partial + S.tile0 + ii);
#pragma unroll
                for (int c = 0; c < NV; ++c) {
                    const double2 t = ld_volatile2(q + c);
                    v[u][c] = (i < S.ntiles) ? t : make_double2(0.0, 0.0);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int c = 0; c < NV; ++c) {
                    acc[2 * c] += v[u][c].x;
                    acc[2 * c + 1] += v[u][c].y;
                }
        }
#pragma unroll
        for (int c = 0; c < 2 * NV; ++c) acc[c] = warp_sum(acc[c]);
        if (lane == 0) {
            sl[j].sx = acc[0];
            sl[j].sy = acc[1];
            if constexpr (NV == 2) {
                sl[j].sz = acc[2 % (2 * NV)];
                sl[j].sw = acc[3 % (2 * NV)];
            }
        }
    }
    __syncthreads();
}

__device__ void retire(const CGArgs& a, SysLocal& L, int converged, int status)
{
    L.active = 0;
    if (status) L.status = status;
    if (L.owner) {
        volatile CGState& s = a.st[L.sys];
        s.converged = converged;
        s.status = L.status;
        s.iters = L.iters;
        s.rr = L.rr;
        s.rr0 = L.rr0;
        s.active = 0;
        __threadfence();
        atomicSub(a.n_active, 1);
    }
}

__device__ void publish(const CGArgs& a, const SysLocal& L, int n_ru)
{
    if (L.owner) {
        volatile CGState& s = a.st[L.sys];
        s.iters = L.iters;
        s.rr = L.rr;
        s.rr0 = L.rr0;
        s.n_ru = n_ru;
    }
}

template <typename W, int K>
__device__ __forceinline__ Site<W, K> apply_d(const W* in, int n, const SysDev& S, bool dag)
{
    const Nbr nb = neighbours(n, S.Nt, S.Nx);
    const Site<W, K> c = YK_LD(W, K, in, n);
    const Site<W, K> tu = YK_LD(W, K, in, nb.tu);
    const Site<W, K> td = YK_LD(W, K, in, nb.td);
    const Site<W, K> xu = YK_LD(W, K, in, nb.xu);
    const Site<W, K> xd = YK_LD(W, K, in, nb.xd);
    const W diag = (W)(2.0 * S.r + S.m0 + S.g * S.sigma[n]);
    return dag ? dirac_combine<W, K, true>(c, tu, td, xu, xd, diag, (W)S.r, (W)nb.sp, (W)nb.sm)
               : dirac_combine<W, K, false>(c, tu, td, xu, xd, diag, (W)S.r, (W)nb.sp, (W)nb.sm);
}

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

// Block partial sums -> the tile's partial slot (thread 0).  z, w: only
// reliable updates pass them (a second block reduction).
__device__ __forceinline__ void put_partial(const CGArgs& a, int tile, double x, double y, double* red,
                                            bool zw = false, double z = 0.0, double w = 0.0)
{
    const double2 s = block_sum2(x, y, red);
    const double2 s2 = zw ? block_sum2(z, w, red + 32) : make_double2(0.0, 0.0);
    if (threadIdx.x == 0) {
#ifdef YK_CG_CHECKED
        if (tile < 0 || tile >= a.tile_end) {
            if (atomicCAS(&g_cg_bad, 0, __LINE__) == 0) printf("cg check: bad partial tile %d end %d\n", tile, a.tile_end);
            return;
        }
#endif
        Partial p;
        p.x = s.x;
        p.y = s.y;
        p.z = s2.x;
        p.w = s2.y;
        a.partial[tile] = p;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Hestenes-Stiefel CG (the reference's algorithm), three phases per iteration:
//   1. reduce |r|^2 -> beta / convergence; p = r + beta p formed on the fly at
//      the five stencil sites; t = D_first p
//   2. Ap = D_second t; partial <p, Ap>
//   3. reduce -> alpha (Smith division); x += alpha p, r -= alpha Ap; |r|^2
// W = double: the plain FP64 solver.  W = float (MIXED): FP32 vectors and
// stencil, FP64 partial sums and scalars.  When the FP32 residual claims
// convergence, every `reliable_every` iterations and at the iteration cap,
// phase 1 is followed by a reliable update -- t64 = D_first (x + xs) and
// r = b - D_second t64 in FP64, x += xs, xs = 0 -- and phase 1 is run again
// for the systems concerned on that FP64 residual; convergence is only
// declared on it.
// ---------------------------------------------------------------------------
template <int K, bool MIXED>
__global__ void __launch_bounds__(kBlock) cg_kernel(CGArgs a)
{
    using W = typename std::conditional<MIXED, float, double>::type;
    __shared__ double red[64];
    __shared__ SysLocal sl[kMaxSysPerBlock];
    __shared__ int nsl;
    __shared__ int tslot[kMaxTilesPerBlock];
    const int tb = a.tile_begin + blockIdx.x * a.tiles_per_block;
    const int te = min(tb + a.tiles_per_block, a.tile_end);
    build_table(a, tb, te, sl, &nsl, tslot);
    const bool first_dag = (a.mtype == YK_NORMAL);   // Normal: A = D D^dag, apply D^dag first
    auto Rv = [](const SysDev& S) -> W* {
        if constexpr (MIXED) return S.r32; else return S.r64;
    };
    auto Pv = [](const SysDev& S, int i) -> W* {
        if constexpr (MIXED) return S.p32[i]; else return S.p64[i];
    };
    auto Tv = [](const SysDev& S) -> W* {
        if constexpr (MIXED) return S.t32; else return S.t64;
    };
    auto Av = [](const SysDev& S) -> W* {
        if constexpr (MIXED) return S.Ap32; else return S.Ap64;
    };
    auto Xv = [](const SysDev& S) -> W* {
        if constexpr (MIXED) return S.xs32; else return S.x;
    };

    // ---------------- init: x = 0 (and xs = 0), r = p_0 = b, |b|^2
    for (int tile = tb; tile < te; ++tile) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + threadIdx.x;
        double pr = 0.0;
        if (n < S.V) {
            const Site<double, K> bv = S.gen_eta ? eta_site<K>(S, n, a.eta_kind) : YK_LD(double, K, S.b, n);
            if (S.gen_eta) YK_ST(double, K, S.b, n, bv);
            Site<double, K> z;
            Site<W, K> bw, zw;
#pragma unroll
            for (int i = 0; i < 4 * K; ++i) {
                z.v[i] = 0.0;
                zw.v[i] = W(0);
                bw.v[i] = (W)bv.v[i];
                pr = fma(bv.v[i], bv.v[i], pr);
            }
            YK_ST(double, K, S.x, n, z);
            if constexpr (MIXED) YK_ST(W, K, S.xs32, n, zw);
            YK_ST(W, K, Rv(S), n, bw);
            YK_ST(W, K, Pv(S, 0), n, bw);
        }
        put_partial(a, tile, pr, 0.0, red);
    }
    if (!gsync(a.bar, a.err)) return;

    int n_ru = 0;
    bool redo = false;   // phase 1 again after a reliable update, same k
    int k = 0;
    while (k <= a.max_iter) {   // every system retires in phase 1 of k = max_iter at the latest
        const int cur = k & 1, prv = cur ^ 1;   // p_k lives in P[cur]
        // ---------------- phase 1
        if (redo)
            reduce_systems<2>(a, sl, nsl);
        else
            reduce_systems<1>(a, sl, nsl);
        if (threadIdx.x == 0) {
            int want_ru = 0;
            for (int j = 0; j < nsl; ++j) {
                SysLocal& L = sl[j];
                L.go = 0;
                if (!L.active || (redo && !L.ru_done)) continue;
                const double rr = L.sx;
                if (k == 0) {
                    L.rr = L.rr0 = rr;
                    L.stop = (a.tol_mode == YK_TOL_ABS) ? a.tol : a.tol * sqrt(rr);
                    L.beta = 0.0;
                    L.rmax = sqrt(rr);
                    if (!isfinite(rr)) retire(a, L, 0, YK_ENAN);
                    else if (!(sqrt(rr) > L.stop)) retire(a, L, 1, 0);
                    else if (a.max_iter <= 0) retire(a, L, 0, YK_ENOCONV);
                    else L.go = 1;
                    continue;
                }
                if (!L.ru_done) L.iters += 1;
                if (!isfinite(rr)) {
                    retire(a, L, 0, YK_ENAN);
                    continue;
                }
                const double rn = sqrt(rr);
                if (MIXED && !L.ru_done) {
                    // reliable update: the FP32 residual claims convergence, has
                    // dropped by reliable_delta since the last update, is due, or
                    // the cap is reached (QUDA-style triggers)
                    L.rmax = fmax(L.rmax, rn);
                    const bool cand = !(rn > L.stop);
                    const bool drop = rn < a.reliable_delta * L.rmax;
                    const bool due = a.reliable_every > 0 && (L.iters % a.reliable_every) == 0;
                    const bool cap = L.iters >= a.max_iter;
                    if (cand || drop || due || cap) {
                        L.ru = 1;
                        want_ru = 1;
                        continue;
                    }
                    L.cre = 1.0;
                    L.cim = 0.0;
                } else {
                    if (!(rn > L.stop)) {
                        L.rr = rr;
                        L.ru_done = 0;
                        retire(a, L, 1, 0);
                        continue;
                    }
                    if (L.iters >= a.max_iter) {
                        L.rr = rr;
                        L.ru_done = 0;
                        retire(a, L, 0, YK_ENOCONV);
                        continue;
                    }
                    if (MIXED) {
                        // after a reliable update p is first made orthogonal to the
                        // new residual: p <- p - gamma r, gamma = <r, p> / |r|^2, so
                        // p_new = r + beta (p - gamma r) = beta p + (1 - beta gamma) r
                        const double beta = rr / L.rr;
                        const double gre = L.sz / rr, gim = L.sw / rr;
                        L.cre = 1.0 - beta * gre;
                        L.cim = -beta * gim;
                        L.rmax = rn;
                        L.ru_done = 0;
                    }
                }
                L.beta = rr / L.rr;
                L.rr = rr;
                L.go = 1;
            }
            if (want_ru) atomicMax(a.any_ru, k + 1);
        }
        __syncthreads();
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (!L.go) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            if (n >= S.V) continue;
            const W beta = (W)L.beta, cre = (W)L.cre, cim = (W)L.cim;
            const W* pold = Pv(S, k == 0 ? 0 : prv);
            const W* rv = Rv(S);
            const Nbr nbr = neighbours(n, S.Nt, S.Nx);
            Site<W, K> st[5];
            const int64_t m5[5] = {n, nbr.tu, nbr.td, nbr.xu, nbr.xd};
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                st[q] = YK_LD(W, K, pold, m5[q]);
                if (k > 0) {
                    // p = beta p + c r  (c = 1 but after a reliable update)
                    const Site<W, K> r = YK_LD(W, K, rv, m5[q]);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        if constexpr (K == 1) {
                            st[q].v[e] = fma(beta, st[q].v[e], cre * r.v[e]);
                        } else {
                            const W re = r.v[2 * e], im = r.v[2 * e + 1];
                            st[q].v[2 * e] = fma(beta, st[q].v[2 * e], fma(cre, re, -cim * im));
                            st[q].v[2 * e + 1] = fma(beta, st[q].v[2 * e + 1], fma(cre, im, cim * re));
                        }
                    }
                }
            }
            const W diag = (W)(2.0 * S.r + S.m0 + S.g * S.sigma[n]);
            const Site<W, K> o = first_dag
                ? dirac_combine<W, K, true>(st[0], st[1], st[2], st[3], st[4], diag, (W)S.r, (W)nbr.sp, (W)nbr.sm)
                : dirac_combine<W, K, false>(st[0], st[1], st[2], st[3], st[4], diag, (W)S.r, (W)nbr.sp, (W)nbr.sm);
            YK_ST(W, K, Tv(S), n, o);
            if (k > 0) YK_ST(W, K, Pv(S, cur), n, st[0]);
        }
        if (!gsync(a.bar, a.err)) return;
        if (*(volatile int*)a.n_active == 0) break;

        if constexpr (MIXED) {
            if (!redo && *(volatile int*)a.any_ru == k + 1) {
                // RU1: t64 = D_first (x + xs), formed on the fly in FP64
                for (int tile = tb; tile < te; ++tile) {
                    const SysLocal& L = sl[tslot[tile - tb]];
                    if (!L.active || !L.ru) continue;
                    const SysDev& S = a.sys[L.sys];
                    const int n = a.tiles[tile].y + threadIdx.x;
                    if (n >= S.V) continue;
                    const Nbr nbr = neighbours(n, S.Nt, S.Nx);
                    Site<double, K> xt[5];
                    const int64_t m5[5] = {n, nbr.tu, nbr.td, nbr.xu, nbr.xd};
#pragma unroll
                    for (int q = 0; q < 5; ++q) {
                        xt[q] = YK_LD(double, K, S.x, m5[q]);
                        const Site<W, K> xs = YK_LD(W, K, S.xs32, m5[q]);
#pragma unroll
                        for (int i = 0; i < 4 * K; ++i) xt[q].v[i] += (double)xs.v[i];
                    }
                    const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
                    const Site<double, K> t = first_dag
                        ? dirac_combine<double, K, true>(xt[0], xt[1], xt[2], xt[3], xt[4], diag, S.r, (double)nbr.sp, (double)nbr.sm)
                        : dirac_combine<double, K, false>(xt[0], xt[1], xt[2], xt[3], xt[4], diag, S.r, (double)nbr.sp, (double)nbr.sm);
                    YK_ST(double, K, S.t64, n, t);
                }
                if (!gsync(a.bar, a.err)) return;
                // RU2: x += xs, xs = 0; r = b - D_second t64 in FP64; |r|^2
                for (int tile = tb; tile < te; ++tile) {
                    const SysLocal& L = sl[tslot[tile - tb]];
                    if (!L.active || !L.ru) continue;
                    const SysDev& S = a.sys[L.sys];
                    const int n = a.tiles[tile].y + threadIdx.x;
                    double rr = 0.0;
                    double2 rp = make_double2(0.0, 0.0);
                    if (n < S.V) {
                        Site<double, K> xv = YK_LD(double, K, S.x, n);
                        const Site<W, K> xs = YK_LD(W, K, S.xs32, n);
                        Site<W, K> zw;
#pragma unroll
                        for (int i = 0; i < 4 * K; ++i) {
                            xv.v[i] += (double)xs.v[i];
                            zw.v[i] = W(0);
                        }
                        YK_ST(double, K, S.x, n, xv);
                        YK_ST(W, K, S.xs32, n, zw);
                        const Site<double, K> ax = apply_d<double, K>(S.t64, n, S, !first_dag);
                        const Site<double, K> bv = YK_LD(double, K, S.b, n);
                        const Site<W, K> pw = YK_LD(W, K, Pv(S, prv), n);   // p_{k-1}
                        Site<W, K> rw;
                        Site<double, K> rd, pd;
#pragma unroll
                        for (int i = 0; i < 4 * K; ++i) {
                            const double r = bv.v[i] - ax.v[i];
                            rr = fma(r, r, rr);
                            rw.v[i] = (W)r;
                            rd.v[i] = r;
                            pd.v[i] = (double)pw.v[i];
                        }
                        rp = site_dot<double, K>(rd, pd);
                        YK_ST(W, K, Rv(S), n, rw);
                    }
                    put_partial(a, tile, rr, 0.0, red, true, rp.x, rp.y);
                }
                __syncthreads();
                if (threadIdx.x == 0)
                    for (int j = 0; j < nsl; ++j)
                        if (sl[j].active && sl[j].ru) {
                            sl[j].ru = 0;
                            sl[j].ru_done = 1;
                        }
                ++n_ru;
                redo = true;
                if (!gsync(a.bar, a.err)) return;
                continue;
            }
        }
        redo = false;

        // ---------------- phase 2: Ap = D_second t, <p, Ap>
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (!L.active) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            double2 d = make_double2(0.0, 0.0);
            if (n < S.V) {
                const Site<W, K> ap = apply_d<W, K>(Tv(S), n, S, !first_dag);
                YK_ST(W, K, Av(S), n, ap);
                d = site_dot<W, K>(YK_LD(W, K, Pv(S, cur), n), ap);
            }
            put_partial(a, tile, d.x, d.y, red);
        }
        if (!gsync(a.bar, a.err)) return;

        // ---------------- phase 3: alpha; x += alpha p, r -= alpha Ap, |r|^2
        reduce_systems<1>(a, sl, nsl);
        if (threadIdx.x == 0) {
            for (int j = 0; j < nsl; ++j) {
                SysLocal& L = sl[j];
                if (!L.active) continue;
                // alpha = rr / (sx + i sy), Smith's complex division (CGsolver.cu:137)
                const double c = L.sx, d = L.sy, num = L.rr;
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
                L.alpha = ar;
                L.alpha_im = ai;
                if (!isfinite(ar) || !isfinite(ai)) retire(a, L, 0, YK_ENAN);
            }
        }
        __syncthreads();
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (!L.active) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            double rr = 0.0;
            if (n < S.V) {
                const Site<W, K> pv = YK_LD(W, K, Pv(S, cur), n);
                const Site<W, K> ap = YK_LD(W, K, Av(S), n);
                Site<W, K> xs = YK_LD(W, K, Xv(S), n);
                Site<W, K> rs = YK_LD(W, K, Rv(S), n);
                site_axpy<W, K>(xs, (W)L.alpha, (W)L.alpha_im, pv);
                site_axpy<W, K>(rs, (W)-L.alpha, (W)-L.alpha_im, ap);
                YK_ST(W, K, Xv(S), n, xs);
                YK_ST(W, K, Rv(S), n, rs);
#pragma unroll
                for (int i = 0; i < 4 * K; ++i) rr = fma((double)rs.v[i], (double)rs.v[i], rr);
            }
            put_partial(a, tile, rr, 0.0, red);
        }
        if (!gsync(a.bar, a.err)) return;
        ++k;
    }
    if (threadIdx.x == 0)
        for (int j = 0; j < nsl; ++j) publish(a, sl[j], n_ru);
}

// Resets the barrier, counters and activity flags before a solve.
__global__ void cg_prepare_kernel(CGArgs a)
{
    for (int i = a.sys_first + threadIdx.x; i < a.sys_first + a.sys_count; i += blockDim.x) {
        a.st[i].active = 1;
        a.st[i].iters = 0;
        a.st[i].converged = 0;
        a.st[i].status = 0;
        a.st[i].n_ru = 0;
        a.st[i].rr = 0.0;
        a.st[i].rr0 = 0.0;
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

int cg_grid_for(int ntiles, int maxg, int* tiles_per_block)
{
    int grid = ntiles < maxg ? ntiles : maxg;
    if (grid < 1) grid = 1;
    int tpb = (ntiles + grid - 1) / grid;
    if (tpb < 1) tpb = 1;
    grid = (ntiles + tpb - 1) / tpb;
    if (grid < 1) grid = 1;
    *tiles_per_block = tpb;
    return grid;
}

template <int K, bool MIXED>
static cudaError_t launch_cg_t(const CGArgs& a0, cudaStream_t stream, int* grid_out)
{
    CGArgs a = a0;
    const int maxg = max_grid_t<K, MIXED>();
    const int nt = a.tile_end - a.tile_begin;
    int tpb = 1;
    const int grid = cg_grid_for(nt, maxg, &tpb);
    if (tpb > kMaxTilesPerBlock || grid > maxg) return cudaErrorInvalidConfiguration;
    a.tiles_per_block = tpb;
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
