// yk_cg.cu -- batched CG on D^dag D (or D D^dag) as one persistent
// cooperative kernel per solve.
//
// FP64 (cg64_kernel): the algorithm of code/src/CGsolver.cu:72-170 --
//   x0 = 0, r = p = b, alpha = |r|^2 / <p, A p>, x += alpha p,
//   r -= alpha A p, beta = |r'|^2 / |r|^2, p = r + beta p, stop when
//   sqrt(|r|^2) <= tol -- in three phases per iteration (the reference pays
//   15 grid syncs): p is formed on the fly inside the first D apply
//   (double-buffered), the second D apply carries <p, Ap>, the axpys carry |r|^2.
//
// MIXED (cgcg_kernel): Chronopoulos-Gear CG (one fused reduction of (r, r)
//   and (A r, r) per iteration) on FP32 vectors with FP64 partial sums, in two
//   phases per iteration: r_{k+1} = r_k - alpha (w_k + beta s_{k-1}) is formed
//   on the fly at the four neighbours inside D, and D^dag follows.  Every
//   `reliable_every` iterations, when the FP32 residual claims convergence,
//   or at the iteration cap, an FP64 reliable update folds the FP32 solution
//   increment into the FP64 solution and recomputes r = b - A x in FP64;
//   convergence is only declared on that FP64 residual.
//
// Both: one launch solves every (chain, rhs) system; each block owns a
// contiguous range of 256-site tiles; a bounded sense-reversing grid barrier
// separates phases; reductions are deterministic (per-tile partials, summed
// in tile order by every block that needs them, right after the barrier).
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
    int last;        // iteration cap reached
    int status;
    int iters_ru;    // iteration of the last reliable update (mixed)
    double rr, rr0, stop, alpha, alpha_im, beta, gamma, gamma_ru;
    double sx, sy, sz, sw, su;   // reduction results of the current phase
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
                L.last = 0;
                L.status = 0;
                L.iters_ru = 0;
                L.rr = L.rr0 = L.stop = L.alpha = L.alpha_im = L.beta = L.gamma = L.gamma_ru = 0.0;
                L.sx = L.sy = L.sz = L.sw = L.su = 0.0;
                ++n;
                last = s;
            }
            tile_slot[t - tb] = n - 1;
        }
        *nsl = n;
    }
    __syncthreads();
}

// Sums the partials of every active system of the block: one warp per
// system; lane l adds tiles l, l+32, l+64, ... in order, then a fixed
// butterfly -- the same bits in every block that reduces the system.  Eight
// tiles per lane are loaded before they are added, so a 256-tile system
// costs one L2 round trip.
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
        for (int q = 0; q < 2 * NV; ++q) acc[q] = 0.0;
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
        for (int q = 0; q < 2 * NV; ++q) acc[q] = warp_sum(acc[q]);
        if (lane == 0) {
            sl[j].sx = acc[0];
            sl[j].sy = acc[1];
            if (NV > 1) {
                sl[j].sz = acc[2 % (2 * NV)];
                sl[j].sw = acc[3 % (2 * NV)];
            }
            if (NV > 2) sl[j].su = acc[4 % (2 * NV)];
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

// Block partial sums -> the tile's partial slot (thread 0), one pass.
// keep_z: the slot's z (the FP64 residual of a reliable update) is kept.
__device__ __forceinline__ void store_partial(const CGArgs& a, int tile, const double4& s, bool keep_z)
{
    if (threadIdx.x == 0) {
        Partial p;
        p.x = s.x;
        p.y = s.y;
        p.z = keep_z ? a.partial[tile].z : s.z;
        p.w = keep_z ? s.z : s.w;
        p.u = keep_z ? s.w : 0.0;
        p.v = 0.0;
#ifdef YK_CG_CHECKED
        if (tile < 0 || tile >= a.tile_end) {
            if (atomicCAS(&g_cg_bad, 0, __LINE__) == 0) printf("cg check: bad partial tile %d end %d\n", tile, a.tile_end);
            return;
        }
#endif
        a.partial[tile] = p;
    }
}

__device__ __forceinline__ void put_partial(const CGArgs& a, int tile, double x, double y, double z, double w,
                                            double u, double* red, bool keep_z = false)
{
    store_partial(a, tile, block_sum4(x, y, keep_z ? w : z, keep_z ? u : w, red), keep_z);
}

// FP32 per-site values: FP32 within each warp, FP64 above (block_sum4f).
__device__ __forceinline__ void put_partial_f(const CGArgs& a, int tile, float x, float y, float z, float w,
                                              float u, double* red, bool keep_z = false)
{
    store_partial(a, tile, block_sum4f(x, y, keep_z ? w : z, keep_z ? u : w, red), keep_z);
}

// Real part of sum conj(a) b over one site, in the vectors' own precision.
template <int K>
__device__ __forceinline__ float site_dotf(const Site<float, K>& a, const Site<float, K>& b)
{
    float re = 0.f;
#pragma unroll
    for (int i = 0; i < 4 * K; ++i) re = fmaf(a.v[i], b.v[i], re);
    return re;
}

}  // namespace

// ---------------------------------------------------------------------------
// FP64 Hestenes-Stiefel CG (the reference's algorithm)
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(kBlock) cg64_kernel(CGArgs a)
{
    __shared__ double red[64];
    __shared__ SysLocal sl[kMaxSysPerBlock];
    __shared__ int nsl;
    __shared__ int tslot[kMaxTilesPerBlock];
    const int tb = a.tile_begin + blockIdx.x * a.tiles_per_block;
    const int te = min(tb + a.tiles_per_block, a.tile_end);
    build_table(a, tb, te, sl, &nsl, tslot);
    const bool first_dag = (a.mtype == YK_NORMAL);   // Normal: A = D D^dag, apply D^dag first

    // ---------------- init: x = 0, r = p_0 = b, |b|^2
    for (int tile = tb; tile < te; ++tile) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + threadIdx.x;
        double pr = 0.0;
        if (n < S.V) {
            const Site<double, K> bv = S.gen_eta ? eta_site<K>(S, n, a.eta_kind) : YK_LD(double, K, S.b, n);
            if (S.gen_eta) YK_ST(double, K, S.b, n, bv);
            Site<double, K> z;
#pragma unroll
            for (int i = 0; i < 4 * K; ++i) {
                z.v[i] = 0.0;
                pr = fma(bv.v[i], bv.v[i], pr);
            }
            YK_ST(double, K, S.x, n, z);
            YK_ST(double, K, S.r64, n, bv);
            YK_ST(double, K, S.p64[0], n, bv);
        }
        put_partial(a, tile, pr, 0.0, 0.0, 0.0, 0.0, red);
    }
    if (!gsync(a.bar, a.err)) return;

    for (int k = 0; k <= a.max_iter + 1; ++k) {
        const bool fresh = (k == 0);
        const int cur = k & 1, prv = (k + 1) & 1;
        // ---------------- phase 1: rr -> beta / stop; p_k on the fly; t = D_first p_k
        reduce_systems<1>(a, sl, nsl);
        if (threadIdx.x == 0) {
            for (int j = 0; j < nsl; ++j) {
                SysLocal& L = sl[j];
                if (!L.active) continue;
                if (fresh) {
                    L.rr = L.rr0 = L.sx;
                    L.stop = (a.tol_mode == YK_TOL_ABS) ? a.tol : a.tol * sqrt(L.sx);
                    L.beta = 0.0;
                    if (!isfinite(L.sx)) retire(a, L, 0, YK_ENAN);
                    else if (!(sqrt(L.sx) > L.stop)) retire(a, L, 1, 0);
                    else if (a.max_iter <= 0) retire(a, L, 0, YK_ENOCONV);
                } else {
                    const double rr = L.sx;
                    L.iters += 1;
                    L.beta = rr / L.rr;
                    L.rr = rr;
                    if (!isfinite(rr)) retire(a, L, 0, YK_ENAN);
                    else if (!(sqrt(rr) > L.stop)) retire(a, L, 1, 0);
                    else if (L.iters >= a.max_iter) retire(a, L, 0, YK_ENOCONV);
                }
            }
        }
        __syncthreads();
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (!L.active) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            if (n >= S.V) continue;
            const double beta = L.beta;
            const double* pold = S.p64[fresh ? 0 : prv];
            const Nbr nbr = neighbours(n, S.Nt, S.Nx);
            auto p_at = [&](int64_t m) {
                Site<double, K> po = YK_LD(double, K, pold, m);
                if (!fresh) {
                    const Site<double, K> rv = YK_LD(double, K, S.r64, m);
#pragma unroll
                    for (int i = 0; i < 4 * K; ++i) po.v[i] = fma(beta, po.v[i], rv.v[i]);
                }
                return po;
            };
            const Site<double, K> c = p_at(n), tu = p_at(nbr.tu), tdn = p_at(nbr.td), xu = p_at(nbr.xu),
                                  xd = p_at(nbr.xd);
            const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
            const Site<double, K> o = first_dag
                ? dirac_combine<double, K, true>(c, tu, tdn, xu, xd, diag, S.r, (double)nbr.sp, (double)nbr.sm)
                : dirac_combine<double, K, false>(c, tu, tdn, xu, xd, diag, S.r, (double)nbr.sp, (double)nbr.sm);
            YK_ST(double, K, S.t64, n, o);
            if (!fresh) YK_ST(double, K, S.p64[cur], n, c);
        }
        if (!gsync(a.bar, a.err)) return;
        if (*(volatile int*)a.n_active == 0) break;

        // ---------------- phase 2: Ap = D_second t, <p, Ap>
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (!L.active) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            double2 d = make_double2(0.0, 0.0);
            if (n < S.V) {
                const Site<double, K> ap = apply_d<double, K>(S.t64, n, S, !first_dag);
                YK_ST(double, K, S.Ap64, n, ap);
                d = site_dot<double, K>(YK_LD(double, K, S.p64[cur], n), ap);
            }
            put_partial(a, tile, d.x, d.y, 0.0, 0.0, 0.0, red);
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
                const Site<double, K> pv = YK_LD(double, K, S.p64[cur], n);
                const Site<double, K> ap = YK_LD(double, K, S.Ap64, n);
                Site<double, K> xs = YK_LD(double, K, S.x, n);
                Site<double, K> rs = YK_LD(double, K, S.r64, n);
                site_axpy<double, K>(xs, L.alpha, L.alpha_im, pv);
                site_axpy<double, K>(rs, -L.alpha, -L.alpha_im, ap);
                YK_ST(double, K, S.x, n, xs);
                YK_ST(double, K, S.r64, n, rs);
#pragma unroll
                for (int i = 0; i < 4 * K; ++i) rr = fma(rs.v[i], rs.v[i], rr);
            }
            put_partial(a, tile, rr, 0.0, 0.0, 0.0, 0.0, red);
        }
        if (!gsync(a.bar, a.err)) return;
    }
    if (threadIdx.x == 0)
        for (int j = 0; j < nsl; ++j) publish(a, sl[j], 0);
}

// ---------------------------------------------------------------------------
// Mixed FP32/FP64 Chronopoulos-Gear CG with reliable updates.
// Buffers of a system: r32 (2 V: r double-buffered), p32[0] (p),
// p32[1] and Ap32 (s = A p, double-buffered), t32 (2 V: t = D r and w = A r),
// xs32 (FP32 solution increment), FP64 x, b, t64.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(kBlock) cgcg_kernel(CGArgs a)
{
    using W = float;
    __shared__ double red[64];
    __shared__ SysLocal sl[kMaxSysPerBlock];
    __shared__ int nsl;
    __shared__ int tslot[kMaxTilesPerBlock];
    __shared__ int s_nru;
    const int tb = a.tile_begin + blockIdx.x * a.tiles_per_block;
    const int te = min(tb + a.tiles_per_block, a.tile_end);
    build_table(a, tb, te, sl, &nsl, tslot);
    if (threadIdx.x == 0) s_nru = 0;
    const bool first_dag = (a.mtype == YK_NORMAL);
    auto Rb = [](const SysDev& S, int i) { return S.r32 + (i ? (int64_t)S.V * 4 * K : 0); };
    auto Sb = [](const SysDev& S, int i) { return i ? S.Ap32 : S.p32[1]; };
    auto Wb = [](const SysDev& S) { return S.t32 + (int64_t)S.V * 4 * K; };

    // ---------------- I0: b (generated or given), x = 0, xs = 0, p = 0, s_{-1} = 0, r_0 = b, |b|^2
    for (int tile = tb; tile < te; ++tile) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + threadIdx.x;
        double bb = 0.0;
        if (n < S.V) {
            const Site<double, K> bv = S.gen_eta ? eta_site<K>(S, n, a.eta_kind) : YK_LD(double, K, S.b, n);
            if (S.gen_eta) YK_ST(double, K, S.b, n, bv);
            Site<double, K> z;
            Site<W, K> bf, zf;
#pragma unroll
            for (int i = 0; i < 4 * K; ++i) {
                z.v[i] = 0.0;
                zf.v[i] = 0.f;
                bf.v[i] = (W)bv.v[i];
                bb = fma(bv.v[i], bv.v[i], bb);
            }
            YK_ST(double, K, S.x, n, z);
            YK_ST(W, K, S.xs32, n, zf);
            YK_ST(W, K, S.p32[0], n, zf);
            YK_ST(W, K, Sb(S, 1), n, zf);
            YK_ST(W, K, Rb(S, 0), n, bf);
        }
        put_partial(a, tile, 0.0, 0.0, bb, 0.0, 0.0, red);
    }
    if (!gsync(a.bar, a.err)) return;
    // ---------------- I1: t = D_first r_0
    for (int tile = tb; tile < te; ++tile) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + threadIdx.x;
        if (n < S.V) YK_ST(W, K, S.t32, n, (apply_d<W, K>(Rb(S, 0), n, S, first_dag)));
    }
    if (!gsync(a.bar, a.err)) return;
    // ---------------- I2: w_0 = D_second t; (r,r), (w,r); |b|^2 kept in z
    for (int tile = tb; tile < te; ++tile) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + threadIdx.x;
        float g = 0.f, d = 0.f;
        if (n < S.V) {
            const Site<W, K> w = apply_d<W, K>(S.t32, n, S, !first_dag);
            YK_ST(W, K, Wb(S), n, w);
            const Site<W, K> r = YK_LD(W, K, Rb(S, 0), n);
            g = site_dotf<K>(r, r);
            d = site_dotf<K>(w, r);
        }
        put_partial_f(a, tile, g, d, 0.f, 0.f, 0.f, red, true);
    }
    if (!gsync(a.bar, a.err)) return;

    for (int k = 0; k <= a.max_iter + 1; ++k) {
        const int cur = k & 1, nxt = (k + 1) & 1;
        // ---------------- phase A: reduce; s_k, p_k, xs += alpha p_k, r_{k+1} (on the fly), t = D r_{k+1}
        reduce_systems<3>(a, sl, nsl);
        if (threadIdx.x == 0) {
            int want_ru = 0;
            for (int j = 0; j < nsl; ++j) {
                SysLocal& L = sl[j];
                if (!L.active) continue;
                const double gam = L.sx, del = L.sy;
                if (k == 0) {
                    L.rr0 = L.sz;
                    L.stop = (a.tol_mode == YK_TOL_ABS) ? a.tol : a.tol * sqrt(L.sz);
                    L.rr = L.sz;
                    if (!isfinite(L.sz)) { retire(a, L, 0, YK_ENAN); continue; }
                    if (!(sqrt(L.sz) > L.stop)) { retire(a, L, 1, 0); continue; }
                    if (a.max_iter <= 0) { retire(a, L, 0, YK_ENOCONV); continue; }
                    L.beta = 0.0;
                    L.alpha = gam / del;
                    L.gamma = gam;
                    L.gamma_ru = gam;
                    L.iters_ru = 0;
                } else {
                    L.iters += 1;
                    const double beta = gam / L.gamma;
                    if (L.ru_done) {
                        // z holds |b - A x|^2 in FP64 from the reliable update; the
                        // recurrence restarts from the recomputed r, w with alpha from
                        // (p, A p) = (r, w) + beta ((r, s) + (p, w)) + beta^2 (p, s)
                        L.ru_done = 0;
                        L.rr = L.sz;
                        if (!isfinite(L.sz)) { retire(a, L, 0, YK_ENAN); continue; }
                        if (!(sqrt(L.sz) > L.stop)) { retire(a, L, 1, 0); continue; }
                        if (L.last) { retire(a, L, 0, YK_ENOCONV); continue; }
                        const double pap = del + beta * L.sw + beta * beta * L.su;
                        L.alpha = gam / pap;
                        L.gamma_ru = gam;
                        L.iters_ru = L.iters;
                    } else {
                        L.rr = gam;
                        const double den = del - beta * gam / L.alpha;
                        L.alpha = gam / den;
                    }
                    L.beta = beta;
                    L.gamma = gam;
                }
                if (!isfinite(gam) || !isfinite(L.beta)) {
                    retire(a, L, 0, YK_ENAN);
                    continue;
                }
                // a breakdown of the short recurrence (alpha <= 0 from rounding):
                // no update this iteration and a reliable update, which recomputes
                // alpha from (p, A p)
                const bool broken = !isfinite(L.alpha) || !(L.alpha > 0.0);
                if (broken) L.alpha = 0.0;
                // reliable update after this iteration: residual down 100x since the
                // last one, FP32 residual below the target, interval, or the cap
                const bool cand = broken || !(sqrt(gam) > L.stop);
                const bool drop = gam < 1e-4 * L.gamma_ru;
                const bool due = drop || (a.reliable_every > 0 && (L.iters + 1 - L.iters_ru) >= a.reliable_every);
                const bool cap = (L.iters + 1) >= a.max_iter;
                if (cand || due || cap) {
                    L.ru = 1;
                    L.last = cap ? 1 : 0;
                    want_ru = 1;
                }
            }
            if (want_ru) atomicMax(a.any_ru, k + 1);
        }
        __syncthreads();
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (!L.active) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            if (n >= S.V) continue;
            const W al = (W)L.alpha, be = (W)L.beta;
            const W* Rc = Rb(S, cur);
            const W* Sp = Sb(S, nxt);   // s_{k-1}
            const W* Wk = Wb(S);
            const Nbr nbr = neighbours(n, S.Nt, S.Nx);
            // r_{k+1}(m) = r_k(m) - alpha (w_k(m) + beta s_{k-1}(m))
            auto rnext = [&](int64_t m, Site<W, K>* s_out) {
                const Site<W, K> rv = YK_LD(W, K, Rc, m);
                const Site<W, K> wv = YK_LD(W, K, Wk, m);
                const Site<W, K> sv = YK_LD(W, K, Sp, m);
                Site<W, K> o;
#pragma unroll
                for (int i = 0; i < 4 * K; ++i) {
                    const W s = fma(be, sv.v[i], wv.v[i]);
                    if (s_out) s_out->v[i] = s;
                    o.v[i] = fma(-al, s, rv.v[i]);
                }
                return o;
            };
            Site<W, K> sk;
            const Site<W, K> c = rnext(n, &sk);
            const Site<W, K> tu = rnext(nbr.tu, nullptr), tdn = rnext(nbr.td, nullptr);
            const Site<W, K> xu = rnext(nbr.xu, nullptr), xd = rnext(nbr.xd, nullptr);
            // p_k = r_k + beta p_{k-1}; xs += alpha p_k
            const Site<W, K> rk = YK_LD(W, K, Rc, n);
            Site<W, K> pk = YK_LD(W, K, S.p32[0], n);
            Site<W, K> xs = YK_LD(W, K, S.xs32, n);
#pragma unroll
            for (int i = 0; i < 4 * K; ++i) {
                pk.v[i] = fma(be, pk.v[i], rk.v[i]);
                xs.v[i] = fma(al, pk.v[i], xs.v[i]);
            }
            YK_ST(W, K, S.p32[0], n, pk);
            YK_ST(W, K, S.xs32, n, xs);
            YK_ST(W, K, Sb(S, cur), n, sk);
            YK_ST(W, K, Rb(S, nxt), n, c);
            const W diag = (W)(2.0 * S.r + S.m0 + S.g * S.sigma[n]);
            const Site<W, K> t = first_dag
                ? dirac_combine<W, K, true>(c, tu, tdn, xu, xd, diag, (W)S.r, (W)nbr.sp, (W)nbr.sm)
                : dirac_combine<W, K, false>(c, tu, tdn, xu, xd, diag, (W)S.r, (W)nbr.sp, (W)nbr.sm);
            YK_ST(W, K, S.t32, n, t);
        }
        if (!gsync(a.bar, a.err)) return;
        if (*(volatile int*)a.n_active == 0) break;

        // ---------------- phase B: w_{k+1} = D_second t; (r,r), (w,r)
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (!L.active) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            float g = 0.f, d = 0.f;
            if (n < S.V) {
                const Site<W, K> w = apply_d<W, K>(S.t32, n, S, !first_dag);
                YK_ST(W, K, Wb(S), n, w);
                const Site<W, K> r = YK_LD(W, K, Rb(S, nxt), n);
                g = site_dotf<K>(r, r);
                d = site_dotf<K>(w, r);
            }
            put_partial_f(a, tile, g, d, 0.f, 0.f, 0.f, red);
        }
        if (!gsync(a.bar, a.err)) return;

        if (*(volatile int*)a.any_ru == k + 1) {
            // RU1: t64 = D_first (x + xs)  (FP64, formed on the fly)
            for (int tile = tb; tile < te; ++tile) {
                const SysLocal& L = sl[tslot[tile - tb]];
                if (!L.active || !L.ru) continue;
                const SysDev& S = a.sys[L.sys];
                const int n = a.tiles[tile].y + threadIdx.x;
                if (n >= S.V) continue;
                const Nbr nbr = neighbours(n, S.Nt, S.Nx);
                auto xat = [&](int64_t m) {
                    Site<double, K> xv = YK_LD(double, K, S.x, m);
                    const Site<W, K> xs = YK_LD(W, K, S.xs32, m);
#pragma unroll
                    for (int i = 0; i < 4 * K; ++i) xv.v[i] += (double)xs.v[i];
                    return xv;
                };
                const Site<double, K> c = xat(n), tu = xat(nbr.tu), tdn = xat(nbr.td), xu = xat(nbr.xu),
                                      xd = xat(nbr.xd);
                const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
                const Site<double, K> t = first_dag
                    ? dirac_combine<double, K, true>(c, tu, tdn, xu, xd, diag, S.r, (double)nbr.sp, (double)nbr.sm)
                    : dirac_combine<double, K, false>(c, tu, tdn, xu, xd, diag, S.r, (double)nbr.sp, (double)nbr.sm);
                YK_ST(double, K, S.t64, n, t);
            }
            if (!gsync(a.bar, a.err)) return;
            // RU2: x += xs, xs = 0; r = b - D_second t64 (FP64) -> r_{k+1}; |r|^2 in z
            for (int tile = tb; tile < te; ++tile) {
                const SysLocal& L = sl[tslot[tile - tb]];
                if (!L.active || !L.ru) continue;
                const SysDev& S = a.sys[L.sys];
                const int n = a.tiles[tile].y + threadIdx.x;
                double rr = 0.0;
                if (n < S.V) {
                    Site<double, K> xv = YK_LD(double, K, S.x, n);
                    const Site<W, K> xs = YK_LD(W, K, S.xs32, n);
                    Site<W, K> zf;
#pragma unroll
                    for (int i = 0; i < 4 * K; ++i) {
                        xv.v[i] += (double)xs.v[i];
                        zf.v[i] = 0.f;
                    }
                    YK_ST(double, K, S.x, n, xv);
                    YK_ST(W, K, S.xs32, n, zf);
                    const Site<double, K> ax = apply_d<double, K>(S.t64, n, S, !first_dag);
                    const Site<double, K> bv = YK_LD(double, K, S.b, n);
                    Site<W, K> rf;
#pragma unroll
                    for (int i = 0; i < 4 * K; ++i) {
                        const double rv = bv.v[i] - ax.v[i];
                        rr = fma(rv, rv, rr);
                        rf.v[i] = (W)rv;
                    }
                    YK_ST(W, K, Rb(S, nxt), n, rf);
                }
                put_partial(a, tile, 0.0, 0.0, rr, 0.0, 0.0, red);
            }
            if (!gsync(a.bar, a.err)) return;
            // RU3: t = D_first r
            for (int tile = tb; tile < te; ++tile) {
                const SysLocal& L = sl[tslot[tile - tb]];
                if (!L.active || !L.ru) continue;
                const SysDev& S = a.sys[L.sys];
                const int n = a.tiles[tile].y + threadIdx.x;
                if (n < S.V) YK_ST(W, K, S.t32, n, (apply_d<W, K>(Rb(S, nxt), n, S, first_dag)));
            }
            if (!gsync(a.bar, a.err)) return;
            // RU4: w = D_second t; (r,r), (w,r), (r,s_k) + (p_k,w), (p_k,s_k); z kept
            for (int tile = tb; tile < te; ++tile) {
                const SysLocal& L = sl[tslot[tile - tb]];
                if (!L.active || !L.ru) continue;
                const SysDev& S = a.sys[L.sys];
                const int n = a.tiles[tile].y + threadIdx.x;
                float g = 0.f, d = 0.f, c1 = 0.f, c2 = 0.f;
                if (n < S.V) {
                    const Site<W, K> w = apply_d<W, K>(S.t32, n, S, !first_dag);
                    YK_ST(W, K, Wb(S), n, w);
                    const Site<W, K> r = YK_LD(W, K, Rb(S, nxt), n);
                    const Site<W, K> sk = YK_LD(W, K, Sb(S, cur), n);
                    const Site<W, K> pk = YK_LD(W, K, S.p32[0], n);
                    g = site_dotf<K>(r, r);
                    d = site_dotf<K>(w, r);
                    c1 = site_dotf<K>(r, sk) + site_dotf<K>(pk, w);
                    c2 = site_dotf<K>(pk, sk);
                }
                put_partial_f(a, tile, g, d, 0.f, c1, c2, red, true);
            }
            if (threadIdx.x == 0) {
                for (int j = 0; j < nsl; ++j)
                    if (sl[j].active && sl[j].ru) {
                        sl[j].ru = 0;
                        sl[j].ru_done = 1;
                    }
                s_nru += 1;
            }
            if (!gsync(a.bar, a.err)) return;
        }
    }
    if (threadIdx.x == 0)
        for (int j = 0; j < nsl; ++j) publish(a, sl[j], s_nru);
}

// Resets the barrier, counters and activity flags before a solve.
__global__ void cg_prepare_kernel(CGArgs a)
{
    for (int i = a.sys_first + threadIdx.x; i < a.sys_first + a.sys_count; i += blockDim.x) {
        a.st[i].counter = 0;
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
static const void* kernel_of()
{
    if constexpr (MIXED)
        return (const void*)cgcg_kernel<K>;
    else
        return (const void*)cg64_kernel<K>;
}

template <int K, bool MIXED>
static int max_grid_t()
{
    static int maxg = -1;
    if (maxg < 0) maxg = max_coresident(kernel_of<K, MIXED>(), kBlock);
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
    if constexpr (MIXED)
        return cudaLaunchKernelEx(&cfg, cgcg_kernel<K>, a);
    else
        return cudaLaunchKernelEx(&cfg, cg64_kernel<K>, a);
}

cudaError_t launch_cg(const CGArgs& a, int K, bool mixed, cudaStream_t stream, int* grid_out)
{
    if (K == 1) return mixed ? launch_cg_t<1, true>(a, stream, grid_out) : launch_cg_t<1, false>(a, stream, grid_out);
    return mixed ? launch_cg_t<2, true>(a, stream, grid_out) : launch_cg_t<2, false>(a, stream, grid_out);
}

}  // namespace yk
