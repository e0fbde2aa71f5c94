// yk_cg.cu -- batched CG on D^dag D (or D D^dag) as one persistent
// cooperative kernel per solve: the algorithm of code/src/CGsolver.cu:72-170
// (x0 = 0, r = p = b, alpha = |r|^2 / <p, A p>, x += alpha p, r -= alpha A p,
// beta = |r'|^2 / |r|^2, p = r + beta p, stop when sqrt(|r|^2) <= tol or after
// IterMax iterations) with one neighbour synchronisation and one grid-wide
// reduction per iteration (the reference pays 15 grid syncs):
//
//   A(k): r_k = r_{k-1} - alpha A p_{k-1} and p_k = r_k + beta p_{k-1} are
//         formed on the fly at each site and its four neighbours, t = D_first
//         p_k is stored, x += alpha p_{k-1}                -> neighbour sync
//   B(k): A p_k = D_second t; per-tile partials of |r_k|^2, |A p_k|^2,
//         <p_k, A p_k> and <r_k, A p_k>                     -> grid reduction
//
// The block that arrives last at the grid barrier sums the partials of every
// system in a fixed order and runs the scalar recurrence: the stopping rule on
// the directly summed |r_k|^2, alpha_k = |r_k|^2 / <p_k, A p_k>, |r_{k+1}|^2 =
// |r_k - alpha_k A p_k|^2 expanded in the sums, beta_k = |r_{k+1}|^2 / |r_k|^2.
// It publishes the coefficients together with the barrier; the other blocks
// wait only for that.  r and p are double-buffered (A(k+1) of one block may
// overlap the neighbour reads of A(k) of another); t and A p are not (a grid
// reduction or a neighbour sync separates their writes from the last reads).
//
// FP64: every vector and scalar in FP64.  MIXED: FP32 vectors, stencils and
// per-warp sums, FP64 partial sums and scalars; the solution is an FP64 x plus
// an FP32 increment.  When |r| reaches the target, drops below reliable_delta
// times its maximum since the last update, every reliable_every iterations and
// at the cap, a reliable update folds the increment into x, recomputes
// r = b - A x in FP64, re-orthogonalises p against it (p <- p - <r, p> r /
// |r|^2) and convergence is only declared on that FP64 residual.
//
// One launch solves every (chain, rhs) system; blocks own contiguous ranges of
// 256-site tiles and wait only for the blocks that hold their stencil
// neighbours.  Every wait is bounded (about 2 s): a block that gives up sets
// YK_ETIMEOUT and every block leaves.
#include <cstdio>
#include <type_traits>

#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

#ifdef YK_CG_CHECKED
// Self-checking build: every site access of the CG kernel is checked against
// the system's volume and for null buffers; the first bad access is printed
// with its source line and skipped.
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
constexpr int kMaxDeps = 64;
constexpr long long kWaitCycles = 4000000000LL;   // about 2 s at 2 GHz

// What a system does in the next pass (published with each grid reduction).
enum CGMode {
    kIdle = 0,   // retired
    kStep = 1,   // ordinary iteration
    kRu = 2,     // reliable update (mixed): fold x, then r = b - A x in FP64
    kRedo = 3,   // after a reliable update: p = c r + beta p from the FP64 residual
    kWait = 4,   // another system's reliable update runs; this one already stepped
};

// Per-block copy of the coefficients of one system whose tiles it owns.
struct SysLocal {
    int sys;
    int mode;
    double alpha_re, alpha_im, beta, c_re, c_im;
};

// Blocks holding stencil neighbours of this block's sites.
struct Deps {
    int n;
    int all;   // more than kMaxDeps: wait for every block
    int b[kMaxDeps];
};

// True when the wait should end: timed out (recorded) or another block failed.
__device__ __forceinline__ bool wait_over(long long t0, int* err)
{
    if (clock64() - t0 > kWaitCycles) {
        atomicCAS(err, 0, YK_ETIMEOUT);
        return true;
    }
    return *(volatile int*)err != 0;
}

__device__ __forceinline__ void wait_flag(const unsigned* f, unsigned epoch, int* err)
{
    const volatile unsigned* q = f;
    const long long t0 = clock64();
    while ((int)(*q - epoch) < 0)
        if (wait_over(t0, err)) return;
}

// Neighbour synchronisation: publish this block's epoch, wait until every
// block in `d` has published it too.  Release: bar.sync + thread 0's fence;
// acquire: each waiting thread's fence + bar.sync.
__device__ bool nsync(const CGArgs& a, unsigned epoch, const Deps& d)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        *(volatile unsigned*)(a.flags + (size_t)blockIdx.x * kFlagStride) = epoch;
    }
    if (d.all) {
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            if (b != (int)blockIdx.x) wait_flag(a.flags + (size_t)b * kFlagStride, epoch, a.err);
        __threadfence();
    } else if ((int)threadIdx.x < d.n) {
        wait_flag(a.flags + (size_t)d.b[threadIdx.x] * kFlagStride, epoch, a.err);
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)a.err == 0;
}

// The block's system table and neighbour blocks, from its tile range [tb, te).
// A tile's stencil reaches at most Nx sites away (wrapping within its system),
// i.e. fewer than Nx / 256 + 2 tiles; only tiles that close to an end of the
// block's range or of their system can reach another block.
__device__ void setup_block(const CGArgs& a, int tb, int te, SysLocal* sl, int* nsl, int* tslot, Deps* dp)
{
    if (threadIdx.x == 0) {
        int n = 0, last = -1, nd = 0, all = 0;
        for (int t = tb; t < te; ++t) {
            const int s = a.tiles[t].x;
            if (s != last) {
                if (n == kMaxSysPerBlock) {
                    atomicCAS(a.err, 0, YK_EINVAL);
                    break;
                }
                SysLocal& L = sl[n];
                L.sys = s;
                L.mode = kStep;
                L.alpha_re = L.alpha_im = L.beta = L.c_im = 0.0;
                L.c_re = 1.0;
                ++n;
                last = s;
            }
            tslot[t - tb] = n - 1;
            const SysDev& S = a.sys[s];
            const int h = S.Nx / kTile + 2;
            const int rel = t - S.tile0;
            if (t - tb >= h && te - 1 - t >= h && rel >= h && S.ntiles - 1 - rel >= h) continue;
            for (int d = -h; d <= h && !all; ++d) {
                if (d == 0) continue;
                int q = (rel + d) % S.ntiles;
                if (q < 0) q += S.ntiles;
                const int blk = (S.tile0 + q - a.tile_begin) / a.tiles_per_block;
                if (blk == (int)blockIdx.x) continue;
                bool seen = false;
                for (int i = 0; i < nd && !seen; ++i) seen = (dp->b[i] == blk);
                if (seen) continue;
                if (nd == kMaxDeps)
                    all = 1;
                else
                    dp->b[nd++] = blk;
            }
        }
        *nsl = n;
        dp->n = nd;
        dp->all = all;
    }
    __syncthreads();
}

// Coefficients of the block's systems after a grid reduction.
__device__ void load_coefs(const CGArgs& a, SysLocal* sl, int nsl, int* s_nact, int* s_anyru)
{
    for (int j = threadIdx.x; j < nsl; j += blockDim.x) {
        const volatile CGCoef& c = a.coef[sl[j].sys];
        sl[j].mode = c.mode;
        sl[j].alpha_re = c.alpha_re;
        sl[j].alpha_im = c.alpha_im;
        sl[j].beta = c.beta;
        sl[j].c_re = c.c_re;
        sl[j].c_im = c.c_im;
    }
    if (threadIdx.x == 0) {
        *s_nact = *(volatile int*)a.n_active;
        *s_anyru = *(volatile int*)a.any_ru;
    }
    __syncthreads();
}

// Scalar recurrence of one system after its partials were summed (one thread).
// s: |r|^2, |Ap|^2, <p,Ap> re/im, <r,Ap> re/im; after a reliable update
// |r|^2 and <r, p_{k-1}> re/im in s[0], s[2], s[3].
template <bool MIXED>
__device__ void scalar_step(const CGArgs& a, int j, int k, bool ru_round, const double* s, int* s_active,
                            int* s_ru)
{
    volatile CGState& st = a.st[j];
    volatile CGCoef& cf = a.coef[j];
    auto retire = [&](int conv, int status) {
        st.active = 0;
        st.converged = conv;
        st.status = status;
        cf.mode = kIdle;
    };
    const double rr = s[0];
    st.rr = rr;
    st.iters = k;
    if (ru_round) {
        st.n_ru = st.n_ru + 1;
        if (!isfinite(rr)) return retire(0, YK_ENAN);
        if (!(sqrt(rr) > st.stop)) return retire(1, 0);
        if (k >= a.max_iter) return retire(0, YK_ENOCONV);
        // p_k = r + beta (p_{k-1} - gamma r), gamma = <r, p_{k-1}> / |r|^2
        const double beta = rr / st.rr_prev;
        cf.beta = beta;
        cf.c_re = 1.0 - beta * (s[2] / rr);
        cf.c_im = -beta * (s[3] / rr);
        cf.mode = kRedo;
        st.rmax = sqrt(rr);
        atomicAdd(s_active, 1);
        return;
    }
    if (k == 0) {
        st.rr0 = rr;
        st.stop = (a.tol_mode == YK_TOL_ABS) ? a.tol : a.tol * sqrt(rr);
        st.rmax = sqrt(rr);
    }
    if (!isfinite(rr)) return retire(0, YK_ENAN);
    // mixed: x is exact only at k = 0 and after a reliable update
    if ((!MIXED || k == 0) && !(sqrt(rr) > st.stop)) return retire(1, 0);
    if (k >= a.max_iter) return retire(0, YK_ENOCONV);
    // alpha = rr / <p, Ap>, Smith's complex division (CGsolver.cu:137)
    const double c = s[2], d = s[3];
    double ar, ai;
    if (fabs(c) >= fabs(d)) {
        const double q = d / c, den = c + d * q;
        ar = rr / den;
        ai = (-rr * q) / den;
    } else {
        const double q = c / d, den = c * q + d;
        ar = (rr * q) / den;
        ai = -rr / den;
    }
    if (!isfinite(ar) || !isfinite(ai)) return retire(0, YK_ENAN);
    // |r - alpha q|^2 = |r|^2 - 2 Re(alpha <r, q>) + |alpha|^2 |q|^2
    double est = rr - 2.0 * (ar * s[4] - ai * s[5]) + (ar * ar + ai * ai) * s[1];
    if (!(est > 0.0)) est = 0.0;
    st.rr_prev = rr;
    cf.alpha_re = ar;
    cf.alpha_im = ai;
    cf.beta = est / rr;
    cf.c_re = 1.0;
    cf.c_im = 0.0;
    int mode = kStep;
    if constexpr (MIXED) {
        const double rn = sqrt(rr), en = sqrt(est);
        const double rmax = fmax(st.rmax, rn);
        st.rmax = rmax;
        const bool cand = !(rn > st.stop) || !(en > st.stop);
        const bool drop = en < a.reliable_delta * rmax;
        const bool due = a.reliable_every > 0 && (k + 1) % a.reliable_every == 0;
        const bool cap = k + 1 >= a.max_iter;
        if (cand || drop || due || cap) {
            mode = kRu;
            atomicOr(s_ru, 1);
        }
    }
    cf.mode = mode;
    atomicAdd(s_active, 1);
}

// The last block at a grid barrier: sums the partials of every system that
// took part in the pass (one warp per system; lane l adds tiles l, l+32, ...
// in order, then a fixed butterfly) and runs the scalar recurrence.
template <bool MIXED>
__device__ void finish_reduction(const CGArgs& a, int k, bool ru_round, int* s_active, int* s_ru)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) {
        *s_active = 0;
        *s_ru = 0;
    }
    __syncthreads();
    constexpr int U = 8;
    for (int j = a.sys_first + w; j < a.sys_first + a.sys_count; j += nw) {
        const int mode = *(volatile int*)&a.coef[j].mode;
        if (mode == kIdle) continue;
        if (ru_round && mode != kRu) {
            if (lane == 0) {
                *(volatile int*)&a.coef[j].mode = kWait;
                atomicAdd(s_active, 1);
            }
            continue;
        }
        const SysDev& S = a.sys[j];
        double acc[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) acc[q] = 0.0;
        for (int base = lane; base < S.ntiles; base += 32 * U) {
            double2 v[U][3];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                // the address is clamped into the system's tiles, so a load issued
                // ahead of the range test never leaves the array
                const int i = base + 32 * u;
                const int ii = i < S.ntiles ? i : S.ntiles - 1;
                const double2* q = reinterpret_cast<const double2*>(a.partial + S.tile0 + ii);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const double2 t = ld_volatile2(q + c);
                    v[u][c] = (i < S.ntiles) ? t : make_double2(0.0, 0.0);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    acc[2 * c] += v[u][c].x;
                    acc[2 * c + 1] += v[u][c].y;
                }
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) acc[q] = warp_sum(acc[q]);
        if (lane == 0) scalar_step<MIXED>(a, j, k, ru_round, acc, s_active, s_ru);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *(volatile int*)a.n_active = *s_active;
        *(volatile int*)a.any_ru = *s_ru;
    }
}

// Grid barrier that also completes the reduction of the pass: the last block
// to arrive sums the partials and publishes the coefficients, then advances
// the generation the others wait on.
template <bool MIXED>
__device__ bool grid_reduce(const CGArgs& a, unsigned& gen, int k, bool ru_round, int* s_flag, int* s_active,
                            int* s_ru)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned old = atomicAdd(&a.bar->arrive, 1u);
        const int last = (old == gridDim.x - 1) ? 1 : 0;
        if (last) __threadfence();
        *s_flag = last;
    }
    __syncthreads();
    if (*s_flag) {
        finish_reduction<MIXED>(a, k, ru_round, s_active, s_ru);
        __syncthreads();
        if (threadIdx.x == 0) {
            *(volatile unsigned*)&a.bar->arrive = 0u;
            __threadfence();
            *(volatile unsigned*)&a.bar->gen = gen + 1u;
        }
    } else if (threadIdx.x == 0) {
        const volatile unsigned* g = &a.bar->gen;
        const long long t0 = clock64();
        while (*g == gen)
            if (wait_over(t0, a.err)) break;
        __threadfence();
    }
    __syncthreads();
    ++gen;
    return *(volatile int*)a.err == 0;
}

template <typename W, bool MIXED>
__device__ __forceinline__ W diag_of(const SysDev& S, int n)
{
    if constexpr (MIXED)
        return S.diag32[n];
    else
        return 2.0 * S.r + S.m0 + S.g * S.sigma[n];
}

template <typename W, int K, bool MIXED>
__device__ __forceinline__ Site<W, K> apply_d(const W* in, int n, const SysDev& S, bool dag)
{
    const Nbr nb = neighbours(n, S.Nt, S.Nx);
    const Site<W, K> c = YK_LD(W, K, in, n);
    const Site<W, K> tu = YK_LD(W, K, in, nb.tu);
    const Site<W, K> td = YK_LD(W, K, in, nb.td);
    const Site<W, K> xu = YK_LD(W, K, in, nb.xu);
    const Site<W, K> xd = YK_LD(W, K, in, nb.xd);
    const W diag = diag_of<W, MIXED>(S, n);
    return dag ? dirac_combine<W, K, true>(c, tu, td, xu, xd, diag, (W)S.r, (W)nb.sp, (W)nb.sm)
               : dirac_combine<W, K, false>(c, tu, td, xu, xd, diag, (W)S.r, (W)nb.sp, (W)nb.sm);
}

// sum conj(a) b over one site, in the vectors' precision
template <typename W, int K>
__device__ __forceinline__ void site_dot(const Site<W, K>& a, const Site<W, K>& b, W& re, W& im)
{
    re = W(0);
    im = W(0);
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
}

template <typename W, int K>
__device__ __forceinline__ W site_norm2(const Site<W, K>& a)
{
    W s = W(0);
#pragma unroll
    for (int i = 0; i < 4 * K; ++i) s = fma(a.v[i], a.v[i], s);
    return s;
}

// y += (ar + i ai) v
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

// c r + beta p  (c complex)
template <typename W, int K>
__device__ __forceinline__ Site<W, K> p_next(const Site<W, K>& r, const Site<W, K>& p, W beta, W cre, W cim)
{
    Site<W, K> o;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if constexpr (K == 1) {
            o.v[e] = fma(beta, p.v[e], cre * r.v[e]);
        } else {
            const W re = r.v[2 * e], im = r.v[2 * e + 1];
            o.v[2 * e] = fma(beta, p.v[2 * e], fma(cre, re, -cim * im));
            o.v[2 * e + 1] = fma(beta, p.v[2 * e + 1], fma(cre, im, cim * re));
        }
    }
    return o;
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

// Block sums of a tile's six values -> its partial slot.  Per-site values and
// warp sums in T (FP32 for the mixed solver), FP64 across the warps.  Values
// listed in `skip` are known to be zero and are not reduced.
template <typename T, int SKIP_MASK>
__device__ __forceinline__ void put_partial(const CGArgs& a, int tile, T (&v)[6], double* red)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < 6; ++i)
        if (!((SKIP_MASK >> i) & 1))
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < 6; ++i) red[w * 6 + i] = (double)v[i];
    __syncthreads();
    if (w == 0) {
        double t[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            t[i] = lane < nw ? red[lane * 6 + i] : 0.0;
            if (!((SKIP_MASK >> i) & 1)) t[i] = warp_sum(t[i]);
        }
        if (lane == 0) {
#ifdef YK_CG_CHECKED
            if (tile < a.tile_begin || tile >= a.tile_end) {
                if (atomicCAS(&g_cg_bad, 0, __LINE__) == 0) printf("cg check: bad partial tile %d\n", tile);
                return;
            }
#endif
            Partial p;
#pragma unroll
            for (int i = 0; i < 6; ++i) p.v[i] = t[i];
            a.partial[tile] = p;
        }
    }
}

}  // namespace

template <int K, bool MIXED>
__global__ void __launch_bounds__(kBlock) cg_kernel(CGArgs a)
{
    using W = typename std::conditional<MIXED, float, double>::type;
    // the imaginary parts (slots 3 and 5) vanish on the real K = 1 path
    constexpr int kSkipIm = (K == 1) ? ((1 << 3) | (1 << 5)) : 0;
    __shared__ double red[64];
    __shared__ SysLocal sl[kMaxSysPerBlock];
    __shared__ int nsl;
    __shared__ int tslot[kMaxTilesPerBlock];
    __shared__ Deps deps;
    __shared__ int s_flag, s_active, s_ru, s_nact, s_anyru;
    const int tb = a.tile_begin + blockIdx.x * a.tiles_per_block;
    const int te = min(tb + a.tiles_per_block, a.tile_end);
    setup_block(a, tb, te, sl, &nsl, tslot, &deps);
    if (*(volatile int*)a.err) return;   // the other blocks' waits see the flag and end
    const bool first_dag = (a.mtype == YK_NORMAL);   // Normal: A = D D^dag, apply D^dag first
    unsigned epoch = 0, gen = 0;

    auto Rv = [](const SysDev& S, int i) -> W* {
        if constexpr (MIXED) return S.r32[i]; else return S.r64[i];
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

    // B(k): Ap = D_second t and the partials of every system that stepped
    auto pass_b = [&](int cur) {
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            if (L.mode == kIdle || L.mode == kRu) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            W v[6] = {W(0), W(0), W(0), W(0), W(0), W(0)};
            if (n < S.V) {
                const Site<W, K> ap = apply_d<W, K, MIXED>(Tv(S), n, S, !first_dag);
                YK_ST(W, K, Av(S), n, ap);
                const Site<W, K> r = YK_LD(W, K, Rv(S, cur), n);
                const Site<W, K> p = YK_LD(W, K, Pv(S, cur), n);
                v[0] = site_norm2<W, K>(r);
                v[1] = site_norm2<W, K>(ap);
                site_dot<W, K>(p, ap, v[2], v[3]);
                site_dot<W, K>(r, ap, v[4], v[5]);
            }
            put_partial<W, kSkipIm>(a, tile, v, red);
        }
    };

    // ---------------- round 0: b, x = 0, r_0 = p_0 = b; t = D_first p_0; B(0)
    for (int tile = tb; tile < te; ++tile) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + threadIdx.x;
        if (n >= S.V) continue;
        const Site<double, K> bv = S.gen_eta ? eta_site<K>(S, n, a.eta_kind) : YK_LD(double, K, S.b, n);
        if (S.gen_eta) YK_ST(double, K, S.b, n, bv);
        Site<double, K> z;
        Site<W, K> bw, zw;
#pragma unroll
        for (int i = 0; i < 4 * K; ++i) {
            z.v[i] = 0.0;
            zw.v[i] = W(0);
            bw.v[i] = (W)bv.v[i];
        }
        YK_ST(double, K, S.x, n, z);
        if constexpr (MIXED) {
            YK_ST(W, K, S.xs32, n, zw);
            S.diag32[n] = (float)(2.0 * S.r + S.m0 + S.g * S.sigma[n]);
        }
        YK_ST(W, K, Rv(S, 0), n, bw);
        YK_ST(W, K, Pv(S, 0), n, bw);
    }
    if (!nsync(a, ++epoch, deps)) return;
    for (int tile = tb; tile < te; ++tile) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + threadIdx.x;
        if (n >= S.V) continue;
        YK_ST(W, K, Tv(S), n, (apply_d<W, K, MIXED>(Pv(S, 0), n, S, first_dag)));
    }
    if (!nsync(a, ++epoch, deps)) return;
    pass_b(0);
    if (!grid_reduce<MIXED>(a, gen, 0, false, &s_flag, &s_active, &s_ru)) return;

    int k = 1;
    while (k <= a.max_iter) {   // every system retires at k = max_iter at the latest
        load_coefs(a, sl, nsl, &s_nact, &s_anyru);
        if (s_nact == 0) break;
        const bool any_ru = MIXED && s_anyru;
        const int cur = k & 1, prv = cur ^ 1;
        // ---------------- A(k)
        for (int tile = tb; tile < te; ++tile) {
            const SysLocal& L = sl[tslot[tile - tb]];
            const int mode = L.mode;
            if (mode != kStep && mode != kRu && mode != kRedo) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + threadIdx.x;
            if (n >= S.V) continue;
            if constexpr (MIXED) {
                if (mode == kRu) {
                    // fold x_k = x + xs + alpha p_{k-1} into the FP64 x; xs = 0
                    Site<double, K> xv = YK_LD(double, K, S.x, n);
                    const Site<W, K> xs = YK_LD(W, K, S.xs32, n);
                    const Site<W, K> pv = YK_LD(W, K, Pv(S, prv), n);
                    Site<double, K> pd;
                    Site<W, K> zw;
#pragma unroll
                    for (int i = 0; i < 4 * K; ++i) {
                        xv.v[i] += (double)xs.v[i];
                        pd.v[i] = (double)pv.v[i];
                        zw.v[i] = W(0);
                    }
                    site_axpy<double, K>(xv, L.alpha_re, L.alpha_im, pd);
                    YK_ST(double, K, S.x, n, xv);
                    YK_ST(W, K, S.xs32, n, zw);
                    continue;
                }
            }
            const Nbr nb = neighbours(n, S.Nt, S.Nx);
            const int64_t m5[5] = {n, nb.tu, nb.td, nb.xu, nb.xd};
            const W beta = (W)L.beta;
            Site<W, K> pn[5];
            if (mode == kStep) {
                const W ar = (W)L.alpha_re, ai = (W)L.alpha_im;
                Site<W, K> r_own, p_old;
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    Site<W, K> r = YK_LD(W, K, Rv(S, prv), m5[q]);
                    const Site<W, K> ap = YK_LD(W, K, Av(S), m5[q]);
                    const Site<W, K> po = YK_LD(W, K, Pv(S, prv), m5[q]);
                    site_axpy<W, K>(r, -ar, -ai, ap);
#pragma unroll
                    for (int i = 0; i < 4 * K; ++i) pn[q].v[i] = fma(beta, po.v[i], r.v[i]);
                    if (q == 0) {
                        r_own = r;
                        p_old = po;
                    }
                }
                Site<W, K> xv = YK_LD(W, K, Xv(S), n);
                site_axpy<W, K>(xv, ar, ai, p_old);
                YK_ST(W, K, Xv(S), n, xv);
                YK_ST(W, K, Rv(S, cur), n, r_own);
            } else {
                // kRedo: r_k is the FP64 residual (rounded) in R[cur]
                const W cre = (W)L.c_re, cim = (W)L.c_im;
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    const Site<W, K> r = YK_LD(W, K, Rv(S, cur), m5[q]);
                    const Site<W, K> po = YK_LD(W, K, Pv(S, prv), m5[q]);
                    pn[q] = p_next<W, K>(r, po, beta, cre, cim);
                }
            }
            const W diag = diag_of<W, MIXED>(S, n);
            const Site<W, K> t = first_dag
                ? dirac_combine<W, K, true>(pn[0], pn[1], pn[2], pn[3], pn[4], diag, (W)S.r, (W)nb.sp, (W)nb.sm)
                : dirac_combine<W, K, false>(pn[0], pn[1], pn[2], pn[3], pn[4], diag, (W)S.r, (W)nb.sp, (W)nb.sm);
            YK_ST(W, K, Tv(S), n, t);
            YK_ST(W, K, Pv(S, cur), n, pn[0]);
        }
        if (!nsync(a, ++epoch, deps)) return;

        if constexpr (MIXED) {
            if (any_ru) {
                // RU1: t64 = D_first x (FP64)
                for (int tile = tb; tile < te; ++tile) {
                    const SysLocal& L = sl[tslot[tile - tb]];
                    if (L.mode != kRu) continue;
                    const SysDev& S = a.sys[L.sys];
                    const int n = a.tiles[tile].y + threadIdx.x;
                    if (n >= S.V) continue;
                    const Nbr nb = neighbours(n, S.Nt, S.Nx);
                    const Site<double, K> c = YK_LD(double, K, S.x, n);
                    const Site<double, K> tu = YK_LD(double, K, S.x, nb.tu);
                    const Site<double, K> td = YK_LD(double, K, S.x, nb.td);
                    const Site<double, K> xu = YK_LD(double, K, S.x, nb.xu);
                    const Site<double, K> xd = YK_LD(double, K, S.x, nb.xd);
                    const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
                    const Site<double, K> t = first_dag
                        ? dirac_combine<double, K, true>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm)
                        : dirac_combine<double, K, false>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm);
                    YK_ST(double, K, S.t64, n, t);
                }
                if (!nsync(a, ++epoch, deps)) return;
                // RU2: r = b - D_second t64 in FP64 -> R[cur]; |r|^2, <r, p_{k-1}>
                for (int tile = tb; tile < te; ++tile) {
                    const SysLocal& L = sl[tslot[tile - tb]];
                    if (L.mode != kRu) continue;
                    const SysDev& S = a.sys[L.sys];
                    const int n = a.tiles[tile].y + threadIdx.x;
                    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                    if (n < S.V) {
                        const Nbr nb = neighbours(n, S.Nt, S.Nx);
                        const Site<double, K> c = YK_LD(double, K, S.t64, n);
                        const Site<double, K> tu = YK_LD(double, K, S.t64, nb.tu);
                        const Site<double, K> td = YK_LD(double, K, S.t64, nb.td);
                        const Site<double, K> xu = YK_LD(double, K, S.t64, nb.xu);
                        const Site<double, K> xd = YK_LD(double, K, S.t64, nb.xd);
                        const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
                        const Site<double, K> ax = first_dag
                            ? dirac_combine<double, K, false>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm)
                            : dirac_combine<double, K, true>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm);
                        const Site<double, K> bv = YK_LD(double, K, S.b, n);
                        const Site<W, K> pw = YK_LD(W, K, Pv(S, prv), n);
                        Site<double, K> rd, pd;
                        Site<W, K> rw;
#pragma unroll
                        for (int i = 0; i < 4 * K; ++i) {
                            rd.v[i] = bv.v[i] - ax.v[i];
                            rw.v[i] = (W)rd.v[i];
                            pd.v[i] = (double)pw.v[i];
                        }
                        YK_ST(W, K, Rv(S, cur), n, rw);
                        v[0] = site_norm2<double, K>(rd);
                        site_dot<double, K>(rd, pd, v[2], v[3]);
                    }
                    // slots 1, 4, 5 unused here
                    put_partial<double, (1 << 1) | (1 << 4) | (1 << 5) | kSkipIm>(a, tile, v, red);
                }
                if (!grid_reduce<MIXED>(a, gen, k, true, &s_flag, &s_active, &s_ru)) return;
                continue;   // same k: the systems that updated redo A(k)
            }
        }

        // ---------------- B(k)
        pass_b(cur);
        if (!grid_reduce<MIXED>(a, gen, k, false, &s_flag, &s_active, &s_ru)) return;
        ++k;
    }
}

// Resets the barrier, flags, counters and per-system state before a solve.
__global__ void cg_prepare_kernel(CGArgs a)
{
    for (int i = a.sys_first + threadIdx.x; i < a.sys_first + a.sys_count; i += blockDim.x) {
        CGState& s = a.st[i];
        s.rr = s.rr0 = s.rr_prev = s.stop = s.rmax = 0.0;
        s.active = 1;
        s.iters = 0;
        s.converged = 0;
        s.status = 0;
        s.n_ru = 0;
        CGCoef& c = a.coef[i];
        c.alpha_re = c.alpha_im = c.beta = c.c_im = 0.0;
        c.c_re = 1.0;
        c.mode = kStep;
    }
    for (int b = threadIdx.x; b < a.grid; b += blockDim.x) a.flags[(size_t)b * kFlagStride] = 0u;
    if (threadIdx.x == 0) {
        *a.n_active = a.sys_count;
        *a.any_ru = 0;
        a.bar->arrive = 0u;
        a.bar->gen = 0u;
        *a.err = 0;
    }
}

static int max_coresident(const void* fn, int block)
{
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0);
    const int g = per * nsm;
    return g < kMaxGrid ? g : kMaxGrid;
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
    if (tpb > kMaxTilesPerBlock || grid > maxg || grid > kMaxGrid) return cudaErrorInvalidConfiguration;
    a.tiles_per_block = tpb;
    a.grid = grid;
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
