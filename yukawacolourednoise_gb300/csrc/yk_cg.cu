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
#include <cfloat>
#include <cstdio>
#include <cstdlib>
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

#ifdef YK_CG_TIMING
// Timing build: block 0 accumulates the clock cycles of each part of an
// iteration and prints the per-iteration averages when the solve ends.
// g_cg_t: arrival cycles / count, finisher cycles / count, release cycles,
// waiter spin cycles / count, arrival spread (ns, first to last arrival).
__device__ unsigned long long g_cg_t[10];
__device__ unsigned long long g_cg_f[8];   // finisher: start->sums ready, ->scalar done, ->end
__device__ unsigned long long g_cg_first;
__device__ unsigned long long g_cg_q[16];   // single-system reduction, block 0: cycles between marks
#define YK_QMARK(i)                                               \
    do {                                                          \
        if (blockIdx.x == 0 && threadIdx.x == 0) {                \
            const long long t_ = clock64();                       \
            atomicAdd(&g_cg_q[i], (unsigned long long)(t_ - ql)); \
            ql = t_;                                              \
        }                                                         \
    } while (0)
__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
#define YK_TMARK(i)                                              \
    do {                                                         \
        if (blockIdx.x == 0 && threadIdx.x == 0) {               \
            const long long t_ = clock64();                      \
            tacc[i] += t_ - tlast;                               \
            tlast = t_;                                          \
        }                                                        \
    } while (0)
#else
#define YK_TMARK(i) \
    do {            \
    } while (0)
#define YK_QMARK(i) \
    do {            \
    } while (0)
#endif

namespace {

constexpr int kMaxSysPerBlock = 48;
constexpr int kFinListMax = 1024;   // batched solves whose finisher compacts the active systems
constexpr int kRuAlign = 10;        // batched solves: iterations at which triggered reliable updates run
constexpr int kMaxDeps = 64;
constexpr long long kWaitCycles = 4000000000LL;   // about 2 s at 2 GHz

// What a system does in the next pass (published with each grid reduction).
enum CGMode {
    kIdle = 0,   // retired
    kStep = 1,   // ordinary iteration
    kRu = 2,     // reliable update (mixed): fold x, then r = b - A x in FP64
    kRedo = 3,   // after a reliable update: p = c r + beta p from the FP64 residual
    kWait = 4,   // another system's reliable update runs; this one already stepped
    kRu2 = 5,    // the patch kernel's update, second round: the odd hop of chi
    kRu3 = 6,    // and third round: the residual and its partials
};

// Per-block copy of the coefficients of one system whose tiles it owns (FP64,
// and FP32 copies for the mixed solver: a conversion from FP64 costs an FP64
// instruction per thread otherwise).
struct SysLocal {
    int sys;
    int mode;
    double alpha_re, alpha_im, beta, c_re, c_im;
    float f_alpha_re, f_alpha_im, f_beta, f_c_re, f_c_im;
};

template <typename W>
__device__ __forceinline__ W pick(double d, float f)
{
    if constexpr (sizeof(W) == sizeof(float))
        return f;
    else
        return d;
}

// ---------------------------------------------------------------------------
// Float-float sums (hi + lo, about 48 significant bits) for the mixed solver:
// GB300 issues FP64 at 1/64 of the FP32 rate, so its reductions run on the
// FP32 pipes.  Knuth's two-sum; no multiplications, so no FMA contraction.
// ---------------------------------------------------------------------------
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const float s = a.hi + b.hi;
    const float bp = s - a.hi;
    float e = (a.hi - (s - bp)) + (b.hi - bp);
    e += a.lo + b.lo;
    const float hi = s + e;
    return FF{hi, e - (hi - s)};
}

__device__ __forceinline__ FF ff_of(double x)
{
    const float hi = (float)x;
    return FF{hi, (float)(x - (double)hi)};
}

__device__ __forceinline__ FF ff_shfl_xor(FF a, int o)
{
    return FF{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}

// Float-float products and the reciprocal (Dekker's product with the exact
// FMA error term; one Newton step from the FP32 reciprocal).  The explicitly
// rounded intrinsics keep the compiler from contracting the product that the
// error term subtracts.
__device__ __forceinline__ FF ff_renorm(float p, float e)
{
    const float hi = __fadd_rn(p, e);
    return FF{hi, __fsub_rn(e, __fsub_rn(hi, p))};
}

__device__ __forceinline__ FF ff_mul(FF a, FF b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_renorm(p, e);
}

__device__ __forceinline__ FF ff_mul_f(FF a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return ff_renorm(p, e);
}

__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add(a, FF{-b.hi, -b.lo}); }
__device__ __forceinline__ double dbl_of(FF a) { return (double)a.hi + (double)a.lo; }

// 1 / d: y = rn(1 / d.hi), then y + y (1 - d y) with d y and the correction in
// float-float (relative error about 2^-47)
__device__ __forceinline__ FF ff_rcp(FF d)
{
    const float y = __frcp_rn(d.hi);
    const FF e = ff_sub(FF{1.f, 0.f}, ff_mul_f(d, y));
    return ff_add(FF{y, 0.f}, ff_mul_f(e, y));
}

// ---------------------------------------------------------------------------
// Fixed-point sums (mixed single-system solves, real path).  Each tile adds
// round(x * 2^e) of its four values (|r|^2, |Ap|^2, <p,Ap>, <r,Ap>) with a
// 64-bit integer atomic: integer addition is exact and associative, so the
// total is the same whatever order the blocks arrive in, and every block reads
// one word per value instead of every tile's partial.  e comes from the
// previous iteration's totals (identical in every block) with 2^12 of headroom
// for growth and 2^-48 resolution relative to the previous total; a total
// that comes out too large for the headroom is detected by every block alike
// and that iteration falls back to the float-float tile partials, which are
// always written too.
// ---------------------------------------------------------------------------
constexpr int kFixBits = 48;                 // resolution: 2^-48 of the previous total
constexpr long long kFixLimit = 1ll << 61;   // a total at or above this is not trusted
constexpr int kFixOverflowWord = 8;          // fsum[b][0][8]: set when a tile's value was too large

// Largest tile value added to a total of ntiles tiles: ntiles values below
// it cannot overflow 63 bits, whatever their signs.  A larger one is not
// added; the tile flags the total instead.
__device__ __forceinline__ long long fix_tile_limit(int ntiles)
{
    return 1ll << (62 - (32 - __clz(ntiles)));
}

// round(x * 2^e) from the bits of x: integer operations only (no FP64).
// Magnitudes beyond the window saturate to kFixLimit, which the readers
// reject; values below 2^-e round to zero.
__device__ __forceinline__ long long f2fix(float x, int e)
{
    const unsigned u = __float_as_uint(x);
    const int ex = (int)((u >> 23) & 0xffu);
    if (ex == 0) return 0;   // zero (subnormals are below every window used)
    const long long m = (long long)((u & 0x7fffffu) | 0x800000u);
    const int sh = ex - 150 + e;   // x = m * 2^(ex - 150)
    long long v;
    if (sh >= 0)
        v = sh > 38 ? kFixLimit : (m << sh);
    else if (sh > -40)
        v = (m + (1ll << (-sh - 1))) >> (-sh);
    else
        v = 0;
    return (u >> 31) ? -v : v;
}

__device__ __forceinline__ long long to_fixed(FF t, int e) { return f2fix(t.hi, e) + f2fix(t.lo, e); }

// scale exponent for a total of magnitude m (> 0): m * 2^e ~ 2^kFixBits
__device__ __forceinline__ int fix_scale(double m)
{
    int ex;
    frexp(m, &ex);
    return kFixBits - ex;
}

// the same from a fixed-point total S (> 0) at scale e: integer operations only
__device__ __forceinline__ int fix_rescale(long long S, int e)
{
    const int bits = 64 - __clzll(S);   // S < 2^bits, so the total < 2^(bits - e)
    return kFixBits - (bits - e);
}

// 2^k as a float, k in [-126, 127]
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// S * 2^-e as a float-float pair, from the integer's bits: the top 24 bits
// give hi exactly, the bits below give lo (truncated to about 24 bits).  No
// FP64 and no 64-bit conversions.  False when the value lies outside
// [2^-80, 2^100), where the caller takes the FP64 route instead.
__device__ __forceinline__ bool fix_to_ff(long long S, int e, FF& out)
{
    if (S == 0) {
        out = FF{0.f, 0.f};
        return true;
    }
    const unsigned long long u = S < 0 ? 0ull - (unsigned long long)S : (unsigned long long)S;
    const int b = 63 - __clzll((long long)u);   // u in [2^b, 2^(b+1)); |S| < 2^61
    if (b - e < -80 || b - e >= 100) return false;
    const int sh = b > 23 ? b - 23 : 0;              // bits below the top 24
    const unsigned top = (unsigned)(u >> sh);         // < 2^24
    const unsigned long long rest = u - ((unsigned long long)top << sh);   // < 2^sh, sh <= 37
    const float scale = pow2f(sh - e);                // sh - e in [-103, 100]
    const float hi = (float)top * scale;
    const float lo_m = fmaf((float)(unsigned)(rest >> 20), 1048576.f, (float)(unsigned)(rest & 0xfffffu));
    const float lo = lo_m * pow2f(-sh) * scale;
    out = S < 0 ? FF{-hi, -lo} : FF{hi, lo};
    return true;
}

// float-float times float (Dekker's product through the FMA, then a fast two-sum)
__device__ __forceinline__ FF ff_mul(FF a, float b)
{
    const float p = a.hi * b;
    float err = fmaf(a.hi, b, -p);
    err = fmaf(a.lo, b, err);
    const float s = p + err;
    return FF{s, err - (s - p)};
}

__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }

// tile slot of value c (|r|^2, |Ap|^2, <p,Ap> re, <r,Ap> re) on the real path
__device__ __forceinline__ int fix_value_of_slot(int i)
{
    return i == 0 ? 0 : i == 1 ? 1 : i == 2 ? 2 : i == 4 ? 3 : -1;
}

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

__device__ __forceinline__ unsigned ld_acquire_flag(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// True when the wait gave up (timed out, or another block failed).  The
// polling load acquires: what the flag's writer released is visible after it.
__device__ __forceinline__ bool wait_flag(const unsigned* f, unsigned epoch, int* err)
{
    const long long t0 = clock64();
    while ((int)(ld_acquire_flag(f) - epoch) < 0)
        if (wait_over(t0, err)) return true;
    return false;
}

// Neighbour synchronisation: publish this block's epoch, wait until every
// block in `d` has published it too.  Release: bar.sync, then thread 0's
// release store of the flag (the barrier orders the block's writes before
// it); acquire: each waiting thread's acquiring poll, then bar.sync.  False
// when a wait gave up (the final barrier ORs the waiters' outcomes: no global
// read of the error flag on the way out).
__device__ bool nsync(const CGArgs& a, unsigned epoch, const Deps& d)
{
    __syncthreads();
    if (threadIdx.x == 0)
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a.flags + (size_t)blockIdx.x * kFlagStride),
                     "r"(epoch)
                     : "memory");
    int bad = 0;
    if (d.all) {
        for (int b = threadIdx.x; b < (int)gridDim.x && !bad; b += blockDim.x)
            if (b != (int)blockIdx.x) bad = wait_flag(a.flags + (size_t)b * kFlagStride, epoch, a.err);
    } else if ((int)threadIdx.x < d.n) {
        bad = wait_flag(a.flags + (size_t)d.b[threadIdx.x] * kFlagStride, epoch, a.err);
    }
    return __syncthreads_or(bad) == 0;
}

// Whether the launch uses work-balanced block ranges.
__device__ __forceinline__ bool balanced(const CGArgs& a)
{
    return a.balance != nullptr && a.balance[0] == (int)gridDim.x;
}

// The block that owns table tile `pos`: uniform ranges, or the last block
// whose balanced range starts at or before pos (empty ranges share starts).
__device__ __forceinline__ int owner_of(const CGArgs& a, int pos)
{
    if (!balanced(a)) return (pos - a.tile_begin) / a.tiles_per_block;
    const int* st = a.balance + 1;
    int lo = 0, hi = (int)gridDim.x - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (st[mid] <= pos) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The block's tile range [tb, te).
__device__ __forceinline__ void block_range(const CGArgs& a, int* tb, int* te)
{
    if (balanced(a)) {
        *tb = a.balance[1 + blockIdx.x];
        *te = a.balance[2 + blockIdx.x];
    } else {
        *tb = a.tile_begin + blockIdx.x * a.tiles_per_block;
        *te = min(*tb + a.tiles_per_block, a.tile_end);
    }
}

// The block's system table and neighbour blocks, from its tile range [tb, te).
// A tile's stencil reaches at most Nx sites away (wrapping within its system),
// i.e. fewer than Nx / 256 + 2 tiles; only tiles that close to an end of the
// block's range or of their system can reach another block.
__device__ void setup_block(const CGArgs& a, int tb, int te, SysLocal* sl, int* nsl, unsigned char* tslot, Deps* dp)
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
                L.f_alpha_re = L.f_alpha_im = L.f_beta = L.f_c_im = 0.f;
                L.f_c_re = 1.f;
                ++n;
                last = s;
            }
            tslot[t - tb] = (unsigned char)(n - 1);
            const SysDev& S = a.sys[s];
            const int h = S.Nx / kTile + 2;
            const int rel = t - S.tile0;
            if (t - tb >= h && te - 1 - t >= h && rel >= h && S.ntiles - 1 - rel >= h) continue;
            for (int d = -h; d <= h && !all; ++d) {
                if (d == 0) continue;
                int q = (rel + d) % S.ntiles;
                if (q < 0) q += S.ntiles;
                const int blk = owner_of(a, S.tile0 + q);
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

// 16-byte load of data another block wrote before the last synchronisation:
// relaxed at gpu scope (served by L2), independent loads stay in flight
// together, and the asm's memory clobber keeps the compiler from moving it
// across the synchronisation.
__device__ __forceinline__ double2 ld_sync2(const void* p)
{
    double2 v;
    asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p) : "memory");
    return v;
}

// Arrival at the single-system barrier (release: this thread's writes, and the
// block's writes ordered before it by bar.sync, are visible to a block that
// acquires the final count) and the acquiring poll of the count.
__device__ __forceinline__ void arrive_release(unsigned* p)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(p) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ float4 ld_sync4f(const void* p)
{
    float4 v;
    asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}

// ---------------------------------------------------------------------------
// Published coefficients.  The block that finishes a grid reduction writes
// every system's next-pass coefficients as 64-bit words, 32 bits of payload
// and the barrier generation in the high half (an aligned 64-bit access is
// single-copy atomic), and the grid word the same way; a waiting block polls
// the words of its systems and the grid word until each carries the new
// generation -- the data is the flag.  The writer fences once before its
// stores (release; it has no stores of its own outstanding then) and each
// poller fences after its last poll (acquire), which also orders the vector
// data of the pass for the next one.
// ---------------------------------------------------------------------------
struct CoefVals {
    double alpha_re, alpha_im, beta, c_re, c_im;
    int mode;
    int par;   // batched even-odd solves: the system's buffer parity in the next pass
};

__device__ __forceinline__ unsigned long long stamp(unsigned payload, unsigned gen)
{
    return ((unsigned long long)gen << 32) | payload;
}

__device__ __forceinline__ void st_pair(unsigned long long* p, unsigned long long a, unsigned long long b)
{
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}

__device__ __forceinline__ ulonglong2 ld_pair(const unsigned long long* p)
{
    ulonglong2 v;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_word(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_word(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// words: alpha_re, alpha_im, beta, c_re, c_im as (low, high) halves, then mode
__device__ __forceinline__ void publish_coef(CGCoef* c, const CoefVals& v, unsigned gen)
{
    const double d[5] = {v.alpha_re, v.alpha_im, v.beta, v.c_re, v.c_im};
    unsigned long long w[12];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const unsigned long long u = (unsigned long long)__double_as_longlong(d[i]);
        w[2 * i] = stamp((unsigned)u, gen);
        w[2 * i + 1] = stamp((unsigned)(u >> 32), gen);
    }
    w[10] = stamp((unsigned)v.mode, gen);
    w[11] = stamp((unsigned)v.par, gen);
#pragma unroll
    for (int i = 0; i < 6; ++i) st_pair(c->w + 2 * i, w[2 * i], w[2 * i + 1]);
}

// Polls one system's words until all carry `gen`; false if the wait ended.
__device__ bool poll_coef(const CGCoef* c, unsigned gen, CoefVals& v, int* err)
{
    const long long t0 = clock64();
    for (;;) {
        ulonglong2 q[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) q[i] = ld_pair(c->w + 2 * i);
        bool ok = true;
#pragma unroll
        for (int i = 0; i < 6; ++i) ok = ok && (unsigned)(q[i].x >> 32) == gen && (unsigned)(q[i].y >> 32) == gen;
        if (ok) {
            double d[5];
            const unsigned long long h[12] = {q[0].x, q[0].y, q[1].x, q[1].y, q[2].x, q[2].y,
                                              q[3].x, q[3].y, q[4].x, q[4].y, q[5].x, q[5].y};
#pragma unroll
            for (int i = 0; i < 5; ++i)
                d[i] = __longlong_as_double((long long)(((h[2 * i + 1] & 0xffffffffull) << 32) |
                                                        (h[2 * i] & 0xffffffffull)));
            v.alpha_re = d[0];
            v.alpha_im = d[1];
            v.beta = d[2];
            v.c_re = d[3];
            v.c_im = d[4];
            v.mode = (int)(unsigned)(h[10] & 0xffffffffull);
            v.par = (int)(unsigned)(h[11] & 0xffffffffull);
            return true;
        }
        if (wait_over(t0, err)) return false;
    }
}

// After a grid reduction: every block polls the words of its systems and the
// grid word (bounded waits), then copies the coefficients into its table.
__device__ bool poll_coefs(const CGArgs& a, SysLocal* sl, int nsl, unsigned gen, int* s_nact, int* s_anyru)
{
    int bad = 0;
    for (int j = threadIdx.x; j < nsl; j += blockDim.x) {
        CoefVals v;
        if (!poll_coef(a.coef + sl[j].sys, gen, v, a.err)) {
            bad = 1;
        } else {
            sl[j].mode = v.mode;
            sl[j].alpha_re = v.alpha_re;
            sl[j].alpha_im = v.alpha_im;
            sl[j].beta = v.beta;
            sl[j].c_re = v.c_re;
            sl[j].c_im = v.c_im;
            sl[j].f_alpha_re = (float)v.alpha_re;
            sl[j].f_alpha_im = (float)v.alpha_im;
            sl[j].f_beta = (float)v.beta;
            sl[j].f_c_re = (float)v.c_re;
            sl[j].f_c_im = (float)v.c_im;
        }
        __threadfence();
    }
    if (threadIdx.x == blockDim.x - 1) {
        const long long t0 = clock64();
        unsigned long long g;
        while ((unsigned)((g = ld_word(&a.bar->gword)) >> 32) != gen)
            if (wait_over(t0, a.err)) {
                bad = 1;
                break;
            }
        *s_nact = (int)(g & 0x7fffffffull);
        *s_anyru = (int)((g >> 31) & 1ull);
        __threadfence();
    }
    return __syncthreads_or(bad) == 0;
}

// Scalar recurrence of one system after its partials were summed (one thread):
// updates the system's state `st` (a copy) and returns the coefficients of
// the next pass.  s: |r|^2, |Ap|^2, <p,Ap> re/im, <r,Ap> re/im; after a
// reliable update |r|^2 and <r, p_{k-1}> re/im in s[0], s[2], s[3].  FP64
// division and square root each cost ~650 cycles of latency on GB300: the
// comparisons are made on squares, the mixed solver divides in FP32.
template <bool MIXED>
__device__ CoefVals scalar_step(const CGArgs& a, int k, bool ru_round, const double* s, CGState& st, int* s_active,
                                int* s_ru)
{
    CoefVals cv = {0.0, 0.0, 0.0, 1.0, 0.0, kIdle};
    auto retire = [&](int conv, int status) {
        st.active = 0;
        st.converged = conv;
        st.status = status;
        // a reliable-update round has just formed t64 = D_first x of this x
        st.chi_ready = ru_round ? 1 : 0;
        return cv;
    };
    const double rr = s[0];
    st.rr = rr;
    st.iters = k;
    if (ru_round) {
        st.n_ru += 1;
        if (!isfinite(rr)) return retire(0, YK_ENAN);
        if (!(rr > st.stop2)) return retire(1, 0);
        if (k >= a.max_iter) return retire(0, YK_ENOCONV);
        // p_k = r + beta (p_{k-1} - gamma r), gamma = <r, p_{k-1}> / |r|^2;
        // the mixed solver divides in FP32 (its p update is FP32; an FP64
        // division is ~650 cycles on the path every block waits for)
        const float rrf = (float)rr, rpf = (float)st.rr_prev;
        if (MIXED && rrf > FLT_MIN && rpf > FLT_MIN && rrf < FLT_MAX && rpf < FLT_MAX) {
            const float inv = 1.f / rrf;
            const float beta = rrf / rpf;
            cv.beta = (double)beta;
            cv.c_re = (double)(1.f - beta * ((float)s[2] * inv));
            cv.c_im = (double)(-beta * ((float)s[3] * inv));
        } else {
            const double beta = rr / st.rr_prev, inv_rr = 1.0 / rr;
            cv.beta = beta;
            cv.c_re = 1.0 - beta * (s[2] * inv_rr);
            cv.c_im = -beta * (s[3] * inv_rr);
        }
        cv.mode = kRedo;
        st.rmax2 = rr;
        atomicAdd(s_active, 1);
        return cv;
    }
    if (k == 0) {
        // even-odd solves: relative to |eta|^2 (slot 5), the rule of the full solve
        const double ref = a.eo ? s[5] : rr;
        st.stop2 = (a.tol_mode == YK_TOL_ABS) ? a.tol * a.tol : a.tol * a.tol * ref;
        st.rmax2 = rr;
        st.rr0 = ref;
    }
    if (!isfinite(rr)) return retire(0, YK_ENAN);
    // mixed: x is exact only at k = 0 and after a reliable update
    if ((!MIXED || k == 0) && !(rr > st.stop2)) return retire(1, 0);
    if (k >= a.max_iter) return retire(0, YK_ENOCONV);
    // alpha = rr / <p, Ap> = rr conj(<p, Ap>) / |<p, Ap>|^2  (CGsolver.cu:137)
    const double c = s[2], d = s[3];
    double ar, ai;
    if constexpr (MIXED) {
        // alpha = (c' - i d') / (c'^2 + d'^2) with c' = c / rr, d' = d / rr:
        // O(1) terms, so no square underflows FP32 when the residual is small
        // in absolute terms (|r|^2 ~ 1e-21 squares to below FLT_MIN)
        const float rinv = 1.f / (float)rr;
        const float cs = (float)c * rinv, ds = (float)d * rinv;
        const float inv = 1.f / fmaf(cs, cs, ds * ds);
        ar = (double)(cs * inv);
        ai = (double)(-ds * inv);
    } else {
        const double inv_pap = 1.0 / fma(c, c, d * d);
        ar = rr * c * inv_pap;
        ai = -rr * d * inv_pap;
    }
    bool force_ru = false;
    if (!isfinite(ar) || !isfinite(ai)) {
        // a batched system whose convergence candidate waits for its aligned
        // reliable update can iterate into breakdown (p -> 0): it takes the
        // update now, without this step (x is unchanged by alpha = 0)
        if (MIXED && a.sys_count > 1 && !(rr > st.stop2)) {
            ar = ai = 0.0;
            force_ru = true;
        } else {
            return retire(0, YK_ENAN);
        }
    }
    // |r - alpha q|^2 = |r|^2 - 2 Re(alpha <r, q>) + |alpha|^2 |q|^2
    double est = rr - 2.0 * (ar * s[4] - ai * s[5]) + (ar * ar + ai * ai) * s[1];
    if (!(est > 0.0)) est = 0.0;
    st.rr_prev = rr;
    cv.alpha_re = ar;
    cv.alpha_im = ai;
    if constexpr (MIXED)
        cv.beta = (double)((float)est / (float)rr);
    else
        cv.beta = est / rr;
    cv.mode = kStep;
    if constexpr (MIXED) {
        st.rmax2 = fmax(st.rmax2, rr);
        const bool cand = !(rr > st.stop2) || !(est > st.stop2);
        const bool drop = est < a.reliable_delta * a.reliable_delta * st.rmax2;
        const bool due = a.reliable_every > 0 && (k + 1) % a.reliable_every == 0;
        const bool cap = k + 1 >= a.max_iter;
        // Batched solves: a system's own triggers (convergence candidate,
        // residual drop) wait for the next iteration divisible by kRuAlign, so
        // that the systems' FP64 updates share iterations.  An update runs on
        // the few SMs that own the system's tiles, at the FP64 rate, and every
        // other block waits for it at the grid barrier.  A candidate far below
        // its target (the recursion nears breakdown) does not wait.
        // (the batched even-odd kernel runs a system's update inside the
        // ordinary pass, on every block: no alignment)
        const bool aligned = a.sys_count == 1 || a.eo || (k + 1) % kRuAlign == 0;
        const bool deep = est < 1e-6 * st.stop2;
        if (force_ru || (cand && (aligned || deep)) || (drop && aligned) || due || cap) {
            cv.mode = kRu;
            atomicOr(s_ru, 1);
        }
    }
    atomicAdd(s_active, 1);
    return cv;
}

// FP32 copies of the state fields the mixed single-system fast step reads and
// writes (rmax2, rr_prev) or compares against (stop2, delta^2).  `valid` says
// the copies are the current values; the FP64 fields of CGState are brought
// up to date from them whenever the FP64 step takes over.
struct FastShadow {
    float rr_prev, rmax2, stop2, d2;
    int valid;
};

// One step of the mixed single-system recurrence from the four totals
// (|r|^2, |Ap|^2, <p, Ap>, <r, Ap>, converted from fixed point to float-float
// by the lanes of warp 0), on the FP32 pipes: the scalar work runs in one
// thread per block on the critical path, where every FP64 instruction would
// cost tens of cycles.  alpha and beta are FP32 as in scalar_step<true>;
// |r_{k+1}|^2 = |r|^2 - alpha (2 <r, Ap> - alpha |Ap|^2) is formed in
// float-float because its terms cancel.  `due`: the periodic reliable update
// falls on k + 1.  Returns false without changing anything when the ordinary
// case does not hold (first iteration, iteration cap, a non-positive
// curvature or a non-finite alpha); the caller then takes the FP64 step.
__device__ bool fast_step(const CGArgs& a, int k, FF rr, FF apap, FF pap, FF rap, bool due, CGState& st,
                          FastShadow& fs, SysLocal& L)
{
#ifdef YK_CG_TIMING
    long long ql = clock64();
#endif
    if (k == 0 || k >= a.max_iter) return false;
    const float rrf = rr.hi + rr.lo, papf = pap.hi + pap.lo;
    if (!(rrf > 0.f) || !(papf > 0.f)) return false;
    // CGsolver.cu:137.  Approximate division (reciprocal and product, within
    // 2 ulp): every block computes the same bits, which is what matters
    const float alpha = __fdividef(rrf, papf);
    if (!isfinite(alpha)) return false;
    if (!fs.valid) {
        fs.rmax2 = (float)st.rmax2;
        fs.stop2 = fmaxf((float)st.stop2, FLT_MIN);
        fs.d2 = (float)(a.reliable_delta * a.reliable_delta);
        fs.valid = 1;
    }
    const FF w = ff_mul(ff_add(FF{2.f * rap.hi, 2.f * rap.lo}, ff_neg(ff_mul(apap, alpha))), alpha);
    const FF e = ff_add(rr, ff_neg(w));
    float est = e.hi + e.lo;
    if (!(est > 0.f)) est = 0.f;
    const float rmax2 = fmaxf(fs.rmax2, rrf);
    fs.rmax2 = rmax2;
    fs.rr_prev = rrf;
    st.iters = k;
    const bool cand = !(rrf > fs.stop2) || !(est > fs.stop2);
    const bool drop = est < fs.d2 * rmax2;
    const bool cap = k + 1 >= a.max_iter;
    int mode = kStep;
    if (cand || drop || due || cap) {
        // the reliable update that follows runs the FP64 step: hand it the state
        mode = kRu;
        st.rr = (double)rrf;
        st.rr_prev = st.rr;
        st.rmax2 = (double)rmax2;
        fs.valid = 0;
        L.alpha_re = (double)alpha;   // the FP64 fold of x uses the FP64 copy
        L.alpha_im = 0.0;
    }
    st.mode = mode;
    L.mode = mode;
    L.f_alpha_re = alpha;
    L.f_alpha_im = 0.f;
    L.f_beta = __fdividef(est, rrf);
    YK_QMARK(12);
    return true;
}

// The scalar step of a reliable update on the FP32 pipes (scalar_step's
// update branch, the mixed solver's FP32 restart coefficients) for an update
// that leaves the solve running: p_k = r + beta (p_{k-1} - gamma r), beta =
// |r|^2 / |r_{k-1}|^2, gamma = <r, p_{k-1}> / |r|^2.  An update near or below
// the stop (the FP64 comparison decides), at the iteration cap, or with a
// value outside FP32's range takes the FP64 step, which also stores the
// host-visible state.
__device__ bool fast_ru_step(const CGArgs& a, int k, FF rr, FF rp, CGState& st, SysLocal& L)
{
    const float rrf = rr.hi + rr.lo, rpf = (float)st.rr_prev, stop2f = (float)st.stop2;
    if (!(rrf > FLT_MIN) || !(rrf < FLT_MAX) || !(rpf > FLT_MIN) || !(rpf < FLT_MAX)) return false;
    if (!(rrf > 1.001f * stop2f) || k >= a.max_iter) return false;
    const float inv = 1.f / rrf, beta = rrf / rpf;
    const float c_re = 1.f - beta * ((rp.hi + rp.lo) * inv);
    st.n_ru += 1;
    st.rr = (double)rrf;
    st.iters = k;
    st.rmax2 = st.rr;
    st.mode = kRedo;
    L.mode = kRedo;
    L.alpha_re = L.alpha_im = 0.0;
    L.beta = (double)beta;
    L.c_re = (double)c_re;
    L.c_im = 0.0;
    L.f_alpha_re = L.f_alpha_im = 0.f;
    L.f_beta = beta;
    L.f_c_re = c_re;
    L.f_c_im = 0.f;
    return true;
}

__device__ __forceinline__ void load_state(const CGState* p, CGState& st)
{
    const volatile CGState& v = *p;
    st.rr = v.rr;
    st.rr0 = v.rr0;
    st.rr_prev = v.rr_prev;
    st.stop2 = v.stop2;
    st.rmax2 = v.rmax2;
    st.active = v.active;
    st.iters = v.iters;
    st.converged = v.converged;
    st.status = v.status;
    st.n_ru = v.n_ru;
    st.mode = v.mode;
    st.chi_ready = v.chi_ready;
}

__device__ __forceinline__ void store_state(CGState* p, const CGState& st)
{
    volatile CGState& v = *p;
    v.rr = st.rr;
    v.rr0 = st.rr0;
    v.rr_prev = st.rr_prev;
    v.stop2 = st.stop2;
    v.rmax2 = st.rmax2;
    v.active = st.active;
    v.iters = st.iters;
    v.converged = st.converged;
    v.status = st.status;
    v.n_ru = st.n_ru;
    v.mode = st.mode;
    v.chi_ready = st.chi_ready;
}

// The last block at a grid barrier: sums the partials of every system that
// took part in the pass, runs the scalar recurrence and publishes the
// coefficients, the same bits whichever block finishes.  Mixed solver:
// float-float sums on the FP32 pipes, the block's warps in groups of
// G = 8 / (systems) warps (at least one), a group's threads adding tiles t,
// t + 32 G, ... in order, a fixed butterfly in each warp and the warps' sums
// in warp order.  FP64 solver: one warp per system (its 1/64-rate
// instructions are the cost), lanes adding tiles l, l + 32, ... in order,
// then a fixed butterfly.  The partial sums and the system's state are loaded
// in one batch; a single-system solve takes its tile range from the
// arguments.  The system state lives in CGState (read and written only here;
// the host reads it after the solve).
template <bool MIXED>
__device__ __noinline__ void finish_reduction(const CGArgs& a, int k, bool ru_round, int* s_active, int* s_ru, double* red,
                                 unsigned gen)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // Batched solves: the systems still iterating, compacted (their order in
    // the list does not matter: each system's sum has a fixed order); a
    // retired system only republishes its idle coefficients, which the
    // blocks that own its tiles poll.
    __shared__ int s_list[kFinListMax];
    __shared__ int s_nlist;
    const bool listed = a.sys_count > 1 && a.sys_count <= kFinListMax;
    if (threadIdx.x == 0) {
        *s_active = 0;
        *s_ru = 0;
        s_nlist = 0;
    }
    __syncthreads();
    if (listed) {
        const CoefVals idle = {0.0, 0.0, 0.0, 1.0, 0.0, kIdle};
        bool any_idle = false;
        for (int q = threadIdx.x; q < a.sys_count; q += blockDim.x) {
            const int j = a.sys_first + q;
            if (*(volatile const int*)&a.st[j].mode != kIdle) {
                s_list[atomicAdd(&s_nlist, 1)] = j;
            } else {
                if (!any_idle) __threadfence();
                any_idle = true;
                publish_coef(a.coef + j, idle, gen);
            }
        }
        __syncthreads();
    }
    const int nsys = listed ? s_nlist : a.sys_count;
    int G = MIXED ? nw : 1;
    while (G > 1 && G * nsys > nw) G >>= 1;
    const int ngroups = nw / G, gid = w / G, wg = w % G, T = 32 * G, tg = wg * 32 + lane;
    float2* red2 = reinterpret_cast<float2*>(red);
    const int rounds = (nsys + ngroups - 1) / ngroups;
#ifdef YK_CG_TIMING
    const long long f0 = clock64();
    long long f1 = 0, f2 = 0, f_ld = 0;
#endif
    if (rounds == 0 && threadIdx.x == 0) {   // every system retired
        __threadfence();
        st_word(&a.bar->gword, stamp((unsigned)*s_active | ((unsigned)(*s_ru != 0) << 31), gen));
    }
    for (int rnd = 0; rnd < rounds; ++rnd) {
        const int q = rnd * ngroups + gid;
        const bool have = q < nsys;
        const int j = listed ? (have ? s_list[q] : a.sys_first) : a.sys_first + q;
        CGState st;
        int tile0 = 0, ntiles = 0;
        if (have) {
            if (tg == 0) load_state(a.st + j, st);
            if (a.sys_count == 1) {
                tile0 = a.tile_begin;
                ntiles = a.tile_end - a.tile_begin;
            } else {
                tile0 = a.sys[j].tile0;
                ntiles = a.sys[j].ntiles;
            }
        }
        double s[6];
        if constexpr (MIXED) {
            FF acc[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[c] = FF{0.f, 0.f};
#pragma unroll 4
            for (int i = tg; i < ntiles; i += T) {
                const Partial* pp = a.partial + tile0 + i;
                const float4 q0 = ld_sync4f(&pp->f[0]), q1 = ld_sync4f(&pp->f[2]), q2 = ld_sync4f(&pp->f[4]);
                acc[0] = ff_add(acc[0], FF{q0.x, q0.y});
                acc[1] = ff_add(acc[1], FF{q0.z, q0.w});
                acc[2] = ff_add(acc[2], FF{q1.x, q1.y});
                acc[3] = ff_add(acc[3], FF{q1.z, q1.w});
                acc[4] = ff_add(acc[4], FF{q2.x, q2.y});
                acc[5] = ff_add(acc[5], FF{q2.z, q2.w});
            }
#ifdef YK_CG_TIMING
            if (threadIdx.x == 0) f_ld = clock64();
#endif
            // level-outer: the six independent chains interleave
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int c = 0; c < 6; ++c) acc[c] = ff_add(acc[c], ff_shfl_xor(acc[c], o));
            if (lane == 0)
#pragma unroll
                for (int c = 0; c < 6; ++c) red2[w * 6 + c] = make_float2(acc[c].hi, acc[c].lo);
            __syncthreads();
            if (have && tg == 0) {
                FF t[6];
#pragma unroll
                for (int c = 0; c < 6; ++c) t[c] = FF{red2[w * 6 + c].x, red2[w * 6 + c].y};
                for (int u = 1; u < G; ++u)
#pragma unroll
                    for (int c = 0; c < 6; ++c) t[c] = ff_add(t[c], FF{red2[(w + u) * 6 + c].x, red2[(w + u) * 6 + c].y});
#pragma unroll
                for (int c = 0; c < 6; ++c) s[c] = (double)t[c].hi + (double)t[c].lo;
            }
        } else {
            constexpr int U = 8;
            double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            for (int base = tg; base < ntiles; base += T * U) {
                double2 v[U][3];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    // the address is clamped into the system's tiles, so a load
                    // issued ahead of the range test never leaves the array
                    const int i = base + T * u;
                    const int ii = i < ntiles ? i : ntiles - 1;
                    const Partial* pp = a.partial + tile0 + ii;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const double2 t = ld_sync2(&pp->d[2 * c]);
                        v[u][c] = (i < ntiles) ? t : make_double2(0.0, 0.0);
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
#ifdef YK_CG_TIMING
            if (threadIdx.x == 0) f_ld = clock64();
#endif
            // G = 1: the warp is the group; level-outer butterfly
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int c = 0; c < 6; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
#pragma unroll
            for (int c = 0; c < 6; ++c) s[c] = acc[c];
            __syncthreads();
        }
#ifdef YK_CG_TIMING
        if (threadIdx.x == 0) f1 = clock64();
#endif
        const bool writer = have && tg == 0;
        CoefVals cv = {0.0, 0.0, 0.0, 1.0, 0.0, kIdle};
        if (writer && st.mode != kIdle) {
            if (a.eo) {
                // batched even-odd: every system keeps its own iteration index;
                // an update ran in this pass for the systems in kRu, at the
                // index after st.iters, and the pass that redoes its step keeps it
                const int ks = k == 0 ? 0 : (st.mode == kRedo ? st.iters : st.iters + 1);
                cv = scalar_step<MIXED>(a, ks, st.mode == kRu, s, st, s_active, s_ru);
                cv.par = (cv.mode == kRedo ? st.iters : st.iters + 1) & 1;
            } else if (ru_round && st.mode != kRu) {
                cv.mode = kWait;
                atomicAdd(s_active, 1);
            } else {
                cv = scalar_step<MIXED>(a, k, ru_round, s, st, s_active, s_ru);
            }
        }
#ifdef YK_CG_TIMING
        if (threadIdx.x == 0) f2 = clock64();
#endif
        __syncthreads();   // the counts of the round are complete
        const bool last_round = rnd == rounds - 1;
        if (writer || (last_round && threadIdx.x == 0)) __threadfence();
        if (writer) publish_coef(a.coef + j, cv, gen);
        if (last_round && threadIdx.x == 0)
            st_word(&a.bar->gword, stamp((unsigned)*s_active | ((unsigned)(*s_ru != 0) << 31), gen));
        if (writer) {
            st.mode = cv.mode;
            store_state(a.st + j, st);
        }
        __syncthreads();
    }
#ifdef YK_CG_TIMING
    if (threadIdx.x == 0) {
        const long long f3 = clock64();
        atomicAdd(&g_cg_f[0], (unsigned long long)(f1 - f0));
        atomicAdd(&g_cg_f[4], (unsigned long long)(f_ld - f0));
        atomicAdd(&g_cg_f[1], (unsigned long long)(f2 - f1));
        atomicAdd(&g_cg_f[2], (unsigned long long)(f3 - f2));
        atomicAdd(&g_cg_f[3], 1ull);
    }
#endif
}

// Grid barrier that also completes the reduction of the pass: the last block
// to arrive (the arrival counter runs on across the solve) sums the partials
// and publishes the coefficients of generation gen + 1; the caller then
// polls them (poll_coefs).
template <bool MIXED>
__device__ void grid_reduce(const CGArgs& a, unsigned& gen, int k, bool ru_round, int* s_flag, int* s_active,
                            int* s_ru, double* red)
{
    __syncthreads();
#ifdef YK_CG_TIMING
    const long long c0 = clock64();
#endif
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned old = atomicAdd(&a.bar->arrive, 1u);
        const int last = (old + 1u == gridDim.x * (gen + 1u)) ? 1 : 0;
#ifdef YK_CG_TIMING
        if (old == gridDim.x * gen) g_cg_first = gtimer();
        if (last) atomicAdd(&g_cg_t[8], gtimer() - *(volatile unsigned long long*)&g_cg_first);
        atomicAdd(&g_cg_t[0], (unsigned long long)(clock64() - c0));
        atomicAdd(&g_cg_t[1], 1ull);
#endif
        if (last) __threadfence();
        *s_flag = last;
    }
    __syncthreads();
    if (*s_flag) {
#ifdef YK_CG_TIMING
        const long long c1 = clock64();
#endif
        finish_reduction<MIXED>(a, k, ru_round, s_active, s_ru, red, gen + 1u);
#ifdef YK_CG_TIMING
        if (threadIdx.x == 0) {
            atomicAdd(&g_cg_t[2], (unsigned long long)(clock64() - c1));
            atomicAdd(&g_cg_t[3], 1ull);
        }
#endif
    }
    ++gen;
}

// Sum of one system's tile partials, the same bits in every block that calls
// it: mixed solver, every thread adds tiles t, t + blockDim, ... in
// float-float, then a fixed butterfly in each warp and the warps' sums in warp
// order; FP64 solver, warp 0 alone (its 1/64-rate instructions are the cost),
// lanes adding tiles l, l + 32, ... in order, then a fixed butterfly.  The sums
// are valid in thread 0.
template <bool MIXED>
__device__ void sum_partials(const CGArgs& a, int tile0, int ntiles, double* red, double* s)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if constexpr (MIXED) {
        float2* red2 = reinterpret_cast<float2*>(red);
        FF acc[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] = FF{0.f, 0.f};
#pragma unroll 2
        for (int i = threadIdx.x; i < ntiles; i += blockDim.x) {
            const Partial* pp = a.partial + tile0 + i;
            const float4 q0 = ld_sync4f(&pp->f[0]), q1 = ld_sync4f(&pp->f[2]), q2 = ld_sync4f(&pp->f[4]);
            acc[0] = ff_add(acc[0], FF{q0.x, q0.y});
            acc[1] = ff_add(acc[1], FF{q0.z, q0.w});
            acc[2] = ff_add(acc[2], FF{q1.x, q1.y});
            acc[3] = ff_add(acc[3], FF{q1.z, q1.w});
            acc[4] = ff_add(acc[4], FF{q2.x, q2.y});
            acc[5] = ff_add(acc[5], FF{q2.z, q2.w});
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[c] = ff_add(acc[c], ff_shfl_xor(acc[c], o));
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 6; ++c) red2[w * 6 + c] = make_float2(acc[c].hi, acc[c].lo);
        __syncthreads();
        if (w == 0) {
            // the warps' sums by a fixed tree in warp 0 (the same order in every
            // block), not a serial chain of float-float additions on thread 0
            FF t[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) t[c] = lane < nw ? FF{red2[lane * 6 + c].x, red2[lane * 6 + c].y} : FF{0.f, 0.f};
            int o0 = 1;
            while (o0 < nw) o0 <<= 1;
            for (int o = o0 >> 1; o > 0; o >>= 1)
#pragma unroll
                for (int c = 0; c < 6; ++c) t[c] = ff_add(t[c], ff_shfl_xor(t[c], o));
            if (lane == 0)
#pragma unroll
                for (int c = 0; c < 6; ++c) s[c] = (double)t[c].hi + (double)t[c].lo;
        }
    } else {
        if (w == 0) {
            constexpr int U = 8;
            double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            for (int base = lane; base < ntiles; base += 32 * U) {
                double2 v[U][3];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    // the address is clamped into the system's tiles, so a load
                    // issued ahead of the range test never leaves the array
                    const int i = base + 32 * u;
                    const int ii = i < ntiles ? i : ntiles - 1;
                    const Partial* pp = a.partial + tile0 + ii;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const double2 t = ld_sync2(&pp->d[2 * c]);
                        v[u][c] = (i < ntiles) ? t : make_double2(0.0, 0.0);
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
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int c = 0; c < 6; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
#pragma unroll
            for (int c = 0; c < 6; ++c) s[c] = acc[c];
        }
    }
    __syncthreads();
}

// Single-system solves: the grid barrier is an arrival counter only; every
// block then sums the system's tile partials itself (sum_partials: the same
// loads in the same order, so the same bits in every block) and runs the
// scalar recurrence on its own copy of the system state.  No block finishes
// for the others and nothing is published: the chain of the other path
// (finisher's loads, release, the others' polls of the published words) is
// replaced by one round of loads in every block.  Block 0 keeps the
// host-visible CGState up to date.
// after_barrier() runs in every thread once the barrier has been passed
// (the other blocks' writes of the pass are visible), before the scalar
// work: the halo kernel issues the next pass's loads there.
struct NoHook {
    __device__ void operator()() const {}
};

// RUFIX: the caller's reliable updates add their partials to the fixed-point
// totals too (put_partial_ff RU_SCALE), so an update round may take the fast
// path (fast_ru_step) like an ordinary one.
template <int K, bool MIXED, bool RUFIX = false, typename Hook = NoHook>
__device__ __forceinline__ bool solo_reduce_body(const CGArgs& a, unsigned& gen, int k, bool ru_round, double* red,
                                                 CGState& lst, SysLocal& L, int* s_nact, int* s_anyru, int* s_cnt,
                                                 int* esc, int* s_fast, FastShadow& fs, Hook after_barrier = Hook())
{
    constexpr bool kFix = MIXED && K == 1;   // fixed-point sums available
    int bad = 0;   // thread 0: its wait gave up
#ifdef YK_CG_TIMING
    long long ql = clock64();
#endif
    __syncthreads();
#ifdef YK_CG_TIMING
    const long long q0 = clock64();
#endif
    YK_QMARK(0);
    if (threadIdx.x == 0) {
        if (kFix && blockIdx.x == 0) {
            // the buffer of the barrier after this one: nobody reads it any more
            // (its last readers arrived here already) and nobody adds to it
            // before this block has arrived
            long long (*z)[16] = a.bar->fsum[(gen + 2u) % 3u];
            for (int c = 0; c < 4; ++c) z[c][0] = 0;
            z[0][kFixOverflowWord] = 0;
        }
        arrive_release(&a.bar->arrive);
        YK_QMARK(1);
        const unsigned target = gridDim.x * (gen + 1u);
        const long long t0 = clock64();
        while ((int)(ld_acquire(&a.bar->arrive) - target) < 0)
            if (wait_over(t0, a.err)) {
                bad = 1;
                break;
            }
        YK_QMARK(2);
        s_cnt[0] = 0;
        s_cnt[1] = 0;
    }
    ++gen;
    if (__syncthreads_or(bad)) return false;
    // the fixed-point totals of this barrier, if the tiles added them: lanes
    // 0-3 load one each, lane 4 the overflow flag -- ahead of the hook's loads
    const bool fix_now = kFix && (!ru_round || RUFIX) && *s_fast;
    long long Sv = 0;
    unsigned long long over_v = 0ull;
    if (fix_now && threadIdx.x < 5) {
        const long long(*f)[16] = a.bar->fsum[gen % 3u];
        if (threadIdx.x < 4)
            Sv = (long long)ld_word(reinterpret_cast<const unsigned long long*>(&f[threadIdx.x][0]));
        else
            over_v = ld_word(reinterpret_cast<const unsigned long long*>(&f[0][kFixOverflowWord]));
    }
    after_barrier();
    YK_QMARK(3);
    double s[6];
#ifdef YK_CG_TIMING
    const long long q1 = clock64();
#endif
    // fixed-point totals of this barrier, if the tiles added them
    bool fast = false, stepped = false;
    int s_scales = 0;   // thread 0: 2 = next scales set from the integer totals
    __shared__ int s_dec;   // thread 0's verdict on the fixed-point totals (0 none, 1 sums, 2 stepped)
    if constexpr (kFix) {
        if (fix_now) {
            if (threadIdx.x < 32) {
                // lanes 0-3: one total each (load, range check, conversion,
                // next scale); lane 4: the overflow flag; lane 5: the
                // periodic trigger; lane 0 then steps
                const unsigned full = 0xffffffffu;
                const int lane = threadIdx.x;
                bool okl = true, conv = true;
                FF fv = {0.f, 0.f};
                int er = 0, due = 0;
                // an update's <r, p> (lane 2) is at the scale of |r|^2
                const int el = (ru_round && lane == 2) ? esc[0] : (lane < 4 ? esc[lane] : 0);
                if (lane < 4) {
                    okl = Sv < kFixLimit && Sv > -kFixLimit;
                    conv = okl && fix_to_ff(Sv, el, fv);
                    if (lane < 3 && Sv > 0) er = fix_rescale(Sv, el);
                } else if (lane == 4) {
                    okl = over_v == 0ull;
                } else if (lane == 5) {
                    due = a.reliable_every > 0 && (k + 1) % a.reliable_every == 0;
                }
                const bool ok = __all_sync(full, okl);
                const bool convall = __all_sync(full, conv);
                const bool pos = __all_sync(full, (ru_round ? lane != 0 : lane >= 3) || Sv > 0);
                FF v[4];
                long long S[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    v[c] = FF{__shfl_sync(full, fv.hi, c), __shfl_sync(full, fv.lo, c)};
                    S[c] = __shfl_sync(full, Sv, c);
                }
                const int e0 = __shfl_sync(full, er, 0), e1 = __shfl_sync(full, er, 1), e2 = __shfl_sync(full, er, 2);
                due = __shfl_sync(full, due, 5);
                YK_QMARK(4);
                __syncwarp();   // every lane has read esc
                if (lane == 0) {
                    bool done = false;
                    if (ok) {
                        // the ordinary step on the FP32 pipes; the FP64 one otherwise
                        done = convall && lst.mode != kIdle &&
                               (ru_round ? fast_ru_step(a, k, v[0], v[2], lst, L)
                                         : fast_step(a, k, v[0], v[1], v[2], v[3], due != 0, lst, fs, L));
                        if (!done) {
                            s[0] = scalbn((double)S[0], -esc[0]);
                            s[1] = scalbn((double)S[1], -esc[1]);
                            s[2] = scalbn((double)S[2], -(ru_round ? esc[0] : esc[2]));
                            s[4] = scalbn((double)S[3], -esc[3]);
                            s[3] = s[5] = 0.0;
                        }
                        // next scales straight from the integer totals (an
                        // update's round renews the |r|^2 scale only)
                        if (pos) {
                            esc[0] = e0;
                            if (!ru_round) {
                                esc[1] = e1;
                                esc[2] = e2;
                                esc[3] = (e0 + e1) / 2 - 1;   // |<r, Ap>| <= |r| |Ap|
                            }
                            s_scales = 2;   // scales already set
                        } else {
                            s_scales = 3;   // no usable scales: the next sums go through the tile partials
                        }
                    }
                    s_dec = ok ? (done ? 2 : 1) : 0;
                    if (done) {
                        // the block's state for the next pass, before the
                        // barrier that publishes the step
                        *s_nact = 1;
                        *s_anyru = lst.mode == kRu;
                        *s_fast = s_scales == 2 ? 1 : 0;
                    }
                    YK_QMARK(5);
                }
            }
            // s_dec is written again only after the barriers of the passes that follow
            __syncthreads();
            fast = s_dec != 0;
            stepped = s_dec == 2;
            if (stepped) {
                YK_QMARK(6);
#ifdef YK_CG_TIMING
                if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&g_cg_f[3], 1ull);
#endif
                return true;   // coefficients, mode and counts published by the barrier above
            }
        }
    }
    if (!fast) sum_partials<MIXED>(a, a.tile_begin, a.tile_end - a.tile_begin, red, s);
#ifdef YK_CG_TIMING
    const long long q2 = clock64();
#endif
    if (threadIdx.x == 0 && stepped) {
        // (the host-visible state is stored by the FP64 steps: every solve
        // ends in one)
        *s_nact = 1;
        *s_anyru = lst.mode == kRu;
        *s_fast = s_scales == 2 ? 1 : 0;
    } else if (threadIdx.x == 0) {
        if (fs.valid) {
            // the FP64 step continues from the fast steps' FP32 state
            lst.rr_prev = (double)fs.rr_prev;
            lst.rmax2 = (double)fs.rmax2;
            fs.valid = 0;
        }
        CoefVals cv = {0.0, 0.0, 0.0, 1.0, 0.0, kIdle};
        if (lst.mode != kIdle) cv = scalar_step<MIXED>(a, k, ru_round, s, lst, s_cnt, s_cnt + 1);
        lst.mode = cv.mode;
        L.mode = cv.mode;
        L.alpha_re = cv.alpha_re;
        L.alpha_im = cv.alpha_im;
        L.beta = cv.beta;
        L.c_re = cv.c_re;
        L.c_im = cv.c_im;
        L.f_alpha_re = (float)cv.alpha_re;
        L.f_alpha_im = (float)cv.alpha_im;
        L.f_beta = (float)cv.beta;
        L.f_c_re = (float)cv.c_re;
        L.f_c_im = (float)cv.c_im;
        *s_nact = s_cnt[0];
        *s_anyru = s_cnt[1] != 0;
        if (blockIdx.x == 0) store_state(a.st + a.sys_first, lst);
        if constexpr (kFix) {
            // scales of the next iteration's sums, from these totals
            if (fast) {
                *s_fast = s_scales == 2 ? 1 : 0;
            } else if (ru_round) {
                if (s[0] > 0.0 && isfinite(s[0])) esc[0] = fix_scale(s[0]);
            } else {
                const bool ok = s[0] > 0.0 && s[1] > 0.0 && s[2] > 0.0 && isfinite(s[0]) && isfinite(s[1]) &&
                                isfinite(s[2]);
                if (ok) {
                    esc[0] = fix_scale(s[0]);
                    esc[1] = fix_scale(s[1]);
                    esc[2] = fix_scale(s[2]);
                    esc[3] = fix_scale(sqrt(s[0] * s[1]));   // |<r, Ap>| <= |r| |Ap|
                }
                *s_fast = ok ? 1 : 0;
            }
        }
    }
    YK_QMARK(6);
#ifdef YK_CG_TIMING
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        atomicAdd(&g_cg_f[0], (unsigned long long)(q1 - q0));
        atomicAdd(&g_cg_f[4], (unsigned long long)(q2 - q1));
        atomicAdd(&g_cg_f[1], (unsigned long long)(clock64() - q2));
        atomicAdd(&g_cg_f[3], 1ull);
    }
#endif
    __syncthreads();
    YK_QMARK(7);
    return true;
}

// Out of line for cg_kernel, whose registers do not leave room for it inline;
// cg_halo_kernel inlines the body (a call costs a save and restore of
// registers through local memory, which the barrier's acquire leaves cold).
template <int K, bool MIXED>
__device__ __noinline__ bool solo_reduce(const CGArgs& a, unsigned& gen, int k, bool ru_round, double* red, CGState& lst,
                                         SysLocal& L, int* s_nact, int* s_anyru, int* s_cnt, int* esc, int* s_fast,
                                         FastShadow& fs)
{
    return solo_reduce_body<K, MIXED>(a, gen, k, ru_round, red, lst, L, s_nact, s_anyru, s_cnt, esc, s_fast, fs);
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
    Site<W, K> o = dag ? dirac_combine<W, K, true>(c, tu, td, xu, xd, diag, (W)S.r, (W)nb.sp, (W)nb.sm)
                       : dirac_combine<W, K, false>(c, tu, td, xu, xd, diag, (W)S.r, (W)nb.sp, (W)nb.sm);
    pion_term<W, K>(o, c, S.pi, n, S.V, S.g, dag);
    return o;
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

// Sums of a tile's six values -> its partial slot.  A block processes
// blockDim / 256 tiles at once, one per 256-thread half; each half reduces its
// own tile (its 8 warps in warp order) and writes the slot if `write`.  Per-site
// values and warp sums in T, FP64 across the warps.  Values listed in
// SKIP_MASK are known to be zero and are not reduced.  Every thread of the
// block calls this (it synchronises the block).
template <typename T, int SKIP_MASK>
__device__ __forceinline__ void put_partial(const CGArgs& a, int tile, bool write, T (&v)[6], double* red)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int hw = kTile / 32;   // warps per tile
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < 6; ++i)
            if (!((SKIP_MASK >> i) & 1)) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < 6; ++i) red[w * 6 + i] = (double)v[i];
    __syncthreads();
    // one thread per value adds the warps' sums in warp order (few FP64
    // instructions: GB300 issues them at 1/64 of the FP32 rate)
    const int ts = threadIdx.x % kTile, w0 = (threadIdx.x / kTile) * hw;
    if (write && ts < 6) {
        const int i = ts;
        double t = red[w0 * 6 + i];
        for (int u = 1; u < hw; ++u) t += red[(w0 + u) * 6 + i];
#ifdef YK_CG_CHECKED
        if (tile < a.tile_begin || tile >= a.tile_end) {
            if (atomicCAS(&g_cg_bad, 0, __LINE__) == 0) printf("cg check: bad partial tile %d\n", tile);
            return;
        }
#endif
        a.partial[tile].d[i] = t;
    }
}

// Sums of a tile's six values -> its partial slot as float-float pairs (mixed
// solver), one tile per 256-thread half as in put_partial.  WARP_FF: the
// per-site values carry a low part (FP64 residuals of a reliable update) and
// the warp butterfly runs in float-float; otherwise the warp sums are plain
// FP32 (the per-site values are FP32 products).  The warps' sums are added in
// warp order by one thread per value.
// RU_SCALE: a reliable update's partials (|r|^2 in slot 0, <r, p> in slot 2)
// go into the fixed-point totals both at the scale of |r|^2.
template <int SKIP_MASK, bool WARP_FF, bool RU_SCALE = false>
__device__ __forceinline__ void put_partial_ff(const CGArgs& a, int tile, bool write, FF (&v)[6], double* red,
                                               long long (*fsum)[16] = nullptr, const int* esc = nullptr)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int hw = kTile / 32;   // warps per tile
    float2* red2 = reinterpret_cast<float2*>(red);
    // level-outer: the independent chains interleave
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < 6; ++i)
            if (!((SKIP_MASK >> i) & 1)) {
                if constexpr (WARP_FF)
                    v[i] = ff_add(v[i], ff_shfl_xor(v[i], o));
                else
                    v[i].hi += __shfl_xor_sync(0xffffffffu, v[i].hi, o);
            }
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < 6; ++i) red2[w * 6 + i] = make_float2(v[i].hi, v[i].lo);
    __syncthreads();
    const int ts = threadIdx.x % kTile, w0 = (threadIdx.x / kTile) * hw;
    // the tile's hw warp sums of slot i by a fixed tree over an aligned group
    // of hw lanes (thread ts < 6 hw: slot ts / hw, warp ts % hw; the groups of
    // slots 0-3 fill the tile's first warp, those of 4-5 half its second)
    static_assert(6 * hw <= 64 && (hw & (hw - 1)) == 0, "six slots' groups in two warps");
    if (ts < 6 * hw) {
        const int i = ts / hw, u = ts % hw;
        const unsigned mask = ts < 32 ? 0xffffffffu : (unsigned)((1ull << (6 * hw - 32)) - 1ull);
        FF t{red2[(w0 + u) * 6 + i].x, red2[(w0 + u) * 6 + i].y};
#pragma unroll
        for (int o = hw / 2; o > 0; o >>= 1)
            t = ff_add(t, FF{__shfl_xor_sync(mask, t.hi, o), __shfl_xor_sync(mask, t.lo, o)});
        if (!write || u != 0) return;
#ifdef YK_CG_CHECKED
        if (tile < a.tile_begin || tile >= a.tile_end) {
            if (atomicCAS(&g_cg_bad, 0, __LINE__) == 0) printf("cg check: bad partial tile %d\n", tile);
            return;
        }
#endif
        a.partial[tile].f[i] = make_float2(t.hi, t.lo);
        if (fsum) {
            const int c = fix_value_of_slot(i);
            if (c >= 0) {
                const long long v = to_fixed(t, esc[(RU_SCALE && c == 2) ? 0 : c]),
                                lim = fix_tile_limit(a.tile_end - a.tile_begin);
                if (v < lim && v > -lim)
                    atomicAdd(reinterpret_cast<unsigned long long*>(&fsum[c][0]), (unsigned long long)v);
                else
                    atomicOr(reinterpret_cast<unsigned long long*>(&fsum[0][kFixOverflowWord]), 1ull);
            }
        }
    }
}

// Reliable update (mixed solver), first part, at one site of a system in
// mode kRu: fold x_k = x + xs + alpha p_{k-1} into the FP64 x; xs = 0.
template <int K>
__device__ __forceinline__ void ru_fold(const SysDev& S, int n, const SysLocal& L, int prv)
{
    Site<double, K> xv = YK_LD(double, K, S.x, n);
    const Site<float, K> xs = YK_LD(float, K, S.xs32, n);
    const Site<float, K> pv = YK_LD(float, K, S.p32[prv], n);
    Site<double, K> pd;
    Site<float, K> zw;
#pragma unroll
    for (int i = 0; i < 4 * K; ++i) {
        xv.v[i] += (double)xs.v[i];
        pd.v[i] = (double)pv.v[i];
        zw.v[i] = 0.f;
    }
    site_axpy<double, K>(xv, L.alpha_re, L.alpha_im, pd);
    YK_ST(double, K, S.x, n, xv);
    YK_ST(float, K, S.xs32, n, zw);
}

// Reliable update (mixed solver), second part, after the fold and a
// neighbour sync: t64 = D_first x in FP64, a neighbour sync, then
// r = b - D_second t64 in FP64, rounded into R[cur], with the partials |r|^2
// and <r, p_{k-1}> of every tile in mode kRu.  The block's tiles go
// blockDim / 256 at a time as in the passes of the kernels calling this.
// False when a neighbour wait gave up.
template <int K>
__device__ bool ru_residual(const CGArgs& a, const SysLocal* sl, const unsigned char* tslot, int tb, int te, bool first_dag,
                            int cur, int prv, unsigned& epoch, const Deps& deps, double* red)
{
    constexpr int kSkipIm = (K == 1) ? ((1 << 3) | (1 << 5)) : 0;
    const int TP = blockDim.x / kTile, hf = threadIdx.x / kTile, ts = threadIdx.x % kTile;
    // RU1: t64 = D_first x (FP64)
    for (int tile = tb + hf; tile < te; tile += TP) {
        const SysLocal& L = sl[tslot[tile - tb]];
        if (L.mode != kRu) continue;
        const SysDev& S = a.sys[L.sys];
        const int n = a.tiles[tile].y + ts;
        if (n >= S.V) continue;
        const Nbr nb = neighbours(n, S.Nt, S.Nx);
        const Site<double, K> c = YK_LD(double, K, S.x, n);
        const Site<double, K> tu = YK_LD(double, K, S.x, nb.tu);
        const Site<double, K> td = YK_LD(double, K, S.x, nb.td);
        const Site<double, K> xu = YK_LD(double, K, S.x, nb.xu);
        const Site<double, K> xd = YK_LD(double, K, S.x, nb.xd);
        const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
        Site<double, K> t = first_dag
            ? dirac_combine<double, K, true>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm)
            : dirac_combine<double, K, false>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm);
        pion_term<double, K>(t, c, S.pi, n, S.V, S.g, first_dag);
        YK_ST(double, K, S.t64, n, t);
    }
    if (!nsync(a, ++epoch, deps)) return false;
    // RU2: r = b - D_second t64 in FP64 -> R[cur]; |r|^2, <r, p_{k-1}>
    for (int base = tb; base < te; base += TP) {   // the same trip count in every thread
        const int tile = base + hf;
        bool on = tile < te;
        const SysLocal& L = sl[tslot[(on ? tile : tb) - tb]];
        on = on && L.mode == kRu;
        const SysDev& S = a.sys[L.sys];
        const int n = on ? a.tiles[tile].y + ts : 0;
        double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (on && n < S.V) {
            const Nbr nb = neighbours(n, S.Nt, S.Nx);
            const Site<double, K> c = YK_LD(double, K, S.t64, n);
            const Site<double, K> tu = YK_LD(double, K, S.t64, nb.tu);
            const Site<double, K> td = YK_LD(double, K, S.t64, nb.td);
            const Site<double, K> xu = YK_LD(double, K, S.t64, nb.xu);
            const Site<double, K> xd = YK_LD(double, K, S.t64, nb.xd);
            const double diag = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
            Site<double, K> ax = first_dag
                ? dirac_combine<double, K, false>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm)
                : dirac_combine<double, K, true>(c, tu, td, xu, xd, diag, S.r, (double)nb.sp, (double)nb.sm);
            pion_term<double, K>(ax, c, S.pi, n, S.V, S.g, !first_dag);
            const Site<double, K> bv = YK_LD(double, K, S.b, n);
            const Site<float, K> pw = YK_LD(float, K, S.p32[prv], n);
            Site<double, K> rd, pd;
            Site<float, K> rw;
#pragma unroll
            for (int i = 0; i < 4 * K; ++i) {
                rd.v[i] = bv.v[i] - ax.v[i];
                rw.v[i] = (float)rd.v[i];
                pd.v[i] = (double)pw.v[i];
            }
            YK_ST(float, K, S.r32[cur], n, rw);
            v[0] = site_norm2<double, K>(rd);
            site_dot<double, K>(rd, pd, v[2], v[3]);
        }
        // slots 1, 4, 5 unused here
        FF f[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) f[i] = ff_of(v[i]);
        put_partial_ff<(1 << 1) | (1 << 4) | (1 << 5) | kSkipIm, true>(a, tile, on, f, red);
    }
    return true;
}

}  // namespace

// Threads per block of the CG kernel: two 256-site tiles at once for the real
// path (one block per SM, so every SM holds the same work and the blocks reach
// the barriers together), one tile for the complex path (its registers).
template <int K>
constexpr int cg_threads()
{
    return K == 1 ? 2 * kTile : kTile;
}

template <int K, bool MIXED>
__global__ void __launch_bounds__(cg_threads<K>()) cg_kernel(CGArgs a)
{
    using W = typename std::conditional<MIXED, float, double>::type;
    // the imaginary parts (slots 3 and 5) vanish on the real K = 1 path
    constexpr int kSkipIm = (K == 1) ? ((1 << 3) | (1 << 5)) : 0;
    constexpr int TP = cg_threads<K>() / kTile;   // tiles processed at once
    const int hf = threadIdx.x / kTile, ts = threadIdx.x % kTile;   // tile slot, thread in tile
    __shared__ double red[128];
    __shared__ SysLocal sl[kMaxSysPerBlock];
    __shared__ int nsl;
    __shared__ unsigned char tslot[kMaxTilesPerBlock];   // local system slot of each tile (< kMaxSysPerBlock)
    __shared__ Deps deps;
    __shared__ int s_flag, s_active, s_ru, s_nact, s_anyru;
    __shared__ int s_cnt[2];
    __shared__ int s_esc[4], s_fast;   // fixed-point scales and whether they hold
    __shared__ CGState lst;   // single-system solves: this block's copy of the state
    __shared__ FastShadow fsh;   // and its FP32 copies for the fast step
    const bool solo = (a.sys_count == 1);
    int tb, te;
    block_range(a, &tb, &te);
    setup_block(a, tb, te, sl, &nsl, tslot, &deps);
    if (*(volatile int*)a.err) return;   // the other blocks' waits see the flag and end
    if (solo && threadIdx.x == 0) {
        s_fast = 0;
        lst.rr = lst.rr0 = lst.rr_prev = lst.stop2 = lst.rmax2 = 0.0;
        lst.active = 1;
        lst.iters = lst.converged = lst.status = lst.n_ru = lst.chi_ready = 0;
        lst.mode = kStep;
        fsh.valid = 0;
    }
    __syncthreads();
    const bool first_dag = (a.mtype == YK_NORMAL);   // Normal: A = D D^dag, apply D^dag first
    unsigned epoch = 0, gen = 0;
#ifdef YK_CG_TIMING
    long long tacc[5] = {0, 0, 0, 0, 0}, tlast = clock64();
    int tit = 0;
#endif

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
        for (int base = tb; base < te; base += TP) {   // the same trip count in every thread
            const int tile = base + hf;
            bool on = tile < te;
            const SysLocal& L = sl[tslot[(on ? tile : tb) - tb]];
            on = on && L.mode != kIdle && L.mode != kRu;
            const SysDev& S = a.sys[L.sys];
            const int n = on ? a.tiles[tile].y + ts : 0;
            W v[6] = {W(0), W(0), W(0), W(0), W(0), W(0)};
            if (on && n < S.V) {
                const Site<W, K> ap = apply_d<W, K, MIXED>(Tv(S), n, S, !first_dag);
                YK_ST(W, K, Av(S), n, ap);
                const Site<W, K> r = YK_LD(W, K, Rv(S, cur), n);
                const Site<W, K> p = YK_LD(W, K, Pv(S, cur), n);
                v[0] = site_norm2<W, K>(r);
                v[1] = site_norm2<W, K>(ap);
                site_dot<W, K>(p, ap, v[2], v[3]);
                site_dot<W, K>(r, ap, v[4], v[5]);
            }
            if constexpr (MIXED) {
                FF f[6];
#pragma unroll
                for (int i = 0; i < 6; ++i) f[i] = FF{v[i], 0.f};
                if (K == 1 && solo && s_fast)
                    put_partial_ff<kSkipIm, false>(a, tile, on, f, red, a.bar->fsum[(gen + 1u) % 3u], s_esc);
                else
                    put_partial_ff<kSkipIm, false>(a, tile, on, f, red);
            } else {
                put_partial<W, kSkipIm>(a, tile, on, v, red);
            }
        }
    };

    // ---------------- round 0: b, x = 0, r_0 = p_0 = b; t = D_first p_0; B(0)
    for (int tile = tb + hf; tile < te; tile += TP) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + ts;
        if (n >= S.V) continue;
        const Site<double, K> bv = S.gen_eta ? eta_of_step<K>(S, n, a.eta_kind) : YK_LD(double, K, S.b, n);
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
    for (int tile = tb + hf; tile < te; tile += TP) {
        const SysDev& S = a.sys[a.tiles[tile].x];
        const int n = a.tiles[tile].y + ts;
        if (n >= S.V) continue;
        YK_ST(W, K, Tv(S), n, (apply_d<W, K, MIXED>(Pv(S, 0), n, S, first_dag)));
    }
    if (!nsync(a, ++epoch, deps)) return;
    pass_b(0);
    // the reduction that ends a pass: see solo_reduce and grid_reduce
    auto reduce = [&](int kk, bool ru) -> bool {
        if (solo) return solo_reduce<K, MIXED>(a, gen, kk, ru, red, lst, sl[0], &s_nact, &s_anyru, s_cnt, s_esc, &s_fast, fsh);
        grid_reduce<MIXED>(a, gen, kk, ru, &s_flag, &s_active, &s_ru, red);
        return true;
    };
    if (!reduce(0, false)) return;

    int k = 1;
    while (k <= a.max_iter) {   // every system retires at k = max_iter at the latest
        if (!solo && !poll_coefs(a, sl, nsl, gen, &s_nact, &s_anyru)) return;
        YK_TMARK(0);   // grid reduction + coefficient load
        if (s_nact == 0) break;
        const bool any_ru = MIXED && s_anyru;
        const int cur = k & 1, prv = cur ^ 1;
        // ---------------- A(k)
        for (int tile = tb + hf; tile < te; tile += TP) {
            const SysLocal& L = sl[tslot[tile - tb]];
            const int mode = L.mode;
            if (mode != kStep && mode != kRu && mode != kRedo) continue;
            const SysDev& S = a.sys[L.sys];
            const int n = a.tiles[tile].y + ts;
            if (n >= S.V) continue;
            if constexpr (MIXED) {
                if (mode == kRu) {
                    ru_fold<K>(S, n, L, prv);
                    continue;
                }
            }
            const Nbr nb = neighbours(n, S.Nt, S.Nx);
            const int64_t m5[5] = {n, nb.tu, nb.td, nb.xu, nb.xd};
            const W beta = pick<W>(L.beta, L.f_beta);
            Site<W, K> pn[5];
            if (mode == kStep) {
                const W ar = pick<W>(L.alpha_re, L.f_alpha_re), ai = pick<W>(L.alpha_im, L.f_alpha_im);
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
                const W cre = pick<W>(L.c_re, L.f_c_re), cim = pick<W>(L.c_im, L.f_c_im);
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    const Site<W, K> r = YK_LD(W, K, Rv(S, cur), m5[q]);
                    const Site<W, K> po = YK_LD(W, K, Pv(S, prv), m5[q]);
                    pn[q] = p_next<W, K>(r, po, beta, cre, cim);
                }
            }
            const W diag = diag_of<W, MIXED>(S, n);
            Site<W, K> t = first_dag
                ? dirac_combine<W, K, true>(pn[0], pn[1], pn[2], pn[3], pn[4], diag, (W)S.r, (W)nb.sp, (W)nb.sm)
                : dirac_combine<W, K, false>(pn[0], pn[1], pn[2], pn[3], pn[4], diag, (W)S.r, (W)nb.sp, (W)nb.sm);
            pion_term<W, K>(t, pn[0], S.pi, n, S.V, S.g, first_dag);
            YK_ST(W, K, Tv(S), n, t);
            YK_ST(W, K, Pv(S, cur), n, pn[0]);
        }
        YK_TMARK(1);   // pass A
        if (!nsync(a, ++epoch, deps)) return;
        YK_TMARK(2);   // neighbour sync

        if constexpr (MIXED) {
            if (any_ru) {
                if (!ru_residual<K>(a, sl, tslot, tb, te, first_dag, cur, prv, epoch, deps, red)) return;
                if (!reduce(k, true)) return;
                continue;   // same k: the systems that updated redo A(k)
            }
        }

        // ---------------- B(k)
        pass_b(cur);
        YK_TMARK(3);   // pass B
        if (!reduce(k, false)) return;
        ++k;
#ifdef YK_CG_TIMING
        ++tit;
#endif
    }
#ifdef YK_CG_TIMING
    if (blockIdx.x == 0 && threadIdx.x == 0 && tit > 0)
    {
        printf("cg timing (block 0, cycles per iteration over %d): reduce+coef %lld  A %lld  nsync %lld  B %lld\n", tit,
               tacc[0] / tit, tacc[1] / tit, tacc[2] / tit, tacc[3] / tit);
        volatile unsigned long long* t = g_cg_t;
        printf("cg timing (all blocks, cycles per event): arrive %llu  finish %llu  arrival spread %llu ns\n",
               t[0] / (t[1] ? t[1] : 1), t[2] / (t[3] ? t[3] : 1), t[8] / (t[3] ? t[3] : 1));
        volatile unsigned long long* f = g_cg_f;
        printf("cg timing (finisher, cycles per event): sums %llu (loads %llu)  scalar %llu  tail %llu\n",
               f[0] / (f[3] ? f[3] : 1), f[4] / (f[3] ? f[3] : 1), f[1] / (f[3] ? f[3] : 1), f[2] / (f[3] ? f[3] : 1));
        for (int i = 0; i < 10; ++i) t[i] = 0;
        for (int i = 0; i < 8; ++i) f[i] = 0;
    }
#endif
}

// ---------------------------------------------------------------------------
// Halo variant of the mixed single-system CG on the real path (K = 1).
//
// Each block owns the contiguous site range [n0, n1) of its tiles.  Every
// iteration it forms p_k itself on that range widened by two time slices on
// each side (2 Nx sites), from r, A p and p of the previous iteration, which
// the grid barrier of that iteration has completed; applies D_first on the
// range widened by one slice; and applies D_second on its own sites -- both
// stencils in shared memory.  An iteration is then one round of bulk copies
// into shared memory, two shared-memory stencils and the reducing grid
// barrier: no neighbour synchronisation and no round trip of D p through L2.
// The price is the redundant work on the four halo slices, so the launcher
// takes this kernel only while 4 Nx <= 2 (n1 - n0) (and the widened range fits
// the lattice and shared memory).
//
// The widened range of r, A p and p (and x on the own sites) is staged into
// shared memory with asynchronous copies (cp.async, each thread the sites it
// forms in A1), issued as soon as the barrier of the previous iteration has
// been passed -- before that iteration's scalar step, on the guess that the
// next iteration is an ordinary step -- so the copies travel while warp 0
// loads the sums and steps the recurrence, and hold no registers meanwhile.
// A1 then forms p (and r) in place in the staging buffers.
//
// Per site the arithmetic is that of cg_kernel<1, true> (the same formation
// of r and p, the same stencil calls, the same tile partials and fixed-point
// sums), so the two kernels produce the same iterates.  A p is double-buffered
// here (S.Ap32 for even k, S.t32 for odd k), because a block may store A p_k
// while a neighbour still reads A p_{k-1} on its halo.  Round 0 and the
// reliable updates run as in cg_kernel, with neighbour synchronisation.
// ---------------------------------------------------------------------------
constexpr int kHaloThreads = 2 * kTile;

__device__ __forceinline__ int wrap_site(int m, int V) { return m < 0 ? m + V : (m >= V ? m - V : m); }

__device__ __forceinline__ Site<float, 1> ld_sm(const float4* s, int j)
{
    const float4 a = s[j];
    Site<float, 1> o;
    o.v[0] = a.x;
    o.v[1] = a.y;
    o.v[2] = a.z;
    o.v[3] = a.w;
    return o;
}

__device__ __forceinline__ void st_sm(float4* s, int j, const Site<float, 1>& v)
{
    s[j] = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}

// Shared-memory address and the per-thread asynchronous copy (cp.async, 16
// bytes, L2 only: the barrier's acquire is what makes other blocks' writes
// visible, and no line of them may come from this SM's L1).
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// D (DAG = false) or D^dag (DAG = true) at site m from a shared-memory copy
// `in` of a contiguous site range holding m at index j and both of m's time
// slices; diag at m given.  sh = log2 Nx when Nx is a power of two, else -1.
template <bool DAG>
__device__ __forceinline__ Site<float, 1> apply_d_sm(const float4* in, int j, int m, int Nt, int Nx, int sh, float diag,
                                                     float r)
{
    const int t = sh >= 0 ? (m >> sh) : m / Nx;
    const int x = m - t * Nx;
    const int ju = j + ((x + 1 == Nx) ? 1 - Nx : 1);   // the hops of neighbours(), as offsets
    const int jd = j + ((x == 0) ? Nx - 1 : -1);
    const float sp = (t + 1 == Nt) ? -1.f : 1.f, sm = (t == 0) ? -1.f : 1.f;
    const Site<float, 1> c = ld_sm(in, j);
    const Site<float, 1> tu = ld_sm(in, j + Nx);
    const Site<float, 1> td = ld_sm(in, j - Nx);
    const Site<float, 1> xu = ld_sm(in, ju);
    const Site<float, 1> xd = ld_sm(in, jd);
    return dirac_combine<float, 1, DAG>(c, tu, td, xu, xd, diag, r, sp, sm);
}

enum { kHaloInit = 0 };   // A1 of round 0: p_0 = b as stored

__global__ void __launch_bounds__(kHaloThreads) cg_halo_kernel(CGArgs a)
{
    constexpr int K = 1;
    constexpr int kSkipIm = (1 << 3) | (1 << 5);
    using W = float;
    extern __shared__ float4 hsm[];
    const int hf = threadIdx.x / kTile, ts = threadIdx.x % kTile;
    __shared__ double red[128];
    __shared__ SysLocal sl[kMaxSysPerBlock];
    __shared__ int nsl;
    __shared__ unsigned char tslot[kMaxTilesPerBlock];   // local system slot of each tile (< kMaxSysPerBlock)
    __shared__ Deps deps;
    __shared__ int s_nact, s_anyru;
    __shared__ int s_cnt[2];
    __shared__ int s_esc[4], s_fast;
    __shared__ CGState lst;
    __shared__ FastShadow fsh;
    // the system record in shared memory: the grid barrier's acquire leaves L1
    // cold, and the vector addresses would otherwise cost a round trip to L2
    // before every pass
    __shared__ SysDev S;
    // and the arguments, for the reduction
    __shared__ CGArgs sa;
    const int tb = a.tile_begin + blockIdx.x * a.tiles_per_block;
    const int te = min(tb + a.tiles_per_block, a.tile_end);
    setup_block(a, tb, te, sl, &nsl, tslot, &deps);
    if (*(volatile int*)a.err) return;
    if (threadIdx.x == 0) {
        s_fast = 0;
        lst.rr = lst.rr0 = lst.rr_prev = lst.stop2 = lst.rmax2 = 0.0;
        lst.active = 1;
        lst.iters = lst.converged = lst.status = lst.n_ru = lst.chi_ready = 0;
        lst.mode = kStep;
        fsh.valid = 0;
        S = a.sys[a.sys_first];
        sa = a;
    }
    __syncthreads();
    const int Nt = S.Nt, Nx = S.Nx, V = S.V;
    const int sh = (Nx & (Nx - 1)) == 0 ? __ffs(Nx) - 1 : -1;
    const int n0 = a.tiles[tb].y;
    const int n1 = min(a.tiles[te - 1].y + kTile, V);
    const int own = n1 - n0;
    const int nP = own + 4 * Nx, nT = own + 2 * Nx;
    const int pfirst = wrap_site(n0 - 2 * Nx, V);        // first site of the widened range
    float4* P_st = hsm;                                  // p on [n0 - 2 Nx, n1 + 2 Nx): staged p_{k-1}, then p_k
    float4* R_st = P_st + nP;                            // r there: staged r_{k-1}, then r_k on the own sites
    float4* A_st = R_st + nP;                            // A p_{k-1} there
    float4* X_st = A_st + nP;                            // x increment on [n0, n1), kept here all solve
    float4* t_s = X_st + own;                            // D_first p_k on [n0 - Nx, n1 + Nx)
    float* d_s = reinterpret_cast<float*>(t_s + nT);     // diag on [n0 - Nx, n1 + Nx)
    const bool first_dag = (a.mtype == YK_NORMAL);       // Normal: A = D D^dag, apply D^dag first
    const float rw = (float)S.r;
    for (int j = threadIdx.x; j < nT; j += kHaloThreads) {
        const int m = wrap_site(n0 - Nx + j, V);
        d_s[j] = (float)(2.0 * S.r + S.m0 + S.g * S.sigma[m]);
    }
    unsigned epoch = 0, gen = 0;
    int staged_k = -1;   // the iteration whose ordinary-step staging is in flight
#ifdef YK_CG_TIMING
    long long tacc[5] = {0, 0, 0, 0, 0}, tlast = clock64();
    int tit = 0;
#endif

    // Stages the inputs of A1 for `mode`, each thread the sites it forms in
    // A1: kStep: r, A p, p of iteration prv; kRedo: r of cur and p of prv;
    // round 0: r and p as stored.
    auto stage = [&](int mode, int cur, int prv) {
        const float* Rl = (mode == kRedo) ? S.r32[cur] : S.r32[prv];
        const float* Pl = S.p32[prv];
        const float* Al = prv == 0 ? S.Ap32 : S.t32;
        for (int j = threadIdx.x; j < nP; j += kHaloThreads) {
            const int m = wrap_site(pfirst + j, V);
            cp_async16(P_st + j, Pl + 4 * (size_t)m);
            cp_async16(R_st + j, Rl + 4 * (size_t)m);
            if (mode == kStep) cp_async16(A_st + j, Al + 4 * (size_t)m);
        }
        cp_async_commit();
    };
    // this thread's staging copies have landed (A1 reads only its own sites)
    auto stage_wait = [&]() -> bool {
        cp_async_wait_all();
        return true;
    };

    // A1: p_k (and r_k, x_k on the own sites) on the widened range, in place
    auto pass_a1 = [&](int mode, int cur, int prv) {
        const SysLocal& L = sl[0];
        const W ar = L.f_alpha_re, beta = L.f_beta, cre = L.f_c_re, cim = L.f_c_im;
        for (int j = threadIdx.x; j < nP; j += kHaloThreads) {
            const int o = j - 2 * Nx;
            const bool is_own = o >= 0 && o < own;
            const int m = n0 + o;   // an own site when is_own
            const Site<W, K> po = ld_sm(P_st, j);
            Site<W, K> p;
            if (mode == kStep) {
                Site<W, K> r = ld_sm(R_st, j);
                site_axpy<W, K>(r, -ar, W(0), ld_sm(A_st, j));
#pragma unroll
                for (int i = 0; i < 4; ++i) p.v[i] = fma(beta, po.v[i], r.v[i]);
                if (is_own) {
                    Site<W, K> x = ld_sm(X_st, o);
                    site_axpy<W, K>(x, ar, W(0), po);
                    st_sm(X_st, o, x);
                    YK_ST(W, K, S.r32[cur], m, r);
                    YK_ST(W, K, S.p32[cur], m, p);
                    st_sm(R_st, j, r);
                }
            } else if (mode == kRedo) {
                p = p_next<W, K>(ld_sm(R_st, j), po, beta, cre, cim);
                if (is_own) YK_ST(W, K, S.p32[cur], m, p);
            } else {
                p = po;   // round 0: r_0 = p_0 = b, both staged
            }
            st_sm(P_st, j, p);
        }
    };

    // A2: t = D_first p_k on [n0 - Nx, n1 + Nx)
    auto pass_a2 = [&]() {
        for (int j = threadIdx.x; j < nT; j += kHaloThreads) {
            const int m = wrap_site(n0 - Nx + j, V);
            const Site<W, K> t = first_dag ? apply_d_sm<true>(P_st, j + Nx, m, Nt, Nx, sh, d_s[j], rw)
                                           : apply_d_sm<false>(P_st, j + Nx, m, Nt, Nx, sh, d_s[j], rw);
            st_sm(t_s, j, t);
        }
    };

    // B(k): A p_k = D_second t on the own sites -> Ap[cur]; the tile partials
    auto pass_b = [&](int cur) {
        float* Ac = cur == 0 ? S.Ap32 : S.t32;
        for (int base = tb; base < te; base += 2) {   // the same trip count in every thread
            const int tile = base + hf;
            const bool tile_on = tile < te;   // the tile writes its partial (every value thread)
            const int n = tile_on ? n0 + (tile - tb) * kTile + ts : V;   // the tiles are contiguous
            const bool on = n < V;
            W v[6] = {W(0), W(0), W(0), W(0), W(0), W(0)};
            if (on) {
                const int o = n - n0, jt = o + Nx;
                const Site<W, K> ap = first_dag ? apply_d_sm<false>(t_s, jt, n, Nt, Nx, sh, d_s[jt], rw)
                                                : apply_d_sm<true>(t_s, jt, n, Nt, Nx, sh, d_s[jt], rw);
                YK_ST(W, K, Ac, n, ap);
                const Site<W, K> r = ld_sm(R_st, o + 2 * Nx);
                const Site<W, K> p = ld_sm(P_st, o + 2 * Nx);
                v[0] = site_norm2<W, K>(r);
                v[1] = site_norm2<W, K>(ap);
                site_dot<W, K>(p, ap, v[2], v[3]);
                site_dot<W, K>(r, ap, v[4], v[5]);
            }
            FF f[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) f[i] = FF{v[i], 0.f};
            if (s_fast)
                put_partial_ff<kSkipIm, false>(a, tile, tile_on, f, red, a.bar->fsum[(gen + 1u) % 3u], s_esc);
            else
                put_partial_ff<kSkipIm, false>(a, tile, tile_on, f, red);
        }
    };

    auto reduce = [&](int kk, bool ru) -> bool {
        // once the barrier of an ordinary iteration is passed, stage the next
        // one on the guess that it is an ordinary step too
        auto prefetch = [&]() {
            if (ru) return;
            const int k1 = kk + 1;
            stage(kStep, k1 & 1, (k1 & 1) ^ 1);
            staged_k = k1;
        };
        return solo_reduce_body<K, true>(sa, gen, kk, ru, red, lst, sl[0], &s_nact, &s_anyru, s_cnt, s_esc, &s_fast, fsh,
                                         prefetch);
    };

    // ---------------- round 0: b, x = 0, r_0 = p_0 = b; t = D_first p_0; B(0)
    for (int tile = tb + hf; tile < te; tile += 2) {
        const int n = a.tiles[tile].y + ts;
        if (n >= V) continue;
        const Site<double, K> bv = S.gen_eta ? eta_of_step<K>(S, n, a.eta_kind) : YK_LD(double, K, S.b, n);
        if (S.gen_eta) YK_ST(double, K, S.b, n, bv);
        Site<double, K> z;
        Site<W, K> bw, zw;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            z.v[i] = 0.0;
            zw.v[i] = W(0);
            bw.v[i] = (W)bv.v[i];
        }
        YK_ST(double, K, S.x, n, z);
        st_sm(X_st, n - n0, zw);
        YK_ST(W, K, S.r32[0], n, bw);
        YK_ST(W, K, S.p32[0], n, bw);
    }
    if (!nsync(a, ++epoch, deps)) return;
    stage(kHaloInit, 0, 0);
    if (!stage_wait()) return;
    pass_a1(kHaloInit, 0, 0);
    __syncthreads();
    pass_a2();
    __syncthreads();
    pass_b(0);
    if (!reduce(0, false)) return;

    int k = 1;
    while (k <= a.max_iter) {   // the system retires at k = max_iter at the latest
        YK_TMARK(0);   // grid reduction
        const int mode = sl[0].mode;
        if (s_nact == 0 || mode == kRu) {
            // the guessed staging is not used: let it land before going on
            if (staged_k == k && !stage_wait()) return;
            staged_k = -1;
        }
        if (s_nact == 0) break;
        const int cur = k & 1, prv = cur ^ 1;
        if (mode == kRu) {
            // fold x_k = x + xs + alpha p_{k-1} into the FP64 x; xs = 0 (as ru_fold,
            // with the increment from shared memory)
            const SysLocal& L = sl[0];
            for (int o = threadIdx.x; o < own; o += kHaloThreads) {
                const int n = n0 + o;
                Site<double, K> xv = YK_LD(double, K, S.x, n);
                const Site<W, K> xs = ld_sm(X_st, o);
                const Site<W, K> pv = YK_LD(W, K, S.p32[prv], n);
                Site<double, K> pd;
                Site<W, K> zw;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    xv.v[i] += (double)xs.v[i];
                    pd.v[i] = (double)pv.v[i];
                    zw.v[i] = W(0);
                }
                site_axpy<double, K>(xv, L.alpha_re, L.alpha_im, pd);
                YK_ST(double, K, S.x, n, xv);
                st_sm(X_st, o, zw);
            }
            if (!nsync(a, ++epoch, deps)) return;
            if (!ru_residual<K>(a, sl, tslot, tb, te, first_dag, cur, prv, epoch, deps, red)) return;
            if (!reduce(k, true)) return;
            continue;   // same k: redo A(k) from the FP64 residual
        }
        if (!(mode == kStep && staged_k == k)) {
            if (staged_k == k && !stage_wait()) return;   // a guess for another mode
            stage(mode, cur, prv);
        }
        staged_k = -1;
        if (!stage_wait()) return;
        pass_a1(mode, cur, prv);
        __syncthreads();
        YK_TMARK(1);
        pass_a2();
        __syncthreads();
        YK_TMARK(2);
        pass_b(cur);
        YK_TMARK(3);
        if (!reduce(k, false)) return;
        ++k;
#ifdef YK_CG_TIMING
        ++tit;
#endif
    }
#ifdef YK_CG_TIMING
    if (blockIdx.x == 0 && threadIdx.x == 0 && tit > 0) {
        printf("cg timing (block 0, cycles per iteration over %d): reduce+coef %lld  A1 %lld  A2 %lld  B %lld\n", tit,
               tacc[0] / tit, tacc[1] / tit, tacc[2] / tit, tacc[3] / tit);
        volatile unsigned long long* f = g_cg_f;
        printf("cg timing (finisher, cycles per event): sums %llu (loads %llu)  scalar %llu  tail %llu\n",
               f[0] / (f[3] ? f[3] : 1), f[4] / (f[3] ? f[3] : 1), f[1] / (f[3] ? f[3] : 1), f[2] / (f[3] ? f[3] : 1));
        volatile unsigned long long* q = g_cg_q;
        const unsigned long long nq = f[3] ? f[3] : 1;
        printf("cg timing (reduction marks): entry-sync %llu  fence+arrive %llu  wait %llu  fence+sync %llu  "
               "loads %llu  step %llu  bcast %llu  end-sync %llu\n",
               q[0] / nq, q[1] / nq, q[2] / nq, q[3] / nq, q[4] / nq, q[5] / nq, q[6] / nq, q[7] / nq);
        printf("cg timing (fast step marks): convert %llu  alpha %llu  estimate %llu  triggers %llu  state %llu\n",
               q[8] / nq, q[9] / nq, q[10] / nq, q[11] / nq, q[12] / nq);
        for (int i = 0; i < 8; ++i) f[i] = 0;
        for (int i = 0; i < 16; ++i) q[i] = 0;
    }
#endif
}

// Shared memory of cg_halo_kernel for own sites per block and Nx: the staged
// widened range (p, r, A p), the own x increment, D_first p and diag.
static size_t halo_smem_bytes(int own, int Nx)
{
    const size_t nP = (size_t)own + 4 * (size_t)Nx, nT = (size_t)own + 2 * (size_t)Nx;
    return (3 * nP + (size_t)own + nT) * sizeof(float4) + nT * sizeof(float);
}

// ---------------------------------------------------------------------------
// Even-odd mixed CG of the step's single-system solves (cg_eo_kernel).
//
// The force needs chi = (D^dag)^-1 eta, which the reference forms as D x from
// CG on D^dag D (FermionicDrift.cu:57-80, CGsolver.cu:72-170).  D = A + H with
// A = 2r + m0 + g sigma per site and H the hops, which join sites of opposite
// parity (t + x) when Nt and Nx are even.  On the even sites D^dag chi = eta is
// the Schur system
//   S chi_e = rhs_e,   S = A_e - H^dag_eo A_o^-1 H^dag_oe,
//   rhs_e = eta_e - H^dag_eo A_o^-1 eta_o,  chi_o = A_o^-1 (eta_o - H^dag_oe chi_e),
// solved by CG on S S^dag with chi_e = S^dag y (CGNE), chi_e kept directly:
// every iteration forms v = S^dag p and q = S v (four half-lattice hops, the
// stencil work of one D^dag D over half the unknowns), alpha = |r|^2 / |v|^2,
// chi_e += alpha v, r -= alpha q.  Its residual rhs_e - S chi_e is the true
// residual of D^dag chi = eta (the odd sites' is zero by construction), the
// quantity CG on D^dag D controls (there r = eta - D^dag (D x)), so the stop is
// the same rule relative to |eta|; it takes about 2.3 times fewer iterations.
//
// Compact lattices: site (t, x) of parity q is t Nh + x / 2 of its class
// (Nh = Nx / 2), full site 2 m + ((t + q) & 1).  a.sys are the systems'
// compact views (Nx = Nh, V = V / 2, tiles over compact sites; the FP32
// vectors compact; x = chi_e (compact) followed by rhs_e; t64 the odd hops
// of the reliable updates and, at the end, chi in the full layout for the
// force, CGState::chi_ready); a.sys_full the full records (eta in b, sigma).
// Both even-odd kernels keep chi_e, rhs_e, the odd hops and dinv in
// float-float (SiteFF).
// A block owns the compact range [c0, c1), stages p, r, q of the previous
// iteration on [c0 - 4Nh, c1 + 4Nh) and forms, in shared memory,
//   w = -A_o^-1 H_oe p      on [c0 - 3Nh, c1 + 3Nh)   (odd)
//   v = A_e p + H_eo w      on [c0 - 2Nh, c1 + 2Nh)   (even; = S^dag p)
//   u = -A_o^-1 H^dag_oe v  on [c0 - Nh,  c1 + Nh)    (odd)
//   q = A_e v + H^dag_eo u  on [c0, c1)               (even; = S v)
// with the one reducing grid barrier per iteration and the scalar steps of
// cg_halo_kernel (its tile partials: |r|^2, |q|^2, |v|^2 in the <p, Ap> slot,
// <r, q>); its reliable updates in float-float on the FP32 pipes.
// cg_eo_kernel<true> owns 16 x 16 patches of the compact lattice instead of
// whole rows: the widened patch (24 x 20 cells) holds 480 sites against
// 1280 for two rows of 128 widened by four rows on each side, and the w, v,
// u passes compute 1200 sites against 2304 (one partial slot per patch).

// Row, x-parity bit and the compact offsets of the x neighbours (opposite
// class) of compact site m of parity q.
__device__ __forceinline__ void eo_geom(int m, int q, int Nh, int sh, int& t, int& b, int& dxu, int& dxd)
{
    t = sh >= 0 ? (m >> sh) : m / Nh;
    const int i = m - t * Nh;
    b = (t + q) & 1;   // x = 2 i + b
    dxu = b ? ((i == Nh - 1) ? 1 - Nh : 1) : 0;
    dxd = b ? 0 : ((i == 0) ? Nh - 1 : -1);
}

// diag c + H (neighbours in `in` at j +- Nh, j + dxu, j + dxd) in FP32 (DAG:
// the hops of D^dag)
template <bool DAG>
__device__ __forceinline__ Site<float, 1> eo_sm(const float4* in, int j, int Nh, int dxu, int dxd,
                                                const Site<float, 1>& c, float diag, float r, float sp, float sm)
{
    return dirac_combine<float, 1, DAG>(c, ld_sm(in, j + Nh), ld_sm(in, j - Nh), ld_sm(in, j + dxu), ld_sm(in, j + dxd),
                                        diag, r, sp, sm);
}

// The even-odd kernels' reliable updates, round 0 and reconstruction in
// float-float (about 48 significant bits, on the FP32 pipes: GB300 issues
// FP64 at 1/64 of the FP32 rate and these passes were bound by it).  chi_e,
// rhs_e and the odd intermediate keep the FP64 vectors' 32 bytes a compact
// site: four hi words, then four lo words; 1 / A_o keeps its 8 bytes as (hi,
// lo).  Only the kernels read them; chi goes out to the force in FP64.
struct SiteFF {
    FF v[4];
};

__device__ __forceinline__ SiteFF ld_ff(const double* base, int m)
{
    const float4* p = reinterpret_cast<const float4*>(base) + 2 * (size_t)m;
    const float4 h = p[0], l = p[1];
    return SiteFF{{FF{h.x, l.x}, FF{h.y, l.y}, FF{h.z, l.z}, FF{h.w, l.w}}};
}

__device__ __forceinline__ void st_ff(double* base, int m, const SiteFF& s)
{
    float4* p = reinterpret_cast<float4*>(base) + 2 * (size_t)m;
    p[0] = make_float4(s.v[0].hi, s.v[1].hi, s.v[2].hi, s.v[3].hi);
    p[1] = make_float4(s.v[0].lo, s.v[1].lo, s.v[2].lo, s.v[3].lo);
}

__device__ __forceinline__ FF ld_ff1(const double* base, int m)
{
    const float2 v = reinterpret_cast<const float2*>(base)[m];
    return FF{v.x, v.y};
}

__device__ __forceinline__ void st_ff1(double* base, int m, FF v)
{
    reinterpret_cast<float2*>(base)[m] = make_float2(v.hi, v.lo);
}

// a source vector's site as float-float: the Langevin sources are FP32 normals
// (exact in FP32) when generated; other right-hand sides are split
__device__ __forceinline__ SiteFF ff_site_of(const Site<double, 1>& e, bool exact32)
{
    SiteFF s;
#pragma unroll
    for (int i = 0; i < 4; ++i) s.v[i] = exact32 ? FF{(float)e.v[i], 0.f} : ff_of(e.v[i]);
    return s;
}

// dirac_combine's hop coefficients in float-float: P = -(r + 1) / 2,
// M = -(r - 1) / 2, A = -r / 2 (the time hops take +-P and +-M by the
// antiperiodic signs, the space hops A and +-1/2)
struct HopFF {
    FF P, M, A;
};

__device__ __forceinline__ HopFF hop_ff(double r)
{
    return HopFF{ff_of(-0.5 * (r + 1.0)), ff_of(-0.5 * (r - 1.0)), ff_of(-0.5 * r)};
}

// the same from r split once (the per-site form: four FP64 operations)
__device__ __forceinline__ HopFF hop_of_r(double r)
{
    const FF rr = ff_of(r);
    const FF rp = ff_add(rr, FF{1.f, 0.f}), rm = ff_add(rr, FF{-1.f, 0.f});
    return HopFF{FF{-0.5f * rp.hi, -0.5f * rp.lo}, FF{-0.5f * rm.hi, -0.5f * rm.lo}, FF{-0.5f * rr.hi, -0.5f * rr.lo}};
}

__device__ __forceinline__ FF ff_sign(FF a, float s) { return FF{s * a.hi, s * a.lo}; }

// dirac_combine<float-float, K = 1, DAG> with the same order of terms:
// MODE 0: H alone; 1: c + H; 2: diag c + H
template <bool DAG, int MODE>
__device__ __forceinline__ SiteFF combine_ff(const SiteFF& c, FF diag, const SiteFF& tu, const SiteFF& td,
                                             const SiteFF& xu, const SiteFF& xd, const HopFF& h, float sp, float sm)
{
    const FF cu_up = ff_sign(DAG ? h.P : h.M, sp), cd_up = ff_sign(DAG ? h.M : h.P, sp);
    const FF cu_dn = ff_sign(DAG ? h.M : h.P, sm), cd_dn = ff_sign(DAG ? h.P : h.M, sm);
    const float bx = DAG ? -0.5f : 0.5f;
    SiteFF o;
#pragma unroll
    for (int f = 0; f < 2; ++f) {
        const int iu = 2 * f, id = 2 * f + 1;
        FF ou, od;
        if (MODE == 0) {
            ou = ff_mul(cu_up, tu.v[iu]);
            od = ff_mul(cd_up, tu.v[id]);
        } else {
            ou = MODE == 1 ? c.v[iu] : ff_mul(diag, c.v[iu]);
            od = MODE == 1 ? c.v[id] : ff_mul(diag, c.v[id]);
            ou = ff_add(ou, ff_mul(cu_up, tu.v[iu]));
            od = ff_add(od, ff_mul(cd_up, tu.v[id]));
        }
        ou = ff_add(ou, ff_mul(cu_dn, td.v[iu]));
        od = ff_add(od, ff_mul(cd_dn, td.v[id]));
        const FF dfu = ff_sub(xu.v[id], xd.v[id]), dfd = ff_sub(xu.v[iu], xd.v[iu]);
        ou = ff_add(ou, FF{bx * dfu.hi, bx * dfu.lo});
        od = ff_add(od, FF{bx * dfd.hi, bx * dfd.lo});
        ou = ff_add(ou, ff_mul(h.A, ff_add(xu.v[iu], xd.v[iu])));
        od = ff_add(od, ff_mul(h.A, ff_add(xu.v[id], xd.v[id])));
        o.v[iu] = ou;
        o.v[id] = od;
    }
    return o;
}

// the odd/even half hop of compact m from a float-float vector (its four
// neighbours at m +- Nh, m + dxu, m + dxd)
template <bool DAG, int MODE>
__device__ __forceinline__ SiteFF eo_ff(const double* in, int m, int Ve, int Nh, int dxu, int dxd, const SiteFF& c,
                                        FF diag, const HopFF& h, float sp, float sm)
{
    const int mu = m + Nh >= Ve ? m + Nh - Ve : m + Nh, md = m - Nh < 0 ? m - Nh + Ve : m - Nh;
    return combine_ff<DAG, MODE>(c, diag, ld_ff(in, mu), ld_ff(in, md), ld_ff(in, m + dxu), ld_ff(in, m + dxd), h, sp,
                                 sm);
}

// Patch geometry of cg_eo_kernel<PX> (PX > 0): each block owns eo_pt(PX) rows x PX
// compact columns and stages them widened by 4 rows and 2 compact columns
// (the reach of the four half hops: two compact columns, since consecutive x
// hops alternate between the compact index's two parities).  Cells at the
// buffer's column edges get values no own q depends on; their x neighbours
// stay inside the buffer (the rows of w, v, u exclude the first and last).
// PX = 16: 512-thread blocks, one per SM; PX = 8: 256-thread blocks, two per
// SM, so that one block's barrier waits overlap the other's passes; PX = 32:
// 32 x 32 patches on 512-thread blocks (156 KB of shared memory), so that a
// 512 x 512 lattice's 128 patches are co-resident (its 16 x 16 patches are
// 512).  PX = 0:
// whole rows (cg_eo_kernel's first form).
__host__ __device__ constexpr int eo_pt(int PX) { return PX == 32 ? 32 : 16; }   // patch rows
__host__ __device__ constexpr int eo_sr(int PX) { return eo_pt(PX) + 8; }        // staged rows
__host__ __device__ constexpr int eo_threads(int PX) { return PX == 8 ? 256 : kHaloThreads; }
__host__ __device__ constexpr int eo_sw(int PX) { return (PX > 0 ? PX : 16) + 4; }

template <int PX>
__global__ void __launch_bounds__(eo_threads(PX), PX == 8 ? 2 : 1) cg_eo_kernel(CGArgs a)
{
    constexpr bool PATCH = PX > 0;
    constexpr int kPX = PATCH ? PX : 16;
    constexpr int kPT = eo_pt(PX), kSR = eo_sr(PX);
    constexpr int kSW = eo_sw(PX), kSN = kSW * kSR;
    constexpr int NT = eo_threads(PX);
    constexpr int K = 1;
    constexpr int kSkipIm = (1 << 3) | (1 << 5);
    using W = float;
    extern __shared__ float4 hsm[];
    const int hf = threadIdx.x / kTile, ts = threadIdx.x % kTile;
    __shared__ double red[128];
    __shared__ SysLocal sl[kMaxSysPerBlock];
    __shared__ int nsl;
    __shared__ unsigned char tslot[kMaxTilesPerBlock];
    __shared__ Deps deps;
    __shared__ int s_nact, s_anyru;
    __shared__ int s_cnt[2];
    __shared__ int s_esc[4], s_fast;
    __shared__ CGState lst;
    __shared__ FastShadow fsh;
    __shared__ SysDev S;    // the compact view
    __shared__ SysDev SF;   // the full record
    __shared__ CGArgs sa;
    __shared__ HopFF s_hop;   // the hop coefficients in float-float (one thread's FP64 work)
    const int tb = a.tile_begin + blockIdx.x * a.tiles_per_block;
    const int te = min(tb + a.tiles_per_block, a.tile_end);
    setup_block(a, tb, te, sl, &nsl, tslot, &deps);
    if (*(volatile int*)a.err) return;
    if constexpr (PATCH) {
        // the eight patches around this one replace the row ranges' neighbours:
        // the widened patch staged after round 0's last neighbour sync reaches
        // into the diagonal ones too
        if (threadIdx.x == 0) {
            const SysDev& V0 = a.sys[a.sys_first];
            const int npx = V0.Nx / kPX, npt = V0.Nt / kPT;
            const int pt = blockIdx.x / npx, px = blockIdx.x % npx;
            int n = 0;
            for (int dt = -1; dt <= 1; ++dt)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int nb = ((pt + dt + npt) % npt) * npx + (px + dx + npx) % npx;
                    bool seen = nb == (int)blockIdx.x;
                    for (int j = 0; j < n && !seen; ++j) seen = deps.b[j] == nb;
                    if (!seen) deps.b[n++] = nb;
                }
            deps.n = n;
            deps.all = 0;
        }
    }
    if (threadIdx.x == 0) {
        s_fast = 0;
        lst.rr = lst.rr0 = lst.rr_prev = lst.stop2 = lst.rmax2 = 0.0;
        lst.active = 1;
        lst.iters = lst.converged = lst.status = lst.n_ru = lst.chi_ready = 0;
        lst.mode = kStep;
        fsh.valid = 0;
        S = a.sys[a.sys_first];
        SF = a.sys_full[a.sys_first];
        sa = a;
        s_hop = hop_ff(a.sys[a.sys_first].r);
    }
    __syncthreads();
    const int Nt = S.Nt, Nh = S.Nx, Ve = S.V;
    const int sh = (Nh & (Nh - 1)) == 0 ? __ffs(Nh) - 1 : -1;
    // The staged buffer: rows (PATCH: the kPT x kPX patch at (t0, i0) widened
    // by 4 rows and 2 compact columns, row stride kSW, wrapped while staging;
    // else the compact range [c0, c0 + own) widened by 4 rows, stride Nh).
    // Stencils in the buffer step by +-SB in t and by the x offsets of cell().
    int c0 = 0, own, t0 = 0, i0 = 0, SB, NB, cbase = 0;
    if constexpr (PATCH) {
        const int npx = Nh / kPX;
        t0 = (blockIdx.x / npx) * kPT;
        i0 = (blockIdx.x % npx) * kPX;
        own = kPT * kPX;
        SB = kSW;
        NB = kSN;
    } else {
        c0 = a.tiles[tb].y;
        own = min(a.tiles[te - 1].y + kTile, Ve) - c0;
        SB = Nh;
        NB = own + 8 * Nh;
        cbase = c0 - 4 * Nh;                       // compact site of buffer index 0
    }
    const int pfirst = PATCH ? 0 : wrap_site(cbase, Ve);
    // compact site of buffer cell j
    auto buf_m = [&](int j) -> int {
        if constexpr (PATCH) {
            const int r = j / kSW, c = j - r * kSW;
            int t = t0 - 4 + r, i = i0 - 2 + c;
            t = t < 0 ? t + Nt : (t >= Nt ? t - Nt : t);
            i = i < 0 ? i + Nh : (i >= Nh ? i - Nh : i);
            return t * Nh + i;
        } else {
            return wrap_site(pfirst + j, Ve);
        }
    };
    // row, x parity bit and buffer x offsets of cell j's site of class q
    auto cell = [&](int j, int q, int& t, int& b, int& du, int& dd) {
        if constexpr (PATCH) {
            const int r = j / kSW;
            t = t0 - 4 + r;
            t = t < 0 ? t + Nt : (t >= Nt ? t - Nt : t);
            b = (t + q) & 1;
            du = b;
            dd = b - 1;
        } else {
            eo_geom(wrap_site(pfirst + j, Ve), q, Nh, sh, t, b, du, dd);
        }
    };
    auto own_j = [&](int o) -> int { return PATCH ? (4 + o / kPX) * kSW + 2 + o % kPX : 4 * Nh + o; };
    auto own_m = [&](int o) -> int { return PATCH ? (t0 + o / kPX) * Nh + i0 + o % kPX : c0 + o; };
    // own index of buffer cell j, or -1
    auto own_of = [&](int j) -> int {
        if constexpr (PATCH) {
            const int r = j / kSW - 4, c = j % kSW - 2;
            return (r >= 0 && r < kPT && c >= 0 && c < kPX) ? r * kPX + c : -1;
        } else {
            const int o = j - 4 * Nh;
            return (o >= 0 && o < own) ? o : -1;
        }
    };
    float4* P_st = hsm;                            // p on [0, NB)
    float4* R_st = P_st + NB;                      // r there
    float4* A_st = R_st + NB;                      // q there
    float4* X_st = A_st + NB;                      // chi_e increment on the own sites
    float4* V_own = X_st + own;                    // v of the previous iteration on the own sites
    float4* Wp = V_own + own;                      // w on [SB, NB - SB), later u on [3SB, NB - 3SB)
    float4* Vp = Wp + NB;                          // v on [2SB, NB - 2SB)
    float* dep = reinterpret_cast<float*>(Vp + NB);   // A_e on [2SB, NB - 2SB)
    float* dip = dep + NB;                             // 1 / A_o on [SB, NB - SB)
    const float rw = (float)S.r;
    for (int j = 2 * SB + threadIdx.x; j < NB - 2 * SB; j += NT) {
        int t, b, du, dd;
        cell(j, 0, t, b, du, dd);
        dep[j] = (float)(2.0 * S.r + S.m0 + S.g * SF.sigma[2 * buf_m(j) + b]);
    }
    const double* rhs_e = S.x + 4 * (size_t)Ve;    // after chi_e (compact float-float)
    // the odd hops of the updates and round 0 (compact float-float, 32 bytes a
    // site) in xs32, which this kernel leaves unused (its chi increment lives
    // in shared memory): t64 is the output, so the last update's u survives
    // the reconstruction of chi
    double* const T = reinterpret_cast<double*>(S.xs32);
    unsigned epoch = 0, gen = 0;
    int staged_k = -1;
#ifdef YK_CG_TIMING
    // block 0's cycles: reduce, A1 (with the staging wait), w/v/u, q, reliable
    // updates, round 0, the reconstruction of chi
    long long tacc[16] = {}, tlast = clock64();
    int tit = 0, tru = 0;
#endif

    auto stage = [&](int mode, int cur, int prv) {
        const float* Rl = (mode == kRedo) ? S.r32[cur] : S.r32[prv];
        const float* Pl = S.p32[prv];
        const float* Al = prv == 0 ? S.Ap32 : S.t32;
        for (int j = threadIdx.x; j < NB; j += NT) {
            const int m = buf_m(j);
            cp_async16(P_st + j, Pl + 4 * (size_t)m);
            cp_async16(R_st + j, Rl + 4 * (size_t)m);
            if (mode == kStep) cp_async16(A_st + j, Al + 4 * (size_t)m);
        }
        cp_async_commit();
    };

    // A1: p_k (r_k and the chi_e increment on the own sites) on [0, NB)
    auto pass_a1 = [&](int mode, int cur, int prv) {
        const SysLocal& L = sl[0];
        const W ar = L.f_alpha_re, beta = L.f_beta, cre = L.f_c_re, cim = L.f_c_im;
        for (int j = threadIdx.x; j < NB; j += NT) {
            const int o = own_of(j);
            const bool is_own = o >= 0;
            const int m = is_own ? own_m(o) : 0;
            const Site<W, K> po = ld_sm(P_st, j);
            Site<W, K> p;
            if (mode == kStep) {
                Site<W, K> r = ld_sm(R_st, j);
                site_axpy<W, K>(r, -ar, W(0), ld_sm(A_st, j));
#pragma unroll
                for (int i = 0; i < 4; ++i) p.v[i] = fma(beta, po.v[i], r.v[i]);
                if (is_own) {
                    Site<W, K> x = ld_sm(X_st, o);
                    site_axpy<W, K>(x, ar, W(0), ld_sm(V_own, o));
                    st_sm(X_st, o, x);
                    YK_ST(W, K, S.r32[cur], m, r);
                    YK_ST(W, K, S.p32[cur], m, p);
                    st_sm(R_st, j, r);
                }
            } else if (mode == kRedo) {
                p = p_next<W, K>(ld_sm(R_st, j), po, beta, cre, cim);
                if (is_own) YK_ST(W, K, S.p32[cur], m, p);
            } else {
                p = po;
            }
            st_sm(P_st, j, p);
        }
    };

    // w, v, u on their ranges (v of the own sites also to V_own)
    auto pass_wvu = [&]() {
        Site<W, K> zero;
#pragma unroll
        for (int i = 0; i < 4; ++i) zero.v[i] = W(0);
        for (int j = SB + threadIdx.x; j < NB - SB; j += NT) {
            int t, b, du, dd;
            cell(j, 1, t, b, du, dd);
            const W sp = (t + 1 == Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
            Site<W, K> h = eo_sm<false>(P_st, j, SB, du, dd, zero, W(0), rw, sp, sm);
            const W s = -dip[j];
#pragma unroll
            for (int i = 0; i < 4; ++i) h.v[i] *= s;
            st_sm(Wp, j, h);
        }
        __syncthreads();
        for (int j = 2 * SB + threadIdx.x; j < NB - 2 * SB; j += NT) {
            int t, b, du, dd;
            cell(j, 0, t, b, du, dd);
            const W sp = (t + 1 == Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
            const Site<W, K> v = eo_sm<false>(Wp, j, SB, du, dd, ld_sm(P_st, j), dep[j], rw, sp, sm);
            st_sm(Vp, j, v);
            const int o = own_of(j);
            if (o >= 0) st_sm(V_own, o, v);
        }
        __syncthreads();
        for (int j = 3 * SB + threadIdx.x; j < NB - 3 * SB; j += NT) {
            int t, b, du, dd;
            cell(j, 1, t, b, du, dd);
            const W sp = (t + 1 == Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
            Site<W, K> h = eo_sm<true>(Vp, j, SB, du, dd, zero, W(0), rw, sp, sm);
            const W s = -dip[j];
#pragma unroll
            for (int i = 0; i < 4; ++i) h.v[i] *= s;
            st_sm(Wp, j, h);   // u
        }
    };

    // q = S v on the own sites -> A p buffer of iteration cur; the tile partials.
    // Round 0 adds |eta|^2 of the compact index's two full sites in slot 5.
    auto pass_q = [&](int cur, bool round0) {
        float* Ac = cur == 0 ? S.Ap32 : S.t32;
        for (int base = tb; base < te; base += 2) {
            const int tile = base + hf;
            const bool tile_on = tile < te;
            const int o = (tile - tb) * kTile + ts;
            const bool on = tile_on && o < own;
            const int m = on ? own_m(o) : 0;
            FF f[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) f[i] = FF{0.f, 0.f};
            if (on) {
                const int j = own_j(o);
                int t, b, du, dd;
                cell(j, 0, t, b, du, dd);
                const W sp = (t + 1 == Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
                const Site<W, K> v = ld_sm(Vp, j);
                const Site<W, K> q = eo_sm<true>(Wp, j, SB, du, dd, v, dep[j], rw, sp, sm);
                YK_ST(W, K, Ac, m, q);
                const Site<W, K> r = ld_sm(R_st, j);
                W rq, dummy;
                site_dot<W, K>(r, q, rq, dummy);
                f[0] = FF{site_norm2<W, K>(r), 0.f};
                f[1] = FF{site_norm2<W, K>(q), 0.f};
                f[2] = FF{site_norm2<W, K>(v), 0.f};
                f[4] = FF{rq, 0.f};
                if (round0) {
                    const Site<double, K> e0 = load_site<double, K>(SF.b, 2 * m);
                    const Site<double, K> e1 = load_site<double, K>(SF.b, 2 * m + 1);
                    f[5] = ff_of(site_norm2<double, K>(e0) + site_norm2<double, K>(e1));
                }
            }
            if (round0)
                put_partial_ff<(1 << 3), true>(a, tile, tile_on, f, red);
            else if (s_fast)
                put_partial_ff<kSkipIm, false>(a, tile, tile_on, f, red, a.bar->fsum[(gen + 1u) % 3u], s_esc);
            else
                put_partial_ff<kSkipIm, false>(a, tile, tile_on, f, red);
        }
    };

    auto reduce = [&](int kk, bool ru) -> bool {
        auto prefetch = [&]() {
            if (ru) return;
            const int k1 = kk + 1;
            stage(kStep, k1 & 1, (k1 & 1) ^ 1);
            staged_k = k1;
        };
        return solo_reduce_body<K, true, true>(sa, gen, kk, ru, red, lst, sl[0], &s_nact, &s_anyru, s_cnt, s_esc, &s_fast, fsh,
                                         prefetch);
    };

    // the reliable update of iteration k, in float-float: fold chi_e += xs +
    // alpha v_{k-1}; u = -A_o^-1 H^dag_oe chi_e on the own odd sites (t64,
    // compact); r = rhs_e - (A_e chi_e + H^dag_eo u) on the own even sites ->
    // r32[cur]; partials |r|^2, <r, p_{k-1}> (FP32 squares of the FP32 r)
    auto reliable = [&](int cur, int prv) -> bool {
        double* chi = S.x;
        const HopFF hop = s_hop;
        const float al = sl[0].f_alpha_re;
        for (int o = threadIdx.x; o < own; o += NT) {
            const int m = own_m(o);
            SiteFF xv = ld_ff(chi, m);
            const Site<W, K> xs = ld_sm(X_st, o);
            const Site<W, K> vv = ld_sm(V_own, o);
            Site<W, K> zw;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float pr = __fmul_rn(al, vv.v[i]);   // alpha v exactly: (pr, its FMA error)
                xv.v[i] = ff_add(xv.v[i], FF{xs.v[i], 0.f});
                xv.v[i] = ff_add(xv.v[i], FF{pr, __fmaf_rn(al, vv.v[i], -pr)});
                zw.v[i] = W(0);
            }
            st_ff(chi, m, xv);
            st_sm(X_st, o, zw);
        }
        YK_TMARK(7);
        if (!nsync(a, ++epoch, deps)) return false;
        YK_TMARK(8);
        SiteFF zero;
#pragma unroll
        for (int i = 0; i < 4; ++i) zero.v[i] = FF{0.f, 0.f};
        for (int o = threadIdx.x; o < own; o += NT) {
            const int m = own_m(o);
            int t, b, du, dd;
            eo_geom(m, 1, Nh, sh, t, b, du, dd);
            const float sp = (t + 1 == Nt) ? -1.f : 1.f, sm = (t == 0) ? -1.f : 1.f;
            SiteFF h = eo_ff<true, 0>(chi, m, Ve, Nh, du, dd, zero, FF{0.f, 0.f}, hop, sp, sm);
            const FF s = ld_ff1(S.dinv, m);
#pragma unroll
            for (int i = 0; i < 4; ++i) h.v[i] = ff_mul(FF{-s.hi, -s.lo}, h.v[i]);
            st_ff(T, m, h);
        }
        YK_TMARK(9);
        if (!nsync(a, ++epoch, deps)) return false;
        YK_TMARK(10);
        for (int base = tb; base < te; base += 2) {
            const int tile = base + hf;
            const bool tile_on = tile < te;
            const int o = (tile - tb) * kTile + ts;
            const bool on = tile_on && o < own;
            const int m = on ? own_m(o) : 0;
            float v0 = 0.f, v2 = 0.f;
            if (on) {
                int t, b, du, dd;
                eo_geom(m, 0, Nh, sh, t, b, du, dd);
                const float sp = (t + 1 == Nt) ? -1.f : 1.f, sm = (t == 0) ? -1.f : 1.f;
                const FF de = ff_of(2.0 * S.r + S.m0 + S.g * SF.sigma[2 * m + b]);
                const SiteFF sx = eo_ff<true, 2>(T, m, Ve, Nh, du, dd, ld_ff(chi, m), de, hop, sp, sm);
                const SiteFF bv = ld_ff(rhs_e, m);
                const Site<W, K> pw = YK_LD(W, K, S.p32[prv], m);
                Site<W, K> rw32;
#pragma unroll
                for (int i = 0; i < 4; ++i) rw32.v[i] = ff_sub(bv.v[i], sx.v[i]).hi;
                YK_ST(W, K, S.r32[cur], m, rw32);
                W dummy;
                v0 = site_norm2<W, K>(rw32);
                site_dot<W, K>(rw32, pw, v2, dummy);
            }
            FF f[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) f[i] = FF{0.f, 0.f};
            f[0] = FF{v0, 0.f};
            f[2] = FF{v2, 0.f};
            if (s_fast)   // the fixed-point totals too, at the scale of |r|^2
                put_partial_ff<(1 << 1) | (1 << 4) | (1 << 5) | kSkipIm, true, true>(
                    a, tile, tile_on, f, red, a.bar->fsum[(gen + 1u) % 3u], s_esc);
            else
                put_partial_ff<(1 << 1) | (1 << 4) | (1 << 5) | kSkipIm, true>(a, tile, tile_on, f, red);
        }
        YK_TMARK(11);
        return true;
    };

    // ---------------- round 0: eta on the own sites of both classes (kept in
    // b for the force); on the odd ones 1 / A_o (dinv: the float-float
    // reciprocal of the FP64 diagonal) and -A_o^-1 eta_o (t64, compact);
    // chi_e = 0; rhs_e; r_0 = p_0 = rhs_e
    const bool eta32 = SF.gen_eta != 0;   // generated sources are FP32 normals
    for (int o = threadIdx.x; o < 2 * own; o += NT) {
        const int m = own_m(o >> 1), q = o & 1;
        int t, b, du, dd;
        eo_geom(m, q, Nh, sh, t, b, du, dd);
        const int n = 2 * m + b;   // the compact index's full site of class q
        const Site<double, K> bv = SF.gen_eta ? eta_of_step<K>(SF, n, a.eta_kind) : load_site<double, K>(SF.b, n);
        if (SF.gen_eta) store_site<double, K>(SF.b, n, bv);
        if (q) {
            const FF inv = ff_rcp(ff_of(2.0 * S.r + S.m0 + S.g * SF.sigma[n]));
            st_ff1(S.dinv, m, inv);
            const SiteFF e = ff_site_of(bv, eta32);
            SiteFF h;
#pragma unroll
            for (int i = 0; i < 4; ++i) h.v[i] = ff_mul(FF{-inv.hi, -inv.lo}, e.v[i]);
            st_ff(T, m, h);
        }
    }
    YK_TMARK(12);
    for (int o = threadIdx.x; o < own; o += NT) {
        Site<double, K> z;
        Site<W, K> zw;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            z.v[i] = 0.0;
            zw.v[i] = W(0);
        }
        store_site<double, K>(S.x, own_m(o), z);
        st_sm(X_st, o, zw);
        st_sm(V_own, o, zw);
    }
    if (!nsync(a, ++epoch, deps)) return;
    YK_TMARK(13);
    // 1 / A_o in FP32 on the widened range, from the owners' dinv
    for (int j = SB + threadIdx.x; j < NB - SB; j += NT) dip[j] = ld_ff1(S.dinv, buf_m(j)).hi;
    if constexpr (PATCH) {
        // r_0 = p_0 = rhs_e on the whole widened patch, formed here: the odd
        // values it reads (T, eta) lie in the eight surrounding patches, which
        // the neighbour sync above waited for, so neither a second sync nor a
        // staging of the neighbours' r_0 and p_0 is needed.  Every block forms
        // a cell's value with the same operations, so the copies agree bit for
        // bit; the own cells also go to rhs_e, r32[0] and p32[0].  Each thread
        // writes the cells that pass_a1 reads in the same thread.
        const HopFF hop = s_hop;
        for (int j = threadIdx.x; j < NB; j += NT) {
            const int m = buf_m(j);
            int t, b, du, dd;
            eo_geom(m, 0, Nh, sh, t, b, du, dd);
            const float sp = (t + 1 == Nt) ? -1.f : 1.f, sm = (t == 0) ? -1.f : 1.f;
            const SiteFF e = ff_site_of(load_site<double, K>(SF.b, 2 * m + b), eta32);
            // eta_e + H^dag_eo (-A_o^-1 eta_o)
            const SiteFF rh = eo_ff<true, 1>(T, m, Ve, Nh, du, dd, e, FF{1.f, 0.f}, hop, sp, sm);
            Site<W, K> rw32;
#pragma unroll
            for (int i = 0; i < 4; ++i) rw32.v[i] = rh.v[i].hi;
            st_sm(P_st, j, rw32);
            st_sm(R_st, j, rw32);
            if (own_of(j) >= 0) {
                st_ff(const_cast<double*>(rhs_e), m, rh);
                YK_ST(W, K, S.r32[0], m, rw32);
                YK_ST(W, K, S.p32[0], m, rw32);
            }
        }
        YK_TMARK(14);
        YK_TMARK(15);
    } else {
        const HopFF hop = s_hop;
        for (int o = threadIdx.x; o < own; o += NT) {
            const int m = own_m(o);
            int t, b, du, dd;
            eo_geom(m, 0, Nh, sh, t, b, du, dd);
            const float sp = (t + 1 == Nt) ? -1.f : 1.f, sm = (t == 0) ? -1.f : 1.f;
            const SiteFF e = ff_site_of(load_site<double, K>(SF.b, 2 * m + b), eta32);
            // eta_e + H^dag_eo (-A_o^-1 eta_o)
            const SiteFF rh = eo_ff<true, 1>(T, m, Ve, Nh, du, dd, e, FF{1.f, 0.f}, hop, sp, sm);
            st_ff(const_cast<double*>(rhs_e), m, rh);
            Site<W, K> rw32;
#pragma unroll
            for (int i = 0; i < 4; ++i) rw32.v[i] = rh.v[i].hi;
            YK_ST(W, K, S.r32[0], m, rw32);
            YK_ST(W, K, S.p32[0], m, rw32);
        }
        YK_TMARK(14);
        if (!nsync(a, ++epoch, deps)) return;
        YK_TMARK(15);
        stage(kHaloInit, 0, 0);
        cp_async_wait_all();
    }
    pass_a1(kHaloInit, 0, 0);
    __syncthreads();
    pass_wvu();
    __syncthreads();
    pass_q(0, true);
    if (!reduce(0, false)) return;
    YK_TMARK(5);

    int k = 1;
    while (k <= a.max_iter) {
        const int mode = sl[0].mode;
        if (s_nact == 0 || mode == kRu) {
            if (staged_k == k) cp_async_wait_all();
            staged_k = -1;
        }
        if (s_nact == 0) break;
        const int cur = k & 1, prv = cur ^ 1;
        if (mode == kRu) {
            if (!reliable(cur, prv)) return;
            if (!reduce(k, true)) return;
            YK_TMARK(4);
#ifdef YK_CG_TIMING
            ++tru;
#endif
            continue;
        }
        if (!(mode == kStep && staged_k == k)) {
            if (staged_k == k) cp_async_wait_all();
            stage(mode, cur, prv);
        }
        staged_k = -1;
        cp_async_wait_all();
        pass_a1(mode, cur, prv);
        __syncthreads();
        YK_TMARK(1);
        pass_wvu();
        __syncthreads();
        YK_TMARK(2);
        pass_q(cur, false);
        YK_TMARK(3);
        if (!reduce(k, false)) return;
        YK_TMARK(0);
        ++k;
#ifdef YK_CG_TIMING
        ++tit;
#endif
    }
    // chi of both classes in the full layout for the force (t64): every
    // block's final chi_e and its own odd sites' chi_o = A_o^-1 (eta_o - H^dag_oe chi_e).
    // A solve that retired converged in an update round (the block's copy of
    // the replicated state says so, alike in every block) has u = -A_o^-1
    // H^dag_oe chi_e of its final chi_e in T already: chi_o = A_o^-1 eta_o + u,
    // own sites only, no neighbour sync
    if (lst.chi_ready && lst.converged) {
        for (int o = threadIdx.x; o < own; o += NT) {
            const int m = own_m(o);
            int t, b, du, dd;
            eo_geom(m, 0, Nh, sh, t, b, du, dd);
            const SiteFF xe = ld_ff(S.x, m);
            Site<double, K> ce;
#pragma unroll
            for (int i = 0; i < 4; ++i) ce.v[i] = dbl_of(xe.v[i]);
            store_site<double, K>(SF.t64, 2 * m + b, ce);
            eo_geom(m, 1, Nh, sh, t, b, du, dd);
            const int n = 2 * m + b;
            const SiteFF e = ff_site_of(load_site<double, K>(SF.b, n), eta32);
            const SiteFF u = ld_ff(T, m);
            const FF inv = ld_ff1(S.dinv, m);
            Site<double, K> co;
#pragma unroll
            for (int i = 0; i < 4; ++i) co.v[i] = dbl_of(ff_add(ff_mul(e.v[i], inv), u.v[i]));
            store_site<double, K>(SF.t64, n, co);
        }
    } else {
        if (!nsync(a, ++epoch, deps)) return;
        const HopFF hop = s_hop;
        SiteFF zero;
#pragma unroll
        for (int i = 0; i < 4; ++i) zero.v[i] = FF{0.f, 0.f};
        for (int o = threadIdx.x; o < own; o += NT) {
            const int m = own_m(o);
            int t, b, du, dd;
            eo_geom(m, 0, Nh, sh, t, b, du, dd);
            const SiteFF xe = ld_ff(S.x, m);
            Site<double, K> ce;
#pragma unroll
            for (int i = 0; i < 4; ++i) ce.v[i] = dbl_of(xe.v[i]);
            store_site<double, K>(SF.t64, 2 * m + b, ce);
            eo_geom(m, 1, Nh, sh, t, b, du, dd);
            const float sp = (t + 1 == Nt) ? -1.f : 1.f, sm = (t == 0) ? -1.f : 1.f;
            const SiteFF h = eo_ff<true, 0>(S.x, m, Ve, Nh, du, dd, zero, FF{0.f, 0.f}, hop, sp, sm);
            const int n = 2 * m + b;
            const SiteFF e = ff_site_of(load_site<double, K>(SF.b, n), eta32);
            const FF inv = ld_ff1(S.dinv, m);
            Site<double, K> co;
#pragma unroll
            for (int i = 0; i < 4; ++i) co.v[i] = dbl_of(ff_mul(ff_sub(e.v[i], h.v[i]), inv));
            store_site<double, K>(SF.t64, n, co);
        }
    }
    // t64 holds chi however the solve ended (also when it retired at k = 0)
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st[a.sys_first].chi_ready = 1;
#ifdef YK_CG_TIMING
    YK_TMARK(6);
    if (blockIdx.x == 0 && threadIdx.x == 0 && tit > 0)
        printf("eo timing (block 0, cycles; %d iterations, %d reliable updates): per iteration reduce %lld  A1 %lld  "
               "wvu %lld  q %lld | per update %lld | round 0 %lld  reconstruction %lld\n",
               tit, tru, tacc[0] / tit, tacc[1] / tit, tacc[2] / tit, tacc[3] / tit, tru ? tacc[4] / tru : 0ll, tacc[5],
               tacc[6]);
    if (blockIdx.x == 0 && threadIdx.x == 0 && tru > 0)
        printf("eo timing (per update): fold %lld  nsync %lld  odd %lld  nsync %lld  even %lld  reduce %lld | round 0: "
               "eta %lld  nsync %lld  rhs %lld  nsync %lld  rest %lld\n",
               tacc[7] / tru, tacc[8] / tru, tacc[9] / tru, tacc[10] / tru, tacc[11] / tru, tacc[4] / tru, tacc[12],
               tacc[13], tacc[14], tacc[15], tacc[5]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        volatile unsigned long long* q = g_cg_q;
        volatile unsigned long long* f = g_cg_f;
        const unsigned long long nq = f[3] ? f[3] : 1;
        printf("eo timing (reduction marks over %llu): entry-sync %llu  arrive %llu  wait %llu  sync %llu  "
               "convert %llu  step %llu  state %llu  end-sync %llu\n",
               nq, q[0] / nq, q[1] / nq, q[2] / nq, q[3] / nq, q[4] / nq, q[5] / nq, q[6] / nq, q[7] / nq);
        for (int i = 0; i < 8; ++i) f[i] = 0;
        for (int i = 0; i < 16; ++i) q[i] = 0;
    }
#endif
}

// ---------------------------------------------------------------------------
// Batched even-odd mixed CG (cg_eob_kernel): the Schur-complement CGNE of
// cg_eo_kernel for every system of a batched step at once (chains of any
// even lattice, several right-hand sides each), and for single systems too
// large for cg_eo_kernel's shared memory.  The systems' compact views share
// one tile table; tile partials, the finisher's per-system scalar steps and
// the coefficient words are those of cg_kernel (finish_reduction,
// scalar_step with the even-odd first threshold).
//
// Work is dealt out per pass, not per block: each pass takes the tiles of
// the systems that work in it (a prefix over the systems' tile counts,
// rebuilt from the published modes every round) and gives every block an
// equal contiguous share.  A system that converges early leaves no block
// idle while the slow ones iterate; passes are separated by grid barriers.
// A round, each system by its mode (kStep, kRedo after an update; kRu):
//   P1 (even)  r, p, chi increment of the own site; w = -A_o^-1 H_oe p at the
//              compact index's odd site, the neighbours' p formed from the
//              previous iteration's r, q, p (the same arithmetic as theirs);
//              kRu: fold chi_e += xs + alpha v in float-float
//   P2 (even)  v = A_e p + H_eo w (= S^dag p);  kRu: R2 u = -A_o^-1 H^dag_oe
//              chi_e in float-float (t64)
//   P3 (odd)   u = -A_o^-1 H^dag_oe v;  kRu: R3 r = rhs_e - (A_e chi_e +
//              H^dag_eo u) in float-float, partials |r|^2, <r, p_{k-1}>
//   P4 (even)  q = A_e v + H^dag_eo u (= S v), tile partials |r|^2, |q|^2,
//              |v|^2, <r, q>; the reducing barrier.
// A system's update thus costs no round of the others: each keeps its own
// iteration index, and its buffers alternate with that index's parity
// (published with its coefficients).
// Round 0: eta (both classes), 1 / A_o (dinv), -A_o^-1 eta_o; rhs_e; then the
// passes of an ordinary round from p_0 = r_0 = rhs_e (slot 5: |eta|^2).
// At the end chi in the full layout (t64) for the force.
// Buffers of a view (compact, Ve = V / 2 sites): x = chi_e then rhs_e (FP64),
// t64 the odd FP64 hops, r32[2], p32[2], q in Ap32 / t32 by iteration parity,
// xs32 the chi increment, v32 and w32 (w, later u), diag32 = A_e then 1 / A_o
// in FP32, dinv 1 / A_o in FP64.
// ---------------------------------------------------------------------------
constexpr int kEobMaxSys = kEobMaxSystems;

// Grid barrier without a reduction (the arrival counter of grid_reduce runs on).
__device__ bool eob_barrier(const CGArgs& a, unsigned& gen)
{
    __syncthreads();
    int bad = 0;
    if (threadIdx.x == 0) {
        arrive_release(&a.bar->arrive);
        const unsigned target = gridDim.x * (gen + 1u);
        const long long t0 = clock64();
        while ((int)(ld_acquire(&a.bar->arrive) - target) < 0)
            if (wait_over(t0, a.err)) {
                bad = 1;
                break;
            }
    }
    ++gen;
    return __syncthreads_or(bad) == 0;
}

// Exclusive prefix over the systems of the tile counts of those whose mode is
// in `mask` (bit per mode); s_pre[nsys] = the total.  Two systems per thread
// (blockDim = 512, nsys <= 1024).
__device__ void eob_scan(int nsys, const int* s_mode, const int* s_nt, int mask, int* s_pre)
{
    __shared__ int ws[kHaloThreads / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int q0 = 2 * t, q1 = 2 * t + 1;
    const int c0 = (q0 < nsys && ((mask >> s_mode[q0]) & 1)) ? s_nt[q0] : 0;
    const int c1 = (q1 < nsys && ((mask >> s_mode[q1]) & 1)) ? s_nt[q1] : 0;
    int v = c0 + c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) ws[w] = v;
    __syncthreads();
    if (w == 0) {
        int x = lane < kHaloThreads / 32 ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane < kHaloThreads / 32) ws[lane] = x;
    }
    __syncthreads();
    const int base = (w > 0 ? ws[w - 1] : 0) + v - (c0 + c1);
    if (q0 < nsys) s_pre[q0] = base;
    if (q1 < nsys) s_pre[q1] = base + c0;
    if (t == 0) s_pre[nsys] = ws[kHaloThreads / 32 - 1];
    __syncthreads();
}

// The system of entry i of the current prefix: the largest q < nsys with
// s_pre[q] <= i (systems without tiles in the pass share their successor's start).
__device__ __forceinline__ int eob_find(int i, int nsys, const int* s_pre)
{
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_pre[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// This block's contiguous share [lo, hi) of `total` entries.
__device__ __forceinline__ void eob_share(int total, int* lo, int* hi)
{
    *lo = (int)(((long long)total * blockIdx.x) / gridDim.x);
    *hi = (int)(((long long)total * (blockIdx.x + 1)) / gridDim.x);
}

// The reducing barrier of a round: after the barrier every block finishes
// the systems q = blockIdx.x, blockIdx.x + gridDim.x, ...: sums their tile
// partials (sum_partials: fixed order), runs the scalar step at the system's
// own iteration index (an update ran in this round for a system in kRu; the
// round that redoes its step keeps the index) and publishes the coefficients,
// mode and buffer parity of the next round.  No block finishes for all.
__device__ bool eob_reduce(const CGArgs& a, unsigned& gen, int k, double* red, int* s_active, int* s_ru)
{
    if (!eob_barrier(a, gen)) return false;
    for (int q = blockIdx.x; q < a.sys_count; q += gridDim.x) {
        const int j = a.sys_first + q;
        const SysDev& S = a.sys[j];
        double s[6];
        sum_partials<true>(a, S.tile0, S.ntiles, red, s);
        if (threadIdx.x == 0) {
            CGState st;
            load_state(a.st + j, st);
            CoefVals cv = {0.0, 0.0, 0.0, 1.0, 0.0, kIdle};
            if (st.mode != kIdle) {
                const int ks = k == 0 ? 0 : (st.mode == kRedo ? st.iters : st.iters + 1);
                cv = scalar_step<true>(a, ks, st.mode == kRu, s, st, s_active, s_ru);
                cv.par = (cv.mode == kRedo ? st.iters : st.iters + 1) & 1;
            }
            st.mode = cv.mode;
            store_state(a.st + j, st);
            __threadfence();
            publish_coef(a.coef + j, cv, gen);
        }
    }
    return true;
}

// Modes of the round from the published coefficient words of every system;
// *nact (every thread) = how many threads saw a system still iterating.
__device__ bool eob_load_coefs(const CGArgs& a, unsigned gen, int nsys, int* s_mode, int* s_par, float* s_fa,
                               float* s_fb, float* s_fc, int* nact)
{
    int bad = 0, act = 0;
    for (int q = threadIdx.x; q < nsys; q += blockDim.x) {
        CoefVals v;
        if (!poll_coef(a.coef + a.sys_first + q, gen, v, a.err)) {
            bad = 1;
        } else {
            s_mode[q] = v.mode;
            s_par[q] = v.par;
            s_fa[q] = (float)v.alpha_re;
            s_fb[q] = (float)v.beta;
            s_fc[q] = (float)v.c_re;
            act += v.mode != kIdle;
        }
    }
    *nact = __syncthreads_count(act > 0);
    return __syncthreads_or(bad) == 0;
}

__global__ void __launch_bounds__(kHaloThreads) cg_eob_kernel(CGArgs a)
{
    constexpr int K = 1;
    constexpr int kSkipIm = (1 << 3) | (1 << 5);
    using W = float;
    const int hf = threadIdx.x / kTile, ts = threadIdx.x % kTile;
    __shared__ double red[128];
    __shared__ int s_mode[kEobMaxSys], s_par[kEobMaxSys], s_nt[kEobMaxSys], s_t0[kEobMaxSys], s_pre[kEobMaxSys + 1];
    __shared__ float s_fa[kEobMaxSys], s_fb[kEobMaxSys], s_fc[kEobMaxSys];
    __shared__ int s_active, s_ru;   // the scalar step's counters (unused here)
    const int nsys = a.sys_count;
    for (int q = threadIdx.x; q < nsys; q += blockDim.x) {
        const SysDev& S = a.sys[a.sys_first + q];
        s_nt[q] = S.ntiles;
        s_t0[q] = S.tile0;
        s_mode[q] = kStep;
        s_par[q] = 0;
        s_fa[q] = s_fb[q] = s_fc[q] = 0.f;
    }
    __syncthreads();
    if (*(volatile int*)a.err) return;
    unsigned gen = 0;
#ifdef YK_CG_TIMING
    // block 0's cycles per round: coefficients, P1, barrier, P2+R2, barrier,
    // P3+R3, barrier, P4, reduce
    long long tacc[10] = {}, tlast = clock64();
    int tit = 0;
#endif
    constexpr int kAll = (1 << kStep) | (1 << kRedo) | (1 << kRu) | (1 << kWait);
    constexpr int kP1 = (1 << kStep) | (1 << kRedo) | (1 << kRu);
    constexpr int kP2 = (1 << kStep) | (1 << kRedo);
    constexpr int kPR = 1 << kRu;
    constexpr int kInit = -1;   // round 0: p_0 as stored

    // Runs f(S, q, m, tile, on) for every site of this block's share of the
    // tiles of the systems in `mask`, two tiles at a time (every thread the
    // same trip count: f may hold block-wide barriers).
    auto for_sites = [&](int mask, auto&& f) {
        eob_scan(nsys, s_mode, s_nt, mask, s_pre);
        int lo, hi;
        eob_share(s_pre[nsys], &lo, &hi);
        int qc = -1;   // the previous tile's system: a contiguous share mostly stays in one
        for (int base = lo; base < hi; base += 2) {
            const int i = base + hf;
            const bool tile_on = i < hi;
            const int ii = tile_on ? i : lo;
            const int q = (qc >= 0 && ii >= s_pre[qc] && ii < s_pre[qc + 1]) ? qc : eob_find(ii, nsys, s_pre);
            qc = q;
            const int lt = ii - s_pre[q];
            const SysDev& S = a.sys[a.sys_first + q];
            const int m = lt * kTile + ts;
            f(S, q, m, s_t0[q] + lt, tile_on, tile_on && m < S.V);
        }
    };

    // the compact geometry of site m of class c: row t, time signs
    struct Geo {
        int t, b, du, dd, mu, md;
        float sp, sm;
    };
    auto geo = [](const SysDev& S, int m, int c) {
        Geo g;
        const int Nh = S.Nx, Ve = S.V;
        g.t = m / Nh;
        const int i = m - g.t * Nh;
        g.b = (g.t + c) & 1;
        g.du = g.b ? ((i == Nh - 1) ? 1 - Nh : 1) : 0;
        g.dd = g.b ? 0 : ((i == 0) ? Nh - 1 : -1);
        g.mu = m + Nh >= Ve ? m + Nh - Ve : m + Nh;
        g.md = m - Nh < 0 ? m - Nh + Ve : m - Nh;
        g.sp = (g.t + 1 == S.Nt) ? -1.f : 1.f;
        g.sm = (g.t == 0) ? -1.f : 1.f;
        return g;
    };
    auto qbuf = [](const SysDev& S, int it) -> float* { return it == 0 ? S.Ap32 : S.t32; };

    // p of iteration `cur` at even compact site n (mode kStep: from r, q, p of
    // prv; kRedo: from the FP64 residual in r[cur]; round 0: p_0 as stored)
    auto p_at = [&](const SysDev& S, int q, int n, int mode, int cur, int prv) -> Site<W, K> {
        if (mode == kStep) {
            Site<W, K> r = YK_LD(W, K, S.r32[prv], n);
            site_axpy<W, K>(r, -s_fa[q], W(0), YK_LD(W, K, qbuf(S, prv), n));
            const Site<W, K> po = YK_LD(W, K, S.p32[prv], n);
            Site<W, K> p;
#pragma unroll
            for (int e = 0; e < 4; ++e) p.v[e] = fma(s_fb[q], po.v[e], r.v[e]);
            return p;
        }
        if (mode == kRedo)
            return p_next<W, K>(YK_LD(W, K, S.r32[cur], n), YK_LD(W, K, S.p32[prv], n), s_fb[q], s_fc[q], W(0));
        return YK_LD(W, K, S.p32[cur], n);
    };

    // P1 of an ordinary round (init: round 0, p_0 as stored) and the fold of
    // a reliable-update round
    auto pass_p1 = [&](bool init) {
        for_sites(init ? kAll : kP1, [&](const SysDev& S, int q, int m, int, bool, bool on) {
            if (!on) return;
            const int mode = init ? kInit : s_mode[q];
            const int cur = s_par[q], prv = cur ^ 1;
            if (mode == kRu) {
                SiteFF xv = ld_ff(S.x, m);
                const Site<W, K> xs = YK_LD(W, K, S.xs32, m);
                const Site<W, K> vv = YK_LD(W, K, S.v32, m);
                const float al = s_fa[q];
                Site<W, K> zw;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float pr = __fmul_rn(al, vv.v[e]);   // alpha v exactly: (pr, its FMA error)
                    xv.v[e] = ff_add(xv.v[e], FF{xs.v[e], 0.f});
                    xv.v[e] = ff_add(xv.v[e], FF{pr, __fmaf_rn(al, vv.v[e], -pr)});
                    zw.v[e] = W(0);
                }
                st_ff(S.x, m, xv);
                YK_ST(W, K, S.xs32, m, zw);
                return;
            }
            if (mode == kStep) {
                Site<W, K> r = YK_LD(W, K, S.r32[prv], m);
                site_axpy<W, K>(r, -s_fa[q], W(0), YK_LD(W, K, qbuf(S, prv), m));
                const Site<W, K> po = YK_LD(W, K, S.p32[prv], m);
                Site<W, K> p;
#pragma unroll
                for (int e = 0; e < 4; ++e) p.v[e] = fma(s_fb[q], po.v[e], r.v[e]);
                Site<W, K> xs = YK_LD(W, K, S.xs32, m);
                site_axpy<W, K>(xs, s_fa[q], W(0), YK_LD(W, K, S.v32, m));
                YK_ST(W, K, S.xs32, m, xs);
                YK_ST(W, K, S.r32[cur], m, r);
                YK_ST(W, K, S.p32[cur], m, p);
            } else if (mode == kRedo) {
                YK_ST(W, K, S.p32[cur], m, (p_at(S, q, m, kRedo, cur, prv)));
            }
            // w at the compact index's odd site from the p of its even neighbours
            const Geo g = geo(S, m, 1);
            Site<W, K> zero;
#pragma unroll
            for (int e = 0; e < 4; ++e) zero.v[e] = W(0);
            Site<W, K> h = dirac_combine<W, K, false>(zero, p_at(S, q, g.mu, mode, cur, prv),
                                                      p_at(S, q, g.md, mode, cur, prv),
                                                      p_at(S, q, m + g.du, mode, cur, prv),
                                                      p_at(S, q, m + g.dd, mode, cur, prv), W(0), (W)S.r, g.sp, g.sm);
            const W s = -S.diag32[S.V + m];
#pragma unroll
            for (int e = 0; e < 4; ++e) h.v[e] *= s;
            YK_ST(W, K, S.w32, m, h);
        });
    };

    // P2: v = A_e p + H_eo w (even)
    auto pass_p2 = [&](int mask) {
        for_sites(mask, [&](const SysDev& S, int q, int m, int, bool, bool on) {
            if (!on) return;
            const int cur = s_par[q];
            const Geo g = geo(S, m, 0);
            const Site<W, K> v = dirac_combine<W, K, false>(
                YK_LD(W, K, S.p32[cur], m), YK_LD(W, K, S.w32, g.mu), YK_LD(W, K, S.w32, g.md),
                YK_LD(W, K, S.w32, m + g.du), YK_LD(W, K, S.w32, m + g.dd), S.diag32[m], (W)S.r, g.sp, g.sm);
            YK_ST(W, K, S.v32, m, v);
        });
    };

    // P3: u = -A_o^-1 H^dag_oe v (odd, into w32)
    auto pass_p3 = [&](int mask) {
        for_sites(mask, [&](const SysDev& S, int, int m, int, bool, bool on) {
            if (!on) return;
            const Geo g = geo(S, m, 1);
            Site<W, K> zero;
#pragma unroll
            for (int e = 0; e < 4; ++e) zero.v[e] = W(0);
            Site<W, K> h = dirac_combine<W, K, true>(zero, YK_LD(W, K, S.v32, g.mu), YK_LD(W, K, S.v32, g.md),
                                                     YK_LD(W, K, S.v32, m + g.du), YK_LD(W, K, S.v32, m + g.dd),
                                                     W(0), (W)S.r, g.sp, g.sm);
            const W s = -S.diag32[S.V + m];
#pragma unroll
            for (int e = 0; e < 4; ++e) h.v[e] *= s;
            YK_ST(W, K, S.w32, m, h);
        });
    };

    // P4: q = A_e v + H^dag_eo u (even) and the tile partials (round 0 adds
    // |eta|^2 of the compact index's two full sites in slot 5)
    auto pass_p4 = [&](int mask, bool round0) {
        for_sites(mask, [&](const SysDev& S, int q, int m, int tile, bool tile_on, bool on) {
            const int cur = s_par[q];
            FF f[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) f[i] = FF{0.f, 0.f};
            if (on) {
                const Geo g = geo(S, m, 0);
                const Site<W, K> v = YK_LD(W, K, S.v32, m);
                const Site<W, K> qv = dirac_combine<W, K, true>(
                    v, YK_LD(W, K, S.w32, g.mu), YK_LD(W, K, S.w32, g.md), YK_LD(W, K, S.w32, m + g.du),
                    YK_LD(W, K, S.w32, m + g.dd), S.diag32[m], (W)S.r, g.sp, g.sm);
                YK_ST(W, K, qbuf(S, cur), m, qv);
                const Site<W, K> r = YK_LD(W, K, S.r32[cur], m);
                W rq, dummy;
                site_dot<W, K>(r, qv, rq, dummy);
                f[0] = FF{site_norm2<W, K>(r), 0.f};
                f[1] = FF{site_norm2<W, K>(qv), 0.f};
                f[2] = FF{site_norm2<W, K>(v), 0.f};
                f[4] = FF{rq, 0.f};
                if (round0) {
                    const Site<double, K> e0 = load_site<double, K>(S.b, 2 * m);
                    const Site<double, K> e1 = load_site<double, K>(S.b, 2 * m + 1);
                    f[5] = ff_of(site_norm2<double, K>(e0) + site_norm2<double, K>(e1));
                }
            }
            if (round0)
                put_partial_ff<(1 << 3), true>(a, tile, tile_on, f, red);
            else
                put_partial_ff<kSkipIm, false>(a, tile, tile_on, f, red);
        });
    };

    // ---------------- round 0
    // eta of both classes (b, full layout), A_e and 1 / A_o, -A_o^-1 eta_o (t64),
    // chi_e = xs = v = 0
    for_sites(kAll, [&](const SysDev& S, int, int m, int, bool, bool on) {
        if (!on) return;
        const int Ve = S.V;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const Geo g = geo(S, m, c);
            const int n = 2 * m + g.b;
            const Site<double, K> bv = S.gen_eta ? eta_of_step<K>(S, n, a.eta_kind) : load_site<double, K>(S.b, n);
            if (S.gen_eta) store_site<double, K>(S.b, n, bv);
            const double d = 2.0 * S.r + S.m0 + S.g * S.sigma[n];
            if (c == 0) {
                S.diag32[m] = (float)d;
            } else {
                const FF inv = ff_rcp(ff_of(d));
                st_ff1(S.dinv, m, inv);
                S.diag32[Ve + m] = inv.hi;
                const SiteFF e = ff_site_of(bv, S.gen_eta != 0);
                SiteFF h;
#pragma unroll
                for (int e2 = 0; e2 < 4; ++e2) h.v[e2] = ff_mul(FF{-inv.hi, -inv.lo}, e.v[e2]);
                st_ff(S.t64, m, h);
            }
        }
        Site<double, K> z;
        Site<W, K> zw;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            z.v[e] = 0.0;
            zw.v[e] = W(0);
        }
        store_site<double, K>(S.x, m, z);
        YK_ST(W, K, S.xs32, m, zw);
        YK_ST(W, K, S.v32, m, zw);
    });
    if (!eob_barrier(a, gen)) return;
    // rhs_e = eta_e + H^dag_eo (-A_o^-1 eta_o); r_0 = p_0 = rhs_e
    for_sites(kAll, [&](const SysDev& S, int, int m, int, bool, bool on) {
        if (!on) return;
        const Geo g = geo(S, m, 0);
        const SiteFF e = ff_site_of(load_site<double, K>(S.b, 2 * m + g.b), S.gen_eta != 0);
        const SiteFF rh =
            eo_ff<true, 1>(S.t64, m, S.V, S.Nx, g.du, g.dd, e, FF{1.f, 0.f}, hop_of_r(S.r), g.sp, g.sm);
        st_ff(S.x + 4 * (size_t)S.V, m, rh);
        Site<W, K> rw;
#pragma unroll
        for (int e2 = 0; e2 < 4; ++e2) rw.v[e2] = rh.v[e2].hi;
        YK_ST(W, K, S.r32[0], m, rw);
        YK_ST(W, K, S.p32[0], m, rw);
    });
    if (!eob_barrier(a, gen)) return;
    pass_p1(true);
    if (!eob_barrier(a, gen)) return;
    pass_p2(kAll);
    if (!eob_barrier(a, gen)) return;
    pass_p3(kAll);
    if (!eob_barrier(a, gen)) return;
    pass_p4(kAll, true);
    if (!eob_reduce(a, gen, 0, red, &s_active, &s_ru)) return;

    // Systems in kRu run their update in the passes of the round (R2 beside P2,
    // R3 beside P3); every system keeps its own iteration index (the
    // finisher's), which advances at least every other round.
    int k = 1;
    const int kmax = 2 * a.max_iter + 2;
    while (k <= kmax) {
        YK_TMARK(8);
        int nact = 0;
        if (!eob_load_coefs(a, gen, nsys, s_mode, s_par, s_fa, s_fb, s_fc, &nact)) return;
        if (nact == 0) break;
        YK_TMARK(0);
        pass_p1(false);
        YK_TMARK(1);
        if (!eob_barrier(a, gen)) return;
        YK_TMARK(2);
        pass_p2(kP2);
        // R2: u = -A_o^-1 H^dag_oe chi_e (float-float, odd, t64)
        for_sites(kPR, [&](const SysDev& S, int, int m, int, bool, bool on) {
            if (!on) return;
            const Geo g = geo(S, m, 1);
            SiteFF zero;
#pragma unroll
            for (int e = 0; e < 4; ++e) zero.v[e] = FF{0.f, 0.f};
            SiteFF h = eo_ff<true, 0>(S.x, m, S.V, S.Nx, g.du, g.dd, zero, FF{0.f, 0.f}, hop_of_r(S.r), g.sp, g.sm);
            const FF sc = ld_ff1(S.dinv, m);
#pragma unroll
            for (int e = 0; e < 4; ++e) h.v[e] = ff_mul(FF{-sc.hi, -sc.lo}, h.v[e]);
            st_ff(S.t64, m, h);
        });
        YK_TMARK(3);
        if (!eob_barrier(a, gen)) return;
        YK_TMARK(4);
        pass_p3(kP2);
        // R3: r = rhs_e - (A_e chi_e + H^dag_eo u) in float-float; |r|^2,
        // <r, p_{k-1}> (FP32 squares of the FP32 r)
        for_sites(kPR, [&](const SysDev& S, int q, int m, int tile, bool tile_on, bool on) {
            const int cur = s_par[q], prv = cur ^ 1;
            float v0 = 0.f, v2 = 0.f;
            if (on) {
                const Geo g = geo(S, m, 0);
                const FF de = ff_of(2.0 * S.r + S.m0 + S.g * S.sigma[2 * m + g.b]);
                const SiteFF sx =
                    eo_ff<true, 2>(S.t64, m, S.V, S.Nx, g.du, g.dd, ld_ff(S.x, m), de, hop_of_r(S.r), g.sp, g.sm);
                const SiteFF bv = ld_ff(S.x + 4 * (size_t)S.V, m);
                const Site<W, K> pw = YK_LD(W, K, S.p32[prv], m);
                Site<W, K> rw;
#pragma unroll
                for (int e = 0; e < 4; ++e) rw.v[e] = ff_sub(bv.v[e], sx.v[e]).hi;
                YK_ST(W, K, S.r32[cur], m, rw);
                W dummy;
                v0 = site_norm2<W, K>(rw);
                site_dot<W, K>(rw, pw, v2, dummy);
            }
            FF f[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) f[i] = FF{0.f, 0.f};
            f[0] = FF{v0, 0.f};
            f[2] = FF{v2, 0.f};
            put_partial_ff<(1 << 1) | (1 << 4) | (1 << 5) | kSkipIm, true>(a, tile, tile_on, f, red);
        });
        YK_TMARK(5);
        if (!eob_barrier(a, gen)) return;
        YK_TMARK(6);
        pass_p4(kP2, false);
        YK_TMARK(7);
        if (!eob_reduce(a, gen, k, red, &s_active, &s_ru)) return;
        ++k;
#ifdef YK_CG_TIMING
        ++tit;
#endif
    }
#ifdef YK_CG_TIMING
    if (blockIdx.x == 0 && threadIdx.x == 0 && tit > 0)
        printf("eob timing (block 0 of %d, cycles per round over %d rounds): coefs %lld  P1 %lld  bar %lld  P2+R2 %lld  "
               "bar %lld  P3+R3 %lld  bar %lld  P4 %lld  reduce %lld\n",
               (int)gridDim.x, tit, tacc[0] / tit, tacc[1] / tit, tacc[2] / tit, tacc[3] / tit, tacc[4] / tit,
               tacc[5] / tit, tacc[6] / tit, tacc[7] / tit, tacc[8] / tit);
#endif
    // chi of both classes in the full layout (t64) for the force: chi_e, and
    // chi_o = A_o^-1 (eta_o - H^dag_oe chi_e)
    if (!eob_barrier(a, gen)) return;
    for_sites(kAll | (1 << kIdle), [&](const SysDev& S, int, int m, int, bool, bool on) {
        if (!on) return;
        Geo g = geo(S, m, 0);
        const SiteFF xe = ld_ff(S.x, m);
        Site<double, K> ce;
#pragma unroll
        for (int e = 0; e < 4; ++e) ce.v[e] = dbl_of(xe.v[e]);
        store_site<double, K>(S.t64, 2 * m + g.b, ce);
        g = geo(S, m, 1);
        SiteFF zero;
#pragma unroll
        for (int e = 0; e < 4; ++e) zero.v[e] = FF{0.f, 0.f};
        const SiteFF h = eo_ff<true, 0>(S.x, m, S.V, S.Nx, g.du, g.dd, zero, FF{0.f, 0.f}, hop_of_r(S.r), g.sp, g.sm);
        const int n = 2 * m + g.b;
        const SiteFF e = ff_site_of(load_site<double, K>(S.b, n), S.gen_eta != 0);
        const FF inv = ld_ff1(S.dinv, m);
        Site<double, K> co;
#pragma unroll
        for (int e2 = 0; e2 < 4; ++e2) co.v[e2] = dbl_of(ff_mul(ff_sub(e.v[e2], h.v[e2]), inv));
        store_site<double, K>(S.t64, n, co);
    });
    if (blockIdx.x == 0)
        for (int q = threadIdx.x; q < nsys; q += blockDim.x) a.st[a.sys_first + q].chi_ready = 1;
}


// ---------------------------------------------------------------------------
// Batched even-odd CG over patches (cg_eop_kernel): the iteration of
// cg_eo_kernel for every system of a batch whose compact lattices 32 x 16
// patches tile (Nt a multiple of 32, Nx / 2 of 16).  The patches of the systems
// that iterate are dealt out to the blocks every round, as cg_eob_kernel
// deals out tiles, and a block takes its share one patch after another: it
// stages the patch's p, r and q of the previous iteration widened by 4 rows
// and 2 compact columns, with A_e and 1 / A_o (the next patch's copies in
// flight while it works on this one), forms p, r, w, v, u and q in shared
// memory, and writes r, p, q, v, the chi increment and the patch's tile
// partials.  w and u never leave the SM, so a round moves fewer bytes than
// cg_eob_kernel's four passes, and it has one grid barrier, the reducing
// one, where cg_eob_kernel has four.  A system's reliable update takes three
// rounds of its own (kRu: the fold; kRu2: the odd hop; kRu3: the residual and
// its partials), run site by site beside the other systems' patches, in
// float-float as in the other even-odd kernels.
// ---------------------------------------------------------------------------
constexpr int kEopPT = 32, kEopPX = 16, kEopSW = kEopPX + 4, kEopNB = kEopSW * (kEopPT + 8),
              kEopOwn = kEopPT * kEopPX;
static_assert(kEopOwn == 2 * kTile, "a patch fills two tiles' partial slots (rows 0-15, 16-31)");

// Shared memory of cg_eop_kernel: two staging sets (p, r, q, A_e, 1 / A_o on
// the widened patch; the chi increment and v on the own sites), w (then u)
// and v.
constexpr size_t kEopSet = 3 * (size_t)kEopNB * sizeof(float4) + 2 * (size_t)kEopNB * sizeof(float) +
                           2 * (size_t)kEopOwn * sizeof(float4);
static size_t eop_smem_bytes() { return 2 * kEopSet + 2 * (size_t)kEopNB * sizeof(float4); }

__device__ __forceinline__ void cp_async4(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// The reducing barrier of cg_eop_kernel: eob_reduce, with the update's first
// two rounds (kRu, kRu2: no partials) moving the system to its next round.
__device__ bool eop_reduce(const CGArgs& a, unsigned& gen, int k, double* red, int* s_active, int* s_ru,
                           const int* s_mode, const int* s_par)
{
    if (!eob_barrier(a, gen)) return false;
    for (int q = blockIdx.x; q < a.sys_count; q += gridDim.x) {
        const int j = a.sys_first + q;
        const SysDev& S = a.sys[j];
        const int mode = s_mode[q];   // this round's (the block's copy: uniform)
        double s[6];
        if (mode != kRu && mode != kRu2 && mode != kIdle) sum_partials<true>(a, S.tile0, S.ntiles, red, s);
        if (threadIdx.x == 0) {
            CGState st;
            load_state(a.st + j, st);
            CoefVals cv = {0.0, 0.0, 0.0, 1.0, 0.0, kIdle};
            cv.par = s_par[q];
            if (st.mode == kRu || st.mode == kRu2) {
                cv.mode = st.mode == kRu ? kRu2 : kRu3;
            } else if (st.mode != kIdle) {
                const int ks = k == 0 ? 0 : (st.mode == kRedo ? st.iters : st.iters + 1);
                cv = scalar_step<true>(a, ks, st.mode == kRu3, s, st, s_active, s_ru);
                cv.par = (cv.mode == kRedo ? st.iters : st.iters + 1) & 1;
            }
            st.mode = cv.mode;
            store_state(a.st + j, st);
            __threadfence();
            publish_coef(a.coef + j, cv, gen);
        }
    }
    return true;
}

__global__ void __launch_bounds__(kHaloThreads, 1) cg_eop_kernel(CGArgs a)
{
    constexpr int K = 1;
    constexpr int kSkipIm = (1 << 3) | (1 << 5);
    constexpr int SB = kEopSW, NB = kEopNB, NT = kHaloThreads;
    using W = float;
    extern __shared__ float4 hsm[];
    // staging set s at hsm + s * kEopSet bytes: p, r, q (NB each), xs, v
    // (own), then A_e, 1 / A_o (NB floats each)
    auto set_base = [&](int set) -> float4* { return reinterpret_cast<float4*>(reinterpret_cast<char*>(hsm) + set * kEopSet); };
    float4* Wp = set_base(2);    // w, later u
    float4* Vp = Wp + NB;        // v
    const int hf = threadIdx.x / kTile, ts = threadIdx.x % kTile;
    __shared__ double red[128];
    __shared__ int s_mode[kEobMaxSys], s_par[kEobMaxSys], s_nt[kEobMaxSys], s_t0[kEobMaxSys], s_pre[kEobMaxSys + 1];
    __shared__ int s_np[kEobMaxSys];   // patches of each system (two tiles each)
    __shared__ float s_fa[kEobMaxSys], s_fb[kEobMaxSys], s_fc[kEobMaxSys];
    __shared__ int s_active, s_ru;   // the scalar step's counters (unused here)
    const int nsys = a.sys_count;
    for (int q = threadIdx.x; q < nsys; q += blockDim.x) {
        const SysDev& S = a.sys[a.sys_first + q];
        s_nt[q] = S.ntiles;
        s_np[q] = S.ntiles / 2;
        s_t0[q] = S.tile0;
        s_mode[q] = kStep;
        s_par[q] = 0;
        s_fa[q] = s_fb[q] = s_fc[q] = 0.f;
    }
    __syncthreads();
    if (*(volatile int*)a.err) return;
    unsigned gen = 0;
    constexpr int kAll = (1 << kStep) | (1 << kRedo) | (1 << kRu) | (1 << kRu2) | (1 << kRu3);
    constexpr int kPass = (1 << kStep) | (1 << kRedo);
    constexpr int kInit = -1;   // round 0: p_0 and r_0 as stored

    // a patch of the current prefix: its system, index and place
    struct Patch {
        int q, lp, t0, i0, Nt, Nh, Ve;
    };
    auto patch_of = [&](int i, int& qc) -> Patch {
        const int q = (qc >= 0 && i >= s_pre[qc] && i < s_pre[qc + 1]) ? qc : eob_find(i, nsys, s_pre);
        qc = q;
        const SysDev& S = a.sys[a.sys_first + q];
        Patch P;
        P.q = q;
        P.lp = i - s_pre[q];
        P.Nt = S.Nt;
        P.Nh = S.Nx;
        P.Ve = S.V;
        const int npx = P.Nh / kEopPX;
        P.t0 = (P.lp / npx) * kEopPT;
        P.i0 = (P.lp % npx) * kEopPX;
        return P;
    };
    // compact site of buffer cell j (the widened patch, wrapped)
    auto buf_m = [](const Patch& P, int j) -> int {
        const int r = j / SB, c = j - r * SB;
        int t = P.t0 - 4 + r, i = P.i0 - 2 + c;
        t = t < 0 ? t + P.Nt : (t >= P.Nt ? t - P.Nt : t);
        i = i < 0 ? i + P.Nh : (i >= P.Nh ? i - P.Nh : i);
        return t * P.Nh + i;
    };
    auto cell_t = [](const Patch& P, int j) -> int {
        const int t = P.t0 - 4 + j / SB;
        return t < 0 ? t + P.Nt : (t >= P.Nt ? t - P.Nt : t);
    };
    auto own_j = [](int o) -> int { return (4 + o / kEopPX) * SB + 2 + o % kEopPX; };
    auto own_m = [](const Patch& P, int o) -> int { return (P.t0 + o / kEopPX) * P.Nh + P.i0 + o % kEopPX; };
    auto own_of = [](int j) -> int {
        const int r = j / SB - 4, c = j % SB - 2;
        return (r >= 0 && r < kEopPT && c >= 0 && c < kEopPX) ? r * kEopPX + c : -1;
    };

    // stage patch P (mode: its system's; kInit: round 0) into set `set`
    auto stage = [&](const Patch& P, int mode, int set) {
        const SysDev& S = a.sys[a.sys_first + P.q];
        const int cur = s_par[P.q], prv = cur ^ 1;
        const float* Rl = (mode == kRedo || mode == kInit) ? S.r32[cur] : S.r32[prv];
        const float* Pl = mode == kInit ? S.p32[cur] : S.p32[prv];
        const float* Al = prv == 0 ? S.Ap32 : S.t32;
        float4* B = set_base(set);
        float4* X = B + 3 * NB;
        float* D = reinterpret_cast<float*>(X + 2 * kEopOwn);
        for (int j = threadIdx.x; j < NB; j += NT) {
            const int m = buf_m(P, j);
            cp_async16(B + j, Pl + 4 * (size_t)m);
            cp_async16(B + NB + j, Rl + 4 * (size_t)m);
            if (mode == kStep) cp_async16(B + 2 * NB + j, Al + 4 * (size_t)m);
            cp_async4(D + j, S.diag32 + m);               // A_e (even)
            cp_async4(D + NB + j, S.diag32 + P.Ve + m);   // 1 / A_o (odd)
        }
        if (mode == kStep)   // the chi increment and v of the own sites
            for (int o = threadIdx.x; o < kEopOwn; o += NT) {
                const int m = own_m(P, o);
                cp_async16(X + o, S.xs32 + 4 * (size_t)m);
                cp_async16(X + kEopOwn + o, S.v32 + 4 * (size_t)m);
            }
        cp_async_commit();
    };

    // the iteration at patch P from staging set `set`
    auto body = [&](const Patch& P, int mode, int set, bool round0) {
        const SysDev& S = a.sys[a.sys_first + P.q];
        float4* P_st = set_base(set);
        float4* R_st = P_st + NB;
        const float4* A_st = R_st + NB;
        const float4* X_st = A_st + NB;
        const float4* Vo_st = X_st + kEopOwn;
        const float* dep = reinterpret_cast<const float*>(Vo_st + kEopOwn);
        const float* dip = dep + NB;
        const int cur = s_par[P.q];
        const W rw = (W)S.r;
        const W ar = s_fa[P.q], beta = s_fb[P.q], cre = s_fc[P.q];
        // A1: p (and r, the chi increment on the own sites) on the buffer
        for (int j = threadIdx.x; j < NB; j += NT) {
            const int o = own_of(j);
            const Site<W, K> po = ld_sm(P_st, j);
            Site<W, K> p;
            if (mode == kStep) {
                Site<W, K> r = ld_sm(R_st, j);
                site_axpy<W, K>(r, -ar, W(0), ld_sm(A_st, j));
#pragma unroll
                for (int i = 0; i < 4; ++i) p.v[i] = fma(beta, po.v[i], r.v[i]);
                if (o >= 0) {
                    const int m = own_m(P, o);
                    Site<W, K> x = ld_sm(X_st, o);
                    site_axpy<W, K>(x, ar, W(0), ld_sm(Vo_st, o));
                    YK_ST(W, K, S.xs32, m, x);
                    YK_ST(W, K, S.r32[cur], m, r);
                    YK_ST(W, K, S.p32[cur], m, p);
                    st_sm(R_st, j, r);
                }
            } else if (mode == kRedo) {
                p = p_next<W, K>(ld_sm(R_st, j), po, beta, cre, W(0));
                if (o >= 0) YK_ST(W, K, S.p32[cur], own_m(P, o), p);
            } else {
                p = po;
            }
            st_sm(P_st, j, p);
        }
        __syncthreads();
        Site<W, K> zero;
#pragma unroll
        for (int i = 0; i < 4; ++i) zero.v[i] = W(0);
        // w = -A_o^-1 H_oe p (odd) on [SB, NB - SB)
        for (int j = SB + threadIdx.x; j < NB - SB; j += NT) {
            const int t = cell_t(P, j), b = (t + 1) & 1;
            const W sp = (t + 1 == P.Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
            Site<W, K> h = eo_sm<false>(P_st, j, SB, b, b - 1, zero, W(0), rw, sp, sm);
            const W sc = -dip[j];
#pragma unroll
            for (int i = 0; i < 4; ++i) h.v[i] *= sc;
            st_sm(Wp, j, h);
        }
        __syncthreads();
        // v = A_e p + H_eo w (even) on [2SB, NB - 2SB); the own sites' to v32
        for (int j = 2 * SB + threadIdx.x; j < NB - 2 * SB; j += NT) {
            const int t = cell_t(P, j), b = t & 1;
            const W sp = (t + 1 == P.Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
            const Site<W, K> v = eo_sm<false>(Wp, j, SB, b, b - 1, ld_sm(P_st, j), dep[j], rw, sp, sm);
            st_sm(Vp, j, v);
            const int o = own_of(j);
            if (o >= 0) YK_ST(W, K, S.v32, own_m(P, o), v);
        }
        __syncthreads();
        // u = -A_o^-1 H^dag_oe v (odd) on [3SB, NB - 3SB)
        for (int j = 3 * SB + threadIdx.x; j < NB - 3 * SB; j += NT) {
            const int t = cell_t(P, j), b = (t + 1) & 1;
            const W sp = (t + 1 == P.Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
            Site<W, K> h = eo_sm<true>(Vp, j, SB, b, b - 1, zero, W(0), rw, sp, sm);
            const W sc = -dip[j];
#pragma unroll
            for (int i = 0; i < 4; ++i) h.v[i] *= sc;
            st_sm(Wp, j, h);
        }
        __syncthreads();
        // q = A_e v + H^dag_eo u on the own sites and the patch's partials
        // (round 0 adds |eta|^2 of the compact index's two full sites)
        FF f[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) f[i] = FF{0.f, 0.f};
        const bool on = true;   // rows 0-15 of the patch in threads 0-255, rows 16-31 in 256-511
        {
            const int o = hf * kTile + ts;
            const int j = own_j(o), m = own_m(P, o);
            const int t = cell_t(P, j), b = t & 1;
            const W sp = (t + 1 == P.Nt) ? W(-1) : W(1), sm = (t == 0) ? W(-1) : W(1);
            const Site<W, K> v = ld_sm(Vp, j);
            const Site<W, K> qv = eo_sm<true>(Wp, j, SB, b, b - 1, v, dep[j], rw, sp, sm);
            YK_ST(W, K, cur == 0 ? S.Ap32 : S.t32, m, qv);
            const Site<W, K> r = ld_sm(R_st, j);
            W rq, dummy;
            site_dot<W, K>(r, qv, rq, dummy);
            f[0] = FF{site_norm2<W, K>(r), 0.f};
            f[1] = FF{site_norm2<W, K>(qv), 0.f};
            f[2] = FF{site_norm2<W, K>(v), 0.f};
            f[4] = FF{rq, 0.f};
            if (round0) {
                const SysDev& SF = a.sys_full[a.sys_first + P.q];
                const Site<double, K> e0 = load_site<double, K>(SF.b, 2 * m);
                const Site<double, K> e1 = load_site<double, K>(SF.b, 2 * m + 1);
                f[5] = ff_of(site_norm2<double, K>(e0) + site_norm2<double, K>(e1));
            }
        }
        const int tile = s_t0[P.q] + 2 * P.lp + hf;
        if (round0)
            put_partial_ff<(1 << 3), true>(a, tile, on, f, red);
        else
            put_partial_ff<kSkipIm, false>(a, tile, on, f, red);
    };

    // this block's share of the patches of the systems in the pass modes
    // (round 0: of every system), the next patch's staging in flight
    auto pass = [&](bool init) {
        eob_scan(nsys, s_mode, s_np, init ? kAll : kPass, s_pre);
        int lo, hi;
        eob_share(s_pre[nsys], &lo, &hi);
        int qc = -1, qn = -1;
        if (lo < hi) {
            const Patch P0 = patch_of(lo, qn);
            stage(P0, init ? kInit : s_mode[P0.q], 0);
        }
        for (int i = lo; i < hi; ++i) {
            const int set = (i - lo) & 1;
            const Patch P = patch_of(i, qc);
            if (i + 1 < hi) {
                const Patch Pn = patch_of(i + 1, qn);
                stage(Pn, init ? kInit : s_mode[Pn.q], set ^ 1);
                cp_async_wait_one();
            } else {
                cp_async_wait_all();
            }
            __syncthreads();
            body(P, init ? kInit : s_mode[P.q], set, init);
        }
    };

    // Runs f(S, q, m, tile, tile_on, on) for every site of this block's share
    // of the tiles of the systems in `mask`, two tiles at a time.
    auto for_sites = [&](int mask, auto&& f) {
        eob_scan(nsys, s_mode, s_nt, mask, s_pre);
        int lo, hi;
        eob_share(s_pre[nsys], &lo, &hi);
        int qc = -1;
        for (int base = lo; base < hi; base += 2) {
            const int i = base + hf;
            const bool tile_on = i < hi;
            const int ii = tile_on ? i : lo;
            const int q = (qc >= 0 && ii >= s_pre[qc] && ii < s_pre[qc + 1]) ? qc : eob_find(ii, nsys, s_pre);
            qc = q;
            const int lt = ii - s_pre[q];
            const SysDev& S = a.sys[a.sys_first + q];
            const int m = lt * kTile + ts;
            f(S, q, m, s_t0[q] + lt, tile_on, tile_on && m < S.V);
        }
    };
    struct Geo {
        int b, du, dd;
        float sp, sm;
    };
    auto geo = [](const SysDev& S, int m, int c) {
        Geo g;
        const int Nh = S.Nx;
        const int t = m / Nh, i = m - t * Nh;
        g.b = (t + c) & 1;
        g.du = g.b ? ((i == Nh - 1) ? 1 - Nh : 1) : 0;
        g.dd = g.b ? 0 : ((i == 0) ? Nh - 1 : -1);
        g.sp = (t + 1 == S.Nt) ? -1.f : 1.f;
        g.sm = (t == 0) ? -1.f : 1.f;
        return g;
    };

    // ---------------- round 0: eta of both classes (b, full layout), A_e and
    // 1 / A_o, -A_o^-1 eta_o (t64), chi_e = xs = v = 0; then rhs_e, r_0 = p_0
    for_sites(kAll, [&](const SysDev& S, int q, int m, int, bool, bool on) {
        if (!on) return;
        const SysDev& SF = a.sys_full[a.sys_first + q];
        const int Ve = S.V;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const Geo g = geo(S, m, c);
            const int n = 2 * m + g.b;
            const Site<double, K> bv =
                SF.gen_eta ? eta_of_step<K>(SF, n, a.eta_kind) : load_site<double, K>(SF.b, n);
            if (SF.gen_eta) store_site<double, K>(SF.b, n, bv);
            const double d = 2.0 * S.r + S.m0 + S.g * SF.sigma[n];
            if (c == 0) {
                S.diag32[m] = (float)d;
            } else {
                const FF inv = ff_rcp(ff_of(d));
                st_ff1(S.dinv, m, inv);
                S.diag32[Ve + m] = inv.hi;
                const SiteFF e = ff_site_of(bv, SF.gen_eta != 0);
                SiteFF h;
#pragma unroll
                for (int e2 = 0; e2 < 4; ++e2) h.v[e2] = ff_mul(FF{-inv.hi, -inv.lo}, e.v[e2]);
                st_ff(S.t64, m, h);
            }
        }
        Site<double, K> z;
        Site<W, K> zw;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            z.v[e] = 0.0;
            zw.v[e] = W(0);
        }
        store_site<double, K>(S.x, m, z);
        YK_ST(W, K, S.xs32, m, zw);
        YK_ST(W, K, S.v32, m, zw);
    });
    if (!eob_barrier(a, gen)) return;
    for_sites(kAll, [&](const SysDev& S, int q, int m, int, bool, bool on) {
        if (!on) return;
        const SysDev& SF = a.sys_full[a.sys_first + q];
        const Geo g = geo(S, m, 0);
        const SiteFF e = ff_site_of(load_site<double, K>(SF.b, 2 * m + g.b), SF.gen_eta != 0);
        const SiteFF rh =
            eo_ff<true, 1>(S.t64, m, S.V, S.Nx, g.du, g.dd, e, FF{1.f, 0.f}, hop_of_r(S.r), g.sp, g.sm);
        st_ff(S.x + 4 * (size_t)S.V, m, rh);
        Site<W, K> rw;
#pragma unroll
        for (int e2 = 0; e2 < 4; ++e2) rw.v[e2] = rh.v[e2].hi;
        YK_ST(W, K, S.r32[0], m, rw);
        YK_ST(W, K, S.p32[0], m, rw);
    });
    if (!eob_barrier(a, gen)) return;
    pass(true);
    if (!eop_reduce(a, gen, 0, red, &s_active, &s_ru, s_mode, s_par)) return;

    // every round: the patches of the systems that iterate, and the update
    // rounds of the others (each system keeps its own iteration index)
    int k = 1;
    const int kmax = 4 * a.max_iter + 4;
    while (k <= kmax) {
        int nact = 0;
        if (!eob_load_coefs(a, gen, nsys, s_mode, s_par, s_fa, s_fb, s_fc, &nact)) return;
        if (nact == 0) break;
        pass(false);
        // kRu: fold chi_e += xs + alpha v (float-float); xs = 0
        for_sites(1 << kRu, [&](const SysDev& S, int q, int m, int, bool, bool on) {
            if (!on) return;
            SiteFF xv = ld_ff(S.x, m);
            const Site<W, K> xs = YK_LD(W, K, S.xs32, m);
            const Site<W, K> vv = YK_LD(W, K, S.v32, m);
            const float al = s_fa[q];
            Site<W, K> zw;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float pr = __fmul_rn(al, vv.v[e]);   // alpha v exactly: (pr, its FMA error)
                xv.v[e] = ff_add(xv.v[e], FF{xs.v[e], 0.f});
                xv.v[e] = ff_add(xv.v[e], FF{pr, __fmaf_rn(al, vv.v[e], -pr)});
                zw.v[e] = W(0);
            }
            st_ff(S.x, m, xv);
            YK_ST(W, K, S.xs32, m, zw);
        });
        // kRu2: u = -A_o^-1 H^dag_oe chi_e (odd, t64)
        for_sites(1 << kRu2, [&](const SysDev& S, int, int m, int, bool, bool on) {
            if (!on) return;
            const Geo g = geo(S, m, 1);
            SiteFF zero;
#pragma unroll
            for (int e = 0; e < 4; ++e) zero.v[e] = FF{0.f, 0.f};
            SiteFF h = eo_ff<true, 0>(S.x, m, S.V, S.Nx, g.du, g.dd, zero, FF{0.f, 0.f}, hop_of_r(S.r), g.sp, g.sm);
            const FF sc = ld_ff1(S.dinv, m);
#pragma unroll
            for (int e = 0; e < 4; ++e) h.v[e] = ff_mul(FF{-sc.hi, -sc.lo}, h.v[e]);
            st_ff(S.t64, m, h);
        });
        // kRu3: r = rhs_e - (A_e chi_e + H^dag_eo u); |r|^2, <r, p_{k-1}>
        for_sites(1 << kRu3, [&](const SysDev& S, int q, int m, int tile, bool tile_on, bool on) {
            const int cur = s_par[q], prv = cur ^ 1;
            float v0 = 0.f, v2 = 0.f;
            if (on) {
                const SysDev& SF = a.sys_full[a.sys_first + q];
                const Geo g = geo(S, m, 0);
                const FF de = ff_of(2.0 * S.r + S.m0 + S.g * SF.sigma[2 * m + g.b]);
                const SiteFF sx =
                    eo_ff<true, 2>(S.t64, m, S.V, S.Nx, g.du, g.dd, ld_ff(S.x, m), de, hop_of_r(S.r), g.sp, g.sm);
                const SiteFF bv = ld_ff(S.x + 4 * (size_t)S.V, m);
                const Site<W, K> pw = YK_LD(W, K, S.p32[prv], m);
                Site<W, K> rw;
#pragma unroll
                for (int e = 0; e < 4; ++e) rw.v[e] = ff_sub(bv.v[e], sx.v[e]).hi;
                YK_ST(W, K, S.r32[cur], m, rw);
                W dummy;
                v0 = site_norm2<W, K>(rw);
                site_dot<W, K>(rw, pw, v2, dummy);
            }
            FF f[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) f[i] = FF{0.f, 0.f};
            f[0] = FF{v0, 0.f};
            f[2] = FF{v2, 0.f};
            put_partial_ff<(1 << 1) | (1 << 4) | (1 << 5) | kSkipIm, true>(a, tile, tile_on, f, red);
        });
        if (!eop_reduce(a, gen, k, red, &s_active, &s_ru, s_mode, s_par)) return;
        ++k;
    }
    // chi of both classes in the full layout (t64) for the force
    if (!eob_barrier(a, gen)) return;
    for_sites(kAll | (1 << kIdle), [&](const SysDev& S, int q, int m, int, bool, bool on) {
        if (!on) return;
        const SysDev& SF = a.sys_full[a.sys_first + q];
        Geo g = geo(S, m, 0);
        const SiteFF xe = ld_ff(S.x, m);
        Site<double, K> ce;
#pragma unroll
        for (int e = 0; e < 4; ++e) ce.v[e] = dbl_of(xe.v[e]);
        store_site<double, K>(SF.t64, 2 * m + g.b, ce);
        g = geo(S, m, 1);
        SiteFF zero;
#pragma unroll
        for (int e = 0; e < 4; ++e) zero.v[e] = FF{0.f, 0.f};
        const SiteFF h = eo_ff<true, 0>(S.x, m, S.V, S.Nx, g.du, g.dd, zero, FF{0.f, 0.f}, hop_of_r(S.r), g.sp, g.sm);
        const int n = 2 * m + g.b;
        const SiteFF e = ff_site_of(load_site<double, K>(SF.b, n), SF.gen_eta != 0);
        const FF inv = ld_ff1(S.dinv, m);
        Site<double, K> co;
#pragma unroll
        for (int e2 = 0; e2 < 4; ++e2) co.v[e2] = dbl_of(ff_mul(ff_sub(e.v[e2], h.v[e2]), inv));
        store_site<double, K>(SF.t64, n, co);
    });
    if (blockIdx.x == 0)
        for (int q = threadIdx.x; q < nsys; q += blockDim.x) a.st[a.sys_first + q].chi_ready = 1;
}


// Shared memory of cg_eo_kernel for `own` compact sites per block and a
// staged buffer of nb cells: p, r, q, w (then u) and v on the buffer, the chi
// increment and v on the own sites, A_e and 1 / A_o in FP32 on the buffer.
static size_t eo_smem_bytes(int own, int nb)
{
    return (5 * (size_t)nb + 2 * (size_t)own) * sizeof(float4) + 2 * (size_t)nb * sizeof(float);
}

// Failure detection without a fault: block 0 waits through nsync on block
// 1's neighbour flag, which block 1 never sets (it returns at once); the
// bounded wait gives up, records YK_ETIMEOUT in *err and the kernel returns.
__device__ unsigned g_probe_flags[2 * kFlagStride];
__device__ int g_probe_err;

__global__ void wait_timeout_probe_kernel(CGArgs a)
{
    if (blockIdx.x == 1) return;
    __shared__ Deps d;
    if (threadIdx.x == 0) {
        d.n = 1;
        d.all = 0;
        d.b[0] = 1;
    }
    __syncthreads();
    nsync(a, 1u, d);
}

int wait_timeout_probe(cudaStream_t stream, int* status)
{
    void* flags = nullptr;
    void* err = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&flags, g_probe_flags);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&err, g_probe_err);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, sizeof(g_probe_flags), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), stream);
    CGArgs a = {};
    a.flags = static_cast<unsigned*>(flags);
    a.err = static_cast<int*>(err);
    if (e == cudaSuccess) {
        wait_timeout_probe_kernel<<<2, 32, 0, stream>>>(a);
        e = cudaGetLastError();
    }
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return -1;
    *status = h;
    return 0;
}

// Resets the barrier, flags, counters and per-system state before a solve.
__global__ void cg_prepare_kernel(CGArgs a)
{
    for (int i = a.sys_first + threadIdx.x; i < a.sys_first + a.sys_count; i += blockDim.x) {
        CGState& s = a.st[i];
        s.rr = s.rr0 = s.rr_prev = s.stop2 = s.rmax2 = 0.0;
        s.active = 1;
        s.iters = 0;
        s.converged = 0;
        s.status = 0;
        s.n_ru = 0;
        s.chi_ready = 0;
        s.mode = kStep;
        // generation 0: the coefficients of round 0 (never polled)
        for (int q = 0; q < 12; ++q) a.coef[i].w[q] = 0ull;
    }
    for (int b = threadIdx.x; b < a.grid; b += blockDim.x) a.flags[(size_t)b * kFlagStride] = 0u;
    if (threadIdx.x == 0) {
        *a.n_active = a.sys_count;
        *a.any_ru = 0;
        a.bar->arrive = 0u;
        a.bar->gword = 0ull;
        for (int b = 0; b < 3; ++b) {
            for (int c = 0; c < 4; ++c) a.bar->fsum[b][c][0] = 0;
            a.bar->fsum[b][0][kFixOverflowWord] = 0;
        }
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

// Largest grid of the CG kernel: the co-resident maximum, capped by the
// environment variable YK_CG_MAX_GRID when it is set (a tuning knob: fewer
// blocks own more tiles each).
template <int K, bool MIXED>
static int max_grid_t()
{
    static int maxg = -1;
    if (maxg < 0) {
        maxg = max_coresident((const void*)cg_kernel<K, MIXED>, cg_threads<K>());
        if (const char* e = getenv("YK_CG_MAX_GRID")) {
            const int cap = atoi(e);
            if (cap > 0 && cap < maxg) maxg = cap;
        }
    }
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

constexpr size_t kHaloMaxSmem = 216 * 1024;

// Whether cg_halo_kernel takes a single-system solve on an Nt x Nx lattice
// whose blocks own tpb tiles each: at most 8 tiles per block, halo work at
// most twice the own work (4 Nx <= 2 * own), the widened range within the
// lattice, and its shared memory within kHaloMaxSmem.  Callers that do not
// give the lattice (Nt = Nx = 0) get cg_kernel.
static bool halo_takes(int Nt, int Nx, int tpb, size_t* smem)
{
    if (Nt < 1 || Nx < 1 || tpb < 1 || tpb > 8) return false;
    const long long own = (long long)tpb * kTile, V = (long long)Nt * Nx;
    if (4LL * Nx > 2 * own || own + 4LL * Nx > V) return false;
    *smem = halo_smem_bytes((int)own, Nx);
    return *smem <= kHaloMaxSmem;
}

// Whether cg_eo_kernel takes the single-system solve of A = D^dag D on an
// Nt x Nx lattice (both even) whose blocks own tpb compact tiles each: at most
// 8 tiles per block, the widened compact range within the compact lattice,
// and its shared memory within kHaloMaxSmem.
static bool eo_takes(int Nt, int Nx, int tpb, size_t* smem)
{
    if (Nt < 2 || Nx < 4 || (Nt & 1) || (Nx & 1) || tpb < 1 || tpb > 8) return false;
    const long long own = (long long)tpb * kTile, Nh = Nx / 2, Ve = (long long)Nt * Nh;
    if (own + 8 * Nh > Ve) return false;
    *smem = eo_smem_bytes((int)own, (int)(own + 8 * Nh));
    return *smem <= kHaloMaxSmem;
}

// Whether cg_eo_kernel<PX> takes it: kPT x PX patches tile the compact
// lattice, one block per patch.
template <int PX>
static bool eo_patch_takes(int Nt, int Nx, int* patches, size_t* smem)
{
    constexpr int PT = eo_pt(PX);
    if (Nt < PT || Nx < 2 * PX || (Nt % PT) || (Nx % (2 * PX))) return false;
    *patches = (Nt / PT) * (Nx / (2 * PX));
    *smem = eo_smem_bytes(PT * PX, eo_sw(PX) * eo_sr(PX));
    return *smem <= kHaloMaxSmem;
}

static int eo_max_grid()
{
    static int maxg = -1;
    if (maxg < 0) {
        cudaFuncSetAttribute((const void*)cg_eo_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kHaloMaxSmem);
        int dev = 0, nsm = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)cg_eo_kernel<0>, kHaloThreads,
                                                      kHaloMaxSmem);
        maxg = per * nsm;
    }
    return maxg;
}

template <int PX>
static int eo_patch_max_grid()
{
    static int maxg = -1;
    if (maxg < 0) {
        const int smem = (int)eo_smem_bytes(eo_pt(PX) * PX, eo_sw(PX) * eo_sr(PX));
        cudaFuncSetAttribute((const void*)cg_eo_kernel<PX>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int dev = 0, nsm = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)cg_eo_kernel<PX>, eo_threads(PX), smem);
        maxg = per * nsm;
        if (maxg > kMaxGrid) maxg = kMaxGrid;
    }
    return maxg;
}

static int eob_max_grid()
{
    static int maxg = -1;
    if (maxg < 0) {
        int dev = 0, nsm = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)cg_eob_kernel, kHaloThreads, 0);
        maxg = per * nsm;
        if (maxg > kMaxGrid) maxg = kMaxGrid;
    }
    return maxg;
}

static int eop_max_grid()
{
    static int maxg = -1;
    if (maxg < 0) {
        const int smem = (int)eop_smem_bytes();
        cudaFuncSetAttribute((const void*)cg_eop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int dev = 0, nsm = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)cg_eop_kernel, kHaloThreads, smem) !=
            cudaSuccess) {
            cudaGetLastError();
            per = 0;
        }
        maxg = per * nsm;
        if (maxg > kMaxGrid) maxg = kMaxGrid;
    }
    return maxg;
}

static int halo_max_grid()
{
    static int maxg = -1;
    if (maxg < 0) {
        cudaFuncSetAttribute((const void*)cg_halo_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kHaloMaxSmem);
        int dev = 0, nsm = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)cg_halo_kernel, kHaloThreads, kHaloMaxSmem);
        maxg = per * nsm;
    }
    return maxg;
}

int cg_eob_max_grid() { return eob_max_grid(); }

void cg_halo_init()
{
    halo_max_grid();
    eo_max_grid();
    eo_patch_max_grid<16>();
    eo_patch_max_grid<8>();
    eo_patch_max_grid<32>();
    eob_max_grid();
    eop_max_grid();
}

static int capped(int maxg, int cap) { return cap > 0 && cap < maxg ? cap : maxg; }

static bool eo_single_variant(const CGArgs& a, int* px, int* grid, int* tpb, size_t* smem);

// The grid launch_cg would use for `a` (the even-odd kernels' when the caller
// gave the compact views, as launch_cg_t picks them).
int cg_predict_grid(const CGArgs& a, bool mixed)
{
    if (mixed && a.sys_eo && a.eo_tiles && a.mtype == YK_DAGGER && a.balance == nullptr &&
        a.sys_count <= kEobMaxSys) {
        int px = 0, eg = 0, etpb = 1;
        size_t es = 0;
        if (eo_single_variant(a, &px, &eg, &etpb, &es)) return eg;
        const int nt = a.eo_tile_end - a.eo_tile_begin;
        const char* pe = getenv("YK_CG_EOP");
        if (a.eo_patches && !(pe && pe[0] == '0') && eop_max_grid() > 0) return std::min(capped(eop_max_grid(), a.grid_cap), std::max(nt, 1));
        return std::min(capped(eob_max_grid(), a.grid_cap), std::max((nt + 1) / 2, 1));
    }
    int tpb = 1;
    return cg_grid_for(a.tile_end - a.tile_begin,
                       capped(mixed ? max_grid_t<1, true>() : max_grid_t<1, false>(), a.grid_cap), &tpb);
}

// The single-system even-odd kernel launch_cg takes for `a` (mixed, K = 1):
// its patch width (16 or 8; 0 whole rows) in *px, *grid blocks of *tpb tiles
// (patches: one), false when none takes it.  YK_CG_EO_PATCH=0, 8 or 16 fixes
// the form.
static bool eo_single_variant(const CGArgs& a, int* px, int* grid, int* tpb, size_t* smem)
{
    if (!(a.sys_eo && a.eo_tiles && a.mtype == YK_DAGGER && a.balance == nullptr && a.sys_count == 1)) return false;
    const char* pe = getenv("YK_CG_EO_PATCH");
    const int want = pe ? atoi(pe) : -1;
    // partial slots: one per patch, within the system's tiles (2 per compact tile)
    const int slots = 2 * (a.eo_tile_end - a.eo_tile_begin);
    int np = 0;
    if ((want == -1 || want == 16) && eo_patch_takes<16>(a.solo_nt, a.solo_nx, &np, smem) &&
        np <= eo_patch_max_grid<16>() && np <= slots) {
        *px = 16;
        *grid = np;
        *tpb = 1;
        return true;
    }
    if ((want == -1 || want == 8) && eo_patch_takes<8>(a.solo_nt, a.solo_nx, &np, smem) &&
        np <= eo_patch_max_grid<8>() && np <= slots) {
        *px = 8;
        *grid = np;
        *tpb = 1;
        return true;
    }
    // 32 x 32 patches: four tiles' partial slots each
    if ((want == -1 || want == 32) && eo_patch_takes<32>(a.solo_nt, a.solo_nx, &np, smem) &&
        np <= eo_patch_max_grid<32>() && 4 * np <= slots) {
        *px = 32;
        *grid = np;
        *tpb = 4;
        return true;
    }
    const int eg = cg_grid_for(a.eo_tile_end - a.eo_tile_begin, capped(eo_max_grid(), a.grid_cap), tpb);
    if (eg <= kMaxGrid && eo_takes(a.solo_nt, a.solo_nx, *tpb, smem)) {
        *px = 0;
        *grid = eg;
        return true;
    }
    return false;
}

template <int K, bool MIXED>
static cudaError_t launch_cg_t(const CGArgs& a0, cudaStream_t stream, int* grid_out, int* kernel_out)
{
    CGArgs a = a0;
    const int maxg = capped(max_grid_t<K, MIXED>(), a.grid_cap);
    const int nt = a.tile_end - a.tile_begin;
    int tpb = 1;
    const int grid = cg_grid_for(nt, maxg, &tpb);
    if (tpb > kMaxTilesPerBlock || grid > maxg || grid > kMaxGrid) return cudaErrorInvalidConfiguration;
    a.tiles_per_block = tpb;
    a.grid = grid;
    if (grid_out) *grid_out = grid;
    const void* fn = (const void*)cg_kernel<K, MIXED>;
    unsigned threads = cg_threads<K>();
    size_t smem = 0;
    if constexpr (K == 1 && MIXED) {
        // the even-odd solve of the step's chi (a single system of A = D^dag D
        // on an even lattice, when the caller gave the compact views)
        if (a.sys_eo && a.eo_tiles && a.mtype == YK_DAGGER && a.balance == nullptr && a.sys_count <= kEobMaxSys) {
            CGArgs e = a;
            e.sys_full = a.sys;
            e.sys = a.sys_eo;
            e.tiles = a.eo_tiles;
            e.tile_begin = a.eo_tile_begin;
            e.tile_end = a.eo_tile_end;
            e.eo = 1;
            // patches first (less halo work per block), then rows of the lattice
            int px = 0, eg = 0, etpb = 1;
            size_t es = 0;
            if (eo_single_variant(a, &px, &eg, &etpb, &es)) {
                if (px > 0) e.tile_end = e.tile_begin + eg * etpb;   // the patches' partial slots
                e.tiles_per_block = etpb;
                e.grid = eg;
                if (grid_out) *grid_out = eg;
                if (kernel_out) *kernel_out = 3;
                cg_prepare_kernel<<<1, 256, 0, stream>>>(e);
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(eg);
                cfg.blockDim = dim3(eo_threads(px));
                cfg.dynamicSmemBytes = es;
                cfg.stream = stream;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeCooperative;
                attr[0].val.cooperative = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                void* args[] = {&e};
                const void* fn = px == 16 ? (const void*)cg_eo_kernel<16>
                               : px == 8  ? (const void*)cg_eo_kernel<8>
                               : px == 32 ? (const void*)cg_eo_kernel<32>
                                          : (const void*)cg_eo_kernel<0>;
                return cudaLaunchKernelExC(&cfg, fn, args);
            }
            // lattices that 16 x 16 patches tile: the batched patch kernel
            // (YK_CG_EOP=0: the four-pass kernel below), one block per SM
            const char* pe = getenv("YK_CG_EOP");
            if (a.eo_patches && !(pe && pe[0] == '0') && eop_max_grid() > 0) {
                int pg = capped(eop_max_grid(), a.grid_cap);
                const int want = a.eo_tile_end - a.eo_tile_begin;   // patches (one tile each)
                if (pg > want) pg = want;
                if (pg < 1) pg = 1;
                e.grid = pg;
                e.tiles_per_block = 1;
                if (grid_out) *grid_out = pg;
                if (kernel_out) *kernel_out = 5;
                cg_prepare_kernel<<<1, 256, 0, stream>>>(e);
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(pg);
                cfg.blockDim = dim3(kHaloThreads);
                cfg.dynamicSmemBytes = eop_smem_bytes();
                cfg.stream = stream;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeCooperative;
                attr[0].val.cooperative = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                void* args[] = {&e};
                return cudaLaunchKernelExC(&cfg, (const void*)cg_eop_kernel, args);
            }
            // the batched even-odd kernel: work dealt out per pass, so the
            // grid does not follow the tiles (at most one block per two tiles)
            int bg = capped(eob_max_grid(), a.grid_cap);
            const int want = (a.eo_tile_end - a.eo_tile_begin + 1) / 2;
            if (bg > want) bg = want;
            if (bg < 1) bg = 1;
            e.grid = bg;
            e.tiles_per_block = 1;
            if (grid_out) *grid_out = bg;
            if (kernel_out) *kernel_out = 4;
            cg_prepare_kernel<<<1, 256, 0, stream>>>(e);
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(bg);
            cfg.blockDim = dim3(kHaloThreads);
            cfg.dynamicSmemBytes = 0;
            cfg.stream = stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeCooperative;
            attr[0].val.cooperative = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            void* args[] = {&e};
            return cudaLaunchKernelExC(&cfg, (const void*)cg_eob_kernel, args);
        }
        // the same tile partition as cg_kernel<1, true>, so the same partials
        size_t hs = 0;
        if (a.sys_count == 1 && halo_takes(a.solo_nt, a.solo_nx, tpb, &hs) && grid <= halo_max_grid()) {
            fn = (const void*)cg_halo_kernel;
            threads = kHaloThreads;
            smem = hs;
        }
    }
    if (kernel_out) *kernel_out = (fn == (const void*)cg_halo_kernel) ? 1 : 0;
    cg_prepare_kernel<<<1, 256, 0, stream>>>(a);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {&a};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

// Work-balanced block ranges for the next solve of the same systems: every
// tile of system s weighs (iterations of s in the solve just finished + 16),
// and blocks take contiguous table ranges of about equal weight, at most
// kMaxTilesPerBlock tiles and kMaxSysPerBlock systems each (greedy over the
// systems' tile runs, one thread).  A partition that cannot meet the caps is
// not published ([0] = 0: the next launch uses the uniform ranges).  The
// iterates of every system do not depend on the ranges (tile partials are
// summed in a fixed order), only the time does: without balancing, the blocks
// that own the slowest systems' tiles run the last iterations alone.
__global__ void cg_balance_kernel(CGArgs a, int grid, int* out)
{
    if (threadIdx.x != 0) return;
    constexpr int kOverhead = 16;
    double W = 0.0;
    for (int s = a.sys_first; s < a.sys_first + a.sys_count; ++s)
        W += (double)a.sys[s].ntiles * (double)(a.st[s].iters + kOverhead);
    const double target = W / grid;
    int b = 0, ntb = 0, nsb = 0, last_sys = -1;
    double acc = 0.0;
    bool ok = true;
    out[1] = a.tile_begin;
    int t = a.tile_begin;
    while (t < a.tile_end && ok) {
        const int s = a.tiles[t].x;
        const SysDev& S = a.sys[s];
        const int run_end = min(a.tile_end, S.tile0 + S.ntiles);   // the system's tiles are contiguous
        const double w = (double)(a.st[s].iters + kOverhead);
        int rem = run_end - t;
        while (rem > 0) {
            if (b < grid - 1 && (ntb == kMaxTilesPerBlock || (nsb == kMaxSysPerBlock && s != last_sys))) {
                out[1 + ++b] = t;
                acc = 0.0;
                ntb = nsb = 0;
                last_sys = -1;
            }
            int take = min(rem, kMaxTilesPerBlock - ntb);
            if (b < grid - 1) {
                const double need = ceil((target - acc) / w);
                take = min(take, need < 1.0 ? 1 : (int)min(need, 1e9));
            }
            if (take < 1) {   // the last block is full
                ok = false;
                break;
            }
            if (s != last_sys) {
                ++nsb;
                last_sys = s;
            }
            acc += take * w;
            ntb += take;
            t += take;
            rem -= take;
            if (b < grid - 1 && acc >= target) {
                out[1 + ++b] = t;
                acc = 0.0;
                ntb = nsb = 0;
                last_sys = -1;
            }
        }
        if (nsb > kMaxSysPerBlock || ntb > kMaxTilesPerBlock) ok = false;
    }
    for (int q = b + 1; q <= grid; ++q) out[1 + q] = a.tile_end;   // trailing empty ranges, and the end
    out[0] = ok ? grid : 0;
}

cudaError_t launch_cg_balance(const CGArgs& a, int grid, int* out, cudaStream_t stream)
{
    if (grid < 1 || grid > kMaxGrid || a.sys_count < 2) return cudaSuccess;
    cg_balance_kernel<<<1, 32, 0, stream>>>(a, grid, out);
    return cudaGetLastError();
}

cudaError_t launch_cg(const CGArgs& a, int K, bool mixed, cudaStream_t stream, int* grid_out, int* kernel_out)
{
    if (K == 1)
        return mixed ? launch_cg_t<1, true>(a, stream, grid_out, kernel_out)
                     : launch_cg_t<1, false>(a, stream, grid_out, kernel_out);
    return mixed ? launch_cg_t<2, true>(a, stream, grid_out, kernel_out)
                 : launch_cg_t<2, false>(a, stream, grid_out, kernel_out);
}

}  // namespace yk
