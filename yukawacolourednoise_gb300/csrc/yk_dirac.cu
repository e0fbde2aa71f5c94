// yk_dirac.cu -- stand-alone Wilson-Dirac apply (the replacement for
// DiracOP<double>::applyD, code/src/Dirac.cu:23-70 and :144-190).
//
// One pass (dirac_kernel): each thread produces one site from its own entries
// and its four neighbours (coalesced 16-byte vector loads, neighbour reuse
// through L1); rows of a multiple of 32 sites take the column-strip form
// (dirac_strip_kernel), which reads each site about once,
// the antiperiodic time signs and neighbour indices are computed instead of
// read from IUP/IDN tables, and the output is written once (the reference
// zeroes `out`, adds the diagonal and adds the hops in three grid-synced
// passes).  Complex (K = 2) applies add the pion term g i gamma5 tau.pi when
// the chain carries pions.
#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

template <typename R, int K, bool DAG>
__global__ void __launch_bounds__(kBlock) dirac_kernel(const R* __restrict__ in, R* __restrict__ out,
                                                       const double* __restrict__ sigma,
                                                       const double* __restrict__ pi, int Nt, int Nx,
                                                       double m0, double g, double r)
{
    const int V = Nt * Nx;
    const R rr = (R)r;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < V; n += gridDim.x * blockDim.x) {
        const Nbr nb = neighbours(n, Nt, Nx);
        const Site<R, K> c = load_site<R, K>(in, n);
        const Site<R, K> tu = load_site<R, K>(in, nb.tu);
        const Site<R, K> td = load_site<R, K>(in, nb.td);
        const Site<R, K> xu = load_site<R, K>(in, nb.xu);
        const Site<R, K> xd = load_site<R, K>(in, nb.xd);
        const R diag = (R)(2.0 * r + m0 + g * sigma[n]);
        Site<R, K> o = dirac_combine<R, K, DAG>(c, tu, td, xu, xd, diag, rr, (R)nb.sp, (R)nb.sm);
        pion_term<R, K>(o, c, pi, n, V, g, DAG);
        store_site<R, K>(out, n, o);
    }
}

// Column-strip form for Nx a multiple of 32: a block of W = 32 w threads owns
// W consecutive columns of one row band of up to kStripRows rows; each thread
// walks its column in t with the sites of rows t - 1, t, t + 1 in registers
// (one new site loaded per output site), and takes its x neighbours from the
// adjacent lanes by warp shuffles (the two lanes at a warp's edges load theirs).
// Every output site is read from memory about once instead of five times.
constexpr int kStripRows = 16;

template <typename R, int K>
__device__ __forceinline__ Site<R, K> shfl_site(const Site<R, K>& s, int delta, bool down)
{
    Site<R, K> o;
#pragma unroll
    for (int i = 0; i < 4 * K; ++i)
        o.v[i] = down ? __shfl_down_sync(0xffffffffu, s.v[i], delta) : __shfl_up_sync(0xffffffffu, s.v[i], delta);
    return o;
}

template <typename R, int K, bool DAG>
__global__ void __launch_bounds__(kBlock) dirac_strip_kernel(const R* __restrict__ in, R* __restrict__ out,
                                                             const double* __restrict__ sigma,
                                                             const double* __restrict__ pi, int Nt, int Nx,
                                                             double m0, double g, double r)
{
    const int V = Nt * Nx;
    const R rr = (R)r;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;   // < Nx: the grid covers the row exactly
    const int lane = threadIdx.x & 31;
    const int xu = (x + 1 == Nx) ? 0 : x + 1;
    const int xd = (x == 0) ? Nx - 1 : x - 1;
    const int t0 = blockIdx.y * kStripRows;
    const int t1 = min(t0 + kStripRows, Nt);
    Site<R, K> prev = load_site<R, K>(in, (int64_t)(t0 == 0 ? Nt - 1 : t0 - 1) * Nx + x);
    Site<R, K> cur = load_site<R, K>(in, (int64_t)t0 * Nx + x);
    for (int t = t0; t < t1; ++t) {
        const int tn = (t + 1 == Nt) ? 0 : t + 1;
        const Site<R, K> next = load_site<R, K>(in, (int64_t)tn * Nx + x);
        const int64_t row = (int64_t)t * Nx;
        Site<R, K> up = shfl_site<R, K>(cur, 1, true);
        Site<R, K> dn = shfl_site<R, K>(cur, 1, false);
        if (lane == 31) up = load_site<R, K>(in, row + xu);
        if (lane == 0) dn = load_site<R, K>(in, row + xd);
        const int n = (int)(row + x);
        const R sp = (t + 1 == Nt) ? R(-1) : R(1);
        const R sm = (t == 0) ? R(-1) : R(1);
        const R diag = (R)(2.0 * r + m0 + g * sigma[n]);
        Site<R, K> o = dirac_combine<R, K, DAG>(cur, next, prev, up, dn, diag, rr, sp, sm);
        pion_term<R, K>(o, cur, pi, n, V, g, DAG);
        store_site<R, K>(out, n, o);
        prev = cur;
        cur = next;
    }
}

// Threads per block of the strip form: 32 w with w <= 8 dividing Nx / 32.
static int strip_width(int Nx)
{
    if (Nx % 32 != 0) return 0;
    const int warps = Nx / 32;
    for (int w = 8; w >= 1; --w)
        if (warps % w == 0) return 32 * w;
    return 32;
}

template <typename R, int K>
static cudaError_t launch_t(const void* in, void* out, const double* sigma, const double* pi, int Nt, int Nx,
                            double m0, double g, double r, int dagger, cudaStream_t stream)
{
    const int V = Nt * Nx;
    if (const int bw = strip_width(Nx)) {
        const dim3 grid(Nx / bw, (Nt + kStripRows - 1) / kStripRows);
        if (dagger)
            dirac_strip_kernel<R, K, true><<<grid, bw, 0, stream>>>((const R*)in, (R*)out, sigma, pi, Nt, Nx, m0, g, r);
        else
            dirac_strip_kernel<R, K, false><<<grid, bw, 0, stream>>>((const R*)in, (R*)out, sigma, pi, Nt, Nx, m0, g,
                                                                     r);
        return cudaGetLastError();
    }
    const int grid = (V + kBlock - 1) / kBlock;
    if (dagger)
        dirac_kernel<R, K, true><<<grid, kBlock, 0, stream>>>((const R*)in, (R*)out, sigma, pi, Nt, Nx, m0, g, r);
    else
        dirac_kernel<R, K, false><<<grid, kBlock, 0, stream>>>((const R*)in, (R*)out, sigma, pi, Nt, Nx, m0, g, r);
    return cudaGetLastError();
}

cudaError_t launch_dirac(const void* in, void* out, const double* sigma, int Nt, int Nx, double m0,
                         double g, double r, int dagger, int prec, int K, cudaStream_t stream, const double* pi)
{
    if (K == 1) pi = nullptr;   // pions need complex sites
    if (prec == YK_FP64)
        return K == 1 ? launch_t<double, 1>(in, out, sigma, pi, Nt, Nx, m0, g, r, dagger, stream)
                      : launch_t<double, 2>(in, out, sigma, pi, Nt, Nx, m0, g, r, dagger, stream);
    return K == 1 ? launch_t<float, 1>(in, out, sigma, pi, Nt, Nx, m0, g, r, dagger, stream)
                  : launch_t<float, 2>(in, out, sigma, pi, Nt, Nx, m0, g, r, dagger, stream);
}

}  // namespace yk
