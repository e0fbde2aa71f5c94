// yk_dirac.cu -- stand-alone Wilson-Dirac apply (the replacement for
// DiracOP<double>::applyD, code/src/Dirac.cu:23-70 and :144-190).
//
// One pass: each thread produces one site from its own entries and its four
// neighbours (coalesced 16-byte vector loads, neighbour reuse through L1),
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

template <typename R, int K>
static cudaError_t launch_t(const void* in, void* out, const double* sigma, const double* pi, int Nt, int Nx,
                            double m0, double g, double r, int dagger, cudaStream_t stream)
{
    const int V = Nt * Nx;
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
