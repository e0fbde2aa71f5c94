// yk_pion.cu -- the pion extension of the Langevin step.
//
// No reference counterpart: the reference's model has the single scalar sigma
// (code/src/params.h:25 nVectorComponents = 1) and the real Yukawa diagonal
// g sigma (Dirac.cu:57-69).  With pions the Yukawa term is
// g (sigma + i gamma5 tau.pi) (pion_add, yk_common.cuh), the operator is
// complex, and the step moves four fields phi = (sigma, pi_1, pi_2, pi_3):
//
//   noise   each field its own coloured noise: sigma the step's usual stream
//           (Philox kind 1, rhs 0), pi_a kind 1 with rhs a (pion_white_kernel
//           draws the white noise, the FFT passes filter it);
//   force   x_j = (D^dag D)^-1 eta_j by the complex CG with the pion term,
//           chi_j = D x_j, and per site
//             F_sigma = -g Re sum_c conj(chi_c) eta_c            (FermionicDrift.cu:83-100)
//             F_pi_a  = -g Re sum_c conj(chi_c) (i gamma5 tau_a eta)_c,
//           the one-noise estimates of -Re tr(D^-1 dD/dphi_a(n));
//   drift   drift_a = F_a + phi_a (m^2 + lambda/6 |phi|^2) - Lap phi_a, the
//           O(4)-symmetric form of PotentialAndMass (langevin_gpu_v2.cu:9-27)
//           with the Laplacian of the sigma path (sorted CSR column order);
//   update  max|drift| over the four fields gives the adaptive eps (or the
//           fixed dt), every field takes phi -= eps drift + sqrt(2 eps) xi
//           (langevin_gpu_v2.cu:29-37), and the last tile writes the step's
//           observables (sum sigma, sum sigma^2, sum pi_a, sum |pi|^2, sum F)
//           and advances time and the Philox step on the device.
//
// At pi = 0 the sigma force, drift and update perform the sigma-only path's
// operations in the same order: with a fixed dt sigma moves exactly as
// without pions.
#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

// White noise of the three pion fields at the chain's current step: element n
// of field a is normal n of Philox stream (kind 1, rhs a), as the sigma noise
// (white_at, yk_noise.cu).
__global__ void __launch_bounds__(kBlock) pion_white_kernel(const ChainDev* __restrict__ C, double* __restrict__ white3)
{
    const int V = C->V;
    const uint64_t step = (uint64_t)C->step;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * V; i += gridDim.x * blockDim.x) {
        const int q = i / V, n = i - q * V;
        const RngStream rs = rng_stream(C->seed, C->chain_id, step, 1u, (uint32_t)(q + 1));
        white3[i] = normal_at(rs, (uint32_t)n);
    }
}

// Complex sources eta_j (j < R) of Philox stream (kind, rhs j) at the chain's
// current step: real Gaussian entries, imaginary parts zero (the entries of
// eta_site_at, FermionicDrift.cu:102-110).
__global__ void __launch_bounds__(kBlock) pion_eta_kernel(const ChainDev* __restrict__ C, double* __restrict__ eta,
                                                          int R, int kind)
{
    const int V = C->V;
    const uint64_t step = (uint64_t)C->step;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R * V; i += gridDim.x * blockDim.x) {
        const int j = i / V, n = i - j * V;
        const RngStream rs = rng_stream(C->seed, C->chain_id, step, (uint32_t)kind, (uint32_t)j);
        const float4 z = normal4(rs, (uint32_t)n);   // normals 4n .. 4n + 3
        double2* e = reinterpret_cast<double2*>(eta + ((size_t)j * V + n) * 8);
        e[0] = make_double2(z.x, 0.0);
        e[1] = make_double2(z.y, 0.0);
        e[2] = make_double2(z.z, 0.0);
        e[3] = make_double2(z.w, 0.0);
    }
}

// F4[q V + n] (q = 0 sigma, 1..3 pi_q) from the solutions x_j of the R
// systems sys[0 .. R-1] (b = eta_j); chi_j = D x_j formed on the fly.  R = 0
// writes zeros.
__global__ void __launch_bounds__(kTile) pion_force_kernel(const ChainDev* __restrict__ C,
                                                           const SysDev* __restrict__ sys, int R,
                                                           const double* __restrict__ pi, double* __restrict__ F4)
{
    const int V = C->V;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= V) return;
    double f[4] = {0.0, 0.0, 0.0, 0.0};
    if (C->g != 0.0 && R > 0) {
        const Nbr nb = neighbours(n, C->Nt, C->Nx);
        const double scale = (C->drift_mode == 1) ? C->cut * C->cut : 1.0;
        const double diag = 2.0 * C->r + C->m0 + C->g * C->phi[n];
        for (int j = 0; j < R; ++j) {
            const SysDev& S = sys[j];
            const Site<double, 2> c = load_site<double, 2>(S.x, n);
            const Site<double, 2> tu = load_site<double, 2>(S.x, nb.tu);
            const Site<double, 2> td = load_site<double, 2>(S.x, nb.td);
            const Site<double, 2> xu = load_site<double, 2>(S.x, nb.xu);
            const Site<double, 2> xd = load_site<double, 2>(S.x, nb.xd);
            Site<double, 2> chi = dirac_combine<double, 2, false>(c, tu, td, xu, xd, diag, C->r, (double)nb.sp,
                                                                  (double)nb.sm);
            pion_term<double, 2>(chi, c, pi, n, V, C->g, false);
            const Site<double, 2> e = load_site<double, 2>(S.b, n);
            // sigma: the contraction of force_drift_kernel, term for term
            double sj = 0.0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                double pq = chi.v[q * 2] * e.v[q * 2];
                pq += chi.v[q * 2 + 1] * e.v[q * 2 + 1];
                sj = (q == 0) ? pq : sj + pq;
            }
            f[0] += -(scale * C->g) * sj;
            // pions: u = i gamma5 tau_a eta
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                Site<double, 2> u;
#pragma unroll
                for (int i = 0; i < 8; ++i) u.v[i] = 0.0;
                pion_add<double>(u, e, a == 0 ? 1.0 : 0.0, a == 1 ? 1.0 : 0.0, a == 2 ? 1.0 : 0.0);
                double sa = 0.0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    double pq = chi.v[q * 2] * u.v[q * 2];
                    pq += chi.v[q * 2 + 1] * u.v[q * 2 + 1];
                    sa = (q == 0) ? pq : sa + pq;
                }
                f[a + 1] += -(scale * C->g) * sa;
            }
        }
        if (R > 1)
#pragma unroll
            for (int q = 0; q < 4; ++q) f[q] /= (double)R;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) F4[(size_t)q * V + n] = f[q];
}

__device__ __forceinline__ void sort5(int* col)
{
    auto cs = [](int& a, int& b) {
        const int lo = min(a, b), hi = max(a, b);
        a = lo;
        b = hi;
    };
    // 5-input sorting network (9 comparators), the order of force_drift_kernel
    cs(col[0], col[1]); cs(col[3], col[4]); cs(col[2], col[4]);
    cs(col[2], col[3]); cs(col[0], col[3]); cs(col[0], col[2]);
    cs(col[1], col[4]); cs(col[1], col[3]); cs(col[1], col[2]);
}

// drift of the four fields (sigma's into C->drift, the pions' into pdrift),
// max|drift| into the chain's word, per-tile sum of F_sigma.
__global__ void __launch_bounds__(kTile) pion_drift_kernel(ChainDev* __restrict__ C, const double* __restrict__ pi,
                                                           const double* __restrict__ F4, double* __restrict__ pdrift,
                                                           double* __restrict__ tile_f)
{
    __shared__ double red[64];
    const int V = C->V;
    const int n = blockIdx.x * kTile + threadIdx.x;
    double fs = 0.0, m = 0.0;
    bool bad = false;
    if (n < V) {
        const Nbr nb = neighbours(n, C->Nt, C->Nx);
        int col[5] = {n, (int)nb.tu, (int)nb.td, (int)nb.xu, (int)nb.xd};
        sort5(col);
        const double s0 = C->phi[n], p1 = pi[n], p2 = pi[V + n], p3 = pi[2 * V + n];
        const double r2 = s0 * s0 + p1 * p1 + p2 * p2 + p3 * p3;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double* f = q == 0 ? C->phi : pi + (size_t)(q - 1) * V;
            double d = F4[(size_t)q * V + n];
            d += f[n] * (C->m2 + C->lambda6 * r2);
            double lap = 0.0;
#pragma unroll
            for (int k = 0; k < 5; ++k) lap += col[k] != n ? f[col[k]] : -4.0 * f[col[k]];
            d -= lap;
            if (q == 0)
                C->drift[n] = d;
            else
                pdrift[(size_t)(q - 1) * V + n] = d;
            bad = bad || !isfinite(d);
            if (!isnan(d)) m = fmax(m, fabs(d));
        }
        fs = F4[n];
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(&C->status, 0, (int)YK_ENAN);
    block_max_bits((unsigned long long)__double_as_longlong(m), &C->dmax_bits);
    const double sf = block_sum(fs, red);
    if (threadIdx.x == 0) tile_f[blockIdx.x] = sf;
}

// Euler update of the four fields and the step's observables; the last tile
// to finish reduces the tiles' sums in a fixed order and advances the chain.
// tile_part: 6 doubles per tile; st: the R solves' states.
__global__ void __launch_bounds__(kTile) pion_update_kernel(ChainDev* __restrict__ C, double* __restrict__ pi,
                                                            const double* __restrict__ pdrift,
                                                            const double* __restrict__ pxi,
                                                            double* __restrict__ tile_part,
                                                            const double* __restrict__ tile_f,
                                                            const CGState* __restrict__ st, int R)
{
    __shared__ double red[64];
    __shared__ double s_eps, s_fact, s_max;
    __shared__ int s_last;
    const int V = C->V, ntiles = (V + kTile - 1) / kTile;
    if (threadIdx.x == 0) {
        double m = __longlong_as_double((long long)*(volatile unsigned long long*)&C->dmax_bits);
        if (m > 1e5) m = 1e5;   // langevin_gpu_v2.cu:83-91
        else if (m < 1e-5) m = 1e-5;
        s_max = m;
        const double e = (C->fixed_dt > 0.0) ? C->fixed_dt : C->eps_bar * 30.0 / m;
        s_eps = e;
        s_fact = sqrt(2.0 * e);
    }
    __syncthreads();
    const double eps = s_eps, fact = s_fact;
    const int n = blockIdx.x * kTile + threadIdx.x;
    double p[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   // sigma, sigma^2, pi_1, pi_2, pi_3, |pi|^2
    if (n < V) {
        double v = C->phi[n];
        v -= eps * C->drift[n] + fact * C->xi[n];
        C->phi[n] = v;
        p[0] = v;
        p[1] = v * v;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const size_t i = (size_t)q * V + n;
            double w = pi[i];
            w -= eps * pdrift[i] + fact * pxi[i];
            pi[i] = w;
            p[2 + q] = w;
            p[5] += w * w;
        }
    }
    double2 t0 = block_sum2(p[0], p[1], red);
    double2 t1 = block_sum2(p[2], p[3], red);
    double2 t2 = block_sum2(p[4], p[5], red);
    if (threadIdx.x == 0) {
        double* tp = tile_part + (size_t)blockIdx.x * 6;
        tp[0] = t0.x;
        tp[1] = t0.y;
        tp[2] = t1.x;
        tp[3] = t1.y;
        tp[4] = t2.x;
        tp[5] = t2.y;
        __threadfence();
        const unsigned prev = atomicAdd(&C->counter, 1u);
        s_last = (prev == (unsigned)ntiles - 1) ? 1 : 0;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double a[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < ntiles; i += blockDim.x) {
#pragma unroll
        for (int q = 0; q < 6; ++q) a[q] += ld_volatile(tile_part + (size_t)i * 6 + q);
        a[6] += ld_volatile(tile_f + i);
    }
    t0 = block_sum2(a[0], a[1], red);
    t1 = block_sum2(a[2], a[3], red);
    t2 = block_sum2(a[4], a[5], red);
    const double f = block_sum(a[6], red);
    if (threadIdx.x == 0) {
        int iters = 0, status = *(volatile int*)&C->status;
        for (int j = 0; j < R; ++j) {
            iters += st[j].iters;
            if (status == 0 && st[j].status) status = st[j].status;
        }
        C->time += eps;
        C->obs.t = C->time;
        C->obs.eps = eps;
        C->obs.max_drift = s_max;
        C->obs.sum_phi = t0.x;
        C->obs.sum_phi2 = t0.y;
        C->obs.sum_pi[0] = t1.x;
        C->obs.sum_pi[1] = t1.y;
        C->obs.sum_pi[2] = t2.x;
        C->obs.sum_pi2 = t2.y;
        C->obs.sum_force = f;
        C->obs.steps += 1;
        C->obs.cg_iterations = iters;
        C->obs.cg_iterations_total += iters;
        if (status == YK_ENOCONV) C->obs.noconv_steps += 1;
        C->obs.status = status;
        C->step += 1;
        if (C->series && C->series_n < C->series_cap) C->series[C->series_n++] = t0.x / (double)V;
        C->counter = 0;
        C->status = 0;
        C->dmax_bits = 0ull;
    }
}

cudaError_t launch_pion_white(const ChainDev* C, double* white3, int V, cudaStream_t s)
{
    const int grid = (3 * V + kBlock - 1) / kBlock;
    pion_white_kernel<<<grid, kBlock, 0, s>>>(C, white3);
    return cudaGetLastError();
}

cudaError_t launch_pion_eta(const ChainDev* C, double* eta, int R, int kind, int V, cudaStream_t s)
{
    if (R <= 0) return cudaSuccess;
    const int grid = (R * V + kBlock - 1) / kBlock;
    pion_eta_kernel<<<grid, kBlock, 0, s>>>(C, eta, R, kind);
    return cudaGetLastError();
}

cudaError_t launch_pion_force(const ChainDev* C, const SysDev* sys, int R, const double* pi, double* F4, int V,
                              cudaStream_t s)
{
    pion_force_kernel<<<(V + kTile - 1) / kTile, kTile, 0, s>>>(C, sys, R, pi, F4);
    return cudaGetLastError();
}

cudaError_t launch_pion_drift_update(ChainDev* C, double* pi, const double* F4, double* pdrift, const double* pxi,
                                     double* tile_part, double* tile_f, const CGState* st, int R, int V,
                                     cudaStream_t s)
{
    const int nt = (V + kTile - 1) / kTile;
    pion_drift_kernel<<<nt, kTile, 0, s>>>(C, pi, F4, pdrift, tile_f);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    pion_update_kernel<<<nt, kTile, 0, s>>>(C, pi, pdrift, pxi, tile_part, tile_f, st, R);
    return cudaGetLastError();
}

}  // namespace yk
