// yk_langevin.cu -- the parts of a Langevin step after the CG solve.
//
// force_drift (mode 0: step, 1: force only, 2: injected force + bosonic drift):
//   chi_j = D x_j is contracted with eta_j:
//   F_n = -g/N sum_j Re sum_c conj(chi_{j,n,c}) eta_{j,n,c}
//   (FermionicDrift.cu:57-100, N = 1 in the reference).  chi_j is read from the
//   CG's t64 when the solve ended in a reliable update (the mixed solver's
//   last round forms exactly D x of the final x there, in FP64), otherwise
//   formed on the fly (never stored).  The bosonic drift
//   phi (m^2 + lambda/6 phi^2) - Lap phi (langevin_gpu_v2.cu:9-27, 41-63,
//   Laplacian columns in the sorted CSR order of Laplace.cu:61-100) is added
//   in the same pass; max|drift| goes into the chain's word by an integer
//   atomic max on the IEEE bits (exact and order-free: non-negative doubles
//   order like their bit patterns), and each tile publishes sum F.
// update: every block reads the chain's max|drift|,
//   applies the clamp and the adaptive step eps = epsBar*30/max|drift| (or a
//   fixed dt) and the Euler update phi -= eps drift + sqrt(2 eps) xi
//   (langevin_gpu_v2.cu:65-118); the last tile of a chain writes the step's
//   observables, advances Langevin time and the Philox step counter on the
//   device, so the host never waits for eps (the reference copies eps to the
//   host every step, main.cu:378-381).
#include "yk_common.cuh"
#include "yk_kernels.h"

namespace yk {

template <int K>
__global__ void __launch_bounds__(kTile) force_drift_kernel(StepArgs s, const SysDev* __restrict__ sys,
                                                            const CGState* __restrict__ st, int mode)
{
    __shared__ double red[64];
    const int2 ct = s.tiles[blockIdx.x];
    ChainDev& C = s.ch[ct.x];
    const int n = ct.y + threadIdx.x;
    double F = 0.0, d = 0.0;
    bool bad = false;
    if (n < C.V) {
        const Nbr nb = neighbours(n, C.Nt, C.Nx);
        if (mode == 2) {
            F = C.drift[n];   // injected force
        } else if (C.g != 0.0 && C.n_rhs > 0) {
            const double scale = (C.drift_mode == 1) ? C.cut * C.cut : 1.0;
            const double diag = 2.0 * C.r + C.m0 + C.g * C.phi[n];
            for (int j = 0; j < C.n_rhs; ++j) {
                const SysDev& S = sys[C.sys0 + j];
                Site<double, K> chi;
                if (st && st[C.sys0 + j].chi_ready) {
                    chi = load_site<double, K>(S.t64, n);
                } else {
                    const Site<double, K> c = load_site<double, K>(S.x, n);
                    const Site<double, K> tu = load_site<double, K>(S.x, nb.tu);
                    const Site<double, K> td = load_site<double, K>(S.x, nb.td);
                    const Site<double, K> xu = load_site<double, K>(S.x, nb.xu);
                    const Site<double, K> xd = load_site<double, K>(S.x, nb.xd);
                    chi = dirac_combine<double, K, false>(c, tu, td, xu, xd, diag, C.r, (double)nb.sp, (double)nb.sm);
                }
                const Site<double, K> e = load_site<double, K>(S.b, n);
                double sj = 0.0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    double pq = chi.v[q * K] * e.v[q * K];
                    if constexpr (K == 2) pq += chi.v[q * K + 1] * e.v[q * K + 1];
                    sj = (q == 0) ? pq : sj + pq;
                }
                F += -(scale * C.g) * sj;
            }
            if (C.n_rhs > 1) F /= (double)C.n_rhs;
        }
        if (mode != 1) {
            d = step_drift(C, n, F);
            C.drift[n] = d;
        } else {
            d = F;
            C.drift[n] = F;
        }
        bad = !isfinite(d);
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(&C.status, 0, (int)YK_ENAN);
    // max|drift| (a NaN does not count, as fmax ignores it) for the update;
    // mode 1 is not followed by one and leaves the word alone
    if (mode != 1) block_max_bits(isnan(d) ? 0ull : (unsigned long long)__double_as_longlong(fabs(d)), &C.dmax_bits);
    const double sf = block_sum(F, red);
    if (threadIdx.x == 0) s.tile_sum2[s.tile_base + blockIdx.x] = sf;
}

__global__ void __launch_bounds__(kTile) update_kernel(StepArgs s, const CGState* __restrict__ st)
{
    __shared__ double red[64];
    __shared__ double s_eps, s_fact, s_max;
    __shared__ int s_last;
    const int2 ct = s.tiles[blockIdx.x];
    ChainDev& C = s.ch[ct.x];
    const int n = ct.y + threadIdx.x;
    // the site's operands first: their loads overlap thread 0's FP64 division
    // and square root below
    double v = 0.0, dr = 0.0, xn = 0.0;
    if (n < C.V) {
        v = C.phi[n];
        dr = C.drift[n];
        xn = C.xi[n];
    }
    if (threadIdx.x == 0) {
        double m = __longlong_as_double((long long)*(volatile unsigned long long*)&C.dmax_bits);
        if (m > 1e5) m = 1e5;               // langevin_gpu_v2.cu:83-91
        else if (m < 1e-5) m = 1e-5;
        s_max = m;
        const double e = (C.fixed_dt > 0.0) ? C.fixed_dt : C.eps_bar * 30.0 / m;
        s_eps = e;
        s_fact = sqrt(2.0 * e);   // once per block: an FP64 square root is a long sequence on GB300
    }
    __syncthreads();
    const double eps = s_eps;
    const double fact = s_fact;
    double p1 = 0.0, p2 = 0.0;
    if (n < C.V) {
        v -= eps * dr + fact * xn;
        C.phi[n] = v;
        p1 = v;
        p2 = v * v;
    }
    const double2 ps = block_sum2(p1, p2, red);
    if (threadIdx.x == 0) {
        s.tile_sum[s.tile_base + blockIdx.x] = ps;
        __threadfence();
        const unsigned prev = atomicAdd(&C.counter, 1u);
        s_last = (prev == (unsigned)C.ntiles - 1) ? 1 : 0;
    }
    __syncthreads();
    if (s_last) {
        // the last tile of the chain: every thread loads its tiles' sums at
        // once (one round trip), then a fixed-order block reduction
        __threadfence();
        double a = 0.0, b = 0.0, f = 0.0;
        for (int i = threadIdx.x; i < C.ntiles; i += blockDim.x) {
            const double2 q = ld_volatile2(s.tile_sum + C.tile0 + i);
            a += q.x;
            b += q.y;
            f += ld_volatile(s.tile_sum2 + C.tile0 + i);
        }
        const double2 ab = block_sum2(a, b, red);
        f = block_sum(f, red);
        a = ab.x;
        b = ab.y;
        if (threadIdx.x == 0) {
            int iters = 0, status = *(volatile int*)&C.status;
            if (C.g != 0.0)
                for (int j = 0; j < C.n_rhs; ++j) {
                    iters += st[C.sys0 + j].iters;
                    if (status == 0 && st[C.sys0 + j].status) status = st[C.sys0 + j].status;
                }
            C.time += eps;
            C.obs.t = C.time;
            C.obs.eps = eps;
            C.obs.max_drift = s_max;
            C.obs.sum_phi = a;
            C.obs.sum_phi2 = b;
            C.obs.sum_force = f;
            C.obs.steps += 1;
            C.obs.cg_iterations = iters;
            C.obs.cg_iterations_total += iters;
            if (status == YK_ENOCONV) C.obs.noconv_steps += 1;
            C.obs.status = status;
            C.step += 1;
            if (C.series && C.series_n < C.series_cap) C.series[C.series_n++] = a / (double)C.V;
            C.counter = 0;
            C.status = 0;
            C.dmax_bits = 0ull;   // every block read it before counting in
        }
    }
}

cudaError_t launch_force_drift(const StepArgs& s, const SysDev* sys, int mode, int K, cudaStream_t stream,
                               const CGState* st)
{
    if (K == 1)
        force_drift_kernel<1><<<s.ntiles, kTile, 0, stream>>>(s, sys, st, mode);
    else
        force_drift_kernel<2><<<s.ntiles, kTile, 0, stream>>>(s, sys, st, mode);
    return cudaGetLastError();
}

// eta (kind 2) of the step after each chain's current one at every site of
// the tiles' systems, into the buffer of that step's parity, tagged with the
// step.  Grid-stride over the tiles, so it can run on a few SMs beside the CG.
__global__ void __launch_bounds__(kTile) eta_ahead_kernel(const SysDev* __restrict__ sys,
                                                          const int2* __restrict__ tiles, int ntiles)
{
    for (int item = blockIdx.x; item < ntiles; item += gridDim.x) {
        const int2 tl = tiles[item];
        const SysDev& S = sys[tl.x];
        const int64_t step = *S.step + 1;
        const int par = (int)(step & 1);
        const int n = tl.y + threadIdx.x;
        if (n < S.V) store_site<double, 1>(S.eta_ahead[par], n, eta_site_at<1>(S, n, 2, step));
        // read only after this kernel has finished (the next step's CG)
        if (tl.y == 0 && threadIdx.x == 0) S.eta_tag[par] = step;
    }
}

cudaError_t launch_eta_ahead(const SysDev* sys, const int2* tiles, int ntiles, int max_blocks, cudaStream_t stream)
{
    if (ntiles <= 0) return cudaSuccess;
    const int grid = (max_blocks > 0 && ntiles > max_blocks) ? max_blocks : ntiles;
    eta_ahead_kernel<<<grid, kTile, 0, stream>>>(sys, tiles, ntiles);
    return cudaGetLastError();
}

cudaError_t launch_update(const StepArgs& s, const CGState* st, cudaStream_t stream)
{
    update_kernel<<<s.ntiles, kTile, 0, stream>>>(s, st);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Field transfers of yk_langevin_step_io through mapped pinned host memory:
// the copy is a kernel in the step's graph instead of a copy-engine node per
// buffer (the upload; the download of the field, the observables' words and
// the error word in one launch).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void io_copy(const double* __restrict__ src, double* __restrict__ dst, int n)
{
    const int stride = gridDim.x * blockDim.x;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
        const double2* s2 = reinterpret_cast<const double2*>(src);
        double2* d2 = reinterpret_cast<double2*>(dst);
        for (int i = i0; i < n / 2; i += stride) d2[i] = s2[i];
        if (i0 == 0 && (n & 1)) dst[n - 1] = src[n - 1];
    } else {
        for (int i = i0; i < n; i += stride) dst[i] = src[i];
    }
}

__global__ void __launch_bounds__(256) io_load_kernel(const double* __restrict__ host, double* __restrict__ phi, int V)
{
    io_copy(host, phi, V);
}

__global__ void __launch_bounds__(256) io_store_kernel(const double* __restrict__ phi, double* __restrict__ host, int V,
                                                       const double* __restrict__ obs, double* __restrict__ hobs,
                                                       int obs_words, const int* __restrict__ err, int* herr)
{
    if (host) io_copy(phi, host, V);
    if (blockIdx.x == gridDim.x - 1) {
        for (int i = threadIdx.x; i < obs_words; i += blockDim.x) hobs[i] = obs[i];
        if (threadIdx.x == 0) *herr = *err;
    }
}

namespace {
int io_blocks(int V)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return std::max(1, std::min((V / 2 + 255) / 256, 2 * nsm));
}
}  // namespace

cudaError_t launch_io_load(const double* host, double* phi, int V, cudaStream_t stream)
{
    io_load_kernel<<<io_blocks(V), 256, 0, stream>>>(host, phi, V);
    return cudaGetLastError();
}

cudaError_t launch_io_store(const double* phi, double* host, int V, const void* obs, void* hobs, size_t obs_bytes,
                            const int* err, int* herr, cudaStream_t stream)
{
    io_store_kernel<<<io_blocks(V), 256, 0, stream>>>(phi, host, V, static_cast<const double*>(obs),
                                                       static_cast<double*>(hobs), (int)(obs_bytes / 8), err, herr);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Observables used by the export block of main.cu:385-483.
// ---------------------------------------------------------------------------
__global__ void time_slices_kernel(const double* __restrict__ phi, double* out, int Nx)
{
    __shared__ double red[64];
    const int t = blockIdx.x;
    double a = 0.0;
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) a += phi[(int64_t)t * Nx + x];
    const double2 r = block_sum2(a, 0.0, red);
    if (threadIdx.x == 0) out[t] = r.x;
}

template <int K>
__global__ void time_slices_spinor_kernel(const double* __restrict__ psi, double* out, int Nx)
{
    __shared__ double red[64];
    const int t = blockIdx.x;
    double a = 0.0;
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        const double* p = psi + ((int64_t)t * Nx + x) * 4 * K;
#pragma unroll
        for (int c = 0; c < 4; ++c) a += p[c * K];
    }
    const double2 r = block_sum2(a, 0.0, red);
    if (threadIdx.x == 0) out[t] = r.x;
}

cudaError_t launch_time_slices(const double* phi, double* out, int Nt, int Nx, cudaStream_t stream)
{
    time_slices_kernel<<<Nt, kBlock, 0, stream>>>(phi, out, Nx);
    return cudaGetLastError();
}

cudaError_t launch_time_slices_spinor(const double* psi, double* corr, int Nt, int Nx, int K,
                                      cudaStream_t stream)
{
    if (K == 1)
        time_slices_spinor_kernel<1><<<Nt, kBlock, 0, stream>>>(psi, corr, Nx);
    else
        time_slices_spinor_kernel<2><<<Nt, kBlock, 0, stream>>>(psi, corr, Nx);
    return cudaGetLastError();
}

}  // namespace yk
