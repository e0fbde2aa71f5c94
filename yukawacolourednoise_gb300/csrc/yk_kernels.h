// yk_kernels.h -- host-side launchers of the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "yk_internal.h"

namespace yk {

// Wilson-Dirac apply on one lattice (K real planes per entry; K = 2 for
// interleaved complex buffers).  prec YK_FP64 (double) or YK_FP32 (float).
// pi: the chain's pions (3 x V doubles) or null for the sigma-only operator.
cudaError_t launch_dirac(const void* in, void* out, const double* sigma, int Nt, int Nx,
                         double m0, double g, double r, int dagger, int prec, int K,
                         cudaStream_t stream, const double* pi = nullptr);

// Batched CG (yk_cg.cu).  Also launches its one-block preparation kernel.
// grid_out: blocks launched; kernel_out: 0 cg_kernel, 1 cg_halo_kernel, 3 cg_eo_kernel
// (the even-odd solve: a.sys_eo given, chi = (D^dag)^-1 b left in t64) (either may be null)
cudaError_t launch_cg(const CGArgs& a, int K, bool mixed, cudaStream_t stream, int* grid_out, int* kernel_out = nullptr);
// Work-balanced block ranges (CGArgs::balance) for the next solve of the
// systems of `a`, from their iteration counts in the solve just finished;
// grid: the grid of that solve's launch.  No-op for a single system.
cudaError_t launch_cg_balance(const CGArgs& a, int grid, int* out, cudaStream_t stream);
// Largest co-resident grid of the CG kernel (cached; call before capturing).
int cg_max_grid(int K, bool mixed);
int cg_eob_max_grid();   // co-resident blocks of the batched even-odd CG
// Kernel attributes and occupancy of the halo CG kernel (call before any stream capture).
void cg_halo_init();
// Runs the wait-timeout probe kernel on `stream`; *status = the device status
// it recorded.  Returns 0, or -1 on a CUDA error.
int wait_timeout_probe(cudaStream_t stream, int* status);

// Cluster-resident mixed CG (yk_cg_cluster.cu): one 16-CTA cluster per system
// of real (K = 1) vectors whose rows fit the cluster (cg_cluster_fits);
// max_sites = the largest per-CTA share (ceil(Nt / 16) * Nx) of the systems.
// cg_cluster_init opts in to the cluster size and shared memory and checks
// residency (call before capturing).  launch_eta draws b = eta for the
// systems of the given tiles (the cluster kernel reads b).
bool cg_cluster_fits(int Nt, int Nx);
bool cg_cluster_init();
cudaError_t launch_cg_cluster(const CGArgs& a, int max_sites, cudaStream_t stream);
cudaError_t launch_eta(const SysDev* sys, const int2* tiles, int ntiles, int kind, cudaStream_t stream);
// Raises the shared-memory limit of the FFT kernels (call before capturing).
void noise_init_attributes();

// Coloured noise of every chain in the tables (yk_noise.cu): xi = filtered
// Philox white noise at each chain's current step, or the filtered `given`
// white field (tables of a single chain).  max_blocks > 0 caps the grids of
// the FFT passes (each block loops over its share of rows / column strips),
// so the passes can run beside a CG that holds the other SMs.
cudaError_t launch_noise_tables(ChainDev* d_chains, const NoiseTables& tb, int max_nx,
                                int max_cols_elems, const double* given, cudaStream_t stream,
                                int max_blocks = 0);
// eta of the next step into the systems' ahead buffers (yk_langevin.cu).
cudaError_t launch_eta_ahead(const SysDev* sys, const int2* tiles, int ntiles, int max_blocks, cudaStream_t stream);
// Blocks (one per SM) of the CG launch_cg would start for `a` (the step's
// persistent CG on the real path).
int cg_predict_grid(const CGArgs& a, bool mixed);

// Force + drift (+ per-tile max|drift| and sum F), then the Euler update and
// observables (yk_langevin.cu).  mode 0: drift = F + bosonic drift;
// mode 1: drift = F (the fermion force alone); mode 2: drift (preset to a
// given force) += bosonic drift.
// st: the solves' states when x was just solved (chi = D x is then reused
// from a solve that ended in a reliable update), else null
cudaError_t launch_force_drift(const StepArgs& s, const SysDev* sys, int mode, int K, cudaStream_t stream,
                               const CGState* st = nullptr);
cudaError_t launch_update(const StepArgs& s, const CGState* st, cudaStream_t stream);
// yk_langevin_step_io's transfers through mapped pinned host memory (device
// addresses of the host buffers): the field's upload; the field's download
// (host null: none) with the observables' bytes (a multiple of 8) and the
// error word
cudaError_t launch_io_load(const double* host, double* phi, int V, cudaStream_t stream);
cudaError_t launch_io_store(const double* phi, double* host, int V, const void* obs, void* hobs, size_t obs_bytes,
                            const int* err, int* herr, cudaStream_t stream);

// The pion extension's step (yk_pion.cu): white noise of the three pion
// fields (3V), the complex sources eta_j of Philox stream `kind` (R x 8V), the
// forces F4 (4V: sigma, pi_1..3) from the R solved systems, and the drift and
// Euler update of the four fields with the step's observables.
cudaError_t launch_pion_white(const ChainDev* C, double* white3, int V, cudaStream_t s);
cudaError_t launch_pion_eta(const ChainDev* C, double* eta, int R, int kind, int V, cudaStream_t s);
cudaError_t launch_pion_force(const ChainDev* C, const SysDev* sys, int R, const double* pi, double* F4, int V,
                              cudaStream_t s);
cudaError_t launch_pion_drift_update(ChainDev* C, double* pi, const double* F4, double* pdrift, const double* pxi,
                                     double* tile_part, double* tile_f, const CGState* st, int R, int V,
                                     cudaStream_t s);

// Gamma-method analysis of a device series of n per-configuration <sigma>
// values on a `volume`-site lattice (yk_series.cu).  Returns a yk_status.
int series_analyse(const double* d_series, int64_t n, int64_t volume, double stau, yk_series_stats* out,
                   cudaStream_t s);

// Point-source / time-slice helpers.
cudaError_t launch_time_slices_spinor(const double* psi, double* corr, int Nt, int Nx, int K,
                                      cudaStream_t stream);
cudaError_t launch_time_slices(const double* phi, double* out, int Nt, int Nx, cudaStream_t stream);

// Learned preconditioner (yk_learned.cu): a linear convolutional network on
// one Nt x Nx lattice (real plane), its training and the flexible GCR that
// uses it.
struct LearnedNet;
// the operator A = D^dag D of a chain (real plane): its field and action
struct NetOp {
    const double* sigma;
    int Nt, Nx;
    double m0, g, r;
};
struct FgcrResult {
    int iterations;   // FGCR iterations (preconditioner applications)
    int outer;        // FP64 refinement rounds
    double rr, rr0;   // final FP64 |r|^2 and |b|^2
    int converged;
};
LearnedNet* net_create(int Nt, int Nx, int layers, cudaError_t* err);
void net_destroy(LearnedNet* n);
int net_size(const LearnedNet* n);
// the convolution tile of the solvers' M and its layers per launch (zeros
// before the first solve tuned them)
void net_tile(const LearnedNet* n, int* rows, int* cols, int* per_launch);
void net_set_skip(LearnedNet* n, float skip);   // M(r) = skip r + N(r)
cudaError_t net_weights(LearnedNet* n, float* host, bool set);
cudaError_t net_forward(LearnedNet* n, const float* r, const double* sigma, float* z, cudaStream_t s);
// the same with BF16 activations and tensor-core convolutions (the form the solvers apply)
cudaError_t net_forward_fast(LearnedNet* n, const float* r, const double* sigma, float* z, cudaStream_t s);
cudaError_t net_zero_grad(LearnedNet* n, cudaStream_t s);
// loss of a pair: (M r - e)^T A (M r - e); accumulates its weight gradient
cudaError_t net_accumulate_grad(LearnedNet* n, const float* r, const float* e, const NetOp& op, cudaStream_t s,
                                double* loss);
cudaError_t net_grad_to_host(LearnedNet* n, float* host, cudaStream_t s);
cudaError_t net_adam_step(LearnedNet* n, float lr, int batch, cudaStream_t s);
cudaError_t net_add_pair(LearnedNet* n, int cap, const double* sigma, double m0, double g, double r, const double* b,
                         const double* xstar, const double* xk, cudaStream_t s);
int net_pairs(const LearnedNet* n);
cudaError_t net_mean_loss(LearnedNet* n, const NetOp& op, cudaStream_t s, double* out);
cudaError_t net_train(LearnedNet* n, const NetOp& op, int steps, int batch, float lr, uint64_t seed, cudaStream_t s);
cudaError_t fgcr_solve(LearnedNet* n, bool use_net, const double* sigma, double m0, double g, double r,
                       const double* b, double* x, double tol, int tol_mode, int max_iter, int restart,
                       double inner_tol, cudaStream_t s, FgcrResult* res);
// preconditioned CG (M SPD) with device-side scalars, inside FP64 refinement;
// inner_tol <= 0: chosen per network by timing 1e-4 against 1e-5
// (pcg_inner_choice: the choice with the network, 0 while undecided)
double pcg_inner_choice(const LearnedNet* n);
cudaError_t pcg_solve(LearnedNet* n, bool use_net, const double* sigma, double m0, double g, double r,
                      const double* b, double* x, double tol, int tol_mode, int max_iter, double inner_tol,
                      cudaStream_t s, FgcrResult* res);

}  // namespace yk
