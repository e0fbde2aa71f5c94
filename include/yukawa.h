/*
 * yukawa.h -- C ABI of libyukawa_gb300.so, the GB300-native Langevin hot path
 * of the 2-D Yukawa model of Matteo294/YukawaColouredNoise.
 *
 * The reference exposes no plugin/FFI API; its boundaries are the in-process
 * C++ classes DiracOP, CGsolver, FermionicDrift, ColouredNoise, the `Run`
 * kernel, the input.toml schema and the `./out input.toml` CLI.  Each entry
 * point below names the reference interface it replaces (paths relative to
 * the reference project).
 *
 * Conventions
 *   - Every function returns a yk_status (YK_OK == 0); yk_last_error() gives
 *     the message of the last failure on the calling thread.
 *   - Buffers passed as `void*`/`double*` to operator calls are DEVICE
 *     pointers unless the name says host.  Spinors are 4 complex per site
 *     ([f1s1, f1s2, f2s1, f2s2], interleaved re/im, code/src/Spinor.cuh:7-16),
 *     site n = t*Nx + x (code/src/Lattice.cu:16-18).
 *   - All work is ordered on the context's stream (yk_ctx_set_stream); calls
 *     that return host values synchronise that stream.
 *   - One context per host thread; a context is not thread-safe.
 */
#ifndef YUKAWA_GB300_H
#define YUKAWA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum yk_status {
    YK_OK = 0,
    YK_EINVAL = 1,    /* bad argument, size or unsupported combination      */
    YK_ENOCONV = 2,   /* CG reached its iteration cap without converging     */
    YK_ENAN = 3,      /* NaN/Inf met in a residual, drift or field           */
    YK_ETIMEOUT = 4,  /* a bounded device-side wait gave up                  */
    YK_ECUDA = 5,     /* CUDA runtime error                                  */
    YK_ENOMEM = 6,    /* device allocation failed                            */
    YK_EIO = 7        /* file could not be read or written                   */
} yk_status;

enum { YK_NORMAL = 0, YK_DAGGER = 1 };          /* MatrixType, code/src/params.h:8 */
enum { YK_FP64 = 0, YK_FP32 = 1, YK_MIXED = 2 }; /* arithmetic of a call           */
enum { YK_TOL_ABS = 0, YK_TOL_REL = 1 };         /* CG stopping rule               */
enum { YK_INIT_DRAND48 = 0, YK_INIT_PHILOX = 1, YK_INIT_NONE = 2 };

/*
 * Run parameters: the reference's input.toml keys (code/input.toml:1-28, read
 * at code/src/main.cu:112-170), the lattice size that the reference fixes at
 * compile time (code/src/params.h:28, patched by runs.py:80-85), and the
 * [gpu] extension keys.  yk_params_default() gives the reference's defaults:
 * compile-time tolerance 1e-8 absolute and IterMax 1000 (code/src/params.h:13-15).
 */
typedef struct yk_params {
    /* [physics] */
    int use_mass;              /* useMass == "true"                              */
    double mass;               /* m^2 when use_mass                              */
    double g;                  /* lambda when use_mass                           */
    double kappa;              /* hopping parameter when !use_mass               */
    double lambda;             /* lattice lambda when !use_mass                  */
    double cut_fraction;       /* cutFraction s: keep |p| <= sqrt(2) pi s        */
    /* [langevin] */
    double average_epsilon;
    double max_langevin_time;
    double export_time;
    int burn_count;
    int measure_drift_count;
    /* [random] */
    int64_t seed;
    /* [fermions] */
    double yukawa_coupling;
    double fermion_mass;
    int drift_mode;            /* 0 normal, 1 rescaled by cutFraction^2          */
    double wilson_param;
    /* [lattice] */
    int Nt, Nx;
    /* [gpu] extensions (not in the reference) */
    int precision;             /* YK_FP64 or YK_MIXED for the CG of each step     */
    int n_rhs;                 /* stochastic right-hand sides per step (1 = ref) */
    int cg_tol_mode;           /* YK_TOL_ABS (reference) or YK_TOL_REL            */
    double cg_tol;             /* 1e-8 (reference)                                */
    int cg_max_iter;           /* 1000 (reference)                                */
    int reliable_every;        /* mixed: also an FP64 update every N iters (0 off)*/
    double reliable_delta;     /* mixed: FP64 update when |r| < delta * max |r|   */
                               /*   since the last one (0.001)                  */
    double fixed_dt;           /* > 0: fixed Euler step instead of adaptive eps   */
    int init;                  /* YK_INIT_DRAND48 (reference), YK_INIT_PHILOX     */
    int learned_layers;        /* yk_run: > 0 trains a network of that many layers */
                               /*   after thermalisation and runs the measurement  */
                               /*   steps with yk_langevin_step_learned (0: off)   */
    int pions;                 /* 1: the pion extension (fields pi_1..3 and the  */
                               /*   Yukawa term g (sigma + i gamma5 tau.pi));    */
                               /*   0: the reference's sigma-only model          */
} yk_params;

/* Parameters after the reference's conversion (main.cu:58-63, 113-170). */
typedef struct yk_action {
    double m2, lambda, kappa, sq2kappa, g, m0, r, cut_fraction, eps_bar;
    int drift_mode, use_mass;
} yk_action;

typedef struct yk_solve_stats {
    int iterations;            /* CG iterations (summed over right-hand sides)   */
    int reliable_updates;      /* FP64 residual recomputations (mixed)           */
    double rr;                 /* final |r|^2 of the solver                      */
    double rr0;                /* |b|^2                                          */
    int converged;             /* 1 if every system met its stopping rule        */
} yk_solve_stats;

/* Per-chain observables of the last step (langevin_gpu_v2.cu:65-118,
 * reductions.cu:106-140, 200-233). */
typedef struct yk_obs {
    double t;                  /* Langevin time accumulated by yk_langevin_step  */
    double eps;                /* step size of the last step                      */
    double max_drift;          /* clamped max |drift| of the last step            */
    double sum_phi;            /* sum_n sigma_n after the step                   */
    double sum_phi2;           /* sum_n sigma_n^2                                 */
    double sum_force;          /* sum_n F_n of the step's fermion force          */
    int64_t steps;             /* steps taken by this chain                       */
    int cg_iterations;         /* CG iterations of the last step                  */
    int64_t cg_iterations_total; /* CG iterations of all steps of this chain       */
    int64_t noconv_steps;      /* steps whose CG hit its iteration cap            */
    int status;                /* yk_status of the last step                      */
    double sum_pi[3];          /* pion extension: sum_n pi_a(n) after the step    */
    double sum_pi2;            /*   sum_n |pi(n)|^2 (zero without pions)          */
} yk_obs;

typedef struct yk_ctx yk_ctx;

const char* yk_last_error(void);
const char* yk_version(void);

/* ---------------------------------------------------------------- params */
/* Defaults of code/input.toml and code/src/params.h. */
void yk_params_default(yk_params* p);
/* Parse an input.toml (code/src/main.cu:112-170; [lattice] and [gpu] optional). */
int yk_params_from_toml(const char* path, yk_params* p);
/* main.cu:58-63 FindKappa and main.cu:113-170 conversion. */
int yk_derive_action(const yk_params* p, yk_action* a);

/* --------------------------------------------------------------- context */
/* One context holds n_chains independent chains (each with its own size and
 * couplings, params[c]).  Replaces the reference's global __constant__
 * parameter set (main.cu:268-278) and the objects built at main.cu:172-242. */
int yk_ctx_create(const yk_params* params, int n_chains, yk_ctx** ctx);
int yk_ctx_destroy(yk_ctx* ctx);
int yk_ctx_set_stream(yk_ctx* ctx, void* cuda_stream);
/* Waits for the context's stream; reports device-side wait timeouts. */
int yk_ctx_synchronize(yk_ctx* ctx);
int yk_ctx_n_chains(const yk_ctx* ctx);
int yk_ctx_volume(const yk_ctx* ctx, int chain);
int yk_ctx_shape(const yk_ctx* ctx, int chain, int* Nt, int* Nx);
/* Scalar field sigma of a chain (main.cu:92-95 initial field).  Host pointers. */
int yk_set_field_host(yk_ctx* ctx, int chain, const double* phi);
int yk_get_field_host(yk_ctx* ctx, int chain, double* phi);
/* Device pointer of the chain's field (V doubles), owned by the context. */
int yk_field_device(yk_ctx* ctx, int chain, double** phi);

/* Pion extension (no reference counterpart: the reference's model has the one
 * scalar sigma, code/src/params.h:25, and the real Yukawa diagonal g sigma,
 * Dirac.cu:57-69).  A context created with params.pions = 1 (every chain)
 * carries three more fields pi_1..3 per chain, initialised iid
 * Uniform[-1, 1] from Philox (stream kind 0, rhs a) unless init is
 * YK_INIT_NONE (zeros), and the Yukawa term becomes
 * g (sigma + i gamma5 tau.pi) with gamma5 = -i gamma_t gamma_x = sigma_2 on
 * spin and the Pauli matrices tau on flavour; D^dag carries
 * g (sigma - i gamma5 tau.pi).  With pions:
 *   - yk_dirac_apply, yk_cg_solve and yk_correlator use that operator;
 *   - yk_fermion_force writes 4V doubles: F_sigma, F_pi1, F_pi2, F_pi3,
 *     F_a(n) = -g Re sum_c conj(chi_c) (dD/dphi_a(n) / g eta)_c;
 *   - yk_langevin_step moves the four fields, each with its own coloured
 *     noise (Philox kind 1, rhs a), by the drift
 *     F_a + phi_a (m^2 + lambda/6 |phi|^2) - Lap phi_a, with max|drift| over
 *     the four fields in the adaptive step; yk_obs gains sum_pi, sum_pi2;
 *   - the learned preconditioner, yk_euler_update and the kernel profile
 *     (real sigma-only operator) return YK_EINVAL.
 * At pi = 0 the operator is the reference's, bit for bit.
 * pi: 3V doubles, component-major (pi[a*V + n]); host buffers. */
int yk_set_pions_host(yk_ctx* ctx, int chain, const double* pi);
int yk_get_pions_host(yk_ctx* ctx, int chain, double* pi);
/* Device pointer of the chain's pions (3V doubles), owned by the context. */
int yk_pions_device(yk_ctx* ctx, int chain, double** pi);

/* ------------------------------------------------------------- operators */
/* DiracOP<double>::applyD(in, out, MatrixType) (code/src/Dirac.cuh:22,
 * Dirac.cu:23-35): out = D in or D^dag in with sigma = the chain's field.
 * precision YK_FP64: double2 buffers; YK_FP32: float2 buffers. */
int yk_dirac_apply(yk_ctx* ctx, int chain, const void* in, void* out, int dagger, int precision);

/* CGsolver::solve(in, out, D, MatrixType) (code/src/CGsolver.cuh:36,
 * CGsolver.cu:42-59): solve A x = b with A = D^dag D (YK_DAGGER) or D D^dag
 * (YK_NORMAL), x0 = 0.  b and x are FP64 complex.  precision YK_FP64 runs the
 * reference's plain CG; YK_MIXED runs FP32 iterations with FP64 reliable
 * updates and an FP64 final residual check.  Returns YK_ENOCONV if the cap
 * is hit (the reference stops silently, CGsolver.cu:107). */
int yk_cg_solve(yk_ctx* ctx, int chain, const void* b, void* x, int mtype, double tol,
                int tol_mode, int max_iter, int precision, yk_solve_stats* stats);

/* No reference counterpart: the FP64 solve of yk_cg_solve for callers that
 * cannot allocate device memory (cudaMalloc / cudaFree can synchronise the
 * whole device and stall other streams, and hosts that embed the solver with
 * a fixed device-memory budget must not grow it).  No context: sigma (V
 * doubles), b and x (4V FP64 complex) are the caller's device buffers and
 * m0, g, r the Dirac parameters of yk_action; the work runs on `stream`
 * (a cudaStream_t, NULL = legacy stream) and the call returns after it.
 * The scratch is one fixed device array sized for V = Nt*Nx <= 16384 sites;
 * larger lattices return YK_EINVAL.  Calls that overlap in time share that
 * array and race.  Make the first call on a device before any stream capture
 * (it looks the array's address up once per device, and again after a
 * cudaDeviceReset has replaced the device's context). */
int yk_cg_solve_static(const double* sigma, int Nt, int Nx, double m0, double g, double r,
                       const void* b, void* x, int mtype, double tol, int tol_mode, int max_iter,
                       void* stream, yk_solve_stats* stats);

/* Learned preconditioner (no reference counterpart; the reference solves with
 * plain CG, code/src/CGsolver.cu:72-170).  Per chain, a linear convolutional
 * network z = M(r) = skip r + N(r) on the chain's lattice, for the real
 * (one-plane) fields of the Langevin step; N: input channels (r, sigma r),
 * `layers` 3x3 convolutions with the fermions' antiperiodic time wrap, 8
 * hidden channels, 4 outputs, weights [layer][tap 9][in][out] FP32.  The skip
 * term keeps every direction of the residual in M(r), so a flexible Krylov
 * method never stalls on directions N nearly annihilates.  Trained on the GPU from (residual,
 * error) pairs that the chain's own CG solves generate, and used in a
 * flexible GCR inside FP64 iterative refinement; a learned solve returns
 * YK_OK only when its FP64 true residual meets the tolerance. */
typedef struct yk_net_train_cfg {
    int n_sources;             /* Philox right-hand sides (streams 100 + i)     */
    int n_levels;              /* CG iterates per source: after base_iter * 2^k */
    int base_iter;             /*   iterations, k < n_levels                    */
    int steps;                 /* Adam steps                                    */
    int batch;                 /* pairs per step                                */
    double lr;                 /* Adam learning rate                            */
    uint64_t seed;             /* batch order                                   */
} yk_net_train_cfg;

typedef struct yk_net_train_stats {
    int pairs;                 /* training pairs generated                      */
    double loss0, loss1;       /* mean (Mr-e)^T A (Mr-e) / e^T A e, before/after */
    double ms;                 /* wall time of pair generation and training     */
} yk_net_train_stats;

/* Creates (or replaces) chain's network with `layers` (2..8) layers, the
 * skip weight `skip` (< 0: 1 / (4r + |m0| + 2)^2, a Richardson step of D^dag D)
 * and deterministic initial weights from `seed`, N starting small next to the
 * skip term. */
int yk_net_setup(yk_ctx* ctx, int chain, int layers, uint64_t seed, double skip);
/* Number of weights of chain's network (0 without one). */
int yk_net_size(yk_ctx* ctx, int chain);
/* Copies the weights to (set = 0) or from (set = 1) host memory. */
int yk_net_weights(yk_ctx* ctx, int chain, float* host, int set);
/* z = M(r) for device r, z (4V floats each, site-major), sigma the chain's field. */
int yk_net_apply(yk_ctx* ctx, int chain, const float* r, float* z);
/* As yk_net_apply, through the BF16 tensor-core convolutions (FP32
 * accumulation) that yk_fgcr_solve, yk_pcg_solve and
 * yk_langevin_step_learned apply. */
int yk_net_apply_tc(yk_ctx* ctx, int chain, const float* r, float* z);
/* Weight gradient (host, yk_net_size floats) and value of the training loss
 * (M r - e)^T A (M r - e) = |D (M r - e)|^2 for device r, e (4V floats
 * each): the energy norm of the error left by the correction M r. */
int yk_net_grad(yk_ctx* ctx, int chain, const float* r, const float* e, float* grad, double* loss);
/* Generates training pairs with the chain's CG (the context's solver and
 * tolerance) and trains the chain's network with Adam. */
int yk_net_train(yk_ctx* ctx, int chain, const yk_net_train_cfg* cfg, yk_net_train_stats* stats);
/* Solves (D^dag D) x = b for real fields (b, x: 4V doubles, device) by
 * flexible GCR with the chain's network (use_net = 1) or the identity
 * (use_net = 0) as preconditioner, inside FP64 iterative refinement; stops
 * at the tolerance rule of yk_cg_solve or after max_iter FGCR iterations.
 * stats->iterations counts preconditioner applications, reliable_updates the
 * FP64 refinement rounds. */
int yk_fgcr_solve(yk_ctx* ctx, int chain, const double* b, double* x, double tol, int tol_mode, int max_iter,
                  int use_net, yk_solve_stats* stats);
/* As yk_fgcr_solve, by flexible preconditioned CG (the network's
 * M = s I + N^T N is symmetric positive definite): FP32 vectors, alpha and
 * beta computed on the device (the host reads |r|^2 every 8 iterations),
 * inside FP64 iterative refinement.  Each inner FP32 solve reduces the
 * residual by 1e-4 or 1e-5, chosen per network by timing its first solves
 * (environment YK_PCG_INNER fixes it). */
int yk_pcg_solve(yk_ctx* ctx, int chain, const double* b, double* x, double tol, int tol_mode, int max_iter,
                 int use_net, yk_solve_stats* stats);

/* No reference counterpart (failure detection): runs on `stream` (NULL =
 * legacy stream) a two-block kernel in which block 0 waits, through the
 * persistent CG's neighbour synchronisation, on a flag that block 1 never
 * sets.  The wait gives up after its bound (about 2 s), records YK_ETIMEOUT
 * and the kernel returns; *status receives the recorded device status.
 * Returns YK_ETIMEOUT when the wait ran out as designed (the device stays
 * usable), YK_OK if it did not, YK_ECUDA on a CUDA error. */
int yk_check_wait_timeout(void* stream, int* status);

/* FermionicDrift::getForce (code/src/FermionicDrift.cuh:15, FermionicDrift.cu:57-100):
 * F_n = -g Re sum_c conj(chi_{n,c}) eta_{n,c}, chi = D (D^dag D)^-1 eta, averaged
 * over the chain's n_rhs right-hand sides; eta (n_rhs * 4V FP64 complex, device)
 * may be NULL, then it is drawn from Philox at the chain's current step.
 * F: V doubles, device. */
int yk_fermion_force(yk_ctx* ctx, int chain, const void* eta, double* F, yk_solve_stats* stats);

/* ColouredNoise::operator() (code/src/colouredNoise.h:33, colouredNoise.cpp:155-178):
 * xi = Z2D(mask * D2Z(w)) with the sharp cutoff mask.  white: V doubles
 * (device) or NULL to draw w from Philox at the chain's current step. */
int yk_coloured_noise(yk_ctx* ctx, int chain, const double* white, double* xi);

/* n_steps Langevin steps of every chain (main.cu:370-381: noise, force,
 * Run kernel langevin_gpu_v2.cu:65-118), fully on the device; the step
 * graph is captured once and replayed. */
int yk_langevin_step(yk_ctx* ctx, int n_steps);

/* One Langevin step of every chain with chain `chain`'s host I/O in one call
 * (the per-step host exchange of main.cu:370-381, which copies eps to the host
 * every step): the field uploaded from phi_in (V doubles, host; NULL keeps the
 * device field), the step, the field downloaded to phi_out (NULL: not read) and
 * the observables to obs (NULL: not read), with one synchronisation at the end
 * (the buffers may be reused when the call returns).  With pinned buffers
 * (or NULL), after the first step, the call is one graph launch: the upload,
 * the step, the downloads and the error word, the transfers made by kernels
 * on the mapped buffers; one graph is kept per (chain, phi_in, phi_out), the
 * last four. */
int yk_langevin_step_io(yk_ctx* ctx, int chain, const double* phi_in, double* phi_out, yk_obs* obs);

/* The autotuner (no reference counterpart: the reference's launch shapes are
 * fixed, main.cu:258-266).  Batched contexts (several CG systems per step):
 * the grid of the step's persistent CG, i.e. how many 256-site tiles each
 * block owns, chosen by timing the step's CG at candidate grids (the
 * co-resident maximum, 3/4 and 1/2 of it, one block per SM, half of that).
 * Where the step's coloured noise and the next step's sources run -- on an
 * auxiliary stream beside the CG, on the SMs the CG's grid leaves free, or on
 * the main stream after the CG -- is chosen by timing whole steps of both forms
 * (the chains' state restored after each).  The learned solver's convolution
 * tile (rows x columns) is chosen by timing candidates on the network's first
 * solve.  Results never depend on either
 * choice.  yk_langevin_step tunes automatically before it captures the step
 * graph (environment YK_AUTOTUNE=0 at context creation: not automatically);
 * yk_autotune tunes now (dropping a captured graph) and reports. */
typedef struct yk_tune_result {
    int cg_grid;               /* chosen grid of the batched step CG (0: not tuned)   */
    int cg_grid_max;           /* the co-resident maximum                            */
    int cg_candidates;         /* candidates timed                                   */
    float cg_ms_chosen;        /* two timed 48-iteration solves at the chosen grid   */
    float cg_ms_max;           /* the same at the co-resident maximum                */
    int conv_rows, conv_cols;  /* chain 0 network's convolution tile (0: none yet)   */
    int conv_layers_per_launch; /* its layers per launch (1 .. 2 x layers)           */
    double pcg_inner_tol;      /* its PCG's inner tolerance, chosen by timing (0: undecided) */
    int noise_overlap;         /* the step's noise and next sources: 1 on an auxiliary stream */
                               /*   beside the CG, 0 on the main stream after it, -1 untuned  */
    float step_ms_overlap, step_ms_serial;   /* two timed steps of each form            */
} yk_tune_result;
int yk_autotune(yk_ctx* ctx, yk_tune_result* out);
/* (Environment YK_NET_TILE=RxW or RxWxG, e.g. 8x64x4, fixes the convolution
 * tile and the layers per launch instead of timing candidates: for profiling
 * and reproducible timing.) */
/* The last tuning's choices (all zero before any). */
int yk_tune_report(yk_ctx* ctx, yk_tune_result* out);

/* As yk_langevin_step, with every fermion solve of the step done by
 * yk_pcg_solve (flexible preconditioned CG inside FP64 refinement, to the
 * context's tolerance) with the chain's network (use_net = 1; every chain
 * with fermions needs one, see yk_net_setup) or the identity (use_net = 0).
 * The same sources, force, update and observables as yk_langevin_step; the
 * solves are driven from the host (not a captured graph).  stats (may be
 * NULL) sums the solver statistics over the steps' solves.  No reference
 * counterpart: the reference solves with plain CG (CGsolver.cu:72-170). */
int yk_langevin_step_learned(yk_ctx* ctx, int n_steps, int use_net, yk_solve_stats* stats);

/* The Run kernel (code/src/langevin_gpu_v2.cu:65-118, launched at main.cu:377)
 * on injected inputs: drift = force + phi (m^2 + lambda/6 phi^2) - Lap phi,
 * eps = epsBar*30/clamp(max|drift|) (or fixed_dt), phi -= eps drift +
 * sqrt(2 eps) xi.  force, xi: V doubles (device).  Advances the chain's step
 * counter and Langevin time like yk_langevin_step; obs may be NULL. */
int yk_euler_update(yk_ctx* ctx, int chain, const double* force, const double* xi, yk_obs* obs);

/* Kernel timing of yk_langevin_step: between begin and end the step runs as
 * direct launches bracketed by CUDA events on the context's stream (instead
 * of the captured graph); end sums the device time per kernel class. */
typedef struct yk_profile {
    int steps;                   /* Langevin steps profiled                       */
    int launches;                /* kernels launched by those steps               */
    int cg_launches;             /* persistent CG launches                        */
    int cg_grid;                 /* blocks of the last CG launch                  */
    int cg_kernel;               /* its kernel: 0 grid-wide, 1 halo, 2 cluster,   */
                                 /*   3 even-odd (Schur complement), 4 batched    */
                                 /*   even-odd (work dealt out per pass), 5       */
                                 /*   batched even-odd over 32 x 16 patches       */
    double noise_ms, cg_ms, force_ms, update_ms;   /* summed device time          */
    int64_t cg_iterations;       /* CG iterations, summed over systems            */
    int64_t cg_site_iterations;  /* sum over chains of iterations x volume        */
    int64_t sites;               /* sum of the chains' volumes                    */
} yk_profile;
int yk_profile_begin(yk_ctx* ctx);
int yk_profile_end(yk_ctx* ctx, yk_profile* out);

/* Host copy of a chain's last-step observables (synchronises the stream). */
int yk_observables(yk_ctx* ctx, int chain, yk_obs* obs);

/* gpuTimeSlices (reductions.cu:65-104): slices[t] = sum_x sigma(t, x); host out (Nt). */
int yk_time_slices(yk_ctx* ctx, int chain, double* slices_host);

/* Point-source fermion correlator (main.cu:441-469 + reductions.cu:176-191):
 * y = D^dag (D D^dag)^-1 e0 with e0 = (1,1,0,0) at site 0, corr[t] = sum_x sum_c Re y;
 * host out (Nt). */
int yk_correlator(yk_ctx* ctx, int chain, double* corr_host, yk_solve_stats* stats);

/* Condensate of main.cu:471-483: a fresh force estimate, tr = sum_n F_n / g
 * (0 when g == 0); returns tr / V in *cond. */
int yk_condensate(yk_ctx* ctx, int chain, double* cond, yk_solve_stats* stats);

/* Langevin time-step control of main.cu:325-352: set the averageEpsilon used
 * by the adaptive rule eps = epsBar * 30 / max|drift|. */
int yk_set_eps_bar(yk_ctx* ctx, int chain, double eps_bar);
int yk_get_step(yk_ctx* ctx, int chain, int64_t* step);
int yk_set_step(yk_ctx* ctx, int chain, int64_t step);
int yk_set_time(yk_ctx* ctx, int chain, double t);

/* Checkpoint / resume of one chain: field, Philox step counter, Langevin time
 * and epsBar in a small binary file.  The reference parses io.startFileName
 * and io.resume (main.cu:146-157) but never reads or writes a configuration. */
int yk_checkpoint_save(yk_ctx* ctx, int chain, const char* path, double eps_bar);
int yk_checkpoint_load(yk_ctx* ctx, int chain, const char* path, double* eps_bar);

/* --------------------------------------------------------------- analysis */
/* Wolff Gamma-method (analysis/AutoCorrelation/ac.cpp:73-181, Wrapper :183-190):
 * out = {mean, error, error of error, tau_int, tau_int error}; host buffers. */
int yk_gamma_method(const double* data, int64_t n, double stau, double* out5);

/* Observables of a time series of per-configuration <sigma> values with
 * Gamma-method errors, computed on the GPU (the reference analyses its
 * traces.csv offline: analysis/functions.py:42-78 with the Gamma-method of
 * analysis/AutoCorrelation/ac.cpp:73-181).  Each entry holds {value, error,
 * error of the error, tau_int, tau_int error}:
 *   sigma      <s>                                  (functions.py:42-45)
 *   abs_sigma  <|s|>                                (:47-49)
 *   chi        V <(s - <s>)^2>, error of that mean  (:54-57)
 *   binder     1 - <s^4> / (3 <s^2>^2), Wolff's derived-quantity error
 *              (U. Wolff, Comput. Phys. Commun. 156 (2004) 143)  (:73-78)
 * Gamma(t) is summed on the device for t <= min(n / 2, 8192). */
typedef struct yk_series_stats {
    int64_t n;
    double sigma[5];
    double abs_sigma[5];
    double chi[5];
    double binder[5];
} yk_series_stats;
/* Records <sigma> = sum_n sigma_n / V after every step of the chain (the
 * update kernel appends it on the device; graph-replayed steps included) into
 * a new device series of `capacity` values; capacity 0 stops and frees. */
int yk_series_record(yk_ctx* ctx, int chain, int64_t capacity);
/* Copies the recorded values (at most cap) to host memory; *n = how many.
 * host == NULL: *n = the number of values recorded so far. */
int yk_series_read(yk_ctx* ctx, int chain, double* host, int64_t cap, int64_t* n);
/* yk_series_stats of the recorded series (stau: Wolff's S_tau, 1.5). */
int yk_series_analyse(yk_ctx* ctx, int chain, double stau, yk_series_stats* out);
/* The same analysis of a host series of n values on a volume-site lattice
 * (e.g. the sigma column of a traces.csv); runs on the current device. */
int yk_series_analyse_host(const double* series, int64_t n, int64_t volume, double stau, yk_series_stats* out);

/* The full reference run protocol of main.cu:73-516 (burn-in, epsBar
 * measurement, export loop, slice.dat / data.csv / traces.csv and stdout)
 * from an input.toml; files are written into out_dir. */
int yk_run_toml(const char* toml_path, const char* out_dir);

#ifdef __cplusplus
}
#endif
#endif /* YUKAWA_GB300_H */
