/*
 * yukawa_oracle.h -- CPU FP64 restatement of the Langevin hot path of
 * Matteo294/YukawaColouredNoise (code/src/*.cu).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may call it; the
 * product library (libyukawa_gb300.so) never links, loads or calls it.
 *
 * Conventions (identical to the reference):
 *   site n = t*Nx + x                               (code/src/Lattice.cu:16-18)
 *   spinor = 4 complex per site, order [f1s1, f1s2, f2s1, f2s2],
 *            stored as interleaved (re, im) doubles  (code/src/Spinor.cuh:7-16)
 *   half spectrum for the r2c mask: Nt x (Nx/2+1), row-major
 *                                                    (code/src/colouredNoise.cpp:138-145)
 */
#ifndef YUKAWA_ORACLE_H
#define YUKAWA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters after the reference's input.toml conversion (main.cu:113-170). */
typedef struct yko_action {
    double m2;          /* bare mass^2 in the bosonic drift        */
    double lambda;      /* quartic coupling (drift uses lambda/6)  */
    double kappa;       /* hopping parameter (derived or given)    */
    double sq2kappa;    /* sqrt(2 kappa): output rescale           */
    double g;           /* Yukawa coupling used by D and the force */
    double m0;          /* bare fermion mass                       */
    double r;           /* Wilson parameter                        */
    double cut_fraction;
    double eps_bar;     /* averageEpsilon                          */
    int drift_mode;     /* 0 normal, 1 rescaled (x cutFraction^2)  */
    int use_mass;       /* useMass == "true"                       */
} yko_action;

/* main.cu:58-63 FindKappa + main.cu:113-170 parameter derivation. */
void yko_derive(int use_mass, double mass, double g_phys, double kappa, double lambda_in,
                double yukawa_in, double fermion_mass, double wilson, double cut_fraction,
                double average_epsilon, int drift_mode, yko_action* out);

/* Dirac.cu:37-70 (diagonal) + Dirac.cu:144-190 (hopping): out = D in (dagger=0) or D^dag in. */
void yko_dirac(int Nt, int Nx, const yko_action* a, const double* sigma,
               const double* in, double* out, int dagger);

/* CGsolver.cu:72-170: CG on D^dag D (mtype=1, "Dagger") or D D^dag (mtype=0, "Normal").
 * tol_mode 0: stop when sqrt(|r|^2) <= tol (reference rule), 1: sqrt(|r|^2) <= tol*|b|.
 * Returns the iteration count; *final_rr receives |r|^2 of the recursive residual. */
int yko_cg(int Nt, int Nx, const yko_action* a, const double* sigma, const double* b,
           double* x, int mtype, double tol, int tol_mode, int max_iter, double* final_rr);

/* FermionicDrift.cu:57-80 + :83-100: F_n = -g Re sum_c conj(chi_{n,c}) eta_{n,c},
 * chi = D (D^dag D)^-1 eta; times cutFraction^2 in rescaled mode.
 * n_rhs right-hand sides (eta has n_rhs*4V complex), averaged. Returns summed CG iterations. */
int yko_force(int Nt, int Nx, const yko_action* a, const double* sigma, const double* eta,
              int n_rhs, double tol, int tol_mode, int max_iter, double* F);

/* colouredNoise.cpp:16-29 + :138-145: the r2c half-spectrum mask, 1/V or 0. */
void yko_mask_half(int Nt, int Nx, double cut_fraction, double* mask);
/* 1 if every mode passes the cut (the filter is the identity). */
int yko_mask_all_kept(int Nt, int Nx, double cut_fraction);

/* Unnormalised 2-D complex DFT in place (sign -1 forward, +1 inverse). */
void yko_fft2(int Nt, int Nx, double* data, int sign);

/* colouredNoise.cpp:155-178: xi = Z2D(mask * D2Z(w)), w real. */
void yko_coloured_noise(int Nt, int Nx, double cut_fraction, const double* white, double* xi);

/* langevin_gpu_v2.cu:9-27 (PotentialAndMass) + :41-63 (gpuSpMV): drift += dV/dphi - Lap phi. */
void yko_bosonic_drift(int Nt, int Nx, double m2, double lambda, const double* phi, double* drift);

/* langevin_gpu_v2.cu:65-118 (Run): max|drift| clamp, adaptive eps, Euler update.
 * fixed_dt > 0 selects a fixed step instead of the adaptive rule.
 * Returns the eps used; *max_drift receives the clamped maximum. */
double yko_euler_update(int V, double eps_bar, double fixed_dt, double* phi, const double* drift,
                        const double* noise, double* max_drift);

/* reductions.cu:106-140, :65-104, :176-191, :200-233 */
double yko_sum(int n, const double* v);
void yko_time_slices(int Nt, int Nx, const double* phi, double* slices);
void yko_time_slices_spinor(int Nt, int Nx, const double* psi, double* corr);

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the framework's counter scheme. */
void yko_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Normals 0 .. n-1 of a stream: FP32 Box-Muller, normals 4e .. 4e+3 from counter e. */
void yko_normals(uint64_t seed, uint32_t chain, uint64_t step, uint32_t kind, uint32_t rhs,
                 int64_t n, double* out);
/* One pair of yko_normals from explicit Philox words a (radius), b (angle). */
void yko_normal_pair_words(uint32_t a, uint32_t b, double out[2]);
/* The GPU even-odd kernels' float-float arithmetic (accuracy tests only):
   sum, product and reciprocal of float-float splits of a[i], b[i]; one site
   of the half hop in float-float. */
void yko_ff_ops(int64_t n, const double* a, const double* b, double* sum, double* prod, double* rcp);
void yko_ff_hop(int dag, int mode, double r, const double* c, double diag, const double* tu, const double* td,
                const double* xu, const double* xd, double sp, double sm, double* out);
/* The same words through FP64 libm Box-Muller (accuracy check of yko_normals). */
void yko_normals_fp64(uint64_t seed, uint32_t chain, uint64_t step, uint32_t kind, uint32_t rhs,
                      int64_t n, double* out);
void yko_uniform_field(uint64_t seed, uint32_t chain, int64_t n, double* out);
void yko_uniform_field_comp(uint64_t seed, uint32_t chain, uint32_t comp, int64_t n, double* out);
/* The reference's initial field 1 - 2*drand48() from glibc's default drand48 state (main.cu:92-95). */
void yko_drand48_field(int64_t n, double* out);

/* One full Langevin step of the framework (noise kind 1, fermion noise kind 2,
 * step counter `step`).  Writes phi in place; returns eps; fills obs[0..5] =
 * {eps, max_drift, sum phi, sum F, cg_iters, sum phi^2}. */
double yko_langevin_step(int Nt, int Nx, const yko_action* a, uint64_t seed, uint32_t chain,
                         uint64_t step, int n_rhs, double tol, int tol_mode, int max_iter,
                         double fixed_dt, double* phi, double* obs);

/* Pion extension (no reference counterpart; the reference is sigma-only,
 * params.h:25, Dirac.cu:57-69): Yukawa term g (sigma + i gamma5 tau.pi),
 * gamma5 = -i gamma_t gamma_x = sigma_2, pi = 3 fields of V doubles
 * (component-major).  pi == NULL gives the sigma-only operator. */
void yko_dirac_pi(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi,
                  const double* in, double* out, int dagger);
int yko_cg_pi(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi, const double* b,
              double* x, int mtype, double tol, int tol_mode, int max_iter, double* final_rr);
/* F4: 4V doubles: F_sigma, F_pi1, F_pi2, F_pi3 (see yukawa_oracle.c). */
int yko_force_pi(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi, const double* eta,
                 int n_rhs, double tol, int tol_mode, int max_iter, double* F4);
/* One step of the four fields phi4 = (sigma, pi1, pi2, pi3); obs[0..9]. */
double yko_langevin_step_pi(int Nt, int Nx, const yko_action* a, uint64_t seed, uint32_t chain,
                            uint64_t step, int n_rhs, double tol, int tol_mode, int max_iter,
                            double fixed_dt, double* phi4, double* obs);

/* Wolff's Gamma-method (U. Wolff, Comput. Phys. Commun. 156 (2004) 143), S_tau = 1.5:
 * out = {mean, error, error_of_error, tau_int, tau_int_error}. */
void yko_gamma_method(const double* data, int64_t n, double stau, double out[5]);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int yko_threads(void);

#ifdef __cplusplus
}
#endif
#endif
