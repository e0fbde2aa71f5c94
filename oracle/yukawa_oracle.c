/*
 * yukawa_oracle.c -- CPU FP64 restatement of the Langevin hot path of
 * Matteo294/YukawaColouredNoise.  Every function cites the reference lines it
 * follows (paths relative to the reference project).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  The product library never links or calls this file.
 *
 * The reference has no CPU path (all of it is CUDA on managed memory); this is
 * a restatement of its arithmetic in plain C with OpenMP over sites.  Complex
 * numbers are interleaved (re, im) doubles, as thrust::complex<double> is laid
 * out in the reference.
 */
#include "yukawa_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int yko_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Parameters: main.cu:58-63 (FindKappa), main.cu:113-170 (conversion).       */
/* ------------------------------------------------------------------------- */
static double find_kappa(double m2, double lambda0)
{
    /* main.cu:58-63, nDim = 2 */
    const double nd2 = 2.0 * 2.0;
    const double delta = (nd2 + m2) * (nd2 + m2) + 4.0 * lambda0 / 3.0;
    return (-(nd2 + m2) + sqrt(delta)) / (2.0 * lambda0 / 3.0);
}

void yko_derive(int use_mass, double mass, double g_phys, double kappa, double lambda_in,
                double yukawa_in, double fermion_mass, double wilson, double cut_fraction,
                double average_epsilon, int drift_mode, yko_action* out)
{
    memset(out, 0, sizeof(*out));
    if (use_mass) {
        /* main.cu:117-122: m2 = mass, lambda = g, kappa from FindKappa */
        out->m2 = mass;
        out->lambda = g_phys;
        out->kappa = find_kappa(mass, g_phys);
    } else {
        /* main.cu:123-129 */
        out->kappa = kappa;
        out->m2 = (1.0 - 2.0 * lambda_in) / kappa - 2.0 * 2.0;
        out->lambda = 6.0 * lambda_in / (kappa * kappa);
    }
    out->sq2kappa = sqrt(2.0 * out->kappa);                         /* main.cu:130 */
    out->g = use_mass ? yukawa_in : yukawa_in / out->sq2kappa;       /* main.cu:166-169 */
    out->m0 = fermion_mass;                                          /* main.cu:163 */
    out->r = wilson;                                                 /* main.cu:164 */
    out->cut_fraction = cut_fraction;                                /* main.cu:131 */
    out->eps_bar = average_epsilon;                                  /* main.cu:137 */
    out->drift_mode = drift_mode;                                    /* main.cu:170 */
    out->use_mass = use_mass;
}

/* ------------------------------------------------------------------------- */
/* Wilson-Dirac operator: Dirac.cu:37-70 (zero, diagonal) + :144-190 (hops).  */
/* ------------------------------------------------------------------------- */
void yko_dirac(int Nt, int Nx, const yko_action* a, const double* sigma,
               const double* in, double* out, int dagger)
{
    const double r = a->r;
    const int V = Nt * Nx;
#pragma omp parallel for schedule(static)
    for (int n = 0; n < V; ++n) {
        const int t = n / Nx, x = n % Nx;                      /* Lattice.cu:26-30 */
        const int tu = ((t + 1) % Nt) * Nx + x;                /* Dirac.cu:10-21   */
        const int td = ((t - 1 + Nt) % Nt) * Nx + x;
        const int xu = t * Nx + (x + 1) % Nx;
        const int xd = t * Nx + (x - 1 + Nx) % Nx;
        /* antiperiodic time: Dirac.cu:161-162 */
        const double s0 = (t == Nt - 1) ? -1.0 : 1.0;   /* hop to n + t   */
        const double s1 = (t == 0) ? -1.0 : 1.0;        /* hop to n - t   */
        const double diag = 2.0 * r + a->m0 + a->g * sigma[n];  /* Dirac.cu:52-69 */
        for (int f = 0; f < 2; ++f) {
            for (int k = 0; k < 2; ++k) {   /* k: real / imaginary plane */
#define U(m) in[((m) * 4 + 2 * f + 0) * 2 + k]
#define Dn(m) in[((m) * 4 + 2 * f + 1) * 2 + k]
                double hu, hd;
                if (!dagger) {
                    /* Dirac.cu:165-174 */
                    hu = -s1 * 0.5 * (r + 1.0) * U(td) - s0 * 0.5 * (r - 1.0) * U(tu)
                         - 0.5 * (r * U(xu) - Dn(xu)) - 0.5 * (r * U(xd) + Dn(xd));
                    hd = -s1 * 0.5 * (r - 1.0) * Dn(td) - s0 * 0.5 * (r + 1.0) * Dn(tu)
                         + 0.5 * (U(xu) - r * Dn(xu)) - 0.5 * (U(xd) + r * Dn(xd));
                } else {
                    /* Dirac.cu:175-185 */
                    hu = -s0 * 0.5 * (r + 1.0) * U(tu) - s1 * 0.5 * (r - 1.0) * U(td)
                         - 0.5 * (r * U(xd) - Dn(xd)) - 0.5 * (r * U(xu) + Dn(xu));
                    hd = -s0 * 0.5 * (r - 1.0) * Dn(tu) - s1 * 0.5 * (r + 1.0) * Dn(td)
                         + 0.5 * (U(xd) - r * Dn(xd)) - 0.5 * (U(xu) + r * Dn(xu));
                }
                out[(n * 4 + 2 * f + 0) * 2 + k] = diag * U(n) + hu;
                out[(n * 4 + 2 * f + 1) * 2 + k] = diag * Dn(n) + hd;
#undef U
#undef Dn
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Pion extension (no reference counterpart: the reference is sigma-only,     */
/* params.h:25 nVectorComponents = 1, diagonal Dirac.cu:57-69).  The Yukawa   */
/* term becomes g (sigma + i gamma5 tau.pi) with gamma5 = -i gamma_t gamma_x  */
/* = sigma_2 on spin (gamma_t = sigma_3, gamma_x = sigma_1 as in Dirac.cu),   */
/* so i gamma5 = [[0, 1], [-1, 0]], and tau the Pauli matrices on flavour.    */
/* D^dag carries g (sigma - i gamma5 tau.pi) (i gamma5 tau_a is              */
/* anti-Hermitian).  pi: 3 fields of V doubles, component-major pi[a*V + n].  */
/* ------------------------------------------------------------------------- */

/* out += (s1 i gamma5 tau_1 + s2 i gamma5 tau_2 + s3 i gamma5 tau_3) in at one
   site: in, out = 4 complex [f1s1, f1s2, f2s1, f2s2] as interleaved doubles */
static void pion_site_add(const double* in, double* out, double s1, double s2, double s3)
{
    /* w_f = i sigma_2 psi_f: (w_f)_0 = psi_{f,1}, (w_f)_1 = -psi_{f,0} */
    double w[2][2][2];
    for (int f = 0; f < 2; ++f)
        for (int k = 0; k < 2; ++k) {
            w[f][0][k] = in[(2 * f + 1) * 2 + k];
            w[f][1][k] = -in[(2 * f + 0) * 2 + k];
        }
    /* tau.s = [[s3, s1 - i s2], [s1 + i s2, -s3]] */
    for (int sp = 0; sp < 2; ++sp) {
        const double ar = w[0][sp][0], ai = w[0][sp][1], br = w[1][sp][0], bi = w[1][sp][1];
        /* flavour 1: s3 a + (s1 - i s2) b */
        out[(0 + sp) * 2 + 0] += s3 * ar + (s1 * br + s2 * bi);
        out[(0 + sp) * 2 + 1] += s3 * ai + (s1 * bi - s2 * br);
        /* flavour 2: (s1 + i s2) a - s3 b */
        out[(2 + sp) * 2 + 0] += (s1 * ar - s2 * ai) - s3 * br;
        out[(2 + sp) * 2 + 1] += (s1 * ai + s2 * ar) - s3 * bi;
    }
}

void yko_dirac_pi(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi,
                  const double* in, double* out, int dagger)
{
    yko_dirac(Nt, Nx, a, sigma, in, out, dagger);
    if (!pi) return;
    const int V = Nt * Nx;
    const double sg = dagger ? -a->g : a->g;
#pragma omp parallel for schedule(static)
    for (int n = 0; n < V; ++n)
        pion_site_add(in + (int64_t)n * 8, out + (int64_t)n * 8, sg * pi[n], sg * pi[V + n], sg * pi[2 * V + n]);
}

/* ------------------------------------------------------------------------- */
/* CG on D^dag D: CGsolver.cu:72-170, gpuSumSpinors :172-177,                 */
/* gpuDotProduct reductions.cu:145-174.                                        */
/* ------------------------------------------------------------------------- */
static void cdot(int64_t n, const double* a, const double* b, double* re, double* im)
{
    /* sum conj(a_i) b_i over n complex: chunks of kDotChunk entries summed in
       order (in parallel over chunks), then the chunk sums in order, so the
       result depends neither on the thread count nor on the threads' timing
       (an OpenMP reduction clause combines the threads' sums in any order) */
    enum { kDotChunk = 4096, kDotStack = 64 };
    const int64_t nc = (n + kDotChunk - 1) / kDotChunk;
    double stack_part[2 * kDotStack];
    double* part = nc <= kDotStack ? stack_part : (double*)malloc(sizeof(double) * 2 * (size_t)nc);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nc; ++c) {
        const int64_t e = (c + 1) * kDotChunk < n ? (c + 1) * kDotChunk : n;
        double sr = 0.0, si = 0.0;
        for (int64_t i = c * kDotChunk; i < e; ++i) {
            const double ar = a[2 * i], ai = a[2 * i + 1], br = b[2 * i], bi = b[2 * i + 1];
            sr += ar * br + ai * bi;
            si += ar * bi - ai * br;
        }
        part[2 * c] = sr;
        part[2 * c + 1] = si;
    }
    double sr = 0.0, si = 0.0;
    for (int64_t c = 0; c < nc; ++c) {
        sr += part[2 * c];
        si += part[2 * c + 1];
    }
    if (part != stack_part) free(part);
    *re = sr;
    *im = si;
}

/* res = s1 + c * s2 (complex c) */
static void csum(int64_t n, const double* s1, const double* s2, double* res, double cr, double ci)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double xr = s2[2 * i], xi = s2[2 * i + 1];
        const double pr = cr * xr - ci * xi, pi = cr * xi + ci * xr;
        res[2 * i] = s1[2 * i] + pr;
        res[2 * i + 1] = s1[2 * i + 1] + pi;
    }
}

static void cdiv(double a, double b, double c, double d, double* re, double* im)
{
    /* (a+ib)/(c+id), Smith's algorithm */
    if (fabs(c) >= fabs(d)) {
        const double q = d / c, den = c + d * q;
        *re = (a + b * q) / den;
        *im = (b - a * q) / den;
    } else {
        const double q = c / d, den = c * q + d;
        *re = (a * q + b) / den;
        *im = (b * q - a) / den;
    }
}

static int cg_any(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi, const double* b,
                  double* x, int mtype, double tol, int tol_mode, int max_iter, double* final_rr);

int yko_cg(int Nt, int Nx, const yko_action* a, const double* sigma, const double* b,
           double* x, int mtype, double tol, int tol_mode, int max_iter, double* final_rr)
{
    return cg_any(Nt, Nx, a, sigma, NULL, b, x, mtype, tol, tol_mode, max_iter, final_rr);
}

int yko_cg_pi(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi, const double* b,
              double* x, int mtype, double tol, int tol_mode, int max_iter, double* final_rr)
{
    return cg_any(Nt, Nx, a, sigma, pi, b, x, mtype, tol, tol_mode, max_iter, final_rr);
}

/* pi == NULL: the reference's operator exactly (yko_dirac) */
static int cg_any(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi, const double* b,
                  double* x, int mtype, double tol, int tol_mode, int max_iter, double* final_rr)
{
    const int64_t n = (int64_t)Nt * Nx * 4;   /* complex entries */
    double* r = (double*)malloc(sizeof(double) * 2 * n);
    double* p = (double*)malloc(sizeof(double) * 2 * n);
    double* t1 = (double*)malloc(sizeof(double) * 2 * n);
    double* t2 = (double*)malloc(sizeof(double) * 2 * n);
    memset(x, 0, sizeof(double) * 2 * n);            /* CGsolver.cu:83 */
    memcpy(r, b, sizeof(double) * 2 * n);            /* :90 */
    memcpy(p, b, sizeof(double) * 2 * n);            /* :92 */
    double re, im;
    cdot(n, r, r, &re, &im);
    double rmodsq = hypot(re, im);                   /* :100 abs(dot) */
    const double stop = (tol_mode == 0) ? tol : tol * sqrt(rmodsq);
    /* Mtype = Dagger (1): first D, then D^dag, i.e. A = D^dag D (:113-125) */
    const int first = (mtype == 1) ? 0 : 1;
    const int second = (mtype == 1) ? 1 : 0;
    int k;
    for (k = 0; k < max_iter && sqrt(rmodsq) > stop; ++k) {
        yko_dirac_pi(Nt, Nx, a, sigma, pi, p, t2, first);
        yko_dirac_pi(Nt, Nx, a, sigma, pi, t2, t1, second);
        cdot(n, p, t1, &re, &im);                    /* :133 */
        double ar, ai;
        cdiv(rmodsq, 0.0, re, im, &ar, &ai);         /* :137 alpha = rmodsq / <p,Ap> */
        csum(n, x, p, x, ar, ai);                    /* :143 x += alpha p */
        csum(n, r, t1, r, -ar, -ai);                 /* :148 r -= alpha Ap */
        cdot(n, r, r, &re, &im);                     /* :152 */
        const double rr = hypot(re, im);
        const double beta = rr / rmodsq;             /* :156 */
        rmodsq = rr;
        csum(n, r, p, p, beta, 0.0);                 /* :162 p = r + beta p */
    }
    if (final_rr) *final_rr = rmodsq;
    free(r); free(p); free(t1); free(t2);
    return k;
}

/* FermionicDrift.cu:57-80 (getForce) and :83-100 (computeDrift). */
int yko_force(int Nt, int Nx, const yko_action* a, const double* sigma, const double* eta,
              int n_rhs, double tol, int tol_mode, int max_iter, double* F)
{
    const int V = Nt * Nx;
    const int64_t n = (int64_t)V * 4;
    double* xs = (double*)malloc(sizeof(double) * 2 * n);
    double* chi = (double*)malloc(sizeof(double) * 2 * n);
    const double scale = (a->drift_mode == 1) ? a->cut_fraction * a->cut_fraction : 1.0;
    int iters = 0;
    for (int i = 0; i < V; ++i) F[i] = 0.0;
    for (int j = 0; j < n_rhs; ++j) {
        const double* e = eta + (int64_t)j * 2 * n;
        iters += yko_cg(Nt, Nx, a, sigma, e, xs, 1, tol, tol_mode, max_iter, NULL);
        yko_dirac(Nt, Nx, a, sigma, xs, chi, 0);     /* chi = D x */
        for (int i = 0; i < V; ++i) {
            double s = 0.0;
            for (int c = 0; c < 4; ++c) {
                const int64_t q = (int64_t)(4 * i + c) * 2;
                s += chi[q] * e[q] + chi[q + 1] * e[q + 1];   /* Re conj(chi) eta */
            }
            F[i] += -(scale * a->g) * s;
        }
    }
    if (n_rhs > 1)
        for (int i = 0; i < V; ++i) F[i] /= (double)n_rhs;
    free(xs); free(chi);
    return iters;
}

/* Pion extension of the force (no reference counterpart; the sigma part is
   FermionicDrift.cu:83-100 with the pion operator): with chi = D x and
   x = (D^dag D)^-1 eta, F_sigma(n) = -g Re sum_c conj(chi_{n,c}) eta_{n,c} and
   F_pi_a(n) = -g Re sum_c conj(chi_{n,c}) (i gamma5 tau_a eta)_{n,c}, the
   one-noise estimates of -Re tr(D^-1 dD/dphi_a(n)); averaged over the
   right-hand sides, times cutFraction^2 in rescaled mode.  F4: 4V doubles
   (sigma, pi_1, pi_2, pi_3).  pi == NULL gives the sigma-only operator (the
   pion forces are still estimated). */
int yko_force_pi(int Nt, int Nx, const yko_action* a, const double* sigma, const double* pi, const double* eta,
                 int n_rhs, double tol, int tol_mode, int max_iter, double* F4)
{
    const int V = Nt * Nx;
    const int64_t n = (int64_t)V * 4;
    double* xs = (double*)malloc(sizeof(double) * 2 * n);
    double* chi = (double*)malloc(sizeof(double) * 2 * n);
    const double scale = (a->drift_mode == 1) ? a->cut_fraction * a->cut_fraction : 1.0;
    int iters = 0;
    for (int64_t i = 0; i < 4 * (int64_t)V; ++i) F4[i] = 0.0;
    for (int j = 0; j < n_rhs; ++j) {
        const double* e = eta + (int64_t)j * 2 * n;
        iters += cg_any(Nt, Nx, a, sigma, pi, e, xs, 1, tol, tol_mode, max_iter, NULL);
        yko_dirac_pi(Nt, Nx, a, sigma, pi, xs, chi, 0);     /* chi = D x */
        for (int i = 0; i < V; ++i) {
            const double* ch = chi + (int64_t)i * 8;
            const double* es = e + (int64_t)i * 8;
            double s = 0.0;
            for (int c = 0; c < 4; ++c) s += ch[2 * c] * es[2 * c] + ch[2 * c + 1] * es[2 * c + 1];
            F4[i] += -(scale * a->g) * s;
            for (int q = 0; q < 3; ++q) {
                double u[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                pion_site_add(es, u, q == 0 ? 1.0 : 0.0, q == 1 ? 1.0 : 0.0, q == 2 ? 1.0 : 0.0);
                double sq = 0.0;
                for (int c = 0; c < 4; ++c) sq += ch[2 * c] * u[2 * c] + ch[2 * c + 1] * u[2 * c + 1];
                F4[(int64_t)(q + 1) * V + i] += -(scale * a->g) * sq;
            }
        }
    }
    if (n_rhs > 1)
        for (int64_t i = 0; i < 4 * (int64_t)V; ++i) F4[i] /= (double)n_rhs;
    free(xs); free(chi);
    return iters;
}

/* ------------------------------------------------------------------------- */
/* Coloured noise: colouredNoise.cpp:5-29 (momenta), :138-145 (mask),         */
/* :155-178 (RNG -> D2Z -> mask -> Z2D).                                       */
/* ------------------------------------------------------------------------- */
/* p^2 of mode (kt, kx) in the reference's operation order (:16-29). */
static double momentum_sq(int kt, int kx, int Nt, int Nx)
{
    const int sizes[2] = {Nt, Nx};
    const int coo[2] = {kt, kx};
    double msq = 0.0;
    for (int d = 0; d < 2; ++d) {
        const int L = sizes[d];
        const double tmp = (coo[d] <= (L / 2) ? coo[d] : coo[d] - L) * 2.0 * M_PI / L;
        msq += tmp * tmp;
    }
    return msq;
}

static double cut_sq(double cut_fraction)
{
    const double momentum_cut = sqrt(2.0) * M_PI * cut_fraction;  /* :139 */
    return momentum_cut * momentum_cut;
}

void yko_mask_half(int Nt, int Nx, double cut_fraction, double* mask)
{
    const double csq = cut_sq(cut_fraction);
    const int Nh = Nx / 2 + 1;
    const double inv = 1.0 / (double)(Nt * Nx);
    for (int kt = 0; kt < Nt; ++kt)
        for (int kx = 0; kx < Nh; ++kx)
            mask[kt * Nh + kx] = (momentum_sq(kt, kx, Nt, Nx) <= csq) ? inv : 0.0;
}

int yko_mask_all_kept(int Nt, int Nx, double cut_fraction)
{
    const double csq = cut_sq(cut_fraction);
    for (int kt = 0; kt < Nt; ++kt)
        for (int kx = 0; kx <= Nx / 2; ++kx)
            if (!(momentum_sq(kt, kx, Nt, Nx) <= csq)) return 0;
    return 1;
}

static void fft1(int n, double* re, double* im, int sign)
{
    /* iterative radix-2 for powers of two, direct DFT otherwise */
    if ((n & (n - 1)) == 0) {
        for (int i = 1, j = 0; i < n; ++i) {
            int bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) {
                double tr = re[i]; re[i] = re[j]; re[j] = tr;
                double ti = im[i]; im[i] = im[j]; im[j] = ti;
            }
        }
        for (int len = 2; len <= n; len <<= 1) {
            const int h = len / 2;
            for (int i = 0; i < n; i += len) {
                for (int k = 0; k < h; ++k) {
                    const double ang = sign * 2.0 * M_PI * k / len;
                    const double wr = cos(ang), wi = sin(ang);
                    const double ur = re[i + k], ui = im[i + k];
                    const double vr = re[i + k + h] * wr - im[i + k + h] * wi;
                    const double vi = re[i + k + h] * wi + im[i + k + h] * wr;
                    re[i + k] = ur + vr; im[i + k] = ui + vi;
                    re[i + k + h] = ur - vr; im[i + k + h] = ui - vi;
                }
            }
        }
    } else {
        double* tr = (double*)malloc(sizeof(double) * n);
        double* ti = (double*)malloc(sizeof(double) * n);
        for (int k = 0; k < n; ++k) {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < n; ++j) {
                const double ang = sign * 2.0 * M_PI * (double)(((int64_t)j * k) % n) / n;
                sr += re[j] * cos(ang) - im[j] * sin(ang);
                si += re[j] * sin(ang) + im[j] * cos(ang);
            }
            tr[k] = sr; ti[k] = si;
        }
        memcpy(re, tr, sizeof(double) * n);
        memcpy(im, ti, sizeof(double) * n);
        free(tr); free(ti);
    }
}

void yko_fft2(int Nt, int Nx, double* data, int sign)
{
    const int L = Nt > Nx ? Nt : Nx;
    double* re = (double*)malloc(sizeof(double) * L);
    double* im = (double*)malloc(sizeof(double) * L);
    for (int t = 0; t < Nt; ++t) {
        for (int x = 0; x < Nx; ++x) { re[x] = data[2 * (t * Nx + x)]; im[x] = data[2 * (t * Nx + x) + 1]; }
        fft1(Nx, re, im, sign);
        for (int x = 0; x < Nx; ++x) { data[2 * (t * Nx + x)] = re[x]; data[2 * (t * Nx + x) + 1] = im[x]; }
    }
    for (int x = 0; x < Nx; ++x) {
        for (int t = 0; t < Nt; ++t) { re[t] = data[2 * (t * Nx + x)]; im[t] = data[2 * (t * Nx + x) + 1]; }
        fft1(Nt, re, im, sign);
        for (int t = 0; t < Nt; ++t) { data[2 * (t * Nx + x)] = re[t]; data[2 * (t * Nx + x) + 1] = im[t]; }
    }
    free(re); free(im);
}

void yko_coloured_noise(int Nt, int Nx, double cut_fraction, const double* white, double* xi)
{
    const int V = Nt * Nx;
    if (yko_mask_all_kept(Nt, Nx, cut_fraction)) {
        /* every mode kept: Z2D(D2Z(w)/V) is w up to rounding */
        memcpy(xi, white, sizeof(double) * V);
        return;
    }
    const double csq = cut_sq(cut_fraction);
    const double inv = 1.0 / (double)V;
    double* c = (double*)malloc(sizeof(double) * 2 * V);
    for (int i = 0; i < V; ++i) { c[2 * i] = white[i]; c[2 * i + 1] = 0.0; }
    yko_fft2(Nt, Nx, c, -1);
    /* full-spectrum mask: the half-spectrum rule extended by k -> -k symmetry */
    for (int kt = 0; kt < Nt; ++kt)
        for (int kx = 0; kx < Nx; ++kx) {
            const int kxh = (kx <= Nx / 2) ? kx : Nx - kx;
            const int kth = (kx <= Nx / 2) ? kt : (Nt - kt) % Nt;
            const double m = (momentum_sq(kth, kxh, Nt, Nx) <= csq) ? inv : 0.0;
            c[2 * (kt * Nx + kx)] *= m;
            c[2 * (kt * Nx + kx) + 1] *= m;
        }
    yko_fft2(Nt, Nx, c, +1);
    for (int i = 0; i < V; ++i) xi[i] = c[2 * i];
    free(c);
}

/* ------------------------------------------------------------------------- */
/* Bosonic drift and Euler update: langevin_gpu_v2.cu:9-37, 41-63, 65-118;    */
/* Laplacian CSR (sorted columns, diag -2d): Laplace.cu:61-100.               */
/* ------------------------------------------------------------------------- */
static int cmp_int(const void* a, const void* b)
{
    const int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

void yko_bosonic_drift(int Nt, int Nx, double m2, double lambda, const double* phi, double* drift)
{
    const int V = Nt * Nx;
    const double my_lambda = lambda / 6.0;                 /* langevin_gpu_v2.cu:13 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < V; ++i) {
        const double v = phi[i];
        drift[i] += v * (m2 + my_lambda * (v * v));        /* :15-24 */
        const int t = i / Nx, x = i % Nx;
        int cols[5] = {i, ((t + 1) % Nt) * Nx + x, ((t - 1 + Nt) % Nt) * Nx + x,
                       t * Nx + (x + 1) % Nx, t * Nx + (x - 1 + Nx) % Nx};
        qsort(cols, 5, sizeof(int), cmp_int);               /* Laplace.cu:88 */
        double out = 0.0;
        for (int j = 0; j < 5; ++j)                         /* :52-59 */
            out += (cols[j] != i ? 1.0 : -4.0) * phi[cols[j]];
        drift[i] -= out;
    }
}

double yko_euler_update(int V, double eps_bar, double fixed_dt, double* phi, const double* drift,
                        const double* noise, double* max_drift)
{
    double eps;
    double m = 0.0;
    for (int i = 0; i < V; ++i) {                           /* reductions.cu:30-63 */
        const double v = fabs(drift[i]);
        m = v > m ? v : m;
    }
    if (m > 1e5) m = 1e5;                                   /* langevin_gpu_v2.cu:83-91 */
    else if (m < 1e-5) m = 1e-5;
    if (max_drift) *max_drift = m;
    if (fixed_dt > 0.0)
        eps = fixed_dt;
    else
        eps = eps_bar * 30.0 / m;                           /* :71, :112 */
    const double fact = sqrt(2.0 * eps);                    /* :32 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < V; ++i)
        phi[i] -= eps * drift[i] + fact * noise[i];         /* :34 */
    return eps;
}

/* ------------------------------------------------------------------------- */
/* Observables: reductions.cu:65-140, 176-191, 200-233.                       */
/* ------------------------------------------------------------------------- */
double yko_sum(int n, const double* v)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += v[i];
    return s;
}

void yko_time_slices(int Nt, int Nx, const double* phi, double* slices)
{
    for (int t = 0; t < Nt; ++t) {
        double s = 0.0;
        for (int x = 0; x < Nx; ++x) s += phi[t * Nx + x];
        slices[t] = s;
    }
}

void yko_time_slices_spinor(int Nt, int Nx, const double* psi, double* corr)
{
    for (int t = 0; t < Nt; ++t) {
        double s = 0.0;
        for (int x = 0; x < Nx; ++x)
            for (int c = 0; c < 4; ++c) s += psi[((t * Nx + x) * 4 + c) * 2];
        corr[t] = s;
    }
}

/* ------------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon et al., SC'11) and Box-Muller.                        */
/* ------------------------------------------------------------------------- */
void yko_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        if (round > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* 52 random bits -> (0,1), exactly representable */
static double u52(uint32_t hi, uint32_t lo)
{
    const uint64_t m = ((uint64_t)hi << 20) | (lo >> 12);
    return ((double)m + 0.5) * 0x1p-52;
}

static void scheme_key_ctr(uint64_t seed, uint32_t chain, uint64_t step, uint32_t kind,
                           uint32_t rhs, uint32_t key[2], uint32_t ctr[4])
{
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32) ^ chain;
    ctr[1] = (uint32_t)step;
    ctr[2] = (uint32_t)(step >> 32);
    ctr[3] = (kind << 24) | (rhs & 0xFFFFFFu);
}

/* Gaussian normals by Box-Muller in FP32 arithmetic: the CUDA generator
   (yk_common.cuh nm_pair) uses IEEE round-to-nearest intrinsics for every
   operation, and this file is compiled with -ffp-contract=off, so both give
   the same bits.  Normals 4e .. 4e+3 of a stream come from Philox counter e:
   pair 0 from words (0, 1), pair 1 from (2, 3).  A pair (a, b):
     R = sqrt(2 E), E = -ln u, u = (a + 1/2) 2^-32, angle 2 pi (b + 1/2) 2^-32.
   ln(1 + f) = 2 atanh(f / (2 + f)) by its Taylor series; sin and cos of
   2 pi y (|y| <= 1/8 turn) by theirs; u >= 1/2 through w = 1 - u, exact from
   the complemented word. */
static float nm_log1p_core(float f)   /* ln(1 + f), f in [-0.293, 0.415] */
{
    const float s = f / (2.0f + f);
    const float t = 2.0f * s;
    const float z = s * s;
    float p = fmaf(z, 0x1.c71c72p-4f, 0x1.24924ap-3f);
    p = fmaf(z, p, 0x1.99999ap-3f);
    p = fmaf(z, p, 0x1.555556p-2f);
    return fmaf(t * z, p, t);
}

static float nm_neglog(uint32_t a)   /* -ln((a + 1/2) 2^-32) */
{
    const float ln2hi = 0x1.62e4p-1f, ln2lo = 0x1.7f7d1cp-20f;
    if (a < 0x80000000u) {
        const float u = (float)(2u * a + 1u) * 0x1p-33f;
        uint32_t bits;
        memcpy(&bits, &u, sizeof bits);
        int e = (int)(bits >> 23) - 127;
        bits = (bits & 0x007FFFFFu) | 0x3F800000u;
        float m;
        memcpy(&m, &bits, sizeof m);
        if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
        const float L = nm_log1p_core(m - 1.0f);
        const float fe = (float)e;
        return -fmaf(fe, ln2hi, fmaf(fe, ln2lo, L));
    }
    const float w = (float)(2u * ~a + 1u) * 0x1p-33f;   /* 1 - u */
    if (w <= 0x1.2bec34p-2f) return -nm_log1p_core(-w);
    return (ln2hi - nm_log1p_core(1.0f - 2.0f * w)) + ln2lo;
}

static void nm_pair(uint32_t a, uint32_t b, float* z0, float* z1)
{
    const float R = sqrtf(2.0f * nm_neglog(a));
    const uint32_t j = (b + 0x20000000u) >> 30;
    const int32_t d = (int32_t)(b - (j << 30));
    const float y = (float)(2 * d + 1) * 0x1p-33f;
    const float y2 = y * y;
    float sp = fmaf(y2, 0x1.507834p+5f, -0x1.32d2ccp+6f);
    sp = fmaf(y2, sp, 0x1.466bc6p+6f);
    sp = fmaf(y2, sp, -0x1.4abbcep+5f);
    sp = fmaf(y2, sp, 0x1.921fb6p+2f);
    const float sn = y * sp;
    float cp = fmaf(y2, -0x1.a6d1f2p+4f, 0x1.e1f506p+5f);
    cp = fmaf(y2, cp, -0x1.55d3c8p+6f);
    cp = fmaf(y2, cp, 0x1.03c1f0p+6f);
    cp = fmaf(y2, cp, -0x1.3bd3ccp+4f);
    const float cs = fmaf(y2, cp, 1.0f);
    float c, s;
    switch (j) {
    case 0: c = cs; s = sn; break;
    case 1: c = -sn; s = cs; break;
    case 2: c = -cs; s = -sn; break;
    default: c = sn; s = -cs; break;
    }
    *z0 = R * c;
    *z1 = R * s;
}

/* One pair from explicit words (edge tests of the transform). */
void yko_normal_pair_words(uint32_t a, uint32_t b, double out[2])
{
    float z0, z1;
    nm_pair(a, b, &z0, &z1);
    out[0] = z0;
    out[1] = z1;
}

void yko_normals(uint64_t seed, uint32_t chain, uint64_t step, uint32_t kind, uint32_t rhs,
                 int64_t n, double* out)
{
    uint32_t key[2], ctr0[4];
    scheme_key_ctr(seed, chain, step, kind, rhs, key, ctr0);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (n + 3) / 4; ++e) {
        uint32_t ctr[4] = {(uint32_t)e, ctr0[1], ctr0[2], ctr0[3]}, o[4];
        yko_philox4x32_10(ctr, key, o);
        float z[4];
        nm_pair(o[0], o[1], &z[0], &z[1]);
        nm_pair(o[2], o[3], &z[2], &z[3]);
        for (int c = 0; c < 4 && 4 * e + c < n; ++c) out[4 * e + c] = (double)z[c];
    }
}

/* Reference transform of the same words in FP64 (libm log, sqrt, cos, sin):
   the test of the FP32 generator's accuracy. */
void yko_normals_fp64(uint64_t seed, uint32_t chain, uint64_t step, uint32_t kind, uint32_t rhs,
                      int64_t n, double* out)
{
    uint32_t key[2], ctr0[4];
    scheme_key_ctr(seed, chain, step, kind, rhs, key, ctr0);
    for (int64_t e = 0; e < (n + 3) / 4; ++e) {
        uint32_t ctr[4] = {(uint32_t)e, ctr0[1], ctr0[2], ctr0[3]}, o[4];
        yko_philox4x32_10(ctr, key, o);
        for (int p = 0; p < 2; ++p) {
            const double u = ((double)o[2 * p] + 0.5) * 0x1p-32, t = ((double)o[2 * p + 1] + 0.5) * 0x1p-32;
            const double R = sqrt(-2.0 * log(u));
            if (4 * e + 2 * p < n) out[4 * e + 2 * p] = R * cos(2.0 * M_PI * t);
            if (4 * e + 2 * p + 1 < n) out[4 * e + 2 * p + 1] = R * sin(2.0 * M_PI * t);
        }
    }
}

void yko_uniform_field(uint64_t seed, uint32_t chain, int64_t n, double* out)
{
    yko_uniform_field_comp(seed, chain, 0u, n, out);
}

/* comp 0: sigma; comp a (1..3): the pion field pi_a of the pion extension */
void yko_uniform_field_comp(uint64_t seed, uint32_t chain, uint32_t comp, int64_t n, double* out)
{
    uint32_t key[2], ctr0[4];
    scheme_key_ctr(seed, chain, 0, 0u, comp, key, ctr0);
    for (int64_t e = 0; e < (n + 1) / 2; ++e) {
        uint32_t ctr[4] = {(uint32_t)e, ctr0[1], ctr0[2], ctr0[3]}, o[4];
        yko_philox4x32_10(ctr, key, o);
        out[2 * e] = 1.0 - 2.0 * u52(o[0], o[1]);
        if (2 * e + 1 < n) out[2 * e + 1] = 1.0 - 2.0 * u52(o[2], o[3]);
    }
}

void yko_drand48_field(int64_t n, double* out)
{
    /* POSIX drand48: X <- (a X + c) mod 2^48, a = 0x5DEECE66D, c = 0xB; glibc's
       state starts at X = 0 when no seeding call is made; value X / 2^48. */
    uint64_t X = 0;
    for (int64_t i = 0; i < n; ++i) {
        X = (0x5DEECE66DULL * X + 0xBULL) & ((1ULL << 48) - 1);
        out[i] = 1.0 - 2.0 * ((double)X * 0x1p-48);
    }
}

/* ------------------------------------------------------------------------- */
/* One full Langevin step (main.cu:370-381): noise, force, bosonic drift,     */
/* update.                                                                    */
/* ------------------------------------------------------------------------- */
double yko_langevin_step(int Nt, int Nx, const yko_action* a, uint64_t seed, uint32_t chain,
                         uint64_t step, int n_rhs, double tol, int tol_mode, int max_iter,
                         double fixed_dt, double* phi, double* obs)
{
    const int V = Nt * Nx;
    double* w = (double*)malloc(sizeof(double) * V);
    double* xi = (double*)malloc(sizeof(double) * V);
    double* F = (double*)malloc(sizeof(double) * V);
    double* drift = (double*)malloc(sizeof(double) * V);
    yko_normals(seed, chain, step, 1u, 0u, V, w);
    yko_coloured_noise(Nt, Nx, a->cut_fraction, w, xi);
    int iters = 0;
    if (a->g != 0.0) {
        const int64_t n = (int64_t)V * 4;
        double* eta = (double*)calloc((size_t)(2 * n * n_rhs), sizeof(double));
        double* re = (double*)malloc(sizeof(double) * n);
        for (int j = 0; j < n_rhs; ++j) {
            yko_normals(seed, chain, step, 2u, (uint32_t)j, n, re);
            for (int64_t i = 0; i < n; ++i) eta[(int64_t)j * 2 * n + 2 * i] = re[i];
        }
        iters = yko_force(Nt, Nx, a, phi, eta, n_rhs, tol, tol_mode, max_iter, F);
        free(eta); free(re);
    } else {
        for (int i = 0; i < V; ++i) F[i] = 0.0;
    }
    memcpy(drift, F, sizeof(double) * V);
    yko_bosonic_drift(Nt, Nx, a->m2, a->lambda, phi, drift);
    double maxd;
    const double eps = yko_euler_update(V, a->eps_bar, fixed_dt, phi, drift, xi, &maxd);
    if (obs) {
        double s2 = 0.0;
        for (int i = 0; i < V; ++i) s2 += phi[i] * phi[i];
        obs[0] = eps; obs[1] = maxd; obs[2] = yko_sum(V, phi); obs[3] = yko_sum(V, F);
        obs[4] = (double)iters; obs[5] = s2;
    }
    free(w); free(xi); free(F); free(drift);
    return eps;
}

/* One Langevin step of the pion extension (no reference counterpart): the
   four fields phi4 = (sigma, pi_1, pi_2, pi_3), each V doubles, get their own
   coloured noise (Philox kind 1, rhs 0 for sigma as in the sigma-only step,
   rhs a for pi_a) and the drift
     drift_a = F_a + phi_a (m^2 + lambda/6 |phi|^2) - Lap phi_a,
   |phi|^2 = sigma^2 + pi^2 (the O(4)-symmetric form of PotentialAndMass,
   langevin_gpu_v2.cu:9-27); max|drift| over all four fields sets the
   adaptive eps; every field takes the Euler update of langevin_gpu_v2.cu:29-37.
   At pi = 0 the sigma field moves exactly as in yko_langevin_step.
   obs[0..9] = {eps, max_drift, sum sigma, sum F_sigma, cg_iters, sum sigma^2,
   sum pi_1, sum pi_2, sum pi_3, sum |pi|^2}. */
double yko_langevin_step_pi(int Nt, int Nx, const yko_action* a, uint64_t seed, uint32_t chain,
                            uint64_t step, int n_rhs, double tol, int tol_mode, int max_iter,
                            double fixed_dt, double* phi4, double* obs)
{
    const int V = Nt * Nx;
    double* w = (double*)malloc(sizeof(double) * V);
    double* xi = (double*)malloc(sizeof(double) * 4 * (size_t)V);
    double* F = (double*)calloc(4 * (size_t)V, sizeof(double));
    double* drift = (double*)malloc(sizeof(double) * 4 * (size_t)V);
    for (int q = 0; q < 4; ++q) {
        yko_normals(seed, chain, step, 1u, (uint32_t)q, V, w);
        yko_coloured_noise(Nt, Nx, a->cut_fraction, w, xi + (size_t)q * V);
    }
    int iters = 0;
    if (a->g != 0.0) {
        const int64_t n = (int64_t)V * 4;
        double* eta = (double*)calloc((size_t)(2 * n * n_rhs), sizeof(double));
        double* re = (double*)malloc(sizeof(double) * n);
        for (int j = 0; j < n_rhs; ++j) {
            yko_normals(seed, chain, step, 2u, (uint32_t)j, n, re);
            for (int64_t i = 0; i < n; ++i) eta[(int64_t)j * 2 * n + 2 * i] = re[i];
        }
        iters = yko_force_pi(Nt, Nx, a, phi4, phi4 + V, eta, n_rhs, tol, tol_mode, max_iter, F);
        free(eta); free(re);
    }
    const double my_lambda = a->lambda / 6.0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < V; ++i) {
        const double s0 = phi4[i], p1 = phi4[V + i], p2 = phi4[2 * V + i], p3 = phi4[3 * V + i];
        const double r2 = s0 * s0 + p1 * p1 + p2 * p2 + p3 * p3;
        const int t = i / Nx, x = i % Nx;
        int cols[5] = {i, ((t + 1) % Nt) * Nx + x, ((t - 1 + Nt) % Nt) * Nx + x,
                       t * Nx + (x + 1) % Nx, t * Nx + (x - 1 + Nx) % Nx};
        qsort(cols, 5, sizeof(int), cmp_int);
        for (int q = 0; q < 4; ++q) {
            const double* f = phi4 + (size_t)q * V;
            double d = F[(size_t)q * V + i];
            d += f[i] * (a->m2 + my_lambda * r2);
            double out = 0.0;
            for (int j = 0; j < 5; ++j) out += (cols[j] != i ? 1.0 : -4.0) * f[cols[j]];
            drift[(size_t)q * V + i] = d - out;
        }
    }
    double maxd;
    const double eps = yko_euler_update(4 * V, a->eps_bar, fixed_dt, phi4, drift, xi, &maxd);
    if (obs) {
        double s2 = 0.0, p2 = 0.0;
        for (int i = 0; i < V; ++i) {
            s2 += phi4[i] * phi4[i];
            p2 += phi4[V + i] * phi4[V + i] + phi4[2 * V + i] * phi4[2 * V + i] + phi4[3 * V + i] * phi4[3 * V + i];
        }
        obs[0] = eps; obs[1] = maxd; obs[2] = yko_sum(V, phi4); obs[3] = yko_sum(V, F);
        obs[4] = (double)iters; obs[5] = s2;
        obs[6] = yko_sum(V, phi4 + V); obs[7] = yko_sum(V, phi4 + 2 * V); obs[8] = yko_sum(V, phi4 + 3 * V);
        obs[9] = p2;
    }
    free(w); free(xi); free(F); free(drift);
    return eps;
}

/* ------------------------------------------------------------------------- */
/* Gamma-method, restated from U. Wolff, CPC 156 (2004) 143, eqs. (31)-(52);   */
/* the reference wraps the same method in analysis/AutoCorrelation/ac.cpp.    */
/* ------------------------------------------------------------------------- */
void yko_gamma_method(const double* data, int64_t n, double stau, double out[5])
{
    double mean = 0.0;
    for (int64_t i = 0; i < n; ++i) mean += data[i];
    mean /= (double)n;
    out[0] = mean; out[1] = out[2] = out[3] = out[4] = 0.0;
    if (n < 2) return;
    const int64_t tmax = n / 2;
    double* gam = (double*)calloc((size_t)tmax + 1, sizeof(double));
    for (int64_t t = 0; t <= tmax; ++t) {
        double s = 0.0;
        for (int64_t i = 0; i + t < n; ++i) s += (data[i] - mean) * (data[i + t] - mean);
        gam[t] = s / (double)(n - t);
    }
    if (gam[0] == 0.0) { free(gam); return; }
    int64_t W = tmax;
    double gint = 0.0;
    int found = 0;
    for (int64_t t = 1; t <= tmax; ++t) {
        gint += gam[t] / gam[0];
        const double tauw = (gint <= 0.0) ? 1e-5 : stau / log((gint + 1.0) / gint);
        const double gw = exp(-(double)t / tauw) - tauw / sqrt((double)t * (double)n);
        if (gw < 0.0) { W = t; found = 1; break; }
    }
    (void)found;
    double cf = gam[0];
    for (int64_t t = 1; t <= W; ++t) cf += 2.0 * gam[t];
    for (int64_t t = 0; t <= tmax; ++t) gam[t] += cf / (double)n;   /* bias correction */
    double cf2 = gam[0], acc = gam[0];
    for (int64_t t = 1; t <= W; ++t) { cf2 += 2.0 * gam[t]; acc += gam[t]; }
    const double tau = acc / gam[0] - 0.5;
    out[1] = sqrt(cf2 / (double)n);
    out[2] = out[1] * sqrt(((double)W + 0.5) / (double)n);
    out[3] = tau;
    out[4] = tau * 2.0 * sqrt(((double)W - tau + 0.5) / (double)n);
    free(gam);
}

/* ------------------------------------------------------------------------
   Float-float arithmetic of the GPU's even-odd reliable updates, round 0 and
   reconstruction of chi, restated for the accuracy tests (test
   infrastructure: tests/test_oracle.py measures it against long-double
   arithmetic; the kernels hold their own copy in csrc/yk_cg.cu).  A value is
   hi + lo, two floats.  Sums use Knuth's two-sum of the high words with the
   low words added; products use Dekker's product with the error term from
   fmaf; the reciprocal takes one Newton step from the correctly rounded float
   reciprocal.  The file is compiled with -ffp-contract=off, so the only
   fused operations are the explicit fmaf calls, as in the kernels. */
typedef struct {
    float hi, lo;
} yko_ff;

static yko_ff ff_add(yko_ff a, yko_ff b)
{
    const float s = a.hi + b.hi;
    const float bp = s - a.hi;
    float e = (a.hi - (s - bp)) + (b.hi - bp);
    e += a.lo + b.lo;
    const float hi = s + e;
    yko_ff r = {hi, e - (hi - s)};
    return r;
}

static yko_ff ff_renorm(float p, float e)
{
    const float hi = p + e;
    yko_ff r = {hi, e - (hi - p)};
    return r;
}

static yko_ff ff_mul(yko_ff a, yko_ff b)
{
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return ff_renorm(p, e);
}

static yko_ff ff_mul_f(yko_ff a, float b)
{
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return ff_renorm(p, e);
}

static yko_ff ff_of(double x)
{
    const float hi = (float)x;
    yko_ff r = {hi, (float)(x - (double)hi)};
    return r;
}

static yko_ff ff_neg(yko_ff a)
{
    yko_ff r = {-a.hi, -a.lo};
    return r;
}

static double ff_dbl(yko_ff a) { return (double)a.hi + (double)a.lo; }

static yko_ff ff_rcp(yko_ff d)
{
    const float y = 1.0f / d.hi;
    const yko_ff one = {1.0f, 0.0f}, y0 = {y, 0.0f};
    const yko_ff e = ff_add(one, ff_neg(ff_mul_f(d, y)));
    return ff_add(y0, ff_mul_f(e, y));
}

void yko_ff_ops(int64_t n, const double* a, const double* b, double* sum, double* prod, double* rcp)
{
    for (int64_t i = 0; i < n; ++i) {
        const yko_ff A = ff_of(a[i]), B = ff_of(b[i]);
        sum[i] = ff_dbl(ff_add(A, B));
        prod[i] = ff_dbl(ff_mul(A, B));
        rcp[i] = ff_dbl(ff_rcp(A));
    }
}

/* One site of the half hop in float-float, in the kernels' order of terms
   (csrc/yk_cg.cu combine_ff, DAG 0 or 1; mode 0: H alone, 1: c + H, 2:
   diag c + H) for a real site of four components (flavour f: upper 2f, lower
   2f + 1); the coefficients from r as the kernels' hop_of_r forms them. */
void yko_ff_hop(int dag, int mode, double r, const double* c, double diag, const double* tu, const double* td,
                const double* xu, const double* xd, double sp, double sm, double* out)
{
    const yko_ff rr = ff_of(r), one = {1.0f, 0.0f}, mone = {-1.0f, 0.0f};
    const yko_ff rp = ff_add(rr, one), rm = ff_add(rr, mone);
    const yko_ff P = {-0.5f * rp.hi, -0.5f * rp.lo}, M = {-0.5f * rm.hi, -0.5f * rm.lo},
                 A = {-0.5f * rr.hi, -0.5f * rr.lo};
    const float fsp = (float)sp, fsm = (float)sm;
    const yko_ff Pp = {fsp * (dag ? P : M).hi, fsp * (dag ? P : M).lo};
    const yko_ff Mp = {fsp * (dag ? M : P).hi, fsp * (dag ? M : P).lo};
    const yko_ff Mm = {fsm * (dag ? M : P).hi, fsm * (dag ? M : P).lo};
    const yko_ff Pm = {fsm * (dag ? P : M).hi, fsm * (dag ? P : M).lo};
    const float bx = dag ? -0.5f : 0.5f;
    const yko_ff dg = ff_of(diag);
    for (int f = 0; f < 2; ++f) {
        const int iu = 2 * f, id = 2 * f + 1;
        yko_ff ou, od;
        const yko_ff tuu = ff_of(tu[iu]), tud = ff_of(tu[id]), tdu = ff_of(td[iu]), tdd = ff_of(td[id]);
        const yko_ff xuu = ff_of(xu[iu]), xud = ff_of(xu[id]), xdu = ff_of(xd[iu]), xdd = ff_of(xd[id]);
        if (mode == 0) {
            ou = ff_mul(Pp, tuu);
            od = ff_mul(Mp, tud);
        } else {
            const yko_ff cu = ff_of(c[iu]), cd = ff_of(c[id]);
            ou = mode == 1 ? cu : ff_mul(dg, cu);
            od = mode == 1 ? cd : ff_mul(dg, cd);
            ou = ff_add(ou, ff_mul(Pp, tuu));
            od = ff_add(od, ff_mul(Mp, tud));
        }
        ou = ff_add(ou, ff_mul(Mm, tdu));
        od = ff_add(od, ff_mul(Pm, tdd));
        const yko_ff dfu = ff_add(xud, ff_neg(xdd)), dfd = ff_add(xuu, ff_neg(xdu));
        const yko_ff bu = {bx * dfu.hi, bx * dfu.lo}, bd = {bx * dfd.hi, bx * dfd.lo};
        ou = ff_add(ou, bu);
        od = ff_add(od, bd);
        ou = ff_add(ou, ff_mul(A, ff_add(xuu, xdu)));
        od = ff_add(od, ff_mul(A, ff_add(xud, xdd)));
        out[iu] = ff_dbl(ou);
        out[id] = ff_dbl(od);
    }
}
