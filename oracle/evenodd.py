"""Even-odd (Schur complement) solve of the fermion force's system (test
infrastructure only: the oracle of a solver the CUDA path does not use yet).

The step needs chi = D (D^dag D)^-1 eta = (D^dag)^-1 eta (code/src/
FermionicDrift.cu:57-100, which forms it from the CG solution of D^dag D x =
eta, code/src/CGsolver.cu:72-170).  D = A + H with A = diag(2 r + m0 + g
sigma_n) (a scalar per site on all four spinor components) and H the hopping
term, which only connects sites of opposite parity (t + x) on a lattice with
even Nt and Nx.  With e / o the even / odd sites, D^dag chi = eta becomes

  S chi_e = eta_e - H^dag_eo A_o^-1 eta_o,  S = A_e - H^dag_eo A_o^-1 H^dag_oe,
  chi_o = A_o^-1 (eta_o - H^dag_oe chi_e),

and S is solved over half the sites, either by CG on the normal equations
S^dag S (CGNR, chi_evenodd) or by CG on S S^dag with chi_e = S^dag y (CGNE,
chi_evenodd_cgne).  CGNE's residual rhs - S S^dag y = rhs - S chi_e is the
true residual of D^dag chi = eta on the even sites (the odd sites' is zero by
the construction of chi_o), the quantity the reference's CG on D^dag D
controls (its residual eta - D^dag D x is eta - D^dag chi with chi = D x), so
the two stop on the same rule |eta - D^dag chi| <= tol |eta|.  Everything here
applies D through the FP64 oracle (oracle.dirac).
"""
from __future__ import annotations

import numpy as np

from . import oracle as O


def parity(Nt, Nx):
    """(t + x) % 2 of every site n = t * Nx + x."""
    t, x = np.divmod(np.arange(Nt * Nx), Nx)
    return (t + x) % 2


def diagonal(a: "O.Action", sigma):
    """The site diagonal of D: 2 r + m0 + g sigma_n."""
    return 2.0 * a.r + a.m0 + a.g * np.asarray(sigma, dtype=np.float64)


def hop_dag(Nt, Nx, a, sigma, v, src, dst):
    """(H^dag v) restricted to the sites of parity dst, for v living on the
    sites of parity src (zero elsewhere); H^dag = D^dag - A."""
    par = parity(Nt, Nx)
    w = np.zeros((Nt * Nx, 4), dtype=np.complex128)
    w[par == src] = v
    out = O.dirac(Nt, Nx, a, sigma, w, True) - diagonal(a, sigma)[:, None] * w
    return out[par == dst]


def schur(Nt, Nx, a, sigma, ve):
    """S v_e = A_e v_e - H^dag_eo A_o^-1 H^dag_oe v_e."""
    par = parity(Nt, Nx)
    d = diagonal(a, sigma)
    vo = hop_dag(Nt, Nx, a, sigma, ve, 0, 1) / d[par == 1][:, None]
    return d[par == 0][:, None] * ve - hop_dag(Nt, Nx, a, sigma, vo, 1, 0)


def schur_dag(Nt, Nx, a, sigma, ve):
    """S^dag v_e = A_e v_e - H_eo A_o^-1 H_oe v_e (H = D - A, real A)."""
    par = parity(Nt, Nx)
    d = diagonal(a, sigma)

    def hop(v, src, dst):
        w = np.zeros((Nt * Nx, 4), dtype=np.complex128)
        w[par == src] = v
        return (O.dirac(Nt, Nx, a, sigma, w, False) - d[:, None] * w)[par == dst]

    vo = hop(ve, 0, 1) / d[par == 1][:, None]
    return d[par == 0][:, None] * ve - hop(vo, 1, 0)


def cg(apply, b, tol, max_iter):
    """Plain CG on a Hermitian positive definite operator; x0 = 0; stops at
    |r| <= tol |b|.  Returns x and the iterations."""
    x = np.zeros_like(b)
    r = b.copy()
    p = r.copy()
    rr = float(np.vdot(r, r).real)
    stop = tol * tol * rr
    it = 0
    while rr > stop and it < max_iter:
        q = apply(p)
        alpha = rr / float(np.vdot(p, q).real)
        x = x + alpha * p
        r = r - alpha * q
        rr_new = float(np.vdot(r, r).real)
        p = r + (rr_new / rr) * p
        rr = rr_new
        it += 1
    return x, it


def chi_evenodd(Nt, Nx, a, sigma, eta, tol=1e-12, max_iter=10000):
    """chi = (D^dag)^-1 eta through the even-odd Schur complement (CGNR on
    the even sites).  Returns chi (V, 4) and the CG iterations."""
    assert Nt % 2 == 0 and Nx % 2 == 0, "the checkerboard needs even extents"
    par = parity(Nt, Nx)
    d = diagonal(a, sigma)
    eta = np.asarray(eta, dtype=np.complex128).reshape(Nt * Nx, 4)
    eta_e, eta_o = eta[par == 0], eta[par == 1]
    rhs = eta_e - hop_dag(Nt, Nx, a, sigma, eta_o / d[par == 1][:, None], 1, 0)
    b = schur_dag(Nt, Nx, a, sigma, rhs)
    chi_e, it = cg(lambda v: schur_dag(Nt, Nx, a, sigma, schur(Nt, Nx, a, sigma, v)), b, tol, max_iter)
    chi_o = (eta_o - hop_dag(Nt, Nx, a, sigma, chi_e, 0, 1)) / d[par == 1][:, None]
    chi = np.empty((Nt * Nx, 4), dtype=np.complex128)
    chi[par == 0] = chi_e
    chi[par == 1] = chi_o
    return chi, it


def chi_full(Nt, Nx, a, sigma, eta, tol=1e-12, max_iter=10000):
    """The reference's way: x from CG on D^dag D, chi = D x."""
    eta = np.asarray(eta, dtype=np.complex128).reshape(Nt * Nx, 4)
    x, it = cg(lambda v: O.dirac(Nt, Nx, a, sigma, O.dirac(Nt, Nx, a, sigma, v, False), True), eta, tol, max_iter)
    return O.dirac(Nt, Nx, a, sigma, x, False), it


def cg_rule(apply, b, stop2, max_iter):
    """CG on a Hermitian positive definite operator, x0 = 0, stopping when
    |r|^2 <= stop2.  Returns x and the iterations."""
    x = np.zeros_like(b)
    r = b.copy()
    p = r.copy()
    rr = float(np.vdot(r, r).real)
    it = 0
    while rr > stop2 and it < max_iter:
        q = apply(p)
        alpha = rr / float(np.vdot(p, q).real)
        x = x + alpha * p
        r = r - alpha * q
        rr_new = float(np.vdot(r, r).real)
        p = r + (rr_new / rr) * p
        rr = rr_new
        it += 1
    return x, it


def chi_evenodd_cgne(Nt, Nx, a, sigma, eta, tol=1e-10, max_iter=10000):
    """chi = (D^dag)^-1 eta by CGNE on the Schur complement: (S S^dag) y =
    rhs_e, chi_e = S^dag y, stopping when the true residual |eta - D^dag chi|
    (= |rhs_e - S chi_e|) reaches tol |eta|.  Returns chi (V, 4) and the CG
    iterations."""
    assert Nt % 2 == 0 and Nx % 2 == 0, "the checkerboard needs even extents"
    par = parity(Nt, Nx)
    d = diagonal(a, sigma)
    eta = np.asarray(eta, dtype=np.complex128).reshape(Nt * Nx, 4)
    eta_e, eta_o = eta[par == 0], eta[par == 1]
    rhs = eta_e - hop_dag(Nt, Nx, a, sigma, eta_o / d[par == 1][:, None], 1, 0)
    stop2 = tol * tol * float(np.vdot(eta, eta).real)
    y, it = cg_rule(lambda v: schur(Nt, Nx, a, sigma, schur_dag(Nt, Nx, a, sigma, v)), rhs, stop2, max_iter)
    chi_e = schur_dag(Nt, Nx, a, sigma, y)
    chi_o = (eta_o - hop_dag(Nt, Nx, a, sigma, chi_e, 0, 1)) / d[par == 1][:, None]
    chi = np.empty((Nt * Nx, 4), dtype=np.complex128)
    chi[par == 0] = chi_e
    chi[par == 1] = chi_o
    return chi, it


def true_residual(Nt, Nx, a, sigma, eta, chi):
    """|eta - D^dag chi| / |eta|."""
    eta = np.asarray(eta, dtype=np.complex128).reshape(Nt * Nx, 4)
    r = eta - O.dirac(Nt, Nx, a, sigma, chi, True)
    return float(np.linalg.norm(r) / np.linalg.norm(eta))
