"""The pion extension of the CPU oracle, pinned by dense linear algebra (no
GPU).  The reference is sigma-only (code/src/params.h:25, Dirac.cu:57-69), so
these pins are independent restatements of the operator's definition:

  D_pi = D + g i gamma5 (tau . pi_n) on each site, gamma5 = -i gamma_t gamma_x
  = sigma_2 (gamma_t = sigma_3, gamma_x = sigma_1), component c = 2 f + s,

the pion force as the gradient of the fermion effective action
-ln|det D_pi| (finite differences of numpy's slogdet), and the exact
reduction to the sigma-only path at pi = 0.
Tolerances: operator 1e-14 relative; CG 1e-9; forces against the dense
trace 1e-8; finite differences 1e-5 relative.
"""
import numpy as np
import pytest

from oracle import oracle as O

S1 = np.array([[0, 1], [1, 0]], dtype=complex)
S2 = np.array([[0, -1j], [1j, 0]], dtype=complex)
S3 = np.array([[1, 0], [0, -1]], dtype=complex)
IG5 = 1j * S2                   # i gamma5 on spin
TAU = (S1, S2, S3)


def setup(Nt=4, Nx=6, seed=3, g=0.7, m0=0.15):
    rng = np.random.default_rng(seed)
    V = Nt * Nx
    a = O.action(m2=-0.5, lam=1.0, g=g, m0=m0, r=1.0)
    sigma = rng.uniform(-1, 1, V)
    pi = rng.uniform(-1, 1, (3, V))
    return a, sigma, pi, rng


def dense(Nt, Nx, a, sigma, pi, dagger=False):
    """D_pi as a dense (4V, 4V) matrix: the sigma-only D column by column from
    the oracle (pinned to the reference's kernels), plus the pion blocks from
    Kronecker products."""
    V = Nt * Nx
    M = np.zeros((4 * V, 4 * V), dtype=complex)
    for k in range(4 * V):
        e = np.zeros(4 * V, dtype=complex)
        e[k] = 1.0
        M[:, k] = O.dirac(Nt, Nx, a, sigma, e.reshape(V, 4), dagger).reshape(-1)
    sg = -a.g if dagger else a.g
    for n in range(V):
        tp = sum(pi[q, n] * TAU[q] for q in range(3))
        M[4 * n:4 * n + 4, 4 * n:4 * n + 4] += sg * np.kron(tp, IG5)
    return M


def test_gamma5_convention():
    assert np.allclose(S2, -1j * S3 @ S1)          # gamma5 = -i gamma_t gamma_x
    for gm in (S3, S1):
        assert np.allclose(S2 @ gm + gm @ S2, 0)
    assert np.allclose(S2 @ S2, np.eye(2))


def test_pion_operator_matches_dense():
    Nt, Nx = 4, 6
    a, sigma, pi, rng = setup(Nt, Nx)
    V = Nt * Nx
    psi = rng.normal(size=(V, 4)) + 1j * rng.normal(size=(V, 4))
    for dag in (False, True):
        M = dense(Nt, Nx, a, sigma, pi, dag)
        got = O.dirac_pi(Nt, Nx, a, sigma, pi, psi, dag).reshape(-1)
        want = M @ psi.reshape(-1)
        assert np.abs(got - want).max() / np.abs(want).max() < 1e-14
    # D^dag is the adjoint of D
    assert np.abs(dense(Nt, Nx, a, sigma, pi, True) - dense(Nt, Nx, a, sigma, pi, False).conj().T).max() < 1e-14


def test_pion_operator_is_complex_and_reduces_at_zero():
    Nt, Nx = 4, 6
    a, sigma, pi, rng = setup(Nt, Nx)
    V = Nt * Nx
    psi = rng.normal(size=(V, 4)).astype(complex)   # real input
    out = O.dirac_pi(Nt, Nx, a, sigma, pi, psi)
    assert np.abs(out.imag).max() > 0.1              # tau_2 makes D complex
    z = np.zeros((3, V))
    for dag in (False, True):
        assert np.array_equal(O.dirac_pi(Nt, Nx, a, sigma, z, psi, dag), O.dirac(Nt, Nx, a, sigma, psi, dag))
        assert np.array_equal(O.dirac_pi(Nt, Nx, a, sigma, None, psi, dag), O.dirac(Nt, Nx, a, sigma, psi, dag))


def test_pion_cg_matches_dense_solve():
    Nt, Nx = 4, 6
    a, sigma, pi, rng = setup(Nt, Nx)
    V = Nt * Nx
    b = rng.normal(size=(V, 4)) + 1j * rng.normal(size=(V, 4))
    D = dense(Nt, Nx, a, sigma, pi)
    for mtype, A in ((1, D.conj().T @ D), (0, D @ D.conj().T)):
        x, it, rr = O.cg_pi(Nt, Nx, a, sigma, pi, b, mtype=mtype, tol=1e-13, tol_mode=1, max_iter=5000)
        want = np.linalg.solve(A, b.reshape(-1))
        assert np.abs(x.reshape(-1) - want).max() / np.abs(want).max() < 1e-9


def test_pion_cg_and_force_reduce_at_zero():
    Nt, Nx = 4, 6
    a, sigma, _, rng = setup(Nt, Nx)
    V = Nt * Nx
    z = np.zeros((3, V))
    eta = np.zeros((2, V, 4), dtype=complex)
    eta.real = rng.normal(size=(2, V, 4))
    x0, it0, _ = O.cg(Nt, Nx, a, sigma, eta[0], tol=1e-12, tol_mode=1)
    x1, it1, _ = O.cg_pi(Nt, Nx, a, sigma, z, eta[0], tol=1e-12, tol_mode=1)
    assert it0 == it1 and np.array_equal(x0, x1)
    F, _ = O.force(Nt, Nx, a, sigma, eta, tol=1e-12, tol_mode=1)
    F4, _ = O.force_pi(Nt, Nx, a, sigma, z, eta, tol=1e-12, tol_mode=1)
    assert np.array_equal(F4[0], F)


def test_pion_force_estimator_matches_dense_trace():
    """Summed over the unit sources the estimator is exact:
    sum_k -g Re e_k^dag D^-1 (dD/dphi_a(n)/g) e_k = -Re tr(D^-1 dD/dphi_a(n))."""
    Nt, Nx = 4, 4
    a, sigma, pi, rng = setup(Nt, Nx, seed=5)
    V = Nt * Nx
    eta = np.zeros((4 * V, V, 4), dtype=complex)
    for k in range(4 * V):
        eta[k].reshape(-1)[k] = 1.0
    F4, _ = O.force_pi(Nt, Nx, a, sigma, pi, eta, tol=1e-13, tol_mode=1, max_iter=5000)
    F4 = F4 * (4 * V)   # the call averages over right-hand sides
    Dinv = np.linalg.inv(dense(Nt, Nx, a, sigma, pi))
    gens = [np.eye(4)] + [np.kron(TAU[q], IG5) for q in range(3)]
    for n in range(V):
        blk = Dinv[4 * n:4 * n + 4, 4 * n:4 * n + 4]
        for q in range(4):
            want = -a.g * np.trace(blk @ gens[q]).real
            assert abs(F4[q, n] - want) < 1e-8 * max(1.0, abs(want)), (q, n)


def test_pion_force_is_gradient_of_fermion_action():
    """F_a(n) = -d ln|det D_pi| / d phi_a(n) (central finite differences)."""
    Nt, Nx = 4, 4
    a, sigma, pi, rng = setup(Nt, Nx, seed=9)
    V = Nt * Nx
    eta = np.zeros((4 * V, V, 4), dtype=complex)
    for k in range(4 * V):
        eta[k].reshape(-1)[k] = 1.0
    F4, _ = O.force_pi(Nt, Nx, a, sigma, pi, eta, tol=1e-13, tol_mode=1, max_iter=5000)
    F4 = F4 * (4 * V)
    h = 1e-5
    for n in (0, 5, 11):
        for q in range(4):
            fields = np.vstack([sigma[None], pi])

            def lndet(f):
                return np.linalg.slogdet(dense(Nt, Nx, a, f[0], f[1:]))[1]

            fp, fm = fields.copy(), fields.copy()
            fp[q, n] += h
            fm[q, n] -= h
            want = -(lndet(fp) - lndet(fm)) / (2 * h)
            assert abs(F4[q, n] - want) < 1e-5 * max(1.0, abs(want)), (q, n, F4[q, n], want)


def test_pion_step_reduces_to_sigma_step_at_zero():
    """Fixed dt, pi = 0 before the step: sigma moves exactly as in the
    sigma-only step; the pions take their first noise and force."""
    Nt, Nx = 8, 8
    a = O.action(m2=-0.5, lam=1.0, g=0.5, m0=0.1, r=1.0, cut_fraction=0.35355339059327373)
    V = Nt * Nx
    sigma = O.uniform_field(1234, 0, V)
    phi4 = np.vstack([sigma[None], np.zeros((3, V))])
    want, ob = O.langevin_step(Nt, Nx, a, sigma, 1234, 0, 0, tol=1e-12, tol_mode=1, fixed_dt=0.01)
    got, obp = O.langevin_step_pi(Nt, Nx, a, phi4, 1234, 0, 0, tol=1e-12, tol_mode=1, fixed_dt=0.01)
    assert np.array_equal(got[0], want)
    assert obp.cg_iters == ob.cg_iters and obp.sum_phi == ob.sum_phi
    assert np.abs(got[1:]).max() > 0.01
    assert obp.sum_pi2 == pytest.approx(float((got[1:] ** 2).sum()), rel=1e-12)
