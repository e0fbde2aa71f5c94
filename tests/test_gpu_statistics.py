"""Time-series observables with Gamma-method errors on the GPU
(yk_series_*), and long-run statistical agreement of the CUDA path with the
FP64 CPU oracle.

1. The device analysis against the oracle's host Gamma-method (itself pinned
   to an independent numpy implementation in test_oracle.py): <sigma>,
   <|sigma|>, chi = V <(s - <s>)^2> (analysis/functions.py:54-57) and the
   Binder cumulant 1 - <s^4>/(3 <s^2>^2) (functions.py:73-78) with Wolff's
   derived-quantity error; values to 1e-12, errors to 1e-9 relative.
2. The step's on-device recorder against the per-step observables.
3. Long runs of the 32 x 32 workload (m^2 = -0.5, lambda = 1, g = 0.5,
   m0 = 0.1, cutoff pi/2, dt = 0.01, CG rel-res 1e-10): the mixed FP32/FP64
   chain, the plain FP64 chain and the learned-preconditioner chain (seed
   1234), and the CPU oracle's FP64 chain from an independent seed (4321),
   300 burn-in steps and 3000 measured steps each.  <sigma>, <|sigma|>, chi
   and the condensate (a fresh force every 25 steps, main.cu:471-483) of every
   GPU chain agree with the oracle's within 4 combined standard errors
   (Gamma-method errors, S_tau = 1.5).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

S_HALF_PI = 0.35355339059327373
BURN, MEAS, COND_EVERY = 300, 3000, 25
BOUND = 4.0   # combined standard errors


def ar1(n, rho, seed, mean=2.0, scale=0.05):
    rng = np.random.default_rng(seed)
    x = np.empty(n)
    v = 0.0
    for i in range(n):
        v = rho * v + np.sqrt(1 - rho * rho) * rng.normal()
        x[i] = mean + scale * v
    return x


def binder_projection(x):
    m2, m4 = (x ** 2).mean(), (x ** 4).mean()
    g1, g2 = -1.0 / (3 * m2 * m2), 2 * m4 / (3 * m2 ** 3)
    return g1 * (x ** 4 - m4) + g2 * (x ** 2 - m2), 1 - m4 / (3 * m2 * m2)


@pytest.mark.parametrize("n,rho", [(4000, 0.9), (501, 0.0), (20000, 0.97)])
def test_series_analysis_matches_the_oracle_gamma_method(ylib, cuda, n, rho):
    yk = ylib
    V = 1024
    x = ar1(n, rho, seed=n)
    st = yk.series_stats(x, V)
    assert st.n == n

    def close(got, want):
        assert abs(got[0] - want[0]) <= 1e-12 * max(1.0, abs(want[0]))
        for k in range(1, 5):
            assert abs(got[k] - want[k]) <= 1e-9 * max(abs(want[k]), 1e-300), (k, got[k], want[k])

    close(list(st.sigma), O.gamma_method(x))
    close(list(st.abs_sigma), O.gamma_method(np.abs(x)))
    chi = O.gamma_method((x - x.mean()) ** 2)
    close(list(st.chi), [V * chi[0], V * chi[1], V * chi[2], chi[3], chi[4]])
    proj, bval = binder_projection(x)
    bw = O.gamma_method(proj)
    close(list(st.binder), [bval, bw[1], bw[2], bw[3], bw[4]])


def params(yk, precision, seed=1234, **kw):
    base = dict(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=0.1, wilson_param=1.0,
                cut_fraction=S_HALF_PI, Nt=32, Nx=32, fixed_dt=0.01, precision=precision, cg_tol=1e-10,
                cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=5000, reliable_every=50, seed=seed,
                init=yk.YK_INIT_PHILOX)
    base.update(kw)
    return yk.Params.default(**base)


def test_series_recorded_by_the_step(ylib, cuda):
    yk = ylib
    V = 32 * 32
    with yk.Context(params(yk, yk.YK_MIXED)) as ctx:
        ctx.series_record(100)
        want = []
        for _ in range(30):
            ctx.step(1)
            want.append(ctx.observables().sum_phi / V)
        ctx.step(20)   # graph replays record too
        rec = ctx.series_read()
        assert rec.size == 50 and np.array_equal(rec[:30], np.array(want))
        a = ctx.series_analyse()
        b = yk.series_stats(rec, V)
        assert list(a.sigma) == list(b.sigma) and list(a.chi) == list(b.chi)
        ctx.step(60)   # the recorder stops at its capacity
        assert ctx.series_read().size == 100


def gpu_chain(yk, precision, learned=False):
    p = params(yk, precision)
    V = p.Nt * p.Nx
    with yk.Context(p) as ctx:
        step = (lambda k: ctx.step_learned(k)) if learned else (lambda k: ctx.step(k))
        if learned:
            ctx.net_setup(2, 7)
            ctx.net_train(n_sources=4, n_levels=5, base_iter=4, steps=200, batch=4, lr=2e-3, seed=3)
        step(BURN)
        ctx.series_record(MEAS)
        cond = []
        for _ in range(MEAS // COND_EVERY):
            step(COND_EVERY)
            cond.append(ctx.condensate()[0])
        st = ctx.series_analyse()
        series = ctx.series_read()
        obs = ctx.observables()
    assert series.size == MEAS and obs.status in (0,)
    return st, np.array(cond), series, V


def oracle_chain(seed=4321):
    a = O.action(m2=-0.5, lam=1.0, g=0.5, m0=0.1, r=1.0, cut_fraction=S_HALF_PI)
    Nt = Nx = 32
    V = Nt * Nx
    phi = O.uniform_field(seed, 0, V)
    sig, cond = [], []
    for s in range(BURN + MEAS):
        phi, ob = O.langevin_step(Nt, Nx, a, phi, seed, 0, s, tol=1e-10, tol_mode=1, max_iter=5000, fixed_dt=0.01)
        if s >= BURN:
            sig.append(ob.sum_phi / V)
            if (s + 1 - BURN) % COND_EVERY == 0:
                eta = O.fermion_eta(seed, 0, s + 1, Nt, Nx, kind=3)
                F, _ = O.force(Nt, Nx, a, phi, eta, tol=1e-10, tol_mode=1, max_iter=5000)
                cond.append(F.sum() / a.g / V)
    return np.array(sig), np.array(cond)


@pytest.fixture(scope="module")
def oracle_run():
    return oracle_chain()


def agree(name, a, ea, b, eb):
    d = abs(a - b)
    lim = BOUND * np.hypot(ea, eb)
    assert d <= lim, f"{name}: {a:.6g} +- {ea:.2g} against the oracle's {b:.6g} +- {eb:.2g}"


@pytest.mark.parametrize("arm", ["mixed", "fp64", "learned"])
def test_long_run_observables_agree_with_the_oracle(ylib, cuda, oracle_run, arm):
    yk = ylib
    prec = yk.YK_FP64 if arm == "fp64" else yk.YK_MIXED
    st, cond, series, V = gpu_chain(yk, prec, learned=(arm == "learned"))
    osig, ocond = oracle_run
    ost = yk.series_stats(osig, V)
    agree("<sigma>", st.sigma[0], st.sigma[1], ost.sigma[0], ost.sigma[1])
    agree("<|sigma|>", st.abs_sigma[0], st.abs_sigma[1], ost.abs_sigma[0], ost.abs_sigma[1])
    agree("chi", st.chi[0], st.chi[1], ost.chi[0], ost.chi[1])
    gc, oc = O.gamma_method(cond), O.gamma_method(ocond)
    agree("condensate", gc[0], gc[1], oc[0], oc[1])
    # the errors are real estimates: tau_int of <sigma> of the order of the
    # oracle chain's, and many independent samples
    assert 0.5 < st.sigma[3] and st.sigma[3] < MEAS / 20
