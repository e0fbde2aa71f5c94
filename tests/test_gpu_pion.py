"""The pion extension on the GPU (through the C ABI) against the CPU oracle's
pion restatement (itself pinned by dense linear algebra and the gradient of
ln|det D| in test_pion_oracle.py), and its exact reduction to the
reference's sigma-only path at pi = 0.

Tolerances: operator 1e-13 relative (FP64), 2e-6 (FP32); CG solutions 1e-9
relative at rel-res 1e-12; forces 1e-9 absolute; Langevin steps 1e-9
absolute on the four fields (CG at rel-res 1e-12), 1e-8 with the mixed
FP32/FP64 CG at rel-res 1e-10.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

S_HALF_PI = 0.35355339059327373


def params(yk, Nt, Nx, **kw):
    base = dict(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=0.1, wilson_param=1.0,
                cut_fraction=S_HALF_PI, Nt=Nt, Nx=Nx, cg_tol=1e-12, cg_tol_mode=yk.YK_TOL_REL, seed=1234,
                init=yk.YK_INIT_PHILOX, pions=1)
    base.update(kw)
    return yk.Params.default(**base)


def act(p):
    return O.action(m2=p.mass, lam=p.g, g=p.yukawa_coupling, m0=p.fermion_mass, r=p.wilson_param,
                    cut_fraction=p.cut_fraction, eps_bar=p.average_epsilon, drift_mode=p.drift_mode)


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def relerr(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_pion_initial_fields(ylib, cuda):
    yk = ylib
    Nt, Nx = 8, 12
    with yk.Context(params(yk, Nt, Nx)) as ctx:
        assert np.array_equal(ctx.get_field(), O.uniform_field(1234, 0, Nt * Nx))
        assert np.array_equal(ctx.get_pions(), O.uniform_pions(1234, 0, Nt * Nx))
    with yk.Context(params(yk, Nt, Nx, init=yk.YK_INIT_NONE)) as ctx:
        assert not ctx.get_pions().any()
    with yk.Context(params(yk, Nt, Nx, pions=0)) as ctx:
        with pytest.raises(yk.YukawaError):
            ctx.get_pions()


@pytest.mark.parametrize("Nt,Nx,r", [(8, 4, 1.0), (16, 16, 0.5), (6, 10, 1.0), (18, 64, 1.0)])
def test_pion_dirac_matches_oracle(ylib, cuda, Nt, Nx, r):
    yk = ylib
    p = params(yk, Nt, Nx, wilson_param=r)
    rng = np.random.default_rng(2)
    V = Nt * Nx
    with yk.Context(p) as ctx:
        sig, pi = rng.uniform(-1, 1, V), rng.uniform(-1, 1, (3, V))
        ctx.set_field(sig)
        ctx.set_pions(pi)
        psi = rng.normal(size=(V, 4)) + 1j * rng.normal(size=(V, 4))
        x = dev(cuda, psi)
        y = cuda.empty_like(x)
        x32 = x.to(cuda.complex64)
        y32 = cuda.empty_like(x32)
        for dag in (False, True):
            want = O.dirac_pi(Nt, Nx, act(p), sig, pi, psi, dag)
            ctx.dirac_apply(x, y, dag)
            ctx.dirac_apply(x32, y32, dag, yk.YK_FP32)
            ctx.synchronize()
            assert relerr(y.cpu().numpy(), want) < 1e-13, dag
            assert relerr(y32.cpu().numpy().astype(complex), want) < 2e-6, dag


def test_pion_dirac_is_sigma_operator_at_zero(ylib, cuda):
    yk = ylib
    Nt, Nx = 16, 8
    rng = np.random.default_rng(4)
    V = Nt * Nx
    sig = rng.uniform(-1, 1, V)
    psi = dev(cuda, rng.normal(size=(V, 4)) + 1j * rng.normal(size=(V, 4)))
    outs = []
    for pions in (1, 0):
        with yk.Context(params(yk, Nt, Nx, pions=pions, init=yk.YK_INIT_NONE)) as ctx:
            ctx.set_field(sig)
            y = cuda.empty_like(psi)
            yd = cuda.empty_like(psi)
            ctx.dirac_apply(psi, y, False)
            ctx.dirac_apply(psi, yd, True)
            ctx.synchronize()
            outs.append((y.cpu().numpy(), yd.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pion_cg_matches_oracle(ylib, cuda, precision):
    yk = ylib
    Nt, Nx = 16, 12
    p = params(yk, Nt, Nx)
    rng = np.random.default_rng(5)
    V = Nt * Nx
    prec = yk.YK_FP64 if precision == "fp64" else yk.YK_MIXED
    with yk.Context(p) as ctx:
        sig, pi = ctx.get_field(), ctx.get_pions()
        b = rng.normal(size=(V, 4)) + 1j * rng.normal(size=(V, 4))
        for mtype in (yk.YK_DAGGER, yk.YK_NORMAL):
            x = cuda.zeros(V, 4, dtype=cuda.complex128, device="cuda")
            st = ctx.cg_solve(dev(cuda, b), x, mtype=mtype, tol=1e-12, tol_mode=yk.YK_TOL_REL, max_iter=5000,
                              precision=prec)
            want, it, _ = O.cg_pi(Nt, Nx, act(p), sig, pi, b, mtype=mtype, tol=1e-12, tol_mode=1, max_iter=5000)
            assert st.converged == 1
            assert relerr(x.cpu().numpy(), want) < (1e-9 if precision == "fp64" else 1e-8), mtype
            if precision == "fp64":
                assert abs(st.iterations - it) <= 2


def test_pion_force_matches_oracle(ylib, cuda):
    yk = ylib
    Nt, Nx = 8, 12
    p = params(yk, Nt, Nx, n_rhs=2)
    rng = np.random.default_rng(6)
    V = Nt * Nx
    with yk.Context(p) as ctx:
        sig, pi = ctx.get_field(), ctx.get_pions()
        eta = np.zeros((2, V, 4), dtype=complex)
        eta.real = rng.normal(size=(2, V, 4))
        F = cuda.empty(4 * V, dtype=cuda.float64, device="cuda")
        ctx.fermion_force(F, eta=dev(cuda, eta))
        want, _ = O.force_pi(Nt, Nx, act(p), sig, pi, eta, tol=1e-12, tol_mode=1)
        got = F.cpu().numpy().reshape(4, V)
        assert np.abs(got - want).max() < 1e-9
        assert np.abs(want[1:]).max() > 1e-3   # the pion forces are not trivially zero


def test_pion_force_reduces_at_zero(ylib, cuda):
    yk = ylib
    Nt, Nx = 8, 12
    rng = np.random.default_rng(7)
    V = Nt * Nx
    sig = rng.uniform(-1, 1, V)
    eta = np.zeros((1, V, 4), dtype=complex)
    eta.real = rng.normal(size=(1, V, 4))
    Fs = []
    for pions in (1, 0):
        with yk.Context(params(yk, Nt, Nx, pions=pions, init=yk.YK_INIT_NONE)) as ctx:
            ctx.set_field(sig)
            F = cuda.zeros((4 if pions else 1) * V, dtype=cuda.float64, device="cuda")
            ctx.fermion_force(F, eta=dev(cuda, eta))
            Fs.append(F.cpu().numpy()[:V])
    assert np.array_equal(Fs[0], Fs[1])


@pytest.mark.parametrize("fixed_dt", [0.0, 0.01])
@pytest.mark.parametrize("Nt,Nx,s,n_rhs", [(16, 16, S_HALF_PI, 1), (8, 12, 1.0, 2)])
def test_pion_steps_match_oracle(ylib, cuda, Nt, Nx, s, n_rhs, fixed_dt):
    yk = ylib
    p = params(yk, Nt, Nx, cut_fraction=s, fixed_dt=fixed_dt, n_rhs=n_rhs)
    a = act(p)
    V = Nt * Nx
    with yk.Context(p) as ctx:
        phi4 = np.vstack([ctx.get_field()[None], ctx.get_pions()])
        for step in range(3):
            ctx.step(1)
            obs = ctx.observables()
            want, ro = O.langevin_step_pi(Nt, Nx, a, phi4, 1234, 0, step, n_rhs=n_rhs, tol=1e-12, tol_mode=1,
                                          fixed_dt=fixed_dt)
            got = np.vstack([ctx.get_field()[None], ctx.get_pions()])
            assert np.abs(got - want).max() < 1e-9, step
            assert abs(obs.eps - ro.eps) < 1e-12 * ro.eps
            assert abs(obs.cg_iterations - ro.cg_iters) <= 2 * n_rhs
            assert np.allclose(list(obs.sum_pi), got[1:].sum(axis=1), rtol=0, atol=1e-10)
            assert obs.sum_pi2 == pytest.approx(float((got[1:] ** 2).sum()), rel=1e-12)
            phi4 = got
        assert ctx.get_step() == 3 and obs.steps == 3


def test_pion_step_mixed_precision(ylib, cuda):
    yk = ylib
    Nt, Nx = 32, 32
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, reliable_every=50, fixed_dt=0.01)
    a = act(p)
    with yk.Context(p) as ctx:
        phi4 = np.vstack([ctx.get_field()[None], ctx.get_pions()])
        for step in range(2):
            ctx.step(1)
            want, _ = O.langevin_step_pi(Nt, Nx, a, phi4, 1234, 0, step, tol=1e-10, tol_mode=1, fixed_dt=0.01)
            got = np.vstack([ctx.get_field()[None], ctx.get_pions()])
            assert np.abs(got - want).max() < 1e-8, step
            phi4 = got


def test_pion_step_at_zero_moves_sigma_as_the_sigma_only_step(ylib, cuda):
    """pi = 0 before the step, fixed dt: sigma takes the sigma-only step (the
    CUDA path's real solver against its complex one: equal to the CG
    tolerance), and the pions their first noise and force."""
    yk = ylib
    Nt, Nx = 16, 16
    V = Nt * Nx
    sig0 = O.uniform_field(1234, 0, V)
    res = {}
    for pions in (1, 0):
        p = params(yk, Nt, Nx, pions=pions, init=yk.YK_INIT_NONE, fixed_dt=0.01)
        with yk.Context(p) as ctx:
            ctx.set_field(sig0)
            ctx.step(1)
            res[pions] = (ctx.get_field(), ctx.get_pions() if pions else None)
    assert np.abs(res[1][0] - res[0][0]).max() < 1e-12
    assert np.abs(res[1][1]).max() > 1e-3
    # and against the oracle's sigma-only step, exactly as the sigma path is
    want, _ = O.langevin_step(Nt, Nx, act(params(yk, Nt, Nx)), sig0, 1234, 0, 0, tol=1e-12, tol_mode=1,
                              fixed_dt=0.01)
    assert np.abs(res[1][0] - want).max() < 1e-9


def test_pion_checkpoint_roundtrip(ylib, cuda, tmp_path):
    yk = ylib
    Nt, Nx = 8, 8
    p = params(yk, Nt, Nx, fixed_dt=0.01)
    with yk.Context(p) as ctx:
        ctx.step(2)
        f = tmp_path / "pion.ckpt"
        ctx.checkpoint_save(f, 0.02)
        sig, pi, step = ctx.get_field(), ctx.get_pions(), ctx.get_step()
        ctx.step(1)
        ref = (ctx.get_field(), ctx.get_pions())
    with yk.Context(p) as ctx2:
        assert ctx2.checkpoint_load(f) == 0.02
        assert np.array_equal(ctx2.get_field(), sig) and np.array_equal(ctx2.get_pions(), pi)
        assert ctx2.get_step() == step
        ctx2.step(1)
        assert np.array_equal(ctx2.get_field(), ref[0]) and np.array_equal(ctx2.get_pions(), ref[1])
    with yk.Context(params(yk, Nt, Nx, pions=0)) as ctx3:
        with pytest.raises(yk.YukawaError):
            ctx3.checkpoint_load(f)


def test_pion_context_refuses_the_real_path_calls(ylib, cuda):
    yk = ylib
    with yk.Context(params(yk, 8, 8)) as ctx:
        with pytest.raises(yk.YukawaError):
            ctx.net_setup(2, 7)
        with pytest.raises(yk.YukawaError):
            ctx.step_learned(1)
        F = cuda.zeros(64, dtype=cuda.float64, device="cuda")
        with pytest.raises(yk.YukawaError):
            ctx.euler_update(F, F)


def test_pion_condensate_and_correlator(ylib, cuda):
    yk = ylib
    Nt, Nx = 8, 8
    p = params(yk, Nt, Nx)
    V = Nt * Nx
    with yk.Context(p) as ctx:
        sig, pi = ctx.get_field(), ctx.get_pions()
        cond, _ = ctx.condensate()
        eta = O.fermion_eta(1234, 0, 0, Nt, Nx, kind=3)
        F, _ = O.force_pi(Nt, Nx, act(p), sig, pi, eta, tol=1e-12, tol_mode=1)
        assert abs(cond - F[0].sum() / p.yukawa_coupling / V) < 1e-10
        corr, _ = ctx.correlator()
        e0 = np.zeros((V, 4), dtype=complex)
        e0[0, 0] = e0[0, 1] = 1.0
        y, _, _ = O.cg_pi(Nt, Nx, act(p), sig, pi, e0, mtype=0, tol=1e-12, tol_mode=1, max_iter=5000)
        y = O.dirac_pi(Nt, Nx, act(p), sig, pi, y, True)
        want = y.real.reshape(Nt, Nx, 4).sum(axis=(1, 2))
        assert np.abs(corr - want).max() < 1e-9
