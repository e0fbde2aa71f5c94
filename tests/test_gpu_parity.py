"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances: FP64 operator applications 1e-13 relative; FP32 Dirac 2e-6
relative; CG solutions to the oracle's FP64 solution at the stated
tolerances; Langevin steps 1e-9 absolute on the field after the CG has
converged to a relative residual of 1e-12.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

S_HALF_PI = 0.35355339059327373   # cutFraction for Lambda = pi/2


def params(yk, Nt, Nx, **kw):
    base = dict(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=0.1, wilson_param=1.0,
                cut_fraction=S_HALF_PI, Nt=Nt, Nx=Nx, cg_tol=1e-12, cg_tol_mode=yk.YK_TOL_REL, seed=1234,
                init=yk.YK_INIT_PHILOX)
    base.update(kw)
    return yk.Params.default(**base)


def act(p):
    return O.action(m2=p.mass, lam=p.g, g=p.yukawa_coupling, m0=p.fermion_mass, r=p.wilson_param,
                    cut_fraction=p.cut_fraction, eps_bar=p.average_epsilon, drift_mode=p.drift_mode)


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def rand_spinor(rng, V):
    return rng.normal(size=(V, 4)) + 1j * rng.normal(size=(V, 4))


# rows of a multiple of 32 sites take the column-strip kernel (blocks of 32,
# 96, 256 threads; bands of 16 rows, the last one partial), the rest the
# site-per-thread kernel
@pytest.mark.parametrize("Nt,Nx,r", [(8, 4, 1.0), (16, 16, 0.5), (6, 10, 1.0), (64, 32, 1.0), (2, 8, 0.0),
                                     (20, 96, 1.0), (3, 256, 0.5), (40, 512, 1.0)])
def test_dirac_fp64(ylib, cuda, Nt, Nx, r):
    yk = ylib
    p = params(yk, Nt, Nx, wilson_param=r)
    rng = np.random.default_rng(1)
    with yk.Context(p) as ctx:
        sig = rng.uniform(-1, 1, Nt * Nx)
        ctx.set_field(sig)
        psi = rand_spinor(rng, Nt * Nx)
        x = dev(cuda, psi)
        y = cuda.empty_like(x)
        for dag in (False, True):
            yk.DiracOP(ctx).applyD(x, y, yk.MatrixType.Dagger if dag else yk.MatrixType.Normal)
            ctx.synchronize()
            want = O.dirac(Nt, Nx, act(p), sig, psi, dag)
            err = np.abs(host(y) - want).max() / np.abs(want).max()
            assert err < 1e-13, (dag, err)


@pytest.mark.parametrize("Nt,Nx", [(32, 16), (36, 64), (16, 288)])
def test_dirac_fp32(ylib, cuda, Nt, Nx):
    yk = ylib
    p = params(yk, Nt, Nx, cut_fraction=1.0)   # white noise: any Nx
    rng = np.random.default_rng(2)
    with yk.Context(p) as ctx:
        sig = rng.uniform(-1, 1, Nt * Nx)
        ctx.set_field(sig)
        psi = rand_spinor(rng, Nt * Nx).astype(np.complex64)
        x = dev(cuda, psi)
        y = cuda.empty_like(x)
        for dag in (False, True):
            ctx.dirac_apply(x, y, dagger=dag, precision=yk.YK_FP32)
            ctx.synchronize()
            want = O.dirac(Nt, Nx, act(p), sig, psi.astype(np.complex128), dag)
            assert np.abs(host(y) - want).max() / np.abs(want).max() < 2e-6, dag


@pytest.mark.parametrize("mtype", [0, 1])
@pytest.mark.parametrize("Nt,Nx", [(8, 4), (32, 32), (6, 10)])
def test_cg_fp64(ylib, cuda, Nt, Nx, mtype):
    yk = ylib
    p = params(yk, Nt, Nx)
    rng = np.random.default_rng(3)
    with yk.Context(p) as ctx:
        sig = rng.uniform(-1, 1, Nt * Nx)
        ctx.set_field(sig)
        b = rand_spinor(rng, Nt * Nx)
        bd, xd = dev(cuda, b), dev(cuda, np.zeros_like(b))
        st = ctx.cg_solve(bd, xd, mtype=mtype, tol=1e-12, tol_mode=yk.YK_TOL_REL)
        want, it, _ = O.cg(Nt, Nx, act(p), sig, b, mtype=mtype, tol=1e-12, tol_mode=1)
        x = host(xd)
        assert np.abs(x - want).max() / np.abs(want).max() < 1e-9
        assert abs(st.iterations - it) <= 1 and st.converged == 1
        # reference stopping rule (absolute 1e-8, IterMax 1000)
        st2 = yk.CGsolver(ctx).solve(bd, xd, None, yk.MatrixType(mtype))
        want2, it2, _ = O.cg(Nt, Nx, act(p), sig, b, mtype=mtype)
        assert abs(st2.iterations - it2) <= 1
        assert np.abs(host(xd) - want2).max() / np.abs(want2).max() < 1e-7


def test_cg_mixed_reaches_fp64_residual(ylib, cuda):
    yk = ylib
    Nt, Nx = 64, 64
    p = params(yk, Nt, Nx)
    rng = np.random.default_rng(4)
    with yk.Context(p) as ctx:
        sig = rng.uniform(-1, 1, Nt * Nx)
        ctx.set_field(sig)
        b = rand_spinor(rng, Nt * Nx)
        bd, xd = dev(cuda, b), dev(cuda, np.zeros_like(b))
        st = ctx.cg_solve(bd, xd, tol=1e-10, tol_mode=yk.YK_TOL_REL, precision=yk.YK_MIXED)
        x = host(xd)
        a = act(p)
        r = b - O.dirac(Nt, Nx, a, sig, O.dirac(Nt, Nx, a, sig, x), True)
        assert np.linalg.norm(r) <= 1.05e-10 * np.linalg.norm(b), np.linalg.norm(r) / np.linalg.norm(b)
        assert st.converged == 1 and st.reliable_updates >= 1
        want, it, _ = O.cg(Nt, Nx, a, sig, b, tol=1e-10, tol_mode=1)
        assert np.abs(x - want).max() / np.abs(want).max() < 1e-7
        assert st.iterations <= 1.5 * it + 60


@pytest.mark.parametrize("scale,tol", [(1e-9, 1e-10), (1.0, 1e-12)])
def test_cg_mixed_small_residuals(ylib, cuda, scale, tol):
    # residuals small in absolute terms (a right-hand side of norm ~1e-7, or a
    # 1e-12 relative target): the FP32 scalar step of the mixed solver stays
    # finite (|<p, Ap>|^2 would underflow FP32) and converges on the FP64 residual
    yk = ylib
    Nt, Nx = 32, 32
    p = params(yk, Nt, Nx)
    rng = np.random.default_rng(12)
    with yk.Context(p) as ctx:
        sig = rng.uniform(-1, 1, Nt * Nx)
        ctx.set_field(sig)
        b = rand_spinor(rng, Nt * Nx) * scale
        xd = dev(cuda, np.zeros_like(b))
        st = ctx.cg_solve(dev(cuda, b), xd, tol=tol, tol_mode=yk.YK_TOL_REL, max_iter=5000, precision=yk.YK_MIXED)
        x = host(xd)
        a = act(p)
        r = b - O.dirac(Nt, Nx, a, sig, O.dirac(Nt, Nx, a, sig, x), True)
        assert st.converged == 1
        assert np.linalg.norm(r) <= 1.05 * tol * np.linalg.norm(b)


def test_cg_iteration_cap_reports_noconv(ylib, cuda):
    yk = ylib
    p = params(yk, 16, 16)
    rng = np.random.default_rng(5)
    with yk.Context(p) as ctx:
        ctx.set_field(rng.uniform(-1, 1, 256))
        b = dev(cuda, rand_spinor(rng, 256))
        x = cuda.zeros_like(b)
        with pytest.raises(yk.YukawaError) as e:
            ctx.cg_solve(b, x, tol=1e-14, tol_mode=yk.YK_TOL_REL, max_iter=3)
        assert e.value.status == yk.YK_ENOCONV
        st = ctx.cg_solve(b, x, tol=1e-14, tol_mode=yk.YK_TOL_REL, max_iter=3, allow_noconv=True)
        assert st.iterations == 3 and st.converged == 0
        z = cuda.zeros_like(b)
        st0 = ctx.cg_solve(z, x)
        assert st0.iterations == 0 and np.abs(host(x)).max() == 0.0


@pytest.mark.parametrize("n_rhs,drift_mode", [(1, 0), (2, 0), (1, 1)])
def test_force_injected_eta(ylib, cuda, n_rhs, drift_mode):
    yk = ylib
    Nt, Nx = 16, 8
    p = params(yk, Nt, Nx, n_rhs=n_rhs, drift_mode=drift_mode, cut_fraction=0.5)
    rng = np.random.default_rng(6)
    with yk.Context(p) as ctx:
        sig = rng.uniform(-1, 1, Nt * Nx)
        ctx.set_field(sig)
        eta = np.zeros((n_rhs, Nt * Nx, 4), complex)
        eta.real = rng.normal(size=eta.shape)
        F = cuda.empty(Nt * Nx, dtype=cuda.float64, device="cuda")
        ctx.fermion_force(F, dev(cuda, eta))
        want, _ = O.force(Nt, Nx, act(p), sig, eta, tol=1e-12, tol_mode=1)
        assert np.abs(host(F) - want).max() < 1e-9


def test_force_philox_eta(ylib, cuda):
    yk = ylib
    Nt, Nx = 16, 16
    p = params(yk, Nt, Nx)
    with yk.Context(p) as ctx:
        sig = ctx.get_field()
        F = cuda.empty(Nt * Nx, dtype=cuda.float64, device="cuda")
        yk.FermionicDrift(ctx).getForce(F)
        eta = O.fermion_eta(1234, 0, 0, Nt, Nx)
        want, _ = O.force(Nt, Nx, act(p), sig, eta, tol=1e-12, tol_mode=1)
        assert np.abs(host(F) - want).max() < 1e-9


@pytest.mark.parametrize("Nt,Nx,s", [(16, 16, S_HALF_PI), (8, 4, 0.25), (6, 10, 0.3), (32, 64, 0.2),
                                     (16, 16, 1.0), (256, 8, 0.3)])
def test_coloured_noise(ylib, cuda, Nt, Nx, s):
    yk = ylib
    p = params(yk, Nt, Nx, cut_fraction=s)
    rng = np.random.default_rng(7)
    with yk.Context(p) as ctx:
        w = rng.normal(size=Nt * Nx)
        xi = cuda.empty(Nt * Nx, dtype=cuda.float64, device="cuda")
        yk.ColouredNoise(ctx, xi)(dev(cuda, w))
        ctx.synchronize()
        assert np.abs(host(xi) - O.coloured_noise(Nt, Nx, s, w)).max() < 1e-13
        # Philox white noise at step 0 of chain 0
        yk.ColouredNoise(ctx, xi)()
        ctx.synchronize()
        w0 = O.normals(1234, 0, 0, 1, 0, Nt * Nx)
        assert np.abs(host(xi) - O.coloured_noise(Nt, Nx, s, w0)).max() < 1e-13


@pytest.mark.parametrize("Nt,Nx,s", [(16, 16, 1.0), (6, 10, 1.0), (32, 64, 1.0), (16, 16, S_HALF_PI)])
def test_philox_white_noise_bit_exact(ylib, cuda, Nt, Nx, s):
    # the GPU's FP32 Box-Muller (IEEE round-to-nearest intrinsics throughout)
    # and the oracle's C restatement give the same normals, bit for bit: with
    # cutFraction >= 1 the noise is the white noise itself; with a cutoff the
    # filter of the oracle's normals matches to rounding
    yk = ylib
    p = params(yk, Nt, Nx, cut_fraction=s)
    with yk.Context(p) as ctx:
        xi = cuda.empty(Nt * Nx, dtype=cuda.float64, device="cuda")
        yk.ColouredNoise(ctx, xi)()
        ctx.synchronize()
        w = O.normals(1234, 0, 0, 1, 0, Nt * Nx)
        if s >= 1.0:
            assert np.array_equal(host(xi), w)
        else:
            assert np.abs(host(xi) - O.coloured_noise(Nt, Nx, s, w)).max() < 1e-13


def test_euler_update_injected(ylib, cuda):
    yk = ylib
    Nt, Nx = 16, 32
    p = params(yk, Nt, Nx)
    rng = np.random.default_rng(8)
    with yk.Context(p) as ctx:
        phi = rng.uniform(-1, 1, Nt * Nx)
        ctx.set_field(phi)
        F, xi = rng.normal(size=Nt * Nx) * 0.3, rng.normal(size=Nt * Nx)
        obs = ctx.euler_update(dev(cuda, F), dev(cuda, xi))
        drift = O.bosonic_drift(Nt, Nx, p.mass, p.g, phi, F)
        want, eps, m = O.euler_update(phi, drift, xi, p.average_epsilon)
        assert abs(obs.eps - eps) <= 1e-15 * eps and abs(obs.max_drift - m) <= 1e-15 * m
        assert np.abs(ctx.get_field() - want).max() < 1e-14
        assert abs(obs.sum_phi - want.sum()) < 1e-10 and obs.steps == 1


@pytest.mark.parametrize("fixed_dt", [0.0, 0.01])
@pytest.mark.parametrize("Nt,Nx,s", [(16, 16, S_HALF_PI), (8, 12, 1.0)])
def test_langevin_steps_match_oracle(ylib, cuda, Nt, Nx, s, fixed_dt):
    yk = ylib
    p = params(yk, Nt, Nx, cut_fraction=s, fixed_dt=fixed_dt)
    a = act(p)
    with yk.Context(p) as ctx:
        phi = ctx.get_field()
        assert np.array_equal(phi, O.uniform_field(1234, 0, Nt * Nx))
        for step in range(4):
            ctx.step(1)
            obs = ctx.observables()
            phi, ro = O.langevin_step(Nt, Nx, a, phi, 1234, 0, step, tol=1e-12, tol_mode=1, fixed_dt=fixed_dt)
            got = ctx.get_field()
            assert np.abs(got - phi).max() < 1e-9, step
            assert abs(obs.eps - ro.eps) < 1e-12 * ro.eps
            assert abs(obs.cg_iterations - ro.cg_iters) <= 2
            phi = got   # keep the chains identical to the last bit of the GPU field
        assert ctx.get_step() == 4 and obs.steps == 4


@pytest.mark.parametrize("cluster", ["1", "0"], ids=["cluster_cg", "grid_cg"])
def test_langevin_mixed_precision_step(ylib, cuda, monkeypatch, cluster):
    # the cluster-resident CG (lattices that fit a 16-CTA cluster, opt-in)
    # and the grid-wide CG kernel
    monkeypatch.setenv("YK_CG_CLUSTER", cluster)
    yk = ylib
    Nt, Nx = 32, 32
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
    a = act(p)
    with yk.Context(p) as ctx:
        phi = ctx.get_field()
        ctx.step(1)
        want, ro = O.langevin_step(Nt, Nx, a, phi, 1234, 0, 0, tol=1e-10, tol_mode=1, fixed_dt=0.01)
        assert np.abs(ctx.get_field() - want).max() < 1e-8
        assert ctx.observables().status == 0


def _mixed_run(yk, monkeypatch, halo, Nt, Nx, steps, eo="0"):
    monkeypatch.setenv("YK_CG_HALO", halo)
    monkeypatch.setenv("YK_CG_EO", eo)
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
    with yk.Context(p) as ctx:
        ctx.profile_begin()
        ctx.step(steps)
        pr = ctx.profile_end()
        return ctx.get_field(), pr.cg_kernel, pr.cg_iterations, ctx.observables().status


@pytest.mark.parametrize("Nt,Nx", [(32, 32), (128, 64), (256, 256), (1024, 64), (40, 24), (41, 25)])
def test_halo_cg_matches_grid_cg(ylib, cuda, monkeypatch, Nt, Nx):
    # the halo CG kernel (single-system mixed solves whose halo slices fit)
    # against cg_kernel on the same trajectory: the same per-site arithmetic,
    # tile partials and fixed-point sums, so the same iterates
    yk = ylib
    f_halo, k_halo, it_halo, st_halo = _mixed_run(yk, monkeypatch, "1", Nt, Nx, 3)
    f_grid, k_grid, it_grid, st_grid = _mixed_run(yk, monkeypatch, "0", Nt, Nx, 3)
    assert (k_halo, k_grid) == (1, 0)
    assert st_halo == 0 and st_grid == 0
    assert it_halo == it_grid
    assert np.array_equal(f_halo, f_grid)


def test_halo_cg_step_against_oracle(ylib, cuda, monkeypatch):
    # one Langevin step through the halo kernel against the FP64 oracle
    monkeypatch.setenv("YK_CG_HALO", "1")
    monkeypatch.setenv("YK_CG_EO", "0")
    yk = ylib
    Nt, Nx = 48, 32
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
    with yk.Context(p) as ctx:
        phi = ctx.get_field()
        ctx.profile_begin()
        ctx.step(1)
        assert ctx.profile_end().cg_kernel == 1
        want, _ = O.langevin_step(Nt, Nx, act(p), phi, 1234, 0, 0, tol=1e-10, tol_mode=1, fixed_dt=0.01)
        assert np.abs(ctx.get_field() - want).max() < 1e-8
        assert ctx.observables().status == 0


@pytest.mark.parametrize("patch", ["16", "8", "32", "0"], ids=["patches16", "patches8", "patches32", "rows"])
@pytest.mark.parametrize("Nt,Nx", [(32, 32), (256, 256), (64, 128), (128, 64), (48, 32)])
def test_evenodd_cg_steps_against_oracle(ylib, cuda, monkeypatch, Nt, Nx, patch):
    # the even-odd Schur-complement solve of the step (CGNE on S S^dag, its
    # residual the true residual of D^dag chi = eta, the same rule relative to
    # |eta|) against the FP64 oracle's CG on D^dag D: the fields of three steps
    # within 1e-8, in fewer iterations than the halo kernel's D^dag D solve;
    # blocks owning 16 x 16, 16 x 8 or 32 x 32 patches of the compact lattice,
    # or rows (a lattice the asked-for patches do not tile runs rows)
    yk = ylib
    monkeypatch.setenv("YK_CG_EO", "1")
    monkeypatch.setenv("YK_CG_EO_PATCH", patch)
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01, reliable_every=50)
    with yk.Context(p) as ctx:
        phi = ctx.get_field()
        ctx.profile_begin()
        ctx.step(1)
        pr = ctx.profile_end()
        assert pr.cg_kernel == 3, "the step's solve runs the even-odd kernel"
        got = [ctx.get_field()]
        ctx.step(2)
        got.append(ctx.get_field())
        obs = ctx.observables()
    assert obs.status == 0
    a = act(p)
    want, _ = O.langevin_step(Nt, Nx, a, phi, 1234, 0, 0, tol=1e-10, tol_mode=1, fixed_dt=0.01)
    assert np.abs(got[0] - want).max() < 1e-8
    w = got[0]
    for s in (1, 2):
        w, _ = O.langevin_step(Nt, Nx, a, w, 1234, 0, s, tol=1e-10, tol_mode=1, fixed_dt=0.01)
    assert np.abs(got[1] - w).max() < 1e-8
    _, k_halo, it_halo, _ = _mixed_run(yk, monkeypatch, "1", Nt, Nx, 1, eo="0")
    assert pr.cg_iterations < 0.7 * it_halo, (pr.cg_iterations, it_halo)


def test_evenodd_512_takes_32x32_patches(ylib, cuda, monkeypatch):
    # 512 x 512: its 16 x 16 patches (512) are more than the GPU holds at
    # once, its 32 x 32 patches (128) are not; the single-system kernel takes
    # them and the step agrees with the FP64 oracle
    yk = ylib
    Nt = Nx = 512
    monkeypatch.delenv("YK_CG_EO_PATCH", raising=False)
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01, reliable_every=50)
    with yk.Context(p) as ctx:
        phi = ctx.get_field()
        ctx.profile_begin()
        ctx.step(1)
        pr = ctx.profile_end()
        assert pr.cg_kernel == 3 and pr.cg_grid == 128, (pr.cg_kernel, pr.cg_grid)
        got = ctx.get_field()
        assert ctx.observables().status == 0
    want, _ = O.langevin_step(Nt, Nx, act(p), phi, 1234, 0, 0, tol=1e-10, tol_mode=1, fixed_dt=0.01)
    assert np.abs(got - want).max() < 1e-8


def test_evenodd_1024_single_chain_takes_the_patch_kernel(ylib, cuda, monkeypatch):
    # 1024 x 1024, one chain: no single-system form fits (its 32 x 32 patches
    # are 512), so the batched patch kernel runs with one system; the step
    # agrees with the FP64 oracle
    yk = ylib
    Nt = Nx = 1024
    monkeypatch.delenv("YK_CG_EOP", raising=False)
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01, reliable_every=50)
    with yk.Context(p) as ctx:
        phi = ctx.get_field()
        ctx.profile_begin()
        ctx.step(1)
        pr = ctx.profile_end()
        assert pr.cg_kernel == 5, pr.cg_kernel
        got = ctx.get_field()
        assert ctx.observables().status == 0
    want, _ = O.langevin_step(Nt, Nx, act(p), phi, 1234, 0, 0, tol=1e-10, tol_mode=1, fixed_dt=0.01)
    assert np.abs(got - want).max() < 1e-8


def test_evenodd_force_and_condensate_match_the_full_solve(ylib, cuda, monkeypatch):
    # yk_fermion_force (the step's Philox source) and yk_condensate through
    # the even-odd solve against the same calls through the D^dag D solve
    yk = ylib
    Nt, Nx = 64, 64
    p = params(yk, Nt, Nx, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
    res = {}
    for eo in ("1", "0"):
        monkeypatch.setenv("YK_CG_EO", eo)
        with yk.Context(p) as ctx:
            F = cuda.empty(Nt * Nx, dtype=cuda.float64, device="cuda")
            ctx.fermion_force(F)
            cond, _ = ctx.condensate()
            res[eo] = (F.cpu().numpy(), cond)
    assert np.abs(res["1"][0] - res["0"][0]).max() < 1e-8 * np.abs(res["0"][0]).max()
    assert abs(res["1"][1] - res["0"][1]) < 1e-8 * abs(res["0"][1])


def test_evenodd_skips_odd_lattices(ylib, cuda, monkeypatch):
    # odd extents have no checkerboard: the halo kernel's D^dag D solve runs
    yk = ylib
    monkeypatch.setenv("YK_CG_EO", "1")
    p = params(yk, 41, 25, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
    with yk.Context(p) as ctx:
        ctx.profile_begin()
        ctx.step(1)
        assert ctx.profile_end().cg_kernel in (0, 1)


def test_batched_chains_equal_single_chains(ylib, cuda):
    yk = ylib
    specs = [(16, 16, 0.1, 0.5, S_HALF_PI), (32, 8, 0.25, 0.3, 0.2), (8, 8, 0.05, 0.8, 1.0)]
    ps = [params(yk, nt, nx, fermion_mass=m0, yukawa_coupling=g, cut_fraction=s, n_rhs=2)
          for nt, nx, m0, g, s in specs]
    with yk.Context(ps) as ctx:
        ctx.step(3)
        batched = [ctx.get_field(c) for c in range(len(ps))]
        obs_b = [ctx.observables(c) for c in range(len(ps))]
    for c, p in enumerate(ps):
        # the Philox key of a chain includes its chain index c
        phi = O.uniform_field(1234, c, p.Nt * p.Nx)
        for step in range(3):
            phi, _ = O.langevin_step(p.Nt, p.Nx, act(p), phi, 1234, c, step, n_rhs=2, tol=1e-12, tol_mode=1)
        assert np.abs(batched[c] - phi).max() < 1e-9, c
        assert obs_b[c].steps == 3


@pytest.mark.parametrize("cluster", ["1", "0"], ids=["cluster_cg", "grid_cg"])
def test_batched_mixed_chains(ylib, cuda, monkeypatch, cluster):
    # batched chains of different shapes (rows not divisible by 16, CTAs of a
    # cluster without rows, two right-hand sides) through the mixed solver
    monkeypatch.setenv("YK_CG_CLUSTER", cluster)
    yk = ylib
    specs = [(40, 24, 0.1, 0.5, S_HALF_PI, 2), (8, 8, 0.25, 0.3, 0.2, 1), (16, 64, 0.05, 0.8, 1.0, 1)]
    ps = [params(yk, nt, nx, fermion_mass=m0, yukawa_coupling=g, cut_fraction=s, n_rhs=nr, precision=yk.YK_MIXED,
                 cg_tol=1e-10, fixed_dt=0.01)
          for nt, nx, m0, g, s, nr in specs]
    with yk.Context(ps) as ctx:
        ctx.step(2)
        got = [ctx.get_field(c) for c in range(len(ps))]
        obs = [ctx.observables(c) for c in range(len(ps))]
    for c, p in enumerate(ps):
        phi = O.uniform_field(1234, c, p.Nt * p.Nx)
        for step in range(2):
            phi, _ = O.langevin_step(p.Nt, p.Nx, act(p), phi, 1234, c, step, n_rhs=p.n_rhs, tol=1e-10, tol_mode=1,
                                     fixed_dt=0.01)
        assert np.abs(got[c] - phi).max() < 1e-8, c
        assert obs[c].steps == 2 and obs[c].status == 0


@pytest.mark.parametrize("balance", ["0", "1"], ids=["uniform_ranges", "balanced_ranges"])
def test_batched_block_ranges_keep_results(ylib, cuda, monkeypatch, balance):
    # batched chains with block ranges balanced by the previous step's
    # iterations: the same fields as the uniform ranges (every tile's partial
    # is summed in a fixed order), checked against the FP64 oracle
    monkeypatch.setenv("YK_CG_BALANCE", balance)
    yk = ylib
    specs = [(40, 24, 0.1, 0.5, S_HALF_PI, 2), (8, 8, 0.25, 0.3, 0.2, 1), (64, 64, 0.05, 0.8, 1.0, 1)]
    ps = [params(yk, nt, nx, fermion_mass=m0, yukawa_coupling=g, cut_fraction=s, n_rhs=nr, precision=yk.YK_MIXED,
                 cg_tol=1e-10, fixed_dt=0.01)
          for nt, nx, m0, g, s, nr in specs]
    with yk.Context(ps) as ctx:
        ctx.step(3)
        got = [ctx.get_field(c) for c in range(len(ps))]
        assert all(ctx.observables(c).status == 0 for c in range(len(ps)))
    for c, p in enumerate(ps):
        phi = O.uniform_field(1234, c, p.Nt * p.Nx)
        for step in range(3):
            phi, _ = O.langevin_step(p.Nt, p.Nx, act(p), phi, 1234, c, step, n_rhs=p.n_rhs, tol=1e-10, tol_mode=1,
                                     fixed_dt=0.01)
        assert np.abs(got[c] - phi).max() < 1e-8, c


@pytest.mark.parametrize("specs,kernel", [
    # even lattices: the batched even-odd CG (work dealt out per pass)
    ([(40, 24, 0.1, 0.5, S_HALF_PI, 2), (8, 8, 0.25, 0.3, 0.2, 1), (64, 64, 0.05, 0.8, 1.0, 3)], 4),
    # one odd lattice: the whole batch keeps the D^dag D grid kernel
    ([(40, 24, 0.1, 0.5, S_HALF_PI, 2), (9, 8, 0.25, 0.3, 1.0, 1)], 0),
    # a single lattice neither 16 x 16 patches nor whole rows fit (18 rows)
    ([(18, 1000, 0.1, 0.5, 1.0, 1)], 4),
], ids=["even_batch", "odd_lattice", "single_wide"])
def test_batched_even_odd_cg(ylib, cuda, specs, kernel):
    # the step's solves of every chain and right-hand side through one
    # even-odd launch; fields within 1e-8 of the FP64 oracle's steps (the
    # reference's D^dag D solve, FermionicDrift.cu:57-100)
    yk = ylib
    ps = [params(yk, nt, nx, fermion_mass=m0, yukawa_coupling=g, cut_fraction=s, n_rhs=nr, precision=yk.YK_MIXED,
                 cg_tol=1e-10, fixed_dt=0.01)
          for nt, nx, m0, g, s, nr in specs]
    with yk.Context(ps) as ctx:
        ctx.profile_begin()
        ctx.step(1)
        pr = ctx.profile_end()
        assert pr.cg_kernel == kernel
        ctx.step(2)
        got = [ctx.get_field(c) for c in range(len(ps))]
        obs = [ctx.observables(c) for c in range(len(ps))]
    for c, p in enumerate(ps):
        assert obs[c].steps == 3 and obs[c].status == 0, c
        phi = O.uniform_field(1234, c, p.Nt * p.Nx)
        for step in range(3):
            phi, _ = O.langevin_step(p.Nt, p.Nx, act(p), phi, 1234, c, step, n_rhs=p.n_rhs, tol=1e-10, tol_mode=1,
                                     fixed_dt=0.01)
        assert np.abs(got[c] - phi).max() < 1e-8, c


@pytest.mark.parametrize("r", [0.7, 1.3])
def test_evenodd_wilson_parameter(ylib, cuda, r):
    # a Wilson parameter r != 1, where the time hops' coefficients -(r -+ 1)/2
    # are both nonzero (in float-float in the reliable updates, round 0 and the
    # reconstruction): the single-system kernel (64 x 64), the batched one
    # (two chains, one with two right-hand sides) and the batched patch
    # kernel against the FP64 oracle
    yk = ylib
    for specs, kernel in (([(64, 64, 0.1, 0.5, 1)], 3), ([(32, 48, 0.1, 0.5, 2), (16, 16, 0.2, 0.7, 1)], 4),
                          ([(32, 64, 0.1, 0.5, 2), (32, 32, 0.2, 0.7, 1)], 5)):
        ps = [params(yk, nt, nx, fermion_mass=m0, yukawa_coupling=g, n_rhs=nr, wilson_param=r,
                     precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
              for nt, nx, m0, g, nr in specs]
        with yk.Context(ps) as ctx:
            ctx.profile_begin()
            ctx.step(1)
            pr = ctx.profile_end()
            assert pr.cg_kernel == kernel, (pr.cg_kernel, kernel)
            ctx.step(1)
            got = [ctx.get_field(c) for c in range(len(ps))]
            assert all(ctx.observables(c).status == 0 for c in range(len(ps)))
        for c, p in enumerate(ps):
            phi = O.uniform_field(1234, c, p.Nt * p.Nx)
            for step in range(2):
                phi, _ = O.langevin_step(p.Nt, p.Nx, act(p), phi, 1234, c, step, n_rhs=p.n_rhs, tol=1e-10,
                                         tol_mode=1, fixed_dt=0.01)
            assert np.abs(got[c] - phi).max() < 1e-8, (c, r)


@pytest.mark.parametrize("eop", ["1", "0"], ids=["patch_kernel", "four_pass_kernel"])
def test_batched_patch_kernel(ylib, cuda, monkeypatch, eop):
    # a batch whose compact lattices 32 x 16 patches tile (32 x 32 and 64 x 32:
    # the staged buffer wraps across the whole compact row; 64 x 64 with three
    # right-hand sides; 32 x 96; different masses, so the systems converge and
    # run their reliable updates in different rounds): the batched patch
    # kernel, and the four-pass kernel, against the FP64 oracle
    monkeypatch.setenv("YK_CG_EOP", eop)
    yk = ylib
    specs = [(32, 32, 0.1, 0.5, 2), (64, 32, 0.3, 0.4, 1), (64, 64, 0.05, 0.8, 3), (32, 96, 0.2, 0.6, 1)]
    ps = [params(yk, nt, nx, fermion_mass=m0, yukawa_coupling=g, n_rhs=nr, precision=yk.YK_MIXED, cg_tol=1e-10,
                 fixed_dt=0.01, reliable_every=50)
          for nt, nx, m0, g, nr in specs]
    with yk.Context(ps) as ctx:
        ctx.profile_begin()
        ctx.step(1)
        pr = ctx.profile_end()
        assert pr.cg_kernel == (5 if eop == "1" else 4), pr.cg_kernel
        ctx.step(2)
        got = [ctx.get_field(c) for c in range(len(ps))]
        obs = [ctx.observables(c) for c in range(len(ps))]
    for c, p in enumerate(ps):
        assert obs[c].steps == 3 and obs[c].status == 0, c
        phi = O.uniform_field(1234, c, p.Nt * p.Nx)
        for step in range(3):
            phi, _ = O.langevin_step(p.Nt, p.Nx, act(p), phi, 1234, c, step, n_rhs=p.n_rhs, tol=1e-10, tol_mode=1,
                                     fixed_dt=0.01)
        assert np.abs(got[c] - phi).max() < 1e-8, c


def test_autotune_keeps_results(ylib, cuda, monkeypatch):
    # batched chains: the tuned CG grid (automatic before the first capture,
    # and again by an explicit call between steps) gives the same fields, bit
    # for bit, as the untuned co-resident grid
    yk = ylib
    specs = [(40, 24, 0.1, 0.5, S_HALF_PI, 2), (8, 8, 0.25, 0.3, 0.2, 1), (64, 64, 0.05, 0.8, 1.0, 1)]
    ps = [params(yk, nt, nx, fermion_mass=m0, yukawa_coupling=g, cut_fraction=s, n_rhs=nr, precision=yk.YK_MIXED,
                 cg_tol=1e-10, fixed_dt=0.01)
          for nt, nx, m0, g, s, nr in specs]
    monkeypatch.setenv("YK_AUTOTUNE", "0")
    with yk.Context(ps) as ctx:
        ctx.step(4)
        assert ctx.tune_report().cg_grid == 0
        want = [ctx.get_field(c) for c in range(len(ps))]
    monkeypatch.delenv("YK_AUTOTUNE")
    with yk.Context(ps) as ctx:
        ctx.step(2)
        t = ctx.tune_report()
        assert t.cg_candidates >= 2 and 8 <= t.cg_grid <= t.cg_grid_max
        assert t.cg_ms_chosen <= t.cg_ms_max
        t2 = ctx.autotune()
        assert t2.cg_candidates >= 2
        ctx.step(2)
        got = [ctx.get_field(c) for c in range(len(ps))]
        assert all(ctx.observables(c).status == 0 for c in range(len(ps)))
    for c in range(len(ps)):
        assert np.array_equal(got[c], want[c]), c


@pytest.mark.parametrize("host", ["pageable", "pinned", "pinned_copies"])
def test_step_io_matches_separate_calls(ylib, cuda, monkeypatch, host):
    # yk_langevin_step_io (upload, step, download, one synchronisation) gives
    # the fields and observables of set_field + step + get_field + observables;
    # with pinned fields after the first step it is one graph per pointer pair
    # (two pairs alternating here, then no upload and no download), its
    # transfers kernels on the mapped buffers or (YK_IO_KERNEL=0) copies
    monkeypatch.setenv("YK_IO_KERNEL", "0" if host == "pinned_copies" else "1")
    yk, torch = ylib, cuda
    p = params(yk, 32, 32, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
    V = 32 * 32
    phi0 = np.random.default_rng(5).uniform(-1, 1, V)
    want, obs_w = [], []
    with yk.Context(p) as ctx:
        ctx.set_field(phi0)
        for _ in range(7):
            ctx.step(1)
            want.append(ctx.get_field())
            obs_w.append(ctx.observables())

    def buf(a):
        if host == "pageable":
            return a.copy()
        t = torch.empty(V, dtype=torch.float64).pin_memory()
        t.copy_(torch.from_numpy(a))
        return t

    def arr(b):
        return b if host == "pageable" else b.numpy()

    with yk.Context(p) as ctx:
        cur, out = buf(phi0), buf(np.zeros(V))
        for s in range(6):
            o = ctx.step_io(cur, out)
            assert np.array_equal(arr(out), want[s]), s
            assert o.status == 0 and o.steps == s + 1 and o.sum_phi == obs_w[s].sum_phi
            assert o.cg_iterations == obs_w[s].cg_iterations
            cur, out = out, cur
        # no upload: the step continues from the device field; no download
        o = ctx.step_io(None, None)
        assert o.steps == 7 and o.sum_phi == obs_w[6].sum_phi
        assert np.array_equal(ctx.get_field(), want[6])
    with pytest.raises(TypeError):
        with yk.Context(p) as ctx:
            ctx.step_io(np.zeros(V, dtype=np.float32))


def test_step_io_graph_cache_eviction(ylib, cuda):
    # six different pinned output buffers, one per step: more pointer pairs
    # than the four io graphs kept, so older graphs are replaced; each buffer
    # holds its step's field, as get_field after the same steps
    yk, torch = ylib, cuda
    p = params(yk, 32, 32, precision=yk.YK_MIXED, cg_tol=1e-10, fixed_dt=0.01)
    V = 32 * 32
    phi0 = np.random.default_rng(6).uniform(-1, 1, V)
    want = []
    with yk.Context(p) as ctx:
        ctx.set_field(phi0)
        for _ in range(8):
            ctx.step(1)
            want.append(ctx.get_field())
    outs = [torch.empty(V, dtype=torch.float64).pin_memory() for _ in range(6)]
    with yk.Context(p) as ctx:
        ctx.set_field(phi0)
        for s in range(8):
            buf = outs[s % 6]
            o = ctx.step_io(None, buf)
            assert o.steps == s + 1 and o.status == 0
            assert np.array_equal(buf.numpy(), want[s]), s


def test_deterministic(ylib, cuda):
    yk = ylib
    p = params(yk, 32, 32)
    out = []
    for _ in range(2):
        with yk.Context(p) as ctx:
            ctx.step(3)
            out.append(ctx.get_field())
    assert np.array_equal(out[0], out[1])


def test_observables(ylib, cuda):
    yk = ylib
    Nt, Nx = 16, 8
    p = params(yk, Nt, Nx)
    with yk.Context(p) as ctx:
        ctx.step(2)
        phi = ctx.get_field()
        assert np.abs(ctx.time_slices() - O.time_slices(Nt, Nx, phi)).max() < 1e-12
        corr, st = ctx.correlator()
        a = act(p)
        src = np.zeros((Nt * Nx, 4), complex)
        src[0, 0] = src[0, 1] = 1.0
        x, _, _ = O.cg(Nt, Nx, a, phi, src, mtype=0, tol=1e-12, tol_mode=1)
        y = O.dirac(Nt, Nx, a, phi, x, True)
        assert np.abs(corr - O.time_slices_spinor(Nt, Nx, y)).max() < 1e-9
        cond, _ = ctx.condensate()
        eta = O.fermion_eta(1234, 0, 2, Nt, Nx, kind=3)
        F, _ = O.force(Nt, Nx, a, phi, eta, tol=1e-12, tol_mode=1)
        assert abs(cond - F.sum() / p.yukawa_coupling / (Nt * Nx)) < 1e-9


def test_checkpoint_roundtrip(ylib, cuda, tmp_path):
    yk = ylib
    p = params(yk, 16, 16)
    with yk.Context(p) as ctx:
        ctx.step(2)
        ctx.checkpoint_save(tmp_path / "c.ckpt", 0.03)
        ctx.step(2)
        f4 = ctx.get_field()
    with yk.Context(p) as ctx2:
        assert ctx2.checkpoint_load(tmp_path / "c.ckpt") == 0.03
        assert ctx2.get_step() == 2
        ctx2.step(2)
        assert np.array_equal(ctx2.get_field(), f4)


def test_bounded_wait_runs_out(ylib, cuda):
    # a device wait on a flag that nothing sets gives up after its bound,
    # records YK_ETIMEOUT for the host and leaves the device usable
    import ctypes as C
    import time
    yk = ylib
    st = C.c_int(-1)
    t0 = time.perf_counter()
    rc = yk.lib().yk_check_wait_timeout(None, C.byref(st))
    dt = time.perf_counter() - t0
    assert rc == yk.YK_ETIMEOUT and st.value == yk.YK_ETIMEOUT
    assert 0.5 < dt < 30.0, dt
    p = params(yk, 16, 16)
    with yk.Context(p) as ctx:
        ctx.step(1)
        assert ctx.observables().status == 0
