"""The learned preconditioner: its oracle (CPU), the CUDA network against the
oracle, training, and what the trained network gains in a flexible Krylov
solve (GPU).

Tolerances: the oracle's gradients against central finite differences 1e-6
relative; the FP32 network against the FP64 oracle 2e-6 (forward) and 2e-5
(weight gradients) relative to the largest entry, its BF16 tensor-core form
(the one the solvers apply) 2e-2; every solve to the FP64 relative residual
1e-10.
"""
import numpy as np
import pytest

from oracle import learned as N
from oracle import oracle as O


def _action(m0=0.1):
    return O.action(m2=-0.5, lam=1.0, g=0.5, m0=m0, r=1.0, cut_fraction=0.35355339059327373, eps_bar=0.01,
                    drift_mode=0)


def _fd_worst(fn, Ws, args):
    L, g = fn(Ws, *args)
    worst = 0.0
    for l in range(len(Ws)):
        for idx in [(0, 0, 0), (4, 3, 2), (8, 7, Ws[l].shape[2] - 1), (2, 5, 1)]:
            W2 = [w.copy() for w in Ws]
            h = 1e-6
            W2[l][idx] += h
            Lp, _ = fn(W2, *args)
            W2[l][idx] -= 2 * h
            Lm, _ = fn(W2, *args)
            fd = (Lp - Lm) / (2 * h)
            worst = max(worst, abs(fd - g[l][idx]) / max(1e-9, abs(fd)))
    return worst


def test_oracle_preconditioner_is_symmetric_positive():
    Nt, Nx = 6, 5
    rng = np.random.default_rng(0)
    Ws = N.init_weights(8, 3, 3)
    sig = rng.uniform(-1, 1, Nt * Nx)
    a, b = rng.normal(size=(2, 4, Nt * Nx))
    Ma = N.apply_M(Ws, a, sig, Nt, Nx, 0.03)[0]
    Mb = N.apply_M(Ws, b, sig, Nt, Nx, 0.03)[0]
    assert abs(np.sum(b * Ma) - np.sum(a * Mb)) < 1e-12 * abs(np.sum(b * Ma))
    assert np.sum(a * Ma) > 0.03 * np.sum(a * a)


@pytest.mark.parametrize("kind", ["plain", "energy"])
def test_oracle_gradients_match_finite_differences(kind):
    Nt, Nx = 6, 5
    rng = np.random.default_rng(1)
    Ws = N.init_weights(8, 3, 3)
    r, e = rng.normal(size=(2, 4, Nt * Nx))
    sig = rng.uniform(-1, 1, Nt * Nx)
    if kind == "plain":
        worst = _fd_worst(N.plain_loss_and_grad, Ws, (r, e, sig, Nt, Nx, 0.03))
    else:
        worst = _fd_worst(N.energy_loss_and_grad, Ws, (r, e, sig, Nt, Nx, _action(), 0.03))
    assert worst < 1e-6, worst


def test_oracle_flexible_pcg_recurrence():
    # the solver's recurrence with the (untrained) network as M on an 8 x 6
    # lattice near the chiral regime: the Polak-Ribiere beta -<z', q>/<p, q>
    # takes the same steps as the classical <r', z'>/<r, z> for a fixed SPD M
    # and converges to 1e-10; with zero weights (M = skip I) it is plain CG
    Nt, Nx = 8, 6
    rng = np.random.default_rng(3)
    a = _action(0.02)
    sig = rng.uniform(-1, 1, Nt * Nx)
    Ws = N.init_weights(8, 2, 5)
    skip = 1.0 / (4 + 0.02 + 2) ** 2
    A = lambda v: N.dirac_real(Nt, Nx, a, sig, N.dirac_real(Nt, Nx, a, sig, v, False), True)
    M = lambda v: N.apply_M(Ws, v, sig, Nt, Nx, skip)[0]
    b = rng.normal(size=(4, Nt * Nx))
    x_pr, it_pr, h_pr = N.flexible_pcg(A, M, b, 1e-10, 2000)
    x_cl, it_cl, h_cl = N.flexible_pcg(A, M, b, 1e-10, 2000, polak_ribiere=False)
    assert np.linalg.norm(A(x_pr) - b) < 1e-9 * np.linalg.norm(b)
    n = min(len(h_pr), len(h_cl), 20)
    assert np.allclose(h_pr[:n], h_cl[:n], rtol=1e-6, atol=0)
    assert abs(it_pr - it_cl) <= 2
    _, it_id, h_id = N.flexible_pcg(A, lambda v: v, b, 1e-10, 2000)
    Z = [np.zeros_like(w) for w in Ws]
    _, it_z, h_z = N.flexible_pcg(A, lambda v: N.apply_M(Z, v, sig, Nt, Nx, skip)[0], b, 1e-10, 2000)
    assert abs(it_z - it_id) <= 1 and np.allclose(h_z[:20], h_id[:20], rtol=1e-8, atol=0)


def _params(yk, Nt, Nx, m0, precision):
    return yk.Params.default(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=m0, wilson_param=1.0,
                             cut_fraction=0.35355339059327373, Nt=Nt, Nx=Nx, cg_tol=1e-10,
                             cg_tol_mode=yk.YK_TOL_REL, seed=1234, init=yk.YK_INIT_PHILOX, precision=precision,
                             fixed_dt=0.01)


@pytest.mark.gpu
@pytest.mark.parametrize("tile", ["8x64x1", "4x16x4", "2x8x8"], ids=["per_layer", "halves_fused", "all_fused"])
def test_network_forward_and_gradient_match_oracle(ylib, cuda, monkeypatch, tile):
    # the solvers' form at three launch shapes: one launch per layer, N and
    # N^T fused, all eight layers fused (a halo of 8 rows around 2-row tiles
    # of the 16 x 12 lattice, so staged rows wrap in time, with 8 + 4 column
    # tiles)
    monkeypatch.setenv("YK_NET_TILE", tile)
    yk, torch = ylib, cuda
    Nt, Nx = 16, 12
    V = Nt * Nx
    rng = np.random.default_rng(0)
    with yk.Context(_params(yk, Nt, Nx, 0.1, yk.YK_FP64)) as ctx:
        sig = rng.uniform(-1, 1, V)
        ctx.set_field(sig)
        ctx.net_setup(4, 1, skip=0.05)
        Ws = N.init_weights(8, 4, 3)
        ctx.net_set_weights(np.concatenate([w.ravel() for w in Ws]))
        assert np.array_equal(ctx.net_get_weights(), np.concatenate([w.ravel() for w in Ws]).astype(np.float32))
        W32 = [w.astype(np.float32).astype(np.float64) for w in Ws]
        r = rng.normal(size=(V, 4)).astype(np.float32)
        e = rng.normal(size=(V, 4)).astype(np.float32)
        rd, ed = torch.from_numpy(r).cuda(), torch.from_numpy(e).cuda()
        zd = torch.empty_like(rd)
        ctx.net_apply(rd, zd)
        want = N.apply_M(W32, r.T.astype(np.float64), sig, Nt, Nx, np.float32(0.05))[0]
        assert np.abs(zd.cpu().numpy().T - want).max() < 2e-6 * np.abs(want).max()
        # the solvers' form: BF16 activations (8-bit significands) through
        # tensor-core convolutions with FP32 accumulation
        ctx.net_apply(rd, zd, tensor_cores=True)
        err = np.abs(zd.cpu().numpy().T - want).max() / np.abs(want).max()
        assert err < 2e-2, err
        g, loss = ctx.net_grad(rd, ed)
        lo, go = N.energy_loss_and_grad(W32, r.T.astype(np.float64), e.T.astype(np.float64), sig, Nt, Nx,
                                        _action(0.1), np.float32(0.05))
        go = np.concatenate([x.ravel() for x in go])
        assert abs(loss - lo) < 1e-5 * lo
        assert np.abs(g - go).max() < 2e-5 * np.abs(go).max()


@pytest.mark.gpu
def test_trained_network_cuts_iterations(ylib, cuda):
    # near the critical mass (m0 = 0.02): the trained network against the
    # method without it (the same flexible solver with z = r) and against the
    # context's mixed CG; every solve must meet the FP64 tolerance
    yk, torch = ylib, cuda
    Nt, Nx = 32, 32
    V = Nt * Nx
    p = _params(yk, Nt, Nx, 0.02, yk.YK_MIXED)
    with yk.Context(p) as ctx:
        ctx.step(20)
        ctx.net_setup(4, 7)
        st = ctx.net_train(n_sources=4, n_levels=5, base_iter=4, steps=400, batch=4, lr=2e-3, seed=3)
        assert st.pairs == 20
        assert st.loss1 < 0.8 * st.loss0
        rng = np.random.default_rng(5)
        b = rng.normal(size=(V, 4))
        bd = torch.from_numpy(b).cuda()
        its = {}
        sig = ctx.get_field()
        a = O.action(m2=p.mass, lam=p.g, g=p.yukawa_coupling, m0=p.fermion_mass, r=p.wilson_param,
                     cut_fraction=p.cut_fraction, eps_bar=p.average_epsilon, drift_mode=p.drift_mode)
        for solver in ("fgcr", "pcg"):
            for use in (False, True):
                x = torch.zeros_like(bd)
                s = getattr(ctx, solver + "_solve")(bd, x, tol=1e-10, max_iter=20000, use_net=use)
                assert s.converged == 1 and s.rr <= 1e-20 * s.rr0
                xs = x.cpu().numpy().astype(np.complex128)
                Ax = O.dirac(Nt, Nx, a, sig, O.dirac(Nt, Nx, a, sig, xs, False), True)
                assert np.linalg.norm(Ax - b) < 1e-9 * np.linalg.norm(b)
                its[solver, use] = s.iterations
        xc = torch.zeros(V, 4, dtype=torch.complex128, device="cuda")
        cg = ctx.cg_solve(torch.complex(bd, torch.zeros_like(bd)).contiguous(), xc, tol=1e-10,
                          tol_mode=yk.YK_TOL_REL, max_iter=20000, precision=yk.YK_MIXED)
        assert its["fgcr", True] * 5 < its["fgcr", False], its
        assert its["fgcr", True] < cg.iterations, (its, cg.iterations)
        assert its["pcg", True] * 2.5 < its["pcg", False], its
        assert its["pcg", True] < cg.iterations, (its, cg.iterations)


@pytest.mark.gpu
@pytest.mark.parametrize("tile", ["8x64x1", "4x16x2", "2x8x4"])
def test_learned_step_odd_lattice(ylib, cuda, monkeypatch, tile):
    # a 41 x 25 lattice (odd in both directions: ragged tiles in rows and
    # columns, a last tile row of one time slice) at three launch shapes of
    # the 2-layer network: two learned steps agree with the FP64 CG step
    monkeypatch.setenv("YK_NET_TILE", tile)
    yk = ylib
    Nt, Nx = 41, 25
    fields = []
    for learned in (False, True):
        with yk.Context(_params(yk, Nt, Nx, 0.05, yk.YK_FP64)) as ctx:
            if learned:
                ctx.net_setup(2, 7)
                ctx.net_train(n_sources=2, n_levels=3, base_iter=4, steps=60, batch=2, lr=2e-3, seed=3)
                st = ctx.step_learned(2)
                assert st.converged == 1
            else:
                ctx.step(2)
            assert ctx.observables().status == 0
            fields.append(ctx.get_field())
    err = np.abs(fields[1] - fields[0]).max() / np.abs(fields[0]).max()
    assert err < 1e-8, err


@pytest.mark.gpu
def test_learned_step_matches_cg_step(ylib, cuda):
    # the same Langevin steps with every fermion solve by the learned PCG
    # (network and identity) and by the step graph's FP64 CG: the fields agree
    # to the solves' tolerance (rel-res 1e-10 gives a force error ~1e-10)
    yk, torch = ylib, cuda
    Nt, Nx = 32, 32
    fields = {}
    for mode in ("cg", "identity", "net"):
        with yk.Context(_params(yk, Nt, Nx, 0.05, yk.YK_FP64)) as ctx:
            if mode == "net":
                ctx.net_setup(4, 7)
                ctx.net_train(n_sources=2, n_levels=4, base_iter=4, steps=100, batch=4, lr=2e-3, seed=3)
            if mode == "cg":
                ctx.step(3)
            else:
                st = ctx.step_learned(3, use_net=(mode == "net"))
                assert st.converged == 1 and st.rr <= 1e-20 * st.rr0 * 3
                t = ctx.tune_report()   # the network's convolution tile, chosen on its first solve
                if mode == "net":
                    assert t.conv_rows in (2, 4, 8) and 1 <= t.conv_cols <= 64
            o = ctx.observables()
            assert o.steps == 3 and o.status == 0 and o.cg_iterations > 0
            fields[mode] = ctx.get_field()
    ref = fields["cg"]
    for mode in ("identity", "net"):
        err = np.abs(fields[mode] - ref).max() / np.abs(ref).max()
        assert err < 1e-8, (mode, err)


@pytest.mark.gpu
@pytest.mark.parametrize("lat", [(32, 32), (41, 25)], ids=["32x32", "41x25"])
def test_persistent_pcg_matches_launched_phases(ylib, cuda, monkeypatch, lat):
    # the persistent PCG chunk (one cooperative launch, grid barriers between
    # the phases) against one launch per phase: the same bodies on the same
    # grid, so the learned steps' fields agree bit for bit, with the network
    # (per-layer convolutions) and with z = r
    monkeypatch.setenv("YK_NET_TILE", "8x64x1")
    yk = ylib
    Nt, Nx = lat
    fields = {}
    for persistent in ("0", "2"):   # off; at most two blocks per SM
        monkeypatch.setenv("YK_PCG_PERSISTENT", persistent)
        for use in (False, True):
            with yk.Context(_params(yk, Nt, Nx, 0.05, yk.YK_FP64)) as ctx:
                ctx.net_setup(2, 7)
                ctx.net_train(n_sources=2, n_levels=3, base_iter=4, steps=40, batch=2, lr=2e-3, seed=3)
                st = ctx.step_learned(2, use_net=use)
                assert st.converged == 1
                assert ctx.observables().status == 0
                fields[persistent, use] = (ctx.get_field(), st.iterations)
    for use in (False, True):
        assert fields["0", use][1] == fields["2", use][1]
        assert np.array_equal(fields["0", use][0], fields["2", use][0]), use


@pytest.mark.gpu
def test_run_protocol_with_learned_solver(ylib, cuda, tmp_path):
    # the reference's run protocol (yk_run_toml) with [gpu] learned_layers = 2:
    # a network is trained after thermalisation and the measurement steps
    # solve with it; the traces agree with the same run by the CG step graph
    # to the solves' tolerance
    yk = ylib
    toml = """
[physics]
useMass = "true"
mass = -0.5
g = 1.0
cutFraction = 0.35355339059327373

[langevin]
averageEpsilon = 0.01
MaxLangevinTime = 0.5
ExportTime = 0.05
burnCount = 2
MeasureDriftCount = 0

[io]
configFileName = "cfg.bin"
export = "false"
timeSliceFileName = "slice.dat"

[random]
seed = 11

[fermions]
yukawa_coupling = 0.5
fermion_mass = 0.05
driftMode = 0
WilsonParam = 1.0

[lattice]
Nt = 32
Nx = 32

[gpu]
precision = "mixed"
cg_tol_mode = "rel"
cg_tol = 1e-10
fixed_dt = 0.01
init = "philox"
"""
    traces = {}
    for name, extra in (("cg", ""), ("learned", "learned_layers = 2\n")):
        d = tmp_path / name
        d.mkdir()
        (d / "input.toml").write_text(toml + extra)
        yk.run(d / "input.toml", d)
        rows = (d / "traces.csv").read_text().strip().splitlines()
        assert rows[0] == "tr,sigma,phi" and len(rows) > 5
        traces[name] = np.array([[float(v) for v in r.split(",")] for r in rows[1:]])
    a, b = traces["cg"], traces["learned"]
    assert a.shape == b.shape
    assert np.abs(a - b).max() < 1e-7 * max(1.0, np.abs(a).max())
