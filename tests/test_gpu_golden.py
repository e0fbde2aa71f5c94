"""The CUDA path against the reference's own outputs (golden fixtures made by
oracle/ref/make_golden.py from the reference kernels).  Tolerances as in
test_golden.py."""
import numpy as np
import pytest

from pathlib import Path

FILES = sorted((Path(__file__).resolve().parent / "golden").glob("ref_*.npz"))
pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not FILES, reason="no golden fixtures")]


def cplx(a):
    return a.view(np.complex128).reshape(-1, 4)


@pytest.fixture(params=FILES, ids=lambda f: f.stem)
def gold(request):
    d = dict(np.load(request.param))
    Nt, Nx = (int(v) for v in d["shape"])
    return d, Nt, Nx, d["params"]


def make_ctx(yk, Nt, Nx, prm, **kw):
    m2, lam, g, m0, eps_bar = prm
    p = yk.Params.default(use_mass=1, mass=m2, g=lam, yukawa_coupling=g, fermion_mass=m0, Nt=Nt, Nx=Nx,
                          average_epsilon=eps_bar, init=yk.YK_INIT_NONE, **kw)
    return yk.Context(p)


def test_gpu_dirac_and_cg(ylib, cuda, gold):
    d, Nt, Nx, prm = gold
    for r, sfx in ((1.0, ""), (0.5, "_r05")):
        with make_ctx(ylib, Nt, Nx, prm, wilson_param=r) as ctx:
            ctx.set_field(d["sigma"])
            x = cuda.from_numpy(cplx(d["psi"]).copy()).cuda()
            y = cuda.empty_like(x)
            for dag, key in ((False, "dirac_D"), (True, "dirac_Ddag")):
                ctx.dirac_apply(x, y, dag)
                ctx.synchronize()
                want = cplx(d[key + sfx])
                assert np.abs(y.cpu().numpy() - want).max() / np.abs(want).max() < 1e-14
            if r == 1.0:
                b = cuda.from_numpy(cplx(d["cg_b"]).copy()).cuda()
                for mtype, key in ((1, "cg_x_dag"), (0, "cg_x_nor")):
                    xs = cuda.zeros_like(b)
                    ctx.cg_solve(b, xs, mtype=mtype)   # reference rule: |r| <= 1e-8, IterMax 1000
                    want = cplx(d[key])
                    assert np.abs(xs.cpu().numpy() - want).max() / np.abs(want).max() < 1e-9


def test_gpu_force_noise_run(ylib, cuda, gold):
    d, Nt, Nx, prm = gold
    V = Nt * Nx
    with make_ctx(ylib, Nt, Nx, prm) as ctx:
        ctx.set_field(d["sigma"])
        F = cuda.empty(V, dtype=cuda.float64, device="cuda")
        ctx.fermion_force(F, cuda.from_numpy(cplx(d["force_eta"]).copy()).cuda())
        assert np.abs(F.cpu().numpy() - d["force_F"]).max() < 3e-9
    for i, s in enumerate(d["noise_cuts"]):
        with make_ctx(ylib, Nt, Nx, prm, cut_fraction=float(s)) as ctx:
            xi = cuda.empty(V, dtype=cuda.float64, device="cuda")
            ctx.coloured_noise(xi, cuda.from_numpy(d["noise_w"].copy()).cuda())
            ctx.synchronize()
            assert np.abs(xi.cpu().numpy() - d[f"noise_xi{i}"]).max() < 1e-13
    with make_ctx(ylib, Nt, Nx, prm) as ctx:
        ctx.set_field(d["run_phi0"])
        obs = ctx.euler_update(cuda.from_numpy(d["run_force"].copy()).cuda(),
                               cuda.from_numpy(d["run_noise"].copy()).cuda())
        assert abs(obs.eps - d["run_eps"][0]) <= 1e-15 * obs.eps
        assert abs(obs.max_drift - d["run_eps"][1]) <= 1e-15 * obs.max_drift
        assert np.abs(ctx.get_field() - d["run_phi1"]).max() < 1e-14
        assert abs(obs.sum_phi - d["obs_mag"][0]) < 1e-12
        assert np.abs(ctx.time_slices() - d["obs_slices"]).max() < 1e-12


def test_gpu_langevin_steps(ylib, cuda, gold):
    d, Nt, Nx, prm = gold
    V = Nt * Nx
    with make_ctx(ylib, Nt, Nx, prm, cut_fraction=float(d["step_cut"][0])) as ctx:
        ctx.set_field(d["step_phi0"])
        xi = cuda.empty(V, dtype=cuda.float64, device="cuda")
        F = cuda.empty(V, dtype=cuda.float64, device="cuda")
        for s in range(3):
            ctx.coloured_noise(xi, cuda.from_numpy(d[f"step_w{s}"].copy()).cuda())
            ctx.fermion_force(F, cuda.from_numpy(cplx(d[f"step_eta{s}"]).copy()).cuda())
            obs = ctx.euler_update(F, xi)
            assert abs(obs.eps - d[f"step_eps{s}"][0]) < 1e-9 * obs.eps
            assert np.abs(ctx.get_field() - d[f"step_phi{s + 1}"]).max() < 1e-10, s
            ctx.set_field(d[f"step_phi{s + 1}"])
