"""Parity of the CUDA path with the CPU oracle at the benchmark
configurations themselves, not only on small lattices.

* C2, the headline step: 256 x 256, mixed FP32/FP64 CG (the even-odd kernel
  of single-system solves) with a reliable update every 50 iterations, CG
  rel-res 1e-10, fixed dt 0.01, from the thermalised start field of the bench
  (tests/golden/start_256x256.npz, Philox step 2000): 4 steps, field within
  1e-8 of the oracle's FP64 steps (code/src/langevin_gpu_v2.cu:65-118,
  FermionicDrift.cu:57-100).
* C1: 32 x 32 in FP64, fixed dt 0.01 and the reference's adaptive step, 12
  steps each, field within 1e-9 (CG rel-res 1e-12).
* C3-shaped batch: 8 chains with L in {32, 64, 128, 256} (two of each),
  seeded m0 ~ U[0.05, 0.3] and g ~ U[0.3, 0.8], 4 right-hand sides, mixed CG
  rel-res 1e-10 (the batched even-odd kernel), all chains in one step graph:
  2 steps, every chain within 1e-8 of its own oracle chain.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

S_HALF_PI = 0.35355339059327373
START = Path(__file__).resolve().parent / "golden" / "start_256x256.npz"


def act(p):
    return O.action(m2=p.mass, lam=p.g, g=p.yukawa_coupling, m0=p.fermion_mass, r=p.wilson_param,
                    cut_fraction=p.cut_fraction, eps_bar=p.average_epsilon, drift_mode=p.drift_mode)


def base(yk, **kw):
    d = dict(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=0.1, wilson_param=1.0,
             cut_fraction=S_HALF_PI, seed=1234, init=yk.YK_INIT_PHILOX)
    d.update(kw)
    return yk.Params.default(**d)


def test_c2_headline_steps_from_the_bench_start(ylib, cuda):
    yk = ylib
    d = np.load(START)
    phi, step0 = d["phi"].copy(), int(d["step"])
    p = base(yk, Nt=256, Nx=256, fixed_dt=0.01, precision=yk.YK_MIXED, cg_tol=1e-10, cg_tol_mode=yk.YK_TOL_REL,
             cg_max_iter=20000, reliable_every=50, reliable_delta=0.001)
    with yk.Context(p) as ctx:
        ctx.set_field(phi)
        ctx.set_step(step0)
        ctx.profile_begin()   # the steps as direct launches: the kernel that ran is reported
        ctx.step(1)
        pr = ctx.profile_end()
        assert pr.cg_kernel == 3, "the headline step's solve runs the even-odd CG kernel"
        got = [ctx.get_field()]
        for _ in range(3):
            ctx.step(1)
            got.append(ctx.get_field())
        obs = ctx.observables()
    assert obs.status == 0 and obs.steps == 4
    a = act(p)
    for s in range(4):
        phi, ro = O.langevin_step(256, 256, a, phi, 1234, 0, step0 + s, tol=1e-10, tol_mode=1, max_iter=20000,
                                  fixed_dt=0.01)
        err = np.abs(got[s] - phi).max()
        assert err < 1e-8, (s, err)
        phi = got[s]


@pytest.mark.parametrize("fixed_dt", [0.01, 0.0])
def test_c1_fp64_steps(ylib, cuda, fixed_dt):
    yk = ylib
    p = base(yk, Nt=32, Nx=32, fixed_dt=fixed_dt, cg_tol=1e-12, cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=5000)
    a = act(p)
    with yk.Context(p) as ctx:
        phi = ctx.get_field()
        for s in range(12):
            ctx.step(1)
            obs = ctx.observables()
            phi, ro = O.langevin_step(32, 32, a, phi, 1234, 0, s, tol=1e-12, tol_mode=1, max_iter=5000,
                                      fixed_dt=fixed_dt)
            got = ctx.get_field()
            assert np.abs(got - phi).max() < 1e-9, s
            assert abs(obs.eps - ro.eps) <= 1e-12 * ro.eps
            phi = got


def test_c3_shaped_batch(ylib, cuda):
    yk = ylib
    rng = np.random.default_rng(1234)
    Ls = [32, 64, 128, 256] * 2
    m0s = rng.uniform(0.05, 0.3, size=len(Ls))
    gs = rng.uniform(0.3, 0.8, size=len(Ls))
    ps = [base(yk, Nt=L, Nx=L, yukawa_coupling=float(g), fermion_mass=float(m0), fixed_dt=0.01, n_rhs=4,
               precision=yk.YK_MIXED, cg_tol=1e-10, cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=20000,
               reliable_every=50)
          for L, m0, g in zip(Ls, m0s, gs)]
    with yk.Context(ps) as ctx:
        ctx.profile_begin()
        ctx.step(1)
        assert ctx.profile_end().cg_kernel == 5, "the batch's solves run the batched even-odd patch kernel"
        ctx.step(1)
        got = [ctx.get_field(c) for c in range(len(ps))]
        obs = [ctx.observables(c) for c in range(len(ps))]
    for c, p in enumerate(ps):
        assert obs[c].status == 0 and obs[c].steps == 2, c
        phi = O.uniform_field(1234, c, p.Nt * p.Nx)
        for s in range(2):
            phi, _ = O.langevin_step(p.Nt, p.Nx, act(p), phi, 1234, c, s, n_rhs=4, tol=1e-10, tol_mode=1,
                                     max_iter=20000, fixed_dt=0.01)
        err = np.abs(got[c] - phi).max()
        assert err < 1e-8, (c, p.Nt, err)


def test_headline_steps_are_reproducible_with_the_auxiliary_stream(ylib, cuda, monkeypatch):
    # the step's coloured noise and the next step's sources run on an
    # auxiliary stream beside the CG; whatever their timing, 30 graph-replayed
    # steps from the bench's start give the same field, bit for bit, as the
    # same steps with everything on one stream, and as a second run
    yk = ylib
    d = np.load(START)
    phi, step0 = d["phi"].copy(), int(d["step"])
    p = base(yk, Nt=256, Nx=256, fixed_dt=0.01, precision=yk.YK_MIXED, cg_tol=1e-10, cg_tol_mode=yk.YK_TOL_REL,
             cg_max_iter=20000, reliable_every=50, reliable_delta=0.001)
    fields = []
    # untuned (the auxiliary stream whenever the CG leaves SMs free), twice;
    # one stream; and the autotuner's choice between the two
    for overlap, tune in (("1", "0"), ("1", "0"), ("0", "0"), ("1", "1")):
        monkeypatch.setenv("YK_NOISE_OVERLAP", overlap)
        monkeypatch.setenv("YK_AUTOTUNE", tune)
        stream = cuda.cuda.Stream()
        with yk.Context(p) as ctx:
            ctx.set_stream(stream.cuda_stream)
            ctx.set_field(phi)
            ctx.set_step(step0)
            ctx.step(30)
            fields.append(ctx.get_field())
            assert ctx.observables().status == 0 and ctx.get_step() == step0 + 30
            t = ctx.tune_report()
            if tune == "1":
                assert t.noise_overlap in (0, 1) and t.step_ms_overlap > 0 and t.step_ms_serial > 0
    for f in fields[1:]:
        assert np.array_equal(fields[0], f)
