"""Golden vectors produced by running the reference's own kernels
(oracle/ref/build_ref.py + oracle/ref/ref_harness.cpp, see
oracle/ref/make_golden.py).  The CPU oracle is pinned against them here (no
GPU); test_gpu_golden.py checks the CUDA path against the same vectors.

Tolerances: operator applications 1e-14 relative (the reference sums in a
different order and uses FMA contraction); CG solutions at the reference's
absolute 1e-8 stopping rule 1e-9 relative; fermion forces from those solves
3e-9 absolute (two FP64 CGs that take the same number of iterations still
differ by rounding amplified through the iteration: the oracle and the
reference differ by up to 6.5e-10 in F on the 8x4 lattice); noise 1e-13
absolute (cuFFT vs radix-2); steps 1e-10 absolute on the field, 1e-9 relative
on eps (it follows max|drift|, whose force carries the CG tolerance).
"""
import numpy as np
import pytest

from oracle import oracle as O

from pathlib import Path

FILES = sorted((Path(__file__).resolve().parent / "golden").glob("ref_*.npz"))
pytestmark = pytest.mark.skipif(not FILES, reason="no golden fixtures")


def load(f):
    d = dict(np.load(f))
    Nt, Nx = (int(v) for v in d["shape"])
    m2, lam, g, m0, eps_bar = d["params"]
    return d, Nt, Nx, (m2, lam, g, m0, eps_bar)


def cplx(a):
    return a.view(np.complex128).reshape(-1, 4)


def relerr(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(params=FILES, ids=lambda f: f.stem)
def gold(request):
    return load(request.param)


def test_dirac(gold):
    d, Nt, Nx, (m2, lam, g, m0, eps_bar) = gold
    for r, sfx in ((1.0, ""), (0.5, "_r05")):
        a = O.action(m2=m2, lam=lam, g=g, m0=m0, r=r)
        for dag, key in ((False, "dirac_D"), (True, "dirac_Ddag")):
            got = O.dirac(Nt, Nx, a, d["sigma"], cplx(d["psi"]), dag)
            assert relerr(got, cplx(d[key + sfx])) < 1e-14, key + sfx


def test_cg(gold):
    d, Nt, Nx, (m2, lam, g, m0, eps_bar) = gold
    a = O.action(m2=m2, lam=lam, g=g, m0=m0)
    for mtype, key in ((1, "cg_x_dag"), (0, "cg_x_nor")):
        x, it, rr = O.cg(Nt, Nx, a, d["sigma"], cplx(d["cg_b"]), mtype=mtype)
        assert relerr(x, cplx(d[key])) < 1e-9, key
        assert np.sqrt(rr) <= 1e-8 and np.sqrt(d[key.replace("x", "rr")][0]) <= 1e-8


def test_force(gold):
    d, Nt, Nx, (m2, lam, g, m0, eps_bar) = gold
    eta = cplx(d["force_eta"])[None]
    F, _ = O.force(Nt, Nx, O.action(m2=m2, lam=lam, g=g, m0=m0), d["sigma"], eta)
    assert np.abs(F - d["force_F"]).max() < 3e-9
    Fr, _ = O.force(Nt, Nx, O.action(m2=m2, lam=lam, g=g, m0=m0, cut_fraction=0.5, drift_mode=1), d["sigma"], eta)
    assert np.abs(Fr - d["force_F_resc"]).max() < 3e-9


def test_mask_and_noise(gold):
    d, Nt, Nx, _ = gold
    for i, s in enumerate(d["noise_cuts"]):
        mh = O.mask_half(Nt, Nx, s).ravel()
        assert np.array_equal(mh, d[f"noise_mask{i}"])
        assert np.abs(O.coloured_noise(Nt, Nx, s, d["noise_w"]) - d[f"noise_xi{i}"]).max() < 1e-13


def test_run_kernel(gold):
    d, Nt, Nx, (m2, lam, g, m0, eps_bar) = gold
    drift = O.bosonic_drift(Nt, Nx, m2, lam, d["run_phi0"], d["run_force"])
    assert np.abs(drift - d["run_drift"]).max() < 1e-13
    phi, eps, m = O.euler_update(d["run_phi0"], drift, d["run_noise"], eps_bar)
    assert abs(eps - d["run_eps"][0]) <= 1e-15 * eps and abs(m - d["run_eps"][1]) <= 1e-15 * m
    assert np.abs(phi - d["run_phi1"]).max() < 1e-14


def test_observables(gold):
    d, Nt, Nx, _ = gold
    assert abs(d["obs_mag"][0] - d["run_phi1"].sum()) < 1e-12
    assert np.abs(d["obs_slices"] - O.time_slices(Nt, Nx, d["run_phi1"])).max() < 1e-12
    assert np.abs(d["obs_corr"] - O.time_slices_spinor(Nt, Nx, cplx(d["psi"]))).max() < 1e-12
    assert abs(d["obs_trace"][0] - d["run_drift"].sum()) < 1e-12


def test_langevin_steps(gold):
    d, Nt, Nx, (m2, lam, g, m0, eps_bar) = gold
    a = O.action(m2=m2, lam=lam, g=g, m0=m0, cut_fraction=d["step_cut"][0], eps_bar=eps_bar)
    phi = d["step_phi0"]
    for s in range(3):
        xi = O.coloured_noise(Nt, Nx, d["step_cut"][0], d[f"step_w{s}"])
        F, _ = O.force(Nt, Nx, a, phi, cplx(d[f"step_eta{s}"])[None])
        drift = O.bosonic_drift(Nt, Nx, m2, lam, phi, F)
        phi, eps, m = O.euler_update(phi, drift, xi, eps_bar)
        assert abs(eps - d[f"step_eps{s}"][0]) < 1e-9 * eps
        assert np.abs(phi - d[f"step_phi{s + 1}"]).max() < 1e-10, s
        phi = d[f"step_phi{s + 1}"]
