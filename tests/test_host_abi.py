"""Host-side logic of the C ABI and its exports (no GPU calls)."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    text = (ROOT / "include" / "yukawa.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(yk_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(ylib):
    declared = header_functions()
    assert len(declared) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", str(ylib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (yk_\w+)", out))
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    for f in declared:
        assert hasattr(ylib.lib(), f)
    assert set(ylib.exported_symbols()) <= set(declared)


def test_defaults_follow_reference(ylib):
    p = ylib.Params.default()
    # code/input.toml and code/src/params.h
    assert (p.use_mass, p.mass, p.g, p.kappa, p.lam, p.cut_fraction) == (0, 0.2, 0.0, 0.18, 0.02, 1.0)
    assert (p.average_epsilon, p.max_langevin_time, p.export_time, p.burn_count, p.measure_drift_count) == \
        (0.02, 100.0, 0.5, 10, 10)
    assert (p.seed, p.yukawa_coupling, p.fermion_mass, p.drift_mode, p.wilson_param) == (1234, 1.0, 1.0, 0, 1.0)
    assert (p.Nt, p.Nx, p.cg_tol, p.cg_max_iter, p.cg_tol_mode) == (16, 16, 1e-8, 1000, ylib.YK_TOL_ABS)


def test_toml_parsing(ylib, tmp_path):
    f = tmp_path / "input.toml"
    f.write_text("""
[physics]
useMass = "true"
mass = -0.5
g = 1.0   # lambda when useMass
kappa = 0.2
lambda = 0.03
cutFraction = 0.35355339059327373

[langevin]
averageEpsilon = 0.01
MaxLangevinTime = 5.0
ExportTime = 0.25
burnCount = 3
MeasureDriftCount = 0

[io]
configFileName = "cfg.bin"
export = "false"
timeSliceFileName = "slice.dat"

[random]
seed = 77

[fermions]
yukawa_coupling = 0.5
fermion_mass = 0.1
driftMode = 1 # rescaled
WilsonParam = 1.0

[lattice]
Nt = 32
Nx = 64

[gpu]
precision = "mixed"
n_rhs = 4
cg_tol_mode = "rel"
cg_tol = 1e-10
reliable_every = 25
fixed_dt = 0.01
init = "philox"
learned_layers = 2
""")
    p = ylib.Params.from_toml(f)
    assert p.use_mass == 1 and p.mass == -0.5 and p.g == 1.0 and p.cut_fraction == 0.35355339059327373
    assert p.average_epsilon == 0.01 and p.export_time == 0.25 and p.burn_count == 3 and p.measure_drift_count == 0
    assert p.seed == 77 and p.yukawa_coupling == 0.5 and p.fermion_mass == 0.1 and p.drift_mode == 1
    assert (p.Nt, p.Nx, p.precision, p.n_rhs, p.cg_tol_mode, p.cg_tol) == (32, 64, ylib.YK_MIXED, 4, 1, 1e-10)
    assert p.reliable_every == 25 and p.fixed_dt == 0.01 and p.init == ylib.YK_INIT_PHILOX
    assert p.learned_layers == 2 and ylib.Params.default().learned_layers == 0
    with pytest.raises(ylib.YukawaError):
        ylib.Params.from_toml(tmp_path / "missing.toml")


@pytest.mark.parametrize("use_mass", [0, 1])
def test_derived_action_matches_oracle(ylib, use_mass):
    p = ylib.Params.default(use_mass=use_mass, mass=-0.5, g=1.0, kappa=0.21, lam=0.03, yukawa_coupling=0.7,
                            fermion_mass=0.15, wilson_param=0.8, cut_fraction=0.4, drift_mode=1)
    a = p.action()
    o = O.derive(use_mass, -0.5, 1.0, 0.21, 0.03, 0.7, 0.15, 0.8, 0.4, 0.02, 1)
    for f in ("m2", "lam", "kappa", "sq2kappa", "g", "m0", "r", "cut_fraction", "eps_bar"):
        assert getattr(a, f) == getattr(o, f), f
    if use_mass:
        # FindKappa (main.cu:58-63) inverts m^2 = (1 - 2 lambda_L)/kappa - 4 with lambda = 6 lambda_L/kappa^2
        lam_l = a.lam * a.kappa**2 / 6.0
        assert abs((1 - 2 * lam_l) / a.kappa - 4.0 - a.m2) < 1e-12


def test_gamma_method_matches_oracle(ylib):
    rng = np.random.default_rng(2)
    x = np.cumsum(rng.normal(size=3000)) * 0.01 + rng.normal(size=3000)
    assert np.allclose(ylib.gamma_method(x), O.gamma_method(x), rtol=1e-12, atol=1e-14)


def test_golden_dump_reader(tmp_path):
    from oracle.ref.make_golden import read_dump
    blob = b""
    for name, arr in [("a", np.arange(3.0)), ("bb", np.array([1.5]))]:
        blob += name.encode().ljust(32, b"\0") + np.int64(arr.size).tobytes() + arr.tobytes()
    (tmp_path / "d.bin").write_bytes(blob)
    d = read_dump(tmp_path / "d.bin")
    assert list(d) == ["a", "bb"] and np.array_equal(d["a"], np.arange(3.0)) and d["bb"][0] == 1.5
