"""The run protocol of the CLI (`yk_run input.toml [out_dir]`, the drop-in for
the reference's `./out input.toml`, code/src/main.cu:73-516), checked
against a restatement of that protocol in Python on the same C ABI:

* burn-in blocks (main.cu:295-313), the drift-measurement phase and the
  epsBar rescale epsBar <- epsBar^2 / <eps> where <eps> averages the LAST
  step size of each export block (main.cu:318-352), the export loop
  (main.cu:368-484);
* the content of slice.dat (time slices / Nx, main.cu:394-400), data.csv (the
  point-source correlator, main.cu:441-469), traces.csv (tr, sigma, phi,
  main.cu:471-483) and the stdout lines (main.cu:403-439), all printed with
  6 significant digits (compared to 1e-5 relative);
* SIGUSR2 during the export loop finishes the run early with the reference's
  lines (main.cu:66-75, 425-428);
* io.resume with io.startFileName continues a run exactly from the
  checkpoint the previous run wrote (main.cu:146-157 parses these keys; the
  reference never implemented them).
"""
import os
import signal
import subprocess
import time
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "yukawacolourednoise_gb300" / "lib" / "yk_run"

TOML = """
[physics]
useMass = "true"
mass = -0.5
g = 1.0
cutFraction = 0.35355339059327373

[langevin]
averageEpsilon = {eps_bar}
MaxLangevinTime = {max_time}
ExportTime = {export_time}
burnCount = {burn}
MeasureDriftCount = {measure}

[io]
configFileName = "cfg.bin"
export = "false"
timeSliceFileName = "slice.dat"
{io_extra}

[random]
seed = 11

[fermions]
yukawa_coupling = 0.5
fermion_mass = 0.1
driftMode = 0
WilsonParam = 1.0

[lattice]
Nt = 16
Nx = 16

[gpu]
cg_tol_mode = "rel"
cg_tol = 1e-12
fixed_dt = {fixed_dt}
init = "philox"
"""


def write_toml(d: Path, **kw):
    v = dict(eps_bar=0.001, max_time=0.06, export_time=0.02, burn=2, measure=2, io_extra="", fixed_dt=0.0)
    v.update(kw)
    d.mkdir(parents=True, exist_ok=True)
    (d / "input.toml").write_text(TOML.format(**v))
    return d / "input.toml"


def run_cli(toml, out_dir, timeout=300):
    r = subprocess.run([str(CLI), str(toml), str(out_dir)], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr
    return r.stdout


def read_outputs(d: Path, Nt):
    blocks = [b for b in (d / "slice.dat").read_text().split("\n\n") if b.strip()]
    slices = np.array([[float(v) for v in b.split()] for b in blocks])
    corr = np.array([float(v) for v in (d / "data.csv").read_text().split()[1:]]).reshape(-1, Nt)
    rows = (d / "traces.csv").read_text().strip().splitlines()
    assert rows[0] == "tr,sigma,phi"
    traces = np.array([[float(v) for v in r.split(",")] for r in rows[1:]])
    return slices, corr, traces


def protocol(yk, toml, burn, measure, max_time, export_time):
    """main.cu:295-484 restated on the C ABI."""
    p = yk.Params.from_toml(toml)
    V = p.Nt * p.Nx
    eps_bar = p.average_epsilon
    with yk.Context(p) as ctx:
        def block():
            t, eps, o = 0.0, None, None
            while t < export_time:
                ctx.step(1)
                o = ctx.observables()
                t += o.eps
                eps = o.eps
            return t, eps, o

        for _ in range(burn):
            block()
        avg_eps = None
        if measure > 0:
            elapsed, s, n = 0.0, 0.0, 0
            while elapsed < measure * export_time:
                t, eps, _ = block()
                elapsed += t
                s += eps
                n += 1
            avg_eps = s / n
            eps_bar *= eps_bar / avg_eps
        ctx.set_eps_bar(eps_bar)
        out = {"avg_eps": avg_eps, "eps": [], "slices": [], "corr": [], "traces": []}
        elapsed = 0.0
        while elapsed < max_time:
            t, eps, o = block()
            elapsed += t
            out["eps"].append(eps)
            out["slices"].append(ctx.time_slices() / p.Nx)
            out["corr"].append(ctx.correlator()[0])
            tr, _ = ctx.condensate()
            avg = o.sum_phi
            out["traces"].append([tr, avg / V, abs(avg) / V])
    return {k: (np.array(v) if k != "avg_eps" else v) for k, v in out.items()}


def test_run_protocol_files_and_eps_bar_rescale(ylib, cuda, tmp_path):
    yk = ylib
    toml = write_toml(tmp_path / "run")
    stdout = run_cli(toml, tmp_path / "run")
    want = protocol(yk, toml, burn=2, measure=2, max_time=0.06, export_time=0.02)
    lines = stdout.splitlines()
    assert "Thermalization done!" in lines and "Drift measuring done!" in lines
    avg_line = [l for l in lines if l.startswith("#Average eps during drift measurement = ")]
    assert len(avg_line) == 1
    assert float(avg_line[0].split("=")[1]) == pytest.approx(want["avg_eps"], rel=1e-5)
    slices, corr, traces = read_outputs(tmp_path / "run", 16)
    assert slices.shape == want["slices"].shape and len(traces) == len(want["traces"]) >= 3
    np.testing.assert_allclose(slices, want["slices"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(corr, want["corr"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(traces, want["traces"], rtol=1e-5, atol=1e-12)
    # the export lines: elapsed, eps, <sigma>, abs. mag, cond, partial avg
    exp = [l for l in lines if "abs. mag:" in l]
    assert len(exp) == len(want["eps"])
    eps_printed = np.array([float(l.split("\t")[1]) for l in exp])
    np.testing.assert_allclose(eps_printed, want["eps"], rtol=1e-5)
    # the rescaled epsBar sets the step: eps = epsBar' * 30 / max|drift|
    assert any(l.startswith("Final abs. magnetisation:") for l in lines)


def test_sigusr2_finishes_the_run_early(ylib, cuda, tmp_path):
    toml = write_toml(tmp_path / "sig", max_time=1e6, burn=0, measure=0, fixed_dt=0.01, export_time=0.05)
    proc = subprocess.Popen([str(CLI), str(toml), str(tmp_path / "sig")], stdout=subprocess.PIPE,
                            stderr=subprocess.PIPE, text=True)
    try:
        seen = []
        deadline = time.time() + 120
        while time.time() < deadline:
            line = proc.stdout.readline()
            if not line:
                break
            seen.append(line)
            if "abs. mag:" in line:
                break
        assert any("abs. mag:" in l for l in seen), "no export line before the deadline"
        os.kill(proc.pid, signal.SIGUSR2)
        rest, err = proc.communicate(timeout=120)
    finally:
        if proc.poll() is None:
            proc.kill()
            proc.wait()
    assert proc.returncode == 0, err
    out = "".join(seen) + rest
    assert "#Early termination signal received.\n#Wrapping up.\n" in out
    assert "Final abs. magnetisation:" in out
    assert (tmp_path / "sig" / "cfg.bin.ckpt").exists()


def test_resume_continues_from_the_checkpoint(ylib, cuda, tmp_path):
    # one run of 8 export blocks against a run of 4 blocks resumed by another 4
    kw = dict(burn=0, measure=0, fixed_dt=0.01, export_time=0.05)
    # limits between block ends, so that float sums of the blocks' times
    # cannot land on either side of them
    whole = write_toml(tmp_path / "whole", max_time=0.38, **kw)
    run_cli(whole, tmp_path / "whole")
    first = write_toml(tmp_path / "first", max_time=0.18, **kw)
    run_cli(first, tmp_path / "first")
    second_dir = tmp_path / "second"
    second_dir.mkdir()
    (second_dir / "start.ckpt").write_bytes((tmp_path / "first" / "cfg.bin.ckpt").read_bytes())
    second = write_toml(second_dir, max_time=0.18, io_extra='startFileName = "start.ckpt"\nresume = "true"', **kw)
    run_cli(second, second_dir)
    _, _, t_whole = read_outputs(tmp_path / "whole", 16)
    _, _, t_first = read_outputs(tmp_path / "first", 16)
    _, _, t_second = read_outputs(second_dir, 16)
    assert len(t_first) + len(t_second) == len(t_whole)
    np.testing.assert_array_equal(np.vstack([t_first, t_second]), t_whole)
