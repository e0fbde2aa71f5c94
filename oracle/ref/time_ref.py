"""Time the reference's own CUDA kernels on this GPU (oracle/ref/ref_harness.cpp
--time, kernels compiled from the reference's sources by
oracle/ref/build_ref.py into oracle/_ref/ref_<Nt>x<Nx>.fatbin).

What is timed, launched and synchronised as the reference does it:
  * the Dirac apply (DiracOP::applyD, Dirac.cu:23-35), 136 B/site;
  * one CG solve on D^dag D of a seeded Gaussian right-hand side with the
    reference's occupancy-sized grid and its compile-time stop (|r| <= 1e-8
    absolute, 1000 iterations; CGsolver.cu:42-59, params.h:13-15); the
    iterations of that solve are counted by the CPU oracle's restatement of
    the same CG (the kernel does not report them);
  * full Langevin steps of main.cu:370-381 (coloured noise with DoRNG, cuFFT
    and ApplyMask; getForce with fillNormalRND, setZero_kernel, the solve,
    applyD, computeDrift; Run; the eps copy), wall clock.
The 256 x 256 field is the bench's thermalised start field
(tests/golden/start_256x256.npz); other lattices start from a seeded uniform
field.  Parameters: m^2 = -0.5, lambda = 1, g = 0.5, m0 = 0.1, r = 1,
cutFraction = 1/(2 sqrt 2), the reference's adaptive step with epsBar 0.01.

TEST AND MEASUREMENT INFRASTRUCTURE ONLY (the reference arm of bench.py).
Run on a GPU machine: python oracle/ref/time_ref.py [--sizes 256x256] [--steps 20]
"""
from __future__ import annotations

import argparse
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF = HERE.parent / "_ref"
sys.path.insert(0, str(ROOT))


def time_size(Nt: int, Nx: int, steps: int) -> dict:
    from oracle import oracle as O
    from oracle.ref.make_golden import build_harness
    fat, sym = REF / f"ref_{Nt}x{Nx}.fatbin", REF / f"symbols_{Nt}x{Nx}.txt"
    if not fat.exists() or not sym.exists():
        return {"lattice": [Nt, Nx], "unavailable": f"{fat.name} not built (oracle/ref/build_ref.py needs the "
                                                    f"reference sources)"}
    V = Nt * Nx
    start = ROOT / "tests" / "golden" / f"start_{Nt}x{Nx}.npz"
    if start.exists():
        phi = np.load(start)["phi"].astype(np.float64)
    else:
        phi = np.random.default_rng(1234).uniform(-1, 1, V)
    b = np.zeros((V, 4), dtype=np.complex128)
    b.real = np.random.default_rng(7).normal(size=(V, 4))
    exe = build_harness()
    with tempfile.TemporaryDirectory(prefix="yk_time_") as td:
        fp, bp, op = Path(td) / "phi.raw", Path(td) / "b.raw", Path(td) / "out.json"
        phi.tofile(fp)
        b.view(np.float64).tofile(bp)
        r = subprocess.run([str(exe), str(fat), str(sym), str(Nt), str(Nx), "--time", str(fp), str(bp), str(steps),
                            str(op)], capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            return {"lattice": [Nt, Nx], "unavailable": f"ref_harness failed ({r.returncode}): {r.stderr[-300:]}"}
        out = json.loads(op.read_text())
    a = O.action(m2=-0.5, lam=1.0, g=0.5, m0=0.1, r=1.0)
    _, it, _ = O.cg(Nt, Nx, a, phi, b, mtype=1, tol=1e-8, tol_mode=0, max_iter=1000)
    out["cg_iterations"] = it
    out["cg_ms_per_iteration"] = round(out["cg_solve_ms"] / max(it, 1), 6)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="32x32,256x256")
    ap.add_argument("--steps", type=int, default=20)
    args = ap.parse_args(argv)
    res = [time_size(*(int(v) for v in s.split("x")), args.steps) for s in args.sizes.split(",")]
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
