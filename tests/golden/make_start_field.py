"""Generate tests/golden/start_256x256.npz: the thermalised starting field of
the bench's 256 x 256 workload.

Both arms of bench.py (this library on the GPU, and the CPU restatement of the
reference on the host cores) start their timed steps from this one field, so
the steps they time are the same stretch of the same trajectory and their
cost does not depend on how many steps are timed (the first steps from the
iid Uniform[-1, 1] start need several times the CG iterations of the
thermalised chain).

The field is the CPU oracle's (FP64 CG to relative residual 1e-10) after
BURN_IN Langevin steps of the workload from the Philox uniform start of seed
1234: m^2 = -0.5, lambda = 1, g = 0.5, m0 = 0.1, r = 1, cutFraction =
1/(2 sqrt 2), fixed dt = 0.01, one right-hand side.  The timed steps continue
the Philox streams at step BURN_IN.

TEST INFRASTRUCTURE: run here (CPU) with `python tests/golden/make_start_field.py`.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

NT = NX = 256
BURN_IN = 2000
SEED = 1234
CUT = 0.35355339059327373


def main() -> int:
    from oracle import oracle as O
    a = O.action(m2=-0.5, lam=1.0, g=0.5, m0=0.1, r=1.0, cut_fraction=CUT)
    phi = O.uniform_field(SEED, 0, NT * NX)
    t0 = time.perf_counter()
    sig = []
    its = []
    for s in range(BURN_IN):
        phi, ob = O.langevin_step(NT, NX, a, phi, SEED, 0, s, tol=1e-10, tol_mode=1, max_iter=20000, fixed_dt=0.01)
        sig.append(ob.sum_phi / (NT * NX))
        its.append(ob.cg_iters)
    out = HERE / f"start_{NT}x{NX}.npz"
    np.savez_compressed(out, phi=phi, step=np.int64(BURN_IN), seed=np.int64(SEED), shape=np.array([NT, NX]),
                        mean_sigma=np.array(sig), cg_iterations=np.array(its))
    print(f"wrote {out}: {BURN_IN} steps in {time.perf_counter() - t0:.1f} s, <sigma> {sig[-1]:.6f}, "
          f"CG iterations first {its[0]} last {its[-1]}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
