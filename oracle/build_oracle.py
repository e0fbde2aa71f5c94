"""Build recipe of the CPU oracle: gcc on yukawa_oracle.c, output in oracle/_build.

-ffp-contract=off keeps the arithmetic free of fused multiply-adds so the
oracle gives the same bits on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libyukawa_oracle.so"


def build(openmp: bool = True) -> Path:
    OUT.mkdir(exist_ok=True)
    src = HERE / "yukawa_oracle.c"
    if LIB.exists() and LIB.stat().st_mtime > max(src.stat().st_mtime, (HERE / "yukawa_oracle.h").stat().st_mtime):
        return LIB
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O3", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", str(src), "-o", str(LIB), "-lm"]
    if openmp:
        cmd.insert(1, "-fopenmp")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build())
