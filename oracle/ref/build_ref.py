"""Compile the reference's own CUDA kernels into device fatbins (oracle/_ref/).

The reference fixes the lattice at compile time (code/src/params.h:28, patched
by runs.py:80-85 with sed before each build).  For each golden lattice size
this recipe copies code/src into a temporary directory OUTSIDE the repository,
patches the Sizes line the same way, and compiles the kernel sources with
nvcc for sm_103a (--expt-relaxed-constexpr, -DUSE_cuFFT: the flags of
code/Makefile) as one translation unit that #includes them, preceded by
consts.cu (the __constant__ symbols that main.cu defines; main.cu itself needs
the absent toml11 header), into oracle/_ref/ref_<Nt>x<Nx>.fatbin.  In that
single unit the sources' `extern __constant__` re-declarations are dropped
from the copies (consts.cu defines the symbols; a non-relocatable unit cannot
hold both), which is the only other edit besides the Sizes line.  The mangled
kernel names are read from the host object of the same unit with `nm` into
oracle/_ref/symbols_<Nt>x<Nx>.txt.  Nothing of
the reference is written into the repository; only compiled device code
lands in oracle/_ref/ (git-ignored).

Runs only where the reference sources are present; the GPU machine uses the
prebuilt fatbins through oracle/ref/ref_harness.cpp.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile
from pathlib import Path

# the reference's code/src directory (environment YK_REFERENCE_SRC overrides the default)
REF_SRC = Path(os.environ.get("YK_REFERENCE_SRC", "/root/reference/code/src"))
HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
SIZES = [(8, 4), (6, 10), (16, 16), (32, 32), (256, 256)]
TUS = ["Dirac.cu", "CGsolver.cu", "FermionicDrift.cu", "reductions.cu", "langevin_gpu_v2.cu", "Lattice.cu"]
KERNELS = ["applyD_gpu", "solve_kernel", "computeDrift", "Run", "gpuMagnetisation", "gpuTimeSlices",
           "gpuTimeSlices_spinors", "gpuTraces", "ApplyMask", "DoRNG", "setup_kernel", "random_setup_kernel",
           "fillNormalRND", "setZero_kernel"]
FLAGS = ["-arch=sm_103a", "--expt-relaxed-constexpr", "-DUSE_cuFFT", "-O3", "-w"]


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_size(Nt: int, Nx: int) -> Path:
    fat = OUT / f"ref_{Nt}x{Nx}.fatbin"
    sym = OUT / f"symbols_{Nt}x{Nx}.txt"
    if fat.exists() and sym.exists():
        return fat
    with tempfile.TemporaryDirectory(prefix="yk_ref_") as td:
        src = Path(td) / "src"
        src.mkdir()
        for f in REF_SRC.iterdir():
            if f.suffix in (".cu", ".cuh", ".h", ".cpp") and f.name not in ("vkFFT.h", "main.cu", "test.cu"):
                shutil.copy(f, src / f.name)
        params = src / "params.h"
        text = params.read_text()
        needle = "dimArray constexpr Sizes = {16, 16};"
        assert needle in text, "Sizes line not found in params.h"
        params.chmod(0o644)
        params.write_text(text.replace(needle, f"dimArray constexpr Sizes = {{{Nt}, {Nx}}};"))
        (src / "consts.cu").write_text(
            '#include "params.h"\n'
            "__constant__ myType epsBar;\n__constant__ myType m2;\n__constant__ myType lambda;\n"
            "__constant__ double yukawa_coupling_gpu;\n__constant__ double fermion_mass_gpu;\n"
            "__constant__ thrust::complex<double> im_gpu;\n__constant__ double cutFraction_gpu;\n"
            "__constant__ double sq2Kappa_gpu;\n__constant__ DriftMode driftMode_gpu;\n"
            "__constant__ double WilsonParam_gpu;\n")
        for f in src.iterdir():
            if f.suffix in (".cu", ".cpp") and f.name != "consts.cu":
                lines = f.read_text().splitlines(keepends=True)
                f.chmod(0o644)
                f.write_text("".join(l for l in lines if not l.lstrip().startswith("extern __constant__")))
        unity = src / "unity.cu"
        unity.write_text("".join(f'#include "{t}"\n' for t in ["consts.cu"] + TUS + ["colouredNoise.cpp"]))
        OUT.mkdir(exist_ok=True)
        obj = Path(td) / "unity.o"
        for extra in (["-fatbin", "-o", str(fat)], ["-c", "-o", str(obj)]):
            r = subprocess.run([_nvcc()] + FLAGS + ["-I", str(src), str(unity)] + extra, capture_output=True,
                               text=True)
            if r.returncode:
                raise RuntimeError(r.stderr)
        objs = [obj]
        names = subprocess.run(["nm", "--defined-only"] + [str(o) for o in objs], capture_output=True,
                               text=True).stdout.split()
        lines = []
        for k in KERNELS:
            pref = f"_Z{len(k)}{k}"
            hits = [n for n in names if n.startswith(pref) and "__device_stub" not in n]
            if not hits:
                raise RuntimeError(f"kernel {k} not found")
            lines.append(f"{k} {hits[0]}")
        sym.write_text("\n".join(lines) + "\n")
    return fat


def build() -> list[Path]:
    if not REF_SRC.exists():
        return []
    return [build_size(nt, nx) for nt, nx in SIZES]


if __name__ == "__main__":
    for p in build():
        print(p)
