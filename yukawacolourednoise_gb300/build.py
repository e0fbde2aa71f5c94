"""Build recipe of libyukawa_gb300.so (sm_103a) and of the yk_run CLI.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library inside the package (``yukawacolourednoise_gb300/lib``).  No
cmake, no torch extension machinery: the product is a plain C-ABI library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libyukawa_gb300.so"
CLI = LIB_DIR / "yk_run"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(CSRC)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cu", ".cpp") and p.name != "yk_run_main.cpp")


def _compile(src: Path, extra: list[str], build_dir: Path) -> Path:
    obj = build_dir / (src.stem + ".o")
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "yukawa.h"]
    if obj.exists() and obj.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra
    if src.suffix == ".cpp":
        cmd += ["-x", "cu"]
    cmd += ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile every translation unit for sm_103a and link the library and CLI."""
    extra = list(extra or [])
    # objects of a build with extra flags live apart from the default build's
    build_dir = BUILD if not extra else BUILD.with_name(BUILD.name + "_" + "_".join(
        f.strip("-").replace("=", "_") for f in extra))
    build_dir.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, build_dir), srcs))
    cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    main = CSRC / "yk_run_main.cpp"
    if main.exists():
        cmd = [nvcc()] + ARCH + ["-O2", "-std=c++17", "-I", str(ROOT / "include"), str(main), "-o", str(CLI),
               "-L", str(LIB_DIR), "-lyukawa_gb300", "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
