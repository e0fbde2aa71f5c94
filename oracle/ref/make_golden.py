"""Generate the golden fixtures tests/golden/ref_<Nt>x<Nx>.npz from the reference.

Builds oracle/ref/ref_harness.cpp (host code of this project; CUDA driver API +
cuFFT) on the machine it runs on, runs it on a GPU against the reference
kernels compiled by oracle/ref/build_ref.py (oracle/_ref/*.fatbin), and packs
each binary dump into an .npz.  Run on a GPU machine:

    python oracle/ref/make_golden.py --out <dir> [--sizes 32x32]

TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import argparse
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE.parent / "_ref"
SIZES = [(8, 4), (6, 10), (16, 16), (32, 32)]


def build_harness() -> Path:
    exe = REF / "ref_harness"
    src = HERE / "ref_harness.cpp"
    if exe.exists() and exe.stat().st_mtime > src.stat().st_mtime:
        return exe
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-O2", "-std=c++17", str(src), "-I", f"{cuda}/include", "-L", f"{cuda}/lib64",
           "-L", f"{cuda}/lib64/stubs", "-lcufft", "-lcudart", "-lcuda", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def read_dump(path: Path) -> dict[str, np.ndarray]:
    raw = path.read_bytes()
    out, off = {}, 0
    while off < len(raw):
        name = raw[off:off + 32].split(b"\0")[0].decode()
        n = int(np.frombuffer(raw, dtype=np.int64, count=1, offset=off + 32)[0])
        out[name] = np.frombuffer(raw, dtype=np.float64, count=n, offset=off + 40).copy()
        off += 40 + 8 * n
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(HERE.parent.parent / "tests" / "golden"))
    ap.add_argument("--sizes", default=None, help="e.g. 32x32,16x16 (default: every size)")
    args = ap.parse_args(argv)
    sizes = SIZES if not args.sizes else [tuple(int(v) for v in s.split("x")) for s in args.sizes.split(",")]
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    exe = build_harness()
    for nt, nx in sizes:
        dump = out / f"ref_{nt}x{nx}.bin"
        subprocess.run([str(exe), str(REF / f"ref_{nt}x{nx}.fatbin"), str(REF / f"symbols_{nt}x{nx}.txt"),
                        str(nt), str(nx), str(dump)], check=True)
        arrays = read_dump(dump)
        np.savez_compressed(out / f"ref_{nt}x{nx}.npz", **arrays)
        dump.unlink()
        print(f"wrote {out / f'ref_{nt}x{nx}.npz'} ({len(arrays)} arrays)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
