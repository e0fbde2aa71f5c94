#!/usr/bin/env python3
"""Langevin steps/sec of the 2-D Yukawa hot path on GB300 (one JSON line).

Workload (the precision configuration of the headline metric): a 256 x 256
lattice, m^2 = -0.5, lambda = 1, Yukawa g = 0.5, m0 = 0.1, Wilson r = 1,
coloured-noise cutoff Lambda = pi/2 (cutFraction = 1/(2 sqrt 2)), fixed Euler
step dt = 0.01, one Gaussian stochastic right-hand side per step, CG on
D^dag D to relative residual 1e-10 with FP32 iterations and FP64 reliable
updates (every 50 iterations, and each time the FP32 residual drops a
hundredfold), FP64 field.  Synthetic data: all noise is drawn from Philox,
and both arms start from one thermalised field (tests/golden/start_256x256.npz:
2000 steps of the CPU oracle from iid Uniform[-1, 1], seed 1234), run the
warm-up steps from it and time the steps that follow, so both time the same
stretch of the same trajectory and the rate does not depend on --steps.

One step = coloured noise + fermion force (CG) + drift/Euler update +
per-step observables, replayed as one CUDA graph.  L2 (129 MB) is flushed by a
256 MiB write between timed steps, outside the timed events.  Every other leg
of the line (kernel profile, e2e through the C ABI with host buffers, the
plain FP64 form, the precision errors) replays that same segment.

  --impl ours (default): the CUDA path; `value` = steps/s of all ranks.
  --impl reference: the CPU oracle (C restatement of the reference's
      algorithm; the reference itself has no CPU path) on the host cores;
      beside it, `reference_gpu`: the reference's own CUDA kernels (compiled
      from its sources) timed on this GPU.

Multi-GPU: chains are independent, so N GPUs run N replicas (weak scaling,
no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Langevin steps/sec @CG rel-res 1e-10, learned+mixed vs plain FP64 CG; Dirac HBM GB/s"
NT = NX = 256
CUT = 0.35355339059327373          # Lambda = pi/2  ->  cutFraction = Lambda / (sqrt(2) pi)
BYTES_CG_ITER_MIXED = 200          # unique bytes per site per FP32 CG iteration of cg_kernel (passes A and B)
BYTES_CG_ITER_HALO = 128           # the same for cg_halo_kernel: D p stays in shared memory, diag is cached
BYTES_CG_ITER_FP64 = 400
BYTES_CG_ITER_EO = 48              # cg_eo_kernel: r, q, p loaded and stored per compact (even) site, 96 B = 48 B per site
# the thermalised start of the workload (both arms time the same steps from it)
START = ROOT / "tests" / "golden" / "start_256x256.npz"
DATA = ("synthetic: Philox noise; the timed steps continue a chain from tests/golden/start_256x256.npz, "
        "the CPU oracle's field after 2000 Langevin steps from iid Uniform[-1, 1] (seed 1234)")


def workload(precision: str) -> dict:
    return {"workload": f"2D {NT}x{NX} Yukawa Langevin step (coloured noise + CG force + Euler), "
                        f"CG rel-res 1e-10, {precision} CG, 1 RHS, fixed dt 0.01",
            "lattice": [NT, NX], "n_rhs": 1, "precision": precision, "cg_tol_rel": 1e-10,
            "reliable_every": 50, "reliable_delta": 1e-5, "m2": -0.5, "lambda": 1.0, "g": 0.5, "m0": 0.1, "cut_fraction": CUT,
            "l2": "flushed between timed steps (256 MiB write)"}


def make_params(yk, precision, seed=1234, Nt=NT, Nx=NX):
    return yk.Params.default(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=0.1,
                             wilson_param=1.0, cut_fraction=CUT, Nt=Nt, Nx=Nx, fixed_dt=0.01,
                             precision=yk.YK_MIXED if precision == "mixed" else yk.YK_FP64,
                             cg_tol=1e-10, cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=20000, reliable_every=50, reliable_delta=1e-5,
                             n_rhs=1, seed=seed, init=yk.YK_INIT_PHILOX)


# ---------------------------------------------------------------- distributed
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4) if "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(kernel):
    """DRAM bytes per CG iteration of `kernel` from its committed ncu summary, if any."""
    f = ROOT / "profiles" / f"{kernel}_256x256_traffic.json"
    if f.exists():
        try:
            return json.loads(f.read_text())
        except Exception:
            return None
    return None


def max_over_ranks(t_sec: float, dist, device) -> float:
    """The job's time: the slowest rank's timed region (all ranks call this)."""
    if dist is None:
        return t_sec
    import torch
    t = torch.tensor([t_sec], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(steps: int, ws: int, t_all: float) -> float:
    """Whole-job steps/s: every rank runs an independent replica of `steps` steps."""
    return steps * ws / t_all


# ---------------------------------------------------------------- our arm
def run_ours(args, ws, rank, local):
    import numpy as np
    import torch
    import yukawacolourednoise_gb300 as yk

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed_steps(ctx, k):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        with torch.cuda.stream(stream):
            for i in range(k):
                starts[i].record(stream)
                ctx.step(1)
                ends[i].record(stream)
                flush.fill_(i & 0xFF)
        stream.synchronize()
        return sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / 1e3

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    phi_start, step_start = start_field()
    ctx = yk.Context(make_params(yk, args.precision, seed=1234 + rank))
    ctx.set_stream(stream.cuda_stream)
    ctx.set_field(phi_start)
    ctx.set_step(step_start)
    ctx.step(args.warmup)
    ctx.synchronize()
    # the timed segment starts here: every other leg of this run replays it
    phi_seg, step_seg = ctx.get_field(), ctx.get_step()
    obs_seg = ctx.observables()

    barrier()
    clocks = Clocks(local)
    t_sec = timed_steps(ctx, args.steps)
    barrier()
    clk = clocks.stop()
    obs = ctx.observables()
    if obs.status not in (0, yk.YK_ENOCONV):
        raise RuntimeError(f"step status {obs.status}")
    phi_end = ctx.get_field()
    seg_iters = obs.cg_iterations_total - obs_seg.cg_iterations_total
    cg_stats = {"iterations_per_step": round(seg_iters / args.steps, 1),
                "steps_at_iteration_cap": int(obs.noconv_steps - obs_seg.noconv_steps), "iteration_cap": 20000}
    t_all = max_over_ranks(t_sec, dist, "cuda")
    value = job_value(args.steps, ws, t_all)

    extras = {}
    if rank == 0 and not args.quick:
        # kernel timing of the same segment: CUDA events around each kernel class
        ctx.set_field(phi_seg)
        ctx.set_step(step_seg)
        ctx.profile_begin()
        with torch.cuda.stream(stream):
            ctx.step(args.steps)
        pr = ctx.profile_end()
        extras["roofline"], extras["kernel_share"] = roofline(pr, args.precision)
        launches_per_step = pr.launches / max(pr.steps, 1)
        extras["e2e"] = e2e(yk, torch, ctx, phi_seg, step_seg, args.steps, flush, phi_end)
        # plain FP64 CG form of the same segment (the metric's denominator)
        if args.precision == "mixed":
            extras["plain_fp64"] = plain_fp64(yk, torch, stream, timed_steps, phi_start, step_start, args, value / ws)
            extras["precision_errors"] = precision_errors(yk, torch, stream, phi_seg, step_seg,
                                                          min(args.steps, 20))
        # Dirac apply HBM bandwidth on a lattice larger than L2 (complex buffers)
        extras["dirac_hbm"] = dirac_hbm(yk, torch, stream)
        # the batching configuration (many chains of uneven sizes in one graph)
        extras["batching"] = batched(yk, torch, stream)
        # the learned-preconditioner configuration (512^2 near the chiral regime)
        if not args.no_learned:
            extras["learned"] = learned(yk, torch, stream, steps=args.learned_steps)
        # the full form at scale (8 chains of 1024^2, 8 RHS), one timed step per arm
        if not args.no_full_scale:
            extras["full_scale"] = full_scale(yk, torch, stream)
        extras["gpu_launches"] = int(round(launches_per_step * args.steps))

    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return None
    line = {"metric": METRIC, "value": round(value, 2), "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_all / args.steps * 1e3, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
            "data": DATA, "config": workload(args.precision), "clocks": clk, "cg": cg_stats}
    line.update(extras)
    if "gpu_launches" not in line:
        line["gpu_launches"] = 7 * args.steps
    if not args.no_cpu and ws == 1:
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds, args.warmup)
    return line


def start_field():
    """The thermalised starting field of the 256^2 workload and the Philox
    step it continues at (tests/golden/make_start_field.py)."""
    import numpy as np
    d = np.load(START)
    return np.ascontiguousarray(d["phi"], dtype=np.float64), int(d["step"])


def roofline(pr, precision):
    """Roofline of the dominant kernel (the persistent CG) from the profiled
    steps: algorithmic bytes per launch / CUDA-event launch time."""
    per_launch_ms = pr.cg_ms / max(pr.cg_launches, 1)
    halo, eo = pr.cg_kernel == 1, pr.cg_kernel == 3
    if precision != "mixed":
        bpi = BYTES_CG_ITER_FP64
    else:
        bpi = BYTES_CG_ITER_EO if eo else (BYTES_CG_ITER_HALO if halo else BYTES_CG_ITER_MIXED)
    kname = "cg_eo_kernel" if eo else ("cg_halo_kernel" if halo else
                                       f"cg_kernel<1,{'mixed' if precision == 'mixed' else 'fp64'}>")
    alg_bytes = pr.cg_site_iterations * bpi / max(pr.cg_launches, 1)
    pk = peaks()
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    tr = ncu_traffic(kname)
    traffic = None
    if tr and tr.get("precision") == precision and tr.get("kernel", "cg_kernel<1,mixed>") == kname:
        traffic = tr["dram_bytes_per_iteration"] * pr.cg_iterations / max(pr.cg_launches, 1)
    roof = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": traffic,
            "peak_source": pk["source"], "bytes_per_site_iteration": bpi,
            "cg_iterations_per_step": pr.cg_iterations / max(pr.steps, 1),
            "ms_per_launch": round(per_launch_ms, 4), "profiled_steps": pr.steps}
    tot = pr.noise_ms + pr.cg_ms + pr.force_ms + pr.update_ms
    share = {k: round(v / tot, 4) for k, v in (("noise", pr.noise_ms), ("cg", pr.cg_ms),
                                                ("force_drift", pr.force_ms), ("update", pr.update_ms))}
    return roof, share


def e2e(yk, torch, ctx, phi_seg, step_seg, k, flush, phi_end):
    """The same k steps as `value` (the timed segment replayed from its first
    field and Philox step) through the C ABI with host buffers: every step
    uploads the field from pinned host memory, steps, and reads the field and
    the observables back (yk_langevin_step_io: one call, one synchronisation).
    Wall clock around each step's call; L2 flushed between steps, outside the
    timed calls."""
    import ctypes as C
    V = NT * NX
    host_in = torch.empty(V, dtype=torch.float64).pin_memory()
    host_out = torch.empty(V, dtype=torch.float64).pin_memory()
    host_in.copy_(torch.from_numpy(phi_seg))
    ctx.set_step(step_seg)
    lib = yk.lib()
    o = yk.Obs()
    sec = 0.0
    for i in range(k):
        flush.fill_(i & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        yk._check(lib.yk_langevin_step_io(ctx.h, 0, C.c_void_p(host_in.data_ptr()), C.c_void_p(host_out.data_ptr()),
                                          C.byref(o)))
        sec += time.perf_counter() - t0
        host_in, host_out = host_out, host_in
    same = bool(torch.equal(host_in, torch.from_numpy(phi_end)))
    return {"value": round(k / sec, 2), "unit": "steps/s", "h2d_bytes_per_step": 8 * V,
            "d2h_bytes_per_step": 8 * V + C.sizeof(yk.Obs), "steps": k,
            "segment": "the steps timed for value, replayed from the segment's first field and step",
            "same_trajectory_as_value": same, "l2": "flushed between steps (outside the timed calls)"}


def plain_fp64(yk, torch, stream, timed_steps, phi_start, step_start, args, value_mixed):
    """The plain FP64 CG form of the same workload and segment (the metric's
    denominator): FP64 stencil and CG (cg_kernel, the grid-wide persistent
    kernel; the halo kernel serves single-system mixed solves)."""
    ctx64 = yk.Context(make_params(yk, "fp64"))
    ctx64.set_stream(stream.cuda_stream)
    ctx64.set_field(phi_start)
    ctx64.set_step(step_start)
    ctx64.step(args.warmup)
    ctx64.synchronize()
    o0 = ctx64.observables()
    k64 = args.fp64_steps or args.steps
    t64 = timed_steps(ctx64, k64)
    o1 = ctx64.observables()
    ctx64.close()
    return {"value": round(k64 / t64, 2), "unit": "steps/s", "steps": k64,
            "cg_iterations_per_step": round((o1.cg_iterations_total - o0.cg_iterations_total) / k64, 1),
            "cg_kernel": "cg_kernel<1,fp64> (grid-wide persistent CG)",
            "speedup_mixed_over_fp64": round(value_mixed / (k64 / t64), 3)}


def precision_errors(yk, torch, stream, phi_seg, step_seg, n, n_ops=5):
    """Errors of the mixed FP32/FP64 path against this library's FP64 path
    (itself pinned to the CPU oracle to 1e-13 by the tests), at the fields of
    the timed segment: per step, the max relative error of the FP32 Dirac
    apply (a Gaussian spinor), of the mixed CG solution (rel-res 1e-10, the
    same Gaussian right-hand side) and of the step's fermion force (the
    step's Philox source, the mixed step solver against the FP64 one); and
    <sigma> of the mixed and FP64 trajectories from the segment's first field
    with the same Philox streams."""
    import numpy as np
    V = NT * NX
    cm = yk.Context(make_params(yk, "mixed"))
    c64 = yk.Context(make_params(yk, "fp64"))
    for c in (cm, c64):
        c.set_stream(stream.cuda_stream)
        c.set_field(phi_seg)
        c.set_step(step_seg)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    d_err, x_err, f_err, sig_m, sig_64 = [], [], [], [], []

    def rel(a, b):
        return float((a - b).abs().max() / b.abs().max())

    with torch.cuda.stream(stream):
        for s in range(n):
            if s < n_ops:
                c64.set_field(cm.get_field())
                c64.set_step(step_seg + s)
                psi = torch.randn(V, 4, dtype=torch.complex128, device="cuda", generator=gen)
                y64 = torch.empty_like(psi)
                y32 = torch.empty(V, 4, dtype=torch.complex64, device="cuda")
                c64.dirac_apply(psi, y64, False, yk.YK_FP64)
                c64.dirac_apply(psi.to(torch.complex64), y32, False, yk.YK_FP32)
                x64, xm = torch.zeros_like(psi), torch.zeros_like(psi)
                c64.cg_solve(psi, x64, yk.YK_DAGGER, 1e-10, yk.YK_TOL_REL, 20000, yk.YK_FP64)
                c64.cg_solve(psi, xm, yk.YK_DAGGER, 1e-10, yk.YK_TOL_REL, 20000, yk.YK_MIXED)
                fm = torch.empty(V, dtype=torch.float64, device="cuda")
                f64 = torch.empty_like(fm)
                cm.fermion_force(fm)
                c64.fermion_force(f64)
                stream.synchronize()
                d_err.append(rel(y32.to(torch.complex128), y64))
                x_err.append(rel(xm, x64))
                f_err.append(rel(fm, f64))
            cm.step(1)
            sig_m.append(cm.observables().sum_phi / V)
        c64.set_field(phi_seg)
        c64.set_step(step_seg)
        for s in range(n):
            c64.step(1)
            sig_64.append(c64.observables().sum_phi / V)
        dphi = float(np.abs(cm.get_field() - c64.get_field()).max())
    cm.close()
    c64.close()
    dsig = [abs(a - b) for a, b in zip(sig_m, sig_64)]
    return {"reference": "this library's FP64 path (pinned to the CPU oracle to 1e-13 in the tests)",
            "steps_checked": n_ops, "dirac_fp32_max_rel": max(d_err), "cg_mixed_max_rel": max(x_err),
            "force_mixed_max_rel": max(f_err),
            "per_step": {"dirac_fp32": [float(f"{v:.3e}") for v in d_err],
                         "cg_mixed": [float(f"{v:.3e}") for v in x_err],
                         "force_mixed": [float(f"{v:.3e}") for v in f_err]},
            "sigma_steps": n, "sigma_mixed_last": sig_m[-1], "sigma_fp64_last": sig_64[-1],
            "sigma_max_abs_diff": max(dsig), "field_max_abs_diff_last": dphi}




# Algorithmic bytes per lattice site and iteration of the batched even-odd
# kernels.  cg_eob_kernel, per compact site and round: P1 reads r, q, p, xs,
# v and writes r, p, xs, w; P2 reads p, w, writes v; P3 reads v, writes u; P4
# reads v, u, r, writes q: 288 B, i.e. 144 B per lattice site.
# cg_eop_kernel: r, q, p, xs, v read and r, p, q, v, xs written per compact
# site (w and u stay in shared memory; the halo re-reads are not counted):
# 160 B, i.e. 80 B per lattice site.
BATCHED_BYTES_PER_SITE_ITERATION = {4: 144, 5: 80}
BATCHED_KERNELS = {0: "cg_kernel (grid-wide D^dag D)", 3: "cg_eo_kernel (single-system even-odd)",
                   4: "cg_eob_kernel (batched even-odd, four passes)",
                   5: "cg_eop_kernel (batched even-odd over 32 x 16 patches)"}


def eob_roofline(yk, torch, stream, ctx):
    """One more step, profiled: the batched even-odd CG's algorithmic bytes
    (BATCHED_BYTES_PER_SITE_ITERATION of the kernel that ran) over its
    CUDA-event time, against the measured HBM copy bandwidth."""
    ctx.profile_begin()
    with torch.cuda.stream(stream):
        ctx.step(1)
    pr = ctx.profile_end()
    pk = peaks()
    bps = BATCHED_BYTES_PER_SITE_ITERATION.get(pr.cg_kernel, 144)
    gbs = pr.cg_site_iterations * bps / (pr.cg_ms / 1e3) / 1e9 if pr.cg_ms > 0 else 0.0
    return {"kernel": BATCHED_KERNELS.get(pr.cg_kernel, str(pr.cg_kernel)), "cg_ms": round(pr.cg_ms, 3),
            "bytes_per_site_iteration": bps, "achieved": round(gbs, 1), "unit": "GB/s",
            "peak": pk["hbm_gbs"], "frac": round(gbs / pk["hbm_gbs"], 4), "peak_source": pk["source"]}


def full_scale(yk, torch, stream, steps=1, L=1024, n_chains=8, n_rhs=8):
    """The full form at scale: 8 chains of 1024^2 (m0 = 0.01, g = 0.6,
    Lambda = pi/4, i.e. cutFraction 0.17678), 8 stochastic right-hand sides
    per step, all chains in one step, every solve to rel-res 1e-10: the mixed
    CG step graph, the plain FP64 CG step graph and the learned PCG step
    (2-layer network trained on chain 0's field, weights shared by the
    chains; training time reported apart).  Each arm times the first `steps`
    steps from the same seeded start (a step takes seconds: thousands of
    iterations over 64 systems of 2^20 sites); the mixed step's grid is tuned
    before the timed step, the FP64 one runs the co-resident grid untuned."""
    def params(prec, c):
        return yk.Params.default(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.6, fermion_mass=0.01,
                                 wilson_param=1.0, cut_fraction=0.17677669529663687, Nt=L, Nx=L, fixed_dt=0.01,
                                 precision=prec, cg_tol=1e-10, cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=50000,
                                 reliable_every=50, reliable_delta=0.001, n_rhs=n_rhs, seed=1234 + c,
                                 init=yk.YK_INIT_PHILOX)

    out = {"config": f"{n_chains} chains of {L}x{L}, m0 0.01, g 0.6, cutFraction 0.17678, {n_rhs} RHS, "
                     f"rel-res 1e-10, the first {steps} step(s) from the seeded start", "steps": steps}
    for name, prec in (("mixed_cg", yk.YK_MIXED), ("plain_fp64", yk.YK_FP64)):
        saved = os.environ.get("YK_AUTOTUNE")
        if prec == yk.YK_FP64:
            os.environ["YK_AUTOTUNE"] = "0"
        try:
            ctx = yk.Context([params(prec, c) for c in range(n_chains)])
        finally:
            if saved is None:
                os.environ.pop("YK_AUTOTUNE", None)
            else:
                os.environ["YK_AUTOTUNE"] = saved
        ctx.set_stream(stream.cuda_stream)
        if prec == yk.YK_MIXED:
            ctx.autotune()
        ctx.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            ctx.step(steps)
            b.record(stream)
        stream.synchronize()
        sec = a.elapsed_time(b) / 1e3
        obs = [ctx.observables(c) for c in range(n_chains)]
        its = sum(o.cg_iterations_total for o in obs)
        out[name] = {"value": round(steps / sec, 4), "unit": "steps/s (all chains)",
                     "chain_steps_per_s": round(steps * n_chains / sec, 3),
                     "site_steps_per_s": round(steps * n_chains * L * L / sec, 1),
                     "cg_iterations_per_system_step": round(its / (steps * n_chains * n_rhs), 1),
                     "status_ok": all(o.status in (0, yk.YK_ENOCONV) for o in obs)}
        if prec == yk.YK_MIXED:
            out[name]["cg_roofline"] = eob_roofline(yk, torch, stream, ctx)
        ctx.close()
    # learned: chain 0's 2-layer network trained at its field, its weights
    # copied to every chain (same couplings; the features adapt to each field)
    ctx = yk.Context([params(yk.YK_MIXED, c) for c in range(n_chains)])
    ctx.set_stream(stream.cuda_stream)
    for c in range(n_chains):
        ctx.net_setup(2, 7, chain=c)
    st = ctx.net_train(n_sources=4, n_levels=5, base_iter=4, steps=400, batch=4, lr=2e-3, seed=3)
    w = ctx.net_get_weights()
    for c in range(1, n_chains):
        ctx.net_set_weights(w, chain=c)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = ctx.step_learned(steps)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    out["learned_2layers"] = {"value": round(steps / sec, 4), "unit": "steps/s (all chains)",
                              "chain_steps_per_s": round(steps * n_chains / sec, 3),
                              "solver_iterations_per_system_step": round(s.iterations / (steps * n_chains * n_rhs), 1),
                              "all_converged": bool(s.converged),
                              "training": {"pairs": st.pairs, "loss_before": round(st.loss0, 4),
                                           "loss_after": round(st.loss1, 4), "ms": round(st.ms, 1)},
                              "value_incl_training_over_10000_steps":
                                  round(10000 / (10000 / (steps / sec) + st.ms / 1e3), 4)}
    ctx.close()
    out["speedup_mixed_over_fp64"] = round(out["mixed_cg"]["value"] / out["plain_fp64"]["value"], 3)
    out["speedup_learned_over_fp64"] = round(out["learned_2layers"]["value"] / out["plain_fp64"]["value"], 3)
    out["speedup_learned_over_mixed"] = round(out["learned_2layers"]["value"] / out["mixed_cg"]["value"], 3)
    return out


def batched(yk, torch, stream, steps=20, warmup=3, n_chains=64, seed=1234):
    """The batching configuration: 64 chains of seeded sizes {32, 64, 128, 256}^2,
    m0 ~ U[0.05, 0.3], g ~ U[0.3, 0.8], 4 stochastic right-hand sides per chain,
    mixed CG at rel-res 1e-10, every chain stepped by one graph replay."""
    import numpy as np
    rng = np.random.default_rng(seed)
    Ls = rng.choice([32, 64, 128, 256], size=n_chains)
    m0s = rng.uniform(0.05, 0.3, size=n_chains)
    gs = rng.uniform(0.3, 0.8, size=n_chains)
    ps = [yk.Params.default(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=float(g), fermion_mass=float(m0),
                            wilson_param=1.0, cut_fraction=CUT, Nt=int(L), Nx=int(L), fixed_dt=0.01,
                            precision=yk.YK_MIXED, cg_tol=1e-10, cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=20000,
                            reliable_every=50, reliable_delta=0.001, n_rhs=4, seed=seed, init=yk.YK_INIT_PHILOX)
          for L, m0, g in zip(Ls, m0s, gs)]
    ctx = yk.Context(ps)
    ctx.set_stream(stream.cuda_stream)
    ctx.step(warmup)
    ctx.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a.record(stream)
        ctx.step(steps)
        b.record(stream)
    stream.synchronize()
    sec = a.elapsed_time(b) / 1e3
    obs = [ctx.observables(c) for c in range(n_chains)]
    t = ctx.tune_report()
    # two more steps as direct launches: the kernel and its iterations
    ctx.profile_begin()
    with torch.cuda.stream(stream):
        ctx.step(2)
    pr = ctx.profile_end()
    ctx.close()
    pk = peaks()
    bps = BATCHED_BYTES_PER_SITE_ITERATION.get(pr.cg_kernel, 144)
    gbs = pr.cg_site_iterations * bps / (pr.cg_ms / 1e3) / 1e9 if pr.cg_ms > 0 else 0.0
    sites = int(sum(int(L) * int(L) for L in Ls))
    return {"config": f"{n_chains} chains, L in {{32,64,128,256}} (seed {seed}), 4 RHS, mixed CG rel-res 1e-10",
            "value": round(steps * n_chains / sec, 2), "unit": "chain-steps/s",
            "site_steps_per_s": round(steps * sites / sec, 1), "steps": steps,
            "ms_per_step": round(sec * 1e3 / steps, 3),
            "cg_kernel": BATCHED_KERNELS.get(pr.cg_kernel, str(pr.cg_kernel)), "cg_grid": pr.cg_grid,
            "cg_iterations_per_system_step": round(pr.cg_iterations / max(pr.steps * n_chains * 4, 1), 1),
            "cg_roofline": {"bytes_per_site_iteration": bps, "achieved": round(gbs, 1),
                            "unit": "GB/s", "peak": pk["hbm_gbs"], "frac": round(gbs / pk["hbm_gbs"], 4)},
            "status_ok": all(o.status in (0, yk.YK_ENOCONV) for o in obs),
            "autotune": {"cg_grid": t.cg_grid, "cg_grid_max": t.cg_grid_max, "candidates": t.cg_candidates,
                         "ms_chosen": round(t.cg_ms_chosen, 3), "ms_at_max": round(t.cg_ms_max, 3)}}


def learned(yk, torch, stream, L=512, m0=0.02, steps=20, burn_in=20, layer_counts=(4, 2)):
    """The learned-preconditioner configuration: a 512^2 lattice near the
    chiral regime (m0 = 0.02, g = 0.5, m^2 = -0.5, lambda = 1), one RHS, every
    solve to FP64 rel-res 1e-10.  From one burnt-in field, the same `steps`
    Langevin steps by (a) the plain FP64 CG step graph, (b) the mixed CG step
    graph and (c) yk_langevin_step_learned: flexible preconditioned CG with the
    trained network (8 hidden channels; 4 layers as specified, and 2), trained
    on the GPU on (residual, error) pairs from the chain's own CG at that
    field.  Wall clock around all the steps of an arm (the learned step is
    host-driven), no L2 flush (the working set, ~40 MB, lives in L2 in every
    arm)."""
    def params(prec):
        return yk.Params.default(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=0.5, fermion_mass=m0,
                                 wilson_param=1.0, cut_fraction=CUT, Nt=L, Nx=L, fixed_dt=0.01, precision=prec,
                                 cg_tol=1e-10, cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=50000, reliable_every=50,
                                 reliable_delta=0.001, n_rhs=1, seed=1234, init=yk.YK_INIT_PHILOX)

    def wall(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, r

    out = {"config": f"{L}x{L}, m0 {m0}, g 0.5, m2 -0.5, lambda 1, 1 RHS, rel-res 1e-10 (FP64 true residual), "
                     f"{steps} steps from a field burnt in for {burn_in} mixed steps", "steps": steps}
    ctx = yk.Context(params(yk.YK_MIXED))
    ctx.set_stream(stream.cuda_stream)
    ctx.step(burn_in)
    phi0, step0 = ctx.get_field(), ctx.get_step()
    arms = {}
    for name, prec in (("plain_fp64", yk.YK_FP64), ("mixed_cg", yk.YK_MIXED)):
        c = yk.Context(params(prec))
        c.set_stream(stream.cuda_stream)
        c.set_field(phi0)
        c.set_step(step0)
        c.step(1)   # capture the step graph
        c.set_field(phi0)
        c.set_step(step0)
        before = c.observables().cg_iterations_total
        sec, _ = wall(lambda: c.step(steps))
        o = c.observables()
        arms[name] = {"value": round(steps / sec, 2), "unit": "steps/s",
                      "cg_iterations_per_step": round((o.cg_iterations_total - before) / steps, 1),
                      "status": int(o.status)}
        c.close()
    for nl in layer_counts:
        ctx.set_field(phi0)
        ctx.set_step(step0)
        ctx.net_setup(nl, 7)
        st = ctx.net_train(n_sources=4, n_levels=5, base_iter=4, steps=400, batch=4, lr=2e-3, seed=3)
        ctx.set_field(phi0)
        ctx.set_step(step0)
        ctx.step_learned(1)   # capture the solver's chunk graph
        ctx.set_field(phi0)
        ctx.set_step(step0)
        sec, s = wall(lambda: ctx.step_learned(steps))
        tile = ctx.tune_report()
        arms[f"learned_{nl}layers"] = {
            "value": round(steps / sec, 2), "unit": "steps/s",
            "solver_iterations_per_step": round(s.iterations / steps, 1),
            "refinement_rounds_per_step": round(s.reliable_updates / steps, 2),
            "all_converged": bool(s.converged),
            "conv_tile_rows_cols": [tile.conv_rows, tile.conv_cols],
            "conv_layers_per_launch": tile.conv_layers_per_launch,
            "pcg_inner_tol": tile.pcg_inner_tol,
            "training": {"pairs": st.pairs, "loss_before": round(st.loss0, 4), "loss_after": round(st.loss1, 4),
                         "ms": round(st.ms, 1)},
            "speedup_over_plain_fp64": round((steps / sec) / arms["plain_fp64"]["value"], 3),
            "speedup_over_mixed_cg": round((steps / sec) / arms["mixed_cg"]["value"], 3),
            # the configuration's 5000 steps with this training's time spread over them
            "value_incl_training_over_5000_steps": round(5000 / (5000 / (steps / sec) + st.ms / 1e3), 2)}
    ctx.close()
    out.update(arms)
    return out


def dirac_hbm(yk, torch, stream, Nt=4096, Nx=4096, reps=20):
    out = {}
    pk = peaks()["hbm_gbs"]
    p = make_params(yk, "fp64", Nt=Nt, Nx=Nx).copy(cut_fraction=1.0, yukawa_coupling=0.0)
    ctx = yk.Context(p)
    ctx.set_stream(stream.cuda_stream)
    V = Nt * Nx
    for prec, dt, bps in (("fp64", torch.complex128, 136), ("fp32", torch.complex64, 72)):
        x = torch.randn(V, 4, dtype=dt, device="cuda")
        y = torch.empty_like(x)
        code = yk.YK_FP64 if prec == "fp64" else yk.YK_FP32
        with torch.cuda.stream(stream):
            for _ in range(3):
                ctx.dirac_apply(x, y, False, code)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                ctx.dirac_apply(x, y, False, code)
            b.record(stream)
        stream.synchronize()
        ms = a.elapsed_time(b) / reps
        gbs = V * bps / (ms * 1e-3) / 1e9
        out[prec] = {"lattice": [Nt, Nx], "bytes_per_site": bps, "ms": round(ms, 4), "GB/s": round(gbs, 1),
                     "frac": round(gbs / pk, 4)}
        del x, y
    ctx.close()
    return out


# ---------------------------------------------------------------- CPU arms
def cpu_steps(seconds_budget: float, max_steps: int, warmup: int):
    """Times full 256x256 Langevin steps of the CPU oracle (all host threads)
    on the segment the GPU arm times: `warmup` untimed steps from the
    thermalised start field, then up to `max_steps` steps within the budget."""
    from oracle import oracle as O
    a = O.action(m2=-0.5, lam=1.0, g=0.5, m0=0.1, r=1.0, cut_fraction=CUT)
    phi, step0 = start_field()

    def one(phi, s):
        return O.langevin_step(NT, NX, a, phi, 1234, 0, step0 + s, tol=1e-10, tol_mode=1, max_iter=20000,
                               fixed_dt=0.01)[0]

    for s in range(warmup):
        phi = one(phi, s)
    t0 = time.perf_counter()
    n = 0
    while n < max_steps and (n == 0 or time.perf_counter() - t0 < seconds_budget):
        phi = one(phi, warmup + n)
        n += 1
    dt = time.perf_counter() - t0
    return n, dt, O.threads()


def cpu_baseline(seconds: float, warmup: int) -> dict:
    n, dt, threads = cpu_steps(seconds, 10_000, warmup)
    return {"value": round(n / dt, 4), "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{n} full {NT}x{NX} Langevin steps from the thermalised start field after {warmup} warm-up "
                      f"steps (FP64 CG rel-res 1e-10, OpenMP over sites)"}


def reference_gpu(steps=20) -> dict:
    """The reference's own CUDA kernels on this GPU at the workload's lattice
    (oracle/ref/time_ref.py: its Dirac apply, CG solve and full Langevin steps,
    launched and synchronised as the reference does, from the thermalised
    start field, with the reference's compile-time CG stop |r| <= 1e-8 and its
    adaptive step).  Reported beside the CPU arm; not the arm's value."""
    try:
        from oracle.ref import time_ref
        return time_ref.time_size(NT, NX, steps)
    except Exception as e:   # the harness needs the fatbins built from the reference's sources
        return {"unavailable": f"{type(e).__name__}: {e}"[:300]}


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    budget = float(os.environ.get("YK_REF_SECONDS", "120"))
    n, dt, threads = cpu_steps(budget, args.steps, args.warmup)
    v = n / dt
    rg = reference_gpu() if not args.no_reference_gpu else {"skipped": "--no-reference-gpu"}
    return {"metric": METRIC, "value": round(v, 4), "unit": "steps/s", "n_gpus": ws, "steps": n,
            "warmup": args.warmup, "ms_per_step": round(dt / n * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": DATA, "config": workload(args.precision),
            "cpu_baseline": {"value": round(v, 4), "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": f"{n} of {args.steps} requested {NT}x{NX} Langevin steps in FP64 from the "
                                       f"thermalised start field after {args.warmup} warm-up steps (the segment "
                                       f"the GPU arm times; CPU restatement of the reference, which has no CPU "
                                       f"path)"},
            "e2e": {"value": round(v, 4), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_gpu": rg}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--profile-steps", type=int, default=100)
    ap.add_argument("--e2e-steps", type=int, default=300)
    ap.add_argument("--fp64-steps", type=int, default=None, help="default: --steps")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner configuration")
    ap.add_argument("--quick", action="store_true", help="timed region only")
    ap.add_argument("--learned-only", action="store_true",
                    help="only the learned-preconditioner configuration (one JSON object; profiling runs)")
    ap.add_argument("--learned-steps", type=int, default=20)
    ap.add_argument("--full-scale", action="store_true",
                    help="only the full form at scale (8 chains of 1024^2, 8 RHS; one JSON object; minutes)")
    ap.add_argument("--no-full-scale", action="store_true", help="skip the full form at scale in the default run")
    ap.add_argument("--steps-only", type=int, default=0, metavar="L",
                    help="only --steps mixed Langevin steps of an L x L lattice after --warmup (the workload's "
                         "couplings, uniform start; one JSON object; profiling runs)")
    ap.add_argument("--dirac-only", type=int, default=0, metavar="L",
                    help="only the Dirac apply on an L x L lattice (one JSON object; profiling runs)")
    ap.add_argument("--batching-only", action="store_true",
                    help="only the batching configuration (one JSON object; profiling runs)")
    ap.add_argument("--batch-case", default="", metavar="L,CHAINS,RHS,STEPS",
                    help="only STEPS steps of CHAINS chains of L x L with RHS right-hand sides, the batching "
                         "configuration's couplings, autotuner off (one JSON object; profiling runs)")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="reference arm: skip timing the reference's own CUDA kernels on the GPU")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.full_scale:
        import torch
        import yukawacolourednoise_gb300 as yk
        stream = torch.cuda.Stream()
        print(json.dumps({"full_scale": full_scale(yk, torch, stream)}), flush=True)
        return 0
    if args.steps_only:
        import torch
        import yukawacolourednoise_gb300 as yk
        L = args.steps_only
        stream = torch.cuda.Stream()
        with yk.Context(make_params(yk, args.precision, Nt=L, Nx=L)) as ctx:
            ctx.set_stream(stream.cuda_stream)
            ctx.step(args.warmup)
            ctx.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
                ctx.step(args.steps)
                b.record(stream)
            stream.synchronize()
            o = ctx.observables()
            print(json.dumps({"steps_only": {"lattice": [L, L], "steps": args.steps,
                                             "ms_per_step": round(a.elapsed_time(b) / args.steps, 4),
                                             "cg_iterations_last_step": o.cg_iterations, "status": o.status}}),
                  flush=True)
        return 0
    if args.dirac_only:
        import torch
        import yukawacolourednoise_gb300 as yk
        stream = torch.cuda.Stream()
        L = args.dirac_only
        print(json.dumps({"dirac_hbm": dirac_hbm(yk, torch, stream, Nt=L, Nx=L)}), flush=True)
        return 0
    if args.batch_case:
        import numpy as np
        import os as _os
        _os.environ["YK_AUTOTUNE"] = "0"
        import yukawacolourednoise_gb300 as yk
        L, nch, nrhs, nsteps = (int(v) for v in args.batch_case.split(","))
        rng = np.random.default_rng(1234)
        ps = [yk.Params.default(use_mass=1, mass=-0.5, g=1.0, yukawa_coupling=float(rng.uniform(0.3, 0.8)),
                                fermion_mass=float(rng.uniform(0.05, 0.3)), wilson_param=1.0, cut_fraction=CUT,
                                Nt=L, Nx=L, fixed_dt=0.01, precision=yk.YK_MIXED, cg_tol=1e-10,
                                cg_tol_mode=yk.YK_TOL_REL, cg_max_iter=20000, reliable_every=50, reliable_delta=0.001,
                                n_rhs=nrhs, seed=1234, init=yk.YK_INIT_PHILOX) for _ in range(nch)]
        with yk.Context(ps) as ctx:
            ctx.step(nsteps)
            ctx.synchronize()
            obs = [ctx.observables(c) for c in range(nch)]
        print(json.dumps({"batch_case": {"lattice": [L, L], "chains": nch, "rhs": nrhs, "steps": nsteps,
                                         "cg_iterations_last_step": [o.cg_iterations for o in obs],
                                         "status": [o.status for o in obs]}}), flush=True)
        return 0
    if args.batching_only:
        import torch
        import yukawacolourednoise_gb300 as yk
        stream = torch.cuda.Stream()
        print(json.dumps({"batching": batched(yk, torch, stream)}), flush=True)
        return 0
    if args.learned_only:
        import torch
        import yukawacolourednoise_gb300 as yk
        stream = torch.cuda.Stream()
        print(json.dumps({"learned": learned(yk, torch, stream, steps=args.learned_steps)}), flush=True)
        return 0
    ws, rank, local = dist_env()
    line = run_reference(args, ws, rank) if args.impl == "reference" else run_ours(args, ws, rank, local)
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
