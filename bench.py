#!/usr/bin/env python
"""Throughput of the plain 3D smoke step on GB300 (cell-steps/s).

One step = one full timestep (force+attenuation, velocity advection, red-black
SOR projection, scalar advection+reinjection) of a device-resident grid,
replayed as a CUDA graph.  Default workload: plain256 (256^3, four seeded
sphere sources, K=600, omega 1.9, 20 backtrace substeps).

Prints one JSON line (rank 0).  --impl reference times the CPU path (the FP32
oracle restatement of the reference's step, all host threads) instead.
Multi-GPU: a single grid does not shard, so N ranks run N independent
replicas ("replicas only"); value = all ranks' cell-steps / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-steps/s on 1 GB300: batched vs plain (rel err ≤1e-4); adjoint/fwd time ratio"
UNIT = "Gcell-steps/s"
SOR_BYTES_PER_CELL_ITER = 13      # read p, div (4+4), flags (1), write p (4)
STEP_BYTES_FIXED = 133            # the non-SOR stages of the algorithmic model


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="plain256")
    ap.add_argument("--sor-depth", type=int, default=0, help="SOR iterations per fused pass (0 = default)")
    ap.add_argument("--sor-variant", type=int, default=-1, help="fused SOR kernel variant (-1 = default)")
    ap.add_argument("--zchunk", type=int, default=0, help="z planes per SOR CTA (0 = automatic)")
    ap.add_argument("--cpu-sample", default="",
                    help="workload of the CPU sample ('' = the bench workload itself, one full step per sample)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--batch", default="batch64", help="mixed-size batch measured beside the plain step ('' or none = skip)")
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--batch-variant", type=int, default=-1)
    ap.add_argument("--batch-zchunk", type=int, default=0)
    ap.add_argument("--adjoint", default="64,128", help="control-problem sizes timed for the reverse mode ('' or none = skip)")
    ap.add_argument("--adjoint-steps", type=int, default=64)
    ap.add_argument("--checkpoint-every", type=int, default=8)
    ap.add_argument("--coarse", default="coarse256",
                    help="coarse-grid projection configuration measured beside the plain step ('' or none = skip)")
    ap.add_argument("--coarse-steps", type=int, default=5)
    ap.add_argument("--large", default="plain512",
                    help="single-grid configuration measured beside the headline ('' or none = skip)")
    ap.add_argument("--large-steps", type=int, default=3)
    ap.add_argument("--render", default="256:1024x768x300",
                    help="headless ray march N:WxHxSTEPS of an N^3 density in the viewer's default view "
                         "('' or none = skip)")
    return ap.parse_args()


def replicas_value(ms_local: float, world: int, cells: int, steps: int, dist=None, device="cuda"):
    """Replicas only (a grid does not shard): every rank steps its own grid; the
    job's time is the slowest rank's (max over ranks) and the value is all
    ranks' cell-steps over that time.  Returns (ms, Gcell-steps/s)."""
    ms = float(ms_local)
    if dist is not None:
        import torch
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * cells * steps / (ms * 1e-3) / 1e9


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name: str, variant: int):
    """DRAM bytes per launch of the SOR kernel from the committed ncu summary:
    the `sor_variant: N` / `traffic_bytes_per_launch: X` pair of the variant
    that ran (None when that variant was not captured)."""
    f = ROOT / "profiles" / f"{name}.md"
    if not f.exists():
        return None
    pairs = re.findall(r"sor_variant:\s*(-?[0-9]+)\s*\n\s*traffic_bytes_per_launch:\s*([0-9.eE+]+)",
                       f.read_text())
    for v, t in pairs:
        if int(v) == variant:
            return float(t)
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nme, val in zip(names, r[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nme)
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


class CpuRun:
    """The FP32 oracle (the CPU restatement of the reference's step) stepping
    the bench's own configuration on all host threads.  The state persists
    across samples, as the GPU grid's does; each sample is one full step."""

    def __init__(self, args, workload: str):
        import numpy as np

        from oracle.binding import Oracle, num_threads
        from zq_smokesimulation_gb300 import workloads as wl
        self.w = wl.make(args.cpu_sample or workload)
        self.o = Oracle(np.float32)
        self.st = self.o.state(self.w)
        self.cores = num_threads()

    def step_seconds(self) -> float:
        w = self.w
        t0 = time.perf_counter()
        rc, _ = self.o.step(w.W, w.H, w.D, self.st, w.occ, w.params, 1)
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(f"oracle step failed: {rc}")
        return dt

    def describe(self, steps: int) -> dict:
        w = self.w
        return {"cores": self.cores, "cpu_model": cpu_model(), "kind": "port", "grid": [w.W, w.H, w.D],
                "sample": f"{steps} full step(s) of {w.name} ({w.W}x{w.H}x{w.D}, K={w.params.sor_iters}), "
                          f"FP32 oracle, state carried across steps"}


def run_reference(args):
    """Reference arm: the CPU path of the step (FP32 oracle port) on the bench's
    own configuration, rank 0 only; one full step per timed step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    run = CpuRun(args, args.workload)
    w = run.w
    for _ in range(max(0, args.warmup)):
        run.step_seconds()
    secs = [run.step_seconds() for _ in range(max(1, args.steps))]
    total = sum(secs)
    value = w.cells * len(secs) / total / 1e9
    cpu = {"value": value, "unit": UNIT}
    cpu.update(run.describe(len(secs)))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": len(secs), "warmup": args.warmup, "ms_per_step": 1000.0 * total / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "grid": [w.W, w.H, w.D],
                       "sor_iters": int(w.params.sor_iters), "omega": round(float(w.params.omega), 6),
                       "substeps": int(w.params.substeps), "advection": "inMAC_outMAC + MAC scalar",
                       "parallelism": "single"},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure_batch(args, stream, rel_check: bool = True):
    """The mixed-size batch: batched step (one persistent launch per stage,
    one CUDA graph) against the same instances stepped one at a time
    (zqs_grid_step per instance, each a CUDA graph of its own)."""
    import numpy as np
    import torch

    from zq_smokesimulation_gb300 import capi
    from zq_smokesimulation_gb300 import workloads as wl

    n = int(args.batch[5:]) if args.batch.startswith("batch") and args.batch[5:].isdigit() else 64
    cases = wl.batch_mixed(n)
    sp = stream.cuda_stream
    cells = sum(w.cells for w in cases)
    K = cases[0].params.sor_iters

    def grids():
        out = []
        for w in cases:
            g = capi.Grid(w.W, w.H, w.D)
            g.set_params(w.params)
            g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
            out.append(g)
        return out

    def timed(fn, steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    gb = grids()
    batch = capi.Batch(gb)
    batch.set_sor_variant(args.batch_variant, args.batch_zchunk)
    batch.step(max(3, args.warmup), sp)
    steps = max(1, args.batch_steps)
    ms_b = timed(lambda: batch.step(1, sp), steps)
    launches = batch.launch_count()
    b_variant, b_us = batch.sor_choice()
    batch.sync(sp)

    gs = grids()
    for g in gs:
        g.step(max(3, args.warmup), sp)
    steps1 = max(1, min(steps, 5))
    ms_1 = timed(lambda: [g.step(1, sp) for g in gs], steps1)
    launches_1 = sum(g.launch_count() for g in gs)
    torch.cuda.synchronize()
    # both ran warmup + a different number of timed steps: compare members after
    # bringing the one-at-a-time set to the same step count
    extra = steps - steps1
    for g in gs:
        g.step(extra, sp)
    torch.cuda.synchronize()
    worst = 0.0
    mism = 0
    if rel_check:
        for ga, gb_ in zip(gs, gb):
            for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_W, capi.FIELD_DENSITY):
                x, y = ga.download(f), gb_.download(f)
                den = float(np.linalg.norm(x.astype(np.float64)))
                err = float(np.linalg.norm((x.astype(np.float64) - y))) / den if den > 0 else 0.0
                worst = max(worst, err)
                mism += int(np.count_nonzero(x != y))
    batch.close()
    for g in gb + gs:
        g.close()
    v_b = cells * steps / (ms_b * 1e-3) / 1e9
    v_1 = cells * steps1 / (ms_1 * 1e-3) / 1e9
    step_alg = (STEP_BYTES_FIXED + SOR_BYTES_PER_CELL_ITER * K) * cells
    return {"workload": args.batch, "instances": n, "cells": cells, "sor_iters": K, "steps": steps,
            "value": v_b, "unit": UNIT, "ms_per_step": ms_b / steps, "gpu_launches_per_step": launches,
            "one_at_a_time": {"value": v_1, "ms_per_step": ms_1 / steps1, "steps": steps1,
                              "gpu_launches_per_step": launches_1},
            "speedup": v_b / v_1, "max_rel_l2_vs_one_at_a_time": worst, "mismatched_values": mism,
            "sor_variant": b_variant, "sor_tuned_us_per_iter": b_us,
            "step_alg_gbs": step_alg / (ms_b / steps * 1e-3) / 1e9}


def measure_coarse(args, stream):
    """The reference's fine256 configuration: COARSE_OPEN_POISSON_SOR with
    subSize 8 (coarse face-ratio SOR, K iterations on the 32^3 grid, then the
    block sub-projection), regular-grid advection, the centred sphere obstacle.
    Full steps through the same C ABI, device-resident, graph-replayed."""
    import torch

    from zq_smokesimulation_gb300 import capi
    from zq_smokesimulation_gb300 import workloads as wl

    w = wl.make(args.coarse)
    sp = stream.cuda_stream
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    g.step(max(3, args.warmup), sp)
    steps = max(1, args.coarse_steps)

    def timed(fn, reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / reps

    ms = timed(lambda: g.step(1, sp), steps)
    launches = g.launch_count()
    g.project(sp)
    ms_proj = timed(lambda: g.project(sp), 3)
    mx = g.stats().max_abs_div
    # the same projection with the obstacle-free blocks on the FP32 SIMT path
    g.set_coarse_gemm(0)
    g.project(sp)
    ms_proj_simt = timed(lambda: g.project(sp), 3)
    g.set_coarse_gemm(1)
    g.sync(sp)
    g.close()
    return {"workload": args.coarse, "grid": [w.W, w.H, w.D], "sub_size": int(w.params.sub_size),
            "coarse_grid": [w.W // w.params.sub_size] * 3, "sor_iters": int(w.params.sor_iters),
            "advection": "inReg_outReg + Reg scalar", "steps": steps, "ms_per_step": ms,
            "value": w.cells / (ms * 1e-3) / 1e9, "unit": UNIT, "gpu_launches_per_step": launches,
            "projection_ms": ms_proj, "max_abs_div_after_projection": mx,
            "block_product": "tcgen05 TF32, 3xTF32 split (zqs_grid_set_coarse_gemm 1)",
            "projection_ms_fp32_simt_blocks": ms_proj_simt}


def measure_large(args, stream):
    """The large single grid of the same configuration (plain512: 512^3, K=600,
    four seeded sphere sources): full steps, device-resident, graph-replayed,
    and the step's algorithmic-byte rate against the HBM peak."""
    import torch

    from zq_smokesimulation_gb300 import capi
    from zq_smokesimulation_gb300 import workloads as wl

    w = wl.make(args.large)
    sp = stream.cuda_stream
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    g.step(2, sp)
    steps = max(1, args.large_steps)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    g.step(steps, sp)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    g.project(sp)
    st = g.stats()
    lay = g.layout()
    K = int(w.params.sor_iters)
    peak, peak_kind = load_peaks()
    step_alg = (STEP_BYTES_FIXED + SOR_BYTES_PER_CELL_ITER * K) * w.cells
    out = {"workload": args.large, "grid": [w.W, w.H, w.D], "sor_iters": K, "steps": steps, "ms_per_step": ms,
           "value": w.cells / (ms * 1e-3) / 1e9, "unit": UNIT, "gpu_launches_per_step": g.launch_count(),
           "step_alg_gbs": step_alg / (ms * 1e-3) / 1e9, "step_frac": step_alg / (ms * 1e-3) / 1e9 / peak,
           "peak_kind": peak_kind, "max_abs_div_after_projection": st.max_abs_div,
           "working_set_gb": lay.field_elems * 4 * 21.25 / 1e9}
    g.close()
    return out


def measure_render(args, stream):
    """The viewer's volume shader as k_raymarch: an N^3 density (seeded uniform
    values; the cost does not depend on them) in the default view, one launch
    per frame, timed with CUDA events; the FP32 oracle on the host cores renders
    the same view at a quarter of the resolution in each direction for the CPU
    rate.  Samples = hit rays x steps; each sample reads 8 texels."""
    import time

    import numpy as np
    import torch

    from zq_smokesimulation_gb300 import capi

    n_s, rest = args.render.split(":")
    N = int(n_s)
    iw, ih, steps = (int(x) for x in rest.split("x"))
    gen = torch.Generator(device="cuda").manual_seed(11)
    vol = torch.rand((N, N, N), generator=gen, device="cuda", dtype=torch.float32)
    cam = capi.default_camera(iw, ih, N, N, N)
    cam.steps = steps
    img = torch.empty((ih, iw, 4), dtype=torch.float32, device="cuda")
    sp = stream.cuda_stream
    for _ in range(3):
        capi.render_density(vol.data_ptr(), N, N, N, cam, img.data_ptr(), sp)
    reps = 10
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        capi.render_density(vol.data_ptr(), N, N, N, cam, img.data_ptr(), sp)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b) / reps
    # rays that met the box: alpha < 1 (the density is positive almost everywhere)
    hits = int((img[..., 3] < 1).sum().item())
    samples = hits * steps
    out = {"volume": [N, N, N], "image": [iw, ih], "steps": steps, "ms_per_frame": ms, "rays_hit": hits,
           "gsamples_per_s": samples / (ms * 1e-3) / 1e9,
           "texel_reads_gbs": samples * 8 * 4 / (ms * 1e-3) / 1e9,
           "hbm_alg_bytes": N ** 3 * 4 + iw * ih * 16,
           "note": "L1/L2-gather bound: the volume (%.0f MB) stays in the 129 MB L2" % (N ** 3 * 4 / 1e6)}
    if not args.no_cpu_baseline:
        from oracle.binding import Oracle, num_threads

        o = Oracle(np.float32)
        small = capi.default_camera(iw // 4, ih // 4, N, N, N)
        small.steps = steps
        small.focal = cam.focal / 4
        host = vol.cpu().numpy()
        t0 = time.perf_counter()
        ref = o.render(host, small)
        dt = time.perf_counter() - t0
        cs = int((ref[..., 3] < 1).sum()) * steps
        out["cpu_baseline"] = {"gsamples_per_s": cs / dt / 1e9, "cores": num_threads(), "kind": "port",
                               "sample": f"{iw // 4}x{ih // 4} image of the same view, {steps} steps, FP32 oracle"}
    return out


def measure_adjoint(args, stream, N: int):
    """The force-field control problem at N^3: forward (nsteps steps with the
    control force, checkpoints every k) and backward (recomputation + adjoint
    kernels) timed with CUDA events; device memory the problem holds."""
    import numpy as np
    import torch

    from zq_smokesimulation_gb300 import capi
    from zq_smokesimulation_gb300 import workloads as wl

    nsteps = args.adjoint_steps
    w, target = wl.control_problem(N, nsteps=nsteps)
    sp = stream.cuda_stream
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    adj = capi.Adjoint(g, nsteps, args.checkpoint_every)
    F = torch.zeros((3, N, N, N), device="cuda", dtype=torch.float32)
    tgt = torch.tensor(target, device="cuda")
    rho = torch.empty((N, N, N), device="cuda", dtype=torch.float32)
    grad = torch.empty_like(F)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def reset():
        for f, arr in ((capi.FIELD_U, w.u), (capi.FIELD_V, w.v), (capi.FIELD_W, w.w),
                       (capi.FIELD_TEMPERATURE, w.T), (capi.FIELD_DENSITY, w.rho)):
            g.upload(f, arr)

    fwd_ms, bwd_ms = [], []
    for rep in range(3):
        reset()
        torch.cuda.synchronize()
        a, b, c = ev(), ev(), ev()
        a.record(stream)
        adj.forward_device(F.data_ptr(), sp)
        b.record(stream)
        capi.check(g.lib.zqs_grid_download(g.h, capi.FIELD_DENSITY, capi.C.c_void_p(rho.data_ptr()), 1,
                                           capi.C.c_void_p(sp)), "download")
        gd = 2.0 * (rho - tgt)
        c0 = ev()
        c0.record(stream)
        adj.backward_device(gd.data_ptr(), grad.data_ptr(), sp)
        c.record(stream)
        c.synchronize()
        fwd_ms.append(a.elapsed_time(b))
        bwd_ms.append(c0.elapsed_time(c))
    free1 = torch.cuda.mem_get_info()[0]
    # plain forward of the same steps (graph replay, no checkpoint copies)
    reset()
    g.set_force_device(F.data_ptr(), sp)
    g.step(1, sp)
    torch.cuda.synchronize()
    a, b = ev(), ev()
    a.record(stream)
    g.step(nsteps, sp)
    b.record(stream)
    b.synchronize()
    plain_ms = a.elapsed_time(b)
    loss = float(((rho - tgt) ** 2).sum())
    inf = adj.info()
    out = {"grid": [N, N, N], "steps": nsteps, "checkpoint_every": args.checkpoint_every,
           "sor_iters": int(w.params.sor_iters), "substeps": int(w.params.substeps),
           "forward_ms": min(fwd_ms), "backward_ms": min(bwd_ms), "plain_forward_ms": plain_ms,
           "ratio_backward_to_forward": min(bwd_ms) / min(fwd_ms),
           "ratio_forward_plus_backward_to_forward": (min(fwd_ms) + min(bwd_ms)) / min(fwd_ms),
           "loss": loss, "grad_norm": float(grad.norm()),
           "session_bytes": int(inf.device_bytes), "device_bytes_used": int(free0 - free1),
           "launches_backward": int(inf.launches_backward)}
    adj.close()
    g.close()
    return out


def run_ours(args):
    import numpy as np
    import torch

    from zq_smokesimulation_gb300 import capi
    from zq_smokesimulation_gb300 import workloads as wl

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    w = wl.make(args.workload)
    K = w.params.sor_iters
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.set_sor_config(args.sor_depth, False)
    g.set_sor_variant(args.sor_variant, args.zchunk)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    # An explicit stream: the library treats a NULL stream as the grid's own
    # stream, so the events must sit on the stream the kernels run on.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp != 0
    cells = w.cells

    sampler = ClockSampler(local)
    sampler.start()
    g.step(max(3, args.warmup), sp)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.step(args.steps, sp)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    barrier()
    launches_per_step = g.launch_count()

    # -- dominant kernel (temporally blocked SOR): per-launch duration, live --
    sor_v, sor_zc, sor_us = g.sor_choice(sp)   # the variant the steps ran (tuned unless forced)
    vinfo = capi.sor_variants()[sor_v] if sor_v >= 0 else None
    depth = vinfo.depth if vinfo is not None else max(1, args.sor_depth)
    passes = math.ceil(2 * K / (2 * depth))
    reps = 3
    p0 = w.params.copy()
    p0.sor_iters = 0

    def time_project(params):
        g.set_params(params)
        g.project(sp)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            g.project(sp)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / reps

    t_K = time_project(w.params)
    t_0 = time_project(p0)
    g.set_params(w.params)
    g.project(sp)
    st_proj = g.stats()
    sor_ms_per_launch = max(1e-9, (t_K - t_0) / passes)
    alg_bytes = SOR_BYTES_PER_CELL_ITER * depth * cells
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (sor_ms_per_launch * 1e-3) / 1e9
    traffic = profile_traffic(f"k_sor_{args.workload}", sor_v)

    # -- end to end through the C ABI with pinned host buffers --
    e2e = None
    if not args.no_e2e:
        fields = [capi.FIELD_U, capi.FIELD_V, capi.FIELD_W, capi.FIELD_TEMPERATURE, capi.FIELD_DENSITY]
        host = {}
        for f in fields:
            n = int(np.prod(capi.field_shape(f, w.W, w.H, w.D)))
            host[f] = torch.empty(n, dtype=torch.float32, pin_memory=True)
            g.download_into(f, host[f].data_ptr(), sp)
        torch.cuda.synchronize()
        nbytes = sum(host[f].numel() * 4 for f in fields)
        e2e_steps = max(1, min(args.steps, 10))
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(e2e_steps):
            for f in fields:
                g.upload_from(f, host[f].data_ptr(), sp)
            g.step(1, sp)
            for f in fields:
                g.download_into(f, host[f].data_ptr(), sp)
        b.record(stream)
        b.synchronize()
        e2e_ms, e2e_value = replicas_value(a.elapsed_time(b), world, cells, e2e_steps, dist)
        e2e = {"value": e2e_value, "unit": UNIT,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "path": "zqs_grid_upload x5 (pinned host) + zqs_grid_step + zqs_grid_download x5"}
    batch = None
    if args.batch not in ("", "none") and world == 1:
        batch = measure_batch(args, stream)
    coarse = None
    if args.coarse not in ("", "none") and world == 1:
        coarse = measure_coarse(args, stream)
    large = None
    if args.large not in ("", "none") and world == 1:
        large = measure_large(args, stream)
    render = None
    if args.render not in ("", "none") and world == 1:
        render = measure_render(args, stream)
    adjoint = None
    if args.adjoint not in ("", "none") and world == 1:
        adjoint = {f"control{n}": measure_adjoint(args, stream, int(n)) for n in args.adjoint.split(",") if n}
    clocks = sampler.stop()

    ms, value = replicas_value(ms, world, cells, args.steps, dist)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        run = CpuRun(args, args.workload)
        secs = run.step_seconds()
        cpu = {"value": run.w.cells / secs / 1e9, "unit": UNIT}
        cpu.update(run.describe(1))

    if rank == 0:
        step_alg = (STEP_BYTES_FIXED + SOR_BYTES_PER_CELL_ITER * K) * cells
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "grid": [w.W, w.H, w.D], "sor_iters": K,
                       "omega": round(float(w.params.omega), 6), "substeps": int(w.params.substeps),
                       "advection": "inMAC_outMAC + MAC scalar", "sor_depth": depth, "graph": True,
                       "sor_variant": sor_v, "sor_zchunk": sor_zc, "sor_tuned_us_per_iter": sor_us,
                       "sor_kernel": (None if vinfo is None else
                                      f"{'k_sor_quad' if vinfo.x_cells_per_thread == 4 else ('k_sor_reg_split' if vinfo.split_barrier else 'k_sor_reg/rb')}"
                                      f"<depth {vinfo.depth}, {vinfo.tile_x}x{vinfo.tile_y}>"),
                       "l2": "working set %.2f GB > 129 MB L2, no flush" % (g.layout().field_elems * 4 * 21.25 / 1e9),
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "kernel": "fused red-black SOR pass", "achieved": achieved, "peak": peak,
                         "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "alg_bytes_per_launch": alg_bytes, "ms_per_launch": sor_ms_per_launch,
                         "step_alg_gbs": step_alg / (ms / args.steps * 1e-3) / 1e9,
                         "step_frac": step_alg / (ms / args.steps * 1e-3) / 1e9 / peak},
            "max_abs_div_after_projection": st_proj.max_abs_div, "residual_l2_after_projection": st_proj.residual_l2,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches_per_step * args.steps, "clocks": clocks,
            "batch": batch, "adjoint": adjoint, "coarse": coarse, "large": large, "render": render,
        }
        print(json.dumps(line), flush=True)
    g.close()
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
