#!/usr/bin/env python
"""Benchmark of the per-substep incremental-potential solve.

Workload: the body scene -- 6,757 strands / 265,108 internal nodes /
258,351 elements on a 225,184-vertex swaying head + torso collider
(scenes.body_scene), 8 base substeps per frame, adaptive doubling up to 64.
A step is one animation frame (khsStepAnimationFrame) with every frame's
root targets and collider vertices already resident in HBM; the metric is
substeps per second.

Prints ONE JSON line (rank 0).  Keys beyond the base contract:
* roofline     -- the dominant kernel's FP64-pipe roofline: executed FP64
                  flops per launch (per-element count measured once with ncu,
                  see profiles/) / its CUDA-event duration measured live in
                  the timed region, against the FMA-pipe peak measured by the
                  library's probe on this GPU; traffic from the ncu capture.
* cpu_baseline -- the CPU oracle (a port of the reference method; the
                  reference has no CPU solver) on this host's cores, on a
                  bounded sample of the same workload.
* e2e          -- the same metric through the public C ABI with host
                  buffers: khsUpdateRootTargets + khsUpdateColliderVertices
                  (pinned host arrays) + khsStep + khsCopyOriginalPositions
                  every step, wall clock.
* clocks       -- nvidia-smi samples taken during the timed region.

``--impl reference`` times the CPU oracle (the reference method restated;
the reference ships no CPU implementation and its CUDA sources do not travel
to this machine) on all host threads, each step one substep of the same
workload.  ``--gpus N`` under torchrun runs N independent replicas (the solve
does not exchange data between strands' GPUs): weak scaling.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
PACKAGE = REPO / "kami-hair-solver_gb300"
sys.path.insert(0, str(PACKAGE))

# One process per GPU: pin the rank's device before any CUDA initialisation.
if int(os.environ.get("WORLD_SIZE", "1")) > 1 and "LOCAL_RANK" in os.environ:
    os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]

import numpy as np  # noqa: E402

METRIC = "substeps/s at 265k nodes, mixed+batched vs plain FP64 on 1 GB300 @≤1e-6 m; p99 latency"
UNIT = "substeps/s"

# Executed FP64 flops per element of the dominant kernel, measured once with
# ncu (smsp__sass_thread_inst_executed_op_{dfma,dmul,dadd}) on the body
# scene; see profiles/.  None until measured.
FP64_FLOPS_PER_ELEMENT = {"k_elem_eval_grad": None, "k_block_solve": None}
DRAM_BYTES_PER_ELEMENT = {"k_elem_eval_grad": None, "k_block_solve": None}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return world, rank


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=lambda: self.lines.extend(iter(self.proc.stdout.readline, "")), daemon=True)
        self.thread.start()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _flush_l2(torch, buf):
    buf.add_(1.0)
    torch.cuda.synchronize()


def cpu_oracle_sample(scene, substeps: int, threads: int | None = None) -> dict:
    """Times the CPU oracle on the first ``substeps`` substeps of frame 1."""
    import khs_native as kn
    import scenes

    subprocess.run(["make", "-s", "-C", str(REPO / "oracle")], check=True)
    lib = kn.Library(REPO / "oracle" / "_build" / "libkhs_oracle.so")
    lib.lib.khsOracleSetThreads.restype = ctypes.c_int
    cores = int(lib.lib.khsOracleSetThreads(ctypes.c_int(threads or os.cpu_count() or 1)))
    lib.lib.khsOracleSetSubstepLimit(ctypes.c_uint32(substeps))
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, frames=2)
    t0 = time.perf_counter()
    r = s._library.khsStepAnimationFrame(s.handle, 1, scene.frame_dt)
    dt = time.perf_counter() - t0
    s.close()
    lib.lib.khsOracleSetSubstepLimit(ctypes.c_uint32(0))
    return {"value": substeps / dt, "unit": UNIT, "cores": cores, "kind": "port", "result": int(r),
            "sample": f"first {substeps} substep(s) of frame 1 of the same body scene, oracle on {cores} threads",
            "seconds": dt}


def run_reference(args) -> None:
    world, rank = _dist()
    if rank != 0:
        return
    import khs_native as kn
    import scenes

    subprocess.run(["make", "-s", "-C", str(REPO / "oracle")], check=True)
    lib = kn.Library(REPO / "oracle" / "_build" / "libkhs_oracle.so")
    lib.lib.khsOracleSetThreads.restype = ctypes.c_int
    cores = int(lib.lib.khsOracleSetThreads(ctypes.c_int(os.cpu_count() or 1)))
    lib.lib.khsOracleSetSubstepLimit(ctypes.c_uint32(1))
    scene = scenes.body_scene(frames=args.warmup + args.steps + 1)
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene)
    for f in range(1, args.warmup + 1):
        s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt)
    t0 = time.perf_counter()
    for f in range(args.warmup + 1, args.warmup + args.steps + 1):
        s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt)
    dt = time.perf_counter() - t0
    s.close()
    value = args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded body scene)",
        "config": _config(scene, "reference-cpu-oracle"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "each step = first substep of one frame of the body scene (CPU FP64 oracle, "
                                   "the reference method restated; the reference has no CPU solver)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _config(scene, mode: str) -> dict:
    return {"workload": "body scene: 6,757 strands / 265,108 nodes / 258,351 elements, 225,184-vertex swaying "
                        "head+torso collider, 8 base substeps (adaptive <= 64) per frame",
            "strands": int(scene.strands), "points": int(len(scene.points)),
            "collider_vertices": int(len(scene.vertices)), "collider_triangles": int(len(scene.triangles)),
            "substeps_base": int(scene.desc["substeps"]), "max_substeps": int(scene.desc["maximum_substeps"]),
            "mode": mode, "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"}


def run_ours(args) -> None:
    world, rank = _dist()
    import torch

    import khs_build
    import khs_native as kn
    import scenes

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(0)
    lib_path = khs_build.build()
    lib = kn.Library(lib_path)
    fp64_peak, fp32_peak = ctypes.c_double(), ctypes.c_double()
    lib.khsxMeasurePipePeaks(ctypes.byref(fp64_peak), ctypes.byref(fp32_peak))
    mode = {"plain": kn.MODE_PLAIN_FP64, "mixed": kn.MODE_MIXED}[args.mode]
    frames = args.warmup + args.steps + 1
    scene = scenes.body_scene(frames=frames)
    solver = kn.HairSolver(lib)
    scenes.load_into(solver, scene)
    solver.set_solve_mode(mode)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for f in range(1, args.warmup + 1):
        solver.step_animation_frame(f, scene.frame_dt)
    solver.set_profiling(True)
    solver.reset_kernel_timings()
    launches0 = solver.kernel_launches()
    clocks = ClockSampler()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    frame_ms, substeps, wall0 = [], 0, time.perf_counter()
    for f in range(args.warmup + 1, frames):
        _flush_l2(torch, flush)
        r = solver._library.khsStepAnimationFrame(solver.handle, f, scene.frame_dt)
        if r != kn.OK:
            raise RuntimeError(f"frame {f} failed ({r}): {solver.last_error()}")
        frame_ms.append(solver.gpu_stats().last_frame_milliseconds)
        substeps += solver.stats().substeps
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clock_info = clocks.stop()
    launches = solver.kernel_launches() - launches0
    timings = solver.kernel_timings()
    solver.set_profiling(False)
    device_s = sum(frame_ms) / 1e3
    t = torch.tensor([device_s], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    device_s = float(t.item())
    value = world * substeps / device_s
    solver.close()

    # End to end through the public API with host buffers.
    e2e = run_e2e(lib, scene, args, torch) if not args.skip_e2e else None

    # Roofline of the dominant kernel.
    total = sum(ms for _, ms in timings.values()) or 1.0
    top = max(timings.items(), key=lambda kv: kv[1][1]) if timings else ("none", (0, 0.0))
    name, (count, ms) = top
    E = 258351
    per_launch_s = (ms / max(count, 1)) / 1e3
    flops_el = FP64_FLOPS_PER_ELEMENT.get(name)
    bytes_el = DRAM_BYTES_PER_ELEMENT.get(name)
    achieved = (flops_el * E / per_launch_s / 1e12) if (flops_el and per_launch_s > 0) else None
    roofline = {"bound": "fp64", "kernel": name, "achieved": achieved, "peak": fp64_peak.value, "unit": "TFLOP/s",
                "frac": (achieved / fp64_peak.value) if achieved else None,
                "traffic": (bytes_el * E) if bytes_el else None,
                "peak_source": "measured FP64 FMA-pipe rate of this GPU (khsxMeasurePipePeaks)",
                "avg_launch_ms": ms / max(count, 1), "launches": count, "share": ms / total,
                "kernel_shares": {k: round(v[1] / total, 4) for k, v in sorted(timings.items(), key=lambda kv: -kv[1][1])}}
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = cpu_oracle_sample(scenes.body_scene(frames=2), substeps=args.cpu_substeps)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * device_s / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.mode == "plain" else "f64+f32",
            "data": "synthetic (seeded body scene, see kami-hair-solver_gb300/scenes.py)",
            "config": _config(scene, args.mode), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clock_info, "gpu_launches": int(launches), "wall_s": wall, "substeps": substeps,
            "fp32_pipe_peak_tflops": fp32_peak.value,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_e2e(lib, scene, args, torch) -> dict:
    import khs_native as kn
    import scenes

    s = kn.HairSolver(lib)
    scenes.apply_settings(s, scene)
    s.create()
    s.set_hair(scene.points, scene.offsets)
    s.set_collider(scene.vertices, scene.triangles)
    s.build()
    mode = {"plain": kn.MODE_PLAIN_FP64, "mixed": kn.MODE_MIXED}[args.mode]
    s.set_solve_mode(mode)
    P, V = len(scene.points), len(scene.vertices)
    # Pinned host staging for the per-step inputs and output.
    roots = torch.empty((P, 3), dtype=torch.float64, pin_memory=True)
    verts = torch.empty((V, 3), dtype=torch.float64, pin_memory=True)
    out = torch.empty((P, 3), dtype=torch.float64, pin_memory=True)
    frames = args.warmup + args.steps + 1
    host_roots = [scene.root_points_at(f) for f in range(frames)]
    host_verts = [scene.collider_at(f) for f in range(frames)]

    def one(f):
        roots.numpy()[:] = host_roots[f]
        verts.numpy()[:] = host_verts[f]
        lib.khsUpdateRootTargets(s.handle, ctypes.c_void_p(roots.data_ptr()), P)
        lib.khsUpdateColliderVertices(s.handle, ctypes.c_void_p(verts.data_ptr()), V)
        r = lib.khsStep(s.handle, scene.frame_dt)
        if r != kn.OK:
            raise RuntimeError(f"e2e frame {f}: {s.last_error()}")
        lib.khsCopyOriginalPositions(s.handle, ctypes.c_void_p(out.data_ptr()), P)
        return s.stats().substeps

    for f in range(1, args.warmup + 1):
        one(f)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sub = 0
    for f in range(args.warmup + 1, frames):
        sub += one(f)
    dt = time.perf_counter() - t0
    s.close()
    N = 265108
    return {"value": sub / dt, "unit": UNIT, "h2d_bytes_per_step": P * 24 + 2 * N * 24 + V * 24,
            "d2h_bytes_per_step": P * 24, "note": "root targets are converted to node positions + rotation vectors "
            "on the host (2 x N x 24 B uploaded) as the reference API does"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["plain", "mixed"], default="plain")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--cpu-substeps", type=int, default=1)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
