#!/usr/bin/env python
"""Benchmark of the per-substep incremental-potential solve.

Workload: the body scene -- 6,757 strands / 265,108 internal nodes /
258,351 elements on a 225,184-vertex swaying head + torso collider
(scenes.body_scene), 8 base substeps per frame, adaptive doubling up to 64.
A step is one animation frame (khsStepAnimationFrame) with every frame's
root targets and collider vertices already resident in HBM; the metric is
substeps per second.

Prints ONE JSON line (rank 0).  ``value`` is the mixed form (FP32 filters,
results identical to the plain form); the plain FP64 form is timed on the
same frames and reported beside it as ``plain_fp64``.  Keys beyond the base
contract:
* roofline     -- the dominant kernel (largest share of device time in an
                  untimed re-run of the first timed frames with per-kernel
                  CUDA-event timing; the timed frames run without it):
                  algorithmic bytes per launch / average launch time against
                  the measured HBM copy bandwidth, and, where the kernel has
                  an algorithmic FP64 flop count, flops per launch against
                  the FMA-pipe rate measured on this GPU by
                  khsxMeasurePipePeaks; ``bound`` names the closer roof.
                  ``traffic`` is DRAM bytes per launch from the ncu capture
                  summarised under profiles/.
* host_gap     -- device time of those frames against the sum of their
                  kernels' times: the share the GPU waits on the host.
* cpu_baseline -- the CPU oracle (a port of the reference method; the
                  reference has no CPU solver) on this host's cores, on the
                  first substeps of the first timed frame from the timed
                  region's GB300 checkpoint.
* same_sample  -- both GB300 forms on exactly those substeps from the same
                  checkpoint: rate, and the maximum position and rotation
                  deviation from the oracle (also max_position_dev_m and
                  max_rotation_dev_rad at the top level, for the mixed form).
* reference_gpu - the reference's own FP64 CUDA backend (its
                  src/cuda_backend.cu built unchanged for sm_103a from the
                  sources staged in oracle/_ref) on the first timed frames
                  from the same checkpoint, beside the mixed form's rate on
                  those frames.
* e2e          -- the same metric through the public C ABI with host
                  buffers: khsUpdateRootTargets + khsUpdateColliderVertices
                  (pinned host arrays) + khsStep + khsCopyOriginalPositions
                  every step, wall clock.
* clocks       -- nvidia-smi samples taken during the timed region.

The baseline legs (cpu_baseline, same_sample's oracle, reference_gpu) are
the only code here that runs anything under oracle/.

``--impl reference`` times the CPU oracle (the reference method restated;
the reference ships no CPU implementation) on all host threads, each step
the first substeps of one frame of the same workload.  ``--gpus N`` under
torchrun runs N independent replicas (the solve does not exchange data
between strands' GPUs): weak scaling.
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

MEASURED_PEAKS = REPO / "MEASURED_PEAKS.json"

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# dominant kernels from one ncu capture of this workload; see profiles/.
# (k_block_solve's traffic does not depend on the contact state.)
NCU_TRAFFIC_BYTES: dict[str, float] = {"k_block_solve": 195.529728e6 + 69.514496e6,
                                      "k_elem_eval_grad": 89.102592e6 + 211.5456e6}

# FP64 operations per unit that the element and node kernels execute (dadd +
# dmul + 2 dfma, thread level, predicated-on), counted by ncu on the body
# scene (profiles/fp64_op_counts_body_scene.md).  The reference method
# differentiates with Dual<12>; these count this implementation's
# closed-form arithmetic, which is the work the FP64 pipe has to do.
COUNTED_FLOPS = {"k_elem_eval_grad": 1089.0, "k_elem_eval_energy": 152.0,
                 "k_node_eval_grad": 365.0, "k_node_eval_energy": 256.0}


def algorithmic(name: str, nodes: int, free_nodes: int, elements: int, candidates: float):
    """Algorithmic (bytes, FP64 flops) of one launch of kernel ``name``.

    Bytes count every input read once and every output written once (FP64
    SoA, the reference layout); flops count the reference method's
    arithmetic, not this implementation's instructions:
    * k_block_solve, per free node: read the diagonal and upper 6x6 blocks
      and the gradient (288 + 288 + 48 B), write the direction (48 B); block
      Thomas = B = D - U^T C (216 FMA), rhs (36), Gauss-Jordan inverse of a
      6x6 with the identity appended (6 x (12 + 5 x 12) ops = 396 FMA-equiv),
      C = B^-1 U (216), d' = B^-1 rhs (36), back substitution (36): 936 FMA
      = 1872 flops.
    * k_contact, per element: both node positions (48 B), node indices and
      flags (10 B), the record written (candidates, triangle, flags, gap, t,
      distance, barycentrics: 57 B); per candidate test 84 B (three vertices
      and the index triple).
    * k_elem_eval_grad, per element: q of both nodes (96 B), R and Jl of both
      (288 B), constants (56 B), the two contributions (2 x (48 + 288) B) and
      the upper block (288 B).
    * k_node_eval_*, per node: q, q_old, v (144 B), constants (88 B),
      gradient and diagonal written (48 + 48 B).
    * k_elem_eval_energy, per element: q and R of both nodes (96 + 144 B),
      constants (56 B), the two energies written (16 B).
    FP64 flops of k_elem_eval_* and k_node_eval_* are the counted ones
    (COUNTED_FLOPS).
    """
    if name == "k_block_solve":
        return 672.0 * free_nodes, 1872.0 * free_nodes
    if name in ("k_contact", "k_contact_query"):
        return 115.0 * elements + 84.0 * candidates, None
    if name == "k_elem_eval_grad":
        return 1400.0 * elements, COUNTED_FLOPS[name] * elements
    if name == "k_elem_eval_energy":
        return 312.0 * elements, COUNTED_FLOPS[name] * elements
    if name.startswith("k_node_eval"):
        return 328.0 * nodes, COUNTED_FLOPS.get(name, 0.0) * nodes or None
    return None, None


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


def _oracle_library():
    import khs_native as kn

    subprocess.run(["make", "-s", "-C", str(REPO / "oracle")], check=True)
    lib = kn.Library(REPO / "oracle" / "_build" / "libkhs_oracle.so")
    lib.lib.khsOracleSetThreads.restype = ctypes.c_int
    lib.lib.khsOracleSetThreads.argtypes = [ctypes.c_int]
    lib.lib.khsOracleSetSubstepLimit.argtypes = [ctypes.c_uint32]
    return lib


def cpu_oracle_sample(scene, full_frames: int, repeats: int, substeps: int, threads: int | None = None) -> dict:
    """Times the CPU oracle on a bounded sample of the workload: frames
    1..full_frames run in full (untimed) and are checkpointed; each of
    ``repeats`` timed samples restores that checkpoint and runs the first
    ``substeps`` substeps of frame full_frames + 1."""
    import khs_native as kn
    import scenes

    lib = _oracle_library()
    cores = int(lib.lib.khsOracleSetThreads(threads or os.cpu_count() or 1))
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, frames=full_frames + 2)
    lib.lib.khsOracleSetSubstepLimit(0)
    for f in range(1, full_frames + 1):
        r = s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt)
        if r != kn.OK:
            raise RuntimeError(f"oracle frame {f} failed ({r}): {s.last_error()}")
    checkpoint = s.save_checkpoint()
    lib.lib.khsOracleSetSubstepLimit(substeps)
    done, newton, seconds, per_step = 0, 0, 0.0, []
    for _ in range(repeats):
        s.restore_checkpoint(checkpoint)
        t0 = time.perf_counter()
        r = s._library.khsStepAnimationFrame(s.handle, full_frames + 1, scene.frame_dt)
        dt = time.perf_counter() - t0
        if r != kn.OK:
            raise RuntimeError(f"oracle frame {full_frames + 1} failed ({r}): {s.last_error()}")
        st = s.stats()
        done += st.converged_substeps
        newton += st.newton_iterations
        seconds += dt
        per_step.append(dt)
    s.close()
    lib.lib.khsOracleSetSubstepLimit(0)
    return {"value": done / seconds, "unit": UNIT, "cores": cores, "kind": "port", "seconds": seconds,
            "substeps": done, "newton_iterations": newton, "per_step_s": per_step,
            "sample": f"first {substeps} substeps of frame {full_frames + 1} of the same body scene ({repeats} "
                      f"run(s) from a checkpoint after frames 1-{full_frames} in full, untimed); CPU FP64 oracle on "
                      f"{cores} threads"}


def oracle_sample_from(scene, checkpoint: bytes, frame: int, substeps: int, repeats: int,
                       threads: int | None = None) -> dict:
    """Times the CPU oracle on the first ``substeps`` substeps of ``frame``,
    starting every repeat from ``checkpoint`` (the GB300 state after frame
    ``frame - 1``); returns the rate and the state reached."""
    import khs_native as kn
    import scenes

    lib = _oracle_library()
    cores = int(lib.lib.khsOracleSetThreads(threads or os.cpu_count() or 1))
    lib.lib.khsOracleSetSubstepLimit(0)
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, frames=frame + 1)
    s.set_substep_limit(substeps)
    done, newton, seconds, per_step = 0, 0, 0.0, []
    for _ in range(repeats):
        s.restore_checkpoint(checkpoint)
        t0 = time.perf_counter()
        r = s._library.khsStepAnimationFrame(s.handle, frame, scene.frame_dt)
        dt = time.perf_counter() - t0
        if r != kn.OK:
            raise RuntimeError(f"oracle frame {frame} failed ({r}): {s.last_error()}")
        st = s.stats()
        done += st.converged_substeps
        newton += st.newton_iterations
        seconds += dt
        per_step.append(dt)
    q = s.state()[0]
    s.close()
    return {"value": done / seconds, "unit": UNIT, "cores": cores, "kind": "port", "seconds": seconds,
            "substeps": done, "newton_iterations": newton, "per_step_s": per_step, "q": q,
            "sample": f"first {substeps} substeps of frame {frame} of the same body scene, {repeats} run(s) from "
                      f"the GB300 checkpoint after frame {frame - 1}; CPU FP64 oracle on {cores} threads"}


def gpu_sample_from(lib, scene, checkpoint: bytes, frame: int, substeps: int, mode: int) -> dict:
    """The GB300 library on exactly the oracle sample's substeps (same
    checkpoint, same substep limit); device time of the second run (the
    first also tunes the block-solve launch shape)."""
    import khs_native as kn
    import scenes

    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, frames=frame + 1)
    s.set_solve_mode(mode)
    s.set_substep_limit(substeps)
    for _ in range(2):
        s.restore_checkpoint(checkpoint)
        if s._library.khsStepAnimationFrame(s.handle, frame, scene.frame_dt) != kn.OK:
            raise RuntimeError(f"sampled frame {frame} failed: {s.last_error()}")
    ms = s.gpu_stats().last_frame_milliseconds
    st = s.stats()
    q = s.state()[0]
    s.close()
    return {"value": st.converged_substeps / (ms / 1e3), "unit": UNIT, "device_ms": ms,
            "substeps": int(st.converged_substeps), "newton_iterations": int(st.newton_iterations), "q": q}


def reference_gpu_frames(scene, checkpoint: bytes, first: int, count: int, frame_ms: list, frame_substeps: list) -> dict:
    """The reference's own FP64 CUDA backend (its src/cuda_backend.cu built
    unchanged for sm_103a, oracle/_ref) on frames first..first+count-1 of the
    same scene from the same checkpoint as the timed frames; beside it the
    mixed form's rate on those frames, from the timed run."""
    sys.path.append(str(REPO / "oracle"))
    import refgpu

    if not refgpu.available():
        return {"unavailable": "the reference CUDA sources are not staged in oracle/_ref/src"}
    ref = refgpu.RefLibrary()
    s = refgpu.RefSolver(ref, _oracle_library(), scene, frames=first + count)
    s.restore_checkpoint(checkpoint)  # module load and first launches outside the timing
    if s.step_animation_frame(first, scene.frame_dt) != 0:
        raise RuntimeError(f"reference frame {first} failed: {s.last_error()}")
    s.restore_checkpoint(checkpoint)
    wall, device, substeps, newton = [], [], [], 0
    for f in range(first, first + count):
        t0 = time.perf_counter()
        r = s.step_animation_frame(f, scene.frame_dt)
        wall.append(time.perf_counter() - t0)
        if r != 0:
            raise RuntimeError(f"reference frame {f} failed ({r}): {s.last_error()}")
        device.append(s.gpu_stats().last_frame_milliseconds)
        st = s.stats()
        substeps.append(int(st.substeps))
        newton += st.newton_iterations
    s.close()
    ours_s = sum(frame_ms[:count]) / 1e3
    return {"value": sum(substeps) / sum(wall), "unit": UNIT, "frames": f"{first}-{first + count - 1}",
            "substeps": substeps, "newton_iterations": newton, "frame_ms": [round(1e3 * w, 1) for w in wall],
            "event_ms": [round(x, 1) for x in device],
            "mixed_same_frames": {"value": sum(frame_substeps[:count]) / ours_s, "substeps": frame_substeps[:count]},
            "note": "the reference's src/cuda_backend.cu compiled unchanged for sm_103a, FP64, stepped from the "
                    "GB300 checkpoint of the timed region's start; its substep counts may differ from ours because "
                    "it sums with atomics"}


def run_reference(args) -> None:
    world, rank = _dist()
    if rank != 0:
        return
    import scenes

    scene = scenes.body_scene(frames=args.warmup + args.steps + 1)
    cpu = cpu_oracle_sample(scenes.body_scene(frames=args.warmup + 3), args.warmup + 1, args.steps, args.cpu_substeps)
    value = cpu["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * cpu["seconds"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded body scene)",
        "config": _config(scene, "reference-cpu-oracle"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu["cores"], "kind": "port",
                         "sample": cpu["sample"] + " (the reference method restated; the reference has no CPU solver)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "substeps": cpu["substeps"], "newton_iterations": cpu["newton_iterations"],
    }
    print(json.dumps(line), flush=True)


def _config(scene, mode: str) -> dict:
    return {"workload": "body scene: 6,757 strands / 265,108 nodes / 258,351 elements, 225,184-vertex swaying "
                        "head+torso collider, 8 base substeps (adaptive <= 64) per frame",
            "strands": int(scene.strands), "points": int(len(scene.points)),
            "collider_vertices": int(len(scene.vertices)), "collider_triangles": int(len(scene.triangles)),
            "substeps_base": int(scene.desc["substeps"]), "max_substeps": int(scene.desc["maximum_substeps"]),
            "mode": mode, "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"}


def time_frames(lib, scene, mode: int, args, torch, flush, world: int, profile_frames: int) -> dict:
    """Warm-up frames, then the timed frames of one solve mode (device time
    of each frame from the library's CUDA events, no per-kernel timing).
    Afterwards, untimed, the first ``profile_frames`` timed frames are run
    again from a checkpoint of the timed region's start with per-kernel
    CUDA-event timing on, for the kernel shares and the roofline."""
    import khs_native as kn
    import scenes

    frames = args.warmup + args.steps + 1
    solver = kn.HairSolver(lib)
    scenes.load_into(solver, scene)
    solver.set_solve_mode(mode)
    for f in range(1, args.warmup + 1):
        solver.step_animation_frame(f, scene.frame_dt)
    start = solver.save_checkpoint()
    launches0 = solver.kernel_launches()
    clocks = ClockSampler()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    frame_ms, frame_substeps, newton, candidates = [], [], 0, 0
    wall0 = time.perf_counter()
    for f in range(args.warmup + 1, frames):
        _flush_l2(torch, flush)
        r = solver._library.khsStepAnimationFrame(solver.handle, f, scene.frame_dt)
        if r != kn.OK:
            raise RuntimeError(f"frame {f} failed ({r}): {solver.last_error()}")
        frame_ms.append(solver.gpu_stats().last_frame_milliseconds)
        st = solver.stats()
        frame_substeps.append(int(st.substeps))
        newton += st.newton_iterations
        candidates += st.contact_candidate_count
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clock_info = clocks.stop()
    launches = solver.kernel_launches() - launches0
    import replicas

    checksum = replicas.state_checksum(solver.state()[0])
    # Untimed profiling pass over the same frames.
    solver.restore_checkpoint(start)
    solver.set_profiling(True)
    solver.reset_kernel_timings()
    profiled_ms, profiled_candidates = [], 0
    for f in range(args.warmup + 1, args.warmup + 1 + profile_frames):
        _flush_l2(torch, flush)
        if solver._library.khsStepAnimationFrame(solver.handle, f, scene.frame_dt) != kn.OK:
            raise RuntimeError(f"profiled frame {f} failed: {solver.last_error()}")
        profiled_ms.append(solver.gpu_stats().last_frame_milliseconds)
        profiled_candidates += solver.stats().contact_candidate_count
    timings = solver.kernel_timings()
    solver.set_profiling(False)
    out = {"device_s": sum(frame_ms) / 1e3, "wall_s": wall, "substeps": sum(frame_substeps), "newton": newton,
           "candidates": candidates, "frame_ms": frame_ms, "frame_substeps": frame_substeps, "clocks": clock_info,
           "launches": launches, "timings": timings, "profiled_frames": profile_frames,
           "profiled_ms": profiled_ms, "profiled_candidates": profiled_candidates,
           "kernel_ms_sum": sum(ms for _, ms in timings.values()),
           "stats": solver.build_stats(), "checksum": checksum, "start_checkpoint": start}
    solver.close()
    return out


def _aggregate(run: dict, world: int) -> dict:
    """Replicas: SUM of substeps over ranks / MAX of device seconds."""
    import replicas

    dist = None
    if world > 1:
        import torch.distributed as dist
    return replicas.aggregate(run["substeps"], run["device_s"], run["checksum"], dist, "cuda")


def _roofline(run: dict, fp64_peak: float) -> dict:
    """Roofline of the kernel with the largest share of device time in the
    profiled frames.  Its algorithmic bytes per launch over its average
    launch time, against the measured HBM copy bandwidth; where the kernel
    has an algorithmic FP64 flop count, also its flops per launch against the
    FP64 FMA-pipe rate measured on this GPU.  ``bound`` names the roof the
    kernel is closer to, and the top-level achieved / peak / frac are that
    roof's; the other roof is kept under ``hbm`` or ``fp64``."""
    timings = run["timings"]
    total = sum(ms for _, ms in timings.values()) or 1.0
    name, (count, ms) = max(timings.items(), key=lambda kv: kv[1][1]) if timings else ("none", (0, 0.0))
    st = run["stats"]
    nodes, elements = int(st.internal_node_count), int(st.element_count)
    free_nodes = nodes - int(st.fixed_node_count)
    grad_evals = timings.get("k_elem_eval_grad", (0, 0.0))[0] or 1
    cand_per_eval = run["profiled_candidates"] / grad_evals
    per_launch_s = (ms / max(count, 1)) / 1e3
    alg_bytes, alg_flops = algorithmic(name, nodes, free_nodes, elements, cand_per_eval)
    peaks = json.loads(MEASURED_PEAKS.read_text()) if MEASURED_PEAKS.exists() else {}
    hbm_peak = peaks.get("hbm_gbs")
    peak_source = "measured (MEASURED_PEAKS.json hbm_gbs)"
    if not hbm_peak:
        # No measured copy bandwidth on this machine: an earlier STREAM-style
        # copy measurement on a GB300.
        hbm_peak, peak_source = 6800.0, "fallback (6.8 TB/s, an earlier copy measurement on a GB300)"
    achieved = alg_bytes / per_launch_s / 1e9 if (alg_bytes and per_launch_s > 0) else None
    hbm = {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
           "frac": achieved / hbm_peak if (achieved and hbm_peak) else None, "peak_source": peak_source,
           "algorithmic_bytes_per_launch": alg_bytes}
    fp64 = None
    if alg_flops:
        tf = alg_flops / per_launch_s / 1e12
        fp64 = {"achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s", "frac": tf / fp64_peak,
                "algorithmic_flops_per_launch": alg_flops,
                "peak_source": "measured FP64 FMA-pipe rate of this GPU (khsxMeasurePipePeaks)"}
    bound = "fp64" if fp64 and (hbm["frac"] or 0.0) < fp64["frac"] else "hbm"
    top = fp64 if bound == "fp64" else hbm
    roof = {"bound": bound, "kernel": name, "achieved": top["achieved"], "peak": top["peak"], "unit": top["unit"],
            "frac": top["frac"], "traffic": NCU_TRAFFIC_BYTES.get(name), "algorithmic_bytes_per_launch": alg_bytes,
            "avg_launch_ms": ms / max(count, 1), "launches": count, "share": ms / total,
            "profiled_frames": run["profiled_frames"],
            "kernel_shares": {k: round(v[1] / total, 4) for k, v in sorted(timings.items(), key=lambda kv: -kv[1][1])}}
    if bound == "fp64":
        roof["hbm"] = hbm
    elif fp64:
        roof["fp64"] = fp64
    # The next kernels by share, against the same FP64 roof.
    others = {}
    for other, (n_other, ms_other) in sorted(timings.items(), key=lambda kv: -kv[1][1])[1:4]:
        b_other, f_other = algorithmic(other, nodes, free_nodes, elements, cand_per_eval)
        t_other = (ms_other / max(n_other, 1)) / 1e3
        if f_other and t_other > 0:
            tf = f_other / t_other / 1e12
            others[other] = {"avg_launch_ms": round(ms_other / max(n_other, 1), 4), "share": round(ms_other / total, 4),
                             "fp64_tflops": round(tf, 4), "fp64_frac": round(tf / fp64_peak, 4),
                             "hbm_gbs": round(b_other / t_other / 1e9, 1) if b_other else None}
    if others:
        roof["next_kernels"] = others
    return roof


def _host_gap(run: dict) -> dict:
    """Device time of the profiled frames against the sum of their kernels'
    CUDA-event times: the difference is time the GPU waited on the host
    (launch gaps and the host-driven Newton loop's synchronisations)."""
    frames_ms = sum(run["profiled_ms"])
    return {"frames_ms": round(frames_ms, 2), "kernel_ms_sum": round(run["kernel_ms_sum"], 2),
            "idle_fraction": round(1.0 - run["kernel_ms_sum"] / frames_ms, 4) if frames_ms else None,
            "frames": run["profiled_frames"]}


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
    scene = scenes.body_scene(frames=args.warmup + args.steps + 1)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    modes = {"plain": kn.MODE_PLAIN_FP64, "mixed": kn.MODE_MIXED}
    profile_frames = min(args.steps, args.profile_frames)
    main = time_frames(lib, scene, modes[args.mode], args, torch, flush, world, profile_frames)
    agg = _aggregate(main, world)
    device_s, value = agg["max_seconds"], agg["value"]
    plain = None
    if args.mode == "mixed" and not args.skip_plain:
        ref = time_frames(lib, scene, kn.MODE_PLAIN_FP64, args, torch, flush, world, min(profile_frames, 2))
        ragg = _aggregate(ref, world)
        plain_s = ragg["max_seconds"]
        plain = {"value": ragg["value"], "unit": UNIT, "ms_per_step": 1e3 * plain_s / args.steps,
                 "substeps": ref["substeps"], "newton_iterations": ref["newton"], "speedup_of_mixed": None,
                 "top_kernels": dict(list(_roofline(ref, fp64_peak.value)["kernel_shares"].items())[:4])}
        plain["speedup_of_mixed"] = value / plain["value"]
        plain["same_iterates"] = ref["substeps"] == main["substeps"] and ref["newton"] == main["newton"]
        plain["same_final_state"] = ref["checksum"] == main["checksum"]

    # End to end through the public API with host buffers.
    e2e = run_e2e(lib, scene, args, torch) if not args.skip_e2e else None
    roofline = _roofline(main, fp64_peak.value)
    cpu, sample, reference_gpu = None, None, None
    first = args.warmup + 1
    if rank == 0 and world == 1 and not args.skip_cpu:
        # Baseline legs, all from the checkpoint of the timed region's start:
        # the CPU oracle and both GB300 forms on the same substeps (rate and
        # deviation), and the reference's own CUDA backend on whole frames.
        ck = main["start_checkpoint"]
        cpu = oracle_sample_from(scene, ck, first, args.cpu_substeps, args.cpu_repeats)
        oq = cpu.pop("q")
        sample = {"frame": first, "substeps": args.cpu_substeps, "oracle_substeps_per_s": cpu["value"]}
        for label, mode in (("mixed", kn.MODE_MIXED), ("plain_fp64", kn.MODE_PLAIN_FP64)):
            g = gpu_sample_from(lib, scene, ck, first, args.cpu_substeps, mode)
            dq = np.abs(g.pop("q") - oq)
            g["max_position_dev_m"] = float(dq[:, :3].max())
            g["max_rotation_dev_rad"] = float(dq[:, 3:].max())
            sample[label] = g
        if not args.skip_reference_gpu:
            reference_gpu = reference_gpu_frames(scene, ck, first, min(args.steps, args.reference_frames),
                                                 main["frame_ms"], main["frame_substeps"])
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * device_s / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.mode == "plain" else "f64+f32",
            "data": "synthetic (seeded body scene, see kami-hair-solver_gb300/scenes.py)",
            "config": _config(scene, args.mode), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "plain_fp64": plain, "same_sample": sample, "reference_gpu": reference_gpu,
            "max_position_dev_m": sample["mixed"]["max_position_dev_m"] if sample else None,
            "max_rotation_dev_rad": sample["mixed"]["max_rotation_dev_rad"] if sample else None,
            "host_gap": _host_gap(main), "clocks": main["clocks"], "gpu_launches": int(main["launches"]),
            "wall_s": main["wall_s"], "substeps": main["substeps"], "newton_iterations": main["newton"],
            "frame_ms": [round(x, 2) for x in main["frame_ms"]], "frame_substeps": main["frame_substeps"],
            "fp64_pipe_peak_tflops": fp64_peak.value, "fp32_pipe_peak_tflops": fp32_peak.value,
            "replica_checksums": agg["checksums"],
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
    return {"value": sub / dt, "unit": UNIT, "h2d_bytes_per_step": P * 24 + V * 24,
            "d2h_bytes_per_step": P * 24, "note": "the source points are uploaded and turned into node position and "
            "rotation-vector targets on the device (k_root_*)"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["plain", "mixed"], default="mixed")
    ap.add_argument("--skip-plain", action="store_true", help="do not time the plain FP64 form beside the mixed one")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--cpu-substeps", type=int, default=1,
                    help="substeps per sampled frame in the CPU oracle legs")
    ap.add_argument("--cpu-repeats", type=int, default=3,
                    help="timed repeats of the CPU oracle sample (each from the same checkpoint)")
    ap.add_argument("--profile-frames", type=int, default=4,
                    help="timed frames re-run untimed with per-kernel timing for the kernel shares")
    ap.add_argument("--reference-frames", type=int, default=3,
                    help="frames of the reference's own CUDA backend timed beside ours")
    ap.add_argument("--skip-reference-gpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
