"""Continuous-batching serving loop for bake requests on one GPU.

A stream of bake requests (each a hair scene and a frame count) is served by
one process on one GPU:

* Admission: a request that has arrived is admitted as soon as a slot is
  free and its device bytes fit the remaining HBM budget (first fit in
  arrival order); finished requests return their slot and bytes at once, so
  requests that arrive while others run join the mix without waiting for a
  batch boundary.  A request reserves a conservative upper bound of its
  bytes (``estimate_bytes``) while it builds; once its solver is resident
  (model, animation frames and rollback ring on the device) the reservation
  is replaced by the bytes the solver itself reports
  (``KhsGpuStats.resident_bytes``, plus its peak temporary bytes), and the
  difference goes back to the budget at once.
* Residency: each admitted request builds its own solver, which keeps the
  rod state, the Gauss-Newton blocks, the BVH and every animation frame in
  one device arena on its own CUDA stream, plus a device-resident rollback
  ring of its last frames (khsxSetRollbackRing).
* Interleaving: each admitted request is driven by its own host thread, one
  animation frame per C-ABI call (the ctypes call releases the GIL), so the
  substeps of different requests overlap on the device.

Every solver computes with fixed-order reductions and its own buffers, so a
request's result is the same alone and in the mix (bit for bit); the tests
check this.  ``summary`` reports p50/p99 per-frame latency (wall time of
each frame call, queueing behind other requests' work included) and the
aggregate node-substeps/s over the whole stream.

Run ``python kami-hair-solver_gb300/serving.py --help`` for the request
stream options (defaults follow the serving workload: Poisson arrivals at
4 req/s, log-uniform strand counts in [100, 20000], node counts U[16, 160],
ellipsoids of 5k-50k triangles, 10 frames of 8 substeps, 150 GB budget,
10-frame rollback ring).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import statistics
import sys
import threading
import time

import numpy as np

import khs_native as kn
import scenes

# Conservative device bytes of a solver before it is built: the arena (state,
# blocks, factors, contact and BVH arrays), every animation frame, and the
# rollback ring.  Used only until the built solver reports its own bytes.
BYTES_PER_NODE = 4096
BYTES_PER_TRIANGLE = 1024
RING_BYTES_PER_NODE = 96


def estimate_bytes(scene: scenes.Scene, ring_slots: int) -> int:
    nodes = int(len(scene.points)) * 2  # internal nodes after resampling are at most ~2x the points
    tris = 0 if scene.triangles is None else int(len(scene.triangles))
    verts = 0 if scene.vertices is None else int(len(scene.vertices))
    anim = scene.frames * (nodes * 48 + verts * 24)
    return nodes * (BYTES_PER_NODE + ring_slots * RING_BYTES_PER_NODE) + tris * BYTES_PER_TRIANGLE + anim


@dataclasses.dataclass
class Request:
    rid: int
    scene: scenes.Scene
    arrival: float          # seconds after the stream starts
    frames: int             # animation frames to step (1 .. frames)


@dataclasses.dataclass
class Result:
    rid: int
    status: int = kn.OK
    error: str = ""
    q: np.ndarray | None = None
    frame_ms: list = dataclasses.field(default_factory=list)
    substeps: list = dataclasses.field(default_factory=list)
    nodes: int = 0
    bytes: int = 0          # bytes reserved at admission (the estimate)
    resident: int = 0       # bytes the built solver reported
    arrival: float = 0.0
    admitted: float = 0.0
    finished: float = 0.0


def resident_bytes(solver: kn.HairSolver) -> int:
    """Device bytes a built solver holds: its resident arrays (model, state,
    animation frames, rollback ring) and its peak temporary allocation."""
    g = solver.gpu_stats()
    return int(g.resident_bytes) + int(g.peak_temporary_bytes)


def run_request(lib, req: Request, mode: int, ring_slots: int, on_resident=None) -> Result:
    """Builds and steps one request on the calling thread.  ``on_resident``
    (if given) is called with the solver's own device bytes once it is
    built, its frames uploaded and its ring allocated, before the first
    frame is stepped."""
    res = Result(rid=req.rid, arrival=req.arrival)
    s = kn.HairSolver(lib)
    try:
        scenes.load_into(s, req.scene, frames=req.frames + 1)
        s.set_solve_mode(mode)
        if ring_slots and hasattr(s._library, "khsxSetRollbackRing"):
            s.set_rollback_ring(ring_slots)
        res.nodes = int(s.build_stats().internal_node_count)
        res.resident = resident_bytes(s)
        if on_resident is not None:
            on_resident(res.resident)
        for f in range(1, req.frames + 1):
            t0 = time.perf_counter()
            r = s._library.khsStepAnimationFrame(s.handle, f, req.scene.frame_dt)
            res.frame_ms.append(1e3 * (time.perf_counter() - t0))
            if r != kn.OK:
                res.status, res.error = r, s.last_error()
                break
            res.substeps.append(int(s.stats().substeps))
        res.q = s.state()[0]
    except Exception as exc:  # a failed request must not stop the server
        res.status, res.error = getattr(exc, "code", kn.ERROR_INTERNAL), str(exc)
    finally:
        s.close()
    return res


class Server:
    """Admits requests by slot and HBM budget and runs them concurrently."""

    def __init__(self, lib, budget_bytes: int, max_slots: int = 8, mode: int = kn.MODE_MIXED, ring_slots: int = 10,
                 estimate=estimate_bytes, runner=run_request, on_result=None):
        self.lib = lib
        self.runner = runner
        self.on_result = on_result  # called with each finished Result (from its worker thread)
        self.budget = int(budget_bytes)
        self.max_slots = int(max_slots)
        self.mode = mode
        self.ring_slots = int(ring_slots)
        self.estimate = estimate
        self.peak_bytes = 0
        self.peak_slots = 0

    def run(self, requests: list[Request]) -> list[Result]:
        waiting = sorted(requests, key=lambda r: (r.arrival, r.rid))
        results: dict[int, Result] = {}
        lock = threading.Condition()
        used = {"bytes": 0, "slots": 0}
        start = time.perf_counter()
        threads = []

        def worker(req: Request, nbytes: int, admitted: float):
            held = {"bytes": nbytes}

            def on_resident(actual: int):
                # Replace the reservation by the solver's own bytes.
                with lock:
                    used["bytes"] += actual - held["bytes"]
                    held["bytes"] = actual
                    self.peak_bytes = max(self.peak_bytes, used["bytes"])
                    lock.notify_all()

            res = self.runner(self.lib, req, self.mode, self.ring_slots, on_resident)
            res.bytes, res.admitted = nbytes, admitted
            res.finished = time.perf_counter() - start
            if self.on_result is not None:
                self.on_result(res)
            with lock:
                results[req.rid] = res
                used["bytes"] -= held["bytes"]
                used["slots"] -= 1
                lock.notify_all()

        with lock:
            while waiting or used["slots"]:
                now = time.perf_counter() - start
                admitted_any = False
                for req in list(waiting):
                    if req.arrival > now:
                        break
                    nbytes = self.estimate(req.scene, self.ring_slots)
                    if nbytes > self.budget:
                        results[req.rid] = Result(rid=req.rid, status=kn.ERROR_INVALID_ARGUMENT,
                                                  error="request exceeds the HBM budget", arrival=req.arrival)
                        waiting.remove(req)
                        continue
                    if used["slots"] < self.max_slots and used["bytes"] + nbytes <= self.budget:
                        waiting.remove(req)
                        used["bytes"] += nbytes
                        used["slots"] += 1
                        self.peak_bytes = max(self.peak_bytes, used["bytes"])
                        self.peak_slots = max(self.peak_slots, used["slots"])
                        t = threading.Thread(target=worker, args=(req, nbytes, now), daemon=True)
                        threads.append(t)
                        t.start()
                        admitted_any = True
                if admitted_any:
                    continue
                # Sleep until the next arrival, until a running request
                # finishes or reports its resident bytes (its worker
                # notifies), whichever comes first.
                now = time.perf_counter() - start
                future = [r.arrival for r in waiting if r.arrival > now]
                lock.wait(timeout=(min(future) - now) if future else None)
        for t in threads:
            t.join()
        self.makespan = time.perf_counter() - start
        return [results[r.rid] for r in sorted(requests, key=lambda r: r.rid)]


def run_serial(lib, requests: list[Request], mode: int, ring_slots: int = 0) -> tuple[list[Result], float]:
    """One request at a time in arrival order (each starts at its arrival or
    when the previous one finished); returns the results and the makespan."""
    out, clock = [], 0.0
    t_start = time.perf_counter()
    for req in sorted(requests, key=lambda r: (r.arrival, r.rid)):
        now = time.perf_counter() - t_start
        if req.arrival > now:
            time.sleep(req.arrival - now)
        res = run_request(lib, req, mode, ring_slots)
        res.admitted = max(req.arrival, clock)
        res.finished = clock = time.perf_counter() - t_start
        out.append(res)
    return sorted(out, key=lambda r: r.rid), time.perf_counter() - t_start


def summary(results: list[Result], makespan: float) -> dict:
    lat = [ms for r in results for ms in r.frame_ms]
    failed = {}
    for r in results:
        if r.status != kn.OK:
            failed[str(r.status)] = failed.get(str(r.status), 0) + 1
    node_substeps = sum(r.nodes * sum(r.substeps) for r in results)
    ok = [r for r in results if r.status == kn.OK]
    return {
        "requests": len(results), "completed": len(ok), "frames": len(lat),
        "p50_frame_ms": float(np.percentile(lat, 50)) if lat else None,
        "p99_frame_ms": float(np.percentile(lat, 99)) if lat else None,
        "mean_frame_ms": statistics.fmean(lat) if lat else None,
        "node_substeps_per_s": node_substeps / makespan if makespan > 0 else None,
        "makespan_s": makespan,
        "mean_queue_s": statistics.fmean(r.admitted - r.arrival for r in results) if results else None,
        "failed_by_result": failed,
        "reserved_bytes_total": sum(r.bytes for r in results),
        "resident_bytes_total": sum(r.resident for r in results),
    }


def make_stream(count: int, rate: float, seed: int, strand_range=(100, 20000), node_range=(16, 160),
                tri_range=(5000, 50000), frames: int = 10, substeps: int = 8) -> list[Request]:
    """Poisson arrivals at ``rate`` requests/s; each request a seeded
    serving scene (scenes.serving_request)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate))
        sc = scenes.serving_request(seed=seed * 100003 + i, strand_range=strand_range, node_range=node_range,
                                    tri_range=tri_range, frames=frames, substeps=substeps)
        out.append(Request(rid=i, scene=sc, arrival=t, frames=frames))
    return out


def main() -> None:
    import khs_build

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--rate", type=float, default=4.0, help="Poisson arrival rate, requests/s")
    ap.add_argument("--min-strands", type=int, default=100)
    ap.add_argument("--max-strands", type=int, default=20000)
    ap.add_argument("--frames", type=int, default=10)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--ring", type=int, default=10)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--serial-plain", action="store_true", help="also run the stream one at a time in plain FP64")
    ap.add_argument("--plain-sample", type=int, default=0,
                    help="also run the first N requests of the stream (same seeds, same arrivals) batched in the "
                         "mixed form and one at a time in plain FP64, for a like-for-like comparison")
    args = ap.parse_args()
    lib = kn.Library(khs_build.build())
    reqs = make_stream(args.requests, args.rate, args.seed, strand_range=(args.min_strands, args.max_strands),
                       frames=args.frames)
    def progress(r: Result) -> None:
        # One write per line: workers finish concurrently.
        sys.stderr.write(json.dumps({"rid": r.rid, "status": r.status, "nodes": r.nodes, "substeps": sum(r.substeps),
                                     "frame_ms": [round(x, 1) for x in r.frame_ms], "arrival": round(r.arrival, 3),
                                     "admitted": round(r.admitted, 3), "finished": round(r.finished, 3),
                                     "resident_bytes": r.resident}) + "\n")
        sys.stderr.flush()

    server = Server(lib, int(args.budget_gb * 1e9), args.slots, kn.MODE_MIXED, args.ring, on_result=progress)
    res = server.run(reqs)
    line = {"workload": f"{args.requests} requests, Poisson {args.rate}/s, strands log-U[{args.min_strands}, "
                        f"{args.max_strands}], {args.frames} frames x 8 substeps",
            "mixed_batched": summary(res, server.makespan), "peak_budget_bytes": server.peak_bytes,
            "peak_slots": server.peak_slots}
    print(json.dumps(line), flush=True)
    if args.serial_plain:
        sres, span = run_serial(lib, reqs, kn.MODE_PLAIN_FP64)
        line["plain_serial"] = summary(sres, span)
    if args.plain_sample:
        sample = reqs[:args.plain_sample]
        sserver = Server(lib, int(args.budget_gb * 1e9), args.slots, kn.MODE_MIXED, args.ring)
        sres = sserver.run(sample)
        pres, span = run_serial(lib, sample, kn.MODE_PLAIN_FP64, args.ring)
        line["sample"] = {"requests": len(sample), "mixed_batched": summary(sres, sserver.makespan),
                          "plain_serial": summary(pres, span),
                          "same_status": all(a.status == b.status for a, b in zip(sres, pres)),
                          "same_final_state": all((a.q == b.q).all() for a, b in zip(sres, pres)
                                                  if a.status == kn.OK and b.status == kn.OK)}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
