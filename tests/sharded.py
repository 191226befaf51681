"""The strand-sharded solve on CPU ranks (the multi-GPU design, exercised
with the CPU oracle and torch.distributed over gloo).

Each rank builds the whole scene (the collider and its BVH are replicated),
takes a contiguous range of strands balanced by node count
(``partition``), and steps only those strands; the global scalars of the
Gauss-Newton loop -- energies, gradient and direction norms, the slope g.d,
the CCD step bound, the largest node translation, candidate and active
counts, feasibility and failure flags -- are combined by the all-reduce
given to khsOracleSetPartition: per evaluation one sum (four exact energy
sums and two counts) and one min (minimum gap, feasibility), plus one
each for the norms, the slope, the bounds and the flags.  Sums are exact, so
the iterates do not depend on the split: any number of ranks gives the bits
of one rank.
"""
from __future__ import annotations

import ctypes

import numpy as np

import khs_native as kn
import scenes

REDUCE = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_uint32, ctypes.c_int)


def partition(offsets_nodes: np.ndarray, world: int) -> list[tuple[int, int]]:
    """Contiguous strand ranges with about equal node counts.
    ``offsets_nodes`` holds each strand's node count."""
    total = int(offsets_nodes.sum())
    cum = np.concatenate([[0], np.cumsum(offsets_nodes)])
    cuts = [0]
    for r in range(1, world):
        cuts.append(int(np.searchsorted(cum, total * r / world)))
    cuts.append(len(offsets_nodes))
    return [(cuts[r], max(cuts[r + 1], cuts[r] + 1)) for r in range(world)]


def make_reduce(dist=None):
    """The all-reduce callback: torch.distributed over the default group, or
    the identity for one process."""
    import torch

    ops = None if dist is None else {0: dist.ReduceOp.SUM, 1: dist.ReduceOp.MIN, 2: dist.ReduceOp.MAX}

    def reduce(_ctx, values, count, op):
        if dist is None:
            return
        a = np.ctypeslib.as_array(values, shape=(count,))
        t = torch.from_numpy(a.copy())
        dist.all_reduce(t, op=ops[op])
        a[:] = t.numpy()

    return REDUCE(reduce)


def strand_node_counts(solver: kn.HairSolver) -> np.ndarray:
    lib = solver._library
    lib.khsOracleModelSizes.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.khsOracleModelSizes.restype = None
    sizes = np.zeros(6, dtype=np.uint32)
    lib.khsOracleModelSizes(solver.handle, sizes.ctypes.data_as(ctypes.c_void_p))
    n, e, s = (int(x) for x in sizes[:3])
    lib.khsOracleExportModel.argtypes = [ctypes.c_void_p] * 9
    lib.khsOracleExportModel.restype = None
    bufs = [np.zeros((n, 18)), np.zeros((n, 4), np.uint32), np.zeros((e, 7)), np.zeros((e, 4), np.uint32),
            np.zeros((s, 2), np.uint32), np.zeros(max(int(sizes[3]), 1), np.uint32),
            np.zeros((max(int(sizes[4]), 1), 3)), np.zeros((max(int(sizes[5]), 1), 3), np.uint32)]
    lib.khsOracleExportModel(solver.handle, *(b.ctypes.data_as(ctypes.c_void_p) for b in bufs))
    return bufs[4][:, 1].astype(np.int64)


def run(oracle_lib, scene, rank: int = 0, world: int = 1, dist=None) -> dict:
    """Steps ``scene`` on strands of this rank's range; returns the node
    range, the state of those nodes and per-frame stats and records."""
    s = kn.HairSolver(oracle_lib)
    scenes.load_into(s, scene)
    counts = strand_node_counts(s)
    s0, s1 = partition(counts, world)[rank]
    cb = make_reduce(dist)
    oracle_lib.lib.khsOracleSetPartition.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, REDUCE,
                                                     ctypes.c_void_p]
    oracle_lib.lib.khsOracleSetPartition.restype = ctypes.c_int
    assert oracle_lib.lib.khsOracleSetPartition(s.handle, s0, s1, cb, None) == kn.OK
    n0 = int(counts[:s0].sum())
    n1 = n0 + int(counts[s0:s1].sum())
    frames = []
    for f in range(1, scene.frames):
        r = s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt)
        st = s.stats()
        frames.append(dict(result=r, stats={k: getattr(st, k) for k, _ in kn.StepStats._fields_},
                           records=[(x.newton_iterations, x.line_search_evaluations, x.steepest_fallbacks,
                                     x.trust_scalings, x.contact_candidates, x.active_contacts)
                                    for x in s.substep_records()]))
        if r != kn.OK:
            break
    q, v = s.state()
    s.close()
    return dict(nodes=(n0, n1), q=q[n0:n1], v=v[n0:n1], frames=frames)
