"""Runs one scene through two libraries and compares them frame by frame."""
from __future__ import annotations

import numpy as np

import khs_native as kn
import scenes


def run(lib, scene, frames=None, mode=None, probe=None, substep_limit=0):
    """Steps ``scene``; per frame returns result, stats, state and the
    contact records of the last gradient evaluation.  ``probe`` is an
    optional second library whose solver is stepped in lockstep only to
    classify contacts at this run's own state (bit-exact integer check).
    ``substep_limit`` > 0 ends every frame after that many substeps."""
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, frames=frames)
    if mode is not None:
        s.set_solve_mode(mode)
    if substep_limit:
        s.set_substep_limit(substep_limit)
    p = None
    if probe is not None:
        p = kn.HairSolver(probe)
        scenes.load_into(p, scene, frames=frames)
    out = []
    n = scene.frames if frames is None else frames
    for f in range(1, n):
        r = s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt)
        st = s.stats()
        q, v = s.state()
        rec = dict(result=r, stats=st, q=q, v=v, contacts=s.contact_records(), records=s.substep_records(),
                   error=s.last_error())
        if p is not None:
            p._library.khsStepAnimationFrame(p.handle, f, scene.frame_dt)
            rec["probe_contacts"] = p.query_contacts(q)
        out.append(rec)
        if r != kn.OK:
            break
    s.close()
    if p is not None:
        p.close()
    return out


def records_equal(a: np.ndarray, b: np.ndarray) -> dict:
    """Field-wise bitwise comparison of two contact-record arrays."""
    res = {}
    for f in ("candidate_count", "closest_triangle", "active"):
        res[f] = int(np.count_nonzero(a[f] != b[f]))
    ga, gb = a["gap"].view(np.uint64), b["gap"].view(np.uint64)
    has = a["closest_triangle"] != 0xFFFFFFFF
    res["gap_bits"] = int(np.count_nonzero((ga != gb) & has))
    return res


def compare(a, b):
    """Max deviations between two runs (lists of frame dicts)."""
    report = []
    for fa, fb in zip(a, b):
        dq = np.abs(fa["q"] - fb["q"])
        entry = dict(
            result=(fa["result"], fb["result"]),
            max_position=float(dq[:, :3].max()), max_rotation=float(dq[:, 3:].max()),
            newton=(fa["stats"].newton_iterations, fb["stats"].newton_iterations),
            line_search=(fa["stats"].line_search_evaluations, fb["stats"].line_search_evaluations),
            substeps=(fa["stats"].substeps, fb["stats"].substeps),
            candidates=(fa["stats"].contact_candidate_count, fb["stats"].contact_candidate_count),
            active=(fa["stats"].active_contact_count, fb["stats"].active_contact_count),
            record_mismatch=records_equal(fa["contacts"], fb["contacts"]),
        )
        if "probe_contacts" in fa:
            entry["own_state_mismatch"] = records_equal(fa["contacts"], fa["probe_contacts"])
        report.append(entry)
    return report
