"""The mixed-precision report's helpers (tests/mixed_precision_report.py) on
CPU with the oracle on both sides: trajectories and one-substep runs from a
checkpoint line up frame by frame, and identical libraries give zero
deviation and identical counts."""
import numpy as np

import khs_native as kn
import mixed_precision_report as report
import scenes


def test_report_helpers_line_up(oracle_lib):
    oracle_lib.lib.khsOracleSetThreads(2)
    make = lambda: scenes.ellipsoid_scene(strands=12, frames=2)  # noqa: E731
    a = report.trajectory(oracle_lib, make)
    b = report.trajectory(oracle_lib, make, kn.MODE_PLAIN_FP64)
    assert len(a["q"]) == len(b["q"]) == len(a["checkpoints"]) == len(a["records"])
    for qa, qb in zip(a["q"], b["q"]):
        assert report._dev(qa, qb) == (0.0, 0.0)
    q1, e1, c1 = report.one_substep(oracle_lib, make, a["checkpoints"][1], 2)
    q2, e2, c2 = report.one_substep(oracle_lib, make, a["checkpoints"][1], 2)
    assert np.array_equal(q1, q2) and e1 == e2 and c1 == c2
    assert report._rel(e1, e2) == 0.0 and c1[0] > 0
