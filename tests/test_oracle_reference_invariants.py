"""Pins the CPU oracle against the reference's own known-answer tests.

The reference ships no golden trajectories; its tests (tests/test_solver.cpp,
tests/test_c_api.c) hold invariants instead.  Every one of them must hold for
the oracle before the oracle is trusted as the parity reference for the GPU
library.
"""
import pytest

import reference_cases as rc


def test_c_api_defaults(oracle_lib):
    rc.case_c_api_defaults(oracle_lib, require_gpu=False)


@pytest.mark.parametrize("case", rc.ALL_SOLVER_CASES, ids=lambda c: c.__name__)
def test_reference_case(oracle_lib, case):
    case(oracle_lib)
