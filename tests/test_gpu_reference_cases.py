"""The reference's own known-answer tests against the GB300 library."""
import pytest

import reference_cases as rc

pytestmark = pytest.mark.gpu


def test_c_api_defaults(gpu_lib):
    rc.case_c_api_defaults(gpu_lib, require_gpu=True)


@pytest.mark.parametrize("case", rc.ALL_SOLVER_CASES, ids=lambda c: c.__name__)
def test_reference_case(gpu_lib, case):
    case(gpu_lib)
