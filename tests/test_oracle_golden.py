"""Pins the CPU oracle against the reference's own golden values
(tests/testthat/test-ci.R), at that suite's 1e-4 tolerance."""
import pytest

import ci_cases
import edm_oracle


@pytest.fixture(scope="module", autouse=True)
def _built():
    edm_oracle.load()


@pytest.mark.parametrize("case", ci_cases.CASES, ids=lambda c: c.__name__)
def test_oracle_matches_reference_goldens(case):
    case(edm_oracle.oracle_edm)
