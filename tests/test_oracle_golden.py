"""The oracle restatement against the reference's own outputs (golden
fixtures generated by tests/golden/make_golden.py from the reference built
from source).  CPU only."""
import pytest

from conftest import (ADAPT_CASES, BIG_CASE, SMALL_CASES, SMALL_CASES_2D, compare_arrays,
                      compare_digest, load_digest, load_golden, run_oracle)

ALL_SMALL = {**SMALL_CASES, **SMALL_CASES_2D}


@pytest.mark.parametrize("case", sorted(ALL_SMALL))
def test_oracle_matches_reference_per_stage(oracle_driver, case):
    golden = load_golden(case)
    got = run_oracle(oracle_driver, ALL_SMALL[case])
    fails, maxerr, ndiff = compare_arrays(golden, got)
    assert not fails, fails[:10]
    # the restatement keeps the reference's operation order: reals are
    # bitwise identical on this platform
    assert maxerr == 0.0 and ndiff == 0


def test_oracle_full_size_pass_matches_reference_digest(oracle_driver):
    name, spec = BIG_CASE
    got = run_oracle(oracle_driver, spec, mode="nostages")
    digest = load_digest(name)
    fails = compare_digest(digest, got)
    assert not fails, fails[:10]
    assert list(got["pass_flags"]) == [0, 1, 1]


@pytest.mark.parametrize("case", sorted(ADAPT_CASES))
def test_oracle_full_adapt_matches_reference(oracle_driver, case):
    golden = load_golden(case)
    got = run_oracle(oracle_driver, ADAPT_CASES[case], mode="adapt")
    keys = [k for k in golden if k.startswith("out_")]
    fails, maxerr, ndiff = compare_arrays(golden, got, keys=keys)
    assert not fails, fails[:10]
    assert maxerr == 0.0 and ndiff == 0
    assert int(got["adapt_result"][0]) == int(golden["adapt_did"][0])
