"""The oracle restatement against the reference's own outputs (golden
fixtures generated by tests/golden/make_golden.py from the reference built
from source on x86-64 with glibc).  CPU only.

The reference's arithmetic on this path calls libm (cbrt, log, exp, acos,
cos), and the last-ulp results of libm differ between platforms.  On
x86-64 the restatement is bitwise identical to the reference.  Elsewhere
(the aarch64 host next to the GPU, glibc 2.39) the same source gives the
reference's integers on every single pass, but reals downstream of the
metric interpolation's cubic solve differ (about 4e-10 on box12_shock), and
the full adapt loop on box8_iso breaks a few ties between equal lengths the
other way (6 of 84,580 edges): the same effects, and the same tolerances,
as the GPU comparison."""
import platform

import numpy as np
import pytest

from conftest import (ADAPT_CASES, BIG_CASE, LIBM_TIE_SENSITIVE, SMALL_CASES, SMALL_CASES_2D,
                      compare_arrays, compare_digest, load_digest, load_golden, run_oracle)

ALL_SMALL = {**SMALL_CASES, **SMALL_CASES_2D}
# the goldens' own platform: bitwise equality expected
SAME_LIBM = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("case", sorted(ALL_SMALL))
def test_oracle_matches_reference_per_stage(oracle_driver, case):
    golden = load_golden(case)
    got = run_oracle(oracle_driver, ALL_SMALL[case])
    fails, maxerr, ndiff = compare_arrays(golden, got)
    print(f"{case}: max real rel err {maxerr:.2e}, {ndiff} reals not bitwise equal")
    assert not fails, fails[:10]
    if SAME_LIBM:
        # the restatement keeps the reference's operation order: reals are
        # bitwise identical on the goldens' platform
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
    if SAME_LIBM:
        fails, maxerr, ndiff = compare_arrays(golden, got, keys=keys)
        assert not fails, fails[:10]
        assert maxerr == 0.0 and ndiff == 0
    else:
        frac = LIBM_TIE_SENSITIVE.get(case, 0.0)
        for k in keys:
            a, b = np.asarray(golden[k]), np.asarray(got[k])
            assert a.shape == b.shape, f"{k}: shape {a.shape} vs {b.shape}"
            if a.dtype.kind != "f":
                nd = int(np.sum(a != b.astype(a.dtype)))
                print(f"  {k}: {nd}/{a.size} differ")
                assert nd <= frac * a.size, f"{k}: {nd}/{a.size} integers differ"
    assert int(got["adapt_result"][0]) == int(golden["adapt_did"][0])
