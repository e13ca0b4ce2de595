"""Which libm function's last ulp the reference's results depend on.

The oracle restatement is bitwise identical to the reference on the
goldens' platform.  Rebuilt with one or more libm functions replaced by
correctly rounded ones (oracle/Makefile, ORC_CR_LIBM), it shows:

* correctly rounded acos, cos, log and exp leave every per-stage array of
  every golden case within 1e-12 relative (measured: at most 4e-14) and
  every integer of every case, the full adapt loop included, bit-exact;
* a correctly rounded cbrt alone moves interpolated metrics by 5e-8 of
  their largest entry (1e-5 relative in their smallest entries; box12_shock)
  and changes the full adapt loop's mesh on box8_iso (14 edges: ties
  between equal edge lengths broken the other way).

So the interpolation tolerances of the GPU comparison stand for cbrt: glibc's
cbrt is not correctly rounded, and CUDA's is another function.  CPU only;
meaningful only against the goldens' own libm (x86-64 glibc)."""
import os
import platform
import subprocess

import numpy as np
import pytest

from conftest import (ADAPT_CASES, ROOT, SMALL_CASES, SMALL_CASES_2D, compare_arrays,
                      load_golden, run_oracle)

pytestmark = pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"),
                                reason="the goldens were written with the x86-64 glibc")

ALL_SMALL = {**SMALL_CASES, **SMALL_CASES_2D}


def _variant(mask):
    target = f"_build/oracle_driver_cr{mask}"
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), target], check=True,
                   stdout=subprocess.DEVNULL)
    return os.path.join(ROOT, "oracle", target)


def _tensor_err(a, b):
    A, B = np.asarray(a).reshape(-1, 6), np.asarray(b).reshape(-1, 6)
    return float(np.max(np.max(np.abs(A - B), axis=1) / np.max(np.abs(A), axis=1)))


def test_correctly_rounded_acos_cos_log_exp_keep_parity():
    drv = _variant(2 | 4 | 8 | 16)
    worst = 0.0
    for case, spec in sorted(ALL_SMALL.items()):
        g = load_golden(case)
        fails, maxerr, _ = compare_arrays(g, run_oracle(drv, spec), interp=False)
        assert not fails, (case, fails[:5])
        worst = max(worst, maxerr)
    for case, spec in sorted(ADAPT_CASES.items()):
        g = load_golden(case)
        keys = [k for k in g if k.startswith("out_")]
        fails, maxerr, _ = compare_arrays(g, run_oracle(drv, spec, mode="adapt"), keys=keys,
                                          interp=False)
        assert not fails, (case, fails[:5])
        worst = max(worst, maxerr)
    print(f"correctly rounded acos, cos, log, exp: max real rel err {worst:.2e}")


def test_a_correctly_rounded_cbrt_alone_moves_interpolated_metrics():
    drv = _variant(1)
    g = load_golden("box12_shock")
    got = run_oracle(drv, SMALL_CASES["box12_shock"])
    err = _tensor_err(g["r_midmetrics"], got["r_midmetrics"])
    print(f"correctly rounded cbrt: box12_shock midpoint metrics differ by {err:.2e}")
    assert err > 1e-9
    # integers of the single pass stay the same
    fails, _, _ = compare_arrays(g, got)
    assert not fails, fails[:5]
    g = load_golden("box8_iso_adapt")
    got = run_oracle(drv, ADAPT_CASES["box8_iso_adapt"], mode="adapt")
    nd = int(np.sum(g["out_down_1"] != got["out_down_1"].astype(g["out_down_1"].dtype))) \
        if g["out_down_1"].shape == got["out_down_1"].shape else -1
    print(f"correctly rounded cbrt: box8_iso_adapt edges differing: {nd}")
    assert nd != 0


def test_only_the_cube_root_changes_the_full_size_digests():
    """At full size (the boundary-layer workloads, a 64^3 box that refines,
    eight batched meshes): the oracle with glibc reproduces every reference
    digest; with correctly rounded acos, cos, log and exp it still does; with
    the correctly rounded cube root alone it differs on exactly the cases
    outside CBRT_NEUTRAL_DIGESTS (near ties between cavity qualities)."""
    from conftest import (BATCH_CASES, CBRT_NEUTRAL_DIGESTS, SCALE_CASES, compare_digest,
                          digest_refined, load_digest)
    cases = {**SCALE_CASES, **BATCH_CASES}
    drivers = {"glibc": os.path.join(ROOT, "oracle", "_build", "oracle_driver"),
               "cr_acos_cos_log_exp": _variant(2 | 4 | 8 | 16), "cr_cbrt": _variant(1)}
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True,
                   stdout=subprocess.DEVNULL)
    differing = {}
    for label, drv in drivers.items():
        differing[label] = set()
        for name, spec in sorted(cases.items()):
            dg = load_digest(name)
            got = run_oracle(drv, spec, mode="nostages")
            if compare_digest(dg, got, interp=digest_refined(dg)):
                differing[label].add(name)
    print({k: sorted(v) for k, v in differing.items()})
    assert differing["glibc"] == set()
    assert differing["cr_acos_cos_log_exp"] == set()
    assert differing["cr_cbrt"] == set(cases) - CBRT_NEUTRAL_DIGESTS
