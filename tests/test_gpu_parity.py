"""GPU parity: every per-stage array and the mesh after each operator of one
adapt pass, computed by the CUDA library through the C ABI, against the
reference's golden outputs (small cases: all arrays; 1.57M-tet pass: sha256
of every integer array and sampled reals) and against the oracle on seeds
without fixtures.  Integers bit-exact; reals within 1e-12 relative."""
import pytest

from conftest import (BATCH_CASES, BIG_CASE, CBRT_NEUTRAL_DIGESTS, SCALAR_CASES, SCALE_CASES,
                      SMALL_CASES, SMALL_CASES_2D, compare_arrays, compare_digest, digest_refined,
                      load_digest, load_golden, run_oracle)

ALL_SMALL = {**SMALL_CASES, **SMALL_CASES_2D, **SCALAR_CASES}

pytestmark = pytest.mark.gpu

# intermediates of the operators that the GPU dump does not expose one by one
# (their effect is pinned by the mesh after each operator)
NOT_DUMPED = ("c_rails2edges", "c_rail_col_dirs", "c_dead_", "s_keep", "s_keys")


@pytest.fixture(scope="module", autouse=True)
def built():
    from omega_h_gb300 import build
    build.build()


@pytest.mark.parametrize("case", list(ALL_SMALL))
def test_gpu_matches_reference_per_stage(case):
    import gpu_dump
    golden = load_golden(case)
    got = gpu_dump.run(*ALL_SMALL[case])
    keys = [k for k in golden if k in got or not k.startswith(NOT_DUMPED)]
    fails, maxerr, ndiff = compare_arrays(golden, got, keys=keys, rtol=1e-12)
    print(f"{case}: max real rel err {maxerr:.3e}, {ndiff} reals not bitwise equal")
    for f in fails:
        print("  FAIL", f)
    assert not fails, fails[:12]


def test_gpu_full_size_pass_matches_reference_digest():
    import gpu_dump
    name, spec = BIG_CASE
    got = gpu_dump.run(*spec, stages=False)
    fails = compare_digest(load_digest(name), got)
    assert not fails, fails[:12]
    assert list(got["pass_flags"]) == [0, 1, 1]


@pytest.mark.parametrize("case", sorted(CBRT_NEUTRAL_DIGESTS))
def test_gpu_pass_matches_reference_digest(case):
    """One pass at full size (2D 1024^2 and 3D 48^3 boundary layers) and on
    batched meshes, against the reference's mesh after its pass: every
    integer array by sha256, reals by sampled entries."""
    import gpu_dump
    spec = {**SCALE_CASES, **BATCH_CASES}[case]
    dg = load_digest(case)
    got = gpu_dump.run(*spec, stages=False)
    errs = {}
    fails = compare_digest(dg, got, interp=digest_refined(dg), errs=errs)
    print(f"{case}: refined {digest_refined(dg)}, max sampled real errors "
          + ", ".join(f"{k} {v:.1e}" for k, v in sorted(errs.items())))
    assert not fails, fails[:12]


@pytest.mark.parametrize("case", sorted(SCALE_CASES) + sorted(BATCH_CASES))
def test_gpu_pass_matches_oracle_with_the_same_cube_root(oracle_cr_driver, case):
    """The same passes (the 64^3 box that refines, coarsens and swaps
    included) against the reference's algorithm run on the host with the
    GPU path's correctly rounded cube root: every array of the mesh after the
    pass, integers bit-exact and reals within 1e-12."""
    import gpu_dump
    spec = {**SCALE_CASES, **BATCH_CASES}[case]
    want = run_oracle(oracle_cr_driver, spec, mode="nostages")
    got = gpu_dump.run(*spec, stages=False)
    keys = [k for k in want if k in got]
    assert len(keys) >= 15
    fails, maxerr, ndiff = compare_arrays(want, got, keys=keys, interp=False)
    print(f"{case}: pass flags {list(want['pass_flags'])}, max real rel err {maxerr:.2e}, "
          f"{ndiff} reals not bitwise equal")
    assert not fails, fails[:12]


def test_gpu_batched_union_matches_oracle_with_the_same_cube_root(oracle_cr_driver):
    """The first 8 meshes of the batched workload run as one union pass
    (ohg_adapt_pass_batch); each part against the reference's algorithm with
    the same cube root, and against the reference's own digest where the
    cube root does not matter."""
    import gpu_dump
    from omega_h_gb300.mesh import Context, Mesh, adapt_opts, adapt_pass_batch
    ctx = Context(0)
    names = sorted(BATCH_CASES)
    ms = []
    for name in names:
        dim, n, kind, seed, _ = BATCH_CASES[name]
        m = Mesh.build_box(ctx, dim, n)
        m.apply_workload(n, seed, kind)
        ms.append(m)
    adapt_pass_batch(ctx, ms, adapt_opts(3, min_quality_allowed=0.2))
    fails = []
    for name, m in zip(names, ms):
        out = {}
        gpu_dump.dump_mesh(m, "out_", out, with_length=True, with_quality=True)
        want = run_oracle(oracle_cr_driver, BATCH_CASES[name], mode="nostages")
        keys = [k for k in want if k in out]
        f, _, _ = compare_arrays(want, out, keys=keys, interp=False)
        fails += [f"{name}: {x}" for x in f]
        if name in CBRT_NEUTRAL_DIGESTS:
            dg = load_digest(name)
            fails += [f"{name} (reference): {x}"
                      for x in compare_digest(dg, out, interp=digest_refined(dg))]
        m.close()
    ctx.close()
    assert not fails, fails[:12]


@pytest.mark.parametrize("case", list(ALL_SMALL))
def test_gpu_matches_oracle_with_the_same_cube_root_per_stage(oracle_cr_driver, case):
    """Every per-stage array of the small cases against the reference's
    algorithm with the GPU path's cube root, reals within 1e-12 throughout
    (no interpolation tolerance)."""
    import gpu_dump
    if ALL_SMALL[case][2] >= 10:
        pytest.skip("the oracle restatement carries packed tensors only")
    want = run_oracle(oracle_cr_driver, ALL_SMALL[case])
    got = gpu_dump.run(*ALL_SMALL[case])
    keys = [k for k in want if k in got]
    fails, maxerr, ndiff = compare_arrays(want, got, keys=keys, interp=False)
    print(f"{case}: max real rel err {maxerr:.2e}, {ndiff} reals not bitwise equal")
    assert not fails, fails[:12]


@pytest.mark.parametrize("spec", [(3, 10, 3, 5, 0.2), (3, 9, 1, 99, 0.25), (3, 14, 2, 11, 0.2),
                                  (2, 40, 1, 9, 0.3), (2, 28, 2, 4, 0.3), (2, 36, 3, 2, 0.3)])
def test_gpu_matches_oracle_other_seeds(oracle_driver, spec):
    import gpu_dump
    want = run_oracle(oracle_driver, spec)
    got = gpu_dump.run(*spec)
    keys = [k for k in want if k in got]
    fails, maxerr, ndiff = compare_arrays(want, got, keys=keys, rtol=1e-12)
    assert not fails, fails[:12]
