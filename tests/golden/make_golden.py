"""Generate the golden fixtures in this directory from the reference itself.

Runs ``oracle/_ref/ref_driver`` (the reference Omega_h library compiled from
its own sources by ``oracle/ref.mk``) on seeded box workloads and stores

* ``<case>.npz``: every per-stage intermediate array and the mesh before and
  after each operator of one adapt pass (small cases);
* ``<case>_digest.json``: sha256 digests of every integer array and
  sum/min/max/strided samples of every real array (full-size cases, whose raw
  arrays are too large to commit);
* ``osh/<case>/{in,out}.osh/``: the mesh before and after one pass, written
  by the reference's own binary::write (its .osh format), with the mesh
  arrays after the pass in ``osh/<case>/out_arrays.npz``;
* ``metric/<case>.npz``: the metric tools' outputs on the box after the
  workload (intersection, clamp, Hessian metrics, implied metrics,
  gradation, expected element count, generate_metrics).

On one rank the reference's global numbers are always 0..n-1 (checked here),
so ``global_*`` arrays are dropped from the fixtures.

Usage (needs the reference sources, i.e. only in the build container)::

    python tests/golden/make_golden.py [--ref /path/to/omega_h] [case ...]

(metric tool cases are named ``metric:<case>``)
"""
import argparse
import hashlib
import json
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# name: (dim, n, metric kind, seed, min_quality_allowed, full fixture?)
CASES = {
    # the 8^3 isotropic box (3072 tets, 729 verts), min_quality_allowed 0.3
    "box8_iso": (3, 8, 0, 12345, 0.3, True),
    # 12^3 shock metric: exercises refine, coarsen and swap
    "box12_shock": (3, 12, 1, 7, 0.2, True),
    # 12^3 boundary layer (aspect up to 1000:1): refine, coarsen and swap
    "box12_blayer": (3, 12, 2, 3, 0.2, True),
    # 64^3 shock metric (1,572,864 tets, 274,625 verts): digests only
    "box64_shock": (3, 64, 1, 2024, 0.2, False),
    # 2D 32^2 boxes (2048 triangles), 2D defaults (min_quality_allowed 0.3):
    # isotropic (coarsen, swap), shock (refine, coarsen, swap), boundary layer
    "sq32_iso": (2, 32, 0, 5, 0.3, True),
    "sq32_shock": (2, 32, 1, 5, 0.3, True),
    "sq32_blayer": (2, 32, 2, 5, 0.3, True),
    # isotropic sine field of the batched workload (seeded h0, a, k)
    "box10_sine": (3, 10, 3, 5, 0.2, True),
    "sq40_sine": (2, 40, 3, 2, 0.3, True),
    # isotropic metrics stored as one scalar per vertex (kind + 10), the
    # reference's isotropic metric tag
    "box8_iso_scalar": (3, 8, 10, 12345, 0.3, True),
    "box10_sine_scalar": (3, 10, 13, 5, 0.2, True),
    "sq32_sine_scalar": (2, 32, 13, 5, 0.3, True),
    # the full adapt() loop (passes until lengths settle, then swaps and
    # sliver collapses): the final mesh only
    "box8_iso_adapt": (3, 8, 0, 12345, 0.3, True, "adapt"),
    "box10_sine_adapt": (3, 10, 3, 5, 0.2, True, "adapt"),
    "sq32_shock_adapt": (2, 32, 1, 5, 0.3, True, "adapt"),
    "sq32_blayer_adapt": (2, 32, 2, 5, 0.3, True, "adapt"),
    "box8_sine_scalar_adapt": (3, 8, 13, 5, 0.2, True, "adapt"),
    # one pass at full size, the mesh after it only (digests): the two
    # boundary-layer workloads of the FP32-screening tier (2D 1024^2,
    # 2,097,152 triangles; 3D 48^3, 663,552 tets) and a 64^3 box whose pass
    # refines, coarsens and swaps (isotropic sine, seed 469: h0 0.0204,
    # amplitude 0.39; 1,572,864 tets in, 2,184,560 out)
    "sq1024_blayer": (2, 1024, 2, 3, 0.3, False, "nostages"),
    "box48_blayer": (3, 48, 2, 3, 0.2, False, "nostages"),
    "box64_sine": (3, 64, 3, 469, 0.2, False, "nostages"),
    # the first 8 meshes of the batched workload's seeded list (1024 boxes,
    # n log-uniform in [4, 40], isotropic sine metric, seed 7)
    "batch_m0_n17": (3, 17, 3, 1504059971, 0.2, False, "nostages"),
    "batch_m1_n32": (3, 32, 3, 1942236769, 0.2, False, "nostages"),
    "batch_m2_n24": (3, 24, 3, 2040772436, 0.2, False, "nostages"),
    "batch_m3_n6": (3, 6, 3, 529044838, 0.2, False, "nostages"),
    "batch_m4_n8": (3, 8, 3, 930072621, 0.2, False, "nostages"),
    "batch_m5_n30": (3, 30, 3, 1543323540, 0.2, False, "nostages"),
    "batch_m6_n4": (3, 4, 3, 881660342, 0.2, False, "nostages"),
    "batch_m7_n27": (3, 27, 3, 664364275, 0.2, False, "nostages"),
}


# .osh fixtures: (dim, n, metric kind, seed, min_quality_allowed)
OSH_CASES = {
    "box4_shock": (3, 4, 1, 7, 0.2),     # refine only: ghosted parting
    "box4_blayer": (3, 4, 2, 1, 0.2),    # refine and swap: element-based parting
    "sq8_blayer": (2, 8, 2, 3, 0.2),     # 2D refine and swap
}


# metric tool fixtures: (dim, n, metric kind, seed); the reference's
# intersect, clamp, Hessian, implied, gradation, expected element count and
# generate_metrics outputs on the box after the workload
METRIC_CASES = {
    "box4_shock": (3, 4, 1, 7),
    "box6_iso": (3, 6, 0, 5),
    "sq8_blayer": (2, 8, 2, 3),
    "sq12_sine": (2, 12, 3, 4),
}


def run_metric_case(name, spec):
    dim, n, kind, seed = spec
    with tempfile.TemporaryDirectory() as tmp:
        args = [os.path.join(ROOT, "oracle/_ref/ref_driver"), str(dim), str(n), str(kind),
                str(seed), "0.2", tmp, "metric"]
        out = subprocess.run(args, check=True, capture_output=True, text=True, timeout=600)
        arrs = {}
        with open(os.path.join(tmp, "manifest.txt")) as f:
            for line in f:
                key, dt, count = line.split()
                if key.startswith("mt_"):
                    arrs[key] = np.fromfile(os.path.join(tmp, key + ".bin"), dtype=np.dtype(dt))
    meta = {"case": name, "dim": dim, "n": n, "metric": kind, "seed": seed,
            "driver_stdout": out.stdout.strip()}
    arrs["meta_json"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    os.makedirs(os.path.join(HERE, "metric"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "metric", name + ".npz"), **arrs)
    print(name, out.stdout.strip())


def run_intersect_case():
    """The reference's intersect_metrics on seeded partially degenerate metric
    pairs (Barral's cases) and on its unit-test pairs."""
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([os.path.join(ROOT, "oracle/_ref/ref_driver"), "intersect", tmp],
                       check=True, capture_output=True, text=True)
        arrs = {}
        with open(os.path.join(tmp, "manifest.txt")) as f:
            for line in f:
                key, dt, count = line.split()
                arrs[key] = np.fromfile(os.path.join(tmp, key + ".bin"), dtype=np.dtype(dt))
    os.makedirs(os.path.join(HERE, "metric"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "metric", "degenerate_intersections.npz"), **arrs)
    print("degenerate_intersections", {k: v.size for k, v in arrs.items()})


def run_osh_case(name, spec):
    import shutil
    dim, n, kind, seed, mqa = spec
    dst = os.path.join(HERE, "osh", name)
    if os.path.isdir(dst):
        shutil.rmtree(dst)
    os.makedirs(dst)
    with tempfile.TemporaryDirectory() as tmp:
        args = [os.path.join(ROOT, "oracle/_ref/ref_driver"), str(dim), str(n),
                str(kind), str(seed), str(mqa), tmp, "osh"]
        out = subprocess.run(args, check=True, capture_output=True, text=True)
        for part in ("in.osh", "out.osh"):
            shutil.copytree(os.path.join(tmp, part), os.path.join(dst, part))
        arrs = {}
        with open(os.path.join(tmp, "manifest.txt")) as f:
            for line in f:
                key, dt, count = line.split()
                if key.startswith("out_"):
                    arrs[key] = np.fromfile(os.path.join(tmp, key + ".bin"), dtype=np.dtype(dt))
    np.savez_compressed(os.path.join(dst, "out_arrays.npz"), **arrs)
    with open(os.path.join(dst, "case.json"), "w") as f:
        json.dump({"case": name, "dim": dim, "n": n, "metric": kind, "seed": seed,
                   "min_quality_allowed": mqa, "driver_stdout": out.stdout.strip()}, f)
    print(name, out.stdout.strip())


def build_ref(ref):
    subprocess.run(["make", "-f", "oracle/ref.mk", f"REF={ref}", "-j8"],
                   cwd=ROOT, check=True, stdout=subprocess.DEVNULL)


def run_case(name, spec):
    dim, n, kind, seed, mqa, full = spec[:6]
    mode = spec[6] if len(spec) > 6 else None
    with tempfile.TemporaryDirectory() as tmp:
        args = [os.path.join(ROOT, "oracle/_ref/ref_driver"), str(dim), str(n),
                str(kind), str(seed), str(mqa), tmp] + ([mode] if mode else [])
        out = subprocess.run(args, check=True, capture_output=True, text=True)
        arrs = {}
        with open(os.path.join(tmp, "manifest.txt")) as f:
            for line in f:
                key, dt, count = line.split()
                a = np.fromfile(os.path.join(tmp, key + ".bin"), dtype=np.dtype(dt))
                assert a.size == int(count), key
                arrs[key] = a
    for key in list(arrs):
        if "global_" in key:
            assert np.array_equal(arrs[key], np.arange(arrs[key].size)), key
            del arrs[key]
        elif "ev2v_1" in key:
            assert np.array_equal(arrs[key], arrs[key.replace("ev2v_1", "down_1")])
            del arrs[key]
    meta = {"case": name, "dim": dim, "n": n, "metric": kind, "seed": seed,
            "min_quality_allowed": mqa, "driver_stdout": out.stdout.strip()}
    if full:
        arrs["meta_json"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
    else:
        digests = {}
        for key, a in arrs.items():
            if a.dtype.kind == "f":
                idx = np.linspace(0, a.size - 1, num=min(a.size, 1024)).astype(np.int64) \
                    if a.size else np.zeros(0, np.int64)
                digests[key] = {"dtype": a.dtype.str, "count": int(a.size),
                                "sum": math.fsum(a.tolist()) if a.size else 0.0,
                                "min": float(a.min()) if a.size else 0.0,
                                "max": float(a.max()) if a.size else 0.0,
                                "sample_idx": idx.tolist(),
                                "sample": a[idx].tolist()}
                ncomp = (6 if dim == 3 else 3) if key.endswith("metric") else 1
                if ncomp > 1 and a.size % ncomp == 0 and a.size:
                    # the largest entry of each sampled entry's tensor: the
                    # scale interpolated metrics are compared against
                    rows = np.abs(a.reshape(-1, ncomp)).max(axis=1)
                    digests[key]["sample_row_scale"] = rows[idx // ncomp].tolist()
            else:
                digests[key] = {"dtype": a.dtype.str, "count": int(a.size),
                                "sha256": hashlib.sha256(
                                    np.ascontiguousarray(a).tobytes()).hexdigest()}
        meta["arrays"] = digests
        with open(os.path.join(HERE, name + "_digest.json"), "w") as f:
            json.dump(meta, f)
    print(name, out.stdout.strip())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("OMEGA_H_REFERENCE_SRC"),
                    help="the reference's source checkout (or set OMEGA_H_REFERENCE_SRC)")
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(a.ref):
        sys.exit(f"reference sources not found: pass --ref or set OMEGA_H_REFERENCE_SRC")
    build_ref(a.ref)
    for name in a.cases or list(CASES) + list(OSH_CASES) + ["metric:" + k for k in METRIC_CASES] + \
            ["intersect"]:
        if name == "intersect":
            run_intersect_case()
            continue
        if name.startswith("metric:"):
            run_metric_case(name[7:], METRIC_CASES[name[7:]])
        elif name in OSH_CASES:
            run_osh_case(name, OSH_CASES[name])
        else:
            run_case(name, CASES[name])


if __name__ == "__main__":
    main()
