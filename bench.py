"""Throughput of one adapt pass (refine -> coarsen -> swap) on the 64^3 box
(1,572,864 tets, 274,625 verts) with the anisotropic shock metric, in mesh
elements per second per pass.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one pass over a fresh device copy of the seeded input mesh.
`value` is timed with CUDA events on the library's stream around the pass
only (inputs resident in HBM); `e2e` goes through the C ABI from pinned host
buffers: upload of the mesh arrays, ohg_mesh_from_arrays, the pass and the
download of the adapted mesh, wall clock with device synchronisation.
Between timed steps L2 is flushed by writing a 256 MiB buffer.  With N > 1
(torchrun) every rank adapts its own replica: the pass does not shard.
"""
import argparse
import hashlib
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {"workload": "box64_shock_pass", "dim": 3, "n": 64, "metric": "shock", "metric_kind": 1,
            "seed": 2024, "min_quality_allowed": 0.2, "elements": 1572864, "verts": 274625}
METRIC = "elements/s per adapt pass"
# the pass's dominant kernel (largest share of device time in its launch
# list): the screened coarsen quality filter; its DRAM traffic per launch
# (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu capture
DOMINANT = "coarsen_filter"
# untimed passes in which the launch-shape autotuner explores its variants
AUTOTUNE_PASSES = 4
# bytes per launch on the 64^3 shock pass: ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one launch of k_coarsen_screen_v<3> (overshoot
# check and quality screen, directions by rail length; per-face invariants,
# cubed tail, queued pairs, one pass over the local vertices per element;
# vertices taken 8 at a time, 1064 blocks of 128 threads, 7 per SM),
# profiles/coarsen_filter_box64_shock.md; to be captured again whenever that
# kernel changes
DOMINANT_TRAFFIC = 139600896 + 20408320
# FP64 add, multiply and fused multiply-add thread instructions per launch of
# the FP64 output kernels on the 64^3 shock box, all edges / all tets (ncu:
# smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum), for their
# FP64-pipe fraction against the measured FMA-chain rate (one such
# instruction per pipe slot)
FP64_OPS_PER_LAUNCH = {"lengths": 63905036 + 70059756 + 30746988,
                       "qualities": 117161842 + 138959394 + 40870410}
# Batched workload: 1024 independent 3D boxes, subdivisions per axis
# log-uniform integers in [4, 40] (seeded), isotropic sine metric with seeded
# h0, amplitude and wave vector per mesh
BATCH = {"workload": "batch1024_sine", "meshes": 1024, "n_min": 4, "n_max": 40, "seed": 7,
         "metric_kind": 3, "plain_sample": 64}


# Serving workload: Poisson arrivals; half 2D squares (n log-uniform in
# [16, 1024]), half 3D boxes (n log-uniform in [4, 64]); metric family
# uniform over isotropic sine, shock and boundary layer; 1 to 3 passes per
# request; 150 GB admission budget.  Requests arrive as box specifications:
# each mesh is built on the device when its request is admitted (served) or
# arrives (plain), inside its latency, and freed when it is done.  The
# default run serves the first requests of the seeded 20,000-request stream
# (the count per rate below; the saturating rate is last);
# --serve-requests 20000 serves the whole stream at the saturating rate.
SERVE = {"workload": "serve_mix", "stream_requests": 20000,
         "rates_per_s": [50.0, 200.0, 800.0], "requests_per_rate": [250, 1000, 2000],
         "budget_gb": 150.0, "seed": 11, "slots_per_dim": 4}


def serve_specs(sv=SERVE, count=None):
    """(dim, n, metric kind, seed, passes) of the seeded stream's first
    ``count`` requests, and their exponential inter-arrival gaps (unit mean)."""
    import numpy as np
    rng = np.random.default_rng(sv["seed"])
    out = []
    total = sv["stream_requests"]
    for _ in range(total):
        dim = 2 if rng.uniform() < 0.5 else 3
        lo, hi = (16, 1024) if dim == 2 else (4, 64)
        n = int(np.clip(np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1)))), lo, hi))
        kind = int(rng.choice([3, 1, 2]))
        out.append((dim, n, kind, int(rng.integers(1, 2 ** 31)), int(rng.integers(1, 4))))
    gaps = rng.exponential(1.0, total)
    count = total if count is None else count
    return out[:count], gaps[:count]


def batch_specs(b=BATCH):
    import numpy as np
    rng = np.random.default_rng(b["seed"])
    u = rng.uniform(np.log(b["n_min"]), np.log(b["n_max"] + 1), b["meshes"])
    ns = np.clip(np.floor(np.exp(u)).astype(int), b["n_min"], b["n_max"])
    seeds = rng.integers(1, 2 ** 31, b["meshes"])
    return [(int(n), int(s)) for n, s in zip(ns, seeds)]


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-workload leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-workload leg")
    ap.add_argument("--serve-slots", type=int, default=0,
                    help="serving contexts per dimension (default: SERVE['slots_per_dim'])")
    ap.add_argument("--serve-requests", type=int, default=0,
                    help="requests served at the saturating rate (default: the bounded "
                         "sample; 20000 serves the whole stream)")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the boundary-layer precision workloads")
    ap.add_argument("--no-tools", action="store_true", help="skip the .osh and metric tools")
    ap.add_argument("--no-autotune", action="store_true",
                    help="launch shapes at their defaults (no exploration passes)")
    ap.add_argument("--profile-pass", action="store_true",
                    help="build the workload, run one warm-up and one timed pass, exit "
                         "(for kernel launch lists under a profiler)")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _oracle_driver():
    path = os.path.join(ROOT, "oracle", "_build", "oracle_driver")
    if not os.path.exists(path):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j4"], check=True,
                       stdout=subprocess.DEVNULL)
    return path


def host_threads():
    """Host threads the CPU legs use: every core this process may run on."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _oracle_pass_seconds(n=None):
    """Times one pass of the oracle restatement (C++, OpenMP over the
    reference's parallel loops, all host threads) on the workload."""
    w = WORKLOAD
    env = dict(os.environ, OMP_NUM_THREADS=str(host_threads()))
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([_oracle_driver(), str(w["dim"]), str(n or w["n"]), str(w["metric_kind"]),
                            str(w["seed"]), str(w["min_quality_allowed"]), d, "time"],
                           capture_output=True, text=True, check=True, env=env)
    toks = r.stdout.split()
    return float(toks[toks.index("pass") + 1])


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    w = WORKLOAD
    for _ in range(args.warmup):
        _oracle_pass_seconds(n=8)  # small untimed warm-up of the same code
    times = [_oracle_pass_seconds() for _ in range(args.steps)]
    total = sum(times)
    value = w["elements"] * len(times) / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "elements/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {k: w[k] for k in ("workload", "dim", "n", "metric", "seed",
                                         "min_quality_allowed", "elements")},
            "cpu_baseline": {"value": value, "unit": "elements/s", "cores": host_threads(),
                             "kind": "port",
                             "sample": "one full adapt pass of the 64^3 shock box per step by the "
                                       "oracle restatement of the reference, its parallel loops "
                                       "on all host threads (OpenMP)"},
            "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# Precision workloads: boundary-layer metric (aspect up to 1000:1) on a 2D
# 1024^2 square (2,097,152 triangles) and a 3D 48^3 box (663,552 tets)
PRECISION = [{"workload": "sq1024_blayer", "dim": 2, "n": 1024, "metric_kind": 2, "seed": 3},
             {"workload": "box48_blayer", "dim": 3, "n": 48, "metric_kind": 2, "seed": 3}]


def precision_report(ctx, lib_stream, flush, m_base, opts):
    """One pass in FP64 throughout and one screened, from clones of m_base:
    pass times, screening counters and whether every output array is
    bitwise the same."""
    import torch
    from omega_h_gb300.mesh import Mesh

    def one(screening):
        ctx.set_screening(screening)
        ctx.screen_counts(reset=True)
        h = ctypes.c_void_p()
        _lib_call("ohg_mesh_clone", m_base.handle, ctypes.byref(h))
        mm = Mesh(ctx, h)
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        mm.adapt_pass(opts)
        e1.record(lib_stream)
        torch.cuda.synchronize()
        counts = ctx.screen_counts(reset=True)
        dg = hashlib.sha256()
        d = mm.dim
        for k in (f"ev2v_{d}", "coords", "metric", "length", "quality", f"class_id_{d}"):
            dg.update(mm.get(k).cpu().numpy().tobytes())
        mm.close()
        ctx.set_screening(True)
        return e0.elapsed_time(e1), counts, dg.hexdigest()

    one(True)  # warm
    fp64_ms, _, fp64_digest = one(False)
    scr_ms, counts, scr_digest = one(True)
    return {"fp64_pass_ms": fp64_ms, "screened_pass_ms": scr_ms,
            "elements_screened": counts[0], "elements_fp64": counts[1],
            "lengths_screened": counts[2], "lengths_fp64": counts[3],
            "element_recheck_fraction": counts[1] / max(counts[0], 1),
            "length_recheck_fraction": counts[3] / max(counts[2], 1),
            "max_error_vs_fp64": 0.0 if fp64_digest == scr_digest else None,
            "outputs_bitwise_equal_to_fp64": fp64_digest == scr_digest}


def run_tools(ctx, lib_stream, flush, base):
    """The tools beside the pass on the 64^3 shock mesh: one part of the
    reference's .osh format written and read back (the device arrays to and
    from the file), and the metric tools (implied metrics, an intersection,
    gradation limiting of the implied metrics, the expected element count,
    generate_metrics).  Each is timed once after one untimed run, with L2
    flushed before it."""
    import shutil
    import tempfile
    import torch
    out = {}

    def timed(fn):
        fn()
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, r

    from omega_h_gb300.mesh import Mesh, intersect_metrics

    def osh_timing():
        tmp = tempfile.mkdtemp(prefix="ohg_osh_")
        holder = []
        try:
            path = os.path.join(tmp, "box64.osh")
            ms_w, _ = timed(lambda: base.write_osh(path))
            nbytes = os.path.getsize(os.path.join(path, "0.osh"))

            def read():
                if holder:
                    holder.pop().close()
                holder.append(Mesh.read_osh(ctx, path))
            ms_r, _ = timed(read)
            return {"file_bytes": nbytes, "write_ms": ms_w, "read_ms": ms_r,
                    "write_gb_s": nbytes / ms_w / 1e6, "read_gb_s": nbytes / ms_r / 1e6,
                    "note": "uncompressed, to the box's local disk; includes the device<->host "
                            "copies of every array"}
        except Exception as e:  # reported, not fatal to the bench line
            return {"error": str(e)}
        finally:
            for h in holder:
                h.close()
            shutil.rmtree(tmp, ignore_errors=True)
    out["osh"] = osh_timing()
    # metric tools on a 64^3 box with the isotropic sine field: gradation's
    # stopping test (every tensor entry within 1e-3 relative, floor 1e-10)
    # settles on it, whereas on anisotropic metrics whose off-diagonal
    # entries sit just above the floor it can keep seeing rounding noise
    # (in the reference as here)
    m = Mesh.build_box(ctx, 3, 64)
    m.apply_workload(64, 5, 3)
    try:
        nv = m.nents(0)
        metric = m.get("metric")
        mt = {"workload": "box64_sine: 64^3 box, isotropic sine metric (seed 5)",
              "vertices": nv, "elements": m.nelems()}
        try:
            ms_i, implied = timed(lambda: m.implied_metrics())
            ms_x, _ = timed(lambda: intersect_metrics(ctx, 3, metric, implied))
            mt.update({"implied_ms": ms_i, "intersect_ms": ms_x,
                       "intersect_verts_per_s": nv / ms_x * 1e3})
            ms_g, (_, sweeps) = timed(lambda: m.limit_metric_gradation(metric, 1.0, 1e-3))
            mt.update({"gradation_ms": ms_g, "gradation_sweeps": sweeps,
                       "gradation_vert_sweeps_per_s": nv * sweeps / ms_g * 1e3})
            ms_n, ne = timed(lambda: m.expected_nelems(metric))
            mt.update({"expected_nelems_ms": ms_n, "expected_nelems": ne})
            ms_gen, (_, nit) = timed(lambda: m.generate_metrics(
                [{"type": "given", "metrics": metric},
                 {"type": "implied", "knob": 2.0, "isotropy": "iso_size", "scales": False}],
                should_limit_gradation=1, max_gradation_rate=1.0))
            mt.update({"generate_metrics_ms": ms_gen, "generate_metrics_iterations": nit})
        except Exception as e:  # reported, not fatal to the bench line
            mt["error"] = str(e)
        out["metric_tools"] = mt
    finally:
        m.close()
    return out


def run_precision(ctx, lib_stream, flush):
    from omega_h_gb300.mesh import Mesh, adapt_opts
    out = []
    for w in PRECISION:
        m = Mesh.build_box(ctx, w["dim"], w["n"])
        m.apply_workload(w["n"], w["seed"], w["metric_kind"])
        r = precision_report(ctx, lib_stream, flush, m, adapt_opts(w["dim"]))
        r.update({"workload": w["workload"], "elements": m.nelems()})
        m.close()
        out.append(r)
    return out


def run_batch(ctx, lib_stream, flush, args):
    """The batched workload as one union pass (timed over the pass only,
    inputs resident) against plain per-mesh passes on a sample of the same
    meshes; elements are those of the input meshes."""
    import torch
    from omega_h_gb300.mesh import Mesh, adapt_opts, adapt_pass_batch
    specs = batch_specs()
    opts = adapt_opts(3)
    base = []
    for n, seed in specs:
        m = Mesh.build_box(ctx, 3, n)
        m.apply_workload(n, seed, BATCH["metric_kind"])
        base.append(m)
    nel = sum(m.nelems() for m in base)

    def clones(ms):
        out = []
        for m in ms:
            h = ctypes.c_void_p()
            _lib_call("ohg_mesh_clone", m.handle, ctypes.byref(h))
            out.append(Mesh(ctx, h))
        return out

    def timed(fn):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        fn()
        e1.record(lib_stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    ms_batch = []
    for step in range(max(1, args.warmup) + 2):
        # the warm-up passes explore launch shapes for the union's sizes
        if not args.no_autotune:
            ctx.autotune("explore" if step < max(1, args.warmup) else "frozen")
        work = clones(base)
        t = timed(lambda: adapt_pass_batch(ctx, work, opts))
        if step >= max(1, args.warmup):
            ms_batch.append(t)
        for m in work:
            m.close()
    stride = max(1, len(base) // BATCH["plain_sample"])
    sample = base[::stride]
    nel_sample = sum(m.nelems() for m in sample)
    work = clones(sample)
    adapt_pass_batch(ctx, clones(sample[:2]), opts)  # warm
    ms_plain = timed(lambda: [m.adapt_pass(opts) for m in work])
    for m in work + base:
        m.close()
    batched = nel / (statistics.median(ms_batch) / 1e3)
    plain = nel_sample / (ms_plain / 1e3)
    return {"workload": BATCH["workload"], "meshes": len(base), "elements": nel,
            "metric_kind": "iso_sine", "batched_ms_per_pass": statistics.median(ms_batch),
            "batched_elements_per_s": batched,
            "plain_elements_per_s": plain,
            "plain_sample": {"meshes": len(sample), "elements": nel_sample, "ms": ms_plain},
            "batched_over_plain": batched / plain}


def run_serve(ctx, args, slots_per_dim=None):
    """The serving workload at each arrival rate: continuous batching against
    one request at a time, on the same requests and arrival times.  Each
    request's mesh is built on the device at admission (served) or arrival
    (plain) and freed when it is done.  Batching routes each request to one
    of slots_per_dim contexts of its dimension, each with its own step loop;
    admission counts device bytes measured by calibrate()."""
    import numpy as np
    from omega_h_gb300.mesh import Context
    from omega_h_gb300.serve import Request, calibrate, serve, serve_one_at_a_time, summary
    k = slots_per_dim or args.serve_slots or SERVE["slots_per_dim"]
    extra = [Context(ctx.device) for _ in range(2 * k - 1)]
    slots = {3: [ctx] + extra[:k - 1], 2: extra[k - 1:]}
    bpe, peak = calibrate({d: c[0] for d, c in slots.items()})
    counts = list(SERVE["requests_per_rate"])
    if args.serve_requests:
        counts = [min(c, args.serve_requests) for c in counts[:-1]] + [args.serve_requests]

    def stream(rate, count):
        specs, gaps = serve_specs(count=count)
        arr = np.cumsum(gaps) / rate
        arr -= arr[0]
        return [Request(rid=i, arrival=float(arr[i]), passes=p, dim=d, n=n, kind=kk, seed=sd)
                for i, (d, n, kk, sd, p) in enumerate(specs)]

    # warm both paths on a few requests
    serve(slots, stream(1e9, 6), bytes_per_element=bpe, pass_peak=peak, release=True)
    serve_one_at_a_time(ctx, stream(1e9, 6), release=True)
    rates = []
    for rate, count in zip(SERVE["rates_per_s"], counts):
        res = {"rate_per_s": rate, "requests": count}
        reqs = stream(rate, count)
        out = serve(slots, reqs, budget_bytes=SERVE["budget_gb"] * 1e9, bytes_per_element=bpe,
                    pass_peak=peak, release=True)
        res["served"] = summary(out)
        res["served"]["build_p50_ms"] = float(np.median([(r.built - r.admitted) * 1e3 for r in out]))
        reqs = stream(rate, count)
        out = serve_one_at_a_time(ctx, reqs, release=True)
        res["plain"] = summary(out)
        res["served_over_plain"] = res["served"]["elements_per_s"] / \
            max(res["plain"]["elements_per_s"], 1e-9)
        rates.append(res)
    for c in extra:
        c.close()
    return {"workload": SERVE["workload"], "stream_requests": SERVE["stream_requests"],
            "budget_gb": SERVE["budget_gb"], "slots_per_dim": k,
            "calibrated_bytes_per_element": bpe, "calibrated_pass_peak_over_resident": peak,
            "meshes": "built on the device at admission (served) or arrival (plain), freed "
                      "when done", "rates": rates}


def _lib_call(name, *a):
    from omega_h_gb300 import _lib
    return _lib.call(name, *a)


def run_ours(args):
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import omega_h_gb300.build as b
    if rank == 0:
        b.build()
    if world > 1:
        torch.distributed.barrier()
    from omega_h_gb300 import _lib
    from omega_h_gb300.mesh import Context, Mesh, adapt_opts
    w = WORKLOAD
    ctx = Context(local)
    sp = ctypes.c_void_p()
    _lib.call("ohg_context_stream", ctx.handle, ctypes.byref(sp))
    lib_stream = torch.cuda.ExternalStream(sp.value, device=dev)
    base = Mesh.build_box(ctx, w["dim"], w["n"])
    base.apply_workload(w["n"], w["seed"], w["metric_kind"])
    opts = adapt_opts(w["dim"], min_quality_allowed=w["min_quality_allowed"])
    nelems = base.nelems()
    assert nelems == w["elements"]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def clone(m):
        h = ctypes.c_void_p()
        _lib.call("ohg_mesh_clone", m.handle, ctypes.byref(h))
        return Mesh(ctx, h)

    def one_pass(timed):
        m = clone(base)
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        st = m.adapt_pass(opts)
        e1.record(lib_stream)
        torch.cuda.synchronize()
        m.close()
        return e0.elapsed_time(e1), st

    # ---- launch-shape autotuning: untimed passes in explore mode, then the
    # choices are frozen for everything that follows
    tune_passes = 0 if args.no_autotune else AUTOTUNE_PASSES
    if tune_passes:
        ctx.autotune("explore")
        for _ in range(tune_passes):
            one_pass(False)
        ctx.autotune("frozen")
    tuning = ctx.tuning()

    if args.profile_pass:
        one_pass(False)
        t, st = one_pass(True)
        print(json.dumps({"profile_pass_ms": t, "pass": st}), flush=True)
        base.close()
        ctx.close()  # with OHG_TRACE_SYNCS set, prints the host waits by call site
        return
    for _ in range(args.warmup):
        one_pass(False)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches()
    syncs0 = ctx.syncs()
    ms, stats = [], None
    ctx.kernel_time(DOMINANT, reset=True)
    ctx.time_kernels(True)  # events around the dominant kernel's launches
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t, stats = one_pass(True)
            ms.append(t)
    torch.cuda.synchronize()
    ctx.time_kernels(False)
    dom_ms, dom_bytes, dom_n = ctx.kernel_time(DOMINANT, reset=True)
    gpu_launches = ctx.launches() - launches0
    host_syncs = ctx.syncs() - syncs0
    total_ms = sum(ms)

    # ---- batched and served workloads
    batched = run_batch(ctx, lib_stream, flush, args) if rank == 0 and not args.no_batch else None
    served = run_serve(ctx, args) if rank == 0 and not args.no_serve else None

    # ---- .osh and metric tools
    tools = run_tools(ctx, lib_stream, flush, base) if rank == 0 and not args.no_tools else None

    # ---- precision mode: FP32 enclosures + FP64 recheck against FP64 throughout
    precision = precision_report(ctx, lib_stream, flush, base, opts)
    precision["workload"] = w["workload"]
    if rank == 0 and not args.no_precision:
        precision = [precision] + run_precision(ctx, lib_stream, flush)
    from omega_h_gb300.replicas import replica_throughput
    value, total_s = replica_throughput(nelems * args.steps, total_ms / 1e3, dev)
    total_ms = total_s * 1e3

    # ---- e2e through the C ABI from pinned host buffers
    names = ["down_1", "down_2", "downcodes_2", "down_3", "downcodes_3", "coords", "metric"] + \
            [f"class_dim_{d}" for d in range(4)] + [f"class_id_{d}" for d in range(4)]
    host = {k: base.get(k).cpu().pin_memory() for k in names}
    nents = (ctypes.c_int * 4)(*[base.nents(d) for d in range(4)])
    h2d = sum(t.numel() * t.element_size() for t in host.values())

    out_host = {}

    cnames = (ctypes.c_char_p * len(names))(*[k.encode() for k in names])

    def e2e_step():
        # the mesh straight from the pinned host arrays: the C ABI copies
        # them into its own device arrays
        P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        down = (ctypes.c_void_p * 4)(None, P(host["down_1"]), P(host["down_2"]), P(host["down_3"]))
        codes = (ctypes.c_void_p * 4)(None, None, P(host["downcodes_2"]), P(host["downcodes_3"]))
        cdim = (ctypes.c_void_p * 4)(*[P(host[f"class_dim_{d}"]) for d in range(4)])
        cid = (ctypes.c_void_p * 4)(*[P(host[f"class_id_{d}"]) for d in range(4)])
        h = ctypes.c_void_p()
        _lib.call("ohg_mesh_from_arrays", ctx.handle, 3, nents, down, codes, cdim, cid,
                  P(host["coords"]), P(host["metric"]), ctypes.byref(h))
        m = Mesh(ctx, h)
        m.adapt_pass(opts)
        # the result's arrays straight into pinned host buffers (allocated in
        # the warm-up steps, whose output sizes are the same), one call
        d2h = 0
        caps = (ctypes.c_longlong * len(names))()
        dsts = (ctypes.c_void_p * len(names))()
        for i, k in enumerate(names):
            nb = ctypes.c_longlong()
            _lib.call("ohg_mesh_array_bytes", m.handle, k.encode(), ctypes.byref(nb))
            buf = out_host.get(k)
            if buf is None or buf.numel() < nb.value:
                buf = torch.empty(nb.value, dtype=torch.uint8).pin_memory()
                out_host[k] = buf
            caps[i] = buf.numel()
            dsts[i] = buf.data_ptr()
            d2h += nb.value
        _lib.call("ohg_mesh_get_arrays", m.handle, len(names), cnames, dsts, caps)
        m.close()
        return d2h

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(args.steps):
        flush.fill_(1)
        d2h = e2e_step()
    torch.cuda.synchronize()
    e2e_value, e2e_s = replica_throughput(nelems * args.steps, time.perf_counter() - t0, dev)

    # ---- roofline: the pass's dominant kernel timed in the timed steps above
    # (CUDA events on the library stream around each launch), plus the
    # stage kernels each timed alone with L2 flushed before every launch
    peak, peak_kind = _peaks()
    dom_avg_ms = dom_ms / max(dom_n, 1)
    dom_bytes_launch = dom_bytes / max(dom_n, 1)
    achieved = dom_bytes_launch / (dom_avg_ms / 1e3) / 1e9 if dom_avg_ms > 0 else 0.0
    m = clone(base)
    kernels = {}
    fp64 = ctypes.c_double()
    _lib.call("ohg_fp64_peak", ctx.handle, 5, ctypes.byref(fp64))
    for stage in ("lengths", "qualities"):
        avg = ctypes.c_float()
        nb = ctypes.c_double()
        _lib.call("ohg_time_stage", m.handle, stage.encode(), 10, ctypes.byref(avg),
                  ctypes.byref(nb))
        kernels[stage] = {"ms": avg.value, "alg_bytes": nb.value,
                          "gbs": nb.value / (avg.value / 1e3) / 1e9 if avg.value > 0 else None,
                          "hbm_frac": (nb.value / (avg.value / 1e3) / 1e9) / peak
                          if avg.value > 0 else None}
        ops = FP64_OPS_PER_LAUNCH[stage]
        if avg.value > 0:
            rate = ops / (avg.value / 1e3) / 1e9  # G instructions / s
            kernels[stage].update({"fp64_ops_per_launch": ops, "fp64_gops": rate,
                                   "fp64_pipe_frac": rate / (fp64.value / 2.0)})
    kernels["fp64_peak_gflops"] = fp64.value
    kernels["fp64_peak_kind"] = ("measured in this run: chains of dependent FP64 FMAs; "
                                 "fp64_pipe_frac divides by half of it (FMA instructions/s)")
    m.close()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        t = _oracle_pass_seconds()
        cpu = {"value": w["elements"] / t, "unit": "elements/s", "cores": host_threads(),
               "kind": "port",
               "sample": "one full adapt pass of the 64^3 shock box (1,572,864 tets) by the "
                         "oracle restatement of the reference, parallel loops on all host "
                         "threads (OpenMP)"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {k: w[k] for k in ("workload", "dim", "n", "metric", "seed",
                                             "min_quality_allowed", "elements")} |
                          {"l2": "flushed (256 MiB write) before every timed step",
                           "parallelism": "replicas" if world > 1 else "single"},
                "pass": {k: stats[k] for k in ("did_refine", "did_coarsen", "did_swap",
                                               "nelems_out", "refine_keys", "coarsen_keys",
                                               "swap_keys", "indset_rounds", "ms_refine",
                                               "ms_coarsen", "ms_swap")},
                "e2e": {"value": e2e_value, "unit": "elements/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "roofline": {"kernel": DOMINANT, "bound": "hbm",
                             "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind,
                             "traffic": DOMINANT_TRAFFIC,
                             "algorithmic_bytes": dom_bytes_launch,
                             "avg_launch_ms": dom_avg_ms, "launches": dom_n,
                             "note": "FP32 enclosure arithmetic bounds this kernel (instruction "
                                     "issue), not HBM; traffic from one ncu capture of it on "
                                     "this workload",
                             "stages": kernels},
                "precision": precision,
                "batched": batched,
                "served": served,
                "tools": tools,
                "cpu_baseline": cpu, "gpu_launches": gpu_launches,
                "host_syncs_per_step": host_syncs / args.steps, "clocks": clk.summary(),
                "autotune": {"passes": tune_passes, "sites": tuning[0], "chosen": tuning[1],
                             "non_default": tuning[2]}}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def main():
    args = _args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
