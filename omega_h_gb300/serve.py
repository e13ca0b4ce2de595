"""Serving loop for adapt-pass requests with continuous batching.

A request names a mesh (a box of given dimension and subdivisions with a
seeded metric family, or a mesh already on the device) and a number of
passes.  Requests arrive over time.  The loop admits them in arrival order
while their device footprint fits the admission budget and routes each to a
slot of its dimension: a context (one stream) with its own step loop on its
own host thread (slots that share a context share its thread, since a
context is driven by one thread at a time).  A slot builds the meshes of
newly routed requests on the device, then runs one adapt pass over the
disjoint union of all its requests (ohg_adapt_pass_batch), and repeats:
requests routed while a step runs join that slot's next step, finished
requests leave and free their memory at once.  Slots on different contexts
do not wait for one another, so a long 3D union does not hold back the 2D
slots.  Because a union pass is bit for bit the
separate passes, a request's result does not depend on what it was batched
with.  The library's calls release the interpreter lock, so the slots' work
overlaps on the device.

Admission counts device bytes.  Before a mesh exists its footprint is
estimated from a per-element figure measured on the device (``calibrate``:
the memory pool's high-water mark over one build and pass); once the slot
has built it, the reservation becomes the mesh's own device bytes scaled by
the measured ratio of a pass's peak to the resident mesh.  A request is
admitted while the larger of the reservations and the pool's bytes in use,
plus its estimate, stays within the budget.

``serve_one_at_a_time`` runs the same stream with one request on the device
at a time and no batching, the baseline the batched loop is measured
against.  Its latencies include the same mesh builds.
"""
import threading
import time
from dataclasses import dataclass, field

from .mesh import Mesh, adapt_opts, adapt_pass_batch

# device bytes per element (build and pass peak) used until calibrate()
# has measured them; upper estimates
BYTES_PER_ELEMENT = {2: 1200, 3: 2400}
# peak bytes of a pass over resident bytes, used until calibrate() measures it
PASS_PEAK_OVER_RESIDENT = {2: 2.5, 3: 2.5}


@dataclass
class Request:
    rid: int
    arrival: float  # seconds from the start of the stream
    passes: int
    dim: int = 0
    n: int = 0      # subdivisions per axis of the box to build
    kind: int = 0   # metric family of the box (the library's workload kinds)
    seed: int = 0
    mesh: object = None  # omega_h_gb300.mesh.Mesh: given, or built on admission
    slot: int = -1
    elements_in: int = 0
    admitted: float = -1.0
    built: float = -1.0
    done: float = -1.0
    reserved: int = 0  # bytes held from admission to completion
    passes_done: int = 0
    element_passes: int = 0
    stats: list = field(default_factory=list)

    def elements(self):
        if self.mesh is not None:
            return self.mesh.nelems()
        return 2 * self.n * self.n if self.dim == 2 else 6 * self.n ** 3

    def build(self, ctx):
        m = Mesh.build_box(ctx, self.dim, self.n)
        m.apply_workload(self.n, self.seed, self.kind)
        self.mesh = m


def route(dims, work, slots):
    """Slot index for each request (in arrival order): the slot of the
    request's dimension with the least work routed to it so far.  ``slots``
    maps a dimension to its number of slots."""
    load = {d: [0.0] * k for d, k in slots.items()}
    out = []
    for d, w in zip(dims, work):
        i = min(range(slots[d]), key=lambda j: load[d][j])
        load[d][i] += w
        out.append(i)
    return out


def calibrate(ctxs, sizes=None):
    """Measures, per dimension, the device bytes per element of a mesh's build
    and pass (the memory pool's high-water mark above its use before) and the
    ratio of a pass's peak to the resident mesh.  ctxs maps a dimension to a
    context.  Returns (bytes_per_element, pass_peak_over_resident)."""
    sizes = sizes or {2: 256, 3: 24}
    bpe, peak = {}, {}
    for d, ctx in ctxs.items():
        r = Request(rid=-1, arrival=0.0, passes=1, dim=d, n=sizes[d], kind=1, seed=1)
        used0, _, _ = ctx.pool_bytes(reset_high=True)
        r.build(ctx)
        resident = r.mesh.device_bytes()
        r.mesh.adapt_pass(adapt_opts(d))
        _, _, high = ctx.pool_bytes()
        n = r.elements()
        bpe[d] = max(1.0, (high - used0) / n)
        peak[d] = max(1.0, (high - used0) / max(resident, 1))
        r.mesh.close()
    return bpe, peak


class _Slot:
    def __init__(self, ctx, dim, index):
        self.ctx, self.dim, self.index = ctx, dim, index
        self.inbox = []
        self.active = []
        self.work = 0.0  # element-passes routed and not finished


def serve(slots, requests, budget_bytes=150e9, opts=None, clock=time.perf_counter,
          bytes_per_element=None, pass_peak=None, release=False, trace=None):
    """Continuous batching.  slots maps a dimension to its contexts (one step
    loop each).  Returns the requests with admitted/built/done times (seconds
    from the stream start), per-pass union stats and their slot.  release:
    free each finished request's mesh at once (else it stays with the
    request for the caller to read and close; its reservation ends either
    way).  trace, if a list, receives (seconds, bytes reserved, pool bytes in
    use) at each admission.  A request whose estimate alone exceeds the
    budget raises ValueError."""
    bpe = bytes_per_element or BYTES_PER_ELEMENT
    peak = pass_peak or PASS_PEAK_OVER_RESIDENT
    reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
    for r in reqs:
        if r.mesh is not None:
            r.dim = r.mesh.dim
        r.elements_in = r.elements()
    all_slots = {d: [_Slot(c, d, i) for i, c in enumerate(cs)] for d, cs in slots.items()}
    any_ctx = next(iter(slots.values()))[0]
    cv = threading.Condition()
    state = {"reserved": 0, "admitting": True, "error": None}
    t0 = clock()

    def estimate(r):
        return int(bpe[r.dim] * r.elements_in)

    def step(s, new):
        """Builds a slot's new meshes, then one union pass over its requests."""
        o = opts[s.dim] if opts else adapt_opts(s.dim)
        for r in new:
            if r.mesh is None:
                r.build(s.ctx)
            r.built = clock() - t0
            actual = int(r.mesh.device_bytes() * peak[s.dim])
            with cv:
                state["reserved"] += actual - r.reserved
                r.reserved = actual
                cv.notify_all()
        s.active.extend(new)
        if not s.active:
            return
        n_before = [r.mesh.nelems() for r in s.active]
        st = adapt_pass_batch(s.ctx, [r.mesh for r in s.active], o)
        still, finished = [], []
        for r, nb in zip(s.active, n_before):
            r.passes_done += 1
            r.element_passes += nb
            r.stats.append(st)
            if r.passes_done >= r.passes:
                r.done = clock() - t0
                finished.append(r)
                if release:
                    r.mesh.close()
                    r.mesh = None
            else:
                still.append(r)
        s.active = still
        with cv:
            for r in finished:
                state["reserved"] -= r.reserved
                s.work -= r.elements_in * r.passes
            cv.notify_all()

    def run_worker(slist):
        # one host thread per context: a context's stream, status word and
        # memory are driven by one thread at a time; slots of different
        # dimensions that share a context take their steps in turn
        try:
            while True:
                with cv:
                    while not any(x.inbox or x.active for x in slist) and \
                            state["admitting"] and state["error"] is None:
                        cv.wait()
                    if state["error"] is not None:
                        return
                    if not any(x.inbox or x.active for x in slist):
                        return
                    news = []
                    for x in slist:
                        news.append(x.inbox)
                        x.inbox = []
                for x, new in zip(slist, news):
                    step(x, new)
        except BaseException as e:  # noqa: BLE001 - reported to the caller
            with cv:
                state["error"] = e
                cv.notify_all()

    workers = {}
    for ss in all_slots.values():
        for x in ss:
            workers.setdefault(id(x.ctx), []).append(x)
    threads = [threading.Thread(target=run_worker, args=(sl,), daemon=True)
               for sl in workers.values()]
    for th in threads:
        th.start()
    try:
        for r in reqs:
            est = estimate(r)
            if est > budget_bytes:
                raise ValueError(f"request {r.rid} alone exceeds the admission budget")
            now = clock() - t0
            if r.arrival > now:
                time.sleep(r.arrival - now)
            with cv:
                while state["error"] is None:
                    used, _, _ = any_ctx.pool_bytes()
                    if max(state["reserved"], used) + est <= budget_bytes or \
                            state["reserved"] == 0:
                        break
                    cv.wait(timeout=0.005)
                if state["error"] is not None:
                    break
                cands = all_slots[r.dim]
                if r.mesh is not None:  # a resident mesh stays on its context
                    cands = [x for x in cands if x.ctx is r.mesh.ctx]
                    if not cands:
                        raise ValueError(f"request {r.rid}: its mesh is on no serving slot")
                s = min(cands, key=lambda x: x.work)
                s.work += r.elements_in * r.passes
                r.slot = s.index
                r.admitted = clock() - t0
                r.reserved = est
                state["reserved"] += est
                if trace is not None:
                    trace.append((r.admitted, state["reserved"], used))
                s.inbox.append(r)
                cv.notify_all()
    finally:
        with cv:
            state["admitting"] = False
            cv.notify_all()
        for th in threads:
            th.join()
    if state["error"] is not None:
        raise state["error"]
    return reqs


def serve_one_at_a_time(ctx, requests, opts=None, clock=time.perf_counter, release=False):
    """The same stream, one request at a time on one context: built on
    arrival (or given), each pass run on its own; freed when done if
    release."""
    reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
    t0 = clock()
    for r in reqs:
        now = clock() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.admitted = clock() - t0
        if r.mesh is None:
            r.build(ctx)
        r.dim = r.mesh.dim
        r.elements_in = r.mesh.nelems()
        r.built = clock() - t0
        o = opts[r.dim] if opts else adapt_opts(r.dim)
        for _ in range(r.passes):
            nb = r.mesh.nelems()
            r.stats.append(r.mesh.adapt_pass(o))
            r.passes_done += 1
            r.element_passes += nb
        r.done = clock() - t0
        if release:
            r.mesh.close()
            r.mesh = None
    return reqs


def summary(reqs):
    """p50/p99 latency (arrival to completion, ms) and element-passes per
    second over the whole stream."""
    lat = sorted((r.done - r.arrival) * 1e3 for r in reqs)

    def pct(p):
        if not lat:
            return 0.0
        i = min(len(lat) - 1, max(0, int(round(p / 100.0 * (len(lat) - 1)))))
        return lat[i]

    span = max(r.done for r in reqs) - min(r.arrival for r in reqs) if reqs else 0.0
    ep = sum(r.element_passes for r in reqs)
    return {"requests": len(reqs), "p50_ms": pct(50), "p99_ms": pct(99),
            "element_passes": ep, "elements_per_s": ep / span if span > 0 else 0.0,
            "span_s": span}
