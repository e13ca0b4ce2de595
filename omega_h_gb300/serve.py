"""Serving loop for adapt-pass requests with continuous batching.

Requests arrive over time, each with a device-resident mesh and a number of
passes.  The loop admits arrived requests in arrival order while their
estimated device footprint fits the admission budget, and every step runs one
adapt pass over the disjoint union of all admitted requests of a dimension
(ohg_adapt_pass_batch): requests that arrive while a step runs join the next
step, finished requests leave and free their memory.  Because a union pass is
bit for bit the separate passes, a request's result does not depend on what
it was batched with.

Each request's mesh lives on a context (a slot: one stream and its memory
pool on the device), chosen when the request is routed; ``route`` spreads a
stream of requests over the slots of each dimension by the work already sent
to each.  A step runs one union pass per slot that holds admitted requests,
all slots at once from a pool of host threads (the library's calls release
the interpreter lock), so the slots' passes overlap on the device.

``serve_one_at_a_time`` runs the same stream with one request on the device
at a time and no batching, the baseline the batched loop is measured against.
"""
import concurrent.futures
import time
from dataclasses import dataclass, field

from .mesh import adapt_opts, adapt_pass_batch

# device bytes per element while a mesh is resident and during its pass:
# arrays of the mesh and its derived adjacencies plus the pass's temporaries
# (upper estimates; 3D tets carry about 3x the adjacency of 2D triangles)
BYTES_PER_ELEMENT = {2: 1200, 3: 2400}


@dataclass
class Request:
    rid: int
    arrival: float  # seconds from the start of the stream
    mesh: object  # omega_h_gb300.mesh.Mesh, resident on the device
    passes: int
    dim: int = 0
    elements_in: int = 0
    admitted: float = -1.0
    done: float = -1.0
    reserved: int = 0  # footprint held from admission to completion
    passes_done: int = 0
    element_passes: int = 0
    stats: list = field(default_factory=list)

    def footprint(self):
        return BYTES_PER_ELEMENT[self.dim] * max(self.elements_in, self.mesh.nelems())


def _prepare(reqs):
    for r in reqs:
        r.dim = r.mesh.dim
        r.elements_in = r.mesh.nelems()
    return sorted(reqs, key=lambda r: (r.arrival, r.rid))


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


def serve(ctx, requests, budget_bytes=150e9, opts=None, clock=time.perf_counter):
    """Continuous batching.  Returns the requests with admitted/done times
    (seconds from the stream start) and per-pass union stats.  The slots are
    the contexts of the requests' meshes (``ctx`` is kept for callers that
    pass one; the meshes decide)."""
    reqs = _prepare(requests)
    slots = []
    for r in reqs:
        if not any(r.mesh.ctx is c for c in slots):
            slots.append(r.mesh.ctx)
    pool = concurrent.futures.ThreadPoolExecutor(len(slots)) if len(slots) > 1 else None

    def run_group(dim, group):
        o = opts[dim] if opts else adapt_opts(dim)
        n_before = [r.mesh.nelems() for r in group]
        st = adapt_pass_batch(group[0].mesh.ctx, [r.mesh for r in group], o)
        for r, nb in zip(group, n_before):
            r.passes_done += 1
            r.element_passes += nb
            r.stats.append(st)

    t0 = clock()
    pending = list(reqs)
    active = []
    used = 0
    while pending or active:
        now = clock() - t0
        # admit arrived requests in order while they fit
        while pending and pending[0].arrival <= now and used + pending[0].footprint() <= budget_bytes:
            r = pending.pop(0)
            r.admitted = now
            r.reserved = r.footprint()
            used += r.reserved
            active.append(r)
        if pending and pending[0].arrival <= now and not active and \
                pending[0].footprint() > budget_bytes:
            raise ValueError(f"request {pending[0].rid} alone exceeds the admission budget")
        if not active:
            time.sleep(max(0.0, pending[0].arrival - now))
            continue
        groups = []
        for c in slots:
            for d in (2, 3):
                g = [r for r in active if r.mesh.ctx is c and r.dim == d]
                if g:
                    groups.append((d, g))
        if pool and len(groups) > 1:
            for f in [pool.submit(run_group, d, g) for d, g in groups]:
                f.result()
        else:
            for d, g in groups:
                run_group(d, g)
        now = clock() - t0
        still = []
        for r in active:
            if r.passes_done >= r.passes:
                r.done = now
                used -= r.reserved
            else:
                still.append(r)
        active = still
    if pool:
        pool.shutdown()
    return reqs


def serve_one_at_a_time(ctx, requests, opts=None, clock=time.perf_counter):
    """The same stream, one request at a time, each pass run on its own."""
    reqs = _prepare(requests)
    t0 = clock()
    for r in reqs:
        now = clock() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.admitted = clock() - t0
        o = opts[r.dim] if opts else adapt_opts(r.dim)
        for _ in range(r.passes):
            nb = r.mesh.nelems()
            r.stats.append(r.mesh.adapt_pass(o))
            r.passes_done += 1
            r.element_passes += nb
        r.done = clock() - t0
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
