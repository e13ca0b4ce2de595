"""Runs the GPU library on a seeded box workload through the C ABI and
returns the same named per-stage arrays the reference dump driver and the
oracle driver write, as numpy arrays.  Stage inputs (candidate lists, codes)
are assembled from the library's own earlier outputs exactly as the
reference operators chain them.
"""
import ctypes

import numpy as np
import torch

from omega_h_gb300 import _lib
from omega_h_gb300.mesh import Context, Mesh, adapt_opts

def mesh_arrays(dim):
    names = ["coords", "metric", "down_1", "ev2v_2", "down_2", "downcodes_2"]
    if dim == 3:
        names += ["ev2v_3", "down_3", "downcodes_3"]
    return names + [f"class_dim_{d}" for d in range(dim + 1)] + \
        [f"class_id_{d}" for d in range(dim + 1)]


def adj_arrays(dim):
    names = [f"up_{k}_{lo}{hi}" for lo in range(dim) for hi in range(lo + 1, dim + 1)
             for k in ("a2ab", "ab2b", "codes")]
    if dim == 3:
        names += ["down31", "downcodes31"]
    return names + ["star_a2ab_0", "star_ab2b_0", "star_a2ab_1", "star_ab2b_1", "dual_a2ab",
                    "dual_ab2b"]


def np_(t):
    return t.detach().cpu().numpy()


def dump_mesh(m, prefix, out, with_length=False, with_quality=False):
    out[prefix + "nents"] = np.array([float(m.nents(0))])
    for name in mesh_arrays(m.dim):
        out[prefix + name] = np_(m.get(name))
    if with_length:
        out[prefix + "length"] = np_(m.get("length"))
    if with_quality:
        out[prefix + "quality"] = np_(m.get("quality"))


def hilbert_perm(ctx, coords, dim):
    perm = torch.empty(coords.numel() // dim, dtype=torch.int32, device=coords.device)
    _lib.call("ohg_hilbert_sort", ctx.handle, ctypes.c_void_p(coords.data_ptr()),
              perm.numel(), dim, ctypes.c_void_p(perm.data_ptr()))
    return perm


def refine_stage(m, o, out):
    lengths = m.get("length")
    cands = (lengths > o.max_length_desired).to(torch.int8)
    out["r_cands"] = np_(cands)
    if not bool(cands.any()):
        return
    c2e = torch.nonzero(cands).flatten().to(torch.int32)
    out["r_cands2edges"] = np_(c2e)
    out["r_midmetrics"] = np_(m.mident_metrics(c2e))
    cq = m.refine_qualities(c2e)
    out["r_cand_quals"] = np_(cq)
    good = cq >= o.min_quality_allowed
    if not bool(good.any()):
        return
    ne = m.nents(1)
    init = torch.zeros(ne, dtype=torch.int8, device=lengths.device)
    eq = torch.zeros(ne, dtype=torch.float64, device=lengths.device)
    init[c2e.long()] = good.to(torch.int8)
    eq[c2e.long()] = cq
    keys, _ = m.find_indset(1, eq, init)
    out["r_keys"] = np_(keys)


def coarsen_stage(m, o, out):
    dev = f"cuda:{m.ctx.device}"
    lengths = m.get("length")
    ec = (lengths < o.min_length_desired).to(torch.int8)
    out["c_edge_is_cand"] = np_(ec)
    if not bool(ec.any()):
        return
    ev = m.get("down_1").long().view(-1, 2)
    vm = torch.zeros(m.nents(0), dtype=torch.int8, device=dev)
    idx = torch.nonzero(ec).flatten()
    vm[ev[idx, 0]] = 1
    vm[ev[idx, 1]] = 1
    out["c_vert_marks"] = np_(vm)
    codes_e = (vm[ev[:, 0]].to(torch.int32) | (vm[ev[:, 1]].to(torch.int32) << 1)).to(torch.int8)
    out["c_edge_codes"] = np_(codes_e)
    c2e = torch.nonzero(codes_e).flatten().to(torch.int32)
    codes = m.check_collapse_class(c2e, codes_e[c2e.long()].contiguous())
    out["c_class_codes"] = np_(codes)
    if int(codes.max()) <= 0:
        return
    keep = codes != 0
    c2e, codes = c2e[keep].contiguous(), codes[keep].contiguous()
    out["c_cands2edges0"] = np_(c2e)
    codes = m.check_collapse_exposure(c2e, codes)
    out["c_expo_codes"] = np_(codes)
    keep = codes != 0
    c2e, codes = c2e[keep].contiguous(), codes[keep].contiguous()
    out["c_cands2edges1"] = np_(c2e)
    codes = m.prevent_coarsen_overshoot(o.max_length_desired, c2e, codes)
    out["c_over_codes"] = np_(codes)
    keep = codes != 0
    c2e, codes = c2e[keep].contiguous(), codes[keep].contiguous()
    out["c_cands2edges2"] = np_(c2e)
    if c2e.numel() == 0:
        return
    q2 = m.coarsen_qualities(c2e, codes)
    out["c_quals"] = np_(q2)
    ok = (q2.view(-1, 2) >= o.min_quality_allowed)
    codes = (codes.to(torch.int32) & (ok[:, 0].to(torch.int32) | (ok[:, 1].to(torch.int32) << 1))).to(torch.int8)
    out["c_minq_codes"] = np_(codes)
    keep = codes != 0
    c2e, codes = c2e[keep].contiguous(), codes[keep].contiguous()
    q2 = q2.view(-1, 2)[keep].contiguous().flatten()
    out["c_cands2edges3"] = np_(c2e)
    out["c_cand_codes3"] = np_(codes)
    if c2e.numel() == 0:
        return
    vc, vq, vr = m.choose_rails(c2e, codes, q2)
    out["c_verts_are_cands"] = np_(vc)
    out["c_vert_quals"] = np_(vq)
    out["c_vert_rails"] = np_(vr)
    keys, _ = m.find_indset(0, vq, vc)
    out["c_keys"] = np_(keys)


def swap_stage(m, o, out):
    ec = m.mark_sliver_layers(o.min_quality_desired, o.nsliver_layers)
    out["s_elem_cands"] = np_(ec)
    dim = m.dim
    a2ab = m.get(f"up_a2ab_1{dim}").long()
    ab2b = m.get(f"up_ab2b_1{dim}").long()
    deg = a2ab[1:] - a2ab[:-1]
    owner = torch.repeat_interleave(torch.arange(deg.numel(), device=deg.device), deg)
    edc = torch.zeros(m.nents(1), dtype=torch.int32, device=deg.device)
    edc.index_reduce_(0, owner, ec[ab2b].to(torch.int32), "amax", include_self=True)
    edc = ((edc > 0) & (m.get("class_dim_1") == dim)).to(torch.int8)
    out["s_edge_cands"] = np_(edc)
    if not bool(edc.any()):
        return
    c2e = torch.nonzero(edc).flatten().to(torch.int32)
    if dim == 3:
        q, cf = m.swap3d_qualities(o.max_length_allowed, c2e)
        out["s_cand_configs"] = np_(cf)
    else:
        q = m.swap2d_qualities(o.max_length_allowed, c2e)
    out["s_cands2edges"] = np_(c2e)
    out["s_cand_quals"] = np_(q)


def run(dim, n, kind, seed, mqa, stages=True, device=0):
    """Returns (arrays, pass flags) of one adapt pass on the GPU."""
    ctx = Context(device)
    out = {}
    m = Mesh.build_box(ctx, dim, n)
    m.apply_workload(n, seed, kind)
    o = adapt_opts(dim, min_quality_allowed=mqa)
    if stages:
        dump_mesh(m, "in_", out)
        for name in adj_arrays(dim):
            out["in_" + name] = np_(m.get(name))
        out["in_length_fresh"] = np_(m.measure_edges_metric())
        out["in_quality_fresh"] = np_(m.measure_qualities())
        out["in_hilbert_perm"] = np_(hilbert_perm(ctx, m.get("coords"), dim))
        refine_stage(m, o, out)
    did_r = m.refine_by_size(o)
    if stages:
        dump_mesh(m, "r_out_", out, with_length=True)
        coarsen_stage(m, o, out)
    did_c = m.coarsen_by_size(o)
    if stages:
        dump_mesh(m, "c_out_", out, with_length=True)
    minq = float(m.get("quality").min())
    did_s = False
    if minq < o.min_quality_desired:
        if stages:
            swap_stage(m, o, out)
        did_s = m.swap_edges(o)
    out["pass_flags"] = np.array([did_r, did_c, did_s], dtype=np.int32)
    dump_mesh(m, "out_", out, with_length=True, with_quality=True)
    m.close()
    ctx.close()
    return out
