"""Spatial queries over the range bounds (src/kd_tree.py) on the GPU.

``construct_uniform_unknown_levelset_tree``, ``hierarchical_marching_cubes``,
``find_any_intersection`` and ``closest_point`` keep the reference's signatures and
return NumPy arrays.  Results that the reference returns in bucket-padded arrays with a
``valid`` mask are returned at their exact size with an all-True mask, so the usual
``lower[valid]`` idiom still works.
"""
from __future__ import annotations

import numpy as np

from . import _io, _lib
from .mlp import device_model

_TREE_CAP0 = 1 << 20
# node capacity that last sufficed, per (model blob, split depth, threshold, flags, offset):
# repeated queries start there instead of failing and retrying from the default
_TREE_CAP_SEEN = {}


def _host3(x):
    a = np.asarray(x.detach().cpu().numpy() if hasattr(x, 'detach') else x, np.float32).reshape(3)
    return (_lib.C.c_float * 3)(*a.tolist())


GROWING_MODES = ('affine_truncate', 'affine_append', 'affine_all')


def _tree_device(func, params, lower, upper, split_depth, node_terminate_thresh, flags, offset, persistent,
                 batch_process_size=2048):
    """Runs the tree on the device; returns (workspace tensor, capacity, counts, model).
    ``persistent``: True (one cooperative launch), False (one launch per level) or
    'batches' (the reference's schedule: launches of ``batch_process_size`` nodes)."""
    t = _io.require_cuda()
    m = device_model(params)
    bo = func.bound_opts()
    L = _lib.load()
    cap = _TREE_CAP0
    if split_depth is not None:
        cap = max(64, min(cap, 2 ** (split_depth + 1)))
    key = (m.fingerprint, split_depth, node_terminate_thresh, flags, float(offset), bo.mode, bo.conservative)
    cap = max(cap, _TREE_CAP_SEEN.get(key, 0))
    growing = func.mode in GROWING_MODES
    if growing:
        # the growing-term modes: the level loop over the growing-term engine (every schedule)
        fn = L.niq_levelset_tree_growing
    elif persistent == 'batches':
        B = int(batch_process_size)

        def fn(*a):
            return L.niq_levelset_tree_batches(*a[:8], B, *a[8:])
    else:
        fn = L.niq_levelset_tree if persistent else L.niq_levelset_tree_plain
    while True:
        ws_bytes = (L.niq_tree_growing_workspace_size(m.handle, _lib.C.byref(bo), cap, flags) if growing
                    else L.niq_tree_workspace_size(cap, flags))
        ws = t.empty(ws_bytes, dtype=t.uint8, device='cuda')
        counts = t.zeros(4, dtype=t.int64, device='cuda')
        try:
            _lib.check(fn(m.handle, _lib.C.byref(bo), _host3(lower), _host3(upper),
                          -1 if split_depth is None else int(split_depth),
                          0 if node_terminate_thresh is None else int(node_terminate_thresh), float(offset), flags,
                          cap, _io.ptr(counts), _io.ptr(ws), ws_bytes, _io.stream_handle()))
            _TREE_CAP_SEEN[key] = cap
            return ws, cap, counts.cpu().numpy(), m
        except _lib.NIQCapacityError:
            del ws
            cap *= 4
            if cap > (1 << 31):
                raise


def _tree_nodes(ws, cap, flags, kind, count):
    t = _io.torch()
    lo = _lib.C.c_void_p()
    hi = _lib.C.c_void_p()
    _lib.check(_lib.load().niq_tree_result(_io.ptr(ws), cap, flags, kind, _lib.C.byref(lo), _lib.C.byref(hi)))
    base = ws.data_ptr()
    flat = ws.view(t.float32) if ws.numel() % 4 == 0 else None
    off_lo = (lo.value - base) // 4
    off_hi = (hi.value - base) // 4
    lo_t = flat[off_lo:off_lo + 3 * count].view(count, 3)
    hi_t = flat[off_hi:off_hi + 3 * count].view(count, 3)
    return lo_t, hi_t


def construct_uniform_unknown_levelset_tree(func, params, lower, upper, node_terminate_thresh=None, split_depth=None,
                                            compress_after=False, with_childern=False, with_interior_nodes=False,
                                            with_exterior_nodes=False, offset=0., batch_process_size=2048,
                                            persistent=True):
    """src/kd_tree.py:103-218.  Adds key ``n_boxes_classified``.  ``persistent``: True
    runs every level in one cooperative launch; False one launch per level; 'batches'
    the reference's own schedule, one launch per ``batch_process_size`` nodes."""
    if node_terminate_thresh is None and split_depth is None:
        raise ValueError("must specify at least one of node_terminate_thresh or split_depth as a terminating condition")
    flags = (1 if with_interior_nodes else 0) | (2 if with_exterior_nodes else 0)
    ws, cap, counts, _ = _tree_device(func, params, lower, upper, split_depth, node_terminate_thresh, flags, offset,
                                      persistent, batch_process_size)
    out = {'n_boxes_classified': int(counts[3])}
    for kind, name, on in ((0, 'unknown', True), (1, 'interior', with_interior_nodes),
                           (2, 'exterior', with_exterior_nodes)):
        if not on:
            continue
        n = int(counts[kind])
        lo, hi = _tree_nodes(ws, cap, flags, kind, n)
        out[f'{name}_node_valid'] = np.ones(n, bool)
        out[f'{name}_node_lower'] = lo.cpu().numpy()
        out[f'{name}_node_upper'] = hi.cpu().numpy()
    return out


def hierarchical_marching_cubes(func, params, lower, upper, depth, n_subcell_depth=2,
                                extract_batch_max_tri_out=1000000, persistent=True, shared_corners=True):
    """src/kd_tree.py:357-399: the tree to split depth 3*(depth - n_subcell_depth), then
    marching cubes on a (2^n_subcell_depth)^3 grid in every unknown leaf.  Returns
    (T, 3, 3) float32 triangles (order differs from the reference's).  With
    n_subcell_depth = 0, ``shared_corners`` evaluates each lattice corner once for all
    the leaves that share it (same triangles)."""
    t = _io.require_cuda()
    k = int(n_subcell_depth)
    ws, cap, counts, m = _tree_device(func, params, lower, upper, 3 * (depth - k), None, 0, 0., persistent)
    n_leaves = int(counts[0])
    if n_leaves == 0:
        return np.zeros((0, 3, 3), np.float32)
    lo, hi = _tree_nodes(ws, cap, 0, 0, n_leaves)
    lo, hi = lo.contiguous(), hi.contiguous()
    L = _lib.load()
    tri_cap = max(1024, n_leaves * (8 ** k) * 2)
    # the leaves are one lattice's cells: with k = 0, shared corners are evaluated once
    lattice = k == 0 and bool(shared_corners)
    rl, ru = _host3(lower), _host3(upper)
    S = 3 * (depth - k)
    if lattice:
        hws_bytes = L.niq_hmc_lattice_workspace_size(rl, ru, S, n_leaves)
        lattice = hws_bytes > 0 and hws_bytes < (8 << 30)
    if not lattice:
        hws_bytes = L.niq_hmc_workspace_size()
    hws = t.empty(hws_bytes, dtype=t.uint8, device='cuda')
    while True:
        tris = t.empty((tri_cap, 3, 3), dtype=t.float32, device='cuda')
        n_t = t.zeros(1, dtype=t.int64, device='cuda')
        try:
            if lattice:
                _lib.check(L.niq_hmc_extract_lattice(m.handle, n_leaves, _io.ptr(lo), _io.ptr(hi), rl, ru, S,
                                                     _io.ptr(tris), tri_cap, _io.ptr(n_t), _io.ptr(hws), hws_bytes,
                                                     _io.stream_handle()))
            else:
                _lib.check(L.niq_hmc_extract(m.handle, n_leaves, _io.ptr(lo), _io.ptr(hi), k, _io.ptr(tris), tri_cap,
                                             _io.ptr(n_t), _io.ptr(hws), hws_bytes, _io.stream_handle()))
            break
        except _lib.NIQCapacityError:
            tri_cap = int(n_t.item()) + 1
    return tris[:int(n_t.item())].cpu().numpy()


def find_any_intersection(func_tuple, params_tuple, lower, upper, eps, viz_nodes=False, max_nodes=1 << 26):
    """src/kd_tree.py:567-655: ``(found, 1, 2, loc)``, or ``(False, 0, 0, (-777,)*3)``.
    The witness ``loc`` is a sample point inside both shapes (or the midpoint of two
    negative samples in an eps-small node); which witness is returned may differ from
    the reference's, the verdict does not.  ``viz_nodes`` is not supported.  A search
    level may hold up to ``max_nodes`` nodes (the workspace grows up to that); beyond it
    the call raises NIQCapacityError."""
    if viz_nodes:
        raise NotImplementedError("viz_nodes (search-tree visualisation) is a GUI feature")
    if len(func_tuple) != 2:
        raise ValueError("intersection supports pairwise only as written")
    t = _io.require_cuda()
    fa, fb = func_tuple
    if (fa.mode, fa.conservative) != (fb.mode, fb.conservative):
        raise ValueError("both functions must share one mode")
    ma, mb = device_model(params_tuple[0]), device_model(params_tuple[1])
    bo = fa.bound_opts()
    L = _lib.load()
    cap = min(1 << 20, int(max_nodes))
    while True:
        ws_bytes = L.niq_intersect_workspace_size(ma.handle, mb.handle, _lib.C.byref(bo), cap)
        ws = t.empty(ws_bytes, dtype=t.uint8, device='cuda')
        found = t.zeros(1, dtype=t.int32, device='cuda')
        loc = t.zeros(3, dtype=t.float32, device='cuda')
        counts = t.zeros(2, dtype=t.int64, device='cuda')
        try:
            _lib.check(L.niq_find_any_intersection(ma.handle, mb.handle, _lib.C.byref(bo), _host3(lower),
                                                   _host3(upper), float(eps), cap, _io.ptr(found), _io.ptr(loc),
                                                   _io.ptr(counts), _io.ptr(ws), ws_bytes, _io.stream_handle()))
            break
        except _lib.NIQCapacityError:
            del ws
            if cap >= max_nodes:
                raise
            cap = min(cap * 4, int(max_nodes))
    f = bool(found.item())
    loc = loc.cpu().numpy()
    if f:
        return True, 1, 2, loc
    return False, 0, 0, np.array((-777., -777., -777.), np.float32)


# Nodes one query may visit in the persistent closest-point forms.  With loose bounds
# (untrained networks) a query must refine every undecided node inside the ball of its
# best distance down to the eps size, which can take millions of nodes; the budget keeps
# such a query from holding the device indefinitely.
NODE_BUDGET = 1 << 22


def closest_point(func, params, lower, upper, query_points, eps=0.001, batch_process_size=2048, persistent=False,
                  node_budget=NODE_BUDGET, strict=True):
    """src/kd_tree.py:766-802: ``(min_dist (Q,), min_loc (Q, 3))``.

    The default runs the reference's schedule (one global LIFO stack, batch pops of
    ``batch_process_size``), which reproduces its results, order-dependent pruning
    included.  ``persistent=True`` gives every query its own depth-first traversal on
    the device in one launch.  It prunes when the query-to-box distance, a true lower
    bound, comes within eps of the best candidate, so its distances are never larger than
    the reference schedule's by more than eps.
    ``node_budget`` caps the nodes one persistent query may visit.  A query that
    exhausts it keeps its best candidate so far, a valid upper bound; the call then
    raises NIQError (code NIQ_ERR_TIMEOUT), or with ``strict=False`` returns those
    results."""
    t = _io.require_cuda()
    m = device_model(params)
    bo = func.bound_opts()
    q, kind = _io.to_dev(query_points)
    q = q.reshape(-1, 3)
    Q = q.shape[0]
    dist = t.empty(Q, dtype=t.float32, device='cuda')
    loc = t.empty((Q, 3), dtype=t.float32, device='cuda')
    L = _lib.load()
    if persistent and func.mode in GROWING_MODES:
        raise ValueError("the persistent closest point takes interval, affine_fixed or slope_interval; the "
                         "reference schedule (persistent=False) takes every mode")
    if persistent:
        ws_bytes = L.niq_closest_point_persistent_workspace_size(Q)
        ws = _io.workspace(ws_bytes)
        rc = L.niq_closest_point_persistent(m.handle, _lib.C.byref(bo), _host3(lower), _host3(upper), Q,
                                            _io.ptr(q), float(eps), int(node_budget or 0), _io.ptr(dist),
                                            _io.ptr(loc), _io.ptr(ws), ws_bytes, _io.stream_handle())
        if strict or rc != _lib.NIQ_ERR_TIMEOUT:
            _lib.check(rc)
    else:
        B = int(batch_process_size)
        cap = max(Q + 2 * B, 1 << 16)
        while True:
            ws_bytes = (L.niq_closest_point_growing_workspace_size(m.handle, _lib.C.byref(bo), Q, B, cap)
                        if func.mode in GROWING_MODES else L.niq_closest_point_workspace_size(Q, B, cap))
            ws = t.empty(ws_bytes, dtype=t.uint8, device='cuda')
            try:
                _lib.check(L.niq_closest_point(m.handle, _lib.C.byref(bo), _host3(lower), _host3(upper), Q,
                                               _io.ptr(q), float(eps), B, cap, _io.ptr(dist), _io.ptr(loc),
                                               _io.ptr(ws), ws_bytes, _io.stream_handle()))
                break
            except _lib.NIQCapacityError:
                del ws
                cap *= 4
                if cap > (1 << 31):
                    raise
    return _io.back(dist, kind), _io.back(loc, kind)


def _seed(rngkey):
    """A 64-bit seed from a JAX-style key ((2,) uint32), an int or None."""
    if rngkey is None:
        return 0
    a = np.asarray(rngkey).reshape(-1).astype(np.uint64)
    v = 0
    for x in a.tolist():
        v = ((v * 0x100000001B3) ^ int(x)) & 0xFFFFFFFFFFFFFFFF
    return v


def sample_surface(func, params, lower, upper, n_samples, width, rngkey, n_node_thresh=4096):
    """src/kd_tree.py:254-292: ``n_samples`` points with |f| < width, drawn uniformly
    from the unknown nodes of a level-set tree built with offset ``width`` and
    ``node_terminate_thresh=n_node_thresh``.  Returns an (n_samples, 3) array."""
    t = _io.require_cuda()
    ws_t, cap, counts, m = _tree_device(func, params, lower, upper, None, n_node_thresh, 0, width, True)
    n_nodes = int(counts[0])
    if n_nodes == 0:
        raise RuntimeError("the level-set tree has no unknown node within the width")
    lo, hi = _tree_nodes(ws_t, cap, 0, 0, n_nodes)
    lo, hi = lo.contiguous(), hi.contiguous()
    per = min(3 * int(n_samples), 100000)    # src/kd_tree.py:276
    L = _lib.load()
    ws_bytes = L.niq_sample_workspace_size(per)
    ws = _io.workspace(ws_bytes)
    out = t.empty((int(n_samples), 3), dtype=t.float32, device='cuda')
    found = _lib.C.c_int64(0)
    _lib.check(L.niq_sample_surface(m.handle, n_nodes, _io.ptr(lo), _io.ptr(hi), int(n_samples), float(width),
                                    _seed(rngkey), per, 100000, _io.ptr(out), _lib.C.byref(found), _io.ptr(ws),
                                    ws_bytes, _io.stream_handle()))
    return out.cpu().numpy()


def bulk_properties(func, params, lower, upper, rngkey, n_expand=int(1e4), n_sample=int(1e6)):
    """src/kd_tree.py:836-863: ``(mass, centroid)`` of the region f < 0: interior nodes of
    a level-set tree (``node_terminate_thresh=n_expand``) exactly, its unknown nodes by
    ``n_sample`` Monte Carlo points."""
    ws_t, cap, counts, m = _tree_device(func, params, lower, upper, None, n_expand, 1, 0., True)
    nu, ni = int(counts[0]), int(counts[1])
    ulo, uhi = _tree_nodes(ws_t, cap, 1, 0, nu)
    ilo, ihi = _tree_nodes(ws_t, cap, 1, 1, ni)
    L = _lib.load()
    ws_bytes = L.niq_sample_workspace_size(int(n_sample))
    ws = _io.workspace(ws_bytes)
    res = (_lib.C.c_double * 4)()
    _lib.check(L.niq_bulk_properties(m.handle, ni, _io.ptr(ilo.contiguous()), _io.ptr(ihi.contiguous()), nu,
                                     _io.ptr(ulo.contiguous()), _io.ptr(uhi.contiguous()), int(n_sample),
                                     _seed(rngkey), res, _io.ptr(ws), ws_bytes, _io.stream_handle()))
    return float(res[0]), np.array([res[1], res[2], res[3]], np.float32)
