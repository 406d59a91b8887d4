"""Many models in one launch: closest-point queries over a table of MLPs.

The reference answers one model's queries per call (src/kd_tree.py:766-802).  Here any
number of (model, query set) jobs run in a single persistent kernel: models of
different widths and depths share the launch, CTAs claim chunks of queries in
longest-job-first order, and each query runs its own depth-first traversal with the
reference's candidate and pruning tests.
"""
from __future__ import annotations

import numpy as np

from . import _io, _lib
from .mlp import device_model


class ModelTable:
    """A list of models resident on the device, addressed by index."""

    def __init__(self, params_list):
        self.models = [device_model(p) for p in params_list]
        self.handles = (_lib.C.c_void_p * len(self.models))(*[m.handle.value for m in self.models])

    def __len__(self):
        return len(self.models)


def closest_point_many(func, table, job_models, query_points_list, lower, upper, eps=0.001):
    """Runs ``len(job_models)`` closest-point jobs in one launch.

    ``table``: a ModelTable (or a list of params dicts); ``job_models[j]`` indexes the
    table; ``query_points_list[j]`` is that job's (Q_j, 3) array.  Returns a list of
    ``(min_dist, min_loc)`` pairs as NumPy arrays (or device tensors with
    ``query_points_list`` given as one CUDA tensor plus offsets, see ``closest_point_packed``)."""
    if not isinstance(table, ModelTable):
        table = ModelTable(table)
    counts = np.array([len(q) for q in query_points_list], np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    allq = np.concatenate([np.asarray(q, np.float32).reshape(-1, 3) for q in query_points_list]) \
        if len(query_points_list) else np.zeros((0, 3), np.float32)
    dist, loc = closest_point_packed(func, table, np.asarray(job_models, np.int32), offsets, counts, allq,
                                     lower, upper, eps)
    dist, loc = _io.back(dist, 'numpy'), _io.back(loc, 'numpy')
    return [(dist[o:o + c], loc[o:o + c]) for o, c in zip(offsets, counts)]


def closest_point_packed(func, table, job_models, offsets, counts, query_points, lower, upper, eps=0.001,
                         status=None, node_budget=None):
    """Device-level form: all queries in one (N, 3) array (host or device), jobs as
    (model index, row offset, row count).  Returns device tensors (dist (N,), loc (N,3)).
    ``node_budget`` (default kd_tree.NODE_BUDGET) caps the nodes one query may visit.
    With ``status`` (a CUDA int32 tensor of one element) the call does not synchronise:
    the traversal status lands there (0; NIQ_ERR_TIMEOUT when a query spent its budget,
    its result then an upper bound; NIQ_ERR_CAPACITY when a traversal stack overflowed)."""
    t = _io.require_cuda()
    if node_budget is None:
        from .kd_tree import NODE_BUDGET as node_budget
    q, _ = _io.to_dev(query_points)
    q = q.reshape(-1, 3)
    n = q.shape[0]
    dist = t.empty(n, dtype=t.float32, device='cuda')
    loc = t.empty((n, 3), dtype=t.float32, device='cuda')
    jm = np.ascontiguousarray(job_models, np.int32)
    jo = np.ascontiguousarray(offsets, np.int64)
    jc = np.ascontiguousarray(counts, np.int64)
    L = _lib.load()
    bo = func.bound_opts()
    ws_bytes = L.niq_batched_closest_point_workspace_size(int(jc.sum()), len(jm))
    ws = _io.workspace(ws_bytes)
    lo = (_lib.C.c_float * 3)(*np.asarray(lower, np.float32).tolist())
    hi = (_lib.C.c_float * 3)(*np.asarray(upper, np.float32).tolist())
    _lib.check(L.niq_batched_closest_point(
        table.handles, len(table), _lib.C.byref(bo), len(jm),
        jm.ctypes.data_as(_lib.C.POINTER(_lib.C.c_int32)), jo.ctypes.data_as(_lib.C.POINTER(_lib.C.c_int64)),
        jc.ctypes.data_as(_lib.C.POINTER(_lib.C.c_int64)), _io.ptr(q), lo, hi, float(eps), _io.ptr(dist),
        _io.ptr(loc), int(node_budget or 0), _io.ptr(status), _io.ptr(ws), ws_bytes, _io.stream_handle()))
    return dist, loc


def stats():
    """Counters of the last ``closest_point_packed`` call on the current device and stream:
    ``(queries stopped at their node budget, nodes bounded)``.  A query past its budget keeps
    its best candidate, an upper bound on its distance.  Synchronises."""
    L = _lib.load()
    spent, nodes = _lib.C.c_int64(0), _lib.C.c_int64(0)
    _lib.check(L.niq_batched_closest_point_stats(_io.ptr(_io.workspace(0)), _lib.C.byref(spent), _lib.C.byref(nodes),
                                                  _io.stream_handle()))
    return int(spent.value), int(nodes.value)
