"""Autotuner for the persistent kernels' launch parameters.

The batched closest-point launch splits every job into chunks of queries that CTAs claim
one at a time, and runs as many CTAs per SM as fit.  The best chunk size and CTA count
depend on the model table (widths, depths) and the query mix: small chunks balance
uneven jobs, large ones restage weights less often.  ``tune_batched`` times the
candidates on the caller's own workload, keeps the fastest and remembers it per device
and workload signature in a JSON cache (``NIQ_AUTOTUNE_CACHE``, default
``niq.autotune.json`` beside this package); ``apply`` sets a remembered choice with
``niq_tune_set``.  The tree's CTAs per SM can be tuned the same way (``tune_tree``).
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import _io, _lib

PARAMS = {'batched_chunk': 0, 'batched_ctas_per_sm': 1, 'tree_ctas_per_sm': 2,
          # 1 + the polls a bounded device wait may make (0: built-in limit, 1: give up at once)
          'barrier_polls': 3, 'mbar_polls': 4,
          # output columns per thread of the per-ray cast (4 or 8)
          'ray_columns': 5}
CACHE = os.environ.get('NIQ_AUTOTUNE_CACHE', os.path.join(os.path.dirname(__file__), 'niq.autotune.json'))


def _device_name():
    return _io.torch().cuda.get_device_name()


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, choice):
    data = _load()
    data[key] = choice
    tmp = CACHE + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def set_params(**kw):
    """Sets launch parameters by name (see PARAMS); 0 restores the built-in choice."""
    L = _lib.load()
    for k, v in kw.items():
        _lib.check(L.niq_tune_set(PARAMS[k], int(v)))


def get_params():
    L = _lib.load()
    out = {}
    for k, p in PARAMS.items():
        v = _lib.C.c_int32()
        _lib.check(L.niq_tune_get(p, _lib.C.byref(v)))
        out[k] = v.value
    return out


def _time(fn, reps):
    t = _io.torch()
    fn()
    t.cuda.synchronize()
    best = float('inf')
    for _ in range(reps):
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        t.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def batched_signature(table, counts):
    """Workload signature: widths and depths of the table, query-count histogram."""
    shapes = sorted((m.max_width, m.n_layers) for m in table.models)
    hist = np.histogram(np.log2(np.maximum(np.asarray(counts), 1)), bins=8, range=(0, 16))[0]
    return 'batched|' + _device_name() + '|' + json.dumps(shapes) + '|' + ','.join(map(str, hist.tolist()))


def apply(key):
    """Sets the remembered choice for ``key``; returns it (or None)."""
    choice = _load().get(key)
    if choice:
        set_params(**choice)
    return choice


def tune_batched(func, table, job_models, offsets, counts, queries, lower, upper, eps=1e-3, node_budget=None,
                 chunks=(32, 64, 128, 256, 512), ctas=(0, 1), reps=2, use_cache=True):
    """Times every (chunk, CTAs per SM) candidate on this batched closest-point workload,
    sets the fastest and returns ``(choice, timings)``."""
    from . import batched
    key = batched_signature(table, counts)
    if use_cache:
        c = apply(key)
        if c:
            return c, None
    t = _io.torch()
    status = t.zeros(1, dtype=t.int32, device='cuda')
    timings = {}
    for ch in chunks:
        for ct in ctas:
            set_params(batched_chunk=ch, batched_ctas_per_sm=ct)
            ms = _time(lambda: batched.closest_point_packed(func, table, job_models, offsets, counts, queries, lower,
                                                            upper, eps, status=status, node_budget=node_budget), reps)
            timings[f'{ch}/{ct}'] = ms
    best = min(timings, key=timings.get)
    ch, ct = (int(x) for x in best.split('/'))
    choice = {'batched_chunk': ch, 'batched_ctas_per_sm': ct}
    set_params(**choice)
    _store(key, choice)
    return choice, timings


def tune_tree(run, candidates=(0, 1, 2), reps=2):
    """Times ``run()`` (a level-set tree call) under each CTAs-per-SM cap and sets the
    fastest; returns ``(choice, timings)``."""
    timings = {}
    for c in candidates:
        set_params(tree_ctas_per_sm=c)
        timings[c] = _time(run, reps)
    best = min(timings, key=timings.get)
    set_params(tree_ctas_per_sm=best)
    return {'tree_ctas_per_sm': best}, timings
