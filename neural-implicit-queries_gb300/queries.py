"""Ray casting (src/queries.py:23-175) and frustum casting (src/queries.py:178-587) on the GPU."""
from __future__ import annotations

import numpy as np

from . import _io, _lib
from .mlp import device_model


def get_default_cast_opts():
    """src/queries.py:23-36."""
    return {
        'hit_eps': 0.001,
        'max_dist': 10.,
        'n_max_step': 512,
        'n_substeps': 1,
        'safety_factor': 0.98,
        'interval_grow_fac': 1.5,
        'interval_shrink_fac': 0.5,
        'interval_init_size': 0.1,
        'refine_width_fac': 2.,
        'n_side_init': 16,
    }


def _common_opts(funcs_tuple):
    modes = {(f.mode, f.conservative) for f in funcs_tuple}
    if len(modes) != 1:
        raise ValueError("all functions of funcs_tuple must share one mode and rounding setting")
    return funcs_tuple[0].bound_opts()


def cast_rays(funcs_tuple, params_tuple, roots, dirs, opts, persistent=True, return_device=False):
    """src/queries.py:134-175: returns ``(t, hit_id, count, N_evals)``.

    ``t`` is the start of the step at termination, ``hit_id`` the 1-based index of the
    function whose sign changed (0: none), ``count`` the steps taken.  ``N_evals`` counts
    the ray-steps actually evaluated (the reference also counts its bucket padding).
    ``persistent=False`` runs the plain form: one launch, one device-to-host sync and one
    compaction per iteration, as the reference's loop does.  ``return_device=True``
    returns CUDA tensors (``N_evals`` as a one-element tensor per function) without
    synchronising the stream."""
    if not isinstance(funcs_tuple, (tuple, list)):
        funcs_tuple, params_tuple = (funcs_tuple,), (params_tuple,)
    if len(funcs_tuple) != len(params_tuple):
        raise ValueError("funcs_tuple and params_tuple must have the same length")
    t = _io.require_cuda()
    bo = _common_opts(funcs_tuple)
    models = [device_model(p) for p in params_tuple]
    rt, kind = _io.to_dev(roots)
    dt, _ = _io.to_dev(dirs)
    rt, dt = rt.reshape(-1, 3), dt.reshape(-1, 3)
    n = rt.shape[0]
    t_out = t.empty(n, dtype=t.float32, device='cuda')
    hit = t.empty(n, dtype=t.int32, device='cuda')
    cnt = t.empty(n, dtype=t.int32, device='cuda')
    nev = t.zeros(len(models), dtype=t.int64, device='cuda')
    L = _lib.load()
    handles = (_lib.C.c_void_p * len(models))(*[m.handle.value for m in models])
    ws_bytes = L.niq_cast_rays_workspace_size(handles, len(models), _lib.C.byref(bo), n)
    ws = _io.workspace(ws_bytes)
    co = _lib.cast_opts(opts)
    fn = L.niq_cast_rays if persistent else L.niq_cast_rays_plain
    _lib.check(fn(handles, len(models), _lib.C.byref(bo), n, _io.ptr(rt), _io.ptr(dt), _lib.C.byref(co),
                  _io.ptr(t_out), _io.ptr(hit), _io.ptr(cnt), _io.ptr(nev), _io.ptr(ws), ws_bytes,
                  _io.stream_handle()))
    if return_device:
        return t_out, hit, cnt, nev
    n_evals = int(nev[0].item()) if n else 0
    return _io.back(t_out, kind), _io.back(hit, kind), _io.back(cnt, kind), n_evals


def cast_rays_frustum(funcs_tuple, params_tuple, cam_params, in_opts):
    """src/queries.py:512-587: ``(out_t, out_hit_id, out_count, N_evals)``, each output a
    (res_x, res_y) array indexed [x, y] as the reference returns it.

    ``cam_params`` is the reference's tuple (root_pos, look_dir, up_dir, left_dir, fov_x,
    fov_y, res_x, res_y); ``in_opts`` the cast options with ``n_side_init`` and
    ``refine_width_fac``.  ``N_evals`` counts frustum steps (the reference also counts its
    bucket padding)."""
    if not isinstance(funcs_tuple, (tuple, list)):
        funcs_tuple, params_tuple = (funcs_tuple,), (params_tuple,)
    if len(funcs_tuple) != len(params_tuple):
        raise ValueError("funcs_tuple and params_tuple must have the same length")
    t = _io.require_cuda()
    bo = _common_opts(funcs_tuple)
    models = [device_model(p) for p in params_tuple]
    root, look, up, left, fov_x, fov_y, res_x, res_y = cam_params
    f3 = lambda a: (_lib.C.c_float * 3)(*np.asarray(_np(a), np.float32).reshape(3).tolist())
    cam = _lib.FrustumCamera(f3(root), f3(look), f3(up), f3(left), float(fov_x), float(fov_y), int(res_x), int(res_y))
    rx, ry = int(res_x), int(res_y)
    t_out = t.empty((rx, ry), dtype=t.float32, device='cuda')
    hit = t.empty((rx, ry), dtype=t.int32, device='cuda')
    cnt = t.empty((rx, ry), dtype=t.int32, device='cuda')
    nev = t.zeros(1, dtype=t.int64, device='cuda')
    L = _lib.load()
    ns = int(in_opts['n_side_init'])
    handles = (_lib.C.c_void_p * len(models))(*[m.handle.value for m in models])
    if bo.mode in (_lib.MODES['affine_truncate'], _lib.MODES['affine_all'], _lib.MODES['affine_append']):
        ws_bytes = L.niq_cast_frustum_growing_workspace_size(handles, len(models), _lib.C.byref(bo), rx, ry, ns)
    else:
        ws_bytes = L.niq_cast_frustum_workspace_size(rx, ry, ns)
    if ws_bytes == 0:
        raise ValueError("bad resolution or n_side_init")
    ws = _io.workspace(ws_bytes)
    co = _lib.cast_opts(in_opts)
    _lib.check(L.niq_cast_frustum(handles, len(models), _lib.C.byref(bo), _lib.C.byref(cam), _lib.C.byref(co),
                                  float(in_opts['refine_width_fac']), ns, _io.ptr(t_out), _io.ptr(hit), _io.ptr(cnt),
                                  _io.ptr(nev), _io.ptr(ws), ws_bytes, _io.stream_handle()))
    return t_out.cpu().numpy(), hit.cpu().numpy(), cnt.cpu().numpy(), int(nev.item())


def _np(a):
    return a.detach().cpu().numpy() if hasattr(a, 'detach') else np.asarray(a)
