"""ctypes binding of libniq.so (declared in include/niq.h).

The library is loaded on first use.  There is no fallback: if ``libniq.so`` is missing
or no CUDA device is present, the call raises.  Tensors cross the boundary as raw device
pointers (``tensor.data_ptr()``) and the current torch CUDA stream handle.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

NIQ_OK = 0
NIQ_ERR_INVALID_ARG = -1
NIQ_ERR_BAD_SPEC = -2
NIQ_ERR_CUDA = -3
NIQ_ERR_CAPACITY = -4
NIQ_ERR_TIMEOUT = -5
NIQ_ERR_UNSUPPORTED = -6

PRODUCTS = {'auto': 0, 'fp32': 1, '3xtf32': 2}
MODES = {'interval': 0, 'affine_fixed': 1, 'affine_truncate': 2, 'affine_append': 3,
         'affine_all': 4, 'slope_interval': 5}
ACTS = {'none': 0, 'relu': 1, 'elu': 2, 'tanh': 3}
NIQ_MAX_LAYERS = 32
NIQ_MAX_WIDTH = 256
NIQ_SPEC_MAGIC = 0x3151494e


class NIQError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"niq error {code}: {msg}")
        self.code = code


class NIQCapacityError(NIQError):
    pass


class BoundOpts(C.Structure):
    _fields_ = [('mode', C.c_int32), ('truncate_count', C.c_int32), ('n_append', C.c_int32),
                ('conservative', C.c_int32), ('products', C.c_int32)]


class FrustumCamera(C.Structure):
    _fields_ = [('root', C.c_float * 3), ('look', C.c_float * 3), ('up', C.c_float * 3), ('left', C.c_float * 3),
                ('fov_x', C.c_float), ('fov_y', C.c_float), ('res_x', C.c_int32), ('res_y', C.c_int32)]


class CastOpts(C.Structure):
    _fields_ = [('hit_eps', C.c_float), ('max_dist', C.c_float), ('n_max_step', C.c_int32),
                ('n_substeps', C.c_int32), ('safety_factor', C.c_float),
                ('interval_grow_fac', C.c_float), ('interval_shrink_fac', C.c_float),
                ('interval_init_size', C.c_float)]


class Request(C.Structure):
    _fields_ = [('kind', C.c_int32), ('model', C.c_void_p), ('model_b', C.c_void_p), ('opts', BoundOpts),
                ('cast', CastOpts), ('n', C.c_int64), ('in0', C.c_void_p), ('in1', C.c_void_p),
                ('out_f', C.c_void_p), ('out_f2', C.c_void_p), ('out_i', C.c_void_p), ('out_i2', C.c_void_p),
                ('eps', C.c_float), ('node_budget', C.c_int64), ('node_capacity', C.c_int64),
                ('lower', C.c_float * 3), ('upper', C.c_float * 3)]


class ServerOpts(C.Structure):
    _fields_ = [('n_lanes', C.c_int32), ('slice_rays', C.c_int64), ('slice_queries', C.c_int64),
                ('lane_scratch_bytes', C.c_int64)]


NIQ_REQ_RAYS, NIQ_REQ_CLOSEST, NIQ_REQ_INTERSECT = 0, 1, 2

_P = C.c_void_p
_I32, _I64, _F32, _SZ = C.c_int32, C.c_int64, C.c_float, C.c_size_t
_PF = C.POINTER(C.c_float)

# name -> (restype, argtypes)
_SIGS = {
    'niq_last_error': (C.c_char_p, []),
    'niq_version': (C.c_int, []),
    'niq_device_info': (C.c_int, [C.POINTER(_I32), C.POINTER(_I32)]),
    'niq_tc_tf32_rate': (C.c_int, [_I32, _PF, _P]),
    'niq_fp32_fma_rate': (C.c_int, [_I32, _PF, _P]),
    'niq_tune_set': (C.c_int, [_I32, _I32]),
    'niq_tune_get': (C.c_int, [_I32, C.POINTER(_I32)]),
    'niq_model_create': (C.c_int, [_P, _SZ, C.POINTER(_P)]),
    'niq_model_destroy': (C.c_int, [_P]),
    'niq_model_info': (C.c_int, [_P, C.POINTER(_I32), C.POINTER(_I32)]),
    'niq_eval_points': (C.c_int, [_P, _I64, _P, _P, _P]),
    'niq_eval_gradients': (C.c_int, [_P, _I64, _P, _P, _P, _P]),
    'niq_classify_workspace_size': (_SZ, [_P, C.POINTER(BoundOpts), _I64, _I32]),
    'niq_classify_boxes': (C.c_int, [_P, C.POINTER(BoundOpts), _I64, _P, _P, _I32, _F32, _P, _P, _P, _SZ, _P]),
    'niq_cast_rays_workspace_size': (_SZ, [C.POINTER(_P), _I32, C.POINTER(BoundOpts), _I64]),
    'niq_cast_rays': (C.c_int, [C.POINTER(_P), _I32, C.POINTER(BoundOpts), _I64, _P, _P, C.POINTER(CastOpts),
                                _P, _P, _P, _P, _P, _SZ, _P]),
    'niq_cast_rays_plain': (C.c_int, [C.POINTER(_P), _I32, C.POINTER(BoundOpts), _I64, _P, _P, C.POINTER(CastOpts),
                                      _P, _P, _P, _P, _P, _SZ, _P]),
    'niq_tree_workspace_size': (_SZ, [_I64, _I32]),
    'niq_levelset_tree': (C.c_int, [_P, C.POINTER(BoundOpts), _PF, _PF, _I32, _I64, _F32, _I32, _I64, _P, _P, _SZ, _P]),
    'niq_cast_frustum_workspace_size': (_SZ, [_I32, _I32, _I32]),
    'niq_cast_frustum_growing_workspace_size': (_SZ, [C.POINTER(_P), _I32, C.POINTER(BoundOpts), _I32, _I32, _I32]),
    'niq_cast_frustum': (C.c_int, [C.POINTER(_P), _I32, C.POINTER(BoundOpts), C.POINTER(FrustumCamera),
                                   C.POINTER(CastOpts), _F32, _I32, _P, _P, _P, _P, _P, _SZ, _P]),
    'niq_sample_workspace_size': (_SZ, [_I64]),
    'niq_sample_surface': (C.c_int, [_P, _I64, _P, _P, _I64, _F32, C.c_uint64, _I64, _I32, _P, C.POINTER(_I64), _P,
                                     _SZ, _P]),
    'niq_bulk_properties': (C.c_int, [_P, _I64, _P, _P, _I64, _P, _P, _I64, C.c_uint64, C.POINTER(C.c_double), _P,
                                      _SZ, _P]),
    'niq_outward_normals_workspace_size': (_SZ, [_I64]),
    'niq_outward_normals': (C.c_int, [C.POINTER(_P), _I32, _I64, _P, _P, _F32, _P, _P, _SZ, _P]),
    'niq_outward_normals_autodiff_workspace_size': (_SZ, [_I64]),
    'niq_outward_normals_autodiff': (C.c_int, [C.POINTER(_P), _I32, _I64, _P, _P, _P, _P, _SZ, _P]),
    'niq_shade_image': (C.c_int, [_I32, _I64, _P, _P, _P, _PF, _P, _I32, _I32, _PF, _I32, _I32, _P, _P]),
    'niq_shade_image_pixel_colors': (C.c_int, [_I64, _P, _P, _P, _PF, _P, _I32, _I32, _P, _I32, _P, _P]),
    'niq_levelset_tree_plain': (C.c_int, [_P, C.POINTER(BoundOpts), _PF, _PF, _I32, _I64, _F32, _I32, _I64, _P, _P,
                                          _SZ, _P]),
    'niq_levelset_tree_batches': (C.c_int, [_P, C.POINTER(BoundOpts), _PF, _PF, _I32, _I64, _F32, _I32, _I64, _I64,
                                            _P, _P, _SZ, _P]),
    'niq_tree_result': (C.c_int, [_P, _I64, _I32, _I32, C.POINTER(_P), C.POINTER(_P)]),
    'niq_tree_engine': (C.c_int, [_P, C.POINTER(BoundOpts), C.POINTER(_I32)]),
    'niq_server_create': (C.c_int, [C.POINTER(ServerOpts), C.POINTER(_P)]),
    'niq_server_destroy': (C.c_int, [_P]),
    'niq_batch_submit': (C.c_int, [_P, C.POINTER(Request), C.POINTER(_I64)]),
    'niq_batch_poll': (C.c_int, [_P, _I64, C.POINTER(_I32), C.POINTER(_I32)]),
    'niq_batch_wait': (C.c_int, [_P, _I64, C.c_double, C.POINTER(_I32)]),
    'niq_server_stats': (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64)]),
    'niq_tree_growing_workspace_size': (_SZ, [_P, C.POINTER(BoundOpts), _I64, _I32]),
    'niq_levelset_tree_growing': (C.c_int, [_P, C.POINTER(BoundOpts), _PF, _PF, _I32, _I64, _F32, _I32, _I64, _P, _P,
                                            _SZ, _P]),
    'niq_levelset_tree_static': (C.c_int, [_P, _P, _SZ, C.POINTER(BoundOpts), _PF, _PF, _I32, _I64, _F32, _I32,
                                           _P, _P, _P, _P, _P, _P, _P, _P]),
    'niq_hmc_workspace_size': (_SZ, []),
    'niq_hmc_extract': (C.c_int, [_P, _I64, _P, _P, _I32, _P, _I64, _P, _P, _SZ, _P]),
    'niq_mc_table': (C.c_int, [C.POINTER(_I32)]),
    'niq_hmc_lattice_workspace_size': (_SZ, [_PF, _PF, _I32, _I64]),
    'niq_hmc_extract_lattice': (C.c_int, [_P, _I64, _P, _P, _PF, _PF, _I32, _P, _I64, _P, _P, _SZ, _P]),
    'niq_intersect_workspace_size': (_SZ, [_P, _P, C.POINTER(BoundOpts), _I64]),
    'niq_find_any_intersection': (C.c_int, [_P, _P, C.POINTER(BoundOpts), _PF, _PF, _F32, _I64, _P, _P, _P, _P, _SZ,
                                            _P]),
    'niq_closest_point_workspace_size': (_SZ, [_I64, _I32, _I64]),
    'niq_closest_point_growing_workspace_size': (_SZ, [_P, C.POINTER(BoundOpts), _I64, _I32, _I64]),
    'niq_closest_point': (C.c_int, [_P, C.POINTER(BoundOpts), _PF, _PF, _I64, _P, _F32, _I32, _I64, _P, _P, _P, _SZ,
                                    _P]),
    'niq_closest_point_persistent_workspace_size': (_SZ, [_I64]),
    'niq_closest_point_persistent': (C.c_int, [_P, C.POINTER(BoundOpts), _PF, _PF, _I64, _P, _F32, _I64, _P, _P, _P,
                                               _SZ, _P]),
    'niq_batched_closest_point_workspace_size': (_SZ, [_I64, _I32]),
    'niq_batched_closest_point_stats': (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64), _P]),
    'niq_batched_closest_point': (C.c_int, [C.POINTER(_P), _I32, C.POINTER(BoundOpts), _I32, C.POINTER(_I32),
                                            C.POINTER(_I64), C.POINTER(_I64), _P, _PF, _PF, _F32, _P, _P, _I64, _P,
                                            _P, _SZ, _P]),
}

_lib = None


def library_path():
    return _build.LIB_PATH


def load(path=None):
    """Load libniq.so and declare every exported function; raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built: run `python -c \"import __graft_entry__ as g; g.build()\"`")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS.keys())


def check(rc):
    if rc == NIQ_OK:
        return
    msg = load().niq_last_error()
    msg = msg.decode() if msg else ''
    if rc in (NIQ_ERR_INVALID_ARG, NIQ_ERR_BAD_SPEC):
        raise ValueError(f"niq error {rc}: {msg}")
    if rc == NIQ_ERR_CAPACITY:
        raise NIQCapacityError(rc, msg)
    raise NIQError(rc, msg)


def bound_opts(mode, truncate_count=-777, n_append=0, conservative=True, products='auto'):
    if mode not in MODES:
        raise ValueError(f"invalid mode {mode!r}")
    if products not in PRODUCTS:
        raise ValueError(f"invalid products {products!r}: one of {sorted(PRODUCTS)}")
    return BoundOpts(MODES[mode], int(truncate_count), int(n_append), 1 if conservative else 0, PRODUCTS[products])


def cast_opts(opts):
    return CastOpts(float(opts['hit_eps']), float(opts['max_dist']), int(opts['n_max_step']),
                    int(opts['n_substeps']), float(opts['safety_factor']), float(opts['interval_grow_fac']),
                    float(opts['interval_shrink_fac']), float(opts['interval_init_size']))
