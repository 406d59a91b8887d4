"""Shared GPU implementation of the ImplicitFunction protocol."""
from __future__ import annotations

import numpy as np

from . import _io, _lib
from .implicit_function import ImplicitFunction, box_to_general
from .mlp import device_model


class GPUImplicitFunction(ImplicitFunction):
    """Point evaluation and box classification through libniq.

    ``mode`` is one of the range-arithmetic names of src/implicit_mlp_utils.py:12-64.
    ``conservative`` (default True) adds the outward rounding terms so that every
    returned bound contains the exact range; False reproduces the reference's
    round-to-nearest arithmetic.  ``products`` ('auto', 'fp32', '3xtf32') chooses how the
    growing-term modes form their dense products (NIQ_PRODUCTS_* in include/niq.h)."""

    def __init__(self, style, mode, truncate_count=-777, n_append=0, conservative=True, products='auto'):
        super().__init__(style)
        self.mode = mode
        self.truncate_count = truncate_count
        self.n_append = n_append
        self.conservative = conservative
        self.products = products

    # -- options as passed to the C ABI
    def bound_opts(self):
        return _lib.bound_opts(self.mode, self.truncate_count, self.n_append, self.conservative, self.products)

    def device_model(self, params):
        return device_model(params)

    def __call__(self, params, x):
        """Plain MLP value at points (3,) or (N, 3) (src/affine.py:26-28)."""
        m = device_model(params)
        xt, kind = _io.to_dev(x)
        single = xt.dim() == 1
        xt = xt.reshape(-1, 3)
        t = _io.torch()
        out = t.empty(xt.shape[0], dtype=t.float32, device='cuda')
        L = _lib.load()
        _lib.check(L.niq_eval_points(m.handle, xt.shape[0], _io.ptr(xt), _io.ptr(out), _io.stream_handle()))
        out = out[0] if single else out
        return _io.back(out, kind)

    def bounds_general_box(self, params, box_center, box_vecs, offset=0.):
        """(sign, lower, upper) over general boxes: center (N,3), vecs (N,v,3)."""
        m = device_model(params)
        ct, kind = _io.to_dev(box_center)
        vt, _ = _io.to_dev(box_vecs)
        single = ct.dim() == 1
        ct = ct.reshape(-1, 3)
        n = ct.shape[0]
        vt = vt.reshape(n, -1, 3)
        v = vt.shape[1]
        t = _io.torch()
        sign = t.empty(n, dtype=t.int32, device='cuda')
        lohi = t.empty((n, 2), dtype=t.float32, device='cuda')
        L = _lib.load()
        opts = self.bound_opts()
        ws_bytes = L.niq_classify_workspace_size(m.handle, _lib.C.byref(opts), n, v)
        ws = _io.workspace(ws_bytes) if ws_bytes else None
        _lib.check(L.niq_classify_boxes(m.handle, _lib.C.byref(opts), n, _io.ptr(ct), _io.ptr(vt), v,
                                        float(offset), _io.ptr(sign), _io.ptr(lohi), _io.ptr(ws),
                                        ws_bytes, _io.stream_handle()))
        if single:
            sign, lohi = sign[0], lohi[0]
        return _io.back(sign, kind), _io.back(lohi[..., 0], kind), _io.back(lohi[..., 1], kind)

    def classify_general_box(self, params, box_center, box_vecs, offset=0.):
        return self.bounds_general_box(params, box_center, box_vecs, offset)[0]

    def bounds_box(self, params, box_lower, box_upper, offset=0.):
        center, vecs = box_to_general(np.asarray(_np(box_lower)), np.asarray(_np(box_upper)))
        return self.bounds_general_box(params, center, vecs, offset)


def _np(x):
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x.detach().cpu().numpy()
    except ImportError:
        pass
    return x
