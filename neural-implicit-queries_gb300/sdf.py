"""Lipschitz sphere test (src/sdf.py) over the GPU point evaluator."""
from __future__ import annotations

import numpy as np

from . import _io
from ._gpu_function import GPUImplicitFunction
from .implicit_function import SIGN_NEGATIVE, SIGN_POSITIVE, SIGN_UNKNOWN


class WeakSDFImplicitFunction(GPUImplicitFunction):
    """src/sdf.py:17-50: a box is classified from one value at its center and the
    box's radius times a Lipschitz bound."""

    def __init__(self, sdf_func=None, lipschitz_bound=1.):
        super().__init__("classify-only", 'affine_fixed')
        self.lipschitz_bound = lipschitz_bound

    def classify_general_box(self, params, box_center, box_vecs, offset=0.):
        t = _io.require_cuda()
        ct, kind = _io.to_dev(box_center)
        vt, _ = _io.to_dev(box_vecs)
        single = ct.dim() == 1
        ct = ct.reshape(-1, 3)
        vt = vt.reshape(ct.shape[0], -1, 3)
        rad = t.sqrt(t.sum(t.square(t.linalg.norm(vt, dim=-1)), dim=1))
        val = GPUImplicitFunction.__call__(self, params, ct)
        can_change = t.abs(val) - rad * self.lipschitz_bound < 0.
        out = t.full_like(val, SIGN_UNKNOWN, dtype=t.int32)
        out = t.where(~can_change & (val > offset), SIGN_POSITIVE, out)
        out = t.where(~can_change & (val < -offset), SIGN_NEGATIVE, out).to(t.int32)
        return _io.back(out[0] if single else out, kind)
