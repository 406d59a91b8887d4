"""The ImplicitFunction interface and sign codes (src/implicit_function.py)."""
from __future__ import annotations

import numpy as np

SIGN_UNKNOWN = 0    # could be anything            (src/implicit_function.py:11)
SIGN_POSITIVE = 1   # definitely positive throughout (src/implicit_function.py:12)
SIGN_NEGATIVE = 2   # definitely negative throughout (src/implicit_function.py:13)


def box_to_general(box_lower, box_upper):
    """center and diagonal vecs of axis-aligned boxes (src/implicit_function.py:28-37);
    accepts (3,) or (N, 3)."""
    lo = np.asarray(box_lower, np.float32)
    hi = np.asarray(box_upper, np.float32)
    center = (np.float32(0.5) * (lo + hi)).astype(np.float32)
    pos_vec = (hi - center).astype(np.float32)
    vecs = pos_vec[..., None, :] * np.eye(3, dtype=np.float32)
    return center, vecs


class ImplicitFunction:
    """Base class: ``__call__`` evaluates points, ``classify_box`` /
    ``classify_general_box`` bound a box and return SIGN_* codes.  Unlike the reference,
    whose methods take a single point or box and are vmapped by the caller, every method
    here also accepts a leading batch axis."""

    def __init__(self, style):
        if style not in ['classify-only', 'classify-and-distance']:
            raise ValueError("unrecognized style")
        self.style = style

    def __call__(self, params, x):
        raise RuntimeError("ImplicitFunction does not implement a __call__() operator. "
                           "Subclasses must provide an implementation if is to be used.")

    def classify_box(self, params, box_lower, box_upper, offset=0.):
        center, vecs = box_to_general(box_lower, box_upper)
        return self.classify_general_box(params, center, vecs, offset=offset)

    def classify_general_box(self, params, box_center, box_vecs, offset=0.):
        raise RuntimeError("ImplicitFunction does not implement classify_general_box(). "
                           "Subclasses must provide an implementation if is to be used.")
