"""Affine-arithmetic ImplicitFunction (src/affine.py) on the GPU."""
from __future__ import annotations

from dataclasses import dataclass

from ._gpu_function import GPUImplicitFunction


@dataclass(frozen=True)
class AffineContext:
    """src/affine.py:62-76.  Only the 'absolute' truncation policy exists here: the
    reference's 'relative' policy divides an (n,) array by a (d,) array and only runs when
    n == d (src/affine.py:145-146)."""
    mode: str = 'affine_fixed'
    truncate_count: int = -777
    truncate_policy: str = 'absolute'
    affine_domain_terms: int = 0
    n_append: int = 0

    def __post_init__(self):
        if self.mode not in ['interval', 'affine_fixed', 'affine_truncate', 'affine_append', 'affine_all']:
            raise ValueError("invalid mode")
        if self.mode == 'affine_truncate':
            if self.truncate_count is None:
                raise ValueError("must specify truncate count")
            if self.truncate_policy != 'absolute':
                raise ValueError("only the 'absolute' truncate policy is supported")


class AffineImplicitFunction(GPUImplicitFunction):
    """src/affine.py:17-55.  ``affine_func`` is accepted for signature compatibility and
    ignored: the spec is evaluated by the CUDA kernels."""

    def __init__(self, affine_func=None, ctx=AffineContext(), conservative=True, products='auto'):
        super().__init__("classify-only", ctx.mode, ctx.truncate_count, ctx.n_append, conservative, products)
        self.ctx = ctx
