"""Factory of ImplicitFunction objects by mode name (src/implicit_mlp_utils.py)."""
from __future__ import annotations

from . import mlp
from .affine import AffineContext, AffineImplicitFunction
from .sdf import WeakSDFImplicitFunction
from .slope_interval import SlopeIntervalImplicitFunction


def generate_implicit_from_params(params, mode, **kwargs):
    """The mode switch of src/implicit_mlp_utils.py:23-64 for an in-memory spec.
    Extra keywords: ``conservative`` (default True) selects outward rounding;
    ``products`` ('auto', 'fp32', '3xtf32') how dense products are formed where there is a
    choice: the affine_truncate/affine_all engine, and the affine_fixed level-set tree
    ('3xtf32' puts its hidden layers on the tensor cores on models of hidden width <= 64;
    by default it runs on the FP32 tile engine, which is faster there)."""
    cons = kwargs.get('conservative', True)
    prod = kwargs.get('products', 'auto')
    if mode == 'sdf':
        return WeakSDFImplicitFunction(lipschitz_bound=kwargs.get('sdf_lipschitz', 1.)), params
    if mode == 'interval':
        return AffineImplicitFunction(None, AffineContext('interval'), cons, prod), params
    if mode == 'affine_fixed':
        return AffineImplicitFunction(None, AffineContext('affine_fixed'), cons, prod), params
    if mode == 'affine_truncate':
        ctx = AffineContext('affine_truncate', truncate_count=kwargs['affine_n_truncate'],
                            truncate_policy=kwargs.get('affine_truncate_policy', 'absolute'))
        return AffineImplicitFunction(None, ctx, cons, prod), params
    if mode == 'affine_append':
        return AffineImplicitFunction(None, AffineContext('affine_append', n_append=kwargs['affine_n_append']),
                                      cons), params
    if mode == 'affine_all':
        return AffineImplicitFunction(None, AffineContext('affine_all'), cons, prod), params
    if mode == 'slope_interval':
        return SlopeIntervalImplicitFunction(None, cons), params
    raise RuntimeError("unrecognized mode")


def generate_implicit_from_file(input_path, mode, **kwargs):
    """src/implicit_mlp_utils.py:12-64."""
    if input_path.endswith(".npz"):
        params = mlp.load(input_path)
    else:
        raise ValueError("unrecognized filetype")
    return generate_implicit_from_params(params, mode, **kwargs)
