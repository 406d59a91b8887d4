"""CPU restatement (NumPy) of the range-analysis hot path of nmwsharp/neural-implicit-queries.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: it is imported by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` and nowhere else.
The product path (the CUDA kernels behind ``include/niq.h``) never calls it.

Every function restates one reference function, vectorised over a leading batch axis
(where the reference uses ``jax.vmap``) and parameterised by ``dtype``:
``np.float32`` mirrors the reference's fp32 JAX arithmetic, ``np.float64`` is the
FP64 affine-arithmetic oracle against which bound widths are measured.

Parity pin: ``tests/golden/make_golden.py`` executes the reference's own ``src/*.py``
(over a NumPy stand-in for the absent ``jax`` package) on seeded inputs and commits the
outputs under ``tests/golden/``; ``tests/test_oracle_golden.py`` checks this module
against them.  The stand-in replaces XLA's arithmetic, so the pin holds within fp32
rounding, not bit for bit.

Citations are ``path:line`` inside the reference project.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SIGN_UNKNOWN = 0   # src/implicit_function.py:11
SIGN_POSITIVE = 1  # src/implicit_function.py:12
SIGN_NEGATIVE = 2  # src/implicit_function.py:13

AFFINE_MODES = ('interval', 'affine_fixed', 'affine_truncate', 'affine_append', 'affine_all')


# ----------------------------------------------------------------------------------------
# Spec walking  (src/mlp.py:117-144)
# ----------------------------------------------------------------------------------------

def n_ops(params):
    """src/mlp.py:135-144: one past the largest 4-digit op prefix."""
    n = 0
    for key in params:
        try:
            i_op = int(key.split(".")[0])
        except ValueError:
            raise ValueError(f"Could not parse out key {key}. Is this a valid mlp spec?")
        n = max(n, i_op + 1)
    return n


def get_op_data(params, i_op):
    """src/mlp.py:117-133: (name, {arg: value}) of op ``i_op``; the ``_`` arg is dropped
    later by the evaluator (src/mlp.py:108-109)."""
    prefix = f"{i_op:04d}"
    name, args = "", {}
    for key in params:
        if key.startswith(prefix):
            tokens = key.split(".")
            name = tokens[1]
            if len(tokens) > 2:
                args[tokens[2]] = params[key]
    if name == "":
        raise ValueError(f"didn't find op {i_op}")
    args.pop("_", None)
    return name, args


def spec_ops(params, dtype=np.float32):
    """Ops in order with their arrays cast to ``dtype``.  ``spatial_transformation`` is
    rewritten into the dense op it applies: ``x @ inv(R) + inv(R) @ (-t)``
    (src/mlp.py:342-346, src/affine_layers.py:175-179)."""
    ops = []
    for i in range(n_ops(params)):
        name, args = get_op_data(params, i)
        if name == 'dense':
            A = np.asarray(args['A'], dtype=dtype)
            b = args.get('b', None)
            b = None if b is None else np.asarray(b, dtype=dtype)
            ops.append(('dense', A, b))
        elif name == 'spatial_transformation':
            R = np.asarray(args['R'], dtype=dtype)
            t = np.asarray(args['t'], dtype=dtype)
            R_inv = np.linalg.inv(R).astype(dtype)
            t_inv = (R_inv @ (-t)).astype(dtype)
            ops.append(('dense', R_inv, t_inv))
        elif name in ('relu', 'elu', 'tanh', 'squeeze_last'):
            ops.append((name,))
        else:
            raise ValueError(f"unsupported op '{name}'")
    return ops


# ----------------------------------------------------------------------------------------
# Point evaluation  (src/mlp.py:253-347, const paths of src/affine_layers.py)
# ----------------------------------------------------------------------------------------

def _elu(x):
    # jax.nn.elu: where(x > 0, x, expm1(where(x > 0, 0, x)))
    return np.where(x > 0, x, np.expm1(np.where(x > 0, 0, x)))


def eval_points(params, x, dtype=np.float32):
    """Plain MLP forward for points ``x`` of shape (N, 3) -> (N,)."""
    x = np.asarray(x, dtype=dtype)
    for op in spec_ops(params, dtype):
        name = op[0]
        if name == 'dense':
            _, A, b = op
            x = x @ A
            if b is not None:
                x = x + b
        elif name == 'relu':
            x = np.maximum(x, 0)
        elif name == 'elu':
            x = _elu(x)
        elif name == 'tanh':
            x = np.tanh(x)
        elif name == 'squeeze_last':
            x = x[..., 0]
    return x


def eval_gradients(params, x, dtype=np.float32):
    """Value and gradient of the MLP at points ``x`` (N, 3) -> ((N,), (N, 3)): forward-mode
    tangents, as jax.jacfwd of the point function (src/render.py:61-63).  The activation
    derivatives are those JAX differentiates: relu' = 1 where x > 0 else 0 (jax.nn.relu),
    elu' = 1 where x > 0 else exp(x) (jax.nn.elu), tanh' = 1 - tanh(x)^2."""
    x = np.asarray(x, dtype=dtype)
    t = np.broadcast_to(np.eye(3, dtype=dtype), x.shape[:-1] + (3, 3)).copy()   # d x / d input, (N, 3 tangents, 3)
    for op in spec_ops(params, dtype):
        name = op[0]
        if name == 'dense':
            _, A, b = op
            x = x @ A
            t = t @ A
            if b is not None:
                x = x + b
        elif name == 'relu':
            d = (x > 0).astype(dtype)
            x = np.maximum(x, 0)
            t = t * d[..., None, :]
        elif name == 'elu':
            d = np.where(x > 0, dtype(1), np.exp(np.minimum(x, 0))).astype(dtype)
            x = _elu(x)
            t = t * d[..., None, :]
        elif name == 'tanh':
            x = np.tanh(x)
            t = t * (1 - x * x)[..., None, :]
        elif name == 'squeeze_last':
            x = x[..., 0]
            t = t[..., 0]
    return x, t


# ----------------------------------------------------------------------------------------
# Affine arithmetic  (src/affine.py, src/affine_layers.py)
# ----------------------------------------------------------------------------------------

@dataclass(frozen=True)
class AffineContext:
    """src/affine.py:62-76."""
    mode: str = 'affine_fixed'
    truncate_count: int = -777
    truncate_policy: str = 'absolute'
    affine_domain_terms: int = 0
    n_append: int = 0

    def __post_init__(self):
        if self.mode not in AFFINE_MODES:
            raise ValueError("invalid mode")
        if self.mode == 'affine_truncate' and self.truncate_count is None:
            raise ValueError("must specify truncate count")


def coordinates_in_general_box(ctx, center, vecs):
    """src/affine.py:109-117, batched: center (N,d), vecs (N,v,d)."""
    base = center
    if ctx.mode == 'interval':
        aff = np.zeros((center.shape[0], 0, center.shape[-1]), dtype=center.dtype)
        err = np.sum(np.abs(vecs), axis=1)
    else:
        aff = vecs
        err = np.zeros_like(center)
    return base, aff, err


def radius(aff, err):
    """src/affine.py:85-91."""
    return np.sum(np.abs(aff), axis=1) + err


def may_contain_bounds(base, aff, err):
    """src/affine.py:119-125."""
    rad = radius(aff, err)
    return base - rad, base + rad


def _boundary_gap(vals_desc, k, gaps):
    """Relative gap between the k-th and (k+1)-th largest values (per row of a
    descending-sorted array), min-folded into ``gaps``: a near tie at the keep/drop
    boundary makes the kept set, and so the bound, depend on last-ulp rounding."""
    if gaps is None or vals_desc.shape[1] <= k or k <= 0:
        return
    a, b = vals_desc[:, k - 1].astype(np.float64), vals_desc[:, k].astype(np.float64)
    g = (a - b) / np.maximum(np.abs(a), 1e-30)
    # a tie between zero magnitudes keeps or drops nothing: not a decision
    g = np.where(a > 0, g, np.inf)
    np.minimum(gaps, g, out=gaps)


def truncate_affine(ctx, base, aff, err, gaps=None):
    """src/affine.py:127-162 ('absolute' policy; rows sorted by decreasing L1 magnitude,
    stable, the first ``truncate_count`` kept, the rest folded into ``err``)."""
    if ctx.mode != 'affine_truncate':
        return base, aff, err
    n_keep = ctx.truncate_count
    if aff.shape[1] <= n_keep:
        return base, aff, err
    if ctx.truncate_policy != 'absolute':
        raise RuntimeError("bad policy")
    mags = np.sum(np.abs(aff), axis=-1)                      # (N, rows)
    order = np.argsort(-mags, axis=-1, kind='stable')        # jnp.argsort is stable
    _boundary_gap(np.take_along_axis(mags, order, axis=-1), n_keep, gaps)
    aff = np.take_along_axis(aff, order[:, :, None], axis=1)
    err = err + np.sum(np.abs(aff[:, n_keep:, :]), axis=1)
    return base, aff[:, :n_keep, :], err


def apply_linear_approx(ctx, base, aff, err, alpha, beta, delta, gaps=None):
    """src/affine.py:164-193.  ``gaps`` (optional, (N,) float64) collects the relative gap
    at the truncation / top-k boundary (see _boundary_gap)."""
    base = alpha * base + beta
    aff = alpha[:, None, :] * aff
    delta = np.abs(delta)
    if ctx.mode in ('interval', 'affine_fixed'):
        err = alpha * err + delta
    elif ctx.mode in ('affine_truncate', 'affine_all'):
        err = alpha * err
        n, d = delta.shape
        new_aff = np.zeros((n, d, d), dtype=delta.dtype)
        new_aff[:, np.arange(d), np.arange(d)] = delta
        aff = np.concatenate((aff, new_aff), axis=1)
        base, aff, err = truncate_affine(ctx, base, aff, err, gaps)
    elif ctx.mode == 'affine_append':
        err = alpha * err
        k = ctx.n_append
        # jax.lax.top_k: descending, ties to the lower index
        order_all = np.argsort(-delta, axis=-1, kind='stable')
        _boundary_gap(np.take_along_axis(delta, order_all, axis=-1), k, gaps)
        order = order_all[:, :k]
        keep_vals = np.take_along_axis(delta, order, axis=-1)
        n, d = delta.shape
        new_aff = np.zeros((n, k, d), dtype=delta.dtype)
        new_aff[np.arange(n)[:, None], np.arange(k)[None, :], order] = keep_vals
        aff = np.concatenate((aff, new_aff), axis=1)
        err = err + (np.sum(delta, axis=-1) - np.sum(keep_vals, axis=-1))[:, None]
    return base, aff, err


def _relu_linearization(lower, upper):
    """src/affine_layers.py:34-56 (Chebyshev bound of relu on [lower, upper])."""
    relu = lambda v: np.maximum(v, 0)
    with np.errstate(divide='ignore', invalid='ignore', over='ignore'):
        alpha = (relu(upper) - relu(lower)) / (upper - lower)
    alpha = np.where(lower >= 0, 1., alpha)
    alpha = np.where(upper < 0, 0., alpha)
    alpha = np.nan_to_num(alpha, nan=0.0)
    alpha = np.clip(alpha, 0., 1.)
    beta = (relu(lower) - alpha * lower) / 2
    delta = beta
    return alpha.astype(lower.dtype), beta.astype(lower.dtype), delta.astype(lower.dtype)


def _elu_linearization(lower, upper):
    """src/affine_layers.py:59-97."""
    with np.errstate(divide='ignore', invalid='ignore', over='ignore'):
        lowerF = _elu(lower)
        upperF = _elu(upper)
        lowerS = np.minimum(np.exp(lower), 1.)
        upperS = np.minimum(np.exp(upper), 1.)
        alpha = (upperF - lowerF) / (upper - lower)
        alpha = np.where(lower >= 0, 1., alpha)
        alpha = np.nan_to_num(alpha, nan=0.0)
        alpha = np.clip(alpha, lowerS, upperS)
        r_upper = lowerF - alpha * lower
        x_lower = np.clip(np.log(alpha), lower, upper)
        r_lower = (alpha - 1.) - alpha * x_lower
    beta = 0.5 * (r_upper + r_lower)
    delta = 0.5 * np.abs(r_upper - r_lower)
    alpha = np.where(lower >= 0, 1., alpha)
    beta = np.where(lower >= 0, 0., beta)
    delta = np.where(lower >= 0, 0., delta)
    dt = lower.dtype
    return alpha.astype(dt), beta.astype(dt), delta.astype(dt)


def _tanh_linearization(lower, upper):
    """TanH has no rule in the reference (its README names TanH, the code has none).
    This rule follows the pattern of the reference's ``sin``/``elu`` rules
    (src/affine_layers.py:59-138): the secant slope ``alpha`` on [lower, upper]; the
    extrema of ``tanh(x) - alpha*x`` are taken over the endpoints and the interior
    stationary points ``x = +-atanh(sqrt(1 - alpha))`` clipped into the interval;
    ``beta`` is their midpoint and ``delta`` their half-range."""
    dt = lower.dtype
    with np.errstate(divide='ignore', invalid='ignore', over='ignore'):
        tl, tu = np.tanh(lower), np.tanh(upper)
        width = upper - lower
        alpha = (tu - tl) / width
        mid = 0.5 * (lower + upper)
        tm = np.tanh(mid)
        alpha = np.where(width > 0, alpha, 1. - tm * tm)
        alpha = np.nan_to_num(alpha, nan=0.0)
        alpha = np.clip(alpha, 0., 1.)
        xs = np.arctanh(np.sqrt(np.clip(1. - alpha, 0., 1.)))   # +inf when alpha == 0
        cands = [lower, upper, np.clip(xs, lower, upper), np.clip(-xs, lower, upper)]
        vals = [np.tanh(c) - alpha * c for c in cands]
        r_lo = np.minimum.reduce(vals)
        r_hi = np.maximum.reduce(vals)
    beta = 0.5 * (r_hi + r_lo)
    delta = 0.5 * (r_hi - r_lo)
    return alpha.astype(dt), beta.astype(dt), delta.astype(dt)


_LINEARIZATIONS = {'relu': _relu_linearization, 'elu': _elu_linearization,
                   'tanh': _tanh_linearization}


def affine_forward(params, ctx, base, aff, err, dtype=np.float32, gaps=None):
    """Walk the spec in affine mode (src/mlp.py:99-111 with apply_func['affine'])."""
    for op in spec_ops(params, dtype):
        name = op[0]
        if name == 'dense':                     # src/affine_layers.py:11-31
            _, A, b = op
            base = base @ A
            aff = aff @ A
            err = err @ np.abs(A)
            if b is not None:
                base = base + b
        elif name in _LINEARIZATIONS:
            lower, upper = may_contain_bounds(base, aff, err)
            alpha, beta, delta = _LINEARIZATIONS[name](lower, upper)
            base, aff, err = apply_linear_approx(ctx, base, aff, err, alpha, beta, delta, gaps)
        elif name == 'squeeze_last':            # src/affine_layers.py:164-172
            base, aff, err = base[..., 0], aff[..., 0], err[..., 0]
    return base, aff, err


def affine_bounds(params, ctx, center, vecs, dtype=np.float32, gaps=None):
    """(lower, upper) of the output over general boxes: center (N,3), vecs (N,v,3)."""
    center = np.asarray(center, dtype=dtype)
    vecs = np.asarray(vecs, dtype=dtype)
    ctx = AffineContext(ctx.mode, ctx.truncate_count, ctx.truncate_policy,
                        vecs.shape[1], ctx.n_append)
    base, aff, err = coordinates_in_general_box(ctx, center, vecs)
    base, aff, err = affine_forward(params, ctx, base, aff, err, dtype, gaps)
    return may_contain_bounds(base, aff, err)


def conservative_affine_bounds_model(params, mode, center, vecs, gammas):
    """FP64 model of the CUDA kernels' outward-rounding scheme for 'interval' and
    'affine_fixed' with ReLU layers: the reference's rules plus, per dense layer with
    rounding factor ``gammas[l]``, the fold gamma(|base| + sum|aff|) into the err input,
    the (1 + 2 gamma) scale and gamma|b| on the err output, and 2^-23 (|base'| + alpha S)
    for the linearisation's rounding.  It isolates the cost of those terms from FP32
    arithmetic: the kernels' widths must agree with it up to FP32 noise."""
    center = np.asarray(center, np.float64)
    vecs = np.asarray(vecs, np.float64)
    layers = [op for op in spec_ops(params, np.float64)]
    dense = [(op[1], op[2] if op[2] is not None else np.zeros(op[1].shape[1])) for op in layers if op[0] == 'dense']
    acts = []
    for op in layers:
        if op[0] == 'dense':
            acts.append('none')
        elif op[0] in ('relu', 'elu', 'tanh'):
            acts[-1] = op[0]
    base = center
    if mode == 'interval':
        aff = np.zeros((center.shape[0], 0, 3))
        err = np.sum(np.abs(vecs), axis=1)
    else:
        aff = vecs
        err = np.zeros_like(center)
    err = err + gammas[0] * (np.abs(base) + np.abs(aff).sum(1))
    for li, ((A, b), act) in enumerate(zip(dense, acts)):
        g = gammas[li]
        base, aff, err = base @ A + b, aff @ A, (err @ np.abs(A)) * (1 + 2 * g) + g * np.abs(b)
        if act == 'relu':
            S = np.abs(aff).sum(1)
            lo, hi = base - (S + err), base + (S + err)
            w = np.where(hi - lo == 0, 1., hi - lo)
            a = np.where(lo >= 0, 1., np.where(hi < 0, 0., (np.maximum(hi, 0) - np.maximum(lo, 0)) / w))
            a = np.clip(np.nan_to_num(a), 0, 1)
            rhi = np.where((lo >= 0) | (hi < 0), 0., np.maximum(np.maximum(-a * lo, hi - a * hi), 0))
            nb = a * base + rhi / 2
            aff = a[:, None, :] * aff
            err = a * err + rhi / 2 + 2 ** -23 * (np.abs(nb) + a * S)
            base = nb
            if li + 1 < len(dense):
                err = err + gammas[li + 1] * (np.abs(base) + a * S)
        elif act != 'none':
            raise ValueError("the model covers ReLU networks only")
        elif li + 1 < len(dense):
            err = err + gammas[li + 1] * (np.abs(base) + np.abs(aff).sum(1))
    base, aff, err = base[:, 0], aff[:, :, 0], err[:, 0]
    rad = np.abs(aff).sum(1) + err
    return base - rad, base + rad


NEAR_REL = 1e-5   # the decision tolerance of the parity rules (relative)


def bound_near(lo, hi, offset=0., rel=NEAR_REL):
    """True where a box's classification (lo > offset, hi < -offset) sits within ``rel``
    of flipping, relative to the bound's scale max(|lo|, |hi|)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    scale = np.maximum(np.abs(lo), np.abs(hi)) + 1e-30
    return (np.abs(lo - offset) <= rel * scale) | (np.abs(hi + offset) <= rel * scale)


def value_near(v0, v1, rel=NEAR_REL):
    """True where the sign test sign(v0) != sign(v1) sits within rounding of flipping:
    either value within rel of zero, relative to max(|v0|, |v1|, 1)."""
    v0 = np.abs(np.asarray(v0, np.float64))
    v1 = np.abs(np.asarray(v1, np.float64))
    scale = np.maximum(np.maximum(v0, v1), 1.0)
    return np.minimum(v0, v1) <= rel * scale


def sign_from_bounds(lower, upper, offset=0.):
    """src/affine.py:50-53 and src/slope_interval.py:44-47."""
    out = np.full(lower.shape, SIGN_UNKNOWN, dtype=np.int32)
    out = np.where(lower > offset, SIGN_POSITIVE, out)
    out = np.where(upper < -offset, SIGN_NEGATIVE, out)
    return out.astype(np.int32)


# ----------------------------------------------------------------------------------------
# Slope intervals  (src/slope_interval.py, src/slope_interval_layers.py)
# ----------------------------------------------------------------------------------------

def slope_forward(params, primal, center, width, dtype=np.float32):
    for op in spec_ops(params, dtype):
        name = op[0]
        if name == 'dense':                     # src/slope_interval_layers.py:11-33
            _, A, b = op
            primal = primal @ A
            if b is not None:
                primal = primal + b
            center = center @ A
            width = width @ np.abs(A)
        elif name in ('relu', 'elu', 'tanh'):   # src/slope_interval_layers.py:36-82
            sl, su = center - width, center + width
            rad = np.sum(np.maximum(su, -sl), axis=1)
            pl, pu = primal - rad, primal + rad
            if name == 'relu':
                dfl = np.where(pl > 0, 1., 0.).astype(dtype)
                dfu = np.where(pu < 0, 0., 1.).astype(dtype)
                primal = np.maximum(primal, 0)
            elif name == 'elu':
                dfl = np.minimum(np.exp(pl), 1.).astype(dtype)
                dfu = np.minimum(np.exp(pu), 1.).astype(dtype)
                primal = _elu(primal)
            else:  # tanh: derivative 1 - tanh^2 is largest at 0, decreasing in |x|
                dl = 1. - np.tanh(pl) ** 2
                du = 1. - np.tanh(pu) ** 2
                straddle = (pl <= 0) & (pu >= 0)
                dfl = np.minimum(dl, du).astype(dtype)
                dfu = np.where(straddle, 1., np.maximum(dl, du)).astype(dtype)
                primal = np.tanh(primal)
            nl = np.minimum(sl * dfl[:, None, :], sl * dfu[:, None, :])
            nu = np.maximum(su * dfl[:, None, :], su * dfu[:, None, :])
            center = 0.5 * (nl + nu)
            width = nu - center
        elif name == 'squeeze_last':
            primal, center, width = primal[..., 0], center[..., 0], width[..., 0]
    return primal, center, width


def slope_bounds_box(params, center, vecs, dtype=np.float32):
    """src/slope_interval.py:29-51,192-210 batched: returns (lower, upper)."""
    center = np.asarray(center, dtype=dtype)
    vecs = np.asarray(vecs, dtype=dtype)
    primal, sc, sw = slope_forward(params, center, vecs, np.zeros_like(vecs), dtype)
    sl, su = sc - sw, sc + sw
    rad = np.sum(np.maximum(su, -sl), axis=1)
    return primal - rad, primal + rad


# ----------------------------------------------------------------------------------------
# ImplicitFunction-like façade (src/implicit_function.py:28-37, src/implicit_mlp_utils.py)
# ----------------------------------------------------------------------------------------

@dataclass
class OracleFunc:
    """A mode-bound evaluator: ``mode`` is one of the names of
    src/implicit_mlp_utils.py:12-64 except 'sdf'."""
    mode: str = 'affine_fixed'
    truncate_count: int = -777
    n_append: int = 0
    dtype: type = np.float32
    ctx: AffineContext = field(init=False, default=None)

    def __post_init__(self):
        if self.mode != 'slope_interval':
            self.ctx = AffineContext(self.mode, truncate_count=self.truncate_count,
                                     n_append=self.n_append)

    def __call__(self, params, x):
        return eval_points(params, x, self.dtype)

    def bounds_general(self, params, center, vecs):
        if self.mode == 'slope_interval':
            return slope_bounds_box(params, center, vecs, self.dtype)
        return affine_bounds(params, self.ctx, center, vecs, self.dtype)

    def bounds_near(self, params, center, vecs, offset=0., rel=NEAR_REL):
        """Bounds plus a flag per box: True where the classification against ``offset``
        sits within ``rel`` (relative) of flipping -- a bound within rel * max(|lo|, |hi|)
        of the threshold, or a near tie at a truncation / top-k boundary -- so that
        last-ulp differences in the dot products can change it."""
        gaps = np.full(np.shape(center)[0], np.inf)
        if self.mode == 'slope_interval':
            lo, hi = slope_bounds_box(params, center, vecs, self.dtype)
        else:
            lo, hi = affine_bounds(params, self.ctx, center, vecs, self.dtype, gaps)
        return lo, hi, bound_near(lo, hi, offset, rel) | (gaps < rel)

    def classify_general_box(self, params, center, vecs, offset=0.):
        lo, hi = self.bounds_general(params, center, vecs)
        return sign_from_bounds(lo, hi, offset)

    def classify_box(self, params, lower, upper, offset=0.):
        lower = np.asarray(lower, self.dtype)
        upper = np.asarray(upper, self.dtype)
        center = 0.5 * (lower + upper)
        vec = upper - center
        vecs = np.zeros(vec.shape[:1] + (3, 3), dtype=self.dtype)
        vecs[:, np.arange(3), np.arange(3)] = vec
        return self.classify_general_box(params, center, vecs, offset)


def generate_implicit(params, mode, **kwargs):
    """src/implicit_mlp_utils.py:12-64 without the file load."""
    if mode == 'affine_truncate':
        f = OracleFunc(mode, truncate_count=kwargs['affine_n_truncate'])
    elif mode == 'affine_append':
        f = OracleFunc(mode, n_append=kwargs['affine_n_append'])
    elif mode in AFFINE_MODES or mode == 'slope_interval':
        f = OracleFunc(mode)
    else:
        raise RuntimeError("unrecognized mode")
    if 'dtype' in kwargs:
        f.dtype = kwargs['dtype']
    return f


# ----------------------------------------------------------------------------------------
# Buckets  (src/bucketing.py:6-36)
# ----------------------------------------------------------------------------------------

BUCKET_SIZES = [2 ** s for s in range(7, 31)]


def get_next_bucket_size(s):
    for b in BUCKET_SIZES:
        if s <= b:
            return b
    raise ValueError("max bucket size exceeded")


def fits_in_smaller_bucket(size, curr_bucket_size):
    return get_next_bucket_size(size) < curr_bucket_size


# ----------------------------------------------------------------------------------------
# Ray casting  (src/queries.py:23-175, src/render.py:17-50)
# ----------------------------------------------------------------------------------------

def get_default_cast_opts():
    """src/queries.py:23-36."""
    return {'hit_eps': 0.001, 'max_dist': 10., 'n_max_step': 512, 'n_substeps': 1,
            'safety_factor': 0.98, 'interval_grow_fac': 1.5, 'interval_shrink_fac': 0.5,
            'interval_init_size': 0.1, 'refine_width_fac': 2., 'n_side_init': 16}


def cast_rays(funcs, params_list, roots, dirs, opts, trace=False):
    """src/queries.py:39-175.  Each ray steps independently; the bucketing only changes
    ``N_evals``, which is reproduced by replaying the bucket sizes.

    With ``trace`` a fifth array is returned: per ray, the step index (the ray's count
    when the decision was taken) of its first near-threshold decision -- a segment bound
    within NEAR_REL of its sign threshold or a hit test with a value within NEAR_REL of
    zero (see bounds_near, value_near) -- or a huge value when it took none.  Two
    implementations that differ only by rounding can send a ray down different paths
    only from such a decision, so their results for the ray may differ only when
    first_near < min(count_a, count_b)."""
    f32 = funcs[0].dtype
    roots = np.asarray(roots, f32)
    dirs = np.asarray(dirs, f32)
    N = roots.shape[0]
    hit_eps = opts['hit_eps']
    out_t = np.zeros(N, f32)
    out_hit = np.zeros(N, np.int32)
    out_count = np.zeros(N, np.int32)
    t = np.zeros(N, f32)
    step = (np.ones(N, f32) * opts['interval_init_size'] * opts['max_dist']).astype(f32)
    count = np.zeros(N, np.int32)
    active = np.arange(N)
    bucket = N
    n_evals = 0
    n_sub = opts['n_substeps']
    first_near = np.full(N, np.iinfo(np.int32).max, np.int64)
    while True:
        r, d = roots[active], dirs[active]
        tt, ss = t[active], step[active]
        is_hit = np.zeros(active.shape[0], bool)
        hit_id = np.zeros(active.shape[0], np.int32)
        n_inner = np.zeros(active.shape[0], np.int32)
        for i_sub in range(n_sub):                          # src/queries.py:44-92
            can_step = ~is_hit
            live = ~is_hit
            n_inner += (~is_hit).astype(np.int32)
            for fid, (func, params) in enumerate(zip(funcs, params_list), start=1):
                pos_start = r + tt[:, None] * d
                half_vec = 0.5 * ss[:, None] * d
                pos_mid = pos_start + half_vec
                if trace:
                    lo, hi, near = func.bounds_near(params, pos_mid, half_vec[:, None, :])
                    btype = sign_from_bounds(lo, hi)
                else:
                    btype = func.classify_general_box(params, pos_mid, half_vec[:, None, :])
                can_step &= (btype == SIGN_POSITIVE) | (btype == SIGN_NEGATIVE)
                pos_eps = r + (tt + np.asarray(hit_eps, f32))[:, None] * d
                v0 = func(params, pos_start)
                v1 = func(params, pos_eps)
                if trace:
                    near = live & (near | value_near(v0, v1))
                    step_idx = count[active] + i_sub
                    idx = active[near]
                    first_near[idx] = np.minimum(first_near[idx], step_idx[near])
                this_hit = np.sign(v0) != np.sign(v1)
                hit_id = np.where(this_hit, fid, hit_id).astype(np.int32)
                is_hit |= this_hit
            this_step = np.where(can_step, ss, np.asarray(hit_eps, f32)).astype(f32)
            tt = np.where(is_hit, tt, tt + this_step * np.asarray(opts['safety_factor'], f32)).astype(f32)
            ss = np.where(can_step, ss * np.asarray(opts['interval_grow_fac'], f32),
                          ss * np.asarray(opts['interval_shrink_fac'], f32)).astype(f32)
            ss = np.maximum(ss, np.asarray(hit_eps, f32)).astype(f32)
        n_evals += bucket * n_sub
        t[active], step[active] = tt, ss
        count[active] += n_inner
        c = count[active]
        term = is_hit | (tt > opts['max_dist']) | (c >= opts['n_max_step'])  # :116-120
        done = active[term]
        out_t[done] = tt[term]
        out_hit[done] = hit_id[term]
        out_count[done] = c[term]
        active = active[~term]
        n_valid = active.shape[0]
        if n_valid == 0:
            break
        if fits_in_smaller_bucket(n_valid, bucket):
            bucket = get_next_bucket_size(n_valid)
    if trace:
        return out_t, out_hit, out_count, n_evals, first_near
    return out_t, out_hit, out_count, n_evals


def jax_linspace(start, stop, num, dtype=np.float32):
    """``jnp.linspace`` for floats: ``start * (1 - s) + stop * s`` with ``s = i / (num - 1)``,
    which keeps both endpoints exact (the formula of jax.numpy's linspace).  ``start`` and
    ``stop`` broadcast against a trailing axis of length ``num``."""
    s = (np.arange(num, dtype=dtype) / np.asarray(num - 1, dtype)).astype(dtype)
    return (np.asarray(start, dtype) * (1 - s) + np.asarray(stop, dtype) * s).astype(dtype)


def normalize(x):
    return x / np.linalg.norm(x, axis=-1, keepdims=True)


def generate_camera_rays(eye_pos, look_dir, up_dir, res=1024, fov_deg=30., dtype=np.float32):
    """src/render.py:26-50 (pinhole, x fastest, image coords linspace(-1, 1, res))."""
    eye_pos = np.asarray(eye_pos, dtype)
    look_dir = np.asarray(look_dir, dtype)
    up_dir = np.asarray(up_dir, dtype)
    ax = jax_linspace(np.asarray(-1., dtype), np.asarray(1., dtype), res, dtype)
    cx, cy = np.meshgrid(ax, ax)
    cx, cy = cx.reshape(-1), cy.reshape(-1)
    up_dir = up_dir - np.dot(look_dir, up_dir) * look_dir
    up_dir = normalize(up_dir)
    left_dir = np.cross(look_dir, up_dir).astype(dtype)
    tanf = np.asarray(np.tan(np.deg2rad(fov_deg) / 2), dtype)
    p = look_dir[None, :] + left_dir[None, :] * (cx * tanf)[:, None] + up_dir[None, :] * (cy * tanf)[:, None]
    dirs = normalize(p).astype(dtype)
    roots = np.tile(eye_pos, (dirs.shape[0], 1))
    return roots, dirs


def look_at(eye_pos, target=None, up_dir='y', dtype=np.float32):
    """src/render.py:229-242."""
    eye_pos = np.asarray(eye_pos, dtype)
    target = np.zeros(3, dtype) if target is None else np.asarray(target, dtype)
    up = np.asarray((0., 1., 0.) if up_dir == 'y' else (0., 0., 1.), dtype)
    look = normalize(target - eye_pos)
    up = normalize(up - np.dot(up, look) * look)
    left = np.cross(look, up)
    return look.astype(dtype), up.astype(dtype), left.astype(dtype)


def camera_ray(look_dir, up_dir, left_dir, fov_x, fov_y, theta_x, theta_y, dtype=np.float32):
    """src/render.py:17-23, batched over theta_x/theta_y (image coords on [-1, 1])."""
    tx = np.asarray(np.tan(np.deg2rad(np.asarray(fov_x, dtype)) / 2), dtype)
    ty = np.asarray(np.tan(np.deg2rad(np.asarray(fov_y, dtype)) / 2), dtype)
    p = (look_dir[None, :] + left_dir[None, :] * (theta_x * tx)[:, None]
         + up_dir[None, :] * (theta_y * ty)[:, None]).astype(dtype)
    return normalize(p).astype(dtype)


def _frust_step(funcs, params_list, cam, rng_, t, size, opts, f32, near=None):
    """The substep loop of one cast_rays_frustum iteration for a batch of frusta
    (src/queries.py:202-321): returns (t, step_size, is_hit, hit_id, demands_subd, steps).
    ``near`` (optional, (n,) bool) is or-ed with the frusta whose box bound or hit test
    sat within NEAR_REL of its threshold."""
    root, look, up, left, fov_x, fov_y, res_x, res_y = cam
    x_lo, y_lo, x_hi, y_hi = rng_[:, 0], rng_[:, 1], rng_[:, 2], rng_[:, 3]
    single = (x_lo + 1 == x_hi) & (y_lo + 1 == y_hi)
    rx1, ry1 = np.asarray(res_x + 1., f32), np.asarray(res_y + 1., f32)
    xc_lo = (np.asarray(2., f32) * x_lo.astype(f32) / rx1 - 1).astype(f32)
    xc_hi = (np.asarray(2., f32) * (x_hi - 1).astype(f32) / rx1 - 1).astype(f32)
    yc_lo = (np.asarray(2., f32) * y_lo.astype(f32) / ry1 - 1).astype(f32)
    yc_hi = (np.asarray(2., f32) * (y_hi - 1).astype(f32) / ry1 - 1).astype(f32)
    ray = lambda a, b: camera_ray(look, up, left, fov_x, fov_y, a, b, f32)
    r_uu, r_lu, r_ul = ray(xc_hi, yc_hi), ray(xc_lo, yc_hi), ray(xc_hi, yc_lo)
    r_ll = ray(xc_lo, yc_lo)
    mid = (np.asarray(0.5, f32) * (r_uu + r_ll)).astype(f32)
    mid_len = np.linalg.norm(mid, axis=-1).astype(f32)
    mid = (mid / mid_len[:, None]).astype(f32)
    expand = (np.asarray(1., f32) / mid_len).astype(f32)
    n = t.shape[0]
    is_hit = np.zeros(n, bool)
    hit_id = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int32)
    demands = np.zeros(n, bool)
    hit_eps = np.asarray(opts['hit_eps'], f32)
    for _ in range(opts['n_substeps']):
        t_up = (t + size).astype(f32)
        t_adj = (t_up * expand).astype(f32)
        right_front = ((r_uu - r_lu) * t_adj[:, None] / 2).astype(f32)
        up_front = ((r_uu - r_ul) * t_adj[:, None] / 2).astype(f32)
        can_step = ~is_hit
        steps += (~is_hit).astype(np.int32)
        center = (root[None, :] + (np.asarray(0.5, f32) * (t + t_adj))[:, None] * mid).astype(f32)
        cvec = ((np.asarray(0.5, f32) * (t_adj - t))[:, None] * mid).astype(f32)
        vecs = np.stack((cvec, right_front, up_front), axis=1)
        live = ~is_hit
        for fid, (func, params) in enumerate(zip(funcs, params_list), start=1):
            if near is not None:
                blo, bhi, bn = func.bounds_near(params, center, vecs)
                btype = sign_from_bounds(blo, bhi)
            else:
                btype = func.classify_general_box(params, center, vecs)
            can_step &= (btype == SIGN_POSITIVE) | (btype == SIGN_NEGATIVE)
            p0 = (root[None, :] + t[:, None] * mid).astype(f32)
            p1 = (root[None, :] + (t + hit_eps)[:, None] * mid).astype(f32)
            v0, v1 = func(params, p0), func(params, p1)
            if near is not None:
                near |= live & (bn | value_near(v0, v1))
            this_hit = np.sign(v0) != np.sign(v1)
            hit_id = np.where(this_hit, fid, hit_id).astype(np.int32)
            is_hit |= this_hit
        this_step = np.where(can_step, size, hit_eps * single.astype(f32)).astype(f32)
        t = np.where(is_hit, t, t + this_step * np.asarray(opts['safety_factor'], f32)).astype(f32)
        size = np.where(can_step, size * np.asarray(opts['interval_grow_fac'], f32),
                        size * np.asarray(opts['interval_shrink_fac'], f32)).astype(f32)
        demands = demands | (size < hit_eps) | is_hit
        size = np.maximum(size, hit_eps).astype(f32)
    return t, size, is_hit, hit_id, demands, steps


def _cmp_near(a, b, rel=NEAR_REL):
    """True where the comparison a > b sits within rel (relative) of flipping."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) <= rel * np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-30)


def cast_rays_frustum(funcs, params_list, cam_params, opts, trace=False):
    """src/queries.py:178-587: frusta over integer pixel ranges march like rays with a
    3-vector box (the frustum's extent at the far end of the step), split in half along
    the wider axis when the step size falls behind the frustum's width, and hit only as
    single pixels.  Returns (out_t, out_hit_id, out_count, n_frustum_steps) with the
    outputs indexed [x, y] as the reference writes them.  The reference's buckets and
    compaction do not change any frustum's result; the frusta are kept compact here.

    With ``trace`` a fifth (res_x, res_y) bool array marks the pixels whose frustum path
    (the pixel's frustum and every frustum it was split from) took a decision within
    NEAR_REL of flipping: a box bound or hit test (bounds_near, value_near), the step
    limit t > max_dist, a refinement comparison of the frustum width with the step, or
    the truncation of the fractional step count.  Two implementations that differ only
    by rounding can give a pixel different results only where it is marked."""
    f32 = funcs[0].dtype
    root, look, up, left, fov_x, fov_y, res_x, res_y = cam_params
    cam = (np.asarray(root, f32), np.asarray(look, f32), np.asarray(up, f32), np.asarray(left, f32),
           float(fov_x), float(fov_y), int(res_x), int(res_y))
    ns = int(opts['n_side_init'])
    xt = jax_linspace(0., float(res_x), ns + 1, np.float32).astype(np.int64)
    yt = jax_linspace(0., float(res_y), ns + 1, np.float32).astype(np.int64)
    rng_ = np.stack((np.tile(xt[:-1], ns), np.repeat(yt[:-1], ns), np.tile(xt[1:], ns), np.repeat(yt[1:], ns)), -1)
    t = np.zeros(ns * ns, f32)
    size = (np.ones(ns * ns, f32) * np.asarray(opts['interval_init_size'], f32) *
            np.asarray(opts['max_dist'], f32)).astype(f32)
    count = np.zeros(ns * ns, f32)
    near = np.zeros(ns * ns, bool)
    fin = []
    it = 0
    n_steps = 0
    fov_x_rad = np.asarray(np.deg2rad(np.asarray(fov_x, f32)), f32)
    fov_y_rad = np.asarray(np.deg2rad(np.asarray(fov_y, f32)), f32)
    while rng_.shape[0]:
        n_steps += rng_.shape[0]
        t, size, is_hit, hit_id, demands, steps = _frust_step(funcs, params_list, cam, rng_, t, size, opts, f32,
                                                              near if trace else None)
        area = ((rng_[:, 2] - rng_[:, 0]) * (rng_[:, 3] - rng_[:, 1])).astype(np.int64)
        count = (count + steps.astype(f32) * (np.asarray(1., f32) / area.astype(f32))).astype(f32)
        is_hit = is_hit & (area == 1)
        term = is_hit | (t > opts['max_dist']) | (it >= opts['n_max_step'])
        if trace:
            near |= _cmp_near(t, opts['max_dist'])
            frac = count.astype(np.float64) - np.floor(count.astype(np.float64))
            near |= term & ((frac <= NEAR_REL * np.maximum(count, 1.)) | (1 - frac <= NEAR_REL * np.maximum(count, 1.)))
        if term.any():
            fin.append((rng_[term], t[term], hit_id[term], count[term], near[term]))
        keep = ~term
        rng_, t, size, count, demands = rng_[keep], t[keep], size[keep], count[keep], demands[keep]
        near = near[keep]
        it += opts['n_substeps']
        if not rng_.shape[0]:
            break
        xw = (rng_[:, 2] - rng_[:, 0]).astype(f32)
        yw = (rng_[:, 3] - rng_[:, 1]).astype(f32)
        wx = (np.asarray(2., f32) * np.sin(fov_x_rad / 2 * xw / np.asarray(res_x, f32)).astype(f32) * t).astype(f32)
        wy = (np.asarray(2., f32) * np.sin(fov_y_rad / 2 * yw / np.asarray(res_y, f32)).astype(f32) * t).astype(f32)
        can = (rng_[:, 2] > rng_[:, 0] + 1) | (rng_[:, 3] > rng_[:, 1] + 1)
        rf = np.asarray(opts['refine_width_fac'], f32)
        refine = ((wx > rf * size) | (wy > rf * size) | demands) & can
        if trace:
            near |= can & ~demands & (_cmp_near(wx, rf * size) | _cmp_near(wy, rf * size))
        if refine.any():                                    # subdivide_frusta, :409-467
            sub = rng_[refine]
            subd_x = (sub[:, 2] - sub[:, 0]) >= (sub[:, 3] - sub[:, 1])
            xm = (sub[:, 0] + sub[:, 2]) // 2
            ym = (sub[:, 1] + sub[:, 3]) // 2
            a = sub.copy()
            a[:, 2] = np.where(subd_x, xm, sub[:, 2])
            a[:, 3] = np.where(~subd_x, ym, sub[:, 3])
            b = sub.copy()
            b[:, 0] = np.where(subd_x, xm, sub[:, 0])
            b[:, 1] = np.where(~subd_x, ym, sub[:, 1])
            rng_ = rng_.copy()
            rng_[refine] = a
            rng_ = np.concatenate((rng_, b))
            t = np.concatenate((t, t[refine]))
            size = np.concatenate((size, size[refine]))
            count = np.concatenate((count, count[refine]))
            near = np.concatenate((near, near[refine]))
    out_t = np.zeros((int(res_x), int(res_y)), f32)
    out_hit = np.zeros((int(res_x), int(res_y)), np.int32)
    out_count = np.zeros((int(res_x), int(res_y)), np.int32)
    out_near = np.zeros((int(res_x), int(res_y)), bool)
    for r_, tt, hh, cc, nn in fin:                          # subdivide to pixels + write, :469-587
        for i in range(r_.shape[0]):
            x0, y0, x1, y1 = r_[i]
            out_t[x0:x1, y0:y1] = tt[i]
            out_hit[x0:x1, y0:y1] = hh[i]
            out_count[x0:x1, y0:y1] = np.trunc(cc[i]).astype(np.int32)
            out_near[x0:x1, y0:y1] = nn[i]
    if trace:
        return out_t, out_hit, out_count, n_steps, out_near
    return out_t, out_hit, out_count, n_steps


_TET = np.array(((1., -1., -1.), (-1., -1., 1.), (-1., 1., -1.), (1., 1., 1.)), np.float32)


def outward_normals(funcs, params_list, hit_pos, hit_ids, eps, method='finite_differences'):
    """src/render.py:53-90: the normalised gradient of the function each point hit, zeros
    where none.  'finite_differences': tetrahedron central differences; 'autodiff': the
    exact gradient (jax.jacfwd, here forward-mode tangents, eval_gradients)."""
    f32 = funcs[0].dtype
    hit_pos = np.asarray(hit_pos, f32)
    if method == 'autodiff':
        out = np.zeros_like(hit_pos)
        for fid, params in enumerate(params_list, start=1):
            _, grad = eval_gradients(params, hit_pos, f32)
            out = np.where((hit_ids == fid)[:, None], normalize(grad.astype(f32)).astype(f32), out)
        return out
    if method != 'finite_differences':
        raise ValueError("unrecognized method")
    offsets = (_TET * np.asarray(eps, f32)).astype(f32)
    out = np.zeros_like(hit_pos)
    for fid, (func, params) in enumerate(zip(funcs, params_list), start=1):
        pts = (hit_pos[:, None, :] + offsets[None]).reshape(-1, 3).astype(f32)
        samples = func(params, pts).reshape(-1, 4)
        grad = np.sum(offsets[None] * samples[:, :, None], axis=1).astype(f32)
        grad = normalize(grad).astype(f32)
        out = np.where((hit_ids == fid)[:, None], grad, out)
    return out


def _map_coordinates_linear_nearest(img, x, y):
    """jax.scipy.ndimage.map_coordinates(img, (x, y), order=1, mode='nearest') for a 2-D
    image: corner weights (1-w, w) per axis, indices clamped to the image."""
    x0, y0 = np.floor(x), np.floor(y)
    wx1, wy1 = (x - x0).astype(np.float32), (y - y0).astype(np.float32)
    wx0, wy0 = (1 - wx1).astype(np.float32), (1 - wy1).astype(np.float32)
    xi = [np.clip(x0.astype(np.int64), 0, img.shape[0] - 1), np.clip(x0.astype(np.int64) + 1, 0, img.shape[0] - 1)]
    yi = [np.clip(y0.astype(np.int64), 0, img.shape[1] - 1), np.clip(y0.astype(np.int64) + 1, 0, img.shape[1] - 1)]
    acc = np.zeros(x.shape, np.float32)
    for a, wa in ((0, wx0), (1, wx1)):
        for b, wb in ((0, wy0), (1, wy1)):
            acc = (acc + img[xi[a], yi[b]] * (wa * wb)).astype(np.float32)
    return acc


def shade_image(shading, ray_dirs, hit_normals, hit_ids, up_dir, matcaps, colors, hit_pos=None,
                shading_color_func=None):
    """src/render.py:161-224 plus the white background of :139; ``shading_color_func``
    (src/render.py:198-206) gives each hit position its color, one position at a time."""
    f32 = np.float32
    n = np.asarray(hit_normals, f32)
    if shading == 'normal':
        c = ((n + 1.) / 2.).astype(f32)
    else:
        d = np.asarray(ray_dirs, f32)
        r = normalize(d).astype(f32)
        up = np.asarray(up_dir, f32)
        ray_up = normalize((up[None] - np.sum(up[None] * r, -1, keepdims=True) * r).astype(f32)).astype(f32)
        ray_left = np.cross(d, ray_up).astype(f32)
        u = (np.sum(-ray_left * n, -1) * f32(.98)).astype(f32)
        v = (np.sum(ray_up * n, -1) * f32(.98)).astype(f32)
        H, W = matcaps[0].shape[:2]
        x = ((u + 1.) / 2. * H).astype(f32)
        y = ((-v + 1.) / 2. * W).astype(f32)
        cols = np.ones((n.shape[0], 3), f32)
        if shading_color_func is not None:
            pos = np.asarray(hit_pos, f32)
            for i in np.nonzero(hit_ids > 0)[0]:
                cols[i] = np.asarray(shading_color_func(pos[i]), f32)
        else:
            for fid, col in enumerate(colors, start=1):
                cols = np.where((hit_ids == fid)[:, None], np.asarray(col, f32)[None], cols)
        ck = (1. - (cols[:, 0] + cols[:, 2] + cols[:, 1])).astype(f32)
        c = np.zeros((n.shape[0], 3), f32)
        for ch in range(3):
            m = [_map_coordinates_linear_nearest(np.asarray(mc, f32)[..., ch], x, y) for mc in matcaps]
            c[:, ch] = cols[:, 0] * m[0] + cols[:, 2] * m[2] + cols[:, 1] * m[1] + ck * m[3]
    return np.where((hit_ids > 0)[:, None], c, f32(1.)).astype(f32)


# ----------------------------------------------------------------------------------------
# Level-set kd-tree  (src/kd_tree.py:19-218)
# ----------------------------------------------------------------------------------------

def split_children(lower, upper):
    """Children of a bisection along the first longest axis (src/kd_tree.py:38,70-77)."""
    split_dim = np.argmax(upper - lower, axis=-1)
    mid = 0.5 * (lower + upper)
    mask = np.arange(3)[None, :] == split_dim[:, None]
    a_lo, a_hi = lower, np.where(mask, mid, upper)
    b_lo, b_hi = np.where(mask, mid, lower), upper
    return (a_lo, a_hi), (b_lo, b_hi)


def construct_uniform_unknown_levelset_tree(func, params, lower, upper, node_terminate_thresh=None,
                                            split_depth=None, with_interior_nodes=False,
                                            with_exterior_nodes=False, offset=0.,
                                            batch_process_size=2048):
    """src/kd_tree.py:103-218.  Returns exactly sized arrays (no bucket padding) in the
    reference's order: per batch of ``batch_process_size`` nodes, the A children then
    the B children of its unknown nodes."""
    if node_terminate_thresh is None and split_depth is None:
        raise ValueError("must specify at least one of node_terminate_thresh or split_depth")
    if node_terminate_thresh is None:
        node_terminate_thresh = 9999999999
    dt = func.dtype
    node_lo = np.asarray(lower, dt)[None, :]
    node_hi = np.asarray(upper, dt)[None, :]
    n_splits = 99999999 if split_depth is None else split_depth + 1
    interior, exterior = [], []
    n_boxes = 0
    for i_split in range(n_splits):
        n_curr = node_lo.shape[0]
        quit_next = (n_curr >= node_terminate_thresh) or (i_split + 1 == n_splits)
        bucket = max(get_next_bucket_size(n_curr), 1) if i_split > 0 else 1
        this_b = min(batch_process_size, bucket)
        types = func.classify_box(params, node_lo, node_hi, offset=offset) if n_curr else np.zeros(0, np.int32)
        n_boxes += n_curr
        if with_interior_nodes:
            m = types == SIGN_NEGATIVE
            interior.append((node_lo[m], node_hi[m]))
        if with_exterior_nodes:
            m = types == SIGN_POSITIVE
            exterior.append((node_lo[m], node_hi[m]))
        unk = types == SIGN_UNKNOWN
        if not quit_next:
            los, his = [], []
            for s in range(0, n_curr, this_b):
                sl = slice(s, s + this_b)
                m = unk[sl]
                (alo, ahi), (blo, bhi) = split_children(node_lo[sl][m], node_hi[sl][m])
                los += [alo, blo]
                his += [ahi, bhi]
            node_lo = np.concatenate(los) if los else np.zeros((0, 3), dt)
            node_hi = np.concatenate(his) if his else np.zeros((0, 3), dt)
        else:
            node_lo, node_hi = node_lo[unk], node_hi[unk]
            break
    out = {'unknown_node_valid': np.ones(node_lo.shape[0], bool),
           'unknown_node_lower': node_lo, 'unknown_node_upper': node_hi,
           'n_boxes_classified': n_boxes}
    for name, lst, flag in (('interior', interior, with_interior_nodes),
                            ('exterior', exterior, with_exterior_nodes)):
        if flag:
            lo = np.concatenate([a for a, _ in lst]) if lst else np.zeros((0, 3), dt)
            hi = np.concatenate([b for _, b in lst]) if lst else np.zeros((0, 3), dt)
            out[f'{name}_node_valid'] = np.ones(lo.shape[0], bool)
            out[f'{name}_node_lower'] = lo
            out[f'{name}_node_upper'] = hi
    return out


# ----------------------------------------------------------------------------------------
# Hierarchical marching cubes  (src/kd_tree.py:338-399, src/extract_cell.py:306-421)
# ----------------------------------------------------------------------------------------

def sample_surface(func, params, lower, upper, n_samples, width, rng, n_node_thresh=4096):
    """src/kd_tree.py:254-292 with NumPy's generator in place of JAX's: uniform node,
    uniform point in it, kept when |f| < width, until n_samples are found."""
    d = construct_uniform_unknown_levelset_tree(func, params, lower, upper, node_terminate_thresh=n_node_thresh,
                                                offset=width)
    lo, hi = d['unknown_node_lower'][d['unknown_node_valid']], d['unknown_node_upper'][d['unknown_node_valid']]
    per = min(3 * n_samples, 100000)
    found = []
    total = 0
    while total < n_samples:
        idx = rng.integers(0, lo.shape[0], per)
        p = (lo[idx] + rng.uniform(0, 1, (per, 3)).astype(np.float32) * (hi[idx] - lo[idx])).astype(np.float32)
        keep = p[np.abs(func(params, p)) < width]
        found.append(keep)
        total += keep.shape[0]
    return np.concatenate(found)[:n_samples], (lo, hi)


def bulk_properties(func, params, lower, upper, rng, n_expand=10000, n_sample=1000000):
    """src/kd_tree.py:836-863 with NumPy's generator: interior nodes exactly, unknown
    nodes by Monte Carlo; returns (mass, centroid) in float64."""
    d = construct_uniform_unknown_levelset_tree(func, params, lower, upper, node_terminate_thresh=n_expand,
                                                with_interior_nodes=True)
    ilo = d['interior_node_lower'][d['interior_node_valid']].astype(np.float64)
    ihi = d['interior_node_upper'][d['interior_node_valid']].astype(np.float64)
    vol = np.prod(ihi - ilo, axis=-1)
    mass_i = vol.sum()
    cen_i = (vol[:, None] * 0.5 * (ilo + ihi)).sum(0)
    lo = d['unknown_node_lower'][d['unknown_node_valid']]
    hi = d['unknown_node_upper'][d['unknown_node_valid']]
    idx = rng.integers(0, lo.shape[0], n_sample)
    p = (lo[idx] + rng.uniform(0, 1, (n_sample, 3)).astype(np.float32) * (hi[idx] - lo[idx])).astype(np.float32)
    inside = func(params, p) < 0
    vps = np.prod((hi - lo).astype(np.float64), axis=-1).sum() / n_sample
    mass = mass_i + vps * inside.sum()
    cen = (cen_i + vps * p[inside].astype(np.float64).sum(0)) / mass
    return mass, cen


def extract_triangles_from_subcells(func, params, mc_data, n_sub_depth, cell_lo, cell_hi):
    """src/extract_cell.py:366-421 batched over leaves: returns tris (L, S*5, 3, 3) and
    valid (L, S*5)."""
    tri_table, edge_verts, vert_logical = mc_data
    dt = func.dtype
    L = cell_lo.shape[0]
    ns = 2 ** n_sub_depth
    npts = ns + 1
    # jnp.linspace(lo, hi, num): lo + i * (hi - lo) / (num - 1), endpoint exact
    coords = [jax_linspace(cell_lo[:, k:k + 1], cell_hi[:, k:k + 1], npts, dt) for k in range(3)]
    gx = np.broadcast_to(coords[0][:, :, None, None], (L, npts, npts, npts))
    gy = np.broadcast_to(coords[1][:, None, :, None], (L, npts, npts, npts))
    gz = np.broadcast_to(coords[2][:, None, None, :], (L, npts, npts, npts))
    pts = np.stack((gx, gy, gz), axis=-1).reshape(-1, 3)
    vals = func(params, pts).reshape(L, npts, npts, npts)
    si = np.stack(np.meshgrid(np.arange(ns), np.arange(ns), np.arange(ns), indexing='ij'), axis=-1).reshape(-1, 3)
    delta = (cell_hi - cell_lo) / np.asarray(ns, dt)
    sub_lo = cell_lo[:, None, :] + si[None, :, :].astype(dt) * delta[:, None, :]
    sub_hi = sub_lo + delta[:, None, :]
    vinds = si[:, None, :] + vert_logical[None, :, :].astype(np.int64)          # (S, 8, 3)
    vvals = vals[:, vinds[..., 0], vinds[..., 1], vinds[..., 2]]               # (L, S, 8)
    vpos = np.where(vert_logical[None, None, :, :], sub_hi[:, :, None, :], sub_lo[:, :, None, :])  # (L,S,8,3)
    # extract_triangles_from_cell (src/extract_cell.py:314-364)
    iA, iB = edge_verts[:, 0], edge_verts[:, 1]
    vA, vB = vvals[:, :, iA], vvals[:, :, iB]
    with np.errstate(divide='ignore', invalid='ignore'):
        tc = -vA / (vB - vA)
    tc = np.clip(np.nan_to_num(tc), 0, 1)
    eloc = (1. - tc)[..., None] * vpos[:, :, iA, :] + tc[..., None] * vpos[:, :, iB, :]  # (L,S,12,3)
    case = np.sum((vvals < 0).astype(np.int64) << np.arange(8)[None, None, :], axis=-1)  # (L,S)
    tris_e = tri_table[case][..., :15].reshape(L, -1, 5, 3)                       # (L,S,5,3)
    valid = tris_e[..., 0] != -1
    ei = np.clip(tris_e, 0, None)
    Ls, Ss = np.meshgrid(np.arange(L), np.arange(eloc.shape[1]), indexing='ij')
    tri = eloc[Ls[:, :, None, None], Ss[:, :, None, None], ei]                    # (L,S,5,3,3)
    return tri.reshape(L, -1, 3, 3), valid.reshape(L, -1)


def hierarchical_marching_cubes(func, params, lower, upper, depth, mc_data, n_subcell_depth=2):
    """src/kd_tree.py:357-399; returns (T, 3, 3) in the reference's order."""
    tree = construct_uniform_unknown_levelset_tree(func, params, lower, upper,
                                                   split_depth=3 * (depth - n_subcell_depth))
    lo, hi = tree['unknown_node_lower'], tree['unknown_node_upper']
    if lo.shape[0] == 0:
        return np.zeros((0, 3, 3), func.dtype)
    out = []
    for s in range(0, lo.shape[0], 4096):
        tri, valid = extract_triangles_from_subcells(func, params, mc_data, n_subcell_depth,
                                                     lo[s:s + 4096], hi[s:s + 4096])
        out.append(tri[valid])
    return np.concatenate(out)


# ----------------------------------------------------------------------------------------
# Pairwise intersection  (src/kd_tree.py:402-655)
# ----------------------------------------------------------------------------------------

def _sample_offsets(d=3):
    return np.concatenate((np.zeros((1, d)), np.eye(d), -np.eye(d)), axis=0)  # (7, d)


def find_any_intersection(funcs, params_list, lower, upper, eps, max_rounds=200):
    """src/kd_tree.py:402-655.  Returns (found, loc, n_nodes_processed)."""
    fA, fB = funcs
    pA, pB = params_list
    dt = fA.dtype
    lo = np.asarray(lower, dt)[None, :]
    hi = np.asarray(upper, dt)[None, :]
    eps_w = np.asarray(eps / np.sqrt(np.asarray(3., dt)), dt)
    offs = _sample_offsets().astype(dt)
    processed = 0
    for _ in range(max_rounds):
        n = lo.shape[0]
        if n == 0:
            return False, np.array((-777., -777., -777.), dt), processed
        processed += n
        width = np.max(hi - lo, axis=-1)
        small = width < eps_w
        center = 0.5 * (lo + hi)
        pts = center[:, None, :] + eps_w * offs[None, :, :]                     # (n,7,3)
        tA = fA.classify_box(pA, lo, hi)
        tB = fB.classify_box(pB, lo, hi)
        sA = fA(pA, pts.reshape(-1, 3)).reshape(n, 7)
        sB = fB(pB, pts.reshape(-1, 3)).reshape(n, 7)
        same = lambda s: np.all(s < 0, axis=1) | np.all(s > 0, axis=1)
        nearA = small & ~same(sA)
        nearB = small & ~same(sB)
        found = np.zeros(n, bool)
        loc = np.full((n, 3), -777., dt)
        iA = np.argmax(sA < 0, axis=1)
        iB = np.argmax(sB < 0, axis=1)
        anyA = sA[np.arange(n), iA] < 0
        anyB = sB[np.arange(n), iB] < 0
        near_neg = small & anyA & anyB
        found |= near_neg
        locA = pts[np.arange(n), iA]
        locB = pts[np.arange(n), iB]
        loc = np.where(near_neg[:, None], 0.5 * (locA + locB), loc)
        both = (sA < 0) & (sB < 0)
        ib = np.argmax(both, axis=1)
        has_both = both[np.arange(n), ib]
        found |= has_both
        loc = np.where(has_both[:, None], pts[np.arange(n), ib], loc)
        cinA = (tA == SIGN_NEGATIVE) | ((tA == SIGN_UNKNOWN) & ~nearA)
        cinB = (tB == SIGN_NEGATIVE) | ((tB == SIGN_UNKNOWN) & ~nearB)
        if np.any(found):
            k = int(np.argmax(found))
            return True, loc[k], processed
        sub = cinA & cinB
        (alo, ahi), (blo, bhi) = split_children(lo[sub], hi[sub])
        m = alo.shape[0]
        lo = np.stack((alo, blo), axis=1).reshape(2 * m, 3)                     # interleave
        hi = np.stack((ahi, bhi), axis=1).reshape(2 * m, 3)
    raise RuntimeError("intersection search did not terminate")


# ----------------------------------------------------------------------------------------
# Closest point  (src/kd_tree.py:659-802)
# ----------------------------------------------------------------------------------------

def closest_point(func, params, lower, upper, query_points, eps=0.001, batch_process_size=2048, trace=False):
    """src/kd_tree.py:659-802 with the same global LIFO stack and batch pops.

    With ``trace`` a third value is returned, a dict: ``near`` (Q,) bool, True for a
    query one of whose node decisions sat within NEAR_REL of flipping (the box
    classification, a sample's sign, or the pruning comparison cdist < best);
    ``first_near_round``, the first round in which any query took such a decision; and
    ``last_round`` (Q,), the last round that processed a node of the query.  All
    queries share one stack, so after the first near decision the batches of two
    implementations may hold different nodes; a query can then differ between them only
    if it is ``near`` itself or still had nodes processed at or after that round."""
    dt = func.dtype
    q = np.asarray(query_points, dt)
    Q = q.shape[0]
    B = batch_process_size
    st_lo = np.repeat(np.asarray(lower, dt)[None, :], Q, axis=0)
    st_hi = np.repeat(np.asarray(upper, dt)[None, :], Q, axis=0)
    st_id = np.arange(Q)
    top = Q
    min_dist = np.full(Q, np.inf, dt)
    min_loc = np.full((Q, 3), -777., dt)
    eps_w = np.asarray(eps / np.sqrt(np.asarray(3., dt)), dt)
    offs = _sample_offsets().astype(dt)
    rounds = 0
    near_q = np.zeros(Q, bool)
    last_round = np.full(Q, -1, np.int64)
    first_near_round = None
    while top > 0:
        pop = max(top - B, 0)
        lo, hi, ids = st_lo[pop:top], st_hi[pop:top], st_id[pop:top]
        n = top - pop
        ql = q[ids]
        qmd = min_dist[ids]
        width = np.max(hi - lo, axis=-1)
        center = 0.5 * (lo + hi)
        diag = np.sqrt(np.sum(np.square(hi - lo), axis=-1))
        cdist = np.linalg.norm(ql - center, axis=-1).astype(dt)
        max_d = cdist + diag
        small = width < eps_w
        pts = center[:, None, :] + (hi - lo)[:, None, :] * offs[None, :, :]
        if trace:
            c_ = 0.5 * (lo + hi)
            v_ = np.zeros((n, 3, 3), dt)
            v_[:, np.arange(3), np.arange(3)] = hi - c_
            blo, bhi, near = func.bounds_near(params, c_, v_)
            types = sign_from_bounds(blo, bhi)
        else:
            types = func.classify_box(params, lo, hi)
        outside = (types == SIGN_NEGATIVE) | (types == SIGN_POSITIVE)
        sv = func(params, pts.reshape(-1, 3)).reshape(n, 7)
        spans = ~(np.all(sv < 0, axis=1) | np.all(sv > 0, axis=1))
        this_d = np.where(spans, max_d, np.inf).astype(dt)
        needs = (~outside) & (~small) & (cdist < qmd)
        if trace:
            svn = np.abs(sv.astype(np.float64))
            near |= np.any(svn <= NEAR_REL * np.maximum(svn.max(axis=1, keepdims=True), 1.0), axis=1)
            fin = np.isfinite(qmd)
            near |= fin & (np.abs(cdist.astype(np.float64) - qmd) <=
                           NEAR_REL * np.maximum(cdist, np.where(fin, qmd, 0)).astype(np.float64))
            near_q[ids[near]] = True
            last_round[ids] = rounds
            if first_near_round is None and near.any():
                first_near_round = rounds
        np.minimum.at(min_dist, ids, this_d)
        newmin = this_d == min_dist[ids]
        min_loc[ids[newmin]] = center[newmin]   # scatter-set; the last duplicate wins
        (alo, ahi), (blo, bhi) = split_children(lo[needs], hi[needs])
        m = alo.shape[0]
        new_lo = np.stack((alo, blo), axis=1).reshape(2 * m, 3)
        new_hi = np.stack((ahi, bhi), axis=1).reshape(2 * m, 3)
        new_id = np.repeat(ids[needs], 2)
        st_lo = np.concatenate((st_lo[:pop], new_lo))
        st_hi = np.concatenate((st_hi[:pop], new_hi))
        st_id = np.concatenate((st_id[:pop], new_id))
        top = pop + 2 * m
        rounds += 1
    if trace:
        return min_dist, min_loc, {'near': near_q, 'last_round': last_round,
                                   'first_near_round': np.iinfo(np.int64).max if first_near_round is None
                                   else first_near_round}
    return min_dist, min_loc
