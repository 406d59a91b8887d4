"""A NumPy stand-in for the parts of ``jax`` that nmwsharp/neural-implicit-queries uses.

Used only by ``make_golden.py`` to execute the reference's own ``src/*.py`` in a
container without JAX.  ``install()`` registers fake ``jax``, ``jax.numpy``,
``jax.lax``, ``jax.nn`` modules plus empty stubs for the GUI-only imports
(polyscope, matplotlib, imageio, igl, skimage) that the reference pulls in at import
time (src/utils.py:10-11, src/queries.py:9, src/render.py:9).

Semantics follow JAX with 64-bit mode off: floats default to float32 and integers to
int32; ``jit`` is the identity; ``vmap`` is a Python loop over the leading axis;
``x.at[idx].set/min/get`` follow JAX's out-of-bounds rules (updates dropped, gathers
clamped unless ``mode='fill'``/``'drop'``, negative indices wrapped); ``argsort`` is
stable; ``lax.top_k`` breaks ties towards the lower index; ``linspace`` uses
``start*(1-s) + stop*s``.  Arithmetic is NumPy's, so results match XLA's only up to
floating-point rounding.
"""
from __future__ import annotations

import sys
import types

import numpy as np

F32, I32 = np.float32, np.int32


def _canon_dtype(dt):
    if dt is None:
        return None
    if dt is float or dt == np.float64:
        return F32
    if dt is int or dt == np.int64:
        return I32
    if dt is bool:
        return np.bool_
    return np.dtype(dt).type


class JArr(np.ndarray):
    """ndarray with JAX's functional ``.at`` indexer."""

    @property
    def at(self):
        return _AtHelper(self)

    def __getitem__(self, idx):
        # NumPy-style retrieval: JAX wraps negative indices and clamps the rest
        tup = idx if isinstance(idx, tuple) else (idx,)
        if any(isinstance(it, (np.ndarray, list, tuple)) and np.asarray(it).dtype.kind in 'iu'
               for it in tup):
            nidx = _norm_index(tup, self.shape)
            dims = _index_dims(nidx, self.shape)
            fixed, k = [], 0
            for it in nidx:
                if it is Ellipsis:
                    fixed.append(it)
                    continue
                if isinstance(it, np.ndarray) and it.dtype.kind in 'iu':
                    it = np.clip(it, 0, self.shape[dims[k]] - 1)
                fixed.append(it)
                k += 1
            return super().__getitem__(tuple(fixed))
        return super().__getitem__(idx)

    def block_until_ready(self):
        return self


def _wrap(x):
    """Canonicalise a result to a JArr of 32-bit type."""
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    a = np.asarray(x)
    if a.dtype == np.float64:
        a = a.astype(F32)
    elif a.dtype == np.int64:
        a = a.astype(I32)
    return a.view(JArr)


def _norm_index(idx, shape):
    """Wrap negative integer-array indices (JAX normalises them like NumPy)."""
    if not isinstance(idx, tuple):
        idx = (idx,)
    out = []
    dim = 0
    for it in idx:
        if it is Ellipsis:
            out.append(it)
            dim = len(shape) - (len(idx) - len(out))
            continue
        if isinstance(it, tuple):  # a tuple from jnp.nonzero nested in the index
            it = np.asarray(it)
        if isinstance(it, (np.ndarray, list)) and np.asarray(it).dtype != np.bool_:
            a = np.asarray(it).astype(np.int64)
            n = shape[dim] if dim < len(shape) else 1
            a = np.where(a < 0, a + n, a)
            out.append(a)
        elif isinstance(it, (int, np.integer)) and not isinstance(it, bool):
            n = shape[dim] if dim < len(shape) else 1
            out.append(int(it) + n if it < 0 else int(it))
        else:
            out.append(it)
        dim += 1
    return tuple(out)


def _index_dims(idx, shape):
    """For each entry of ``idx``, the axis it indexes (ints and arrays only)."""
    dims = []
    dim = 0
    n_real = sum(1 for it in idx if it is not Ellipsis)
    for it in idx:
        if it is Ellipsis:
            dim = len(shape) - (n_real - len(dims))
            continue
        dims.append(dim)
        dim += 1
    return dims


class _AtRef:
    def __init__(self, arr, idx):
        self.arr = np.asarray(arr)
        self.idx = _norm_index(idx, self.arr.shape)

    def _inbounds_mask(self):
        """Broadcast mask of index tuples whose integer components are in bounds, and a
        clipped copy of the index."""
        shape = self.arr.shape
        dims = _index_dims(self.idx, shape)
        arrays, clipped = [], []
        k = 0
        for it in self.idx:
            if it is Ellipsis:
                clipped.append(it)
                continue
            d = dims[k]
            k += 1
            if isinstance(it, np.ndarray):
                arrays.append((it >= 0) & (it < shape[d]))
                clipped.append(np.clip(it, 0, shape[d] - 1))
            else:
                clipped.append(it)
        mask = np.broadcast_arrays(*arrays)[0].copy() if arrays else None
        if arrays:
            for m in arrays[1:]:
                mask &= np.broadcast_to(m, mask.shape)
        return mask, tuple(clipped)

    def get(self, mode=None, fill_value=None, **_):
        mask, clipped = self._inbounds_mask()
        out = self.arr[clipped]
        if mode in ('fill', 'drop') and mask is not None and not mask.all():
            if fill_value is None:
                # jax's gather fill: NaN for floats, min for signed, max for unsigned, True for bool
                if np.issubdtype(out.dtype, np.inexact):
                    fill_value = np.nan
                elif out.dtype == np.bool_:
                    fill_value = True
                elif np.issubdtype(out.dtype, np.unsignedinteger):
                    fill_value = np.iinfo(out.dtype).max
                else:
                    fill_value = np.iinfo(out.dtype).min
            out = np.array(out)
            bad = ~mask
            out[bad] = np.asarray(fill_value).astype(out.dtype)
        return _wrap(out)

    def _scatter(self, vals, op):
        arr = np.array(self.arr)
        mask, clipped = self._inbounds_mask()
        vals = np.asarray(vals).astype(arr.dtype)
        if mask is None:
            if op == 'set':
                arr[self.idx] = vals
            else:
                arr[self.idx] = np.minimum(arr[self.idx], vals)
            return _wrap(arr)
        # drop out-of-bounds updates: restrict the index arrays and the values
        target_shape = arr[clipped].shape
        vals = np.broadcast_to(vals, target_shape)
        lead = mask.ndim
        keep = mask.reshape(-1)
        vflat = vals.reshape((-1,) + target_shape[lead:]) if lead else vals
        sel = []
        for it in clipped:
            if isinstance(it, np.ndarray):
                sel.append(np.broadcast_to(it, mask.shape).reshape(-1)[keep])
            else:
                sel.append(it)
        sel = tuple(sel)
        if op == 'set':
            arr[sel] = vflat[keep]
        else:
            np.minimum.at(arr, sel, vflat[keep])
        return _wrap(arr)

    def set(self, vals, mode=None, **_):
        return self._scatter(vals, 'set')

    def min(self, vals, mode=None, **_):
        return self._scatter(vals, 'min')


class _AtHelper:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtRef(self.arr, idx)


# ------------------------------------------------------------------ jax.numpy
def _mk_jnp():
    m = types.ModuleType('jax.numpy')
    m.ndarray = JArr
    m.pi, m.inf, m.nan = np.pi, np.inf, np.nan
    m.float32, m.int32, m.bool_ = F32, I32, np.bool_

    def array(x, dtype=None):
        a = np.array(x, dtype=_canon_dtype(dtype))
        return _wrap(a)

    def _ctor(fn):
        def f(shape, dtype=None, *a, **k):
            return _wrap(fn(shape, *a, dtype=_canon_dtype(dtype) or F32, **k))
        return f

    m.array = array
    m.asarray = array
    m.zeros = _ctor(np.zeros)
    m.ones = _ctor(np.ones)

    def full(shape, fill_value, dtype=None):
        dt = _canon_dtype(dtype)
        if dt is None:
            dt = F32 if isinstance(fill_value, float) else (I32 if isinstance(fill_value, int) else None)
        return _wrap(np.full(shape, fill_value, dtype=dt))
    m.full = full
    m.zeros_like = lambda a, dtype=None: _wrap(np.zeros_like(a, dtype=_canon_dtype(dtype)))
    m.ones_like = lambda a, dtype=None: _wrap(np.ones_like(a, dtype=_canon_dtype(dtype)))

    def arange(*a, dtype=None, **k):
        dt = _canon_dtype(dtype)
        if dt is None:
            dt = F32 if any(isinstance(v, float) for v in list(a) + list(k.values())) else I32
        return _wrap(np.arange(*a, **k).astype(dt))
    m.arange = arange
    m.eye = lambda n, dtype=None: _wrap(np.eye(n, dtype=_canon_dtype(dtype) or F32))

    def linspace(start, stop, num=50, dtype=None):
        start = np.asarray(start, F32)
        stop = np.asarray(stop, F32)
        s = (np.arange(num, dtype=F32) / F32(num - 1)).astype(F32)
        out = start[..., None] * (1 - s) + stop[..., None] * s if start.ndim else start * (1 - s) + stop * s
        if dtype is not None and np.issubdtype(np.dtype(dtype), np.integer):
            # jax computes in floating point and converts (toward zero) to the integer type
            out = np.trunc(out).astype(np.int32)
        return _wrap(out)
    m.linspace = linspace

    def _f(fn):
        def g(*a, **k):
            return _wrap(fn(*a, **k))
        return g

    for name in ['where', 'sum', 'max', 'min', 'abs', 'sign', 'sqrt', 'square', 'exp', 'log', 'tan',
                 'sin', 'cos', 'arccos', 'deg2rad', 'logical_and', 'logical_or', 'logical_not',
                 'all', 'any', 'mean', 'cumsum', 'maximum', 'minimum', 'power', 'floor', 'ceil',
                 'dot', 'inner', 'cross', 'diag', 'reshape', 'squeeze', 'repeat', 'tile', 'roll',
                 'meshgrid', 'isnan', 'argmax', 'argmin', 'concatenate', 'stack', 'isinf']:
        setattr(m, name, _f(getattr(np, name)))
    m.product = _f(np.prod)
    m.prod = _f(np.prod)
    m.nan_to_num = lambda x, copy=True, nan=0.0, **k: _wrap(np.nan_to_num(np.asarray(x), nan=nan, **k))
    m.clip = lambda a, a_min=None, a_max=None: _wrap(np.clip(a, a_min, a_max))
    m.argsort = lambda a, axis=-1, **k: _wrap(np.argsort(a, axis=axis, kind='stable'))

    def nonzero(a, size=None, fill_value=None):
        res = np.nonzero(np.asarray(a))
        if size is None:
            return tuple(_wrap(r) for r in res)
        fv = 0 if fill_value is None else fill_value
        out = []
        for r in res:
            r = r[:size]
            if r.shape[0] < size:
                r = np.concatenate((r, np.full(size - r.shape[0], fv, dtype=r.dtype)))
            out.append(_wrap(r))
        return tuple(out)
    m.nonzero = nonzero

    lin = types.ModuleType('jax.numpy.linalg')
    lin.norm = lambda x, axis=None, **k: _wrap(np.linalg.norm(x, axis=axis, **k))
    lin.inv = lambda x: _wrap(np.linalg.inv(np.asarray(x)))
    m.linalg = lin
    return m, lin


# ------------------------------------------------------------------ jax, lax, nn
def _vmap(fn, in_axes=0, out_axes=0):
    def g(*args):
        n = None
        for a in args:
            if a is not None and np.ndim(a) > 0:
                n = np.shape(a)[0]
                break
        if n == 0:
            # mapped axis of length zero: trace one dummy element for the output shapes
            call = [None if a is None else _wrap(np.zeros(np.shape(a)[1:], np.asarray(a).dtype)) for a in args]
            o = fn(*call)
            mk = lambda r: _wrap(np.zeros((0,) + np.shape(r), np.asarray(r).dtype))
            return tuple(None if r is None else mk(r) for r in o) if isinstance(o, tuple) else mk(o)
        outs = []
        for i in range(n):
            call = [None if a is None else _wrap(np.asarray(a)[i]) for a in args]
            outs.append(fn(*call))
        if isinstance(outs[0], tuple):
            res = []
            for j in range(len(outs[0])):
                col = [o[j] for o in outs]
                if col[0] is None:
                    res.append(None)
                else:
                    res.append(_wrap(np.stack([np.asarray(c) for c in col])))
            return tuple(res)
        return _wrap(np.stack([np.asarray(o) for o in outs]))
    return g


def _jit(fn=None, **_):
    if fn is None:
        return lambda f: f
    return fn


def _mk_lax():
    lax = types.ModuleType('jax.lax')

    def fori_loop(lo, hi, body, init):
        # the carry becomes arrays, as in JAX (so ~ on a bool carry is a logical not)
        v = tuple(_wrap(x) for x in init) if isinstance(init, tuple) else _wrap(init)
        for i in range(lo, hi):
            v = body(i, v)
        return v
    lax.fori_loop = fori_loop
    lax.map = lambda f, xs: _wrap(np.stack([np.asarray(f(_wrap(x))) for x in np.asarray(xs)]))

    def top_k(x, k):
        x = np.asarray(x)
        order = np.argsort(-x, axis=-1, kind='stable')[..., :k]
        return _wrap(np.take_along_axis(x, order, axis=-1)), _wrap(order)
    lax.top_k = top_k

    def dynamic_slice_in_dim(x, start, size, axis=0):
        x = np.asarray(x)
        start = int(np.clip(int(start), 0, x.shape[axis] - size))
        return _wrap(np.take(x, np.arange(start, start + size), axis=axis))
    lax.dynamic_slice_in_dim = dynamic_slice_in_dim

    def dynamic_update_slice_in_dim(x, upd, start, axis=0):
        x = np.array(x)
        upd = np.asarray(upd)
        n = upd.shape[axis]
        start = int(np.clip(int(start), 0, x.shape[axis] - n))
        sl = [slice(None)] * x.ndim
        sl[axis] = slice(start, start + n)
        x[tuple(sl)] = upd
        return _wrap(x)
    lax.dynamic_update_slice_in_dim = dynamic_update_slice_in_dim
    lax.pow = lambda a, b: _wrap(np.power(a, b))
    return lax


def _mk_nn():
    nn = types.ModuleType('jax.nn')
    nn.relu = lambda x: _wrap(np.maximum(x, 0))
    nn.elu = lambda x: _wrap(np.where(np.asarray(x) > 0, x, np.expm1(np.where(np.asarray(x) > 0, 0, x))))
    init = types.ModuleType('jax.nn.initializers')

    def _unavailable(*a, **k):
        raise NotImplementedError("random initialisers are not part of the stand-in")
    init.glorot_normal = _unavailable
    init.normal = _unavailable
    nn.initializers = init
    return nn, init


def install():
    jnp, lin = _mk_jnp()
    lax = _mk_lax()
    nn, init = _mk_nn()
    jax = types.ModuleType('jax')
    jax.numpy, jax.lax, jax.nn = jnp, lax, nn
    jax.jit = _jit
    jax.vmap = _vmap
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    rnd = types.ModuleType('jax.random')

    def _no_rng(*a, **k):
        raise NotImplementedError("jax.random is not part of the stand-in")
    rnd.PRNGKey = rnd.split = rnd.uniform = rnd.randint = rnd.normal = rnd.permutation = _no_rng
    jax.random = rnd
    scipy = types.ModuleType('jax.scipy')
    scipy.ndimage = types.ModuleType('jax.scipy.ndimage')
    jax.scipy = scipy
    mods = {'jax': jax, 'jax.numpy': jnp, 'jax.numpy.linalg': lin, 'jax.lax': lax, 'jax.nn': nn,
            'jax.nn.initializers': init, 'jax.random': rnd, 'jax.scipy': scipy,
            'jax.scipy.ndimage': scipy.ndimage}
    for name in ['polyscope', 'polyscope.imgui', 'matplotlib', 'matplotlib.pyplot', 'imageio',
                 'igl', 'skimage', 'skimage.measure']:
        mods[name] = types.ModuleType(name)
    mods['polyscope'].imgui = mods['polyscope.imgui']
    mods['matplotlib'].pyplot = mods['matplotlib.pyplot']
    sys.modules.update(mods)
    return jax
