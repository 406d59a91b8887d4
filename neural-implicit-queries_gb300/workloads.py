"""Seeded synthetic workloads for the query engine (NumPy only, no GPU).

Models are produced in the reference's dict spec format (``"%04d.<op>.<arg>"`` keys,
``dense.A`` of shape (in, out) applied as ``x @ A + b``; src/mlp.py:14-24,218-249) so they
load through the same code as the reference's ``.npz`` files.

The reference has no random-MLP generator of its own beyond Glorot init inside
training (src/mlp.py:260-276); these generators are this project's:

* ``he_mlp``: He-normal weights ``N(0, 2/fan_in)``, zero hidden biases, and (by default)
  the output bias shifted so that the median of the output over a 64^3 grid in
  [-1, 1]^3 is zero, which places a closed-ish level set inside the unit box.
* ``spheres_sdf_model``: a 3->64x4->1 ReLU MLP fitted with Adam to the signed distance
  of a union of 12 spheres; the fitted weights are committed next to this file and
  regenerated by ``data/make_models.py``.
"""
from __future__ import annotations

import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))


def build_spec(op_list):
    """src/mlp.py:14-24: prefix each op's keys with its 4-digit index."""
    out = {}
    for i, op in enumerate(op_list):
        for k, v in op.items():
            out[f"{i:04d}.{k}"] = v
    return out


def _forward_np(params_ops, x):
    for kind, A, b in params_ops:
        x = x @ A + b
        if kind == 'relu':
            x = np.maximum(x, 0)
        elif kind == 'tanh':
            x = np.tanh(x)
        elif kind == 'elu':
            x = np.where(x > 0, x, np.expm1(np.minimum(x, 0)))
    return x[:, 0]


def he_mlp(sizes, activation='relu', seed=0, median_bias=True, grid=64):
    """ReLU/TanH/ELU MLP ``sizes[0] -> ... -> sizes[-1]`` with He-normal weights."""
    rng = np.random.default_rng(seed)
    ops = []
    layers = []
    for i in range(len(sizes) - 1):
        fin, fout = sizes[i], sizes[i + 1]
        A = (rng.standard_normal((fin, fout)) * np.sqrt(2.0 / fin)).astype(np.float32)
        b = np.zeros(fout, np.float32)
        last = i + 2 == len(sizes)
        layers.append(('none' if last else activation, A, b))
    if median_bias:
        ax = np.linspace(-1., 1., grid, dtype=np.float32)
        g = np.stack(np.meshgrid(ax, ax, ax, indexing='ij'), -1).reshape(-1, 3)
        vals = np.concatenate([_forward_np(layers, g[s:s + 65536]) for s in range(0, g.shape[0], 65536)])
        layers[-1][2][:] -= np.float32(np.median(vals))
    for kind, A, b in layers:
        ops.append({'dense.A': A, 'dense.b': b})
        if kind != 'none':
            ops.append({f'{kind}._': np.zeros((0,), np.float32)})
    ops.append({'squeeze_last._': np.zeros((0,), np.float32)})
    return build_spec(ops)


def prepend_spatial_transformation(params, R=None, t=None):
    """src/mlp.py:149-167 + src/mlp.py:335-339: shift every op index up by one and put a
    ``spatial_transformation`` (R, t) in slot 0000."""
    out = {}
    for k, v in params.items():
        parts = k.split('.')
        parts[0] = f"{int(parts[0]) + 1:04d}"
        out['.'.join(parts)] = v
    out['0000.spatial_transformation.R'] = np.eye(3, dtype=np.float32) if R is None else np.asarray(R, np.float32)
    out['0000.spatial_transformation.t'] = np.zeros(3, np.float32) if t is None else np.asarray(t, np.float32)
    return out


def random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], np.float32)


# ------------------------------------------------------------------ the five workloads

def plain_small_model():
    """3->32->32->32->1 ReLU, He-normal seed 0, median-biased output."""
    return he_mlp([3, 32, 32, 32, 1], 'relu', seed=0)


def precision_model():
    """3->256x8->1 ReLU, He-normal seed 7, median-biased output."""
    return he_mlp([3] + [256] * 8 + [1], 'relu', seed=7)


SPHERES_NPZ = os.path.join(_HERE, 'data', 'spheres12_relu64x4.npz')


def spheres_scene(seed=1):
    """12 spheres: centers U[-0.6, 0.6]^3, radii U[0.1, 0.3]."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-0.6, 0.6, (12, 3))
    radii = rng.uniform(0.1, 0.3, 12)
    return centers, radii


def spheres_sdf(x, centers, radii):
    d = np.linalg.norm(x[:, None, :] - centers[None, :, :], axis=-1) - radii[None, :]
    return d.min(axis=1)


def spheres_sdf_model():
    """The fitted 3->64x4->1 ReLU level-set model (loads the committed npz)."""
    with np.load(SPHERES_NPZ) as d:
        return {k: d[k] for k in d.files}


def batched_models(n=512, seed0=0):
    """``n`` MLPs: widths U{16..128}, hidden depths U{2..6}, ReLU or TanH (p=0.5),
    He-normal with seeds ``seed0 .. seed0+n-1``."""
    out = []
    for i in range(n):
        rng = np.random.default_rng(10_000 + seed0 + i)
        w = int(rng.integers(16, 129))
        d = int(rng.integers(2, 7))
        act = 'relu' if rng.random() < 0.5 else 'tanh'
        out.append(he_mlp([3] + [w] * d + [1], act, seed=seed0 + i, grid=24))
    return out


def batched_queries(n_models=512, seed=0):
    """Per model: round(exp(U[ln 64, ln 4096])) query points uniform in [-1.2, 1.2]^3."""
    rng = np.random.default_rng(seed)
    counts = np.round(np.exp(rng.uniform(np.log(64), np.log(4096), n_models))).astype(np.int64)
    pts = [rng.uniform(-1.2, 1.2, (int(c), 3)).astype(np.float32) for c in counts]
    return pts


def serving_models(n=64, seed0=100):
    """``n`` resident MLPs: widths U{32..256}, hidden depths U{3..8}, seeds 100..163."""
    out = []
    for i in range(n):
        rng = np.random.default_rng(20_000 + seed0 + i)
        w = int(rng.integers(32, 257))
        d = int(rng.integers(3, 9))
        act = 'relu' if rng.random() < 0.5 else 'tanh'
        out.append(he_mlp([3] + [w] * d + [1], act, seed=seed0 + i, grid=24))
    return out


def fit_sdf_mlp(sizes, sdf_fn, steps=2000, lr=1e-3, seed=1, n_points=2 ** 18, box=1.0,
                batch=None, log_every=0):
    """Fit a ReLU MLP to a signed distance function with Adam on the CPU (torch).

    ``n_points`` samples uniform in [-box, box]^3 are drawn once with ``seed``; each of
    the ``steps`` Adam steps uses all of them (``batch=None``) or a seeded minibatch.
    Returns the model in the reference's dict spec format."""
    import torch
    g = torch.Generator().manual_seed(seed)
    rng = np.random.default_rng(seed)
    x = rng.uniform(-box, box, (n_points, 3)).astype(np.float32)
    y = sdf_fn(x).astype(np.float32)
    X, Y = torch.from_numpy(x), torch.from_numpy(y)
    layers = []
    for i in range(len(sizes) - 1):
        lin = torch.nn.Linear(sizes[i], sizes[i + 1])
        with torch.no_grad():
            lin.weight.normal_(0.0, float(np.sqrt(2.0 / sizes[i])), generator=g)
            lin.bias.zero_()
        layers.append(lin)
    net = torch.nn.ModuleList(layers)

    def fwd(z):
        for i, l in enumerate(net):
            z = l(z)
            if i + 1 < len(net):
                z = torch.relu(z)
        return z[:, 0]
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    for s in range(steps):
        if batch is None:
            xb, yb = X, Y
        else:
            idx = torch.randint(0, n_points, (batch,), generator=g)
            xb, yb = X[idx], Y[idx]
        loss = torch.mean((fwd(xb) - yb) ** 2)
        opt.zero_grad()
        loss.backward()
        opt.step()
        if log_every and s % log_every == 0:
            print(f"fit step {s} loss {loss.item():.3e}", flush=True)
    ops = []
    for i, l in enumerate(net):
        ops.append({'dense.A': l.weight.detach().numpy().T.copy().astype(np.float32),
                    'dense.b': l.bias.detach().numpy().copy().astype(np.float32)})
        if i + 1 < len(net):
            ops.append({'relu._': np.zeros((0,), np.float32)})
    ops.append({'squeeze_last._': np.zeros((0,), np.float32)})
    return build_spec(ops)


def sphere_sdf_fn(center, radius):
    c = np.asarray(center, np.float64)
    return lambda x: (np.linalg.norm(x - c[None, :], axis=-1) - radius)
