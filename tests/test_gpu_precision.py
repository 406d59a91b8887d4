"""Precision of the bounds on the deep model: ReLU 3->256x8->1 (He-normal seed 7,
median-biased output), 'affine_fixed' and 'affine_truncate' with up to 256 noise terms.

* Containment: 1000 boxes x 1000 FP64 samples (10^6 in all) of the same network, zero
  samples outside the conservative bound.
* Width: the conservative bound against the FP64 oracle's affine bound (the oracle
  restates src/affine.py in float64), reported as the median relative excess; held
  below 0.5 for 'affine_fixed'.  With 256 kept rows the rigorous rounding terms of eight
  256-wide layers create a symbol per neuron per layer; truncation drops most of them
  into err, whose |A| propagation grows about 9x per layer, so the truncated bound's
  excess is reported only.
* Parity: the reference-arithmetic bound (conservative=False) against the FP32 oracle,
  within 3e-4 of the bound scale max(|lo|, |hi|) + 1e-3 (256-term dot products summed in
  a different order, then truncation near-ties, across eight layers).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODES = [('affine_fixed', {}, 'auto'), ('affine_truncate', {'affine_n_truncate': 256}, 'fp32'),
         ('affine_truncate', {'affine_n_truncate': 256}, '3xtf32')]
N_BOXES = 1000
N_SAMPLES = 1000


def _boxes(rng, n):
    """Half the boxes are ray segments (v=1), half axis-aligned boxes (v=3), centred
    where the network is near its level set and small enough to be undecided."""
    c = rng.uniform(-0.8, 0.8, (n, 3)).astype(np.float32)
    v3 = np.zeros((n // 2, 3, 3), np.float32)
    half = np.exp(rng.uniform(np.log(1e-3), np.log(0.1), (n // 2, 3))).astype(np.float32)
    v3[:, np.arange(3), np.arange(3)] = half
    d = rng.standard_normal((n - n // 2, 1, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    v1 = (d * np.exp(rng.uniform(np.log(1e-3), np.log(0.1), (n - n // 2, 1, 1)))).astype(np.float32)
    return (c[:n // 2], v3), (c[n // 2:], v1)


def _fp64_forward(params, R, pts):
    out = np.empty(pts.shape[0])
    for s in range(0, pts.shape[0], 1 << 17):
        out[s:s + (1 << 17)] = R.eval_points(params, pts[s:s + (1 << 17)], np.float64)
    return out


@pytest.mark.parametrize('mode,kw,products', MODES)
def test_deep_model_containment_and_width(niq, R, gpu_ready, mode, kw, products):
    params = niq.workloads.precision_model()
    rng = np.random.default_rng(7)
    f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=True, products=products,
                                                                **kw)
    o = R.generate_implicit(params, mode, dtype=np.float64, **kw)
    excess = []
    n_checked = 0
    for c, vv in _boxes(rng, N_BOXES):
        sign, lo, hi = f.bounds_general_box(params, c, vv)
        v = vv.shape[1]
        eps = rng.uniform(-1, 1, (N_SAMPLES, v))
        eps[:2 ** v] = np.array(np.meshgrid(*[[-1., 1.]] * v, indexing='ij')).reshape(v, -1).T
        pts = c[None].astype(np.float64) + np.einsum('sv,nvd->snd', eps, vv.astype(np.float64))
        vals = _fp64_forward(params, R, pts.reshape(-1, 3)).reshape(N_SAMPLES, -1)
        bad = (vals < lo[None]) | (vals > hi[None])
        assert not bad.any(), (mode, v, int(bad.sum()))
        n_checked += vals.size
        for s in range(0, c.shape[0], 100):
            rlo, rhi = o.bounds_general(params, c[s:s + 100].astype(np.float64), vv[s:s + 100].astype(np.float64))
            excess.append(((hi[s:s + 100] - lo[s:s + 100]) - (rhi - rlo)) / np.maximum(rhi - rlo, 1e-30))
    assert n_checked == N_BOXES * N_SAMPLES
    ex = np.concatenate(excess)
    print('deep model width excess over FP64 (median, p90)', mode, products, float(np.median(ex)),
          float(np.percentile(ex, 90)))
    if mode == 'affine_fixed':
        assert np.median(ex) < 0.5, (mode, products, float(np.median(ex)))


@pytest.mark.parametrize('mode,kw,products', MODES)
def test_deep_model_matches_oracle(niq, R, gpu_ready, mode, kw, products):
    params = niq.workloads.precision_model()
    rng = np.random.default_rng(8)
    f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=False, products=products,
                                                                **kw)
    o = R.generate_implicit(params, mode, **kw)
    for c, vv in _boxes(rng, 128):
        sign, lo, hi = f.bounds_general_box(params, c, vv)
        rlo, rhi = o.bounds_general(params, c, vv)
        scale = np.maximum(np.abs(rlo), np.abs(rhi)) + 1e-3
        err = max(np.max(np.abs(lo - rlo) / scale), np.max(np.abs(hi - rhi) / scale))
        assert err <= 3e-4, (mode, products, vv.shape[1], err)


@pytest.mark.parametrize('act', ['relu', 'tanh'])
@pytest.mark.parametrize('mode,kw', [('affine_truncate', {'affine_n_truncate': 64}),
                                     ('affine_truncate', {'affine_n_truncate': 200}), ('affine_all', {})])
def test_tensor_core_products_match_fp32(niq, R, gpu_ready, act, mode, kw):
    """The 3xTF32 engine against the oracle and the FP32 engine on narrower models:
    widths 64..256, depth 2..4, ReLU and TanH (affine_all on a model whose rows stay
    within 256)."""
    rng = np.random.default_rng(11)
    shapes = [[3, 128, 128, 1], [3, 256, 96, 160, 1], [3, 64, 64, 64, 64, 1]] if mode != 'affine_all' else \
        [[3, 64, 96, 1], [3, 48, 48, 48, 1]]
    for i, sizes in enumerate(shapes):
        params = niq.workloads.he_mlp(sizes, act, seed=20 + i, grid=16)
        o = R.generate_implicit(params, mode, **kw)
        for v in (3, 1):
            c = rng.uniform(-1, 1, (200, 3)).astype(np.float32)
            vv = (rng.standard_normal((200, v, 3)) * np.exp(rng.uniform(np.log(1e-3), np.log(0.2), (200, v, 1))))
            vv = vv.astype(np.float32)
            rlo, rhi = o.bounds_general(params, c, vv)
            scale = np.maximum(np.abs(rlo), np.abs(rhi)) + 1e-3
            got = {}
            for products in ('fp32', '3xtf32'):
                f, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=False,
                                                                            products=products, **kw)
                _, lo, hi = f.bounds_general_box(params, c, vv)
                err = max(np.max(np.abs(lo - rlo) / scale), np.max(np.abs(hi - rhi) / scale))
                # TanH secant slopes amplify last-ulp differences into truncation near-ties
                assert err <= (3e-4 if act == 'relu' else 3e-3), (sizes, act, mode, v, products, err)
                got[products] = (lo, hi)
                # conservative bounds contain the reference-arithmetic ones up to FP32 noise
                fc, _ = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=True,
                                                                             products=products, **kw)
                _, clo, chi = fc.bounds_general_box(params, c, vv)
                assert np.all(clo <= rlo + 1e-4 * scale) and np.all(chi >= rhi - 1e-4 * scale), (sizes, products)
