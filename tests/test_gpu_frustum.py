"""queries.cast_rays_frustum on the GPU against the oracle (oracle/ref_np.py) and the
reference's golden vectors.

Frusta march and split on sign decisions of bounds.  A pixel (hit id, count, t within
1e-4 relative) may differ from the oracle's only where the oracle's trace marks a
decision within rounding of its threshold on the pixel's frustum path -- a box bound, a
hit test, the refinement of a frustum, the step limit or the truncation of the count
(tests/parity.py, oracle.ref_np.cast_rays_frustum(trace=True))."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, model_from

pytestmark = pytest.mark.gpu


def gf(niq, params, mode='affine_fixed', conservative=False):
    return niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=conservative)[0]


def pixel_match(a, b):
    t, h, c = a[:3]
    rt, rh, rc = b[:3]
    return (h == rh) & (c == rc) & np.isclose(t, rt, rtol=1e-4, atol=1e-5)


def unexplained_pixels(got, ref, near):
    bad = ~pixel_match(got, ref)
    print(f'frustum: {int(bad.sum())} of {bad.size} pixels differ, {int((bad & near).sum())} explained '
          f'({int(near.sum())} pixels took a near decision)')
    return np.argwhere(bad & ~near)


def camera(R, eye, res_x, res_y, fov_x, fov_y):
    look, up, left = R.look_at(np.asarray(eye, np.float32))
    return (np.asarray(eye, np.float32), look, up, left, fov_x, fov_y, res_x, res_y)


@pytest.mark.parametrize('mode', ['affine_fixed', 'interval', 'slope_interval'])
def test_frustum_matches_oracle(niq, R, gpu_ready, mode):
    params = niq.workloads.plain_small_model()
    cam = camera(R, [0.3, 0.4, 2.8], 40, 32, 60., 50.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 96
    opts['n_side_init'] = 4
    got = niq.queries.cast_rays_frustum((gf(niq, params, mode),), (params,), cam, opts)
    ref = R.cast_rays_frustum((R.generate_implicit(params, mode),), (params,), cam, opts, trace=True)
    assert got[0].shape == (40, 32) and got[1].dtype == np.int32
    bad = unexplained_pixels(got, ref, ref[4])
    assert len(bad) == 0, (mode, bad[:10])
    if mode != 'interval':               # interval bounds stay undecided near the surface here
        assert (ref[1] > 0).sum() > 0    # the view holds surface


@pytest.mark.parametrize('mode,kw', [('affine_truncate', {'affine_n_truncate': 8}), ('affine_all', {}),
                                     ('affine_append', {'affine_n_append': 4})])
def test_frustum_growing_modes_match_oracle(niq, R, gpu_ready, mode, kw):
    """The growing-term modes: each substep's boxes go through the growing-term engine."""
    params = niq.workloads.plain_small_model()
    cam = camera(R, [0.3, 0.4, 2.8], 24, 20, 60., 50.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    opts['n_side_init'] = 4
    opts['n_substeps'] = 2
    f = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=False, **kw)[0]
    got = niq.queries.cast_rays_frustum((f,), (params,), cam, opts)
    ref = R.cast_rays_frustum((R.generate_implicit(params, mode, **kw),), (params,), cam, opts, trace=True)
    assert got[0].shape == (24, 20)
    bad = unexplained_pixels(got, ref, ref[4])
    assert len(bad) == 0, (mode, bad[:10])
    assert (ref[1] > 0).sum() > 0
    # the conservative growing-term cast terminates everywhere
    fc = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=True, **kw)[0]
    t, hid, cnt, nev = niq.queries.cast_rays_frustum((fc,), (params,), cam, opts)
    assert nev > 0 and np.all(np.isfinite(t)) and np.all(cnt >= 0)


def test_frustum_two_functions_substeps(niq, R, gpu_ready):
    p1 = niq.workloads.plain_small_model()
    p2 = niq.workloads.he_mlp([3, 64, 64, 1], 'tanh', seed=5, grid=16)
    cam = camera(R, [0., 0., 3.], 33, 27, 45., 45.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    opts['n_side_init'] = 3
    opts['n_substeps'] = 2
    f = gf(niq, p1)
    got = niq.queries.cast_rays_frustum((f, f), (p1, p2), cam, opts)
    o = R.generate_implicit(p1, 'affine_fixed')
    ref = R.cast_rays_frustum((o, o), (p1, p2), cam, opts, trace=True)
    bad = unexplained_pixels(got, ref, ref[4])
    assert len(bad) == 0, bad[:10]
    assert set(np.unique(got[1])) <= {0, 1, 2}


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, 'frustum.npz')), reason='no frustum fixture')
@pytest.mark.parametrize('name', ['one', 'two'])
def test_frustum_golden(niq, R, gpu_ready, name):
    g = golden('frustum.npz')
    c = g['frustum/cam']
    cam = (c[0:3], c[3:6], c[6:9], c[9:12], float(c[12]), float(c[13]), int(c[14]), int(c[15]))
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 32
    opts['n_side_init'] = 2
    opts['n_substeps'] = 1 if name == 'one' else 2
    p1 = model_from(g, 'model/relu32x3')
    ps = (p1,) if name == 'one' else (p1, model_from(g, 'model/relu16'))
    f = gf(niq, p1)
    got = niq.queries.cast_rays_frustum(tuple(f for _ in ps), ps, cam, opts)
    ref = (g[f'frustum/{name}/t'], g[f'frustum/{name}/hit_id'], g[f'frustum/{name}/count'])
    o = R.generate_implicit(p1, 'affine_fixed')
    near = R.cast_rays_frustum(tuple(o for _ in ps), ps, cam, opts, trace=True)[4]
    bad = unexplained_pixels(got, ref, near)
    assert len(bad) == 0, (name, bad[:10])


def test_frustum_conservative_covers_rays(niq, R, gpu_ready):
    """Conservative bounds: every pixel terminates, and hits sit where the ray cast of the
    same pixel's central ray finds the surface (within a few hit_eps steps)."""
    params = niq.workloads.plain_small_model()
    cam = camera(R, [0., 0., 3.], 32, 32, 60., 60.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 128
    opts['n_side_init'] = 4
    t, hid, cnt, nev = niq.queries.cast_rays_frustum((gf(niq, params, conservative=True),), (params,), cam, opts)
    assert nev > 0 and np.all(cnt >= 0) and np.all(np.isfinite(t))
    ref = R.cast_rays_frustum((R.generate_implicit(params, 'affine_fixed'),), (params,), cam, opts)
    both = (hid > 0) & (ref[1] > 0)
    assert both.sum() >= 0.9 * (ref[1] > 0).sum()
    assert np.all(np.abs(t[both] - ref[0][both]) <= 0.05 * np.maximum(ref[0][both], 1.))
