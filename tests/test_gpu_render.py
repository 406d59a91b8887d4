"""render.outward_normals / shade_image / render_image on the GPU against the oracle.

Gradients (niq_eval_gradients, outward_normal(method='autodiff')): the forward-mode
derivatives against the oracle's in float32 within 1e-5 relative to the gradient's
size (the same products in another summation order), and against float64 within 1e-4.
Normals: unit vectors within 2e-3 (the finite-difference quotient divides sample
differences of about 1e-3 by eps, so last-ulp differences of the samples show at the
1e-4 level).  Shading: within 1e-4 per channel for 'normal'; 'matcap_color' within 2e-3
(a normal differing in the last bits moves the bilinear lookup)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(niq, R, res=48):
    params = niq.workloads.plain_small_model()
    f = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=False)[0]
    eye = np.array([0.2, 0.3, 2.9], np.float32)
    look, up, left = R.look_at(eye)
    roots, dirs = R.generate_camera_rays(eye, look, up, res=res, fov_deg=60.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 96
    t, hid, cnt, _ = niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
    pos = (roots + t[:, None] * dirs).astype(np.float32)
    return params, f, eye, look, up, left, roots, dirs, pos, hid, opts


def test_normals_match_oracle(niq, R, gpu_ready):
    params, f, eye, look, up, left, roots, dirs, pos, hid, opts = _scene(niq, R)
    assert (hid > 0).sum() > 100
    got = niq.render.outward_normals((f,), (params,), pos, hid, 1e-3)
    ref = R.outward_normals((R.generate_implicit(params, 'affine_fixed'),), (params,), pos, hid, 1e-3)
    h = hid > 0
    assert np.all(got[~h] == 0)
    np.testing.assert_allclose(np.linalg.norm(got[h], axis=1), 1., atol=1e-5)
    assert np.max(np.abs(got[h] - ref[h])) <= 2e-3


@pytest.mark.parametrize('act', ['relu', 'elu', 'tanh'])
def test_gradients_match_oracle(niq, R, gpu_ready, act):
    """Value and gradient at points through the C ABI against the oracle's forward-mode
    derivatives (jax.jacfwd of the point function, src/render.py:61-63), widths 32-256."""
    import importlib
    import torch
    lib = importlib.import_module('neural-implicit-queries_gb300._lib')
    L = lib.load()
    rng = np.random.default_rng(21)
    for i, sizes in enumerate([[3, 32, 32, 1], [3, 64, 64, 64, 1], [3, 256, 128, 1]]):
        params = niq.workloads.he_mlp(sizes, act, seed=40 + i, grid=8)
        x = rng.uniform(-1, 1, (1000, 3)).astype(np.float32)
        m = niq.mlp.device_model(params)
        xt = torch.from_numpy(x).cuda()
        val = torch.empty(1000, dtype=torch.float32, device='cuda')
        grad = torch.empty((1000, 3), dtype=torch.float32, device='cuda')
        lib.check(L.niq_eval_gradients(m.handle, 1000, xt.data_ptr(), val.data_ptr(), grad.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream))
        v32, g32 = R.eval_gradients(params, x, np.float32)
        v64, g64 = R.eval_gradients(params, x.astype(np.float64), np.float64)
        gv, gg = val.cpu().numpy(), grad.cpu().numpy()
        scale = np.linalg.norm(g64, axis=1, keepdims=True) + 1e-6
        np.testing.assert_allclose(gv, v32, rtol=1e-5, atol=1e-5 * (np.abs(v32).max() + 1e-3))
        assert np.max(np.abs(gg - g32) / scale) <= 1e-5, (sizes, act)
        assert np.max(np.abs(gg - g64) / scale) <= 1e-4, (sizes, act)
        # the value matches the point evaluation
        np.testing.assert_allclose(gv, niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed')[0](
            params, x), rtol=1e-5, atol=1e-6)


def test_autodiff_normals_match_oracle(niq, R, gpu_ready):
    params, f, eye, look, up, left, roots, dirs, pos, hid, opts = _scene(niq, R)
    assert (hid > 0).sum() > 100
    got = niq.render.outward_normals((f,), (params,), pos, hid, 1e-3, method='autodiff')
    ref = R.outward_normals((R.generate_implicit(params, 'affine_fixed'),), (params,), pos, hid, 1e-3,
                            method='autodiff')
    h = hid > 0
    assert np.all(got[~h] == 0)
    np.testing.assert_allclose(np.linalg.norm(got[h], axis=1), 1., atol=1e-5)
    assert np.max(np.abs(got[h] - ref[h])) <= 1e-5
    # close to the finite-difference normals away from ReLU kinks
    fd = niq.render.outward_normals((f,), (params,), pos, hid, 1e-3)
    assert np.median(np.abs(got[h] - fd[h]).max(axis=1)) <= 1e-2


@pytest.mark.parametrize('shading', ['normal', 'matcap_color'])
def test_shading_matches_oracle(niq, R, gpu_ready, shading):
    params, f, eye, look, up, left, roots, dirs, pos, hid, opts = _scene(niq, R)
    nrm = R.outward_normals((R.generate_implicit(params, 'affine_fixed'),), (params,), pos, hid, 1e-3)
    rng = np.random.default_rng(4)
    matcaps = tuple(rng.uniform(0, 1, (32, 40, 3)).astype(np.float32) for _ in range(4))
    colors = ((0.157, 0.613, 1.000),)
    got = niq.render.shade_image(shading, dirs, pos, nrm, hid, up, matcaps, colors)
    ref = R.shade_image(shading, dirs, nrm, hid, up, matcaps, colors)
    tol = 1e-4 if shading == 'normal' else 2e-3
    assert np.max(np.abs(got - ref)) <= tol
    assert np.all(got[hid == 0] == 1.)


def test_shading_color_func_matches_oracle(niq, R, gpu_ready):
    """shading_color_func (src/render.py:198-206): a color per hit position, here a
    function that only takes one position at a time and one that takes the array."""
    params, f, eye, look, up, left, roots, dirs, pos, hid, opts = _scene(niq, R)
    nrm = R.outward_normals((R.generate_implicit(params, 'affine_fixed'),), (params,), pos, hid, 1e-3)
    rng = np.random.default_rng(6)
    matcaps = tuple(rng.uniform(0, 1, (32, 40, 3)).astype(np.float32) for _ in range(4))

    def one(p):
        assert np.shape(p) == (3,)
        return np.clip(np.abs(np.asarray(p, np.float32)), 0, 1)

    def many(p):
        return np.clip(np.abs(np.asarray(p, np.float32)), 0, 1)
    ref = R.shade_image('matcap_color', dirs, nrm, hid, up, matcaps, None, hit_pos=pos, shading_color_func=one)
    for fn in (one, many):
        got = niq.render.shade_image('matcap_color', dirs, pos, nrm, hid, up, matcaps, ((0.2, 0.2, 0.2),),
                                     shading_color_func=fn)
        assert np.max(np.abs(got - ref)) <= 2e-3
        assert np.all(got[hid == 0] == 1.)


@pytest.mark.parametrize('frustum', [False, True])
def test_render_image(niq, R, gpu_ready, frustum):
    params = niq.workloads.plain_small_model()
    f = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=True)[0]
    eye = np.array([0., 0., 3.], np.float32)
    look, up, left = R.look_at(eye)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 96
    opts['n_side_init'] = 4
    rng = np.random.default_rng(5)
    matcaps = tuple(rng.uniform(0, 1, (16, 16, 3)).astype(np.float32) for _ in range(4))
    img, depth, counts, hits, n_eval, _ = niq.render.render_image(f, params, eye, look, up, left, 40, 60., frustum,
                                                                  opts, shading='matcap_color', matcaps=matcaps)
    assert img.shape == (40, 40, 3) and depth.shape == (40, 40) and hits.shape == (40, 40)
    assert n_eval > 0 and (hits > 0).sum() > 50
    assert np.all(img[hits == 0] == 1.) and np.all(np.isfinite(img))
