"""render.outward_normals / shade_image / render_image on the GPU against the oracle.

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
