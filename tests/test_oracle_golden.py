"""The oracle (oracle/ref_np.py) against golden vectors produced by running the
reference's own source (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from parity import ray_match, unexplained_rays
from conftest import golden, model_from

MODES = {'interval': {}, 'affine_fixed': {}, 'affine_all': {},
         'affine_truncate': {'affine_n_truncate': 8}, 'affine_append': {'affine_n_append': 4},
         'slope_interval': {}}


@pytest.fixture(scope='module')
def gb():
    return golden('bounds.npz')


@pytest.mark.parametrize('mname', ['relu16', 'elu16', 'relu32x3'])
def test_points(R, gb, mname):
    params = model_from(gb, f'model/{mname}')
    f = R.eval_points(params, gb[f'points/{mname}/x'])
    np.testing.assert_allclose(f, gb[f'points/{mname}/f'], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize('mname', ['relu16', 'elu16', 'relu32x3'])
@pytest.mark.parametrize('v', [3, 1, 2])
@pytest.mark.parametrize('mode', list(MODES))
def test_bounds(R, gb, mname, v, mode):
    params = model_from(gb, f'model/{mname}')
    f = R.generate_implicit(params, mode, **MODES[mode])
    c = gb[f'boxes/{mname}/v{v}/center']
    vv = gb[f'boxes/{mname}/v{v}/vecs']
    lo, hi = f.bounds_general(params, c, vv)
    glo, ghi = gb[f'boxes/{mname}/v{v}/{mode}/lower'], gb[f'boxes/{mname}/v{v}/{mode}/upper']
    scale = np.maximum(np.abs(glo), np.abs(ghi)) + 1e-3
    assert np.all(np.abs(lo - glo) <= 2e-5 * scale), np.max(np.abs(lo - glo) / scale)
    assert np.all(np.abs(hi - ghi) <= 2e-5 * scale), np.max(np.abs(hi - ghi) / scale)
    sign = R.sign_from_bounds(lo, hi, 0.01)
    gsign = gb[f'boxes/{mname}/v{v}/{mode}/sign_off0.01']
    # a sign may differ only where the bound sits within rounding of the threshold
    diff = sign != gsign
    near = (np.abs(glo - 0.01) < 1e-4 * scale) | (np.abs(ghi + 0.01) < 1e-4 * scale)
    assert np.all(~diff | near)


def test_fp64_oracle_contains_fp32_reference_values(R, gb):
    """Sanity: the FP64 bounds of every mode contain FP64 samples of the network."""
    params = model_from(gb, 'model/relu32x3')
    rng = np.random.default_rng(0)
    c = gb['boxes/relu32x3/v3/center'].astype(np.float64)
    vv = gb['boxes/relu32x3/v3/vecs'].astype(np.float64)
    for mode in MODES:
        f = R.generate_implicit(params, mode, dtype=np.float64, **MODES[mode])
        lo, hi = f.bounds_general(params, c, vv)
        eps = rng.uniform(-1, 1, (64, c.shape[0], vv.shape[1]))
        pts = c[None] + np.einsum('snv,nvd->snd', eps, vv)
        vals = R.eval_points(params, pts.reshape(-1, 3), np.float64).reshape(64, -1)
        assert np.all(vals >= lo[None] - 1e-9) and np.all(vals <= hi[None] + 1e-9), mode


@pytest.fixture(scope='module')
def gr():
    return golden('rays.npz')


@pytest.mark.parametrize('mode', ['affine_fixed', 'interval', 'slope_interval'])
def test_cast_rays(R, gr, mode):
    params = model_from(gr, 'model/relu32x3')
    f = R.generate_implicit(params, mode)
    opts = R.get_default_cast_opts()
    opts['n_max_step'] = 64
    t, hid, cnt, nev, near = R.cast_rays([f], [params], gr['rays/roots'], gr['rays/dirs'], opts, trace=True)
    gt, ghid, gcnt = gr[f'rays/{mode}/t'], gr[f'rays/{mode}/hit_id'], gr[f'rays/{mode}/count']
    # a ray may differ from the reference only after a decision within rounding of its
    # threshold (tests/parity.py)
    assert unexplained_rays(t, hid, cnt, gt, ghid, gcnt, near).size == 0
    assert int(nev) == int(gr[f'rays/{mode}/n_evals']) or not ray_match(t, hid, cnt, gt, ghid, gcnt).all()


def test_cast_rays_two_functions_substeps(R, gr):
    p1 = model_from(gr, 'model/relu32x3')
    p2 = model_from(gr, 'model/relu16')
    f = R.generate_implicit(p1, 'affine_fixed')
    opts = R.get_default_cast_opts()
    opts['n_max_step'] = 48
    opts['n_substeps'] = 2
    sub = slice(0, gr['rays/roots'].shape[0], 3)
    t, hid, cnt, nev, near = R.cast_rays([f, f], [p1, p2], gr['rays/roots'][sub], gr['rays/dirs'][sub], opts,
                                         trace=True)
    assert unexplained_rays(t, hid, cnt, gr['rays2/t'], gr['rays2/hit_id'], gr['rays2/count'], near).size == 0


def _sorted_boxes(lo, hi):
    a = np.concatenate([lo, hi], axis=1)
    return a[np.lexsort(a.T[::-1])]


@pytest.fixture(scope='module')
def gt_():
    return golden('tree.npz')


@pytest.mark.parametrize('mode', ['affine_fixed', 'interval'])
def test_levelset_tree(R, gt_, mode):
    params = model_from(gt_, 'model/relu32x3')
    f = R.generate_implicit(params, mode)
    d = R.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=9,
                                                  with_interior_nodes=True, with_exterior_nodes=True)
    for kind in ('unknown', 'interior', 'exterior'):
        lo, hi = d[f'{kind}_node_lower'], d[f'{kind}_node_upper']
        glo, ghi = gt_[f'tree/{mode}/{kind}/lower'], gt_[f'tree/{mode}/{kind}/upper']
        # same order as the reference, not just the same set
        np.testing.assert_array_equal(lo, glo)
        np.testing.assert_array_equal(hi, ghi)


def test_levelset_tree_thresh(R, gt_):
    params = model_from(gt_, 'model/relu32x3')
    f = R.generate_implicit(params, 'affine_fixed')
    d = R.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), node_terminate_thresh=200,
                                                  offset=0.05, batch_process_size=128)
    np.testing.assert_array_equal(d['unknown_node_lower'], gt_['tree_thresh/lower'])
    np.testing.assert_array_equal(d['unknown_node_upper'], gt_['tree_thresh/upper'])


@pytest.mark.parametrize('name', ['one', 'two'])
def test_cast_rays_frustum(R, name):
    """The frustum cast restated in oracle/ref_np.py against the reference's own
    cast_rays_frustum: t, hit id and count on every pixel."""
    g = golden('frustum.npz')
    c = g['frustum/cam']
    cam = (c[0:3], c[3:6], c[6:9], c[9:12], float(c[12]), float(c[13]), int(c[14]), int(c[15]))
    opts = R.get_default_cast_opts()
    opts['n_max_step'] = 32
    opts['n_side_init'] = 2
    opts['n_substeps'] = 1 if name == 'one' else 2
    p1 = model_from(g, 'model/relu32x3')
    ps = (p1,) if name == 'one' else (p1, model_from(g, 'model/relu16'))
    fs = tuple(R.generate_implicit(p, 'affine_fixed') for p in ps)
    t, hid, cnt, _, near = R.cast_rays_frustum(fs, ps, cam, opts, trace=True)
    m = (hid == g[f'frustum/{name}/hit_id']) & (cnt == g[f'frustum/{name}/count']) & \
        np.isclose(t, g[f'frustum/{name}/t'], rtol=1e-5, atol=1e-6)
    assert np.all(m | near), np.argwhere(~m & ~near)[:10]
    assert (g[f'frustum/{name}/hit_id'] > 0).sum() > 0


def test_c_restatement_matches_numpy_oracle(R):
    """oracle/cpu_tree.c (the CPU baseline) builds the same leaf set, in the same order,
    as the NumPy oracle."""
    from oracle import cpu_tree
    import importlib
    niq = importlib.import_module('neural-implicit-queries_gb300')
    params = niq.workloads.spheres_sdf_model()
    n, nb, leaves = cpu_tree.levelset_tree(niq.mlp.spec_layers(params), -np.ones(3), np.ones(3), 12,
                                           want_leaves=True)
    d = R.construct_uniform_unknown_levelset_tree(R.generate_implicit(params, 'affine_fixed'), params,
                                                  -np.ones(3), np.ones(3), split_depth=12)
    ref = np.concatenate([d['unknown_node_lower'], d['unknown_node_upper']], 1)
    assert n == ref.shape[0] and nb == d['n_boxes_classified']
    np.testing.assert_array_equal(leaves, ref)


SAMPLE_NAMES = ('fox', 'hammer', 'bunny', 'birdcage_occ')
SAMPLE_MODES = {'interval': {}, 'affine_fixed': {}, 'slope_interval': {},
                'affine_truncate': {'affine_n_truncate': 8}}


@pytest.fixture(scope='module')
def gs_():
    return golden('samples.npz'), golden('sample_models.npz')


@pytest.mark.parametrize('name', SAMPLE_NAMES)
def test_sample_models_oracle(R, gs_, name):
    """The oracle against the reference's outputs on its own sample models: point values,
    bounds in four modes, the 12-bisection level-set tree (same boxes in the same order)
    and a 12 x 12 ray cast."""
    g, m = gs_
    params = model_from(m, f'model/{name}')
    np.testing.assert_allclose(R.eval_points(params, g[f'{name}/points/x']), g[f'{name}/points/f'],
                               rtol=1e-5, atol=1e-6)
    c, vv = g[f'{name}/boxes/center'], g[f'{name}/boxes/vecs']
    for mode, kw in SAMPLE_MODES.items():
        f = R.generate_implicit(params, mode, **kw)
        lo, hi = f.bounds_general(params, c, vv)
        glo, ghi = g[f'{name}/boxes/{mode}/lower'], g[f'{name}/boxes/{mode}/upper']
        scale = np.maximum(np.abs(glo), np.abs(ghi)) + 1e-3
        assert np.max(np.abs(lo - glo) / scale) <= 1e-5 and np.max(np.abs(hi - ghi) / scale) <= 1e-5, mode
    f = R.generate_implicit(params, 'affine_fixed')
    d = R.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=12,
                                                  with_interior_nodes=True, with_exterior_nodes=True)
    for kind in ('unknown', 'interior', 'exterior'):
        np.testing.assert_array_equal(d[f'{kind}_node_lower'], g[f'{name}/tree/{kind}/lower'])
        np.testing.assert_array_equal(d[f'{kind}_node_upper'], g[f'{name}/tree/{kind}/upper'])
    opts = R.get_default_cast_opts()
    opts['n_max_step'] = 48
    t, hid, cnt, _, near = R.cast_rays([f], [params], g['rays/roots'], g['rays/dirs'], opts, trace=True)
    assert unexplained_rays(t, hid, cnt, g[f'{name}/rays/t'], g[f'{name}/rays/hit_id'], g[f'{name}/rays/count'],
                            near).size == 0


def test_c_marching_cubes_matches_numpy_oracle(R):
    """oracle/cpu_tree.c's marching cubes on the leaves (n_subcell_depth 0, the CPU
    baseline's second phase) gives the NumPy oracle's triangles, in the same order, to
    fp32 rounding of the point values."""
    from oracle import cpu_tree, mc_table
    import importlib
    niq = importlib.import_module('neural-implicit-queries_gb300')
    params = niq.workloads.spheres_sdf_model()
    layers = niq.mlp.spec_layers(params)
    _, _, leaves = cpu_tree.levelset_tree(layers, -np.ones(3), np.ones(3), 12, want_leaves=True)
    tris = cpu_tree.hmc_leaves(layers, leaves)
    o = R.generate_implicit(params, 'affine_fixed')
    ref = R.hierarchical_marching_cubes(o, params, -np.ones(3), np.ones(3), 4,
                                        (mc_table.make_table(), mc_table.EDGE, mc_table.VERT), n_subcell_depth=0)
    assert tris.shape == ref.shape and tris.shape[0] > 500
    np.testing.assert_allclose(tris, ref, atol=1e-5)
    assert cpu_tree.hmc_leaves(layers, leaves, want_tris=False) == tris.shape[0]


@pytest.mark.parametrize('name,mode,kw', [('truncate8', 'affine_truncate', {'affine_n_truncate': 8}),
                                          ('truncate64', 'affine_truncate', {'affine_n_truncate': 64}),
                                          ('append4', 'affine_append', {'affine_n_append': 4}),
                                          ('all', 'affine_all', {})])
def test_levelset_tree_growing_modes(R, name, mode, kw):
    """The oracle's tree in the growing-term modes against the reference's, box for box
    and in the same order."""
    g = golden('tree_growing.npz')
    params = model_from(g, 'model/relu32x3')
    f = R.generate_implicit(params, mode, **kw)
    d = R.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=8,
                                                  with_interior_nodes=True, with_exterior_nodes=True)
    for kind in ('unknown', 'interior', 'exterior'):
        np.testing.assert_array_equal(d[f'{kind}_node_lower'], g[f'tree/{name}/{kind}/lower'])
        np.testing.assert_array_equal(d[f'{kind}_node_upper'], g[f'tree/{name}/{kind}/upper'])


@pytest.mark.parametrize('name,K', [('truncate8', 8), ('truncate64', 64)])
def test_closest_point_truncate(R, name, K):
    """The oracle's closest point in affine_truncate against the reference's."""
    g = golden('tree_growing.npz')
    A = model_from(g, 'model/A')
    f = R.generate_implicit(A, 'affine_truncate', affine_n_truncate=K)
    for B in (8, 2048):
        d, _ = R.closest_point(f, A, -np.ones(3), np.ones(3), g['cp/q'], eps=0.05, batch_process_size=B)
        np.testing.assert_allclose(d, g[f'cp/{name}/B{B}/dist'], rtol=1e-5, atol=1e-6)
