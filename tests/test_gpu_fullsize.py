"""Size-independent properties at the benchmark's full sizes (too large for the oracle):
the 256^3 level-set tree of the 12-sphere model, its marching cubes, and the 1024^2 ray
cast."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _func(niq, params, conservative=True):
    return niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=conservative)[0]


def test_tree_24_bisections_partitions_the_root(niq, gpu_ready):
    """Unknown leaves, interior and exterior nodes tile the root box: their volumes add up
    to 8, leaves have the uniform size 2/256, and every interior/exterior node is aligned
    to the dyadic grid of its own size."""
    params = niq.workloads.spheres_sdf_model()
    f = _func(niq, params)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, lo, hi, split_depth=24,
                                                            with_interior_nodes=True, with_exterior_nodes=True)
    vol = 0.0
    for kind in ('unknown', 'interior', 'exterior'):
        a, b = d[f'{kind}_node_lower'].astype(np.float64), d[f'{kind}_node_upper'].astype(np.float64)
        assert np.all(b > a) and np.all(a >= -1) and np.all(b <= 1)
        w = b - a
        vol += np.prod(w, axis=1).sum()
        # dyadic alignment: lower corner is a multiple of the node's width along each axis
        k = (a + 1) / w
        assert np.allclose(k, np.round(k), atol=1e-6), kind
    assert vol == pytest.approx(8.0, rel=1e-12)
    leaf_w = d['unknown_node_upper'] - d['unknown_node_lower']
    assert np.allclose(leaf_w, 2.0 / 256, rtol=1e-6)
    assert 500000 < d['unknown_node_lower'].shape[0] < 1000000


def test_hmc_depth8_vertices_lie_in_leaves_and_surface(niq, R, gpu_ready):
    """Every triangle of the 256^3 extraction lies in one leaf box, and the network
    changes sign along the edge its vertices interpolate (checked on a sample)."""
    params = niq.workloads.spheres_sdf_model()
    f = _func(niq, params)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    tris = niq.kd_tree.hierarchical_marching_cubes(f, params, lo, hi, 8, n_subcell_depth=0)
    assert tris.shape[0] > 100000 and tris.shape[1:] == (3, 3)
    h = 2.0 / 256
    # the cell of a triangle from its centroid; interpolated vertices may round one ulp
    # past the cell's faces
    cell = np.floor((tris.mean(axis=1).astype(np.float64) + 1) / h)
    assert np.all(tris.min(axis=1) >= -1 + cell * h - 1e-5)
    assert np.all(tris.max(axis=1) <= -1 + (cell + 1) * h + 1e-5)
    rng = np.random.default_rng(0)
    s = tris[rng.integers(0, tris.shape[0], 2000)].reshape(-1, 3)
    assert np.max(np.abs(R.eval_points(params, s))) < 0.05   # vertices sit near the zero set


def test_rays_1024_persistent_equals_plain(niq, gpu_ready):
    params = niq.workloads.plain_small_model()
    f = _func(niq, params, conservative=False)
    look, up, _ = niq.render.look_at(np.array([0., 0., 3.], np.float32))
    roots, dirs = niq.render.generate_camera_rays(np.array([0., 0., 3.], np.float32), look, up, res=1024, fov_deg=60.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    a = niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
    b = niq.queries.cast_rays((f,), (params,), roots, dirs, opts, persistent=False)
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    assert (a[1] > 0).sum() > 500000


def test_tree_24_bisections_matches_c_oracle(niq, gpu_ready):
    """The level-set tree of the 12-sphere model to 24 bisections (256^3 leaves) in the
    reference's arithmetic (conservative=False) against the oracle's C restatement
    (oracle/cpu_tree.c) at the same size: identical leaf sets except boxes whose path
    from the root holds a decision within rounding of its threshold (tests/parity.py)."""
    from oracle import cpu_tree
    from parity import box_set_diff, unexplained_boxes
    params = niq.workloads.spheres_sdf_model()
    f = _func(niq, params, conservative=False)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, lo, hi, split_depth=24)
    n, nb, leaves = cpu_tree.levelset_tree(niq.mlp.spec_layers(params), lo, hi, 24, want_leaves=True)
    assert n == leaves.shape[0] > 500000
    extra, missing = box_set_diff(d['unknown_node_lower'], d['unknown_node_upper'], leaves[:, :3], leaves[:, 3:])
    print(f'24-bisection tree: {len(extra)} extra, {len(missing)} missing of {n} leaves')
    bad = unexplained_boxes(params, np.concatenate([extra, missing]), lo, hi)
    assert len(bad) == 0, bad[:5]
