"""CUDA queries (cast_rays, level-set tree, HMC, intersection, closest point) against the
oracle and the golden vectors of the reference.

Decision parity (tests/parity.py): results depend on sign decisions of bounds and point
values; every difference from the oracle or the reference must trace back to a
decision that sat within 1e-5 (relative) of its threshold in the oracle's own
computation.  No test passes on a fraction of matching results."""
import numpy as np
import pytest

from conftest import golden, model_from
from parity import box_set_diff, ray_match, unexplained_boxes, unexplained_queries, unexplained_rays

pytestmark = pytest.mark.gpu


def gf(niq, params, mode='affine_fixed', conservative=False, **kw):
    return niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=conservative, **kw)[0]


@pytest.mark.parametrize('mode', ['affine_fixed', 'interval', 'slope_interval'])
def test_cast_rays_golden(niq, R, gpu_ready, mode):
    g = golden('rays.npz')
    params = model_from(g, 'model/relu32x3')
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    f = gf(niq, params, mode)
    t, hid, cnt, nev = niq.queries.cast_rays((f,), (params,), g['rays/roots'], g['rays/dirs'], opts)
    *_, near = R.cast_rays([R.generate_implicit(params, mode)], [params], g['rays/roots'], g['rays/dirs'], opts,
                           trace=True)
    bad = unexplained_rays(t, hid, cnt, g[f'rays/{mode}/t'], g[f'rays/{mode}/hit_id'], g[f'rays/{mode}/count'],
                           near)
    assert bad.size == 0, bad


def test_cast_rays_two_functions_golden(niq, R, gpu_ready):
    g = golden('rays.npz')
    p1, p2 = model_from(g, 'model/relu32x3'), model_from(g, 'model/relu16')
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 48
    opts['n_substeps'] = 2
    sub = slice(0, g['rays/roots'].shape[0], 3)
    f = gf(niq, p1)
    roots, dirs = g['rays/roots'][sub], g['rays/dirs'][sub]
    t, hid, cnt, _ = niq.queries.cast_rays((f, f), (p1, p2), roots, dirs, opts)
    o = R.generate_implicit(p1, 'affine_fixed')
    *_, near = R.cast_rays([o, o], [p1, p2], roots, dirs, opts, trace=True)
    bad = unexplained_rays(t, hid, cnt, g['rays2/t'], g['rays2/hit_id'], g['rays2/count'], near)
    assert bad.size == 0, bad


@pytest.mark.parametrize('width', [32, 64, 128, 256])
def test_cast_rays_oracle_and_plain(niq, R, gpu_ready, width):
    params = niq.workloads.he_mlp([3, width, width, width, 1], 'relu', seed=width, grid=16)
    roots, dirs = R.generate_camera_rays([0., 0., 3.], [0., 0., -1.], [0., 1., 0.], res=24, fov_deg=60.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    f = gf(niq, params)
    t, hid, cnt, nev = niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
    tp, hidp, cntp, nevp = niq.queries.cast_rays((f,), (params,), roots, dirs, opts, persistent=False)
    # the persistent and plain forms run the same per-ray arithmetic
    np.testing.assert_array_equal(t, tp)
    np.testing.assert_array_equal(hid, hidp)
    np.testing.assert_array_equal(cnt, cntp)
    assert nev == nevp == int(cnt.sum())
    o = R.generate_implicit(params, 'affine_fixed')
    rt, rhid, rcnt, _, near = R.cast_rays([o], [params], roots, dirs, opts, trace=True)
    bad = unexplained_rays(t, hid, cnt, rt, rhid, rcnt, near)
    assert bad.size == 0, bad


def test_cast_rays_plain_method_full_size(niq, R, gpu_ready):
    """The plain-method workload at its full size: 128 x 128 rays on the 3->32x3->1 ReLU
    model, affine_fixed, 64 steps, from the reference's camera (eye at distance 3 on +z,
    60 degree field of view), against the oracle ray by ray; persistent and plain forms."""
    params = niq.workloads.plain_small_model()
    eye = np.array([0., 0., 3.], np.float32)
    look, up, _ = niq.render.look_at(eye)
    roots, dirs = niq.render.generate_camera_rays(eye, look, up, res=128, fov_deg=60.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    f = gf(niq, params)
    o = R.generate_implicit(params, 'affine_fixed')
    rt, rhid, rcnt, _, near = R.cast_rays([o], [params], roots, dirs, opts, trace=True)
    assert (rhid > 0).sum() > 1000
    for persistent in (True, False):
        t, hid, cnt, _ = niq.queries.cast_rays((f,), (params,), roots, dirs, opts, persistent=persistent)
        bad = unexplained_rays(t, hid, cnt, rt, rhid, rcnt, near)
        assert bad.size == 0, (persistent, bad[:20])


@pytest.mark.parametrize('mode', ['affine_fixed', 'interval', 'slope_interval'])
@pytest.mark.parametrize('conservative', [False, True])
def test_ray_tile_columns_agree(niq, gpu_ready, mode, conservative):
    """The narrow ray tile (4 columns per thread, 8 lanes per ray; the default for models
    at most 32 wide) and the 8-column tile give identical casts, persistent and plain."""
    at = niq.autotune
    old = at.get_params()
    try:
        for width in (16, 32):
            params = niq.workloads.he_mlp([3, width, width, width, 1], 'relu', seed=40 + width, grid=16)
            eye = np.array([0., 0., 3.], np.float32)
            look, up, _ = niq.render.look_at(eye)
            roots, dirs = niq.render.generate_camera_rays(eye, look, up, res=40, fov_deg=60.)
            opts = niq.queries.get_default_cast_opts()
            opts['n_max_step'] = 64
            f = gf(niq, params, mode, conservative=conservative)
            res = {}
            for cols in (8, 4):
                at.set_params(ray_columns=cols)
                for persistent in (True, False):
                    res[cols, persistent] = niq.queries.cast_rays((f,), (params,), roots, dirs, opts,
                                                                  persistent=persistent)[:3]
            ref = res[8, True]
            assert int(ref[2].sum()) > 0
            if mode != 'interval':   # interval bounds of this model are too loose to reach a hit
                assert (ref[1] > 0).sum() > 100
            for key, r in res.items():
                for a, b in zip(r, ref):
                    np.testing.assert_array_equal(a, b, err_msg=str((width, key)))
    finally:
        at.set_params(**old)


@pytest.mark.parametrize('mode,kw', [('affine_all', {}), ('affine_truncate', {'affine_n_truncate': 8}),
                                     ('affine_append', {'affine_n_append': 4})])
def test_cast_rays_growing_modes(niq, R, gpu_ready, mode, kw):
    params = niq.workloads.he_mlp([3, 16, 16, 1], 'relu', seed=3, grid=16)
    roots, dirs = R.generate_camera_rays([0., 0., 3.], [0., 0., -1.], [0., 1., 0.], res=14, fov_deg=60.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 48
    f = gf(niq, params, mode, **kw)
    t, hid, cnt, nev = niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
    tp, hidp, cntp, _ = niq.queries.cast_rays((f,), (params,), roots, dirs, opts, persistent=False)
    np.testing.assert_array_equal(t, tp)
    o = R.generate_implicit(params, mode, **kw)
    rt, rhid, rcnt, _, near = R.cast_rays([o], [params], roots, dirs, opts, trace=True)
    bad = unexplained_rays(t, hid, cnt, rt, rhid, rcnt, near)
    assert bad.size == 0, bad


def test_cast_rays_conservative_hits(niq, R, gpu_ready):
    params = niq.workloads.plain_small_model()
    roots, dirs = R.generate_camera_rays([0., 0., 3.], [0., 0., -1.], [0., 1., 0.], res=32, fov_deg=60.)
    opts = niq.queries.get_default_cast_opts()
    opts['n_max_step'] = 64
    f = gf(niq, params, conservative=True)
    t, hid, cnt, _ = niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
    # every reported hit brackets a sign change of the FP64 network within hit_eps
    hit = hid > 0
    p0 = roots[hit].astype(np.float64) + t[hit, None].astype(np.float64) * dirs[hit]
    p1 = p0 + 1e-3 * dirs[hit]
    v0, v1 = R.eval_points(params, p0, np.float64), R.eval_points(params, p1, np.float64)
    assert np.mean(np.sign(v0) != np.sign(v1)) > 0.98


def tree_diff_unexplained(params, d, ref, mode, root=(-1., 1.), offset=0., kinds=('unknown', 'interior', 'exterior'),
                          ref_fmt='{kind}_node_{side}'):
    """Boxes in one tree's node sets and not the other's that no near-threshold decision
    on their path from the root explains (tests/parity.py)."""
    lo, hi = np.full(3, root[0], np.float32), np.full(3, root[1], np.float32)
    out = {}
    for kind in kinds:
        extra, missing = box_set_diff(d[f'{kind}_node_lower'], d[f'{kind}_node_upper'],
                                      ref[ref_fmt.format(kind=kind, side='lower')],
                                      ref[ref_fmt.format(kind=kind, side='upper')])
        print(f'{kind}: {len(extra)} extra, {len(missing)} missing of {len(d[f"{kind}_node_lower"])}')
        out[kind] = unexplained_boxes(params, np.concatenate([extra, missing]), lo, hi, mode, offset)
    return out


@pytest.mark.parametrize('mode', ['affine_fixed', 'interval'])
def test_tree_golden(niq, R, gpu_ready, mode):
    g = golden('tree.npz')
    params = model_from(g, 'model/relu32x3')
    f = gf(niq, params, mode)
    for persistent in (True, False):
        d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=9,
                                                                with_interior_nodes=True, with_exterior_nodes=True,
                                                                persistent=persistent)
        bad = tree_diff_unexplained(params, d, g, mode, ref_fmt='tree/' + mode + '/{kind}/{side}')
        assert all(len(v) == 0 for v in bad.values()), bad


def test_tree_thresh_golden(niq, gpu_ready):
    g = golden('tree.npz')
    params = model_from(g, 'model/relu32x3')
    f = gf(niq, params)
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3),
                                                            node_terminate_thresh=200, offset=0.05)
    extra, missing = box_set_diff(d['unknown_node_lower'], d['unknown_node_upper'], g['tree_thresh/lower'],
                                  g['tree_thresh/upper'])
    assert len(extra) == 0 and len(missing) == 0


@pytest.mark.parametrize('conservative', [False, True])
def test_tree_oracle_spheres(niq, R, gpu_ready, conservative):
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params, conservative=conservative)
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=12)
    o = R.generate_implicit(params, 'affine_fixed')
    r = R.construct_uniform_unknown_levelset_tree(o, params, -np.ones(3), np.ones(3), split_depth=12)
    extra, missing = box_set_diff(d['unknown_node_lower'], d['unknown_node_upper'], r['unknown_node_lower'],
                                  r['unknown_node_upper'])
    # conservative bounds are never narrower: they can only keep more boxes unknown
    if conservative:
        assert len(missing) == 0
        assert len(extra) <= 0.001 * len(r['unknown_node_lower']) + 2
    else:
        bad = unexplained_boxes(params, np.concatenate([extra, missing]), -np.ones(3), np.ones(3))
        assert len(bad) == 0, bad


@pytest.mark.parametrize('conservative', [False, True])
def test_tree_oracle_spheres_slope(niq, R, gpu_ready, conservative):
    """slope_interval trees of the 12-sphere model against the oracle's: the node sets
    agree except boxes that a near decision on their path explains; outward rounding may
    keep more boxes unknown, and drops one only where such a decision explains it."""
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params, 'slope_interval', conservative=conservative)
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=12)
    o = R.generate_implicit(params, 'slope_interval')
    r = R.construct_uniform_unknown_levelset_tree(o, params, -np.ones(3), np.ones(3), split_depth=12)
    n_ref = len(r['unknown_node_lower'])
    assert n_ref > 100
    extra, missing = box_set_diff(d['unknown_node_lower'], d['unknown_node_upper'], r['unknown_node_lower'],
                                  r['unknown_node_upper'])
    if conservative:
        assert len(extra) <= 0.01 * n_ref + 2, (len(extra), n_ref)
        bad = unexplained_boxes(params, missing, -np.ones(3), np.ones(3), mode='slope_interval')
    else:
        bad = unexplained_boxes(params, np.concatenate([extra, missing]), -np.ones(3), np.ones(3),
                                mode='slope_interval')
    assert len(bad) == 0, bad


def test_hmc_oracle_and_golden(niq, R, gpu_ready):
    from oracle import mc_table
    g = golden('tree.npz')
    params = model_from(g, 'model/relu32x3')
    f = gf(niq, params)
    o = R.generate_implicit(params, 'affine_fixed')
    T = mc_table.make_table()
    mc = (T, mc_table.EDGE, mc_table.VERT)
    for depth, k in ((4, 1), (3, 0), (5, 2)):
        tris = niq.kd_tree.hierarchical_marching_cubes(f, params, -np.ones(3), np.ones(3), depth, n_subcell_depth=k)
        rt = R.hierarchical_marching_cubes(o, params, -np.ones(3), np.ones(3), depth, mc, n_subcell_depth=k)
        assert tris.shape == rt.shape
        a = np.sort(np.round(tris.reshape(-1, 9), 4), axis=0)
        b = np.sort(np.round(rt.reshape(-1, 9), 4), axis=0)
        assert np.max(np.abs(a - b)) < 1e-3
        key = f'hmc/d{depth}s{k}/tris'
        if key in g:
            ref = g[key]
            assert ref.shape == tris.shape
            # same crossing vertices and the same total vector area (triangulation-invariant)
            va = np.unique(np.round(tris.reshape(-1, 3), 4), axis=0)
            vb = np.unique(np.round(ref.reshape(-1, 3), 4), axis=0)
            assert va.shape == vb.shape and np.max(np.abs(va - vb)) < 1e-3
            area = lambda x: 0.5 * np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]).sum(0)
            np.testing.assert_allclose(area(tris), area(ref), atol=1e-4)


@pytest.mark.parametrize('mode', ['affine_all', 'affine_fixed'])
def test_intersection_golden(niq, gpu_ready, mode):
    g = golden('queries.npz')
    A = model_from(g, 'model/A')
    for name in ('near', 'far'):
        Bp = model_from(g, f'model/B_{name}')
        fa, fb = gf(niq, A, mode), gf(niq, Bp, mode)
        found, ia, ib, loc = niq.kd_tree.find_any_intersection((fa, fb), (A, Bp), -np.ones(3), np.ones(3), 0.02)
        assert found == bool(g[f'isect/{name}/{mode}/found']), name
        if found:
            va = niq.implicit_mlp_utils.generate_implicit_from_params(A, 'affine_fixed')[0](A, loc)
            vb = niq.implicit_mlp_utils.generate_implicit_from_params(Bp, 'affine_fixed')[0](Bp, loc)
            assert va < 0.05 and vb < 0.05


def test_intersection_persistent_vs_plain(niq, gpu_ready):
    g = golden('queries.npz')
    A = model_from(g, 'model/A')
    for name in ('near', 'far'):
        Bp = model_from(g, f'model/B_{name}')
        r1 = niq.kd_tree.find_any_intersection((gf(niq, A), gf(niq, Bp)), (A, Bp), -np.ones(3), np.ones(3), 0.02)
        # affine_truncate runs the plain host loop of the growing-term engine
        ft = dict(affine_n_truncate=64, affine_truncate_policy='absolute')
        r2 = niq.kd_tree.find_any_intersection((gf(niq, A, 'affine_truncate', **ft), gf(niq, Bp, 'affine_truncate', **ft)),
                                               (A, Bp), -np.ones(3), np.ones(3), 0.02)
        assert r1[0] == r2[0]


def test_closest_point_golden(niq, R, gpu_ready):
    g = golden('queries.npz')
    A = model_from(g, 'model/A')
    f = gf(niq, A)
    q = g['cp/q']
    o = R.generate_implicit(A, 'affine_fixed')
    for B in (8, 2048):
        dist, loc = niq.kd_tree.closest_point(f, A, -np.ones(3), np.ones(3), q, eps=0.05, batch_process_size=B)
        rd, rl = g[f'cp/B{B}/dist'], g[f'cp/B{B}/loc']
        od, ol, tr = R.closest_point(o, A, -np.ones(3), np.ones(3), q, eps=0.05, batch_process_size=B, trace=True)
        for ref in (rd, od):
            bad = unexplained_queries(dist, ref, tr)
            assert bad.size == 0, (B, bad)
        # queries whose distance agrees also agree on the location (the node center)
        same = np.isclose(dist, rd, rtol=1e-4, atol=1e-5) & np.isfinite(rd)
        assert np.allclose(loc[same], rl[same], atol=1e-5) or (~same).all()


def test_closest_point_queries_alone(niq, R, gpu_ready):
    """Each golden query run alone (its own stack, no coupling through shared batches)
    matches the oracle unless its own path holds a near-threshold decision."""
    g = golden('queries.npz')
    A = model_from(g, 'model/A')
    f = gf(niq, A)
    o = R.generate_implicit(A, 'affine_fixed')
    for i, qi in enumerate(g['cp/q']):
        q1 = qi[None].astype(np.float32)
        dist, _ = niq.kd_tree.closest_point(f, A, -np.ones(3), np.ones(3), q1, eps=0.05, batch_process_size=8)
        od, _, tr = R.closest_point(o, A, -np.ones(3), np.ones(3), q1, eps=0.05, batch_process_size=8, trace=True)
        assert unexplained_queries(dist, od, tr).size == 0, i


def test_closest_point_persistent_and_batched(niq, R, gpu_ready):
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params, conservative=True)
    rng = np.random.default_rng(3)
    q = rng.uniform(-1.2, 1.2, (300, 3)).astype(np.float32)
    eps = 1e-3
    d_ref, l_ref = niq.kd_tree.closest_point(f, params, -np.ones(3), np.ones(3), q, eps=eps)
    d_p, l_p = niq.kd_tree.closest_point(f, params, -np.ones(3), np.ones(3), q, eps=eps, persistent=True)
    fin = np.isfinite(d_ref)
    assert np.array_equal(fin, np.isfinite(d_p))
    # the persistent traversal prunes with a true lower bound less eps, so it visits every
    # node that could hold a candidate better by more than eps: never worse than the
    # reference schedule by more than eps
    assert np.all(d_p[fin] <= d_ref[fin] + eps + 1e-5)
    # every reported distance is cd + diag of a node whose samples change sign, so the
    # FP64 network changes sign within diag of the reported location
    o = R.generate_implicit(params, 'affine_fixed', dtype=np.float64)
    g = np.linspace(-1, 1, 11)
    grid = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    for i in np.nonzero(fin)[0][:40]:
        c = l_p[i].astype(np.float64)
        diag = float(d_p[i]) - np.linalg.norm(q[i] - c)
        assert diag >= -1e-5
        v = o(params, c + max(diag, 1e-6) * grid)
        assert v.min() <= 0 <= v.max(), i
    # the batched form over a model table returns the persistent form's results
    other = niq.workloads.he_mlp([3, 48, 48, 1], 'tanh', seed=9, grid=16)
    out = niq.batched.closest_point_many(f, [params, other], [0, 1, 0], [q[:100], q[100:200], q[200:]],
                                         -np.ones(3), np.ones(3), eps)
    np.testing.assert_array_equal(out[0][0], d_p[:100])
    np.testing.assert_array_equal(out[2][0], d_p[200:])
    d_o, _ = niq.kd_tree.closest_point(f, other, -np.ones(3), np.ones(3), q[100:200], eps=eps, persistent=True)
    np.testing.assert_array_equal(out[1][0], d_o)


def test_batched_results_independent_of_tuning(niq, gpu_ready):
    """The autotuner's parameters change the work split, never a query's result."""
    models = [niq.workloads.he_mlp([3, w, w, 1], 'relu', seed=30 + i, grid=16) for i, w in enumerate((32, 64, 96))]
    table = niq.batched.ModelTable(models)
    f = gf(niq, models[0], conservative=True)
    rng = np.random.default_rng(9)
    counts = np.array([70, 300, 45], np.int64)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    q = rng.uniform(-1.2, 1.2, (int(counts.sum()), 3)).astype(np.float32)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    jm = np.arange(3, dtype=np.int32)
    at = niq.autotune
    old = at.get_params()
    try:
        ref = None
        for ch, ct in ((128, 0), (32, 1), (512, 0)):
            at.set_params(batched_chunk=ch, batched_ctas_per_sm=ct)
            import torch
            st = torch.zeros(1, dtype=torch.int32, device='cuda')
            d, l_ = niq.batched.closest_point_packed(f, table, jm, offs, counts, q, lo, hi, 1e-2, status=st,
                                                     node_budget=4096)
            d = d.cpu().numpy()
            if ref is None:
                ref = d
            np.testing.assert_array_equal(d, ref)
        choice, timings = at.tune_batched(f, table, jm, offs, counts, q, lo, hi, 1e-2, node_budget=4096,
                                          chunks=(32, 128), ctas=(0,), reps=1, use_cache=False)
        assert choice['batched_chunk'] in (32, 128) and len(timings) == 2
    finally:
        at.set_params(**old)


def test_batched_jobs_over_a_subset_of_a_large_table(niq, gpu_ready):
    """Jobs that use a few models of a large table (as the autotuner's sample does) fit the
    workspace sized by the job count, and return the same distances as the table of just
    those models."""
    models = [niq.workloads.he_mlp([3, 32, 32, 1], 'relu', seed=60 + i, grid=8) for i in range(40)]
    table = niq.batched.ModelTable(models)
    f = gf(niq, models[0], conservative=True)
    rng = np.random.default_rng(12)
    qs = [rng.uniform(-1.2, 1.2, (n, 3)).astype(np.float32) for n in (50, 80, 30)]
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    big = niq.batched.closest_point_many(f, table, [37, 5, 37], qs, lo, hi, 1e-2)
    small = niq.batched.closest_point_many(f, [models[37], models[5]], [0, 1, 0], qs, lo, hi, 1e-2)
    for (d_big, _), (d_small, _) in zip(big, small):
        np.testing.assert_array_equal(d_big, d_small)


def test_batched_counts_queries_past_their_budget(niq, gpu_ready):
    """niq_batched_closest_point_stats: the queries stopped at a node budget of one node are
    counted, none with the default budget; each query bounds at least its root node, and no
    more than one node under a budget of one."""
    import torch
    models = [niq.workloads.he_mlp([3, 32, 32, 1], 'relu', seed=70 + i, grid=8) for i in range(3)]
    table = niq.batched.ModelTable(models)
    f = gf(niq, models[0], conservative=True)
    rng = np.random.default_rng(13)
    counts = np.array([40, 25, 60], np.int64)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    q = rng.uniform(-1.2, 1.2, (int(counts.sum()), 3)).astype(np.float32)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    jm = np.arange(3, dtype=np.int32)
    st = torch.zeros(1, dtype=torch.int32, device='cuda')
    niq.batched.closest_point_packed(f, table, jm, offs, counts, q, lo, hi, 1e-2, status=st, node_budget=1)
    torch.cuda.synchronize()
    assert int(st.item()) == niq._lib.NIQ_ERR_TIMEOUT
    spent, nodes = niq.batched.stats()
    nq = int(counts.sum())
    assert 0 < spent <= nq and nodes == nq
    niq.batched.closest_point_packed(f, table, jm, offs, counts, q, lo, hi, 1e-2, status=st)
    torch.cuda.synchronize()
    spent, nodes = niq.batched.stats()
    assert int(st.item()) == 0 and spent == 0 and nodes > nq


@pytest.mark.parametrize('B', [2048, 100])
def test_tree_schedules_agree(niq, gpu_ready, B):
    """The persistent tree, one launch per level, and the reference's schedule (launches
    of batch_process_size nodes) produce the same node sets."""
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params, conservative=True)
    sets = []
    for persistent in (True, False, 'batches'):
        d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=15,
                                                                with_interior_nodes=True, batch_process_size=B,
                                                                persistent=persistent)
        sets.append({k: {tuple(r) for r in np.concatenate([d[f'{k}_node_lower'], d[f'{k}_node_upper']], 1).tolist()}
                     for k in ('unknown', 'interior')})
        assert d['n_boxes_classified'] > 0
    assert sets[0] == sets[1] == sets[2]


def test_hmc_shared_corners_same_triangles(niq, gpu_ready):
    """Evaluating each lattice corner once gives exactly the triangles of the per-leaf
    evaluation (same values at shared corners, same arithmetic), in another order."""
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params, conservative=True)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    for root in ((lo, hi), (np.array([-1.2, -0.9, -1.1], np.float32), np.array([1.1, 1.0, 0.95], np.float32))):
        a = niq.kd_tree.hierarchical_marching_cubes(f, params, root[0], root[1], 6, n_subcell_depth=0,
                                                    shared_corners=True)
        b = niq.kd_tree.hierarchical_marching_cubes(f, params, root[0], root[1], 6, n_subcell_depth=0,
                                                    shared_corners=False)
        assert a.shape == b.shape and a.shape[0] > 1000
        key = lambda t: t.reshape(t.shape[0], 9)[np.lexsort(t.reshape(t.shape[0], 9).T[::-1])]
        np.testing.assert_array_equal(key(a), key(b))
