"""The request loop: results in a concurrent mix equal the same requests run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_serve_mix_equals_alone(niq, gpu_ready):
    wl = niq.workloads
    models = [wl.he_mlp([3] + [w] * d + [1], act, seed=100 + i, grid=16)
              for i, (w, d, act) in enumerate([(32, 3, 'relu'), (64, 3, 'tanh'), (128, 2, 'relu'),
                                                (48, 4, 'tanh'), (256, 2, 'relu'), (96, 3, 'relu')])]
    srv = niq.serve.Server(models, budget_bytes=1 << 30, n_streams=3)
    rng = np.random.default_rng(0)
    reqs = []
    for i in range(12):
        reqs.append(niq.serve.ClosestRequest(int(rng.integers(6)),
                                             rng.uniform(-1.2, 1.2, (int(rng.integers(1, 300)), 3)).astype(np.float32),
                                             eps=1e-2))
    for i in range(5):
        eye = rng.standard_normal(3)
        eye = (3.0 * eye / np.linalg.norm(eye)).astype(np.float32)
        look, up, _ = niq.render.look_at(eye)
        roots, dirs = niq.render.generate_camera_rays(eye, look, up, res=24, fov_deg=60.)
        opts = niq.queries.get_default_cast_opts()
        opts['n_max_step'] = 48
        reqs.append(niq.serve.RayRequest(int(rng.integers(6)), roots, dirs, opts))
    for i in range(2):
        R = wl.random_rotation(rng)
        reqs.append(niq.serve.IntersectRequest(0, 1, R, rng.uniform(-0.3, 0.3, 3).astype(np.float32), eps=0.02))
    order = rng.permutation(len(reqs))
    futs = {int(k): srv.submit(reqs[k]) for k in order}
    got = {k: f.result(timeout=300) for k, f in futs.items()}
    srv.close()
    st = srv.stats()
    assert st['completed'] == len(reqs) and st['p99_ms'] >= st['p50_ms'] > 0
    f = srv.func
    for k, r in enumerate(reqs):
        if isinstance(r, niq.serve.ClosestRequest):
            d, l_ = niq.kd_tree.closest_point(f, models[r.model], srv.lower, srv.upper, r.points, eps=r.eps,
                                              persistent=True, node_budget=r.node_budget, strict=False)
            np.testing.assert_array_equal(got[k][0], d)
            np.testing.assert_array_equal(got[k][1], l_)
        elif isinstance(r, niq.serve.RayRequest):
            t, hid, cnt, _ = niq.queries.cast_rays((f,), (models[r.model],), r.roots, r.dirs, r.opts)
            np.testing.assert_array_equal(got[k][0], t)
            np.testing.assert_array_equal(got[k][1], hid)
            np.testing.assert_array_equal(got[k][2], cnt)
        else:
            pa = niq.mlp.prepend_op(models[r.model_a], niq.mlp.spatial_transformation())
            pa['0000.spatial_transformation.R'] = r.R
            pa['0000.spatial_transformation.t'] = r.t
            pb = niq.mlp.prepend_op(models[r.model_b], niq.mlp.spatial_transformation())
            alone = niq.kd_tree.find_any_intersection((f, f), (pa, pb), srv.lower, srv.upper, r.eps)
            assert got[k][0] == alone[0]
