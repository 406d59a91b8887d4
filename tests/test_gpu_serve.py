"""The request loops (the Python scheduler and the library's native runtime): results in a
concurrent mix equal the same requests run alone."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('native', [False, True])
def test_serve_mix_equals_alone(niq, gpu_ready, native):
    wl = niq.workloads
    models = [wl.he_mlp([3] + [w] * d + [1], act, seed=100 + i, grid=16)
              for i, (w, d, act) in enumerate([(32, 3, 'relu'), (64, 3, 'tanh'), (128, 2, 'relu'),
                                                (48, 4, 'tanh'), (256, 2, 'relu'), (96, 3, 'relu')])]
    if native:
        # small slices, so that every request is cut into several and the slices of
        # different requests interleave on the lanes
        srv = niq.serve.NativeServer(models, n_lanes=3, slice_rays=200, slice_queries=64,
                                     lane_scratch_bytes=256 << 20)
    else:
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



def test_native_server_c_abi(niq, gpu_ready):
    """niq_server_create / niq_batch_submit / niq_batch_poll / niq_batch_wait through ctypes:
    a ray tile cut into slices gives the results of one niq_cast_rays call; a request
    with a null output is refused at submit; an unknown ticket is an error."""
    import torch
    L = niq._lib
    lib = L.load()
    params = niq.workloads.plain_small_model()
    m = niq.mlp.device_model(params)
    f = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=True)[0]
    so = L.ServerOpts(2, 500, 64, 64 << 20)
    h = C.c_void_p()
    L.check(lib.niq_server_create(C.byref(so), C.byref(h)))
    try:
        roots, dirs = niq.render.generate_camera_rays([0., 0., 3.], [0., 0., -1.], [0., 1., 0.], res=40, fov_deg=60.)
        opts = niq.queries.get_default_cast_opts()
        opts['n_max_step'] = 64
        rt, dt = torch.from_numpy(roots).cuda(), torch.from_numpy(dirs).cuda()
        n = rt.shape[0]
        t = torch.empty(n, dtype=torch.float32, device='cuda')
        hit = torch.empty(n, dtype=torch.int32, device='cuda')
        cnt = torch.empty(n, dtype=torch.int32, device='cuda')
        r = L.Request()
        r.kind, r.model, r.opts, r.cast, r.n = L.NIQ_REQ_RAYS, m.handle.value, f.bound_opts(), L.cast_opts(opts), n
        r.in0, r.in1, r.out_f, r.out_i, r.out_i2 = rt.data_ptr(), dt.data_ptr(), t.data_ptr(), hit.data_ptr(), \
            cnt.data_ptr()
        torch.cuda.synchronize()
        tk = C.c_int64()
        L.check(lib.niq_batch_submit(h, C.byref(r), C.byref(tk)))
        status = C.c_int32(-1)
        L.check(lib.niq_batch_wait(h, tk.value, 60.0, C.byref(status)))
        assert status.value == 0
        ref = niq.queries.cast_rays((f,), (params,), roots, dirs, opts)
        np.testing.assert_array_equal(t.cpu().numpy(), ref[0])
        np.testing.assert_array_equal(hit.cpu().numpy(), ref[1])
        np.testing.assert_array_equal(cnt.cpu().numpy(), ref[2])
        done = C.c_int32()
        assert lib.niq_batch_poll(h, tk.value, C.byref(done), C.byref(status)) == L.NIQ_ERR_INVALID_ARG
        r.out_f = None
        assert lib.niq_batch_submit(h, C.byref(r), C.byref(tk)) == L.NIQ_ERR_INVALID_ARG
        comp, infl = C.c_int64(), C.c_int64()
        L.check(lib.niq_server_stats(h, C.byref(comp), C.byref(infl)))
        assert comp.value == 1 and infl.value == 0
    finally:
        L.check(lib.niq_server_destroy(h))
