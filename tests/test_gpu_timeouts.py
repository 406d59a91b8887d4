"""The bounded device-side waits give up with NIQ_ERR_TIMEOUT, and the library recovers.

Every spin of a kernel here has a poll limit (niq_tune_set NIQ_TUNE_BARRIER_POLLS /
NIQ_TUNE_MBAR_POLLS, 1 + the polls allowed).  These tests set a limit of zero polls --
the wait gives up at once, deterministically, without any fault or hang -- check the
error code, restore the built-in limit and check that the next call gives the result a
clean run gives.  A closest-point query past its node budget is the host-visible form
of the same rule (src/kd_tree.py:659-802 has no budget; NIQ_ERR_TIMEOUT with strict)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gf(niq, params, mode='affine_fixed', products='auto', **kw):
    return niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=True, products=products,
                                                                **kw)[0]


def tree_sets(niq, f, params, depth=12):
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=depth,
                                                            with_interior_nodes=True)
    return {k: {tuple(r) for r in np.concatenate([d[f'{k}_node_lower'], d[f'{k}_node_upper']], 1).tolist()}
            for k in ('unknown', 'interior')}


@pytest.fixture
def tune(niq):
    at = niq.autotune
    old = at.get_params()
    yield at
    at.set_params(**old)


@pytest.mark.parametrize('products', ['fp32', '3xtf32'])
def test_grid_barrier_gives_up_and_recovers(niq, gpu_ready, tune, products):
    """The persistent tree's level barrier (FP32 tile engine and tensor-core form)."""
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params, products=products)
    ref = tree_sets(niq, f, params)
    tune.set_params(barrier_polls=1)
    with pytest.raises(niq._lib.NIQError) as e:
        tree_sets(niq, f, params)
    assert e.value.code == niq._lib.NIQ_ERR_TIMEOUT
    tune.set_params(barrier_polls=0)
    assert tree_sets(niq, f, params) == ref


def test_tensor_core_tree_mbarrier_gives_up_and_recovers(niq, gpu_ready, tune):
    """The tensor-core tree's wait on its MMAs: the kernel gives up, still waits for the
    MMAs in flight with the built-in limit, releases tensor memory and returns."""
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params, products='3xtf32')
    ref = tree_sets(niq, f, params)
    tune.set_params(mbar_polls=1)
    with pytest.raises(niq._lib.NIQError) as e:
        tree_sets(niq, f, params)
    assert e.value.code == niq._lib.NIQ_ERR_TIMEOUT
    tune.set_params(mbar_polls=0)
    assert tree_sets(niq, f, params) == ref


def test_growing_term_engine_mbarrier_gives_up_and_recovers(niq, gpu_ready, tune):
    """The 3xTF32 growing-term engine (affine_truncate on a 128-wide model)."""
    params = niq.workloads.he_mlp([3, 128, 128, 128, 1], 'relu', seed=21, grid=8)
    f = gf(niq, params, 'affine_truncate', products='3xtf32', affine_n_truncate=64)
    rng = np.random.default_rng(2)
    c = rng.uniform(-0.8, 0.8, (64, 3)).astype(np.float32)
    vv = np.tile((0.05 * np.eye(3, dtype=np.float32))[None], (64, 1, 1))
    ref = f.bounds_general_box(params, c, vv)
    tune.set_params(mbar_polls=1)
    with pytest.raises(niq._lib.NIQError) as e:
        f.bounds_general_box(params, c, vv)
    assert e.value.code == niq._lib.NIQ_ERR_TIMEOUT
    tune.set_params(mbar_polls=0)
    got = f.bounds_general_box(params, c, vv)
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)


def test_intersection_barrier_gives_up_and_recovers(niq, gpu_ready, tune):
    from conftest import golden, model_from
    g = golden('queries.npz')
    A, Bp = model_from(g, 'model/A'), model_from(g, 'model/B_near')
    fa, fb = gf(niq, A), gf(niq, Bp)
    ref = niq.kd_tree.find_any_intersection((fa, fb), (A, Bp), -np.ones(3), np.ones(3), 0.02)
    tune.set_params(barrier_polls=1)
    with pytest.raises(niq._lib.NIQError) as e:
        niq.kd_tree.find_any_intersection((fa, fb), (A, Bp), -np.ones(3), np.ones(3), 0.02)
    assert e.value.code == niq._lib.NIQ_ERR_TIMEOUT
    tune.set_params(barrier_polls=0)
    got = niq.kd_tree.find_any_intersection((fa, fb), (A, Bp), -np.ones(3), np.ones(3), 0.02)
    assert got[0] == ref[0]
    np.testing.assert_array_equal(got[3], ref[3])


def test_closest_point_node_budget(niq, gpu_ready):
    """A persistent closest-point query past its node budget: NIQ_ERR_TIMEOUT with
    strict=True; with strict=False every result is written and each is an upper bound of
    the unbudgeted distance."""
    params = niq.workloads.spheres_sdf_model()
    f = gf(niq, params)
    q = np.random.default_rng(4).uniform(-1.2, 1.2, (64, 3)).astype(np.float32)
    full, _ = niq.kd_tree.closest_point(f, params, -np.ones(3), np.ones(3), q, eps=1e-3, persistent=True)
    with pytest.raises(niq._lib.NIQError) as e:
        niq.kd_tree.closest_point(f, params, -np.ones(3), np.ones(3), q, eps=1e-3, persistent=True, node_budget=8)
    assert e.value.code == niq._lib.NIQ_ERR_TIMEOUT
    d, _ = niq.kd_tree.closest_point(f, params, -np.ones(3), np.ones(3), q, eps=1e-3, persistent=True,
                                     node_budget=8, strict=False)
    fin = np.isfinite(d)
    assert np.all(d[fin] >= full[fin] - 1e-6)


def test_tensor_core_rate_probe_gives_up_and_recovers(niq, gpu_ready, tune):
    """niq_tc_tf32_rate (the roofline calibration of the 3xTF32 engine): a plausible rate,
    NIQ_ERR_TIMEOUT when its MMA waits may not poll, and a rate again afterwards."""
    import ctypes
    lib = niq._lib
    L = lib.load()
    v = ctypes.c_float(0.)
    lib.check(L.niq_tc_tf32_rate(256, ctypes.byref(v), None))
    assert 100. < v.value < 10000., v.value
    tune.set_params(mbar_polls=1)
    rc = L.niq_tc_tf32_rate(256, ctypes.byref(v), None)
    assert rc == lib.NIQ_ERR_TIMEOUT
    tune.set_params(mbar_polls=0)
    lib.check(L.niq_tc_tf32_rate(256, ctypes.byref(v), None))
    assert 100. < v.value < 10000., v.value


def test_fp32_rate_probe_is_plausible(niq, gpu_ready):
    """niq_fp32_fma_rate (the roofline calibration of the FP32 tile engine): a rate between a
    quarter of and the nominal FP32 FMA peak (SMs x 128 lanes x 2 FLOP x the maximum clock),
    and bad arguments rejected."""
    import ctypes
    import torch
    lib = niq._lib
    L = lib.load()
    v = ctypes.c_float(0.)
    lib.check(L.niq_fp32_fma_rate(2048, ctypes.byref(v), None))
    props = torch.cuda.get_device_properties(0)
    nominal = props.multi_processor_count * 128 * 2 * 2.2e9 / 1e12
    assert 0.25 * nominal < v.value < 1.05 * nominal, (v.value, nominal)
    assert L.niq_fp32_fma_rate(0, ctypes.byref(v), None) == lib.NIQ_ERR_INVALID_ARG
    assert L.niq_fp32_fma_rate(16, None, None) == lib.NIQ_ERR_INVALID_ARG
