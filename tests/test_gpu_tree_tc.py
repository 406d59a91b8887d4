"""The level-set tree with tensor-core products (csrc/k_tree_tc.cu, products='3xtf32';
affine_fixed with outward rounding on models whose hidden layers are at most 64 wide).

Its bounds are conservative like the FP32 engine's, with a larger rounding term (3xTF32
products), so it keeps somewhat more boxes unknown and against the reference's
arithmetic it may only keep MORE; interior and exterior nodes must hold the right sign
at every FP64 sample; and it gives the same node sets in all three schedules."""
import ctypes as C

import numpy as np
import pytest

from parity import box_set_diff

pytestmark = pytest.mark.gpu


def gf(niq, params, products='3xtf32', conservative=True, mode='affine_fixed'):
    return niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=conservative,
                                                                products=products)[0]


def engine(niq, params, f):
    v = C.c_int32(-1)
    bo = f.bound_opts()
    niq._lib.check(niq._lib.load().niq_tree_engine(niq.mlp.device_model(params).handle, C.byref(bo), C.byref(v)))
    return v.value


def models(niq):
    wl = niq.workloads
    return {'spheres': wl.spheres_sdf_model(),
            'relu32x3': wl.plain_small_model(),
            'tanh48x2': wl.he_mlp([3, 48, 48, 1], 'tanh', seed=11, grid=16),
            'elu64x3': wl.he_mlp([3, 64, 64, 64, 1], 'elu', seed=12, grid=16)}


def fp64_signs_hold(R, params, lo, hi, want_negative, n=200000, seed=0):
    """Every FP64 value of the network at random points of the nodes has the sign the
    tree gave the node (interior: < 0, exterior: > 0)."""
    if len(lo) == 0:
        return True
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, len(lo), n)
    u = rng.uniform(0, 1, (n, 3))
    x = lo[idx].astype(np.float64) + u * (hi[idx] - lo[idx]).astype(np.float64)
    v = R.eval_points(params, x, np.float64)
    return bool(np.all(v < 0)) if want_negative else bool(np.all(v > 0))


@pytest.mark.parametrize('name', ['spheres', 'relu32x3', 'tanh48x2', 'elu64x3'])
def test_tc_tree_conservative(niq, R, gpu_ready, name):
    params = models(niq)[name]
    assert engine(niq, params, gf(niq, params)) == 1
    assert engine(niq, params, gf(niq, params, 'fp32')) == 0
    assert engine(niq, params, gf(niq, params, 'auto')) == 0
    lo3, hi3 = -np.ones(3, np.float32), np.ones(3, np.float32)
    depth = 15
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(gf(niq, params), params, lo3, hi3, split_depth=depth,
                                                            with_interior_nodes=True, with_exterior_nodes=True)
    d32 = niq.kd_tree.construct_uniform_unknown_levelset_tree(gf(niq, params, 'fp32'), params, lo3, hi3,
                                                              split_depth=depth, with_interior_nodes=True,
                                                              with_exterior_nodes=True)
    n = len(d['unknown_node_lower'])
    assert n > 0
    # against the FP32 engine: the split products' rounding bound (about 3.5e-5 relative
    # at 64 terms against 3.9e-6) keeps more boxes near the surface unknown, and almost
    # never fewer
    extra, missing = box_set_diff(d['unknown_node_lower'], d['unknown_node_upper'], d32['unknown_node_lower'],
                                  d32['unknown_node_upper'])
    print(f'{name}: {n} leaves; against the FP32 engine {len(extra)} extra, {len(missing)} missing')
    assert len(missing) <= 0.002 * n + 2
    assert len(extra) <= 0.05 * n + 2
    # against the reference's arithmetic (oracle, no outward rounding): conservative bounds
    # are never narrower, so no leaf of the reference goes missing
    if name in ('spheres', 'relu32x3'):
        o = R.generate_implicit(params, 'affine_fixed')
        r = R.construct_uniform_unknown_levelset_tree(o, params, lo3, hi3, split_depth=depth)
        extra, missing = box_set_diff(d['unknown_node_lower'], d['unknown_node_upper'], r['unknown_node_lower'],
                                      r['unknown_node_upper'])
        print(f'{name}: against the reference arithmetic {len(extra)} extra of {len(r["unknown_node_lower"])}')
        assert len(missing) == 0
        assert len(extra) <= 0.05 * len(r['unknown_node_lower']) + 2
    # interior and exterior nodes: the FP64 network has their sign everywhere sampled
    assert fp64_signs_hold(R, params, d['interior_node_lower'], d['interior_node_upper'], True)
    assert fp64_signs_hold(R, params, d['exterior_node_lower'], d['exterior_node_upper'], False, seed=1)
    # the volumes still tile the root box
    vol = sum(np.prod((d[f'{k}_node_upper'] - d[f'{k}_node_lower']).astype(np.float64), axis=1).sum()
              for k in ('unknown', 'interior', 'exterior'))
    assert vol == pytest.approx(8.0, rel=1e-12)


def test_tc_tree_offset_and_threshold(niq, gpu_ready):
    """node_terminate_thresh and a nonzero offset (the sample_surface call of
    src/kd_tree.py:267) through the tensor-core tree: same stopping rule as the FP32
    engine, and only near-threshold boxes differ."""
    params = niq.workloads.spheres_sdf_model()
    lo3, hi3 = -np.ones(3, np.float32), np.ones(3, np.float32)
    a = niq.kd_tree.construct_uniform_unknown_levelset_tree(gf(niq, params), params, lo3, hi3,
                                                            node_terminate_thresh=4096, offset=0.02)
    b = niq.kd_tree.construct_uniform_unknown_levelset_tree(gf(niq, params, 'fp32'), params, lo3, hi3,
                                                            node_terminate_thresh=4096, offset=0.02)
    n = len(a['unknown_node_lower'])
    assert n >= 4096
    extra, missing = box_set_diff(a['unknown_node_lower'], a['unknown_node_upper'], b['unknown_node_lower'],
                                  b['unknown_node_upper'])
    assert len(missing) <= 0.002 * n + 2 and len(extra) <= 0.05 * n + 2
