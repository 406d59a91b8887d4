"""The level-set tree and closest point in the growing-term modes: the reference's loops
over the growing-term engine (niq_levelset_tree_growing, niq_closest_point), against the
reference's own results in affine_truncate (8 and 64 terms), affine_append (4) and
affine_all (tests/golden/tree_growing.npz), every difference explained by a
near-threshold decision (a bound at its threshold or a tie at a truncation boundary)
on the path that led to it (tests/parity.py)."""
import ctypes as C
import importlib

import numpy as np
import pytest

from conftest import golden, model_from
from parity import box_set_diff, unexplained_boxes, unexplained_queries

pytestmark = pytest.mark.gpu

CASES = {'truncate8': ('affine_truncate', {'affine_n_truncate': 8}),
         'truncate64': ('affine_truncate', {'affine_n_truncate': 64}),
         'append4': ('affine_append', {'affine_n_append': 4}),
         'all': ('affine_all', {})}


@pytest.mark.parametrize('name', list(CASES))
def test_tree_growing_golden(niq, R, gpu_ready, name):
    g = golden('tree_growing.npz')
    params = model_from(g, 'model/relu32x3')
    mode, kw = CASES[name]
    f = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=False, **kw)[0]
    d = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=8,
                                                            with_interior_nodes=True, with_exterior_nodes=True)
    o = R.generate_implicit(params, mode, **kw)
    for kind in ('unknown', 'interior', 'exterior'):
        extra, missing = box_set_diff(d[f'{kind}_node_lower'], d[f'{kind}_node_upper'],
                                      g[f'tree/{name}/{kind}/lower'], g[f'tree/{name}/{kind}/upper'])
        print(name, kind, len(extra), len(missing), len(d[f'{kind}_node_lower']))
        bad = unexplained_boxes(params, np.concatenate([extra, missing]), -np.ones(3), np.ones(3), func=o)
        assert len(bad) == 0, (kind, bad[:5])


@pytest.mark.parametrize('mode', ['affine_fixed', 'interval'])
def test_tree_growing_entry_in_fixed_modes(niq, gpu_ready, mode):
    """The host loop over niq_classify_boxes gives the persistent kernel's node sets in
    the fixed modes (same tile-engine arithmetic, another schedule)."""
    L = importlib.import_module('neural-implicit-queries_gb300._lib')
    lib = L.load()
    import torch
    params = niq.workloads.spheres_sdf_model()
    f = niq.implicit_mlp_utils.generate_implicit_from_params(params, mode, conservative=True, products='fp32')[0]
    ref = niq.kd_tree.construct_uniform_unknown_levelset_tree(f, params, -np.ones(3), np.ones(3), split_depth=12,
                                                              with_interior_nodes=True)
    m = niq.mlp.device_model(params)
    bo = f.bound_opts()
    cap, flags = 1 << 16, 1
    nb = lib.niq_tree_growing_workspace_size(m.handle, C.byref(bo), cap, flags)
    ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
    counts = torch.zeros(4, dtype=torch.int64, device='cuda')
    lo3, hi3 = (C.c_float * 3)(-1., -1., -1.), (C.c_float * 3)(1., 1., 1.)
    L.check(lib.niq_levelset_tree_growing(m.handle, C.byref(bo), lo3, hi3, 12, 0, 0.0, flags, cap,
                                          counts.data_ptr(), ws.data_ptr(), nb, torch.cuda.current_stream().cuda_stream))
    c = counts.cpu().numpy()
    assert int(c[3]) == ref['n_boxes_classified']
    for kind, name in ((0, 'unknown'), (1, 'interior')):
        lo, hi = niq.kd_tree._tree_nodes(ws, cap, flags, kind, int(c[kind]))
        extra, missing = box_set_diff(lo.cpu().numpy(), hi.cpu().numpy(), ref[f'{name}_node_lower'],
                                      ref[f'{name}_node_upper'])
        assert len(extra) == 0 and len(missing) == 0, (name, len(extra), len(missing))


def test_hmc_in_a_growing_mode(niq, gpu_ready):
    """hierarchical_marching_cubes with an affine_truncate function: the tree through the
    growing-term engine, then the same extraction.  A leaf whose corners change sign
    holds a zero, so every conservative bound keeps it: the triangles are the fixed
    mode's."""
    params = niq.workloads.spheres_sdf_model()
    ft = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_truncate', conservative=True,
                                                              affine_n_truncate=16)[0]
    ff = niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=True)[0]
    a = niq.kd_tree.hierarchical_marching_cubes(ft, params, -np.ones(3), np.ones(3), 5, n_subcell_depth=1)
    b = niq.kd_tree.hierarchical_marching_cubes(ff, params, -np.ones(3), np.ones(3), 5, n_subcell_depth=1)
    key = lambda t: {tuple(r) for r in np.round(t.reshape(-1, 9), 5).tolist()}
    assert a.shape[0] > 1000 and key(b) <= key(a)


@pytest.mark.parametrize('name', ['truncate8', 'truncate64'])
def test_closest_point_growing_golden(niq, R, gpu_ready, name):
    """closest_point in affine_truncate through the reference schedule (each popped batch
    classified by the growing-term engine) against the reference's distances."""
    g = golden('tree_growing.npz')
    A = model_from(g, 'model/A')
    mode, kw = CASES[name]
    f = niq.implicit_mlp_utils.generate_implicit_from_params(A, mode, conservative=False, **kw)[0]
    o = R.generate_implicit(A, mode, **kw)
    q = g['cp/q']
    for B in (8, 2048):
        dist, loc = niq.kd_tree.closest_point(f, A, -np.ones(3), np.ones(3), q, eps=0.05, batch_process_size=B)
        _, _, tr = R.closest_point(o, A, -np.ones(3), np.ones(3), q, eps=0.05, batch_process_size=B, trace=True)
        bad = unexplained_queries(dist, g[f'cp/{name}/B{B}/dist'], tr)
        assert bad.size == 0, (B, bad)
