"""CPU-only checks: the C-ABI library, the spec packer, the triangle table."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope='module')
def lib(niq):
    import importlib
    b = importlib.import_module('neural-implicit-queries_gb300._build')
    b.build()
    L = importlib.import_module('neural-implicit-queries_gb300._lib')
    return L, L.load()


def header_functions():
    src = open(os.path.join(ROOT, 'include', 'niq.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(niq_[a-z0-9_]+)\s*\(', src)))


def test_library_exports_every_header_function(lib):
    L, so = lib
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(so, n), n
    assert set(names) == set(L.exported_symbols())


def test_mc_table_library_matches_oracle(lib):
    from oracle import mc_table
    L, so = lib
    out = (L.C.c_int32 * 4096)()
    assert so.niq_mc_table(out) == 0
    T = np.frombuffer(out, dtype=np.int32).reshape(256, 16)
    np.testing.assert_array_equal(T, mc_table.make_table())


def test_mc_table_equivalent_to_reference():
    """Same polygons (edge sets per connected piece) and orientation as the reference's
    third-party table, case by case."""
    from oracle import mc_table
    from test_oracle_golden import reference_mc_table
    ref = reference_mc_table()
    T = mc_table.make_table()
    mid = (mc_table.VERT[mc_table.EDGE[:, 0]] + mc_table.VERT[mc_table.EDGE[:, 1]]) / 2.0

    def tris(row):
        return [tuple(row[i:i + 3]) for i in range(0, 15, 3) if row[i] != -1]

    def comps(ts):
        groups = []
        for t in ts:
            hit = [g for g in groups if set(t) & {x for tt in g for x in tt}]
            groups = [g for g in groups if g not in hit] + [[t] + [tt for g in hit for tt in g]]
        return groups

    def vec_area(g):
        return sum(np.cross(mid[b] - mid[a], mid[c] - mid[a]) for a, b, c in g)

    for c in range(256):
        gr, gm = comps(tris(ref[c])), comps(tris(T[c]))
        assert sorted(sorted({x for t in g for x in t}) for g in gr) == \
            sorted(sorted({x for t in g for x in t}) for g in gm), c
        for g in gr:
            es = {x for t in g for x in t}
            h = [x for x in gm if {y for t in x for y in t} == es][0]
            assert np.dot(vec_area(g), vec_area(h)) > 0, c


def test_pack_roundtrip_and_errors(niq):
    import struct
    mlp = niq.mlp
    params = niq.workloads.he_mlp([3, 20, 7, 1], 'tanh', seed=3, grid=8)
    blob = mlp.pack(params)
    magic, ver, nl, din, dout, maxw, nw, _ = struct.unpack('<Iiiiiiii', blob[:32])
    assert (magic, nl, din, dout, maxw) == (0x3151494e, 3, 3, 1, 20)
    assert len(blob) == 32 + 32 * 32 + 4 * nw
    rec = struct.unpack('<iiiiiiif', blob[32:64])
    assert rec[:5] == (3, 20, 4, 20, 3)
    w = np.frombuffer(blob[32 + 32 * 32:], np.float32)
    A0 = w[rec[5]:rec[5] + 4 * 20].reshape(4, 20)
    np.testing.assert_array_equal(A0[:3], params['0000.dense.A'])
    assert np.all(A0[3] == 0)
    bad = dict(params)
    bad['0007.sin._'] = np.zeros(0, np.float32)
    with pytest.raises(ValueError):
        mlp.pack(bad)
    with pytest.raises(ValueError):
        mlp.pack({'zz.dense.A': np.zeros((3, 1), np.float32)})
    two = dict(params)
    two['0001.dense.A'] = np.zeros((5, 5), np.float32)   # op 1 is now dense, chain breaks
    with pytest.raises(ValueError):
        mlp.pack(two)


def test_spatial_transformation_pack(niq, R):
    wl = niq.workloads
    params = wl.prepend_spatial_transformation(wl.he_mlp([3, 8, 1], 'relu', seed=1, grid=8),
                                               R=wl.random_rotation(np.random.default_rng(0)),
                                               t=np.array([0.1, 0.2, 0.3], np.float32))
    layers = niq.mlp.spec_layers(params)
    assert len(layers) == 3 and layers[0][2] == 'none' and layers[1][2] == 'relu'
    x = np.random.default_rng(1).uniform(-1, 1, (5, 3)).astype(np.float32)
    y = x
    for A, b, act in layers:
        y = y @ A + b
        if act == 'relu':
            y = np.maximum(y, 0)
    np.testing.assert_allclose(y[:, 0], R.eval_points(params, x), rtol=1e-5, atol=1e-6)


def test_generate_implicit_modes(niq):
    u = niq.implicit_mlp_utils
    p = niq.workloads.he_mlp([3, 8, 1], 'relu', seed=1, grid=8)
    for mode in ['interval', 'affine_fixed', 'affine_all', 'slope_interval', 'sdf']:
        f, q = u.generate_implicit_from_params(p, mode)
        assert q is p
    f, _ = u.generate_implicit_from_params(p, 'affine_truncate', affine_n_truncate=8, affine_truncate_policy='absolute')
    assert f.truncate_count == 8
    with pytest.raises(RuntimeError):
        u.generate_implicit_from_params(p, 'bogus')
    with pytest.raises(ValueError):
        niq.affine.AffineContext('nope')


def test_tuning_parameters_roundtrip(niq):
    """niq_tune_set/get on the host (no device work): values stick, bad ones are refused."""
    at = niq.autotune
    old = at.get_params()
    try:
        at.set_params(batched_chunk=64, batched_ctas_per_sm=1, tree_ctas_per_sm=2)
        assert at.get_params() == {'batched_chunk': 64, 'batched_ctas_per_sm': 1, 'tree_ctas_per_sm': 2}
        with pytest.raises(ValueError):
            at.set_params(batched_chunk=7)
        with pytest.raises(ValueError):
            at.set_params(tree_ctas_per_sm=-1)
    finally:
        at.set_params(**old)
