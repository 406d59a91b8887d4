"""CPU-only checks: the C-ABI library, the spec packer, the triangle table."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden


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


def test_c_abi_checks_arguments_before_device_work(lib, niq):
    """The C ABI's argument and spec checks return their status before any device work,
    so they hold on a machine without a GPU: bad counts, null pointers, and packed specs
    whose header does not validate (src/mlp.py:131,142), each with a message."""
    import ctypes
    L, so = lib
    v = ctypes.c_float(0.)
    assert so.niq_fp32_fma_rate(0, ctypes.byref(v), None) == L.NIQ_ERR_INVALID_ARG
    assert b'iters' in so.niq_last_error()
    assert so.niq_tc_tf32_rate(0, ctypes.byref(v), None) == L.NIQ_ERR_INVALID_ARG
    assert b'chunks' in so.niq_last_error()
    out = ctypes.c_void_p()
    assert so.niq_model_create(None, 0, ctypes.byref(out)) == L.NIQ_ERR_INVALID_ARG
    blob = bytes(niq.mlp.pack(niq.workloads.he_mlp([3, 8, 1], 'relu', seed=1, grid=8)))
    buf = ctypes.create_string_buffer(blob[:16], 16)
    assert so.niq_model_create(buf, 16, ctypes.byref(out)) == L.NIQ_ERR_BAD_SPEC
    assert b'too short' in so.niq_last_error()
    bad = bytearray(blob)
    bad[0] ^= 0xFF                                   # magic
    buf = ctypes.create_string_buffer(bytes(bad), len(bad))
    assert so.niq_model_create(buf, len(bad), ctypes.byref(out)) == L.NIQ_ERR_BAD_SPEC
    assert b'magic' in so.niq_last_error()
    buf = ctypes.create_string_buffer(blob, len(blob))
    assert so.niq_model_create(buf, len(blob) - 4, ctypes.byref(out)) == L.NIQ_ERR_BAD_SPEC
    assert b'does not match' in so.niq_last_error()
    assert out.value is None


def test_mc_table_library_matches_oracle(lib):
    from oracle import mc_table
    L, so = lib
    out = (L.C.c_int32 * 4096)()
    assert so.niq_mc_table(out) == 0
    T = np.frombuffer(out, dtype=np.int32).reshape(256, 16)
    np.testing.assert_array_equal(T, mc_table.make_table())


def test_mc_table_equivalent_to_reference():
    """Same polygons (edge sets per connected piece) and orientation (vector area, which
    does not depend on the triangulation) as the reference's third-party table, case by
    case: the digests in mc_digest.npz were computed from the reference's table by
    tests/golden/make_golden.py."""
    import sys
    sys.path.insert(0, GOLDEN)
    import mc_canon
    from oracle import mc_table
    ref = golden('mc_digest.npz')['mc/digest']
    ours = mc_canon.case_digests(mc_table.make_table(), mc_table.VERT, mc_table.EDGE)
    bad = np.nonzero(ref != ours)[0]
    assert bad.size == 0, f'cases differing from the reference table: {bad.tolist()}'


def test_camera_rays_golden(niq):
    """render.generate_camera_rays / look_at bit for bit against the reference's own
    functions (src/render.py:17-50,229-242) run over the NumPy stand-in."""
    g = golden('camera.npz')
    R = niq.render
    eyes = g['look_at/eyes']
    for up in ('y', 'z'):
        for i, e in enumerate(eyes):
            with np.errstate(invalid='ignore'):
                got = R.look_at(e, up_dir=up)
            for j, name in enumerate(('look', 'up', 'left')):
                np.testing.assert_array_equal(got[j], g[f'look_at/{up}/{name}'][i])
    for res in (5, 33, 128, 16):
        k = f'cam/{res}/'
        roots, dirs = R.generate_camera_rays(g[k + 'eye'], g[k + 'look'], g[k + 'up'], res=res,
                                             fov_deg=float(g[k + 'fov']))
        assert roots.dtype == np.float32 and dirs.dtype == np.float32
        np.testing.assert_array_equal(roots, g[k + 'roots'])
        np.testing.assert_array_equal(dirs, g[k + 'dirs'])


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


def test_autotune_cache_roundtrip(niq, tmp_path, monkeypatch):
    """The autotuner's cache on the host: a stored choice is found again by its key and
    applied through niq_tune_set; unknown keys and a corrupt file give no choice."""
    at = niq.autotune
    old = at.get_params()
    monkeypatch.setattr(at, 'CACHE', str(tmp_path / 'tune.json'))
    try:
        assert at.apply('batched|none') is None
        at._store('batched|k1', {'batched_chunk': 256, 'batched_ctas_per_sm': 1})
        at._store('tree|k2', {'tree_ctas_per_sm': 2})
        assert at.apply('batched|k1') == {'batched_chunk': 256, 'batched_ctas_per_sm': 1}
        p = at.get_params()
        assert p['batched_chunk'] == 256 and p['batched_ctas_per_sm'] == 1
        assert at.apply('tree|k2') == {'tree_ctas_per_sm': 2} and at.get_params()['tree_ctas_per_sm'] == 2
        (tmp_path / 'tune.json').write_text('{not json')
        assert at.apply('batched|k1') is None
    finally:
        at.set_params(**old)


def test_tuning_parameters_roundtrip(niq):
    """niq_tune_set/get on the host (no device work): values stick, bad ones are refused."""
    at = niq.autotune
    old = at.get_params()
    try:
        at.set_params(batched_chunk=64, batched_ctas_per_sm=1, tree_ctas_per_sm=2, barrier_polls=5, mbar_polls=1,
                      ray_columns=8)
        assert at.get_params() == {'batched_chunk': 64, 'batched_ctas_per_sm': 1, 'tree_ctas_per_sm': 2,
                                   'barrier_polls': 5, 'mbar_polls': 1, 'ray_columns': 8}
        with pytest.raises(ValueError):
            at.set_params(batched_chunk=7)
        with pytest.raises(ValueError):
            at.set_params(ray_columns=6)
        with pytest.raises(ValueError):
            at.set_params(tree_ctas_per_sm=-1)
    finally:
        at.set_params(**old)
