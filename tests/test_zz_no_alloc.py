"""The allocation-free level-set tree (niq_levelset_tree_static), through the C ABI.

Some callers cannot allocate device memory at the moment they issue work: hosts that own
a fixed memory pool they cannot grow, plug-ins given only pre-allocated buffers, loops that
must not enter the allocator.  For them the tree keeps its scratch in a static device
array of the library, and the model blob, root box and outputs are the caller's.  This
file checks that entry point against the allocating one (niq_levelset_tree) on two calls
in a row, so the second call also proves the scratch is cleared between calls.  It is
collected last so that a run stopping at the first failure has run everything else.
"""
import ctypes as C
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATIC_NODES = 65536


def box_set(lo, hi):
    return {tuple(r) for r in np.concatenate([lo, hi], 1).tolist()}


def test_static_tree_matches_allocating_tree(niq, gpu_ready):
    import torch
    L = importlib.import_module('neural-implicit-queries_gb300._lib')
    lib = L.load()
    params = niq.workloads.spheres_sdf_model()
    blob = niq.mlp.pack(params)
    dev_blob = torch.frombuffer(bytearray(blob), dtype=torch.uint8).cuda()
    assert dev_blob.data_ptr() % 16 == 0
    opts = L.bound_opts('affine_fixed', conservative=True)
    lo3 = (C.c_float * 3)(-1., -1., -1.)
    hi3 = (C.c_float * 3)(1., 1., 1.)
    flags = 3   # interior and exterior lists too
    depth = 15
    stream = torch.cuda.current_stream().cuda_stream

    # the allocating entry point, for comparison
    m = niq.mlp.device_model(params)
    cap = 1 << 18
    ws_bytes = lib.niq_tree_workspace_size(cap, flags)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device='cuda')
    ref_counts = torch.zeros(4, dtype=torch.int64, device='cuda')
    L.check(lib.niq_levelset_tree(m.handle, C.byref(opts), lo3, hi3, depth, 0, 0.0, flags, cap,
                                  ref_counts.data_ptr(), ws.data_ptr(), ws_bytes, stream))
    ref = {}
    rc = ref_counts.cpu().numpy()
    kd = niq.kd_tree
    for kind in range(3):
        lo, hi = kd._tree_nodes(ws, cap, flags, kind, int(rc[kind]))
        ref[kind] = box_set(lo.cpu().numpy(), hi.cpu().numpy())

    for call in range(2):
        outs = [torch.full((STATIC_NODES, 3), -5.0, dtype=torch.float32, device='cuda') for _ in range(6)]
        counts = torch.zeros(4, dtype=torch.int64, device='cuda')
        L.check(lib.niq_levelset_tree_static(blob, dev_blob.data_ptr(), len(blob), C.byref(opts), lo3, hi3, depth, 0,
                                             0.0, flags, *[o.data_ptr() for o in outs], counts.data_ptr(), stream))
        c = counts.cpu().numpy()
        np.testing.assert_array_equal(c, rc)
        for kind in range(3):
            n = int(c[kind])
            got = box_set(outs[2 * kind][:n].cpu().numpy(), outs[2 * kind + 1][:n].cpu().numpy())
            assert got == ref[kind], (call, kind)


def test_static_tree_rejects_levels_beyond_the_scratch(niq, gpu_ready):
    import torch
    L = importlib.import_module('neural-implicit-queries_gb300._lib')
    lib = L.load()
    params = niq.workloads.spheres_sdf_model()
    blob = niq.mlp.pack(params)
    dev_blob = torch.frombuffer(bytearray(blob), dtype=torch.uint8).cuda()
    opts = L.bound_opts('affine_fixed', conservative=True)
    outs = [torch.empty((STATIC_NODES, 3), dtype=torch.float32, device='cuda') for _ in range(2)]
    counts = torch.zeros(4, dtype=torch.int64, device='cuda')
    rc = lib.niq_levelset_tree_static(blob, dev_blob.data_ptr(), len(blob), C.byref(opts),
                                      (C.c_float * 3)(-1., -1., -1.), (C.c_float * 3)(1., 1., 1.), 20, 0, 0.0, 0,
                                      outs[0].data_ptr(), outs[1].data_ptr(), None, None, None, None,
                                      counts.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == L.NIQ_ERR_CAPACITY
    assert b'static scratch' in lib.niq_last_error()


def test_static_tree_rejects_a_device_spec_unlike_the_host_spec(niq, gpu_ready):
    """Launch planning reads the host copy of the spec, the kernel the device copy: a
    device copy with another header is refused before any launch, and the next call with
    matching copies still succeeds."""
    import torch
    L = importlib.import_module('neural-implicit-queries_gb300._lib')
    lib = L.load()
    params = niq.workloads.spheres_sdf_model()
    blob = niq.mlp.pack(params)
    other = niq.mlp.pack(niq.workloads.he_mlp([3, 32, 32, 1], 'relu', seed=4, grid=8))
    opts = L.bound_opts('affine_fixed', conservative=True)
    lo3, hi3 = (C.c_float * 3)(-1., -1., -1.), (C.c_float * 3)(1., 1., 1.)
    outs = [torch.empty((STATIC_NODES, 3), dtype=torch.float32, device='cuda') for _ in range(2)]
    counts = torch.zeros(4, dtype=torch.int64, device='cuda')
    stream = torch.cuda.current_stream().cuda_stream
    for dev, want in ((other, L.NIQ_ERR_BAD_SPEC), (blob, 0)):
        dev_blob = torch.frombuffer(bytearray(dev), dtype=torch.uint8).cuda()
        rc = lib.niq_levelset_tree_static(blob, dev_blob.data_ptr(), len(blob), C.byref(opts), lo3, hi3, 8, 0, 0.0, 0,
                                          outs[0].data_ptr(), outs[1].data_ptr(), None, None, None, None,
                                          counts.data_ptr(), stream)
        assert rc == want, lib.niq_last_error()
    assert int(counts[0]) > 0
