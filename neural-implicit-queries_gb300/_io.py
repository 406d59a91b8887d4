"""Array plumbing between user arrays (NumPy or torch) and device pointers.

Inputs may be NumPy arrays, CPU tensors or CUDA tensors; they are staged as contiguous
float32 CUDA tensors and results come back in the kind of the input (NumPy in, NumPy
out; CUDA tensor in, CUDA tensor out).  torch is used for device memory and streams only.
"""
from __future__ import annotations

import numpy as np


def torch():
    import torch as _t
    return _t


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise RuntimeError("no CUDA device: the query engine runs on the GPU only")
    return t


def to_dev(x, dtype='float32'):
    """(contiguous CUDA tensor, kind) for an array-like."""
    t = require_cuda()
    td = {'float32': t.float32, 'int32': t.int32, 'int64': t.int64}[dtype]
    if isinstance(x, t.Tensor):
        kind = 'cuda' if x.is_cuda else 'cpu'
        return x.to(device='cuda', dtype=td).contiguous(), kind
    a = np.ascontiguousarray(np.asarray(x, dtype=dtype))
    return t.from_numpy(a).to('cuda', non_blocking=False), 'numpy'


def to_numpy(x):
    """A NumPy array of an array-like or a (CPU or CUDA) tensor."""
    t = torch()
    if isinstance(x, t.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def back(t, kind):
    if kind == 'cuda':
        return t
    if kind == 'cpu':
        return t.cpu()
    return t.cpu().numpy()


def stream_handle():
    return torch().cuda.current_stream().cuda_stream


def ptr(t):
    return None if t is None else t.data_ptr()


_WS = {}


def workspace(nbytes):
    """A reusable scratch buffer for the current device and stream (>= nbytes)."""
    t = torch()
    key = (t.cuda.current_device(), stream_handle())
    buf = _WS.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = t.empty(max(int(nbytes), 256), dtype=t.uint8, device='cuda')
        _WS[key] = buf
    return buf


def release_workspaces():
    _WS.clear()
