"""ctypes wrapper of oracle/cpu_tree.c (test infrastructure and CPU baseline only): the
affine_fixed level-set tree and the marching cubes on its leaves on the host cores with
OpenMP."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, '_build', 'libcpu_tree.so')
ACTS = {'none': 0, 'relu': 1, 'elu': 2}


def build(force=False):
    """gcc -O3 -fopenmp, no FMA contraction (the reference rounds every product)."""
    src = os.path.join(HERE, 'cpu_tree.c')
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + '.tmp'
    base = ['gcc', '-O3', '-ffp-contract=off', '-fPIC', '-shared', '-o', tmp, src, '-lm']
    r = subprocess.run(base[:1] + ['-fopenmp'] + base[1:], capture_output=True, text=True)
    if r.returncode != 0:   # no OpenMP runtime: build the serial form
        subprocess.run(base, check=True)
    os.replace(tmp, LIB)
    return LIB


def _load():
    lib = C.CDLL(build())
    lib.cpu_hmc_leaves.restype = C.c_int64
    lib.cpu_hmc_leaves.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_void_p, C.c_int64,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int64]
    lib.cpu_levelset_tree.restype = C.c_int64
    lib.cpu_levelset_tree.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_float),
                                      C.POINTER(C.c_float), C.c_int, C.c_float, C.c_int, C.POINTER(C.c_int64),
                                      C.c_void_p, C.c_int64]
    return lib


def _net(layers):
    n = len(layers)
    A = [np.ascontiguousarray(l[0], np.float32) for l in layers]
    b = [np.ascontiguousarray(l[1], np.float32) for l in layers]
    keep = (A, b)
    return (n, (C.c_int * n)(*[a.shape[0] for a in A]), (C.c_int * n)(*[a.shape[1] for a in A]),
            (C.c_int * n)(*[ACTS[l[2]] for l in layers]), (C.c_void_p * n)(*[a.ctypes.data for a in A]),
            (C.c_void_p * n)(*[x.ctypes.data for x in b])), keep


def hmc_leaves(layers, leaves, threads=0, want_tris=True):
    """Marching cubes on every leaf box (leaves (n, 6): lower | upper) as one cell, the
    n_subcell_depth = 0 extraction of src/kd_tree.py:357-399.  Returns (T, 3, 3) float32
    triangles in leaf order (or their count when want_tris is False)."""
    from oracle import mc_table
    lib = _load()
    net, keep = _net(layers)
    leaves = np.ascontiguousarray(leaves, np.float32)
    table = np.ascontiguousarray(mc_table.make_table(), np.int32)
    edge = np.ascontiguousarray(mc_table.EDGE, np.int32)
    vert = np.ascontiguousarray(mc_table.VERT, np.int32)
    n = leaves.shape[0]
    count = lib.cpu_hmc_leaves(*net, leaves.ctypes.data, n, table.ctypes.data, edge.ctypes.data, vert.ctypes.data,
                               int(threads), None, 0)
    if count < 0:
        raise ValueError("unsupported network for the C restatement")
    if not want_tris:
        return int(count)
    tris = np.zeros((max(count, 1), 3, 3), np.float32)
    lib.cpu_hmc_leaves(*net, leaves.ctypes.data, n, table.ctypes.data, edge.ctypes.data, vert.ctypes.data,
                       int(threads), tris.ctypes.data, count)
    return tris[:count]


def levelset_tree(layers, lower, upper, split_depth, offset=0., threads=0, want_leaves=False):
    """``layers``: [(A (in, out), b (out,), act_name)].  Returns (n_leaves, n_boxes,
    leaves (n, 6) or None)."""
    lib = _load()
    n = len(layers)
    A = [np.ascontiguousarray(l[0], np.float32) for l in layers]
    b = [np.ascontiguousarray(l[1], np.float32) for l in layers]
    ins = (C.c_int * n)(*[a.shape[0] for a in A])
    outs = (C.c_int * n)(*[a.shape[1] for a in A])
    acts = (C.c_int * n)(*[ACTS[l[2]] for l in layers])
    Ap = (C.c_void_p * n)(*[a.ctypes.data for a in A])
    bp = (C.c_void_p * n)(*[x.ctypes.data for x in b])
    lo = (C.c_float * 3)(*np.asarray(lower, np.float32).tolist())
    hi = (C.c_float * 3)(*np.asarray(upper, np.float32).tolist())
    nb = C.c_int64(0)
    cap = 1 << 22 if want_leaves else 0
    leaves = np.zeros((cap, 6), np.float32) if want_leaves else None
    r = lib.cpu_levelset_tree(n, ins, outs, acts, Ap, bp, lo, hi, int(split_depth), float(offset), int(threads),
                              C.byref(nb), leaves.ctypes.data if want_leaves else None, cap)
    if r < 0:
        raise ValueError("unsupported network for the C restatement")
    return int(r), int(nb.value), (leaves[:min(r, cap)] if want_leaves else None)
