"""Marching-cubes data (src/extract_cell.py:270-310).

Corner and edge numbering are the reference's.  The triangle table comes from
libniq's generator (niq_mc_table): per case the same polygons and orientation as the
reference's table (src/extract_cell.py:12-268), with polygons of four or more vertices
fan-triangulated from their lowest edge.  The extraction itself runs on the GPU
(kd_tree.hierarchical_marching_cubes).
"""
import numpy as np

from . import _lib

# src/extract_cell.py:274-287
EDGE_VERTS_NP = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6], [6, 7], [7, 4],
                          [0, 4], [1, 5], [2, 6], [3, 7]])
# src/extract_cell.py:293-302
VERT_LOGICAL_COORDS_NP = np.array([[0, 1, 0], [1, 1, 0], [1, 0, 0], [0, 0, 0],
                                   [0, 1, 1], [1, 1, 1], [1, 0, 1], [0, 0, 1]], dtype=bool)


def tri_table():
    out = (_lib.C.c_int32 * (256 * 16))()
    _lib.check(_lib.load().niq_mc_table(out))
    return np.frombuffer(out, dtype=np.int32).reshape(256, 16).astype(np.int64)


def get_mc_data():
    """src/extract_cell.py:306-310."""
    return tri_table(), EDGE_VERTS_NP.copy(), VERT_LOGICAL_COORDS_NP.copy()
