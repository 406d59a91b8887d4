"""Canonical form of a marching-cubes triangle table, for comparing two tables that may
triangulate the same polygons differently.

For every case the triangles are grouped into connected pieces (triangles sharing an
edge index).  A piece is described by its sorted set of cut edges and by its vector
area, computed from the edge midpoints of the unit cube: for a closed polygon the vector
area does not depend on how the polygon was triangulated, and with midpoints on the
cube's edges it is an exact multiple of 1/8.  The description of a case is the sorted
list of its pieces; ``case_digests`` hashes it, so a committed fixture can pin a table
without holding the table itself.
"""
import hashlib

import numpy as np


def _pieces(row):
    tris = [tuple(int(x) for x in row[i:i + 3]) for i in range(0, len(row) - 2, 3) if row[i] != -1]
    groups = []
    for t in tris:
        hit = [g for g in groups if set(t) & {x for tt in g for x in tt}]
        groups = [g for g in groups if g not in hit] + [[t] + [tt for g in hit for tt in g]]
    return groups


def canonical_case(row, vert, edge):
    mid = (vert[edge[:, 0]] + vert[edge[:, 1]]) / 2.0
    out = []
    for g in _pieces(row):
        area = sum(np.cross(mid[b] - mid[a], mid[c] - mid[a]) for a, b, c in g) * 0.5
        out.append((tuple(sorted({x for t in g for x in t})), tuple(int(round(8 * v)) for v in area)))
    return tuple(sorted(out))


def case_digests(table, vert, edge):
    """(256,) uint64: the first 8 bytes of the SHA-256 of each case's canonical form."""
    d = np.zeros(len(table), np.uint64)
    for c, row in enumerate(table):
        h = hashlib.sha256(repr(canonical_case(row, vert, edge)).encode()).digest()
        d[c] = np.frombuffer(h[:8], np.uint64)[0]
    return d
