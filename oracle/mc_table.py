"""Programmatic marching-cubes triangle table (test infrastructure copy).

The reference ships a third-party 256-case table (src/extract_cell.py:12-268) with its
own corner numbering (src/extract_cell.py:293-302) and edge numbering
(src/extract_cell.py:274-287).  This module derives an equivalent table from those two
numberings alone: for each case the cut edges of every cube face are joined into
segments (an ambiguous face keeps its inside corners apart), segments chain into
closed loops, each loop is oriented so its normal points from the inside (value < 0)
corners to the outside ones, and loops are fan-triangulated from their lowest edge.
The CUDA library builds the same table in C++ (csrc/k_hmc.cu, exported as
niq_mc_table); tests compare the two, and compare this one case by case with digests
of the reference's table (tests/golden/mc_digest.npz).
"""
import numpy as np

# corner i -> logical (x, y, z), src/extract_cell.py:293-302
VERT = np.array([[0, 1, 0], [1, 1, 0], [1, 0, 0], [0, 0, 0],
                 [0, 1, 1], [1, 1, 1], [1, 0, 1], [0, 0, 1]])
# edge e -> (corner a, corner b), src/extract_cell.py:274-287
EDGE = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6], [6, 7], [7, 4],
                 [0, 4], [1, 5], [2, 6], [3, 7]])


def _faces():
    """Each cube face as a 4-cycle of corners."""
    faces = []
    for axis in range(3):
        for side in (0, 1):
            cs = [i for i in range(8) if VERT[i][axis] == side]
            # order the 4 corners cyclically around the face
            o = [a for a in range(3) if a != axis]
            ang = [np.arctan2(VERT[c][o[1]] - 0.5, VERT[c][o[0]] - 0.5) for c in cs]
            faces.append([cs[k] for k in np.argsort(ang)])
    return faces


def _edge_id(a, b):
    for e, (p, q) in enumerate(EDGE):
        if (p, q) == (a, b) or (p, q) == (b, a):
            return e
    raise KeyError((a, b))


def case_loops(case):
    inside = [(case >> i) & 1 for i in range(8)]
    segs = []
    for f in _faces():
        cut = []
        for k in range(4):
            a, b = f[k], f[(k + 1) % 4]
            if inside[a] != inside[b]:
                cut.append((k, _edge_id(a, b)))
        if len(cut) == 2:
            segs.append((cut[0][1], cut[1][1]))
        elif len(cut) == 4:
            # ambiguous face: cut off each inside corner on its own
            for k in range(4):
                c = f[k]
                if inside[c]:
                    segs.append((_edge_id(f[(k - 1) % 4], c), _edge_id(c, f[(k + 1) % 4])))
    adj = {}
    for a, b in segs:
        adj.setdefault(a, []).append(b)
        adj.setdefault(b, []).append(a)
    loops, seen = [], set()
    for start in sorted(adj):
        if start in seen:
            continue
        loop = [start]
        seen.add(start)
        prev, cur = None, start
        while True:
            nxt = [x for x in adj[cur] if x != prev and (x not in seen or (x == start and len(loop) > 2))]
            if not nxt:
                break
            x = nxt[0]
            if x == start:
                break
            loop.append(x)
            seen.add(x)
            prev, cur = cur, x
        loops.append(loop)
    # orient: normal from inside corners towards outside corners
    mid = (VERT[EDGE[:, 0]] + VERT[EDGE[:, 1]]) / 2.0
    out = []
    for loop in loops:
        P = mid[loop]
        n = np.zeros(3)
        for i in range(len(loop)):
            p, q = P[i], P[(i + 1) % len(loop)]
            n += np.cross(p, q)
        ins = [EDGE[e][0] if inside[EDGE[e][0]] else EDGE[e][1] for e in loop]
        outs = [EDGE[e][1] if inside[EDGE[e][0]] else EDGE[e][0] for e in loop]
        d = VERT[outs].mean(0) - VERT[ins].mean(0)
        if np.dot(n, d) < 0:
            loop = loop[::-1]
        k = int(np.argmin(loop))
        out.append(loop[k:] + loop[:k])
    return out


def make_table(flip=False):
    """(256, 16) int table: up to 5 triangles of edge ids, -1 padded."""
    T = -np.ones((256, 16), np.int64)
    for case in range(256):
        tris = []
        for loop in case_loops(case):
            for i in range(1, len(loop) - 1):
                tri = [loop[0], loop[i], loop[i + 1]]
                tris.append(tri[::-1] if flip else tri)
        assert len(tris) <= 5, case
        flat = [e for t in tris for e in t]
        T[case, :len(flat)] = flat
    return T
