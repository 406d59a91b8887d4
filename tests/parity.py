"""Parity rules shared by the GPU tests: every difference between the CUDA path and the
oracle (or the reference's golden outputs) must be explained by a decision that sat
within rounding of its threshold; nothing passes on a fraction.

- Rays (src/queries.py:44-120): a ray's path is a sequence of decisions (segment bound
  sign, hit test).  Two implementations that differ only in last-ulp rounding take the
  same path until one of them meets a decision within NEAR_REL of flipping.  The
  oracle's trace gives, per ray, the step index of its first such decision; a ray may
  differ only if that index is below both implementations' step counts.
- Closest point (src/kd_tree.py:659-802): the reference schedule pops batches from one
  stack shared by all queries, so after the first near decision anywhere the batches can
  hold different nodes.  A query may differ only if one of its own decisions was near,
  or if it still had nodes processed at or after the first near round.
- Trees (src/kd_tree.py:19-218): a box may be present in one set and not the other only
  if its oracle bound straddles the threshold by less than NEAR_REL of its scale.
"""
import numpy as np

from oracle import ref_np as R

NEAR_REL = R.NEAR_REL


def ray_match(t, hid, cnt, rt, rhid, rcnt):
    """Same hit id and step count, hit distance within 1e-4 relative."""
    return (hid == rhid) & (cnt == rcnt) & np.isclose(t, rt, rtol=1e-4, atol=1e-5)


def unexplained_rays(t, hid, cnt, rt, rhid, rcnt, first_near):
    """Indices of rays that differ without a near-threshold decision on the shared part
    of their path; also prints the mismatch count for the log."""
    bad = ~ray_match(t, hid, cnt, rt, rhid, rcnt)
    ok = np.asarray(first_near) < np.minimum(cnt, rcnt)
    print(f'rays: {int(bad.sum())} of {bad.size} differ, {int((bad & ok).sum())} explained by a '
          f'near-threshold decision ({int((np.asarray(first_near) < 2 ** 31 - 1).sum())} rays took one)')
    return np.nonzero(bad & ~ok)[0]


def unexplained_queries(dist, rdist, trace, rtol=1e-4, atol=1e-5):
    """Closest-point queries whose distance differs (beyond 1e-4 relative) without an
    explanation from the oracle's trace."""
    d, r = np.asarray(dist), np.asarray(rdist)
    same = (np.isinf(d) & np.isinf(r)) | np.isclose(d, r, rtol=rtol, atol=atol)
    ok = trace['near'] | (trace['last_round'] >= trace['first_near_round'])
    print(f'closest point: {int((~same).sum())} of {same.size} differ, {int((~same & ok).sum())} explained')
    return np.nonzero(~same & ~ok)[0]


def box_rows(lo, hi):
    return np.ascontiguousarray(np.concatenate([np.asarray(lo, np.float32), np.asarray(hi, np.float32)], 1))


def box_set_diff(lo, hi, rlo, rhi):
    """Rows (lower | upper) present in one set only: (extra, missing) as (n, 6) arrays."""
    a, b = box_rows(lo, hi), box_rows(rlo, rhi)
    va = a.view(np.dtype((np.void, 24))).ravel()
    vb = b.view(np.dtype((np.void, 24))).ravel()
    return a[~np.isin(va, vb)], b[~np.isin(vb, va)]


def straddle_rows(params, boxes, mode='affine_fixed', offset=0., func=None):
    """Rows of ``boxes`` ((n, 6): lower | upper) whose FP32 oracle bound does NOT sit
    within NEAR_REL of the classification threshold."""
    b = np.asarray(boxes, np.float32).reshape(-1, 6)
    if len(b) == 0:
        return b
    f = func or R.generate_implicit(params, mode)
    c = (0.5 * (b[:, :3] + b[:, 3:])).astype(np.float32)
    v = (b[:, 3:] - c)[:, :, None] * np.eye(3, dtype=np.float32)
    _, _, near = f.bounds_near(params, c, v, offset)
    return b[~near]


def unexplained_boxes(params, rows, root_lo, root_hi, mode='affine_fixed', offset=0., func=None):
    """Rows ((n, 6): lower | upper) of boxes found in one tree's node sets and not the
    other's that no near-threshold decision explains.  A box's fate is decided along its
    path from the root, so the first decision where two trees part must lie on that path:
    the box is explained when its own oracle bound, or that of one of its ancestors (the
    bisection rule of src/kd_tree.py:38,70-77 replayed from the root), sits within
    NEAR_REL of the threshold."""
    b = np.asarray(rows, np.float32).reshape(-1, 6)
    if len(b) == 0:
        return b
    f = func or R.generate_implicit(params, mode)
    target_c = 0.5 * (b[:, :3] + b[:, 3:])
    lo = np.repeat(np.asarray(root_lo, np.float32)[None], len(b), 0)
    hi = np.repeat(np.asarray(root_hi, np.float32)[None], len(b), 0)
    path = []
    for _ in range(64):
        live = np.any(hi - lo > (b[:, 3:] - b[:, :3]) * 1.5, axis=1)
        path.append(np.concatenate([lo, hi], 1))
        if not live.any():
            break
        (alo, ahi), (blo, bhi) = R.split_children(lo, hi)
        in_b = np.all(target_c >= blo, axis=1)
        nlo, nhi = np.where(in_b[:, None], blo, alo), np.where(in_b[:, None], bhi, ahi)
        lo, hi = np.where(live[:, None], nlo, lo), np.where(live[:, None], nhi, hi)
    explained = np.zeros(len(b), bool)
    for p in path:
        c = (0.5 * (p[:, :3] + p[:, 3:])).astype(np.float32)
        v = (p[:, 3:] - c)[:, :, None] * np.eye(3, dtype=np.float32)
        _, _, near = f.bounds_near(params, c, v, offset)
        explained |= near
    return b[~explained]
