"""kd_tree.sample_surface and kd_tree.bulk_properties on the GPU.

The reference draws its candidates from JAX's threefry generator and the kernels from a
counter-based generator of their own, so samples are compared by their properties and
the Monte Carlo estimates statistically: every sample lies in the tree's unknown nodes
and within the width of the surface; mass and centroid agree with the oracle's estimate
(NumPy generator, same tree) within five standard errors, and the mass with the interior
volume plus the boundary volume as bounds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _func(niq, params):
    return niq.implicit_mlp_utils.generate_implicit_from_params(params, 'affine_fixed', conservative=False)[0]


def test_sample_surface(niq, R, gpu_ready):
    params = niq.workloads.spheres_sdf_model()
    f = _func(niq, params)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    width = 0.02
    pts = niq.kd_tree.sample_surface(f, params, lo, hi, 20000, width, np.array([0, 7], np.uint32), n_node_thresh=4096)
    assert pts.shape == (20000, 3) and np.all(np.isfinite(pts))
    vals = R.eval_points(params, pts)
    assert np.all(np.abs(vals) < width * (1 + 1e-4) + 1e-6)
    # inside the oracle tree's unknown nodes (same construction: offset = width)
    ref, (nlo, nhi) = R.sample_surface(R.generate_implicit(params, 'affine_fixed'), params, lo, hi, 1000, width,
                                       np.random.default_rng(0), n_node_thresh=4096)
    inside = np.zeros(pts.shape[0], bool)
    for s in range(0, nlo.shape[0], 512):
        a, b = nlo[s:s + 512], nhi[s:s + 512]
        inside |= np.any(np.all((pts[:, None] >= a[None]) & (pts[:, None] <= b[None]), -1), 1)
    assert inside.all()
    # another seed gives other points
    pts2 = niq.kd_tree.sample_surface(f, params, lo, hi, 20000, width, np.array([0, 8], np.uint32))
    assert not np.array_equal(pts, pts2)


def test_bulk_properties(niq, R, gpu_ready):
    params = niq.workloads.spheres_sdf_model()
    f = _func(niq, params)
    lo, hi = -np.ones(3, np.float32), np.ones(3, np.float32)
    n = 1000000
    mass, cen = niq.kd_tree.bulk_properties(f, params, lo, hi, np.array([0, 3], np.uint32), n_expand=10000,
                                            n_sample=n)
    rm, rc = R.bulk_properties(R.generate_implicit(params, 'affine_fixed'), params, lo, hi,
                               np.random.default_rng(1), n_expand=10000, n_sample=n)
    # standard error of the boundary estimate: boundary volume * sqrt(p (1 - p) / n)
    d = R.construct_uniform_unknown_levelset_tree(R.generate_implicit(params, 'affine_fixed'), params, lo, hi,
                                                  node_terminate_thresh=10000, with_interior_nodes=True)
    vb = np.prod((d['unknown_node_upper'] - d['unknown_node_lower']).astype(np.float64), -1).sum()
    vi = np.prod((d['interior_node_upper'] - d['interior_node_lower']).astype(np.float64), -1).sum()
    p = (rm - vi) / vb
    se = vb * np.sqrt(max(p * (1 - p), 1e-12) / n)
    assert abs(mass - rm) <= 5 * np.sqrt(2) * se + 1e-9, (mass, rm, se)
    assert vi <= mass <= vi + vb
    # seed-to-seed spread of the oracle's own centroid estimate is about 2e-3 per axis
    assert np.max(np.abs(cen - rc)) <= 1e-2, (cen, rc)
