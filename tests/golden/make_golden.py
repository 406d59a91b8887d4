"""Generate the golden vectors in this folder by running the reference's own code.

    python tests/golden/make_golden.py --reference <path of the reference checkout> [--only NAME]

(or set NIQ_REFERENCE to that path).

The reference (nmwsharp/neural-implicit-queries) is pure JAX and JAX is not installed
here, so its ``src/*.py`` modules are imported unchanged over the NumPy stand-in in
``jax_standin.py``.  Inputs are seeded synthetic models (``workloads.he_mlp``) and
seeded boxes/rays/queries; each ``.npz`` written here holds the model parameters, the
inputs and the reference's outputs, so the tests that read them need neither the
reference nor this script.  Only this script reads the reference tree.
"""
from __future__ import annotations

import argparse
import dataclasses
import importlib
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import jax_standin  # noqa: E402

workloads = importlib.import_module('neural-implicit-queries_gb300.workloads')


def flat(prefix, params):
    return {f'{prefix}/{k}': np.asarray(v) for k, v in params.items()}


def rand_boxes(rng, n, v):
    """Boxes for the bound cases: centers in [-1,1]^3, half extents log-uniform in
    [1e-3, 0.5]; v=3 axis-aligned diagonal vecs, v=1 ray segments, v=2 random."""
    center = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    if v == 3:
        half = np.exp(rng.uniform(np.log(1e-3), np.log(0.5), (n, 3))).astype(np.float32)
        vecs = np.zeros((n, 3, 3), np.float32)
        vecs[:, np.arange(3), np.arange(3)] = half
    else:
        vecs = rng.standard_normal((n, v, 3)).astype(np.float32)
        vecs *= (np.exp(rng.uniform(np.log(1e-3), np.log(0.3), (n, v, 1))) /
                 np.linalg.norm(vecs, axis=-1, keepdims=True)).astype(np.float32)
    return center, vecs.astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=os.environ.get('NIQ_REFERENCE'),
                    help='root of the reference checkout (default: $NIQ_REFERENCE)')
    ap.add_argument('--only', default=None,
                    help='write one fixture only: frustum, camera, mc, samples, tree_growing')
    args = ap.parse_args()
    if not args.reference or not os.path.isdir(os.path.join(args.reference, 'src')):
        ap.error('--reference (or NIQ_REFERENCE) must name the reference checkout')
    jax_standin.install()
    sys.path.insert(0, os.path.join(args.reference, 'src'))
    import jax.numpy as jnp
    import affine, mlp, implicit_mlp_utils, slope_interval, queries, kd_tree, extract_cell  # noqa

    tmp = tempfile.mkdtemp()

    def load_as_reference(params, name, mode, **kw):
        path = os.path.join(tmp, name + '.npz')
        np.savez(path, **params)
        return implicit_mlp_utils.generate_implicit_from_file(path, mode=mode, **kw)

    models = {
        'relu16': workloads.he_mlp([3, 16, 16, 1], 'relu', seed=0),
        'elu16': workloads.he_mlp([3, 16, 16, 1], 'elu', seed=1),
        'relu32x3': workloads.plain_small_model(),
    }
    t0 = time.time()
    if args.only == 'frustum':
        frustum_fixture(queries, load_as_reference, models, t0)
        return
    if args.only == 'camera':
        camera_fixture()
        return
    if args.only == 'mc':
        mc_fixture(extract_cell)
        return
    if args.only == 'tree_growing':
        tree_growing_fixture(kd_tree, load_as_reference, models)
        return
    if args.only == 'samples':
        samples_fixture(args.reference, affine, slope_interval, queries, kd_tree, load_as_reference, t0)
        return

    # ---------------------------------------------------------------- point evals + bounds
    mode_kw = {'interval': {}, 'affine_fixed': {}, 'affine_all': {},
               'affine_truncate': {'affine_n_truncate': 8, 'affine_truncate_policy': 'absolute'},
               'affine_append': {'affine_n_append': 4}, 'slope_interval': {}}
    out = {}
    rng = np.random.default_rng(1234)
    for mname, params in models.items():
        out.update(flat(f'model/{mname}', params))
        pts = rng.uniform(-1.2, 1.2, (128, 3)).astype(np.float32)
        f, p = load_as_reference(params, mname, 'affine_fixed')
        out[f'points/{mname}/x'] = pts
        out[f'points/{mname}/f'] = np.asarray(jax_standin._vmap(lambda x: f(p, x))(pts))
        for v in (3, 1, 2):
            center, vecs = rand_boxes(rng, 48, v)
            out[f'boxes/{mname}/v{v}/center'] = center
            out[f'boxes/{mname}/v{v}/vecs'] = vecs
            for mode, kw in mode_kw.items():
                f, p = load_as_reference(params, mname, mode, **kw)
                if mode == 'slope_interval':
                    def bounds_one(c, vv):
                        inp = slope_interval.coordinates_in_general_box(c, vv)
                        o = f.slope_interval_func(p, inp)
                        sl, su = slope_interval.slope_bounds(o)
                        return slope_interval.primal_may_contain_bounds(o, sl, su)
                else:
                    def bounds_one(c, vv):
                        ctx = dataclasses.replace(f.ctx, affine_domain_terms=vv.shape[0])
                        inp = affine.coordinates_in_general_box(ctx, c, vv)
                        o = f.affine_func(p, inp, {'ctx': ctx})
                        return affine.may_contain_bounds(ctx, o)
                lo, hi = jax_standin._vmap(bounds_one)(center, vecs)
                sign = jax_standin._vmap(lambda c, vv: f.classify_general_box(p, c, vv, offset=0.01))(center, vecs)
                out[f'boxes/{mname}/v{v}/{mode}/lower'] = np.asarray(lo)
                out[f'boxes/{mname}/v{v}/{mode}/upper'] = np.asarray(hi)
                out[f'boxes/{mname}/v{v}/{mode}/sign_off0.01'] = np.asarray(sign)
    np.savez_compressed(os.path.join(HERE, 'bounds.npz'), **out)
    print(f'bounds done {time.time() - t0:.1f}s', flush=True)

    # ---------------------------------------------------------------- cast_rays
    out = {}
    params = models['relu32x3']
    out.update(flat('model/relu32x3', params))
    out.update(flat('model/relu16', models['relu16']))
    eye = np.array([0., 0., 3.], np.float32)
    look, up, left = (np.array(v, np.float32) for v in ([0, 0, -1.], [0, 1., 0], [1., 0, 0]))
    roots, dirs = (np.asarray(a) for a in _camera(eye, look, up, 20, 60.))
    out['rays/roots'], out['rays/dirs'] = roots, dirs
    for mode in ('affine_fixed', 'interval', 'slope_interval'):
        f, p = load_as_reference(params, 'relu32x3', mode)
        opts = queries.get_default_cast_opts()
        opts['n_max_step'] = 64
        t, hid, cnt, nev = queries.cast_rays((f,), (p,), jnp.array(roots), jnp.array(dirs), opts)
        out[f'rays/{mode}/t'], out[f'rays/{mode}/hit_id'] = np.asarray(t), np.asarray(hid)
        out[f'rays/{mode}/count'], out[f'rays/{mode}/n_evals'] = np.asarray(cnt), np.asarray(nev)
        print(f'rays {mode} {time.time() - t0:.1f}s', flush=True)
    # two functions, the second one shifted
    f1, p1 = load_as_reference(params, 'relu32x3', 'affine_fixed')
    f2, p2 = load_as_reference(models['relu16'], 'relu16', 'affine_fixed')
    opts = queries.get_default_cast_opts()
    opts['n_max_step'] = 48
    opts['n_substeps'] = 2
    sub = slice(0, roots.shape[0], 3)
    t, hid, cnt, nev = queries.cast_rays((f1, f2), (p1, p2), jnp.array(roots[sub]), jnp.array(dirs[sub]), opts)
    out['rays2/t'], out['rays2/hit_id'], out['rays2/count'] = np.asarray(t), np.asarray(hid), np.asarray(cnt)
    out['rays2/n_evals'] = np.asarray(nev)
    np.savez_compressed(os.path.join(HERE, 'rays.npz'), **out)
    print(f'rays done {time.time() - t0:.1f}s', flush=True)

    # ---------------------------------------------------------------- tree, hmc
    out = {}
    out.update(flat('model/relu32x3', params))
    lower = jnp.array((-1., -1., -1.))
    upper = jnp.array((1., 1., 1.))
    for mode in ('affine_fixed', 'interval'):
        f, p = load_as_reference(params, 'relu32x3', mode)
        d = kd_tree.construct_uniform_unknown_levelset_tree(f, p, lower, upper, split_depth=9,
                                                            with_interior_nodes=True,
                                                            with_exterior_nodes=True, offset=0.)
        for kind in ('unknown', 'interior', 'exterior'):
            valid = np.asarray(d[f'{kind}_node_valid'])
            out[f'tree/{mode}/{kind}/lower'] = np.asarray(d[f'{kind}_node_lower'])[valid]
            out[f'tree/{mode}/{kind}/upper'] = np.asarray(d[f'{kind}_node_upper'])[valid]
    f, p = load_as_reference(params, 'relu32x3', 'affine_fixed')
    d = kd_tree.construct_uniform_unknown_levelset_tree(f, p, lower, upper, node_terminate_thresh=200,
                                                        offset=0.05, batch_process_size=128)
    valid = np.asarray(d['unknown_node_valid'])
    out['tree_thresh/lower'] = np.asarray(d['unknown_node_lower'])[valid]
    out['tree_thresh/upper'] = np.asarray(d['unknown_node_upper'])[valid]
    print(f'tree done {time.time() - t0:.1f}s', flush=True)
    tris = kd_tree.hierarchical_marching_cubes(f, p, lower, upper, 4, n_subcell_depth=1)
    out['hmc/d4s1/tris'] = np.asarray(tris)
    tris = kd_tree.hierarchical_marching_cubes(f, p, lower, upper, 3, n_subcell_depth=0)
    out['hmc/d3s0/tris'] = np.asarray(tris)
    np.savez_compressed(os.path.join(HERE, 'tree.npz'), **out)
    print(f'hmc done {time.time() - t0:.1f}s', flush=True)

    # ---------------------------------------------------------------- intersection, closest point
    out = {}
    # bounded shapes for the pairwise search: small MLPs fitted to spheres
    A = workloads.fit_sdf_mlp([3, 16, 16, 1], workloads.sphere_sdf_fn([0., 0., 0.], 0.35),
                              steps=400, lr=1e-2, seed=3, n_points=4096)
    B = workloads.prepend_spatial_transformation(
        workloads.fit_sdf_mlp([3, 16, 16, 1], workloads.sphere_sdf_fn([0., 0., 0.], 0.3),
                              steps=400, lr=1e-2, seed=4, n_points=4096))
    out.update(flat('model/A', A))
    rot = workloads.random_rotation(np.random.default_rng(5))
    # the shape moves by (R, t): points are mapped by x @ inv(R) + inv(R) @ (-t)
    cases = {'near': (rot, rot @ np.array([0.55, 0.1, 0.0], np.float32)),
             'far': (rot, rot @ np.array([0.8, 0.35, 0.0], np.float32))}
    for name, (R, tr) in cases.items():
        Bp = dict(B)
        Bp['0000.spatial_transformation.R'] = R
        Bp['0000.spatial_transformation.t'] = tr.astype(np.float32)
        out.update(flat(f'model/B_{name}', Bp))
        for mode in ('affine_all', 'affine_fixed'):
            fa, pa = load_as_reference(A, 'A', mode)
            fb, pb = load_as_reference(Bp, 'B' + name, mode)
            found, ia, ib, loc = kd_tree.find_any_intersection((fa, fb), (pa, pb), lower, upper, 0.02)
            out[f'isect/{name}/{mode}/found'] = np.asarray(bool(found))
            out[f'isect/{name}/{mode}/loc'] = np.asarray(loc)
            print(f'isect {name} {mode} found={bool(found)} {time.time() - t0:.1f}s', flush=True)
    f, p = load_as_reference(A, 'A', 'affine_fixed')
    q = np.random.default_rng(77).uniform(-1.2, 1.2, (20, 3)).astype(np.float32)
    out['cp/q'] = q
    for B_ in (8, 2048):
        dist, loc = kd_tree.closest_point(f, p, lower, upper, jnp.array(q), eps=0.05, batch_process_size=B_)
        out[f'cp/B{B_}/dist'] = np.asarray(dist)
        out[f'cp/B{B_}/loc'] = np.asarray(loc)
        print(f'cp B{B_} {time.time() - t0:.1f}s', flush=True)
    np.savez_compressed(os.path.join(HERE, 'queries.npz'), **out)
    print(f'all done {time.time() - t0:.1f}s')


def frustum_fixture(queries, load_as_reference, models, t0):
    """cast_rays_frustum (src/queries.py:178-587) on the 3x32x3 ReLU model: a 12x10 image,
    2x2 initial frusta, 32 steps; affine_fixed alone and with two functions and two
    substeps (the stand-in runs every frustum through Python, so the image is small)."""
    import jax.numpy as jnp
    out = {}
    params = models['relu32x3']
    out.update(flat('model/relu32x3', params))
    out.update(flat('model/relu16', models['relu16']))
    eye = np.array([0., 0., 3.], np.float32)
    look, up, left = (np.array(v, np.float32) for v in ([0, 0, -1.], [0, 1., 0], [-1., 0, 0]))
    for name, fs, n_sub in (('one', ('relu32x3',), 1), ('two', ('relu32x3', 'relu16'), 2)):
        funcs, ps = [], []
        for m in fs:
            f, p = load_as_reference(models[m], m, 'affine_fixed')
            funcs.append(f)
            ps.append(p)
        opts = queries.get_default_cast_opts()
        opts['n_max_step'] = 32
        opts['n_side_init'] = 2
        opts['n_substeps'] = n_sub
        cam = (jnp.array(eye), jnp.array(look), jnp.array(up), jnp.array(left), 40., 30., 12, 10)
        t, hid, cnt, nev = queries.cast_rays_frustum(tuple(funcs), tuple(ps), cam, opts)
        out[f'frustum/{name}/t'], out[f'frustum/{name}/hit_id'] = np.asarray(t), np.asarray(hid)
        out[f'frustum/{name}/count'] = np.asarray(cnt)
        print(f'frustum {name} {time.time() - t0:.1f}s', flush=True)
    out['frustum/cam'] = np.concatenate([eye, look, up, left, [40., 30., 12, 10]]).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, 'frustum.npz'), **out)


def tree_growing_fixture(kd_tree, load_as_reference, models):
    """construct_uniform_unknown_levelset_tree (src/kd_tree.py:19-218) in the growing-term
    modes on the 3x32x3 ReLU model, 8 bisections: affine_truncate with 8 and 64 terms,
    affine_append with 4, affine_all; and closest_point in affine_truncate (8 and 64
    terms) on the fitted sphere model of queries.npz."""
    import jax.numpy as jnp
    out = {}
    params = models['relu32x3']
    out.update(flat('model/relu32x3', params))
    lower, upper = jnp.array((-1., -1., -1.)), jnp.array((1., 1., 1.))
    cases = {'truncate8': ('affine_truncate', {'affine_n_truncate': 8, 'affine_truncate_policy': 'absolute'}),
             'truncate64': ('affine_truncate', {'affine_n_truncate': 64, 'affine_truncate_policy': 'absolute'}),
             'append4': ('affine_append', {'affine_n_append': 4}),
             'all': ('affine_all', {})}
    for name, (mode, kw) in cases.items():
        f, p = load_as_reference(params, 'relu32x3', mode, **kw)
        d = kd_tree.construct_uniform_unknown_levelset_tree(f, p, lower, upper, split_depth=8,
                                                            with_interior_nodes=True, with_exterior_nodes=True)
        for kind in ('unknown', 'interior', 'exterior'):
            valid = np.asarray(d[f'{kind}_node_valid'])
            out[f'tree/{name}/{kind}/lower'] = np.asarray(d[f'{kind}_node_lower'])[valid]
            out[f'tree/{name}/{kind}/upper'] = np.asarray(d[f'{kind}_node_upper'])[valid]
        print(f'tree {name}', flush=True)
    gq = dict(np.load(os.path.join(HERE, 'queries.npz')))
    A = {k[len('model/A/'):]: v for k, v in gq.items() if k.startswith('model/A/')}
    out.update(flat('model/A', A))
    q = gq['cp/q']
    out['cp/q'] = q
    for name in ('truncate8', 'truncate64'):
        mode, kw = cases[name]
        f, p = load_as_reference(A, 'A', mode, **kw)
        for B_ in (8, 2048):
            dist, loc = kd_tree.closest_point(f, p, lower, upper, jnp.array(q), eps=0.05, batch_process_size=B_)
            out[f'cp/{name}/B{B_}/dist'] = np.asarray(dist)
            out[f'cp/{name}/B{B_}/loc'] = np.asarray(loc)
            print(f'cp {name} B{B_}', flush=True)
    np.savez_compressed(os.path.join(HERE, 'tree_growing.npz'), **out)


def camera_fixture():
    """render.generate_camera_rays and render.look_at (src/render.py:17-50,229-242): the
    default plain-method camera (eye at distance 3 on +z, 60 degree field of view) at
    three resolutions, and look_at for a few eyes and both up axes."""
    import render
    import jax.numpy as jnp
    out = {}
    eyes = np.array([[0., 0., 3.], [1.5, 2., -2.1], [-2.5, 0.3, 1.2], [0.2, -3., 0.4]], np.float32)
    out['look_at/eyes'] = eyes
    for up in ('y', 'z'):
        res = [tuple(np.asarray(x) for x in render.look_at(jnp.array(e), up_dir=up)) for e in eyes]
        for j, name in enumerate(('look', 'up', 'left')):
            out[f'look_at/{up}/{name}'] = np.stack([r[j] for r in res]).astype(np.float32)
    look, up, _ = (np.asarray(x) for x in render.look_at(jnp.array(eyes[0])))
    for res_, fov in ((5, 60.), (33, 60.), (128, 60.), (16, 35.)):
        e = eyes[0] if fov == 60. else eyes[1]
        lk, u, _ = (np.asarray(x) for x in render.look_at(jnp.array(e)))
        roots, dirs = render.generate_camera_rays(jnp.array(e), jnp.array(lk), jnp.array(u), res=res_, fov_deg=fov)
        out[f'cam/{res_}/eye'], out[f'cam/{res_}/look'], out[f'cam/{res_}/up'] = e, lk, u
        out[f'cam/{res_}/fov'] = np.float32(fov)
        out[f'cam/{res_}/roots'], out[f'cam/{res_}/dirs'] = np.asarray(roots), np.asarray(dirs)
    np.savez_compressed(os.path.join(HERE, 'camera.npz'), **out)
    print('camera done', flush=True)


def mc_fixture(extract_cell):
    """Per-case digests of the reference's marching-cubes table (src/extract_cell.py:12-268)
    in the triangulation-independent canonical form of mc_canon.py: the tests pin this
    project's generated table against them without the table itself being committed."""
    import mc_canon
    from oracle import mc_table
    ref = np.asarray(extract_cell.MC_TRI_TABLE_RAW)
    out = {'mc/digest': mc_canon.case_digests(ref, mc_table.VERT, mc_table.EDGE)}
    np.savez_compressed(os.path.join(HERE, 'mc_digest.npz'), **out)
    print('mc digests done', flush=True)


SAMPLE_MODELS = ('fox', 'hammer', 'bunny', 'birdcage_occ')


def samples_fixture(reference, affine, slope_interval, queries, kd_tree, load_as_reference, t0):
    """The reference's own sample models (sample_inputs/*.npz: ReLU 3->32x8, ReLU 3->64x8,
    ELU 3->64x8, ReLU 3->64x8): their parameters go to sample_models.npz, the reference's
    outputs on them to samples.npz -- point values, box bounds in four modes, the
    level-set tree (12 bisections) and a small ray cast."""
    import jax.numpy as jnp
    params_out, out = {}, {}
    rng = np.random.default_rng(4321)
    mode_kw = {'interval': {}, 'affine_fixed': {}, 'slope_interval': {},
               'affine_truncate': {'affine_n_truncate': 8, 'affine_truncate_policy': 'absolute'}}
    eye = np.array([0., 0., 3.], np.float32)
    import render
    look, up, _ = (np.asarray(x) for x in render.look_at(jnp.array(eye)))
    roots, dirs = (np.asarray(a) for a in render.generate_camera_rays(jnp.array(eye), jnp.array(look),
                                                                        jnp.array(up), res=12, fov_deg=60.))
    out['rays/roots'], out['rays/dirs'] = roots, dirs
    lower, upper = jnp.array((-1., -1., -1.)), jnp.array((1., 1., 1.))
    for name in SAMPLE_MODELS:
        src = dict(np.load(os.path.join(reference, 'sample_inputs', name + '.npz')))
        params_out.update(flat(f'model/{name}', src))
        pts = rng.uniform(-1.1, 1.1, (64, 3)).astype(np.float32)
        f, p = load_as_reference(src, name, 'affine_fixed')
        out[f'{name}/points/x'] = pts
        out[f'{name}/points/f'] = np.asarray(jax_standin._vmap(lambda x: f(p, x))(pts))
        center, vecs = rand_boxes(rng, 32, 3)
        out[f'{name}/boxes/center'], out[f'{name}/boxes/vecs'] = center, vecs
        for mode, kw in mode_kw.items():
            f, p = load_as_reference(src, name, mode, **kw)
            if mode == 'slope_interval':
                def bounds_one(c, vv):
                    inp = slope_interval.coordinates_in_general_box(c, vv)
                    o = f.slope_interval_func(p, inp)
                    sl, su = slope_interval.slope_bounds(o)
                    return slope_interval.primal_may_contain_bounds(o, sl, su)
            else:
                def bounds_one(c, vv):
                    ctx = dataclasses.replace(f.ctx, affine_domain_terms=vv.shape[0])
                    inp = affine.coordinates_in_general_box(ctx, c, vv)
                    o = f.affine_func(p, inp, {'ctx': ctx})
                    return affine.may_contain_bounds(ctx, o)
            lo, hi = jax_standin._vmap(bounds_one)(center, vecs)
            out[f'{name}/boxes/{mode}/lower'], out[f'{name}/boxes/{mode}/upper'] = np.asarray(lo), np.asarray(hi)
        print(f'{name} bounds {time.time() - t0:.1f}s', flush=True)
        f, p = load_as_reference(src, name, 'affine_fixed')
        d = kd_tree.construct_uniform_unknown_levelset_tree(f, p, lower, upper, split_depth=12,
                                                            with_interior_nodes=True,
                                                            with_exterior_nodes=True, offset=0.)
        for kind in ('unknown', 'interior', 'exterior'):
            valid = np.asarray(d[f'{kind}_node_valid'])
            out[f'{name}/tree/{kind}/lower'] = np.asarray(d[f'{kind}_node_lower'])[valid]
            out[f'{name}/tree/{kind}/upper'] = np.asarray(d[f'{kind}_node_upper'])[valid]
        print(f'{name} tree {time.time() - t0:.1f}s', flush=True)
        opts = queries.get_default_cast_opts()
        opts['n_max_step'] = 48
        t, hid, cnt, nev = queries.cast_rays((f,), (p,), jnp.array(roots), jnp.array(dirs), opts)
        out[f'{name}/rays/t'], out[f'{name}/rays/hit_id'] = np.asarray(t), np.asarray(hid)
        out[f'{name}/rays/count'] = np.asarray(cnt)
        print(f'{name} rays {time.time() - t0:.1f}s', flush=True)
    np.savez_compressed(os.path.join(HERE, 'sample_models.npz'), **params_out)
    np.savez_compressed(os.path.join(HERE, 'samples.npz'), **out)


def _camera(eye, look, up, res, fov):
    import render  # the reference's module (imported over the stand-in)
    return render.generate_camera_rays(eye, look, up, res=res, fov_deg=fov)


if __name__ == '__main__':
    main()
