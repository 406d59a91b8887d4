"""Camera rays, normals, shading and whole images (src/render.py).

Rays are generated on the host in float32 with the reference's formulas; the cast,
the finite-difference normals and the shading run on the GPU and the image stays a
device buffer until it is returned.  The reference's window and GUI paths are not part
of this package; matcaps are passed as arrays (``load_matcap`` reads the reference's
PNG files when imageio is installed).
"""
import numpy as np

from . import _io, _lib, geometry


def _linspace(start, stop, num):
    # jnp.linspace for floats: start*(1-s) + stop*s, s = i/(num-1)
    s = (np.arange(num, dtype=np.float32) / np.float32(num - 1)).astype(np.float32)
    return (np.float32(start) * (1 - s) + np.float32(stop) * s).astype(np.float32)


def camera_ray(look_dir, up_dir, left_dir, fov_deg_x, fov_deg_y, theta_x, theta_y):
    """src/render.py:17-24."""
    tx = np.float32(np.tan(np.float32(np.deg2rad(np.float32(fov_deg_x))) / 2))
    ty = np.float32(np.tan(np.float32(np.deg2rad(np.float32(fov_deg_y))) / 2))
    p = look_dir + left_dir * (theta_x * tx) + up_dir * (theta_y * ty)
    return geometry.normalize(p).astype(np.float32)


def generate_camera_rays(eye_pos, look_dir, up_dir, res=1024, fov_deg=30.):
    """src/render.py:26-50: (roots, dirs), each (res*res, 3) float32, x fastest."""
    eye_pos = np.asarray(eye_pos, np.float32)
    look_dir = np.asarray(look_dir, np.float32)
    up_dir = np.asarray(up_dir, np.float32)
    ax = _linspace(-1., 1., res)
    cx, cy = np.meshgrid(ax, ax)
    cx, cy = cx.reshape(-1), cy.reshape(-1)
    up_dir = (up_dir - np.dot(look_dir, up_dir) * look_dir).astype(np.float32)
    up_dir = geometry.normalize(up_dir).astype(np.float32)
    left_dir = np.cross(look_dir, up_dir).astype(np.float32)
    t = np.float32(np.tan(np.float32(np.deg2rad(np.float32(fov_deg))) / 2))
    p = look_dir[None] + left_dir[None] * (cx * t)[:, None] + up_dir[None] * (cy * t)[:, None]
    dirs = geometry.normalize(p.astype(np.float32)).astype(np.float32)
    roots = np.tile(eye_pos, (dirs.shape[0], 1))
    return roots, dirs


def look_at(eye_pos, target=None, up_dir='y'):
    """src/render.py:229-242."""
    eye_pos = np.asarray(eye_pos, np.float32)
    target = np.zeros(3, np.float32) if target is None else np.asarray(target, np.float32)
    up = np.array((0., 1., 0.) if up_dir == 'y' else (0., 0., 1.), np.float32)
    look_dir = geometry.normalize(target - eye_pos).astype(np.float32)
    up = geometry.orthogonal_dir(up, look_dir).astype(np.float32)
    left_dir = np.cross(look_dir, up).astype(np.float32)
    return look_dir, up, left_dir


def outward_normals(funcs_tuple, params_tuple, hit_pos, hit_ids, eps, method='finite_differences'):
    """src/render.py:53-90: (N, 3) unit normals of the function each point hit (hit id
    1-based; zeros where none).  'finite_differences': tetrahedron central differences;
    'autodiff': the normalised exact gradient (forward-mode derivatives on the device, the
    jax.jacfwd of the reference).  Device tensors in give device tensors out."""
    if method not in ('finite_differences', 'autodiff'):
        raise ValueError("unrecognized method")
    if not isinstance(funcs_tuple, (tuple, list)):
        funcs_tuple, params_tuple = (funcs_tuple,), (params_tuple,)
    t = _io.require_cuda()
    from .mlp import device_model
    models = [device_model(p) for p in params_tuple]
    pos, kind = _io.to_dev(hit_pos)
    pos = pos.reshape(-1, 3)
    hid, _ = _io.to_dev(hit_ids, dtype='int32')
    n = pos.shape[0]
    out = t.empty((n, 3), dtype=t.float32, device='cuda')
    L = _lib.load()
    handles = (_lib.C.c_void_p * len(models))(*[m.handle.value for m in models])
    if method == 'autodiff':
        ws_bytes = L.niq_outward_normals_autodiff_workspace_size(n)
        ws = _io.workspace(ws_bytes)
        _lib.check(L.niq_outward_normals_autodiff(handles, len(models), n, _io.ptr(pos), _io.ptr(hid.reshape(-1)),
                                                  _io.ptr(out), _io.ptr(ws), ws_bytes, _io.stream_handle()))
        return _io.back(out, kind)
    ws_bytes = L.niq_outward_normals_workspace_size(n)
    ws = _io.workspace(ws_bytes)
    _lib.check(L.niq_outward_normals(handles, len(models), n, _io.ptr(pos), _io.ptr(hid.reshape(-1)), float(eps),
                                     _io.ptr(out), _io.ptr(ws), ws_bytes, _io.stream_handle()))
    return _io.back(out, kind)


def _shading_colors(fn, hit_pos, hit_ids, n):
    """(n, 3) float32 colors of ``fn`` at the hit positions (white where nothing was hit,
    which the shading replaces by the background)."""
    pos = np.asarray(_io.to_numpy(hit_pos), np.float32).reshape(-1, 3)
    hit = np.asarray(_io.to_numpy(hit_ids)).reshape(-1) > 0
    out = np.ones((n, 3), np.float32)
    if not hit.any():
        return out
    sel = pos[hit]
    try:
        cols = np.asarray(fn(sel), np.float32)
        if cols.shape != (sel.shape[0], 3):
            raise ValueError
    except Exception:
        cols = np.stack([np.asarray(fn(p), np.float32).reshape(3) for p in sel])
    out[hit] = cols
    return out


def shade_image(shading, ray_dirs, hit_pos, hit_normals, hit_ids, up_dir, matcaps, shading_color_tuple,
                shading_color_func=None, tonemap=False):
    """src/render.py:161-224 (plus the white background of :139 and, optionally,
    tonemap_image): (N, 3) colors.  ``matcaps`` is the (r, g, b, k) tuple of (H, W, 3)
    images.  ``shading_color_func`` (a callable of a hit position, as the reference
    vmaps it) gives each hit pixel its color in place of ``shading_color_tuple``: it runs
    on the host over the hit positions (once on the whole (N, 3) array if it accepts one,
    else per position) and the colors go to the device with the matcap shading."""
    t = _io.require_cuda()
    dirs, kind = _io.to_dev(ray_dirs)
    nrm, _ = _io.to_dev(hit_normals)
    hid, _ = _io.to_dev(hit_ids, dtype='int32')
    n = dirs.reshape(-1, 3).shape[0]
    out = t.empty((n, 3), dtype=t.float32, device='cuda')
    L = _lib.load()
    up = (_lib.C.c_float * 3)(*np.asarray(up_dir, np.float32).reshape(3).tolist())
    if shading == 'normal':
        code, mc, mh, mw = 0, None, 1, 1
        cols = (_lib.C.c_float * 3)(1., 1., 1.)
        ncol = 1
    elif shading == 'matcap_color':
        if matcaps is None or len(matcaps) != 4:
            raise ValueError("matcap_color shading needs the (r, g, b, k) matcap images")
        stack = np.stack([np.asarray(m, np.float32)[..., :3] for m in matcaps])
        mc = t.from_numpy(np.ascontiguousarray(stack)).cuda()
        code, mh, mw = 1, stack.shape[1], stack.shape[2]
        ct = shading_color_tuple
        if not isinstance(ct[0], (tuple, list, np.ndarray)):
            ct = (ct,)
        colf = np.asarray(ct, np.float32).reshape(-1, 3)
        cols = (_lib.C.c_float * colf.size)(*colf.reshape(-1).tolist())
        ncol = colf.shape[0]
    else:
        raise RuntimeError("Unrecognized shading parameter")
    if shading_color_func is not None and code == 1:
        pix = t.from_numpy(_shading_colors(shading_color_func, hit_pos, hit_ids, n)).cuda()
        _lib.check(L.niq_shade_image_pixel_colors(n, _io.ptr(dirs.reshape(-1, 3)), _io.ptr(nrm.reshape(-1, 3)),
                                                  _io.ptr(hid.reshape(-1)), up, _io.ptr(mc), mh, mw, _io.ptr(pix),
                                                  1 if tonemap else 0, _io.ptr(out), _io.stream_handle()))
        return _io.back(out, kind)
    _lib.check(L.niq_shade_image(code, n, _io.ptr(dirs.reshape(-1, 3)), _io.ptr(nrm.reshape(-1, 3)),
                                 _io.ptr(hid.reshape(-1)), up, _io.ptr(mc) if mc is not None else None, mh, mw, cols,
                                 ncol, 1 if tonemap else 0, _io.ptr(out), _io.stream_handle()))
    return _io.back(out, kind)


def render_image(funcs_tuple, params_tuple, eye_pos, look_dir, up_dir, left_dir, res, fov_deg, frustum, opts,
                 shading="normal", shading_color_tuple=((0.157, 0.613, 1.000)), matcaps=None, tonemap=False,
                 shading_color_func=None):
    """src/render.py:94-150: ``(img (res, res, 3), depth (res, res), counts, hit_ids,
    n_eval, -1)``, the cast by queries.cast_rays or queries.cast_rays_frustum, then normals
    and shading on the device."""
    from . import queries
    if isinstance(funcs_tuple, list):
        funcs_tuple = tuple(funcs_tuple)
    if isinstance(params_tuple, list):
        params_tuple = tuple(params_tuple)
    if not isinstance(funcs_tuple, tuple):
        funcs_tuple = (funcs_tuple,)
    if not isinstance(params_tuple, tuple):
        params_tuple = (params_tuple,)
    if not isinstance(shading_color_tuple[0], (tuple, list)):
        shading_color_tuple = (shading_color_tuple,)
    if len(params_tuple) != len(funcs_tuple) or (shading == 'matcap_color' and
                                                 len(shading_color_tuple) != len(funcs_tuple)):
        raise ValueError("render_image tuple arguments should all be same length")
    t = _io.require_cuda()
    roots, dirs = generate_camera_rays(eye_pos, look_dir, up_dir, res=res, fov_deg=fov_deg)
    if frustum:
        cam = (eye_pos, look_dir, up_dir, left_dir, fov_deg, fov_deg, res, res)
        tt, hit, cnt, n_eval = queries.cast_rays_frustum(funcs_tuple, params_tuple, cam, opts)
        # the reference transposes the [x, y] outputs to the ray order
        tt, hit, cnt = tt.T.reshape(-1), hit.T.reshape(-1), cnt.T.reshape(-1)
        tt, hit, cnt = (t.from_numpy(np.ascontiguousarray(a)).cuda() for a in (tt, hit, cnt))
    else:
        tt, hit, cnt, nev = queries.cast_rays(funcs_tuple, params_tuple, roots, dirs, opts, return_device=True)
        n_eval = int(nev[0].item())
    rt = t.from_numpy(roots).cuda()
    dt = t.from_numpy(dirs).cuda()
    hit_pos = rt + tt[:, None] * dt
    normals = outward_normals(funcs_tuple, params_tuple, hit_pos, hit, opts['hit_eps'])
    img = shade_image(shading, dt, hit_pos, normals, hit, up_dir, matcaps, shading_color_tuple,
                      shading_color_func=shading_color_func, tonemap=tonemap)
    img = img.reshape(res, res, 3).cpu().numpy()
    return (img, tt.reshape(res, res).cpu().numpy(), cnt.reshape(res, res).cpu().numpy(),
            hit.reshape(res, res).cpu().numpy(), n_eval, -1)


def load_matcap(fname_pattern):
    """src/render.py:245-254: the r, g, b, k images of a matcap, scaled by 1/256."""
    try:
        import imageio
    except ImportError as e:
        raise ImportError("load_matcap reads PNG files with imageio, which is not installed; "
                          "pass the four images as arrays instead") from e
    return tuple(np.asarray(imageio.imread(fname_pattern.format(c)), np.float32) / 256. for c in 'rgbk')
