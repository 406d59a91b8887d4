"""Camera rays (src/render.py:17-50, 229-242).

Rays are generated on the host in float32 with the reference's formulas; the cast itself
runs on the GPU (queries.cast_rays).  Window, matcap and GUI paths of the reference are
not part of this package.
"""
import numpy as np

from . import geometry


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
