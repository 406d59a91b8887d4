"""Small vector helpers (src/geometry.py:6-19)."""
import numpy as np


def norm(x):
    return np.linalg.norm(x, axis=-1)


def norm2(x):
    return np.inner(x, x)


def normalize(x):
    return x / norm(x)[..., None] if np.ndim(x) > 1 else x / norm(x)


def orthogonal_dir(x, remove_dir):
    remove_dir = normalize(remove_dir)
    x = x - np.dot(x, remove_dir) * remove_dir
    return normalize(x)


def dot(x, y):
    return np.sum(x * y, axis=-1)
