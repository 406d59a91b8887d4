"""Regenerate the fitted model files in this folder (run once, results committed).

    python neural-implicit-queries_gb300/data/make_models.py

``spheres12_relu64x4.npz``: a 3->64x4->1 ReLU MLP fitted by 2000 full-batch Adam steps
(lr 1e-3, seed 1) to the signed distance of a union of 12 spheres (centers
U[-0.6,0.6]^3, radii U[0.1,0.3]) sampled at 2^18 uniform points in [-1,1]^3.
"""
import importlib
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
wl = importlib.import_module('neural-implicit-queries_gb300.workloads')

if __name__ == '__main__':
    t0 = time.time()
    centers, radii = wl.spheres_scene(seed=1)
    params = wl.fit_sdf_mlp([3, 64, 64, 64, 64, 1], lambda x: wl.spheres_sdf(x, centers, radii),
                            steps=2000, lr=1e-3, seed=1, n_points=2 ** 18, log_every=200)
    np.savez(wl.SPHERES_NPZ, **params)
    print(f"wrote {wl.SPHERES_NPZ} in {time.time() - t0:.0f}s")
