"""GB300-native range-analysis query engine for neural implicit surfaces.

Drop-in for the range-analysis path of nmwsharp/neural-implicit-queries: the reference's
dict MLP spec, ImplicitFunction modes and query signatures, computed by sm_103a CUDA
kernels behind the C ABI in include/niq.h (libniq.so).  Modules keep the reference's
names: ``mlp``, ``implicit_function``, ``affine``, ``slope_interval``, ``sdf``,
``implicit_mlp_utils``, ``queries``, ``kd_tree``, ``extract_cell``, ``render``,
``geometry``; plus ``batched`` (many models in one launch) and ``serve`` (the request
loop).  Submodules load lazily; nothing touches the GPU until a query runs.
"""
import importlib

__all__ = ['mlp', 'implicit_function', 'affine', 'slope_interval', 'sdf', 'implicit_mlp_utils',
           'queries', 'kd_tree', 'extract_cell', 'render', 'geometry', 'batched', 'serve',
           'workloads', 'autotune']


def __getattr__(name):
    if name in __all__:
        return importlib.import_module(f'.{name}', __name__)
    raise AttributeError(name)
