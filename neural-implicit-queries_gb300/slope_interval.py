"""Slope-interval ImplicitFunction (src/slope_interval.py) on the GPU."""
from __future__ import annotations

from ._gpu_function import GPUImplicitFunction


class SlopeIntervalImplicitFunction(GPUImplicitFunction):
    """src/slope_interval.py:16-51.  The reference's ``min_distance_to_zero*`` methods
    (src/slope_interval.py:53-158) have no caller in the reference's queries and are not
    provided."""

    def __init__(self, slope_interval_func=None, conservative=True):
        super().__init__("classify-and-distance", 'slope_interval', conservative=conservative)
