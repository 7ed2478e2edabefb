"""Host-side helpers of the post-processing API (no device work)."""
from __future__ import annotations

import numpy as np


def xy_extent(kind: str, width: float, depth: float, tilt: float = 0.0):
    """x_min, x_max, y_min, y_max of a scan geometry, in FP32 as
    SectorScanGeometry / LinearScanGeometry::get_xy_extent compute them
    (src/utils/ScanGeometry.hpp:49-77)."""
    f = np.float32
    if kind == "sector":
        pi = f(4.0 * float(np.arctan(f(1.0))))
        min_angle = f(f(f(0.5) * pi) - f(f(0.5) * f(width))) + f(tilt)
        max_angle = f(f(f(0.5) * pi) + f(f(0.5) * f(width))) + f(tilt)
        return (f(f(depth) * np.cos(f(max_angle))), f(f(depth) * np.cos(f(min_angle))), f(0.0), f(depth))
    return (f(-0.5) * f(width), f(0.5) * f(width), f(0.0), f(depth))


def image_size(kind: str, width: float, depth: float, dots_per_meter: float, tilt: float = 0.0):
    x0, x1, y0, y1 = xy_extent(kind, width, depth, tilt)
    w, h = np.float32(x1 - x0), np.float32(y1 - y0)
    dpm = np.float32(dots_per_meter)
    return int(np.float32(w * dpm)), int(np.float32(h * dpm))
