"""Batches of views for ne_views: cameras orbiting a scene with seeded resolutions.

The multi-view configuration: 64 views, resolutions drawn uniformly from {64, 128, 256,
512}^2 with a fixed seed, 16 samples per pixel, cameras on a ring around the scene looking
at its centre.
"""
from __future__ import annotations

import numpy as np

SIZES = (64, 128, 256, 512)


def orbit_views(n: int = 64, seed: int = 0x4E415256, spp: int = 16, center=(0.0, 1.0, 0.0), radius: float = 4.5,
                height: float = 1.8, vfov: float = 45.0, sizes=SIZES, camera_look_at=None):
    """[(camera, width, height, spp)] for n cameras evenly spaced on a ring. `camera_look_at`
    (position, look_at, vfov, width, height) -> ne_camera defaults to the library's."""
    if camera_look_at is None:
        from . import camera_look_at
    rng = np.random.default_rng(seed)
    picks = rng.integers(0, len(sizes), size=n)
    views = []
    for i in range(n):
        a = 2.0 * np.pi * i / n
        pos = [center[0] + radius * np.sin(a), height, center[2] - radius * np.cos(a)]
        s = int(sizes[picks[i]])
        views.append((camera_look_at(pos, center, vfov, s, s), s, s, spp))
    return views
