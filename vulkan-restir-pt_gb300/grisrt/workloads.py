"""Seeded workload definitions shared by the benchmark and the tests.

batched_views: many independent views of uneven size and path length, each with its own
box-or-terrain scene of 10k-200k triangles (resolution drawn from {64,128,256,512}^2, max depth
uniform in [2, 10]); the batch renders them all with one launch per pass.
"""
import math

import numpy as np

RESOLUTIONS = (64, 128, 256, 512)


def batched_views(n=64, seed=7, min_tris=10_000, max_tris=200_000, resolutions=RESOLUTIONS, depths=(2, 10)):
    """Returns a list of dicts {kind, grid, spheres, seed, width, height, maxDepth, target_tris}.

    kind 3 (box room + icospheres) or kind 1 (fBm terrain + icospheres) with equal odds; the
    triangle target is log-uniform in [min_tris, max_tris]; a terrain spends ~60% of it on the
    heightfield (2 (grid-1)^2 triangles) and the rest on 320-triangle icospheres."""
    rng = np.random.default_rng(seed)
    views = []
    for i in range(n):
        res = int(resolutions[int(rng.integers(0, len(resolutions)))])
        target = math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))
        box = bool(rng.uniform() < 0.5)
        depth = int(rng.integers(depths[0], depths[1] + 1))
        if box:
            kind, grid, spheres = 3, 0, max(1, int(round((target - 36) / 320.0)))
        else:
            kind = 1
            grid = int(math.sqrt(0.6 * target / 2.0)) + 1
            spheres = max(1, int(round(0.4 * target / 320.0)))
        views.append(dict(kind=kind, grid=grid, spheres=spheres, seed=seed * 1000 + i, width=res, height=res,
                          maxDepth=depth, target_tris=int(target)))
    return views
