"""The threaded oracle (cpv_oracle_render_threaded) against the
single-threaded one (no GPU).

The threaded form exists so that the GPU can be checked at the workloads'
full sizes; it must give the same image bit for bit and the same counts on
every kind of scene: depth and stencil, blending (where per-pixel order
matters), points and lines, instancing, many draws, and thread counts that
do and do not divide the image height.
"""
import numpy as np
import pytest

import cpvulkan_gb300 as c

SCENES = [
    (c.CUBE, 1, [30]),
    (c.HEIGHTFIELD, 1, [96, 320, 200]),
    (c.BLEND, 3, [1500, 320, 200]),
    (c.BATCH, 4, [40, 3000, 320, 200]),
    (c.SERVE, 5, [256, 5000, 3]),
    (c.PROGRAM, 2, [c.PROGRAM_CUBE, 0x18 | 0x100, 64, 48, 24]),
    (c.PROGRAM, 2, [c.PROGRAM_POINTS, 0x10000 | 0x20 | 0x8, 64, 48, 24]),
    (c.PROGRAM, 3, [c.PROGRAM_CUBE, 0x10000 | 0x800 | 0x20 | 0x20000, 64, 48, 24]),
    (c.PROGRAM, 1, [c.PROGRAM_TEXLIT, 0x10 | 0x8000 | 0x20, 64, 48, 24]),
    (c.PROGRAM, 2, [c.PROGRAM_FETCH, 0x20, 64, 48, 24, 9]),
    (c.PROGRAM, 2, [c.PROGRAM_CUBE, 0x10, 64, 48, 24, 92]),
]


@pytest.mark.parametrize("config,seed,params", SCENES)
@pytest.mark.parametrize("threads", [1, 3, 8])
def test_threaded_equals_single(oracle, config, seed, params, threads):
    scene = c.Scene(config, seed, params)
    color, depth, stats = oracle.render(scene)
    tcolor, tdepth, tstats = oracle.render_threaded(scene, threads)
    assert np.array_equal(color, tcolor)
    if depth is not None:
        assert np.array_equal(depth, tdepth)
    assert stats == tstats
    assert stats["fragments"] > 0
