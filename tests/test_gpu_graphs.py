"""Command buffers replayed as CUDA graphs: the first submission on a queue
runs eagerly, the second is captured, later ones replay the graph. Every
frame must be bit-identical to the eager one, and to the oracle."""
import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import compare

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("config,params", [(c.CUBE, [45]), (c.HEIGHTFIELD, [96, 320, 200]), (c.BLEND, [500, 320, 200]),
                                           (c.PROGRAM, [c.PROGRAM_TEXLIT, 0x10 | 0x4000, 64, 48, 24]),
                                           (c.PROGRAM, [c.PROGRAM_CUBE, 0x18 | 0x100, 64, 48, 24])])
def test_graph_replay_is_bit_identical(gpu_ctx, oracle, config, params):
    scene = c.Scene(config, 4, params)
    r = c.Renderer(gpu_ctx, scene)
    try:
        frames = []
        for _ in range(4):  # eager, capture, replay, replay
            r.render(1)
            frames.append(r.readback())
    finally:
        r.close()
    for col, dep in frames[1:]:
        assert np.array_equal(col, frames[0][0])
        if dep is not None:
            assert np.array_equal(dep, frames[0][1])
    ocol, odep, _ = oracle.render(scene)
    report = compare(scene, frames[-1][0], frames[-1][1], ocol, odep)
    assert report["color_pixels_differing"] == 0, report


def test_graphs_off_matches(gpu_ctx, monkeypatch):
    scene = c.Scene(c.HEIGHTFIELD, 2, [64, 256, 160])
    monkeypatch.setenv("CPV_CB_GRAPH", "0")
    r = c.Renderer(gpu_ctx, scene)
    try:
        r.render(3)
        eager = r.readback()
    finally:
        r.close()
    monkeypatch.setenv("CPV_CB_GRAPH", "1")
    r = c.Renderer(gpu_ctx, scene)
    try:
        r.render(3)
        graphed = r.readback()
    finally:
        r.close()
    assert np.array_equal(eager[0], graphed[0]) and np.array_equal(eager[1], graphed[1])
