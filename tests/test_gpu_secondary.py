"""Secondary command buffers (vkCmdExecuteCommands, CPVulkan/CommandBuffer.cpp:704-730).

The harness records each frame's draws into two secondary command buffers
(the first and second half of the scene's draws, each binding its own
state) executed inside the render pass; the images must equal the
oracle's, on the per-draw path, the batched path (a pass of many draws)
and with a sampled texture, on two frames in a row (the second replays the
primary's recorded commands, or its CUDA graph)."""
import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import compare

pytestmark = pytest.mark.gpu


@pytest.fixture
def secondary_ctx(native, monkeypatch):
    monkeypatch.setenv("CPVH_SECONDARY", "1")
    ctx = c.Context()
    yield ctx
    ctx.close()


@pytest.mark.parametrize("config,seed,params", [
    (c.CUBE, 1, [30]),
    (c.BATCH, 4, [48, 3000, 640, 360]),
    (c.PROGRAM, 2, [c.PROGRAM_TEXLIT, 0x10 | 0x20, 64, 48, 24]),
    (c.PROGRAM, 1, [c.PROGRAM_CUBE, 0x18 | 0x100, 64, 48, 24]),
])
def test_secondary_equals_oracle(secondary_ctx, oracle, config, seed, params):
    scene = c.Scene(config, seed, params)
    r = c.Renderer(secondary_ctx, scene)
    try:
        images = []
        for _ in range(2):
            r.render(1)
            images.append(r.readback())
    finally:
        r.close()
    ref_color, ref_depth, _ = oracle.render(scene)
    for color, depth in images:
        report = compare(scene, color, depth, ref_color, ref_depth)
        assert report["color_pixels_differing"] == 0, report
    assert np.array_equal(images[0][0], images[1][0])
