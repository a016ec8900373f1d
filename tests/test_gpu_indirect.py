"""vkCmdDrawIndirect / vkCmdDrawIndexedIndirect: the same draws issued
through indirect argument records give the same images as direct draws
(the records are read from a host-visible buffer at replay)."""
import numpy as np
import pytest

import cpvulkan_gb300 as c

pytestmark = pytest.mark.gpu


def render(ctx, scene, frames=2):
    r = c.Renderer(ctx, scene)
    try:
        r.render(frames)
        return r.readback()
    finally:
        r.close()


@pytest.mark.parametrize("config,params", [(c.CUBE, [20]), (c.BATCH, [24, 3000, 320, 200]), (c.HEIGHTFIELD, [64, 256, 160]),
                                           (c.PROGRAM, [c.PROGRAM_CUBE, 0x400 | 0x10, 64, 48, 24]),
                                           (c.PROGRAM, [c.PROGRAM_MESHPC, 0x10 | 0x20, 64, 48, 24])])
def test_indirect_equals_direct(gpu_ctx, monkeypatch, config, params):
    scene = c.Scene(config, 6, params)
    direct = render(gpu_ctx, scene)
    monkeypatch.setenv("CPVH_INDIRECT", "1")
    indirect = render(gpu_ctx, scene)
    assert np.array_equal(direct[0], indirect[0])
    if direct[1] is not None:
        assert np.array_equal(direct[1], indirect[1])
