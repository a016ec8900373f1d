"""cpv_queue_submit_no_alloc against vkQueueSubmit.

The allocation-free submit bins every draw through the ICD's fixed device
scratch array instead of the queue's grow-only scratch. Its images must equal
those of vkQueueSubmit (the kernels are the same; the tolerance is zero), on
two submissions in a row, without ever allocating the queue's own scratch,
and a draw too large for the fixed array, direct or indirect, must be
rejected before any work is enqueued. This file sorts last so that it also
runs after every other GPU test of the session.
"""
import ctypes

import numpy as np
import pytest

import cpvulkan_gb300 as c

pytestmark = pytest.mark.gpu

SCENES = [
    # binned path (primitives × tiles above the direct limit)
    (c.HEIGHTFIELD, [256, 640, 360]),
    (c.BLEND, [3000, 640, 360]),
    (c.BATCH, [32, 3000, 640, 360]),
    # direct path (no bins)
    (c.CUBE, []),
]


def _images(ctx, scene, frames_each=1, calls=1):
    r = c.Renderer(ctx, scene)
    try:
        out = []
        for _ in range(calls):
            r.render(frames_each)
            out.append(r.readback())
        return out
    finally:
        r.close()


@pytest.fixture
def no_alloc_ctx(native, monkeypatch):
    monkeypatch.setenv("CPVH_SUBMIT", "no_alloc")
    ctx = c.Context()
    yield ctx
    ctx.close()


def _scratch_generation(ctx):
    lib = ctypes.CDLL(c.ICD_PATH)
    lib.cpv_queue_scratch_generation.restype = ctypes.c_uint64
    lib.cpv_queue_scratch_generation.argtypes = [ctypes.c_void_p]
    return lib.cpv_queue_scratch_generation(ctx.queue)


@pytest.mark.parametrize("config,params", SCENES)
def test_no_alloc_matches_queue_submit(gpu_ctx, no_alloc_ctx, config, params):
    scene = c.Scene(config, 5, params)
    (ref_color, ref_depth), = _images(gpu_ctx, scene)
    before = c.kernel_launches()
    runs = _images(no_alloc_ctx, scene, calls=2)
    assert c.kernel_launches() > before
    # the queue's own grow-only scratch was never allocated
    assert _scratch_generation(no_alloc_ctx) == 0
    for color, depth in runs:
        assert np.count_nonzero(np.any(color != ref_color, axis=-1)) == 0
        if ref_depth is not None:
            assert np.count_nonzero(np.any(depth != ref_depth, axis=-1)) == 0


def _expect_rejected(ctx, scene):
    r = c.Renderer(ctx, scene)
    try:
        before = c.kernel_launches()
        with pytest.raises(RuntimeError):
            r.render(1)
        lib = ctypes.CDLL(c.ICD_PATH)
        lib.cpv_last_error.restype = ctypes.c_char_p
        msg = lib.cpv_last_error().decode()
        assert "cpv_queue_submit_no_alloc" in msg and "fixed scratch holds 33554432" in msg, msg
        assert c.kernel_launches() == before
    finally:
        r.close()


def test_no_alloc_rejects_oversized_draw(no_alloc_ctx):
    # 2 × 1499² ≈ 4.49 million triangles: 36 MB of tile rectangles alone,
    # more than the 32 MiB fixed scratch.
    _expect_rejected(no_alloc_ctx, c.Scene(c.HEIGHTFIELD, 1, [1500, 640, 360]))


@pytest.mark.parametrize("mode", ["1", "2"])
def test_no_alloc_rejects_oversized_indirect_draw(native, monkeypatch, mode):
    # The same draw issued as vkCmdDrawIndexedIndirect (mode 1) or as an
    # indirect-count draw (mode 2): its record is read at submission and the
    # submission is refused before any of its work is enqueued.
    monkeypatch.setenv("CPVH_SUBMIT", "no_alloc")
    monkeypatch.setenv("CPVH_INDIRECT", mode)
    ctx = c.Context()
    try:
        _expect_rejected(ctx, c.Scene(c.HEIGHTFIELD, 1, [1500, 640, 360]))
    finally:
        ctx.close()
