"""vkCmdDrawIndirect / vkCmdDrawIndexedIndirect: the same draws issued
through indirect argument records give the same images as direct draws
(the records are read from a host-visible buffer at replay), per draw and
batched, also when the records change between submissions."""
import ctypes

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


@pytest.mark.parametrize("mode", ["1", "2"])  # indirect, indirect-count draws
@pytest.mark.parametrize("config,params", [(c.CUBE, [20]), (c.BATCH, [24, 3000, 320, 200]), (c.HEIGHTFIELD, [64, 256, 160]),
                                           (c.PROGRAM, [c.PROGRAM_CUBE, 0x400 | 0x10, 64, 48, 24]),
                                           (c.PROGRAM, [c.PROGRAM_MESHPC, 0x10 | 0x20, 64, 48, 24])])
def test_indirect_equals_direct(gpu_ctx, monkeypatch, config, params, mode):
    scene = c.Scene(config, 6, params)
    direct = render(gpu_ctx, scene)
    monkeypatch.setenv("CPVH_INDIRECT", mode)
    indirect = render(gpu_ctx, scene)
    assert np.array_equal(direct[0], indirect[0])
    if direct[1] is not None:
        assert np.array_equal(direct[1], indirect[1])


def batch_raster_launches():
    icd = ctypes.CDLL(c.ICD_PATH)
    icd.cpv_profile_get.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double)]
    n, ms = ctypes.c_uint64(0), ctypes.c_double(0.0)
    icd.cpv_profile_get(b"cpv_batch_raster", ctypes.byref(n), ctypes.byref(ms))
    return n.value


def test_batched_indirect_follows_record_changes(gpu_ctx, monkeypatch):
    """A pass of 24 indirect draws runs batched, its records read at every
    submission. Records rewritten between submissions (half the draws without
    instances, one drawn from a later first index with fewer indices) rebuild
    the batch: every image equals the per-draw path's under the same records,
    and restoring the records restores the first image."""
    monkeypatch.setenv("CPVH_INDIRECT", "1")
    scene = c.Scene(c.BATCH, 6, [24, 3000, 320, 200])
    original = [scene.indirect_record(i) for i in range(scene.draws)]
    changed = [list(r) for r in original]
    for k in range(0, scene.draws, 2):
        changed[k][1] = 0
    d = scene.draw(1)
    changed[1][0] = (d.count // 3 // 2) * 3
    changed[1][2] = d.first + (d.count // 3 - d.count // 3 // 2) * 3

    def run(batched):
        if batched:
            monkeypatch.delenv("CPV_BATCH", raising=False)
        else:
            monkeypatch.setenv("CPV_BATCH", "0")
        r = c.Renderer(gpu_ctx, scene)
        try:
            images = []
            for records in (original, changed, original):
                for i, rec in enumerate(records):
                    r.set_indirect(i, rec)
                r.render(2)
                images.append(r.readback())
            return images
        finally:
            r.close()

    icd = ctypes.CDLL(c.ICD_PATH)
    icd.cpv_profile_reset()
    icd.cpv_profile_enable(1)
    try:
        batched = run(True)
    finally:
        icd.cpv_profile_enable(0)
    assert batch_raster_launches() >= 6
    plain = run(False)
    for (bc, bd), (pc, pd) in zip(batched, plain):
        assert np.array_equal(bc, pc) and np.array_equal(bd, pd)
    assert not np.array_equal(batched[0][0], batched[1][0])
    assert np.array_equal(batched[0][0], batched[2][0]) and np.array_equal(batched[0][1], batched[2][1])


@pytest.mark.parametrize("batched", [True, False])
def test_indirect_count_words(gpu_ctx, monkeypatch, batched):
    """vkCmdDraw(Indexed)IndirectCountKHR (CPVulkan/CommandBuffer.Draw.cpp:
    2226-2348): each draw is at most one record, drawn min(maxDrawCount = 1,
    count word) times. Count words of 0 skip their draws, words above 1 are
    clamped to 1: the image equals the indirect path's with those draws
    given no instances, batched and per draw."""
    if not batched:
        monkeypatch.setenv("CPV_BATCH", "0")
    scene = c.Scene(c.BATCH, 7, [30, 3000, 320, 200])
    skip = set(range(1, scene.draws, 3))  # 20 draws remain: the pass still batches
    monkeypatch.setenv("CPVH_INDIRECT", "2")
    r = c.Renderer(gpu_ctx, scene)
    icd = ctypes.CDLL(c.ICD_PATH)
    icd.cpv_profile_reset()
    icd.cpv_profile_enable(1)
    try:
        for i in range(scene.draws):
            r.set_indirect_count(i, 0 if i in skip else (7 if i % 2 else 1))
        r.render(2)
        got = r.readback()
    finally:
        icd.cpv_profile_enable(0)
        r.close()
    assert (batch_raster_launches() >= 2) == batched
    monkeypatch.setenv("CPVH_INDIRECT", "1")
    r = c.Renderer(gpu_ctx, scene)
    try:
        for i in skip:
            rec = scene.indirect_record(i)
            rec[1] = 0
            r.set_indirect(i, rec)
        r.render(2)
        want = r.readback()
    finally:
        r.close()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    assert not np.array_equal(got[0], render(gpu_ctx, scene)[0])
