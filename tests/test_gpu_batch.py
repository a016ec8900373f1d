"""Batched render passes (one kernel sequence, captured in a CUDA graph, for
every draw of a render pass) against the per-draw path and the oracle.

Batching changes no draw's arithmetic: its images must equal the per-draw
images bit for bit, on every frame (the first eager run and the graph
replays), for every tile size and fragment schedule, and when the pair
buffers overflow (the raster then scans the tile rectangles).
"""
import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import compare

pytestmark = pytest.mark.gpu


def frames(ctx, scene, n=1):
    r = c.Renderer(ctx, scene)
    try:
        out = []
        for _ in range(n):
            r.render(1)
            out.append(r.readback())
        return out
    finally:
        r.close()


def same(a, b):
    (ca, da), (cb, db) = a, b
    assert np.count_nonzero(np.any(ca != cb, axis=-1)) == 0
    if da is not None:
        assert np.count_nonzero(np.any(da != db, axis=-1)) == 0


@pytest.fixture
def plain(monkeypatch):
    def run(ctx, scene, n=1):
        monkeypatch.setenv("CPV_BATCH", "0")
        out = frames(ctx, scene, n)
        monkeypatch.setenv("CPV_BATCH", "1")
        return out
    return run


@pytest.mark.parametrize("seed", [1, 2])
def test_batched_equals_plain_and_oracle(gpu_ctx, oracle, plain, seed):
    scene = c.Scene(c.BATCH, seed, [64, 4000, 640, 360])
    ref = plain(gpu_ctx, scene)[0]
    before = c.kernel_launches()
    runs = frames(gpu_ctx, scene, 3)  # eager first run, then graph replays
    assert c.kernel_launches() > before
    for got in runs:
        same(got, ref)
    ocol, odep, _ = oracle.render(scene)
    report = compare(scene, runs[-1][0], runs[-1][1], ocol, odep)
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("tile", ["8", "16", "32"])
@pytest.mark.parametrize("schedule", ["0", "1", "2"])
def test_batched_schedules(gpu_ctx, plain, monkeypatch, tile, schedule):
    monkeypatch.setenv("CPV_TILE", tile)
    monkeypatch.setenv("CPV_SCHEDULE", schedule)
    scene = c.Scene(c.BATCH, 3, [40, 3000, 400, 272])
    ref = plain(gpu_ctx, scene)[0]
    same(frames(gpu_ctx, scene)[0], ref)


def test_batched_pair_overflow_scans_rectangles(gpu_ctx, plain, monkeypatch):
    scene = c.Scene(c.BATCH, 4, [24, 2000, 320, 200])
    ref = plain(gpu_ctx, scene)[0]
    monkeypatch.setenv("CPV_BATCH_PAIR_CAPACITY", "100")
    for got in frames(gpu_ctx, scene, 3):  # overflowing launch, then regrown buffers
        same(got, ref)


def test_batched_blend_scene(gpu_ctx, plain, monkeypatch):
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.BLEND, 5, [1500, 480, 270])  # one draw: a batch of one
    ref = plain(gpu_ctx, scene)[0]
    same(frames(gpu_ctx, scene, 2)[1], ref)


def test_batched_program_variants(gpu_ctx, plain, monkeypatch):
    """Stencil, D16, CW, strips, discard, points, lines, a logic op, a
    colour write mask, the depth bounds test and a depth-only pass through
    the batched kernels."""
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    for program, variant in [(c.PROGRAM_CUBE, 0x18 | 0x100), (c.PROGRAM_CUBE, 0x8 | 0x4 | 0x1), (c.PROGRAM_CUBE, 0x400 | 0x10),
                             (c.PROGRAM_DISCARD, 0x10), (c.PROGRAM_TEXLIT, 0x10 | 0x4000), (c.PROGRAM_MESHPC, 0x10 | 0x20),
                             (c.PROGRAM_POINTS, 0x10000 | 0x20), (c.PROGRAM_CUBE, 0x10000 | 0x800 | 0x20000 | 0x10),
                             (c.PROGRAM_FLATQUAD, 0x20 | 0x40000 | (6 << 20)), (c.PROGRAM_CUBE, 0x10 | 0x80000 | (0xB << 24)),
                             (c.PROGRAM_CUBE, 0x18 | 0x100 | (2 << 28)), (c.PROGRAM_CUBE, 0x40000000 | 0x18 | 0x100)]:
        scene = c.Scene(c.PROGRAM, 2, [program, variant, 64, 48, 24])
        ref = plain(gpu_ctx, scene)[0]
        same(frames(gpu_ctx, scene)[0], ref)


@pytest.mark.parametrize("seed", [6, 7])
def test_tuned_batch_equals_plain(gpu_ctx, plain, monkeypatch, seed):
    """The tuner runs the pass once per candidate (tile 8/16/32, warps per
    tile, batch size, schedule and, for the sparse schedule, the per-pixel
    fragment-list depth) on its first submission, restoring the attachments
    around each run: the frames must still equal the per-draw path's, and
    the report must name every candidate and the choice."""
    monkeypatch.setenv("CPV_AUTOTUNE", "1")
    scene = c.Scene(c.BATCH, seed, [32, 3000, 352, 208])
    ref = plain(gpu_ctx, scene)[0]
    runs = frames(gpu_ctx, scene, 3)
    report = c.batch_tuning()
    assert report.count(" ms") == 9 and "chosen tile" in report, report
    assert "depth 16" in report and "depth 32" in report, report
    for got in runs:
        same(got, ref)


def test_large_single_draw_runs_batched(gpu_ctx, oracle, plain, monkeypatch):
    """A pass of one draw with at least CPV_BATCH_MIN_PRIMS primitives (and no
    blend tables) runs batched: its image equals the per-draw image and the
    oracle's, and the batched raster is what ran."""
    import ctypes
    monkeypatch.setenv("CPV_BATCH_MIN_PRIMS", "20000")
    scene = c.Scene(c.HEIGHTFIELD, 3, [128, 480, 270])  # 32,258 triangles in one draw
    ref = plain(gpu_ctx, scene)[0]
    icd = ctypes.CDLL(c.ICD_PATH)
    icd.cpv_profile_get.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double)]
    icd.cpv_profile_reset()
    icd.cpv_profile_enable(1)
    try:
        got = frames(gpu_ctx, scene, 2)
    finally:
        icd.cpv_profile_enable(0)
    n, ms = ctypes.c_uint64(0), ctypes.c_double(0.0)
    icd.cpv_profile_get(b"cpv_batch_raster", ctypes.byref(n), ctypes.byref(ms))
    assert n.value >= 2
    for g in got:
        same(g, ref)
    ocol, odep, _ = oracle.render(scene)
    assert compare(scene, got[-1][0], got[-1][1], ocol, odep)["color_pixels_differing"] == 0


def _profiled_launches(name, fn):
    import ctypes
    icd = ctypes.CDLL(c.ICD_PATH)
    icd.cpv_profile_get.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double)]
    icd.cpv_profile_reset()
    icd.cpv_profile_enable(1)
    try:
        out = fn()
    finally:
        icd.cpv_profile_enable(0)
    n, ms = ctypes.c_uint64(0), ctypes.c_double(0.0)
    icd.cpv_profile_get(name.encode(), ctypes.byref(n), ctypes.byref(ms))
    return out, n.value


@pytest.mark.parametrize("trim", ["0", "1", "7"])
def test_vertex_stage(gpu_ctx, plain, monkeypatch, trim):
    """The vertex stage shades each vertex of an indexed triangle draw once
    per frame into slots that the set-up and raster kernels read. With the
    ranges narrowed (CPV_VS_TRIM), the vertices outside them are shaded by
    the set-up itself, in the same triangles as slot vertices: every frame
    must still equal the per-draw path's, and the stage must have run."""
    monkeypatch.setenv("CPV_VS_TRIM", trim)
    scene = c.Scene(c.BATCH, 8, [48, 3000, 400, 240])
    ref = plain(gpu_ctx, scene)[0]
    runs, n = _profiled_launches("cpv_batch_vs", lambda: frames(gpu_ctx, scene, 2))
    assert n >= 2
    for got in runs:
        same(got, ref)


def test_vertex_stage_off_and_textured_grid(gpu_ctx, plain, monkeypatch):
    """CPV_VERTEX_STAGE=0 gives the same frames without the stage; a
    textured heightfield grid (each vertex in six triangles, texture
    coordinates and normals as outputs) through the stage equals the
    per-draw path."""
    scene = c.Scene(c.BATCH, 9, [24, 2000, 320, 200])
    ref = plain(gpu_ctx, scene)[0]
    monkeypatch.setenv("CPV_VERTEX_STAGE", "0")
    runs, n = _profiled_launches("cpv_batch_vs", lambda: frames(gpu_ctx, scene, 2))
    assert n == 0
    for got in runs:
        same(got, ref)
    monkeypatch.setenv("CPV_VERTEX_STAGE", "1")
    monkeypatch.setenv("CPV_BATCH_MIN_PRIMS", "20000")
    grid = c.Scene(c.HEIGHTFIELD, 4, [160, 480, 270])
    ref = plain(gpu_ctx, grid)[0]
    runs, n = _profiled_launches("cpv_batch_vs", lambda: frames(gpu_ctx, grid, 2))
    assert n >= 2
    for got in runs:
        same(got, ref)
