"""The labelled quad-derivative LOD mode on the GPU (CPV_SPEC_LOD=1).

Implicit-LOD sampling in fragment shaders takes λ_base = log2(max(ρx, ρy))
from fine derivatives within each 2x2 quad: the shader runs for the pixel's
horizontal and vertical neighbours (helper runs that record coordinates and
write nothing), then for the pixel (cpv_quad_helpers, cpv_sample_quad). The
images must equal the oracle's render of the same mode bit for bit, per
draw under every schedule and tile size, batched, for points and lines, and
at the heightfield's full size; and the mode must actually change the image
where the texture is minified.
"""
import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import compare

pytestmark = pytest.mark.gpu

SPEC_VARIANTS = [
    (c.PROGRAM_TEXLIT, 0x10), (c.PROGRAM_TEXLIT, 0x10 | 0x4000), (c.PROGRAM_TEXLIT, 0x10 | 0x8000 | 0x20),
    (c.PROGRAM_TEXLIT, 0x0 | 0x1 | 0x4),
]


def _render(ctx, scene):
    r = c.Renderer(ctx, scene)
    try:
        r.render(1)
        return r.readback()
    finally:
        r.close()


def _check(ctx, oracle, scene):
    scene.spec_lod = 1
    gc, gd = _render(ctx, scene)
    rc, rd, stats = oracle.render(scene)
    report = compare(scene, gc, gd, rc, rd)
    assert report["color_pixels_differing"] == 0, report
    if rd is not None:
        assert report["depth_pixels_differing"] == 0, report
    return gc, rc, stats


@pytest.mark.parametrize("program,variant", SPEC_VARIANTS)
@pytest.mark.parametrize("seed", [1, 2])
def test_spec_lod_variants(gpu_ctx, oracle, monkeypatch, program, variant, seed):
    monkeypatch.setenv("CPV_SPEC_LOD", "1")
    scene = c.Scene(c.PROGRAM, seed, [program, variant, 64, 48, 24])
    gc, _, stats = _check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    # the mode took effect: the reference's λ 0 gives another image
    scene.spec_lod = 0
    lod0, _, _ = oracle.render(scene)
    assert np.count_nonzero(np.any(gc != lod0, axis=-1)) > 0


@pytest.mark.parametrize("tile", ["8", "16", "32"])
@pytest.mark.parametrize("schedule", ["0", "1", "2"])
def test_spec_lod_schedules(gpu_ctx, oracle, monkeypatch, tile, schedule):
    monkeypatch.setenv("CPV_SPEC_LOD", "1")
    monkeypatch.setenv("CPV_TILE", tile)
    monkeypatch.setenv("CPV_SCHEDULE", schedule)
    _check(gpu_ctx, oracle, c.Scene(c.HEIGHTFIELD, 2, [96, 320, 200]))


@pytest.mark.parametrize("variant", [0x10000 | 0x10, 0x10000 | 0x400 | 0x10 | 0x20000, 0x10000 | 0x800 | 0x10])
def test_spec_lod_points_lines(gpu_ctx, oracle, monkeypatch, variant):
    # points: every neighbour has the same inputs (λ -∞, the least level);
    # lines: the neighbours' line parameter
    monkeypatch.setenv("CPV_SPEC_LOD", "1")
    _, _, stats = _check(gpu_ctx, oracle, c.Scene(c.PROGRAM, 3, [c.PROGRAM_TEXLIT, variant, 96, 64, 60]))
    assert stats["fragments"] > 0


@pytest.mark.parametrize("config,params", [(c.PROGRAM, [c.PROGRAM_TEXLIT, 0x10 | 0x8000 | 0x20, 64, 48, 24]),
                                           (c.HEIGHTFIELD, [128, 480, 270])])
def test_spec_lod_batched(gpu_ctx, oracle, monkeypatch, config, params):
    monkeypatch.setenv("CPV_SPEC_LOD", "1")
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    _check(gpu_ctx, oracle, c.Scene(config, 4, params))


def test_spec_lod_heightfield_full(gpu_ctx, oracle, monkeypatch):
    """The heightfield at its full size (1024² grid, 1920x1080, trilinear
    over a full mip chain) against the threaded oracle in the same mode."""
    monkeypatch.setenv("CPV_SPEC_LOD", "1")
    scene = c.Scene(c.HEIGHTFIELD, 1, [])
    scene.spec_lod = 1
    gc, gd = _render(gpu_ctx, scene)
    rc, rd, stats = oracle.render_threaded(scene)
    report = compare(scene, gc, gd, rc, rd)
    print("spec-LOD full-size parity", report, stats)
    assert report["color_pixels_differing"] == 0 and report["depth_pixels_differing"] == 0, report
    assert stats["triangles"] == 2 * 1023 * 1023
