"""GPU parity at the workloads' full sizes.

Every benchmarked image is rendered through the ICD and compared with the
oracle (its threaded form, which is bit-identical to the single-threaded
one): the heightfield (1024² grid, 1920x1080), the blend scene (200k quads,
1920x1080) through the blend-table path, the general blend path, the
batched kernels and with interpolated colour, the 4096-draw frame
(2560x1440, 758 M triangles) batched and per draw, and four 2048² serving
requests of 500k triangles. Tolerances are those of tests/parity.py (colour
1 LSB, D32 1 ULP); the differing-pixel counts are printed and, so far,
always 0.
"""
import functools

import pytest

import cpvulkan_gb300 as c
from tests.parity import compare

pytestmark = pytest.mark.gpu


@functools.lru_cache(maxsize=4)
def _reference(oracle, config, seed, params):
    scene = c.Scene(config, seed, list(params))
    color, depth, stats = oracle.render_threaded(scene)
    return scene, color, depth, stats


def _check(ctx, oracle, config, seed, params):
    scene, ref_color, ref_depth, stats = _reference(oracle, config, seed, tuple(params))
    r = c.Renderer(ctx, scene)
    try:
        r.render(1)
        color, depth = r.readback()
    finally:
        r.close()
    report = compare(scene, color, depth, ref_color, ref_depth)
    print("full-size parity", config, seed, list(params), report, stats)
    assert report["color_pixels_differing"] == 0, report
    if ref_depth is not None:
        assert report["depth_pixels_differing"] == 0, report
    return stats


def test_heightfield_full(gpu_ctx, oracle):
    stats = _check(gpu_ctx, oracle, c.HEIGHTFIELD, 1, ())
    assert stats["triangles"] == 2 * 1023 * 1023


@pytest.mark.parametrize("path", ["tables", "general", "batched"])
def test_blend_full(gpu_ctx, oracle, monkeypatch, path):
    if path == "general":
        monkeypatch.setenv("CPV_BLEND_TABLES", "0")
    if path == "batched":
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    stats = _check(gpu_ctx, oracle, c.BLEND, 3, ())
    assert stats["fragments_written"] > 600_000_000


def test_blend_interpolated_full(gpu_ctx, oracle):
    _check(gpu_ctx, oracle, c.BLEND, 3, (200000, 1920, 1080, 1))


@pytest.mark.parametrize("path", ["batched", "per_draw"])
def test_batch_full(gpu_ctx, oracle, monkeypatch, path):
    if path == "per_draw":
        monkeypatch.setenv("CPV_BATCH", "0")
    stats = _check(gpu_ctx, oracle, c.BATCH, 4, ())
    assert stats["triangles"] > 700_000_000


@pytest.mark.parametrize("client", [0, 1, 2, 3])
def test_serve_request_2048(gpu_ctx, oracle, client):
    _check(gpu_ctx, oracle, c.SERVE, 5, (2048, 500000, client))
