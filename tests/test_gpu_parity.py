"""GPU parity: images rendered through the ICD (Vulkan API → NVRTC-compiled
sm_103a kernels) against the CPU oracle on the same seeded scenes."""
import itertools

import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import compare

pytestmark = pytest.mark.gpu


def render_gpu(ctx, scene):
    r = c.Renderer(ctx, scene)
    try:
        r.render(1)
        return r.readback()
    finally:
        r.close()


def check(ctx, oracle, scene):
    gc, gd = render_gpu(ctx, scene)
    rc, rd, stats = oracle.render(scene)
    report = compare(scene, gc, gd, rc, rd)
    return report, stats


# (program, variant) combinations: cull modes, both windings, D16/D32/D32S8,
# stencil, blending, BGRA targets, strips and fans, 16-bit indices.
VARIANTS = [
    (c.PROGRAM_CUBE, 0x0), (c.PROGRAM_CUBE, 0x8 | 0x2), (c.PROGRAM_CUBE, 0x10 | 0x4 | 0x1), (c.PROGRAM_CUBE, 0x18 | 0x100),
    (c.PROGRAM_CUBE, 0x10 | 0x40), (c.PROGRAM_CUBE, 0x10 | 0x80), (c.PROGRAM_CUBE, 0x10 | 0xC0), (c.PROGRAM_CUBE, 0x20 | 0x200),
    (c.PROGRAM_CUBE, 0x400 | 0x10), (c.PROGRAM_CUBE, 0x800 | 0x10), (c.PROGRAM_CUBE, 0x1000 | 0x10), (c.PROGRAM_CUBE, 0x2000 | 0x10 | 0x20),
    (c.PROGRAM_DISCARD, 0x10), (c.PROGRAM_NOPERSP, 0x8), (c.PROGRAM_FLATQUAD, 0x20), (c.PROGRAM_FLATQUAD, 0x20 | 0x200),
    (c.PROGRAM_TEXLIT, 0x10), (c.PROGRAM_TEXLIT, 0x10 | 0x4000), (c.PROGRAM_TEXLIT, 0x10 | 0x8000 | 0x20),
    (c.PROGRAM_MESHPC, 0x10 | 0x2 | 0x4), (c.PROGRAM_MESHPC, 0x10 | 0x20),
]


# Points and lines (variant bit 16; bits 10-11 then pick points, line list,
# line strip; bit 17 a 3.5 px line width): sizes from the POINTS program's
# gl_PointSize (0-16 px) or the default 1, perspective / linear / flat
# varyings, depth, blending, BGRA, discard and a sampled texture.
POINTS_LINES = [
    (c.PROGRAM_POINTS, 0x10000 | 0x10), (c.PROGRAM_POINTS, 0x10000 | 0x20 | 0x8), (c.PROGRAM_POINTS, 0x10000 | 0x200 | 0x18 | 0x100),
    (c.PROGRAM_FLATQUAD, 0x10000 | 0x20), (c.PROGRAM_CUBE, 0x10000 | 0x400), (c.PROGRAM_CUBE, 0x10000 | 0x400 | 0x20000 | 0x10),
    (c.PROGRAM_CUBE, 0x10000 | 0x800 | 0x20 | 0x20000), (c.PROGRAM_NOPERSP, 0x10000 | 0x400 | 0x20000),
    (c.PROGRAM_FLATQUAD, 0x10000 | 0x400 | 0x20000 | 0x20), (c.PROGRAM_DISCARD, 0x10000 | 0x20000 | 0x400),
    (c.PROGRAM_TEXLIT, 0x10000 | 0x800 | 0x10 | 0x20000), (c.PROGRAM_POINTS, 0x10000 | 0x400 | 0x20000 | 0x1000),
]


# Logic ops (bit 18, VkLogicOp in bits 20-23; blending is then off) and
# partial colour write masks (bit 19, mask in bits 24-27), on interpolated,
# flat-shaded (blend-table candidates), textured, line and BGRA pipelines.
LOGIC_MASK = [
    (c.PROGRAM_CUBE, 0x10 | 0x40000 | (6 << 20)), (c.PROGRAM_FLATQUAD, 0x20 | 0x40000 | (7 << 20)),
    (c.PROGRAM_FLATQUAD, 0x20 | 0x200 | 0x40000 | (2 << 20)), (c.PROGRAM_TEXLIT, 0x10 | 0x40000 | (12 << 20) | 0x80000 | (0x7 << 24)),
    (c.PROGRAM_CUBE, 0x10000 | 0x400 | 0x20000 | 0x40000 | (9 << 20)), (c.PROGRAM_FLATQUAD, 0x40000 | (14 << 20)),
    (c.PROGRAM_FLATQUAD, 0x20 | 0x80000 | (0x9 << 24)), (c.PROGRAM_CUBE, 0x18 | 0x100 | 0x200 | 0x80000 | (0x6 << 24)),
    (c.PROGRAM_POINTS, 0x10000 | 0x20 | 0x80000 | (0x3 << 24)),
]

# The depth bounds test (bits 28-29: [0, 1], [0.3, 1], [0.8, 1] against a
# depth cleared to 0.75) with D32, D32S8 + stencil, D16, blending and lines.
DEPTH_BOUNDS = [
    (c.PROGRAM_CUBE, 0x10 | (2 << 28)), (c.PROGRAM_CUBE, 0x18 | 0x100 | (2 << 28)), (c.PROGRAM_CUBE, 0x18 | 0x100 | (3 << 28)),
    (c.PROGRAM_FLATQUAD, 0x8 | 0x20 | (2 << 28)), (c.PROGRAM_MESHPC, 0x10 | 0x20 | (1 << 28)),
    (c.PROGRAM_CUBE, 0x10000 | 0x400 | 0x20000 | 0x10 | (2 << 28)),
]

# Depth-only passes (bit 30: no colour attachment): depth and stencil
# against the oracle, with D32, D32S8 + stencil, D16 + discard, a sampled
# texture, lines and the depth bounds test.
DEPTH_ONLY = [
    (c.PROGRAM_CUBE, 0x40000000 | 0x10), (c.PROGRAM_CUBE, 0x40000000 | 0x18 | 0x100), (c.PROGRAM_DISCARD, 0x40000000 | 0x8),
    (c.PROGRAM_TEXLIT, 0x40000000 | 0x10), (c.PROGRAM_CUBE, 0x40000000 | 0x10000 | 0x800 | 0x20000 | 0x10),
    (c.PROGRAM_FLATQUAD, 0x40000000 | 0x8 | 0x20 | (2 << 28)),
]


@pytest.mark.parametrize("program,variant", VARIANTS + POINTS_LINES + LOGIC_MASK + DEPTH_BOUNDS + DEPTH_ONLY)
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_program_variants(gpu_ctx, oracle, program, variant, seed):
    scene = c.Scene(c.PROGRAM, seed, [program, variant, 64, 48, 24])
    report, stats = check(gpu_ctx, oracle, scene)
    if (variant >> 28) & 3 != 3:  # depth bounds above the stored depth: nothing passes
        assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("frame", [0, 37, 90, 200])
def test_cube_frames(gpu_ctx, oracle, frame):
    scene = c.Scene(c.CUBE, 1, [frame])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 1000
    assert report["color_pixels_differing"] == 0 and report["depth_pixels_differing"] == 0, report


def test_heightfield_small(gpu_ctx, oracle):
    scene = c.Scene(c.HEIGHTFIELD, 1, [128, 480, 270])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


def test_blend_small(gpu_ctx, oracle):
    scene = c.Scene(c.BLEND, 3, [2000, 640, 360])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


def test_batch_small(gpu_ctx, oracle):
    scene = c.Scene(c.BATCH, 4, [48, 3000, 640, 360])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


def test_serve_request(gpu_ctx, oracle):
    scene = c.Scene(c.SERVE, 5, [256, 5000, 3])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("tile", ["8", "16", "32"])
@pytest.mark.parametrize("schedule", ["0", "1", "2"])
@pytest.mark.parametrize("config,params", [(c.HEIGHTFIELD, [96, 320, 200]), (c.BLEND, [600, 320, 200]), (c.BATCH, [24, 2000, 320, 200])])
def test_schedule_invariance(gpu_ctx, oracle, monkeypatch, tile, schedule, config, params):
    """Tile size and fragment schedule change only the work distribution:
    every combination must reproduce the oracle's image exactly."""
    monkeypatch.setenv("CPV_TILE", tile)
    monkeypatch.setenv("CPV_SCHEDULE", schedule)
    scene = c.Scene(config, 7, params)
    report, _ = check(gpu_ctx, oracle, scene)
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("tile", ["8", "16", "32"])
@pytest.mark.parametrize("schedule", ["0", "1", "2"])
@pytest.mark.parametrize("program,variant", [(c.PROGRAM_POINTS, 0x10000 | 0x20), (c.PROGRAM_CUBE, 0x10000 | 0x800 | 0x20000 | 0x20)])
def test_points_lines_schedule_invariance(gpu_ctx, oracle, monkeypatch, tile, schedule, program, variant):
    monkeypatch.setenv("CPV_TILE", tile)
    monkeypatch.setenv("CPV_SCHEDULE", schedule)
    scene = c.Scene(c.PROGRAM, 4, [program, variant, 96, 64, 120])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments"] > 0
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("schedule", ["0", "2"])
@pytest.mark.parametrize("tile", ["8", "16"])
def test_coverage_kats(gpu_ctx, oracle, monkeypatch, tile, schedule):
    """The hand-placed coverage cases (pixel centres on edges, a shared edge,
    both windings under every cull mode, a sliver, a degenerate and an
    off-screen triangle) through the device: images equal to the oracle's,
    whose coverage the numpy restatement pins, under two tile sizes and
    both the immediate and the sparse schedule."""
    from tests import coverage_kat as kat
    monkeypatch.setenv("CPV_TILE", tile)
    monkeypatch.setenv("CPV_SCHEDULE", schedule)
    for case in kat.CASES:
        report, stats = check(gpu_ctx, oracle, kat.scene(case))
        assert stats["fragments"] == int(kat.coverage(case).sum())
        assert report["color_pixels_differing"] == 0, (case[0], report)


@pytest.mark.parametrize("config,params", [(c.PROGRAM, [c.PROGRAM_CUBE, 0x18 | 0x100, 64, 48, 24]), (c.HEIGHTFIELD, [64, 256, 160]),
                                           (c.PROGRAM, [c.PROGRAM_FLATQUAD, 0x20, 64, 48, 24]), (c.BATCH, [24, 3000, 320, 200]),
                                           (c.CUBE, [45])])
def test_second_subpass(gpu_ctx, oracle, monkeypatch, config, params):
    """vkCmdNextSubpass (CPVulkan/CommandBuffer.cpp:649-664): the frame draws
    in subpass 1 of a two-subpass render pass whose subpass 0 references only
    the depth attachment, with pipelines created for subpass 1; the image
    equals the oracle's (a pass of several subpasses runs per draw)."""
    monkeypatch.setenv("CPVH_SUBPASSES", "2")
    scene = c.Scene(config, 3, params)
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


# Vertex attribute formats (scene parameter 5): the CUBE program's colour
# attribute read from a second binding in normalised 8/16-bit formats (1-4
# channels, B8G8R8A8) and half floats, raw bytes over the whole code range.
VERTEX_FORMATS = [9, 10, 16, 17, 23, 24, 37, 38, 44, 70, 71, 77, 78, 84, 85, 91, 92, 97]


@pytest.mark.parametrize("fmt", VERTEX_FORMATS)
@pytest.mark.parametrize("seed", [1, 2])
def test_vertex_attribute_formats(gpu_ctx, oracle, fmt, seed):
    scene = c.Scene(c.PROGRAM, seed, [c.PROGRAM_CUBE, 0x10, 64, 48, 24, fmt])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("fmt", [38, 97])
def test_vertex_attribute_formats_batched(gpu_ctx, oracle, monkeypatch, fmt):
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 3, [c.PROGRAM_CUBE, 0x10, 64, 48, 24, fmt])
    report, _ = check(gpu_ctx, oracle, scene)
    assert report["color_pixels_differing"] == 0, report


# The FETCH program: OpImage + OpImageFetch (level 0, zeros outside),
# OpBitCount, OpCopyMemory and a specialisation constant folded through
# OpSpecConstantOp, with the constant's default (parameter 5 = 0) and two
# VkSpecializationInfo values; opaque and blended.
@pytest.mark.parametrize("variant", [0x0, 0x20, 0x4])
@pytest.mark.parametrize("k", [0, 1, 9])
@pytest.mark.parametrize("seed", [1, 2])
def test_fetch_program(gpu_ctx, oracle, variant, k, seed):
    scene = c.Scene(c.PROGRAM, seed, [c.PROGRAM_FETCH, variant, 64, 48, 24, k])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 1000
    assert report["color_pixels_differing"] == 0, report


def test_fetch_program_batched(gpu_ctx, oracle, monkeypatch):
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 3, [c.PROGRAM_FETCH, 0x20, 64, 48, 24, 9])
    report, _ = check(gpu_ctx, oracle, scene)
    assert report["color_pixels_differing"] == 0, report


# Colour attachments beyond RGBA8/BGRA8 (parameter 6): R8, R8G8, R16, R16G16
# UNORM, R8G8B8A8 SNORM, R16G16 and R32 SFLOAT, cleared to a colour outside
# [0, 1]; opaque, blended (destination alpha 1 where the format has none),
# blended under a partial write mask, wide lines and flat quads. The colour
# attribute is half-float with channels in [-2, 2], so the encoders clamp.
COLOUR_ATTACHMENTS = [9, 16, 38, 70, 77, 83, 100]
COLOUR_VARIANTS = [(c.PROGRAM_CUBE, 0x10), (c.PROGRAM_CUBE, 0x10 | 0x20), (c.PROGRAM_CUBE, 0x10 | 0x20 | 0x80000 | (0x5 << 24)),
                   (c.PROGRAM_CUBE, 0x10000 | 0x400 | 0x20000 | 0x20), (c.PROGRAM_FLATQUAD, 0x20)]


@pytest.mark.parametrize("fmt", COLOUR_ATTACHMENTS)
@pytest.mark.parametrize("program,variant", COLOUR_VARIANTS)
@pytest.mark.parametrize("seed", [1, 2])
def test_colour_attachment_formats(gpu_ctx, oracle, fmt, program, variant, seed):
    scene = c.Scene(c.PROGRAM, seed, [program, variant, 64, 48, 24, 97, fmt])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("fmt", [9, 16, 38])
@pytest.mark.parametrize("op", [3, 6, 12])
def test_colour_attachment_logic_ops(gpu_ctx, oracle, fmt, op):
    scene = c.Scene(c.PROGRAM, 4, [c.PROGRAM_CUBE, 0x10 | 0x40000 | (op << 20) | 0x80000 | (0xB << 24), 64, 48, 24, 97, fmt])
    report, _ = check(gpu_ctx, oracle, scene)
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("fmt", [9, 38, 83, 100])
def test_colour_attachment_formats_batched(gpu_ctx, oracle, monkeypatch, fmt):
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 3, [c.PROGRAM_CUBE, 0x10 | 0x20, 64, 48, 24, 97, fmt])
    report, _ = check(gpu_ctx, oracle, scene)
    assert report["color_pixels_differing"] == 0, report


# 8- and 16-byte colour texels on the first attachment: R16G16B16A16
# UNORM and SFLOAT, R32G32 and R32G32B32A32 SFLOAT, under the same variants
# (opaque, blended, write mask with a logic op, wide lines, flat quads).
WIDE_COLOUR_ATTACHMENTS = [91, 97, 103, 109]


@pytest.mark.parametrize("fmt", WIDE_COLOUR_ATTACHMENTS)
@pytest.mark.parametrize("program,variant", COLOUR_VARIANTS)
def test_wide_colour_attachment_formats(gpu_ctx, oracle, fmt, program, variant):
    scene = c.Scene(c.PROGRAM, 5, [program, variant, 64, 48, 24, 97, fmt])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


@pytest.mark.parametrize("fmt", WIDE_COLOUR_ATTACHMENTS)
def test_wide_colour_attachment_formats_batched(gpu_ctx, oracle, monkeypatch, fmt):
    monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 6, [c.PROGRAM_CUBE, 0x10 | 0x20, 64, 48, 24, 97, fmt])
    report, _ = check(gpu_ctx, oracle, scene)
    assert report["color_pixels_differing"] == 0, report


def _pack(values):
    """Bytes of a packed scene parameter (byte k = values[k])."""
    out = 0
    for k, v in enumerate(values):
        out |= int(v) << (8 * k)
    return out


# Several colour attachments (the MRT program writes locations 0-7): the
# formats of attachments 1 .. (0: an unused reference in the middle) and
# each one's blend byte (bit 0 src-over, bit 1 additive colour with MAX
# alpha, bits 4-7 a write mask), with the first attachment's variant.
MRT_CASES = [
    ([37], [0x01], 0x10),                                   # two RGBA8, the second blended
    ([83, 100, 9], [0x02, 0x00, 0x00], 0x10 | 0x20),        # half, float, R8; the first blended too
    ([38, 0, 77, 16, 70, 37, 44], [0x00, 0x00, 0x30, 0x01, 0x02, 0x90, 0x01], 0x18 | 0x100),  # eight, one unused; stencil
    ([37, 9, 16], [0x00, 0x00, 0x10], 0x10 | 0x40000 | (6 << 20)),  # a logic op on every 8-bit attachment
]


@pytest.mark.parametrize("case", range(len(MRT_CASES)))
@pytest.mark.parametrize("batched", [False, True])
def test_colour_attachments(gpu_ctx, oracle, monkeypatch, case, batched):
    """Up to eight colour attachments per subpass, each with its own format,
    blend state and write mask, fed by the fragment shader's output at its
    location (LLVMRuntime/PipelineCompiler.cpp:1415-1429): every attachment
    equals the oracle's, per draw and batched."""
    if batched:
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    fmts, blends, variant = MRT_CASES[case]
    scene = c.Scene(c.PROGRAM, 3 + case, [c.PROGRAM_MRT, variant, 64, 48, 24, 0, 0, _pack(fmts), _pack(blends)])
    r = c.Renderer(gpu_ctx, scene)
    try:
        r.render(1)
        gc, gd = r.readback()
        gx = [r.readback_extra(k + 1) for k in range(len(fmts))]
    finally:
        r.close()
    rc, rx, rd, stats = oracle.render_extra(scene)
    assert stats["fragments_written"] > 0
    report = compare(scene, gc, gd, rc, rd)
    assert report["color_pixels_differing"] == 0, report
    for k, (g, o) in enumerate(zip(gx, rx)):
        assert np.count_nonzero(np.any(g != o, axis=-1)) == 0, "attachment %d (format %d)" % (k + 1, fmts[k])


# Integer colour attachments (UINT / SINT): the integer-output program's
# vec4, uvec4(c * 300), ivec4(c * 400 - 200) and floatBitsToUint(c) into
# integer formats of every width, clamped to each channel's range; blend
# states on integer attachments are ignored (Vulkan: integer formats are not
# blended); the render pass clears them with the integers round(clear * 100).
INT_CASES = [
    (37, [41, 42, 98], [0x00, 0x00, 0x00]),
    (99, [81, 75, 13], [0x01, 0x02, 0x30]),
    (42, [20, 82, 99], [0x00, 0x10, 0x00]),
]


@pytest.mark.parametrize("case", range(len(INT_CASES)))
@pytest.mark.parametrize("batched", [False, True])
def test_integer_colour_attachments(gpu_ctx, oracle, monkeypatch, case, batched):
    if batched:
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    fmt0, fmts, blends = INT_CASES[case]
    scene = c.Scene(c.PROGRAM, 7 + case, [c.PROGRAM_MRTI, 0x10, 64, 48, 24, 0, fmt0, _pack(fmts), _pack(blends)])
    r = c.Renderer(gpu_ctx, scene)
    try:
        r.render(1)
        gc, gd = r.readback()
        gx = [r.readback_extra(k + 1) for k in range(len(fmts))]
    finally:
        r.close()
    rc, rx, rd, stats = oracle.render_extra(scene)
    assert stats["fragments_written"] > 0
    assert np.count_nonzero(np.any(gc != rc, axis=-1)) == 0, "attachment 0 (format %d)" % fmt0
    assert np.count_nonzero(np.any(gd != rd, axis=-1)) == 0
    for k, (g, o) in enumerate(zip(gx, rx)):
        assert np.count_nonzero(np.any(g != o, axis=-1)) == 0, "attachment %d (format %d)" % (k + 1, fmts[k])


# Integer formats with 8- and 16-byte texels on the first attachment: the
# MRTI program's location 0 output read as integers (16-bit channels
# clamp, 32-bit channels keep the bits); few triangles, so the integer
# clear stays visible.
WIDE_INT_ATTACHMENTS = [95, 96, 101, 102, 107, 108]


@pytest.mark.parametrize("fmt", WIDE_INT_ATTACHMENTS)
@pytest.mark.parametrize("batched", [False, True])
def test_wide_integer_colour_attachments(gpu_ctx, oracle, monkeypatch, fmt, batched):
    if batched:
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 9, [c.PROGRAM_MRTI, 0x10, 64, 48, 5, 0, fmt, _pack([98]), 0])
    r = c.Renderer(gpu_ctx, scene)
    try:
        r.render(1)
        gc, gd = r.readback()
        g1 = r.readback_extra(1)
    finally:
        r.close()
    rc, rx, rd, stats = oracle.render_extra(scene)
    assert stats["fragments_written"] > 0
    assert gc.shape[-1] == c.colour_texel_bytes(fmt)
    assert np.count_nonzero(np.any(gc != rc, axis=-1)) == 0, "attachment 0 (format %d)" % fmt
    assert np.count_nonzero(np.any(gd != rd, axis=-1)) == 0
    assert np.count_nonzero(np.any(g1 != rx[0], axis=-1)) == 0


# Textures bound other than as one combined image sampler (the reference
# binds SAMPLED_IMAGE, STORAGE_IMAGE and SAMPLER descriptors alike,
# CPVulkan/CommandBuffer.Draw.cpp:356-377): a storage image read with
# imageLoad (OpImageRead), and a sampled image joined with a sampler from
# another binding (OpSampledImage). Nearest filtering with mirrored and
# border addressing, a LOD bias with blending; per draw and batched.
IMAGE_BINDING_VARIANTS = [0x10, 0x10 | 0x4000, 0x10 | 0x8000 | 0x20]


@pytest.mark.parametrize("program", [c.PROGRAM_STORAGE, c.PROGRAM_SEPARATE])
@pytest.mark.parametrize("variant", IMAGE_BINDING_VARIANTS)
@pytest.mark.parametrize("batched", [False, True])
def test_image_bindings(gpu_ctx, oracle, monkeypatch, program, variant, batched):
    if batched:
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 3, [program, variant, 64, 48, 24])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


def test_separate_sampler_equals_combined(gpu_ctx):
    # the same texture and sampler, bound separately or combined
    for variant in IMAGE_BINDING_VARIANTS:
        a, _ = render_gpu(gpu_ctx, c.Scene(c.PROGRAM, 4, [c.PROGRAM_SEPARATE, variant, 64, 48, 24]))
        b, _ = render_gpu(gpu_ctx, c.Scene(c.PROGRAM, 4, [c.PROGRAM_TEXLIT, variant, 64, 48, 24]))
        assert np.array_equal(a, b), hex(variant)


# GLSL.std.450 instructions the reference registers beyond the programs
# above (CPVulkan/GlslFunctions.cpp:36-40, 184-310): NMin / NMax / NClamp
# with a NaN operand, FindSMsb / FindILsb / SSign / FindUMsb on integers
# converted from the colour, Reflect.
@pytest.mark.parametrize("variant", [0x10, 0x10 | 0x20, 0x8 | 0x2])
@pytest.mark.parametrize("batched", [False, True])
def test_glsl_builtins_program(gpu_ctx, oracle, monkeypatch, variant, batched):
    if batched:
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 5, [c.PROGRAM_MATHX, variant, 64, 48, 24])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report


# Function calls (OpFunctionCall): a function that scales the variable it
# is given (a pointer parameter) and returns a value, and one that
# discards; per draw, batched, and under the deferred schedule.
@pytest.mark.parametrize("variant", [0x10, 0x10 | 0x20, 0x8 | 0x2])
@pytest.mark.parametrize("mode", ["plain", "batched", "deferred"])
def test_function_calls_program(gpu_ctx, oracle, monkeypatch, variant, mode):
    if mode == "batched":
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    if mode == "deferred":
        monkeypatch.setenv("CPV_SCHEDULE", "1")
    scene = c.Scene(c.PROGRAM, 6, [c.PROGRAM_CALLS, variant, 64, 48, 24])
    report, stats = check(gpu_ctx, oracle, scene)
    assert 0 < stats["fragments_written"] < stats["fragments"]
    assert report["color_pixels_differing"] == 0, report


# A read-only storage buffer (Uniform storage with BufferBlock, a runtime
# array; bound as STORAGE_BUFFER): the uniform buffer bound again at
# binding 3, its row 1 multiplying the colour.
@pytest.mark.parametrize("batched", [False, True])
def test_storage_buffer_program(gpu_ctx, oracle, monkeypatch, batched):
    if batched:
        monkeypatch.setenv("CPV_BATCH_MIN_DRAWS", "1")
    scene = c.Scene(c.PROGRAM, 7, [c.PROGRAM_SSBO, 0x10 | 0x20, 64, 48, 24])
    report, stats = check(gpu_ctx, oracle, scene)
    assert stats["fragments_written"] > 0
    assert report["color_pixels_differing"] == 0, report

