"""vkCmdClearColorImage, vkCmdClearDepthStencilImage, vkCmdCopyImage and
vkCmdClearAttachments (CPVulkan/CommandBuffer.Draw.cpp:2142-2224, 2380-2396;
CPVulkan/CommandBuffer.Copy.cpp:1091-1095) on the device, byte for byte
against numpy: colour through the reference's UNORM8 encoder in the
format's byte order, D16 quantised, D32 as its bits, the stencil in the
second word of a D32S8 texel; a clear writes only the aspects it names and
only the levels and rectangles it names."""
import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import encode_colour

pytestmark = pytest.mark.gpu

RGBA, BGRA = 37, 44
COLOR, DEPTH, STENCIL = 1, 2, 4
REMAINING = 0xFFFFFFFF


def chain(w, h, levels, texel):
    out, off = [], 0
    for _ in range(levels):
        out.append((off, w, h))
        off += w * h * texel
        w, h = max(w // 2, 1), max(h // 2, 1)
    return out, off


def level_view(buf, lv, texel):
    off, w, h = lv
    return buf[off:off + w * h * texel].reshape(h, w, texel)


def colour_bytes(oracle, colour, fmt):
    b = [oracle.lib.cpv_oracle_encode_unorm8(float(x)) for x in colour]
    return np.array([b[2], b[1], b[0], b[3]] if fmt == BGRA else b, np.uint8)


def ds_texel(oracle, fmt, depth, stencil):
    if fmt == c.VK_FORMAT_D16_UNORM:
        return np.frombuffer(np.uint16(oracle.lib.cpv_oracle_encode_unorm16(depth)).tobytes(), np.uint8)
    lo = np.frombuffer(np.float32(depth).tobytes(), np.uint8)
    if fmt == c.VK_FORMAT_D32_SFLOAT:
        return lo
    return np.concatenate([lo, np.frombuffer(np.uint32(stencil & 0xFF).tobytes(), np.uint8)])


@pytest.mark.parametrize("fmt", [RGBA, BGRA])
def test_clear_color_image(gpu_ctx, oracle, fmt):
    rng = np.random.default_rng(1)
    levels, (w, h) = 5, (37, 23)
    lv, total = chain(w, h, levels, 4)
    init = rng.integers(0, 256, total, dtype=np.uint8)
    a, b = (0.2, 0.51, 1.3, -0.1), (0.0, 1.0, 0.5, 0.25)
    out = gpu_ctx.image_ops(fmt, (w, h), levels, init, [
        dict(kind=c.OP_CLEAR_COLOR_IMAGE, aspect=COLOR, level=1, level_count=2, colour=a),
        dict(kind=c.OP_CLEAR_COLOR_IMAGE, aspect=COLOR, level=4, level_count=REMAINING, colour=b)])
    want = init.copy()
    for l in (1, 2):
        level_view(want, lv[l], 4)[:] = colour_bytes(oracle, a, fmt)
    level_view(want, lv[4], 4)[:] = colour_bytes(oracle, b, fmt)
    assert np.array_equal(out, want)


@pytest.mark.parametrize("fmt", [c.VK_FORMAT_D16_UNORM, c.VK_FORMAT_D32_SFLOAT, c.VK_FORMAT_D32_SFLOAT_S8_UINT])
def test_clear_depth_stencil_image(gpu_ctx, oracle, fmt):
    texel = c.depth_texel_bytes(fmt)
    rng = np.random.default_rng(2)
    levels, (w, h) = 3, (29, 17)
    lv, total = chain(w, h, levels, texel)
    init = rng.integers(0, 256, total, dtype=np.uint8)
    ops = [dict(kind=c.OP_CLEAR_DEPTH_STENCIL_IMAGE, aspect=DEPTH, level=0, level_count=1, depth=0.625, stencil=9),
           dict(kind=c.OP_CLEAR_DEPTH_STENCIL_IMAGE, aspect=STENCIL, level=1, level_count=1, depth=0.125, stencil=0x1A7),
           dict(kind=c.OP_CLEAR_DEPTH_STENCIL_IMAGE, aspect=DEPTH | STENCIL, level=2, level_count=1, depth=1.0 / 3.0, stencil=200)]
    out = gpu_ctx.image_ops(fmt, (w, h), levels, init, ops)
    want = init.copy()
    l0 = level_view(want, lv[0], texel)
    l0[..., :min(texel, 4)] = ds_texel(oracle, fmt, 0.625, 9)[:min(texel, 4)]
    if texel == 8:  # stencil only: the depth word stays
        level_view(want, lv[1], texel)[..., 4:] = ds_texel(oracle, fmt, 0.125, 0x1A7)[4:]
    level_view(want, lv[2], texel)[:] = ds_texel(oracle, fmt, 1.0 / 3.0, 200)
    assert np.array_equal(out, want)


@pytest.mark.parametrize("fmt", [RGBA, c.VK_FORMAT_D32_SFLOAT_S8_UINT, c.VK_FORMAT_D16_UNORM])
def test_copy_image(gpu_ctx, fmt):
    texel = 4 if fmt == RGBA else c.depth_texel_bytes(fmt)
    rng = np.random.default_rng(3)
    levels, (w, h) = 3, (41, 30)
    lv, total = chain(w, h, levels, texel)
    init0 = rng.integers(0, 256, total, dtype=np.uint8)
    init1 = rng.integers(0, 256, total, dtype=np.uint8)
    aspect = COLOR if fmt == RGBA else DEPTH
    out = gpu_ctx.image_ops(fmt, (w, h), levels, init0, [
        dict(kind=c.OP_COPY_IMAGE, aspect=aspect, src_level=1, src_x=3, src_y=2, level=0, x=5, y=7, w=9, h=6),
        dict(kind=c.OP_COPY_IMAGE, aspect=aspect, src_level=0, src_x=0, src_y=0, level=2, x=0, y=0, w=10, h=7)], init1=init1)
    want = init0.copy()
    level_view(want, lv[0], texel)[7:13, 5:14] = level_view(init1, lv[1], texel)[2:8, 3:12]
    level_view(want, lv[2], texel)[:] = level_view(init1, lv[0], texel)[0:7, 0:10]
    assert np.array_equal(out, want)


@pytest.mark.parametrize("fmt", [RGBA, BGRA, c.VK_FORMAT_D16_UNORM, c.VK_FORMAT_D32_SFLOAT_S8_UINT])
def test_clear_attachments(gpu_ctx, oracle, fmt):
    colour = fmt in (RGBA, BGRA)
    texel = 4 if colour else c.depth_texel_bytes(fmt)
    rng = np.random.default_rng(4)
    levels, (w, h) = 2, (48, 20)
    lv, total = chain(w, h, levels, texel)
    init = rng.integers(0, 256, total, dtype=np.uint8)
    value = (0.9, 0.05, 0.4, 0.7)
    if colour:
        ops = [dict(kind=c.OP_CLEAR_ATTACHMENTS, aspect=COLOR, level=1, x=2, y=3, w=10, h=4, colour=value),
               dict(kind=c.OP_CLEAR_ATTACHMENTS, aspect=COLOR, level=0, x=40, y=0, w=8, h=20, colour=(1, 1, 1, 1))]
    else:
        ops = [dict(kind=c.OP_CLEAR_ATTACHMENTS, aspect=DEPTH | STENCIL, level=1, x=2, y=3, w=10, h=4, depth=0.75, stencil=3),
               dict(kind=c.OP_CLEAR_ATTACHMENTS, aspect=STENCIL if texel == 8 else DEPTH, level=0, x=40, y=0, w=8, h=20, depth=0.5, stencil=77)]
    out = gpu_ctx.image_ops(fmt, (w, h), levels, init, ops)
    want = init.copy()
    if colour:
        level_view(want, lv[1], 4)[3:7, 2:12] = colour_bytes(oracle, value, fmt)
        level_view(want, lv[0], 4)[0:20, 40:48] = colour_bytes(oracle, (1, 1, 1, 1), fmt)
    else:
        level_view(want, lv[1], texel)[3:7, 2:12] = ds_texel(oracle, fmt, 0.75, 3)
        if texel == 8:
            level_view(want, lv[0], texel)[0:20, 40:48, 4:] = ds_texel(oracle, fmt, 0.5, 77)[4:]
        else:
            level_view(want, lv[0], texel)[0:20, 40:48] = ds_texel(oracle, fmt, 0.5, 77)
    assert np.array_equal(out, want)


# Colour formats beyond RGBA8/BGRA8: 1-, 2- and 4-byte texels, UNORM, SNORM
# and float channels, each through the format's own encoder.
OTHER_COLOUR = [9, 16, 38, 70, 77, 83, 100]


@pytest.mark.parametrize("fmt", OTHER_COLOUR)
def test_clear_other_colour_formats(gpu_ctx, fmt):
    texel = c.colour_texel_bytes(fmt)
    rng = np.random.default_rng(6)
    levels, (w, h) = 3, (37, 23)
    lv, total = chain(w, h, levels, texel)
    init = rng.integers(0, 256, total, dtype=np.uint8)
    a, b = (-0.3, 0.6, 1.7, 0.45), (0.1234, -1.5, 0.5, 0.25)
    out = gpu_ctx.image_ops(fmt, (w, h), levels, init, [
        dict(kind=c.OP_CLEAR_COLOR_IMAGE, aspect=COLOR, level=1, level_count=REMAINING, colour=a),
        dict(kind=c.OP_CLEAR_ATTACHMENTS, aspect=COLOR, level=0, x=3, y=2, w=9, h=5, colour=b)])
    want = init.copy()
    for l in (1, 2):
        level_view(want, lv[l], texel)[:] = encode_colour(fmt, a)
    level_view(want, lv[0], texel)[2:7, 3:12] = encode_colour(fmt, b)
    assert np.array_equal(out, want)
