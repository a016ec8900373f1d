"""vkCmdBlitImage on the device against the oracle's restatement of the
reference blit (CPVulkan/CommandBuffer.cpp:57-232): mip-chain generation
with LINEAR, NEAREST at arbitrary scales, mirrored regions and RGBA8/BGRA8
conversions. The bar is bit-exact bytes."""
import numpy as np
import pytest

import cpvulkan_gb300 as c

pytestmark = pytest.mark.gpu

RGBA8, BGRA8 = 37, 44


def chain_shapes(w, h, levels):
    shapes = []
    for _ in range(levels):
        shapes.append((h, w))
        w, h = max(w // 2, 1), max(h // 2, 1)
    return shapes


def split(packed, shapes):
    out, off = [], 0
    for h, w in shapes:
        out.append(packed[off:off + h * w * 4].reshape(h, w, 4))
        off += h * w * 4
    return out


def random_image(rng, w, h, levels=1):
    n = sum(hh * ww * 4 for hh, ww in chain_shapes(w, h, levels))
    return rng.integers(0, 256, n, dtype=np.uint8)


def check_equal(gpu, ref, what):
    diff = np.any(gpu != ref, axis=-1)
    n = int(diff.sum())
    if n:
        ys, xs = np.nonzero(diff)
        raise AssertionError("%s: %d texels differ, first at (%d, %d): gpu %s oracle %s" %
                             (what, n, xs[0], ys[0], gpu[ys[0], xs[0]].tolist(), ref[ys[0], xs[0]].tolist()))


@pytest.mark.parametrize("w,h,fmt", [(256, 256, RGBA8), (300, 77, RGBA8), (129, 64, BGRA8)])
def test_mip_chain_linear(gpu_ctx, oracle, w, h, fmt):
    """Each level blitted from the one above it, inside one image."""
    rng = np.random.default_rng(w * 7 + h)
    shapes = chain_shapes(w, h, 6)
    img = random_image(rng, w, h, 6)
    regions = []
    for l in range(1, 6):
        (sh, sw), (dh, dw) = shapes[l - 1], shapes[l]
        regions.append((l - 1, 0, 0, sw, sh, l, 0, 0, dw, dh))
    ref = split(img.copy(), shapes)
    for g in regions:
        oracle.blit(ref[g[0]], fmt, ref[g[5]], fmt, g[1:5] + g[6:10], 1)
    gpu = img.copy()
    gpu_ctx.blit(gpu, (w, h), 6, fmt, regions, 1)
    for l, (a, b) in enumerate(zip(split(gpu, shapes), ref)):
        check_equal(a, b, "level %d" % l)


@pytest.mark.parametrize("filter", [0, 1])
@pytest.mark.parametrize("region", [
    (0, 0, 37, 23, 0, 0, 64, 50),       # upscale by a non-integer ratio
    (5, 3, 37, 23, 10, 4, 25, 11),      # downscale of a sub-rectangle
    (0, 0, 37, 23, 64, 0, 0, 50),       # mirrored in x
    (0, 23, 37, 0, 3, 49, 60, 2),       # source flipped in y, destination flipped in y
    (36, 22, 1, 1, 0, 0, 64, 50),       # source reversed in both axes
])
def test_regions(gpu_ctx, oracle, filter, region):
    rng = np.random.default_rng(sum(region) + filter)
    src = random_image(rng, 37, 23)
    dst = random_image(rng, 64, 50)
    ref = dst.copy().reshape(50, 64, 4)
    oracle.blit(src.reshape(23, 37, 4), RGBA8, ref, RGBA8, region, filter)
    gpu = dst.copy()
    g = (0,) + tuple(region[:4]) + (0,) + tuple(region[4:])
    gpu_ctx.blit(src, (37, 23), 1, RGBA8, [g], filter, dst=gpu, dst_size=(64, 50), dst_levels=1, dst_format=RGBA8)
    check_equal(gpu.reshape(50, 64, 4), ref, "region %s" % (region,))


@pytest.mark.parametrize("src_fmt,dst_fmt", [(BGRA8, RGBA8), (RGBA8, BGRA8), (BGRA8, BGRA8)])
def test_format_conversion(gpu_ctx, oracle, src_fmt, dst_fmt):
    rng = np.random.default_rng(src_fmt * 3 + dst_fmt)
    src = random_image(rng, 48, 40)
    dst = random_image(rng, 100, 90, 2)
    shapes = chain_shapes(100, 90, 2)
    ref = split(dst.copy(), shapes)
    regions = [(0, 0, 0, 48, 40, 0, 0, 0, 100, 90), (0, 8, 8, 40, 32, 1, 49, 44, 1, 1)]
    for g in regions:
        oracle.blit(src.reshape(40, 48, 4), src_fmt, ref[g[5]], dst_fmt, g[1:5] + g[6:10], 1)
    gpu = dst.copy()
    gpu_ctx.blit(src, (48, 40), 1, src_fmt, regions, 1, dst=gpu, dst_size=(100, 90), dst_levels=2, dst_format=dst_fmt)
    for l, (a, b) in enumerate(zip(split(gpu, shapes), ref)):
        check_equal(a, b, "level %d" % l)


def test_identity_nearest_is_copy(gpu_ctx):
    rng = np.random.default_rng(5)
    src = random_image(rng, 64, 64)
    dst = np.zeros_like(src)
    gpu_ctx.blit(src, (64, 64), 1, RGBA8, [(0, 0, 0, 64, 64, 0, 0, 0, 64, 64)], 0, dst=dst, dst_size=(64, 64), dst_levels=1,
                 dst_format=RGBA8)
    assert np.array_equal(src, dst)
