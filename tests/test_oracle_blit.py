"""Known answers of the oracle's blit (CPVulkan/CommandBuffer.cpp:57-232,
sampling as CPVulkan/ImageSampler.cpp:676-681 with CLAMP_TO_EDGE): a
same-size NEAREST blit is a copy, a mirrored one is a flip, an exact 2x
LINEAR reduction is the lerp of lerps at delta 0.5, BGRA8 and RGBA8 swap
red and blue, and texels outside the region are untouched."""
import numpy as np

RGBA8, BGRA8 = 37, 44


def img(seed, h, w):
    return np.random.default_rng(seed).integers(0, 256, (h, w, 4), dtype=np.uint8)


def test_same_size_nearest_is_copy(oracle):
    src = img(1, 19, 23)
    dst = np.zeros_like(src)
    oracle.blit(src, RGBA8, dst, RGBA8, (0, 0, 23, 19, 0, 0, 23, 19), 0)
    assert np.array_equal(src, dst)


def test_mirrored_nearest_is_flip(oracle):
    src = img(2, 16, 20)
    dst = np.zeros_like(src)
    oracle.blit(src, RGBA8, dst, RGBA8, (0, 0, 20, 16, 20, 16, 0, 0), 0)
    assert np.array_equal(dst, src[::-1, ::-1])


def test_half_linear_is_mean_of_quads(oracle):
    src = img(3, 8, 8)
    dst = np.zeros((4, 4, 4), np.uint8)
    oracle.blit(src, RGBA8, dst, RGBA8, (0, 0, 8, 8, 0, 0, 4, 4), 1)
    f = src.astype(np.float64) / 255.0
    top = f[0::2, 0::2] + (f[0::2, 1::2] - f[0::2, 0::2]) * 0.5
    bottom = f[1::2, 0::2] + (f[1::2, 1::2] - f[1::2, 0::2]) * 0.5
    v = top + (bottom - top) * 0.5
    assert np.max(np.abs(dst.astype(np.int32) - np.floor(v * 255.0 + 0.5).astype(np.int32))) <= 1


def test_bgra_rgba_swap(oracle):
    src = img(4, 6, 6)
    dst = np.zeros_like(src)
    oracle.blit(src, BGRA8, dst, RGBA8, (0, 0, 6, 6, 0, 0, 6, 6), 0)
    assert np.array_equal(dst, src[..., [2, 1, 0, 3]])
    back = np.zeros_like(src)
    oracle.blit(dst, RGBA8, back, BGRA8, (0, 0, 6, 6, 0, 0, 6, 6), 0)
    assert np.array_equal(back, src)


def test_outside_region_untouched(oracle):
    src = img(5, 10, 10)
    dst = img(6, 12, 12)
    before = dst.copy()
    oracle.blit(src, RGBA8, dst, RGBA8, (0, 0, 10, 10, 2, 3, 7, 9), 1)
    mask = np.zeros((12, 12), bool)
    mask[3:9, 2:7] = True
    assert np.array_equal(dst[~mask], before[~mask])
    assert not np.array_equal(dst[mask], before[mask])
