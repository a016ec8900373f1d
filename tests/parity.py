"""Image comparison with the tolerances of the draw path's parity contract:
coverage, stencil and integer formats bit-exact; D16 exact; D32 within 1 ULP;
UNORM colour within 1 LSB per channel. Always reports differing pixels."""
import numpy as np

from cpvulkan_gb300 import VK_FORMAT_D16_UNORM, VK_FORMAT_D32_SFLOAT, VK_FORMAT_D32_SFLOAT_S8_UINT

COLOR_LSB = 1
DEPTH_ULP = 1


def _ordered(bits):
    """Maps float32 bit patterns to integers ordered like the floats (for ULP distance)."""
    b = bits.astype(np.int64)
    return np.where(b & 0x80000000, 0x80000000 - (b & 0x7FFFFFFF), b + 0x80000000)


def compare(scene, gpu_color, gpu_depth, ref_color, ref_depth):
    """Returns a dict of differing-pixel counts; raises AssertionError beyond tolerance."""
    report = {}
    cdiff = np.abs(gpu_color.astype(np.int16) - ref_color.astype(np.int16))
    report["color_pixels_differing"] = int(np.count_nonzero(cdiff.max(axis=2)))
    report["color_max_lsb"] = int(cdiff.max()) if cdiff.size else 0
    fmt = scene.depth_format
    if fmt:
        if fmt == VK_FORMAT_D16_UNORM:
            g = gpu_depth.view(np.uint16)[..., 0]
            r = ref_depth.view(np.uint16)[..., 0]
            report["depth_pixels_differing"] = int(np.count_nonzero(g != r))
            report["depth_max_ulp"] = int(np.abs(g.astype(np.int64) - r.astype(np.int64)).max())
            depth_tol = 0
        else:
            g = gpu_depth[..., :4].copy().view(np.uint32)[..., 0]
            r = ref_depth[..., :4].copy().view(np.uint32)[..., 0]
            ulp = np.abs(_ordered(g) - _ordered(r))
            report["depth_pixels_differing"] = int(np.count_nonzero(g != r))
            report["depth_max_ulp"] = int(ulp.max())
            depth_tol = DEPTH_ULP
        if fmt == VK_FORMAT_D32_SFLOAT_S8_UINT:
            report["stencil_pixels_differing"] = int(np.count_nonzero(gpu_depth[..., 4] != ref_depth[..., 4]))
            assert report["stencil_pixels_differing"] == 0, report
        assert report["depth_max_ulp"] <= depth_tol, report
    assert report["color_max_lsb"] <= COLOR_LSB, report
    return report


def unorm(x, bits):
    """numpy restatement of the UNORM encoder: clamp to [0, 1] (NaN → 0),
    scale in float32, round half away from zero."""
    m = np.float32(2 ** bits - 1)
    v = np.clip(np.nan_to_num(np.asarray(x, np.float32), nan=0.0), 0, 1).astype(np.float32) * m
    return np.floor(v + np.float32(0.5)).astype(np.int64)


def snorm(x, bits):
    """numpy restatement of the SNORM encoder: clamp to [-1, 1], scale in
    float32, round half away from zero."""
    m = np.float32(2 ** (bits - 1) - 1)
    v = np.clip(np.asarray(x, np.float32), -1, 1).astype(np.float32) * m
    return (np.sign(v) * np.floor(np.abs(v) + np.float32(0.5))).astype(np.int64)


def encode_colour(fmt, colour):
    """The texel bytes of an RGBA float colour in a colour attachment format."""
    x = np.asarray(colour, np.float32)
    if fmt in (37, 44):
        b = unorm(x, 8).astype(np.uint8)
        return b[[2, 1, 0, 3]] if fmt == 44 else b
    return np.frombuffer({9: lambda: unorm(x[:1], 8).astype(np.uint8).tobytes(),
                          16: lambda: unorm(x[:2], 8).astype(np.uint8).tobytes(),
                          38: lambda: snorm(x, 8).astype(np.int8).tobytes(),
                          70: lambda: unorm(x[:1], 16).astype(np.uint16).tobytes(),
                          77: lambda: unorm(x[:2], 16).astype(np.uint16).tobytes(),
                          83: lambda: x[:2].astype(np.float16).tobytes(),
                          100: lambda: x[:1].tobytes()}[fmt](), np.uint8)
