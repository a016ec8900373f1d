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
