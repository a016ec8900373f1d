"""The oracle's MATHX program (no GPU): GLSL.std.450 NClamp with NMin /
NMax against a NaN (CPVulkan/GlslFunctions.cpp:264-310) keeps the red
channel within the clamp; FindUMsb of a 16-bit value stays within 15."""
import numpy as np

import cpvulkan_gb300 as c


def test_mathx_channels_stay_in_their_ranges(oracle):
    scene = c.Scene(c.PROGRAM, 2, [c.PROGRAM_MATHX, 0x10, 64, 48, 24])
    col, _, st = oracle.render(scene)
    assert st["fragments_written"] > 0
    drawn = np.any(col != np.array([64, 128, 191, 255], np.uint8), axis=-1)
    assert drawn.any()
    red = col[drawn][:, 0].astype(np.int64)
    # NClamp to [0.25, 0.75] encodes to [64, 191]; NMin(NaN, r) and NMax(r, NaN) keep r
    assert red.min() >= 64 and red.max() <= 191
    # findMSB of a value in [0, 65535] is at most 15: 15 / 16 encodes to 239
    assert col[drawn][:, 2].max() <= 239
