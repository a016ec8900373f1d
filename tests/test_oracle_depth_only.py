"""Depth-only passes (no colour attachment; variant bit 30 of the PROGRAM
scenes): the oracle runs the same fragment operations without the colour
write, so depth and stencil equal those of the same scene with a colour
attachment, and the colour buffer is left untouched."""
import numpy as np
import pytest

import cpvulkan_gb300 as c

DEPTH_ONLY = 0x40000000


@pytest.mark.parametrize("program,variant", [(c.PROGRAM_CUBE, 0x10), (c.PROGRAM_CUBE, 0x18 | 0x100), (c.PROGRAM_DISCARD, 0x8),
                                             (c.PROGRAM_CUBE, 0x0), (c.PROGRAM_CUBE, 0x10000 | 0x400 | 0x20000 | 0x10)])
def test_depth_only_matches_depth_of_full_pass(native, oracle, program, variant):
    full = c.Scene(c.PROGRAM, 2, [program, variant, 48, 40, 24])
    only = c.Scene(c.PROGRAM, 2, [program, variant | DEPTH_ONLY, 48, 40, 24])
    assert only.color_format == 0 and only.depth_format != 0
    if variant & 0x18 == 0:
        assert only.depth_format == c.VK_FORMAT_D32_SFLOAT  # a depth-only pass needs a depth attachment
        full = c.Scene(c.PROGRAM, 2, [program, variant | 0x10, 48, 40, 24])
    fc, fd, fs = oracle.render(full)
    oc, od, os_ = oracle.render(only)
    assert np.array_equal(fd, od)
    assert not oc.any()
    assert fs["fragments"] == os_["fragments"] and fs["fragments_written"] == os_["fragments_written"]
