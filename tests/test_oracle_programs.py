"""Relations between the oracle's programs (no GPU): the same texture
through a separate sampler renders as through a combined one, and the
storage-buffer program is the cube program's colour times row 1 of the
buffer (the uniform buffer bound again), one binary32 multiply per channel."""
import ctypes

import numpy as np

import cpvulkan_gb300 as c


def test_separate_sampler_renders_as_combined(oracle):
    for variant in (0x10, 0x10 | 0x4000, 0x10 | 0x8000 | 0x20):
        a, da, _ = oracle.render(c.Scene(c.PROGRAM, 3, [c.PROGRAM_SEPARATE, variant, 64, 48, 24]))
        b, db, _ = oracle.render(c.Scene(c.PROGRAM, 3, [c.PROGRAM_TEXLIT, variant, 64, 48, 24]))
        assert np.array_equal(a, b) and np.array_equal(da, db)


def test_storage_buffer_program_scales_the_colour(oracle):
    # R32_SFLOAT attachment (parameter 6 = 100) keeps the first channel exact
    ssbo = c.Scene(c.PROGRAM, 4, [c.PROGRAM_SSBO, 0x10, 64, 48, 24, 0, 100])
    cube = c.Scene(c.PROGRAM, 4, [c.PROGRAM_CUBE, 0x10, 64, 48, 24, 0, 100])
    hdr = c.SceneHeader.from_address(ssbo.ptr)
    assert hdr.uniform_as_storage == 1 and hdr.uniform_bytes >= 32
    row = np.ctypeslib.as_array(ctypes.cast(hdr.uniform_data, ctypes.POINTER(ctypes.c_float)), shape=(8,))[4:8].copy()
    a, da, st = oracle.render(ssbo)
    b, db, _ = oracle.render(cube)
    assert st["fragments_written"] > 0 and np.array_equal(da, db)
    fa, fb = a.view(np.float32)[..., 0], b.view(np.float32)[..., 0]
    clear = np.float32(-0.3)
    drawn = fb != clear
    assert drawn.any()
    assert np.array_equal(fa[drawn], fb[drawn] * row[0])
