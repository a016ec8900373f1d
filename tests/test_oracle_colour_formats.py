"""The oracle's colour attachment formats (the reference's encoder,
LLVMRuntime/ImageCompiler.cpp:1077-1185, and decoder, :161-230): one seeded
scene rendered into each format must agree, channel by channel, with its
render into R32_SFLOAT (the shader's colour as stored) run through numpy's
own UNORM / SNORM / binary16 conversions, and the clear colour must be
stored through the same encoders."""
import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import encode_colour, snorm, unorm

W = H = 48
# CUBE program, depth-tested, with a half-float colour attribute whose
# channels reach [-2, 2] (so the encoders clamp); cleared to (-0.3, 0.6, 1.7, 0.45)
CLEAR = np.array([-0.3, 0.6, 1.7, 0.45], np.float32)


def render(oracle, fmt, variant=0x10, attribute=97):
    colour, _, stats = oracle.render(c.Scene(c.PROGRAM, 3, [c.PROGRAM_CUBE, variant, W, H, 24, attribute, fmt]))
    return colour, stats


@pytest.fixture(scope="module")
def reference_channels(oracle):
    """The red channel the fragment shader wrote, as R32_SFLOAT stores it."""
    colour, stats = render(oracle, 100)
    assert stats["fragments_written"] > 200
    return colour.view(np.float32)[..., 0]


@pytest.mark.parametrize("fmt,kind,bits", [(9, "u", 8), (16, "u", 8), (70, "u", 16), (77, "u", 16), (38, "s", 8), (83, "f", 16)])
def test_red_channel_is_the_encoded_float(oracle, reference_channels, fmt, kind, bits):
    colour, _ = render(oracle, fmt)
    red = reference_channels
    if kind == "f":
        got = colour.view(np.uint16)[..., 0]
        assert np.array_equal(got, red.astype(np.float16).view(np.uint16))
        return
    dtype = {("u", 8): np.uint8, ("u", 16): np.uint16, ("s", 8): np.int8}[(kind, bits)]
    got = colour.view(dtype)[..., 0].astype(np.int64)
    want = unorm(red, bits) if kind == "u" else snorm(red, bits)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("fmt", [9, 16, 38, 70, 77, 83, 100])
def test_clear_colour_encoded(oracle, fmt):
    colour, _, _ = oracle.render(c.Scene(c.PROGRAM, 3, [c.PROGRAM_CUBE, 0x10, W, H, 24, 97, fmt]), draw_end=0)
    texel = colour[0, 0]
    assert (colour == texel).all()
    want = encode_colour(fmt, CLEAR).tobytes()
    assert texel.tobytes() == want


def test_two_channel_formats_agree(oracle):
    """R8G8 and R16G16 UNORM hold the same two channels at different widths;
    R16G16_SFLOAT's channels, encoded to 8 and 16 bits, give both."""
    rg8, _ = render(oracle, 16)
    rg16, _ = render(oracle, 77)
    rgh, _ = render(oracle, 83)
    f = rgh.view(np.float16).astype(np.float32)
    # half-float rounding can move a value across an 8-bit rounding boundary
    assert np.abs(unorm(f, 8) - rg8.astype(np.int64)).max() <= 1
    assert np.abs(unorm(f, 16) - rg16.view(np.uint16).astype(np.int64)).max() <= 40


@pytest.mark.parametrize("fmt", [9, 38, 77, 83])
def test_write_mask_keeps_absent_and_masked_channels(oracle, fmt):
    """Mask 0 leaves the cleared image; a blended pass into a format
    without alpha reads the destination alpha as 1."""
    none, _, _ = oracle.render(c.Scene(c.PROGRAM, 3, [c.PROGRAM_CUBE, 0x10 | 0x80000, W, H, 24, 97, fmt]))
    cleared, _, _ = oracle.render(c.Scene(c.PROGRAM, 3, [c.PROGRAM_CUBE, 0x10, W, H, 24, 97, fmt]), draw_end=0)
    assert np.array_equal(none, cleared)
    blended, stats = render(oracle, fmt, variant=0x10 | 0x20)
    assert stats["fragments_written"] > 200
    assert not np.array_equal(blended, cleared)
