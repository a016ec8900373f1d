"""The oracle's colour attachments after the first (CPU): each attachment
receives the fragment shader's output at its location, through its own
format, blend state and write mask."""
import numpy as np

import cpvulkan_gb300 as c


def _pack(values):
    out = 0
    for k, v in enumerate(values):
        out |= int(v) << (8 * k)
    return out


def test_first_attachment_equals_single_attachment_render(oracle):
    # the MRT program's location 0 is the cube program's output
    mrt = c.Scene(c.PROGRAM, 2, [c.PROGRAM_MRT, 0x10 | 0x20, 64, 48, 24, 0, 0, _pack([83, 9]), _pack([0x01, 0x00])])
    cube = c.Scene(c.PROGRAM, 2, [c.PROGRAM_CUBE, 0x10 | 0x20, 64, 48, 24])
    col, extras, dep, st = oracle.render_extra(mrt)
    col0, dep0, st0 = oracle.render(cube)
    assert np.array_equal(col, col0) and np.array_equal(dep, dep0)
    assert st["fragments_written"] == st0["fragments_written"] > 0
    assert [e.shape[-1] for e in extras] == [4, 1]


def test_float_attachments_follow_their_outputs(oracle):
    # every attachment R32_SFLOAT, no blending: location 1 holds 1 - c.r and
    # location 3 c.r * 0.5 (exact in binary32), location 0 c.r
    scene = c.Scene(c.PROGRAM, 5, [c.PROGRAM_MRT, 0x10, 64, 48, 24, 0, 100, _pack([100, 100, 100]), 0])
    col, extras, _, st = oracle.render_extra(scene)
    r0 = col.view(np.float32)[..., 0]
    r1 = extras[0].view(np.float32)[..., 0]
    r3 = extras[2].view(np.float32)[..., 0]
    clear = np.float32(-0.3)
    drawn = r0 != clear
    assert drawn.any()
    assert np.array_equal(r1[drawn], np.float32(1.0) - r0[drawn])
    assert np.array_equal(r3[drawn], r0[drawn] * np.float32(0.5))
    assert np.all(r1[~drawn] == clear) and np.all(r3[~drawn] == clear)


def test_write_mask_and_unused_reference(oracle):
    # attachment 2 unused (zeros), attachment 1 with a green-only write mask
    # keeps the clear colour's other channels
    scene = c.Scene(c.PROGRAM, 6, [c.PROGRAM_MRT, 0x10, 64, 48, 24, 0, 0, _pack([37, 0, 37]), _pack([0x20, 0x00, 0x00])])
    col, extras, _, _ = oracle.render_extra(scene)
    assert not extras[1].any()
    m = extras[0]
    assert np.all(m[..., [0, 2, 3]] == np.array([64, 191, 255], np.uint8))  # clear (0.25, 0.5, 0.75, 1) encoded, kept
    assert (m[..., 1] != 128).any()  # green written somewhere


def test_integer_attachments_hold_the_outputs_bits(oracle):
    # R32_SFLOAT at location 0 (c.r), R32_UINT at location 1 (uint(c.r * 300))
    # and location 3 (floatBitsToUint(c).r): exact relations between them
    scene = c.Scene(c.PROGRAM, 3, [c.PROGRAM_MRTI, 0x10, 64, 48, 24, 0, 100, _pack([98, 99, 98]), 0])
    col, extras, _, _ = oracle.render_extra(scene)
    f0 = col.view(np.float32)[..., 0]
    u1 = extras[0].view(np.uint32)[..., 0]
    i2 = extras[1].view(np.int32)[..., 0]
    u3 = extras[2].view(np.uint32)[..., 0]
    drawn = f0 != np.float32(-0.3)
    assert drawn.any()
    assert np.array_equal(u3[drawn], col.view(np.uint32)[..., 0][drawn])
    assert np.array_equal(u1[drawn], (f0[drawn] * np.float32(300.0)).astype(np.uint32))
    assert np.array_equal(i2[drawn], (f0[drawn] * np.float32(400.0) - np.float32(200.0)).astype(np.int32))
    # cleared pixels hold the integer clear: round(-0.3 * 100) = -30
    assert np.all(i2[~drawn] == -30) and np.all(u1[~drawn] == np.uint32(2**32 - 30))


def test_integer_channels_clamp(oracle):
    # 8-bit UINT and SINT channels clamp uint(c * 300) to 255 and
    # int(c * 400 - 200) to [-128, 127]
    scene = c.Scene(c.PROGRAM, 4, [c.PROGRAM_MRTI, 0x10, 64, 48, 24, 0, 100, _pack([41, 42]), 0])
    col, extras, _, _ = oracle.render_extra(scene)
    f0 = col.view(np.float32)[..., 0]
    drawn = f0 != np.float32(-0.3)
    r1 = extras[0][..., 0][drawn].astype(np.int64)
    r2 = extras[1][..., 0][drawn].view(np.int8).astype(np.int64)
    want1 = np.minimum((f0[drawn] * np.float32(300.0)).astype(np.int64), 255)
    want2 = np.clip((f0[drawn] * np.float32(400.0) - np.float32(200.0)).astype(np.int64), -128, 127)
    assert np.array_equal(r1, want1) and np.array_equal(r2, want2)
    assert (want1 == 255).any() and (want2 == 127).any() and (want2 == -128).any()


def _render0(oracle, program, fmt, seed=7, tris=5):
    scene = c.Scene(c.PROGRAM, seed, [program, 0x10, 64, 48, tris, 0, fmt, 0, 0])
    col, _, _, st = oracle.render_extra(scene)
    assert col.shape == (48, 64, c.colour_texel_bytes(fmt))
    return col, st


def test_wide_float_attachments_narrow_the_same_outputs(oracle):
    # R32G32B32A32_SFLOAT holds the outputs as they are; R32G32_SFLOAT its
    # first two channels; R16G16B16A16_SFLOAT them narrowed to binary16
    # (round to nearest even) and R16G16B16A16_UNORM them clamped and scaled
    f32, st = _render0(oracle, c.PROGRAM_CUBE, 109)
    f32 = f32.view(np.float32)
    g32, _ = _render0(oracle, c.PROGRAM_CUBE, 103)
    h16, _ = _render0(oracle, c.PROGRAM_CUBE, 97)
    u16, _ = _render0(oracle, c.PROGRAM_CUBE, 91)
    assert st["fragments_written"] > 0
    assert np.array_equal(g32.view(np.float32), f32[..., :2])
    assert np.array_equal(h16.view(np.float16), f32.astype(np.float16))
    drawn = np.any(f32 != f32[0, 0], axis=-1)
    assert drawn.any() and not drawn.all()
    from tests.parity import unorm
    assert np.array_equal(u16.view(np.uint16)[drawn].astype(np.int64), unorm(f32[drawn], 16))


def test_wide_integer_attachments_keep_or_clamp_the_bits(oracle):
    # the MRTI program's location 0 is a float vector: 32-bit integer
    # channels keep its bits, 16-bit UINT channels clamp them to 65535 and
    # SINT ones to [-32768, 32767]; the clear (-0.3, 0.6, 1.7, 0.45) is
    # stored as round(clear * 100)
    raw, _ = _render0(oracle, c.PROGRAM_MRTI, 109)
    f32, bits = raw.view(np.float32), raw.view(np.uint32)
    u128, _ = _render0(oracle, c.PROGRAM_MRTI, 107)
    s64, _ = _render0(oracle, c.PROGRAM_MRTI, 102)
    u16, _ = _render0(oracle, c.PROGRAM_MRTI, 95)
    s16, _ = _render0(oracle, c.PROGRAM_MRTI, 96)
    clear = np.array([-0.3, 0.6, 1.7, 0.45], np.float32)
    drawn = np.any(f32 != clear, axis=-1)
    assert drawn.any() and not drawn.all()
    assert np.array_equal(u128.view(np.uint32)[drawn], bits[drawn])
    assert np.array_equal(s64.view(np.uint32)[drawn], bits[drawn][:, :2])
    assert np.array_equal(u16.view(np.uint16)[drawn].astype(np.int64), np.minimum(bits[drawn].astype(np.int64), 65535))
    s = bits[drawn].view(np.int32).astype(np.int64)
    assert np.array_equal(s16.view(np.int16)[drawn].astype(np.int64), np.clip(s, -32768, 32767))
    assert np.all(u128.view(np.int32)[~drawn] == [-30, 60, 170, 45]) and np.all(s16.view(np.int16)[~drawn] == [-30, 60, 170, 45])
    assert np.all(u16.view(np.uint16)[~drawn] == [65535, 60, 170, 45])

