"""The oracle's logic operations and colour write mask (Vulkan 1.1, "Logical
Operations" and "Color Write Mask"; the reference aborts on both,
LLVMRuntime/PipelineCompiler.cpp:1687-1700): the 16 operations against the
specification's table, and relations between renders of one seeded scene
under different operations and masks."""
import numpy as np
import pytest

import cpvulkan_gb300 as c

# Vulkan 1.1, table "Logical Operations": VkLogicOp value -> s op d
VK_LOGIC = [lambda s, d: 0, lambda s, d: s & d, lambda s, d: s & ~d, lambda s, d: s, lambda s, d: ~s & d, lambda s, d: d,
            lambda s, d: s ^ d, lambda s, d: s | d, lambda s, d: ~(s | d), lambda s, d: ~(s ^ d), lambda s, d: ~d,
            lambda s, d: s | ~d, lambda s, d: ~s, lambda s, d: ~s | d, lambda s, d: ~(s & d), lambda s, d: 0xFF]
CLEAR, COPY, NO_OP, INVERT, COPY_INVERTED, AND, OR, SET = 0, 3, 5, 10, 12, 1, 7, 15

# (program, variant): a depth-tested interpolated cube mesh, flat-shaded
# src-over quads, and the same quads into B8G8R8A8
SCENES = [(c.PROGRAM_CUBE, 0x10), (c.PROGRAM_FLATQUAD, 0x20), (c.PROGRAM_FLATQUAD, 0x20 | 0x200)]


def logic(op):
    return 0x40000 | (op << 20)


def mask(m):
    return 0x80000 | (m << 24)


def render(oracle, program, variant, size=48, prims=24):
    colour, depth, _ = oracle.render(c.Scene(c.PROGRAM, 5, [program, variant, size, size, prims]))
    return colour.reshape(size, size, 4), depth


def test_logic_op_table(oracle):
    rng = np.random.default_rng(7)
    pairs = rng.integers(0, 256, size=(64, 2))
    for op in range(16):
        for s, d in pairs:
            assert oracle.lib.cpv_oracle_logic_op(op, int(s), int(d)) == VK_LOGIC[op](int(s), int(d)) & 0xFF, (op, s, d)


@pytest.mark.parametrize("program,variant", SCENES)
def test_write_mask_keeps_the_stored_channels(native, oracle, program, variant):
    full, depth = render(oracle, program, variant)
    none, depth_none = render(oracle, program, variant | mask(0))
    assert (depth is None and depth_none is None) or np.array_equal(depth, depth_none)
    # B8G8R8A8 stores R, G, B, A at byte offsets 2, 1, 0, 3
    offsets = [2, 1, 0, 3] if variant & 0x200 else [0, 1, 2, 3]
    for m in (0x1, 0x6, 0x8, 0xB):
        part, _ = render(oracle, program, variant | mask(m))
        for comp in range(4):
            ref = full if (m >> comp) & 1 else none
            assert np.array_equal(part[..., offsets[comp]], ref[..., offsets[comp]]), (m, comp)
    assert not np.array_equal(full, none)


@pytest.mark.parametrize("program,variant", SCENES)
def test_logic_op_relations(native, oracle, program, variant):
    base = variant & ~0x20  # a logic op turns blending off: COPY is the unblended render
    opaque, _ = render(oracle, program, base)
    clear, _ = render(oracle, program, base | mask(0))
    res = {op: render(oracle, program, variant | logic(op))[0] for op in (CLEAR, COPY, NO_OP, INVERT, COPY_INVERTED, AND, OR, SET)}
    written = (res[SET] == 255).all(axis=-1)
    assert written.any() and not (clear == 255).all(axis=-1).any()
    assert np.array_equal(res[COPY], opaque)
    assert np.array_equal(res[NO_OP], clear)
    assert np.array_equal(res[COPY_INVERTED][written], 255 - res[COPY][written])
    assert np.array_equal(res[COPY_INVERTED][~written], clear[~written])
    assert (res[CLEAR][written] == 0).all() and np.array_equal(res[CLEAR][~written], clear[~written])
    inv = res[INVERT]
    assert ((inv == clear) | (inv == 255 - clear)).all()
    assert not (res[AND] & ~clear).any()
    assert np.array_equal(res[OR] & clear, clear)
    # a logic op and a write mask: the masked-out channels keep the clear value
    part, _ = render(oracle, program, variant | logic(COPY_INVERTED) | mask(0x5))
    offsets = [2, 1, 0, 3] if variant & 0x200 else [0, 1, 2, 3]
    for comp in range(4):
        ref = res[COPY_INVERTED] if (0x5 >> comp) & 1 else clear
        assert np.array_equal(part[..., offsets[comp]], ref[..., offsets[comp]])


def bounds(mode):
    return mode << 28


@pytest.mark.parametrize("program,variant", [(c.PROGRAM_CUBE, 0x10), (c.PROGRAM_CUBE, 0x18 | 0x100), (c.PROGRAM_FLATQUAD, 0x8 | 0x20)])
def test_depth_bounds_relations(native, oracle, program, variant):
    """The depth bounds test (LLVMRuntime/PipelineCompiler.cpp:1128-1166)
    compares the stored depth: bounds [0, 1] change nothing; bounds [0.8, 1]
    reject every fragment of a target cleared to depth 0.75, which then keeps
    its clear colour, depth and stencil; bounds [0.3, 1] stop a pixel from
    changing once its stored depth falls below 0.3."""
    off_c, off_d = render(oracle, program, variant)
    full_c, full_d = render(oracle, program, variant | bounds(1))
    assert np.array_equal(off_c, full_c) and np.array_equal(off_d, full_d)
    none_c, none_d = render(oracle, program, variant | bounds(3))
    clear_c, clear_d = render(oracle, program, variant | bounds(3) | mask(0))
    assert np.array_equal(none_c, clear_c) and np.array_equal(none_d, clear_d)
    assert not np.array_equal(off_c, none_c)
    # bounds [0.3, 1]: a pixel that ends unlike the unbounded render was
    # frozen by a stored depth below 0.3
    part_c, part_d = render(oracle, program, variant | bounds(2))
    if part_d.shape[-1] == 2:
        stored = part_d.view(np.uint16)[..., 0] / np.float32(65535)
    else:
        stored = np.ascontiguousarray(part_d[..., :4]).view(np.float32)[..., 0]
    changed = (part_c != off_c).any(axis=-1) | (part_d != off_d).any(axis=-1)
    assert (stored[changed] < 0.3).all()
