"""The CPU oracle against the golden fixtures (no GPU).

kat.npz holds known-answer vectors from an independent numpy restatement of
the reference lines each oracle helper follows (tests/golden/make_golden.py);
every value must match bit for bit. oracle_scenes.json pins whole renders of
small seeded scenes.
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.oracle_binding import SamplerDesc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def kat():
    return dict(np.load(os.path.join(GOLDEN, "kat.npz")))


def _bits(x):
    return np.asarray(x, np.float32).view(np.uint32)


def test_edge_function(oracle, kat):
    pts, want = kat["edge_in"], kat["edge_out"]
    got = np.array([oracle.lib.cpv_oracle_edge(*map(float, p)) for p in pts], np.float32)
    assert np.array_equal(_bits(got), _bits(want))


def test_unorm_encode_decode(oracle, kat):
    x = kat["encode_in"]
    e8 = np.array([oracle.lib.cpv_oracle_encode_unorm8(float(v)) for v in x], np.uint8)
    e16 = np.array([oracle.lib.cpv_oracle_encode_unorm16(float(v)) for v in x], np.uint16)
    assert np.array_equal(e8, kat["encode8_out"])
    assert np.array_equal(e16, kat["encode16_out"])
    d8 = np.array([oracle.lib.cpv_oracle_decode_unorm8(int(u)) for u in kat["decode8_in"]], np.float32)
    assert np.array_equal(_bits(d8), _bits(kat["decode8_out"]))
    # round trip of every UNORM8 code
    assert np.array_equal(np.array([oracle.lib.cpv_oracle_encode_unorm8(float(v)) for v in d8], np.uint8), kat["decode8_in"])


def test_image_sampler(oracle, kat):
    tex = np.ascontiguousarray(kat["sample_texels"])
    out = (ctypes.c_float * 4)()
    bad = []
    for row, want in zip(kat["sample_in"], kat["sample_out"]):
        f = row[[6, 7, 8, 10, 11, 12]].view(np.float32)
        s = SamplerDesc(int(row[0]), int(row[1]), int(row[2]), int(row[3]), int(row[4]), int(row[5]), float(f[0]), float(f[1]),
                        float(f[2]), int(row[9]))
        oracle.lib.cpv_oracle_sample(tex.ctypes.data, 8, 8, 4, ctypes.byref(s), float(f[3]), float(f[4]), float(f[5]), ctypes.byref(out))
        if not np.array_equal(_bits(np.array(out[:], np.float32)), _bits(want)):
            bad.append((row.tolist(), out[:], want.tolist()))
    assert not bad, "%d of %d samples differ, first: %s" % (len(bad), len(kat["sample_in"]), bad[0])


def test_blend_equations(oracle, kat):
    F4 = ctypes.c_float * 4
    out = F4()
    bad = 0
    for row, want in zip(kat["blend_in"], kat["blend_out"]):
        src, dst, const = (F4(*row[k:k + 4].view(np.float32).tolist()) for k in (0, 4, 8))
        ops = [int(v) for v in row[12:18]]
        oracle.lib.cpv_oracle_blend(ctypes.byref(src), ctypes.byref(dst), ctypes.byref(const), *ops, ctypes.byref(out))
        bad += not np.array_equal(_bits(np.array(out[:], np.float32)), _bits(want))
    assert bad == 0


def _pins():
    with open(os.path.join(GOLDEN, "oracle_scenes.json")) as f:
        return sorted(json.load(f).items())


@pytest.mark.parametrize("name,pin", _pins(), ids=[n for n, _ in _pins()])
def test_oracle_scene_pins(native, oracle, name, pin):
    scene = c.Scene(pin["config"], pin["seed"], pin["params"])
    assert scene.triangles == pin["triangles"]
    color, depth, st = oracle.render(scene)
    assert {k: int(v) for k, v in st.items()} == pin["stats"]
    assert hashlib.sha256(color.tobytes()).hexdigest() == pin["color_sha256"]
    if pin["depth_sha256"] is not None:
        assert hashlib.sha256(depth.tobytes()).hexdigest() == pin["depth_sha256"]


def test_oracle_draw_ranges_compose(native, oracle):
    """Rendering draws [0, k) then [k, n) onto the same attachments equals
    rendering [0, n) at once (the API-order property the binning keeps)."""
    scene = c.Scene(c.BATCH, 11, [6, 300, 128, 80])
    full_c, full_d, _ = oracle.render(scene)
    part_c, part_d, _ = oracle.render(scene, 0, 3)
    part_c, part_d, _ = oracle.render(scene, 3, None, color=part_c, depth=part_d, clear=False)
    assert np.array_equal(full_c, part_c) and np.array_equal(full_d, part_d)
