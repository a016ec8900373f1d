"""The oracle against the reference's own code (no GPU).

oracle/refpin/extract.py compiles the reference's functions for the parts of
the draw path that are plain C++ (not LLVM-JIT output) from the reference's
files into oracle/_ref/librefpin.so: EdgeFunction, GetFragmentInput with
SetDatum, ApplyBlendFactor / ApplyBlend (CPVulkan/CommandBuffer.Draw.cpp),
wrap, lerp, frac, GetPixelLinear, SampleImageOfLevel and SampleImage
(CPVulkan/ImageSampler.cpp). Each oracle restatement must give the same
bits on about a million seeded and edge-case inputs (NaN compares equal to
NaN). The reference sources exist only on the build machine; without them
the library cannot be built and these tests are skipped.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = "/root/reference"
LIB = os.path.join(ROOT, "oracle", "_ref", "librefpin.so")


@pytest.fixture(scope="module")
def ref():
    if not os.path.isdir(REFERENCE):
        pytest.skip("the reference sources are not on this machine")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], stdout=subprocess.DEVNULL)
    return ctypes.CDLL(LIB)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _same(a, b):
    """Bitwise equality of float arrays, NaN equal to NaN."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    nan = np.isnan(a) & np.isnan(b)
    return (a.view(np.uint32) == b.view(np.uint32)) | nan


def _call(lib, name, *arrays, n):
    fn = getattr(lib, name)
    fn.restype = None
    fn(*[_p(a) if isinstance(a, np.ndarray) else a for a in arrays], ctypes.c_uint64(n))


def _specials(rng, n):
    vals = np.array([0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 1e-38, -1e-38, 1e-45, 3e38, -3e38, np.inf, -np.inf, 1.0 / 3, 2.0 / 3], np.float32)
    return rng.choice(vals, size=n)


def test_edge_function(ref, oracle):
    rng = np.random.default_rng(11)
    n = 1_000_000
    pts = rng.uniform(-2, 2, size=(n, 6)).astype(np.float32)
    pts[: n // 4] = np.round(pts[: n // 4] * 8) / 8                      # grid points: exact zeros and ties
    pts[n // 4: n // 2] *= np.float32(1e-20)                             # tiny magnitudes (underflow, denormals)
    mask = rng.random((n, 6)) < 0.02
    pts[mask] = _specials(rng, int(mask.sum()))
    got = np.zeros(n, np.float32)
    want = np.zeros(2 * n, np.float32)
    _call(oracle.lib, "cpv_oracle_edge_n", pts, got, n=n)
    _call(ref, "cpv_ref_edge_n", pts, want, n=n)
    assert _same(got, want[0::2]).all()
    assert _same(got, want[1::2]).all()


def test_wrap(ref, oracle):
    rng = np.random.default_rng(12)
    n = 1_000_000
    size = rng.integers(1, 70, n).astype(np.int32)
    v = (rng.integers(-4, 5, n) * size + rng.integers(-3, 4, n)).astype(np.int32)
    mode = rng.integers(0, 5, n).astype(np.uint32)
    got, want = np.zeros(n, np.int32), np.zeros(n, np.int32)
    _call(oracle.lib, "cpv_oracle_wrap_n", v, size, mode, got, n=n)
    _call(ref, "cpv_ref_wrap_n", v, size, mode, want, n=n)
    assert np.array_equal(got, want)


def test_blend(ref, oracle):
    rng = np.random.default_rng(13)
    # every colour factor pair x colour op, alpha factors and op random,
    # 60 colour sets each; then 300k fully random cases
    combos = np.array([(s, d, o) for s in range(15) for d in range(15) for o in range(5)], np.uint32)
    per = 60
    n1 = len(combos) * per
    modes = np.zeros((n1, 6), np.uint32)
    modes[:, :3] = np.repeat(combos, per, axis=0)
    modes[:, 3] = rng.integers(0, 15, n1)
    modes[:, 4] = rng.integers(0, 15, n1)
    modes[:, 5] = rng.integers(0, 5, n1)
    n2 = 300_000
    modes2 = np.stack([rng.integers(0, 15, n2), rng.integers(0, 15, n2), rng.integers(0, 5, n2), rng.integers(0, 15, n2),
                       rng.integers(0, 15, n2), rng.integers(0, 5, n2)], axis=1).astype(np.uint32)
    modes = np.ascontiguousarray(np.concatenate([modes, modes2]))
    n = len(modes)
    cols = rng.uniform(0, 1, size=(3, n, 4)).astype(np.float32)
    cols[:, ::7] = rng.uniform(-0.5, 1.5, size=cols[:, ::7].shape)   # out-of-range inputs
    cols[:, ::11] = np.round(cols[:, ::11] * 255) / 255              # UNORM8 values
    src, dst, const = [np.ascontiguousarray(c) for c in cols]
    got, want = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)
    _call(oracle.lib, "cpv_oracle_blend_n", src, dst, const, modes, got, n=n)
    _call(ref, "cpv_ref_blend_n", src, dst, const, modes, want, n=n)
    ok = _same(got, want).all(axis=1)
    assert ok.all(), "%d of %d differ, first modes %s" % ((~ok).sum(), n, modes[~ok][0].tolist())


def test_fragment_input(ref, oracle):
    rng = np.random.default_rng(14)
    n = 1_000_000
    pts = np.zeros((n, 14), np.float32)
    xy = rng.uniform(-1.2, 1.2, size=(n, 3, 2)).astype(np.float32)
    xy[: n // 5] = np.round(xy[: n // 5] * 16) / 16                     # vertices on a grid
    pts[:, 0:12:4] = xy[:, :, 0]
    pts[:, 1:12:4] = xy[:, :, 1]
    pts[:, 2:12:4] = rng.uniform(0, 1, size=(n, 3))
    pts[:, 3:12:4] = rng.uniform(0.05, 20, size=(n, 3))
    # pixel centres: inside the triangle's box, some exactly on a vertex or
    # on a grid line shared with the vertices
    lo, hi = xy.min(axis=1), xy.max(axis=1)
    pts[:, 12:14] = rng.uniform(lo, hi)
    on_vertex = rng.random(n) < 0.05
    pts[on_vertex, 12] = pts[on_vertex, 0]
    pts[on_vertex, 13] = pts[on_vertex, 1]
    grid = rng.random(n) < 0.2
    pts[grid, 12:14] = np.round(pts[grid, 12:14] * 16) / 16
    degenerate = rng.random(n) < 0.01                                   # zero-area triangles
    pts[degenerate, 8:10] = pts[degenerate, 0:2]
    vars_ = rng.uniform(-4, 4, size=(n, 27)).astype(np.float32)
    cull = rng.integers(0, 4, n).astype(np.uint32)
    provoking = rng.integers(0, 3, n).astype(np.uint32)
    got, want = np.zeros((n, 12), np.float32), np.zeros((n, 12), np.float32)
    _call(oracle.lib, "cpv_oracle_fragment_input_n", pts, vars_, cull, provoking, got, n=n)
    _call(ref, "cpv_ref_fragment_input_n", pts, vars_, cull, provoking, want, n=n)
    ok = _same(got, want).all(axis=1)
    assert ok.all(), "%d of %d differ, first %s" % ((~ok).sum(), n, pts[~ok][0].tolist())
    assert 0.1 * n < got[:, 0].sum() < 0.9 * n  # both covered and uncovered cases occur


def test_sample(ref, oracle):
    rng = np.random.default_rng(15)
    w = h = 8
    levels = 4
    tex = rng.integers(0, 256, size=(w * h + 16 + 4 + 1) * 4).astype(np.uint8)
    n = 600_000
    modes = np.stack([rng.integers(0, 2, n), rng.integers(0, 2, n), rng.integers(0, 2, n), rng.integers(0, 5, n), rng.integers(0, 5, n),
                      rng.integers(0, 6, n)], axis=1).astype(np.uint32)
    uvl = np.zeros((n, 3), np.float32)
    uvl[:, :2] = rng.uniform(-2, 3, size=(n, 2))
    uvl[: n // 4, :2] = (np.round(uvl[: n // 4, :2] * 16) + 0.5) / 16   # texel centres and edges
    uvl[:, 2] = rng.choice(np.array([-1, 0, 0.25, 0.5, 1, 1.5, 2, 2.75, 3, 7], np.float32), n)
    got, want = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)
    _call(oracle.lib, "cpv_oracle_sample_n", tex, ctypes.c_uint32(w), ctypes.c_uint32(h), ctypes.c_uint32(levels), modes, uvl, got, n=n)
    _call(ref, "cpv_ref_sample_n", tex, ctypes.c_uint32(w), ctypes.c_uint32(h), ctypes.c_uint32(levels), modes, uvl, want, n=n)
    ok = _same(got, want).all(axis=1)
    assert ok.all(), "%d of %d differ, first %s %s" % ((~ok).sum(), n, modes[~ok][0].tolist(), uvl[~ok][0].tolist())
