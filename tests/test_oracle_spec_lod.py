"""The oracle's labelled quad-derivative LOD mode (no GPU).

In this mode (the ICD's CPV_SPEC_LOD=1, cpv_scene.spec_lod for the oracle)
implicit-LOD sampling takes λ_base = log2(max(ρx, ρy)) from fine quad
derivatives of the coordinates (Vulkan 1.1, "Scale Factor Operation") instead
of the reference's λ = 0 (CPVulkan/GlslFunctions.cpp:657-672); bias, clamp
and level selection stay the reference's (CPVulkan/ImageSampler.cpp:562-673).
These tests check the oracle's own log2 series against numpy and relations
between renders in the two modes.
"""
import ctypes

import numpy as np

import cpvulkan_gb300 as c


def _half_log2(oracle, x):
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    fn = oracle.lib.cpv_oracle_half_log2_n
    fn.restype = None
    fn(x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(x.size))
    return out


def test_half_log2_series(oracle):
    rng = np.random.default_rng(3)
    x = np.concatenate([np.exp2(rng.uniform(-140.0, 127.0, 200000)).astype(np.float32),
                        np.float32([1.0, 2.0, 0.5, 4.0, 1.41421356, 0.70710678, 1e-45, 1e-40, 3.4e38])])
    got = _half_log2(oracle, x).astype(np.float64)
    want = 0.5 * np.log2(x.astype(np.float64))
    # a few binary32 roundings of values up to |64|: well below 1e-5 absolute
    assert np.max(np.abs(got - want)) < 1e-5
    # powers of two are exact
    p = np.float32([2.0 ** k for k in range(-149, 128, 3)])
    assert np.array_equal(_half_log2(oracle, p), (0.5 * np.log2(p.astype(np.float64))).astype(np.float32))
    special = _half_log2(oracle, np.float32([0.0, -0.0, -1.0, np.nan, np.inf]))
    assert list(special[:4]) == [-np.inf] * 4 and special[4] == np.inf


def test_quad_lambda_follows_the_scale_factor_definition(oracle):
    # Vulkan 1.1, "Scale Factor Operation": rho_x = |(du/dx * w, dv/dx * h)|,
    # rho_y likewise, lambda_base = log2(max(rho_x, rho_y)); fine
    # derivatives: P(x | 1) - P(x & ~1). numpy in binary64 against the oracle.
    rng = np.random.default_rng(9)
    n = 100000
    u = rng.uniform(-2, 2, n).astype(np.float32)
    v = rng.uniform(-2, 2, n).astype(np.float32)
    scale = np.exp2(rng.uniform(-14, 2, (n, 4))).astype(np.float32) * rng.choice([-1, 1], (n, 4)).astype(np.float32)
    ux, vx, uy, vy = u + scale[:, 0], v + scale[:, 1], u + scale[:, 2], v + scale[:, 3]
    odd = rng.integers(0, 4, n).astype(np.uint32)
    w, h = 1024, 512
    packed = np.ascontiguousarray(np.stack([u, v, ux, vx, uy, vy], axis=1), np.float32)
    out = np.empty(n, np.float32)
    fn = oracle.lib.cpv_oracle_quad_lambda_n
    fn.restype = None
    fn(packed.ctypes.data_as(ctypes.c_void_p), odd.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint32(w), ctypes.c_uint32(h),
       out.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(n))
    sx = np.where(odd & 1, 1.0, -1.0)  # x odd: the neighbour is x - 1
    sy = np.where(odd & 2, 1.0, -1.0)
    f64 = np.float64
    dudx, dvdx = sx * (u.astype(f64) - ux), sx * (v.astype(f64) - vx)
    dudy, dvdy = sy * (u.astype(f64) - uy), sy * (v.astype(f64) - vy)
    rho_x = np.hypot(dudx * w, dvdx * h)
    rho_y = np.hypot(dudy * w, dvdy * h)
    want = np.log2(np.maximum(rho_x, rho_y))
    # binary32 differences and squares: a few ulps of rho, i.e. ~1e-6 in log2
    assert np.max(np.abs(out.astype(f64) - want)) < 2e-5


def _scene(variant=0x10, seed=1, lod_range=None):
    s = c.Scene(c.PROGRAM, seed, [c.PROGRAM_TEXLIT, variant, 64, 48, 24])
    if lod_range is not None:
        hdr = c.SceneHeader.from_address(s.ptr)
        hdr.sampler.min_lod, hdr.sampler.max_lod = lod_range
    return s


def test_spec_lod_changes_minified_pixels(oracle):
    # the scene's texture (64x64, 7 levels) is minified over much of the
    # frame, so quad derivatives select coarser levels there
    for variant in (0x10, 0x10 | 0x4000, 0x10 | 0x8000 | 0x20):
        s = _scene(variant)
        a, da, st = oracle.render(s)
        s.spec_lod = 1
        b, db, st2 = oracle.render(s)
        assert st["fragments_written"] > 0 and st == st2
        assert np.array_equal(da, db)  # depth and coverage do not depend on λ
        assert np.count_nonzero(np.any(a != b, axis=-1)) > st["fragments_written"] // 20


def test_clamped_lod_equals_reference_mode(oracle):
    # with minLod = maxLod the clamp fixes λ in both modes: equal images
    for lod in (0.0, 1.0, 2.5):
        s = _scene(0x10, 2, (lod, lod))
        a, _, _ = oracle.render(s)
        s.spec_lod = 1
        b, _, _ = oracle.render(s)
        assert np.array_equal(a, b), lod


def test_spec_lod_without_texture_sampling_is_unchanged(oracle):
    # programs without implicit-LOD sampling render the same in both modes
    for program, variant in ((c.PROGRAM_CUBE, 0x10), (c.PROGRAM_FETCH, 0x0), (c.PROGRAM_MESHPC, 0x10 | 0x20)):
        s = c.Scene(c.PROGRAM, 3, [program, variant, 64, 48, 24])
        a, _, _ = oracle.render(s)
        s.spec_lod = 1
        b, _, _ = oracle.render(s)
        assert np.array_equal(a, b), program


def test_spec_lod_threaded_equals_single_thread(oracle):
    s = c.Scene(c.HEIGHTFIELD, 1, [128, 480, 270])
    s.spec_lod = 1
    a, da, _ = oracle.render(s)
    b, db, _ = oracle.render_threaded(s, threads=4)
    assert np.array_equal(a, b) and np.array_equal(da, db)
