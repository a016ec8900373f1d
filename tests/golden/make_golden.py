"""Generates the golden fixtures of tests/golden/.

kat.npz — known-answer vectors for the oracle's single-step helpers, computed
here by an independent numpy restatement of the reference lines each helper
follows (float32 arithmetic, one rounding per operation, no fused
multiply-add; binary64 where the reference computes in double):

  edge      EdgeFunction, CPVulkan/CommandBuffer.Draw.cpp:410-418
  encode8   UNORM8 store: clamp to [0, 1], * 255, round half away from zero
  encode16  UNORM16 (D16) store, * 65535 (CPVulkanBase/Formats.cpp,
            LLVMRuntime/PipelineCompiler.cpp colour/depth writers)
  decode8   UNORM8 load: u / 255.0f
  sample    wrap (CPVulkan/ImageSampler.cpp:12-38), lerp in double (:51-55),
            SampleImageOfLevel NEAREST/LINEAR with the border table (:403-531),
            SampleImage level selection (:562-673) after the λ clamp of
            ImageSampleExplicitLod (CPVulkan/GlslFunctions.cpp:598-630)
  blend     ApplyBlendFactor / ApplyBlend (CPVulkan/CommandBuffer.Draw.cpp:956-1262)

oracle_scenes.json — regression pins of whole oracle renders of small seeded
scenes (image hashes and fragment statistics). These are produced by the
oracle itself and guard it against unintended change; they are not evidence
of parity with the reference.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
F = np.float32

# ---------------------------------------------------------------- helpers --


def edge(ax, ay, bx, by, cx, cy):
    return (cx - ax) * (by - ay) - (cy - ay) * (bx - ax)


def round_half_away(v):
    """roundf for non-negative float32 values, exactly."""
    fl = np.floor(v)
    return fl + (v - fl >= F(0.5)).astype(F)


def encode(x, maxv):
    v = np.where(np.isnan(x), F(0), x).astype(F)
    v = np.minimum(np.maximum(v, F(0)), F(1)).astype(F)
    return round_half_away((v * F(maxv)).astype(F)).astype(np.uint32)


def decode8(u):
    return (u.astype(F) / F(255)).astype(F)


def wrap(v, size, mode):
    if mode == 0:
        return (v % size + size) % size  # Python % is already non-negative; same result
    if mode == 1:
        two = 2 * size
        n = (v % two + two) % two - size
        return size - 1 - (n if n >= 0 else -(1 + n))
    if mode == 2:
        return min(max(v, 0), size - 1)
    if mode == 3:
        return min(max(v, -1), size)
    if mode == 4:
        return min(max(v if v >= 0 else -(1 + v), 0), size - 1)
    raise ValueError(mode)


BORDER = [(0, 0, 0, 0), (0, 0, 0, 0), (0, 0, 0, 1), (0, 0, 0, 1), (1, 1, 1, 1), (1, 1, 1, 1)]


def texel(levels, level, x, y, border):
    img = levels[level]
    h, w = img.shape[:2]
    if x < 0 or x >= w or y < 0 or y >= h:
        return np.array(BORDER[border], F)
    return decode8(img[y, x])


def lerp(a, b, delta):
    diff = (b - a).astype(F)
    return (a.astype(np.float64) + diff.astype(np.float64) * np.float64(delta)).astype(F)


def sample_level(levels, level, u, v, filt, s):
    h, w = levels[level].shape[:2]
    rng = (w, h)
    coord = (F(u), F(v))
    modes = (s["address_u"], s["address_v"])
    if filt == 0:
        c = [wrap(int(np.floor(coord[i] * F(rng[i]) + F(0))), rng[i], modes[i]) for i in range(2)]
        return texel(levels, level, c[0], c[1], s["border_color"])
    c0, c1, fr = [], [], []
    for i in range(2):
        scaled = F(coord[i] * F(rng[i])) - F(0.5)
        scaled = F(scaled)
        fl = F(np.floor(scaled))
        base = int(fl)
        c1.append(wrap(base + 1, rng[i], modes[i]))
        c0.append(wrap(base, rng[i], modes[i]))
        fr.append(F(scaled - fl))
    b = s["border_color"]
    t00 = texel(levels, level, c0[0], c0[1], b)
    t01 = texel(levels, level, c0[0], c1[1], b)
    t10 = texel(levels, level, c1[0], c0[1], b)
    t11 = texel(levels, level, c1[0], c1[1], b)
    ij0 = lerp(t00, t10, fr[0])
    ij1 = lerp(t01, t11, fr[0])
    return lerp(ij0, ij1, fr[1])


def sample(levels, s, u, v, lod):
    bias = F(min(max(F(s["mip_lod_bias"]) + F(0), F(-32)), F(32)))
    lam = F(F(lod) + bias)
    lam = F(min(max(lam, F(s["min_lod"])), F(s["max_lod"])))
    if lam <= 0:
        return sample_level(levels, 0, u, v, s["mag_filter"], s)
    max_level = F(len(levels) - 1)
    mip = F(min(max(lam, F(0)), max_level))
    if s["mipmap_mode"] == 0:
        real = int(np.ceil(F(mip + F(0.5)))) - 1
        return sample_level(levels, real, u, v, s["min_filter"], s)
    l1 = int(np.floor(mip))
    delta = F(mip - F(l1))
    p1 = sample_level(levels, l1, u, v, s["min_filter"], s)
    if delta == 0:
        return p1
    p2 = sample_level(levels, l1 + 1, u, v, s["min_filter"], s)
    return lerp(p1, p2, delta)


def blend_factor(src, dst, const, cf, af):
    one = F(1)
    table = {
        0: np.zeros(4, F), 1: np.ones(4, F), 2: src.copy(), 3: (one - src).astype(F), 4: dst.copy(), 5: (one - dst).astype(F),
        6: np.full(4, src[3], F), 7: np.full(4, F(one - src[3]), F), 8: np.full(4, dst[3], F), 9: np.full(4, F(one - dst[3]), F),
        10: const.copy(), 11: (one - const).astype(F), 12: np.full(4, const[3], F), 13: np.full(4, F(one - const[3]), F),
    }
    if cf == 14:
        a, b = src[3], F(one - dst[3])
        f = b if b < a else a  # std::min(a, b)
        value = np.array([f, f, f, one], F)
    else:
        value = table[cf]
    if cf != af:
        alpha = {0: F(0), 1: one, 14: one, 2: src[3], 6: src[3], 3: F(one - src[3]), 7: F(one - src[3]), 4: dst[3], 8: dst[3],
                 5: F(one - dst[3]), 9: F(one - dst[3]), 10: const[3], 12: const[3], 11: F(one - const[3]), 13: F(one - const[3])}[af]
        value[3] = alpha
    return value


def blend_op(s, sf, d, df, op):
    a = F(s * sf)
    b = F(d * df)
    if op == 0:
        return F(a + b)
    if op == 1:
        return F(a - b)
    if op == 2:
        return F(b - a)
    if op == 3:
        return d if d < s else s  # glm::min / std::min
    if op == 4:
        return d if s < d else s  # glm::max / std::max
    raise ValueError(op)


def blend(src, dst, const, sc, dc, cop, sa, da, aop):
    sf = blend_factor(src, dst, const, sc, sa)
    df = blend_factor(src, dst, const, dc, da)
    out = np.array([blend_op(src[i], sf[i], dst[i], df[i], cop) for i in range(4)], F)
    if cop != aop:
        out[3] = blend_op(src[3], sf[3], dst[3], df[3], aop)
    return out


# --------------------------------------------------------------- vectors --


def make_kat(rng):
    kat = {}
    # edge: random NDC points, exact-zero (collinear) cases and wide ranges
    n = 2000
    pts = rng.uniform(-1.5, 1.5, size=(n, 6)).astype(F)
    pts[:200, 4:6] = pts[:200, 0:2]                      # c == a
    pts[200:400, 4:6] = pts[200:400, 2:4]                # c == b
    pts[400:600] = (pts[400:600] * F(1e-4)).astype(F)    # tiny triangles
    pts[600:800] = (pts[600:800] * F(1e4)).astype(F)     # huge coordinates
    kat["edge_in"] = pts
    kat["edge_out"] = edge(*[pts[:, i] for i in range(6)]).astype(F)
    # encode / decode
    x = np.concatenate([rng.uniform(-0.5, 1.5, 6000).astype(F), (np.arange(256, dtype=F) / F(255)).astype(F),
                        ((np.arange(512, dtype=F) + F(0.5)) / F(255)).astype(F),
                        ((np.arange(2048, dtype=F) * F(32) + F(0.5)) / F(65535)).astype(F),
                        np.array([np.nan, -0.0, 0.0, 1.0, 1.0000001, -1e-30, np.inf, -np.inf], F)]).astype(F)
    kat["encode_in"] = x
    kat["encode8_out"] = encode(x, 255.0).astype(np.uint8)
    kat["encode16_out"] = encode(x, 65535.0).astype(np.uint16)
    kat["decode8_in"] = np.arange(256, dtype=np.uint8)
    kat["decode8_out"] = decode8(kat["decode8_in"])
    # sampling: 8x8 RGBA8 texture, full chain (8, 4, 2, 1)
    levels = [rng.integers(0, 256, size=(8 >> l, 8 >> l, 4), dtype=np.uint8) for l in range(4)]
    kat["sample_texels"] = np.concatenate([lv.reshape(-1) for lv in levels])
    sin, sout = [], []
    for i in range(2000):
        s = {
            "mag_filter": int(rng.integers(0, 2)), "min_filter": int(rng.integers(0, 2)), "mipmap_mode": int(rng.integers(0, 2)),
            "address_u": int(rng.integers(0, 5)), "address_v": int(rng.integers(0, 5)), "address_w": 0,
            "mip_lod_bias": float(rng.choice([0.0, 0.75, -1.5, 40.0])), "min_lod": float(rng.choice([0.0, 0.5])),
            "max_lod": float(rng.choice([4.0, 1.5, 0.25])), "border_color": int(rng.integers(0, 6)),
        }
        if i % 4 == 0:  # exact texel centres and edges
            u = F((int(rng.integers(-8, 16)) + 0.5 * int(rng.integers(0, 2))) / 8.0)
            v = F((int(rng.integers(-8, 16)) + 0.5 * int(rng.integers(0, 2))) / 8.0)
        else:
            u, v = F(rng.uniform(-1.5, 2.5)), F(rng.uniform(-1.5, 2.5))
        lod = F(rng.choice([0.0, -1.0, 0.3, 1.0, 1.5, 2.7, 3.0, 5.0]))
        out = sample(levels, s, u, v, lod)
        sin.append([s["mag_filter"], s["min_filter"], s["mipmap_mode"], s["address_u"], s["address_v"], s["address_w"],
                    np.float32(s["mip_lod_bias"]).view(np.uint32), np.float32(s["min_lod"]).view(np.uint32),
                    np.float32(s["max_lod"]).view(np.uint32), s["border_color"], u.view(np.uint32), v.view(np.uint32),
                    lod.view(np.uint32)])
        sout.append(out)
    kat["sample_in"] = np.array(sin, np.uint32)
    kat["sample_out"] = np.array(sout, F)
    # blend: every factor pair class and op, random colours
    bin_, bout = [], []
    for i in range(1500):
        sc, dc, sa, da = (int(rng.integers(0, 15)) for _ in range(4))
        if i % 3 == 0:
            sa, da = sc, dc
        cop, aop = int(rng.integers(0, 5)), int(rng.integers(0, 5))
        if i % 2 == 0:
            aop = cop
        src, dst, const = (rng.uniform(0, 1, 4).astype(F) for _ in range(3))
        if i % 7 == 0:
            src = rng.uniform(-0.5, 1.5, 4).astype(F)
        out = blend(src, dst, const, sc, dc, cop, sa, da, aop)
        bin_.append(np.concatenate([src.view(np.uint32), dst.view(np.uint32), const.view(np.uint32),
                                    np.array([sc, dc, cop, sa, da, aop], np.uint32)]))
        bout.append(out)
    kat["blend_in"] = np.array(bin_, np.uint32)
    kat["blend_out"] = np.array(bout, F)
    return kat


SCENES = [
    # name, config, seed, params
    ("cube_frame30", 1, 1, [30]),
    ("heightfield_64", 2, 3, [64, 160, 96]),
    ("blend_300", 3, 4, [300, 160, 96]),
    ("batch_6", 4, 5, [6, 400, 160, 96]),
    ("serve_small", 6, 6, [96, 2000, 2]),
    ("program_texlit_mirror", 5, 7, [1, 0x10 | 0x4000, 48, 40, 12]),
    ("program_cube_stencil", 5, 8, [0, 0x18 | 0x100, 48, 40, 12]),
    ("program_points", 5, 9, [6, 0x10000 | 0x10, 48, 40, 12]),
    ("program_wide_line_strip", 5, 10, [0, 0x10000 | 0x800 | 0x20000 | 0x10, 48, 40, 12]),
    ("program_flatquad_logic_xor", 5, 11, [2, 0x20 | 0x40000 | (6 << 20), 48, 40, 12]),
    ("program_cube_write_mask", 5, 12, [0, 0x10 | 0x80000 | (0x5 << 24), 48, 40, 12]),
    ("program_cube_depth_bounds", 5, 13, [0, 0x18 | 0x100 | (2 << 28), 48, 40, 12]),
    ("program_cube_depth_only", 5, 14, [0, 0x40000000 | 0x18 | 0x100, 48, 40, 12]),
]


def scene_pins():
    sys.path.insert(0, ROOT)
    import cpvulkan_gb300 as c
    from tests import oracle_binding
    c.build()
    oracle = oracle_binding.load()
    pins = {}
    for name, cfg, seed, params in SCENES:
        scene = c.Scene(cfg, seed, params)
        color, depth, st = oracle.render(scene)
        pins[name] = {
            "config": cfg, "seed": seed, "params": params, "triangles": scene.triangles,
            "color_sha256": hashlib.sha256(color.tobytes()).hexdigest(),
            "depth_sha256": hashlib.sha256(depth.tobytes()).hexdigest() if depth is not None else None,
            "stats": {k: int(v) for k, v in st.items()},
        }
    return pins


def main():
    # --scenes-only rewrites the scene pins and leaves kat.npz as it is
    if "--scenes-only" not in sys.argv:
        rng = np.random.default_rng(20261203)
        kat = make_kat(rng)
        np.savez_compressed(os.path.join(HERE, "kat.npz"), **kat)
    with open(os.path.join(HERE, "oracle_scenes.json"), "w") as f:
        json.dump(scene_pins(), f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
