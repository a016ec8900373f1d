"""The oracle's point and line rasterisation (CPVulkan/CommandBuffer.Draw.cpp:
1315-1508) against an independent numpy restatement of the same lines: the
number of fragments each seeded scene produces (depth and blending off, so
every covered pixel is one fragment). numpy float32 arithmetic is one IEEE
binary32 operation per array operation, as the reference's scalar code."""
import ctypes

import numpy as np
import pytest

import cpvulkan_gb300 as c

f32 = np.float32


def scene_arrays(scene):
    hdr = c.SceneHeader.from_address(scene.ptr)
    raw = ctypes.string_at(hdr.vertex_data, hdr.vertex_bytes)
    v = np.frombuffer(raw, dtype=np.float32).reshape(-1, 8)
    return hdr, v[:, :4], v[:, 4:]


def draws(vcount):
    # build_program: one draw of every vertex, a second from vertex 3 on
    return [(0, vcount), (3, vcount - 3)] if vcount > 6 else [(0, vcount)]


def ndc_centres(n, extent):
    extent = f32(extent)
    half = (f32(1.0) / extent) * f32(0.5)
    return (np.arange(n, dtype=np.float32) / extent + half) * f32(2.0) - f32(1.0)


def f2i(x):
    return int(np.trunc(np.float64(x))) if np.isfinite(x) else 0


def point_fragments(pos, colour, w, h):
    total = 0
    for p, col in zip(pos, colour):
        wc = f32(p[3])
        nx, ny = f32(p[0]) / wc, f32(p[1]) / wc
        sx = f2i((nx + f32(1)) * f32(0.5) * (f32(w) - f32(1)))
        sy = f2i((ny + f32(1)) * f32(0.5) * (f32(h) - f32(1)))
        size = col[3] * f32(16.0)
        half = f2i(np.ceil(size / f32(2)))
        xs = np.arange(max(0, sx - half), min(w, sx + half + 1))
        ys = np.arange(max(0, sy - half), min(h, sy + half + 1))
        s = f32(0.5) + (xs - sx).astype(np.float32) / size
        t = f32(0.5) + (ys - sy).astype(np.float32) / size
        total += int(((s >= 0) & (s <= 1)).sum()) * int(((t >= 0) & (t <= 1)).sum())
    return total


def edge(a, b, px, py):
    return (px - a[0]) * (b[1] - a[1]) - (py - a[1]) * (b[0] - a[0])


def line_fragments(pos, pairs, w, h, width):
    xf = ndc_centres(w, w)[None, :]
    yf = ndc_centres(h, h)[:, None]
    lw = (f32(width) / f32(w), f32(width) / f32(h))
    total = 0
    for i0, i1 in pairs:
        P = []
        for i in (i0, i1):
            wc = f32(pos[i][3])
            P.append(np.array([f32(pos[i][0]) / wc, f32(pos[i][1]) / wc, f32(pos[i][2]) / wc, wc], dtype=np.float32))
        d = P[1] - P[0]
        sq = d * d
        inv = f32(1.0) / np.sqrt((sq[0] + sq[1]) + (sq[2] + sq[3]))
        dx, dy = d[0] * inv, d[1] * inv
        ox, oy = dy * lw[0], -dx * lw[1]
        c00, c01 = (P[0][0] + ox, P[0][1] + oy), (P[0][0] - ox, P[0][1] - oy)
        c10, c11 = (P[1][0] + ox, P[1][1] + oy), (P[1][0] - ox, P[1][1] - oy)
        with np.errstate(invalid="ignore"):
            inside = (edge(c00, c01, xf, yf) >= 0) & (edge(c11, c10, xf, yf) >= 0) & (edge(c10, c00, xf, yf) >= 0) & (edge(c01, c11, xf, yf) >= 0)
        total += int(inside.sum())
    return total


@pytest.mark.parametrize("seed", [1, 2, 4])
def test_point_fragments(oracle, seed):
    scene = c.Scene(c.PROGRAM, seed, [c.PROGRAM_POINTS, 0x10000, 64, 48, 24])
    hdr, pos, colour = scene_arrays(scene)
    expected = sum(point_fragments(pos[a:a + n], colour[a:a + n], 64, 48) for a, n in draws(len(pos)))
    _, _, stats = oracle.render(scene)
    assert stats["fragments"] == expected > 0


@pytest.mark.parametrize("seed", [1, 2, 4])
@pytest.mark.parametrize("strip,wide", [(False, False), (True, False), (False, True), (True, True)])
def test_line_fragments(oracle, seed, strip, wide):
    variant = 0x10000 | (0x800 if strip else 0x400) | (0x20000 if wide else 0)
    scene = c.Scene(c.PROGRAM, seed, [c.PROGRAM_CUBE, variant, 64, 48, 24])
    hdr, pos, _ = scene_arrays(scene)
    expected = 0
    for a, n in draws(len(pos)):
        idx = list(range(a, a + n))
        pairs = list(zip(idx[:-1], idx[1:])) if strip else list(zip(idx[0::2], idx[1::2]))[: n // 2]
        expected += line_fragments(pos, pairs, 64, 48, 3.5 if wide else 1.0)
    _, _, stats = oracle.render(scene)
    assert stats["fragments"] == expected > 0
