"""One-triangle coverage known-answer cases: hand-placed triangles on 8 x 8
and 16 x 16 targets (vertices on pixel centres, shared edges, both windings
under every cull mode, a degenerate triangle, one reaching off screen), with
an independent numpy restatement of the reference's coverage rule
(CPVulkan/CommandBuffer.Draw.cpp:410-418 EdgeFunction, 874-904
GetFragmentInput, 1510-1594 ProcessTriangles) in float32, one IEEE
operation per array operation.

A case is rendered as the PROGRAM scene of the CUBE program (identity MVP,
w = 1, one draw of the case's vertices) with its seeded vertices replaced by
the case's, in red over the scene's clear colour; no depth attachment."""
import ctypes

import numpy as np

import cpvulkan_gb300 as c

f32 = np.float32


def centre(i, extent):
    """NDC of pixel i's centre: (i / extent + (1 / extent) * 0.5) * 2 - 1."""
    extent = f32(extent)
    return (f32(i) / extent + (f32(1) / extent) * f32(0.5)) * f32(2) - f32(1)


# (name, size, vertices as pixel coordinates (fractional allowed), cull, front CW)
def _cases():
    out = []
    tri = [(2, 2), (12, 3), (5, 13)]  # counter-clockwise in NDC (y down the image)
    for cull in (0, 1, 2, 3):
        for cw in (False, True):
            out.append(("centres_cull%d_%s" % (cull, "cw" if cw else "ccw"), 16, tri, cull, cw))
            out.append(("reversed_cull%d_%s" % (cull, "cw" if cw else "ccw"), 16, tri[::-1], cull, cw))
    a, b, cc, d = (1, 1), (13, 1), (1, 13), (13, 13)  # the shared edge x + y = 14 crosses 13 pixel centres
    out.append(("shared_edge_first", 16, [a, b, cc], 0, False))
    out.append(("shared_edge_second", 16, [cc, b, d], 0, False))
    out.append(("axis_aligned", 8, [(1, 1), (6, 1), (1, 6)], 0, False))
    out.append(("sliver", 16, [(0.5, 0.2), (15.2, 1.0), (0.9, 1.4)], 0, False))
    out.append(("off_screen", 8, [(-5.3, 2.0), (11.5, -3.2), (4.0, 12.7)], 0, False))
    out.append(("degenerate", 16, [(2, 2), (8, 8), (13, 13)], 0, False))
    return out


CASES = _cases()


def clip_positions(case):
    """The case's vertices in clip space (w = 1)."""
    _, size, verts, _, _ = case
    return [(float(centre(x, size)) if float(x).is_integer() else float((f32(x) + f32(0.5)) / f32(size) * f32(2) - f32(1)),
             float(centre(y, size)) if float(y).is_integer() else float((f32(y) + f32(0.5)) / f32(size) * f32(2) - f32(1)))
            for x, y in verts]


def scene(case):
    name, size, verts, cull, cw = case
    variant = cull | (0x4 if cw else 0)
    s = c.Scene(c.PROGRAM, 1, [c.PROGRAM_CUBE, variant, size, size, 1])
    hdr = c.SceneHeader.from_address(s.ptr)
    assert s.draws == 1 and s.draw(0).count == 3 and hdr.vertex_bytes >= 3 * 32
    data = np.zeros((3, 8), np.float32)
    for i, (x, y) in enumerate(clip_positions(case)):
        data[i] = (x, y, 0.5, 1.0, 1.0, 0.0, 0.0, 1.0)
    ctypes.memmove(hdr.vertex_data, data.ctypes.data, data.nbytes)
    return s


def edge(a, b, px, py):
    return (px - a[0]) * (b[1] - a[1]) - (py - a[1]) * (b[0] - a[0])


def coverage(case):
    """Pixels the reference rasterises for the case (a size x size mask)."""
    _, size, _, cull, cw = case
    p = [np.array(v, np.float32) for v in clip_positions(case)]
    if cw:
        p[0], p[2] = p[2], p[0]
    mask = np.zeros((size, size), bool)
    screen = [(int(np.trunc((q[0] + f32(1)) * f32(0.5) * f32(size))), int(np.trunc((q[1] + f32(1)) * f32(0.5) * f32(size)))) for q in p]
    x0 = max(0, min(s[0] for s in screen))
    y0 = max(0, min(s[1] for s in screen))
    x1 = min(size, max(s[0] for s in screen) + 1)
    y1 = min(size, max(s[1] for s in screen) + 1)
    if x1 <= x0 or y1 <= y0:
        return mask
    xs = centre(np.arange(x0, x1), size)[None, :]
    ys = centre(np.arange(y0, y1), size)[:, None]
    area = edge(p[0], p[1], p[2][0], p[2][1])
    front = not (area < 0)
    if front:
        w = [edge(p[1], p[2], xs, ys), edge(p[2], p[0], xs, ys), edge(p[0], p[1], xs, ys)]
    else:
        w = [edge(p[2], p[1], xs, ys), edge(p[0], p[2], xs, ys), edge(p[1], p[0], xs, ys)]
    culled = ((cull & 2) and not front) or ((cull & 1) and front)  # VK_CULL_MODE_FRONT_BIT 1, BACK_BIT 2
    if culled:
        return mask
    inside = ~((w[0] < 0) | (w[1] < 0) | (w[2] < 0))
    mask[y0:y1, x0:x1] = inside
    return mask
