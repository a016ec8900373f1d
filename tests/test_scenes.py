"""The seeded scene generator (no GPU): determinism, documented sizes, and
the parameters of the benchmark workloads."""
import numpy as np
import pytest

import cpvulkan_gb300 as c


def test_heightfield_full_size_triangle_count(native):
    # 1024 x 1024 vertex grid: 2 * 1023^2 triangles, 1920 x 1080 target
    s = c.Scene(c.HEIGHTFIELD, 1, [])
    assert s.triangles == 2 * 1023 * 1023
    assert (s.width, s.height) == (1920, 1080)


def test_cube_is_the_sample_cube(native):
    s = c.Scene(c.CUBE, 1, [0])
    assert s.triangles == 12 and (s.width, s.height) == (500, 500)


def test_blend_scene_size(native):
    s = c.Scene(c.BLEND, 1, [])
    assert s.triangles == 400000 and (s.width, s.height) == (1920, 1080)


@pytest.mark.parametrize("config,params", [(c.HEIGHTFIELD, [32, 64, 48]), (c.BLEND, [50, 64, 48]), (c.BATCH, [5, 200, 64, 48]),
                                           (c.SERVE, [64, 500, 1])])
def test_seeded_scenes_are_deterministic(native, oracle, config, params):
    a, b, other = c.Scene(config, 9, params), c.Scene(config, 9, params), c.Scene(config, 10, params)
    ca, da, _ = oracle.render(a)
    cb, db, _ = oracle.render(b)
    co, _, _ = oracle.render(other)
    assert np.array_equal(ca, cb)
    assert (da is None and db is None) or np.array_equal(da, db)
    assert not np.array_equal(ca, co)


def test_batch_scene_has_4096_draws_by_default(native):
    s = c.Scene(c.BATCH, 1, [])
    assert s.draws == 4096 and (s.width, s.height) == (2560, 1440)


def test_scene_draw_view_matches_the_triangle_count(native):
    """The ctypes view of cpv_scene_draw: its counts give the scene's
    primitive total (triangle lists in the batch scene)."""
    import ctypes
    assert ctypes.sizeof(c.SceneDraw) == 200
    s = c.Scene(c.BATCH, 3, [12, 2000, 64, 48])
    total = sum(s.draw(i).count // 3 * s.draw(i).instance_count for i in range(s.draws))
    assert total == s.triangles
    rec = s.indirect_record(0)
    assert len(rec) == 5 and rec[0] == s.draw(0).count


@pytest.mark.parametrize("variant,per_draw", [(0x10000, lambda n: n), (0x10000 | 0x400, lambda n: n // 2),
                                              (0x10000 | 0x800, lambda n: max(n - 1, 0)), (0x0, lambda n: n // 3),
                                              (0x400, lambda n: max(n - 2, 0)), (0x800, lambda n: max(n - 2, 0))])
def test_primitive_counts_by_topology(native, variant, per_draw):
    """Primitives of a draw per topology (CPVulkan/CommandBuffer.Draw.cpp:
    567-673): points n, line list n/2, line strip n-1, triangle list n/3,
    strip and fan n-2."""
    s = c.Scene(c.PROGRAM, 1, [c.PROGRAM_CUBE, variant, 32, 32, 7])
    assert s.triangles == sum(per_draw(s.draw(i).count) * s.draw(i).instance_count for i in range(s.draws))
