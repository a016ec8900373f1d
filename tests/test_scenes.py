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
