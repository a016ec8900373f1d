"""The oracle's triangle coverage against the numpy restatement of the
reference's rule on hand-placed triangles (tests/coverage_kat.py): the
fragment count always, and the covered pixels where the shading is defined
(every case but the zero-area one, whose barycentric weights divide by 0)."""
import numpy as np
import pytest

from tests import coverage_kat as kat


@pytest.mark.parametrize("case", kat.CASES, ids=[k[0] for k in kat.CASES])
def test_coverage_kat(native, oracle, case):
    want = kat.coverage(case)
    s = kat.scene(case)
    colour, _, stats = oracle.render(s)
    assert stats["fragments"] == int(want.sum()), (stats, int(want.sum()))
    if case[0] != "degenerate":
        got = (colour.reshape(case[1], case[1], 4) == [255, 0, 0, 255]).all(axis=-1)
        assert np.array_equal(got, want)


def test_kat_cases_cover_the_edge_rules(native):
    """The cases exercise what they are named for: pixel centres on edges
    (edge function exactly 0 and covered), a shared edge covered by both
    triangles, culling by winding, and a zero-area line of fragments."""
    by = {k[0]: k for k in kat.CASES}
    first, second = kat.coverage(by["shared_edge_first"]), kat.coverage(by["shared_edge_second"])
    assert (first & second).sum() >= 10
    n = {name: int(kat.coverage(by[name]).sum()) for name in by}
    for face in ("ccw", "cw"):
        # culling front or back faces keeps exactly one winding of the triangle
        assert (n["centres_cull1_" + face] == 0) != (n["centres_cull2_" + face] == 0)
        assert (n["centres_cull1_" + face] == 0) == (n["reversed_cull2_" + face] == 0)
        assert (n["reversed_cull1_" + face] == 0) != (n["reversed_cull2_" + face] == 0)
    # the front-face setting flips which winding is culled
    assert (n["centres_cull1_ccw"] == 0) != (n["centres_cull1_cw"] == 0)
    assert kat.coverage(by["centres_cull3_cw"]).sum() == 0
    assert kat.coverage(by["degenerate"]).sum() == 12
