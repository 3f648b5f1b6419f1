"""Even-odd fill rule (extension: the reference fills nonzero only, so this
is pinned against its definition rather than reference output).  Coverage
under even-odd is the distance from the accumulated signed area to the
nearest even integer; nonzero is min(|area|, 1)."""
import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import scenes
from canvas_ity_gb300 import trace as T
import golden_util as G

W, H = 64, 48


def _two_squares(rule):
    t = T.TraceWriter(W, H)
    t.set_fill_rule(rule)
    t.set_color(T.FILL_STYLE, 1.0, 1.0, 1.0, 1.0)
    t.begin_path()
    for x0, y0 in ((8, 8), (24, 16)):       # same orientation: winding 2 where they overlap
        t.move_to(x0, y0); t.line_to(x0 + 24, y0); t.line_to(x0 + 24, y0 + 24); t.line_to(x0, y0 + 24)
        t.close_path()
    t.fill()
    t.is_point_in_path(30.5, 20.5)            # in both squares
    t.is_point_in_path(12.5, 12.5)            # in the first only
    return t.finish()


def _alpha(tb, rule_ties="reference"):
    img = G.split_images(tb, oracle.replay(tb, ties=rule_ties)[0])[-1]
    return img[..., 3]


def test_nonzero_fills_the_overlap_even_odd_leaves_it_empty():
    a_nz = _alpha(_two_squares(T.NONZERO))
    a_eo = _alpha(_two_squares(T.EVEN_ODD))
    overlap = (slice(17, 31), slice(25, 31))   # rows 16..32, cols 24..32, inside both
    only_first = (slice(9, 15), slice(9, 23))
    assert (a_nz[overlap] == 255).all() and (a_eo[overlap] == 0).all()
    assert (a_nz[only_first] == 255).all() and (a_eo[only_first] == 255).all()
    assert (a_nz[0:4, :] == 0).all() and (a_eo[0:4, :] == 0).all()


def test_point_in_path_follows_the_rule():
    assert oracle.replay(_two_squares(T.NONZERO))[1] == [1.0, 1.0]
    assert oracle.replay(_two_squares(T.EVEN_ODD))[1] == [0.0, 1.0]


def test_partial_coverage_matches_the_definition():
    """Along the overlap's edge the accumulated area s lies in (1, 2):
    even-odd coverage is 2 - s where nonzero gives 1."""
    t = T.TraceWriter(W, H)
    t.set_fill_rule(T.EVEN_ODD)
    t.set_color(T.FILL_STYLE, 1.0, 1.0, 1.0, 1.0)
    t.begin_path()
    t.rectangle(4, 4, 40, 30)
    t.rectangle(10.25, 10.5, 20.5, 12.75)      # inside the first, same orientation
    t.fill()
    tb = t.finish()
    a = oracle.replay_linear(tb, W, H)[..., 3]
    # inner rectangle's left column x=10: area from the inner edge is 0.75,
    # so s = 1 + 0.75 and even-odd coverage 0.25
    assert abs(a[15, 10] - 0.25) < 1e-6
    assert a[15, 20] == 0.0 and a[15, 6] == 1.0


@pytest.mark.reference
def test_reference_rejects_even_odd():
    if not oracle.reference_available():
        pytest.skip("reference sources are not present here")
    with pytest.raises(ValueError):
        oracle.reference_replay(_two_squares(T.EVEN_ODD))
