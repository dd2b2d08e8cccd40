"""The sliding-window extrema restatement (oracle tuo_extrema: the
reference's extrema_finder deque, BoxFilter.h:196-233, run down the columns
and then along the rows as BoxFilter2::convolve does) against an independent
brute force of the same rule, and known answers."""
import numpy as np
import pytest


def brute(img, wV, wH, is_max, shift):
    """Per window: each column's best value and its topmost row, then the
    leftmost column holding the best of those."""
    rows, cols = img.shape
    val = np.full((rows, cols), np.nan)
    pos = np.full((rows, cols, 2), -1, np.int32)
    oy, ox = (wV // 2, wH // 2) if shift else (0, 0)
    better = (lambda a, b: a > b) if is_max else (lambda a, b: a < b)
    for y in range(rows + 1 - wV):
        for x in range(cols + 1 - wH):
            bc = None
            for c in range(x, x + wH):
                br = y
                for r in range(y + 1, y + wV):
                    if better(img[r, c], img[br, c]):
                        br = r
                if bc is None or better(img[br, c], img[bc[1], bc[0]]):
                    bc = (c, br)
            val[y + oy, x + ox] = img[bc[1], bc[0]]
            pos[y + oy, x + ox] = bc
    return val, pos


@pytest.mark.parametrize("wV,wH", [(1, 1), (1, 4), (4, 1), (3, 3), (2, 5), (5, 7), (9, 2)])
@pytest.mark.parametrize("is_max", [False, True])
@pytest.mark.parametrize("shift", [True, False])
def test_deque_matches_brute_force_with_ties(oracle, wV, wH, is_max, shift):
    rng = np.random.default_rng(wV * 100 + wH + 7 * is_max)
    img = rng.integers(0, 4, (23, 31)).astype(np.float64)  # many ties
    v, p = oracle.extrema(img, wV, wH, is_max, shift)
    bv, bp = brute(img, wV, wH, is_max, shift)
    assert np.array_equal(np.isnan(v), np.isnan(bv))
    assert np.array_equal(v[~np.isnan(v)], bv[~np.isnan(bv)])
    assert np.array_equal(p, bp)


def test_known_answers(oracle):
    # constant image: every window's first element (left column, top row)
    img = np.full((10, 12), 3.0)
    v, p = oracle.extrema(img, 3, 4, False, False)
    assert np.all(v[:8, :9] == 3)
    ys, xs = np.mgrid[0:8, 0:9]
    assert np.array_equal(p[:8, :9, 0], xs) and np.array_equal(p[:8, :9, 1], ys)
    # one minimum: every window that holds it reports it
    img = np.full((9, 9), 5.0)
    img[4, 6] = -1.0
    v, p = oracle.extrema(img, 3, 3, False, True)
    for y in range(7):
        for x in range(7):
            inside = y <= 4 < y + 3 and x <= 6 < x + 3
            assert v[y + 1, x + 1] == (-1.0 if inside else 5.0)
            if inside:
                assert tuple(p[y + 1, x + 1]) == (6, 4)
    # image smaller than the window: no-op
    assert oracle.extrema(np.zeros((2, 9)), 3, 3)[0] is None
    # maxima of a ramp: the window's last column, top row
    img = np.tile(np.arange(10, dtype=np.float64), (6, 1))
    v, p = oracle.extrema(img, 2, 3, True, False)
    assert np.all(v[:5, :8] == np.arange(2, 10)) and np.all(p[:5, :8, 0] == np.arange(2, 10))
    assert np.all(p[:5, :8, 1] == np.arange(5)[:, None])
