"""The oracle's DisparitySelector restatement (tuo_select_disparity) against a
plain-Python transcription of select_disparity's rule (StereoUtility.h:56-107)
with exact right-image minima, on small integer volumes full of ties."""
import numpy as np
import pytest


def brute(costs, dmax, inc):
    D, rows, cols = costs.shape
    out = np.zeros((rows, cols))
    for y in range(rows):
        dR = []
        for xr in range(cols):
            best, db = np.inf, 0
            for d in range(min(D, xr + 1)):
                c = costs[d, y, xr - d]
                if c < best:
                    best, db = c, d
            dR.append(db)
        for x in range(cols):
            best, dl = np.inf, 0
            for d in range(D):
                if costs[d, y, x] < best:
                    best, dl = costs[d, y, x], d
            xr = x + dl
            out[y, x] = dmax - dl if xr < cols and abs(dl - dR[xr]) < inc else 0
    return out


@pytest.mark.parametrize("D,rows,cols,inc", [(1, 3, 5, 1), (4, 5, 9, 1), (7, 4, 12, 2), (16, 3, 20, 3)])
def test_select_matches_rule(oracle, D, rows, cols, inc):
    rng = np.random.default_rng(D * 31 + cols)
    costs = rng.integers(0, 4, (D, rows, cols)).astype(np.float64)  # many ties
    got = oracle.select_disparity(costs, 40, inc)
    assert np.array_equal(got, brute(costs, 40, inc))


def test_select_known_answer(oracle):
    """One row, two disparities: left minima dL = [1, 0, 1], right minima
    dR = [0, 0, 1]; pixel 0: xr = 1, |1 - dR[1]| = 1 is not < 1 -> 0; pixel 1:
    |0 - dR[1]| = 0 -> 10 - 0; pixel 2: xr = 3 is past the row -> 0."""
    costs = np.array([[[5, 1, 9]], [[2, 3, 0]]], np.float64)
    assert oracle.select_disparity(costs, 10, 1).tolist() == [[0, 10, 0]]
