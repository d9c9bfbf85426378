"""The marker kernels compute cell indices ceil(d/h + add) from the product
d * (1/h) and divide only when that product lies within a few units in the
last place of an integer (ceil_quot in csrc/mdz_internal.cuh).  This checks
the rule on the CPU in IEEE double arithmetic against the plain division, on
random positions and on positions placed exactly on, and a few ulps either
side of, every grid line of the lithosphere grid and of small grids."""
import numpy as np
import pytest

EPS = np.finfo(np.float64).eps


def ceil_quot(d, h, ih, add, fma):
    q = (np.longdouble(d) * np.longdouble(ih) + np.longdouble(add)).astype(np.float64) if fma else d * ih + add
    c = np.ceil(q)
    tol = 16.0 * EPS * 65538.0
    f = c - q
    fast = (f > tol) & (f < 1.0 - tol)
    return np.where(fast, c, np.ceil(d / h + add))


def lines(x0, h, n):
    """The reference's grid lines: x0 + k h accumulated as SetGridCoordinates does."""
    out = np.empty(n)
    out[0] = x0
    for k in range(1, n):
        out[k] = out[k - 1] + h
    return out


@pytest.mark.parametrize("fma", [False, True])
@pytest.mark.parametrize("add", [0.0, 0.5])
@pytest.mark.parametrize("n,x0,x1", [(1025, -1.0, 1.0), (513, -0.5, 0.0), (65, 0.0, 3.0), (33, -7.3, 11.9)])
def test_ceil_quot_matches_division(n, x0, x1, add, fma):
    h = (x1 - x0) / (n - 1)
    ih = 1.0 / h
    rng = np.random.default_rng(n)
    L = lines(x0, h, n)
    pts = [rng.uniform(x0 - 2 * h, x1 + 2 * h, 200000), L, L + h / 2]
    for k in range(1, 9):
        pts += [np.nextafter(L, np.inf) if k == 1 else L + k * EPS * np.maximum(np.abs(L), 1.0),
                np.nextafter(L, -np.inf) if k == 1 else L - k * EPS * np.maximum(np.abs(L), 1.0)]
    x = np.concatenate(pts)
    for X0 in (x0, L[0] + h / 2):   # node lines and the staggered (centroid) lines
        d = x - X0
        np.testing.assert_array_equal(ceil_quot(d, h, ih, add, fma), np.ceil(d / h + add))
