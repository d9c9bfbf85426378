"""Batched marker transfers (mdz_set_marker_state / mdz_get_marker_state):
the same resident state and the same host arrays as the per-array entry
points, with registered and with plain host memory, and the capacity
error before anything is written."""
import numpy as np
import pytest

import mdz

pytestmark = pytest.mark.gpu


def _ctx(cap):
    g = mdz.Grid(33, 17, 0.0, 2.0, 0.0, 1.0).set_bc_pureshear(1.0)
    return g, mdz.Context(g, 2, cap)


@pytest.mark.parametrize("register", [False, True])
def test_batched_round_trip(register):
    rng = np.random.default_rng(4)
    n = 200_003
    g, ctx = _ctx(n + 10)
    x, z = rng.uniform(0, 2, n), rng.uniform(0, 1, n)
    ph = rng.integers(0, 2, n).astype(np.int32)
    attrs = {a: rng.normal(size=n) for a in (mdz.M_SXXD, mdz.M_T, mdz.M_P)}
    if register:
        for a in [x, z, ph] + list(attrs.values()):
            mdz.host_register(a)
    ctx.set_marker_state(x, z, ph, attrs)
    assert ctx.n_markers == n
    gx, gz, gph, _, _ = ctx.get_markers()
    assert np.array_equal(gx, x) and np.array_equal(gz, z) and np.array_equal(gph, ph)
    for a, v in attrs.items():
        assert np.array_equal(ctx.get_marker_attr(a), v)
    out = [np.empty(n), np.empty(n), np.empty(n, np.int32), None, None]
    back = {a: np.empty(n) for a in attrs}
    ctx.get_marker_state(out, back)
    assert np.array_equal(out[0], x) and np.array_equal(out[1], z) and np.array_equal(out[2], ph)
    for a in attrs:
        assert np.array_equal(back[a], attrs[a])
    if register:
        for a in [x, z, ph] + list(attrs.values()):
            mdz.host_unregister(a)
    ctx.close()


def test_batched_capacity_error():
    g, ctx = _ctx(100)
    x = np.zeros(101)
    with pytest.raises(mdz.MdzError) as e:
        ctx.set_marker_state(x, x, np.zeros(101, np.int32), {})
    assert e.value.status == 3
    assert ctx.n_markers == 0
    ctx.close()
