"""The deforming pure-shear box (PureShearALE): the wall means, the new box and
the regenerated grid lines against the oracle bit for bit, for host and for
resident velocities; a breakpoint carries the moved box into a fresh context;
new Dirichlet values reach the next step."""
import ctypes as C

import numpy as np
import pytest

import mdz
import oracle_step

pytestmark = pytest.mark.gpu

BOX = (-0.5, 0.5, -0.3, 0.4)


def _grid():
    return mdz.Grid(37, 29, *BOX).set_bc_pureshear(1.0)


def _lines(ctx, g):
    box = (C.c_double * 6)()
    out = [np.empty(n) for n in (g.Nx, g.Nz, g.Nx - 1, g.Nz - 1, g.Nx + 1, g.Nz + 1)]
    ctx._check(ctx.L.mdz_get_grid(ctx.h, box, *[mdz._dptr(a) for a in out]))
    return tuple(box), out


def test_pure_shear_ale_matches_oracle():
    rng = np.random.default_rng(5)
    g = _grid()
    u = rng.standard_normal(g.size(-1))
    v = rng.standard_normal(g.size(-2))
    ctx = mdz.Context(g, 1, 16)
    try:
        got = ctx.pure_shear_ale(0.01, u, v)
        want_g = _grid()
        want = oracle_step.pure_shear_ale(want_g, u, v, 0.01)
        assert got == want
        box, lines = _lines(ctx, g)
        assert box[:4] == want and box[4:] == (want_g.dx, want_g.dz)
        for a, b in zip(lines, (want_g.xg, want_g.zg, want_g.xc, want_g.zc, want_g.xvz, want_g.zvx)):
            assert np.array_equal(a, b)
        # the Python grid followed the context
        assert (g.xmin, g.xmax, g.zmin, g.zmax) == want and np.array_equal(g.xvz, want_g.xvz)
        # second call on the resident velocities (uploaded by the first)
        got2 = ctx.pure_shear_ale(0.02)
        assert got2 == oracle_step.pure_shear_ale(want_g, u, v, 0.02)
    finally:
        ctx.close()


def test_breakpoint_restores_the_moved_box(tmp_path):
    g = _grid()
    x = np.linspace(-0.45, 0.45, 50)
    z = np.linspace(-0.25, 0.35, 50)
    ctx = mdz.Context(g, 1, 64)
    try:
        ctx.set_markers(x, z, np.zeros(50, np.int32))
        u, v = np.zeros(g.size(-1)), np.zeros(g.size(-2))
        u.reshape(g.Nz + 1, g.Nx)[:, 0] = 0.3
        v.reshape(g.Nz, g.Nx + 1)[-1, :] = 0.2
        moved = ctx.pure_shear_ale(0.1, u, v)
        assert moved != BOX
        path = tmp_path / "ale.brk"
        ctx.save_breakpoint(path)
    finally:
        ctx.close()
    g2 = _grid()
    ctx2 = mdz.Context(g2, 1, 64)
    try:
        ctx2.load_breakpoint(path)
        assert ctx2.get_box()[:4] == moved
        assert (g2.xmin, g2.xmax, g2.zmin, g2.zmax) == moved
        x2, z2, ph2, _, _ = ctx2.get_markers()
        assert np.array_equal(x2, x) and np.array_equal(z2, z)
    finally:
        ctx2.close()
