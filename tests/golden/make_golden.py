"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own C
functions (MDOODZ 6.0 compiled in place by `make -C oracle ref`, driven through
oracle/ref_harness.c).  Run in a container that has the reference sources:

    python tests/golden/make_golden.py

Each fixture is a small .npz holding the inputs and the reference outputs.
The GPU tests and the oracle self-tests read these files; nothing at test time
needs the reference itself.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "mdoodz6.0_gb300")]

import mdz  # noqa: E402  (grid / tag helpers only; no GPU use)
import mdz_setups  # noqa: E402
from refharness import RefMDOODZ  # noqa: E402

# small, non-square grid; two phases; 4x4 jittered markers per cell
NX, NZ, XMIN, XMAX, ZMIN, ZMAX = 21, 17, -0.5, 0.5, -0.4, 0.4


def _grid():
    return mdz.Grid(NX, NZ, XMIN, XMAX, ZMIN, ZMAX).set_bc_pureshear(1.0)


def _markers(g, seed=7):
    x, z = mdz_setups.seed_markers(g, 4, 4, 0.5, seed)
    ph = mdz_setups.inclusion_phase(x, z, 0.05, -0.02, 0.18)
    # a few inactive markers, and a third phase stripe
    ph[(z > 0.25) & (x < -0.2)] = 2
    ph[::97] = -1
    return x, z, ph


def make_markers_fixture():
    g = _grid()
    r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
    r.set_bc_pureshear(1.0)
    # the harness grid must equal ours bit for bit
    for name, ours in [("xg_coord", g.xg), ("zg_coord", g.zg), ("xc_coord", g.xc), ("zc_coord", g.zc),
                       ("xvz_coord", g.xvz), ("zvx_coord", g.zvx)]:
        assert np.array_equal(r.field(name), ours), name
    assert np.array_equal(r.tags("BCu"), g.BCu) and np.array_equal(r.tags("BCv"), g.BCv)
    assert np.array_equal(r.field("BCu_val"), g.BCu_val) and np.array_equal(r.field("BCv_val"), g.BCv_val)
    x, z, ph = _markers(g)
    r.set_markers(x, z, ph)
    rng = np.random.default_rng(3)
    per_phase = np.array([1.0, 1e3, 7.5])
    per_marker = np.exp(rng.normal(0.0, 1.0, len(x)))
    out = dict(Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]), x=x, z=z, phase=ph, per_phase=per_phase,
               per_marker=per_marker)
    for centroid in (1, 0, -1, -2):
        for stencil in (1, 9):
            for avg in (0, 1, 2):
                for flag in (0, 1):
                    vals = per_phase if flag == 0 else per_marker
                    init = np.full(g.size(centroid), -7.0)   # untouched nodes keep this
                    out["p2g_c%d_s%d_a%d_f%d" % (centroid, stencil, avg, flag)] = r.p2g(vals, flag, avg, 0, centroid,
                                                                                       stencil, init)
    for centroid in (1, 0):
        for stencil in (1, 9):
            r.p2g(per_phase, 0, 0, 1, centroid, stencil)
            out["pp_c%d_s%d" % (centroid, stencil)] = np.array([r.phase_perc(centroid, p).copy() for p in range(3)])
    # counts (CountPartCell_Old): totals, and per-phase counts recovered from
    # the phase fractions it stores (fraction x total is an exact small integer)
    r.count_old()
    cc, cv = r.counts(1).copy(), r.counts(0).copy()
    out["count_cell"], out["count_vert"] = cc, cv
    out["pcount_cell"] = np.rint(np.array([r.phase_perc(1, p) * cc for p in range(3)])).astype(np.int32)
    out["pcount_vert"] = np.rint(np.array([r.phase_perc(0, p) * cv for p in range(3)])).astype(np.int32)
    # grid -> marker
    fv = np.sin(3 * g.xg)[None, :] * np.cos(2 * g.zg)[:, None]
    fc = np.cos(2 * g.xc)[None, :] * (1 + g.zc)[:, None] ** 2
    out["g2p_vertex_field"], out["g2p_centroid_field"] = fv.ravel(), fc.ravel()
    out["g2p_vertex"] = r.g2p(fv.ravel(), 0)
    out["g2p_centroid"] = r.g2p(fc.ravel(), 1)
    # RK4 in a pure-shear + vortex velocity (some markers leave the box)
    U = (-g.xg[None, :] * 1.0 + 0.3 * np.sin(np.pi * g.zvx[:, None])).ravel()
    V = (g.zg[:, None] * 1.0 + 0.2 * np.cos(np.pi * g.xvz[None, :])).ravel()
    r.field("u_in")[:] = U
    r.field("v_in")[:] = V
    r.set_param("dt", 0.07)
    r.rk4()
    out["rk4_u"], out["rk4_v"], out["rk4_dt"] = U, V, 0.07
    out["rk4_x"], out["rk4_z"] = r.marker_field("x").copy(), r.marker_field("z").copy()
    out["rk4_vx"], out["rk4_vz"] = r.marker_field("Vx").copy(), r.marker_field("Vz").copy()
    out["rk4_phase"] = r.marker_phase().copy()
    np.savez_compressed(os.path.join(HERE, "markers_ref.npz"), **out)
    print("markers_ref.npz:", len(out), "arrays")


if __name__ == "__main__":
    what = sys.argv[1:] or ["markers"]
    if "markers" in what:
        make_markers_fixture()
