"""The reference-signature drop-ins (libmdoodz_refshim.so: P2Mastah,
Interp_Grid2P, Interp_Grid2P_centroids2, RogerGuntherII,
StrainRateComponents, NonNewtonianViscosityGrid, RheologicalOperators,
EvaluateStokesResidualDecoupled, UpdateParticleStress, CountPartCell), called
with the reference's own structures and argument lists, as Main_DOODZ.c calls
them, against the golden vectors of the reference's functions."""
import ctypes as C
import os

import numpy as np
import pytest

import mdz
from refstructs import Ref, grid_of, phase_perc

pytestmark = pytest.mark.gpu

LIB = os.path.join(os.path.dirname(mdz.LIB_PATH), "libmdoodz_refshim.so")


@pytest.fixture(scope="module")
def shim():
    mdz.load_library()
    L = C.CDLL(LIB)
    L.LineSearchDecoupled.restype = C.c_double
    yield L
    L.mdz_gpu_finalize()


def _grid(ref):
    if "box" in ref:
        xmin, xmax, zmin, zmax = ref["box"]
        return mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    # fixtures without the box were made on the generator's standard grid
    from golden.make_golden import NX, NZ, XMIN, XMAX, ZMIN, ZMAX
    return mdz.Grid(NX, NZ, XMIN, XMAX, ZMIN, ZMAX).set_bc_pureshear(1.0)


def _params(g, nph, **kw):
    p = Ref("params", Nx=g.Nx, Nz=g.Nz, xmin=g.xmin, xmax=g.xmax, zmin=g.zmin, zmax=g.zmax, dx=g.dx, dz=g.dz,
            Nb_phases=nph, itp_stencil=1, isperiodic_x=0)
    for k, v in kw.items():
        p.set(k, v)
    return p


def _markers(x, z, ph, cap=None, **attrs):
    n = len(x)
    m = Ref("markers", Nb_part=n, Nb_part_max=cap or n, min_part_cell=16,
            x=np.array(x, np.float64), z=np.array(z, np.float64), phase=np.array(ph, np.int32))
    for k in ("Vx", "Vz", "P", "sxxd", "szzd", "sxz", "T", "strain", "strain_pl"):
        a = np.zeros(cap or n)
        if k in attrs:
            a[:n] = attrs[k]
        m.set(k, a)
    return m


def test_markers_through_reference_signatures(shim, golden):
    ref = golden("markers_ref.npz")
    g = _grid(ref)
    prm = _params(g, 3)
    mesh = grid_of(g, 3)
    mk = _markers(ref["x"], ref["z"], ref["phase"])
    shim.mdz_gpu_finalize()
    assert shim.mdz_gpu_init(prm.ptr, mesh.ptr, mk.ptr) == 0
    for centroid, stencil, avg, flag in ((1, 1, 0, 0), (0, 9, 1, 1), (-1, 1, 2, 1), (-2, 9, 0, 0)):
        vals = np.array(ref["per_phase"] if flag == 0 else ref["per_marker"], np.float64)
        out = np.full(g.size(centroid), -7.0)
        tags = np.ascontiguousarray(g.tags(centroid), np.int8)
        prm.set("itp_stencil", stencil)
        shim.P2Mastah(prm.ptr, mk.obj, vals.ctypes.data_as(C.c_void_p), mesh.ptr, out.ctypes.data_as(C.c_void_p),
                      tags.ctypes.data_as(C.c_void_p), C.c_int(flag), C.c_int(avg), C.c_int(0), C.c_int(centroid),
                      C.c_int(stencil))
        np.testing.assert_allclose(out, ref["p2g_c%d_s%d_a%d_f%d" % (centroid, stencil, avg, flag)], rtol=1e-12)
    for centroid in (1, 0):   # phase fractions land in the reference's per-phase arrays
        prm.set("itp_stencil", 9)
        shim.P2Mastah(prm.ptr, mk.obj, np.zeros(3).ctypes.data_as(C.c_void_p), mesh.ptr, None,
                      np.ascontiguousarray(g.tags(centroid), np.int8).ctypes.data_as(C.c_void_p), C.c_int(0),
                      C.c_int(0), C.c_int(1), C.c_int(centroid), C.c_int(9))
        np.testing.assert_allclose(phase_perc(mesh, centroid), ref["pp_c%d_s9" % centroid], rtol=1e-12, atol=1e-15)
    # counts (CountPartCell without reseeding)
    topo = Ref("surface")
    sc = Ref("scale", eta=1.0, L=1.0, V=1.0, T=1.0, t=1.0, E=1.0, S=1.0)
    shim.CountPartCell(mk.ptr, mesh.ptr, prm.obj, topo.obj, topo.obj, C.c_int(0), sc.obj)
    assert np.array_equal(mesh.keep["nb_part_cell"], ref["count_cell"])
    assert np.array_equal(mesh.keep["nb_part_vert"], ref["count_vert"])
    # grid -> markers
    out = np.zeros(len(ref["x"]))
    fv = np.ascontiguousarray(ref["g2p_vertex_field"], np.float64)
    shim.Interp_Grid2P(mk.obj, out.ctypes.data_as(C.c_void_p), mesh.ptr, fv.ctypes.data_as(C.c_void_p),
                       C.c_void_p(mesh.keep["xg_coord"].ctypes.data), C.c_void_p(mesh.keep["zg_coord"].ctypes.data),
                       C.c_int(g.Nx), C.c_int(g.Nz), C.c_void_p(mesh.keep["BCg.type"].ctypes.data))
    np.testing.assert_allclose(out, ref["g2p_vertex"], rtol=1e-13, atol=1e-15)
    fc = np.ascontiguousarray(ref["g2p_centroid_field"], np.float64)
    shim.Interp_Grid2P_centroids2(mk.obj, out.ctypes.data_as(C.c_void_p), mesh.ptr, fc.ctypes.data_as(C.c_void_p),
                                  C.c_void_p(mesh.keep["xvz_coord"].ctypes.data),
                                  C.c_void_p(mesh.keep["zvx_coord"].ctypes.data), C.c_int(g.Nx - 1),
                                  C.c_int(g.Nz - 1), C.c_void_p(mesh.keep["BCp.type"].ctypes.data), prm.ptr)
    np.testing.assert_allclose(out, ref["g2p_centroid"], rtol=1e-13, atol=1e-15)
    # RK4: velocities in the grid's u_in / v_in, dt in params, grid and params by value
    mesh.keep["u_in"][:] = ref["rk4_u"]
    mesh.keep["v_in"][:] = ref["rk4_v"]
    prm.set("dt", float(ref["rk4_dt"]))
    shim.RogerGuntherII(mk.ptr, prm.obj, mesh.obj, C.c_int(0), sc.obj)
    assert np.array_equal(mk.keep["phase"], ref["rk4_phase"])
    np.testing.assert_allclose(mk.keep["x"], ref["rk4_x"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(mk.keep["z"], ref["rk4_z"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(mk.keep["Vx"], ref["rk4_vx"], rtol=1e-13, atol=1e-15)
    shim.mdz_gpu_finalize()


def _mat_prop(phases, R):
    from golden.make_golden import RHEO_PHASES  # noqa: F401  (the phases below are RHEO_PHASES)
    mp = Ref("mat_prop", Nb_phases=len(phases), R=R)
    keys = {}
    for p, props in enumerate(phases):
        for k, v in props.items():
            keys.setdefault(k, [0.0] * 20)[p] = v
    for k, v in keys.items():
        mp.set(k, v)
    return mp


def test_rheology_and_residual_through_reference_signatures(shim, golden):
    from golden.make_golden import RHEO_PHASES, RHEO_MODEL, RHEO_R
    ref = golden("rheology_ref.npz")
    g = _grid(ref)
    fields = {k[3:]: ref[k] for k in ref if k.startswith("in_")}
    pp_n, pp_s = fields.pop("phase_perc_n"), fields.pop("phase_perc_s")
    mesh = grid_of(g, 3, fields)
    mesh.set("phase_perc_n", list(pp_n))
    mesh.set("phase_perc_s", list(pp_s))
    prm = _params(g, 3, dt=RHEO_MODEL["dt"], iselastic=RHEO_MODEL["iselastic"], step=RHEO_MODEL["step"],
                  eta_avg=0, mineta=RHEO_MODEL["mineta"], maxeta=RHEO_MODEL["maxeta"], loc_iter=1)
    mp = _mat_prop(RHEO_PHASES, RHEO_R)
    sc = Ref("scale", eta=1.0, L=1.0, V=1.0, T=1.0, t=1.0, E=1.0, S=1.0)
    nm = Ref("Nparams")
    mk = _markers([0.0], [0.0], [0])
    shim.mdz_gpu_finalize()
    assert shim.mdz_gpu_init(prm.ptr, mesh.ptr, mk.ptr) == 0
    shim.StrainRateComponents(mesh.ptr, sc.obj, prm.ptr)
    for k in ("div_u", "exxd", "ezzd", "exz", "exz_n", "exxd_s", "ezzd_s"):
        want = ref["sr_" + k]
        assert np.abs(mesh.keep[k] - want).max() <= 1e-13 * max(np.abs(want).max(), 1e-300), k
    shim.NonNewtonianViscosityGrid(mesh.ptr, mp.ptr, prm.ptr, nm.obj, sc.ptr)
    for k in ref:
        if k.startswith("vg_") and k[3:] in mesh.keep:
            want = ref[k]
            assert np.abs(mesh.keep[k[3:]] - want).max() <= 1e-10 * max(np.abs(want).max(), 1e-300), k
    shim.RheologicalOperators(mesh.ptr, prm.ptr, sc.ptr, C.c_int(0))
    for k in ref:
        if k.startswith("op0_"):
            want = ref[k]
            assert np.abs(mesh.keep[k[4:]] - want).max() <= 1e-10 * max(np.abs(want).max(), 1e-300), k
    # residual of the reference's state (its p_corr, right-hand side and
    # Picard operators), in the reference's equation numbering
    for k in ("p_corr", "roger_x", "roger_z", "rhs_p"):
        mesh.keep[k][:] = ref["vg_p_corr"] if k == "p_corr" else ref["rhs_" + k]
    for k in ("D11_n", "D22_n", "D33_s"):
        mesh.keep[k][:] = ref["op0_" + k]
    eq = [np.ascontiguousarray(ref["st_eqn%d" % w], np.int32) for w in range(3)]
    nmom = int(max(eq[0].max(), eq[1].max()) + 1)
    ncont = int(eq[2].max() + 1 - nmom)
    stokes = Ref("SparseMat", eqn_u=eq[0], eqn_v=eq[1], eqn_p=eq[2], neq_mom=nmom, neq_cont=ncont,
                 neq=nmom + ncont)
    A, Cm = Ref("SparseMat", F=np.zeros(nmom)), Ref("SparseMat", F=np.zeros(ncont))
    B, D = Ref("SparseMat"), Ref("SparseMat")
    shim.EvaluateStokesResidualDecoupled(stokes.ptr, A.ptr, B.ptr, Cm.ptr, D.ptr, nm.ptr, mesh.ptr, prm.obj, sc.obj,
                                         C.c_int(1))
    got = [nm.get("resx"), nm.get("resz"), nm.get("resp")]
    np.testing.assert_allclose(got, ref["st_norms"], rtol=1e-12)
    Fm = A.keep["F"]
    sel = (eq[0] >= 0) & (g.BCu == -1)
    np.testing.assert_allclose(Fm[eq[0][sel]], ref["st_ru"][sel], rtol=1e-12, atol=1e-12 * np.abs(ref["st_ru"]).max())
    # marker stresses (UpdateParticleStress, no rotation): increments of the grid stresses
    sref = golden("stress_ref.npz")
    mk2 = _markers(sref["x"], sref["z"], sref["phase"], sxxd=sref["m0_sxxd"], szzd=sref["m0_szzd"],
                   sxz=sref["m0_sxz"])
    for k in ("sxxd", "szzd", "sxz", "sxxd0", "szzd0", "sxz0"):
        mesh.keep[k][:] = sref[k]
    shim.UpdateParticleStress(mesh.ptr, mk2.ptr, prm.ptr, mp.ptr, sc.ptr)
    for k in ("sxxd", "szzd", "sxz"):
        np.testing.assert_allclose(mk2.keep[k], sref["m_" + k], rtol=1e-12, atol=1e-13)
    shim.mdz_gpu_finalize()
