"""Breakpoint of the resident state (mdz_save_breakpoint / mdz_load_breakpoint,
the counterpart of MakeBreakpointParticles / LoadBreakpointParticles): a run
restarted from a breakpoint continues as the uninterrupted one, and a
breakpoint of another grid or a truncated file is refused without touching
the context."""
import numpy as np
import pytest

import mdz
from test_step_gpu import vep_case, _rel

pytestmark = pytest.mark.gpu


def _context(g, m, u, v, p, mat, cap):
    ctx = mdz.Context(g, mat.n_phases, cap)
    ctx.set_markers(m["x"], m["z"], m["phase"])
    for attr, key in ((mdz.M_SXXD, "sxxd"), (mdz.M_SZZD, "szzd"), (mdz.M_SXZ, "sxz"), (mdz.M_STRAIN_PL, "strain_pl"),
                      (mdz.M_STRAIN, "strain"), (mdz.M_T, "T"), (mdz.M_CMUL, "cmul")):
        ctx.set_marker_attr(attr, m[key])
    f = mdz.GridFields(g, mat.n_phases)
    f["u"], f["v"], f["p"] = u, v, p
    s = f.struct()
    for name in mdz.FIELD_NAMES:
        if name not in ("u", "v", "p"):
            setattr(s, name, None)
    ctx._check(ctx.L.mdz_sync_fields(ctx.h, mdz.C.byref(s), 1))
    return ctx


def _state(ctx, g, nph):
    out = mdz.GridFields(g, nph)
    ctx.download_fields(out)
    x, z, ph, vx, vz = ctx.get_markers()
    return dict(u=out["u"], v=out["v"], p=out["p"] - out["p"].mean(), x=x, z=z, phase=ph, vx=vx,
                sxxd=ctx.get_marker_attr(mdz.M_SXXD), strain_pl=ctx.get_marker_attr(mdz.M_STRAIN_PL))


def test_restart_continues_as_uninterrupted(tmp_path):
    g, m, u, v, p, mat = vep_case()
    prm = mdz.RheoParams.make(dt=0.05, iselastic=1, step=1)
    model = mdz.Model.make(prm, newton=1, nit_max=12, rel_tol=1e-11, lin_rtol=1e-9, line_search=0, precision=64,
                           reseed=1, min_part_cell=16, direct_neighbour=0)
    cap = len(m["x"]) + 8 * g.ncx * g.ncz
    path = str(tmp_path / "step1.brk")
    a = _context(g, m, u, v, p, mat, cap)
    a.time_step(mat, model)
    a.save_breakpoint(path)
    n1 = a.n_markers
    ra = a.time_step(mat, model)
    sa = _state(a, g, mat.n_phases)
    a.close()
    # a fresh context of the same grid, nothing uploaded but the breakpoint
    b = mdz.Context(g, mat.n_phases, cap)
    b.load_breakpoint(path)
    assert b.n_markers == n1
    rb = b.time_step(mat, model)
    sb = _state(b, g, mat.n_phases)
    b.close()
    assert ra.converged == 1 and rb.converged == 1
    assert ra.nonlinear_its == rb.nonlinear_its and ra.markers_added == rb.markers_added
    assert np.array_equal(sa["phase"], sb["phase"])
    for k in ("u", "v", "p", "x", "z", "vx", "sxxd", "strain_pl"):
        assert _rel(sb[k], sa[k]) < 1e-12, (k, _rel(sb[k], sa[k]))


def test_restart_into_a_context_that_has_stepped(tmp_path):
    """Loading into a context that already ran steps of its own (other
    markers, fields and multigrid hierarchy) gives the same next step as the
    uninterrupted run; a breakpoint saved before any field existed zeroes the
    loaded context's u, v, p as well."""
    g, m, u, v, p, mat = vep_case()
    prm = mdz.RheoParams.make(dt=0.05, iselastic=1, step=1)
    model = mdz.Model.make(prm, newton=1, nit_max=12, rel_tol=1e-11, lin_rtol=1e-9, line_search=0, precision=64,
                           reseed=1, min_part_cell=16, direct_neighbour=0)
    cap = len(m["x"]) + 8 * g.ncx * g.ncz
    path = str(tmp_path / "step1.brk")
    a = _context(g, m, u, v, p, mat, cap)
    a.time_step(mat, model)
    a.save_breakpoint(path)
    ra = a.time_step(mat, model)
    sa = _state(a, g, mat.n_phases)
    a.close()
    c = _context(g, m, u, v, p, mat, cap)
    for _ in range(3):
        c.time_step(mat, model)
    c.load_breakpoint(path)
    rc = c.time_step(mat, model)
    sc = _state(c, g, mat.n_phases)
    assert rc.nonlinear_its == ra.nonlinear_its and rc.markers_added == ra.markers_added
    for k in ("u", "v", "p", "x", "z", "vx", "sxxd", "strain_pl"):
        assert _rel(sc[k], sa[k]) < 1e-12, (k, _rel(sc[k], sa[k]))
    # a field-less breakpoint (saved by a context that never had fields)
    empty = str(tmp_path / "markers_only.brk")
    d = mdz.Context(g, mat.n_phases, cap)
    d.set_markers(m["x"], m["z"], m["phase"])
    d.save_breakpoint(empty)
    d.close()
    c.load_breakpoint(empty)
    out = mdz.GridFields(g, mat.n_phases)
    c.download_fields(out)
    c.close()
    assert not out["u"].any() and not out["v"].any() and not out["p"].any()


def test_breakpoint_refused(tmp_path):
    g, m, u, v, p, mat = vep_case()
    path = str(tmp_path / "b.brk")
    a = _context(g, m, u, v, p, mat, len(m["x"]))
    a.save_breakpoint(path)
    before = a.get_markers()
    other = mdz.Grid(g.Nx + 2, g.Nz, g.xmin, g.xmax, g.zmin, g.zmax).set_bc_pureshear(1.0)
    c = mdz.Context(other, mat.n_phases, len(m["x"]))
    with pytest.raises(mdz.MdzError) as e:
        c.load_breakpoint(path)
    assert e.value.status == 1
    c.close()
    raw = open(path, "rb").read()
    short = str(tmp_path / "short.brk")
    open(short, "wb").write(raw[:len(raw) // 2])
    with pytest.raises(mdz.MdzError) as e:
        a.load_breakpoint(short)
    assert e.value.status == 1
    after = a.get_markers()
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    a.close()


def test_restart_from_reference_breakpoint_file(tmp_path):
    """A file written by the reference's own MakeBreakpointParticles (scaled
    lithosphere-like units, iselastic = 1) loads into a context exactly as the
    reference's LoadBreakpointParticles reads it back: markers, phases,
    velocities, P, stresses, strains, T, u_in / v_in / p_in, dt, time and the
    box, bit for bit; wrong flags, a truncated file and another grid are
    refused with the context unchanged."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "breakpoint_ref.npz"))
    scales = dict(zip(("L", "V", "S", "T", "t"), d["scale"]))
    Nx, Nz, nph, n = int(d["Nx"]), int(d["Nz"]), int(d["n_phases"]), int(d["n"])
    box = d["box"]
    path = tmp_path / "Breakpoint00001.dat"
    path.write_bytes(d["image"].tobytes())
    g = mdz.Grid(Nx, Nz, box[0], box[1], box[2], box[3]).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, nph, n + 64)
    # refusals first: the context must stay empty
    with pytest.raises(mdz.MdzError):
        ctx.load_reference_breakpoint(str(path), scales, iselastic=0)
    short = tmp_path / "short.dat"
    short.write_bytes(d["image"].tobytes()[:-8])
    with pytest.raises(mdz.MdzError):
        ctx.load_reference_breakpoint(str(short), scales)
    assert ctx.n_markers == 0
    other = mdz.Context(mdz.Grid(Nx + 2, Nz, box[0], box[1], box[2], box[3]).set_bc_pureshear(1.0), nph, n + 64)
    with pytest.raises(mdz.MdzError):
        other.load_reference_breakpoint(str(path), scales)
    other.close()
    dt, time = ctx.load_reference_breakpoint(str(path), scales)
    assert dt == float(d["dt"]) and time == float(d["time"])
    assert ctx.n_markers == n
    x, z, ph, vx, vz = ctx.get_markers()
    assert np.array_equal(ph, d["phase"])
    for k, a in (("x", x), ("z", z), ("Vx", vx), ("Vz", vz)):
        assert np.array_equal(a, d["m_" + k]), k
    for k, a in (("P", mdz.M_P), ("sxxd", mdz.M_SXXD), ("szzd", mdz.M_SZZD), ("sxz", mdz.M_SXZ),
                 ("strain", mdz.M_STRAIN), ("strain_pl", mdz.M_STRAIN_PL), ("T", mdz.M_T)):
        assert np.array_equal(ctx.get_marker_attr(a), d["m_" + k]), k
    assert np.all(ctx.get_marker_attr(mdz.M_CMUL) == 1.0)
    out = mdz.GridFields(g, nph)
    ctx.download_fields(out)
    for k in ("u", "v", "p"):
        assert np.array_equal(out[k], d[k]), k
    ctx.close()
