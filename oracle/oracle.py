"""ctypes wrapper of the CPU oracle (oracle/mdz_oracle.c, built to
oracle/_build/libmdz_oracle.so).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, always as the reference the GPU results are
compared with or as the reported CPU time, never as the thing measured or shipped.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmdz_oracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_sp = C.POINTER(C.c_int8)

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle not built: run `make -C oracle port`")
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _s(a):
    return a.ctypes.data_as(_sp) if a is not None else None


class Oracle:
    """Oracle bound to one grid (an mdz.Grid) and one marker set."""

    def __init__(self, grid, n_phases):
        self.grid = grid
        self.n_phases = n_phases
        self._desc = grid.desc()
        self.L = lib()
        self.x = self.z = self.phase = None

    def set_markers(self, x, z, phase):
        self.x = np.array(x, np.float64)
        self.z = np.array(z, np.float64)
        self.phase = np.array(phase, np.int32)

    @property
    def n(self):
        return 0 if self.x is None else len(self.x)

    def P2Mastah(self, mat_prop, node_field, node_type, flag, avg, prop, centroid, itp_stencil):
        nn = self.grid.size(centroid)
        nf = np.array(node_field if node_field is not None else np.zeros(nn), np.float64)
        mp = np.ascontiguousarray(mat_prop, np.float64) if mat_prop is not None else None
        tags = np.ascontiguousarray(node_type, np.int8) if node_type is not None else None
        pp = np.zeros((self.n_phases, nn)) if prop == 1 else None
        r = self.L.orc_p2g(C.byref(self._desc), C.c_int(self.n), _d(self.x), _d(self.z), _i(self.phase),
                           C.c_int(self.n_phases), _d(mp), _d(nf), _s(tags), C.c_int(flag), C.c_int(avg),
                           C.c_int(prop), C.c_int(centroid), C.c_int(itp_stencil), _d(pp))
        assert r == 0
        return pp if prop == 1 else nf

    def count_markers(self):
        g = self.grid
        nc, nv = g.size(1), g.size(0)
        c, v = np.zeros(nc, np.int32), np.zeros(nv, np.int32)
        pc, pv = np.zeros((self.n_phases, nc), np.int32), np.zeros((self.n_phases, nv), np.int32)
        self.L.orc_count(C.byref(self._desc), C.c_int(self.n), _d(self.x), _d(self.z), _i(self.phase),
                         C.c_int(self.n_phases), _i(c), _i(v), _i(pc), _i(pv))
        return c, v, pc, pv

    def Interp_Grid2P(self, node_field, node_set):
        nf = np.ascontiguousarray(node_field, np.float64)
        out = np.zeros(self.n)
        self.L.orc_g2p(C.byref(self._desc), C.c_int(self.n), _d(self.x), _d(self.z), _i(self.phase), _d(nf),
                       C.c_int(node_set), _d(out))
        return out

    def RogerGuntherII(self, u, v, dt):
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        vx, vz = np.zeros(self.n), np.zeros(self.n)
        self.L.orc_rk4(C.byref(self._desc), C.c_int(self.n), _d(self.x), _d(self.z), _i(self.phase), _d(vx),
                       _d(vz), _d(u), _d(v), C.c_double(dt))
        return vx, vz


# marker attribute order of include/mdoodz_gpu.h (MDZ_M_SXXD ... MDZ_M_P)
MARKER_ATTRS = ("sxxd", "szzd", "sxz", "strain_pl", "strain", "T", "cmul", "P")


def reseed(grid, markers, cap, min_part_cell=16, direct=0, T_n=None, sxxd_n=None, szzd_n=None, sxz_s=None,
           p_n=None):
    """Marker reseeding of CountPartCell (RESEED = 1, one thread): returns a
    new markers dict (keys x, z, phase, vx, vz and MARKER_ATTRS, length = the
    new count) and the number of markers created.  Raises RuntimeError where
    the reference exits."""
    n = len(markers["x"])
    out = {}
    for k in ("x", "z", "vx", "vz") + MARKER_ATTRS:
        a = np.zeros(cap)
        a[:n] = markers[k]
        out[k] = a
    out["phase"] = np.full(cap, -1, np.int32)
    out["phase"][:n] = markers["phase"]
    attrs = (_dp * len(MARKER_ATTRS))(*[_d(out[k]) for k in MARKER_ATTRS])
    g = grid
    nc, nv = (g.Nx - 1) * (g.Nz - 1), g.Nx * g.Nz
    z0 = np.zeros(max(nc, nv))
    fld = [np.ascontiguousarray(a if a is not None else z0, np.float64) for a in (T_n, sxxd_n, szzd_n, sxz_s, p_n)]
    added = C.c_int(0)
    desc = grid.desc()
    r = lib().orc_reseed(C.byref(desc), C.c_int(n), C.c_int(cap), _d(out["x"]), _d(out["z"]), _i(out["phase"]),
                         _d(out["vx"]), _d(out["vz"]), attrs, C.c_int(min_part_cell), C.c_int(direct),
                         _d(fld[0]), _d(fld[1]), _d(fld[2]), _d(fld[3]), _d(fld[4]), C.byref(added))
    if r == -1:
        raise RuntimeError("reseed: a deficient quarter cell has no marker within two quarter cells")
    if r == -2:
        raise RuntimeError("reseed: capacity exceeded")
    return {k: v[:r].copy() for k, v in out.items()}, added.value


def strain_rates(grid, fields):
    s = fields.struct()
    lib().orc_strain_rates(C.byref(grid.desc()), C.byref(s))


def viscosity_grid(grid, mat, prm, fields):
    s = fields.struct()
    nc = np.zeros(2, np.int32)
    lib().orc_viscosity_grid(C.byref(grid.desc()), C.byref(mat), C.byref(prm), C.byref(s), _i(nc))
    return nc


def rheo_operators(grid, prm, fields, jacobian):
    s = fields.struct()
    lib().orc_rheo_operators(C.byref(grid.desc()), C.byref(prm), C.byref(s), C.c_int(jacobian))


def rhs(grid, prm, gx, gz, fields):
    s = fields.struct()
    lib().orc_rhs(C.byref(grid.desc()), C.byref(prm), C.c_double(gx), C.c_double(gz), C.byref(s))


def stokes_apply(grid, fields, jacobian, xu, xv, xp, residual=False):
    s = fields.struct()
    xu, xv, xp = (np.ascontiguousarray(a, np.float64) for a in (xu, xv, xp))
    yu, yv, yp = np.zeros_like(xu), np.zeros_like(xv), np.zeros_like(xp)
    lib().orc_stokes_apply(C.byref(grid.desc()), C.byref(s), C.c_int(jacobian), C.c_int(int(residual)), _d(xu),
                           _d(xv), _d(xp), _d(yu), _d(yv), _d(yp))
    return yu, yv, yp


def residual(grid, fields):
    s = fields.struct()
    norms = np.zeros(3)
    lib().orc_residual(C.byref(grid.desc()), C.byref(s), _d(norms))
    return norms
