"""Host-side mirror of the reference's C entry points for the GB300 path.

Thin ctypes layer over libmdoodz_gb300.so (include/mdoodz_gpu.h).  Function
names follow the reference (P2Mastah, Interp_Grid2P, RogerGuntherII, ...) and
take the same arguments; errors raise MdzError carrying the library's message
where the reference would have printed and exit()ed.

There is no CPU fallback: if the library or a CUDA device is missing, every
entry point raises.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libmdoodz_gb300.so")

MDZ_MAX_PHASES = 20
MDZ_P2G_MAX_FIELDS = 8
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_CAPACITY", 4: "ERR_UNSUPPORTED", 5: "ERR_NOT_CONVERGED",
          6: "ERR_NAN", 7: "ERR_STATE"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_sp = C.POINTER(C.c_int8)


class MdzError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class GridDesc(C.Structure):
    _fields_ = [("Nx", C.c_int), ("Nz", C.c_int), ("dx", C.c_double), ("dz", C.c_double),
                ("xmin", C.c_double), ("xmax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double),
                ("xg", _dp), ("zg", _dp), ("xc", _dp), ("zc", _dp), ("xvz", _dp), ("zvx", _dp),
                ("BCu_type", _sp), ("BCv_type", _sp), ("BCp_type", _sp), ("BCg_type", _sp),
                ("BCu_val", _dp), ("BCv_val", _dp), ("isperiodic_x", C.c_int)]


_lib = None


def load_library(path=LIB_PATH):
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise MdzError(2, "CUDA library not built: %s (run __graft_entry__.build())" % path)
    L = C.CDLL(path)
    L.mdz_last_error.restype = C.c_char_p
    L.mdz_kernel_launches.restype = C.c_longlong
    L.mdz_marker_count.restype = C.c_int
    L.mdz_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(GridDesc), C.c_int, C.c_longlong]
    L.mdz_host_register.argtypes = [C.c_void_p, C.c_size_t]
    L.mdz_host_unregister.argtypes = [C.c_void_p]
    _lib = L
    return L


def host_register(a):
    """Page-lock the memory of a contiguous numpy array (mdz_host_register) so
    that uploads from it and downloads into it run as DMA copies."""
    st = load_library().mdz_host_register(C.c_void_p(a.ctypes.data), C.c_size_t(a.nbytes))
    if st:
        raise MdzError(st, "mdz_host_register: %d bytes refused" % a.nbytes)


def host_unregister(a):
    st = load_library().mdz_host_unregister(C.c_void_p(a.ctypes.data))
    if st:
        raise MdzError(st, "mdz_host_unregister refused")


def _dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _sptr(a):
    return a.ctypes.data_as(_sp) if a is not None else None


class Grid:
    """Staggered grid with the reference's coordinate lines and BC tags.

    Coordinates accumulate exactly as SetGridCoordinates does
    (SOURCE/GridRoutines.c:230-300), so index formulas agree bit for bit."""

    def __init__(self, Nx, Nz, xmin, xmax, zmin, zmax):
        self.Nx, self.Nz = int(Nx), int(Nz)
        self.regrid(xmin, xmax, zmin, zmax)
        self.BCu = np.full(Nx * (Nz + 1), -1, np.int8)
        self.BCv = np.full((Nx + 1) * Nz, -1, np.int8)
        self.BCp = np.full((Nx - 1) * (Nz - 1), -1, np.int8)
        self.BCg = np.full(Nx * Nz, -1, np.int8)
        self.BCu_val = np.zeros(Nx * (Nz + 1))
        self.BCv_val = np.zeros((Nx + 1) * Nz)

    def regrid(self, xmin, xmax, zmin, zmax):
        """Move the box to the given bounds and regenerate the grid lines over
        it (SetGridCoordinates; PureShearALE calls it after moving the walls).
        Tags and Dirichlet values are kept."""
        Nx, Nz = self.Nx, self.Nz
        self.xmin, self.xmax, self.zmin, self.zmax = float(xmin), float(xmax), float(zmin), float(zmax)
        self.dx = (self.xmax - self.xmin) / (Nx - 1)
        self.dz = (self.zmax - self.zmin) / (Nz - 1)
        lines = dict(xg=self._accum(self.xmin, self.dx, Nx), zg=self._accum(self.zmin, self.dz, Nz),
                     xc=self._accum(self.xmin + self.dx / 2.0, self.dx, Nx - 1),
                     zc=self._accum(self.zmin + self.dz / 2.0, self.dz, Nz - 1),
                     xvz=self._accum(self.xmin - self.dx / 2.0, self.dx, Nx + 1),
                     zvx=self._accum(self.zmin - self.dz / 2.0, self.dz, Nz + 1))
        for k, a in lines.items():   # in place: descriptions made earlier keep valid pointers
            if hasattr(self, k):
                getattr(self, k)[:] = a
            else:
                setattr(self, k, a)
        return self

    @staticmethod
    def _accum(x0, h, n):
        out = np.empty(n)
        v = x0
        for i in range(n):
            out[i] = v
            v = v + h
        return out

    @property
    def ncx(self):
        return self.Nx - 1

    @property
    def ncz(self):
        return self.Nz - 1

    def size(self, centroid):
        Nx, Nz = self.Nx, self.Nz
        return {1: (Nx - 1) * (Nz - 1), 0: Nx * Nz, -1: Nx * (Nz + 1), -2: (Nx + 1) * Nz}[centroid]

    def tags(self, centroid):
        return {1: self.BCp, 0: self.BCg, -1: self.BCu, -2: self.BCv}[centroid]

    def set_bc_pureshear(self, eps_bg):
        """Free-slip pure shear: the tag and value rules of the reference's
        shear_style = 0 setup (SOURCE/set_Shear_VEVP.c:177-265)."""
        Nx, Nz = self.Nx, self.Nz
        bu = self.BCu.reshape(Nz + 1, Nx)
        vu = self.BCu_val.reshape(Nz + 1, Nx)
        bu[:] = -1
        vu[:] = 0.0
        for k in (0, Nx - 1):
            bu[:, k] = 0
            vu[:, k] = -self.xg[k] * eps_bg
        bu[0, :] = 13
        bu[Nz, :] = 13
        vu[0, :] = 0.0
        vu[Nz, :] = 0.0
        bv = self.BCv.reshape(Nz, Nx + 1)
        vv = self.BCv_val.reshape(Nz, Nx + 1)
        bv[:] = -1
        vv[:] = 0.0
        for l in (0, Nz - 1):
            bv[l, :] = 0
            vv[l, :] = self.zg[l] * eps_bg
        bv[:, 0] = 13
        bv[:, Nx] = 13
        vv[:, 0] = 0.0
        vv[:, Nx] = 0.0
        self.BCp[:] = -1
        self.BCg[:] = -1
        return self

    def desc(self):
        d = GridDesc()
        d.Nx, d.Nz, d.dx, d.dz = self.Nx, self.Nz, self.dx, self.dz
        d.xmin, d.xmax, d.zmin, d.zmax = self.xmin, self.xmax, self.zmin, self.zmax
        d.xg, d.zg, d.xc, d.zc = _dptr(self.xg), _dptr(self.zg), _dptr(self.xc), _dptr(self.zc)
        d.xvz, d.zvx = _dptr(self.xvz), _dptr(self.zvx)
        d.BCu_type, d.BCv_type = _sptr(self.BCu), _sptr(self.BCv)
        d.BCp_type, d.BCg_type = _sptr(self.BCp), _sptr(self.BCg)
        d.BCu_val, d.BCv_val = _dptr(self.BCu_val), _dptr(self.BCv_val)
        d.isperiodic_x = 0
        return d


class RefBreakpointDesc(C.Structure):
    """mdz_ref_breakpoint_desc: the flags and scales of the reference run that
    wrote a Breakpoint%05d.dat."""
    _fields_ = [(n, C.c_int) for n in ("free_surf", "iselastic", "fstrain", "aniso", "rec_T_P_x_z")] + \
               [(n, C.c_double) for n in ("L", "V", "S", "T", "t")]


class ThermalBC(C.Structure):
    """mdz_thermal_bc (the reference's BCT BCt)."""
    _fields_ = [("type", _sp), ("typW", _sp), ("typE", _sp), ("typS", _sp), ("typN", _sp),
                ("valW", _dp), ("valE", _dp), ("valS", _dp), ("valN", _dp)]


class Context:
    """One device context: grid mirror + resident markers (mdz_create)."""

    def __init__(self, grid, n_phases, max_markers):
        self.L = load_library()
        self.grid = grid
        self.n_phases = int(n_phases)
        self._desc = grid.desc()
        h = C.c_void_p()
        st = self.L.mdz_create(C.byref(h), C.byref(self._desc), C.c_int(n_phases), C.c_longlong(max_markers))
        if st != 0:
            raise MdzError(st, "mdz_create failed (no usable CUDA device or bad grid)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.mdz_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            raise MdzError(st, self.L.mdz_last_error(self.h).decode())

    @property
    def kernel_launches(self):
        return int(self.L.mdz_kernel_launches(self.h))

    # markers ---------------------------------------------------------------
    def set_markers(self, x, z, phase):
        x = np.ascontiguousarray(x, np.float64)
        z = np.ascontiguousarray(z, np.float64)
        phase = np.ascontiguousarray(phase, np.int32)
        self._check(self.L.mdz_set_markers(self.h, C.c_int(len(x)), _dptr(x), _dptr(z), _iptr(phase)))

    def save_breakpoint(self, path):
        self._check(self.L.mdz_save_breakpoint(self.h, os.fsencode(path)))

    def load_breakpoint(self, path):
        """Restore a breakpoint; the context's grid (and self.grid) move to
        the box it was saved with."""
        self._check(self.L.mdz_load_breakpoint(self.h, os.fsencode(path)))
        self._follow_box()

    def load_reference_breakpoint(self, path, scales, iselastic=1, free_surf=0, fstrain=0, aniso=0,
                                  rec_T_P_x_z=0):
        """Restart from the reference's own breakpoint file (LoadBreakpointParticles'
        reading): scales = dict of the run's L, V, S, T, t.  Returns (dt, time)
        in scaled units; the context's grid follows the restored box."""
        d = RefBreakpointDesc(free_surf, iselastic, fstrain, aniso, rec_T_P_x_z,
                              *(float(scales[k]) for k in ("L", "V", "S", "T", "t")))
        dt, tm = C.c_double(0.0), C.c_double(0.0)
        self._check(self.L.mdz_load_reference_breakpoint(self.h, os.fsencode(path), C.byref(d), C.byref(dt),
                                                          C.byref(tm)))
        self._follow_box()
        return dt.value, tm.value

    # the box (PureShearALE) ---------------------------------------------------
    def get_box(self):
        """(xmin, xmax, zmin, zmax, dx, dz) of the grid the context works on."""
        b = (C.c_double * 6)()
        self._check(self.L.mdz_get_grid(self.h, b, None, None, None, None, None, None))
        return tuple(b)

    def _follow_box(self):
        b = self.get_box()
        g = self.grid
        if (b[0], b[1], b[2], b[3]) != (g.xmin, g.xmax, g.zmin, g.zmax):
            g.regrid(*b[:4])

    def pure_shear_ale(self, dt, u=None, v=None):
        """mdz_PureShearALE on host velocities u, v (or the resident ones):
        returns the new (xmin, xmax, zmin, zmax); self.grid follows."""
        b = (C.c_double * 4)()
        uu = None if u is None else np.ascontiguousarray(u, np.float64)
        vv = None if v is None else np.ascontiguousarray(v, np.float64)
        self._check(self.L.mdz_PureShearALE(self.h, _dptr(uu), _dptr(vv), C.c_double(dt), b))
        self._follow_box()
        return tuple(b)

    def set_boundary_values(self, grid=None):
        """Upload the Dirichlet values of `grid` (default self.grid)."""
        g = grid or self.grid
        self._check(self.L.mdz_set_boundary_values(self.h, _dptr(g.BCu_val), _dptr(g.BCv_val)))

    def set_marker_velocity(self, vx, vz):
        vx = np.ascontiguousarray(vx, np.float64)
        vz = np.ascontiguousarray(vz, np.float64)
        self._check(self.L.mdz_set_marker_velocity(self.h, C.c_int(len(vx)), _dptr(vx), _dptr(vz)))

    @property
    def n_markers(self):
        """Resident marker count (grows when reseeding appends markers)."""
        return int(self.L.mdz_marker_count(self.h)) if self.h else 0

    def get_markers(self, out=None):
        """(x, z, phase, vx, vz) of the resident markers; `out` may hold five
        preallocated arrays (e.g. registered with host_register) to fill."""
        n = self.n_markers
        if out is not None:
            x, z, ph, vx, vz = out
            for a, dt in ((x, np.float64), (z, np.float64), (ph, np.int32), (vx, np.float64), (vz, np.float64)):
                if a.dtype != dt or a.size < n or not a.flags.c_contiguous:
                    raise MdzError(1, "get_markers: out arrays must be contiguous x, z, vx, vz float64 and phase int32")
        else:
            x, z, vx, vz = np.empty(n), np.empty(n), np.empty(n), np.empty(n)
            ph = np.empty(n, np.int32)
        self._check(self.L.mdz_get_markers(self.h, C.c_int(n), _dptr(x), _dptr(z), _iptr(ph), _dptr(vx), _dptr(vz)))
        return x, z, ph, vx, vz

    # reference entry points -------------------------------------------------
    def P2Mastah(self, mat_prop, node_field, node_type, flag, avg, prop, centroid, itp_stencil):
        """P2Mastah (SOURCE/ParticleRoutines.c:3226).  Returns node_field (updated
        copy) for prop == 0, or the phase fractions (n_phases x nnodes) for prop == 1."""
        nn = self.grid.size(centroid)
        nf = np.array(node_field if node_field is not None else np.zeros(nn), np.float64)
        mp = np.ascontiguousarray(mat_prop, np.float64) if mat_prop is not None else None
        tags = np.ascontiguousarray(node_type, np.int8) if node_type is not None else None
        pp = np.zeros((self.n_phases, nn)) if prop == 1 else None
        self._check(self.L.mdz_P2Mastah(self.h, _dptr(mp), _dptr(nf), _sptr(tags), C.c_int(flag), C.c_int(avg),
                                        C.c_int(prop), C.c_int(centroid), C.c_int(itp_stencil), _dptr(pp)))
        return pp if prop == 1 else nf

    def count_markers(self):
        g = self.grid
        nc, nv = g.size(1), g.size(0)
        c, v = np.zeros(nc, np.int32), np.zeros(nv, np.int32)
        pc, pv = np.zeros((self.n_phases, nc), np.int32), np.zeros((self.n_phases, nv), np.int32)
        self._check(self.L.mdz_count_markers(self.h, _iptr(c), _iptr(v), _iptr(pc), _iptr(pv)))
        return c, v, pc, pv

    def CountPartCell(self, reseed=1, min_part_cell=16, direct_neighbour=0, T_n=None, sxxd_n=None, szzd_n=None,
                      sxz_s=None, p_n=None):
        """CountPartCell (SOURCE/ParticleRoutines.c:3543) with RESEED = reseed
        on the resident markers; returns the number of markers created."""
        a = [None if v is None else np.ascontiguousarray(v, np.float64) for v in (T_n, sxxd_n, szzd_n, sxz_s, p_n)]
        added = C.c_int(0)
        self._check(self.L.mdz_CountPartCell(self.h, C.c_int(reseed), C.c_int(min_part_cell),
                                             C.c_int(direct_neighbour), *[_dptr(v) if v is not None else None for v in a],
                                             C.byref(added)))
        return added.value

    def UpdateParticlePressure(self, fields):
        """UpdateParticlePressure (SOURCE/RheologyParticles.c:1004): the resident
        markers' pressure += the centroid increment p - p0_n of `fields`."""
        s = fields.struct()
        self._check(self.L.mdz_UpdateParticlePressure(self.h, C.byref(s)))

    def Interp_Grid2P(self, node_field, node_set):
        nf = np.ascontiguousarray(node_field, np.float64)
        out = np.zeros(self.n_markers)
        self._check(self.L.mdz_Interp_Grid2P(self.h, _dptr(nf), C.c_int(node_set), _dptr(out)))
        return out

    def RogerGuntherII(self, u, v, dt):
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        self._check(self.L.mdz_RogerGuntherII(self.h, _dptr(u), _dptr(v), C.c_double(dt)))

    # grid-side entry points (fields: a GridFields) --------------------------
    def StrainRateComponents(self, fields):
        s = fields.struct()
        self._check(self.L.mdz_StrainRateComponents(self.h, C.byref(s)))

    def NonNewtonianViscosityGrid(self, mat, prm, fields):
        s = fields.struct()
        nc = C.c_int(0)
        self._check(self.L.mdz_NonNewtonianViscosityGrid(self.h, C.byref(mat), C.byref(prm), C.byref(s),
                                                         C.byref(nc)))
        return nc.value

    def NonNewtonianViscosityGrid_learned(self, mat, prm, fields, learned):
        """Local rheology with or without the learned start; returns the
        statistics (not converged, fall-backs, learned starts, local updates)."""
        s = fields.struct()
        st = (C.c_longlong * 4)()
        self._check(self.L.mdz_NonNewtonianViscosityGrid_learned(self.h, C.byref(mat), C.byref(prm), C.byref(s),
                                                                 C.c_int(learned), st))
        return dict(failures=st[0], fallbacks=st[1], learned=st[2], iterations=st[3])

    # learned guess --------------------------------------------------------------
    MLP_NPARAM = 4866

    def mlp_init(self, seed):
        self._check(self.L.mdz_mlp_init(self.h, C.c_ulonglong(seed)))

    def mlp_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == self.MLP_NPARAM
        self._check(self.L.mdz_mlp_set_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float))))

    def mlp_get_weights(self):
        w = np.zeros(self.MLP_NPARAM, np.float32)
        self._check(self.L.mdz_mlp_get_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float))))
        return w

    def mlp_generate(self, mat, prm, n, seed, lo, hi):
        lo = np.ascontiguousarray(lo, np.float64)
        hi = np.ascontiguousarray(hi, np.float64)
        self._check(self.L.mdz_mlp_generate(self.h, C.byref(mat), C.byref(prm), C.c_longlong(n), C.c_ulonglong(seed),
                                            _dptr(lo), _dptr(hi)))

    def mlp_train(self, steps, batch, lr):
        loss = C.c_double(0)
        self._check(self.L.mdz_mlp_train(self.h, C.c_int(steps), C.c_int(batch), C.c_double(lr), C.byref(loss)))
        return loss.value

    def mlp_gradients(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(self.MLP_NPARAM, np.float32)
        loss = C.c_double(0)
        fp = C.POINTER(C.c_float)
        self._check(self.L.mdz_mlp_gradients(self.h, C.c_int(len(x)), x.ctypes.data_as(fp), y.ctypes.data_as(fp),
                                             g.ctypes.data_as(fp), C.byref(loss)))
        return g, loss.value

    def mlp_infer(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((len(x), 2), np.float32)
        fp = C.POINTER(C.c_float)
        self._check(self.L.mdz_mlp_infer(self.h, C.c_longlong(len(x)), x.ctypes.data_as(fp), y.ctypes.data_as(fp)))
        return y

    def EnergyDirectSolve(self, fields, bc, dt, gz=0.0, shear_heating=0, adiab_heating=0, scale_T=1.0, rel_tol=0.0,
                          max_iterations=0):
        """mdz_EnergyDirectSolve: one implicit energy step on `fields` (T and
        dT are written back); bc: dict of the thermal boundary arrays (type,
        typW, typE, typS, typN as int8, valW, valE, valS, valN).  Returns
        (iterations, relative residual)."""
        arrs = {k: np.ascontiguousarray(bc[k], np.int8) for k in ("type", "typW", "typE", "typS", "typN")}
        arrs.update({k: np.ascontiguousarray(bc[k], np.float64) for k in ("valW", "valE", "valS", "valN")})
        b = ThermalBC(*[(_sptr if k.startswith("t") else _dptr)(arrs[k]) for k, _ in ThermalBC._fields_])
        s = fields.struct()
        its, rel = C.c_int(0), C.c_double(0)
        self._check(self.L.mdz_EnergyDirectSolve(self.h, C.byref(s), C.byref(b), C.c_double(dt), C.c_double(gz),
                                                 C.c_int(shear_heating), C.c_int(adiab_heating),
                                                 C.c_double(scale_T), C.c_double(rel_tol), C.c_int(max_iterations),
                                                 C.byref(its), C.byref(rel)))
        return its.value, rel.value

    def mlp_set_engine(self, engine):
        """Inference and training kernels: 0 tcgen05 (tensor memory accumulators), 1 mma.sync."""
        self._check(self.L.mdz_mlp_set_engine(self.h, C.c_int(engine)))

    def mlp_benchmark(self, batch, reps):
        a, b, c = C.c_double(0), C.c_double(0), C.c_double(0)
        self._check(self.L.mdz_mlp_benchmark(self.h, C.c_int(batch), C.c_int(reps), C.byref(a), C.byref(b),
                                             C.byref(c)))
        return dict(ms_infer=a.value, ms_train_step=b.value, rms_error=c.value)

    def ShearModCompExpGrid(self, mat, fields):
        """ShearModCompExpGrid (SOURCE/RheologyDensity.c:1666): mu_n, mu_s,
        bet_n, bet_s of `fields` from its phase fractions."""
        s = fields.struct()
        self._check(self.L.mdz_ShearModCompExpGrid(self.h, C.byref(mat), C.byref(s)))

    def CohesionFrictionDilationGrid(self, mat, itp_stencil, fields):
        """CohesionFrictionDilationGrid (SOURCE/RheologyDensity.c:1422): C, fric,
        dil (and strain) at centroids and vertices of `fields` from its phase
        fractions and the resident markers' plastic strain."""
        s = fields.struct()
        self._check(self.L.mdz_CohesionFrictionDilationGrid(self.h, C.byref(mat), C.c_int(itp_stencil), C.byref(s)))

    def RheologicalOperators(self, prm, fields, jacobian):
        s = fields.struct()
        self._check(self.L.mdz_RheologicalOperators(self.h, C.byref(prm), C.byref(s), C.c_int(jacobian)))

    def EvaluateRHS(self, prm, gx, gz, fields):
        s = fields.struct()
        self._check(self.L.mdz_EvaluateRHS(self.h, C.byref(prm), C.c_double(gx), C.c_double(gz), C.byref(s)))

    def EvaluateStokesResidualDecoupled(self, fields):
        s = fields.struct()
        norms = np.zeros(3)
        self._check(self.L.mdz_EvaluateStokesResidualDecoupled(self.h, C.byref(s), _dptr(norms)))
        return norms

    # resident state and the time step -----------------------------------------
    def set_marker_attr(self, attr, values):
        v = np.ascontiguousarray(values, np.float64)
        self._check(self.L.mdz_set_marker_attr(self.h, C.c_int(attr), C.c_int(len(v)), _dptr(v)))

    def set_marker_state(self, x, z, phase, attrs):
        """Upload positions, phases and attributes ({attr index: array}) in
        one batched call (mdz_set_marker_state); arrays are used in place and
        must be contiguous float64 (phase int32)."""
        n = len(x)
        for a in [x, z] + list(attrs.values()):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size < n:
                raise MdzError(1, "set_marker_state: contiguous float64 arrays of the marker count")
        if phase.dtype != np.int32 or not phase.flags.c_contiguous:
            raise MdzError(1, "set_marker_state: phase must be contiguous int32")
        tab = (_dp * M_NATTR)()
        for a, v in attrs.items():
            tab[a] = _dptr(v)
        self._check(self.L.mdz_set_marker_state(self.h, C.c_int(n), _dptr(x), _dptr(z), _iptr(phase), tab))

    def get_marker_state(self, out, attrs):
        """Download (x, z, phase, vx, vz) into the five arrays of `out` (None
        to skip one) and the attributes into {attr index: array}, in one batched
        call (mdz_get_marker_state)."""
        n = self.n_markers
        x, z, ph, vx, vz = out
        tab = (_dp * M_NATTR)()
        for a, v in attrs.items():
            if v.dtype != np.float64 or v.size < n or not v.flags.c_contiguous:
                raise MdzError(1, "get_marker_state: contiguous float64 arrays of the marker count")
            tab[a] = _dptr(v)
        self._check(self.L.mdz_get_marker_state(self.h, C.c_int(n), _dptr(x), _dptr(z), _iptr(ph), _dptr(vx),
                                                _dptr(vz), tab))

    def Interp_Phase2VizGrid(self, res_fact):
        """(compo as int8, xviz, zviz) of the visualisation grid of res_fact x
        the grid resolution (mdz_Interp_Phase2VizGrid)."""
        g = self.grid
        nxv, nzv = res_fact * (g.Nx - 1) + 1, res_fact * (g.Nz - 1) + 1
        compo = np.zeros((nxv - 1) * (nzv - 1), np.int8)
        xv, zv = np.zeros(nxv), np.zeros(nzv)
        self._check(self.L.mdz_Interp_Phase2VizGrid(self.h, C.c_int(res_fact), _sptr(compo), _dptr(xv), _dptr(zv)))
        return compo, xv, zv

    def output_field(self, name, scale, size):
        """float32 copy of a resident field, scaled back (mdz_output_field)."""
        out = np.zeros(size, np.float32)
        self._check(self.L.mdz_output_field(self.h, os.fsencode(name), C.c_double(scale),
                                            out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def get_marker_attr(self, attr, out=None):
        n = self.n_markers
        v = np.zeros(n) if out is None else out
        if v.dtype != np.float64 or v.size < n or not v.flags.c_contiguous:
            raise MdzError(1, "get_marker_attr: out must be a contiguous float64 array of the marker count")
        self._check(self.L.mdz_get_marker_attr(self.h, C.c_int(attr), C.c_int(n), _dptr(v)))
        return v

    def upload_fields(self, fields):
        s = fields.struct()
        self._check(self.L.mdz_sync_fields(self.h, C.byref(s), C.c_int(1)))

    def download_fields(self, fields):
        s = fields.struct()
        self._check(self.L.mdz_sync_fields(self.h, C.byref(s), C.c_int(0)))

    def set_profiling(self, on):
        self._check(self.L.mdz_set_profiling(self.h, C.c_int(int(on))))

    KERNEL_CLASSES = ["local_rheology", "stokes_apply", "mg_vcycle", "projection", "mlp_guess", "krylov", "mg_setup"]

    def kernel_timing(self):
        """Summed event time, algorithmic bytes and launch count per kernel class,
        plus the dominant class (largest time)."""
        out = {}
        for i, name in enumerate(self.KERNEL_CLASSES):
            ms, by, n = C.c_double(0), C.c_double(0), C.c_longlong(0)
            self._check(self.L.mdz_kernel_timing(self.h, C.c_int(i), C.byref(ms), C.byref(by), C.byref(n)))
            out[name] = dict(ms=ms.value, bytes=by.value, launches=n.value)
        dom = max(out, key=lambda k: out[k]["ms"])
        d = dict(out[dom])
        d["name"] = dom
        d["classes"] = out
        return d

    def time_step(self, mat, model):
        """mdz_time_step; with model.ispureshear_ale the box moves and
        self.grid follows it (its Dirichlet values for the next step are the
        setup's to renew: set_boundary_values)."""
        rep = StepReport()
        self._check(self.L.mdz_time_step(self.h, C.byref(mat), C.byref(model), C.byref(rep)))
        if model.ispureshear_ale:
            self._follow_box()
        return rep

    def SolveStokesDefect(self, fields, jacobian, precision, rtol, maxit, Fu, Fv, Fp):
        """Solve K dx = F; returns (dxu, dxv, dxp, iterations, relative residual)."""
        s = fields.struct()
        Fu, Fv, Fp = (np.ascontiguousarray(a, np.float64) for a in (Fu, Fv, Fp))
        du, dv, dp = np.zeros_like(Fu), np.zeros_like(Fv), np.zeros_like(Fp)
        its, rel = C.c_int(0), C.c_double(0)
        self._check(self.L.mdz_SolveStokesDefect(self.h, C.byref(s), C.c_int(jacobian), C.c_int(precision),
                                                 C.c_double(rtol), C.c_int(maxit), _dptr(Fu), _dptr(Fv), _dptr(Fp),
                                                 _dptr(du), _dptr(dv), _dptr(dp), C.byref(its), C.byref(rel)))
        return du, dv, dp, its.value, rel.value

    def set_solver_options(self, nu1=2, nu2=1, omega=0.7, restart=30, check=1, mg_jacobian=0):
        self._check(self.L.mdz_set_solver_options(self.h, C.c_int(nu1), C.c_int(nu2), C.c_double(omega),
                                                  C.c_int(restart), C.c_int(check), C.c_int(mg_jacobian)))

    def set_schur_scaling(self, mode):
        """Pressure block of Newton solves: 0 eta_n / cell volume, 1 the
        Jacobian's tangent D11 / 2 where positive."""
        self._check(self.L.mdz_set_schur_scaling(self.h, C.c_int(mode)))

    def mg_stencils(self, precision, level):
        """(levels, Nx, Nz, su[31, Nx*(Nz+1)], sv[31, (Nx+1)*Nz]) of one multigrid level."""
        nl, nx, nz = C.c_int(0), C.c_int(0), C.c_int(0)
        self._check(self.L.mdz_mg_stencils(self.h, C.c_int(precision), C.c_int(level), C.byref(nl), C.byref(nx),
                                           C.byref(nz), None, None))
        su = np.zeros((31, nx.value * (nz.value + 1)))
        sv = np.zeros((31, (nx.value + 1) * nz.value))
        self._check(self.L.mdz_mg_stencils(self.h, C.c_int(precision), C.c_int(level), C.byref(nl), C.byref(nx),
                                           C.byref(nz), _dptr(su), _dptr(sv)))
        return nl.value, nx.value, nz.value, su, sv

    def StokesOperatorApply(self, fields, jacobian, xu, xv, xp):
        s = fields.struct()
        xu, xv, xp = (np.ascontiguousarray(a, np.float64) for a in (xu, xv, xp))
        yu, yv, yp = np.zeros_like(xu), np.zeros_like(xv), np.zeros_like(xp)
        self._check(self.L.mdz_StokesOperatorApply(self.h, C.byref(s), C.c_int(jacobian), _dptr(xu), _dptr(xv),
                                                   _dptr(xp), _dptr(yu), _dptr(yv), _dptr(yp)))
        return yu, yv, yp


# ---- grid fields / rheology structures (mdz_fields, mdz_materials, mdz_rheo_params) ----
FIELD_NAMES = [
    "u", "v", "p", "p_corr",
    "div_u", "div_u_s", "exxd", "ezzd", "exz", "exz_n", "exxd_s", "ezzd_s",
    "sxxd0", "szzd0", "sxz0", "sxxd0_s", "szzd0_s", "sxz0_n",
    "mu_n", "mu_s", "T", "T_s", "P_s", "d0_n", "d0_s", "phi0_n", "phi0_s", "X0_n", "X0_s",
    "strain_n", "strain_s", "dil_n", "dil_s", "fric_n", "fric_s", "C_n", "C_s", "p0_n", "p0_s",
    "bet_n", "bet_s", "rho_n", "rho_s",
    "phase_perc_n", "phase_perc_s",
    "eta_n", "eta_s", "eta_phys_n", "eta_phys_s", "VE_n", "VE_s", "sxxd", "szzd", "sxz", "sxz_n",
    "eII_el", "eII_pl", "eII_pwl", "eII_lin", "eII_cst", "d_n",
    "exx_el", "ezz_el", "exz_el", "exx_diss", "ezz_diss", "exz_diss",
    "detadexx_n", "detadezz_n", "detadgxz_n", "detadp_n",
    "ddivpdexx_n", "ddivpdezz_n", "ddivpdgxz_n", "ddivpdp_n",
    "detadexx_s", "detadezz_s", "detadgxz_s", "detadp_s",
    "div_u_el", "div_u_pl", "div_u_r", "Wtot", "Wel", "Wdiss", "X_n", "X_s", "OverS_n", "OverS_s",
    "D11_n", "D12_n", "D13_n", "D14_n", "D21_n", "D22_n", "D23_n", "D24_n",
    "D31_s", "D32_s", "D33_s", "D34_s",
    "roger_x", "roger_z", "rhs_p", "gx", "gz",
    "ru", "rv", "rp", "eII_exp", "eII_gbs",
    "kx", "kz", "Cv", "Qr", "dT", "alp",
]

VERTEX_FIELDS = {"div_u_s", "exz", "exxd_s", "ezzd_s", "sxz0", "sxxd0_s", "szzd0_s", "mu_s", "T_s", "P_s", "d0_s",
                 "phi0_s", "X0_s", "strain_s", "dil_s", "fric_s", "C_s", "p0_s", "bet_s", "rho_s", "eta_s",
                 "eta_phys_s", "VE_s", "sxz", "exz_el", "exz_diss", "detadexx_s", "detadezz_s", "detadgxz_s",
                 "detadp_s", "X_s", "OverS_s", "D31_s", "D32_s", "D33_s", "D34_s"}
VX_FIELDS = {"u", "roger_x", "gx", "ru", "kx"}
VZ_FIELDS = {"v", "roger_z", "gz", "rv", "kz"}


def field_size(grid, name, n_phases=1):
    if name in VX_FIELDS:
        return grid.size(-1)
    if name in VZ_FIELDS:
        return grid.size(-2)
    if name == "phase_perc_n":
        return n_phases * grid.size(1)
    if name == "phase_perc_s":
        return n_phases * grid.size(0)
    if name in VERTEX_FIELDS:
        return grid.size(0)
    return grid.size(1)


class FieldsStruct(C.Structure):
    _fields_ = [(n, _dp) for n in FIELD_NAMES]


class GridFields:
    """Host arrays for every mdz_fields member (zero-initialised), by name."""

    def __init__(self, grid, n_phases, init=None):
        self.grid, self.n_phases = grid, n_phases
        self.a = {n: np.zeros(field_size(grid, n, n_phases)) for n in FIELD_NAMES}
        for k, v in (init or {}).items():
            self.a[k][:] = np.asarray(v, np.float64).ravel()

    def __getitem__(self, k):
        return self.a[k]

    def __setitem__(self, k, v):
        self.a[k][:] = np.asarray(v, np.float64).ravel()

    def struct(self):
        s = FieldsStruct()
        for n in FIELD_NAMES:
            setattr(s, n, self.a[n].ctypes.data_as(_dp))
        return s


MAT_INT = ["cstv", "pwlv", "linv", "expv", "gbsv", "gs", "is_tensile", "reac_soft", "phase_mix"]
MAT_DBL = ["eta0", "rho", "alp", "gs_ref", "Slim", "eta_vp", "n_vp",
           "npwl", "Apwl", "Qpwl", "Vpwl", "mpwl", "rpwl", "fpwl", "apwl", "Fpwl", "pref_pwl",
           "nlin", "Alin", "Qlin", "Vlin", "mlin", "rlin", "flin", "alin", "Flin"]
MAT_DBL2 = ["mu", "bet", "C", "phi", "psi", "C_end", "phi_end", "psi_end", "pls_start", "pls_end"]
MAT_INT2 = ["coh_soft", "phi_soft", "psi_soft"]
MAT_DBL3 = ["Qexp", "Sexp", "Eexp", "Gexp", "nexp",
            "ngbs", "Agbs", "Qgbs", "Vgbs", "mgbs", "rgbs", "fgbs", "agbs", "Fgbs"]


class Materials(C.Structure):
    _fields_ = ([("n_phases", C.c_int), ("R", C.c_double)]
                + [(n, C.c_int * MDZ_MAX_PHASES) for n in MAT_INT]
                + [(n, C.c_double * MDZ_MAX_PHASES) for n in MAT_DBL]
                + [(n, C.c_double * MDZ_MAX_PHASES) for n in MAT_DBL2]
                + [(n, C.c_int * MDZ_MAX_PHASES) for n in MAT_INT2]
                + [(n, C.c_double * MDZ_MAX_PHASES) for n in MAT_DBL3])

    @classmethod
    def from_phases(cls, phases, R=8.314510):
        m = cls()
        m.n_phases = len(phases)
        m.R = R
        for p, props in enumerate(phases):
            for k, v in props.items():
                getattr(m, k)[p] = v
        return m


class RheoParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("iselastic", C.c_int), ("step", C.c_int), ("eta_avg", C.c_int),
                ("mineta", C.c_double), ("maxeta", C.c_double), ("scale_T", C.c_double), ("scale_E", C.c_double),
                ("scale_S", C.c_double), ("scale_eta", C.c_double), ("scale_L", C.c_double),
                ("clamp_tangent", C.c_int)]

    @classmethod
    def make(cls, dt, iselastic=1, step=1, eta_avg=0, mineta=1e-100, maxeta=1e100, scale_T=1.0, scale_E=1.0,
             scale_S=1.0, scale_eta=1.0, scale_L=1.0, clamp_tangent=0):
        return cls(dt, iselastic, step, eta_avg, mineta, maxeta, scale_T, scale_E, scale_S, scale_eta, scale_L,
                   clamp_tangent)


# marker attributes (enum in include/mdoodz_gpu.h)
M_SXXD, M_SZZD, M_SXZ, M_STRAIN_PL, M_STRAIN, M_T, M_CMUL, M_P = range(8)
M_NATTR = 8


class Model(C.Structure):
    """mdz_model: switches of one time step."""
    _fields_ = [("rheo", RheoParams), ("gx", C.c_double), ("gz", C.c_double), ("newton", C.c_int),
                ("nit_max", C.c_int), ("rel_tol", C.c_double), ("abs_tol", C.c_double), ("lin_rtol", C.c_double),
                ("lin_maxit", C.c_int), ("line_search", C.c_int), ("line_search_min", C.c_double),
                ("precision", C.c_int), ("learned_guess", C.c_int), ("itp_stencil", C.c_int),
                ("softening", C.c_int), ("advect", C.c_int), ("picard2newton", C.c_int),
                ("pic2newt_cond", C.c_double), ("nit_pic_max", C.c_int), ("newton_maxit", C.c_int),
                ("adaptive_lin_tol", C.c_int), ("fp32_rheology_its", C.c_int), ("mg_reuse_below", C.c_double),
                ("reseed", C.c_int), ("min_part_cell", C.c_int), ("direct_neighbour", C.c_int),
                ("ispureshear_ale", C.c_int)]

    @classmethod
    def make(cls, rheo, gx=0.0, gz=0.0, newton=1, nit_max=10, rel_tol=1e-8, abs_tol=1e-300, lin_rtol=1e-5,
             lin_maxit=500, line_search=0, line_search_min=0.0, precision=64, learned_guess=0, itp_stencil=1,
             softening=0, advect=1, picard2newton=0, pic2newt_cond=1e-1, nit_pic_max=10, newton_maxit=0,
             adaptive_lin_tol=0, fp32_rheology_its=0, mg_reuse_below=0.0, reseed=0, min_part_cell=16,
             direct_neighbour=0, ispureshear_ale=0):
        return cls(rheo, gx, gz, newton, nit_max, rel_tol, abs_tol, lin_rtol, lin_maxit, line_search,
                   line_search_min, precision, learned_guess, itp_stencil, softening, advect, picard2newton,
                   pic2newt_cond, nit_pic_max, newton_maxit, adaptive_lin_tol, fp32_rheology_its, mg_reuse_below,
                   reseed, min_part_cell, direct_neighbour, ispureshear_ale)


class StepReport(C.Structure):
    _fields_ = [("nonlinear_its", C.c_int), ("linear_its", C.c_int), ("converged", C.c_int), ("stagnated", C.c_int),
                ("picard_fallbacks", C.c_int), ("res0", C.c_double * 3), ("res", C.c_double * 3), ("local_solves", C.c_longlong),
                ("local_fallbacks", C.c_longlong), ("local_failures", C.c_longlong),
                ("ms_projection", C.c_double), ("ms_rheology", C.c_double), ("ms_residual", C.c_double),
                ("ms_solve", C.c_double), ("ms_line_search", C.c_double), ("ms_markers", C.c_double),
                ("ms_total", C.c_double), ("newton_its", C.c_int), ("local_iterations", C.c_longlong),
                ("res_history", (C.c_double * 3) * 32), ("lin_its_history", C.c_int * 32),
                ("lin_rel_history", C.c_double * 32), ("newton_history", C.c_int * 32),
                ("precision_fallbacks", C.c_int), ("markers_added", C.c_int),
                ("xmin", C.c_double), ("xmax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double)]

    def as_dict(self):
        def plain(v):
            return [plain(x) for x in v] if hasattr(v, "__len__") else v
        d = {}
        for name, _ in self._fields_:
            d[name] = plain(getattr(self, name))
        if d["nonlinear_its"] < 32:   # history rows past the last iteration are empty
            n = d["nonlinear_its"] + 1
            for key in ("res_history", "lin_its_history", "lin_rel_history", "newton_history"):
                d[key] = d[key][:n]
        return d
