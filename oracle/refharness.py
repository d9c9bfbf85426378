"""ctypes wrapper around oracle/_ref/libmdoodz_ref.so: the reference's own
hot-path C functions, compiled in place from the reference sources
(``make -C oracle ref``).

Test infrastructure only.  Used to generate the golden fixtures under
tests/golden/ and to pin the C restatement (oracle/mdz_oracle.c) against the
reference in this container; the reference sources are not present on the GPU
machine, so nothing that runs there imports this module.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libmdoodz_ref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_cp = C.POINTER(C.c_char)


def available():
    return os.path.exists(LIB_PATH)


class RefMDOODZ:
    """One reference grid + marker set.  The library keeps global state, so
    only one instance is meaningful per process."""

    def __init__(self, Nx, Nz, xmin, xmax, zmin, zmax, nphases):
        self.lib = L = C.CDLL(LIB_PATH)
        L.ref_field.restype = _dp
        L.ref_tags.restype = _cp
        L.ref_phase_perc.restype = _dp
        L.ref_count_array.restype = _ip
        L.ref_marker_field.restype = _dp
        L.ref_marker_phase.restype = _ip
        L.ref_dx.restype = C.c_double
        L.ref_dz.restype = C.c_double
        L.ref_get_model.restype = C.c_double
        L.ref_eqn.restype = _ip
        L.ref_residual_vec.restype = _dp
        L.ref_rhs_vec.restype = _dp
        L.ref_bct_tags.restype = _cp
        L.ref_bct_vals.restype = _dp
        L.ref_set_param.argtypes = [C.c_char_p, C.c_double]
        L.ref_set_mat.argtypes = [C.c_char_p, C.c_int, C.c_double]
        L.ref_setup(C.c_int(Nx), C.c_int(Nz), C.c_double(xmin), C.c_double(xmax), C.c_double(zmin),
                    C.c_double(zmax), C.c_int(nphases))
        self.Nx, self.Nz, self.nph = Nx, Nz, nphases
        self.n_markers = 0

    # sizes of each node set
    def size(self, kind):
        Nx, Nz = self.Nx, self.Nz
        return {"n": (Nx - 1) * (Nz - 1), "s": Nx * Nz, "u": Nx * (Nz + 1), "v": (Nx + 1) * Nz,
                "xg": Nx, "zg": Nz, "xc": Nx - 1, "zc": Nz - 1, "xvz": Nx + 1, "zvx": Nz + 1}[kind]

    _KIND = {
        "u_in": "u", "v_in": "v", "roger_x": "u", "ru": "u", "BCu_val": "u", "gx": "u", "kx": "u", "kz": "v",
        "roger_z": "v", "rv": "v", "BCv_val": "v", "gz": "v",
        "xg_coord": "xg", "zg_coord": "zg", "xc_coord": "xc", "zc_coord": "zc", "xvz_coord": "xvz",
        "zvx_coord": "zvx",
    }
    _VERTEX = {"exz", "exxd_s", "ezzd_s", "sxz", "sxz0", "sxxd0_s", "szzd0_s", "eta_s", "eta_phys_s", "VE_s", "mu_s",
               "T_s", "P_s", "d0_s", "phi0_s", "X0_s", "strain_s", "p0_s", "bet_s", "rho_s", "C_s", "fric_s", "dil_s",
               "exz_el", "exz_diss", "OverS_s", "X_s", "D31_s", "D32_s", "D33_s", "D34_s", "detadexx_s",
               "detadezz_s", "detadgxz_s", "detadp_s", "div_u_s"}

    def field(self, name):
        """numpy view of a reference grid array (writes go into the reference)."""
        kind = self._KIND.get(name, "s" if name in self._VERTEX else "n")
        ptr = self.lib.ref_field(name.encode())
        if not ptr:
            raise KeyError(name)
        return np.ctypeslib.as_array(ptr, shape=(self.size(kind),))

    def tags(self, name):
        kind = {"BCu": "u", "BCv": "v", "BCp": "n", "BCg": "s"}[name]
        ptr = self.lib.ref_tags(name.encode())
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_int8)), shape=(self.size(kind),))

    def phase_perc(self, centroid, p):
        ptr = self.lib.ref_phase_perc(C.c_int(centroid), C.c_int(p))
        return np.ctypeslib.as_array(ptr, shape=(self.size("n" if centroid else "s"),))

    def counts(self, centroid):
        ptr = self.lib.ref_count_array(C.c_int(centroid))
        return np.ctypeslib.as_array(ptr, shape=(self.size("n" if centroid else "s"),))

    def set_param(self, name, v):
        if self.lib.ref_set_param(name.encode(), float(v)) != 0:
            raise KeyError(name)

    def set_mat(self, name, p, v):
        if self.lib.ref_set_mat(name.encode(), int(p), float(v)) != 0:
            raise KeyError(name)

    def set_bc_pureshear(self, eps_bg):
        self.lib.ref_set_bc_pureshear(C.c_double(eps_bg))

    @property
    def dx(self):
        return self.lib.ref_dx()

    @property
    def dz(self):
        return self.lib.ref_dz()

    # markers -------------------------------------------------------------
    def set_markers(self, x, z, phase):
        x = np.ascontiguousarray(x, np.float64)
        z = np.ascontiguousarray(z, np.float64)
        phase = np.ascontiguousarray(phase, np.int32)
        self.n_markers = len(x)
        self.lib.ref_set_markers(C.c_int(len(x)), x.ctypes.data_as(_dp), z.ctypes.data_as(_dp),
                                 phase.ctypes.data_as(_ip))

    def set_markers_cap(self, x, z, phase, cap):
        """Markers with room for cap of them (reseeding)."""
        x = np.ascontiguousarray(x, np.float64)
        z = np.ascontiguousarray(z, np.float64)
        phase = np.ascontiguousarray(phase, np.int32)
        self.n_markers = len(x)
        self.cap = cap
        self.lib.ref_set_markers_cap(C.c_int(len(x)), C.c_int(cap), x.ctypes.data_as(_dp), z.ctypes.data_as(_dp),
                                     phase.ctypes.data_as(_ip))

    def accumulated_strain(self):
        """AccumulatedStrainII on the current markers (adds to strain, strain_pl)."""
        self.lib.ref_accumulated_strain()

    def reseed(self, direct, min_part_cell):
        """CountPartCell(RESEED = 1) on one thread; returns the new marker count."""
        self.n_markers = self.lib.ref_reseed(C.c_int(direct), C.c_int(min_part_cell))
        return self.n_markers

    def marker_field(self, name):
        ptr = self.lib.ref_marker_field(name.encode())
        return np.ctypeslib.as_array(ptr, shape=(self.n_markers,))

    def marker_phase(self):
        return np.ctypeslib.as_array(self.lib.ref_marker_phase(), shape=(self.n_markers,))

    def p2g(self, values, flag, avg, prop, centroid, stencil, init=None):
        kind = {1: "n", 0: "s", -1: "u", -2: "v"}[centroid]
        out = np.zeros(self.size(kind)) if init is None else np.array(init, np.float64)
        values = np.ascontiguousarray(values, np.float64)
        self.lib.ref_p2g(values.ctypes.data_as(_dp), out.ctypes.data_as(_dp), C.c_int(flag), C.c_int(avg),
                         C.c_int(prop), C.c_int(centroid), C.c_int(stencil))
        return out

    def g2p(self, node_field, which):
        node_field = np.ascontiguousarray(node_field, np.float64)
        out = np.zeros(self.n_markers)
        self.lib.ref_g2p(node_field.ctypes.data_as(_dp), out.ctypes.data_as(_dp), C.c_int(which))
        return out

    def count_old(self):
        self.lib.ref_count_old()

    def rk4(self):
        self.lib.ref_rk4()

    def phase_viz(self, res_fact):
        """Interp_Phase2VizGrid on the visualisation grid of res_fact x the
        grid resolution: (compo as int8, xviz, zviz)."""
        nxv, nzv = res_fact * (self.Nx - 1) + 1, res_fact * (self.Nz - 1) + 1
        compo = np.zeros((nxv - 1) * (nzv - 1), np.int8)
        xv, zv = np.zeros(nxv), np.zeros(nzv)
        self.lib.ref_phase_viz(C.c_int(res_fact), compo.ctypes.data_as(C.c_char_p), xv.ctypes.data_as(_dp),
                               zv.ctypes.data_as(_dp))
        return compo, xv, zv

    def set_scale(self, name, v):
        if self.lib.ref_set_scale(name.encode(), C.c_double(v)) != 0:
            raise KeyError(name)

    def make_breakpoint(self):
        """MakeBreakpointParticles into BreakpointXXXXX.dat in the working directory."""
        if self.lib.ref_make_breakpoint() != 0:
            raise RuntimeError("make_breakpoint: no grid or markers")

    def load_breakpoint(self):
        """LoadBreakpointParticles from BreakpointXXXXX.dat in the working directory."""
        n = self.lib.ref_load_breakpoint()
        if n < 0:
            raise RuntimeError("load_breakpoint: no grid or markers")
        self.n_markers = n
        return n

    def model(self, name):
        return self.lib.ref_get_model(name.encode())

    # grid operators --------------------------------------------------------
    def strain_rates(self):
        self.lib.ref_strain_rates()

    def viscosity_grid(self):
        self.lib.ref_viscosity_grid()

    def rheo_operators(self, jacobian):
        self.lib.ref_rheo_operators(C.c_int(jacobian))

    def rhs(self):
        self.lib.ref_rhs()

    def update_particle_stress(self):
        self.lib.ref_update_particle_stress()

    def update_particle_pressure(self):
        self.lib.ref_update_particle_pressure()

    def shear_mod_grid(self):
        self.lib.ref_shear_mod_grid()

    def cohesion_grid(self):
        self.lib.ref_cohesion_grid()

    def setup_equations(self):
        self.lib.ref_setup_equations()

    def eqn(self, which):
        self.setup_equations()
        kind = {0: "u", 1: "v", 2: "n"}[which]
        return np.ctypeslib.as_array(self.lib.ref_eqn(C.c_int(which)), shape=(self.size(kind),)).copy()

    def neq(self, which):
        self.setup_equations()
        return self.lib.ref_neq(C.c_int(which))

    def residual(self):
        norms = np.zeros(3)
        self.lib.ref_residual(norms.ctypes.data_as(_dp))
        Fm = np.ctypeslib.as_array(self.lib.ref_residual_vec(0), shape=(self.neq(0),)).copy()
        Fc = np.ctypeslib.as_array(self.lib.ref_residual_vec(1), shape=(self.neq(1),)).copy()
        return norms, Fm, Fc

    def assemble(self, jacobian):
        """Return the four blocks as scipy CSR matrices plus their BC vectors."""
        import scipy.sparse as sp
        self.lib.ref_assemble(C.c_int(jacobian))
        nm, nc = self.neq(0), self.neq(1)
        out = []
        for b, (nr, ncol) in enumerate([(nm, nm), (nm, nc), (nc, nm), (nc, nc)]):
            Ic, J, A, bbc = _ip(), _ip(), _dp(), _dp()
            n = self.lib.ref_block(C.c_int(jacobian), C.c_int(b), C.byref(Ic), C.byref(J), C.byref(A), C.byref(bbc))
            ic = np.ctypeslib.as_array(Ic, shape=(n + 1,)).copy()
            nnz = int(ic[-1])
            j = np.ctypeslib.as_array(J, shape=(max(nnz, 1),))[:nnz].copy() if nnz else np.zeros(0, np.int32)
            a = np.ctypeslib.as_array(A, shape=(max(nnz, 1),))[:nnz].copy() if nnz else np.zeros(0)
            out.append(sp.csr_matrix((a, j, ic), shape=(nr, ncol)))
        return out

    # ---- energy equation (EnergyDirectSolve with the harness's dense stand-in solve)
    def bct_tags(self, name):
        """numpy int8 view of BCt.type (centroids) or BCt.typW/E (Nz-1), typS/N (Nx-1)."""
        n = {"type": self.size("n"), "typW": self.Nz - 1, "typE": self.Nz - 1, "typS": self.Nx - 1,
             "typN": self.Nx - 1}[name]
        return np.ctypeslib.as_array(C.cast(self.lib.ref_bct_tags(name.encode()), C.POINTER(C.c_int8)), shape=(n,))

    def bct_vals(self, name):
        n = {"valW": self.Nz - 1, "valE": self.Nz - 1, "valS": self.Nx - 1, "valN": self.Nx - 1}[name]
        return np.ctypeslib.as_array(self.lib.ref_bct_vals(name.encode()), shape=(n,))

    def energy_solve(self, dt, shear_heating, adiab_heating):
        self.lib.ref_energy_solve(C.c_double(dt), C.c_int(shear_heating), C.c_int(adiab_heating))

    def energy_system(self):
        """(CSR matrix, right-hand side b + bbc, solution) of the last energy solve."""
        import scipy.sparse as sp
        ia, ja, a, b, x = _ip(), _ip(), _dp(), _dp(), _dp()
        n = self.lib.ref_energy_system(C.byref(ia), C.byref(ja), C.byref(a), C.byref(b), C.byref(x))
        ic = np.ctypeslib.as_array(ia, shape=(n + 1,)).copy()
        nnz = int(ic[-1])
        j = np.ctypeslib.as_array(ja, shape=(nnz,)).copy()
        v = np.ctypeslib.as_array(a, shape=(nnz,)).copy()
        return (sp.csr_matrix((v, j, ic), shape=(n, n)), np.ctypeslib.as_array(b, shape=(n,)).copy(),
                np.ctypeslib.as_array(x, shape=(n,)).copy())
