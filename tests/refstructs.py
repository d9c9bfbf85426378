"""Instances of the reference's structures (grid, markers, params, mat_prop,
scale, Nparams, SparseMat) in plain byte buffers, laid out by the generated
table refshim/ref_layout.py, for calling the reference-signature drop-ins
(libmdoodz_refshim.so) from the tests as a reference build would."""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "mdoodz6.0_gb300", "refshim"))
from ref_layout import LAYOUT  # noqa: E402

_CLASSES = {}


def _cls(name):
    if name not in _CLASSES:
        size = LAYOUT[name][0]
        assert size % 8 == 0
        _CLASSES[name] = type("ref_" + name, (C.Structure,), {"_fields_": [("raw", C.c_double * (size // 8))]})
    return _CLASSES[name]


class Ref:
    """A zeroed instance of reference structure `name`; set(member, value)
    writes a member at its offset (arrays are referenced, and kept alive)."""

    def __init__(self, name, **members):
        self.name = name
        self.members = LAYOUT[name][1]
        self.obj = _cls(name)()
        self.keep = {}
        for k, v in members.items():
            self.set(k, v)

    @property
    def addr(self):
        return C.addressof(self.obj)

    @property
    def ptr(self):
        return C.c_void_p(self.addr)

    def set(self, member, value):
        off, ctype = self.members[member]
        a = self.addr + off
        if ctype == "int":
            C.c_int.from_address(a).value = int(value)
        elif ctype == "double":
            C.c_double.from_address(a).value = float(value)
        elif ctype in ("double[20]", "int[20]"):
            t = C.c_double if ctype.startswith("double") else C.c_int
            arr = (t * 20).from_address(a)
            for i, v in enumerate(value):
                arr[i] = int(v) if t is C.c_int else float(v)
        elif ctype in ("BC", "BCT"):           # (tags, values); BCT keeps the tags only
            tags, vals = value if isinstance(value, tuple) else (value, None)
            self._point(a, np.ascontiguousarray(tags, np.int8), member + ".type")
            if ctype == "BC" and vals is not None:
                self._point(a + 8, np.ascontiguousarray(vals, np.float64), member + ".val")
        elif ctype == "double **":              # one array per phase
            arrs = [np.ascontiguousarray(x, np.float64) for x in value]
            table = (C.c_void_p * len(arrs))(*[x.ctypes.data for x in arrs])
            self.keep[member + "[]"] = arrs
            self.keep[member] = table
            C.c_void_p.from_address(a).value = C.addressof(table)
        else:                                   # a pointer member: a numpy array (kept) or None
            self._point(a, value, member)

    def _point(self, addr, arr, key):
        if arr is None:
            C.c_void_p.from_address(addr).value = None
            return
        self.keep[key] = arr
        C.c_void_p.from_address(addr).value = arr.ctypes.data

    def get(self, member):
        off, ctype = self.members[member]
        a = self.addr + off
        if ctype == "int":
            return C.c_int.from_address(a).value
        if ctype == "double":
            return C.c_double.from_address(a).value
        return self.keep.get(member)


def grid_of(g, nph, fields=None):
    """A reference grid for mdz.Grid g: sizes, coordinate lines, BC tags and
    values, the phase-fraction arrays, and every field of `fields` (a dict of
    numpy arrays by the reference's member names; missing ones are zeros)."""
    import mdz
    nc, nv = g.size(1), g.size(0)
    r = Ref("grid", Nx=g.Nx, Nz=g.Nz, dx=g.dx, dz=g.dz, xg_coord=g.xg, zg_coord=g.zg, xc_coord=g.xc,
            zc_coord=g.zc, xvz_coord=g.xvz, zvx_coord=g.zvx, BCu=(g.BCu, g.BCu_val), BCv=(g.BCv, g.BCv_val),
            BCp=(g.BCp, np.zeros(nc)), BCg=g.BCg, BCt=g.BCp)
    r.set("phase_perc_n", [np.zeros(nc) for _ in range(nph)])
    r.set("phase_perc_s", [np.zeros(nv) for _ in range(nph)])
    r.set("nb_part_cell", np.zeros(nc, np.int32))
    r.set("nb_part_vert", np.zeros(nv, np.int32))
    fields = dict(fields or {})
    for name, (off, ctype) in LAYOUT["grid"][1].items():
        if ctype != "double *" or name in r.keep:
            continue
        ours = {"u_in": "u", "v_in": "v", "p_in": "p"}.get(name, name)
        size = mdz.field_size(g, ours, nph) if ours in mdz.FIELD_NAMES else {
            "p_lith": nc, "p_lith0": nc, "dp": nc, "phi_n": nc, "eII_exp": nc, "eII_gbs": nc}.get(name, nc)
        val = fields.get(name, fields.get(ours))
        r.set(name, np.array(val, np.float64) if val is not None else np.zeros(size))
    return r


def phase_perc(r, centroid):
    return np.array(r.keep[("phase_perc_n" if centroid == 1 else "phase_perc_s") + "[]"])
