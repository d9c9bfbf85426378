"""Shared set-up for the Stokes tests: the reference state stored in the
rheology golden fixture (operators, RHS, p_corr) and its assembled blocks."""
import numpy as np
import scipy.sparse as sp

import mdz


def reference_state(ref, jacobian):
    """GridFields holding the reference's inputs to the Stokes rows: velocities,
    p_corr, RHS and the Picard (jacobian=0) or Newton (jacobian=1) D tensor."""
    from golden.make_golden import NX, NZ, XMIN, XMAX, ZMIN, ZMAX
    g = mdz.Grid(NX, NZ, XMIN, XMAX, ZMIN, ZMAX).set_bc_pureshear(1.0)
    if "bc_BCu" in ref:   # a fixture with its own boundary tags and values (Neumann walls)
        g.BCu[:], g.BCu_val[:] = ref["bc_BCu"], ref["bc_BCu_val"]
        g.BCv[:], g.BCv_val[:] = ref["bc_BCv"], ref["bc_BCv_val"]
    f = mdz.GridFields(g, 3)
    f["u"], f["v"], f["p"] = ref["in_u"], ref["in_v"], ref["in_p"]
    f["eta_n"], f["eta_s"] = ref["vg_eta_n"], ref["vg_eta_s"]   # read by the Neumann rows
    f["p_corr"] = ref["vg_p_corr"]
    for k in ref:
        if k.startswith("op%d_" % jacobian):
            f[k[4:]] = ref[k]
    f["roger_x"], f["roger_z"], f["rhs_p"] = ref["rhs_roger_x"], ref["rhs_roger_z"], ref["rhs_rhs_p"]
    return g, f


def assembled(ref, jacobian):
    blocks = []
    for b in "ABCD":
        key = "st_J%d_%s_" % (jacobian, b)
        blocks.append(sp.csr_matrix((ref[key + "data"], ref[key + "indices"], ref[key + "indptr"]),
                                    shape=tuple(ref[key + "shape"])))
    A, B, Cm, D = blocks
    return sp.bmat([[A, B], [Cm, D]]).tocsr()


def eqn_maps(ref):
    """index arrays (grid node -> equation number, -1 if none) for u, v, p."""
    return ref["st_eqn0"], ref["st_eqn1"], ref["st_eqn2"]


def to_grid(x, maps, g):
    eu, ev, ep = maps
    xu, xv, xp = np.zeros(g.size(-1)), np.zeros(g.size(-2)), np.zeros(g.size(1))
    m = eu >= 0
    xu[m] = x[eu[m]]
    m = ev >= 0
    xv[m] = x[ev[m]]
    m = ep >= 0
    xp[m] = x[ep[m]]
    return xu, xv, xp


def to_eqn(yu, yv, yp, maps, n):
    eu, ev, ep = maps
    y = np.zeros(n)
    y[eu[eu >= 0]] = yu[eu >= 0]
    y[ev[ev >= 0]] = yv[ev >= 0]
    y[ep[ep >= 0]] = yp[ep >= 0]
    return y
