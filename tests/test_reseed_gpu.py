"""GPU parity of the marker reseeding (CountPartCell with RESEED = 1) through
the C ABI: against the reference's own golden vectors, and against the CPU
oracle on random cases up to the 1025x513 lithosphere marker count.  Positions,
phases, slot assignment and copied attributes are bit for bit; attributes
interpolated from the grid (DirectNeighbour = 0) agree to 1e-14 (the GPU
fuses multiply-adds in the bilinear sums)."""
import numpy as np
import pytest

import mdz
import mdz_setups
import oracle

pytestmark = pytest.mark.gpu

ATTR_IDS = (("sxxd", mdz.M_SXXD), ("szzd", mdz.M_SZZD), ("sxz", mdz.M_SXZ), ("strain_pl", mdz.M_STRAIN_PL),
            ("strain", mdz.M_STRAIN), ("T", mdz.M_T), ("cmul", mdz.M_CMUL), ("P", mdz.M_P))
INTERP = ("T", "sxxd", "szzd", "sxz", "P")
INTERP_TOL = 1e-14


def _load(g, m, cap, nph):
    ctx = mdz.Context(g, nph, cap)
    ctx.set_markers(m["x"], m["z"], m["phase"])
    ctx.set_marker_velocity(m["vx"], m["vz"])
    for k, a in ATTR_IDS:
        ctx.set_marker_attr(a, m[k])
    return ctx


def _read(ctx):
    x, z, ph, vx, vz = ctx.get_markers()
    out = dict(x=x, z=z, phase=ph, vx=vx, vz=vz)
    for k, a in ATTR_IDS:
        out[k] = ctx.get_marker_attr(a)
    return out


def _compare(gpu, ref, direct, keys=None):
    assert len(gpu["x"]) == len(ref["x"])
    for k in keys or ref:
        if not direct and k in INTERP:
            d = np.abs(gpu[k] - ref[k])
            assert np.all(d <= INTERP_TOL * np.maximum(1.0, np.abs(ref[k]))), (k, d.max())
        else:
            assert np.array_equal(gpu[k], ref[k]), (k, np.flatnonzero(gpu[k] != ref[k])[:5])


def _case(ref):
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    m = {k: np.array(ref["in_" + k]) for k in ("x", "z", "phase", "vx", "vz", "sxxd", "szzd", "sxz", "strain",
                                                "strain_pl", "T", "P")}
    m["cmul"] = np.arange(len(m["x"]), dtype=np.float64)
    return g, m


@pytest.mark.parametrize("direct", [1, 0])
@pytest.mark.parametrize("mpc", [16, 9])
def test_reseed_matches_reference_golden(golden, direct, mpc):
    ref = golden("reseed_ref.npz")
    g, m = _case(ref)
    n = len(m["x"])
    cap = n + 4 * g.ncx * g.ncz
    ctx = _load(g, m, cap, 3)
    added = ctx.CountPartCell(1, mpc, direct, ref["T_n"], ref["sxxd_n"], ref["szzd_n"], ref["sxz_s"], ref["p_n"])
    tag = "d%d_m%d_" % (direct, mpc)
    assert ctx.n_markers == int(ref[tag + "n"]) and added > 0
    out = _read(ctx)
    slots = ref[tag + "slots"]
    _compare({k: out[k][slots] for k in out}, {k: ref[tag + k] for k in ("x", "z", "phase", "vx", "vz", "sxxd",
                                                                         "szzd", "sxz", "strain", "strain_pl", "T",
                                                                         "P")},
             direct)
    # the whole marker store against the oracle, the cohesion multiplier included
    o, o_added = oracle.reseed(g, m, cap, mpc, direct, ref["T_n"], ref["sxxd_n"], ref["szzd_n"], ref["sxz_s"],
                               ref["p_n"])
    assert o_added == added
    _compare(out, o, direct)
    ctx.close()


def _random_case(Nx, Nz, nm, thin, seed, nph=4):
    rng = np.random.default_rng(seed)
    g = mdz.Grid(Nx, Nz, -1.0, 1.0, -0.6, 0.0).set_bc_pureshear(1.0)
    x, z = mdz_setups.seed_markers(g, nm, nm, 0.5, seed)
    keep = rng.random(len(x)) > thin
    x, z = x[keep], z[keep]
    m = dict(x=x, z=z, phase=rng.integers(0, nph, len(x)).astype(np.int32))
    m["phase"][rng.random(len(x)) < 0.01] = -1          # markers that left the box: slots to reuse
    for k in ("vx", "vz", "sxxd", "szzd", "sxz", "strain", "strain_pl", "T", "cmul", "P"):
        m[k] = rng.normal(size=len(x))
    nc, nv = g.ncx * g.ncz, Nx * Nz
    flds = [rng.normal(size=nc), rng.normal(size=nc), rng.normal(size=nc), rng.normal(size=nv), rng.normal(size=nc)]
    return g, m, flds


@pytest.mark.parametrize("Nx,Nz,nm,thin,direct", [(129, 65, 4, 0.3, 0), (129, 65, 4, 0.3, 1),
                                                 (1025, 513, 4, 0.05, 0)])
def test_reseed_random_vs_oracle(Nx, Nz, nm, thin, direct):
    g, m, flds = _random_case(Nx, Nz, nm, thin, seed=Nx + Nz)
    n = len(m["x"])
    cap = n + 8 * g.ncx * g.ncz          # room for two passes (one marker per quarter cell each)
    ctx = _load(g, m, cap, 4)
    added = ctx.CountPartCell(1, 16, direct, *flds)
    o, o_added = oracle.reseed(g, m, cap, 16, direct, *flds)
    assert added == o_added and added > 0
    _compare(_read(ctx), o, direct)
    # a second pass finds every inner quarter cell at the threshold or above
    # only where the first one could not add (it adds one marker per cell)
    again = ctx.CountPartCell(1, 16, 1)
    o2, again_o = oracle.reseed(g, o, cap, 16, 1)
    assert again == again_o
    _compare(_read(ctx), o2, 1, keys=("x", "z", "phase"))
    ctx.close()


def test_reseed_capacity_and_empty_neighbourhood():
    g, m, flds = _random_case(65, 33, 4, 0.3, seed=3)
    n = len(m["x"])
    ctx = _load(g, m, n + 1, 4)
    before = _read(ctx)
    with pytest.raises(mdz.MdzError) as e:
        ctx.CountPartCell(1, 16, 1)
    assert e.value.status == 3
    _compare(_read(ctx), before, 1)
    ctx.close()
    keep = m["x"] > 0.0          # an empty west half: its quarter cells have no neighbours
    mm = {k: v[keep] for k, v in m.items()}
    ctx = _load(g, mm, len(mm["x"]) + 4 * g.ncx * g.ncz, 4)
    before = _read(ctx)
    with pytest.raises(mdz.MdzError) as e:
        ctx.CountPartCell(1, 16, 1)
    assert e.value.status == 7
    _compare(_read(ctx), before, 1)
    ctx.close()
