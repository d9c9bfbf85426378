"""The allocation-free residual-norm entry point against the context entry
point (EvaluateStokesResidualDecoupled's norms) on the reference fixture's
state: two calls in a row, each equal to it within 1e-12 and to each other
bit for bit.  Named to be collected last: it must also pass after every
other test has used the device."""
import ctypes as C

import numpy as np
import pytest

import mdz
from stokes_case import reference_state

pytestmark = pytest.mark.gpu


def test_residual_norms_without_allocation(golden):
    torch = pytest.importorskip("torch")
    ref = golden("rheology_ref.npz")
    g, f = reference_state(ref, 0)
    ctx = mdz.Context(g, 3, 1)
    want = ctx.EvaluateStokesResidualDecoupled(f)
    ctx.close()
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(np.ascontiguousarray(f[k])).to(dev) for k in ("ru", "rv", "rp")}
    tags = {k: torch.from_numpy(np.ascontiguousarray(a)).to(dev) for k, a in (("u", g.BCu), ("v", g.BCv), ("p", g.BCp))}
    out = torch.zeros(3, dtype=torch.float64, device=dev)
    L = mdz.load_library()
    P = C.c_void_p
    got = []
    for _ in range(2):
        out.zero_()
        st = L.mdz_dev_residual_norms_noalloc(C.c_int(g.Nx), C.c_int(g.Nz), P(t["ru"].data_ptr()),
                                              P(t["rv"].data_ptr()), P(t["rp"].data_ptr()),
                                              P(tags["u"].data_ptr()), P(tags["v"].data_ptr()),
                                              P(tags["p"].data_ptr()), P(out.data_ptr()), None)
        assert st == 0
        torch.cuda.synchronize()
        got.append(out.cpu().numpy().copy())
    for r in got:
        assert np.all(np.abs(r - want) <= 1e-12 * np.abs(want) + 1e-300), (r, want)
    assert np.array_equal(got[0], got[1])
    # a grid whose index box has more rows than the scratch holds is refused
    st = L.mdz_dev_residual_norms_noalloc(C.c_int(g.Nx), C.c_int(8192), P(t["ru"].data_ptr()),
                                          P(t["rv"].data_ptr()), P(t["rp"].data_ptr()), P(tags["u"].data_ptr()),
                                          P(tags["v"].data_ptr()), P(tags["p"].data_ptr()), P(out.data_ptr()), None)
    assert st == 3


def test_no_allocation_stream_large_grid_and_empty():
    """On a side stream, a grid of more than 256 index rows (the second pass
    strides over rows) against the context norms; then every tag != -1, where
    all three norms are zero."""
    torch = pytest.importorskip("torch")
    g = mdz.Grid(65, 301, 0.0, 1.0, 0.0, 4.0).set_bc_pureshear(1.0)
    rng = np.random.default_rng(5)
    f = mdz.GridFields(g, 1)
    for k in ("ru", "rv", "rp"):
        f[k] = rng.normal(size=len(f[k]))
    f["ru"] = f["ru"] * (g.BCu == -1)
    f["rv"] = f["rv"] * (g.BCv == -1)
    f["rp"] = f["rp"] * (g.BCp == -1)
    want = np.array([np.sqrt(np.sum(f[k] ** 2) / np.sum(t == -1))
                     for k, t in (("ru", g.BCu), ("rv", g.BCv), ("rp", g.BCp))])
    dev = torch.device("cuda:0")
    s = torch.cuda.Stream()
    L = mdz.load_library()
    P = C.c_void_p

    def run(tu, tv, tp):
        t = {k: torch.from_numpy(np.ascontiguousarray(f[k])).to(dev) for k in ("ru", "rv", "rp")}
        tg = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (tu, tv, tp)]
        out = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            st = L.mdz_dev_residual_norms_noalloc(C.c_int(g.Nx), C.c_int(g.Nz), P(t["ru"].data_ptr()),
                                                  P(t["rv"].data_ptr()), P(t["rp"].data_ptr()), P(tg[0].data_ptr()),
                                                  P(tg[1].data_ptr()), P(tg[2].data_ptr()), P(out.data_ptr()),
                                                  P(s.cuda_stream))
        s.synchronize()
        assert st == 0
        return out.cpu().numpy()

    got = run(g.BCu, g.BCv, g.BCp)
    assert np.all(np.abs(got - want) <= 1e-12 * want), (got, want)
    none = run(np.full_like(g.BCu, 0), np.full_like(g.BCv, 0), np.full_like(g.BCp, 30))
    assert np.array_equal(none, np.zeros(3))
