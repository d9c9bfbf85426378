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
