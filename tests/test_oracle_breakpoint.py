"""The restated reader of the reference's breakpoint file against a file
written by the reference's own MakeBreakpointParticles and what its own
LoadBreakpointParticles read back from it (CPU only)."""
import os

import numpy as np
import pytest

import oracle_breakpoint as ob

GOLD = os.path.join(os.path.dirname(__file__), "golden", "breakpoint_ref.npz")


def _fixture():
    d = np.load(GOLD)
    scales = dict(zip(("L", "V", "S", "T", "t"), d["scale"]))
    return d, scales


def test_reader_matches_reference_loader():
    d, scales = _fixture()
    Nx, Nz, nph = int(d["Nx"]), int(d["Nz"]), int(d["n_phases"])
    out = ob.read(d["image"], Nx, Nz, nph, scales, iselastic=1)
    assert out["n"] == int(d["n"])
    assert out["rest"] == ob.trailing_bytes(Nx, Nz, nph)
    assert np.array_equal(out["phase"], d["phase"])
    for k in ("x", "z", "P", "Vx", "Vz", "sxxd", "szzd", "sxz", "strain", "strain_pl", "T"):
        assert np.array_equal(out[k], d["m_" + k]), k
    for k in ("u", "v", "p"):
        assert np.array_equal(out[k], d[k]), k
    assert out["dt"] == float(d["dt"]) and out["time"] == float(d["time"])
    assert np.array_equal(out["box"], d["box"])


def test_wrong_flags_change_the_layout():
    d, scales = _fixture()
    Nx, Nz, nph = int(d["Nx"]), int(d["Nz"]), int(d["n_phases"])
    out = ob.read(d["image"], Nx, Nz, nph, scales, iselastic=0)
    assert out["rest"] != ob.trailing_bytes(Nx, Nz, nph)
    with pytest.raises(ValueError):
        ob.read(d["image"][: d["image"].size // 2], Nx, Nz, nph, scales, iselastic=1)
