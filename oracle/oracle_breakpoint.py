"""CPU restatement of reading the reference's breakpoint file (test
infrastructure only).

The layout is the one MakeBreakpointParticles writes
(SOURCE/InputOutput.c:515-903) and LoadBreakpointParticles reads back
(SOURCE/InputOutput.c:160-514): a 4-byte size header, dt, dt0, time and the
box, the topography chains when free_surf, Nb_part and the marker arrays in
their fixed order (sections switched by iselastic, fstrain, aniso and
rec_T_P_x_z), the grid arrays of the previous step, u_in, v_in, p_in, and the
trailing topography, boundary, phase-proportion and count arrays.  The values
the library keeps are divided by the run's scales as the reference's loader
divides them.  Pinned to a file written by the reference's own
MakeBreakpointParticles and to what its own LoadBreakpointParticles read back
(tests/golden/breakpoint_ref.npz).
"""
import numpy as np


def trailing_bytes(Nx, Nz, n_phases, free_surf=0):
    """Bytes after p_in (InputOutput.c:798-851): p_lith, p_lith0, Ut, W, L0,
    the two topographies, BC tags (char) and values, phase proportions, counts."""
    nc, ns, nu, nv = (Nx - 1) * (Nz - 1), Nx * Nz, Nx * (Nz + 1), (Nx + 1) * Nz
    topo = 2 * 8 * (4 * Nx + 1 + 4 * (Nx - 1)) if free_surf else 0
    return (8 * (2 * nc + 3) + topo + (2 * nc + nu + nv + ns) + 8 * (nc + nu + nv + ns)
            + 8 * n_phases * (nc + ns) + 4 * (nc + ns))


def read(data, Nx, Nz, n_phases, scales, iselastic=1, free_surf=0, fstrain=0, aniso=0, rec_T_P_x_z=0):
    """Parse a breakpoint image; returns the kept arrays in scaled units and
    the number of bytes left after p_in (to compare with trailing_bytes)."""
    buf = bytes(data)
    pos = 0

    def take(dtype, count):
        nonlocal pos
        dt = np.dtype(dtype)
        end = pos + dt.itemsize * count
        if end > len(buf):
            raise ValueError("truncated at byte %d" % pos)
        a = np.frombuffer(buf[pos:end], dt).copy()
        pos = end
        return a

    sizes = take(np.uint8, 4)
    if list(sizes) != [4, 8, 8, 1]:
        raise ValueError("size header %s" % list(sizes))
    dt, _, time, xmin, xmax, zmin, zmax = take(np.float64, 7)
    if free_surf:
        for _ in range(2):
            nb = int(take(np.int32, 1)[0])
            take(np.float64, 4 * nb)
    n = int(take(np.int32, 1)[0])
    nc, ns, nu, nv = (Nx - 1) * (Nz - 1), Nx * Nz, Nx * (Nz + 1), (Nx + 1) * Nz
    out = {}
    out["x"], out["z"], out["P"], out["Vx"], out["Vz"] = (take(np.float64, n) for _ in range(5))
    take(np.float64, 2 * n)                                   # phi, X
    out["phase"] = take(np.int32, n)
    if iselastic:
        out["sxxd"], out["szzd"], out["sxz"] = (take(np.float64, n) for _ in range(3))
        take(np.float64, 3 * n + 2 * nc + 2 * ns)             # dsxxd, dszzd, dsxz, eta_n, VE_n, eta_s, VE_s
    out["strain"] = take(np.float64, n)
    take(np.float64, n)                                       # strain_el
    out["strain_pl"] = take(np.float64, n)
    take(np.float64, 5 * n)                                   # strain_pwl, _exp, _lin, _gbs, d
    take(np.float64, n * (4 * bool(fstrain) + 4 * bool(aniso) + 6 * bool(rec_T_P_x_z)))
    take(np.float64, n)                                       # divth
    out["T"] = take(np.float64, n)
    take(np.float64, n)                                       # rho
    take(np.float64, 9 * nc + (2 * nc if aniso else 0) + 2 * ns + (2 * ns if aniso else 0) + nc + ns)
    out["u"], out["v"], out["p"] = take(np.float64, nu), take(np.float64, nv), take(np.float64, nc)
    L, V, S, T, t = (scales[k] for k in ("L", "V", "S", "T", "t"))
    for k in ("x", "z"):
        out[k] = out[k] / L
    for k in ("Vx", "Vz", "u", "v"):
        out[k] = out[k] / V
    for k in ("P", "p") + (("sxxd", "szzd", "sxz") if iselastic else ()):
        out[k] = out[k] / S
    out["T"] = out["T"] / T
    out.update(n=n, dt=dt / t, time=time / t, box=np.array([xmin, xmax, zmin, zmax]) / L,
               rest=len(buf) - pos)
    return out
