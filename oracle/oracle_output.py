"""CPU restatement of the output preparation for the tests: the closest-marker
phase map of Interp_Phase2VizGrid (SOURCE/ParticleRoutines.c:3004-3095) on the
visualisation grid WriteOutputHDF5 builds (SOURCE/HDF5Output.c:266-297), and
the float cast + ScaleBack of a field (HDF5Output.c:44-73).

Test infrastructure only: the parity checker of mdz_Interp_Phase2VizGrid and
mdz_output_field, pinned to the phase maps the reference itself produced
(tests/golden/phasemap_ref.npz)."""
import math

import numpy as np


def viz_lines(x0, h, res_fact, ncells):
    """res_fact * ncells + 1 lines by accumulation from x0 (HDF5Output.c:270-276)."""
    out = np.empty(res_fact * ncells + 1)
    out[0] = x0
    step = h / res_fact
    for k in range(1, len(out)):
        out[k] = out[k - 1] + step
    return out


def phase_viz(xg0, zg0, dx, dz, xc0, zc0, ncx, ncz, bcp, x, z, phase, res_fact):
    """compo (int8), xviz, zviz: the marker of largest tent weight per
    visualisation cell, the first in index order among equal weights; markers
    in air centroids (BCp 30 / 31) and inactive ones left out."""
    X = viz_lines(xg0, dx, res_fact, ncx)
    Z = viz_lines(zg0, dz, res_fact, ncz)
    nx, nz = len(X) - 1, len(Z) - 1
    dxv, dzv = X[1] - X[0], Z[1] - Z[0]
    compo = np.full(nx * nz, -1, np.int8)
    wm = np.zeros(nx * nz)
    for k in range(len(x)):
        if phase[k] == -1:
            continue
        j = math.ceil((x[k] - (X[0] + 0.5 * dxv)) / dxv + 0.5) - 1
        j = min(max(j, 0), nx - 1)
        i = math.ceil((z[k] - (Z[0] + 0.5 * dzv)) / dzv + 0.5) - 1
        i = min(max(i, 0), nz - 1)
        dxm = abs(0.5 * (X[j] + X[j + 1]) - x[k])
        dzm = abs(0.5 * (Z[i + 1] + Z[i]) - z[k])
        ic = min(max(math.ceil((x[k] - xc0) / dx + 0.5) - 1, 0), ncx - 1)
        jc = min(max(math.ceil((z[k] - zc0) / dz + 0.5) - 1, 0), ncz - 1)
        flag = bcp[ic + jc * ncx]
        w = (1.0 - (dxm / dxv)) * (1.0 - (dzm / dzv))
        if flag not in (30, 31) and w > wm[j + i * nx]:
            wm[j + i * nx] = w
            compo[j + i * nx] = phase[k]
    return compo, X, Z


def cast_scale(a, scale):
    """(float) a, then float * scale rounded to float (DoubleToFloat + ScaleBack)."""
    f = np.asarray(a, np.float64).astype(np.float32)
    return (f.astype(np.float64) * scale).astype(np.float32)
