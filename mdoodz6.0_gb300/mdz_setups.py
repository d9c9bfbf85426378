"""Synthetic model setups: the harness's own SetParticles / SetBCs for the
benchmark configurations (the reference keeps these in per-model plugins,
SOURCE/set_*.c).  Markers are seeded on a regular sub-grid of each cell with a
uniform jitter from a fixed seed; BCs are the reference's free-slip pure-shear
tags (shear_style = 0).
"""
import numpy as np


def seed_markers(grid, nmx, nmz, jitter=0.5, seed=12345):
    """nmx x nmz markers per cell, each displaced uniformly by up to
    +/- jitter x (marker spacing) in x and z, clipped into the box.
    Returned in cell-major order (all markers of cell 0, then cell 1, ...)."""
    rng = np.random.default_rng(seed)
    ncx, ncz = grid.ncx, grid.ncz
    hx, hz = grid.dx / nmx, grid.dz / nmz
    # sub-grid of the whole box, then reorder cell-major
    ix = np.arange(ncx * nmx)
    iz = np.arange(ncz * nmz)
    X, Z = np.meshgrid(grid.xmin + (ix + 0.5) * hx, grid.zmin + (iz + 0.5) * hz)
    cx = (ix // nmx)[None, :].repeat(len(iz), 0)
    cz = (iz // nmz)[:, None].repeat(len(ix), 1)
    order = np.lexsort((X.ravel(), Z.ravel(), cx.ravel(), cz.ravel()))
    x = X.ravel()[order]
    z = Z.ravel()[order]
    n = x.size
    x = x + rng.uniform(-jitter, jitter, n) * hx
    z = z + rng.uniform(-jitter, jitter, n) * hz
    x = np.clip(x, grid.xmin, grid.xmax)
    z = np.clip(z, grid.zmin, grid.zmax)
    return x, z


def inclusion_phase(x, z, xc, zc, r):
    return (np.hypot(x - xc, z - zc) < r).astype(np.int32)
