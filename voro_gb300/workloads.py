"""Seeded synthetic particle sets for the benchmark and test workloads.

The reference publishes no dataset for its cell computation, so every workload
is generated here from a fixed seed with numpy's PCG64 (portable across x86-64
and aarch64).  Each generator returns a dict with the container description in
the reference's own constructor terms:

* ``kind``      0 container, 1 container_poly, 2 container_periodic,
                3 container_periodic_poly (src/container.hh:289,511;
                src/container_prd.hh:213,434)
* ``geom``      container: (ax,bx,ay,by,az,bz); periodic: (bx,bxy,by,bxz,byz,bz)
* ``grid``      (nx,ny,nz) block counts passed to the constructor
* ``periodic``  (xperiodic,yperiodic,zperiodic) flags (container kinds only)
* ``ids``       int32 particle IDs
* ``xyzr``      float64 (n,4): x, y, z and radius (radius ignored for mono kinds)
"""
from __future__ import annotations

import numpy as np

KIND_CONTAINER = 0
KIND_CONTAINER_POLY = 1
KIND_PERIODIC = 2
KIND_PERIODIC_POLY = 3


def _pack(kind, geom, grid, periodic, xyz, r=None, ids=None):
    n = xyz.shape[0]
    xyzr = np.zeros((n, 4), dtype=np.float64)
    xyzr[:, :3] = xyz
    if r is not None:
        xyzr[:, 3] = r
    else:
        xyzr[:, 3] = 0.5
    if ids is None:
        ids = np.arange(n, dtype=np.int32)
    return {
        "kind": int(kind),
        "geom": tuple(float(g) for g in geom),
        "grid": tuple(int(g) for g in grid),
        "periodic": tuple(bool(p) for p in periodic),
        "ids": np.ascontiguousarray(ids, dtype=np.int32),
        "xyzr": np.ascontiguousarray(xyzr),
    }


def unit_cube(n=100_000, seed=1001, grid=(6, 6, 6)):
    """Plain non-periodic container on [0,1]^3, positions i.i.d. uniform."""
    rng = np.random.default_rng(seed)
    xyz = rng.random((n, 3))
    return _pack(KIND_CONTAINER, (0, 1, 0, 1, 0, 1), grid, (False,) * 3, xyz)


def periodic_cube(n=4_000_000, L=100.0, seed=1002, grid=None, kind=KIND_PERIODIC):
    """Cubic periodic box of side L.  ``kind`` 2 uses container_periodic
    (unit-cell initialisation); kind 0 the flag-periodic container."""
    rng = np.random.default_rng(seed)
    xyz = rng.random((n, 3)) * L
    if grid is None:
        g = max(1, int(round((n / 5.0) ** (1.0 / 3.0))))
        grid = (g, g, g)
    if kind == KIND_PERIODIC:
        return _pack(kind, (L, 0, L, 0, 0, L), grid, (True,) * 3, xyz)
    return _pack(KIND_CONTAINER, (0, L, 0, L, 0, L), grid, (True,) * 3, xyz)


def sheared_periodic(n=4_000_000, L=100.0, shear=(0.3, 0.2, -0.25), seed=1006, grid=None):
    """container_periodic of lattice vectors (L,0,0), (sxy L, L, 0),
    (sxz L, syz L, L) (shear = (sxy, sxz, syz)), positions uniform over the
    box [0, L)^3 (a fundamental domain of the lattice)."""
    rng = np.random.default_rng(seed)
    xyz = rng.random((n, 3)) * L
    if grid is None:
        g = max(1, int(round((n / 5.0) ** (1.0 / 3.0))))
        grid = (g, g, g)
    sxy, sxz, syz = shear
    return _pack(KIND_PERIODIC, (L, sxy * L, L, sxz * L, syz * L, L), grid, (True,) * 3, xyz)


def radical_box(n=2_000_000, L=200.0, seed=1003, grid=None):
    """container_poly on [0,L]^3 with log-normal radii (median 0.5, sigma 0.3)
    clipped to [0.1, 1.5]."""
    rng = np.random.default_rng(seed)
    xyz = rng.random((n, 3)) * L
    r = np.clip(rng.lognormal(mean=np.log(0.5), sigma=0.3, size=n), 0.1, 1.5)
    if grid is None:
        g = max(1, int(round((n / 5.0) ** (1.0 / 3.0))))
        grid = (g, g, g)
    return _pack(KIND_CONTAINER_POLY, (0, L, 0, L, 0, L), grid, (False,) * 3, xyz, r)


def fcc_jitter(cells=64, sigma=1e-7, seed=1004, kind=KIND_PERIODIC):
    """FCC lattice with cubic lattice constant a = 1 (4 sites per unit cell),
    ``cells``^3 unit cells in a periodic cube of side ``cells``; every
    coordinate jittered by N(0, sigma^2)."""
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], dtype=np.float64)
    g = np.arange(cells, dtype=np.float64)
    cx, cy, cz = np.meshgrid(g, g, g, indexing="ij")
    corners = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], axis=1)
    xyz = (corners[:, None, :] + base[None, :, :]).reshape(-1, 3)
    xyz = xyz + rng.normal(0.0, sigma, size=xyz.shape)
    L = float(cells)
    xyz = np.mod(xyz, L)
    grid = (cells, cells, cells)
    if kind == KIND_PERIODIC:
        return _pack(kind, (L, 0, L, 0, 0, L), grid, (True,) * 3, xyz)
    return _pack(KIND_CONTAINER, (0, L, 0, L, 0, L), grid, (True,) * 3, xyz)


def batched(count=4096, nmin=64, nmax=1_000_000, seed=1005):
    """Many independent containers: N log-uniform in [nmin, nmax], unit density
    (box side N^(1/3)), blocks round((N/5)^(1/3)).  Even-indexed containers are
    container_periodic, odd ones walled containers; every fourth (index 1 mod
    4, walled) is radical with radii U[0.3, 1.0]."""
    rng = np.random.default_rng(seed)
    out = []
    for c in range(count):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        L = n ** (1.0 / 3.0)
        g = max(1, int(round((n / 5.0) ** (1.0 / 3.0))))
        xyz = rng.random((n, 3)) * L
        if c % 2 == 0:
            out.append(_pack(KIND_PERIODIC, (L, 0, L, 0, 0, L), (g, g, g), (True,) * 3, xyz))
        elif c % 4 == 1:
            r = rng.uniform(0.3, 1.0, size=n)
            out.append(_pack(KIND_CONTAINER_POLY, (0, L, 0, L, 0, L), (g, g, g), (False,) * 3, xyz, r))
        else:
            out.append(_pack(KIND_CONTAINER, (0, L, 0, L, 0, L), (g, g, g), (False,) * 3, xyz))
    return out


def small_random(n, kind=KIND_CONTAINER, L=1.0, periodic=(False, False, False), grid=None,
                 seed=0, rmin=0.3, rmax=1.0):
    """Small mixed-geometry case for parity tests."""
    rng = np.random.default_rng(seed)
    xyz = rng.random((n, 3)) * L
    if grid is None:
        g = max(1, int(round((n / 5.0) ** (1.0 / 3.0))))
        grid = (g, g, g)
    r = None
    if kind in (KIND_CONTAINER_POLY, KIND_PERIODIC_POLY):
        r = rng.uniform(rmin, rmax, size=n) * L / max(1.0, n ** (1.0 / 3.0))
    if kind in (KIND_PERIODIC, KIND_PERIODIC_POLY):
        return _pack(kind, (L, 0, L, 0, 0, L), grid, (True,) * 3, xyz, r)
    return _pack(kind, (0, L, 0, L, 0, L), grid, periodic, xyz, r)
