"""Generates the golden per-cell fixtures from the unmodified reference.

Run in a tree where the reference sources exist (oracle/Makefile builds
oracle/_ref/libvoro_ref.so from them):

    python tests/golden/make_golden.py

Each case stores its inputs (so the fixture does not depend on a random
number generator) and the reference's per-cell records in loop order:
ids, stored positions, volume, centroid, face count, vertex count,
max_radius_squared, ok flag and the neighbour lists (CSR, each list sorted).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import RefLib, build_ref  # noqa: E402
from voro_gb300 import workloads as W  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    out = {}
    # container on the unit cube, non-periodic (the 100k shape, scaled down)
    out["unit_cube_1000"] = W.unit_cube(n=1000, seed=2001, grid=(3, 3, 3))
    # container_periodic, density 4 (the 4M / L=100 shape)
    n = 2000
    L = 100.0 * (n / 4e6) ** (1 / 3)
    out["periodic_2000"] = W.periodic_cube(n=n, L=L, seed=2002, grid=(7, 7, 7))
    # flag-periodic container on the same kind of box
    out["flagperiodic_1500"] = W.periodic_cube(n=1500, L=100.0 * (1500 / 4e6) ** (1 / 3), seed=2003,
                                              grid=(6, 6, 6), kind=W.KIND_CONTAINER)
    # container_poly, log-normal radii (the 2M / 200^3 shape)
    n = 1200
    out["radical_1200"] = W.radical_box(n=n, L=200.0 * (n / 2e6) ** (1 / 3), seed=2004, grid=(6, 6, 6))
    # jittered FCC, container_periodic
    out["fcc_6"] = W.fcc_jitter(cells=6, sigma=1e-7, seed=2005)
    # mixed walls: periodic in x only
    out["xperiodic_600"] = W.small_random(600, kind=W.KIND_CONTAINER, L=2.0, periodic=(True, False, False),
                                          grid=(4, 5, 3), seed=2006)
    # a few particles in a mostly empty grid, including out-of-range ones that put() drops
    w = W.small_random(40, kind=W.KIND_CONTAINER, L=2.0, grid=(6, 6, 6), seed=2007)
    w["xyzr"][:, :3] -= 1.0  # container is [0,2]^3: about half of these fall outside and are dropped
    w["geom"] = (-0.5, 1.0, -0.5, 1.0, -0.5, 1.0)
    out["sparse_dropped_40"] = w
    # container_periodic_poly
    w = W.small_random(800, kind=W.KIND_PERIODIC_POLY, L=8.0, grid=(5, 5, 5), seed=2008, rmin=0.2, rmax=0.8)
    out["periodic_poly_800"] = w
    # exactly degenerate input: a simple-cubic lattice (every cell a cube with
    # twelve further neighbours touching it only along edges and at corners)
    g = np.arange(6, dtype=float) + 0.5
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    out["degenerate_cubic_216"] = W._pack(W.KIND_CONTAINER, (0, 6, 0, 6, 0, 6), (3, 3, 3), (False,) * 3, xyz)
    out.update(degenerate_cases())
    return out


# Exactly degenerate lattices whose cells have vertices of order 4: the FCC
# lattice (every cell a rhombic dodecahedron, six of its fourteen vertices of
# order 4), periodic and in a walled box.
def degenerate_cases():
    out = {}
    out["degenerate_fcc_256"] = W.fcc_jitter(cells=4, sigma=0.0, seed=2010)
    w = W.fcc_jitter(cells=4, sigma=0.0, seed=2011, kind=W.KIND_CONTAINER)
    w["periodic"] = (False, False, False)
    # shifted so that no wall of the box passes through a lattice vertex; the
    # walls still meet the lattice's degenerate edges
    w["xyzr"][:, :3] += 0.3
    w["geom"] = (0.0, 4.5, 0.0, 4.5, 0.0, 4.5)
    w["grid"] = (3, 3, 3)
    out["degenerate_fcc_walled_256"] = w
    return out


# Edge cases of placement and of tiny inputs (edge_*.npz): coordinates
# exactly on the box's faces and on block boundaries (put_remap's step_int
# and its range checks, src/container.cc:174-191: a point at the upper face
# of a non-periodic box is dropped), their neighbouring doubles, signed
# zero, points many periods away (the remaps of src/container.cc:178-186
# and src/container_prd.cc:189-216), and containers of one and two
# particles (a periodic box's lone particle is its own neighbour).
def edge_cases():
    out = {}
    rng = np.random.default_rng(2301)
    special = [0.0, -0.0, 0.25, 0.5, 0.75, 1.0, np.nextafter(1.0, 0.0), np.nextafter(0.25, 0.0),
               np.nextafter(0.25, 1.0), np.nextafter(0.75, 1.0), 1e-300, 0.5 + 2.0 ** -40]
    rows = []
    for v in special:
        for a in range(3):
            q = rng.uniform(0.05, 0.95, size=3)
            q[a] = v
            rows.append(q)
    xyz = np.concatenate([rng.random((260, 3)), np.array(rows)])
    out["edge_box_boundaries_296"] = W._pack(W.KIND_CONTAINER, (0, 1, 0, 1, 0, 1), (4, 4, 4), (False,) * 3, xyz)
    r = rng.uniform(0.02, 0.08, size=len(xyz))
    out["edge_poly_boundaries_296"] = W._pack(W.KIND_CONTAINER_POLY, (0, 1, 0, 1, 0, 1), (4, 4, 4), (False,) * 3,
                                              xyz, r=r)
    # periodic: exact faces, one period and many periods away
    L = 2.0
    wrap = [0.0, L, -L, 2 * L + 0.3, -1000 * L + 0.7, np.nextafter(L, 0.0), np.nextafter(L, 4.0), -0.0, 1e-300,
            1e6 * L + 0.123, 0.5 * L, -0.5 * L]
    rows = []
    for v in wrap:
        for a in range(3):
            q = rng.uniform(0.1, 1.9, size=3)
            q[a] = v
            rows.append(q)
    xyz = np.concatenate([rng.uniform(0, L, size=(264, 3)), np.array(rows)])
    out["edge_periodic_wraps_300"] = W._pack(W.KIND_PERIODIC, (L, 0, L, 0, 0, L), (4, 4, 4), (True,) * 3, xyz)
    out["edge_flagperiodic_wraps_300"] = W._pack(W.KIND_CONTAINER, (0, L, 0, L, 0, L), (4, 4, 4), (True,) * 3, xyz)
    # one and two particles
    out["edge_single_1"] = W._pack(W.KIND_CONTAINER, (0, 1, 0, 1, 0, 1), (1, 1, 1), (False,) * 3,
                                   np.array([[0.3, 0.6, 0.2]]))
    out["edge_pair_2"] = W._pack(W.KIND_CONTAINER, (0, 2, 0, 1, 0, 1), (2, 1, 1), (False,) * 3,
                                 np.array([[0.4, 0.5, 0.5], [1.7, 0.2, 0.9]]))
    out["edge_single_periodic_1"] = W._pack(W.KIND_PERIODIC, (3, 0, 3, 0, 0, 3), (2, 2, 2), (True,) * 3,
                                            np.array([[1.1, 2.2, 0.4]]))
    out["edge_pair_periodic_2"] = W._pack(W.KIND_PERIODIC, (3, 0, 3, 0, 0, 3), (2, 2, 2), (True,) * 3,
                                          np.array([[1.1, 2.2, 0.4], [2.5, 0.9, 1.6]]))
    # a box far from the origin (coordinates near 1e5, spacing about 0.13)
    x0 = 100000.0
    xyz = x0 + rng.random((500, 3))
    out["edge_far_box_500"] = W._pack(W.KIND_CONTAINER, (x0, x0 + 1, x0, x0 + 1, x0, x0 + 1), (4, 4, 4),
                                      (False,) * 3, xyz)
    # strongly anisotropic boxes, walled and periodic
    xyz = rng.random((600, 3)) * np.array([20.0, 1.0, 0.5])
    out["edge_aniso_600"] = W._pack(W.KIND_CONTAINER, (0, 20, 0, 1, 0, 0.5), (20, 2, 1), (False,) * 3, xyz)
    xyz = rng.random((500, 3)) * np.array([5.0, 1.0, 0.7])
    out["edge_periodic_aniso_500"] = W._pack(W.KIND_PERIODIC, (5.0, 0, 1.0, 0, 0, 0.7), (10, 2, 2), (True,) * 3, xyz)
    # radical: zero radii among a wide spread, and all radii equal (the
    # power diagram is then the plain Voronoi diagram)
    xyz = rng.random((400, 3)) * 2.0
    r = rng.uniform(0.0, 0.3, size=400)
    r[::7] = 0.0
    out["edge_radical_zero_r_400"] = W._pack(W.KIND_CONTAINER_POLY, (0, 2, 0, 2, 0, 2), (4, 4, 4), (False,) * 3,
                                             xyz, r=r)
    xyz = rng.random((400, 3)) * 3.0
    out["edge_periodic_poly_equal_r_400"] = W._pack(W.KIND_PERIODIC_POLY, (3, 0, 3, 0, 0, 3), (4, 4, 4),
                                                    (True,) * 3, xyz, r=np.full(400, 0.25))
    # radical cells cut away entirely (compute_cell false): a few large
    # particles among many small ones
    xyz = rng.random((300, 3)) * 2.0
    r = np.full(300, 0.02)
    r[:6] = 0.9
    out["edge_radical_deleted_300"] = W._pack(W.KIND_CONTAINER_POLY, (0, 2, 0, 2, 0, 2), (4, 4, 4), (False,) * 3,
                                              xyz, r=r)
    # nearly coincident pairs (1e-7 and 1e-9 apart) in a walled box: tiny cells
    xyz = rng.random((300, 3))
    xyz[1] = xyz[0] + np.array([1e-7, 0.0, 0.0])
    xyz[3] = xyz[2] + np.array([3e-9, -2e-9, 1e-9])
    out["edge_near_coincident_300"] = W._pack(W.KIND_CONTAINER, (0, 1, 0, 1, 0, 1), (4, 4, 4), (False,) * 3, xyz)
    # a simple-cubic lattice jittered by 1e-12: vertices of order 4 split by
    # far less than the reference's tolerance (about 1e-13 of the box here)
    g = np.arange(6, dtype=float) + 0.5
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) + rng.normal(0.0, 1e-12, size=(216, 3))
    out["edge_cubic_jitter_1e-12_216"] = W._pack(W.KIND_CONTAINER, (0, 6, 0, 6, 0, 6), (3, 3, 3), (False,) * 3, xyz)
    # a dense cluster in a mostly empty box: most blocks empty, a few holding
    # hundreds of particles (the search's long runs of candidates per block)
    xyz = np.concatenate([0.5 + 0.02 * rng.standard_normal((1500, 3)), rng.random((60, 3))])
    out["edge_cluster_1560"] = W._pack(W.KIND_CONTAINER, (0, 1, 0, 1, 0, 1), (5, 5, 5), (False,) * 3, xyz)
    # particles on a line and on a plane: every bisector parallel to the
    # others (slabs), or to one axis (prisms), the box closing the cells
    t = np.sort(rng.random(80))
    xyz = np.stack([t, np.full(80, 0.37), np.full(80, 0.61)], 1)
    out["edge_line_80"] = W._pack(W.KIND_CONTAINER, (0, 1, 0, 1, 0, 1), (4, 2, 2), (False,) * 3, xyz)
    uv = rng.random((150, 2))
    xyz = np.stack([uv[:, 0], uv[:, 1], np.full(150, 0.5)], 1)
    out["edge_plane_150"] = W._pack(W.KIND_CONTAINER, (0, 1, 0, 1, 0, 1), (4, 4, 2), (False,) * 3, xyz)
    # a sheared periodic box with positions up to fifty periods away (the
    # z-y-x remap along the lattice vectors, src/container_prd.cc:189-216)
    geom = (7.3, -1.9, 6.1, 2.7, 1.3, 5.9)
    xyz = rng.uniform(-50.0, 50.0, size=(800, 3)) * np.array([geom[0], geom[2], geom[5]])
    out["edge_tric_far_800"] = W._pack(W.KIND_PERIODIC, geom, (4, 3, 4), (True,) * 3, xyz)
    # a periodic box so small that a cell's neighbours are mostly images
    xyz = rng.random((20, 3)) * 0.5
    out["edge_periodic_small_box_20"] = W._pack(W.KIND_PERIODIC, (0.5, 0, 0.5, 0, 0, 0.5), (2, 2, 2), (True,) * 3, xyz)
    # voids: a slab of particles in a box periodic across it (the cells
    # reach through the empty part to the slab's images, some 20 engine
    # blocks away), and three tight clusters in a periodic box with a few
    # particles between them (cells spanning much of the box)
    xyz = rng.random((9000, 3)) * np.array([0.2, 1.0, 1.0])
    out["edge_slab_periodic_9000"] = W._pack(W.KIND_CONTAINER, (0, 1, 0, 1, 0, 1), (14, 14, 14),
                                             (True, False, False), xyz)
    cen = rng.random((3, 3))
    xyz = np.mod(cen[rng.integers(0, 3, 6000)] + rng.normal(0.0, 0.02, (6000, 3)), 1.0)
    xyz = np.concatenate([xyz, rng.random((8, 3))])
    out["edge_voids_periodic_6008"] = W._pack(W.KIND_PERIODIC, (1, 0, 1, 0, 0, 1), (12, 12, 12), (True,) * 3, xyz)
    return out


# Sheared periodic boxes (tric_*.npz: the same per-cell records, plus
# locate_tric_* and ghost_tric_*): container_periodic(_poly) with bxy, bxz,
# byz != 0.  Positions are drawn over a larger range than the box, so put()
# remaps them along the lattice vectors.  The dyadic boxes make every image
# displacement exact (the reference's lazily built image blocks sum the
# displacements in several orders, which other boxes round differently).
def tric_cases():
    out = {}

    def tric(kind, geom, grid, n, seed, rmin=None, rmax=None):
        rng = np.random.default_rng(seed)
        span = np.array([geom[0], geom[2], geom[5]])
        xyz = rng.uniform(-0.5, 1.5, size=(n, 3)) * span
        r = rng.uniform(rmin, rmax, size=n) if rmin is not None else None
        return W._pack(kind, geom, grid, (True,) * 3, xyz, r)

    out["tric_dyadic_1500"] = tric(W.KIND_PERIODIC, (8.0, 2.5, 7.0, 1.25, -1.5, 6.5), (4, 4, 4), 1500, 2201)
    out["tric_generic_1200"] = tric(W.KIND_PERIODIC, (7.3, -1.9, 6.1, 2.7, 1.3, 5.9), (4, 3, 4), 1200, 2202)
    out["tric_poly_1000"] = tric(W.KIND_PERIODIC_POLY, (8.0, -3.0, 7.5, 2.0, 2.5, 7.0), (4, 4, 4), 1000, 2203,
                                 0.2, 0.5)
    # strongly sheared (bxy > bx/2: the reduced lattice differs from the box)
    out["tric_skew_800"] = tric(W.KIND_PERIODIC, (6.0, 5.0, 5.0, -4.5, 3.5, 6.0), (3, 3, 3), 800, 2204)
    # a few particles: the unit cell's own faces (neighbour 0) survive, and
    # where the search meets a particle's own image, whose plane is one of
    # those faces, the reference relabels the face with the particle's ID
    out["degenerate_tric_small_5"] = tric(W.KIND_PERIODIC, (4.0, 1.0, 3.5, 0.5, -1.25, 3.0), (2, 2, 2), 5, 2205)
    return out


def make_cell_fixture(ref, name, w):
    rec = ref.compute(w)
    nb = [np.sort(rec.neighbors(k)) for k in range(len(rec))]
    nb_off = np.zeros(len(rec) + 1, np.int64)
    nb_off[1:] = np.cumsum([len(x) for x in nb])
    nb_flat = np.concatenate(nb).astype(np.int32) if nb else np.zeros(0, np.int32)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(
        path, kind=w["kind"], geom=np.asarray(w["geom"]), grid=np.asarray(w["grid"], np.int32),
        periodic=np.asarray(w["periodic"], np.int32), in_ids=w["ids"], in_xyzr=w["xyzr"],
        ids=rec.ids, pos=rec.pos, vol=rec.vol, cen=rec.cen, nf=rec.nf, nv=rec.nv, ok=rec.ok, mrs=rec.mrs,
        nb=nb_flat, nb_off=nb_off)
    print(f"{name}: {len(rec)} cells, sum vol {rec.vol.sum():.15g}, {os.path.getsize(path)} bytes")


# Wall fixtures (wall_*.npz): containers with walls (wall_sphere, wall_plane,
# wall_cylinder, wall_cone), particles filling the box (those outside a wall
# get no cell), the same per-cell records plus the walls.
def wall_cases():
    out = {}
    w = W.small_random(2000, kind=W.KIND_CONTAINER, L=2.0, grid=(6, 6, 6), seed=2101)
    w["walls"] = [(0, [1.0, 1.0, 1.0, 0.9], -7)]
    out["wall_sphere_2000"] = w
    w = W.small_random(1500, kind=W.KIND_CONTAINER_POLY, L=2.0, grid=(6, 6, 6), seed=2102, rmin=0.02, rmax=0.06)
    w["walls"] = [(2, [1.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.8], -7), (1, [0.0, 0.0, 1.0, 1.6], -8)]
    out["wall_cylinder_plane_poly_1500"] = w
    w = W.small_random(2000, kind=W.KIND_CONTAINER, L=2.0, grid=(6, 6, 6), seed=2103)
    w["xyzr"][:, :2] -= 1.0
    w["geom"] = (-1.0, 1.0, -1.0, 1.0, 0.0, 2.0)
    w["walls"] = [(3, [0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.5], -7), (1, [0.0, 0.0, 1.0, 1.8], -8)]
    out["wall_cone_2000"] = w
    w = W.small_random(1000, kind=W.KIND_CONTAINER, L=1.0, periodic=(True, False, False), grid=(8, 4, 4), seed=2104)
    w["xyzr"][:, 0] *= 2.0
    w["geom"] = (0.0, 2.0, 0.0, 1.0, 0.0, 1.0)
    w["walls"] = [(1, [0.0, -1.0, 0.0, -0.1], -7), (1, [0.0, 1.0, 0.0, 0.9], -8)]
    out["wall_planes_xperiodic_1000"] = w
    # a sphere wall on a box far from the origin
    x0 = 50000.0
    rng = np.random.default_rng(2104)
    w = W._pack(W.KIND_CONTAINER, (x0, x0 + 2, x0, x0 + 2, x0, x0 + 2), (5, 5, 5), (False,) * 3,
                x0 + rng.random((800, 3)) * 2.0)
    w["walls"] = [(0, [x0 + 1.0, x0 + 1.0, x0 + 1.0, 0.95], -7)]
    out["wall_far_sphere_800"] = w
    # a plane wall with particles lying exactly on it
    rng = np.random.default_rng(2105)
    xyz = rng.random((600, 3)) * 2.0
    xyz[:25, 0] = 1.25
    w = W._pack(W.KIND_CONTAINER, (0, 2, 0, 2, 0, 2), (4, 4, 4), (False,) * 3, xyz)
    w["walls"] = [(1, [1.0, 0.0, 0.0, 1.25], -7)]
    out["wall_plane_through_600"] = w
    return out


def make_wall_fixtures(ref):
    for name, w in wall_cases().items():
        rec = ref.compute(w)
        nb = [np.sort(rec.neighbors(k)) for k in range(len(rec))]
        nb_off = np.zeros(len(rec) + 1, np.int64)
        nb_off[1:] = np.cumsum([len(x) for x in nb])
        nb_flat = np.concatenate(nb).astype(np.int32) if nb else np.zeros(0, np.int32)
        wt = np.array([x[0] for x in w["walls"]], np.int32)
        wp = np.zeros((len(w["walls"]), 7))
        for i, x in enumerate(w["walls"]):
            wp[i, :len(x[1])] = x[1]
        wid = np.array([x[2] for x in w["walls"]], np.int32)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(
            path, kind=w["kind"], geom=np.asarray(w["geom"]), grid=np.asarray(w["grid"], np.int32),
            periodic=np.asarray(w["periodic"], np.int32), in_ids=w["ids"], in_xyzr=w["xyzr"],
            ids=rec.ids, pos=rec.pos, vol=rec.vol, cen=rec.cen, nf=rec.nf, nv=rec.nv, ok=rec.ok, mrs=rec.mrs,
            nb=nb_flat, nb_off=nb_off, wall_type=wt, wall_params=wp, wall_id=wid)
        print(f"{name}: {len(rec)} cells, {int(rec.ok.sum())} kept, sum vol {rec.vol.sum():.15g}")


# Polytope fixtures: the reference's own polytope of the first POLY_CELLS cells
# (vertices, faces in its traversal order with neighbour, area, perimeter,
# normal and vertex loop; surface area; total edge distance) and its
# print_custom output for every cell over the fields that do not depend on
# vertex or face numbering.
POLY_NAMES = ["unit_cube_1000", "radical_1200", "periodic_poly_800", "sparse_dropped_40", "degenerate_cubic_216",
              "degenerate_fcc_256", "degenerate_fcc_walled_256"]
POLY_CELLS = 200
# polytopes of the edge cases (vertices near 1e5, a dense cluster, slabs and
# prisms of collinear and coplanar particles, a box's faces and block
# boundaries)
EDGE_POLY_NAMES = ["edge_far_box_500", "edge_cluster_1560", "edge_line_80", "edge_plane_150",
                   "edge_box_boundaries_296"]
# point location and ghost cells in the void containers (queries and ghosts
# deep inside the voids; a ghost in the slab container's void touches up to
# 327 of the slab's particles, beyond the engines' 128 vertices, so only the
# clustered one gets ghosts)
EDGE_LOCATE_NAMES = ["edge_slab_periodic_9000", "edge_voids_periodic_6008"]
EDGE_GHOST_NAMES = ["edge_voids_periodic_6008"]
CUSTOM_FORMAT = "%i %q %r %w %s %v %c %C %m %g %F %E %A %o"


def make_poly_fixtures(ref, all_cases, names=None):
    import tempfile
    for name in names or POLY_NAMES:
        w = all_cases[name]
        cells = ref.polytopes(w)[:POLY_CELLS]
        flat = []
        for c in cells:
            flat += [1.0 if c["ok"] else 0.0, len(c["verts"]), len(c["faces"]), c["sa"], c["ted"]]
            flat += list(np.asarray(c["verts"]).ravel())
            for nb, area, perim, nrm, loop in c["faces"]:
                flat += [nb, len(loop), area, perim, *nrm, *loop]
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "custom.txt")
            ref.print_custom(w, CUSTOM_FORMAT, path)
            text = open(path).read()
        out = os.path.join(HERE, f"poly_{name}.npz")
        np.savez_compressed(out, flat=np.asarray(flat, np.float64), ncells=len(cells),
                            custom_format=np.array(CUSTOM_FORMAT), custom_text=np.array(text))
        print(f"poly_{name}: {len(cells)} cells, {os.path.getsize(out)} bytes")


# Normal fixtures: the reference's print_custom of "%i %n %l" over every cell,
# each face's neighbour beside its normal, so that a test can pair them
# whatever the face order (faces whose normals_search finds no pair above
# the tolerance print 0 0 0).
NORMAL_FORMAT = "%i %n %l"
NORMAL_NAMES = ["unit_cube_1000", "radical_1200", "periodic_poly_800", "edge_box_boundaries_296",
                "edge_far_box_500"]


def make_normal_fixtures(ref, all_cases):
    import tempfile
    for name in NORMAL_NAMES:
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "custom.txt")
            ref.print_custom(all_cases[name], NORMAL_FORMAT, path)
            text = open(path).read()
        out = os.path.join(HERE, f"normals_{name}.npz")
        np.savez_compressed(out, custom_format=np.array(NORMAL_FORMAT), custom_text=np.array(text))
        print(f"normals_{name}: {os.path.getsize(out)} bytes")


# Point-location fixtures: query points and the reference's find_voronoi_cell
# answer for each (found flag, particle ID, returned particle position): points
# spread over the domain grown by 20% on every side (outside a non-periodic
# wall: not found), the stored particle positions themselves, and, where an
# axis is periodic, points several box lengths away.
LOCATE_QUERIES = 400


def locate_queries(w, seed):
    rng = np.random.default_rng(seed)
    g = np.asarray(w["geom"], float)
    if w["kind"] in (W.KIND_PERIODIC, W.KIND_PERIODIC_POLY):
        lo, hi = np.zeros(3), np.array([g[0], g[2], g[5]])
    else:
        lo, hi = g[0::2], g[1::2]
    span = hi - lo
    a = rng.uniform(lo - 0.2 * span, hi + 0.2 * span, size=(LOCATE_QUERIES - 100, 3))
    b = w["xyzr"][rng.choice(len(w["ids"]), 50), :3]
    c = rng.uniform(lo, hi, size=(50, 3)) + rng.integers(-3, 4, size=(50, 3)) * span
    return np.concatenate([a, b, c])


def make_locate_fixtures(ref, all_cases, seed0=3000):
    for i, (name, w) in enumerate(all_cases.items()):
        q = locate_queries(w, seed0 + i)
        found, pid, r = ref.find_voronoi_cells(w, q)
        out = os.path.join(HERE, f"locate_{name}.npz")
        np.savez_compressed(out, q=q, found=found, pid=pid, r=r)
        print(f"locate_{name}: {len(q)} queries, {int(found.sum())} found, {os.path.getsize(out)} bytes")


# Ghost-cell fixtures: ghost particles and the reference's compute_ghost_cell
# record for each (ok, volume, centroid, faces, vertices, max_radius_squared,
# sorted neighbours): ghosts spread over the domain grown by 10% (outside a
# non-periodic wall: no cell) and, where periodic, some boxes away; radical
# kinds give each ghost a radius from the particles' own range.
GHOST_COUNT = 200


def ghost_particles(w, seed):
    rng = np.random.default_rng(seed)
    g = np.asarray(w["geom"], float)
    if w["kind"] in (W.KIND_PERIODIC, W.KIND_PERIODIC_POLY):
        lo, hi = np.zeros(3), np.array([g[0], g[2], g[5]])
    else:
        lo, hi = g[0::2], g[1::2]
    span = hi - lo
    a = rng.uniform(lo - 0.1 * span, hi + 0.1 * span, size=(GHOST_COUNT - 40, 3))
    c = rng.uniform(lo, hi, size=(40, 3)) + rng.integers(-2, 3, size=(40, 3)) * span
    xyz = np.concatenate([a, c])
    r = w["xyzr"][:, 3]
    rad = rng.uniform(r.min(), r.max(), size=len(xyz)) if w["kind"] in (W.KIND_CONTAINER_POLY,
                                                                          W.KIND_PERIODIC_POLY) else np.full(len(xyz), 0.5)
    return np.concatenate([xyz, rad[:, None]], 1)


def make_ghost_fixtures(ref, all_cases, seed0=4000, nb_per_cell=60):
    for i, (name, w) in enumerate(all_cases.items()):
        gx = ghost_particles(w, seed0 + i)
        rec = ref.ghost_cells(w, gx, nb_per_cell=nb_per_cell)
        nb = [np.sort(rec.neighbors(k)) for k in range(len(rec))]
        nb_off = np.zeros(len(rec) + 1, np.int64)
        nb_off[1:] = np.cumsum([len(x) for x in nb])
        nb_flat = np.concatenate(nb).astype(np.int32) if nb else np.zeros(0, np.int32)
        out = os.path.join(HERE, f"ghost_{name}.npz")
        np.savez_compressed(out, g=gx, ok=rec.ok, vol=rec.vol, cen=rec.cen, nf=rec.nf, nv=rec.nv, mrs=rec.mrs,
                            nb=nb_flat, nb_off=nb_off)
        print(f"ghost_{name}: {len(gx)} ghosts, {int(rec.ok.sum())} cells, {os.path.getsize(out)} bytes")


# Command-line fixtures (cli_*.npz): the reference's own voro++ utility
# (oracle/_ref/voro++, built from src/cmd_line.cc) run on seeded particle
# files with the flags of each case; stored: the arguments, the input file's
# text, the .vol text, with -v the printed summary, and any drawing outputs.
# A format's %n (face order: numbering dependent) is always its last field.
def cli_cases():
    rng = np.random.default_rng(5001)

    def text(n, lo, hi, radii=None):
        xyz = rng.uniform(lo, hi, size=(n, 3))
        lines = []
        for i in range(n):
            row = "%d %.17g %.17g %.17g" % (i, xyz[i, 0], xyz[i, 1], xyz[i, 2])
            if radii is not None:
                row += " %.17g" % radii[i]
            lines.append(row)
        return "\n".join(lines) + "\n"

    out = {}
    out["cli_cube_default"] = (["0", "1", "0", "1", "0", "1"], text(1000, 0.0, 1.0))
    out["cli_periodic_custom"] = (["-p", "-v", "-c", "%i %q %v %s %w %g %F %E %A %C %m %n", "0", "2", "0", "2", "0", "2"],
                                  text(2000, 0.0, 2.0))
    r = rng.uniform(0.02, 0.06, size=1500)
    out["cli_poly_ordered_sphere"] = (["-r", "-o", "-ws", "1", "1", "1", "0.9", "-c", "%i %v %s %r %n",
                                       "0", "2", "0", "2", "0", "2"], text(1500, -0.1, 2.1, radii=r))
    out["cli_length_scale_xy_periodic"] = (["-l", "0.15", "-px", "-py", "-v", "0", "1.5", "0", "1.5", "0", "1.5"],
                                           text(1200, -0.2, 1.7))
    r = rng.uniform(0.3, 1.0, size=800)
    out["cli_grid_ordered_poly"] = (["-n", "3", "4", "5", "-o", "-r", "-c", "%i %q %v %s %w %c", "0", "8", "0", "8",
                                     "0", "8"], text(800, 0.0, 8.0, radii=r))
    out["cli_box_walls"] = (["-wb", "0.1", "0.9", "0.15", "0.85", "0.2", "0.8", "-c", "%i %v %s %F %n",
                             "0", "1", "0", "1", "0", "1"], text(900, 0.0, 1.0))
    out["cli_cylinder_cone"] = (["-wc", "1", "1", "0", "0", "0", "1", "0.8", "-wo", "1", "1", "2.2", "0", "0", "-1",
                                 "0.6", "-c", "%i %v %s %w", "0", "2", "0", "2", "0", "2"], text(1500, 0.0, 2.0))
    out["cli_drawing"] = (["-g", "-y", "0", "1", "0", "1", "0", "1"], text(120, 0.0, 1.0))
    return out


def make_cli_fixtures():
    import subprocess
    import tempfile
    exe = os.path.join(ROOT, "oracle", "_ref", "voro++")
    if not os.path.exists(exe):
        raise SystemExit("the reference command-line utility was not built (make -C oracle ref)")
    for name, (args, txt) in cli_cases().items():
        with tempfile.TemporaryDirectory() as td:
            fn = os.path.join(td, "pts")
            open(fn, "w").write(txt)
            r = subprocess.run([exe] + args + [fn], capture_output=True, text=True, check=True)
            vol = open(fn + ".vol").read()
            extra = {}
            for suffix, key in ((".gnu", "gnu"), ("_p.pov", "povp"), ("_v.pov", "povv")):
                if os.path.exists(fn + suffix):
                    extra[key] = np.array(open(fn + suffix).read())
        out = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(out, args=np.array(args), input=np.array(txt), vol=np.array(vol),
                            stdout=np.array(r.stdout.replace(td, "<dir>")), **extra)
        print(f"{name}: {len(vol.splitlines())} cells, {os.path.getsize(out)} bytes")


def main():
    if not build_ref():
        raise SystemExit("reference sources not available; cannot generate fixtures")
    if "--cli-only" in sys.argv:
        make_cli_fixtures()
        return
    ref = RefLib()
    if "--poly-only" in sys.argv:
        make_poly_fixtures(ref, cases())
        return
    if "--locate-only" in sys.argv:
        make_locate_fixtures(ref, cases())
        return
    if "--ghost-only" in sys.argv:
        make_ghost_fixtures(ref, cases())
        return
    if "--walls-only" in sys.argv:
        make_wall_fixtures(ref)
        return
    if "--tric-only" in sys.argv:
        make_tric_fixtures(ref)
        return
    if "--degenerate-only" in sys.argv:
        dc = degenerate_cases()
        for name, w in dc.items():
            make_cell_fixture(ref, name, w)
        make_poly_fixtures(ref, dc, names=list(dc))
        return
    if "--edge-only" in sys.argv:
        ec = edge_cases()
        for name, w in ec.items():
            make_cell_fixture(ref, name, w)
        make_poly_fixtures(ref, ec, names=EDGE_POLY_NAMES)
        make_locate_fixtures(ref, {k: ec[k] for k in EDGE_LOCATE_NAMES}, seed0=3900)
        make_ghost_fixtures(ref, {k: ec[k] for k in EDGE_GHOST_NAMES}, seed0=4901, nb_per_cell=1000)
        return
    if "--normals-only" in sys.argv:
        make_normal_fixtures(ref, {**cases(), **edge_cases()})
        return
    if "--tric-large-only" in sys.argv:
        make_tric_large_fixture(ref)
        return
    for name, w in cases().items():
        make_cell_fixture(ref, name, w)
    make_poly_fixtures(ref, cases())
    make_normal_fixtures(ref, {**cases(), **edge_cases()})
    make_locate_fixtures(ref, cases())
    make_ghost_fixtures(ref, cases())
    make_wall_fixtures(ref)
    make_tric_fixtures(ref)
    make_tric_large_fixture(ref)
    ec = edge_cases()
    for name, w in ec.items():
        make_cell_fixture(ref, name, w)
    make_poly_fixtures(ref, ec, names=EDGE_POLY_NAMES)
    make_locate_fixtures(ref, {k: ec[k] for k in EDGE_LOCATE_NAMES}, seed0=3900)
    make_ghost_fixtures(ref, {k: ec[k] for k in EDGE_GHOST_NAMES}, seed0=4901, nb_per_cell=1000)
    make_cli_fixtures()


# A larger sheared box (cells only): 20,000 particles, so that the first
# compute's thin image layers hold (no rerun at the reference's depth).
def make_tric_large_fixture(ref):
    rng = np.random.default_rng(2207)
    geom = (20.0, -6.3, 18.5, 7.1, 4.9, 17.2)
    xyz = rng.uniform(-0.5, 1.5, size=(20000, 3)) * np.array([geom[0], geom[2], geom[5]])
    make_cell_fixture(ref, "tric_large_20000", W._pack(W.KIND_PERIODIC, geom, (9, 9, 8), (True,) * 3, xyz))


def make_tric_fixtures(ref):
    tc = tric_cases()
    for name, w in tc.items():
        make_cell_fixture(ref, name, w)
    make_locate_fixtures(ref, tc, seed0=3100)
    make_ghost_fixtures(ref, tc, seed0=4100)


if __name__ == "__main__":
    main()
