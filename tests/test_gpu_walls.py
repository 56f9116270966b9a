"""Walls (wall_sphere, wall_plane, wall_cylinder, wall_cone) on the GPU
against the reference's records for containers with walls: which cells are
kept, face and vertex counts and neighbour lists (wall IDs included)
exactly, volumes and centroids within the engine's tolerance; single
computes and a batch."""
import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G

TOL = {"fp64": (1e-12, 1e-12), "mixed": (1e-10, 1e-10)}


@pytest.mark.gpu
@pytest.mark.parametrize("name", G.wall_names())
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_walls_match_reference(gpu, name, mode):
    w, z = G.load(name)
    con = vg.from_workload(w, mode=mode)
    con.compute_all_cells()
    errs = G.compare_cells(con.cells(), z, *TOL[mode], label=f"{name}/{mode}")
    assert not errs, "\n".join(errs)


@pytest.mark.gpu
def test_walls_in_a_batch(gpu):
    names = G.wall_names()
    cons = [vg.from_workload(G.load(n)[0], mode="mixed") for n in names]
    b = vg.batch(cons)
    b.compute_all_cells(mode="mixed")
    for n, c in zip(names, cons):
        errs = G.compare_cells(c.cells(), G.load(n)[1], *TOL["mixed"], label=f"batch/{n}")
        assert not errs, "\n".join(errs)


@pytest.mark.gpu
def test_point_inside_walls(gpu):
    """point_inside_walls (src/container.hh:75-78) with the walls' own tests
    (src/wall.cc:17-95)."""
    w, z = G.load("wall_cone_2000")
    con = vg.from_workload(w, mode="mixed")
    p = z["pos"]
    # cone: apex 0, axis z, angle 0.5; plane z < 1.8
    rad2 = p[:, 0] ** 2 + p[:, 1] ** 2
    pa = p[:, 2] * np.tan(0.5)
    expect = (pa >= 0) & (rad2 < pa * pa) & (p[:, 2] < 1.8)
    got = np.array([con.point_inside_walls(*q) for q in p])
    assert np.array_equal(got, expect)


@pytest.mark.gpu
def test_point_inside_box_and_walls(gpu):
    """container_base::point_inside (src/container.cc:484-487): the box
    first, then the walls."""
    w, z = G.load("wall_cone_2000")
    con = vg.from_workload(w, mode="mixed")
    g = w["geom"]
    rng = np.random.default_rng(5)
    q = rng.uniform([g[0] - 0.5, g[2] - 0.5, g[4] - 0.5], [g[1] + 0.5, g[3] + 0.5, g[5] + 0.5], size=(400, 3))
    in_box = np.all((q >= [g[0], g[2], g[4]]) & (q <= [g[1], g[3], g[5]]), axis=1)
    walls = np.array([con.point_inside_walls(*p) for p in q])
    got = np.array([con.point_inside(*p) for p in q])
    assert np.array_equal(got, in_box & walls)
    assert in_box.any() and (~in_box).any() and (in_box & walls).any()
