"""Ghost cells (compute_ghost_cell) on the GPU against the reference's own
records in the fixtures: which ghosts have a cell, face and vertex counts and
sorted neighbour lists exactly, volumes and centroids within the engine's
tolerance; the container's own results stay as they were."""
import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G

TOL = {"fp64": 1e-12, "mixed": 1e-10}


@pytest.mark.gpu
@pytest.mark.parametrize("name", G.ghost_names())
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_ghost_cells_match_reference(gpu, name, mode):
    w, _ = G.load(name)
    g, z = G.load_ghost(name)
    con = vg.from_workload(w, mode=mode)
    res = con.compute_ghost_cells(g[:, :3], g[:, 3])
    ok = z["ok"] != 0
    assert np.array_equal(res.ok, ok)
    assert np.array_equal(res.nf[ok], z["nf"][ok])
    # vertex counts exactly, also in cells with vertices of order 4 or more (a
    # ghost among exactly degenerate lattice points: the engine merges the
    # coincident vertices of its cuts as the reference does)
    assert np.array_equal(res.nv[ok], z["nv"][ok])
    for k in np.nonzero(ok)[0]:
        ref = z["nb"][z["nb_off"][k]:z["nb_off"][k + 1]]
        assert np.array_equal(np.sort(res.neighbors(k)), ref), k
    if ok.any():
        rel = np.abs(res.vol[ok] - z["vol"][ok]) / z["vol"][ok]
        assert rel.max() <= TOL[mode]
        scale = np.cbrt(z["vol"][ok])[:, None]
        assert (np.abs(res.cen[ok] - z["cen"][ok]) / scale).max() <= TOL[mode]


@pytest.mark.gpu
def test_ghost_cells_leave_the_container_results(gpu):
    name = "periodic_2000"
    w, _ = G.load(name)
    g, z = G.load_ghost(name)
    con = vg.from_workload(w, mode="mixed")
    before = con.cells()
    vol0, nb0 = before.vol.copy(), before.nb.copy()
    con.compute_ghost_cells(g[:, :3], g[:, 3])
    after = con.cells()
    assert np.array_equal(after.vol, vol0)
    assert np.array_equal(after.nb, nb0)
    # and a ghost compute with polytopes on gives every kept ghost its polytope
    con.set_polytopes(True)
    con.compute_all_cells()
    res = con.compute_ghost_cells(g[:, :3], g[:, 3])
    for k in np.nonzero(res.ok)[0][:20]:
        p = res.polytope(k)
        assert p is not None and np.asarray(p.vertices()).reshape(-1, 3).shape[0] == res.nv[k]
