"""Point location (find_voronoi_cell) on the GPU against the reference's own
answers stored in the fixtures: found flags, particle IDs and returned
positions, bit for bit; once on a freshly filled container (the call bins it)
and once after a compute (the compute's binning is reused).  A sheared box
whose lattice terms are not dyadic returns image positions whose
displacements the reference summed in another order: there within a few
units in the last place of the box size."""
import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G


@pytest.mark.gpu
@pytest.mark.parametrize("name", G.locate_names())
@pytest.mark.parametrize("after_compute", [False, True])
def test_find_voronoi_cells_match_reference(gpu, name, after_compute):
    w, _ = G.load(name)
    q, found, pid, r = G.load_locate(name)
    con = vg.from_workload(w, mode="mixed")
    if after_compute:
        con.compute_all_cells()
    f, p, rr = con.find_voronoi_cells(q)
    assert np.array_equal(f, found != 0)
    m = found != 0
    assert np.array_equal(p[m], pid[m])
    if name.startswith("tric_generic"):
        L = float(np.abs(np.asarray(w["geom"])).sum())
        assert np.abs(rr[m] - r[m]).max() <= 64 * np.finfo(float).eps * L
    else:
        assert np.array_equal(rr[m], r[m])


@pytest.mark.gpu
def test_find_voronoi_cell_single_point_signature(gpu):
    name = G.locate_names()[0]
    w, _ = G.load(name)
    q, found, pid, r = G.load_locate(name)
    con = vg.from_workload(w, mode="mixed")
    k = int(np.nonzero(found)[0][0])
    ok, rx, ry, rz, i = con.find_voronoi_cell(*q[k])
    assert ok and i == pid[k] and (rx, ry, rz) == tuple(r[k])
