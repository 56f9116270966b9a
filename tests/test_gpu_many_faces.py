"""Cells of many faces: a radical container where a few large particles get
cells of up to about 43 faces and 82 vertices.  Their neighbour lists pass the
fixed 32-slot row (the rest goes to the overflow store) and their vertices the
64-slot engine (the 128-slot rerun takes them); everything must still match
the CPU port cell by cell, exactly in topology."""
import numpy as np
import pytest

import oracle
import voro_gb300 as vg
from voro_gb300 import workloads as W


def _workload():
    rng = np.random.default_rng(11)
    n = 6000
    xyz = rng.random((n, 3))
    r = np.full(n, 0.02)
    r[rng.choice(n, 40, replace=False)] = 0.065
    return W._pack(W.KIND_CONTAINER_POLY, (0, 1, 0, 1, 0, 1), (10, 10, 10), (False,) * 3, xyz, r)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_cells_with_more_faces_than_a_neighbour_row(gpu, mode):
    oracle.build_port()
    port = oracle.PortLib()
    w = _workload()
    ref = port.compute_selected(w, np.arange(len(w["ids"])))
    assert ref.nf.max() > 32 and ref.nv.max() > 64   # the case exercises both paths
    con = vg.from_workload(w, mode=mode)
    con.compute_all_cells()
    st = con.stats()
    assert st["failed_cells"] == 0
    assert st["overflow_reruns"] > 0
    res = con.cells()
    assert np.array_equal(res.ids, ref.ids)
    assert np.array_equal(res.nf, ref.nf)
    assert np.array_equal(res.nv, ref.nv)
    for k in range(len(res)):
        assert np.array_equal(np.sort(res.neighbors(k)), np.sort(ref.neighbors(k))), k
    tol = 1e-12 if mode == "fp64" else 1e-10
    m = ref.ok != 0   # (radical cells can vanish: volume 0 in both)
    assert np.array_equal(res.ok, m)
    assert (np.abs(res.vol[m] - ref.vol[m]) / ref.vol[m]).max() <= tol
    # the same through a batch
    c2 = vg.from_workload(w, mode=mode)
    b = vg.batch([c2])
    b.compute_all_cells(mode=mode)
    r2 = c2.cells()
    assert np.array_equal(r2.nb_off, res.nb_off)
    assert np.array_equal(r2.nb, res.nb)
