"""Full-size workloads (the bench configurations) checked by size-independent
properties, plus bit-exact topology against the CPU port on a seeded sample:

* Σ cell volumes = container volume;
* neighbour relation symmetric with multiplicity (j lists i as often as i
  lists j — periodic images included);
* Euler's relation for simple polyhedra, V = 2F − 4 (every vertex the engine
  produces has order 3);
* MIXED and FP64 engines give the same topology on every cell, volumes and
  centroids within 1e-10;
* a seeded sample of cells matches the CPU port (which is bit-exact with the
  reference) in face count, vertex count and neighbour multiset, with volume
  and centroid within the engine's tolerance."""
import numpy as np
import pytest

import oracle
import voro_gb300 as vg
from tests import _golden as G
from voro_gb300 import workloads as W

CASES = {
    "unit_cube_100k": (lambda: W.unit_cube(), "fp64"),
    "periodic_4m": (lambda: W.periodic_cube(), "mixed"),
    "radical_2m": (lambda: W.radical_box(), "mixed"),
    "fcc_jitter_1m": (lambda: W.fcc_jitter(), "mixed"),
}
TOL = {"fp64": 1e-12, "mixed": 1e-10}
SAMPLE = 1500


def _symmetric(res):
    ids = res.ids.astype(np.int64)
    owner = np.repeat(ids, np.diff(res.nb_off))
    m = res.nb >= 0
    a, b = owner[m], res.nb[m].astype(np.int64)
    n = int(ids.max()) + 1
    return np.array_equal(np.sort(a * n + b), np.sort(b * n + a))


@pytest.fixture(scope="module")
def port():
    oracle.build_port()
    return oracle.PortLib()


@pytest.mark.gpu
def test_sheared_box_full_size_invariants(gpu):
    """A 1M-particle sheared periodic box (images stored in ghost layers):
    volumes tile the box, Euler's relation, a symmetric neighbour relation,
    and the MIXED and FP64 engines agree on every cell's topology."""
    w = W.sheared_periodic(n=1_000_000, L=100.0 * (1 / 4) ** (1 / 3))
    res = {}
    for mode in ("mixed", "fp64"):
        con = vg.from_workload(w, mode=mode)
        con.compute_all_cells()
        st = con.stats()
        assert st["failed_cells"] == 0 and st["marginal_cells"] == 0
        r = con.cells()
        vbox = G.box_volume(w)
        assert abs(con.sum_cell_volumes() - vbox) <= 1e-9 * vbox
        assert np.all(r.ok)
        simple = (r.flags & vg.VGPU_CELL_MARGINAL) == 0   # (merged vertices: V < 2F - 4)
        assert np.array_equal(r.nv[simple], 2 * r.nf[simple] - 4), "Euler relation V = 2F - 4"
        assert _symmetric(r), "neighbour relation not symmetric"
        res[mode] = r
    a, b = res["mixed"], res["fp64"]
    assert np.array_equal(a.ids, b.ids) and np.array_equal(a.pos, b.pos)
    assert np.array_equal(a.nf, b.nf) and np.array_equal(a.nv, b.nv)
    assert np.array_equal(a.nb_off, b.nb_off) and np.array_equal(a.nb, b.nb)
    assert (np.abs(a.vol - b.vol) / b.vol).max() <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_full_size_invariants_and_sample_parity(gpu, port, name):
    make, mode = CASES[name]
    w = make()
    con = vg.from_workload(w, mode=mode)
    con.compute_all_cells()
    st = con.stats()
    assert st["failed_cells"] == 0
    res = con.cells()
    ok = res.ok
    vbox = G.box_volume(w)
    assert abs(con.sum_cell_volumes() - vbox) <= 1e-9 * vbox
    # Euler's relation: V = 2F - 4 where every vertex has order 3, V < 2F - 4
    # where the tolerance band merged vertices into ones of higher order
    simple = ok & ((res.flags & vg.VGPU_CELL_MARGINAL) == 0)
    assert np.array_equal(res.nv[simple], 2 * res.nf[simple] - 4), "Euler relation V = 2F - 4"
    assert np.all(res.nv[ok] <= 2 * res.nf[ok] - 4)
    assert _symmetric(res), "neighbour relation not symmetric"

    rng = np.random.default_rng(7)
    sel = np.sort(rng.choice(len(res), size=min(SAMPLE, len(res)), replace=False))
    ref = port.compute_selected(w, sel)
    assert np.array_equal(res.ids[sel], ref.ids)
    assert np.array_equal(res.pos[sel], ref.pos)
    assert np.array_equal(ok[sel], ref.ok != 0)
    m = ref.ok != 0
    assert np.array_equal(res.nf[sel][m], ref.nf[m])
    assert np.array_equal(res.nv[sel][m], ref.nv[m])
    for r, k in enumerate(sel):
        if m[r]:
            assert np.array_equal(np.sort(res.neighbors(k)), np.sort(ref.neighbors(r))), f"cell {k}"
    rel = np.abs(res.vol[sel][m] - ref.vol[m]) / ref.vol[m]
    assert rel.max() <= TOL[mode]
    scale = np.cbrt(ref.vol[m])[:, None]
    assert (np.abs(res.cen[sel][m] - ref.cen[m]) / scale).max() <= TOL[mode]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["periodic_4m", "radical_2m", "fcc_jitter_1m", "unit_cube_100k"])
def test_mixed_and_fp64_agree_on_every_cell(gpu, name):
    """The mixed engine against the plain FP64 engine on every cell of the
    full-size workloads: identical deleted flags, face and vertex counts and
    neighbour lists; volume within 1e-10 relative and centroid within 1e-10
    of the cell size."""
    w = CASES[name][0]()
    a = vg.from_workload(w, mode="mixed")
    a.set_fp64_fallback(1.0)   # the FP32 engine on every cell, even where its filter band is saturated
    b = vg.from_workload(w, mode="fp64")
    ra, rb = a.cells(), b.cells()
    assert a.stats()["fp64_engine_cells"] == 0
    assert np.array_equal(ra.ok, rb.ok)
    assert np.array_equal(ra.nf, rb.nf)
    assert np.array_equal(ra.nv, rb.nv)
    assert np.array_equal(ra.nb_off, rb.nb_off)
    assert np.array_equal(ra.nb, rb.nb)
    ok = rb.ok
    assert (np.abs(ra.vol[ok] - rb.vol[ok]) / rb.vol[ok]).max() <= 1e-10
    scale = np.cbrt(rb.vol[ok])[:, None]
    assert (np.abs(ra.cen[ok] - rb.cen[ok]) / scale).max() <= 1e-10
    sa, sb = a.stats(), b.stats()
    assert sa["failed_cells"] == 0 and sb["failed_cells"] == 0
    if name != "fcc_jitter_1m":
        # generic input: few FP64 repairs, and even the FP64 engine's own
        # rounding band is never met (the jittered lattice meets both on purpose)
        assert sa["fp64_repairs"] <= 0.01 * sa["side_tests"]
        assert sb["marginal_cells"] == 0


@pytest.mark.gpu
def test_saturated_filter_band_switches_to_the_fp64_engine(gpu):
    """A mixed compute samples its FP32 first pass; on the jittered FCC lattice
    (every cell meets the filter band) the whole container runs on the FP64
    engine, with the same topology as the FP32 engine forced through; on
    uniform input nothing switches."""
    w = W.fcc_jitter()
    a = vg.from_workload(w, mode="mixed")
    ra = a.cells()
    assert a.stats()["fp64_engine_cells"] == len(ra)
    f = vg.from_workload(w, mode="mixed")
    f.set_fp64_fallback(1.0)
    rf = f.cells()
    assert np.array_equal(ra.nf, rf.nf) and np.array_equal(ra.nv, rf.nv)
    assert np.array_equal(ra.nb_off, rf.nb_off) and np.array_equal(ra.nb, rf.nb)
    assert (np.abs(ra.vol - rf.vol) / ra.vol).max() <= 1e-10
    u = vg.from_workload(W.periodic_cube(n=500_000, L=50.0, grid=(46, 46, 46)), mode="mixed")
    u.compute_all_cells()
    assert u.stats()["fp64_engine_cells"] == 0


@pytest.mark.gpu
def test_large_container_24m(gpu):
    """A container whose polytope records pass 4G words of offsets (24M
    cells): no cell fails, volumes still sum to the box."""
    n = 24_000_000
    L = 100.0 * (n / 4e6) ** (1 / 3)
    g = int(round((n / 5.0) ** (1 / 3)))
    w = W.periodic_cube(n=n, L=L, seed=1010, grid=(g, g, g))
    con = vg.from_workload(w, mode="mixed")
    con.compute_all_cells()
    st = con.stats()
    assert st["cells"] == n and st["failed_cells"] == 0
    assert abs(con.sum_cell_volumes() - L ** 3) <= 1e-9 * L ** 3
