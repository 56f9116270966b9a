"""GPU engine vs the reference on the golden fixtures, through the C ABI.

Bars: loop order, stored positions, deleted flags, face counts, vertex counts
and neighbour multisets exact; volume relative error <= 1e-12 (FP64 engine) or
1e-10 (mixed engine); centroid error <= the same bound times the cell size."""
import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G

NAMES = G.names()
TOL = {"fp64": (1e-12, 1e-12), "mixed": (1e-10, 1e-10)}
EXACTLY_COPLANAR = {"edge_single_periodic_1", "edge_pair_periodic_2"}


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("name", NAMES)
def test_fixture_parity(gpu, name, mode):
    if name in G.KNOWN_LIMIT:
        pytest.xfail(G.KNOWN_LIMIT[name])
    w, z = G.load(name)
    con = vg.from_workload(w, mode=mode)
    skip = None
    if name in G.CAPACITY_LIMIT:
        lim = G.CAPACITY_LIMIT[name]
        with pytest.raises(vg.VoroError) as e:
            con.compute_all_cells()
        assert e.value.code == vg.VGPU_ERR_CAPACITY
        got = con.cells()
        skip = (got.flags & vg.VGPU_CELL_FAILED) != 0
        assert sorted(got.ids[skip].tolist()) == sorted(lim["ids"])
        assert np.all(((got.flags[skip] >> 8) & 15) == lim["reason"])
    else:
        con.compute_all_cells()
    got = con.cells()
    st = con.stats()
    errs = G.compare_cells(got, z, *G.tolerance(name, mode, TOL[mode]), label=f"{name}/{mode}", skip=skip)
    assert not errs, "\n".join(errs) + f"\nstats {st}"
    if name in EXACTLY_COPLANAR:
        # a lone particle (or a pair) in a periodic box: its images' planes lie
        # exactly on the initial cell's faces, inside the tolerance band
        assert st["marginal_cells"] == len(z["ids"])
    elif not name.startswith("degenerate"):
        # generic inputs never touch the reference's tolerance band
        assert st["marginal_cells"] == 0
    assert st["failed_cells"] == (0 if skip is None else int(skip.sum()))
    if skip is None:
        s = con.sum_cell_volumes()
        assert abs(s - G.box_volume(w)) <= 1e-9 * G.box_volume(w)


@pytest.mark.gpu
def test_max_radius_matches_reference(gpu):
    w, z = G.load("periodic_2000")
    con = vg.from_workload(w, mode="fp64")
    got = con.cells(neighbors=False)
    # engine reports max |v|^2 in real units; the reference's is in doubled coordinates
    assert np.allclose(got.maxr2 * 4.0, z["mrs"], rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_recompute_is_deterministic(gpu):
    w, _ = G.load("radical_1200")
    con = vg.from_workload(w, mode="mixed")
    a = con.cells()
    con.compute_all_cells()
    b = con.cells()
    assert np.array_equal(a.vol, b.vol)
    assert np.array_equal(a.nb, b.nb)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["periodic_2000", "radical_1200", "wall_sphere_2000"])
def test_autotune_keeps_results(gpu, tmp_path, monkeypatch, name):
    """The tuning (engine-grid density, warps per CTA, cells per chunk)
    changes the search, never the cells; a cached choice is reused."""
    monkeypatch.setenv("VORO_GB300_TUNE_CACHE", str(tmp_path / "tune.txt"))
    w, z = G.load(name)
    con = vg.from_workload(w, mode="mixed")
    t, ms = con.autotune(cache=True)
    assert 0.3 <= t["particles_per_block"] <= 3.0 and ms > 0
    assert 1 <= t["warps_per_cta"] <= 8 and 1 <= t["cells_per_chunk"] <= 16
    assert con.tuning()["cells_per_chunk"] == t["cells_per_chunk"]
    errs = G.compare_cells(con.cells(), z, *TOL["mixed"], label="autotuned")
    assert not errs, "\n".join(errs)
    # other tuples of the search space give the same cells too
    for tup in [(0.35, 1, 1), (3.0, 2, 16), (1.0, 4, 4)]:
        con.set_tuning(*tup)
        errs = G.compare_cells(con.cells(), z, *TOL["mixed"], label=f"tuning {tup}")
        assert not errs, "\n".join(errs)
    # the cache: a second container of the same signature takes the stored tuple
    assert len(open(tmp_path / "tune.txt").read().split()) == 5
    con2 = vg.from_workload(w, mode="mixed")
    t2, _ = con2.autotune(cache=True)
    assert t2 == t


@pytest.mark.gpu
@pytest.mark.parametrize("spacings", [0.5, -1.0])
@pytest.mark.parametrize("name", ["tric_dyadic_1500", "tric_poly_1000", "tric_skew_800"])
def test_sheared_ghost_depth_never_changes_cells(gpu, name, spacings):
    """Image layers half a spacing deep (so most boundary cells reach past
    them and the compute is redone at the reference's depth), and always the
    reference's depth: the same cells as the reference either way."""
    w, z = G.load(name)
    con = vg.from_workload(w, mode="mixed")
    con.set_ghost_depth(spacings)
    con.compute_all_cells()
    errs = G.compare_cells(con.cells(), z, *TOL["mixed"], label=f"{name}/depth {spacings}")
    assert not errs, "\n".join(errs)
    assert con.stats()["failed_cells"] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(G.KNOWN_LIMIT))
def test_known_limit_fixtures_keep_their_geometry(gpu, name, mode):
    """Where the topology inside the tolerance band is not reproduced, the
    cells are still the reference's up to faces of vanishing area: every cell
    kept, volumes to 1e-12 relative (a mixed compute whose first pass is
    saturated reruns on the FP64 engine), the box filled."""
    w, z = G.load(name)
    con = vg.from_workload(w, mode=mode)
    con.compute_all_cells()
    got = con.cells()
    st = con.stats()
    assert st["failed_cells"] == 0
    assert np.array_equal(got.ids, z["ids"]) and np.array_equal(got.ok, z["ok"] != 0)
    rel = np.abs(got.vol - z["vol"]) / z["vol"]
    assert rel.max() <= 1e-12, rel.max()
    assert abs(con.sum_cell_volumes() - G.box_volume(w)) <= 1e-12 * G.box_volume(w)
    if mode == "mixed":
        assert st["fp64_engine_cells"] == len(z["ids"])
    # the same as a batch member beside a generic container: the member is
    # rerun on the FP64 engine after the batch, the other is untouched
    con2 = vg.from_workload(w, mode=mode)
    other_w, other_z = G.load("periodic_2000")
    other = vg.from_workload(other_w, mode=mode)
    b = vg.batch([con2, other])
    b.compute_all_cells(mode=mode)
    got2 = con2.cells()
    rel2 = np.abs(got2.vol - z["vol"]) / z["vol"]
    assert rel2.max() <= 1e-12, rel2.max()
    assert not G.compare_cells(other.cells(), other_z, *TOL[mode], label="batch/periodic_2000")
    if mode == "mixed":
        assert b.stats()["fp64_engine_cells"] == len(z["ids"])
