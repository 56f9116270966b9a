"""Batched containers (vgpu_batch_*): many containers computed by one
persistent launch give the per-container results (same topology exactly,
volumes and centroids to the last few bits)."""
import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G
from voro_gb300 import workloads as W

TOL = {"fp64": (1e-12, 1e-12), "mixed": (1e-10, 1e-10)}


def test_batch_needs_a_device():
    try:
        if vg.device_count() > 0:
            pytest.skip("a GPU is present")
    except vg.VoroError:
        pass
    with pytest.raises(vg.VoroError):
        vg.batch()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_batch_of_golden_fixtures_matches_reference(gpu, mode):
    # every kind, sheared periodic boxes included (not the known limits,
    # whose topology or capacity is tested one container at a time)
    names = [n for n in G.names() if n not in G.KNOWN_LIMIT and n not in G.CAPACITY_LIMIT]
    cons, refs = [], []
    for name in names:
        w, z = G.load(name)
        cons.append(vg.from_workload(w, mode=mode))
        refs.append((w, z))
    b = vg.batch(cons)
    b.compute_all_cells(mode=mode)
    st = b.stats()
    assert st["cells"] == sum(len(z["ids"]) for _, z in refs)
    assert st["failed_cells"] == 0
    for name, con, (w, z) in zip(names, cons, refs):
        errs = G.compare_cells(con.cells(), z, *G.tolerance(name, mode, TOL[mode]), label=f"batch/{name}/{mode}")
        assert not errs, "\n".join(errs)
        assert abs(con.sum_cell_volumes() - G.box_volume(w)) <= 1e-9 * G.box_volume(w)


@pytest.mark.gpu
def test_batch_equals_one_container_at_a_time(gpu):
    ws = W.batched(count=48, nmin=64, nmax=20000, seed=77)
    single = []
    for w in ws:
        c = vg.from_workload(w, mode="mixed")
        c.compute_all_cells()
        single.append(c.cells())
    cons = [vg.from_workload(w, mode="mixed") for w in ws]
    b = vg.batch(cons)
    b.compute_all_cells(mode="mixed")
    for k, (c, a) in enumerate(zip(cons, single)):
        r = c.cells()
        assert np.array_equal(r.ids, a.ids), k
        assert np.array_equal(r.flags, a.flags), k
        assert np.array_equal(r.nf, a.nf), k
        assert np.array_equal(r.nv, a.nv), k
        assert np.array_equal(r.nb_off, a.nb_off), k
        assert np.array_equal(r.nb, a.nb), k
        # the finish kernel sums a cell's terms in an order that depends on
        # which cell shares its warp, so the last bits may differ
        assert np.allclose(r.vol, a.vol, rtol=1e-13, atol=0), k
        scale = np.cbrt(np.maximum(a.vol, 1e-300))[:, None]
        assert (np.abs(r.cen - a.cen) / scale).max() <= 1e-13, k
    # a second compute of the same batch gives exactly the same again
    first = cons[3].cells().vol.copy()
    b.compute_all_cells(mode="mixed")
    assert np.array_equal(cons[3].cells().vol, first)


@pytest.mark.gpu
def test_batch_edge_members(gpu):
    """Members binned by the one-CTA path next to ones binned by the
    multi-kernel path: an empty container, one that drops particles outside
    its walls, one of exactly the small-path limit and one just above it."""
    rng = np.random.default_rng(5)

    def walled(n):
        c = vg.container(0, 1, 0, 1, 0, 1, 6, 6, 6, False, False, False, mode="mixed")
        xyz = rng.uniform(-0.2, 1.2, size=(n, 3))
        c.put_array(np.arange(n, dtype=np.int32), xyz)
        return c

    def periodic(n):
        c = vg.container_periodic(10, 0, 10, 0, 0, 10, 8, 8, 8, mode="mixed")
        c.put_array(np.arange(n, dtype=np.int32), rng.uniform(0, 10, size=(n, 3)))
        return c

    # sizes either side of the two shared-memory binning tiers (4096, 16384)
    makers = [lambda: walled(0), lambda: walled(3000), lambda: periodic(4096), lambda: periodic(4097),
              lambda: walled(1), lambda: periodic(16384), lambda: periodic(16385), lambda: walled(9000)]
    state = rng.bit_generator.state
    single = []
    for m in makers:
        c = m()
        c.compute_all_cells()
        single.append(c.cells())
    rng.bit_generator.state = state
    cons = [m() for m in makers]
    b = vg.batch(cons)
    b.compute_all_cells(mode="mixed")
    for k, (c, a) in enumerate(zip(cons, single)):
        r = c.cells()
        assert len(r) == len(a), k
        assert np.array_equal(r.ids, a.ids), k
        assert np.array_equal(r.pos, a.pos), k
        assert np.array_equal(r.nf, a.nf), k
        assert np.array_equal(r.nb, a.nb), k
        assert np.allclose(r.vol, a.vol, rtol=1e-13, atol=0), k
    assert len(cons[0].cells()) == 0
    assert 0 < len(cons[1].cells()) < 3000


@pytest.mark.gpu
def test_batch_reports_duplicates_in_a_small_member(gpu):
    c = vg.container_periodic(10, 0, 10, 0, 0, 10, 4, 4, 4, mode="mixed")
    xyz = np.random.default_rng(2).uniform(0, 10, size=(50, 3))
    xyz[17] = xyz[3]
    c.put_array(np.arange(50, dtype=np.int32), xyz)
    with pytest.raises(vg.VoroError):
        c.compute_all_cells()
    b = vg.batch([c])
    with pytest.raises(vg.VoroError):
        b.compute_all_cells(mode="mixed")


@pytest.mark.gpu
@pytest.mark.parametrize("with_small", [False, True])
def test_batch_reports_duplicates_in_a_large_member(gpu, with_small):
    """A member binned by the multi-kernel path (more than 16384 particles),
    whose duplicate check is read back only once the batch has waited for
    every member's binning: the batch still fails with VGPU_ERR_DUPLICATE."""
    rng = np.random.default_rng(5)
    n = 20000
    c = vg.container_periodic(30, 0, 30, 0, 0, 30, 16, 16, 16, mode="mixed")
    xyz = rng.uniform(0, 30, size=(n, 3))
    xyz[12345] = xyz[678]
    c.put_array(np.arange(n, dtype=np.int32), xyz)
    cons = [c]
    if with_small:
        s = vg.container_periodic(10, 0, 10, 0, 0, 10, 4, 4, 4, mode="mixed")
        s.put_array(np.arange(300, dtype=np.int32), rng.uniform(0, 10, size=(300, 3)))
        cons.append(s)
    b = vg.batch(cons)
    with pytest.raises(vg.VoroError) as e:
        b.compute_all_cells(mode="mixed")
    assert e.value.code == vg.VGPU_ERR_DUPLICATE
    # the same member without the duplicate computes
    xyz[12345] = rng.uniform(0, 30, size=3)
    c2 = vg.container_periodic(30, 0, 30, 0, 0, 30, 16, 16, 16, mode="mixed")
    c2.put_array(np.arange(n, dtype=np.int32), xyz)
    b2 = vg.batch([c2] + cons[1:])
    b2.compute_all_cells(mode="mixed")
    assert abs(c2.sum_cell_volumes() - 27000.0) < 1e-8 * 27000.0


@pytest.mark.gpu
def test_batch_in_record_waves_matches_one_wave(gpu):
    """A record budget far below the batch's records runs it in waves of
    cells (each clipped and finished before the next): the same results."""
    ws = W.batched(count=24, nmin=64, nmax=30000, seed=91)
    one = [vg.from_workload(w, mode="mixed") for w in ws]
    b1 = vg.batch(one)
    b1.compute_all_cells(mode="mixed")
    assert b1.waves() == 1
    many = [vg.from_workload(w, mode="mixed") for w in ws]
    b2 = vg.batch(many)
    b2.set_record_budget(40 << 20)   # about 40k cells per wave
    b2.compute_all_cells(mode="mixed")
    assert b2.waves() >= 3
    assert b2.stats()["failed_cells"] == 0
    for k, (c, a) in enumerate(zip(many, one)):
        r, q = c.cells(), a.cells()
        assert np.array_equal(r.ids, q.ids), k
        assert np.array_equal(r.flags, q.flags), k
        assert np.array_equal(r.nf, q.nf), k
        assert np.array_equal(r.nb, q.nb), k
        # (a wave may pair cells differently in the finish kernel's warps)
        assert np.allclose(r.vol, q.vol, rtol=1e-13, atol=0), k
        scale = np.cbrt(np.maximum(q.vol, 1e-300))[:, None]
        assert (np.abs(r.cen - q.cen) / scale).max() <= 1e-13, k


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_sheared_members_in_a_batch_of_mixed_kinds(gpu, mode):
    """Sheared container_periodic members (their images stored at the
    reference's depth) beside rectangular, radical and walled ones, in waves
    of the record store: the same cells as the reference."""
    names = ["tric_dyadic_1500", "periodic_2000", "tric_poly_1000", "radical_1200", "tric_skew_800",
             "wall_sphere_2000", "tric_generic_1200", "degenerate_tric_small_5"]
    cons, refs = [], []
    for name in names:
        w, z = G.load(name)
        cons.append(vg.from_workload(w, mode=mode))
        refs.append(z)
    b = vg.batch(cons)
    b.set_record_budget(4 << 20)   # a few waves
    b.compute_all_cells(mode=mode)
    assert b.waves() > 1
    assert b.stats()["failed_cells"] == 0
    for name, con, z in zip(names, cons, refs):
        errs = G.compare_cells(con.cells(), z, *TOL[mode], label=f"batch/{name}/{mode}")
        assert not errs, "\n".join(errs)
