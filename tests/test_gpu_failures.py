"""Failure paths, driven without faulting anything.

* A record store too small for the compute: the clipping kernels check every
  record against the store's capacity before writing it, so the cells that do
  not fit are reported (VGPU_CELL_FAILED, reason VGPU_FAIL_RECORDS) and the
  compute returns VGPU_ERR_CAPACITY, while the cells that fit are complete and
  still match the reference.
* Non-finite particle coordinates: put() rejects them on the host before
  anything is staged; device-resident input (put_device) is checked by the
  binning kernels and the compute is refused before any cell is computed.
"""
import numpy as np
import pytest

import voro_gb300 as vg
from voro_gb300 import workloads as W
from tests import _golden as G

TOL = {"fp64": 1e-12, "mixed": 1e-10}


def _reason(flags):
    return (flags >> 8) & 15


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_small_record_store_fails_cells_not_the_gpu(gpu, mode):
    w, z = G.load("periodic_2000")
    con = vg.from_workload(w, mode=mode)
    con.set_record_budget(300_000)   # room for a few hundred of the 2000 cells' records
    with pytest.raises(vg.VoroError) as e:
        con.compute_all_cells()
    assert e.value.code == vg.VGPU_ERR_CAPACITY
    got = con.cells()
    st = con.stats()
    failed = (got.flags & vg.VGPU_CELL_FAILED) != 0
    assert 0 < failed.sum() < len(got)
    assert st["failed_cells"] == failed.sum()
    assert np.all(_reason(got.flags[failed]) == vg.VGPU_FAIL_RECORDS)
    assert np.all(got.vol[failed] == 0.0) and np.all(got.nf[failed] == 0)
    # the cells that fit are complete and match the reference
    done = ~failed
    assert np.all(got.ok[done])
    assert np.array_equal(got.nf[done], z["nf"][done])
    assert np.array_equal(got.nv[done], z["nv"][done])
    rel = np.abs(got.vol[done] - z["vol"][done]) / z["vol"][done]
    assert rel.max() <= TOL[mode]
    for k in np.nonzero(done)[0][:200]:
        ref = z["nb"][z["nb_off"][k]:z["nb_off"][k + 1]]
        assert np.array_equal(np.sort(got.neighbors(k)), ref)
    # the default budget again: every cell, exact
    con.set_record_budget(0)
    con.compute_all_cells()
    errs = G.compare_cells(con.cells(), z, TOL[mode], TOL[mode], label=f"after/{mode}")
    assert not errs, "\n".join(errs)


@pytest.mark.gpu
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_put_rejects_nonfinite_positions(gpu, bad):
    rng = np.random.default_rng(7)
    xyz = rng.random((300, 3))
    ids = np.arange(300, dtype=np.int32)
    con = vg.container(0, 1, 0, 1, 0, 1, 4, 4, 4, False, False, False, 8)
    con.put_array(ids[:200], xyz[:200])
    tail = xyz[200:].copy()
    tail[37, 1] = bad
    with pytest.raises(vg.VoroError) as e:
        con.put_array(ids[200:], tail)
    assert e.value.code == vg.VGPU_ERR_ARG
    # nothing of the rejected call was staged: the container holds the first 200
    ref = vg.container(0, 1, 0, 1, 0, 1, 4, 4, 4, False, False, False, 8)
    ref.put_array(ids[:200], xyz[:200])
    a, b = con.cells(), ref.cells()
    assert np.array_equal(a.ids, b.ids) and np.array_equal(a.vol, b.vol)
    assert abs(con.sum_cell_volumes() - 1.0) < 1e-9


@pytest.mark.gpu
def test_put_radius_checked_only_for_radical_containers(gpu):
    rng = np.random.default_rng(8)
    xyz = rng.random((100, 3))
    ids = np.arange(100, dtype=np.int32)
    r = np.full(100, 0.05)
    r[5] = np.nan
    mono = vg.container(0, 1, 0, 1, 0, 1, 3, 3, 3, False, False, False, 8)
    mono.put_array(ids, xyz, r)   # the radius is ignored by a monodisperse container
    assert abs(mono.sum_cell_volumes() - 1.0) < 1e-9
    poly = vg.container_poly(0, 1, 0, 1, 0, 1, 3, 3, 3, False, False, False, 8)
    with pytest.raises(vg.VoroError) as e:
        poly.put_array(ids, xyz, r)
    assert e.value.code == vg.VGPU_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("n", [500, 6000, 20000])   # both shared-memory binning tiers, the multi-kernel binning
def test_put_device_nonfinite_refused_by_compute(gpu, n):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    xyzr = np.zeros((n, 4))
    xyzr[:, :3] = rng.random((n, 3)) * 10.0
    xyzr[n // 3, 2] = np.nan
    d_ids = torch.arange(n, dtype=torch.int32, device="cuda")
    d_xyzr = torch.from_numpy(xyzr).to("cuda")
    con = vg.container_periodic(10, 0, 10, 0, 0, 10, 5, 5, 5, 8)
    con.put_device(n, d_ids.data_ptr(), d_xyzr.data_ptr(), keepalive=(d_ids, d_xyzr))
    with pytest.raises(vg.VoroError) as e:
        con.compute_all_cells()
    assert e.value.code == vg.VGPU_ERR_ARG
    # in a batch, too (members of at most 16384 particles are binned together)
    con2 = vg.container_periodic(10, 0, 10, 0, 0, 10, 5, 5, 5, 8)
    con2.put_device(n, d_ids.data_ptr(), d_xyzr.data_ptr(), keepalive=(d_ids, d_xyzr))
    b = vg.batch([con2])
    with pytest.raises(vg.VoroError) as e:
        b.compute_all_cells()
    assert e.value.code == vg.VGPU_ERR_ARG
    # the same arrays made finite compute normally
    d_xyzr[n // 3, 2] = 5.0
    con.compute_all_cells()
    assert abs(con.sum_cell_volumes() - 1000.0) < 1e-9 * 1000.0


@pytest.mark.gpu
def test_destroyed_containers_free_their_device_memory(gpu):
    """Every device buffer a container allocates (binning, a sheared box's
    images, hand-on lists) goes back when it is destroyed: a run of sheared,
    periodic and plain containers created, computed and dropped leaves
    device memory where it was."""
    import gc
    import torch
    ws = [W.small_random(20000, kind=k, L=10.0, seed=s) for s, k in enumerate((2, 3, 0, 1))]
    ws.append(W.sheared_periodic(n=20000, L=30.0, seed=7))
    for w in ws:   # warm: the library's own one-off allocations
        c = vg.from_workload(w, mode="mixed")
        c.compute_all_cells()
        del c
    gc.collect()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(12):
        for w in ws:
            c = vg.from_workload(w, mode="mixed")
            c.compute_all_cells()
            c.cells()
            del c
    gc.collect()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < 64 << 20, f"{(free0 - free1) >> 20} MiB not returned"
