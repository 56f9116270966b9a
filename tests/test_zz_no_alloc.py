"""vgpu_sum_volumes_noalloc: Σ cell volumes from device-resident results with
its partial sums in a fixed static device array (no allocation), checked
against vgpu_sum_cell_volumes through the C ABI on two calls in a row.

Collected last on purpose (file name): the entry point's one-time per-device
set-up must work both in a fresh process and after every other test has used
the library."""
import ctypes

import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G

MAX_CELLS = 4096 * 8192


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = vg.load_library()
    fake = ctypes.c_void_p(256)   # never dereferenced: the size check comes first
    assert lib.vgpu_sum_volumes_noalloc(fake, MAX_CELLS + 1, fake, None) == 16
    msg = lib.vgpu_last_error().decode()
    assert "scratch capacity" in msg and str(MAX_CELLS) in msg
    assert lib.vgpu_sum_volumes_noalloc(fake, -1, fake, None) == 16
    assert lib.vgpu_sum_volumes_noalloc(fake, 10, None, None) == 16


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["periodic_2000", "radical_1200", "sparse_dropped_40"])
def test_noalloc_sum_matches_sum_cell_volumes(gpu, name):
    torch = pytest.importorskip("torch")
    lib = vg.load_library()
    w, _ = G.load(name)
    con = vg.from_workload(w, mode="mixed")
    con.compute_all_cells()
    ref = con.sum_cell_volumes()
    n = con.total_particles()
    dev_vol = ctypes.c_void_p()
    assert lib.vgpu_device_results(con._h, ctypes.byref(dev_vol), None) == 0
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        rc = lib.vgpu_sum_volumes_noalloc(dev_vol, n, ctypes.c_void_p(out.data_ptr() + 8 * call), stream)
        assert rc == 0, lib.vgpu_last_error().decode()
    torch.cuda.synchronize()
    first, second = out.tolist()
    assert first == second   # fixed summation order
    assert abs(first - ref) <= 1e-12 * abs(ref), (first, ref)
    assert abs(first - G.box_volume(w)) <= 1e-9 * G.box_volume(w)


@pytest.mark.gpu
def test_noalloc_sum_of_nothing_is_zero(gpu):
    torch = pytest.importorskip("torch")
    lib = vg.load_library()
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.vgpu_sum_volumes_noalloc(None, 0, ctypes.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    assert out.item() == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3 * 4096 + 17, MAX_CELLS])
def test_noalloc_many_tiles_and_the_size_limit(gpu, n):
    """Several tile partials, a partial last tile, and exactly the largest n
    the scratch holds, against a host sum; repeated calls give identical bits."""
    import math
    torch = pytest.importorskip("torch")
    lib = vg.load_library()
    g = torch.Generator(device="cuda:0")
    g.manual_seed(11)
    vol = torch.rand(n, dtype=torch.float64, device="cuda:0", generator=g)
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        rc = lib.vgpu_sum_volumes_noalloc(ctypes.c_void_p(vol.data_ptr()), n,
                                          ctypes.c_void_p(out.data_ptr() + 8 * call), stream)
        assert rc == 0, lib.vgpu_last_error().decode()
    torch.cuda.synchronize()
    first, second = out.tolist()
    assert first == second
    host = vol.cpu().numpy()
    exact = math.fsum(host.tolist()) if n < 100_000 else float(host.sum(dtype=np.float64))
    assert abs(first - exact) <= 1e-12 * exact, (first, exact)


@pytest.mark.gpu
def test_noalloc_refuses_host_pointers(gpu):
    """A host array passed as device memory is refused before any launch."""
    torch = pytest.importorskip("torch")
    lib = vg.load_library()
    host = np.ones(100)
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.vgpu_sum_volumes_noalloc(host.ctypes.data_as(ctypes.c_void_p), 100,
                                        ctypes.c_void_p(out.data_ptr()), stream) == 16
    assert "not device memory" in lib.vgpu_last_error().decode()
    dev = torch.ones(100, dtype=torch.float64, device="cuda:0")
    hout = np.zeros(1)
    assert lib.vgpu_sum_volumes_noalloc(ctypes.c_void_p(dev.data_ptr()), 100,
                                        hout.ctypes.data_as(ctypes.c_void_p), stream) == 16
    # still usable afterwards
    assert lib.vgpu_sum_volumes_noalloc(ctypes.c_void_p(dev.data_ptr()), 100,
                                        ctypes.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    assert out.item() == 100.0
