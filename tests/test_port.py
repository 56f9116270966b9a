"""The CPU oracle port (oracle/port) against the reference.

The port restates the reference's cell algorithm with the same arithmetic
order; on the golden fixtures it must reproduce the reference bit for bit
(volumes, centroids, counts and even the order of neighbour IDs).  Where the
reference tree is present it is also compared directly on fresh inputs."""
import os
import re

import numpy as np
import pytest

from tests import _golden as G


@pytest.fixture(scope="module")
def port():
    from oracle import PortLib, build_port
    assert build_port()
    return PortLib()


# Fixtures whose volumes and centroids the port reproduces to a few units in
# the last place rather than bit for bit (topology and neighbours exact):
#  * degenerate_fcc_256: the reference merges exactly coincident vertices of
#    order 4 with arithmetic the port does not restate step by step;
#  * edge_periodic_wraps_300: container_periodic with particles exactly on
#    block faces.  The reference fills its y/z image layers lazily, re-bucketing
#    each particle by x against the image block's face (create_side_image,
#    src/container_prd.cc:583-624, where a particle on the face goes to the
#    block on its left, shifted by bx at the box edge, or stays, depending on
#    which neighbouring image block was created first); the port's image
#    layers are plain shifted copies, so those particles' planes are tested in
#    another order or computed from a position one box length over.
ULP_FIXTURES = {"degenerate_fcc_256", "edge_periodic_wraps_300"}


@pytest.mark.parametrize("name", G.names())
def test_port_matches_golden_bit_for_bit(port, name):
    if "tric_" in name:
        pytest.skip("the port restates the rectangular periodic box only")
    w, z = G.load(name)
    r = port.compute(w)
    assert np.array_equal(r.ids, z["ids"])
    assert np.array_equal(r.pos, z["pos"])
    assert np.array_equal(r.ok, z["ok"])
    assert np.array_equal(r.nf, z["nf"])
    assert np.array_equal(r.nv, z["nv"])
    if name in ULP_FIXTURES:
        # exactly coincident vertices of order 4: the topology is exact, the
        # arithmetic of the reference's vertex merging is not restated step by
        # step, so volumes and centroids agree to a few units in the last place
        assert np.allclose(r.vol, z["vol"], rtol=1e-15, atol=0)
        assert np.allclose(r.cen, z["cen"], rtol=0, atol=1e-15)
        assert np.allclose(r.mrs, z["mrs"], rtol=1e-15, atol=0)
    else:
        assert np.array_equal(r.vol, z["vol"])
        assert np.array_equal(r.cen, z["cen"])
        assert np.array_equal(r.mrs, z["mrs"])
    for k in range(len(r.ids)):
        assert np.array_equal(np.sort(r.neighbors(k)), z["nb"][z["nb_off"][k]:z["nb_off"][k + 1]])


def test_port_counts_side_tests(port):
    w, _ = G.load("periodic_2000")
    r = port.compute(w)
    assert r.tests.min() > 0
    assert 200 < r.tests.mean() < 2000


def test_port_threads_give_same_work(port):
    w, _ = G.load("radical_1200")
    t1, m1 = port.time_cells(w, threads=1)
    s1 = port.last_side_tests
    t4, m4 = port.time_cells(w, threads=4)
    assert m1 == m4 == len(w["ids"])
    assert port.last_side_tests == s1


def test_worklists_match_reference_table(port):
    from oracle import ref_src
    ref_wl = os.path.join(ref_src(), "v_base_wl.cc")
    if not os.path.exists(ref_wl):
        pytest.skip("reference tree not present")
    txt = open(ref_wl).read()
    body = txt[txt.index("{") + 1:txt.rindex("}")]
    vals = np.array([int(t, 0) for t in re.findall(r"0x[0-9a-f]+|\b\d+\b", body)], dtype=np.uint32)
    assert np.array_equal(vals, port.worklists())


@pytest.mark.parametrize("kind,periodic,seed", [(0, (False,) * 3, 11), (0, (True, False, True), 12),
                                                (1, (False,) * 3, 13), (2, (True,) * 3, 14), (3, (True,) * 3, 15)])
def test_port_matches_reference_on_fresh_inputs(port, kind, periodic, seed):
    from oracle import REF_SO, RefLib
    if not os.path.exists(REF_SO):
        pytest.skip("reference library not built here")
    from voro_gb300 import workloads as W
    w = W.small_random(700, kind=kind, L=3.0, periodic=periodic, seed=seed)
    a = port.compute(w)
    b = RefLib().compute(w)
    assert np.array_equal(a.vol, b.vol)
    assert np.array_equal(a.nb, b.nb)
    assert np.array_equal(a.nv, b.nv)
