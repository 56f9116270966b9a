"""A seeded sweep of containers unlike the fixtures: clustered particles with
voids between the clusters, slabs in boxes periodic across them (cells that
reach across most of the box, to images many blocks away), random periodic
flags and block grids.  Both engines against the CPU port, which follows the
reference operation for operation: topology exact, volumes and centroids to
the engines' bounds."""
import numpy as np
import pytest

import oracle
import voro_gb300 as vg
from voro_gb300 import workloads as W
from tests import _golden as G

TOL = {"fp64": (1e-12, 1e-12), "mixed": (1e-10, 1e-10)}
CASES = 24


def sweep_case(c):
    r = np.random.default_rng(70000 + c)
    kind = (W.KIND_CONTAINER, W.KIND_PERIODIC)[c % 2]
    n = int(np.exp(r.uniform(np.log(200), np.log(8000))))
    L = float(np.exp(r.uniform(np.log(0.5), np.log(20.0))))
    dist = ("uniform", "clusters", "slab")[(c // 2) % 3]
    if dist == "uniform":
        xyz = r.random((n, 3)) * L
    elif dist == "clusters":
        k = int(r.integers(1, 6))
        cen = r.random((k, 3)) * L
        xyz = np.mod(cen[r.integers(0, k, n)] + r.normal(0.0, L * float(r.uniform(0.01, 0.1)), (n, 3)), L)
    else:
        xyz = r.random((n, 3)) * L
        xyz[:, int(r.integers(0, 3))] *= float(r.uniform(0.05, 0.3))
    g = max(1, int(round((n / float(r.uniform(1.5, 8.0))) ** (1 / 3))))
    if kind == W.KIND_PERIODIC:
        return W._pack(kind, (L, 0, L, 0, 0, L), (g, g, g), (True,) * 3, xyz)
    per = tuple(bool(v) for v in r.integers(0, 2, 3))
    return W._pack(kind, (0, L, 0, L, 0, L), (g, g, g), per, xyz)


@pytest.fixture(scope="module")
def port():
    return oracle.PortLib()


@pytest.mark.gpu
@pytest.mark.parametrize("c", range(CASES))
def test_sweep_matches_port(gpu, port, c):
    w = sweep_case(c)
    ref = port.compute(w)
    nb = np.concatenate([np.sort(ref.neighbors(k)) for k in range(len(ref))])
    z = {"ids": ref.ids, "pos": ref.pos, "vol": ref.vol, "cen": ref.cen, "nf": ref.nf, "nv": ref.nv,
         "ok": ref.ok, "nb": nb, "nb_off": ref.nb_off}
    for mode in ("mixed", "fp64"):
        con = vg.from_workload(w, mode=mode)
        con.compute_all_cells()
        st = con.stats()
        errs = G.compare_cells(con.cells(), z, *TOL[mode], label=f"sweep {c}/{mode}")
        assert not errs, "\n".join(errs) + f"\nstats {st}"
        assert st["marginal_cells"] == 0 and st["failed_cells"] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_sweep_as_one_batch_matches_port(gpu, port, mode):
    """The same containers as members of one batch (binned together, one
    launch per pass): every member against the port."""
    ws = [sweep_case(c) for c in range(CASES)]
    cons = [vg.from_workload(w, mode=mode) for w in ws]
    b = vg.batch(cons)
    b.compute_all_cells(mode=mode)
    for c, (w, con) in enumerate(zip(ws, cons)):
        ref = port.compute(w)
        nb = np.concatenate([np.sort(ref.neighbors(k)) for k in range(len(ref))])
        z = {"ids": ref.ids, "pos": ref.pos, "vol": ref.vol, "cen": ref.cen, "nf": ref.nf, "nv": ref.nv,
             "ok": ref.ok, "nb": nb, "nb_off": ref.nb_off}
        errs = G.compare_cells(con.cells(), z, *TOL[mode], label=f"batch sweep {c}/{mode}")
        assert not errs, "\n".join(errs)
