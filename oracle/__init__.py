"""Oracle for the per-cell Voronoi path — TEST INFRASTRUCTURE ONLY.

Two checkers live here; neither is part of the product and only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
them:

* ``RefLib``  — the unmodified reference (Voro++), compiled from its own
  sources into ``oracle/_ref/libvoro_ref.so`` by ``oracle/Makefile``.  It only
  exists where the reference tree exists.
* ``PortLib`` — the CPU restatement of the reference's cell algorithm in
  ``oracle/port/`` (built into ``oracle/_build/libvoro_port.so``).  It builds
  anywhere and is pinned against ``RefLib`` and the committed golden fixtures.

Both return per-cell records in the reference's loop order (c_loop_all,
src/c_loops.hh:165-210; c_loop_all_periodic, src/c_loops.hh:325-393).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libvoro_ref.so")
PORT_SO = os.path.join(HERE, "_build", "libvoro_port.so")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def ref_src() -> str:
    """The reference's src/ directory: $VORO_REF_SRC when set, else a checkout
    named "reference" beside this repository (the reference tree is absent on
    hosts that only run the tests)."""
    return os.environ.get("VORO_REF_SRC") or os.path.abspath(os.path.join(HERE, "..", "..", "reference", "src"))


def build_ref(quiet=True) -> bool:
    """Builds the reference library if its sources are present."""
    ref_src_dir = ref_src()
    if not os.path.isfile(os.path.join(ref_src_dir, "voro++.cc")):
        return False
    subprocess.run(["make", "-C", HERE, "ref", f"REF_SRC={ref_src_dir}"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return os.path.isfile(REF_SO)


def build_port(quiet=True) -> bool:
    subprocess.run(["make", "-C", HERE, "port"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return os.path.isfile(PORT_SO)


class CellRecords:
    """Per-cell results in loop order; neighbours in CSR form."""

    def __init__(self, ids, pos, vol, cen, nf, nv, ok, mrs, nb, nb_off, tests=None):
        self.ids, self.pos, self.vol, self.cen = ids, pos, vol, cen
        self.nf, self.nv, self.ok, self.mrs = nf, nv, ok, mrs
        self.nb, self.nb_off = nb, nb_off
        self.tests = tests

    def __len__(self):
        return len(self.ids)

    def neighbors(self, k):
        return self.nb[self.nb_off[k]:self.nb_off[k + 1]]

    def sorted_neighbors(self, k):
        return np.sort(self.neighbors(k))

    def by_id(self):
        """Index permutation that orders records by particle ID."""
        return np.argsort(self.ids, kind="stable")


class _Lib:
    path = None

    def __init__(self):
        if not os.path.isfile(self.path):
            raise FileNotFoundError(self.path)
        self.lib = ctypes.CDLL(self.path)
        f = self.lib.ref_compute_cells if hasattr(self.lib, "ref_compute_cells") else None
        self._setup(f)

    def _setup(self, f):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p,
                      ctypes.c_int, _i32p, _f64p, _f64p, _f64p, _i32p, _i32p, _i32p, _f64p,
                      ctypes.c_long, _i32p, _i64p]
        self._compute = f

    def compute(self, w, nb_per_cell=40) -> CellRecords:
        n = len(w["ids"])
        geom = np.asarray(w["geom"], dtype=np.float64)
        grid = np.asarray(w["grid"], dtype=np.int32)
        per = np.asarray([1 if p else 0 for p in w["periodic"]], dtype=np.int32)
        cap = max(n, 1)
        nb_cap = max(64, n * nb_per_cell)
        while True:
            ids = np.zeros(cap, np.int32); pos = np.zeros(3 * cap); vol = np.zeros(cap)
            cen = np.zeros(3 * cap); nf = np.zeros(cap, np.int32); nv = np.zeros(cap, np.int32)
            ok = np.zeros(cap, np.int32); mrs = np.zeros(cap)
            nb = np.zeros(nb_cap, np.int32); nb_off = np.zeros(cap + 1, np.int64)
            m = self._compute(int(w["kind"]), geom, grid, per, n, w["ids"], w["xyzr"], cap,
                              ids, pos, vol, cen, nf, nv, ok, mrs, nb_cap, nb, nb_off)
            if m >= 0:
                break
            if m == -2:
                raise ValueError("bad container kind")
            nb_cap *= 2
        return CellRecords(ids[:m], pos[:3 * m].reshape(m, 3), vol[:m], cen[:3 * m].reshape(m, 3),
                           nf[:m], nv[:m], ok[:m], mrs[:m], nb[:nb_off[m]], nb_off[:m + 1])


class RefLib(_Lib):
    path = REF_SO

    def compute(self, w, nb_per_cell=40) -> CellRecords:
        _walls(self.lib, w)
        return super().compute(w, nb_per_cell)

    def polytopes(self, w):
        """The reference's polytope of every cell (parse_polytopes format)."""
        _walls(self.lib, w)
        f = self.lib.ref_polytopes
        f.restype = ctypes.c_long
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p, ctypes.c_long, _f64p]
        cap = max(1024, 300 * len(w["ids"]))
        while True:
            out = np.zeros(cap)
            m = f(*_args(w), cap, out)
            if m >= 0:
                return parse_polytopes(out[:m])
            cap = -m

    def print_custom(self, w, fmt, path):
        """The reference's container::print_custom(fmt, path) output."""
        _walls(self.lib, w)
        f = self.lib.ref_print_custom
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p, ctypes.c_char_p,
                      ctypes.c_char_p]
        if f(*_args(w), fmt.encode(), str(path).encode()) != 0:
            raise ValueError("bad container kind")

    def find_voronoi_cells(self, w, q):
        """The reference's find_voronoi_cell for each row of q (n x 3):
        (found, pid, r) with r the returned particle positions (n x 3)."""
        _walls(self.lib, w)
        f = self.lib.ref_find_voronoi_cells
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p, ctypes.c_int, _f64p,
                      _i32p, _i32p, _f64p]
        q = np.ascontiguousarray(q, np.float64)
        nq = len(q)
        found = np.zeros(nq, np.int32)
        pid = np.zeros(nq, np.int32)
        r = np.zeros((nq, 3), np.float64)
        if f(*_args(w), nq, q, found, pid, r) != 0:
            raise ValueError("bad container kind")
        return found, pid, r

    def ghost_cells(self, w, gxyzr, nb_per_cell=60) -> CellRecords:
        """The reference's compute_ghost_cell for each row of gxyzr (x, y, z,
        r): one record per ghost (ids -1, pos = the given position)."""
        _walls(self.lib, w)
        f = self.lib.ref_ghost_cells
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p, ctypes.c_int, _f64p,
                      _i32p, _f64p, _f64p, _i32p, _i32p, _f64p, ctypes.c_long, _i32p, _i64p]
        g = np.ascontiguousarray(gxyzr, np.float64).reshape(-1, 4)
        m = len(g)
        ok = np.zeros(m, np.int32); vol = np.zeros(m); cen = np.zeros((m, 3)); nf = np.zeros(m, np.int32)
        nv = np.zeros(m, np.int32); mrs = np.zeros(m)
        cap = nb_per_cell * max(m, 1)
        nb = np.zeros(cap, np.int32); nb_off = np.zeros(m + 1, np.int64)
        if f(*_args(w), m, g, ok, vol, cen, nf, nv, mrs, cap, nb, nb_off) != 0:
            raise ValueError("ghost cells: bad kind or neighbour capacity")
        return CellRecords(np.full(m, -1, np.int32), g[:, :3].copy(), vol, cen, nf, nv, ok, mrs,
                           nb[:nb_off[m]], nb_off)

    def time_compute_all(self, w):
        f = self.lib.ref_time_compute_all
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p,
                      ctypes.POINTER(ctypes.c_double)]
        sv = ctypes.c_double(0)
        t = f(int(w["kind"]), np.asarray(w["geom"], np.float64), np.asarray(w["grid"], np.int32),
              np.asarray([1 if p else 0 for p in w["periodic"]], np.int32), len(w["ids"]),
              w["ids"], w["xyzr"], ctypes.byref(sv))
        return t, sv.value


def parse_polytopes(flat):
    """Splits a flat polytope stream (see ref_polytopes in oracle/ref_capi.cc)
    into per-cell dicts: ok, verts (nv,3), sa, ted, faces [(nb, area,
    perimeter, normal(3), [vertex indices])]."""
    cells = []
    i = 0
    n = len(flat)
    while i < n:
        ok, nv, nf, sa, ted = flat[i:i + 5]
        i += 5
        nv, nf = int(nv), int(nf)
        verts = np.asarray(flat[i:i + 3 * nv]).reshape(nv, 3)
        i += 3 * nv
        faces = []
        for _ in range(nf):
            nb, order, area, perim, nx, ny, nz = flat[i:i + 7]
            i += 7
            order = int(order)
            faces.append((int(nb), float(area), float(perim), (float(nx), float(ny), float(nz)),
                          [int(v) for v in flat[i:i + order]]))
            i += order
        cells.append({"ok": bool(ok), "verts": verts, "sa": float(sa), "ted": float(ted), "faces": faces})
    return cells


def _walls(lib, w):
    """Hands the workload's walls (list of (type, params, id)) to the
    reference driver; they apply to kind 0/1 containers."""
    f = lib.ref_set_walls
    f.restype = None
    f.argtypes = [ctypes.c_int, _i32p, _f64p, _i32p]
    walls = w.get("walls") or []
    t = np.array([x[0] for x in walls], np.int32)
    p = np.zeros((len(walls), 7), np.float64)
    for i, x in enumerate(walls):
        p[i, :len(x[1])] = x[1]
    ids = np.array([x[2] for x in walls], np.int32)
    f(len(walls), t, np.ascontiguousarray(p), ids)


def _args(w):
    return (int(w["kind"]), np.asarray(w["geom"], np.float64), np.asarray(w["grid"], np.int32),
            np.asarray([1 if p else 0 for p in w["periodic"]], np.int32), len(w["ids"]),
            np.ascontiguousarray(w["ids"], np.int32), np.ascontiguousarray(w["xyzr"], np.float64))


class PortLib(_Lib):
    """The CPU restatement (oracle/port), same records as RefLib plus the
    per-cell count of vertex-plane side tests."""
    path = PORT_SO

    def _setup(self, f):
        f = self.lib.port_compute_cells
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p,
                      ctypes.c_int, _i32p, _f64p, _f64p, _f64p, _i32p, _i32p, _i32p, _f64p,
                      ctypes.c_long, _i32p, _i64p, _i64p]
        self._compute_port = f
        t = self.lib.port_time_cells
        t.restype = ctypes.c_double
        t.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p, ctypes.c_long,
                      ctypes.c_long, ctypes.c_int, ctypes.POINTER(ctypes.c_long),
                      ctypes.POINTER(ctypes.c_ulonglong)]
        self._time = t

    def compute(self, w, nb_per_cell=40) -> CellRecords:
        n = len(w["ids"])
        geom = np.asarray(w["geom"], dtype=np.float64)
        grid = np.asarray(w["grid"], dtype=np.int32)
        per = np.asarray([1 if p else 0 for p in w["periodic"]], dtype=np.int32)
        cap = max(n, 1)
        nb_cap = max(64, n * nb_per_cell)
        while True:
            ids = np.zeros(cap, np.int32); pos = np.zeros(3 * cap); vol = np.zeros(cap)
            cen = np.zeros(3 * cap); nf = np.zeros(cap, np.int32); nv = np.zeros(cap, np.int32)
            ok = np.zeros(cap, np.int32); mrs = np.zeros(cap)
            nb = np.zeros(nb_cap, np.int32); nb_off = np.zeros(cap + 1, np.int64); tests = np.zeros(cap, np.int64)
            m = self._compute_port(int(w["kind"]), geom, grid, per, n, w["ids"], w["xyzr"], cap,
                                   ids, pos, vol, cen, nf, nv, ok, mrs, nb_cap, nb, nb_off, tests)
            if m >= 0:
                break
            if m == -2:
                raise ValueError("unsupported container for the port")
            nb_cap *= 2
        return CellRecords(ids[:m], pos[:3 * m].reshape(m, 3), vol[:m], cen[:3 * m].reshape(m, 3),
                           nf[:m], nv[:m], ok[:m], mrs[:m], nb[:nb_off[m]], nb_off[:m + 1], tests[:m])

    def compute_selected(self, w, sel, nb_per_cell=40) -> CellRecords:
        """Records of the cells at loop-order positions ``sel`` only."""
        f = self.lib.port_compute_selected
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, _f64p, _i32p, _i32p, ctypes.c_int, _i32p, _f64p, ctypes.c_int, _i64p,
                      _i32p, _f64p, _f64p, _f64p, _i32p, _i32p, _i32p, _f64p, ctypes.c_long, _i32p, _i64p]
        sel = np.ascontiguousarray(sel, dtype=np.int64)
        m = len(sel)
        cap = max(m, 1)
        nb_cap = max(64, m * nb_per_cell)
        while True:
            ids = np.zeros(cap, np.int32); pos = np.zeros(3 * cap); vol = np.zeros(cap)
            cen = np.zeros(3 * cap); nf = np.zeros(cap, np.int32); nv = np.zeros(cap, np.int32)
            ok = np.zeros(cap, np.int32); mrs = np.zeros(cap)
            nb = np.zeros(nb_cap, np.int32); nb_off = np.zeros(cap + 1, np.int64)
            r = f(int(w["kind"]), np.asarray(w["geom"], np.float64), np.asarray(w["grid"], np.int32),
                  np.asarray([1 if p else 0 for p in w["periodic"]], np.int32), len(w["ids"]), w["ids"], w["xyzr"],
                  m, sel, ids, pos, vol, cen, nf, nv, ok, mrs, nb_cap, nb, nb_off)
            if r >= 0:
                break
            if r != -1:
                raise ValueError(f"port_compute_selected failed ({r})")
            nb_cap *= 2
        return CellRecords(ids[:m], pos[:3 * m].reshape(m, 3), vol[:m], cen[:3 * m].reshape(m, 3),
                           nf[:m], nv[:m], ok[:m], mrs[:m], nb[:nb_off[m]], nb_off[:m + 1])

    def time_cells(self, w, first=0, count=None, threads=1):
        """Seconds to compute cells [first, first+count) of the loop order with
        `threads` threads; returns (seconds, cells)."""
        n = len(w["ids"])
        count = n if count is None else count
        done = ctypes.c_long(0)
        tests = ctypes.c_ulonglong(0)
        t = self._time(int(w["kind"]), np.asarray(w["geom"], np.float64), np.asarray(w["grid"], np.int32),
                       np.asarray([1 if p else 0 for p in w["periodic"]], np.int32), n, w["ids"], w["xyzr"],
                       int(first), int(count), int(threads), ctypes.byref(done), ctypes.byref(tests))
        self.last_side_tests = tests.value
        return t, done.value

    def worklists(self):
        f = self.lib.port_worklists
        f.restype = ctypes.c_int
        out = np.zeros(4096, np.uint32)
        f.argtypes = [np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS"), ctypes.c_int]
        m = f(out, 4096)
        return out[:m]
