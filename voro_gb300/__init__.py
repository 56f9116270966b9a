"""GB300 engine for Voro++'s per-particle Voronoi cell computation.

The host classes mirror the reference's container API (src/container.hh,
src/container_prd.hh) and call the CUDA engine through its C ABI
(include/vorogpu.h, built into ``voro_gb300/_lib/libvorogpu.so``).  There is
no CPU fallback: if the library or a GPU is missing, construction raises.

    from voro_gb300 import container
    con = container(0, 1, 0, 1, 0, 1, 6, 6, 6, False, False, False, 8)
    for i, (x, y, z) in enumerate(points):
        con.put(i, x, y, z)
    vol = con.sum_cell_volumes()
    con.print_custom("%i %q %v %s %n", "out.vol")
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

from . import _build

VGPU_OK = 0
VGPU_FP64 = 0
VGPU_MIXED = 1
VGPU_CELL_OK = 1
VGPU_CELL_MARGINAL = 2
VGPU_CELL_REPAIRED = 4
VGPU_OUTPUT_POLYTOPES = 1
VGPU_CELL_FAILED = 8   # bits 8-11: reason (1 planes, 2 adjacency, 3 vertices, 4 search, 5 records)
VGPU_FAIL_RECORDS = 5
VGPU_ERR_ARG = 16
VGPU_ERR_DUPLICATE = 19
VGPU_ERR_CAPACITY = 21

KIND_CONTAINER = 0
KIND_CONTAINER_POLY = 1
KIND_PERIODIC = 2
KIND_PERIODIC_POLY = 3

# Reference status codes (src/config.hh:105-119) plus the engine's own.
STATUS_NAMES = {
    0: "VGPU_OK", 1: "VGPU_ERR_FILE", 2: "VGPU_ERR_MEMORY", 3: "VGPU_ERR_INTERNAL", 16: "VGPU_ERR_ARG",
    17: "VGPU_ERR_CUDA", 18: "VGPU_ERR_UNSUPPORTED", 19: "VGPU_ERR_DUPLICATE", 20: "VGPU_ERR_NOT_COMPUTED",
    21: "VGPU_ERR_CAPACITY", 22: "VGPU_ERR_NO_DEVICE",
}

# Every symbol include/vorogpu.h declares.
EXPORTED = [
    "vgpu_version", "vgpu_device_count", "vgpu_last_error", "vgpu_container_create", "vgpu_container_destroy",
    "vgpu_put", "vgpu_put_device", "vgpu_clear", "vgpu_compute", "vgpu_sum_cell_volumes", "vgpu_get_stats",
    "vgpu_num_cells", "vgpu_num_neighbors", "vgpu_get_cells", "vgpu_get_neighbors", "vgpu_device_results",
    "vgpu_set_tuning", "vgpu_set_ghost_depth", "vgpu_phase_cycles", "vgpu_get_radii",
    "vgpu_sum_volumes_noalloc", "vgpu_batch_create", "vgpu_batch_add", "vgpu_batch_compute",
    "vgpu_batch_get_stats", "vgpu_batch_destroy", "vgpu_batch_set_record_budget", "vgpu_batch_waves",
    "vgpu_set_output", "vgpu_get_polytopes", "vgpu_find_voronoi_cells", "vgpu_compute_ghost_cells",
    "vgpu_get_ghost_cells", "vgpu_get_ghost_neighbors", "vgpu_get_ghost_polytopes", "vgpu_add_wall",
    "vgpu_clear_walls", "vgpu_point_inside_walls",
    "vgpu_autotune", "vgpu_set_record_budget", "vgpu_phase_counts", "vgpu_set_fp64_fallback",
    "vgpu_get_input_rows", "vgpu_get_tuning", "vgpu_set_tuning_ex", "vgpu_autotune_ex",
    "vgpu_get_tolerance",
]


class Tuning(ctypes.Structure):
    """vgpu_tuning: the engine's per-container tuning (see include/vorogpu.h)."""
    _fields_ = [("particles_per_block", ctypes.c_double), ("warps_per_cta", ctypes.c_int),
                ("cells_per_chunk", ctypes.c_int), ("fp64_fallback", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


VGPU_TUNE_USE_CACHE = 1
VGPU_TUNE_WRITE_CACHE = 2


class VoroError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("cells", ctypes.c_int64), ("deleted", ctypes.c_int64), ("marginal_cells", ctypes.c_int64),
                ("side_tests", ctypes.c_int64), ("fp64_repairs", ctypes.c_int64),
                ("planes_tested", ctypes.c_int64), ("planes_cut", ctypes.c_int64),
                ("overflow_reruns", ctypes.c_int64), ("failed_cells", ctypes.c_int64),
                ("kernel_ms", ctypes.c_double), ("bin_ms", ctypes.c_double), ("step_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("clip_ms", ctypes.c_double),
                ("finish_ms", ctypes.c_double), ("fp64_engine_cells", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def library_path():
    return os.environ.get("VORO_GB300_LIB", _build.LIB)


def load_library(build_if_missing=True):
    """Loads libvorogpu.so (building it from source if absent).  Raises if it
    cannot be built or loaded: the engine has no CPU path."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if path == _build.LIB and (not os.path.exists(path) or (build_if_missing and not _build.up_to_date())):
        if not build_if_missing:
            raise RuntimeError(f"engine library missing: {path}")
        _build.build()
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    i64 = ctypes.c_int64
    pd = ctypes.POINTER(ctypes.c_double)
    pi = ctypes.POINTER(ctypes.c_int32)
    lib.vgpu_version.restype = ctypes.c_char_p
    lib.vgpu_last_error.restype = ctypes.c_char_p
    lib.vgpu_device_count.argtypes = [ctypes.POINTER(ctypes.c_int)]
    lib.vgpu_container_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, pd, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_int)]
    lib.vgpu_container_destroy.argtypes = [vp]
    lib.vgpu_put.argtypes = [vp, i64, vp, vp]
    lib.vgpu_put_device.argtypes = [vp, i64, vp, vp]
    lib.vgpu_clear.argtypes = [vp]
    lib.vgpu_compute.argtypes = [vp, ctypes.c_int]
    lib.vgpu_sum_cell_volumes.argtypes = [vp, pd]
    lib.vgpu_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.vgpu_num_cells.argtypes = [vp, ctypes.POINTER(i64)]
    lib.vgpu_num_neighbors.argtypes = [vp, ctypes.POINTER(i64)]
    lib.vgpu_get_cells.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.vgpu_get_neighbors.argtypes = [vp, vp, vp]
    lib.vgpu_device_results.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    lib.vgpu_set_tuning.argtypes = [vp, ctypes.c_double, ctypes.c_int]
    lib.vgpu_set_ghost_depth.argtypes = [vp, ctypes.c_double]
    lib.vgpu_set_record_budget.argtypes = [vp, ctypes.c_int64]
    lib.vgpu_set_fp64_fallback.argtypes = [vp, ctypes.c_double]
    lib.vgpu_get_tolerance.argtypes = [vp, pd]
    lib.vgpu_get_input_rows.argtypes = [vp, vp]
    lib.vgpu_get_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.vgpu_set_tuning_ex.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.vgpu_autotune_ex.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Tuning), pd]
    lib.vgpu_phase_cycles.argtypes = [vp, pd]
    lib.vgpu_phase_counts.argtypes = [vp, pd]
    lib.vgpu_get_radii.argtypes = [vp, vp]
    lib.vgpu_sum_volumes_noalloc.argtypes = [vp, i64, vp, vp]
    lib.vgpu_set_output.argtypes = [vp, ctypes.c_int]
    lib.vgpu_autotune.argtypes = [vp, ctypes.c_int, pd, pd]
    lib.vgpu_get_polytopes.argtypes = [vp, vp, vp]
    lib.vgpu_batch_create.argtypes = [ctypes.POINTER(vp)]
    lib.vgpu_batch_add.argtypes = [vp, vp]
    lib.vgpu_batch_compute.argtypes = [vp, ctypes.c_int]
    lib.vgpu_batch_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.vgpu_batch_destroy.argtypes = [vp]
    lib.vgpu_batch_set_record_budget.argtypes = [vp, ctypes.c_int64]
    lib.vgpu_find_voronoi_cells.argtypes = [vp, ctypes.c_int64, vp, vp, vp, vp]
    lib.vgpu_compute_ghost_cells.argtypes = [vp, ctypes.c_int, ctypes.c_int64, vp]
    lib.vgpu_add_wall.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int]
    lib.vgpu_clear_walls.argtypes = [vp]
    lib.vgpu_point_inside_walls.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_int)]
    lib.vgpu_get_ghost_cells.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    lib.vgpu_get_ghost_neighbors.argtypes = [vp, vp, vp]
    lib.vgpu_get_ghost_polytopes.argtypes = [vp, vp, vp]
    lib.vgpu_batch_waves.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    for name in EXPORTED:
        if name not in ("vgpu_version", "vgpu_last_error"):
            getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def _check(rc):
    if rc != VGPU_OK:
        raise VoroError(rc, _lib.vgpu_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def device_count():
    lib = load_library()
    c = ctypes.c_int(0)
    _check(lib.vgpu_device_count(ctypes.byref(c)))
    return c.value


class CellResults:
    """Per-cell results in the reference's loop order."""

    def __init__(self, ids, pos, vol, cen, nf, nv, maxr2, flags, nb=None, nb_off=None):
        self.ids, self.pos, self.vol, self.cen = ids, pos, vol, cen
        self.nf, self.nv, self.maxr2, self.flags = nf, nv, maxr2, flags
        self.nb, self.nb_off = nb, nb_off
        self.rad = None   # stored radii (put's r), filled by cells()
        self.poly_off = None   # polytope CSR (VGPU_OUTPUT_POLYTOPES), filled by cells()
        self.poly_data = None
        self.poly_tol = 0.0    # the container's length tolerance (vgpu_get_tolerance)

    def __len__(self):
        return len(self.ids)

    @property
    def ok(self):
        return (self.flags & VGPU_CELL_OK) != 0

    def neighbors(self, k):
        return self.nb[self.nb_off[k]:self.nb_off[k + 1]]

    def polytope(self, k):
        """Cell k's Polytope (needs the container's polytope output)."""
        if self.poly_off is None:
            raise ValueError("polytope output was not requested: call set_polytopes(True) before computing")
        a, b = self.poly_off[k], self.poly_off[k + 1]
        return Polytope.from_stream(self.poly_data[a:b], self.poly_tol) if b > a else None


class Polytope:
    """One cell's polytope as the engine returns it (VGPU_OUTPUT_POLYTOPES):
    vertices relative to the particle and faces as vertex loops, ordered by
    neighbour ID like ``neighbors()``.  The query names follow
    voronoicell_base (src/cell.hh:132-211) and compute the same quantities.
    ``tol`` is the container's length tolerance (vgpu_get_tolerance), the
    threshold below which normals() reports a face's normal as zero."""

    def __init__(self, verts, faces, tol=0.0):
        self.verts = verts                      # (nv, 3)
        self.faces = faces                      # [(neighbour, [vertex indices])]
        self.tol = float(tol)

    @classmethod
    def from_stream(cls, d, tol=0.0):
        nv, nf = int(d[0]), int(d[1])
        verts = np.asarray(d[2:2 + 3 * nv]).reshape(nv, 3)
        faces = []
        i = 2 + 3 * nv
        for _ in range(nf):
            nb, m = int(d[i]), int(d[i + 1])
            faces.append((nb, [int(v) for v in d[i + 2:i + 2 + m]]))
            i += 2 + m
        faces.sort(key=lambda f: f[0])          # stable: the order of neighbors()
        return cls(verts, faces, tol)

    @property
    def p(self):
        return len(self.verts)

    def vertices(self, x=0.0, y=0.0, z=0.0):
        return self.verts + np.array([x, y, z])

    def neighbors(self):
        return [f[0] for f in self.faces]

    def face_vertices(self):
        return [f[1] for f in self.faces]

    def face_orders(self):
        return [len(f[1]) for f in self.faces]

    def _newell(self, loop):
        # twice the vector area, from vectors relative to the first vertex
        # (small faces keep their precision)
        P = self.verts[loop] - self.verts[loop[0]]
        return np.cross(P[1:-1], P[2:]).sum(axis=0) if len(loop) > 2 else np.zeros(3)

    def face_areas(self):
        return [0.5 * float(np.linalg.norm(self._newell(f[1]))) for f in self.faces]

    def normals(self):
        """Outward unit normals, by the rule of voronoicell_base::normals_search
        (src/cell.cc:2108-2164): walking the loop from its second edge, the
        first edge longer than the tolerance is paired with each later edge
        until their vector product is above it; that product, normalised, is
        the normal.  The tests are on the reference's doubled coordinates (2x
        these vertices).  The reference walks from its lowest-numbered vertex
        of the face, a numbering the engine does not share; so each start is
        tried in turn, and a face gets (0, 0, 0) only when no start finds
        such a pair (a sliver, or a face whose edges are all shorter than the
        tolerance), where the reference's answer cannot depend on its start."""
        out = []
        for f in self.faces:
            P = self.verts[f[1]]
            E = np.roll(P, -1, axis=0) - P             # edge t: loop[t] -> loop[t+1]
            n = len(P)
            nrm = (0.0, 0.0, 0.0)
            for r in range(n):
                w = self._normal_walk(E, n, r)
                if w is not None:
                    nrm = tuple(w / np.sqrt(float(w @ w)))
                    break
            out.append(nrm)
        return out

    def _normal_walk(self, E, n, r):
        """normals_search from loop vertex r: the first edge product above the
        tolerance, or None."""
        for t in range(1, n):
            u = E[(r + t) % n]
            if 4.0 * float(u @ u) > self.tol:
                for s in range(t + 1, n):
                    w = np.cross(E[(r + s) % n], u)
                    if 16.0 * float(w @ w) > self.tol:
                        return w
                return None
        return None

    def face_perimeters(self):
        out = []
        for f in self.faces:
            P = self.verts[f[1]]
            out.append(float(np.linalg.norm(P - np.roll(P, -1, axis=0), axis=1).sum()))
        return out

    def surface_area(self):
        return float(sum(self.face_areas()))

    def total_edge_distance(self):
        return 0.5 * float(sum(self.face_perimeters()))   # every edge bounds two faces

    def vertex_orders(self):
        cnt = np.zeros(len(self.verts), np.int64)
        for f in self.faces:
            cnt[f[1]] += 1
        return [int(c) for c in cnt]

    def number_of_edges(self):
        return sum(self.vertex_orders()) // 2

    def face_freq_table(self):
        orders = self.face_orders()
        v = [0] * (max(orders) + 1 if orders else 0)
        for o in orders:
            v[o] += 1
        return v


class _ContainerBase:
    """Shared implementation of the four reference container classes."""

    _kind = None

    def __init__(self, kind, geom, grid, periodic, mode="mixed"):
        self._lib = load_library()
        self._h = ctypes.c_void_p()
        g = (ctypes.c_double * 6)(*[float(v) for v in geom])
        gr = (ctypes.c_int * 3)(*[int(v) for v in grid])
        pe = (ctypes.c_int * 3)(*[1 if p else 0 for p in periodic])
        _check(self._lib.vgpu_container_create(ctypes.byref(self._h), kind, g, gr, pe))
        t = ctypes.c_double(0.0)
        _check(self._lib.vgpu_get_tolerance(self._h, ctypes.byref(t)))
        self.tol = t.value
        self.kind = kind
        self.geom = tuple(float(v) for v in geom)
        self.grid = tuple(int(v) for v in grid)
        self.periodic = tuple(bool(p) for p in periodic)
        self.mode = mode
        self._pending_ids = []
        self._pending_xyzr = []
        self._n_put = 0
        self._dirty = True
        self._dev_keep = None
        self._polytopes = False

    def set_polytopes(self, on=True):
        """Keep every cell's polytope (vertices, face loops) from the next
        compute on (VGPU_OUTPUT_POLYTOPES): what voronoicell's vertex and face
        queries and the print_custom fields %p %P %o %g %E %e %F %A %a %f %t %l
        need."""
        self._polytopes = bool(on)
        _check(self._lib.vgpu_set_output(self._h, VGPU_OUTPUT_POLYTOPES if on else 0))
        self._dirty = True

    def __del__(self):
        try:
            if self._h:
                self._lib.vgpu_container_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    # ---- put(): src/container.cc:90-111, src/container_prd.cc:94-119
    def _put(self, n, x, y, z, r):
        self._pending_ids.append(int(n))
        self._pending_xyzr.extend((float(x), float(y), float(z), float(r)))
        self._dirty = True

    def _flush_pending(self):
        if self._pending_ids:
            ids = np.asarray(self._pending_ids, dtype=np.int32)
            xyzr = np.asarray(self._pending_xyzr, dtype=np.float64)
            _check(self._lib.vgpu_put(self._h, len(ids), _ptr(ids), _ptr(xyzr)))
            self._count_put(len(ids))
            self._pending_ids = []
            self._pending_xyzr = []

    def _count_put(self, n):
        if self._dev_keep is not None:   # a host put() replaces device-resident input
            self._dev_keep = None
            self._n_put = 0
        self._n_put += int(n)

    def put_array(self, ids, xyz, r=None):
        """Vectorised put(): ids (n,), xyz (n,3), optional radii (n,)."""
        self._flush_pending()
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        xyz = np.asarray(xyz, dtype=np.float64)
        n = len(ids)
        xyzr = np.empty((n, 4), dtype=np.float64)
        xyzr[:, :3] = xyz
        xyzr[:, 3] = 0.5 if r is None else r
        _check(self._lib.vgpu_put(self._h, n, _ptr(ids), _ptr(xyzr)))
        self._count_put(n)
        self._dirty = True

    # ---- walls: src/container.hh:56-103 (wall_list), src/wall.hh:25-130
    def add_wall(self, w):
        """Adds a wall (wall_sphere, wall_plane, wall_cylinder, wall_cone);
        it cuts every cell from the next compute on."""
        params = np.zeros(7, np.float64)
        params[:len(w.params)] = w.params
        _check(self._lib.vgpu_add_wall(self._h, w.type, _ptr(params), int(w.w_id)))
        self._dirty = True

    def clear_walls(self):
        _check(self._lib.vgpu_clear_walls(self._h))
        self._dirty = True

    def point_inside_walls(self, x, y, z):
        out = ctypes.c_int(0)
        _check(self._lib.vgpu_point_inside_walls(self._h, float(x), float(y), float(z), ctypes.byref(out)))
        return bool(out.value)

    def point_inside(self, x, y, z):
        """container_base::point_inside (src/container.cc:484-487): inside
        the box on every axis, periodic or not, and inside every wall
        (container and container_poly)."""
        if self.kind not in (KIND_CONTAINER, KIND_CONTAINER_POLY):
            raise AttributeError("point_inside belongs to container and container_poly")
        g = self.geom
        if x < g[0] or x > g[1] or y < g[2] or y > g[3] or z < g[4] or z > g[5]:
            return False
        return self.point_inside_walls(x, y, z)

    # ---- import: src/container.cc:333-376, src/container_prd.cc:400-433
    def import_file(self, f):
        """container::import: entries "id x y z" ("id x y z r" for the
        radical kinds) read as whitespace-separated numbers until the end of
        the file (a file name or an open text file); an incomplete or
        malformed entry is the reference's "File import error"."""
        text = open(f).read() if isinstance(f, (str, bytes, os.PathLike)) else f.read()
        poly = self.kind in (KIND_CONTAINER_POLY, KIND_PERIODIC_POLY)
        k = 5 if poly else 4
        tok = text.split()
        if len(tok) % k:
            raise VoroError(1, "File import error")
        try:
            ids = np.array([int(t) for t in tok[0::k]], dtype=np.int32)
            vals = np.array([[float(t) for t in tok[i + 1:i + k]] for i in range(0, len(tok), k)],
                            dtype=np.float64).reshape(-1, k - 1)
        except ValueError:
            raise VoroError(1, "File import error") from None
        if len(ids):
            self.put_array(ids, vals[:, :3], vals[:, 3] if poly else None)

    def put_xyzr(self, ids, xyzr):
        """put() of int32 ids (n,) and float64 xyzr (n,4) without a host copy."""
        self._flush_pending()
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        xyzr = np.ascontiguousarray(xyzr, dtype=np.float64)
        assert xyzr.shape == (len(ids), 4)
        _check(self._lib.vgpu_put(self._h, len(ids), _ptr(ids), _ptr(xyzr)))
        self._count_put(len(ids))
        self._dirty = True

    def put_device(self, n, dev_ids_ptr, dev_xyzr_ptr, keepalive=None):
        """Points the container at particle arrays already in device memory
        (int32 ids, float64 (n,4) xyzr); ``keepalive`` holds their owner."""
        self._pending_ids, self._pending_xyzr = [], []
        _check(self._lib.vgpu_put_device(self._h, int(n), ctypes.c_void_p(dev_ids_ptr),
                                         ctypes.c_void_p(dev_xyzr_ptr)))
        self._n_put = int(n)
        self._dev_keep = keepalive if keepalive is not None else ()
        self._dirty = True

    def clear(self):
        """container::clear (src/container.cc:385-387)."""
        self._pending_ids, self._pending_xyzr = [], []
        self._dev_keep = None
        _check(self._lib.vgpu_clear(self._h))
        self._n_put = 0
        self._dirty = True

    def autotune(self, mode=None, cache=False):
        """The engine's autotuner on this container's particles: engine-grid
        density, warps per CTA and cells per chunk, fastest tuple kept (and,
        with ``cache``, read from / written to the per-GPU cache file);
        returns (tuning dict, ms per compute)."""
        self._flush_pending()
        t, ms = Tuning(), ctypes.c_double(0)
        flags = (VGPU_TUNE_USE_CACHE | VGPU_TUNE_WRITE_CACHE) if cache else 0
        _check(self._lib.vgpu_autotune_ex(self._h, self._mode_code(mode), flags, ctypes.byref(t), ctypes.byref(ms)))
        self._dirty = False
        return t.as_dict(), ms.value

    def set_tuning(self, particles_per_block=0.0, warps_per_cta=0, cells_per_chunk=0, fp64_fallback=0.0):
        """vgpu_set_tuning_ex: zero keeps a setting."""
        t = Tuning(float(particles_per_block), int(warps_per_cta), int(cells_per_chunk), float(fp64_fallback))
        _check(self._lib.vgpu_set_tuning_ex(self._h, ctypes.byref(t)))
        self._dirty = True

    def tuning(self):
        t = Tuning()
        _check(self._lib.vgpu_get_tuning(self._h, ctypes.byref(t)))
        return t.as_dict()

    def set_ghost_depth(self, spacings=0.0):
        """Sheared periodic boxes: depth of the image layers a compute stores
        first, in mean particle spacings (0: default 8; negative: always the
        reference's depth).  Results never depend on it."""
        _check(self._lib.vgpu_set_ghost_depth(self._h, float(spacings)))
        self._dirty = True

    def _mode_code(self, mode):
        mode = mode or self.mode
        return VGPU_FP64 if mode == "fp64" else VGPU_MIXED

    # ---- compute_all_cells: src/container.cc:438-453
    def compute_all_cells(self, mode=None):
        self._flush_pending()
        rc = self._lib.vgpu_compute(self._h, self._mode_code(mode))
        if rc in (VGPU_OK, VGPU_ERR_CAPACITY):
            # a capacity failure still leaves results: the cells that failed
            # carry VGPU_CELL_FAILED and a reason, the others are complete
            self._dirty = False
        _check(rc)

    def set_fp64_fallback(self, fraction=0.25):
        """Mixed computes of large containers: the fraction of a sample of
        cells needing FP64 above which the whole container runs on the FP64
        engine (>= 1: never)."""
        _check(self._lib.vgpu_set_fp64_fallback(self._h, float(fraction)))
        self._dirty = True

    def set_record_budget(self, nbytes=0):
        """Record-store budget of one compute in bytes (0: the default).  Cells
        whose records do not fit fail with VGPU_FAIL_RECORDS and the compute
        raises VGPU_ERR_CAPACITY; the rest are complete."""
        _check(self._lib.vgpu_set_record_budget(self._h, int(nbytes)))
        self._dirty = True

    def _ensure(self):
        if self._dirty:
            self.compute_all_cells()

    # ---- sum_cell_volumes: src/container.cc:459-477
    def sum_cell_volumes(self):
        self._ensure()
        out = ctypes.c_double(0)
        _check(self._lib.vgpu_sum_cell_volumes(self._h, ctypes.byref(out)))
        return out.value

    # ---- find_voronoi_cell: src/container.cc:237-301, src/container_prd.cc:303-359
    def find_voronoi_cells(self, points):
        """Point location for many points (n, 3): (found, pid, r) with found
        a bool array, pid the IDs and r (n, 3) the particles' positions (the
        periodic image nearest each point), as the reference's
        find_voronoi_cell returns them point by point."""
        self._flush_pending()
        q = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = len(q)
        found = np.zeros(n, np.int32)
        pid = np.zeros(n, np.int32)
        r = np.zeros((n, 3), np.float64)
        _check(self._lib.vgpu_find_voronoi_cells(self._h, n, _ptr(q), _ptr(pid), _ptr(r), _ptr(found)))
        return found != 0, pid, r

    # ---- compute_ghost_cell: src/container.hh:487-498, 710-721; src/container_prd.hh:414-422, 635-644
    def compute_ghost_cells(self, xyz, r=None):
        """The cells of ghost particles at the rows of xyz (radii r for the
        radical kinds), each as if it alone were added to the container;
        returns a GhostResults (vol, cen, nf, nv, maxr2, flags, ok,
        neighbors(k), and polytope(k) when set_polytopes is on)."""
        self._flush_pending()
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = len(xyz)
        xyzr = np.zeros((n, 4), np.float64)
        xyzr[:, :3] = xyz
        xyzr[:, 3] = 0.5 if r is None else r
        _check(self._lib.vgpu_compute_ghost_cells(self._h, VGPU_FP64 if self.mode == "fp64" else VGPU_MIXED, n,
                                                  _ptr(xyzr)))
        vol = np.zeros(n); cen = np.zeros((n, 3)); nf = np.zeros(n, np.int32); nv = np.zeros(n, np.int32)
        mr2 = np.zeros(n); fl = np.zeros(n, np.int32)
        _check(self._lib.vgpu_get_ghost_cells(self._h, _ptr(vol), _ptr(cen), _ptr(nf), _ptr(nv), _ptr(mr2),
                                              _ptr(fl)))
        res = CellResults(np.full(n, -1, np.int32), xyz.copy(), vol, cen, nf, nv, mr2, fl)
        off = np.zeros(n + 1, np.int64)
        _check(self._lib.vgpu_get_ghost_neighbors(self._h, _ptr(off), None))
        nb = np.zeros(max(int(off[-1]), 1), np.int32)
        _check(self._lib.vgpu_get_ghost_neighbors(self._h, _ptr(off), _ptr(nb)))
        res.nb, res.nb_off = nb[:int(off[-1])], off
        if self._polytopes:
            poff = np.zeros(n + 1, np.int64)
            _check(self._lib.vgpu_get_ghost_polytopes(self._h, _ptr(poff), None))
            data = np.zeros(max(int(poff[-1]), 1))
            _check(self._lib.vgpu_get_ghost_polytopes(self._h, _ptr(poff), _ptr(data)))
            res.poly_off, res.poly_data, res.poly_tol = poff, data, self.tol
        return res

    def find_voronoi_cell(self, x, y, z):
        """The reference's signature: (found, rx, ry, rz, pid)."""
        f, pid, r = self.find_voronoi_cells([[x, y, z]])
        return bool(f[0]), float(r[0, 0]), float(r[0, 1]), float(r[0, 2]), int(pid[0])

    def stats(self):
        st = Stats()
        _check(self._lib.vgpu_get_stats(self._h, ctypes.byref(st)))
        return st.as_dict()

    def phase_cycles(self):
        """Per-phase clock totals (diagnostics builds only; zeros otherwise)."""
        out = (ctypes.c_double * 8)()
        _check(self._lib.vgpu_phase_cycles(self._h, out))
        names = ["init", "gather", "sort", "test", "cut", "finish", "gather_flush", "kernel"]
        return dict(zip(names, list(out)))

    def phase_counts(self):
        """Per-compute event counts of the cell kernel (diagnostics builds only)."""
        out = (ctypes.c_double * 8)()
        _check(self._lib.vgpu_phase_counts(self._h, out))
        names = ["flushes", "sorts64", "block_passes", "cand_passes", "cands_kept", "new_vertices",
                 "segments", "cells_run"]
        return dict(zip(names, list(out)))

    def input_rows(self):
        """particle_order / c_loop_order (src/c_loops.hh:268-317): for each
        particle put since the last clear, in put order, its row in cells(),
        or -1 where put() dropped it."""
        self._flush_pending()
        self._ensure()
        rows = np.empty(self._n_put, np.int32)
        _check(self._lib.vgpu_get_input_rows(self._h, _ptr(rows)))
        return rows

    def total_particles(self):
        self._ensure()
        n = ctypes.c_int64(0)
        _check(self._lib.vgpu_num_cells(self._h, ctypes.byref(n)))
        return n.value

    def cells(self, neighbors=True, out=None, alloc=None):
        """All per-cell results (CellResults) from the last compute.
        ``out``: the CellResults of an earlier call, whose arrays are reused
        when they fit; ``alloc(shape, dtype)``: allocator for new arrays (for
        example pinned host memory, which the device copies faster)."""
        self._ensure()
        n = self.total_particles()
        alloc = alloc or (lambda shape, dt: np.empty(shape, dt))

        def get(name, shape, dt, at_least=False):
            a = getattr(out, "_buf_" + name, None) if out is not None else None
            size = int(np.prod(shape))
            if a is not None and a.dtype == np.dtype(dt) and (a.size >= size if at_least else a.shape == shape):
                return a
            return alloc(shape, dt)

        ids = get("ids", (n,), np.int32); pos = get("pos", (n, 3), np.float64); vol = get("vol", (n,), np.float64)
        cen = get("cen", (n, 3), np.float64); nf = get("nf", (n,), np.int32); nv = get("nv", (n,), np.int32)
        mr2 = get("mr2", (n,), np.float64); fl = get("fl", (n,), np.int32)
        _check(self._lib.vgpu_get_cells(self._h, _ptr(ids), _ptr(pos), _ptr(vol), _ptr(cen), _ptr(nf),
                                        _ptr(nv), _ptr(mr2), _ptr(fl)))
        res = CellResults(ids, pos, vol, cen, nf, nv, mr2, fl)
        rad = get("rad", (n,), np.float64)
        _check(self._lib.vgpu_get_radii(self._h, _ptr(rad)))
        res.rad = rad
        for name, a in (("ids", ids), ("pos", pos), ("vol", vol), ("cen", cen), ("nf", nf), ("nv", nv),
                        ("mr2", mr2), ("fl", fl), ("rad", rad)):
            setattr(res, "_buf_" + name, a)
        if neighbors:
            tot = ctypes.c_int64(0)
            _check(self._lib.vgpu_num_neighbors(self._h, ctypes.byref(tot)))
            off = get("nb_off", (n + 1,), np.int64)
            nbuf = get("nb", (max(tot.value, 1),), np.int32, at_least=True)
            _check(self._lib.vgpu_get_neighbors(self._h, _ptr(off), _ptr(nbuf)))
            res.nb, res.nb_off = nbuf[:tot.value], off
            res._buf_nb, res._buf_nb_off = nbuf, off
        if self._polytopes:
            poff = np.zeros(n + 1, np.int64)
            _check(self._lib.vgpu_get_polytopes(self._h, _ptr(poff), None))
            data = np.zeros(max(int(poff[-1]), 1))
            _check(self._lib.vgpu_get_polytopes(self._h, _ptr(poff), _ptr(data)))
            res.poly_off, res.poly_data, res.poly_tol = poff, data, self.tol
        return res

    # ---- print_custom: src/container.hh:434-451, src/cell.cc:2485-2558
    def print_custom(self, fmt, fp=None):
        """Writes one line per computed cell with the reference's %-fields.
        ``fp`` is a file object, a filename, or None (stdout).  Fields that
        need the polytope switch its output on and recompute."""
        if _needs_polytope(fmt) and not self._polytopes:
            self.set_polytopes(True)
        res = self.cells(neighbors=("%n" in fmt))
        close = False
        if fp is None:
            fp = sys.stdout
        elif isinstance(fp, (str, os.PathLike)):
            fp = open(fp, "w")
            close = True
        try:
            poly = self.kind in (KIND_CONTAINER_POLY, KIND_PERIODIC_POLY)
            radius = (lambda k: float(res.rad[k]) if poly else 0.5)
            for k in range(len(res)):
                if not res.ok[k]:
                    continue
                fp.write(_format_custom(fmt, res, k, radius) + "\n")
        finally:
            if close:
                fp.close()


_POLY_FIELDS = "pPoEeFAaftl"


def _needs_polytope(fmt):
    i = 0
    while i < len(fmt) - 1:
        if fmt[i] == "%":
            if fmt[i + 1] in _POLY_FIELDS:
                return True
            i += 2
        else:
            i += 1
    return False


def _g(v):
    return "%g" % v


def _poly_field(f, c, x, y, z):
    """A polytope field of output_custom (src/cell.cc:2485-2558), formatted as
    the reference's printers (src/common.cc:37-136)."""
    if f == "p":
        return " ".join("(%g,%g,%g)" % tuple(v) for v in c.verts)
    if f == "P":
        return " ".join("(%g,%g,%g)" % (x + v[0], y + v[1], z + v[2]) for v in c.verts)
    if f == "o":
        return " ".join(str(o) for o in c.vertex_orders())
    if f == "E":
        return _g(c.total_edge_distance())
    if f == "e":
        return " ".join(_g(v) for v in c.face_perimeters())
    if f == "F":
        return _g(c.surface_area())
    if f == "A":
        return " ".join(str(v) for v in c.face_freq_table())
    if f == "a":
        return " ".join(str(v) for v in c.face_orders())
    if f == "f":
        return " ".join(_g(v) for v in c.face_areas())
    if f == "t":
        return " ".join("(" + ",".join(str(i) for i in loop) + ")" for loop in c.face_vertices())
    if f == "l":
        return " ".join("(%g,%g,%g)" % n for n in c.normals())
    raise ValueError(f)


def _vec(v):
    return " ".join(str(int(x)) for x in v)


def _format_custom(fmt, res, k, radius):
    out = []
    i = 0
    n = len(fmt)
    while i < n:
        ch = fmt[i]
        if ch != "%":
            out.append(ch)
            i += 1
            continue
        i += 1
        if i >= n:
            break
        f = fmt[i]
        x, y, z = res.pos[k]
        if f == "i":
            out.append("%d" % res.ids[k])
        elif f == "x":
            out.append("%g" % x)
        elif f == "y":
            out.append("%g" % y)
        elif f == "z":
            out.append("%g" % z)
        elif f == "q":
            out.append("%g %g %g" % (x, y, z))
        elif f == "r":
            out.append("%g" % radius(k))
        elif f == "w":
            out.append("%d" % res.nv[k])
        elif f == "o":
            out.append(_poly_field("o", res.polytope(k), x, y, z))
        elif f == "m":
            out.append("%g" % res.maxr2[k])
        elif f == "g":   # Euler's relation: E = V + F - 2 for vertices of any order
            out.append("%d" % (int(res.nv[k]) + int(res.nf[k]) - 2))
        elif f == "s":
            out.append("%d" % res.nf[k])
        elif f == "n":
            out.append(_vec(res.neighbors(k)))
        elif f == "v":
            out.append("%g" % res.vol[k])
        elif f == "c":
            out.append("%g %g %g" % tuple(res.cen[k]))
        elif f == "C":
            cx, cy, cz = res.cen[k]
            out.append("%g %g %g" % (x + cx, y + cy, z + cz))
        elif f in "pPEeFAaftl":
            out.append(_poly_field(f, res.polytope(k), x, y, z))
        else:
            out.append("%" + f)
        i += 1
    return "".join(out)


class container(_ContainerBase):
    """container(ax,bx,ay,by,az,bz,nx,ny,nz,xperiodic,yperiodic,zperiodic,init_mem)
    (src/container.hh:289-291)."""

    def __init__(self, ax, bx, ay, by, az, bz, nx, ny, nz, xperiodic, yperiodic, zperiodic, init_mem=8,
                 mode="mixed"):
        super().__init__(KIND_CONTAINER, (ax, bx, ay, by, az, bz), (nx, ny, nz),
                         (xperiodic, yperiodic, zperiodic), mode)

    def put(self, n, x, y, z):
        self._put(n, x, y, z, 0.5)


class container_poly(_ContainerBase):
    """container_poly(...) (src/container.hh:511-513): radical tessellation."""

    def __init__(self, ax, bx, ay, by, az, bz, nx, ny, nz, xperiodic, yperiodic, zperiodic, init_mem=8,
                 mode="mixed"):
        super().__init__(KIND_CONTAINER_POLY, (ax, bx, ay, by, az, bz), (nx, ny, nz),
                         (xperiodic, yperiodic, zperiodic), mode)

    def put(self, n, x, y, z, r):
        self._put(n, x, y, z, r)


class container_periodic(_ContainerBase):
    """container_periodic(bx,bxy,by,bxz,byz,bz,nx,ny,nz,init_mem)
    (src/container_prd.hh:213-216): the periodic parallelepiped of lattice
    vectors (bx,0,0), (bxy,by,0), (bxz,byz,bz); rectangular or sheared."""

    def __init__(self, bx, bxy, by, bxz, byz, bz, nx, ny, nz, init_mem=8, mode="mixed"):
        super().__init__(KIND_PERIODIC, (bx, bxy, by, bxz, byz, bz), (nx, ny, nz), (True, True, True), mode)

    def put(self, n, x, y, z):
        self._put(n, x, y, z, 0.5)


class container_periodic_poly(_ContainerBase):
    """container_periodic_poly (src/container_prd.hh:434-437)."""

    def __init__(self, bx, bxy, by, bxz, byz, bz, nx, ny, nz, init_mem=8, mode="mixed"):
        super().__init__(KIND_PERIODIC_POLY, (bx, bxy, by, bxz, byz, bz), (nx, ny, nz), (True, True, True), mode)

    def put(self, n, x, y, z, r):
        self._put(n, x, y, z, r)


class _Wall:
    type = None

    def __init__(self, *params, w_id=-99):
        self.params = [float(v) for v in params]
        self.w_id = int(w_id)


class wall_sphere(_Wall):
    """wall_sphere(xc, yc, zc, rc, w_id=-99) (src/wall.hh:25-45)."""
    type = 0


class wall_plane(_Wall):
    """wall_plane(xc, yc, zc, ac, w_id=-99) (src/wall.hh:47-68): x.c < ac inside."""
    type = 1


class wall_cylinder(_Wall):
    """wall_cylinder(xc, yc, zc, xa, ya, za, rc, w_id=-99) (src/wall.hh:70-95)."""
    type = 2


class wall_cone(_Wall):
    """wall_cone(xc, yc, zc, xa, ya, za, ang, w_id=-99) (src/wall.hh:97-130)."""
    type = 3


class batch:
    """Many containers computed together by one persistent launch of the cell
    engine (vgpu_batch_*).  Members keep their own results (``cells()``,
    ``sum_cell_volumes()``, ``print_custom``)."""

    def __init__(self, containers=()):
        self._lib = load_library()
        self._h = ctypes.c_void_p()
        _check(self._lib.vgpu_batch_create(ctypes.byref(self._h)))
        self.members = []
        for c in containers:
            self.add(c)

    def add(self, con):
        con._flush_pending()
        _check(self._lib.vgpu_batch_add(self._h, con._h))
        self.members.append(con)

    def compute_all_cells(self, mode="mixed"):
        for c in self.members:
            c._flush_pending()
        _check(self._lib.vgpu_batch_compute(self._h, VGPU_FP64 if mode == "fp64" else VGPU_MIXED))
        for c in self.members:
            c._dirty = False

    def stats(self):
        st = Stats()
        _check(self._lib.vgpu_batch_get_stats(self._h, ctypes.byref(st)))
        return st.as_dict()

    def set_record_budget(self, nbytes):
        """Budget of the record store (0 = default 8 GiB); larger batches run in waves."""
        _check(self._lib.vgpu_batch_set_record_budget(self._h, int(nbytes)))

    def waves(self):
        """Record-store waves of the last compute."""
        w = ctypes.c_int()
        _check(self._lib.vgpu_batch_waves(self._h, ctypes.byref(w)))
        return w.value

    def __del__(self):
        try:
            if self._h:
                self._lib.vgpu_batch_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass


def from_workload(w, mode="mixed"):
    """Builds a container from a ``voro_gb300.workloads`` dict and puts its particles."""
    kind = w["kind"]
    if kind == KIND_CONTAINER:
        c = container(*w["geom"], *w["grid"], *w["periodic"], 8, mode=mode)
    elif kind == KIND_CONTAINER_POLY:
        c = container_poly(*w["geom"], *w["grid"], *w["periodic"], 8, mode=mode)
    elif kind == KIND_PERIODIC:
        c = container_periodic(*w["geom"], *w["grid"], 8, mode=mode)
    else:
        c = container_periodic_poly(*w["geom"], *w["grid"], 8, mode=mode)
    for t, params, wid in w.get("walls") or []:
        c.add_wall([wall_sphere, wall_plane, wall_cylinder, wall_cone][t](*params[:4 if t < 2 else 7], w_id=wid))
    xyzr = w["xyzr"]
    c.put_array(w["ids"], xyzr[:, :3], xyzr[:, 3])
    return c
