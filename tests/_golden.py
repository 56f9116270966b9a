"""Loading and comparison helpers for the golden fixtures."""
import glob
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# Fixtures whose per-cell topology the engine does not reproduce, with the
# reason; their geometry is checked instead (test_gpu_parity.py).
KNOWN_LIMIT = {
    "edge_cubic_jitter_1e-12_216":
        "a lattice jittered at the scale of the reference's tolerance: which of the split "
        "vertices' tiny faces survive is decided inside the band, cell by cell (the reference's "
        "own neighbour lists are not symmetric there)",
}

# Fixtures whose volumes are determined only to u * kappa: vertices where two
# nearly parallel bisectors meet (a pair of particles 3e-9 apart seen from a
# third one: kappa about spacing / separation, 5e7 here), computed by the
# reference along its edges and by the engine from three planes.
CONDITIONING_TOL = {
    "edge_near_coincident_300": {"fp64": (1e-9, 1e-9), "mixed": (1e-7, 1e-7)},
}


# Fixtures with a cell beyond the engines' capacity (the 128-vertex engine's
# slots): the compute returns VGPU_ERR_CAPACITY with exactly these cells
# flagged VGPU_CELL_FAILED and this reason (bits 8-11), every other cell as
# the reference's.  A large radical particle among small ones: its cell of 84
# vertices and 44 faces needs more than 128 vertex slots while it is cut.
CAPACITY_LIMIT = {
    "edge_radical_deleted_300": {"ids": [1], "reason": 3},
}


def tolerance(name, mode, default):
    return CONDITIONING_TOL.get(name, {}).get(mode, default)


def names():
    """The per-cell record fixtures (poly_*.npz hold polytopes, see load_poly;
    locate_*.npz point-location answers, see load_locate; ghost_*.npz ghost
    cells, see load_ghost; normals_*.npz print_custom normals, see
    load_normals)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "*.npz"))
                  if not os.path.basename(p).startswith(("poly_", "locate_", "ghost_", "wall_", "cli_", "normals_")))


def normal_names():
    return sorted(os.path.basename(p)[8:-4] for p in glob.glob(os.path.join(HERE, "normals_*.npz")))


def load_normals(name):
    """The reference's print_custom text of fixture ``name`` for "%i %n %l"
    (format, text)."""
    with np.load(os.path.join(HERE, f"normals_{name}.npz")) as z:
        return str(z["custom_format"]), str(z["custom_text"])


def face_normals_by_neighbour(text):
    """Per particle ID of a "%i %n %l" print_custom text: its faces as
    (neighbour, (nx, ny, nz)) pairs, sorted."""
    out = {}
    for line in text.splitlines():
        f = line.split()
        if not f:
            continue
        pid = int(f[0])
        rest = f[1:]
        nf = len(rest) // 2   # nf neighbour IDs, then nf "(x,y,z)" normals
        nbs = [int(v) for v in rest[:nf]]
        nrms = []
        for tok in rest[nf:]:
            x, y, z = (float(v) for v in tok.strip("()").split(","))
            nrms.append((x, y, z))
        out[pid] = sorted(zip(nbs, nrms))
    return out


def wall_names():
    """Fixtures of containers with walls (the same records; load() adds the walls)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "wall_*.npz")))


def locate_names():
    return sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(HERE, "locate_*.npz")))


def ghost_names():
    return sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(HERE, "ghost_*.npz")))


def load_ghost(name):
    """Ghost particles of fixture ``name`` (n x 4: x, y, z, r) and the
    reference's compute_ghost_cell records (npz fields ok, vol, cen, nf, nv,
    mrs, nb, nb_off)."""
    with np.load(os.path.join(HERE, f"ghost_{name}.npz")) as f:
        z = {k: f[k] for k in f.files}
    return z["g"], z


def load_locate(name):
    """Query points of fixture ``name`` and the reference's find_voronoi_cell
    answers: (q, found, pid, r)."""
    z = np.load(os.path.join(HERE, f"locate_{name}.npz"))
    return z["q"], z["found"], z["pid"], z["r"]


def poly_names():
    return sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(HERE, "poly_*.npz")))


def load_poly(name):
    """The reference's polytopes of the first cells of fixture ``name`` (list
    of dicts: ok, verts, sa, ted, faces [(nb, area, perimeter, normal, loop)])
    and its print_custom text over every cell for the stored format."""
    z = np.load(os.path.join(HERE, f"poly_{name}.npz"))
    flat = z["flat"]
    cells = []
    i = 0
    while i < len(flat):
        ok, nv, nf, sa, ted = flat[i:i + 5]
        i += 5
        nv, nf = int(nv), int(nf)
        verts = flat[i:i + 3 * nv].reshape(nv, 3)
        i += 3 * nv
        faces = []
        for _ in range(nf):
            nb, m, area, perim, nx, ny, nz = flat[i:i + 7]
            i += 7
            m = int(m)
            faces.append((int(nb), float(area), float(perim), np.array([nx, ny, nz]), [int(v) for v in flat[i:i + m]]))
            i += m
        cells.append({"ok": bool(ok), "verts": verts, "sa": float(sa), "ted": float(ted), "faces": faces})
    return cells, str(z["custom_format"]), str(z["custom_text"])


def compare_custom_text(got, ref, rtol=2e-6, atol=1e-12):
    """Line-by-line, token-by-token comparison of print_custom outputs: tokens
    equal as text, or numbers equal to the last printed digit (%g prints six
    significant digits, so values within rounding of a boundary may differ in
    it)."""
    import re
    gl, rl = got.splitlines(), ref.splitlines()
    if len(gl) != len(rl):
        return [f"{len(gl)} lines vs reference {len(rl)}"]
    num = re.compile(r"[-+0-9.eE]+")
    errs = []
    for li, (a, b) in enumerate(zip(gl, rl)):
        if a == b:
            continue
        ta = re.split(r"([ (),])", a)
        tb = re.split(r"([ (),])", b)
        if len(ta) != len(tb):
            errs.append(f"line {li}: {a!r} vs {b!r}")
            continue
        for x, y in zip(ta, tb):
            if x == y:
                continue
            if num.fullmatch(x) and num.fullmatch(y):
                try:
                    fx, fy = float(x), float(y)
                except ValueError:
                    errs.append(f"line {li}: {x!r} vs {y!r}")
                    break
                if abs(fx - fy) <= max(rtol * max(abs(fx), abs(fy)), atol):
                    continue
            errs.append(f"line {li}: {x!r} vs {y!r} in {a!r} / {b!r}")
            break
        if len(errs) > 10:
            break
    return errs


def load(name):
    # every array read once (an NpzFile decompresses on each access)
    with np.load(os.path.join(HERE, name + ".npz")) as f:
        z = {k: f[k] for k in f.files}
    w = {
        "kind": int(z["kind"]),
        "geom": tuple(float(v) for v in z["geom"]),
        "grid": tuple(int(v) for v in z["grid"]),
        "periodic": tuple(bool(v) for v in z["periodic"]),
        "ids": z["in_ids"],
        "xyzr": z["in_xyzr"],
    }
    if "wall_type" in z:
        w["walls"] = [(int(t), [float(v) for v in p], int(i))
                      for t, p, i in zip(z["wall_type"], z["wall_params"], z["wall_id"])]
    return w, z


def reference_tol(w):
    """The reference cell's length tolerance for workload ``w``:
    10 * DBL_EPSILON * max_len_sq (src/cell.cc:26), max_len_sq by
    src/container.cc:34-35 or, for a rectangular periodic box, the unit
    cell's max_radius_squared in doubled coordinates (bx^2 + by^2 + bz^2)."""
    g = w["geom"]
    if w["kind"] in (0, 1):
        m = sum((g[2 * a + 1] - g[2 * a]) ** 2 * (0.25 if w["periodic"][a] else 1.0) for a in range(3))
    else:
        assert g[1] == g[3] == g[4] == 0.0, "sheared unit cells need the engine's unit-cell computation"
        m = g[0] ** 2 + g[2] ** 2 + g[5] ** 2
    return 10.0 * np.finfo(np.float64).eps * m


def normal_start_dependent(verts, loop, tol):
    """Whether the reference's normals_search (src/cell.cc:2108-2164) finds
    a normal for this face from some loop vertices and none from others: its
    answer then rests on its own vertex numbering."""
    P = np.asarray(verts)[loop]
    E = np.roll(P, -1, axis=0) - P
    n = len(loop)

    def found(r):
        for t in range(1, n):
            u = E[(r + t) % n]
            if 4.0 * (u @ u) > tol:
                return any(16.0 * float(np.sum(np.cross(E[(r + s) % n], u) ** 2)) > tol for s in range(t + 1, n))
        return False

    outcomes = {found(r) for r in range(n)}
    return len(outcomes) == 2


def box_volume(w):
    g = w["geom"]
    if w["kind"] in (0, 1):
        return (g[1] - g[0]) * (g[3] - g[2]) * (g[5] - g[4])
    return g[0] * g[2] * g[5]


def compare_cells(got, ref, vol_rtol, cen_rtol, label="", skip=None):
    """got: object with ids,pos,vol,cen,nf,nv,ok and neighbors(k) sorted;
    ref: the fixture arrays; skip: a mask of cells left out (the cells of a
    known capacity limit).  Returns a list of human-readable mismatches."""
    errs = []
    n = len(ref["ids"])
    if len(got.ids) != n:
        return [f"{label}: {len(got.ids)} cells vs reference {n}"]
    if not np.array_equal(got.ids, ref["ids"]):
        errs.append(f"{label}: loop order (ids) differs")
    if not np.array_equal(got.pos, ref["pos"]):
        errs.append(f"{label}: stored positions differ (max {np.abs(got.pos - ref['pos']).max():.3g})")
    ok_ref = ref["ok"] != 0
    ok_got = np.asarray(got.ok, dtype=bool)
    if skip is not None:
        ok_ref = ok_ref & ~skip
        ok_got = ok_got & ~skip
    if not np.array_equal(ok_got, ok_ref):
        errs.append(f"{label}: deleted-cell flags differ at {np.nonzero(ok_got != ok_ref)[0][:10]}")
    m = ok_ref & ok_got
    bad_nf = np.nonzero((got.nf != ref["nf"]) & m)[0]
    bad_nv = np.nonzero((got.nv != ref["nv"]) & m)[0]
    if len(bad_nf):
        errs.append(f"{label}: face counts differ at {len(bad_nf)} cells, e.g. {bad_nf[:5]}")
    if len(bad_nv):
        errs.append(f"{label}: vertex counts differ at {len(bad_nv)} cells, e.g. {bad_nv[:5]}")
    nbad = 0
    for k in np.nonzero(m)[0]:
        a = np.asarray(got.neighbors(k))
        b = ref["nb"][ref["nb_off"][k]:ref["nb_off"][k + 1]]
        if len(a) != len(b) or not np.array_equal(np.sort(a), b):
            nbad += 1
    if nbad:
        errs.append(f"{label}: neighbour lists differ at {nbad} cells")
    v = ref["vol"][m]
    rel = np.abs(got.vol[m] - v) / np.maximum(np.abs(v), 1e-300)
    if len(rel) and rel.max() > vol_rtol:
        errs.append(f"{label}: max relative volume error {rel.max():.3g} > {vol_rtol}")
    scale = np.cbrt(np.maximum(np.abs(v), 1e-300))[:, None]
    cerr = np.abs(got.cen[m] - ref["cen"][m]) / scale
    if len(cerr) and cerr.max() > cen_rtol:
        errs.append(f"{label}: max centroid error / cell size {cerr.max():.3g} > {cen_rtol}")
    return errs
