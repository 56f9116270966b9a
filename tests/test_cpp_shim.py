"""The C++ drop-in header (include/voro_gb300.hh): a reference-style program
(container / c_loop_all / voronoicell_neighbor / compute_cell / print_custom,
as the reference's examples are written) compiles against it and, on a GPU,
reproduces the reference's golden per-cell records and the Python API's
print_custom output."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_cells.cc")
LIBDIR = os.path.dirname(vg.library_path())


def _compile(tmp_path, extra=()):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    vg.load_library()  # builds libvorogpu.so if needed
    exe = str(tmp_path / "shim_cells")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT}/include", SRC,
           f"-L{LIBDIR}", "-lvorogpu", f"-Wl,-rpath,{LIBDIR}", "-o", exe, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _write_input(path, w):
    g, gr, per = w["geom"], w["grid"], w["periodic"]
    with open(path, "w") as f:
        f.write(f"{w['kind']} " + " ".join(repr(float(v)) for v in g) + " " + " ".join(str(v) for v in gr) + " " +
                " ".join(str(int(p)) for p in per) + f" {len(w['ids'])}\n")
        walls = w.get("walls") or []
        if walls:
            f.write(f"walls {len(walls)}\n")
            for t, p, wid in walls:
                pp = list(p) + [0.0] * (7 - len(p))
                f.write(f"{t} {wid} " + " ".join(repr(float(v)) for v in pp) + "\n")
        for i, (x, y, z, r) in zip(w["ids"], w["xyzr"]):
            f.write(f"{int(i)} {float(x)!r} {float(y)!r} {float(z)!r} {float(r)!r}\n")


class _Parsed:
    def __init__(self, path):
        ids, ok, pos, vol, cen, nf, nv, mrs, nbs = [], [], [], [], [], [], [], [], []
        self.sum = None
        for line in open(path):
            t = line.split()
            if t[0] == "sum":
                self.sum = float(t[1])
                continue
            ids.append(int(t[0]))
            ok.append(int(t[1]))
            pos.append([float(v) for v in t[2:5]])
            if t[1] == "1":
                vol.append(float(t[5])); cen.append([float(v) for v in t[6:9]])
                nf.append(int(t[9])); nv.append(int(t[10])); mrs.append(float(t[11]))
                nbs.append(np.sort(np.array([int(v) for v in t[12:]], np.int32)))
            else:
                vol.append(0.0); cen.append([0, 0, 0]); nf.append(0); nv.append(0); mrs.append(0.0)
                nbs.append(np.zeros(0, np.int32))
        self.ids = np.array(ids, np.int32)
        self.ok = np.array(ok, bool)
        self.pos = np.array(pos)
        self.vol = np.array(vol)
        self.cen = np.array(cen, float)
        self.nf = np.array(nf, np.int32)
        self.nv = np.array(nv, np.int32)
        self.mrs = np.array(mrs)
        self._nb = nbs

    def neighbors(self, k):
        return self._nb[k]


def test_shim_compiles(tmp_path):
    _compile(tmp_path)
    _compile(tmp_path, ["-DVORO_GB300_THROW"])


def test_shim_reports_errors_like_the_reference(tmp_path):
    """Without a GPU the engine's status reaches the program as the
    reference's fatal-error path: a 'voro++:' message and a VOROPP_* exit code."""
    try:
        if vg.device_count() > 0:
            pytest.skip("a GPU is present: the no-device path cannot be exercised")
    except vg.VoroError:
        pass
    exe = _compile(tmp_path)
    w, _ = G.load("unit_cube_1000")
    inp = tmp_path / "in.txt"
    _write_input(inp, w)
    r = subprocess.run([exe, str(inp), str(tmp_path / "out.txt")], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert r.stderr.startswith("voro++: container:")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["unit_cube_1000", "periodic_2000", "radical_1200", "periodic_poly_800",
                                  "sparse_dropped_40", "tric_dyadic_1500", "tric_poly_1000"])
def test_shim_matches_reference_records(gpu, tmp_path, name):
    exe = _compile(tmp_path)
    w, z = G.load(name)
    inp = tmp_path / "in.txt"
    _write_input(inp, w)
    out = tmp_path / "out.txt"
    custom = tmp_path / "custom.txt"
    fmt = "%i %q %r %v %s %w %g %m %c %C %n %% %"
    r = subprocess.run([exe, str(inp), str(out), fmt, str(custom)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = _Parsed(out)
    errs = G.compare_cells(got, z, 1e-10, 1e-10, label=f"shim/{name}")
    assert not errs, "\n".join(errs)
    m = got.ok
    assert np.allclose(got.mrs[m], z["mrs"][m], rtol=1e-10, atol=0)
    assert abs(got.sum - G.box_volume(w)) <= 1e-9 * G.box_volume(w)
    # print_custom from C++ and from the Python mirror agree character for character
    con = vg.from_workload(w, mode="mixed")
    py = tmp_path / "custom_py.txt"
    con.print_custom(fmt, str(py))
    assert open(custom).read() == open(py).read()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["radical_1200", "unit_cube_1000"])
def test_shim_polytope_fields(gpu, tmp_path, name):
    """print_custom's polytope fields from the C++ header agree with the
    Python mirror, and its numbering-independent fields with the reference."""
    exe = _compile(tmp_path)
    w, z = G.load(name)
    _, ref_fmt, ref_text = G.load_poly(name)
    inp = tmp_path / "in.txt"
    _write_input(inp, w)
    for fmt, ref in [("%i %p %P %o %g %E %e %F %A %a %f %t %l %n", None), (ref_fmt, ref_text)]:
        custom = tmp_path / "custom.txt"
        r = subprocess.run([exe, str(inp), str(tmp_path / "out.txt"), fmt, str(custom)], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
        got = open(custom).read()
        if ref is None:
            con = vg.from_workload(w, mode="mixed")
            py = tmp_path / "custom_py.txt"
            con.print_custom(fmt, str(py))
            # unit normals of faces with areas near 1e-12 are only resolved to ~1e-10
            errs = G.compare_custom_text(got, open(py).read(), atol=1e-9)
        else:
            errs = G.compare_custom_text(got, ref)
        assert not errs, "\n".join(errs[:10])


@pytest.mark.gpu
@pytest.mark.parametrize("name", G.wall_names())
def test_shim_walls_match_reference(gpu, tmp_path, name):
    """Walls added through the header's wall classes reproduce the reference's
    records for containers with walls."""
    exe = _compile(tmp_path)
    w, z = G.load(name)
    inp = tmp_path / "in.txt"
    _write_input(inp, w)
    out = tmp_path / "out.txt"
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    errs = G.compare_cells(_Parsed(out), z, 1e-10, 1e-10, label=f"shim/{name}")
    assert not errs, "\n".join(errs)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["unit_cube_1000", "periodic_poly_800"])
def test_shim_point_location_and_ghost_cells(gpu, tmp_path, name):
    """find_voronoi_cell and compute_ghost_cell through the C++ header give
    the reference's answers stored in the fixtures."""
    exe = _compile(tmp_path)
    w, _ = G.load(name)
    g, z = G.load_ghost(name)
    inp = tmp_path / "in.txt"
    _write_input(inp, w)
    qf = tmp_path / "q.txt"
    with open(qf, "w") as f:
        for x, y, zz, r in g[:60]:
            f.write(f"{float(x)!r} {float(y)!r} {float(zz)!r} {float(r)!r}\n")
    out = tmp_path / "q_out.txt"
    r = subprocess.run([exe, str(inp), str(tmp_path / "o.txt"), "%i", str(tmp_path / "c.txt"), str(qf), str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = open(out).read().splitlines()
    finds = [l.split() for l in lines if l.startswith("find")]
    ghosts = [l.split() for l in lines if l.startswith("ghost")]
    assert len(finds) == len(ghosts) == 60
    con = vg.from_workload(w, mode="mixed")
    f, pid, rr = con.find_voronoi_cells(g[:60, :3])
    for k, t in enumerate(finds):
        assert int(t[1]) == int(f[k])
        if f[k]:
            assert int(t[2]) == pid[k] and [float(v) for v in t[3:6]] == list(rr[k])
    for k, t in enumerate(ghosts):
        assert int(t[1]) == int(z["ok"][k]), k
        if z["ok"][k]:
            assert abs(float(t[2]) - z["vol"][k]) <= 1e-10 * z["vol"][k]
            assert int(t[6]) == z["nf"][k]
            nb = np.sort(np.array([int(v) for v in t[8:]], np.int32))
            assert np.array_equal(nb, z["nb"][z["nb_off"][k]:z["nb_off"][k + 1]])
