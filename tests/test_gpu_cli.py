"""The voro++ command-line utility on the GPU engine against the reference's
own utility (src/cmd_line.cc), whose outputs for the same particle files and
flags are the cli_*.npz fixtures (tests/golden/make_golden.py).

The .vol files must agree line by line: every token equal as text, or as a
number to the digit %g prints; a format's %n list (last field; the reference
lists a cell's neighbours in its own face order) is compared as a multiset.
The -v summary agrees line by line.  Drawings (-g, -y) hold the same edges:
the reference walks them in the order of its vertex tables, so gnuplot
segments and POV-Ray spheres and cylinders are compared as multisets (per
cell for POV-Ray), with coordinates compared to 1e-9 (%g prints rounding
noise of a coordinate that is zero in different ways)."""
import glob
import os
import re
import subprocess

import numpy as np
import pytest

from voro_gb300 import _build

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "cli_*.npz")))
NUM = re.compile(r"[-+0-9.eE]+")


def load(name):
    with np.load(os.path.join(HERE, name + ".npz")) as f:
        return {k: (f[k].tolist() if f[k].dtype.kind in "US" else f[k]) for k in f.files}


def same_token(a, b, rtol=2e-6, atol=1e-12):
    if a == b:
        return True
    if NUM.fullmatch(a) and NUM.fullmatch(b):
        try:
            fa, fb = float(a), float(b)
        except ValueError:
            return False
        return abs(fa - fb) <= max(rtol * max(abs(fa), abs(fb)), atol)
    return False


def nb_count(fmt, tokens):
    """Tokens of the trailing %n list: the %s value (the face count)."""
    width = {"%q": 3, "%c": 3, "%C": 3}
    pos = 0
    for f in fmt.split():
        if f == "%s":
            return int(tokens[pos])
        if f == "%A":
            raise AssertionError("%A before %s: its width varies")
        pos += width.get(f, 1)
    raise AssertionError("a format with %n must hold %s")


def compare_vol(got, ref, fmt):
    gl, rl = got.splitlines(), ref.splitlines()
    assert len(gl) == len(rl), f"{len(gl)} cells vs reference {len(rl)}"
    has_nb = fmt.rstrip().endswith("%n")
    for li, (a, b) in enumerate(zip(gl, rl)):
        ta, tb = a.split(), b.split()
        if has_nb:
            k = nb_count(fmt, tb)
            assert k == nb_count(fmt, ta), f"line {li}: {a!r} vs {b!r}"
            assert sorted(map(int, ta[len(ta) - k:])) == sorted(map(int, tb[len(tb) - k:])), f"line {li}"
            ta, tb = ta[:len(ta) - k], tb[:len(tb) - k]
        assert len(ta) == len(tb), f"line {li}: {a!r} vs {b!r}"
        for x, y in zip(ta, tb):
            assert same_token(x, y), f"line {li}: {x!r} vs {y!r} in {a!r} / {b!r}"


def run_cli(tmp_path, z):
    fn = str(tmp_path / "pts")
    open(fn, "w").write(z["input"])
    r = subprocess.run([_build.CLI] + list(z["args"]) + [fn], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return fn, r


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in NAMES if n != "cli_drawing"])
def test_cli_matches_reference(gpu, tmp_path, name):
    z = load(name)
    fn, r = run_cli(tmp_path, z)
    args = list(z["args"])
    fmt = args[args.index("-c") + 1] if "-c" in args else ("%i %q %v %r" if "-r" in args else "%i %q %v")
    compare_vol(open(fn + ".vol").read(), z["vol"], fmt)
    if "-v" in args:
        got = [ln for ln in r.stdout.splitlines() if not ln.startswith("Filename")]
        ref = [ln for ln in z["stdout"].splitlines() if not ln.startswith("Filename")]
        assert len(got) == len(ref)
        for a, b in zip(got, ref):
            ta, tb = a.split(), b.split()
            assert len(ta) == len(tb) and all(same_token(x, y) for x, y in zip(ta, tb)), (a, b)


def _point(text):
    """A printed point as a canonical tuple (1e-9 grid, no negative zero)."""
    return tuple(round(float(v), 9) + 0.0 for v in re.split(r"[ ,]+", text.strip()))


def gnu_segments(text):
    segs = []
    for chain in text.split("\n\n\n"):
        pts = [_point(ln) for ln in chain.splitlines() if ln.strip()]
        segs += [tuple(sorted((pts[i], pts[i + 1]))) for i in range(len(pts) - 1)]
    return sorted(segs)


def pov_cells(text):
    cells, cur = {}, None
    for ln in text.splitlines():
        if ln.startswith("// cell"):
            cur = int(ln.split()[2])
            cells[cur] = []
        elif ln.startswith("cylinder"):
            a, b = re.findall(r"<([^>]*)>", ln)
            cells[cur].append(("c",) + tuple(sorted((_point(a), _point(b)))))
        elif ln.startswith("sphere"):
            cells[cur].append(("s", _point(re.findall(r"<([^>]*)>", ln)[0])))
    return {k: sorted(v) for k, v in cells.items()}


@pytest.mark.gpu
def test_cli_drawings_hold_the_reference_edges(gpu, tmp_path):
    z = load("cli_drawing")
    fn, _ = run_cli(tmp_path, z)
    assert gnu_segments(open(fn + ".gnu").read()) == gnu_segments(z["gnu"])
    assert open(fn + "_p.pov").read() == z["povp"]
    assert pov_cells(open(fn + "_v.pov").read()) == pov_cells(z["povv"])


def test_cli_usage_and_errors_match_the_reference():
    """Arguments only: the utility stops before it touches a GPU."""
    exe = _build.CLI
    if not os.path.exists(exe):
        pytest.skip("voro++ not built")
    r = subprocess.run([exe, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "Syntax: voro++ [options]" in r.stdout
    r = subprocess.run([exe, "-hc"], capture_output=True, text=True)
    assert r.returncode == 0 and "%n A list of neighboring particle" in r.stdout
    r = subprocess.run([exe, "-x"], capture_output=True, text=True)
    assert r.returncode == 4 and "Unrecognized command-line options" in r.stderr   # VOROPP_CMD_LINE_ERROR
    r = subprocess.run([exe, "0", "1", "0", "1", "0"], capture_output=True, text=True)
    assert r.returncode == 4
    r = subprocess.run([exe, "-l", "0.1", "-n", "2", "2", "2", "0", "1", "0", "1", "0", "1", "f"],
                       capture_output=True, text=True)
    assert r.returncode == 4 and "Conflicting options" in r.stderr
    r = subprocess.run([exe, "0", "1", "1", "0", "0", "1", "f"], capture_output=True, text=True)
    assert r.returncode == 4 and "Minimum y coordinate exceeds maximum y coordinate" in r.stderr
    r = subprocess.run([exe, "-m", "0", "0", "1", "0", "1", "0", "1", "f"], capture_output=True, text=True)
    assert r.returncode == 4 and "memory allocation must be positive" in r.stderr
    r = subprocess.run([exe, "-n", "1000", "1000", "1000", "0", "1", "0", "1", "0", "1", "f"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "exceeds the maximum allowed" in r.stderr   # VOROPP_MEMORY_ERROR
