"""The point-location fixtures (the reference's find_voronoi_cell answers,
tests/golden/make_golden.py) checked against a brute-force nearest-cell
search in numpy: every found answer is a stored particle (an image of it
across periodic axes) at the smallest power distance |q - p|^2 - r^2 over
all particles and their images, and every 'not found' is a point outside a
non-periodic wall.  CPU only."""
import numpy as np
import pytest

from tests import _golden as G

PERIODIC_KINDS = (2, 3)
POLY_KINDS = (1, 3)


def _domain(z):
    g = np.asarray(z["geom"], float)
    if int(z["kind"]) in PERIODIC_KINDS:
        return np.zeros(3), np.array([g[0], g[2], g[5]]), np.ones(3, bool)
    return g[0::2], g[1::2], np.asarray(z["periodic"], bool)


@pytest.mark.parametrize("name", G.locate_names())
def test_locate_fixture_is_the_nearest_cell(name):
    w, z = G.load(name)
    q, found, pid, r = G.load_locate(name)
    lo, hi, per = _domain(z)
    L = hi - lo
    pos = z["pos"]                       # stored (remapped) positions, loop order
    ids = z["ids"]
    rad = (z["in_xyzr"][:, 3] if int(z["kind"]) in POLY_KINDS else np.zeros(len(z["in_ids"])))
    rad_of = dict(zip(z["in_ids"].tolist(), rad.tolist()))
    rads = np.array([rad_of[i] for i in ids.tolist()]) if len(ids) else np.zeros(0)
    shifts = np.array([[a, b, c] for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)], float)
    shifts = shifts[np.all((shifts == 0) | per, axis=1)]
    for i in range(len(q)):
        x = q[i].copy()
        inside = np.all(per | ((x >= lo) & (x < hi)))
        if not inside or len(ids) == 0:
            assert found[i] == 0, i
            continue
        assert found[i] == 1, i
        # the query in the domain, and its periodic frame
        k = np.where(per, np.floor((x - lo) / L), 0.0)
        xd = x - k * L
        cand = (pos[None, :, :] + shifts[:, None, :] * L) - xd
        d = (cand ** 2).sum(-1) - rads[None, :] ** 2
        best = d.min()
        # the answer: particle pid, at r = its image in the query's frame
        rr = r[i] - k * L
        j = np.nonzero(ids == pid[i])[0]
        assert len(j) == 1, i
        off = (rr - pos[j[0]]) / np.where(per, L, 1.0)
        assert np.allclose(off, np.round(off), atol=1e-9) and np.all((np.round(off) == 0) | per), i
        dr = ((rr - xd) ** 2).sum() - rads[j[0]] ** 2
        assert dr <= best + 1e-9 * max(1.0, abs(best)), (i, dr, best)
