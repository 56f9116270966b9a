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
    """Lower corner, lattice basis (rows: the periodic translations a, b, c;
    for a non-periodic axis its box length) and periodic flags."""
    g = np.asarray(z["geom"], float)
    if int(z["kind"]) in PERIODIC_KINDS:
        A = np.array([[g[0], 0, 0], [g[1], g[2], 0], [g[3], g[4], g[5]]])
        return np.zeros(3), A, np.ones(3, bool)
    return g[0::2], np.diag(g[1::2] - g[0::2]), np.asarray(z["periodic"], bool)


def _frame(x, lo, A, per):
    """The query remapped into the domain along the lattice vectors, z then
    y then x as the reference remaps, and its image counts."""
    x = x.copy()
    k = np.zeros(3)
    for ax in (2, 1, 0):
        if per[ax]:
            k[ax] = np.floor((x[ax] - lo[ax]) / A[ax, ax])
            x = x - k[ax] * A[ax]
    return x, k


@pytest.mark.parametrize("name", G.locate_names())
def test_locate_fixture_is_the_nearest_cell(name):
    w, z = G.load(name)
    q, found, pid, r = G.load_locate(name)
    lo, A, per = _domain(z)
    hi = lo + np.diag(A)
    pos = z["pos"]                       # stored (remapped) positions, loop order
    ids = z["ids"]
    rad = (z["in_xyzr"][:, 3] if int(z["kind"]) in POLY_KINDS else np.zeros(len(z["in_ids"])))
    rad_of = dict(zip(z["in_ids"].tolist(), rad.tolist()))
    rads = np.array([rad_of[i] for i in ids.tolist()]) if len(ids) else np.zeros(0)
    rng = range(-2, 3)
    coef = np.array([[a, b, c] for a in rng for b in rng for c in rng], float)
    coef = coef[np.all((coef == 0) | per, axis=1)]
    shifts = coef @ A
    Ainv = np.linalg.inv(A)
    for i in range(len(q)):
        x = q[i].copy()
        inside = np.all(per | ((x >= lo) & (x < hi)))
        if not inside or len(ids) == 0:
            assert found[i] == 0, i
            continue
        assert found[i] == 1, i
        # the query in the domain, and its periodic frame
        xd, k = _frame(x, lo, A, per)
        cand = (pos[None, :, :] + shifts[:, None, :]) - xd
        d = (cand ** 2).sum(-1) - rads[None, :] ** 2
        best = d.min()
        # the answer: particle pid, at r = an image of it in the query's frame
        rr = r[i] - k @ A
        j = np.nonzero(ids == pid[i])[0]
        assert len(j) == 1, i
        off = (rr - pos[j[0]]) @ Ainv
        assert np.allclose(off, np.round(off), atol=1e-9) and np.all((np.round(off) == 0) | per), i
        dr = ((rr - xd) ** 2).sum() - rads[j[0]] ** 2
        assert dr <= best + 1e-9 * max(1.0, abs(best)), (i, dr, best)
