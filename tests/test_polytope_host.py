"""Host-side polytope queries (voro_gb300.Polytope, the basis of the
print_custom fields %p %P %o %g %E %e %F %A %a %f %t %l and of the C++
header's voronoicell queries) against the reference's own values, on the
reference's polytopes: no GPU needed."""
import numpy as np
import pytest

import voro_gb300 as vg
from tests import _golden as G


@pytest.mark.parametrize("name", G.poly_names())
def test_polytope_queries_match_reference(name):
    cells, _, _ = G.load_poly(name)
    tol = G.reference_tol(G.load(name)[0])
    checked = 0
    for c in cells:
        if not c["ok"]:
            continue
        pt = vg.Polytope(c["verts"], [(f[0], f[4]) for f in c["faces"]], tol)
        areas = pt.face_areas()
        perims = pt.face_perimeters()
        normals = pt.normals()
        for (nb, area, perim, nrm, loop), a, p_, n in zip(c["faces"], areas, perims, normals):
            assert abs(a - area) <= 1e-12 * max(area, 1e-300) + 1e-14
            assert abs(p_ - perim) <= 1e-12 * perim
            # the zero normals of slivers included; a face whose outcome
            # depends on the loop's start vertex may differ (the reference's
            # own start gave zero, another start does not)
            if bool(np.any(nrm)) != bool(np.any(n)):
                assert not np.any(nrm) and G.normal_start_dependent(c["verts"], loop, tol), (n, nrm)
            else:
                assert np.allclose(n, nrm, atol=1e-9), (n, nrm)
        assert abs(pt.surface_area() - c["sa"]) <= 1e-12 * c["sa"]
        assert abs(pt.total_edge_distance() - c["ted"]) <= 1e-12 * c["ted"]
        assert pt.number_of_edges() == sum(pt.vertex_orders()) // 2
        assert sum(pt.face_freq_table()) == len(c["faces"])
        checked += 1
    assert checked > 0


def test_normals_follow_the_tolerance():
    # the z = 0 face of the unit cube, clockwise seen from below (outside)
    verts = np.array([[x, y, 0.0] for y in (0.0, 1.0) for x in (0.0, 1.0)])
    face = [(-5, [0, 1, 3, 2])]
    assert np.allclose(vg.Polytope(verts, face).normals()[0], (0.0, 0.0, -1.0))
    # in doubled coordinates the edges' squared lengths are 4 and their
    # products' 16: a tolerance of 5 (or 17) leaves no first edge, one of 3
    # keeps the normal
    assert vg.Polytope(verts, face, tol=5.0).normals()[0] == (0.0, 0.0, 0.0)
    assert vg.Polytope(verts, face, tol=17.0).normals()[0] == (0.0, 0.0, 0.0)
    assert np.allclose(vg.Polytope(verts, face, tol=3.0).normals()[0], (0.0, 0.0, -1.0))

