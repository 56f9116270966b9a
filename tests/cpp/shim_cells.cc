// A reference-style program (container + c_loop_all + voronoicell_neighbor,
// as in the reference's examples) built against the drop-in header.
//
// usage: shim_cells <input> <records-out> [<print_custom format> <custom-out>
//                   [<queries> <queries-out>]]
// input: "kind ax bx ay by az bz nx ny nz xp yp zp n", optionally "walls k" and k
// lines "type id p0 .. p6" (0 sphere, 1 plane, 2 cylinder, 3 cone), then n
// lines "id x y z r"
// queries: lines "x y z r": find_voronoi_cell and compute_ghost_cell of each
#include <cstdio>
#include <cstring>
#include <vector>

#include "voro_gb300.hh"
using namespace voro;

template <class C>
static void dump(C &con, FILE *out) {
    c_loop_all vl(con);
    voronoicell_neighbor c(con);
    std::vector<int> neigh;
    double x, y, z, cx, cy, cz;
    if (vl.start()) do {
            if (con.compute_cell(c, vl)) {
                vl.pos(x, y, z);
                c.centroid(cx, cy, cz);
                c.neighbors(neigh);
                fprintf(out, "%d 1 %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d %d %.17g", vl.pid(), x, y, z,
                        c.volume(), cx, cy, cz, c.number_of_faces(), c.p, c.max_radius_squared());
                for (int v : neigh) fprintf(out, " %d", v);
                fputc('\n', out);
            } else {
                vl.pos(x, y, z);
                fprintf(out, "%d 0 %.17g %.17g %.17g\n", vl.pid(), x, y, z);
            }
        } while (vl.inc());
    fprintf(out, "sum %.17g\n", con.sum_cell_volumes());
}

static void put_one(container &con, int id, double x, double y, double z, double) { con.put(id, x, y, z); }
static void put_one(container_poly &con, int id, double x, double y, double z, double r) { con.put(id, x, y, z, r); }
static void put_one(container_periodic &con, int id, double x, double y, double z, double) { con.put(id, x, y, z); }
static void put_one(container_periodic_poly &con, int id, double x, double y, double z, double r) {
    con.put(id, x, y, z, r);
}

template <class C>
static int queries(C &con, const char *qpath, const char *opath) {
    FILE *q = fopen(qpath, "r");
    FILE *out = fopen(opath, "w");
    if (!q || !out) return 4;
    double x, y, z, r, rx, ry, rz, cx, cy, cz;
    int pid;
    voronoicell_neighbor c(con);
    std::vector<int> neigh;
    while (fscanf(q, "%lg %lg %lg %lg", &x, &y, &z, &r) == 4) {
        const bool f = con.find_voronoi_cell(x, y, z, rx, ry, rz, pid);
        fprintf(out, "find %d %d %.17g %.17g %.17g\n", f ? 1 : 0, f ? pid : -1, f ? rx : 0.0, f ? ry : 0.0,
                f ? rz : 0.0);
        const bool g = con.compute_ghost_cell(c, x, y, z, r);
        if (g) {
            c.centroid(cx, cy, cz);
            c.neighbors(neigh);
            fprintf(out, "ghost 1 %.17g %.17g %.17g %.17g %d %d", c.volume(), cx, cy, cz, c.number_of_faces(), c.p);
            for (int v : neigh) fprintf(out, " %d", v);
            fputc('\n', out);
        } else {
            fprintf(out, "ghost 0\n");
        }
    }
    fclose(q);
    fclose(out);
    return 0;
}

// the optional wall lines, added with the reference's wall classes
template <class C>
static void read_walls(C &con, FILE *in, std::vector<wall *> &owned) {
    const long at = ftell(in);
    char tag[16];
    int k = 0;
    if (fscanf(in, "%15s", tag) != 1 || strcmp(tag, "walls") != 0 || fscanf(in, "%d", &k) != 1) {
        fseek(in, at, SEEK_SET);
        return;
    }
    for (int i = 0; i < k; i++) {
        int t, id;
        double p[7];
        if (fscanf(in, "%d %d %lg %lg %lg %lg %lg %lg %lg", &t, &id, p, p + 1, p + 2, p + 3, p + 4, p + 5, p + 6) != 9)
            return;
        wall *w = t == 0   ? (wall *)new wall_sphere(p[0], p[1], p[2], p[3], id)
                  : t == 1 ? (wall *)new wall_plane(p[0], p[1], p[2], p[3], id)
                  : t == 2 ? (wall *)new wall_cylinder(p[0], p[1], p[2], p[3], p[4], p[5], p[6], id)
                           : (wall *)new wall_cone(p[0], p[1], p[2], p[3], p[4], p[5], p[6], id);
        owned.push_back(w);
        con.add_wall(w);
    }
}

template <class C>
static int run(C &con, FILE *in, int n, int argc, char **argv) {
    for (int k = 0; k < n; k++) {
        int id;
        double x, y, z, r;
        if (fscanf(in, "%d %lg %lg %lg %lg", &id, &x, &y, &z, &r) != 5) return 2;
        put_one(con, id, x, y, z, r);
    }
    FILE *out = fopen(argv[2], "w");
    if (!out) return 3;
    dump(con, out);
    fclose(out);
    if (argc > 4) con.print_custom(argv[3], argv[4]);
    if (argc > 6) return queries(con, argv[5], argv[6]);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 3) return 1;
    FILE *in = fopen(argv[1], "r");
    if (!in) return 1;
    int kind, nx, ny, nz, xp, yp, zp, n;
    double g[6];
    if (fscanf(in, "%d %lg %lg %lg %lg %lg %lg %d %d %d %d %d %d %d", &kind, g, g + 1, g + 2, g + 3, g + 4, g + 5, &nx,
               &ny, &nz, &xp, &yp, &zp, &n) != 14)
        return 1;
    int rc = 1;
    std::vector<wall *> owned;
    if (kind == 0) {
        container con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, xp, yp, zp, 8);
        read_walls(con, in, owned);
        rc = run(con, in, n, argc, argv);
    } else if (kind == 1) {
        container_poly con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, xp, yp, zp, 8);
        read_walls(con, in, owned);
        rc = run(con, in, n, argc, argv);
    } else if (kind == 2) {
        container_periodic con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, 8);
        rc = run(con, in, n, argc, argv);
    } else {
        container_periodic_poly con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, 8);
        rc = run(con, in, n, argc, argv);
    }
    for (wall *w : owned) delete w;
    fclose(in);
    return rc;
}
