// A reference-style program (container + c_loop_all + voronoicell_neighbor,
// as in the reference's examples) built against the drop-in header.
//
// usage: shim_cells <input> <records-out> [<print_custom format> <custom-out>]
// input: "kind ax bx ay by az bz nx ny nz xp yp zp n" then n lines "id x y z r"
#include <cstdio>
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
    if (kind == 0) {
        container con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, xp, yp, zp, 8);
        rc = run(con, in, n, argc, argv);
    } else if (kind == 1) {
        container_poly con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, xp, yp, zp, 8);
        rc = run(con, in, n, argc, argv);
    } else if (kind == 2) {
        container_periodic con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, 8);
        rc = run(con, in, n, argc, argv);
    } else {
        container_periodic_poly con(g[0], g[1], g[2], g[3], g[4], g[5], nx, ny, nz, 8);
        rc = run(con, in, n, argc, argv);
    }
    fclose(in);
    return rc;
}
