// Test infrastructure only: a C-ABI driver around the unmodified reference
// library (Voro++), compiled from the reference's own sources by
// oracle/Makefile into oracle/_ref/.  Nothing in the product links it; the
// tests use it to pin the oracle port and to generate golden fixtures.
//
// Container kinds mirror the reference classes:
//   0 container            (src/container.hh:289-483)
//   1 container_poly       (src/container.hh:511-705)
//   2 container_periodic   (src/container_prd.hh:213-432)
//   3 container_periodic_poly (src/container_prd.hh:434-655)
// Per-cell records follow the reference's own loop order: c_loop_all
// (src/c_loops.hh:165-210) or c_loop_all_periodic (src/c_loops.hh:325-393).
#include <algorithm>
#include <chrono>
#include <type_traits>
#include <vector>
#include "voro++.hh"

using namespace voro;

namespace {

struct rec_sink {
    int cap;
    int n;
    int *id;
    double *pos, *vol, *cen, *mrs;
    int *nf, *nv, *ok;
    int *nb;
    long nb_cap, nb_used;
    long *nb_off;
    int overflow;
};

template <class con_t, class loop_t>
void run_cells(con_t &con, loop_t &vl, rec_sink &s) {
    voronoicell_neighbor c(con);
    std::vector<int> v;
    s.n = 0;
    s.nb_used = 0;
    if (!vl.start()) { if (s.nb_off) s.nb_off[0] = 0; return; }
    do {
        if (s.n >= s.cap) { s.overflow = 1; return; }
        int k = s.n++;
        double x, y, z, r;
        int pid;
        vl.pos(pid, x, y, z, r);
        s.id[k] = pid;
        s.pos[3 * k] = x; s.pos[3 * k + 1] = y; s.pos[3 * k + 2] = z;
        if (s.nb_off) s.nb_off[k] = s.nb_used;
        bool ok = con.compute_cell(c, vl);
        s.ok[k] = ok ? 1 : 0;
        if (ok) {
            double cx, cy, cz;
            s.vol[k] = c.volume();
            c.centroid(cx, cy, cz);
            s.cen[3 * k] = cx; s.cen[3 * k + 1] = cy; s.cen[3 * k + 2] = cz;
            s.nf[k] = c.number_of_faces();
            s.nv[k] = c.p;
            s.mrs[k] = c.max_radius_squared();
            c.neighbors(v);
            for (size_t j = 0; j < v.size(); j++) {
                if (s.nb_used >= s.nb_cap) { s.overflow = 1; return; }
                s.nb[s.nb_used++] = v[j];
            }
        } else {
            s.vol[k] = 0; s.cen[3 * k] = s.cen[3 * k + 1] = s.cen[3 * k + 2] = 0;
            s.nf[k] = 0; s.nv[k] = 0; s.mrs[k] = 0;
        }
    } while (vl.inc());
    if (s.nb_off) s.nb_off[s.n] = s.nb_used;
}

// Walls to add to the next containers of kinds 0 and 1 (ref_set_walls): type
// (0 sphere, 1 plane, 2 cylinder, 3 cone), 7 parameters, ID.
struct wall_rec {
    int type, id;
    double p[7];
};
std::vector<wall_rec> g_walls;

template <class con_t>
void add_walls(con_t &con, std::vector<wall *> &owned) {
    for (const wall_rec &w : g_walls) {
        wall *o = nullptr;
        const double *p = w.p;
        if (w.type == 0) o = new wall_sphere(p[0], p[1], p[2], p[3], w.id);
        else if (w.type == 1) o = new wall_plane(p[0], p[1], p[2], p[3], w.id);
        else if (w.type == 2) o = new wall_cylinder(p[0], p[1], p[2], p[3], p[4], p[5], p[6], w.id);
        else o = new wall_cone(p[0], p[1], p[2], p[3], p[4], p[5], p[6], w.id);
        owned.push_back(o);
        con.add_wall(o);
    }
}

// Builds the container of the given kind, puts the particles, and calls
// f(con, loop).  Returns false on an unknown kind.
template <class F>
bool with_container(int kind, const double *geom, const int *grid, const int *periodic, int n, const int *ids,
                    const double *xyzr, F f) {
    std::vector<wall *> owned;
    if (kind == 0) {
        container con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2],
                      periodic[0] != 0, periodic[1] != 0, periodic[2] != 0, 8);
        add_walls(con, owned);
        for (int i = 0; i < n; i++) con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2]);
        c_loop_all vl(con);
        f(con, vl);
    } else if (kind == 1) {
        container_poly con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2],
                           periodic[0] != 0, periodic[1] != 0, periodic[2] != 0, 8);
        add_walls(con, owned);
        for (int i = 0; i < n; i++)
            con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2], xyzr[4 * i + 3]);
        c_loop_all vl(con);
        f(con, vl);
    } else if (kind == 2) {
        container_periodic con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2], 8);
        for (int i = 0; i < n; i++) con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2]);
        c_loop_all_periodic vl(con);
        f(con, vl);
    } else if (kind == 3) {
        container_periodic_poly con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2], 8);
        for (int i = 0; i < n; i++)
            con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2], xyzr[4 * i + 3]);
        c_loop_all_periodic vl(con);
        f(con, vl);
    } else {
        return false;
    }
    for (wall *w : owned) delete w;
    return true;
}

// Every periodic image block of a container_periodic(_poly), built before any
// ghost: the reference builds them lazily, and a block first built while a
// ghost sits in its primary block keeps a copy of the ghost (which that
// ghost, and any later one, then sees); built first, a ghost cell depends on
// the particles alone.
template <class con_t>
void images_first(con_t &con) {
    if constexpr (std::is_same<con_t, container_periodic>::value ||
                  std::is_same<con_t, container_periodic_poly>::value)
        con.create_all_images();
}

// compute_ghost_cell of the container's kind (radius for the radical kinds)
template <class con_t>
bool ghost_of(con_t &con, voronoicell_neighbor &c, const double *g) {
    if constexpr (std::is_same<con_t, container_poly>::value || std::is_same<con_t, container_periodic_poly>::value)
        return con.compute_ghost_cell(c, g[0], g[1], g[2], g[3]);
    else
        return con.compute_ghost_cell(c, g[0], g[1], g[2]);
}

}  // namespace

extern "C" {

// The walls later calls add to kind 0/1 containers (n = 0: none).
void ref_set_walls(int n, const int *type, const double *params, const int *id) {
    g_walls.clear();
    for (int i = 0; i < n; i++) {
        wall_rec w;
        w.type = type[i];
        w.id = id[i];
        for (int a = 0; a < 7; a++) w.p[a] = params[7 * i + a];
        g_walls.push_back(w);
    }
}

// The polytope of every cell in loop order, flattened into doubles:
//   ok, nv, nf, surface_area, total_edge_distance, vertices (3 nv, particle-
//   relative), then per face: neighbour, order, area, perimeter, normal (3),
//   vertex indices (order)
// with the faces in the reference's own traversal order (the one
// neighbors / face_areas / face_vertices share, src/cell.cc:2189-2308).
// Returns the number of doubles, or -(needed) if cap is too small.
long ref_polytopes(int kind, const double *geom, const int *grid, const int *periodic, int n, const int *ids,
                   const double *xyzr, long cap, double *out) {
    std::vector<double> buf;
    bool ok = with_container(kind, geom, grid, periodic, n, ids, xyzr, [&](auto &con, auto &vl) {
        voronoicell_neighbor c(con);
        std::vector<int> nb, fv, fo;
        std::vector<double> vs, fa, fp, nm;
        if (!vl.start()) return;
        do {
            if (!con.compute_cell(c, vl)) {
                buf.insert(buf.end(), {0.0, 0.0, 0.0, 0.0, 0.0});
                continue;
            }
            c.vertices(vs);
            c.neighbors(nb);
            c.face_vertices(fv);
            c.face_orders(fo);
            c.face_areas(fa);
            c.face_perimeters(fp);
            c.normals(nm);
            buf.push_back(1.0);
            buf.push_back((double)c.p);
            buf.push_back((double)nb.size());
            buf.push_back(c.surface_area());
            buf.push_back(c.total_edge_distance());
            buf.insert(buf.end(), vs.begin(), vs.end());
            size_t q = 0;
            for (size_t f = 0; f < nb.size(); f++) {
                const int ord = fv[q];
                buf.push_back((double)nb[f]);
                buf.push_back((double)ord);
                buf.push_back(fa[f]);
                buf.push_back(fp[f]);
                buf.push_back(nm[3 * f]);
                buf.push_back(nm[3 * f + 1]);
                buf.push_back(nm[3 * f + 2]);
                for (int j = 0; j < ord; j++) buf.push_back((double)fv[q + 1 + j]);
                q += 1 + ord;
            }
        } while (vl.inc());
    });
    if (!ok) return 0;
    if ((long)buf.size() > cap) return -(long)buf.size();
    std::copy(buf.begin(), buf.end(), out);
    return (long)buf.size();
}

// Point location with the reference: find_voronoi_cell for each query point
// (container::find_voronoi_cell, src/container.cc:237-263 and 275-301;
// container_periodic::find_voronoi_cell, src/container_prd.cc:303-359).
// found[i] = 0 where it returns false; else pid[i] and r[3i..3i+2].
int ref_find_voronoi_cells(int kind, const double *geom, const int *grid, const int *periodic, int n, const int *ids,
                           const double *xyzr, int nq, const double *q, int *found, int *pid, double *r) {
    bool ok = with_container(kind, geom, grid, periodic, n, ids, xyzr, [&](auto &con, auto &) {
        for (int i = 0; i < nq; i++) {
            double rx = 0, ry = 0, rz = 0;
            int id = -1;
            const bool f = con.find_voronoi_cell(q[3 * i], q[3 * i + 1], q[3 * i + 2], rx, ry, rz, id);
            found[i] = f ? 1 : 0;
            pid[i] = f ? id : -1;
            r[3 * i] = f ? rx : 0.0;
            r[3 * i + 1] = f ? ry : 0.0;
            r[3 * i + 2] = f ? rz : 0.0;
        }
    });
    return ok ? 0 : -2;
}

// Ghost cells with the reference: compute_ghost_cell for each ghost
// (gxyzr: x, y, z, r; r used by the radical kinds), one record per ghost as
// ref_compute_cells writes them (ok, vol, centroid, faces, vertices,
// max_radius_squared, neighbours in CSR).  Returns 0, or -1 if nb_cap was
// too small.
int ref_ghost_cells(int kind, const double *geom, const int *grid, const int *periodic, int n, const int *ids,
                    const double *xyzr, int ng, const double *gxyzr, int *out_ok, double *out_vol, double *out_cen,
                    int *out_nf, int *out_nv, double *out_mrs, long nb_cap, int *out_nb, long *out_nb_off) {
    int status = 0;
    bool ok = with_container(kind, geom, grid, periodic, n, ids, xyzr, [&](auto &con, auto &) {
        voronoicell_neighbor c(con);
        std::vector<int> v;
        long used = 0;
        images_first(con);
        for (int i = 0; i < ng; i++) {
            out_nb_off[i] = used;
            const bool q = ghost_of(con, c, gxyzr + 4 * i);
            out_ok[i] = q ? 1 : 0;
            if (!q) {
                out_vol[i] = 0;
                out_cen[3 * i] = out_cen[3 * i + 1] = out_cen[3 * i + 2] = 0;
                out_nf[i] = out_nv[i] = 0;
                out_mrs[i] = 0;
                continue;
            }
            double cx, cy, cz;
            out_vol[i] = c.volume();
            c.centroid(cx, cy, cz);
            out_cen[3 * i] = cx; out_cen[3 * i + 1] = cy; out_cen[3 * i + 2] = cz;
            out_nf[i] = c.number_of_faces();
            out_nv[i] = c.p;
            out_mrs[i] = c.max_radius_squared();
            c.neighbors(v);
            for (size_t j = 0; j < v.size(); j++) {
                if (used >= nb_cap) { status = -1; return; }
                out_nb[used++] = v[j];
            }
        }
        out_nb_off[ng] = used;
    });
    if (!ok) return -2;
    return status;
}

// The reference's own print_custom output for every cell, written to path
// (container::print_custom(format, filename), src/container.cc:401-417).
int ref_print_custom(int kind, const double *geom, const int *grid, const int *periodic, int n, const int *ids,
                     const double *xyzr, const char *format, const char *path) {
    bool ok = with_container(kind, geom, grid, periodic, n, ids, xyzr,
                             [&](auto &con, auto &) { con.print_custom(format, path); });
    return ok ? 0 : -2;
}

// Computes every cell with the reference and writes one record per stored
// particle.  Returns the number of records, or -1 if a capacity was too small.
int ref_compute_cells(int kind, const double *geom, const int *grid, const int *periodic,
                      int n, const int *ids, const double *xyzr,
                      int cap, int *out_id, double *out_pos, double *out_vol, double *out_cen,
                      int *out_nf, int *out_nv, int *out_ok, double *out_mrs,
                      long nb_cap, int *out_nb, long *out_nb_off) {
    rec_sink s{cap, 0, out_id, out_pos, out_vol, out_cen, out_mrs, out_nf, out_nv, out_ok,
               out_nb, nb_cap, 0, out_nb_off, 0};
    if (!with_container(kind, geom, grid, periodic, n, ids, xyzr,
                        [&](auto &con, auto &vl) { run_cells(con, vl, s); }))
        return -2;
    return s.overflow ? -1 : s.n;
}

// Times the reference's own compute_all_cells() (the "dummy" computation of
// src/container.cc:438-453) after put(); returns seconds, or -1 on a bad kind.
double ref_time_compute_all(int kind, const double *geom, const int *grid, const int *periodic,
                            int n, const int *ids, const double *xyzr, double *sum_vol) {
    using clk = std::chrono::steady_clock;
    double secs = -1;
    auto timed = [&](auto &con) {
        auto t0 = clk::now();
        con.compute_all_cells();
        auto t1 = clk::now();
        secs = std::chrono::duration<double>(t1 - t0).count();
        if (sum_vol) *sum_vol = con.sum_cell_volumes();
    };
    if (kind == 0) {
        container con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2],
                      periodic[0] != 0, periodic[1] != 0, periodic[2] != 0, 8);
        for (int i = 0; i < n; i++) con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2]);
        timed(con);
    } else if (kind == 1) {
        container_poly con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2],
                           periodic[0] != 0, periodic[1] != 0, periodic[2] != 0, 8);
        for (int i = 0; i < n; i++)
            con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2], xyzr[4 * i + 3]);
        timed(con);
    } else if (kind == 2) {
        container_periodic con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2], 8);
        for (int i = 0; i < n; i++) con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2]);
        timed(con);
    } else if (kind == 3) {
        container_periodic_poly con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2], 8);
        for (int i = 0; i < n; i++)
            con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2], xyzr[4 * i + 3]);
        timed(con);
    }
    return secs;
}

}  // extern "C"
