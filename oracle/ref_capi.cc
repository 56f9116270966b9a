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
#include <chrono>
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

}  // namespace

extern "C" {

// Computes every cell with the reference and writes one record per stored
// particle.  Returns the number of records, or -1 if a capacity was too small.
int ref_compute_cells(int kind, const double *geom, const int *grid, const int *periodic,
                      int n, const int *ids, const double *xyzr,
                      int cap, int *out_id, double *out_pos, double *out_vol, double *out_cen,
                      int *out_nf, int *out_nv, int *out_ok, double *out_mrs,
                      long nb_cap, int *out_nb, long *out_nb_off) {
    rec_sink s{cap, 0, out_id, out_pos, out_vol, out_cen, out_mrs, out_nf, out_nv, out_ok,
               out_nb, nb_cap, 0, out_nb_off, 0};
    if (kind == 0) {
        container con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2],
                      periodic[0] != 0, periodic[1] != 0, periodic[2] != 0, 8);
        for (int i = 0; i < n; i++) con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2]);
        c_loop_all vl(con);
        run_cells(con, vl, s);
    } else if (kind == 1) {
        container_poly con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2],
                           periodic[0] != 0, periodic[1] != 0, periodic[2] != 0, 8);
        for (int i = 0; i < n; i++)
            con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2], xyzr[4 * i + 3]);
        c_loop_all vl(con);
        run_cells(con, vl, s);
    } else if (kind == 2) {
        container_periodic con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2], 8);
        for (int i = 0; i < n; i++) con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2]);
        c_loop_all_periodic vl(con);
        run_cells(con, vl, s);
    } else if (kind == 3) {
        container_periodic_poly con(geom[0], geom[1], geom[2], geom[3], geom[4], geom[5], grid[0], grid[1], grid[2], 8);
        for (int i = 0; i < n; i++)
            con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2], xyzr[4 * i + 3]);
        c_loop_all_periodic vl(con);
        run_cells(con, vl, s);
    } else {
        return -2;
    }
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
