// Drop-in C++ host API for the GB300 Voronoi cell engine.
//
// A program written against the reference's container API (src/voro++.hh:
// container, container_poly, container_periodic, container_periodic_poly,
// c_loop_all, c_loop_all_periodic, voronoicell, voronoicell_neighbor) builds
// against this header instead by replacing
//     #include "voro++.hh"            ->   #include "voro_gb300.hh"
//     -lvoro++                        ->   -lvorogpu
// The classes keep the reference's names, constructor arguments and
// semantics; every cell is computed on the GPU through the C ABI of
// vorogpu.h, once per compute_all_cells() (or lazily on first use).
//
// What a cell exposes after compute_cell(c, vl) is what the engine returns per
// cell: volume(), centroid(), number_of_faces(), number_of_edges(), p (vertex
// count), max_radius_squared() and, for voronoicell_neighbor, neighbors().
// The queries that need the polytope itself (vertices(), face_vertices(),
// face_areas(), face_orders(), face_perimeters(), normals(), surface_area(),
// total_edge_distance(), vertex_orders(), face_freq_table()) work once the
// container keeps polytopes: con.set_polytopes(true) before computing
// (print_custom switches it on by itself for the fields that need it).
// Vertex and face numbering is the engine's own: faces are listed in the
// order of neighbors() (ascending neighbour ID), each as a vertex loop
// clockwise seen from outside like the reference's.
//
// Errors follow the reference (src/common.cc:27-30): the message is printed
// and the process exits with the status code, unless VORO_GB300_THROW is
// defined, in which case voro::gpu_error is thrown instead.
#ifndef VORO_GB300_HH
#define VORO_GB300_HH

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <initializer_list>
#include <vector>

#include "vorogpu.h"

namespace voro {

// Status codes and the default radius of the reference (src/config.hh:88-119).
const int VOROPP_FILE_ERROR = 1;
const int VOROPP_MEMORY_ERROR = 2;
const int VOROPP_INTERNAL_ERROR = 3;
const int VOROPP_CMD_LINE_ERROR = 4;
const double default_radius = 0.5;

struct gpu_error : std::runtime_error {
    int status;
    gpu_error(const std::string &m, int s) : std::runtime_error(m), status(s) {}
};

inline void voro_fatal_error(const char *p, int status) {
#ifdef VORO_GB300_THROW
    throw gpu_error(p, status);
#else
    fprintf(stderr, "voro++: %s\n", p);
    exit(status);
#endif
}

namespace gpu_detail {
// Argument packs for the C ABI's fixed-size arrays (temporaries that live
// until the end of the constructor call that uses them).
struct d6 {
    double v[6];
};
struct i3 {
    int v[3];
};
inline void check(int rc, const char *what) {
    if (rc == VGPU_OK) return;
    std::string m = std::string(what) + ": " + vgpu_last_error();
    // engine codes 1..3 are the reference's; the GPU-specific ones map to an internal error
    voro_fatal_error(m.c_str(), rc <= VOROPP_INTERNAL_ERROR ? rc : VOROPP_INTERNAL_ERROR);
}
}  // namespace gpu_detail

class container_gpu_base;

// Walls (src/wall.hh:25-130): the reference's constructors; the container
// hands their parameters to the engine (vgpu_add_wall), which cuts every
// cell with them as the reference's cut_cell does.
class wall {
  public:
    virtual ~wall() {}
    int type_ = 0, w_id_ = -99;
    double p_[7] = {0, 0, 0, 0, 0, 0, 0};

  protected:
    wall(int type, int id, std::initializer_list<double> p) : type_(type), w_id_(id) {
        int i = 0;
        for (double v : p) p_[i++] = v;
    }
};
class wall_sphere : public wall {
  public:
    wall_sphere(double xc_, double yc_, double zc_, double rc_, int w_id_ = -99)
        : wall(VGPU_WALL_SPHERE, w_id_, {xc_, yc_, zc_, rc_}) {}
};
class wall_plane : public wall {
  public:
    wall_plane(double xc_, double yc_, double zc_, double ac_, int w_id_ = -99)
        : wall(VGPU_WALL_PLANE, w_id_, {xc_, yc_, zc_, ac_}) {}
};
class wall_cylinder : public wall {
  public:
    wall_cylinder(double xc_, double yc_, double zc_, double xa_, double ya_, double za_, double rc_,
                  int w_id_ = -99)
        : wall(VGPU_WALL_CYLINDER, w_id_, {xc_, yc_, zc_, xa_, ya_, za_, rc_}) {}
};
class wall_cone : public wall {
  public:
    wall_cone(double xc_, double yc_, double zc_, double xa_, double ya_, double za_, double ang, int w_id_ = -99)
        : wall(VGPU_WALL_CONE, w_id_, {xc_, yc_, zc_, xa_, ya_, za_, ang}) {}
};

// Per-cell results of one compute_cell call (voronoicell, src/cell.hh:93-350).
class voronoicell {
  public:
    int p = 0;   // vertex count (voronoicell_base::p)
    voronoicell() {}
    template <class C>
    explicit voronoicell(C &) {}
    double volume() const { return vol_; }
    void centroid(double &cx, double &cy, double &cz) const {
        cx = cen_[0];
        cy = cen_[1];
        cz = cen_[2];
    }
    int number_of_faces() const { return nf_; }
    // Euler's relation for a convex polyhedron, V - E + F = 2: it holds with
    // vertices of any order, as the reference's edge count does
    // (src/cell.cc:2469)
    int number_of_edges() const { return p + nf_ - 2; }
    // in the reference's doubled coordinates (src/cell.cc:1907-1917)
    double max_radius_squared() const { return 4.0 * mr2_; }

    // ---- polytope queries (src/cell.hh:132-184); need set_polytopes(true)
    void vertices(std::vector<double> &v) const {
        need_poly();
        v = verts_;
    }
    void vertices(double x, double y, double z, std::vector<double> &v) const {
        need_poly();
        v = verts_;
        for (size_t i = 0; i < v.size(); i += 3) {
            v[i] += x;
            v[i + 1] += y;
            v[i + 2] += z;
        }
    }
    // per face: vertex count, then the loop (as voronoicell_base::face_vertices)
    void face_vertices(std::vector<int> &v) const {
        need_poly();
        v.clear();
        for (size_t f = 0; f < fstart_.size(); f++) {
            v.push_back(forder(f));
            for (int j = 0; j < forder(f); j++) v.push_back(floops_[fstart_[f] + j]);
        }
    }
    void face_orders(std::vector<int> &v) const {
        need_poly();
        v.resize(fstart_.size());
        for (size_t f = 0; f < fstart_.size(); f++) v[f] = forder(f);
    }
    void face_areas(std::vector<double> &v) const {
        need_poly();
        v.resize(fstart_.size());
        for (size_t f = 0; f < fstart_.size(); f++) {
            double n[3];
            newell(f, n);
            v[f] = 0.5 * std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        }
    }
    void face_perimeters(std::vector<double> &v) const {
        need_poly();
        v.resize(fstart_.size());
        for (size_t f = 0; f < fstart_.size(); f++) {
            double per = 0;
            for (int j = 0; j < forder(f); j++) {
                const double *a = vert(floops_[fstart_[f] + j]);
                const double *b = vert(floops_[fstart_[f] + (j + 1) % forder(f)]);
                per += std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                                 (a[2] - b[2]) * (a[2] - b[2]));
            }
            v[f] = per;
        }
    }
    // outward unit normals, three per face, by the rule of
    // voronoicell_base::normals_search (src/cell.cc:2108-2164): from the
    // loop's second edge on, the first edge longer than the tolerance is
    // paired with each later edge until their vector product is above it.
    // The tests are on the reference's doubled coordinates, 2x these
    // vertices.  The reference starts at its lowest-numbered vertex of the
    // face, a numbering the engine does not share: each start is tried in
    // turn, and a face gets (0, 0, 0) only when none finds such a pair.
    void normals(std::vector<double> &v) const {
        need_poly();
        v.assign(3 * fstart_.size(), 0.0);
        for (size_t f = 0; f < fstart_.size(); f++) {
            const int m = forder(f);
            auto edge = [&](int t, double e[3]) {
                const double *a = vert(floops_[fstart_[f] + t % m]);
                const double *b = vert(floops_[fstart_[f] + (t + 1) % m]);
                for (int c = 0; c < 3; c++) e[c] = b[c] - a[c];
            };
            bool found = false;
            for (int r = 0; r < m && !found; r++) {
                for (int t = 1; t < m; t++) {
                    double u[3];
                    edge(r + t, u);
                    if (4.0 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) <= tol_) continue;
                    for (int s = t + 1; s < m; s++) {
                        double e[3];
                        edge(r + s, e);
                        const double w[3] = {e[1] * u[2] - e[2] * u[1], e[2] * u[0] - e[0] * u[2],
                                             e[0] * u[1] - e[1] * u[0]};
                        const double wm = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
                        if (16.0 * wm > tol_) {
                            const double q = 1.0 / std::sqrt(wm);
                            for (int c = 0; c < 3; c++) v[3 * f + c] = w[c] * q;
                            found = true;
                            break;
                        }
                    }
                    break;
                }
            }
        }
    }
    double surface_area() const {
        std::vector<double> a;
        face_areas(a);
        double s = 0;
        for (double x : a) s += x;
        return s;
    }
    double total_edge_distance() const {
        std::vector<double> p_;
        face_perimeters(p_);
        double s = 0;
        for (double x : p_) s += x;
        return 0.5 * s;   // every edge bounds two faces
    }
    void vertex_orders(std::vector<int> &v) const {
        if (!has_poly_ && p == 2 * nf_ - 4) {
            v.assign(p, 3);   // V = 2F - 4: every vertex has order 3
            return;
        }
        need_poly();
        v.assign(p, 0);
        for (int x : floops_) v[x]++;
    }
    void face_freq_table(std::vector<int> &v) const {
        std::vector<int> o;
        face_orders(o);
        v.clear();
        for (int k : o) {
            if ((int)v.size() <= k) v.resize(k + 1, 0);
            v[k]++;
        }
    }
    // voronoicell_base::output_custom (src/cell.cc:2485-2558): the
    // print_custom fields of this cell, for particle i at (x, y, z), radius r
    void output_custom(const char *format, int i, double x, double y, double z, double r, FILE *fp = stdout) const;

  protected:
    friend class container_gpu_base;
    double vol_ = 0, cen_[3] = {0, 0, 0}, mr2_ = 0;
    double tol_ = 0;   // the container's length tolerance, for normals()
    int nf_ = 0;
    bool has_poly_ = false;
    std::vector<double> verts_;   // 3 per vertex, particle-relative
    std::vector<int> fstart_;     // per face (neighbour order): start in floops_
    std::vector<int> floops_;     // concatenated vertex loops
    std::vector<int> fnb_;        // per face: neighbour ID
    int forder(size_t f) const {
        return (f + 1 < fstart_.size() ? fstart_[f + 1] : (int)floops_.size()) - fstart_[f];
    }
    const double *vert(int i) const { return &verts_[3 * i]; }
    // twice the face's vector area, from vectors relative to its first vertex
    // (small faces keep their precision)
    void newell(size_t f, double n[3]) const {
        n[0] = n[1] = n[2] = 0;
        const int m = forder(f);
        const double *o = vert(floops_[fstart_[f]]);
        for (int j = 1; j + 1 < m; j++) {
            const double *pa = vert(floops_[fstart_[f] + j]);
            const double *pb = vert(floops_[fstart_[f] + j + 1]);
            const double a[3] = {pa[0] - o[0], pa[1] - o[1], pa[2] - o[2]};
            const double b[3] = {pb[0] - o[0], pb[1] - o[1], pb[2] - o[2]};
            n[0] += a[1] * b[2] - a[2] * b[1];
            n[1] += a[2] * b[0] - a[0] * b[2];
            n[2] += a[0] * b[1] - a[1] * b[0];
        }
    }
    void need_poly() const {
        if (!has_poly_)
            voro_fatal_error("this query needs the cell polytope: call set_polytopes(true) on the container "
                             "before computing",
                             VOROPP_INTERNAL_ERROR);
    }
};

// voronoicell_neighbor (src/cell.hh:470-560): adds the neighbour ID per face.
class voronoicell_neighbor : public voronoicell {
  public:
    voronoicell_neighbor() {}
    template <class C>
    explicit voronoicell_neighbor(C &) {}
    // one ID per face, ascending (the reference lists them in face order)
    void neighbors(std::vector<int> &v) const { v = nb_; }
    void output_custom(const char *format, int i, double x, double y, double z, double r, FILE *fp = stdout) const;

  protected:
    friend class container_gpu_base;
    std::vector<int> nb_;
};

// The fields of output_custom (src/cell.cc:2485-2558), printed as the
// reference's printers do (src/common.cc:37-136); nb: the neighbour IDs
// (voronoicell_neighbor), NULL for a plain voronoicell (whose %n is empty).
inline void gpu_detail_print_cell(const voronoicell &c, const std::vector<int> *nb, const char *format, int id,
                                  double x, double y, double z, double r, FILE *fp) {
    std::vector<double> d;
    std::vector<int> iv;
    auto print_d = [&](const std::vector<double> &v) {
        for (size_t i = 0; i < v.size(); i++) fprintf(fp, i ? " %g" : "%g", v[i]);
    };
    auto print_i = [&](const std::vector<int> &v) {
        for (size_t i = 0; i < v.size(); i++) fprintf(fp, i ? " %d" : "%d", v[i]);
    };
    auto print_xyz = [&](const std::vector<double> &v, double ox, double oy, double oz) {
        for (size_t i = 0; i < v.size(); i += 3)
            fprintf(fp, i ? " (%g,%g,%g)" : "(%g,%g,%g)", ox + v[i], oy + v[i + 1], oz + v[i + 2]);
    };
    for (const char *f = format; *f; f++) {
        if (*f != '%') {
            putc(*f, fp);
            continue;
        }
        f++;
        switch (*f) {
            case 'i': fprintf(fp, "%d", id); break;
            case 'x': fprintf(fp, "%g", x); break;
            case 'y': fprintf(fp, "%g", y); break;
            case 'z': fprintf(fp, "%g", z); break;
            case 'q': fprintf(fp, "%g %g %g", x, y, z); break;
            case 'r': fprintf(fp, "%g", r); break;
            case 'w': fprintf(fp, "%d", c.p); break;
            case 'p': c.vertices(d); print_xyz(d, 0, 0, 0); break;
            case 'P': c.vertices(d); print_xyz(d, x, y, z); break;
            case 'o': c.vertex_orders(iv); print_i(iv); break;
            case 'm': fprintf(fp, "%g", 0.25 * c.max_radius_squared()); break;
            case 'g': fprintf(fp, "%d", c.number_of_edges()); break;
            case 'E': fprintf(fp, "%g", c.total_edge_distance()); break;
            case 'e': c.face_perimeters(d); print_d(d); break;
            case 's': fprintf(fp, "%d", c.number_of_faces()); break;
            case 'F': fprintf(fp, "%g", c.surface_area()); break;
            case 'A': c.face_freq_table(iv); print_i(iv); break;
            case 'a': c.face_orders(iv); print_i(iv); break;
            case 'f': c.face_areas(d); print_d(d); break;
            case 't': {
                c.face_vertices(iv);
                size_t i = 0;
                bool first = true;
                while (i < iv.size()) {
                    const int m = iv[i++];
                    fputs(first ? "(" : " (", fp);
                    first = false;
                    for (int j = 0; j < m; j++) fprintf(fp, j ? ",%d" : "%d", iv[i + j]);
                    fputs(")", fp);
                    i += m;
                }
            } break;
            case 'l': c.normals(d); print_xyz(d, 0, 0, 0); break;
            case 'n':
                if (nb) print_i(*nb);
                break;
            case 'v': fprintf(fp, "%g", c.volume()); break;
            case 'c': {
                double cx, cy, cz;
                c.centroid(cx, cy, cz);
                fprintf(fp, "%g %g %g", cx, cy, cz);
            } break;
            case 'C': {
                double cx, cy, cz;
                c.centroid(cx, cy, cz);
                fprintf(fp, "%g %g %g", x + cx, y + cy, z + cz);
            } break;
            case 0: f--; break;
            default:
                putc('%', fp);
                putc(*f, fp);
        }
    }
    fputs("\n", fp);
}
inline void voronoicell::output_custom(const char *format, int i, double x, double y, double z, double r,
                                       FILE *fp) const {
    gpu_detail_print_cell(*this, nullptr, format, i, x, y, z, r, fp);
}
inline void voronoicell_neighbor::output_custom(const char *format, int i, double x, double y, double z, double r,
                                                FILE *fp) const {
    gpu_detail_print_cell(*this, &nb_, format, i, x, y, z, r, fp);
}

// particle_order (src/c_loops.hh:27-71): the order in which particles were
// put through it (put / import with a particle_order); c_loop_order visits
// their cells in that order.
class particle_order {
  public:
    explicit particle_order(int init_size = 16) { idx_.reserve(init_size > 0 ? init_size : 16); }
    void add(int64_t put_index) { idx_.push_back(put_index); }
    size_t size() const { return idx_.size(); }
    int64_t operator[](size_t i) const { return idx_[i]; }

  private:
    std::vector<int64_t> idx_;
};

// Shared implementation of the four container classes.
class container_gpu_base {
  public:
    container_gpu_base(const container_gpu_base &) = delete;
    container_gpu_base &operator=(const container_gpu_base &) = delete;
    ~container_gpu_base() {
        if (h_) vgpu_container_destroy(h_);
    }

    // Keep every cell's polytope from the next compute on (needed by the
    // voronoicell vertex/face queries; no counterpart in the reference, whose
    // cells always carry their polytope).
    void set_polytopes(bool on) {
        gpu_detail::check(vgpu_set_output(h_, on ? VGPU_OUTPUT_POLYTOPES : 0), "set_polytopes");
        poly_on_ = on;
        dirty_ = true;
    }

    // Precision of the engine: VGPU_MIXED (default) or VGPU_FP64.
    void set_mode(int mode) {
        mode_ = mode;
        dirty_ = true;
    }

    // Sheared container_periodic: depth of the image layers a compute stores
    // first, in mean particle spacings (0: default; < 0: the reference's
    // depth from the start); the cells never depend on it.
    void set_ghost_depth(double spacings) {
        gpu_detail::check(vgpu_set_ghost_depth(h_, spacings), "set_ghost_depth");
        dirty_ = true;
    }

    // container::clear (src/container.cc:385-387)
    void clear() {
        ids_in_.clear();
        xyzr_in_.clear();
        gpu_detail::check(vgpu_clear(h_), "clear");
        n_put_ = 0;
        dirty_ = true;
    }

    // For c_loop_order: per particle put since the last clear (put order), its
    // row in the loop-order results, -1 where put() dropped it.
    const std::vector<int32_t> &input_rows() {
        ensure();
        if (!rows_valid_) {
            rows_.assign((size_t)n_put_, -1);
            if (n_put_ > 0) gpu_detail::check(vgpu_get_input_rows(h_, rows_.data()), "input_rows");
            rows_valid_ = true;
        }
        return rows_;
    }

    // container::compute_all_cells (src/container.cc:438-453)
    void compute_all_cells() {
        flush();
        gpu_detail::check(vgpu_compute(h_, mode_), "compute_all_cells");
        int64_t n = 0;
        gpu_detail::check(vgpu_num_cells(h_, &n), "compute_all_cells");
        n_ = n;
        ids_.resize(n);
        pos_.resize(3 * n);
        vol_.resize(n);
        cen_.resize(3 * n);
        nf_.resize(n);
        nv_.resize(n);
        mr2_.resize(n);
        flags_.resize(n);
        rad_.resize(n);
        if (n > 0) {
            gpu_detail::check(vgpu_get_cells(h_, ids_.data(), pos_.data(), vol_.data(), cen_.data(), nf_.data(),
                                             nv_.data(), mr2_.data(), flags_.data()),
                              "compute_all_cells");
            gpu_detail::check(vgpu_get_radii(h_, rad_.data()), "compute_all_cells");
        }
        have_nb_ = false;
        rows_valid_ = false;
        poff_.clear();
        pdata_.clear();
        if (poly_on_ && n > 0) {
            poff_.assign(n + 1, 0);
            gpu_detail::check(vgpu_get_polytopes(h_, poff_.data(), nullptr), "polytopes");
            pdata_.resize(poff_[n] > 0 ? poff_[n] : 1);
            gpu_detail::check(vgpu_get_polytopes(h_, poff_.data(), pdata_.data()), "polytopes");
        }
        dirty_ = false;
    }

    // container::sum_cell_volumes (src/container.cc:459-465)
    double sum_cell_volumes() {
        ensure();
        double s = 0;
        gpu_detail::check(vgpu_sum_cell_volumes(h_, &s), "sum_cell_volumes");
        return s;
    }

    // wall_list::add_wall (src/container.hh:62-69) and point_inside_walls (75-78)
    void add_wall(wall &w) {
        gpu_detail::check(vgpu_add_wall(h_, w.type_, w.p_, w.w_id_), "add_wall");
        dirty_ = true;
    }
    void add_wall(wall *w) { add_wall(*w); }
    bool point_inside_walls(double x, double y, double z) {
        int in = 0;
        gpu_detail::check(vgpu_point_inside_walls(h_, x, y, z, &in), "point_inside_walls");
        return in != 0;
    }

    // container::find_voronoi_cell (src/container.cc:237-301,
    // src/container_prd.cc:303-359): the particle whose Voronoi cell holds
    // (x, y, z); false outside a non-periodic wall or with no particles.
    bool find_voronoi_cell(double x, double y, double z, double &rx, double &ry, double &rz, int &pid) {
        flush();
        const double q[3] = {x, y, z};
        double r[3] = {0, 0, 0};
        int32_t id = -1, found = 0;
        gpu_detail::check(vgpu_find_voronoi_cells(h_, 1, q, &id, r, &found), "find_voronoi_cell");
        if (!found) return false;
        rx = r[0];
        ry = r[1];
        rz = r[2];
        pid = id;
        return true;
    }

    // container_base::total_particles (src/container.hh:150-155)
    int total_particles() {
        ensure();
        return (int)n_;
    }

    // compute_cell (src/container.hh:462-465): fills c with cell k of the loop
    // and returns false if the cell was cut away entirely.
    template <class c_loop>
    bool compute_cell(voronoicell &c, c_loop &vl) {
        ensure();
        return fill(c, vl.index());
    }
    template <class c_loop>
    bool compute_cell(voronoicell_neighbor &c, c_loop &vl) {
        ensure();
        ensure_neighbors();
        if (!fill(c, vl.index())) return false;
        const int64_t k = vl.index();
        c.nb_.assign(nb_.begin() + off_[k], nb_.begin() + off_[k + 1]);
        return true;
    }

    // compute_ghost_cell (src/container.hh:487-498 and 710-721,
    // src/container_prd.hh:414-422 and 635-644): the cell of a ghost particle
    // at (x, y, z) (radius r for the radical kinds) among the particles;
    // false if it has none (outside a non-periodic wall, or cut away).
    bool compute_ghost_cell(voronoicell &c, double x, double y, double z, double r = default_radius) {
        return ghost(c, nullptr, x, y, z, r);
    }
    bool compute_ghost_cell(voronoicell_neighbor &c, double x, double y, double z, double r = default_radius) {
        return ghost(c, &c.nb_, x, y, z, r);
    }

    // container::print_custom (src/container.hh:434-451; fields
    // src/cell.cc:2485-2558)
    void print_custom(const char *format, FILE *fp = stdout) {
        if (needs_polytope(format) && !poly_on_) set_polytopes(true);
        ensure();
        if (contains_neighbor(format)) ensure_neighbors();
        voronoicell_neighbor c;
        for (int64_t k = 0; k < n_; k++) print_cell(c, format, k, fp);
    }
    // the same over the cells of a loop (c_loop_all, c_loop_order), as the
    // reference's command-line utility prints them (src/cmd_line.cc:75-121)
    template <class c_loop>
    void print_custom_loop(c_loop &vl, const char *format, FILE *fp = stdout) {
        if (needs_polytope(format) && !poly_on_) set_polytopes(true);
        ensure();
        if (contains_neighbor(format)) ensure_neighbors();
        voronoicell_neighbor c;
        if (vl.start()) do print_cell(c, format, vl.index(), fp);
            while (vl.inc());
    }
    void print_custom(const char *format, const char *filename) {
        FILE *fp = fopen(filename, "w");
        if (!fp) voro_fatal_error("Unable to open file", VOROPP_FILE_ERROR);
        print_custom(format, fp);
        fclose(fp);
    }

    // Loop-order record access used by c_loop_all.
    int64_t size() {
        ensure();
        return n_;
    }
    int pid_at(int64_t k) const { return ids_[k]; }
    const double *pos_at(int64_t k) const { return &pos_[3 * k]; }
    double radius_at(int64_t k) const { return poly_ ? rad_[k] : default_radius; }

    vgpu_container *handle() { return h_; }

  protected:
    container_gpu_base(int kind, const double geom[6], const int grid[3], const int per[3])
        : poly_(kind == VGPU_CONTAINER_POLY || kind == VGPU_CONTAINER_PERIODIC_POLY) {
        gpu_detail::check(vgpu_container_create(&h_, kind, geom, grid, per), "container");
        gpu_detail::check(vgpu_get_tolerance(h_, &tol_), "container");
        for (int i = 0; i < 6; i++) geom_[i] = geom[i];
    }

    // container_base::point_inside (src/container.cc:484-487): inside the
    // box (every axis, periodic or not) and inside every wall
    bool point_inside_box_and_walls(double x, double y, double z) {
        if (x < geom_[0] || x > geom_[1] || y < geom_[2] || y > geom_[3] || z < geom_[4] || z > geom_[5])
            return false;
        return point_inside_walls(x, y, z);
    }
    double geom_[6];

    void stage(int n, double x, double y, double z, double r) {
        n_put_++;
        ids_in_.push_back(n);
        xyzr_in_.push_back(x);
        xyzr_in_.push_back(y);
        xyzr_in_.push_back(z);
        xyzr_in_.push_back(r);
        dirty_ = true;
    }

    // put with a particle_order (src/container.hh:294,516): the order records
    // the particle's place in the put sequence
    void stage(particle_order &vo, int n, double x, double y, double z, double r) {
        vo.add(n_put_);
        stage(n, x, y, z, r);
    }

    // container::import (src/container.cc:333-376): "id x y z" (+ " r") per line
    void import_stream(FILE *fp, bool with_r, particle_order *vo = nullptr) {
        int i, j;
        double x, y, z, r = default_radius;
        while ((j = with_r ? fscanf(fp, "%d %lg %lg %lg %lg", &i, &x, &y, &z, &r)
                           : fscanf(fp, "%d %lg %lg %lg", &i, &x, &y, &z)) == (with_r ? 5 : 4)) {
            if (vo) stage(*vo, i, x, y, z, r);
            else stage(i, x, y, z, r);
        }
        if (j != EOF) voro_fatal_error("File import error", VOROPP_FILE_ERROR);
    }
    void import_file(const char *filename, bool with_r, particle_order *vo = nullptr) {
        FILE *fp = fopen(filename, "r");
        if (!fp) voro_fatal_error("Unable to open file", VOROPP_FILE_ERROR);
        import_stream(fp, with_r, vo);
        fclose(fp);
    }

  private:
    vgpu_container *h_ = nullptr;
    double tol_ = 0;   // the reference cell's length tolerance (vgpu_get_tolerance)
    bool poly_;
    bool poly_on_ = false;
    std::vector<int64_t> poff_;
    std::vector<double> pdata_;
    int mode_ = VGPU_MIXED;
    bool dirty_ = true, have_nb_ = false;
    std::vector<int32_t> ids_in_;
    std::vector<double> xyzr_in_;
    int64_t n_ = 0;
    int64_t n_put_ = 0;          // particles put since the last clear
    bool rows_valid_ = false;
    std::vector<int32_t> rows_;  // input_rows() of the last compute
    std::vector<int32_t> ids_, nf_, nv_, flags_, nb_;
    std::vector<double> pos_, vol_, cen_, mr2_, rad_;
    std::vector<int64_t> off_;

    void flush() {
        if (!ids_in_.empty()) {
            gpu_detail::check(vgpu_put(h_, (int64_t)ids_in_.size(), ids_in_.data(), xyzr_in_.data()), "put");
            ids_in_.clear();
            xyzr_in_.clear();
        }
    }
    void ensure() {
        if (dirty_) compute_all_cells();
    }
    void ensure_neighbors() {
        if (have_nb_) return;
        int64_t tot = 0;
        gpu_detail::check(vgpu_num_neighbors(h_, &tot), "neighbors");
        off_.assign(n_ + 1, 0);
        nb_.resize(tot > 0 ? tot : 1);
        gpu_detail::check(vgpu_get_neighbors(h_, off_.data(), nb_.data()), "neighbors");
        nb_.resize(tot);
        have_nb_ = true;
    }
    bool ghost(voronoicell &c, std::vector<int> *nb, double x, double y, double z, double r) {
        flush();
        const double g[4] = {x, y, z, r};
        gpu_detail::check(vgpu_compute_ghost_cells(h_, mode_, 1, g), "compute_ghost_cell");
        double vol = 0, cen[3] = {0, 0, 0}, mr2 = 0;
        int32_t nf = 0, nv = 0, fl = 0;
        gpu_detail::check(vgpu_get_ghost_cells(h_, &vol, cen, &nf, &nv, &mr2, &fl), "compute_ghost_cell");
        c.has_poly_ = false;
        c.p = nv;
        c.vol_ = vol;
        c.cen_[0] = cen[0];
        c.cen_[1] = cen[1];
        c.cen_[2] = cen[2];
        c.nf_ = nf;
        c.mr2_ = mr2;
        if (!(fl & VGPU_CELL_OK)) return false;
        if (nb) {
            int64_t off[2] = {0, 0};
            gpu_detail::check(vgpu_get_ghost_neighbors(h_, off, nullptr), "compute_ghost_cell");
            nb->assign((size_t)off[1], 0);
            gpu_detail::check(vgpu_get_ghost_neighbors(h_, off, nb->data()), "compute_ghost_cell");
        }
        if (poly_on_) {
            int64_t off[2] = {0, 0};
            gpu_detail::check(vgpu_get_ghost_polytopes(h_, off, nullptr), "compute_ghost_cell");
            std::vector<double> d((size_t)std::max<int64_t>(off[1], 1));
            gpu_detail::check(vgpu_get_ghost_polytopes(h_, off, d.data()), "compute_ghost_cell");
            if (off[1] > 0) load_polytope(c, d.data(), tol_);
        }
        return true;
    }
    bool fill(voronoicell &c, int64_t k) {
        c.has_poly_ = false;
        if (poly_on_ && !poff_.empty() && poff_[k + 1] > poff_[k]) load_polytope(c, &pdata_[poff_[k]], tol_);
        c.p = nv_[k];
        c.vol_ = vol_[k];
        c.cen_[0] = cen_[3 * k];
        c.cen_[1] = cen_[3 * k + 1];
        c.cen_[2] = cen_[3 * k + 2];
        c.nf_ = nf_[k];
        c.mr2_ = mr2_[k];
        return (flags_[k] & VGPU_CELL_OK) != 0;
    }
    // [nv, nf, vertices, per face: neighbour, m, loop] -> faces in neighbour order
    static void load_polytope(voronoicell &c, const double *d, double tol) {
        const int nv = (int)d[0], nf = (int)d[1];
        c.tol_ = tol;
        c.verts_.assign(d + 2, d + 2 + 3 * nv);
        std::vector<int> fs(nf), order(nf);
        int i = 2 + 3 * nv;
        for (int f = 0; f < nf; f++) {
            fs[f] = i;
            order[f] = f;
            i += 2 + (int)d[i + 1];
        }
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return d[fs[a]] < d[fs[b]]; });
        c.fstart_.clear();
        c.floops_.clear();
        c.fnb_.clear();
        for (int f : order) {
            c.fstart_.push_back((int)c.floops_.size());
            c.fnb_.push_back((int)d[fs[f]]);
            const int m = (int)d[fs[f] + 1];
            for (int j = 0; j < m; j++) c.floops_.push_back((int)d[fs[f] + 2 + j]);
        }
        c.has_poly_ = true;
    }
    static bool needs_polytope(const char *format) {
        for (const char *f = format; *f; f++)
            if (f[0] == '%' && f[1]) {
                if (strchr("pPoEeFAaftl", f[1])) return true;
                f++;
            }
        return false;
    }
    static bool contains_neighbor(const char *format) {
        for (const char *f = format; *f; f++)
            if (f[0] == '%' && f[1] == 'n') return true;
        return false;
    }
    // cell k (loop order) as a voronoicell_neighbor, printed if it has a cell
    void print_cell(voronoicell_neighbor &c, const char *format, int64_t k, FILE *fp) {
        if (!fill(c, k)) return;
        if (have_nb_) c.nb_.assign(nb_.begin() + off_[k], nb_.begin() + off_[k + 1]);
        else c.nb_.clear();
        c.output_custom(format, ids_[k], pos_[3 * k], pos_[3 * k + 1], pos_[3 * k + 2], radius_at(k), fp);
    }
};

// container (src/container.hh:289-291)
class container : public container_gpu_base {
  public:
    container(double ax_, double bx_, double ay_, double by_, double az_, double bz_, int nx_, int ny_, int nz_,
              bool xperiodic_, bool yperiodic_, bool zperiodic_, int /*init_mem*/)
        : container_gpu_base(VGPU_CONTAINER, gpu_detail::d6{{ax_, bx_, ay_, by_, az_, bz_}}.v,
                             gpu_detail::i3{{nx_, ny_, nz_}}.v, gpu_detail::i3{{xperiodic_, yperiodic_, zperiodic_}}.v) {}
    void put(int n, double x, double y, double z) { stage(n, x, y, z, default_radius); }
    void import(FILE *fp = stdin) { import_stream(fp, false); }
    void import(const char *filename) { import_file(filename, false); }
    void put(particle_order &vo, int n, double x, double y, double z) { stage(vo, n, x, y, z, default_radius); }
    void import(particle_order &vo, FILE *fp = stdin) { import_stream(fp, false, &vo); }
    void import(particle_order &vo, const char *filename) { import_file(filename, false, &vo); }
    bool point_inside(double x, double y, double z) { return point_inside_box_and_walls(x, y, z); }
};

// container_poly (src/container.hh:511-513)
class container_poly : public container_gpu_base {
  public:
    container_poly(double ax_, double bx_, double ay_, double by_, double az_, double bz_, int nx_, int ny_, int nz_,
                   bool xperiodic_, bool yperiodic_, bool zperiodic_, int /*init_mem*/)
        : container_gpu_base(VGPU_CONTAINER_POLY, gpu_detail::d6{{ax_, bx_, ay_, by_, az_, bz_}}.v,
                             gpu_detail::i3{{nx_, ny_, nz_}}.v, gpu_detail::i3{{xperiodic_, yperiodic_, zperiodic_}}.v) {}
    void put(int n, double x, double y, double z, double r) { stage(n, x, y, z, r); }
    void import(FILE *fp = stdin) { import_stream(fp, true); }
    void import(const char *filename) { import_file(filename, true); }
    void put(particle_order &vo, int n, double x, double y, double z, double r) { stage(vo, n, x, y, z, r); }
    void import(particle_order &vo, FILE *fp = stdin) { import_stream(fp, true, &vo); }
    void import(particle_order &vo, const char *filename) { import_file(filename, true, &vo); }
    bool point_inside(double x, double y, double z) { return point_inside_box_and_walls(x, y, z); }
};

// container_periodic (src/container_prd.hh:213-216): the periodic
// parallelepiped of lattice vectors (bx,0,0), (bxy,by,0), (bxz,byz,bz).
class container_periodic : public container_gpu_base {
  public:
    container_periodic(double bx_, double bxy_, double by_, double bxz_, double byz_, double bz_, int nx_, int ny_,
                       int nz_, int /*init_mem*/)
        : container_gpu_base(VGPU_CONTAINER_PERIODIC, gpu_detail::d6{{bx_, bxy_, by_, bxz_, byz_, bz_}}.v,
                             gpu_detail::i3{{nx_, ny_, nz_}}.v, gpu_detail::i3{{1, 1, 1}}.v) {}
    void put(int n, double x, double y, double z) { stage(n, x, y, z, default_radius); }
    void import(FILE *fp = stdin) { import_stream(fp, false); }
    void import(const char *filename) { import_file(filename, false); }
    void put(particle_order &vo, int n, double x, double y, double z) { stage(vo, n, x, y, z, default_radius); }
    void import(particle_order &vo, FILE *fp = stdin) { import_stream(fp, false, &vo); }
    void import(particle_order &vo, const char *filename) { import_file(filename, false, &vo); }
};

// container_periodic_poly (src/container_prd.hh:434-437)
class container_periodic_poly : public container_gpu_base {
  public:
    container_periodic_poly(double bx_, double bxy_, double by_, double bxz_, double byz_, double bz_, int nx_,
                            int ny_, int nz_, int /*init_mem*/)
        : container_gpu_base(VGPU_CONTAINER_PERIODIC_POLY, gpu_detail::d6{{bx_, bxy_, by_, bxz_, byz_, bz_}}.v,
                             gpu_detail::i3{{nx_, ny_, nz_}}.v, gpu_detail::i3{{1, 1, 1}}.v) {}
    void put(int n, double x, double y, double z, double r) { stage(n, x, y, z, r); }
    void import(FILE *fp = stdin) { import_stream(fp, true); }
    void import(const char *filename) { import_file(filename, true); }
    void put(particle_order &vo, int n, double x, double y, double z, double r) { stage(vo, n, x, y, z, r); }
    void import(particle_order &vo, FILE *fp = stdin) { import_stream(fp, true, &vo); }
    void import(particle_order &vo, const char *filename) { import_file(filename, true, &vo); }
};

// c_loop_all (src/c_loops.hh:165-210) and c_loop_all_periodic (325-393): the
// reference's loop order, which is the order of the engine's records.
class c_loop_all {
  public:
    template <class C>
    explicit c_loop_all(C &con) : con_(&con) {}
    bool start() {
        k_ = 0;
        return con_->size() > 0;
    }
    bool inc() { return ++k_ < con_->size(); }
    int pid() const { return con_->pid_at(k_); }
    void pos(double &x, double &y, double &z) const {
        const double *p = con_->pos_at(k_);
        x = p[0];
        y = p[1];
        z = p[2];
    }
    void pos(int &pid_, double &x, double &y, double &z, double &r) const {
        pid_ = pid();
        pos(x, y, z);
        r = con_->radius_at(k_);
    }
    double x() const { return con_->pos_at(k_)[0]; }
    double y() const { return con_->pos_at(k_)[1]; }
    double z() const { return con_->pos_at(k_)[2]; }
    int64_t index() const { return k_; }

  private:
    container_gpu_base *con_;
    int64_t k_ = 0;
};
typedef c_loop_all c_loop_all_periodic;

// c_loop_order (src/c_loops.hh:268-317) and c_loop_order_periodic (398-446):
// the cells of the particles of a particle_order, in its order (particles
// that put() dropped have no cell and are skipped).
class c_loop_order {
  public:
    template <class C>
    c_loop_order(C &con, particle_order &vo) : con_(&con), vo_(&vo) {}
    bool start() {
        rows_ = &con_->input_rows();
        i_ = 0;
        return seek();
    }
    bool inc() {
        i_++;
        return seek();
    }
    int pid() const { return con_->pid_at(k_); }
    void pos(double &x, double &y, double &z) const {
        const double *p = con_->pos_at(k_);
        x = p[0];
        y = p[1];
        z = p[2];
    }
    void pos(int &pid_, double &x, double &y, double &z, double &r) const {
        pid_ = pid();
        pos(x, y, z);
        r = con_->radius_at(k_);
    }
    double x() const { return con_->pos_at(k_)[0]; }
    double y() const { return con_->pos_at(k_)[1]; }
    double z() const { return con_->pos_at(k_)[2]; }
    int64_t index() const { return k_; }

  private:
    container_gpu_base *con_;
    particle_order *vo_;
    const std::vector<int32_t> *rows_ = nullptr;
    size_t i_ = 0;
    int64_t k_ = 0;
    bool seek() {
        for (; i_ < vo_->size(); i_++) {
            const int64_t j = (*vo_)[i_];
            if (j >= 0 && j < (int64_t)rows_->size() && (*rows_)[j] >= 0) {
                k_ = (*rows_)[j];
                return true;
            }
        }
        return false;
    }
};
typedef c_loop_order c_loop_order_periodic;

}  // namespace voro

#endif
