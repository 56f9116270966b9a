// CPU restatement of the reference's plane-cutting cell — TEST INFRASTRUCTURE.
//
// This is the oracle: a restatement, in this project's own code and storage
// layout, of voronoicell_base / voronoicell_neighbor (src/cell.hh, src/cell.cc).
// It keeps the reference's floating-point operation order so that it can be
// pinned bit for bit against the real library, and it counts the vertex-plane
// side tests (the reference's m_calc calls) for the roofline arithmetic.
//
// Storage differs from the reference: each vertex owns a block in one pool
// holding its edges, the relation table and the neighbour IDs
// ([edges | relations | ids], 3*cap ints).  The reference's back pointer
// slot (ed[i][2*nu[i]], used as a marker in the marginal-vertex code) is the
// separate array bp[].
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace vport {

extern const double kTolerance;   // 10*DBL_EPSILON (src/config.hh:80)
extern const double kBigTolFac;   // 20 (src/config.hh:82)

struct Cell {
    // vertex data
    int p = 0;     // vertex count (src/cell.hh:54)
    int up = 0;    // search start vertex (src/cell.hh:62)
    std::vector<double> pts;  // 4 per vertex: doubled coordinates + cached plane value
    std::vector<int> nu, off, cap, bp;
    std::vector<unsigned> mask;
    std::vector<int> pool;
    unsigned maskc = 0;
    double tol, tol_cu, big_tol;
    // current plane (src/cell.hh:282-289)
    double px = 0, py = 0, pz = 0, prsq = 0;
    // stacks: delete (ds), auxiliary delete (ds2), extra search (xse)
    std::vector<int> ds, ds2, xse;
    // count of vertex-plane side tests (m_calc calls)
    uint64_t side_tests = 0;

    explicit Cell(double max_len_sq);

    // accessors
    inline int &E(int i, int k) { return pool[off[i] + k]; }
    inline int &R(int i, int k) { return pool[off[i] + cap[i] + k]; }
    inline int &N(int i, int k) { return pool[off[i] + 2 * cap[i] + k]; }
    inline int cycle_up(int a, int q) const { return a == nu[q] - 1 ? 0 : a + 1; }
    inline int cycle_down(int a, int q) const { return a == 0 ? nu[q] - 1 : a - 1; }

    void reset_pool(int vertices_hint);
    int new_block(int order);                 // returns pool offset, block of capacity >= order
    void ensure_vertex(int i);                // room for vertex index i in per-vertex arrays
    void set_order(int i, int order);         // (re)allocate vertex i's block for `order` edges (content lost)

    void init_box(double xmin, double xmax, double ymin, double ymax, double zmin, double zmax,
                  const int ids[6]);
    void copy_from(const Cell &o);

    bool nplane(double x, double y, double z, double rsq, int p_id);
    bool plane_intersects(double x, double y, double z, double rsq);
    bool plane_intersects_guess(double x, double y, double z, double rsq);
    double max_radius_squared() const;

    double volume();
    void centroid(double &cx, double &cy, double &cz);
    int number_of_faces();
    void neighbors(std::vector<int> &v);

   private:
    inline unsigned m_test(int n, double &ans) {
        if (mask[n] >= maskc) {
            ans = pts[4 * n + 3];
            return mask[n] & 3;
        }
        return m_calc(n, ans);
    }
    unsigned m_calc(int n, double &ans);
    unsigned m_testx(int n, double &ans);
    void reset_mask();
    bool search_for_outside_edge(int &upv);
    void add_to_stack(int sc2, int lp);
    bool search_upward(unsigned &uw, int &lp, int &ls, int &us, double &l, double &u);
    bool definite_max(int &lp, int &ls, double &l, double &u, unsigned &uw);
    bool search_downward(unsigned &lw, int &lp, int &ls, int &us, double &l, double &u);
    bool definite_min(int &lp, int &us, double &l, double &u, unsigned &lw);
    bool create_facet(int lp, int ls, double l, int us, double u, int p_id);
    bool collapse_order2();
    bool collapse_order1();
    bool delete_connection(int j, int k, bool hand);
    void move_vertex(int dst, int src);
    inline void flip(int tp) { bp[tp] = -1 - bp[tp]; }
    void reset_edges();
};

}  // namespace vport
