// C ABI of the engine (declared in include/vorogpu.h).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <mutex>
#include <sys/stat.h>
#include <string>
#include <vector>
#include "vgpu_internal.cuh"
#include "../../include/vorogpu.h"

#include <atomic>

namespace vgpu {
static std::atomic<long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
}

using namespace vgpu;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

}  // namespace

// Error reporting for the library's other translation units.
int vgpu::report_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

namespace {

#define VG_CUDA(expr)                                                                        \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return fail(_e == cudaErrorMemoryAllocation ? VGPU_ERR_MEMORY : VGPU_ERR_CUDA,   \
                        "%s: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, __LINE__); \
    } while (0)

// A device buffer that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want) {
        if (want <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t b = want + std::min<size_t>(want / 8, (size_t)64 << 20) + 256;   // headroom for regrowth
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T *as() const { return reinterpret_cast<T *>(p); }
};


struct OffsetTable {
    std::vector<int> codes;
    std::vector<int> group_start;
    std::vector<int> group_lb2;
};

const OffsetTable &offset_table() {
    static OffsetTable t = [] {
        OffsetTable o;
        struct E { int lb2, r2, code; };
        std::vector<E> es;
        const int R = kOffsetRadius;
        for (int dk = -R; dk <= R; dk++)
            for (int dj = -R; dj <= R; dj++)
                for (int di = -R; di <= R; di++) {
                    int a = std::max(std::abs(di) - 1, 0), b = std::max(std::abs(dj) - 1, 0),
                        c = std::max(std::abs(dk) - 1, 0);
                    int lb2 = a * a + b * b + c * c;
                    if (lb2 > kTableLb2Max) continue;
                    int code = (di + 16) | ((dj + 16) << 5) | ((dk + 16) << 10);
                    es.push_back({lb2, di * di + dj * dj + dk * dk, code});
                }
        std::stable_sort(es.begin(), es.end(), [](const E &x, const E &y) {
            if (x.lb2 != y.lb2) return x.lb2 < y.lb2;
            return x.r2 < y.r2;
        });
        // one group per lower bound lb2, then a small group (at most 24
        // offsets) joins the one before it when that saves a 32-lane pass of
        // the gather: a group is gathered and its candidates tested (nearest
        // first) before the next, so merging saves a pass and a sort, and its
        // lower bound (the first group's) still ends the search correctly
        std::vector<int> start, lb2;
        for (size_t i = 0; i < es.size(); i++) {
            if (i == 0 || es[i].lb2 != es[i - 1].lb2) {
                start.push_back((int)i);
                lb2.push_back(es[i].lb2);
            }
            o.codes.push_back(es[i].code);
        }
        start.push_back((int)es.size());
        auto passes = [](int n) { return (n + 31) / 32; };
        for (size_t g = 0; g + 1 < start.size(); g++) {
            const int n = start[g + 1] - start[g];
            if (!o.group_start.empty()) {
                const int prev = start[g] - o.group_start.back();
                if (n <= 24 && passes(prev + n) < passes(prev) + passes(n)) continue;   // joins the previous group
            }
            o.group_start.push_back(start[g]);
            o.group_lb2.push_back(lb2[g]);
        }
        o.group_start.push_back((int)es.size());
        return o;
    }();
    return t;
}

}  // namespace

// Polytope record store, words per cell: the mean record of a uniform
// periodic box is about 186 words with FP32 vertices (MIXED engine) and 268
// with FP64 ones; a cell that finds the store full fails with
// VGPU_FAIL_RECORDS.  Polytope output: 2 + 6 nv + 2 nf doubles per cell
// (about 195).
constexpr unsigned long long kRecWordsPerCell[2] = {384, 256};   // FP64, MIXED
constexpr unsigned long long kPolyDoublesPerCell = 256;
// neighbour overflow store (ints) for n cells: cells with more than kNbStride
// faces are rare (Poisson cells average 15.5); this holds a quarter of an int
// per cell, e.g. 6 % of the cells at 36 faces
inline size_t nb_ovf_ints(size_t n) { return std::min<size_t>(n / 4 + 4096, (size_t)1 << 30); }

// default budget of a batch's record store (records are scratch between the
// clipping and finish kernels; larger batches are processed in waves)
constexpr unsigned long long kBatchRecordBytes = 8ull << 30;

struct vgpu_container {
    Geometry g;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6];
    double target_density = 0.6;   // the autotuner's choice on the 4M periodic box
    int warps_per_cta = 4;
    // particles put() so far, staged on the device in put() order
    int64_t staged = 0;
    // device input (either owned copies or caller's device arrays)
    const int32_t *dev_ids_ext = nullptr;
    const double *dev_xyzr_ext = nullptr;
    int64_t dev_n_ext = 0;
    bool use_device_input = false;
    DevBuf ids_in, xyzr_in;
    DevBuf chk;   // put(): index of the first non-finite particle
    // pinned host words the binning reads back asynchronously: [0] kept and
    // non-finite counts, [1] largest radius (bits), [2] duplicate flag
    unsigned long long *host_rb = nullptr;
    bool dup_pending = false;   // the duplicate flag of a deferred check is in host_rb[2]
    // work buffers
    DevBuf rem, ukey, gkey, idx, idx2, keys_alt, vals_alt, hist, scan_tmp, outpos_in, kept;
    DevBuf p64, lffh, lffl, pid, outpos, gblock, bstart, offsets, ovf_list, ovf_list2, counters, counters2;
    // results
    DevBuf rec_off, poly, poly_off;
    DevBuf loc_q, loc_found, loc_pid, loc_r;   // point-location queries and answers
    // ghost cells: engine arrays (the particles, then the ghosts), their
    // record offsets, work lists and results
    DevBuf gh_p64, gh_lffh, gh_lffl, gh_pid, gh_gblock, gh_outpos, gh_rec_off, gh_q, gh_keep, gh_list, gh_ovf, gh_ovf2,
        gh_cnt, gh_vol, gh_cen, gh_nf, gh_nv, gh_mr2, gh_flags, gh_nb, gh_nb_ovf, gh_nb_off, gh_nb_out, gh_poly,
        gh_poly_off;
    std::vector<WallSpec> lattice;  // sheared periodic boxes: the unit cell's face planes (after the walls)
    double full_lo[3] = {0, 0, 0}, full_ext[3] = {0, 0, 0};   // ... their ghost layers at the reference's depth
    bool tric_thin = false;         // the last binning stored thinner ghost layers
    double ghost_spacings = 8.0;    // their depth in mean particle spacings (< 0: never thin)
    int nengine = 0;                // engine entries of the last binning: the particles, then any images
    DevBuf x_rem, x_gkey, x_idx, x_kalt, x_valt, img_cnt, img_off, img_src, cell_list;   // images (sheared boxes)
    std::vector<WallSpec> walls;    // walls, in the order added
    DevBuf walls_dev;               // their device copy (uploaded when changed)
    bool walls_dirty = false;
    int64_t ghost_n = 0;            // ghosts of the last ghost compute
    bool ghost_poly = false;        // their polytopes were kept
    unsigned long long ghost_poly_used = 0;
    DevBuf r_vol, r_cen, r_nf, r_nv, r_mr2, r_flags, r_nb, r_nb_ovf, r_ids, r_pos, r_rad, nb_off, nb_out, nb_tmp, sum_tmp;
    int64_t ncells = 0;
    int nkept = 0;              // cells of the compute in progress
    int output = 0;             // VGPU_OUTPUT_* flags
    unsigned long long poly_used = 0;   // doubles of polytope output of the last compute
    long long launches0 = 0;    // launch counter at its start
    bool computed = false;
    // the CSR neighbour offsets of the last compute are in nb_off (csr_total
    // neighbours), so that get_neighbors after num_neighbors scans once
    bool csr_valid = false;
    int64_t csr_total = 0;
    bool binned = false;        // engine-order arrays match the particles (after a compute or a locate)
    vgpu_stats stats{};
    double phase[16] = {};
    int64_t record_bytes = 0;   // record-store budget of one compute (0: kRecWordsPerCell per cell)
    double fp64_fallback = 0.25;   // hand-on fraction of the sample above which a mixed compute runs FP64
    int cell_chunk = 0;            // cells per work-queue grab (0: built-in default)
};

namespace {

// The Voronoi cell about the origin of the lattice of a sheared periodic box
// (unitcell::unitcell, src/unitcell.cc:26-79): a large box (max_unit_voro_shells
// box lengths, src/config.hh:93) is cut by the bisecting planes of the lattice
// vectors i*a + j*b + k*c shell by shell (Chebyshev index l = 1, 2, ...) until
// no vector of a shell cuts it.  Kept as its vertices, each with the planes
// it lies on: a cut keeps the vertices inside and adds a vertex on each edge
// (two vertices sharing two planes) that crosses the plane.
struct UnitCell {
    std::vector<std::array<double, 3>> v;       // vertices
    std::vector<std::array<double, 4>> faces;   // lattice vectors (x, y, z, |d|^2) whose bisectors are faces
};

bool build_unit_cell(const double B[6], UnitCell &U) {
    const double bx = B[0], bxy = B[1], by = B[2], bxz = B[3], byz = B[4], bz = B[5];
    constexpr int kShells = 10;
    struct Vert {
        std::array<double, 3> x;
        std::vector<int> pl;
    };
    std::vector<std::array<double, 4>> planes;   // n.x <= h
    const double uc[3] = {kShells * bx, kShells * by, kShells * bz};
    for (int a = 0; a < 3; a++)
        for (int sgn = -1; sgn <= 1; sgn += 2) {
            std::array<double, 4> q = {0, 0, 0, uc[a]};
            q[a] = sgn;
            planes.push_back(q);
        }
    std::vector<Vert> V;
    for (int c = 0; c < 8; c++) {
        Vert w;
        for (int a = 0; a < 3; a++) {
            const int hi = (c >> a) & 1;
            w.x[a] = hi ? uc[a] : -uc[a];
            w.pl.push_back(2 * a + hi);
        }
        V.push_back(w);
    }
    const double scale = std::fabs(bx) + std::fabs(bxy) + std::fabs(by) + std::fabs(bxz) + std::fabs(byz) + std::fabs(bz);
    const double eps = 1e-11 * scale;
    auto side = [](const Vert &w, const std::array<double, 4> &q) {
        return q[0] * w.x[0] + q[1] * w.x[1] + q[2] * w.x[2] - q[3];
    };
    auto cut = [&](const std::array<double, 4> &q) {
        const double e = eps * (1.0 + std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]));
        std::vector<double> sv(V.size());
        bool any = false;
        for (size_t i = 0; i < V.size(); i++) {
            sv[i] = side(V[i], q);
            any |= sv[i] > e;
        }
        if (!any) return;
        const int idx = (int)planes.size();
        planes.push_back(q);
        std::vector<Vert> out;
        for (size_t i = 0; i < V.size(); i++)
            if (sv[i] <= e) {
                out.push_back(V[i]);
                if (sv[i] >= -e) out.back().pl.push_back(idx);
            }
        for (size_t i = 0; i < V.size(); i++) {
            if (!(sv[i] < -e)) continue;
            for (size_t j = 0; j < V.size(); j++) {
                if (!(sv[j] > e)) continue;
                std::vector<int> common;
                for (int p : V[i].pl)
                    if (std::find(V[j].pl.begin(), V[j].pl.end(), p) != V[j].pl.end()) common.push_back(p);
                if (common.size() < 2) continue;
                const double t = sv[i] / (sv[i] - sv[j]);
                Vert w;
                for (int a = 0; a < 3; a++) w.x[a] = V[i].x[a] + t * (V[j].x[a] - V[i].x[a]);
                w.pl = common;
                w.pl.push_back(idx);
                out.push_back(w);
            }
        }
        V.swap(out);
    };
    for (int l = 1; l < 2 * kShells; l++) {
        std::vector<std::array<double, 4>> shell;
        for (int k = -l; k <= l; k++)
            for (int j = -l; j <= l; j++)
                for (int i = -l; i <= l; i++) {
                    if (std::max(std::abs(i), std::max(std::abs(j), std::abs(k))) != l) continue;
                    const double x = i * bx + j * bxy + k * bxz, y = j * by + k * byz, z = k * bz;
                    shell.push_back({x, y, z, 0.5 * (x * x + y * y + z * z)});
                }
        bool cuts = false;
        for (const auto &q : shell) {
            const double e = eps * (1.0 + std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]));
            for (const Vert &w : V)
                if (side(w, q) > e) {
                    cuts = true;
                    break;
                }
            if (cuts) break;
        }
        if (!cuts) {
            U.v.clear();
            for (const Vert &w : V) {
                for (int p : w.pl)
                    if (p < 6) return false;   // the box still bounds the cell
                U.v.push_back(w.x);
            }
            U.faces.clear();
            for (size_t p = 6; p < planes.size(); p++) {
                int on = 0;
                for (const Vert &w : V) on += std::find(w.pl.begin(), w.pl.end(), (int)p) != w.pl.end();
                if (on >= 3) U.faces.push_back({planes[p][0], planes[p][1], planes[p][2], 2.0 * planes[p][3]});
            }
            return !U.v.empty() && U.faces.size() <= (size_t)kMaxWalls;
        }
        for (const auto &q : shell) cut(q);
    }
    return false;   // src/unitcell.cc:76-79: VOROPP_MEMORY_ERROR
}

int setup_geometry(vgpu_container *h, int kind, const double geom[6], const int grid[3], const int periodic[3]) {
    Geometry &g = h->g;
    memset(&g, 0, sizeof(g));
    g.kind = kind;
    g.poly = (kind == VGPU_CONTAINER_POLY || kind == VGPU_CONTAINER_PERIODIC_POLY) ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        if (grid[a] < 1) return fail(VGPU_ERR_ARG, "grid[%d] = %d must be >= 1", a, grid[a]);
        g.un[a] = grid[a];
    }
    double max_len_sq;
    if (kind == VGPU_CONTAINER || kind == VGPU_CONTAINER_POLY) {
        g.unit_cell = 0;
        for (int a = 0; a < 3; a++) {
            g.lo[a] = geom[2 * a];
            g.hi[a] = geom[2 * a + 1];
            g.len[a] = g.hi[a] - g.lo[a];
            if (!(g.len[a] > 0)) return fail(VGPU_ERR_ARG, "empty container extent on axis %d", a);
            g.per[a] = periodic ? (periodic[a] != 0) : 0;
            g.ext[a] = g.len[a];
            g.ubox[a] = g.len[a] / g.un[a];   // src/container.cc:31
            g.usp[a] = 1 / g.ubox[a];          // src/v_base.cc:26
        }
        // src/container.cc:34-35
        max_len_sq = g.len[0] * g.len[0] * (g.per[0] ? 0.25 : 1) + g.len[1] * g.len[1] * (g.per[1] ? 0.25 : 1) +
                     g.len[2] * g.len[2] * (g.per[2] ? 0.25 : 1);
    } else if (kind == VGPU_CONTAINER_PERIODIC || kind == VGPU_CONTAINER_PERIODIC_POLY) {
        // geom = (bx, bxy, by, bxz, byz, bz)
        g.unit_cell = 1;
        double L[3] = {geom[0], geom[2], geom[5]};
        g.shear[0] = geom[1];
        g.shear[1] = geom[3];
        g.shear[2] = geom[4];
        for (int a = 0; a < 3; a++) {
            if (!(L[a] > 0)) return fail(VGPU_ERR_ARG, "periodic length on axis %d must be > 0", a);
            if (!std::isfinite(g.shear[a])) return fail(VGPU_ERR_ARG, "shear terms must be finite");
            g.lo[a] = 0;
            g.len[a] = L[a];
            g.hi[a] = L[a];
            g.ext[a] = L[a];
            g.per[a] = 1;
            g.half[a] = 0.5 * L[a];
            g.ubox[a] = L[a] / g.un[a];        // src/container_prd.cc:31
            g.usp[a] = 1 / g.ubox[a];
        }
        h->lattice.clear();
        if (g.shear[0] != 0.0 || g.shear[1] != 0.0 || g.shear[2] != 0.0) {
            UnitCell U;
            if (!build_unit_cell(geom, U)) return fail(VGPU_ERR_MEMORY, "periodic cell computation failed");
            // max_len_sq = unit_voro.max_radius_squared() (doubled
            // coordinates); ghost layers ey, ez from the largest y and z a
            // cutting particle can have (src/unitcell.cc:60-70,
            // src/container_prd.cc:31-33)
            double mr = 0, muy = 0, muz = 0, mab[3] = {0, 0, 0};
            for (const auto &v : U.v) {
                const double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                mr = std::max(mr, 4.0 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
                muy = std::max(muy, v[1] + r);
                muz = std::max(muz, v[2] + r);
                for (int a = 0; a < 3; a++) mab[a] = std::max(mab[a], std::fabs(v[a]));
            }
            max_len_sq = mr;
            const int ey = (int)(muy * g.usp[1] + 1), ez = (int)(muz * g.usp[2] + 1);
            g.tric = 1;
            g.per[1] = g.per[2] = 0;
            g.lo[1] = -(ey * g.ubox[1]);
            g.lo[2] = -(ez * g.ubox[2]);
            g.ext[1] = (g.un[1] + 2 * ey) * g.ubox[1];
            g.ext[2] = (g.un[2] + 2 * ez) * g.ubox[2];
            // the initial box: just larger than the unit cell (its own face
            // planes cut it to the unit cell); the FP32 side tests' error
            // bounds grow with the vertices' distance, so no larger
            for (int a = 0; a < 3; a++) g.half[a] = 1.02 * mab[a];
            for (const auto &f : U.faces) {
                WallSpec w;
                memset(&w, 0, sizeof(w));
                w.type = kWallLattice;
                w.id = 0;   // the unit cell's faces carry neighbour 0 (src/cell.cc:86-94)
                for (int a = 0; a < 3; a++) w.c[a] = f[a];
                w.r = f[3];
                h->lattice.push_back(w);
            }
            h->walls_dirty = true;
            for (int a = 0; a < 3; a++) {
                h->full_lo[a] = g.lo[a];
                h->full_ext[a] = g.ext[a];
            }
        } else {
            // unit_voro.max_radius_squared() of the rectangular unit cell
            // (src/container_prd.cc:32), in the reference's doubled coordinates
            max_len_sq = L[0] * L[0] + L[1] * L[1] + L[2] * L[2];
        }
    } else {
        return fail(VGPU_ERR_ARG, "unknown container kind %d", kind);
    }
    double tol = 10.0 * 2.220446049250313e-16 * max_len_sq;  // src/config.hh:80, src/cell.cc:24
    g.tol_h = 0.5 * tol;
    g.tol_h32 = std::nextafter((float)g.tol_h, 3.0e38f);
    g.tol_cu = tol * std::sqrt(tol);
    return VGPU_OK;
}

// n particles in the domain; the engine region (ghost layers included)
// holds them at the same density.
void choose_engine_grid(Geometry &g, int64_t n, double density) {
    double vol = g.len[0] * g.len[1] * g.len[2];
    double nn = (double)std::max<int64_t>(n, 1);
    double bs = std::cbrt(vol * density / nn);
    long long total = 1;
    for (int a = 0; a < 3; a++) {
        int m = (int)std::floor(g.ext[a] / bs + 0.5);
        m = std::max(1, std::min(m, 1 << 10));
        g.gn[a] = m;
        total *= m;
    }
    while (total > (1ll << 26)) {
        total = 1;
        for (int a = 0; a < 3; a++) {
            g.gn[a] = std::max(1, g.gn[a] / 2);
            total *= g.gn[a];
        }
    }
    float bmin = 3.4e38f, bmax = 0.0f;
    for (int a = 0; a < 3; a++) {
        g.gbs[a] = g.ext[a] / g.gn[a];
        g.gbs32[a] = (float)g.gbs[a];
        g.gbs_h[a] = g.gbs32[a];
        g.gbs_l[a] = (float)(g.gbs[a] - (double)g.gbs32[a]);
        bmin = std::min(bmin, g.gbs32[a]);
        bmax = std::max(bmax, g.gbs32[a]);
    }
    g.gbs_min = bmin * (1.0f - 1e-6f);
    g.gbs_max = bmax * (1.0f + 1e-6f);
}

int ensure_device(vgpu_container *h) {
    int dev = 0;
    VG_CUDA(cudaGetDevice(&dev));
    h->device = dev;
    return VGPU_OK;
}

}  // namespace

extern "C" {

const char *vgpu_version(void) { return "vorogpu 0.1 (sm_103a)"; }

const char *vgpu_last_error(void) { return g_last_error.c_str(); }

int vgpu_device_count(int *count) {
    if (!count) return fail(VGPU_ERR_ARG, "null count");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) c = 0;
    *count = c;
    return VGPU_OK;
}

int vgpu_container_create(vgpu_container **out, int kind, const double geom[6], const int grid[3],
                          const int periodic[3]) {
    if (!out || !geom || !grid) return fail(VGPU_ERR_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(VGPU_ERR_NO_DEVICE, "no CUDA device");
    vgpu_container *h = new vgpu_container();
    int rc = setup_geometry(h, kind, geom, grid, periodic);
    if (rc != VGPU_OK) {
        delete h;
        return rc;
    }
    rc = ensure_device(h);
    if (rc != VGPU_OK) {
        delete h;
        return rc;
    }
    cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(VGPU_ERR_CUDA, "stream creation failed");
    }
    for (int i = 0; i < 6; i++) cudaEventCreate(&h->ev[i]);
    *out = h;
    return VGPU_OK;
}

int vgpu_container_destroy(vgpu_container *h) {
    if (!h) return VGPU_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    DevBuf *bufs[] = {&h->ids_in, &h->xyzr_in, &h->rem, &h->ukey, &h->gkey, &h->idx, &h->idx2, &h->keys_alt,
                      &h->vals_alt, &h->hist, &h->scan_tmp, &h->outpos_in, &h->kept, &h->p64,
                      &h->lffh, &h->lffl, &h->pid,
                      &h->outpos, &h->gblock, &h->bstart, &h->offsets, &h->ovf_list, &h->ovf_list2, &h->counters, &h->counters2,
                      &h->r_vol, &h->r_cen, &h->r_nf, &h->r_nv, &h->r_mr2, &h->r_flags, &h->r_nb, &h->r_nb_ovf, &h->r_ids,
                      &h->loc_q, &h->loc_found, &h->loc_pid, &h->loc_r, &h->gh_p64, &h->gh_lffh, &h->gh_lffl,
                      &h->gh_pid, &h->gh_gblock, &h->gh_outpos, &h->gh_rec_off, &h->gh_q, &h->gh_keep, &h->gh_list,
                      &h->gh_ovf, &h->gh_ovf2, &h->gh_cnt, &h->gh_vol, &h->gh_cen, &h->gh_nf, &h->gh_nv, &h->gh_mr2, &h->gh_flags,
                      &h->gh_nb, &h->gh_nb_ovf, &h->gh_nb_off, &h->gh_nb_out, &h->gh_poly, &h->gh_poly_off,
                      &h->walls_dev,
                      &h->r_pos, &h->r_rad, &h->rec_off, &h->poly, &h->poly_off, &h->nb_off, &h->nb_out, &h->nb_tmp, &h->sum_tmp,
                      &h->chk, &h->cell_list, &h->img_cnt, &h->img_off, &h->img_src, &h->x_gkey, &h->x_idx,
                      &h->x_kalt, &h->x_rem, &h->x_valt};
    for (DevBuf *b : bufs) b->release();
    if (h->host_rb) cudaFreeHost(h->host_rb);
    for (int i = 0; i < 6; i++) cudaEventDestroy(h->ev[i]);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return VGPU_OK;
}

}  // extern "C"


extern "C" {

int vgpu_put(vgpu_container *h, int64_t n, const int32_t *ids, const double *xyzr) {
    if (!h || n < 0 || (n > 0 && (!ids || !xyzr))) return fail(VGPU_ERR_ARG, "bad put arguments");
    if (h->use_device_input) {
        h->use_device_input = false;
        h->dev_ids_ext = nullptr;
        h->dev_xyzr_ext = nullptr;
        h->dev_n_ext = 0;
        h->staged = 0;
    }
    if (n == 0) return VGPU_OK;
    if (h->staged + n > (int64_t)INT32_MAX / 2) return fail(VGPU_ERR_MEMORY, "too many particles");
    const size_t want = (size_t)(h->staged + n);
    if (want * 32 > h->xyzr_in.bytes || want * 4 > h->ids_in.bytes) {
        // grow the device staging area, keeping what is already there
        DevBuf ni, nx;
        size_t cap = std::max(want, (size_t)(h->staged * 2));
        VG_CUDA(ni.ensure(cap * 4));
        VG_CUDA(nx.ensure(cap * 32));
        if (h->staged > 0) {
            VG_CUDA(cudaMemcpyAsync(ni.p, h->ids_in.p, (size_t)h->staged * 4, cudaMemcpyDeviceToDevice, h->stream));
            VG_CUDA(cudaMemcpyAsync(nx.p, h->xyzr_in.p, (size_t)h->staged * 32, cudaMemcpyDeviceToDevice, h->stream));
            VG_CUDA(cudaStreamSynchronize(h->stream));
        }
        h->ids_in.release();
        h->xyzr_in.release();
        h->ids_in = ni;
        h->xyzr_in = nx;
        ni.p = nx.p = nullptr;
    }
    // synchronous with respect to the caller's arrays: they may be reused on return
    VG_CUDA(cudaMemcpyAsync(h->ids_in.as<int32_t>() + h->staged, ids, (size_t)n * 4, cudaMemcpyHostToDevice,
                            h->stream));
    VG_CUDA(cudaMemcpyAsync(h->xyzr_in.as<double>() + 4 * h->staged, xyzr, (size_t)n * 32,
                            cudaMemcpyHostToDevice, h->stream));
    // non-finite input is rejected here, by a scan of what was just copied
    // (on the device: the host's one-thread scan of 4M particles took longer
    // than the copy); the staged count does not advance, so nothing of this
    // call is kept
    VG_CUDA(h->chk.ensure(sizeof(unsigned long long)));
    VG_CUDA(cudaMemsetAsync(h->chk.p, 0xff, sizeof(unsigned long long), h->stream));
    VG_CUDA(launch_first_nonfinite(h->xyzr_in.as<double>() + 4 * h->staged, n, h->g.poly,
                                   h->chk.as<unsigned long long>(), h->stream));
    unsigned long long bad = ~0ull;
    VG_CUDA(cudaMemcpyAsync(&bad, h->chk.p, sizeof(bad), cudaMemcpyDeviceToHost, h->stream));
    VG_CUDA(cudaStreamSynchronize(h->stream));
    if (bad != ~0ull)
        return fail(VGPU_ERR_ARG, "particle %lld (id %d) has a non-finite position or radius", (long long)bad,
                    (int)ids[bad]);
    h->staged += n;
    h->computed = false;
    h->binned = false;
    return VGPU_OK;
}

int vgpu_put_device(vgpu_container *h, int64_t n, const int32_t *dev_ids, const double *dev_xyzr) {
    if (!h || n < 0 || (n > 0 && (!dev_ids || !dev_xyzr))) return fail(VGPU_ERR_ARG, "bad put_device arguments");
    if (n > (int64_t)INT32_MAX / 2) return fail(VGPU_ERR_MEMORY, "too many particles");
    h->staged = 0;
    h->use_device_input = true;
    h->dev_ids_ext = dev_ids;
    h->dev_xyzr_ext = dev_xyzr;
    h->dev_n_ext = n;
    h->computed = false;
    h->binned = false;
    return VGPU_OK;
}

int vgpu_clear(vgpu_container *h) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    h->staged = 0;
    h->use_device_input = false;
    h->dev_ids_ext = nullptr;
    h->dev_xyzr_ext = nullptr;
    h->dev_n_ext = 0;
    h->computed = false;
    h->binned = false;
    h->ncells = 0;
    return VGPU_OK;
}

int vgpu_add_wall(vgpu_container *h, int type, const double params[7], int id) {
    if (!h || !params) return fail(VGPU_ERR_ARG, "null argument");
    if (h->g.unit_cell) return fail(VGPU_ERR_UNSUPPORTED, "walls belong to container / container_poly only");
    if (type < VGPU_WALL_SPHERE || type > VGPU_WALL_CONE) return fail(VGPU_ERR_ARG, "unknown wall type %d", type);
    if ((int)h->walls.size() >= kMaxWalls) return fail(VGPU_ERR_ARG, "at most %d walls", kMaxWalls);
    WallSpec w;
    memset(&w, 0, sizeof(w));
    w.type = type;
    w.id = id;
    for (int a = 0; a < 3; a++) w.c[a] = params[a];
    if (type == VGPU_WALL_SPHERE || type == VGPU_WALL_PLANE) {
        w.r = params[3];
    } else {
        // the constructors' precomputed terms (src/wall.hh:76-105)
        for (int a = 0; a < 3; a++) w.a[a] = params[3 + a];
        w.asi = 1 / (params[3] * params[3] + params[4] * params[4] + params[5] * params[5]);
        if (type == VGPU_WALL_CYLINDER) {
            w.r = params[6];
        } else {
            w.gra = std::tan(params[6]);
            w.sang = std::sin(params[6]);
            w.cang = std::cos(params[6]);
        }
    }
    h->walls.push_back(w);
    h->walls_dirty = true;
    h->computed = false;
    return VGPU_OK;
}

int vgpu_clear_walls(vgpu_container *h) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    h->walls.clear();
    h->walls_dirty = true;
    h->computed = false;
    return VGPU_OK;
}

// point_inside (src/wall.cc:17-95) of every wall
int vgpu_point_inside_walls(vgpu_container *h, double x, double y, double z, int *inside) {
    if (!h || !inside) return fail(VGPU_ERR_ARG, "null argument");
    *inside = 1;
    for (const WallSpec &w : h->walls) {
        bool in;
        if (w.type == VGPU_WALL_SPHERE) {
            in = (x - w.c[0]) * (x - w.c[0]) + (y - w.c[1]) * (y - w.c[1]) + (z - w.c[2]) * (z - w.c[2]) < w.r * w.r;
        } else if (w.type == VGPU_WALL_PLANE) {
            in = x * w.c[0] + y * w.c[1] + z * w.c[2] < w.r;
        } else {
            double xd = x - w.c[0], yd = y - w.c[1], zd = z - w.c[2];
            double pa = (xd * w.a[0] + yd * w.a[1] + zd * w.a[2]) * w.asi;
            xd -= w.a[0] * pa;
            yd -= w.a[1] * pa;
            zd -= w.a[2] * pa;
            if (w.type == VGPU_WALL_CYLINDER) {
                in = xd * xd + yd * yd + zd * zd < w.r * w.r;
            } else {
                pa *= w.gra;
                in = pa >= 0 && xd * xd + yd * yd + zd * zd < pa * pa;
            }
        }
        if (!in) {
            *inside = 0;
            break;
        }
    }
    return VGPU_OK;
}

int vgpu_set_ghost_depth(vgpu_container *h, double spacings) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    if (!std::isfinite(spacings)) return fail(VGPU_ERR_ARG, "ghost depth must be finite");
    const double v = spacings == 0 ? 8.0 : spacings;
    if (v != h->ghost_spacings) {
        h->ghost_spacings = v;
        h->binned = false;
    }
    return VGPU_OK;
}

int vgpu_set_fp64_fallback(vgpu_container *h, double fraction) {
    if (!h || !(fraction >= 0.0)) return fail(VGPU_ERR_ARG, "bad fallback fraction");
    h->fp64_fallback = fraction;
    return VGPU_OK;
}

int vgpu_get_tolerance(vgpu_container *h, double *tol) {
    if (!h || !tol) return fail(VGPU_ERR_ARG, "null argument");
    *tol = 2.0 * h->g.tol_h;   // tol_h holds half of it (exact in binary)
    return VGPU_OK;
}

int vgpu_set_record_budget(vgpu_container *h, int64_t bytes) {
    if (!h || bytes < 0) return fail(VGPU_ERR_ARG, "bad record budget");
    h->record_bytes = bytes;
    return VGPU_OK;
}

int vgpu_set_tuning(vgpu_container *h, double particles_per_block, int warps_per_cta) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    if (particles_per_block > 0 && particles_per_block != h->target_density) {
        h->target_density = particles_per_block;
        h->binned = false;   // the engine grid changes
    }
    if (warps_per_cta > 8) return fail(VGPU_ERR_ARG, "at most 8 warps per CTA (got %d)", warps_per_cta);
    if (warps_per_cta > 0) h->warps_per_cta = warps_per_cta;
    return VGPU_OK;
}

}  // extern "C"

namespace {

void fill_cell_params(vgpu_container *h, CellParams &cp);

// Everything of a compute before the cell kernel: remap, loop-order sort,
// duplicate check, engine-order sort and gather; fills cp for the engine.
// Leaves the gather queued on the handle's stream (event ev[1] after it).
// The walls' device copy, when they changed since the last upload.
int upload_walls(vgpu_container *h) {
    if (!h->walls_dirty) return VGPU_OK;
    std::vector<WallSpec> all(h->walls);
    all.insert(all.end(), h->lattice.begin(), h->lattice.end());
    if ((int)all.size() > kMaxWalls) return fail(VGPU_ERR_ARG, "at most %d walls", kMaxWalls);
    if (!all.empty()) {
        VG_CUDA(h->walls_dev.ensure(all.size() * sizeof(WallSpec)));
        VG_CUDA(cudaMemcpyAsync(h->walls_dev.p, all.data(), all.size() * sizeof(WallSpec), cudaMemcpyHostToDevice,
                                h->stream));
        VG_CUDA(cudaStreamSynchronize(h->stream));
    }
    h->walls_dirty = false;
    return VGPU_OK;
}

// thin: a sheared periodic box may store its images only ghost_spacings mean
// particle spacings deep (a compute checks afterwards that every cell's reach
// stayed inside; see reach_check_kernel); else at the reference's depth.
// Binning runs in two parts around its one wait for the device: bin_begin
// enqueues the remap and the read-back of its counts (into pinned memory),
// bin_finish (once the container's stream has reached them) the sorts, the
// gather and the engine's parameters.  A batch begins every large member
// before it finishes any, so that their remaps run together instead of one
// host round trip after another.
int bin_begin(vgpu_container *h, int mode, bool thin) {
    if (mode != VGPU_FP64 && mode != VGPU_MIXED) return fail(VGPU_ERR_ARG, "bad mode %d", mode);
    if (int rc = upload_walls(h)) return rc;
    cudaStream_t s = h->stream;
    const int64_t n64 = h->use_device_input ? h->dev_n_ext : h->staged;
    const int n = (int)n64;
    Geometry &g = h->g;
    memset(&h->stats, 0, sizeof(h->stats));
    h->computed = false;
    if (g.tric) {
        h->tric_thin = false;
        const double sp = std::cbrt(g.len[0] * g.len[1] * g.len[2] / (double)std::max<int64_t>(n64, 1));
        for (int a = 1; a < 3; a++) {
            g.lo[a] = h->full_lo[a];
            g.ext[a] = h->full_ext[a];
            const double d = h->ghost_spacings * sp;
            if (thin && h->ghost_spacings >= 0 && d < -h->full_lo[a]) {
                g.lo[a] = -d;
                g.ext[a] = g.len[a] + 2.0 * d;
                h->tric_thin = true;
            }
        }
    }
    choose_engine_grid(g, n64, h->target_density);
    const int nblocks = g.gn[0] * g.gn[1] * g.gn[2];
    const size_t nn = (size_t)std::max(n, 1);
    // inputs
    const int32_t *d_ids;
    const double *d_xyzr;
    if (h->use_device_input) {
        d_ids = h->dev_ids_ext;
        d_xyzr = h->dev_xyzr_ext;
    } else {
        VG_CUDA(h->ids_in.ensure(nn * 4));
        VG_CUDA(h->xyzr_in.ensure(nn * 32));
        d_ids = h->ids_in.as<int32_t>();
        d_xyzr = h->xyzr_in.as<double>();
    }
    if ((reinterpret_cast<uintptr_t>(d_xyzr) & 15u) != 0)
        return fail(VGPU_ERR_ARG, "device xyzr must be 16-byte aligned");

    // work buffers
    size_t scan_n = scan_tmp_ints(std::max<int>((int)radix_hist_ints(n), nblocks + 1)) + 64;
    VG_CUDA(h->rem.ensure(nn * 32));
    VG_CUDA(h->ukey.ensure(nn * 4));
    VG_CUDA(h->gkey.ensure(nn * 4));
    VG_CUDA(h->idx.ensure((nn + 1) * 4));
    VG_CUDA(h->idx2.ensure(nn * 4));
    VG_CUDA(h->keys_alt.ensure(nn * 4));
    VG_CUDA(h->vals_alt.ensure(nn * 4));
    VG_CUDA(h->hist.ensure(radix_hist_ints(n) * 4));
    VG_CUDA(h->scan_tmp.ensure(scan_n * 8));
    VG_CUDA(h->outpos_in.ensure(nn * 4));
    VG_CUDA(h->kept.ensure(64));
    VG_CUDA(h->counters.ensure(sizeof(Counters)));
    VG_CUDA(h->counters2.ensure(2 * sizeof(Counters)));

    h->launches0 = launch_count();
    cudaEventRecord(h->ev[0], s);
    VG_CUDA(cudaMemsetAsync(h->kept.p, 0, 64, s));
    if (n > 0) VG_CUDA(cudaMemsetAsync(h->outpos_in.p, 0xff, (size_t)n * 4, s));   // -1: dropped by put()
    BinParams bp;
    bp.g = g;
    bp.n = n;
    bp.ids_in = d_ids;
    bp.xyzr_in = reinterpret_cast<const double4 *>(d_xyzr);
    bp.rem = h->rem.as<double4>();
    bp.ukey = h->ukey.as<unsigned>();
    bp.gkey = h->gkey.as<unsigned>();
    bp.idx = h->idx.as<int>();
    int *d_kept = h->kept.as<int>();
    unsigned long long *d_rmax = reinterpret_cast<unsigned long long *>(h->kept.as<char>() + 16);
    VG_CUDA(launch_remap(bp, d_kept, d_rmax, s));
    if (!h->host_rb) VG_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&h->host_rb), 64, cudaHostAllocDefault));
    // kept particles and particles with a non-finite position or radius
    // (two ints), then the largest radius
    VG_CUDA(cudaMemcpyAsync(h->host_rb, d_kept, 8, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaMemcpyAsync(h->host_rb + 1, d_rmax, 8, cudaMemcpyDeviceToHost, s));
    // identity copy for the second sort
    if (n > 0) VG_CUDA(cudaMemcpyAsync(h->idx2.p, h->idx.p, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    return VGPU_OK;
}

// The rest of the binning, after bin_begin's read-back has landed (the
// caller synchronised the container's stream).  defer_dup: the duplicate
// check's flag is read back without waiting (dup_pending; the caller checks
// it after its next synchronisation) instead of being waited for here.
int bin_finish(vgpu_container *h, int mode, CellParams &cp, bool defer_dup) {
    (void)mode;
    cudaStream_t s = h->stream;
    const int64_t n64 = h->use_device_input ? h->dev_n_ext : h->staged;
    const int n = (int)n64;
    Geometry &g = h->g;
    const int nblocks = g.gn[0] * g.gn[1] * g.gn[2];
    const int nub = g.un[0] * g.un[1] * g.un[2];
    const size_t nn = (size_t)std::max(n, 1);
    const int32_t *d_ids = h->use_device_input ? h->dev_ids_ext : h->ids_in.as<int32_t>();
    int kept2[2];
    memcpy(kept2, h->host_rb, 8);
    if (kept2[1] > 0)
        return fail(VGPU_ERR_ARG, "%d particles have a non-finite position or radius", kept2[1]);
    const int nkept = kept2[0];
    double rmax = 0.0;
    memcpy(&rmax, h->host_rb + 1, 8);
    g.rmax = rmax;
    g.rmax32 = (float)rmax * (1.0f + 1e-6f);
    h->dup_pending = false;

    int ubits = 1, gbits = 1;
    while ((1u << ubits) <= (unsigned)nub) ubits++;
    while ((1u << gbits) <= (unsigned)nblocks) gbits++;
    ubits = (ubits + 7) / 8 * 8;
    gbits = (gbits + 7) / 8 * 8;
    bool alt = false;
    VG_CUDA(radix_sort_pairs(h->ukey.as<unsigned>(), h->idx.as<int>(), h->keys_alt.as<unsigned>(),
                             h->vals_alt.as<int>(), n, ubits, h->hist.as<int>(), h->hist.bytes / 4,
                             h->scan_tmp.as<int>(), h->scan_tmp.bytes / 4, s, &alt));
    const unsigned *ukey_sorted = alt ? h->keys_alt.as<unsigned>() : h->ukey.as<unsigned>();
    const int *uorder = alt ? h->vals_alt.as<int>() : h->idx.as<int>();

    // sheared periodic boxes: the images in the ghost layers, counted per
    // particle (every particle is kept), then written after the particles
    int nengine = nkept;
    if (g.tric && n > 0) {
        VG_CUDA(h->img_cnt.ensure(nn * 4));
        VG_CUDA(h->img_off.ensure(nn * 4));
        VG_CUDA(h->scan_tmp.ensure((scan_tmp_ints(n) + 64) * 8));
        VG_CUDA(launch_image_count(g, n, h->rem.as<double4>(), h->img_cnt.as<int>(), s));
        VG_CUDA(exclusive_scan_int(h->img_cnt.as<int>(), h->img_off.as<int>(), n, h->scan_tmp.as<int>(),
                                   h->scan_tmp.bytes / 4, s));
        int last[2] = {0, 0};
        VG_CUDA(cudaMemcpyAsync(&last[0], h->img_cnt.as<int>() + (n - 1), 4, cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaMemcpyAsync(&last[1], h->img_off.as<int>() + (n - 1), 4, cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
        const long long total = (long long)n + last[0] + last[1];
        if (total > (long long)INT32_MAX / 2) return fail(VGPU_ERR_MEMORY, "too many periodic images");
        nengine = (int)total;
    }
    h->nengine = nengine;

    // results arrays
    const size_t nk = (size_t)std::max(nkept, 1);
    const size_t ne = (size_t)std::max(nengine, 1);
    VG_CUDA(h->r_vol.ensure(nk * 8));
    VG_CUDA(h->r_cen.ensure(nk * 24));
    VG_CUDA(h->r_nf.ensure(nk * 4));
    VG_CUDA(h->r_nv.ensure(nk * 4));
    VG_CUDA(h->r_mr2.ensure(nk * 8));
    VG_CUDA(h->r_flags.ensure(nk * 4));
    VG_CUDA(h->r_nb.ensure(nk * kNbStride * 4));
    VG_CUDA(h->r_nb_ovf.ensure(nb_ovf_ints(nk) * 4));
    VG_CUDA(h->r_ids.ensure(nk * 4));
    VG_CUDA(h->r_pos.ensure(nk * 24));
    VG_CUDA(h->r_rad.ensure(nk * 8));
    VG_CUDA(h->p64.ensure(ne * 32));
    VG_CUDA(h->lffh.ensure(ne * 16));
    VG_CUDA(h->lffl.ensure(ne * 16));
    VG_CUDA(h->pid.ensure(ne * 4));
    VG_CUDA(h->outpos.ensure(ne * 4));
    VG_CUDA(h->gblock.ensure(ne * 4));
    VG_CUDA(h->bstart.ensure(((size_t)nblocks + 2) * 4));
    VG_CUDA(h->ovf_list.ensure(nk * 4));

    if (g.unit_cell && nkept > 1) {
        int *dflag = h->kept.as<int>() + 8;
        VG_CUDA(cudaMemsetAsync(dflag, 0, 4, s));
        VG_CUDA(launch_duplicate_check(ukey_sorted, uorder, h->rem.as<double4>(), nkept, dflag, s));
        h->host_rb[2] = 0;
        VG_CUDA(cudaMemcpyAsync(h->host_rb + 2, dflag, 4, cudaMemcpyDeviceToHost, s));
        if (defer_dup) {
            h->dup_pending = true;
        } else {
            VG_CUDA(cudaStreamSynchronize(s));
            if (h->host_rb[2]) return fail(VGPU_ERR_DUPLICATE, "duplicate particle positions (|d|^2 < 1e-10) in one block");
        }
    }

    // engine order: the u-sort consumed idx, so sort (gkey, idx2)
    bool galt = false;
    const unsigned *gkey_sorted;
    const int *gorder;
    const double4 *erem = h->rem.as<double4>();
    const int *img_src = nullptr;
    if (g.tric && n > 0) {
        // the particles and their images, in buffers of their own
        const size_t nx = (size_t)nengine;
        VG_CUDA(h->x_rem.ensure(nx * 32));
        VG_CUDA(h->x_gkey.ensure(nx * 4));
        VG_CUDA(h->x_idx.ensure(nx * 4));
        VG_CUDA(h->x_kalt.ensure(nx * 4));
        VG_CUDA(h->x_valt.ensure(nx * 4));
        VG_CUDA(h->img_src.ensure(std::max<size_t>(nx - (size_t)n, 1) * 4));
        VG_CUDA(h->hist.ensure(radix_hist_ints(nengine) * 4));
        const size_t xscan = scan_tmp_ints(std::max<int>((int)radix_hist_ints(nengine), nblocks + 1)) + 64;
        VG_CUDA(h->scan_tmp.ensure(xscan * 8));
        VG_CUDA(cudaMemcpyAsync(h->x_rem.p, h->rem.p, (size_t)n * 32, cudaMemcpyDeviceToDevice, s));
        VG_CUDA(cudaMemcpyAsync(h->x_gkey.p, h->gkey.p, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        VG_CUDA(cudaMemcpyAsync(h->x_idx.p, h->idx2.p, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        VG_CUDA(launch_image_write(g, n, h->rem.as<double4>(), h->img_off.as<int>(), n, h->x_rem.as<double4>(),
                                   h->x_gkey.as<unsigned>(), h->x_idx.as<int>(), h->img_src.as<int>(), s));
        VG_CUDA(radix_sort_pairs(h->x_gkey.as<unsigned>(), h->x_idx.as<int>(), h->x_kalt.as<unsigned>(),
                                 h->x_valt.as<int>(), nengine, gbits, h->hist.as<int>(), h->hist.bytes / 4,
                                 h->scan_tmp.as<int>(), h->scan_tmp.bytes / 4, s, &galt));
        gkey_sorted = galt ? h->x_kalt.as<unsigned>() : h->x_gkey.as<unsigned>();
        gorder = galt ? h->x_valt.as<int>() : h->x_idx.as<int>();
        erem = h->x_rem.as<double4>();
        img_src = h->img_src.as<int>();
    } else {
        unsigned *gk_alt = alt ? h->ukey.as<unsigned>() : h->keys_alt.as<unsigned>();
        int *gv_alt = alt ? h->idx.as<int>() : h->vals_alt.as<int>();
        // keep uorder intact: the g-sort ping-pongs between gkey/idx2 and the buffers not holding uorder
        VG_CUDA(radix_sort_pairs(h->gkey.as<unsigned>(), h->idx2.as<int>(), gk_alt, gv_alt, n, gbits,
                                 h->hist.as<int>(), h->hist.bytes / 4, h->scan_tmp.as<int>(), h->scan_tmp.bytes / 4,
                                 s, &galt));
        gkey_sorted = galt ? gk_alt : h->gkey.as<unsigned>();
        gorder = galt ? gv_alt : h->idx2.as<int>();
        if (galt && (gk_alt == (const unsigned *)ukey_sorted || gv_alt == uorder))
            return fail(VGPU_ERR_INTERNAL, "sort buffer aliasing");
    }

    VG_CUDA(launch_gather(g, nkept, nengine, n, img_src, uorder, gorder, gkey_sorted, erem, d_ids,
                          h->outpos_in.as<int>(), h->p64.as<double4>(), h->lffh.as<float4>(),
                          h->lffl.as<float4>(), h->pid.as<int>(),
                          h->outpos.as<int>(), h->gblock.as<int>(), h->bstart.as<int>(), nblocks,
                          h->r_ids.as<int>(), h->r_pos.as<double>(), h->r_rad.as<double>(), s));
    if (g.tric) {   // the cells to compute: the particles, not their images, in engine order
        VG_CUDA(h->cell_list.ensure(nk * 4));
        VG_CUDA(h->scan_tmp.ensure((scan_tmp_ints(nengine) + 64) * 8));
        // (the sort buffers x_idx and x_gkey are free once the gather has run)
        VG_CUDA(launch_cell_list(h->outpos.as<int>(), nengine, h->cell_list.as<int>(), h->x_idx.as<int>(),
                                 h->x_gkey.as<int>(), h->scan_tmp.as<int>(), h->scan_tmp.bytes / 4, s));
    }
    cudaEventRecord(h->ev[1], s);

    // cell engine parameters
    const OffsetTable &ot = offset_table();
    VG_CUDA(h->offsets.ensure(ot.codes.size() * 4));
    VG_CUDA(cudaMemcpyAsync(h->offsets.p, ot.codes.data(), ot.codes.size() * 4, cudaMemcpyHostToDevice, s));
    VG_CUDA(cudaMemsetAsync(h->counters.p, 0, sizeof(Counters), s));
    VG_CUDA(cudaMemsetAsync(h->counters2.p, 0, 2 * sizeof(Counters), s));
    h->nkept = nkept;
    h->binned = true;
    fill_cell_params(h, cp);
    return VGPU_OK;
}

int prepare_cells(vgpu_container *h, int mode, CellParams &cp, bool thin = false) {
    int rc = bin_begin(h, mode, thin);
    if (rc != VGPU_OK) return rc;
    VG_CUDA(cudaStreamSynchronize(h->stream));
    return bin_finish(h, mode, cp, false);
}

// The cell engine's parameters for the binned container h (h->nkept set).
void fill_cell_params(vgpu_container *h, CellParams &cp) {
    const OffsetTable &ot = offset_table();
    const Geometry &g = h->g;
    const int nkept = h->nkept;
    memset(&cp, 0, sizeof(cp));
    cp.cell_chunk = h->cell_chunk;
    cp.g = g;
    cp.a.p64 = h->p64.as<double4>();
    cp.a.l32 = h->lffh.as<float4>();
    cp.a.lffh = h->lffh.as<float4>();
    cp.a.lffl = h->lffl.as<float4>();
    cp.a.pid = h->pid.as<int>();
    cp.a.outpos = h->outpos.as<int>();
    cp.a.gblock = h->gblock.as<int>();
    cp.a.bstart = h->bstart.as<int>();
    cp.r.vol = h->r_vol.as<double>();
    cp.r.cen = h->r_cen.as<double>();
    cp.r.nf = h->r_nf.as<int>();
    cp.r.nv = h->r_nv.as<int>();
    cp.r.maxr2 = h->r_mr2.as<double>();
    cp.r.flags = h->r_flags.as<int>();
    cp.r.nb = h->r_nb.as<int>();
    cp.r.nb_ovf = h->r_nb_ovf.as<int>();
    cp.r.nb_ovf_cap = nb_ovf_ints((size_t)std::max(nkept, 1));
    cp.cnt = h->counters.as<Counters>();
    cp.ncells = nkept;
    cp.cell_list = g.tric ? h->cell_list.as<int>() : nullptr;
    cp.overflow_list = h->ovf_list.as<int>();
    cp.offsets = h->offsets.as<int>();
    cp.noffsets = (int)ot.codes.size();
    cp.ngroups = (int)ot.group_lb2.size();
    for (int i = 0; i <= cp.ngroups; i++) cp.group_start[i] = ot.group_start[i];
    for (int i = 0; i < cp.ngroups; i++) cp.group_lb2[i] = ot.group_lb2[i];
    box_tables(cp.box_tri, cp.box_adj);
    // A sheared box binned with thin ghost layers leaves out the unit cell's
    // face planes: a cell they could cut reaches half a lattice vector, past
    // the layers, and the reach check reruns the compute at full depth (with
    // them); a lattice vector shorter than the layers' depth has its image
    // stored, whose plane is the same.
    cp.nwalls = (int)(h->walls.size() + (h->g.tric && h->tric_thin ? 0 : h->lattice.size()));
    cp.walls = cp.nwalls == 0 ? nullptr : h->walls_dev.as<WallSpec>();
}

// A batch member of at most kSmallBinMax particles is binned by one CTA of
// small_bin_kernel: its buffers are sized for every particle (the number
// kept is known only afterwards) and its job filled here; no launch.
int prepare_small(vgpu_container *h, int mode, SmallBinJob &job, unsigned long long *result) {
    if (mode != VGPU_FP64 && mode != VGPU_MIXED) return fail(VGPU_ERR_ARG, "bad mode %d", mode);
    if (int rc = upload_walls(h)) return rc;
    const int64_t n64 = h->use_device_input ? h->dev_n_ext : h->staged;
    const int n = (int)n64;
    Geometry &g = h->g;
    memset(&h->stats, 0, sizeof(h->stats));
    h->computed = false;
    choose_engine_grid(g, n64, h->target_density);
    const int nblocks = g.gn[0] * g.gn[1] * g.gn[2];
    const size_t nn = (size_t)std::max(n, 1);
    const int32_t *d_ids = h->use_device_input ? h->dev_ids_ext : h->ids_in.as<int32_t>();
    const double *d_xyzr = h->use_device_input ? h->dev_xyzr_ext : h->xyzr_in.as<double>();
    if (n > 0 && (!d_ids || !d_xyzr)) return fail(VGPU_ERR_INTERNAL, "container inputs missing");
    if ((reinterpret_cast<uintptr_t>(d_xyzr) & 15u) != 0)
        return fail(VGPU_ERR_ARG, "device xyzr must be 16-byte aligned");
    VG_CUDA(h->rem.ensure(nn * 32));
    VG_CUDA(h->outpos_in.ensure(nn * 4));
    VG_CUDA(h->counters.ensure(sizeof(Counters)));
    VG_CUDA(h->counters2.ensure(2 * sizeof(Counters)));
    VG_CUDA(h->r_vol.ensure(nn * 8));
    VG_CUDA(h->r_cen.ensure(nn * 24));
    VG_CUDA(h->r_nf.ensure(nn * 4));
    VG_CUDA(h->r_nv.ensure(nn * 4));
    VG_CUDA(h->r_mr2.ensure(nn * 8));
    VG_CUDA(h->r_flags.ensure(nn * 4));
    VG_CUDA(h->r_nb.ensure(nn * kNbStride * 4));
    VG_CUDA(h->r_nb_ovf.ensure(nb_ovf_ints(nn) * 4));
    VG_CUDA(h->r_ids.ensure(nn * 4));
    VG_CUDA(h->r_pos.ensure(nn * 24));
    VG_CUDA(h->r_rad.ensure(nn * 8));
    VG_CUDA(h->p64.ensure(nn * 32));
    VG_CUDA(h->lffh.ensure(nn * 16));
    VG_CUDA(h->lffl.ensure(nn * 16));
    VG_CUDA(h->pid.ensure(nn * 4));
    VG_CUDA(h->outpos.ensure(nn * 4));
    VG_CUDA(h->gblock.ensure(nn * 4));
    VG_CUDA(h->bstart.ensure(((size_t)nblocks + 2) * 4));
    VG_CUDA(h->ovf_list.ensure(nn * 4));
    memset(&job, 0, sizeof(job));
    job.g = g;
    job.n = n;
    job.nub = g.un[0] * g.un[1] * g.un[2];
    job.nblocks = nblocks;
    job.ids_in = d_ids;
    job.xyzr_in = reinterpret_cast<const double4 *>(d_xyzr);
    job.rem = h->rem.as<double4>();
    job.outpos_in = h->outpos_in.as<int>();
    job.p64 = h->p64.as<double4>();
    job.lffh = h->lffh.as<float4>();
    job.lffl = h->lffl.as<float4>();
    job.pid = h->pid.as<int>();
    job.outpos = h->outpos.as<int>();
    job.gblock = h->gblock.as<int>();
    job.bstart = h->bstart.as<int>();
    job.res_ids = h->r_ids.as<int>();
    job.res_pos = h->r_pos.as<double>();
    job.res_rad = h->r_rad.as<double>();
    job.result = result;
    h->launches0 = launch_count();
    return VGPU_OK;
}

// After small_bin_kernel: the kept count, largest radius and duplicate flag of h.
int finish_small(vgpu_container *h, const unsigned long long res[2]) {
    if ((res[0] >> 33) & 1ull) return fail(VGPU_ERR_ARG, "a particle has a non-finite position or radius");
    if ((res[0] >> 32) & 1ull) return fail(VGPU_ERR_DUPLICATE, "duplicate particle positions (|d|^2 < 1e-10) in one block");
    h->nkept = (int)(res[0] & 0xffffffffu);
    h->nengine = h->nkept;
    h->binned = true;
    double rmax = 0.0;
    memcpy(&rmax, &res[1], 8);
    h->g.rmax = rmax;
    h->g.rmax32 = (float)rmax * (1.0f + 1e-6f);
    return VGPU_OK;
}

// The record store: scratch between the clipping kernels and the finish
// kernel of one compute, shared by all containers of a device so that many
// containers hold no records between computes.  A compute holds it (mutex)
// from before its first clipping launch until its finish kernel completed.
struct RecordStore {
    std::mutex m;
    DevBuf buf;
};
RecordStore &record_store(int device) {
    static RecordStore stores[64];
    return stores[device & 63];
}

// The record store (held by the caller) as the clipping kernels' output,
// and the optional polytope output, for the compute of h described by cp;
// the offset arrays are reset on stream s.
int setup_records(vgpu_container *h, int mode, CellParams &cp, Counters *cnt, cudaStream_t s, DevBuf &store) {
    cp.rec = nullptr;
    cp.poly = nullptr;
    if (h->nkept <= 0) return VGPU_OK;
    unsigned long long cap = std::min<unsigned long long>(
        (unsigned long long)h->nkept * kRecWordsPerCell[mode == VGPU_MIXED ? 1 : 0] + (1u << 20), ~0ull >> 8);
    if (h->record_bytes > 0) cap = std::min<unsigned long long>(cap, (unsigned long long)h->record_bytes / 4);
    VG_CUDA(store.ensure(cap * 4));
    VG_CUDA(h->rec_off.ensure((size_t)h->nengine * 8));
    VG_CUDA(cudaMemsetAsync(h->rec_off.p, 0xff, (size_t)h->nengine * 8, s));
    cp.rec = store.as<unsigned>();
    cp.rec_cap = cap;
    cp.rec_used = &cnt->rec_used;
    cp.rec_off = h->rec_off.as<unsigned long long>();
    if (h->output & VGPU_OUTPUT_POLYTOPES) {
        const unsigned long long pcap = (unsigned long long)h->nkept * kPolyDoublesPerCell + (1u << 16);
        VG_CUDA(h->poly.ensure(pcap * 8));
        VG_CUDA(h->poly_off.ensure((size_t)h->nkept * 8));
        VG_CUDA(cudaMemsetAsync(h->poly_off.p, 0xff, (size_t)h->nkept * 8, s));
        cp.poly = h->poly.as<double>();
        cp.poly_cap = pcap;
        cp.poly_used = &cnt->poly_used;
        cp.poly_off = h->poly_off.as<long long>();
    }
    return VGPU_OK;
}

// A batch member's record offsets (reset) and optional polytope output; its
// records go to the batch's store (fields rec, rec_cap, rec_used set later).
int setup_member_records(vgpu_container *h, CellParams &cp, Counters *cnt, cudaStream_t s) {
    cp.rec = nullptr;
    cp.poly = nullptr;
    if (h->nkept <= 0) return VGPU_OK;
    // by engine index: the particles, then (sheared boxes) their images
    VG_CUDA(h->rec_off.ensure((size_t)h->nengine * 8));
    VG_CUDA(cudaMemsetAsync(h->rec_off.p, 0xff, (size_t)h->nengine * 8, s));
    cp.rec_off = h->rec_off.as<unsigned long long>();
    if (h->output & VGPU_OUTPUT_POLYTOPES) {
        const unsigned long long pcap = (unsigned long long)h->nkept * kPolyDoublesPerCell + (1u << 16);
        VG_CUDA(h->poly.ensure(pcap * 8));
        VG_CUDA(h->poly_off.ensure((size_t)h->nkept * 8));
        VG_CUDA(cudaMemsetAsync(h->poly_off.p, 0xff, (size_t)h->nkept * 8, s));
        cp.poly = h->poly.as<double>();
        cp.poly_cap = pcap;
        cp.poly_used = &cnt->poly_used;
        cp.poly_off = h->poly_off.as<long long>();
    }
    return VGPU_OK;
}

// Counters of the last compute into the handle's stats; marks it computed.
// The clipping passes over cp's cells (cp.cnt, cp.overflow_list: the first
// pass's counters and hand-on list).  MIXED: the FP64-free first pass, the
// full 64-slot engine on the cells it handed on (counters cnt1, hand-on
// list list2), then the 128-slot engine on what that handed on (cnt2).
// FP64: 64 slots, then 128 slots (cnt2).  sum: the passes' counters added,
// overflow = cells the first pass handed on, failed = cells the last pass
// run could not complete.
// first: cells at the start of cp's range whose first pass has already run
// (with the same counters, whose work counters the caller has reset).
// clip_passes' answer when a mixed first pass handed on more than switch_above
// of its cells (the caller reruns the container on the FP64 engine)
constexpr int kSwitchToFp64 = -1;

int clip_passes(cudaStream_t s, int sms, int warps, int mode, const CellParams &cp, Counters *cnt1, Counters *cnt2,
                int *list2, Counters &sum, int first = 0, double switch_above = -1.0) {
    Counters c[3];
    memset(c, 0, sizeof(c));
    CellParams p0 = cp;
    if (first > 0) {
        if (cp.cell_list) p0.cell_list = cp.cell_list + first;
        else p0.cell_begin = cp.cell_begin + first;
        p0.ncells = cp.ncells - first;
    }
    VG_CUDA(launch_cells(p0, mode, 0, sms, s, warps));
    VG_CUDA(cudaMemcpyAsync(&c[0], cp.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    unsigned long long pending = c[0].overflow;
    if (mode == VGPU_MIXED && switch_above >= 0.0 && (double)pending > switch_above * p0.ncells)
        return kSwitchToFp64;
    const int *list = cp.overflow_list;
    if (pending > 0 && mode == VGPU_MIXED) {
        CellParams p1 = cp;
        p1.cnt = cnt1;
        p1.ncells = (int)pending;
        p1.cell_list = list;
        p1.overflow_list = list2;
        VG_CUDA(launch_cells(p1, mode, 1, sms, s, warps));
        VG_CUDA(cudaMemcpyAsync(&c[1], cnt1, sizeof(Counters), cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
        pending = c[1].overflow;
        list = list2;
    }
    unsigned long long last_failed = 0;
    if (pending > 0) {
        CellParams p2 = cp;
        p2.cnt = cnt2;
        p2.ncells = (int)pending;
        p2.cell_list = list;
        p2.overflow_list = nullptr;
        VG_CUDA(launch_cells(p2, mode, 2, sms, s, warps));
        VG_CUDA(cudaMemcpyAsync(&c[2], cnt2, sizeof(Counters), cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
        last_failed = c[2].overflow;
    }
    sum = c[0];
    for (int k = 1; k < 3; k++) {
        sum.side_tests += c[k].side_tests;
        sum.fp64_repairs += c[k].fp64_repairs;
        sum.planes_tested += c[k].planes_tested;
        sum.planes_cut += c[k].planes_cut;
        sum.deleted += c[k].deleted;
        sum.marginal += c[k].marginal;
        sum.failed += c[k].failed;
        for (int i = 0; i < 16; i++) sum.phase_cycles[i] += c[k].phase_cycles[i];
    }
    sum.overflow = c[0].overflow;
    sum.failed += last_failed;
    return VGPU_OK;
}

// c: the compute's counters summed over its clipping passes, overflow = the
// cells the first pass handed on, failed = the cells no pass completed.
int finish_compute(vgpu_container *h, const Counters &c, float cell_ms) {
    float bin_ms = 0, step_ms = 0;
    cudaEventElapsedTime(&bin_ms, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&step_ms, h->ev[0], h->ev[3]);
    h->ncells = h->nkept;
    h->stats.cells = h->nkept;
    h->stats.deleted = (int64_t)c.deleted;
    h->stats.marginal_cells = (int64_t)c.marginal;
    h->stats.side_tests = (int64_t)c.side_tests;
    h->stats.fp64_repairs = (int64_t)c.fp64_repairs;
    h->stats.planes_tested = (int64_t)c.planes_tested;
    h->stats.planes_cut = (int64_t)c.planes_cut;
    h->stats.overflow_reruns = (int64_t)c.overflow;
    h->stats.failed_cells = (int64_t)(c.failed + c.nb_failed);
    for (int i = 0; i < 16; i++) h->phase[i] = (double)c.phase_cycles[i];
    h->stats.kernel_ms = cell_ms;
    h->stats.bin_ms = bin_ms;
    h->stats.step_ms = step_ms;
    h->stats.kernel_launches = launch_count() - h->launches0;
    h->computed = true;
    h->csr_valid = false;
    if (h->stats.failed_cells > 0)
        return fail(VGPU_ERR_CAPACITY, "%lld cells exceeded the engine capacity", (long long)h->stats.failed_cells);
    return VGPU_OK;
}

int compute_cells(vgpu_container *h, int mode, bool thin);

}  // namespace

extern "C" {

int vgpu_compute(vgpu_container *h, int mode) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    int rc = compute_cells(h, mode, true);
    if (h->g.tric && h->tric_thin && (rc == VGPU_OK || rc == VGPU_ERR_CAPACITY)) {
        // thin ghost layers: every cell's reach must lie inside them, else
        // again at the reference's depth
        int *flag = h->kept.as<int>() + 12;
        VG_CUDA(cudaMemsetAsync(flag, 0, 4, h->stream));
        VG_CUDA(launch_reach_check(h->g, h->nkept, h->r_pos.as<double>(), h->r_mr2.as<double>(),
                                   h->r_flags.as<int>(), flag, h->stream));
        int out = 0;
        VG_CUDA(cudaMemcpyAsync(&out, flag, 4, cudaMemcpyDeviceToHost, h->stream));
        VG_CUDA(cudaStreamSynchronize(h->stream));
        if (out) rc = compute_cells(h, mode, false);
    }
    return rc;
}

}  // extern "C"

namespace {

// One compute: binning (thin: a sheared box may store thin ghost layers),
// the clipping passes and the finish kernel.
// Mixed computes of containers of at least kSampleMinCells cells sample the
// FP64-free first pass on their first cells (engine order: a compact region);
// measured on the jittered 64^3 FCC lattice (1M cells), where every cell meets
// the FP32 filter band, the mixed engine ran at 6.9M cells/s and the FP64
// engine at 10.0M, while on uniform input 2.3 % of the cells are handed on.
constexpr int kSampleMinCells = 1 << 18;
constexpr int kSampleFraction = 64;

int compute_cells(vgpu_container *h, int mode, bool thin) {
    CellParams cp;
    int rc = prepare_cells(h, mode, cp, thin);
    if (rc != VGPU_OK) return rc;
    cudaStream_t s = h->stream;
    RecordStore &store = record_store(h->device);
    std::lock_guard<std::mutex> hold(store.m);
    rc = setup_records(h, mode, cp, h->counters.as<Counters>(), h->stream, store.buf);
    if (rc != VGPU_OK) return rc;
    // clipping (the passes of clip_passes), then the finish kernel over every record
    cudaEventRecord(h->ev[2], s);
    VG_CUDA(h->ovf_list2.ensure((size_t)std::max(h->nkept, 1) * 4));
    VG_CUDA(cudaMemsetAsync(h->counters2.p, 0, 2 * sizeof(Counters), s));
    int first = 0;
    bool switched = false;
    if (mode == VGPU_MIXED && h->fp64_fallback < 1.0 && cp.ncells >= kSampleMinCells) {
        CellParams ps = cp;
        ps.ncells = cp.ncells / kSampleFraction;
        VG_CUDA(launch_cells(ps, mode, 0, h->sms, s, h->warps_per_cta));
        Counters c0;
        VG_CUDA(cudaMemcpyAsync(&c0, cp.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
        if ((double)c0.overflow > h->fp64_fallback * ps.ncells) {
            // the filter band is saturated: the whole container on the FP64 engine
            mode = VGPU_FP64;
            switched = true;
            VG_CUDA(cudaMemsetAsync(cp.cnt, 0, sizeof(Counters), s));
            rc = setup_records(h, mode, cp, cp.cnt, s, store.buf);
            if (rc != VGPU_OK) return rc;
        } else {
            first = ps.ncells;   // the first pass continues after the sample
            // (a launch over a cell list, as a sheared box's, takes its work
            // from the second queue counter)
            VG_CUDA(cudaMemsetAsync(&cp.cnt->work, 0, sizeof(unsigned long long), s));
            VG_CUDA(cudaMemsetAsync(&cp.cnt->overflow_work, 0, sizeof(unsigned long long), s));
        }
    }
    Counters c1;
    // a container below the sampled size is assessed on its whole first pass:
    // with the band saturated (a lattice jittered at the tolerance's scale,
    // where the FP32 engine's band handling met its limits) it reruns on the
    // FP64 engine like a sampled one
    const bool whole_first = mode == VGPU_MIXED && h->fp64_fallback < 1.0 && cp.ncells < kSampleMinCells;
    rc = clip_passes(s, h->sms, h->warps_per_cta, mode, cp, h->counters2.as<Counters>(),
                     h->counters2.as<Counters>() + 1, h->ovf_list2.as<int>(), c1, first,
                     whole_first ? h->fp64_fallback : -1.0);
    if (rc == kSwitchToFp64) {
        mode = VGPU_FP64;
        switched = true;
        VG_CUDA(cudaMemsetAsync(cp.cnt, 0, sizeof(Counters), s));
        VG_CUDA(cudaMemsetAsync(h->counters2.p, 0, 2 * sizeof(Counters), s));
        rc = setup_records(h, mode, cp, cp.cnt, s, store.buf);
        if (rc != VGPU_OK) return rc;
        rc = clip_passes(s, h->sms, h->warps_per_cta, mode, cp, h->counters2.as<Counters>(),
                         h->counters2.as<Counters>() + 1, h->ovf_list2.as<int>(), c1, 0);
    }
    if (rc != VGPU_OK) return rc;
    cudaEventRecord(h->ev[4], s);
    VG_CUDA(launch_finish(cp, mode, h->sms, s));
    cudaEventRecord(h->ev[3], s);
    Counters c3;   // after the finish kernel: polytope output used, neighbour store failures
    VG_CUDA(cudaMemcpyAsync(&c3, h->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    h->poly_used = c3.poly_used;
    c1.nb_failed = c3.nb_failed;
    VG_CUDA(cudaGetLastError());
    float cell_ms = 0, clip_ms = 0, fin_ms = 0;
    cudaEventElapsedTime(&cell_ms, h->ev[2], h->ev[3]);
    cudaEventElapsedTime(&clip_ms, h->ev[2], h->ev[4]);
    cudaEventElapsedTime(&fin_ms, h->ev[4], h->ev[3]);
    rc = finish_compute(h, c1, cell_ms);
    h->stats.clip_ms = clip_ms;
    h->stats.finish_ms = fin_ms;
    h->stats.fp64_engine_cells = switched ? h->nkept : 0;
    return rc;
}

}  // namespace

extern "C" {

int vgpu_get_tuning(vgpu_container *h, vgpu_tuning *out) {
    if (!h || !out) return fail(VGPU_ERR_ARG, "null argument");
    out->particles_per_block = h->target_density;
    out->warps_per_cta = h->warps_per_cta;
    out->cells_per_chunk = h->cell_chunk > 0 ? h->cell_chunk : kDefaultCellChunk;
    out->fp64_fallback = h->fp64_fallback;
    return VGPU_OK;
}

int vgpu_set_tuning_ex(vgpu_container *h, const vgpu_tuning *t) {
    if (!h || !t) return fail(VGPU_ERR_ARG, "null argument");
    if (t->warps_per_cta < 0 || t->warps_per_cta > kBuiltCtaWarps)
        return fail(VGPU_ERR_ARG, "warps per CTA must be 1-%d (got %d)", kBuiltCtaWarps, t->warps_per_cta);
    if (t->cells_per_chunk < 0 || t->cells_per_chunk > 64)
        return fail(VGPU_ERR_ARG, "cells per chunk must be 1-64 (got %d)", t->cells_per_chunk);
    if (!(t->fp64_fallback >= 0.0)) return fail(VGPU_ERR_ARG, "bad fallback fraction");
    int rc = vgpu_set_tuning(h, t->particles_per_block, t->warps_per_cta);
    if (rc != VGPU_OK) return rc;
    if (t->cells_per_chunk > 0) h->cell_chunk = t->cells_per_chunk;
    if (t->fp64_fallback > 0.0) h->fp64_fallback = t->fp64_fallback;
    return VGPU_OK;
}

}  // extern "C"

namespace {

// The autotuner's cache: one line per (GPU, workload signature) with the
// tuple it chose, in $VORO_GB300_TUNE_CACHE, else
// $XDG_CACHE_HOME/voro_gb300/autotune.txt, else ~/.cache/voro_gb300/autotune.txt.
// Unreadable or unwritable files only cost a fresh search.
std::string tune_cache_path() {
    if (const char *e = getenv("VORO_GB300_TUNE_CACHE")) return e;
    std::string base;
    if (const char *x = getenv("XDG_CACHE_HOME")) base = x;
    else if (const char *home = getenv("HOME")) base = std::string(home) + "/.cache";
    else return "";
    return base + "/voro_gb300/autotune.txt";
}

// The signature the choice depends on: the device, the container kind and
// precision, the particle count to within a factor of two, the box's shape
// (its largest over smallest side, rounded) and its walls.
std::string tune_key(vgpu_container *h, int mode) {
    cudaDeviceProp prop;
    std::string dev = cudaGetDeviceProperties(&prop, h->device) == cudaSuccess ? prop.name : "unknown";
    for (char &c : dev)
        if (c == ' ' || c == '\t') c = '_';
    const int64_t n = h->use_device_input ? h->dev_n_ext : h->staged;
    int lg = 0;
    while (lg < 62 && (int64_t(1) << (lg + 1)) <= n) lg++;
    const double e0 = std::max({h->g.len[0], h->g.len[1], h->g.len[2]});
    const double e1 = std::max(1e-300, std::min({h->g.len[0], h->g.len[1], h->g.len[2]}));
    char buf[256];
    snprintf(buf, sizeof(buf), "%s|kind%d|mode%d|n2^%d|aspect%d|walls%d|sm%d", dev.c_str(), h->g.kind, mode, lg,
             (int)std::lround(e0 / e1), (int)h->walls.size(), h->sms);
    return buf;
}

bool tune_cache_read(const std::string &key, vgpu_tuning &t) {
    const std::string path = tune_cache_path();
    if (path.empty()) return false;
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return false;
    char line[512];
    bool found = false;
    while (fgets(line, sizeof(line), f)) {
        char k[300];
        vgpu_tuning v{};
        if (sscanf(line, "%299s %lf %d %d %lf", k, &v.particles_per_block, &v.warps_per_cta, &v.cells_per_chunk,
                   &v.fp64_fallback) == 5 &&
            key == k && v.particles_per_block > 0 && v.warps_per_cta >= 1 && v.warps_per_cta <= kBuiltCtaWarps &&
            v.cells_per_chunk >= 1 && v.cells_per_chunk <= 64) {
            t = v;   // the last matching line wins
            found = true;
        }
    }
    fclose(f);
    return found;
}

void tune_cache_write(const std::string &key, const vgpu_tuning &t) {
    const std::string path = tune_cache_path();
    if (path.empty()) return;
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {   // mkdir -p of the directory
        const std::string dir = path.substr(0, slash);
        for (size_t i = 1; i <= dir.size(); i++)
            if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
    }
    FILE *f = fopen(path.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s %.17g %d %d %.17g\n", key.c_str(), t.particles_per_block, t.warps_per_cta, t.cells_per_chunk,
            t.fp64_fallback);
    fclose(f);
}

// the best step time of two computes at tuning t (the first compute of a new
// size also allocates)
int time_tuning(vgpu_container *h, int mode, const vgpu_tuning &t, double *ms) {
    int rc = vgpu_set_tuning_ex(h, &t);
    if (rc != VGPU_OK) return rc;
    double best = 1e300;
    for (int rep = 0; rep < 2; rep++) {
        rc = vgpu_compute(h, mode);
        if (rc != VGPU_OK) return rc;
        best = std::min(best, (double)h->stats.step_ms);
    }
    *ms = best;
    return VGPU_OK;
}

}  // namespace

extern "C" {

int vgpu_autotune_ex(vgpu_container *h, int mode, int flags, vgpu_tuning *chosen, double *best_ms) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    if (flags & ~(VGPU_TUNE_USE_CACHE | VGPU_TUNE_WRITE_CACHE)) return fail(VGPU_ERR_ARG, "unknown flags 0x%x", flags);
    const std::string key = tune_key(h, mode);
    vgpu_tuning best;
    vgpu_get_tuning(h, &best);
    double best_t = 1e300;
    if ((flags & VGPU_TUNE_USE_CACHE) && tune_cache_read(key, best)) {
        int rc = time_tuning(h, mode, best, &best_t);   // leaves the results of the cached choice
        if (chosen) *chosen = best;
        if (best_ms) *best_ms = best_t;
        return rc;
    }
    // coordinate search: the engine-grid density (particles per block: the
    // search visits fewer, fuller blocks as it grows), then the warps (cells
    // in flight) per CTA, then the cells a warp takes from the queue at once
    static const double kDensities[] = {0.35, 0.5, 0.6, 0.75, 0.9, 1.0, 1.25, 1.5, 2.0, 3.0};
    static const int kWarps[] = {1, 2, 4, 8};
    static const int kChunks[] = {1, 2, 4, 8, 16};
    auto consider = [&](const vgpu_tuning &t) -> int {
        double ms;
        const int rc = time_tuning(h, mode, t, &ms);
        if (rc == VGPU_OK && ms < best_t) {
            best_t = ms;
            best = t;
        }
        return rc;
    };
    for (double d : kDensities) {
        vgpu_tuning t = best;
        t.particles_per_block = d;
        if (int rc = consider(t)) return rc;
    }
    for (int w : kWarps) {
        if (w > kBuiltCtaWarps) continue;
        vgpu_tuning t = best;
        t.warps_per_cta = w;
        if (int rc = consider(t)) return rc;
    }
    for (int c : kChunks) {
        vgpu_tuning t = best;
        t.cells_per_chunk = c;
        if (int rc = consider(t)) return rc;
    }
    double ms;
    int rc = time_tuning(h, mode, best, &ms);   // leave the results of the chosen setting
    if (rc != VGPU_OK) return rc;
    if (flags & VGPU_TUNE_WRITE_CACHE) tune_cache_write(key, best);
    if (chosen) *chosen = best;
    if (best_ms) *best_ms = best_t;
    return VGPU_OK;
}

int vgpu_autotune(vgpu_container *h, int mode, double *best_density, double *best_ms) {
    vgpu_tuning t;
    const int rc = vgpu_autotune_ex(h, mode, 0, &t, best_ms);
    if (rc == VGPU_OK && best_density) *best_density = t.particles_per_block;
    return rc;
}

int vgpu_set_output(vgpu_container *h, int flags) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    if (flags & ~VGPU_OUTPUT_POLYTOPES) return fail(VGPU_ERR_ARG, "unknown output flags 0x%x", flags);
    h->output = flags;
    h->computed = false;
    return VGPU_OK;
}

}  // extern "C"

namespace {

// The polytopes of n cells from a store (offsets poff, doubles used) as CSR.
int assemble_polytopes(vgpu_container *h, size_t n, const DevBuf &poff, const DevBuf &poly, unsigned long long pused,
                       int64_t *offsets, double *data) {
    offsets[0] = 0;
    if (n == 0) return VGPU_OK;
    cudaStream_t s = h->stream;
    std::vector<long long> off(n);
    VG_CUDA(cudaMemcpyAsync(off.data(), poff.p, n * 8, cudaMemcpyDeviceToHost, s));
    const unsigned long long used = std::min<unsigned long long>(pused, poly.bytes / 8);
    std::vector<double> store(used);
    if (used > 0) VG_CUDA(cudaMemcpyAsync(store.data(), poly.p, used * 8, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    for (size_t k = 0; k < n; k++) {
        if (off[k] == -2) return fail(VGPU_ERR_CAPACITY, "polytope output store full");
        int64_t len = 0;
        if (off[k] >= 0) {
            if ((unsigned long long)off[k] + 2 > used)
                return fail(VGPU_ERR_INTERNAL, "polytope offset %lld beyond the store (%llu)", off[k], used);
            // [nv, nf, 3 nv coordinates, then per face: neighbour, order, loop]
            // (the orders sum to 3 nv unless the cell has merged vertices)
            const int64_t nvk = (int64_t)store[off[k]], nfk = (int64_t)store[off[k] + 1];
            len = 2 + 3 * nvk;
            for (int64_t f = 0; f < nfk; f++) {
                if ((unsigned long long)(off[k] + len + 2) > used)
                    return fail(VGPU_ERR_INTERNAL, "polytope of cell %zu runs beyond the store", k);
                len += 2 + (int64_t)store[off[k] + len + 1];
            }
            if ((unsigned long long)(off[k] + len) > used)
                return fail(VGPU_ERR_INTERNAL, "polytope of cell %zu runs beyond the store", k);
        }
        offsets[k + 1] = offsets[k] + len;
        if (data && len > 0) memcpy(data + offsets[k], store.data() + off[k], (size_t)len * 8);
    }
    return VGPU_OK;
}

}  // namespace

extern "C" {

int vgpu_get_polytopes(vgpu_container *h, int64_t *offsets, double *data) {
    if (!h || !offsets) return fail(VGPU_ERR_ARG, "null argument");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    if (!(h->output & VGPU_OUTPUT_POLYTOPES))
        return fail(VGPU_ERR_ARG, "polytope output was not requested (vgpu_set_output) for the last compute");
    return assemble_polytopes(h, (size_t)h->ncells, h->poly_off, h->poly, h->poly_used, offsets, data);
}

int vgpu_get_stats(vgpu_container *h, vgpu_stats *out) {
    if (!h || !out) return fail(VGPU_ERR_ARG, "null argument");
    *out = h->stats;
    return VGPU_OK;
}

int vgpu_num_cells(vgpu_container *h, int64_t *n) {
    if (!h || !n) return fail(VGPU_ERR_ARG, "null argument");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    *n = h->ncells;
    return VGPU_OK;
}

int vgpu_get_cells(vgpu_container *h, int32_t *ids, double *pos, double *vol, double *cen, int32_t *nfaces,
                   int32_t *nverts, double *maxr2, int32_t *flags) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    size_t n = (size_t)h->ncells;
    if (n == 0) return VGPU_OK;
    cudaStream_t s = h->stream;
    if (ids) VG_CUDA(cudaMemcpyAsync(ids, h->r_ids.p, n * 4, cudaMemcpyDeviceToHost, s));
    if (pos) VG_CUDA(cudaMemcpyAsync(pos, h->r_pos.p, n * 24, cudaMemcpyDeviceToHost, s));
    if (vol) VG_CUDA(cudaMemcpyAsync(vol, h->r_vol.p, n * 8, cudaMemcpyDeviceToHost, s));
    if (cen) VG_CUDA(cudaMemcpyAsync(cen, h->r_cen.p, n * 24, cudaMemcpyDeviceToHost, s));
    if (nfaces) VG_CUDA(cudaMemcpyAsync(nfaces, h->r_nf.p, n * 4, cudaMemcpyDeviceToHost, s));
    if (nverts) VG_CUDA(cudaMemcpyAsync(nverts, h->r_nv.p, n * 4, cudaMemcpyDeviceToHost, s));
    if (maxr2) VG_CUDA(cudaMemcpyAsync(maxr2, h->r_mr2.p, n * 8, cudaMemcpyDeviceToHost, s));
    if (flags) VG_CUDA(cudaMemcpyAsync(flags, h->r_flags.p, n * 4, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    return VGPU_OK;
}

int vgpu_get_radii(vgpu_container *h, double *radii) {
    if (!h || !radii) return fail(VGPU_ERR_ARG, "null argument");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    size_t n = (size_t)h->ncells;
    if (n == 0) return VGPU_OK;
    VG_CUDA(cudaMemcpyAsync(radii, h->r_rad.p, n * 8, cudaMemcpyDeviceToHost, h->stream));
    VG_CUDA(cudaStreamSynchronize(h->stream));
    return VGPU_OK;
}

static int build_csr(vgpu_container *h, int64_t *total_out) {
    if (h->csr_valid) {
        *total_out = h->csr_total;
        return VGPU_OK;
    }
    size_t n = (size_t)h->ncells;
    cudaStream_t s = h->stream;
    VG_CUDA(h->nb_off.ensure((n + 1) * 8));
    VG_CUDA(h->nb_tmp.ensure((scan_tmp_ints((int)n + 1) + 64) * 8));
    VG_CUDA(launch_nf_to_ll(h->r_nf.as<int>(), h->nb_off.as<long long>(), (int)n, s));
    VG_CUDA(cudaMemsetAsync(h->nb_off.as<long long>() + n, 0, 8, s));
    VG_CUDA(exclusive_scan_ll(h->nb_off.as<long long>(), h->nb_off.as<long long>(), (int)n + 1,
                              h->nb_tmp.as<long long>(), s));
    long long total = 0;
    VG_CUDA(cudaMemcpyAsync(&total, h->nb_off.as<long long>() + n, 8, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    *total_out = total;
    h->csr_total = total;
    h->csr_valid = true;
    return VGPU_OK;
}

int vgpu_num_neighbors(vgpu_container *h, int64_t *total) {
    if (!h || !total) return fail(VGPU_ERR_ARG, "null argument");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    if (h->ncells == 0) { *total = 0; return VGPU_OK; }
    return build_csr(h, total);
}

int vgpu_get_neighbors(vgpu_container *h, int64_t *offsets, int32_t *ids) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    size_t n = (size_t)h->ncells;
    if (n == 0) {
        if (offsets) offsets[0] = 0;
        return VGPU_OK;
    }
    int64_t total = 0;
    int rc = build_csr(h, &total);
    if (rc != VGPU_OK) return rc;
    cudaStream_t s = h->stream;
    if (offsets) VG_CUDA(cudaMemcpyAsync(offsets, h->nb_off.p, (n + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (ids && total > 0) {
        VG_CUDA(h->nb_out.ensure((size_t)total * 4));
        VG_CUDA(launch_compact_neighbors(h->r_nf.as<int>(), h->r_nb.as<int>(), h->r_nb_ovf.as<int>(),
                                         h->nb_off.as<long long>(), (int)n,
                                         h->nb_out.as<int>(), s));
        VG_CUDA(cudaMemcpyAsync(ids, h->nb_out.p, (size_t)total * 4, cudaMemcpyDeviceToHost, s));
    }
    VG_CUDA(cudaStreamSynchronize(s));
    return VGPU_OK;
}

int vgpu_sum_cell_volumes(vgpu_container *h, double *out) {
    if (!h || !out) return fail(VGPU_ERR_ARG, "null argument");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    *out = 0.0;
    if (h->ncells == 0) return VGPU_OK;
    cudaStream_t s = h->stream;
    VG_CUDA(h->sum_tmp.ensure(64 * 8));
    VG_CUDA(launch_sum_volumes(h->r_vol.as<double>(), h->r_flags.as<int>(), (int)h->ncells, h->sum_tmp.as<double>(), s));
    double part[64];
    VG_CUDA(cudaMemcpyAsync(part, h->sum_tmp.p, sizeof(part), cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for (int i = 0; i < 64; i++) t += part[i];
    *out = t;
    return VGPU_OK;
}

int vgpu_compute_ghost_cells(vgpu_container *h, int mode, int64_t n, const double *xyzr) {
    if (!h || n < 0 || (n > 0 && !xyzr)) return fail(VGPU_ERR_ARG, "bad arguments");
    if (mode != VGPU_FP64 && mode != VGPU_MIXED) return fail(VGPU_ERR_ARG, "bad mode %d", mode);
    if (n > (int64_t)INT32_MAX / 4) return fail(VGPU_ERR_MEMORY, "too many ghosts");
    h->ghost_n = 0;
    if (n == 0) return VGPU_OK;
    CellParams cp;
    if (h->g.tric && h->tric_thin) h->binned = false;   // images at the reference's depth
    if (!h->binned) {   // bin the particles as a compute would
        int rc = prepare_cells(h, mode, cp);
        if (rc != VGPU_OK) return rc;
    } else {
        fill_cell_params(h, cp);
    }
    cudaStream_t s = h->stream;
    const size_t nk = (size_t)h->nengine, ng = (size_t)n, tot = nk + ng;
    // engine arrays: the particles and any images (copied), then the ghosts
    VG_CUDA(h->gh_p64.ensure(tot * 32));
    VG_CUDA(h->gh_lffh.ensure(tot * 16));
    VG_CUDA(h->gh_lffl.ensure(tot * 16));
    VG_CUDA(h->gh_pid.ensure(tot * 4));
    VG_CUDA(h->gh_gblock.ensure(tot * 4));
    VG_CUDA(h->gh_outpos.ensure(tot * 4));
    VG_CUDA(h->gh_rec_off.ensure(tot * 8));
    VG_CUDA(h->gh_q.ensure(ng * 32));
    VG_CUDA(h->gh_keep.ensure(ng * 4));
    VG_CUDA(h->gh_list.ensure(ng * 4));
    VG_CUDA(h->gh_ovf.ensure(ng * 4));
    VG_CUDA(h->gh_ovf2.ensure(ng * 4));
    VG_CUDA(h->gh_cnt.ensure(3 * sizeof(Counters)));
    VG_CUDA(h->gh_vol.ensure(ng * 8));
    VG_CUDA(h->gh_cen.ensure(ng * 24));
    VG_CUDA(h->gh_nf.ensure(ng * 4));
    VG_CUDA(h->gh_nv.ensure(ng * 4));
    VG_CUDA(h->gh_mr2.ensure(ng * 8));
    VG_CUDA(h->gh_flags.ensure(ng * 4));
    VG_CUDA(h->gh_nb.ensure(ng * kNbStride * 4));
    VG_CUDA(h->gh_nb_ovf.ensure(nb_ovf_ints(ng) * 4));
    if (nk > 0) {
        VG_CUDA(cudaMemcpyAsync(h->gh_p64.p, cp.a.p64, nk * 32, cudaMemcpyDeviceToDevice, s));
        VG_CUDA(cudaMemcpyAsync(h->gh_lffh.p, cp.a.lffh, nk * 16, cudaMemcpyDeviceToDevice, s));
        VG_CUDA(cudaMemcpyAsync(h->gh_lffl.p, cp.a.lffl, nk * 16, cudaMemcpyDeviceToDevice, s));
        VG_CUDA(cudaMemcpyAsync(h->gh_pid.p, cp.a.pid, nk * 4, cudaMemcpyDeviceToDevice, s));
        VG_CUDA(cudaMemcpyAsync(h->gh_gblock.p, cp.a.gblock, nk * 4, cudaMemcpyDeviceToDevice, s));
    }
    VG_CUDA(cudaMemcpyAsync(h->gh_q.p, xyzr, ng * 32, cudaMemcpyHostToDevice, s));
    VG_CUDA(launch_ghost_setup(h->g, (int)ng, h->gh_q.as<double4>(), (int)nk, h->gh_p64.as<double4>(),
                               h->gh_lffh.as<float4>(), h->gh_lffl.as<float4>(), h->gh_pid.as<int>(),
                               h->gh_outpos.as<int>(), h->gh_gblock.as<int>(), h->gh_keep.as<int>(), s));
    std::vector<int> keep(ng);
    VG_CUDA(cudaMemcpyAsync(keep.data(), h->gh_keep.p, ng * 4, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    std::vector<int> list;
    list.reserve(ng);
    double rmax = h->g.rmax;
    for (size_t i = 0; i < ng; i++)
        if (keep[i]) {
            list.push_back((int)(nk + i));
            if (h->g.poly) rmax = std::max(rmax, xyzr[4 * i + 3]);
        }
    const int nl = (int)list.size();
    // results of ghosts that are not computed (outside a wall): no cell
    VG_CUDA(cudaMemsetAsync(h->gh_vol.p, 0, ng * 8, s));
    VG_CUDA(cudaMemsetAsync(h->gh_cen.p, 0, ng * 24, s));
    VG_CUDA(cudaMemsetAsync(h->gh_nf.p, 0, ng * 4, s));
    VG_CUDA(cudaMemsetAsync(h->gh_nv.p, 0, ng * 4, s));
    VG_CUDA(cudaMemsetAsync(h->gh_mr2.p, 0, ng * 8, s));
    VG_CUDA(cudaMemsetAsync(h->gh_flags.p, 0, ng * 4, s));
    VG_CUDA(cudaMemsetAsync(h->gh_rec_off.as<char>() + nk * 8, 0xff, ng * 8, s));
    VG_CUDA(cudaMemsetAsync(h->gh_cnt.p, 0, 3 * sizeof(Counters), s));
    if (nl > 0) VG_CUDA(cudaMemcpyAsync(h->gh_list.p, list.data(), (size_t)nl * 4, cudaMemcpyHostToDevice, s));
    // the engine over the ghosts only, against the particles
    Counters *gc = h->gh_cnt.as<Counters>();
    cp.a.p64 = h->gh_p64.as<double4>();
    cp.a.l32 = cp.a.lffh = h->gh_lffh.as<float4>();
    cp.a.lffl = h->gh_lffl.as<float4>();
    cp.a.pid = h->gh_pid.as<int>();
    cp.a.gblock = h->gh_gblock.as<int>();
    cp.a.outpos = h->gh_outpos.as<int>();
    cp.r.vol = h->gh_vol.as<double>();
    cp.r.cen = h->gh_cen.as<double>();
    cp.r.nf = h->gh_nf.as<int>();
    cp.r.nv = h->gh_nv.as<int>();
    cp.r.maxr2 = h->gh_mr2.as<double>();
    cp.r.flags = h->gh_flags.as<int>();
    cp.r.nb = h->gh_nb.as<int>();
    cp.r.nb_ovf = h->gh_nb_ovf.as<int>();
    cp.r.nb_ovf_cap = nb_ovf_ints(ng);
    cp.g.rmax = rmax;   // a larger ghost radius widens the search (compute_ghost_cell raises max_radius)
    cp.g.rmax32 = (float)rmax * (1.0f + 1e-6f);
    cp.cnt = gc;
    cp.ncells = nl;
    cp.cell_list = h->gh_list.as<int>();
    cp.overflow_list = h->gh_ovf.as<int>();
    h->ghost_poly = (h->output & VGPU_OUTPUT_POLYTOPES) != 0;
    h->ghost_poly_used = 0;
    RecordStore &store = record_store(h->device);
    std::lock_guard<std::mutex> hold(store.m);
    const unsigned long long cap =
        (unsigned long long)nl * kRecWordsPerCell[mode == VGPU_MIXED ? 1 : 0] + (1u << 20);
    VG_CUDA(store.buf.ensure(cap * 4));
    cp.rec = store.buf.as<unsigned>();
    cp.rec_cap = cap;
    cp.rec_used = &gc->rec_used;
    cp.rec_off = h->gh_rec_off.as<unsigned long long>();
    cp.poly = nullptr;
    if (h->ghost_poly) {
        const unsigned long long pcap = (unsigned long long)ng * kPolyDoublesPerCell + (1u << 16);
        VG_CUDA(h->gh_poly.ensure(pcap * 8));
        VG_CUDA(h->gh_poly_off.ensure(ng * 8));
        VG_CUDA(cudaMemsetAsync(h->gh_poly_off.p, 0xff, ng * 8, s));
        cp.poly = h->gh_poly.as<double>();
        cp.poly_cap = pcap;
        cp.poly_used = &gc->poly_used;
        cp.poly_off = h->gh_poly_off.as<long long>();
    }
    Counters c1, c3;
    if (nl > 0) {
        int rc = clip_passes(s, h->sms, h->warps_per_cta, mode, cp, gc + 1, gc + 2, h->gh_ovf2.as<int>(), c1);
        if (rc != VGPU_OK) return rc;
        VG_CUDA(launch_finish(cp, mode, h->sms, s));
        VG_CUDA(cudaMemcpyAsync(&c3, gc, sizeof(Counters), cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
        h->ghost_poly_used = c3.poly_used;
        const unsigned long long failed = c1.failed + c3.nb_failed;
        h->ghost_n = n;
        if (failed > 0) return fail(VGPU_ERR_CAPACITY, "%llu ghost cells exceeded the engine capacity", failed);
    }
    VG_CUDA(cudaStreamSynchronize(s));
    VG_CUDA(cudaGetLastError());
    h->ghost_n = n;
    return VGPU_OK;
}

int vgpu_get_ghost_cells(vgpu_container *h, double *vol, double *cen, int32_t *nfaces, int32_t *nverts, double *maxr2,
                         int32_t *flags) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    const size_t n = (size_t)h->ghost_n;
    if (n == 0) return VGPU_OK;
    cudaStream_t s = h->stream;
    if (vol) VG_CUDA(cudaMemcpyAsync(vol, h->gh_vol.p, n * 8, cudaMemcpyDeviceToHost, s));
    if (cen) VG_CUDA(cudaMemcpyAsync(cen, h->gh_cen.p, n * 24, cudaMemcpyDeviceToHost, s));
    if (nfaces) VG_CUDA(cudaMemcpyAsync(nfaces, h->gh_nf.p, n * 4, cudaMemcpyDeviceToHost, s));
    if (nverts) VG_CUDA(cudaMemcpyAsync(nverts, h->gh_nv.p, n * 4, cudaMemcpyDeviceToHost, s));
    if (maxr2) VG_CUDA(cudaMemcpyAsync(maxr2, h->gh_mr2.p, n * 8, cudaMemcpyDeviceToHost, s));
    if (flags) VG_CUDA(cudaMemcpyAsync(flags, h->gh_flags.p, n * 4, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    return VGPU_OK;
}

int vgpu_get_ghost_neighbors(vgpu_container *h, int64_t *offsets, int32_t *ids) {
    if (!h || !offsets) return fail(VGPU_ERR_ARG, "null argument");
    const size_t n = (size_t)h->ghost_n;
    offsets[0] = 0;
    if (n == 0) return VGPU_OK;
    cudaStream_t s = h->stream;
    std::vector<int32_t> nf(n);
    VG_CUDA(cudaMemcpyAsync(nf.data(), h->gh_nf.p, n * 4, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    for (size_t k = 0; k < n; k++) offsets[k + 1] = offsets[k] + nf[k];
    const int64_t total = offsets[n];
    if (ids && total > 0) {
        VG_CUDA(h->gh_nb_off.ensure((n + 1) * 8));
        VG_CUDA(h->gh_nb_out.ensure((size_t)total * 4));
        VG_CUDA(cudaMemcpyAsync(h->gh_nb_off.p, offsets, (n + 1) * 8, cudaMemcpyHostToDevice, s));
        VG_CUDA(launch_compact_neighbors(h->gh_nf.as<int>(), h->gh_nb.as<int>(), h->gh_nb_ovf.as<int>(),
                                         h->gh_nb_off.as<long long>(), (int)n, h->gh_nb_out.as<int>(), s));
        VG_CUDA(cudaMemcpyAsync(ids, h->gh_nb_out.p, (size_t)total * 4, cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
    }
    return VGPU_OK;
}

int vgpu_get_ghost_polytopes(vgpu_container *h, int64_t *offsets, double *data) {
    if (!h || !offsets) return fail(VGPU_ERR_ARG, "null argument");
    if (!h->ghost_poly)
        return fail(VGPU_ERR_ARG, "polytope output was not requested (vgpu_set_output) for the last ghost compute");
    return assemble_polytopes(h, (size_t)h->ghost_n, h->gh_poly_off, h->gh_poly, h->ghost_poly_used, offsets, data);
}

int vgpu_find_voronoi_cells(vgpu_container *h, int64_t n, const double *xyz, int32_t *pid, double *rxyz,
                            int32_t *found) {
    if (!h || n < 0 || (n > 0 && (!xyz || !pid || !rxyz || !found))) return fail(VGPU_ERR_ARG, "bad arguments");
    if (n == 0) return VGPU_OK;
    if (n > (int64_t)INT32_MAX / 4) return fail(VGPU_ERR_MEMORY, "too many query points");
    CellParams cp;
    if (h->g.tric && h->tric_thin) h->binned = false;   // images at the reference's depth
    if (!h->binned) {   // bin the particles as a compute would (no cells computed)
        int rc = prepare_cells(h, VGPU_MIXED, cp);
        if (rc != VGPU_OK) return rc;
    } else {
        fill_cell_params(h, cp);
    }
    cudaStream_t s = h->stream;
    VG_CUDA(h->loc_q.ensure((size_t)n * 24));
    VG_CUDA(h->loc_r.ensure((size_t)n * 24));
    VG_CUDA(h->loc_found.ensure((size_t)n * 4));
    VG_CUDA(h->loc_pid.ensure((size_t)n * 4));
    VG_CUDA(cudaMemcpyAsync(h->loc_q.p, xyz, (size_t)n * 24, cudaMemcpyHostToDevice, s));
    VG_CUDA(launch_locate(cp, (int)n, h->loc_q.as<double>(), h->loc_found.as<int>(), h->loc_pid.as<int>(),
                          h->loc_r.as<double>(), s));
    VG_CUDA(cudaMemcpyAsync(found, h->loc_found.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaMemcpyAsync(pid, h->loc_pid.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaMemcpyAsync(rxyz, h->loc_r.p, (size_t)n * 24, cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    return VGPU_OK;
}

int vgpu_phase_cycles(vgpu_container *h, double out[8]) {
    if (!h || !out) return fail(VGPU_ERR_ARG, "null argument");
    for (int i = 0; i < 8; i++) out[i] = h->phase[i];
    return VGPU_OK;
}

int vgpu_get_input_rows(vgpu_container *h, int32_t *rows) {
    if (!h || !rows) return fail(VGPU_ERR_ARG, "null argument");
    if (!h->binned) return fail(VGPU_ERR_NOT_COMPUTED, "no compute since the last put");
    const int64_t n = h->use_device_input ? h->dev_n_ext : h->staged;
    if (n <= 0) return VGPU_OK;
    VG_CUDA(cudaMemcpyAsync(rows, h->outpos_in.p, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
    VG_CUDA(cudaStreamSynchronize(h->stream));
    return VGPU_OK;
}

int vgpu_phase_counts(vgpu_container *h, double out[8]) {
    if (!h || !out) return fail(VGPU_ERR_ARG, "null argument");
    for (int i = 0; i < 8; i++) out[i] = h->phase[8 + i];
    return VGPU_OK;
}

int vgpu_device_results(vgpu_container *h, const double **dev_vol, const int32_t **dev_nfaces) {
    if (!h) return fail(VGPU_ERR_ARG, "null handle");
    if (!h->computed) return fail(VGPU_ERR_NOT_COMPUTED, "vgpu_compute has not run");
    if (dev_vol) *dev_vol = h->r_vol.as<double>();
    if (dev_nfaces) *dev_nfaces = h->r_nf.as<int32_t>();
    return VGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- batches

struct vgpu_batch {
    std::vector<vgpu_container *> members;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4];
    DevBuf cps, starts, counters, work, ovf_list, ovf_list2, jobs, bin_res, offsets, rec;
    bool offsets_ready = false;
    int64_t record_bytes = 0;   // record store budget (0: kBatchRecordBytes)
    int waves = 0;              // record-store waves of the last compute
    vgpu_stats stats{};
};

extern "C" {

int vgpu_batch_create(vgpu_batch **out) {
    if (!out) return fail(VGPU_ERR_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(VGPU_ERR_NO_DEVICE, "no CUDA device");
    vgpu_batch *b = new vgpu_batch();
    VG_CUDA(cudaGetDevice(&b->device));
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return fail(VGPU_ERR_CUDA, "stream creation failed");
    }
    for (int i = 0; i < 4; i++) cudaEventCreate(&b->ev[i]);
    *out = b;
    return VGPU_OK;
}

int vgpu_batch_add(vgpu_batch *b, vgpu_container *h) {
    if (!b || !h) return fail(VGPU_ERR_ARG, "null argument");
    if (h->device != b->device) return fail(VGPU_ERR_ARG, "container and batch are on different devices");
    b->members.push_back(h);
    return VGPU_OK;
}

int vgpu_batch_destroy(vgpu_batch *b) {
    if (!b) return VGPU_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    DevBuf *bufs[] = {&b->cps, &b->starts, &b->counters, &b->work, &b->ovf_list, &b->ovf_list2, &b->jobs, &b->bin_res,
                      &b->offsets,
                      &b->rec};
    for (DevBuf *d : bufs) d->release();
    for (int i = 0; i < 4; i++) cudaEventDestroy(b->ev[i]);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return VGPU_OK;
}

int vgpu_batch_compute(vgpu_batch *b, int mode) {
    if (!b) return fail(VGPU_ERR_ARG, "null handle");
    if (mode != VGPU_FP64 && mode != VGPU_MIXED) return fail(VGPU_ERR_ARG, "bad mode %d", mode);
    const auto t0 = std::chrono::steady_clock::now();
    memset(&b->stats, 0, sizeof(b->stats));
    const long long launches0 = launch_count();
    const int nc = (int)b->members.size();
    if (nc == 0) return VGPU_OK;
    cudaStream_t s = b->stream;
    VG_CUDA(b->counters.ensure((size_t)nc * sizeof(Counters)));
    VG_CUDA(cudaMemsetAsync(b->counters.p, 0, (size_t)nc * sizeof(Counters), s));
    const OffsetTable &ot = offset_table();
    if (!b->offsets_ready) {
        VG_CUDA(b->offsets.ensure(ot.codes.size() * 4));
        VG_CUDA(cudaMemcpyAsync(b->offsets.p, ot.codes.data(), ot.codes.size() * 4, cudaMemcpyHostToDevice, s));
        b->offsets_ready = true;
    }
    std::vector<CellParams> cps(nc);
    std::vector<long long> starts(nc + 1, 0);
    // members of at most kSmallBinMax particles: binned together, one CTA
    // each, in two launches by size (the jobs of at most kSmallBinTier
    // particles first)
    std::vector<int> small;
    std::vector<char> is_small(nc, 0);
    int ns_tier = 0;
    for (int pass = 0; pass < 2; pass++) {
        for (int i = 0; i < nc; i++) {
            const vgpu_container *h = b->members[i];
            const int64_t n = h->use_device_input ? h->dev_n_ext : h->staged;
            // (a sheared box stores images of its particles: the multi-kernel binning)
            if (h->g.tric || n > kSmallBinMax || (n <= kSmallBinTier) != (pass == 0)) continue;
            small.push_back(i);
            is_small[i] = 1;
        }
        if (pass == 0) ns_tier = (int)small.size();
    }
    const int ns = (int)small.size();
    if (ns > 0) {
        std::vector<SmallBinJob> jobs(ns);
        VG_CUDA(b->bin_res.ensure((size_t)ns * 16));
        VG_CUDA(b->jobs.ensure((size_t)ns * sizeof(SmallBinJob)));
        for (int j = 0; j < ns; j++) {
            int rc = prepare_small(b->members[small[j]], mode, jobs[j], b->bin_res.as<unsigned long long>() + 2 * j);
            if (rc != VGPU_OK) return rc;
        }
        VG_CUDA(cudaMemcpyAsync(b->jobs.p, jobs.data(), (size_t)ns * sizeof(SmallBinJob), cudaMemcpyHostToDevice, s));
        for (int j = 0; j < ns; j++) cudaEventRecord(b->members[small[j]]->ev[0], s);
        VG_CUDA(launch_small_bin(b->jobs.as<SmallBinJob>(), ns_tier, kSmallBinTier, s));
        VG_CUDA(launch_small_bin(b->jobs.as<SmallBinJob>() + ns_tier, ns - ns_tier, kSmallBinMax, s));
        for (int j = 0; j < ns; j++) cudaEventRecord(b->members[small[j]]->ev[1], s);
    }
    // the others on their own streams: every remap first, then the rest of
    // each member's binning as its remap's counts land; the batch stream
    // waits for each gather
    for (int i = 0; i < nc; i++) {
        if (is_small[i]) continue;
        int rc = bin_begin(b->members[i], mode, false);
        if (rc != VGPU_OK) return rc;
    }
    bool dup_check = false;
    for (int i = 0; i < nc; i++) {
        if (is_small[i]) continue;
        vgpu_container *h = b->members[i];
        VG_CUDA(cudaStreamSynchronize(h->stream));
        int rc = bin_finish(h, mode, cps[i], true);
        if (rc != VGPU_OK) return rc;
        dup_check = dup_check || h->dup_pending;
        cps[i].cnt = b->counters.as<Counters>() + i;
        rc = setup_member_records(h, cps[i], cps[i].cnt, h->stream);
        if (rc != VGPU_OK) return rc;
        cudaEventRecord(h->ev[2], h->stream);   // after the gather and the record resets
        VG_CUDA(cudaStreamWaitEvent(s, h->ev[2], 0));
    }
    if (dup_check && ns == 0) VG_CUDA(cudaStreamSynchronize(s));
    if (ns > 0) {
        std::vector<unsigned long long> res((size_t)ns * 2);
        VG_CUDA(cudaMemcpyAsync(res.data(), b->bin_res.p, (size_t)ns * 16, cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
        for (int j = 0; j < ns; j++) {
            const int i = small[j];
            vgpu_container *h = b->members[i];
            int rc = finish_small(h, &res[2 * (size_t)j]);
            if (rc != VGPU_OK) return rc;
            fill_cell_params(h, cps[i]);
            cps[i].cnt = b->counters.as<Counters>() + i;
            rc = setup_member_records(h, cps[i], cps[i].cnt, s);
            if (rc != VGPU_OK) return rc;
        }
    }
    // the large members' deferred duplicate checks (the batch stream has
    // passed every member's gather, which follows its check)
    for (int i = 0; dup_check && i < nc; i++) {
        vgpu_container *h = b->members[i];
        if (!h->dup_pending) continue;
        h->dup_pending = false;
        if (h->host_rb[2])
            return fail(VGPU_ERR_DUPLICATE, "member %d: duplicate particle positions (|d|^2 < 1e-10) in one block", i);
    }
    for (int i = 0; i < nc; i++) {
        if (!b->members[i]->g.tric) cps[i].cell_list = nullptr;   // (sheared: the particles among the images)
        cps[i].overflow_list = nullptr;
        cps[i].offsets = b->offsets.as<int>();   // the same table for every container
        starts[i + 1] = starts[i] + b->members[i]->nkept;
    }
    const long long total = starts[nc];
    const auto t1 = std::chrono::steady_clock::now();
    // one record store for the whole batch, reused by waves of cells when
    // the batch's records would not fit the budget: each wave is clipped,
    // rerun where it overflowed, and finished before the next starts
    const unsigned long long per_cell = kRecWordsPerCell[mode == VGPU_MIXED ? 1 : 0];
    const unsigned long long slack = 1ull << 20;
    const unsigned long long budget_words =
        std::max<unsigned long long>((b->record_bytes > 0 ? (unsigned long long)b->record_bytes : kBatchRecordBytes) / 4,
                                     slack + per_cell);
    const unsigned long long cap = std::min<unsigned long long>((unsigned long long)total * per_cell + slack, budget_words);
    const long long wave = std::max<long long>(1, (long long)((cap - slack) / per_cell));
    VG_CUDA(b->rec.ensure(cap * 4));
    VG_CUDA(b->cps.ensure((size_t)nc * sizeof(CellParams)));
    VG_CUDA(b->starts.ensure((size_t)(nc + 1) * 8));
    VG_CUDA(b->work.ensure(64));
    VG_CUDA(b->ovf_list.ensure((size_t)std::max<long long>(total, 1) * 8));
    VG_CUDA(b->ovf_list2.ensure((size_t)std::max<long long>(total, 1) * 8));
    // work, hand-ons, second pass work, records used, third pass work, second hand-ons
    unsigned long long *wk = b->work.as<unsigned long long>();
    for (int i = 0; i < nc; i++) {
        cps[i].rec = b->rec.as<unsigned>();
        cps[i].rec_cap = cap;
        cps[i].rec_used = wk + 3;
    }
    VG_CUDA(cudaMemcpyAsync(b->cps.p, cps.data(), (size_t)nc * sizeof(CellParams), cudaMemcpyHostToDevice, s));
    VG_CUDA(cudaMemcpyAsync(b->starts.p, starts.data(), (size_t)(nc + 1) * 8, cudaMemcpyHostToDevice, s));
    BatchParams bp;
    memset(&bp, 0, sizeof(bp));
    bp.cps = b->cps.as<CellParams>();
    bp.cell_start = b->starts.as<long long>();
    bp.ncont = nc;
    bp.cell_list = nullptr;
    bp.overflow_list = b->ovf_list.as<long long>();
    bp.work = wk;
    bp.overflow_count = wk + 1;
    bp.offsets = b->offsets.as<int>();
    bp.noffsets = (int)ot.codes.size();
    float clip_ms = 0, fin_ms = 0;
    b->waves = 0;
    for (long long w0 = 0; w0 < total; w0 += wave) {
        bp.cell_begin = w0;
        bp.ncells = std::min<long long>(wave, total - w0);
        VG_CUDA(cudaMemsetAsync(b->work.p, 0, 64, s));
        cudaEventRecord(b->ev[0], s);
        // the passes of clip_passes: first pass, (MIXED) the full 64-slot
        // engine on the cells it handed on, the 128-slot engine on the rest
        VG_CUDA(launch_cells_batch(bp, mode, 0, b->sms, s));
        unsigned long long novf = 0;
        VG_CUDA(cudaMemcpyAsync(&novf, wk + 1, 8, cudaMemcpyDeviceToHost, s));
        VG_CUDA(cudaStreamSynchronize(s));
        const long long *pending = b->ovf_list.as<long long>();
        if (novf > 0 && mode == VGPU_MIXED) {
            BatchParams bp1 = bp;
            bp1.ncells = (long long)novf;
            bp1.cell_list = pending;
            bp1.overflow_list = b->ovf_list2.as<long long>();
            bp1.overflow_count = wk + 5;
            bp1.work = wk + 2;
            VG_CUDA(launch_cells_batch(bp1, mode, 1, b->sms, s));
            VG_CUDA(cudaMemcpyAsync(&novf, wk + 5, 8, cudaMemcpyDeviceToHost, s));
            VG_CUDA(cudaStreamSynchronize(s));
            pending = b->ovf_list2.as<long long>();
        }
        if (novf > 0) {
            BatchParams bp2 = bp;
            bp2.ncells = (long long)novf;
            bp2.cell_list = pending;
            bp2.overflow_list = nullptr;
            bp2.work = wk + 4;
            VG_CUDA(launch_cells_batch(bp2, mode, 2, b->sms, s));
        }
        cudaEventRecord(b->ev[2], s);
        VG_CUDA(launch_finish_batch(bp, mode, b->sms, s));
        cudaEventRecord(b->ev[1], s);
        VG_CUDA(cudaEventSynchronize(b->ev[1]));
        float a = 0, f = 0;
        cudaEventElapsedTime(&a, b->ev[0], b->ev[2]);
        cudaEventElapsedTime(&f, b->ev[2], b->ev[1]);
        clip_ms += a;
        fin_ms += f;
        b->waves++;
    }
    for (int i = 0; i < nc; i++) cudaEventRecord(b->members[i]->ev[3], s);
    std::vector<Counters> cs(nc);
    VG_CUDA(cudaMemcpyAsync(cs.data(), b->counters.p, (size_t)nc * sizeof(Counters), cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    VG_CUDA(cudaGetLastError());
    const float cell_ms = clip_ms + fin_ms;
    int first_err = VGPU_OK;
    for (int i = 0; i < nc; i++) {
        vgpu_container *h = b->members[i];
        int rc;
        if (mode == VGPU_MIXED && h->fp64_fallback < 1.0 && h->nkept > 0 &&
            (double)cs[i].overflow > h->fp64_fallback * h->nkept) {
            // the member's filter band was saturated (more than the fallback
            // fraction of its cells handed on, as a single compute assesses
            // it): the member alone again, on the FP64 engine
            rc = compute_cells(h, VGPU_FP64, false);
            h->stats.fp64_engine_cells = h->nkept;
        } else {
            h->poly_used = cs[i].poly_used;
            rc = finish_compute(h, cs[i], cell_ms);
        }
        if (rc != VGPU_OK && first_err == VGPU_OK) first_err = rc;
        vgpu_stats &t = b->stats;
        t.cells += h->stats.cells;
        t.deleted += h->stats.deleted;
        t.marginal_cells += h->stats.marginal_cells;
        t.side_tests += h->stats.side_tests;
        t.fp64_repairs += h->stats.fp64_repairs;
        t.planes_tested += h->stats.planes_tested;
        t.planes_cut += h->stats.planes_cut;
        t.overflow_reruns += h->stats.overflow_reruns;
        t.failed_cells += h->stats.failed_cells;
        t.fp64_engine_cells += h->stats.fp64_engine_cells;
    }
    const auto t2 = std::chrono::steady_clock::now();
    b->stats.kernel_ms = cell_ms;
    b->stats.clip_ms = clip_ms;
    b->stats.finish_ms = fin_ms;
    b->stats.bin_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    b->stats.step_ms = std::chrono::duration<double, std::milli>(t2 - t0).count();
    b->stats.kernel_launches = launch_count() - launches0;
    if (first_err != VGPU_OK)
        return fail(first_err, "%lld cells exceeded the engine capacity", (long long)b->stats.failed_cells);
    return VGPU_OK;
}

int vgpu_batch_get_stats(vgpu_batch *b, vgpu_stats *out) {
    if (!b || !out) return fail(VGPU_ERR_ARG, "null argument");
    *out = b->stats;
    return VGPU_OK;
}

int vgpu_batch_set_record_budget(vgpu_batch *b, int64_t bytes) {
    if (!b || bytes < 0) return fail(VGPU_ERR_ARG, "bad record budget");
    b->record_bytes = bytes;
    return VGPU_OK;
}

int vgpu_batch_waves(vgpu_batch *b, int *waves) {
    if (!b || !waves) return fail(VGPU_ERR_ARG, "null argument");
    *waves = b->waves;
    return VGPU_OK;
}

}  // extern "C"
