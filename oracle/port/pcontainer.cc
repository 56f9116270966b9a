// CPU restatement of the reference's containers and cell search — TEST
// INFRASTRUCTURE (oracle + timed CPU baseline).  Restates:
//   worklist generation   src/worklist_gen.pl:94-197 (the table src/v_base_wl.cc)
//   radius bounds (mrad)  src/v_base.cc:23-94
//   container put/remap   src/container.cc:90-191; src/container_prd.cc:94-256
//   periodic images       src/container_prd.cc:583-774 (rectangular boxes)
//   unit Voronoi cell     src/unitcell.cc:26-85,90-200
//   compute_cell          src/v_compute.cc:289-944
//   loops                 src/c_loops.hh:165-210,325-393
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "pcell.hh"

namespace vport {

namespace {

constexpr int kHGrid = 4, kFGrid = 8, kSeqLen = 64, kHGridCu = 64;
constexpr double kLarge = 1.7976931348623157e308;
constexpr int kMaxUnitShells = 10;  // src/config.hh:93

inline int step_int(double a) { return a < 0 ? int(a) - 1 : int(a); }
inline int step_mod(int a, int b) { return a >= 0 ? a % b : b - 1 - (b - 1 - a) % b; }
inline int step_div(int a, int b) { return a >= 0 ? a / b : -1 + (a + 1) / b; }

// ----------------------------------------------------------------- worklists
// For each of the 4^3 sub-regions of the lower octant of a block, a greedy
// ordering of 63 nearby blocks by distance from the sub-region centre (plus a
// small penalty for jumping away from the previous pick), followed by flags
// that name the neighbouring blocks not on the list (bits 21-28) and, in the
// first word, the length of the prefix whose neighbours are all on the list.
std::vector<unsigned> build_worklists() {
    const int hr = kHGrid, r = kFGrid, ls = kSeqLen - 1, dis = 8;
    const int d = 2 * dis + 1, dd = d * d, d0 = (1 + d + dd) * dis;
    std::vector<int> m(d * d * d, 0), la(d * d * d, 0);
    std::vector<unsigned> out;
    int v = 0;
    for (int kk = 0; kk < hr; kk++)
        for (int jj = 0; jj < hr; jj++)
            for (int ii = 0; ii < hr; ii++) {
                std::vector<int> a, b;
                v += 2;
                int xp = 0, yp = 0, zp = 0;
                double x = (ii + 0.5) / r, y = (jj + 0.5) / r, z = (kk + 0.5) / r;
                m[d0] = v;
                auto add = [&](int i, int j, int k) {
                    int idx = d0 + i + d * j + dd * k;
                    if (m[idx] != v) {
                        a.push_back(i); a.push_back(j); a.push_back(k);
                        m[idx] = v;
                    }
                };
                auto adis = [&](int xt, int yt, int zt) {
                    double xco = 0, yco = 0, zco = 0;
                    if (xt > 0) xco = x - xt;
                    if (xt < 0) xco = x - xt - 1;
                    if (yt > 0) yco = y - yt;
                    if (yt < 0) yco = y - yt - 1;
                    if (zt > 0) zco = z - zt;
                    if (zt < 0) zco = z - zt - 1;
                    return std::sqrt(xco * xco + yco * yco + zco * zco);
                };
                add(1, 0, 0); add(0, 1, 0); add(0, 0, 1);
                add(-1, 0, 0); add(0, -1, 0); add(0, 0, -1);
                for (int l = 1; l <= ls; l++) {
                    double minwei = 1e9;
                    int nx = 0;
                    int ac = (int)a.size() / 3;
                    for (int t = 0; t < ac; t++) {
                        int xt = a[3 * t], yt = a[3 * t + 1], zt = a[3 * t + 2];
                        double dx = xt - xp, dy = yt - yp, dz = zt - zp;
                        double wei = adis(xt, yt, zt) + 0.02 * std::sqrt(dx * dx + dy * dy + dz * dz);
                        if (wei < minwei) { nx = t; minwei = wei; }
                    }
                    xp = a[3 * nx]; yp = a[3 * nx + 1]; zp = a[3 * nx + 2];
                    add(xp + 1, yp, zp); add(xp, yp + 1, zp); add(xp, yp, zp + 1);
                    add(xp - 1, yp, zp); add(xp, yp - 1, zp); add(xp, yp, zp - 1);
                    b.push_back(a[3 * nx]); b.push_back(a[3 * nx + 1]); b.push_back(a[3 * nx + 2]);
                    a.erase(a.begin() + 3 * nx, a.begin() + 3 * nx + 3);
                }
                m[d0] = ++v;
                int nb = (int)b.size() / 3;
                for (int t = 0; t < nb; t++) m[d0 + b[3 * t] + d * b[3 * t + 1] + dd * b[3 * t + 2]] = v;
                for (int t = 0; t < nb; t++) {
                    int xt = b[3 * t], yt = b[3 * t + 1], zt = b[3 * t + 2];
                    int k = d0 + xt + yt * d + zt * dd;
                    if (xt >= 0 && m[k + 1] != v) { la[k + 1] = t; m[k + 1] = v + 1; }
                    if (yt >= 0 && m[k + d] != v) { la[k + d] = t; m[k + d] = v + 1; }
                    if (zt >= 0 && m[k + dd] != v) { la[k + dd] = t; m[k + dd] = v + 1; }
                    if (xt <= 0 && m[k - 1] != v) { la[k - 1] = t; m[k - 1] = v + 1; }
                    if (yt <= 0 && m[k - d] != v) { la[k - d] = t; m[k - d] = v + 1; }
                    if (zt <= 0 && m[k - dd] != v) { la[k - dd] = t; m[k - dd] = v + 1; }
                }
                int j = 0;
                for (; j < nb; j++) {
                    int k = d0 + b[3 * j] + b[3 * j + 1] * d + b[3 * j + 2] * dd;
                    if (m[k + 1] != v || m[k + d] != v || m[k + dd] != v || m[k - 1] != v || m[k - d] != v ||
                        m[k - dd] != v)
                        break;
                }
                out.push_back((unsigned)j);
                for (int t = 0; t < nb; t++) {
                    int xt = b[3 * t], yt = b[3 * t + 1], zt = b[3 * t + 2];
                    int k = d0 + xt + yt * d + zt * dd;
                    unsigned o = 0;
                    if (m[k + 1] != v && la[k + 1] == t) o |= 1;
                    if (m[k - 1] != v && la[k - 1] == t) o ^= 3;
                    if (m[k + d] != v && la[k + d] == t) o |= 8;
                    if (m[k - d] != v && la[k - d] == t) o ^= 24;
                    if (m[k + dd] != v && la[k + dd] == t) o |= 64;
                    if (m[k - dd] != v && la[k - dd] == t) o ^= 192;
                    out.push_back((unsigned)((xt + 64) | (yt + 64) << 7 | (zt + 64) << 14) | (o << 21));
                }
            }
    return out;
}

const std::vector<unsigned> &worklists() {
    static const std::vector<unsigned> wl = build_worklists();
    return wl;
}

}  // namespace

// ----------------------------------------------------------------- containers
struct Container {
    int kind = 0;
    bool poly = false, prd = false;
    bool xper = false, yper = false, zper = false;
    double ax = 0, bx = 0, ay = 0, by = 0, az = 0, bz = 0;  // container bounds / periodic lengths
    int nx, ny, nz, nxy, nxyz;
    double boxx, boxy, boxz, xsp, ysp, zsp;
    int ps;
    double max_len_sq;
    double max_radius = 0;
    // block storage: flat arrays, block b holds particles [bstart[b], bstart[b+1])
    int nblocks;
    std::vector<int> bstart;
    std::vector<int> fid;
    std::vector<double> fp;
    // put() staging per primary block (insertion order)
    std::vector<std::vector<int>> sid;
    std::vector<std::vector<double>> sp;
    int ghost_y = 0, ghost_z = 0;  // ghost layers materialised (periodic)
    // periodic: ghost layers
    int ey = 0, ez = 0, wy = 0, wz = 0, oy = 0, oz = 0;
    Cell unit_voro{1.0};
    // search
    std::vector<double> mrad;
    int hx, hy, hz;

    int co(int ijk) const { return bstart[ijk + 1] - bstart[ijk]; }
    const double *pp(int ijk) const { return fp.data() + (size_t)bstart[ijk] * ps; }
    const int *ids(int ijk) const { return fid.data() + bstart[ijk]; }

    void setup_radii() {
        // voro_base::voro_base (src/v_base.cc:23-69)
        const unsigned b1 = 1 << 21, b2 = 1 << 22, b3 = 1 << 24, b4 = 1 << 25, b5 = 1 << 27, b6 = 1 << 28;
        const double xstep = boxx / kFGrid, ystep = boxy / kFGrid, zstep = boxz / kFGrid;
        mrad.assign(kHGridCu * kSeqLen, 0.0);
        const std::vector<unsigned> &wl = worklists();
        const unsigned *e = wl.data();
        double *radp = mrad.data();
        double xlo, ylo, zlo, xhi, yhi, zhi, minr;
        int lx, ly, lz, i, j, k, q;
        unsigned f;
        auto cmin = [&](int ti, int tj, int tk) {
            double radsq, temp;
            if (ti > 0) { temp = boxx * ti - xhi; radsq = temp * temp; }
            else if (ti < 0) { temp = xlo - boxx * (1 + ti); radsq = temp * temp; }
            else radsq = 0;
            if (tj > 0) { temp = boxy * tj - yhi; radsq += temp * temp; }
            else if (tj < 0) { temp = ylo - boxy * (1 + tj); radsq += temp * temp; }
            if (tk > 0) { temp = boxz * tk - zhi; radsq += temp * temp; }
            else if (tk < 0) { temp = zlo - boxz * (1 + tk); radsq += temp * temp; }
            if (radsq < minr) minr = radsq;
        };
        for (zlo = 0, zhi = zstep, lz = 0; lz < kHGrid; zlo = zhi, zhi += zstep, lz++)
            for (ylo = 0, yhi = ystep, ly = 0; ly < kHGrid; ylo = yhi, yhi += ystep, ly++)
                for (xlo = 0, xhi = xstep, lx = 0; lx < kHGrid; xlo = xhi, xhi += xstep, lx++) {
                    minr = kLarge;
                    for (q = e[0] + 1; q < kSeqLen; q++) {
                        f = e[q];
                        i = (f & 127) - 64;
                        j = (f >> 7 & 127) - 64;
                        k = (f >> 14 & 127) - 64;
                        if ((f & b2) == b2) {
                            cmin(i - 1, j, k);
                            if ((f & b1) == 0) cmin(i + 1, j, k);
                        } else if ((f & b1) == b1) cmin(i + 1, j, k);
                        if ((f & b4) == b4) {
                            cmin(i, j - 1, k);
                            if ((f & b3) == 0) cmin(i, j + 1, k);
                        } else if ((f & b3) == b3) cmin(i, j + 1, k);
                        if ((f & b6) == b6) {
                            cmin(i, j, k - 1);
                            if ((f & b5) == 0) cmin(i, j, k + 1);
                        } else if ((f & b5) == b5) cmin(i, j, k + 1);
                    }
                    q--;
                    while (q > 0) {
                        radp[q] = minr;
                        f = e[q];
                        i = (f & 127) - 64;
                        j = (f >> 7 & 127) - 64;
                        k = (f >> 14 & 127) - 64;
                        cmin(i, j, k);
                        q--;
                    }
                    *radp = minr;
                    e += kSeqLen;
                    radp += kSeqLen;
                }
    }

    // container / container_poly (src/container.cc:30-44,90-191)
    void init_container(int k, const double *g, const int *grid, const int *per) {
        kind = k;
        poly = (k == 1);
        prd = false;
        ax = g[0]; bx = g[1]; ay = g[2]; by = g[3]; az = g[4]; bz = g[5];
        xper = per[0] != 0; yper = per[1] != 0; zper = per[2] != 0;
        nx = grid[0]; ny = grid[1]; nz = grid[2];
        nxy = nx * ny; nxyz = nxy * nz;
        boxx = (bx - ax) / nx; boxy = (by - ay) / ny; boxz = (bz - az) / nz;
        xsp = 1 / boxx; ysp = 1 / boxy; zsp = 1 / boxz;
        ps = poly ? 4 : 3;
        max_len_sq = (bx - ax) * (bx - ax) * (xper ? 0.25 : 1) + (by - ay) * (by - ay) * (yper ? 0.25 : 1) +
                     (bz - az) * (bz - az) * (zper ? 0.25 : 1);
        nblocks = nxyz;
        sid.assign(nxyz, {});
        sp.assign(nxyz, {});
        hx = xper ? 2 * nx + 1 : nx;
        hy = yper ? 2 * ny + 1 : ny;
        hz = zper ? 2 * nz + 1 : nz;
        setup_radii();
    }

    bool put_remap(int &ijk, double &x, double &y, double &z) const {
        int l;
        ijk = step_int((x - ax) * xsp);
        if (xper) { l = step_mod(ijk, nx); x += boxx * (l - ijk); ijk = l; }
        else if (ijk < 0 || ijk >= nx) return false;
        int j = step_int((y - ay) * ysp);
        if (yper) { l = step_mod(j, ny); y += boxy * (l - j); j = l; }
        else if (j < 0 || j >= ny) return false;
        int k = step_int((z - az) * zsp);
        if (zper) { l = step_mod(k, nz); z += boxz * (l - k); k = l; }
        else if (k < 0 || k >= nz) return false;
        ijk += nx * j + nxy * k;
        return true;
    }

    // container_periodic (src/container_prd.cc:29-50), unit cell (src/unitcell.cc:26-85)
    void init_periodic(int k, const double *g, const int *grid) {
        kind = k;
        poly = (k == 3);
        prd = true;
        bx = g[0]; by = g[2]; bz = g[5];
        ax = ay = az = 0;
        xper = yper = zper = true;
        nx = grid[0]; ny = grid[1]; nz = grid[2];
        nxy = nx * ny; nxyz = nxy * nz;
        boxx = bx / nx; boxy = by / ny; boxz = bz / nz;
        xsp = 1 / boxx; ysp = 1 / boxy; zsp = 1 / boxz;
        ps = poly ? 4 : 3;
        build_unit_cell();
        max_len_sq = unit_voro.max_radius_squared();
        ey = int(max_uv_y * ysp + 1);
        ez = int(max_uv_z * zsp + 1);
        wy = ny + ey; wz = nz + ez;
        oy = ny + 2 * ey; oz = nz + 2 * ez;
        nblocks = nx * oy * oz;
        sid.assign(nxyz, {});
        sp.assign(nxyz, {});
        hx = 2 * nx + 1; hy = 2 * ey + 1; hz = 2 * ez + 1;
        setup_radii();
    }

    double max_uv_y = 0, max_uv_z = 0;

    void build_unit_cell() {
        const double bxy = 0, bxz = 0, byz = 0;
        unit_voro = Cell(kMaxUnitShells * kMaxUnitShells * 4 * (bx * bx + by * by + bz * bz));
        const double ucx = kMaxUnitShells * bx, ucy = kMaxUnitShells * by, ucz = kMaxUnitShells * bz;
        const int zero_ids[6] = {0, 0, 0, 0, 0, 0};
        unit_voro.init_box(-ucx, ucx, -ucy, ucy, -ucz, ucz, zero_ids);
        auto apply = [&](int i, int j, int k) {
            double x = i * bx + j * bxy + k * bxz, y = j * by + k * byz, z = k * bz;
            unit_voro.nplane(x, y, z, x * x + y * y + z * z, 0);
            unit_voro.nplane(-x, -y, -z, x * x + y * y + z * z, 0);
        };
        auto test = [&](int i, int j, int k) {
            double x = i * bx + j * bxy + k * bxz, y = j * by + k * byz, z = k * bz;
            double rsq = x * x + y * y + z * z;
            return unit_voro.plane_intersects(x, y, z, rsq);
        };
        auto intersect = [&](int l) {
            if (test(l, 0, 0)) return true;
            for (int i = 1; i < l; i++) {
                if (test(l, i, 0)) return true;
                if (test(-l, i, 0)) return true;
            }
            for (int i = -l; i <= l; i++)
                if (test(i, l, 0)) return true;
            for (int i = 1; i < l; i++)
                for (int j = -l + 1; j <= l; j++) {
                    if (test(l, j, i)) return true;
                    if (test(-j, l, i)) return true;
                    if (test(-l, -j, i)) return true;
                    if (test(j, -l, i)) return true;
                }
            for (int i = -l; i <= l; i++)
                for (int j = -l; j <= l; j++)
                    if (test(i, j, l)) return true;
            return false;
        };
        int l = 1;
        while (l < 2 * kMaxUnitShells) {
            if (intersect(l)) {
                apply(l, 0, 0);
                for (int i = 1; i < l; i++) {
                    apply(l, i, 0);
                    apply(-l, i, 0);
                }
                for (int i = -l; i <= l; i++) apply(i, l, 0);
                for (int i = 1; i < l; i++)
                    for (int j = -l + 1; j <= l; j++) {
                        apply(l, j, i);
                        apply(-j, l, i);
                        apply(-l, -j, i);
                        apply(j, -l, i);
                    }
                for (int i = -l; i <= l; i++)
                    for (int j = -l; j <= l; j++) apply(i, j, l);
            } else {
                max_uv_y = max_uv_z = 0;
                for (int v = 0; v < unit_voro.p; v++) {
                    double q = unit_voro.pts[4 * v], y = unit_voro.pts[4 * v + 1], z = unit_voro.pts[4 * v + 2];
                    q = std::sqrt(q * q + y * y + z * z);
                    if (y + q > max_uv_y) max_uv_y = y + q;
                    if (z + q > max_uv_z) max_uv_z = z + q;
                }
                max_uv_z *= 0.5;
                max_uv_y *= 0.5;
                return;
            }
            l++;
        }
    }

    // container_periodic_base::put_locate_block (src/container_prd.cc:189-216)
    int put_locate_periodic(double &x, double &y, double &z) const {
        int k = step_int(z * zsp);
        if (k < 0 || k >= nz) {
            int ak = step_div(k, nz);
            z -= ak * bz; y -= ak * 0.0; x -= ak * 0.0; k -= ak * nz;
        }
        int j = step_int(y * ysp);
        if (j < 0 || j >= ny) {
            int aj = step_div(j, ny);
            y -= aj * by; x -= aj * 0.0; j -= aj * ny;
        }
        int i = step_int(x * xsp);
        if (i < 0 || i >= nx) {
            int ai = step_div(i, nx);
            x -= ai * bx; i -= ai * nx;
        }
        return i + nx * (j + ny * k);  // primary block index (staging)
    }

    void put(int n, double x, double y, double z, double r) {
        int ijk;
        if (prd) {
            ijk = put_locate_periodic(x, y, z);
        } else if (!put_remap(ijk, x, y, z)) {
            return;
        }
        sid[ijk].push_back(n);
        sp[ijk].push_back(x);
        sp[ijk].push_back(y);
        sp[ijk].push_back(z);
        if (poly) {
            sp[ijk].push_back(r);
            if (max_radius < r) max_radius = r;
        }
    }

    // Flat block storage.  For periodic boxes the ghost blocks are shifted
    // copies of the primary blocks, in their order (src/container_prd.cc:
    // 551-554,583-774, rectangular case).  The reference creates them lazily;
    // here they are all built up front (for a rectangular box at most about
    // nine times the primary particles): a cell beside a void reaches across
    // most of the box, to images many layers deep.
    void finalize() {
        bstart.assign(nblocks + 1, 0);
        auto src_of = [&](int b, int &sb, int &aj, int &ak) {
            if (!prd) { sb = b; aj = ak = 0; return true; }
            int i = b % nx, j = (b / nx) % oy, k = b / (nx * oy);
            int lj = j - ey, lk = k - ez;
            aj = step_div(lj, ny);
            ak = step_div(lk, nz);
            int dj = lj < 0 ? -lj : (lj >= ny ? lj - ny + 1 : 0);
            int dk = lk < 0 ? -lk : (lk >= nz ? lk - nz + 1 : 0);
            if (dj > ghost_y || dk > ghost_z) return false;
            sb = i + nx * ((lj - aj * ny) + ny * (lk - ak * nz));
            return true;
        };
        if (prd) {
            ghost_y = ey;
            ghost_z = ez;
        }
        for (int b = 0; b < nblocks; b++) {
            int sb, aj, ak;
            bstart[b + 1] = bstart[b] + (src_of(b, sb, aj, ak) ? (int)sid[sb].size() : 0);
        }
        fid.resize(bstart[nblocks]);
        fp.resize((size_t)bstart[nblocks] * ps);
        for (int b = 0; b < nblocks; b++) {
            int sb, aj, ak;
            if (!src_of(b, sb, aj, ak)) continue;
            int o = bstart[b];
            for (size_t l = 0; l < sid[sb].size(); l++) {
                fid[o + l] = sid[sb][l];
                double *d = &fp[(size_t)(o + l) * ps];
                const double *q = &sp[sb][ps * l];
                d[0] = q[0];
                d[1] = (aj == 0) ? q[1] : q[1] + by * aj;
                d[2] = (ak == 0) ? q[2] : q[2] + bz * ak;
                if (ps == 4) d[3] = q[3];
            }
        }
        sid.clear(); sid.shrink_to_fit();
        sp.clear(); sp.shrink_to_fit();
    }

    // loop order: c_loop_all (src/c_loops.hh:165-210) or c_loop_all_periodic (325-393)
    void loop_order(std::vector<int> &blk, std::vector<int> &slot, std::vector<int> &ci, std::vector<int> &cj,
                    std::vector<int> &ck) const {
        blk.clear(); slot.clear(); ci.clear(); cj.clear(); ck.clear();
        if (!prd) {
            for (int k = 0; k < nz; k++)
                for (int j = 0; j < ny; j++)
                    for (int i = 0; i < nx; i++) {
                        int ijk = i + nx * (j + ny * k);
                        for (int q = 0; q < co(ijk); q++) {
                            blk.push_back(ijk); slot.push_back(q); ci.push_back(i); cj.push_back(j); ck.push_back(k);
                        }
                    }
        } else {
            for (int k = ez; k < wz; k++)
                for (int j = ey; j < wy; j++)
                    for (int i = 0; i < nx; i++) {
                        int ijk = i + nx * (j + oy * k);
                        for (int q = 0; q < co(ijk); q++) {
                            blk.push_back(ijk); slot.push_back(q); ci.push_back(i); cj.push_back(j); ck.push_back(k);
                        }
                    }
        }
    }
};

// ----------------------------------------------------------------- compute_cell
struct Computer {
    const Container &con;
    Cell c;
    std::vector<unsigned> mask;
    unsigned mv = 0;
    std::vector<int> qu;
    double bxsq;
    double r_rad = 0, r_mul = 0, r_val = 0;

    explicit Computer(const Container &cn)
        : con(cn), c(cn.max_len_sq), mask((size_t)cn.hx * cn.hy * cn.hz, 0u),
          qu(3 * (3 + cn.hx * cn.hy + cn.hz * (cn.hx + cn.hy))),
          bxsq(cn.boxx * cn.boxx + cn.boxy * cn.boxy + cn.boxz * cn.boxz) {}

    // radius policy (src/rad_option.hh:299-434)
    inline bool r_ctest(double crs, double mrs) const {
        if (!con.poly) return crs > mrs;
        double cc = crs + r_mul;
        return cc > 0 && cc * cc > mrs * crs;
    }
    inline void r_prime(double rv) { if (con.poly) r_val = 1 + r_mul / rv; }
    inline double r_cutoff(double lrs) const { return con.poly ? lrs * r_val : lrs; }
    inline double r_scale(double rs, int ijk, int q) const {
        if (!con.poly) return rs;
        double rj = con.pp(ijk)[4 * q + 3];
        return rs + r_rad - rj * rj;
    }
    inline bool r_scale_check(double &rs, double mrs, int ijk, int q) const {
        if (!con.poly) return rs < mrs;
        double trs = rs;
        double rj = con.pp(ijk)[4 * q + 3];
        rs += r_rad - rj * rj;
        return rs <= 0 || rs * rs < mrs * trs;
    }

    int region_index(int ci, int cj, int ck, int ei, int ej, int ek, double &qx, double &qy, double &qz, int disp) const {
        if (!con.prd) {
            const int nx = con.nx, ny = con.ny, nz = con.nz;
            if (con.xper) { if (ci + ei < nx) { ei += nx; qx = -(con.bx - con.ax); } else if (ci + ei >= (nx << 1)) { ei -= nx; qx = con.bx - con.ax; } else qx = 0; }
            if (con.yper) { if (cj + ej < ny) { ej += ny; qy = -(con.by - con.ay); } else if (cj + ej >= (ny << 1)) { ej -= ny; qy = con.by - con.ay; } else qy = 0; }
            if (con.zper) { if (ck + ek < nz) { ek += nz; qz = -(con.bz - con.az); } else if (ck + ek >= (nz << 1)) { ek -= nz; qz = con.bz - con.az; } else qz = 0; }
            return disp + ei + nx * (ej + ny * ek);
        }
        int qi = ci + (ei - con.nx), qj = cj + (ej - con.ey), qk = ck + (ek - con.ez);
        int iv = step_div(qi, con.nx);
        if (iv != 0) { qx = iv * con.bx; qi -= con.nx * iv; } else qx = 0;
        return qi + con.nx * (qj + con.oy * qk);
    }

    bool compute_min_max_radius(int di, int dj, int dk, double fx, double fy, double fz, double gxs, double gys,
                                double gzs, double &crs, double mrs) const;
    bool corner_test(double xl, double yl, double zl, double xh, double yh, double zh);
    bool edge_x_test(double x0, double yl, double zl, double x1, double yh, double zh);
    bool edge_y_test(double xl, double y0, double zl, double xh, double y1, double zh);
    bool edge_z_test(double xl, double yl, double z0, double xh, double yh, double z1);
    bool face_x_test(double xl, double y0, double z0, double y1, double z1);
    bool face_y_test(double x0, double yl, double z0, double x1, double z1);
    bool face_z_test(double x0, double y0, double zl, double x1, double y1);

    void add_to_mask(int ei, int ej, int ek, size_t &qe);
    void scan_bits_mask_add(unsigned q, size_t mijk, int ei, int ej, int ek, size_t &qe);
    void qpush(size_t &qe, int a, int b, int d) {
        if (qe + 3 > qu.size()) qu.resize(qu.size() * 2 + 18);
        qu[qe++] = a; qu[qe++] = b; qu[qe++] = d;
    }

    bool compute_cell(int ijk, int s, int ci, int cj, int ck);
};

bool Computer::compute_min_max_radius(int di, int dj, int dk, double fx, double fy, double fz, double gxs,
                                      double gys, double gzs, double &crs, double mrs) const {
    // src/v_compute.cc:796-944
    const double boxx = con.boxx, boxy = con.boxy, boxz = con.boxz;
    double xlo, ylo, zlo;
    if (di > 0) {
        xlo = di * boxx - fx;
        crs = xlo * xlo;
        if (dj > 0) {
            ylo = dj * boxy - fy;
            crs += ylo * ylo;
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (boxx * xlo + boxy * ylo + boxz * zlo);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (boxx * xlo + boxy * ylo - boxz * zlo);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += boxx * (2 * xlo + boxx) + boxy * (2 * ylo + boxy) + gzs;
            }
        } else if (dj < 0) {
            ylo = (dj + 1) * boxy - fy;
            crs += ylo * ylo;
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (boxx * xlo - boxy * ylo + boxz * zlo);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (boxx * xlo - boxy * ylo - boxz * zlo);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += boxx * (2 * xlo + boxx) + boxy * (-2 * ylo + boxy) + gzs;
            }
        } else {
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (2 * zlo + boxz);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (-2 * zlo + boxz);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += gzs;
            }
            crs += gys + boxx * (2 * xlo + boxx);
        }
    } else if (di < 0) {
        xlo = (di + 1) * boxx - fx;
        crs = xlo * xlo;
        if (dj > 0) {
            ylo = dj * boxy - fy;
            crs += ylo * ylo;
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (-boxx * xlo + boxy * ylo + boxz * zlo);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (-boxx * xlo + boxy * ylo - boxz * zlo);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += boxx * (-2 * xlo + boxx) + boxy * (2 * ylo + boxy) + gzs;
            }
        } else if (dj < 0) {
            ylo = (dj + 1) * boxy - fy;
            crs += ylo * ylo;
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (-boxx * xlo - boxy * ylo + boxz * zlo);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += bxsq + 2 * (-boxx * xlo - boxy * ylo - boxz * zlo);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += boxx * (-2 * xlo + boxx) + boxy * (-2 * ylo + boxy) + gzs;
            }
        } else {
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (2 * zlo + boxz);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (-2 * zlo + boxz);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += gzs;
            }
            crs += gys + boxx * (-2 * xlo + boxx);
        }
    } else {
        if (dj > 0) {
            ylo = dj * boxy - fy;
            crs = ylo * ylo;
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (2 * zlo + boxz);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (-2 * zlo + boxz);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += gzs;
            }
            crs += boxy * (2 * ylo + boxy);
        } else if (dj < 0) {
            ylo = (dj + 1) * boxy - fy;
            crs = ylo * ylo;
            if (dk > 0) {
                zlo = dk * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (2 * zlo + boxz);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz;
                crs += zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (-2 * zlo + boxz);
            } else {
                if (r_ctest(crs, mrs)) return true;
                crs += gzs;
            }
            crs += boxy * (-2 * ylo + boxy);
        } else {
            if (dk > 0) {
                zlo = dk * boxz - fz; crs = zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (2 * zlo + boxz);
            } else if (dk < 0) {
                zlo = (dk + 1) * boxz - fz; crs = zlo * zlo; if (r_ctest(crs, mrs)) return true;
                crs += boxz * (-2 * zlo + boxz);
            } else {
                crs = 0;
            }
            crs += gys;
        }
        crs += gxs;
    }
    return false;
}

// corner/edge/face tests (src/v_compute.cc:632-780)
bool Computer::corner_test(double xl, double yl, double zl, double xh, double yh, double zh) {
    r_prime(xl * xl + yl * yl + zl * zl);
    if (c.plane_intersects_guess(xh, yl, zl, r_cutoff(xl * xh + yl * yl + zl * zl))) return false;
    if (c.plane_intersects(xh, yh, zl, r_cutoff(xl * xh + yl * yh + zl * zl))) return false;
    if (c.plane_intersects(xl, yh, zl, r_cutoff(xl * xl + yl * yh + zl * zl))) return false;
    if (c.plane_intersects(xl, yh, zh, r_cutoff(xl * xl + yl * yh + zl * zh))) return false;
    if (c.plane_intersects(xl, yl, zh, r_cutoff(xl * xl + yl * yl + zl * zh))) return false;
    if (c.plane_intersects(xh, yl, zh, r_cutoff(xl * xh + yl * yl + zl * zh))) return false;
    return true;
}
bool Computer::edge_x_test(double x0, double yl, double zl, double x1, double yh, double zh) {
    r_prime(yl * yl + zl * zl);
    if (c.plane_intersects_guess(x0, yl, zh, r_cutoff(yl * yl + zl * zh))) return false;
    if (c.plane_intersects(x1, yl, zh, r_cutoff(yl * yl + zl * zh))) return false;
    if (c.plane_intersects(x1, yl, zl, r_cutoff(yl * yl + zl * zl))) return false;
    if (c.plane_intersects(x0, yl, zl, r_cutoff(yl * yl + zl * zl))) return false;
    if (c.plane_intersects(x0, yh, zl, r_cutoff(yl * yh + zl * zl))) return false;
    if (c.plane_intersects(x1, yh, zl, r_cutoff(yl * yh + zl * zl))) return false;
    return true;
}
bool Computer::edge_y_test(double xl, double y0, double zl, double xh, double y1, double zh) {
    r_prime(xl * xl + zl * zl);
    if (c.plane_intersects_guess(xl, y0, zh, r_cutoff(xl * xl + zl * zh))) return false;
    if (c.plane_intersects(xl, y1, zh, r_cutoff(xl * xl + zl * zh))) return false;
    if (c.plane_intersects(xl, y1, zl, r_cutoff(xl * xl + zl * zl))) return false;
    if (c.plane_intersects(xl, y0, zl, r_cutoff(xl * xl + zl * zl))) return false;
    if (c.plane_intersects(xh, y0, zl, r_cutoff(xl * xh + zl * zl))) return false;
    if (c.plane_intersects(xh, y1, zl, r_cutoff(xl * xh + zl * zl))) return false;
    return true;
}
bool Computer::edge_z_test(double xl, double yl, double z0, double xh, double yh, double z1) {
    r_prime(xl * xl + yl * yl);
    if (c.plane_intersects_guess(xl, yh, z0, r_cutoff(xl * xl + yl * yh))) return false;
    if (c.plane_intersects(xl, yh, z1, r_cutoff(xl * xl + yl * yh))) return false;
    if (c.plane_intersects(xl, yl, z1, r_cutoff(xl * xl + yl * yl))) return false;
    if (c.plane_intersects(xl, yl, z0, r_cutoff(xl * xl + yl * yl))) return false;
    if (c.plane_intersects(xh, yl, z0, r_cutoff(xl * xh + yl * yl))) return false;
    if (c.plane_intersects(xh, yl, z1, r_cutoff(xl * xh + yl * yl))) return false;
    return true;
}
bool Computer::face_x_test(double xl, double y0, double z0, double y1, double z1) {
    r_prime(xl * xl);
    if (c.plane_intersects_guess(xl, y0, z0, r_cutoff(xl * xl))) return false;
    if (c.plane_intersects(xl, y0, z1, r_cutoff(xl * xl))) return false;
    if (c.plane_intersects(xl, y1, z1, r_cutoff(xl * xl))) return false;
    if (c.plane_intersects(xl, y1, z0, r_cutoff(xl * xl))) return false;
    return true;
}
bool Computer::face_y_test(double x0, double yl, double z0, double x1, double z1) {
    r_prime(yl * yl);
    if (c.plane_intersects_guess(x0, yl, z0, r_cutoff(yl * yl))) return false;
    if (c.plane_intersects(x0, yl, z1, r_cutoff(yl * yl))) return false;
    if (c.plane_intersects(x1, yl, z1, r_cutoff(yl * yl))) return false;
    if (c.plane_intersects(x1, yl, z0, r_cutoff(yl * yl))) return false;
    return true;
}
bool Computer::face_z_test(double x0, double y0, double zl, double x1, double y1) {
    r_prime(zl * zl);
    if (c.plane_intersects_guess(x0, y0, zl, r_cutoff(zl * zl))) return false;
    if (c.plane_intersects(x0, y1, zl, r_cutoff(zl * zl))) return false;
    if (c.plane_intersects(x1, y1, zl, r_cutoff(zl * zl))) return false;
    if (c.plane_intersects(x1, y0, zl, r_cutoff(zl * zl))) return false;
    return true;
}

// add_to_mask / scan_bits_mask_add (src/v_compute.cc:235-264); the queue here
// is a growing array read from the front, equivalent to the reference's ring
void Computer::add_to_mask(int ei, int ej, int ek, size_t &qe) {
    const int hx = con.hx, hy = con.hy, hz = con.hz, hxy = hx * hy;
    size_t mijk = ei + (size_t)hx * (ej + (size_t)hy * ek);
    if (ek > 0 && mask[mijk - hxy] != mv) { mask[mijk - hxy] = mv; qpush(qe, ei, ej, ek - 1); }
    if (ej > 0 && mask[mijk - hx] != mv) { mask[mijk - hx] = mv; qpush(qe, ei, ej - 1, ek); }
    if (ei > 0 && mask[mijk - 1] != mv) { mask[mijk - 1] = mv; qpush(qe, ei - 1, ej, ek); }
    if (ei < hx - 1 && mask[mijk + 1] != mv) { mask[mijk + 1] = mv; qpush(qe, ei + 1, ej, ek); }
    if (ej < hy - 1 && mask[mijk + hx] != mv) { mask[mijk + hx] = mv; qpush(qe, ei, ej + 1, ek); }
    if (ek < hz - 1 && mask[mijk + hxy] != mv) { mask[mijk + hxy] = mv; qpush(qe, ei, ej, ek + 1); }
}

void Computer::scan_bits_mask_add(unsigned q, size_t mijk, int ei, int ej, int ek, size_t &qe) {
    const unsigned b1 = 1 << 21, b2 = 1 << 22, b3 = 1 << 24, b4 = 1 << 25, b5 = 1 << 27, b6 = 1 << 28;
    const int hx = con.hx, hy = con.hy, hz = con.hz, hxy = hx * hy;
    if ((q & b2) == b2) {
        if (ei > 0) { mask[mijk - 1] = mv; qpush(qe, ei - 1, ej, ek); }
        if ((q & b1) == 0 && ei < hx - 1) { mask[mijk + 1] = mv; qpush(qe, ei + 1, ej, ek); }
    } else if ((q & b1) == b1 && ei < hx - 1) { mask[mijk + 1] = mv; qpush(qe, ei + 1, ej, ek); }
    if ((q & b4) == b4) {
        if (ej > 0) { mask[mijk - hx] = mv; qpush(qe, ei, ej - 1, ek); }
        if ((q & b3) == 0 && ej < hy - 1) { mask[mijk + hx] = mv; qpush(qe, ei, ej + 1, ek); }
    } else if ((q & b3) == b3 && ej < hy - 1) { mask[mijk + hx] = mv; qpush(qe, ei, ej + 1, ek); }
    if ((q & b6) == b6) {
        if (ek > 0) { mask[mijk - hxy] = mv; qpush(qe, ei, ej, ek - 1); }
        if ((q & b5) == 0 && ek < hz - 1) { mask[mijk + hxy] = mv; qpush(qe, ei, ej, ek + 1); }
    } else if ((q & b5) == b5 && ek < hz - 1) { mask[mijk + hxy] = mv; qpush(qe, ei, ej, ek + 1); }
}

// compute_cell (src/v_compute.cc:289-621)
bool Computer::compute_cell(int ijk, int s, int ci, int cj, int ck) {
    static const int count_list[8] = {7, 11, 15, 19, 26, 35, 45, 59};
    const int *count_e = count_list + 8;
    double x, y, z, x1, y1, z1, qx = 0, qy = 0, qz = 0;
    double xlo, ylo, zlo, xhi, yhi, zhi, x2, y2, z2, rs;
    int i, j, k, di, dj, dk, ei, ej, ek, f, g, l, disp = 0;
    double fx, fy, fz, gxs, gys, gzs;
    const double *radp;
    unsigned q;
    const unsigned *e;
    const int ps = con.ps;
    const double boxx = con.boxx, boxy = con.boxy, boxz = con.boxz;
    const int hx = con.hx, hy = con.hy, hz = con.hz;

    // initialize_voronoicell
    {
        const double *pp = con.pp(ijk) + ps * s;
        x = pp[0]; y = pp[1]; z = pp[2];
        if (con.prd) {
            c.copy_from(con.unit_voro);
            i = con.nx; j = con.ey; k = con.ez;
        } else {
            double xa1, xa2, ya1, ya2, za1, za2;
            if (con.xper) { xa1 = -(xa2 = 0.5 * (con.bx - con.ax)); i = con.nx; } else { xa1 = con.ax - x; xa2 = con.bx - x; i = ci; }
            if (con.yper) { ya1 = -(ya2 = 0.5 * (con.by - con.ay)); j = con.ny; } else { ya1 = con.ay - y; ya2 = con.by - y; j = cj; }
            if (con.zper) { za1 = -(za2 = 0.5 * (con.bz - con.az)); k = con.nz; } else { za1 = con.az - z; za2 = con.bz - z; k = ck; }
            const int box_ids[6] = {-1, -2, -3, -4, -5, -6};
            c.init_box(xa1, xa2, ya1, ya2, za1, za2, box_ids);
            disp = ijk - i - con.nx * (j + con.ny * k);
        }
    }
    if (con.poly) {
        double r = con.pp(ijk)[4 * s + 3];
        r_rad = r * r;
        r_mul = (r - con.max_radius) * (r + con.max_radius);
    }
    double crs, mrs;
    int next_count = 3;
    const int *count_p = count_list;
    const int co0 = con.co(ijk);
    for (l = 0; l < s; l++) {
        x1 = con.pp(ijk)[ps * l] - x;
        y1 = con.pp(ijk)[ps * l + 1] - y;
        z1 = con.pp(ijk)[ps * l + 2] - z;
        rs = r_scale(x1 * x1 + y1 * y1 + z1 * z1, ijk, l);
        if (!c.nplane(x1, y1, z1, rs, con.ids(ijk)[l])) return false;
    }
    l++;
    while (l < co0) {
        x1 = con.pp(ijk)[ps * l] - x;
        y1 = con.pp(ijk)[ps * l + 1] - y;
        z1 = con.pp(ijk)[ps * l + 2] - z;
        rs = r_scale(x1 * x1 + y1 * y1 + z1 * z1, ijk, l);
        if (!c.nplane(x1, y1, z1, rs, con.ids(ijk)[l])) return false;
        l++;
    }
    mrs = c.max_radius_squared();
    unsigned m1, m2;
    if (con.prd) {
        fx = x - boxx * ci;
        fy = y - boxy * (cj - con.ey);
        fz = z - boxz * (ck - con.ez);
    } else {
        fx = x - con.ax - boxx * ci;
        fy = y - con.ay - boxy * cj;
        fz = z - con.az - boxz * ck;
    }
    di = int(fx * con.xsp * kFGrid); dj = int(fy * con.ysp * kFGrid); dk = int(fz * con.zsp * kFGrid);
    if (di >= kHGrid) {
        gxs = fx;
        m1 = 127 + (3 << 21); m2 = 1 + (1 << 21); di = kFGrid - 1 - di; if (di < 0) di = 0;
    } else { m1 = m2 = 0; gxs = boxx - fx; }
    if (dj >= kHGrid) {
        gys = fy;
        m1 |= (127 << 7) + (3 << 24); m2 |= (1 << 7) + (1 << 24); dj = kFGrid - 1 - dj; if (dj < 0) dj = 0;
    } else gys = boxy - fy;
    if (dk >= kHGrid) {
        gzs = fz;
        m1 |= (127 << 14) + (3 << 27); m2 |= (1 << 14) + (1 << 27); dk = kFGrid - 1 - dk; if (dk < 0) dk = 0;
    } else gzs = boxz - fz;
    gxs *= gxs; gys *= gys; gzs *= gzs;
    int wl_index = di + kHGrid * (dj + kHGrid * dk);
    radp = con.mrad.data() + wl_index * kSeqLen;
    e = worklists().data() + wl_index * kSeqLen;
    f = e[0];
    g = 0;
    int cijk;
    do {
        if (g == next_count) {
            mrs = c.max_radius_squared();
            if (count_p != count_e) next_count = *(count_p++);
        }
        if (r_ctest(radp[g], mrs)) return true;
        g++;
        q = e[g]; q ^= m1; q += m2;
        di = q & 127; di -= 64;
        dj = (q >> 7) & 127; dj -= 64;
        dk = (q >> 14) & 127; dk -= 64;
        ei = di + i; if (ei < 0 || ei >= hx) continue;
        ej = dj + j; if (ej < 0 || ej >= hy) continue;
        ek = dk + k; if (ek < 0 || ek >= hz) continue;
        if (compute_min_max_radius(di, dj, dk, fx, fy, fz, gxs, gys, gzs, crs, mrs)) continue;
        cijk = region_index(ci, cj, ck, ei, ej, ek, qx, qy, qz, disp);
        if (con.co(cijk) > 0) {
            l = 0; x2 = x - qx; y2 = y - qy; z2 = z - qz;
            if (!r_ctest(crs, mrs)) {
                do {
                    x1 = con.pp(cijk)[ps * l] - x2;
                    y1 = con.pp(cijk)[ps * l + 1] - y2;
                    z1 = con.pp(cijk)[ps * l + 2] - z2;
                    rs = r_scale(x1 * x1 + y1 * y1 + z1 * z1, cijk, l);
                    if (!c.nplane(x1, y1, z1, rs, con.ids(cijk)[l])) return false;
                    l++;
                } while (l < con.co(cijk));
            } else {
                do {
                    x1 = con.pp(cijk)[ps * l] - x2;
                    y1 = con.pp(cijk)[ps * l + 1] - y2;
                    z1 = con.pp(cijk)[ps * l + 2] - z2;
                    rs = x1 * x1 + y1 * y1 + z1 * z1;
                    if (r_scale_check(rs, mrs, cijk, l) && !c.nplane(x1, y1, z1, rs, con.ids(cijk)[l])) return false;
                    l++;
                } while (l < con.co(cijk));
            }
        }
    } while (g < f);
    mv++;
    if (mv == 0) {
        std::fill(mask.begin(), mask.end(), 0u);
        mv = 1;
    }
    size_t qs = 0, qe = 0;
    while (g < kSeqLen - 1) {
        if (g == next_count) {
            mrs = c.max_radius_squared();
            if (count_p != count_e) next_count = *(count_p++);
        }
        if (r_ctest(radp[g], mrs)) return true;
        g++;
        q = e[g]; q ^= m1; q += m2;
        di = q & 127; di -= 64;
        dj = (q >> 7) & 127; dj -= 64;
        dk = (q >> 14) & 127; dk -= 64;
        ei = di + i; if (ei < 0 || ei >= hx) continue;
        ej = dj + j; if (ej < 0 || ej >= hy) continue;
        ek = dk + k; if (ek < 0 || ek >= hz) continue;
        size_t mijk = ei + (size_t)hx * (ej + (size_t)hy * ek);
        mask[mijk] = mv;
        if (compute_min_max_radius(di, dj, dk, fx, fy, fz, gxs, gys, gzs, crs, mrs)) continue;
        cijk = region_index(ci, cj, ck, ei, ej, ek, qx, qy, qz, disp);
        if (con.co(cijk) > 0) {
            l = 0; x2 = x - qx; y2 = y - qy; z2 = z - qz;
            if (!r_ctest(crs, mrs)) {
                do {
                    x1 = con.pp(cijk)[ps * l] - x2;
                    y1 = con.pp(cijk)[ps * l + 1] - y2;
                    z1 = con.pp(cijk)[ps * l + 2] - z2;
                    rs = r_scale(x1 * x1 + y1 * y1 + z1 * z1, cijk, l);
                    if (!c.nplane(x1, y1, z1, rs, con.ids(cijk)[l])) return false;
                    l++;
                } while (l < con.co(cijk));
            } else {
                do {
                    x1 = con.pp(cijk)[ps * l] - x2;
                    y1 = con.pp(cijk)[ps * l + 1] - y2;
                    z1 = con.pp(cijk)[ps * l + 2] - z2;
                    rs = x1 * x1 + y1 * y1 + z1 * z1;
                    if (r_scale_check(rs, mrs, cijk, l) && !c.nplane(x1, y1, z1, rs, con.ids(cijk)[l])) return false;
                    l++;
                } while (l < con.co(cijk));
            }
        }
        scan_bits_mask_add(q, mijk, ei, ej, ek, qe);
    }
    if (r_ctest(radp[g], mrs)) return true;
    while (qs != qe) {
        ei = qu[qs++]; ej = qu[qs++]; ek = qu[qs++];
        xlo = (ei - i) * boxx - fx; xhi = xlo + boxx;
        ylo = (ej - j) * boxy - fy; yhi = ylo + boxy;
        zlo = (ek - k) * boxz - fz; zhi = zlo + boxz;
        if (ei > i) {
            if (ej > j) {
                if (ek > k) { if (corner_test(xlo, ylo, zlo, xhi, yhi, zhi)) continue; }
                else if (ek < k) { if (corner_test(xlo, ylo, zhi, xhi, yhi, zlo)) continue; }
                else { if (edge_z_test(xlo, ylo, zlo, xhi, yhi, zhi)) continue; }
            } else if (ej < j) {
                if (ek > k) { if (corner_test(xlo, yhi, zlo, xhi, ylo, zhi)) continue; }
                else if (ek < k) { if (corner_test(xlo, yhi, zhi, xhi, ylo, zlo)) continue; }
                else { if (edge_z_test(xlo, yhi, zlo, xhi, ylo, zhi)) continue; }
            } else {
                if (ek > k) { if (edge_y_test(xlo, ylo, zlo, xhi, yhi, zhi)) continue; }
                else if (ek < k) { if (edge_y_test(xlo, ylo, zhi, xhi, yhi, zlo)) continue; }
                else { if (face_x_test(xlo, ylo, zlo, yhi, zhi)) continue; }
            }
        } else if (ei < i) {
            if (ej > j) {
                if (ek > k) { if (corner_test(xhi, ylo, zlo, xlo, yhi, zhi)) continue; }
                else if (ek < k) { if (corner_test(xhi, ylo, zhi, xlo, yhi, zlo)) continue; }
                else { if (edge_z_test(xhi, ylo, zlo, xlo, yhi, zhi)) continue; }
            } else if (ej < j) {
                if (ek > k) { if (corner_test(xhi, yhi, zlo, xlo, ylo, zhi)) continue; }
                else if (ek < k) { if (corner_test(xhi, yhi, zhi, xlo, ylo, zlo)) continue; }
                else { if (edge_z_test(xhi, yhi, zlo, xlo, ylo, zhi)) continue; }
            } else {
                if (ek > k) { if (edge_y_test(xhi, ylo, zlo, xlo, yhi, zhi)) continue; }
                else if (ek < k) { if (edge_y_test(xhi, ylo, zhi, xlo, yhi, zlo)) continue; }
                else { if (face_x_test(xhi, ylo, zlo, yhi, zhi)) continue; }
            }
        } else {
            if (ej > j) {
                if (ek > k) { if (edge_x_test(xlo, ylo, zlo, xhi, yhi, zhi)) continue; }
                else if (ek < k) { if (edge_x_test(xlo, ylo, zhi, xhi, yhi, zlo)) continue; }
                else { if (face_y_test(xlo, ylo, zlo, xhi, zhi)) continue; }
            } else if (ej < j) {
                if (ek > k) { if (edge_x_test(xlo, yhi, zlo, xhi, ylo, zhi)) continue; }
                else if (ek < k) { if (edge_x_test(xlo, yhi, zhi, xhi, ylo, zlo)) continue; }
                else { if (face_y_test(xlo, yhi, zlo, xhi, zhi)) continue; }
            } else {
                if (ek > k) { if (face_z_test(xlo, ylo, zlo, xhi, yhi)) continue; }
                else if (ek < k) { if (face_z_test(xlo, ylo, zhi, xhi, yhi)) continue; }
                else continue;  // the reference treats this as an internal error
            }
        }
        cijk = region_index(ci, cj, ck, ei, ej, ek, qx, qy, qz, disp);
        if (con.co(cijk) > 0) {
            l = 0; x2 = x - qx; y2 = y - qy; z2 = z - qz;
            do {
                x1 = con.pp(cijk)[ps * l] - x2;
                y1 = con.pp(cijk)[ps * l + 1] - y2;
                z1 = con.pp(cijk)[ps * l + 2] - z2;
                rs = r_scale(x1 * x1 + y1 * y1 + z1 * z1, cijk, l);
                if (!c.nplane(x1, y1, z1, rs, con.ids(cijk)[l])) return false;
                l++;
            } while (l < con.co(cijk));
        }
        add_to_mask(ei, ej, ek, qe);
    }
    return true;
}

// ----------------------------------------------------------------- C API
namespace {

bool build(Container &con, int kind, const double *geom, const int *grid, const int *periodic, int n,
           const int *ids, const double *xyzr) {
    if (kind == 0 || kind == 1) con.init_container(kind, geom, grid, periodic);
    else if (kind == 2 || kind == 3) {
        if (geom[1] != 0.0 || geom[3] != 0.0 || geom[4] != 0.0) return false;
        con.init_periodic(kind, geom, grid);
    } else return false;
    for (int i = 0; i < n; i++) con.put(ids[i], xyzr[4 * i], xyzr[4 * i + 1], xyzr[4 * i + 2], xyzr[4 * i + 3]);
    con.finalize();
    return true;
}

}  // namespace
}  // namespace vport

using namespace vport;

extern "C" {

// Same records and layout as ref_compute_cells (oracle/ref_capi.cc), plus the
// per-cell count of vertex-plane side tests when out_tests is not NULL.
// Computes the cells at loop-order positions sel[0..m) and writes their
// records at output rows 0..m; returns m, -1 if nb_cap is too small.
static int record_cells(Container &con, const std::vector<int> &blk, const std::vector<int> &slot,
                        const std::vector<int> &ci, const std::vector<int> &cj, const std::vector<int> &ck,
                        const long *sel, int m, int *out_id, double *out_pos, double *out_vol, double *out_cen,
                        int *out_nf, int *out_nv, int *out_ok, double *out_mrs, long nb_cap, int *out_nb,
                        long *out_nb_off, long long *out_tests) {
    Computer comp(con);
    std::vector<int> v;
    long used = 0;
    for (int r = 0; r < m; r++) {
        const long t = sel ? sel[r] : r;
        int ijk = blk[t], q = slot[t];
        out_id[r] = con.ids(ijk)[q];
        out_pos[3 * r] = con.pp(ijk)[con.ps * q];
        out_pos[3 * r + 1] = con.pp(ijk)[con.ps * q + 1];
        out_pos[3 * r + 2] = con.pp(ijk)[con.ps * q + 2];
        out_nb_off[r] = used;
        uint64_t t0 = comp.c.side_tests;
        bool ok = comp.compute_cell(ijk, q, ci[t], cj[t], ck[t]);
        if (out_tests) out_tests[r] = (long long)(comp.c.side_tests - t0);
        out_ok[r] = ok ? 1 : 0;
        if (ok) {
            out_vol[r] = comp.c.volume();
            comp.c.centroid(out_cen[3 * r], out_cen[3 * r + 1], out_cen[3 * r + 2]);
            out_nf[r] = comp.c.number_of_faces();
            out_nv[r] = comp.c.p;
            out_mrs[r] = comp.c.max_radius_squared();
            comp.c.neighbors(v);
            for (int x : v) {
                if (used >= nb_cap) return -1;
                out_nb[used++] = x;
            }
        } else {
            out_vol[r] = 0; out_cen[3 * r] = out_cen[3 * r + 1] = out_cen[3 * r + 2] = 0;
            out_nf[r] = 0; out_nv[r] = 0; out_mrs[r] = 0;
        }
    }
    out_nb_off[m] = used;
    return m;
}

int port_compute_cells(int kind, const double *geom, const int *grid, const int *periodic, int n, const int *ids,
                       const double *xyzr, int cap, int *out_id, double *out_pos, double *out_vol, double *out_cen,
                       int *out_nf, int *out_nv, int *out_ok, double *out_mrs, long nb_cap, int *out_nb,
                       long *out_nb_off, long long *out_tests) {
    Container con;
    if (!build(con, kind, geom, grid, periodic, n, ids, xyzr)) return -2;
    std::vector<int> blk, slot, ci, cj, ck;
    con.loop_order(blk, slot, ci, cj, ck);
    int m = (int)blk.size();
    if (m > cap) return -1;
    return record_cells(con, blk, slot, ci, cj, ck, nullptr, m, out_id, out_pos, out_vol, out_cen, out_nf, out_nv,
                        out_ok, out_mrs, nb_cap, out_nb, out_nb_off, out_tests);
}

// The records of the cells at loop-order positions sel[0..nsel) only (a
// sample of a container too large to compute whole on the CPU).  Returns
// nsel, -1 if nb_cap is too small, -3 if a position is out of range.
int port_compute_selected(int kind, const double *geom, const int *grid, const int *periodic, int n,
                          const int *ids, const double *xyzr, int nsel, const long *sel, int *out_id,
                          double *out_pos, double *out_vol, double *out_cen, int *out_nf, int *out_nv, int *out_ok,
                          double *out_mrs, long nb_cap, int *out_nb, long *out_nb_off) {
    Container con;
    if (!build(con, kind, geom, grid, periodic, n, ids, xyzr)) return -2;
    std::vector<int> blk, slot, ci, cj, ck;
    con.loop_order(blk, slot, ci, cj, ck);
    for (int r = 0; r < nsel; r++)
        if (sel[r] < 0 || sel[r] >= (long)blk.size()) return -3;
    return record_cells(con, blk, slot, ci, cj, ck, sel, nsel, out_id, out_pos, out_vol, out_cen, out_nf, out_nv,
                        out_ok, out_mrs, nb_cap, out_nb, out_nb_off, nullptr);
}

// Times compute_cell over the cells [first, first+count) of the loop order
// with `threads` worker threads (each with its own cell and search scratch,
// sharing the read-only container), the work the reference's
// compute_all_cells() does per cell (src/container.cc:438-443).  Returns
// seconds; *done = cells computed; *tests = side tests performed.
double port_time_cells(int kind, const double *geom, const int *grid, const int *periodic, int n, const int *ids,
                       const double *xyzr, long first, long count, int threads, long *done,
                       unsigned long long *tests) {
    Container con;
    if (!build(con, kind, geom, grid, periodic, n, ids, xyzr)) return -1;
    std::vector<int> blk, slot, ci, cj, ck;
    con.loop_order(blk, slot, ci, cj, ck);
    long m = (long)blk.size();
    long lo = std::min(first, m), hi = std::min(first + count, m);
    if (threads < 1) threads = 1;
    std::vector<unsigned long long> tc(threads, 0);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) {
        pool.emplace_back([&, t]() {
            Computer comp(con);
            // interleaved chunks of 64 cells keep the work balanced
            for (long s = lo + 64L * t; s < hi; s += 64L * threads)
                for (long u = s; u < std::min(s + 64, hi); u++) comp.compute_cell(blk[u], slot[u], ci[u], cj[u], ck[u]);
            tc[t] = comp.c.side_tests;
        });
    }
    for (auto &th : pool) th.join();
    auto t1 = std::chrono::steady_clock::now();
    if (done) *done = hi - lo;
    if (tests) {
        unsigned long long s = 0;
        for (auto x : tc) s += x;
        *tests = s;
    }
    return std::chrono::duration<double>(t1 - t0).count();
}

// The worklist table this restatement generates (64 lists x 64 words), for
// comparison with the reference's src/v_base_wl.cc.
int port_worklists(unsigned *out, int cap) {
    const std::vector<unsigned> &w = worklists();
    int m = std::min(cap, (int)w.size());
    for (int i = 0; i < m; i++) out[i] = w[i];
    return (int)w.size();
}

}  // extern "C"
