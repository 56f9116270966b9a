// CPU restatement of the reference's plane-cutting cell — TEST INFRASTRUCTURE.
// Each routine names the reference routine (src/cell.cc) whose steps it follows.
#include "pcell.hh"

#include <cfloat>
#include <cstring>

namespace vport {

const double kTolerance = 10.0 * DBL_EPSILON;
const double kBigTolFac = 20.0;

// voronoicell_base::voronoicell_base (src/cell.cc:20-45)
Cell::Cell(double max_len_sq)
    : tol(kTolerance * max_len_sq), tol_cu(tol * std::sqrt(tol)), big_tol(kBigTolFac * tol) {
    reset_pool(256);
}

void Cell::reset_pool(int hint) {
    pool.clear();
    pool.reserve(hint * 12);
    if ((int)pts.size() < 4 * hint) {
        pts.resize(4 * hint);
        nu.resize(hint);
        off.resize(hint);
        cap.resize(hint);
        bp.resize(hint);
        mask.resize(hint, 0u);
    }
}

void Cell::ensure_vertex(int i) {
    if (i < (int)nu.size()) return;
    int n = (int)nu.size() * 2;
    while (n <= i) n *= 2;
    pts.resize(4 * n);
    nu.resize(n);
    off.resize(n);
    cap.resize(n);
    bp.resize(n);
    mask.resize(n, 0u);
}

int Cell::new_block(int order) {
    int c = 4;
    while (c < order) c *= 2;
    int o = (int)pool.size();
    pool.resize(pool.size() + 3 * c, 0);
    return o | (c << 24);  // packed: offset (low 24 bits) and capacity
}

void Cell::set_order(int i, int order) {
    int b = new_block(order);
    off[i] = b & 0xffffff;
    cap[i] = b >> 24;
}

// Moves vertex `src` into index `dst` (reference: ed[dst]=ed[src]; nu[dst]=nu[src];
// relation fix-up; back pointer reset), e.g. src/cell.cc:850-858,1435-1444
void Cell::move_vertex(int dst, int src) {
    pts[4 * dst] = pts[4 * src];
    pts[4 * dst + 1] = pts[4 * src + 1];
    pts[4 * dst + 2] = pts[4 * src + 2];
    off[dst] = off[src];
    cap[dst] = cap[src];
    nu[dst] = nu[src];
    for (int i = 0; i < nu[dst]; i++) E(E(dst, i), R(dst, i)) = dst;
    bp[dst] = dst;
}

// voronoicell_base::init_base + voronoicell_neighbor::init (src/cell.cc:294-318,
// 2567-2580).  Corner c has bits (x,y,z); its three edges run counter-clockwise
// seen from outside, starting along x for even parity and along y for odd
// parity; the neighbour ID of edge j is the face spanned by edges j-1 and j.
void Cell::init_box(double xmin, double xmax, double ymin, double ymax, double zmin, double zmax,
                    const int ids[6]) {
    reset_pool(256);
    up = 0;
    p = 8;
    xmin *= 2; xmax *= 2; ymin *= 2; ymax *= 2; zmin *= 2; zmax *= 2;
    for (int c = 0; c < 8; c++) {
        pts[4 * c] = (c & 1) ? xmax : xmin;
        pts[4 * c + 1] = (c & 2) ? ymax : ymin;
        pts[4 * c + 2] = (c & 4) ? zmax : zmin;
        pts[4 * c + 3] = 0;
        set_order(c, 3);
        nu[c] = 3;
        bp[c] = c;
        // edge axes in order: choose first axis by parity, then the order with
        // det(e0,e1,e2) < 0 for the edge direction vectors
        int par = __builtin_popcount((unsigned)c) & 1;
        int a0 = par ? 1 : 0;
        int rest[2];
        int m = 0;
        for (int a = 0; a < 3; a++)
            if (a != a0) rest[m++] = a;
        int ax[3] = {a0, rest[0], rest[1]};
        auto dirsign = [&](int a) { return ((c >> a) & 1) ? -1 : 1; };
        // determinant of the signed axis permutation
        int perm_sign = 1;
        {
            int q[3] = {ax[0], ax[1], ax[2]};
            for (int i = 0; i < 3; i++)
                for (int j = i + 1; j < 3; j++)
                    if (q[i] > q[j]) perm_sign = -perm_sign;
        }
        int det = perm_sign * dirsign(ax[0]) * dirsign(ax[1]) * dirsign(ax[2]);
        if (det > 0) { int t = ax[1]; ax[1] = ax[2]; ax[2] = t; }
        for (int j = 0; j < 3; j++) {
            E(c, j) = c ^ (1 << ax[j]);
            R(c, j) = 2 - j;
        }
        for (int j = 0; j < 3; j++) {
            int a = ax[(j + 2) % 3], b = ax[j];
            int face_axis = 3 - a - b;
            int side = (c >> face_axis) & 1;
            N(c, j) = ids[2 * face_axis + side];
        }
    }
    // relation table: R(c,j) = index of the edge at the far vertex pointing back
    for (int c = 0; c < 8; c++)
        for (int j = 0; j < 3; j++) {
            int d = E(c, j);
            for (int q = 0; q < 3; q++)
                if (E(d, q) == c) R(c, j) = q;
        }
}

// voronoicell_neighbor::operator=(voronoicell&) (src/cell.cc:86-95): copies the
// polytope; neighbour IDs become 0
void Cell::copy_from(const Cell &o) {
    reset_pool(std::max(256, o.p + 16));
    ensure_vertex(o.p + 1);
    p = o.p;
    up = 0;
    for (int i = 0; i < p; i++) {
        pts[4 * i] = o.pts[4 * i];
        pts[4 * i + 1] = o.pts[4 * i + 1];
        pts[4 * i + 2] = o.pts[4 * i + 2];
        pts[4 * i + 3] = o.pts[4 * i + 3];
        set_order(i, o.nu[i]);
        nu[i] = o.nu[i];
        bp[i] = i;
        for (int j = 0; j < nu[i]; j++) {
            E(i, j) = o.pool[o.off[i] + j];
            R(i, j) = o.pool[o.off[i] + o.cap[i] + j];
            N(i, j) = 0;
        }
    }
}

void Cell::reset_mask() {
    for (size_t i = 0; i < mask.size(); i++) mask[i] = 0;
    maskc = 4;
}

// m_calc (src/cell.cc:2050-2059)
unsigned Cell::m_calc(int n, double &ans) {
    side_tests++;
    const double *pp = &pts[4 * n];
    ans = pp[0] * px;
    ans += pp[1] * py;
    ans += pp[2] * pz - prsq;
    pts[4 * n + 3] = ans;
    unsigned maskr = ans < -tol ? 0 : (ans > tol ? 2 : 1);
    mask[n] = maskc | maskr;
    return maskr;
}

// m_testx (src/cell.cc:2071-2083)
unsigned Cell::m_testx(int n, double &ans) {
    unsigned maskr;
    if (mask[n] >= maskc) {
        ans = pts[4 * n + 3];
        maskr = mask[n] & 3;
    } else maskr = m_calc(n, ans);
    if (maskr == 0 && ans > -big_tol && bp[n] != -1) {
        bp[n] = -1;
        xse.push_back(n);
    }
    return maskr;
}

// search_for_outside_edge / add_to_stack (src/cell.cc:444-472)
bool Cell::search_for_outside_edge(int &upv) {
    size_t sc2 = ds2.size();
    ds2.push_back(upv);
    size_t j = sc2;
    double l;
    while (j < ds2.size()) {
        upv = ds2[j++];
        for (int i = 0; i < nu[upv]; i++) {
            int lp = E(upv, i);
            unsigned lw = m_test(lp, l);
            if (lw == 0) {
                ds2.resize(sc2);
                return true;
            } else if (lw == 1) add_to_stack((int)sc2, lp);
        }
    }
    ds2.resize(sc2);
    return false;
}

void Cell::add_to_stack(int sc2, int lp) {
    for (size_t k = sc2; k < ds2.size(); k++)
        if (ds2[k] == lp) return;
    ds2.push_back(lp);
}

// search_upward (src/cell.cc:480-518)
bool Cell::search_upward(unsigned &uw, int &lp, int &ls, int &us, double &l, double &u) {
    int vs;
    lp = up;
    l = u;
    for (ls = 0; ls < nu[lp]; ls++) {
        up = E(lp, ls);
        uw = m_test(up, u);
        if (u > l) break;
    }
    if (ls == nu[lp])
        if (definite_max(lp, ls, l, u, uw)) {
            up = lp;
            return false;
        }
    while (uw == 0) {
        vs = R(lp, ls);
        lp = up;
        l = u;
        for (ls = 0; ls < nu[lp]; ls++) {
            if (ls == vs) continue;
            up = E(lp, ls);
            uw = m_test(up, u);
            if (u > l) break;
        }
        if (ls == nu[lp] && definite_max(lp, ls, l, u, uw)) {
            up = lp;
            return false;
        }
    }
    us = R(lp, ls);
    return true;
}

// definite_max (src/cell.cc:520-588)
bool Cell::definite_max(int &lp, int &ls, double &l, double &u, unsigned &uw) {
    int tp = lp, ts, qp = 0;
    unsigned qw;
    double q;
    for (ts = 0; ts < nu[tp]; ts++) {
        qp = E(tp, ts);
        m_test(qp, q);
        if (q > l - big_tol) break;
    }
    if (ts == nu[tp]) return true;
    std::vector<int> st;
    flip(lp);
    flip(qp);
    st.push_back(qp);
    ts++;
    while (ts < nu[tp]) {
        qp = E(tp, ts);
        m_test(qp, q);
        if (q > l - big_tol) {
            st.push_back(up);
            flip(up);
        }
        ts++;
    }
    size_t spp = 0;
    while (spp < st.size()) {
        tp = st[spp++];
        for (ts = 0; ts < nu[tp]; ts++) {
            qp = E(tp, ts);
            if (bp[qp] < 0) continue;
            qw = m_test(qp, q);
            if (q > l) {
                flip(lp);
                lp = tp;
                ls = ts;
                m_test(lp, l);
                up = qp;
                uw = qw;
                u = q;
                while (!st.empty()) { flip(st.back()); st.pop_back(); }
                return false;
            }
            if (q > l - big_tol) {
                st.push_back(qp);
                flip(qp);
            }
        }
    }
    flip(lp);
    while (!st.empty()) { flip(st.back()); st.pop_back(); }
    return true;
}

// search_downward (src/cell.cc:590-628)
bool Cell::search_downward(unsigned &lw, int &lp, int &ls, int &us, double &l, double &u) {
    int vs;
    for (us = 0; us < nu[up]; us++) {
        lp = E(up, us);
        lw = m_test(lp, l);
        if (u > l) break;
    }
    if (us == nu[up])
        if (definite_min(lp, us, l, u, lw)) return false;
    while (lw == 2) {
        vs = R(up, us);
        up = lp;
        u = l;
        for (us = 0; us < nu[up]; us++) {
            if (us == vs) continue;
            lp = E(up, us);
            lw = m_test(lp, l);
            if (u > l) break;
        }
        if (us == nu[up] && definite_min(lp, us, l, u, lw)) return false;
    }
    ls = R(up, us);
    return true;
}

// definite_min (src/cell.cc:630-708)
bool Cell::definite_min(int &lp, int &us, double &l, double &u, unsigned &lw) {
    int tp = up, ts, qp = 0;
    unsigned qw;
    double q;
    for (ts = 0; ts < nu[tp]; ts++) {
        qp = E(tp, ts);
        m_test(qp, q);
        if (q < u + big_tol) break;
    }
    if (ts == nu[tp]) return true;
    std::vector<int> st;
    flip(up);
    flip(qp);
    st.push_back(qp);
    ts++;
    while (ts < nu[tp]) {
        qp = E(tp, ts);
        m_test(qp, q);
        if (q < u + big_tol) {
            st.push_back(lp);
            flip(lp);
        }
        ts++;
    }
    size_t spp = 0;
    while (spp < st.size()) {
        tp = st[spp++];
        for (ts = 0; ts < nu[tp]; ts++) {
            qp = E(tp, ts);
            if (bp[qp] < 0) continue;
            qw = m_test(qp, q);
            if (q < u) {
                flip(up);
                up = tp;
                us = ts;
                m_test(up, u);
                lp = qp;
                lw = qw;
                l = q;
                while (!st.empty()) { flip(st.back()); st.pop_back(); }
                return false;
            }
            if (q < u + big_tol) {
                st.push_back(qp);
                flip(qp);
            }
        }
    }
    flip(up);
    while (!st.empty()) { flip(st.back()); st.pop_back(); }
    return true;
}

// nplane (src/cell.cc:718-870)
bool Cell::nplane(double x, double y, double z, double rsq, int p_id) {
    int i, j, lp = up, cp, qp;
    int us = 0, ls = 0;
    unsigned uw, lw;
    double u, l = 0;
    up = 0;
    ds.clear();
    px = x; py = y; pz = z; prsq = rsq;
    maskc += 4;
    if (maskc < 4) reset_mask();
    uw = m_test(up, u);
    if (uw == 2) {
        if (!search_downward(lw, lp, ls, us, l, u)) return false;
        if (lw == 1) { up = lp; lp = -1; }
    } else if (uw == 0) {
        if (!search_upward(uw, lp, ls, us, l, u)) return true;
        if (uw == 1) lp = -1;
    } else {
        lp = -1;
    }
    ds.clear(); ds2.clear(); xse.clear();
    int op = p;
    if (create_facet(lp, ls, l, us, u, p_id)) return false;
    size_t k = 0;
    while (k < xse.size()) {
        lp = xse[k++];
        uw = m_test(lp, l);
        for (ls = 0; ls < nu[lp]; ls++) {
            up = E(lp, ls);
            uw = m_test(up, u);
            if (up >= op) continue;
            if (uw == 0) {
                if (u > -big_tol && bp[up] != -1) {
                    bp[up] = -1;
                    xse.push_back(up);
                }
            } else if (uw == 1) {
                if (create_facet(-1, 0, 0, 0, u, p_id)) return false;
            } else {
                us = R(lp, ls);
                m_test(lp, l);
                if (create_facet(lp, ls, l, us, u, p_id)) return false;
            }
        }
    }
    for (int v : xse) bp[v] = v;
    // delete stacked vertices: remove duplicates
    size_t dsp = 0;
    while (dsp < ds.size()) {
        j = ds[dsp];
        if (R(j, 0) != -1) {
            R(j, 0) = -1;
            dsp++;
        } else {
            ds[dsp] = ds.back();
            ds.pop_back();
        }
    }
    // auxiliary delete stack
    for (int v : ds2) {
        bp[v] = v;
        if (R(v, 0) != -1) {
            R(v, 0) = -1;
            ds.push_back(v);
        }
    }
    // vertices reachable through deleted ones
    for (dsp = 0; dsp < ds.size(); dsp++) {
        cp = ds[dsp];
        for (int e = 0; e < nu[cp]; e++) {
            qp = E(cp, e);
            if (qp != -1 && R(qp, 0) != -1) {
                ds.push_back(qp);
                R(qp, 0) = -1;
            }
        }
    }
    up = 0;
    while (!ds.empty()) {
        --p;
        while (R(p, 0) == -1) --p;
        up = ds.back();
        ds.pop_back();
        if (up < p) {
            move_vertex(up, p);
        } else up = p++;
    }
    (void)i;
    return collapse_order2();
}

// create_facet (src/cell.cc:874-1364)
bool Cell::create_facet(int lp, int ls, double l, int us, double u, int p_id) {
    int i, j, k, qp, qs, iqs, cp, cs, rp;
    unsigned lw, qw;
    bool new_double_edge = false, double_edge = false;
    double q, r;
    ensure_vertex(p + 1);
    if (lp == -1) {
        if (!search_for_outside_edge(up)) return true;
        pts[4 * p] = pts[4 * up];
        pts[4 * p + 1] = pts[4 * up + 1];
        pts[4 * p + 2] = pts[4 * up + 2];
        i = 0;
        lp = E(up, 0);
        lw = m_testx(lp, l);
        if (lw != 0) {
            unsigned rw = lw;
            do {
                i++;
                if (i == nu[up]) return true;
                lp = E(up, i);
                lw = m_testx(lp, l);
            } while (lw != 0);
            j = i + 1;
            while (j < nu[up]) {
                lp = E(up, j);
                lw = m_testx(lp, l);
                if (lw != 0) break;
                j++;
            }
            int order;
            if (j == nu[up] && i == 1 && rw == 1) {
                order = nu[up];
                double_edge = true;
            } else order = j - i + 2;
            k = 1;
            set_order(p, order);
            nu[p] = order;
            bp[p] = p;
            us = cycle_down(i, up);
            while (i < j) {
                qp = E(up, i);
                qs = R(up, i);
                N(p, k) = N(up, i);
                E(p, k) = qp;
                R(p, k) = qs;
                E(qp, qs) = p;
                R(qp, qs) = k;
                E(up, i) = -1;
                i++;
                k++;
            }
            qs = i == nu[up] ? 0 : i;
        } else {
            i = nu[up] - 1;
            lp = E(up, i);
            lw = m_testx(lp, l);
            while (lw == 0) {
                i--;
                if (i == 0) return false;
                lp = E(up, i);
                lw = m_testx(lp, l);
            }
            j = 1;
            qp = E(up, j);
            qw = m_testx(qp, q);
            while (qw == 0) {
                j++;
                qp = E(up, j);
                qw = m_testx(qp, l);
            }
            int order;
            if (i == j && qw == 1) {
                double_edge = true;
                order = nu[up];
            } else order = nu[up] - i + j + 1;
            k = 1;
            set_order(p, order);
            nu[p] = order;
            bp[p] = p;
            us = i++;
            while (i < nu[up]) {
                qp = E(up, i);
                qs = R(up, i);
                N(p, k) = N(up, i);
                E(p, k) = qp;
                R(p, k) = qs;
                E(qp, qs) = p;
                R(qp, qs) = k;
                E(up, i) = -1;
                i++;
                k++;
            }
            i = 0;
            while (i < j) {
                qp = E(up, i);
                qs = R(up, i);
                N(p, k) = N(up, i);
                E(p, k) = qp;
                R(p, k) = qs;
                E(qp, qs) = p;
                R(qp, qs) = k;
                E(up, i) = -1;
                i++;
                k++;
            }
            qs = j;
        }
        if (!double_edge) {
            N(p, k) = N(up, qs);
            N(p, 0) = p_id;
        } else N(p, 0) = N(up, qs);
        ds2.push_back(up);
        cs = k;
        qp = up;
        q = u;
        i = E(up, us);
        us = R(up, us);
        up = i;
        bp[qp] = -p;
    } else {
        ds.push_back(up);
        r = u / (u - l);
        l = 1 - r;
        pts[4 * p] = pts[4 * lp] * r + pts[4 * up] * l;
        pts[4 * p + 1] = pts[4 * lp + 1] * r + pts[4 * up + 1] * l;
        pts[4 * p + 2] = pts[4 * lp + 2] * r + pts[4 * up + 2] * l;
        nu[p] = 3;
        set_order(p, 3);
        bp[p] = p;
        N(p, 0) = p_id;
        N(p, 1) = N(up, us);
        N(p, 2) = N(lp, ls);
        E(up, us) = -1;
        E(lp, ls) = p;
        R(lp, ls) = 1;
        E(p, 1) = lp;
        R(p, 1) = ls;
        cs = 2;
        qs = cycle_up(us, up);
        qp = up;
        q = u;
    }
    cp = p;
    rp = p;
    p++;
    while (qp != up || qs != us) {
        lp = E(qp, qs);
        lw = m_testx(lp, l);
        if (lw == 2) {
            qs = cycle_up(R(qp, qs), lp);
            qp = lp;
            q = l;
            ds.push_back(qp);
        } else if (lw == 0) {
            ensure_vertex(p + 1);
            r = q / (q - l);
            l = 1 - r;
            pts[4 * p] = pts[4 * lp] * r + pts[4 * qp] * l;
            pts[4 * p + 1] = pts[4 * lp + 1] * r + pts[4 * qp + 1] * l;
            pts[4 * p + 2] = pts[4 * lp + 2] * r + pts[4 * qp + 2] * l;
            nu[p] = 3;
            set_order(p, 3);
            ls = R(qp, qs);
            N(p, 0) = p_id;
            N(p, 1) = N(qp, qs);
            N(p, 2) = N(lp, ls);
            E(p, 0) = cp;
            E(p, 1) = lp;
            R(p, 0) = cs;
            R(p, 1) = ls;
            bp[p] = p;
            E(lp, ls) = p;
            R(lp, ls) = 1;
            E(cp, cs) = p;
            R(cp, cs) = 0;
            E(qp, qs) = -1;
            qs = cycle_up(qs, qp);
            cp = p++;
            cs = 2;
        } else {
            ensure_vertex(p + 1);
            k = double_edge ? 0 : 1;
            qs = R(qp, qs);
            qp = lp;
            iqs = qs;
            do {
                k++;
                qs = cycle_up(qs, qp);
                lp = E(qp, qs);
                lw = m_testx(lp, l);
            } while (lw == 0);
            j = -bp[qp];
            if (qp == up && qs == us) {
                new_double_edge = false;
                if (j > 0) k += nu[j];
            } else {
                if (j > 0) {
                    k += nu[j];
                    if (lw == 1) {
                        i = -bp[lp];
                        if (i > 0) {
                            if (E(i, nu[i] - 1) == j) {
                                new_double_edge = true;
                                k -= 1;
                            } else new_double_edge = false;
                        } else {
                            if (j == rp && lp == up && R(qp, qs) == us) {
                                new_double_edge = true;
                                k -= 1;
                            } else new_double_edge = false;
                        }
                    } else new_double_edge = false;
                } else {
                    if (lw == 1) {
                        i = -bp[lp];
                        if (i == cp) {
                            new_double_edge = true;
                            k -= 1;
                        } else new_double_edge = false;
                    } else new_double_edge = false;
                }
            }
            if (j > 0) {
                if (nu[j] != k) {
                    // grow vertex j to order k, keeping its edges (src/cell.cc:1237-1270)
                    int oo = off[j], oc = cap[j], on = nu[j];
                    std::vector<int> te(on), tr(on), tn(on);
                    for (int t = 0; t < on; t++) {
                        te[t] = pool[oo + t];
                        tr[t] = pool[oo + oc + t];
                        tn[t] = pool[oo + 2 * oc + t];
                    }
                    set_order(j, k);
                    for (int t = 0; t < on; t++) {
                        E(j, t) = te[t];
                        R(j, t) = tr[t];
                        N(j, t) = tn[t];
                    }
                    bp[j] = j;
                    i = on;
                } else i = nu[j];
            } else {
                set_order(p, k);
                bp[p] = p;
                ds2.push_back(qp);
                pts[4 * p] = pts[4 * qp];
                pts[4 * p + 1] = pts[4 * qp + 1];
                pts[4 * p + 2] = pts[4 * qp + 2];
                bp[qp] = -p;
                j = p++;
                i = 0;
            }
            nu[j] = k;
            if (!double_edge) {
                E(j, i) = cp;
                R(j, i) = cs;
                N(j, i) = p_id;
                E(cp, cs) = j;
                R(cp, cs) = i;
                i++;
            }
            qs = iqs;
            while (i < (new_double_edge ? k : k - 1)) {
                qs = cycle_up(qs, qp);
                lp = E(qp, qs);
                ls = R(qp, qs);
                N(j, i) = N(qp, qs);
                E(j, i) = lp;
                R(j, i) = ls;
                E(lp, ls) = j;
                R(lp, ls) = i;
                E(qp, qs) = -1;
                i++;
            }
            qs = cycle_up(qs, qp);
            cs = i;
            cp = j;
            N(j, new_double_edge ? 0 : cs) = N(qp, qs);
            double_edge = new_double_edge;
        }
    }
    E(cp, cs) = rp;
    E(rp, 0) = cp;
    R(cp, cs) = 0;
    R(rp, 0) = cs;
    return false;
}

// collapse_order2 (src/cell.cc:1376-1428).  The reference takes order-two
// vertices from its per-order memory pool; this restatement takes the highest
// index, which only matters in degenerate cases.
bool Cell::collapse_order2() {
    if (!collapse_order1()) return false;
    for (;;) {
        int i = -1;
        for (int v = p - 1; v >= 0; v--)
            if (nu[v] == 2) { i = v; break; }
        if (i < 0) break;
        int j = E(i, 0), k = E(i, 1);
        if (j == k) return false;
        int l;
        for (l = 0; l < nu[j]; l++)
            if (E(j, l) == k) break;
        int a = R(i, 0), b = R(i, 1);
        if (l == nu[j]) {
            E(j, a) = k;
            E(k, b) = j;
            R(j, a) = b;
            R(k, b) = a;
        } else {
            if (!delete_connection(j, a, false)) return false;
            if (!delete_connection(k, b, true)) return false;
        }
        --p;
        if (up == i) up = 0;
        if (p != i) {
            if (up == p) up = i;
            move_vertex(i, p);
        }
        if (!collapse_order1()) return false;
    }
    return true;
}

// collapse_order1 (src/cell.cc:1436-1464)
bool Cell::collapse_order1() {
    for (;;) {
        int i = -1;
        for (int v = p - 1; v >= 0; v--)
            if (nu[v] == 1) { i = v; break; }
        if (i < 0) break;
        up = 0;
        int j = E(i, 0), k = R(i, 0);
        if (!delete_connection(j, k, false)) return false;
        --p;
        if (up == i) up = 0;
        if (p != i) {
            if (up == p) up = i;
            move_vertex(i, p);
        }
    }
    return true;
}

// delete_connection (src/cell.cc:1472-1513)
bool Cell::delete_connection(int j, int k, bool hand) {
    int q = hand ? k : cycle_up(k, j);
    int i = nu[j] - 1;
    if (i < 1) return false;
    int on = nu[j];
    std::vector<int> te(i), tr(i), tn(i);
    int l;
    for (l = 0; l < q; l++) tn[l] = N(j, l);
    while (l < i) {
        tn[l] = N(j, l + 1);
        l++;
    }
    for (l = 0; l < k; l++) {
        te[l] = E(j, l);
        tr[l] = R(j, l);
    }
    while (l < i) {
        int m = E(j, l + 1);
        te[l] = m;
        int kk = R(j, l + 1);
        tr[l] = kk;
        R(m, kk)--;
        l++;
    }
    (void)on;
    set_order(j, i);
    for (l = 0; l < i; l++) {
        E(j, l) = te[l];
        R(j, l) = tr[l];
        N(j, l) = tn[l];
    }
    bp[j] = j;
    nu[j] = i;
    return true;
}

// reset_edges (src/cell.cc:2025-2031)
void Cell::reset_edges() {
    for (int i = 0; i < p; i++)
        for (int j = 0; j < nu[i]; j++) E(i, j) = -1 - E(i, j);
}

// volume (src/cell.cc:1584-1616)
double Cell::volume() {
    const double fe = 1 / 48.0;
    double vol = 0;
    int i, j, k, l, m, n;
    double ux, uy, uz, vx, vy, vz, wx, wy, wz;
    for (i = 1; i < p; i++) {
        ux = pts[0] - pts[4 * i];
        uy = pts[1] - pts[4 * i + 1];
        uz = pts[2] - pts[4 * i + 2];
        for (j = 0; j < nu[i]; j++) {
            k = E(i, j);
            if (k >= 0) {
                E(i, j) = -1 - k;
                l = cycle_up(R(i, j), k);
                vx = pts[4 * k] - pts[0];
                vy = pts[4 * k + 1] - pts[1];
                vz = pts[4 * k + 2] - pts[2];
                m = E(k, l);
                E(k, l) = -1 - m;
                while (m != i) {
                    n = cycle_up(R(k, l), m);
                    wx = pts[4 * m] - pts[0];
                    wy = pts[4 * m + 1] - pts[1];
                    wz = pts[4 * m + 2] - pts[2];
                    vol += ux * vy * wz + uy * vz * wx + uz * vx * wy - uz * vy * wx - uy * vx * wz - ux * vz * wy;
                    k = m;
                    l = n;
                    vx = wx;
                    vy = wy;
                    vz = wz;
                    m = E(k, l);
                    E(k, l) = -1 - m;
                }
            }
        }
    }
    reset_edges();
    return vol * fe;
}

// centroid (src/cell.cc:1861-1901)
void Cell::centroid(double &cx, double &cy, double &cz) {
    double tvol, vol = 0;
    cx = cy = cz = 0;
    int i, j, k, l, m, n;
    double ux, uy, uz, vx, vy, vz, wx, wy, wz;
    for (i = 1; i < p; i++) {
        ux = pts[0] - pts[4 * i];
        uy = pts[1] - pts[4 * i + 1];
        uz = pts[2] - pts[4 * i + 2];
        for (j = 0; j < nu[i]; j++) {
            k = E(i, j);
            if (k >= 0) {
                E(i, j) = -1 - k;
                l = cycle_up(R(i, j), k);
                vx = pts[4 * k] - pts[0];
                vy = pts[4 * k + 1] - pts[1];
                vz = pts[4 * k + 2] - pts[2];
                m = E(k, l);
                E(k, l) = -1 - m;
                while (m != i) {
                    n = cycle_up(R(k, l), m);
                    wx = pts[4 * m] - pts[0];
                    wy = pts[4 * m + 1] - pts[1];
                    wz = pts[4 * m + 2] - pts[2];
                    tvol = ux * vy * wz + uy * vz * wx + uz * vx * wy - uz * vy * wx - uy * vx * wz - ux * vz * wy;
                    vol += tvol;
                    cx += (wx + vx - ux) * tvol;
                    cy += (wy + vy - uy) * tvol;
                    cz += (wz + vz - uz) * tvol;
                    k = m;
                    l = n;
                    vx = wx;
                    vy = wy;
                    vz = wz;
                    m = E(k, l);
                    E(k, l) = -1 - m;
                }
            }
        }
    }
    reset_edges();
    if (vol > tol_cu) {
        vol = 0.125 / vol;
        cx = cx * vol + 0.5 * pts[0];
        cy = cy * vol + 0.5 * pts[1];
        cz = cz * vol + 0.5 * pts[2];
    } else cx = cy = cz = 0;
}

// max_radius_squared (src/cell.cc:1907-1917)
double Cell::max_radius_squared() const {
    double r = pts[0] * pts[0] + pts[1] * pts[1] + pts[2] * pts[2], s;
    for (int i = 1; i < p; i++) {
        s = pts[4 * i] * pts[4 * i];
        s += pts[4 * i + 1] * pts[4 * i + 1];
        s += pts[4 * i + 2] * pts[4 * i + 2];
        if (s > r) r = s;
    }
    return r;
}

// number_of_faces (src/cell.cc:2168-2187)
int Cell::number_of_faces() {
    int i, j, k, l, m, s = 0;
    for (i = 1; i < p; i++)
        for (j = 0; j < nu[i]; j++) {
            k = E(i, j);
            if (k >= 0) {
                s++;
                E(i, j) = -1 - k;
                l = cycle_up(R(i, j), k);
                do {
                    m = E(k, l);
                    E(k, l) = -1 - m;
                    l = cycle_up(R(k, l), m);
                    k = m;
                } while (k != i);
            }
        }
    reset_edges();
    return s;
}

// voronoicell_neighbor::neighbors (src/cell.cc:2660-2678)
void Cell::neighbors(std::vector<int> &v) {
    v.clear();
    int i, j, k, l, m;
    for (i = 1; i < p; i++)
        for (j = 0; j < nu[i]; j++) {
            k = E(i, j);
            if (k >= 0) {
                v.push_back(N(i, j));
                E(i, j) = -1 - k;
                l = cycle_up(R(i, j), k);
                do {
                    m = E(k, l);
                    E(k, l) = -1 - m;
                    l = cycle_up(R(k, l), m);
                    k = m;
                } while (k != i);
            }
        }
    reset_edges();
}

// plane_intersects, plane_intersects_guess, plane_intersects_track (src/cell.cc:2366-2409)
bool Cell::plane_intersects(double x, double y, double z, double rsq) {
    double g = x * pts[4 * up] + y * pts[4 * up + 1] + z * pts[4 * up + 2];
    if (g < rsq) {
        for (int tp = 0; tp < p; tp++)
            if (x * pts[4 * tp] + y * pts[4 * tp + 1] + z * pts[4 * tp + 2] > rsq) return true;
        return false;
    }
    return true;
}

bool Cell::plane_intersects_guess(double x, double y, double z, double rsq) {
    up = 0;
    double g = x * pts[4 * up] + y * pts[4 * up + 1] + z * pts[4 * up + 2];
    if (g < rsq) {
        int ca = 1, cc = p >> 3, mp = 1;
        double m;
        while (ca < cc) {
            m = x * pts[4 * mp] + y * pts[4 * mp + 1] + z * pts[4 * mp + 2];
            if (m > g) {
                if (m > rsq) return true;
                g = m;
                up = mp;
            }
            ca += mp++;
        }
        for (int tp = 0; tp < p; tp++)
            if (x * pts[4 * tp] + y * pts[4 * tp + 1] + z * pts[4 * tp + 2] > rsq) return true;
        return false;
    }
    return true;
}

}  // namespace vport
