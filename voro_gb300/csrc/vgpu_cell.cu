// The per-cell engine: one warp computes one Voronoi cell.
//
// It replaces voro_compute::compute_cell (src/v_compute.cc:289-621) and the
// voronoicell_base plane-cutting engine (nplane, src/cell.cc:718-870;
// create_facet 874-1364; collapse_order2/1 1376-1464; delete_connection
// 1472-1513; plane_intersects 2366-2409) plus the per-cell reductions
// (volume 1584-1616, centroid 1861-1901, number_of_faces 2168-2187,
// neighbors 2660-2678), with a different representation chosen for warps:
//
//  * A cell is a convex polyhedron stored by its vertices.  Every vertex is
//    the meeting point of three planes (a,b,c), stored as a "triangle" of
//    plane indices oriented so that det(n_a,n_b,n_c) > 0 (faces counter-
//    clockwise seen from outside), plus the three neighbouring vertices across
//    its three edges.  Lane l owns vertex slots l, l+32, ... in registers.
//  * A candidate plane is tested against all vertices at once (one side test
//    per lane and slot, then a ballot).  The common case — the plane misses —
//    costs a handful of instructions.  A cut removes the vertices outside,
//    finds the boundary of the removed region (a cycle of edges), and adds one
//    new vertex per boundary edge; slots are reused through bit masks.
//  * Side tests run in FP32 (MIXED mode) under a forward error bound: a test
//    is certain when |value| exceeds the bound plus the reference tolerance;
//    otherwise it is redone in FP64 from the planes' double-precision source.
//    A vertex still inside the reference's tolerance band (|value| <= tol,
//    src/cell.cc:2050-2059) marks the cell MARGINAL: there the reference
//    merges vertices and the topology depends on its insertion order.
//  * Candidates come from the engine's own block grid, gathered shell by shell
//    in order of the blocks' lower-bound distance and sorted by (power)
//    distance inside a batch, with the same radius cut-off as the reference's
//    r_ctest / r_scale_check (src/rad_option.hh:320-341,387-431).
//  * Final vertices are rebuilt in FP64 from their three planes; volume and
//    centroid are accumulated in FP64 over the cell's edges.
#include <cfloat>
#include <cstdio>
#include "vgpu_internal.cuh"
#include "../../include/vorogpu.h"

namespace vgpu {

namespace {

constexpr float kU32 = 5.9604645e-08f;          // 2^-24
constexpr double kU64 = 1.1102230246251565e-16; // 2^-53
constexpr unsigned kFull = 0xffffffffu;

// Initial box: eight corners as plane triangles and their neighbours.  Planes
// 0..5 are -x,+x,-y,+y,-z,+z.  Filled from the host (see build_box_tables).
__constant__ unsigned c_box_tri[8];
__constant__ unsigned c_box_adj[8];

// ------------------------------------------------------------------ masks
template <int K>
struct Mask {
    static constexpr int W = (K + 1) / 2;
    unsigned long long w[W];
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int i = 0; i < W; i++) w[i] = 0ull;
    }
    __device__ __forceinline__ bool test(int t) const { return (w[t >> 6] >> (t & 63)) & 1ull; }
    __device__ __forceinline__ void set(int t) { w[t >> 6] |= 1ull << (t & 63); }
    __device__ __forceinline__ int popc() const {
        int c = 0;
#pragma unroll
        for (int i = 0; i < W; i++) c += __popcll(w[i]);
        return c;
    }
    __device__ __forceinline__ bool any() const {
        unsigned long long o = 0;
#pragma unroll
        for (int i = 0; i < W; i++) o |= w[i];
        return o != 0ull;
    }
    __device__ __forceinline__ bool equals(const Mask &o) const {
        bool e = true;
#pragma unroll
        for (int i = 0; i < W; i++) e = e && (w[i] == o.w[i]);
        return e;
    }
    // position of the j-th (0-based) set bit, or -1
    __device__ __forceinline__ int nth(int j) const {
#pragma unroll
        for (int i = 0; i < W; i++) {
            int c = __popcll(w[i]);
            if (j < c) {
                unsigned long long x = w[i];
                for (int q = 0; q < j; q++) x &= x - 1ull;
                return i * 64 + __ffsll((long long)x) - 1;
            }
            j -= c;
        }
        return -1;
    }
};

// ballot of a per-slot predicate into a mask: slot s of lane l is bit l+32s
template <int K>
__device__ __forceinline__ Mask<K> ballot_mask(const bool (&pred)[K]) {
    Mask<K> m;
    m.clear();
#pragma unroll
    for (int s = 0; s < K; s++) {
        unsigned b = __ballot_sync(kFull, pred[s]);
        m.w[s >> 1] |= (unsigned long long)b << (32 * (s & 1));
    }
    return m;
}

__device__ __forceinline__ unsigned long long warp_or64(unsigned long long x) {
    unsigned lo = __reduce_or_sync(kFull, (unsigned)x);
    unsigned hi = __reduce_or_sync(kFull, (unsigned)(x >> 32));
    return ((unsigned long long)hi << 32) | lo;
}
__device__ __forceinline__ float warp_maxf(float x) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x = fmaxf(x, __shfl_xor_sync(kFull, x, d));
    return x;
}
__device__ __forceinline__ double warp_sumd(double x) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(kFull, x, d);
    return x;
}
__device__ __forceinline__ double warp_maxd(double x) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x = fmax(x, __shfl_xor_sync(kFull, x, d));
    return x;
}

// plane indices are always < kMaxPlanes; the mask keeps every shared-memory
// index in bounds even if a slot held inconsistent data
__device__ __forceinline__ int tri_plane(unsigned t, int e) { return (t >> (8 * e)) & (kMaxPlanes - 1); }

// Sortable key of a float (total order as unsigned)
__device__ __forceinline__ unsigned float_key(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ------------------------------------------------------------------ shared memory per warp
template <int K>
struct WarpShared {
    float4 pl[kMaxPlanes];      // plane n.x, n.y, n.z, h  (n.v <= h inside)
    float4 pe[kMaxPlanes];      // |n|, en (abs error of n), eh (abs error of h), |h|
    double4 pl64[kMaxPlanes];   // FP64 plane (box planes always; others when needed)
    int pid[kMaxPlanes];        // neighbour ID of the plane
    int psrc[kMaxPlanes];       // engine index of the generating particle, -1 for initial faces
    int pshift[kMaxPlanes];     // packed periodic image counts
    unsigned tri[32 * K];
    unsigned adj[32 * K];
    unsigned char startN[kMaxPlanes];
    unsigned char endN[kMaxPlanes];
    unsigned ck[kCandBuf];      // candidate sort keys
    int cj[kCandBuf];           // candidate engine index
    int cs[kCandBuf];           // candidate packed image counts
    union {
        struct {
            float4 cd[kCandBuf];      // candidate plane (FP32): n, h
            float4 ce[kCandBuf];      // en, eh, dist2, rs
            double4 cd64[kCandBuf];   // candidate plane (FP64), FP64 mode
        } c;
        struct {
            double4 vtx[32 * K];      // final FP64 vertices (after the search)
        } f;
    } u;
    double4 foot[kMaxPlanes];   // final stage: foot point of each live plane
};

// ------------------------------------------------------------------ per-lane vertex registers
template <int MODE, int K>
struct Verts {
    unsigned tri[K];
    float x[K], y[K], z[K], a[K], e[K];   // FP32 position, |v|, error bound
    double dx[K], dy[K], dz[K];           // FP64 mode positions
};

struct CellCtx {
    double4 me64;     // particle (remapped position, radius)
    float4 me32;      // local coords, radius
    int bi, bj, bk;   // engine block coordinates
    int k;            // engine index
    float R2;         // upper bound of max |v|^2
    float cutoff2;    // squared distance bound for candidates / blocks
    float ri2;        // particle radius squared (poly)
    bool deleted;
    bool overflow;
    bool marginal;
    bool repaired;
    unsigned long long freeplanes;
    int ncand;
    unsigned long long tests, repairs, ptested, pcut;
};

__device__ __forceinline__ int unpack_shift(int code, int a) { return ((code >> (8 * a)) & 255) - 128; }

// FP64 plane of a candidate (engine index j, image counts) relative to the
// particle, with the reference's own arithmetic: x1 = p_j - (x - qx)
// (src/v_compute.cc:383-397) and rs = x1*x1+y1*y1+z1*z1 [+ r_i^2 - r_j^2]
// (r_scale, src/rad_option.hh:414-416).  h = rs/2 (the reference works in
// doubled coordinates; halving is exact).
__device__ __forceinline__ double4 plane64_from(const CellParams &P, const CellCtx &C, int j, int code) {
    double4 q = P.a.p64[j];
    double sx = unpack_shift(code, 0) * P.g.len[0];
    double sy = unpack_shift(code, 1) * P.g.len[1];
    double sz = unpack_shift(code, 2) * P.g.len[2];
    double x1 = __dsub_rn(q.x, __dsub_rn(C.me64.x, sx));
    double y1 = __dsub_rn(q.y, __dsub_rn(C.me64.y, sy));
    double z1 = __dsub_rn(q.z, __dsub_rn(C.me64.z, sz));
    double rs = __dadd_rn(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)), __dmul_rn(z1, z1));
    if (P.g.poly) rs = __dsub_rn(__dadd_rn(rs, __dmul_rn(C.me64.w, C.me64.w)), __dmul_rn(q.w, q.w));
    return make_double4(x1, y1, z1, 0.5 * rs);
}

template <int K>
__device__ __forceinline__ double4 plane64_of(const CellParams &P, const CellCtx &C, WarpShared<K> &S, int p) {
    int src = S.psrc[p];
    if (src < 0) return S.pl64[p];
    return plane64_from(P, C, src, S.pshift[p]);
}

// Vertex of planes (a,b,c) in FP32 with a forward error bound (absolute,
// Euclidean) covering the planes' own storage error and the rounding of this
// Cramer solve.  Returns false if the planes are (numerically) dependent.
template <int K>
__device__ __forceinline__ bool solve_f32(const WarpShared<K> &S, unsigned t, float &x, float &y, float &z,
                                          float &va, float &ve) {
    const int a = tri_plane(t, 0), b = tri_plane(t, 1), c = tri_plane(t, 2);
    const float4 A = S.pl[a], B = S.pl[b], Cc = S.pl[c];
    const float4 EA = S.pe[a], EB = S.pe[b], EC = S.pe[c];
    float bcx = B.y * Cc.z - B.z * Cc.y, bcy = B.z * Cc.x - B.x * Cc.z, bcz = B.x * Cc.y - B.y * Cc.x;
    float cax = Cc.y * A.z - Cc.z * A.y, cay = Cc.z * A.x - Cc.x * A.z, caz = Cc.x * A.y - Cc.y * A.x;
    float abx = A.y * B.z - A.z * B.y, aby = A.z * B.x - A.x * B.z, abz = A.x * B.y - A.y * B.x;
    float D = A.x * bcx + A.y * bcy + A.z * bcz;
    float inv = 1.0f / D;
    x = (A.w * bcx + B.w * cax + Cc.w * abx) * inv;
    y = (A.w * bcy + B.w * cay + Cc.w * aby) * inv;
    z = (A.w * bcz + B.w * caz + Cc.w * abz) * inv;
    va = sqrtf(x * x + y * y + z * z);
    float nbc = fabsf(bcx) + fabsf(bcy) + fabsf(bcz);
    float nca = fabsf(cax) + fabsf(cay) + fabsf(caz);
    float nab = fabsf(abx) + fabsf(aby) + fabsf(abz);
    const float r8 = 8.0f * kU32;
    float ra = EA.z + EA.y * va + r8 * (EA.w + EA.x * va);
    float rb = EB.z + EB.y * va + r8 * (EB.w + EB.x * va);
    float rc = EC.z + EC.y * va + r8 * (EC.w + EC.x * va);
    ve = 2.0f * (nbc * ra + nca * rb + nab * rc) / fabsf(D) + r8 * va;
    bool good = D > 0.0f && isfinite(x) && isfinite(y) && isfinite(z) && isfinite(ve);
    if (!good) { ve = 3.0e38f; }
    return good;
}

// Vertex of three FP64 planes by Cramer's rule.
__device__ __forceinline__ void solve_f64(const double4 A, const double4 B, const double4 C, double &x, double &y,
                                          double &z, double &D, double &kappa_num) {
    double bcx = B.y * C.z - B.z * C.y, bcy = B.z * C.x - B.x * C.z, bcz = B.x * C.y - B.y * C.x;
    double cax = C.y * A.z - C.z * A.y, cay = C.z * A.x - C.x * A.z, caz = C.x * A.y - C.y * A.x;
    double abx = A.y * B.z - A.z * B.y, aby = A.z * B.x - A.x * B.z, abz = A.x * B.y - A.y * B.x;
    D = A.x * bcx + A.y * bcy + A.z * bcz;
    double inv = 1.0 / D;
    x = (A.w * bcx + B.w * cax + C.w * abx) * inv;
    y = (A.w * bcy + B.w * cay + C.w * aby) * inv;
    z = (A.w * bcz + B.w * caz + C.w * abz) * inv;
    // sum over rows of |cofactor row| * (|h| + |n||v|), used for the error bound
    float vv = (float)sqrt(x * x + y * y + z * z);
    float nbc = fabsf((float)bcx) + fabsf((float)bcy) + fabsf((float)bcz);
    float nca = fabsf((float)cax) + fabsf((float)cay) + fabsf((float)caz);
    float nab = fabsf((float)abx) + fabsf((float)aby) + fabsf((float)abz);
    float na = fabsf((float)A.x) + fabsf((float)A.y) + fabsf((float)A.z);
    float nb = fabsf((float)B.x) + fabsf((float)B.y) + fabsf((float)B.z);
    float nc = fabsf((float)C.x) + fabsf((float)C.y) + fabsf((float)C.z);
    kappa_num = nbc * (fabsf((float)A.w) + na * vv) + nca * (fabsf((float)B.w) + nb * vv) +
                nab * (fabsf((float)C.w) + nc * vv);
}

// FP64 side test of one vertex against plane Q, returning 2 outside, 0 inside,
// 1 inside the reference tolerance band (marginal).
__device__ __forceinline__ int side64(const double4 Q, double x, double y, double z, double D, double kappa_num,
                                      double tol_h) {
    double s = fma(Q.x, x, fma(Q.y, y, fma(Q.z, z, -Q.w)));
    double vv = sqrt(x * x + y * y + z * z);
    double nq = fabs(Q.x) + fabs(Q.y) + fabs(Q.z);
    double verr = 16.0 * kU64 * kappa_num / fabs(D) + 64.0 * kU64 * vv;
    double bnd = nq * verr + 8.0 * kU64 * (nq * vv + fabs(Q.w));
    if (s > tol_h + bnd) return 2;
    if (s < -(tol_h + bnd)) return 0;
    return 1;
}

// ------------------------------------------------------------------ warp sort of candidate keys
__device__ __forceinline__ void bitonic32(unsigned &x, int lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            unsigned y = __shfl_xor_sync(kFull, x, j);
            bool up = (lane & k) == 0;
            bool lower = (lane & j) == 0;
            x = (lower == up) ? min(x, y) : max(x, y);
        }
    }
}
__device__ __forceinline__ void bitonic64(unsigned &x0, unsigned &x1, int lane) {
#pragma unroll
    for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j == 32) {
                unsigned a = min(x0, x1), b = max(x0, x1);
                x0 = a;
                x1 = b;
            } else {
                unsigned y0 = __shfl_xor_sync(kFull, x0, j);
                unsigned y1 = __shfl_xor_sync(kFull, x1, j);
                bool lower = (lane & j) == 0;
                bool up0 = ((lane)&k) == 0;
                bool up1 = ((lane + 32) & k) == 0;
                x0 = (lower == up0) ? min(x0, y0) : max(x0, y0);
                x1 = (lower == up1) ? min(x1, y1) : max(x1, y1);
            }
        }
    }
}

// ------------------------------------------------------------------ the engine
template <int MODE, int K>
struct Engine {
    const CellParams &P;
    WarpShared<K> &S;
    const int *offsets;   // shared copy of the offset table
    int lane;
    Verts<MODE, K> V;
    Mask<K> Vm;           // valid vertex slots
    CellCtx C;

    __device__ Engine(const CellParams &p, WarpShared<K> &s, const int *off, int l) : P(p), S(s), offsets(off), lane(l) {}

    // ---- bound of max |v|^2 and the candidate cut-off
    __device__ void update_radius() {
        float m = 0.0f;
#pragma unroll
        for (int s = 0; s < K; s++) {
            if (Vm.test(lane + 32 * s)) {
                float r;
                if (MODE == VGPU_FP64) {
                    r = (float)sqrt(V.dx[s] * V.dx[s] + V.dy[s] * V.dy[s] + V.dz[s] * V.dz[s]);
                    r = r * (1.0f + 4.0f * kU32);
                } else {
                    r = (V.a[s] + V.e[s]) * (1.0f + 4.0f * kU32);
                }
                m = fmaxf(m, r * r);
            }
        }
        C.R2 = warp_maxf(m) * (1.0f + 4.0f * kU32);
        if (P.g.poly) {
            float R = sqrtf(C.R2);
            float q = C.R2 + P.g.rmax32 * P.g.rmax32 - C.ri2;
            float D = R + sqrtf(fmaxf(q, 0.0f));
            C.cutoff2 = D * D * (1.0f + 8.0f * kU32);
        } else {
            C.cutoff2 = 4.0f * C.R2;
        }
    }

    // ---- initial cell: container box (src/container.hh:191-203, src/cell.cc:294-318,2567-2580)
    //      or the periodic unit cell (src/container_prd.hh:124-131)
    __device__ void init_cell(int k) {
        C.k = k;
        C.me64 = P.a.p64[k];
        C.me32 = P.a.l32[k];
        int b = P.a.gblock[k];
        C.bi = b % P.g.gn[0];
        C.bj = (b / P.g.gn[0]) % P.g.gn[1];
        C.bk = b / (P.g.gn[0] * P.g.gn[1]);
        C.ri2 = C.me32.w * C.me32.w;
        C.deleted = C.overflow = C.marginal = C.repaired = false;
        C.freeplanes = ~0x3full;
        C.ncand = 0;
        C.tests = C.repairs = C.ptested = C.pcut = 0;
        if (lane < 6) {
            int ax = lane >> 1;
            bool hiside = lane & 1;
            double xa = ax == 0 ? C.me64.x : (ax == 1 ? C.me64.y : C.me64.z);
            double h;
            if (P.g.unit_cell || P.g.per[ax]) {
                h = 0.5 * P.g.len[ax];
            } else {
                h = hiside ? __dsub_rn(P.g.hi[ax], xa) : -__dsub_rn(P.g.lo[ax], xa);
            }
            double n = hiside ? 1.0 : -1.0;
            double4 q = make_double4(ax == 0 ? n : 0.0, ax == 1 ? n : 0.0, ax == 2 ? n : 0.0, h);
            S.pl64[lane] = q;
            S.pl[lane] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)h);
            float hf = fabsf((float)h);
            S.pe[lane] = make_float4(1.0f, 0.0f, 2.0f * kU32 * hf, hf);
            S.pid[lane] = P.g.unit_cell ? 0 : -(lane + 1);
            S.psrc[lane] = -1;
            S.pshift[lane] = 0;
        }
        Vm.clear();
#pragma unroll
        for (int s = 0; s < K; s++) V.tri[s] = 0;
        if (lane < 8) {
            S.tri[lane] = c_box_tri[lane];
            S.adj[lane] = c_box_adj[lane];
            V.tri[0] = c_box_tri[lane];
        }
        for (int t = 0; t < 8; t++) Vm.set(t);
        __syncwarp();
        if (lane < 8) compute_vertex(0);
        update_radius();
    }

    // ---- vertex of slot s (planes from shared memory)
    __device__ void compute_vertex(int s) {
        unsigned t = V.tri[s];
        if (MODE == VGPU_FP64) {
            double D, kn;
            solve_f64(S.pl64[tri_plane(t, 0)], S.pl64[tri_plane(t, 1)], S.pl64[tri_plane(t, 2)], V.dx[s], V.dy[s],
                      V.dz[s], D, kn);
            V.e[s] = (float)(16.0 * kU64 * kn / fabs(D) + 64.0 * kU64 * sqrt(V.dx[s] * V.dx[s] + V.dy[s] * V.dy[s] + V.dz[s] * V.dz[s]));
            V.a[s] = (float)D;   // orientation check value
            if (!(D > 0.0)) C.marginal = true;
        } else {
            bool ok = solve_f32<K>(S, t, V.x[s], V.y[s], V.z[s], V.a[s], V.e[s]);
            (void)ok;  // a dependent triple leaves an infinite error bound: every test on it is repaired in FP64
        }
    }

    // ---- plane slot allocation with recycling of dead planes
    __device__ int alloc_plane() {
        if (C.freeplanes == 0ull) {
            unsigned long long live = 0ull;
#pragma unroll
            for (int s = 0; s < K; s++)
                if (Vm.test(lane + 32 * s)) {
                    unsigned t = V.tri[s];
                    live |= (1ull << tri_plane(t, 0)) | (1ull << tri_plane(t, 1)) | (1ull << tri_plane(t, 2));
                }
            live = warp_or64(live);
            C.freeplanes = ~live;
            if (C.freeplanes == 0ull) return -1;
        }
        int p = __ffsll((long long)C.freeplanes) - 1;
        C.freeplanes &= ~(1ull << p);
        return p;
    }

    // ---- test candidate (buffer slot cb) and cut the cell if it intersects.
    __device__ void test_and_cut(int cb) {
        const float4 Q = S.u.c.cd[cb];
        const float4 E = S.u.c.ce[cb];
        C.ptested++;
        bool out[K], unc[K];
        const int nvalid = Vm.popc();
        C.tests += nvalid;
        if (MODE == VGPU_FP64) {
            const double4 Q64 = S.u.c.cd64[cb];
#pragma unroll
            for (int s = 0; s < K; s++) {
                out[s] = unc[s] = false;
                if (Vm.test(lane + 32 * s)) {
                    double v = fma(Q64.x, V.dx[s], fma(Q64.y, V.dy[s], fma(Q64.z, V.dz[s], -Q64.w)));
                    double vv = sqrt(V.dx[s] * V.dx[s] + V.dy[s] * V.dy[s] + V.dz[s] * V.dz[s]);
                    double nq = fabs(Q64.x) + fabs(Q64.y) + fabs(Q64.z);
                    double bnd = nq * (double)V.e[s] + 8.0 * kU64 * (nq * vv + fabs(Q64.w)) + P.g.tol_h;
                    out[s] = v > bnd;
                    if (!out[s] && v >= -bnd) { unc[s] = true; }
                }
            }
            Mask<K> Um = ballot_mask<K>(unc);
            if (Um.any()) C.marginal = true;   // inside the tolerance band: kept, cell flagged
        } else {
            const float nabs = sqrtf(E.z);
            const float A = E.x + 3.0f * kU32 * nabs;
            const float Cq = E.y + 3.0f * kU32 * fabsf(Q.w) + (float)P.g.tol_h;
#pragma unroll
            for (int s = 0; s < K; s++) {
                out[s] = unc[s] = false;
                if (Vm.test(lane + 32 * s)) {
                    float v = fmaf(Q.x, V.x[s], fmaf(Q.y, V.y[s], fmaf(Q.z, V.z[s], -Q.w)));
                    float bnd = 1.5f * fmaf(A, V.a[s], fmaf(nabs, V.e[s], Cq));
                    out[s] = v > bnd;
                    unc[s] = !out[s] && v >= -bnd;
                }
            }
            Mask<K> Um = ballot_mask<K>(unc);
            if (Um.any()) {
                // FP64 repair of the uncertain tests
                C.repaired = true;
                C.repairs += Um.popc();
                bool anym = false;
#pragma unroll
                for (int s = 0; s < K; s++) {
                    if (unc[s]) {
                        unsigned t = V.tri[s];
                        double4 Q64 = plane64_from(P, C, S.cj[cb], S.cs[cb]);
                        double4 A64 = plane64_of<K>(P, C, S, tri_plane(t, 0));
                        double4 B64 = plane64_of<K>(P, C, S, tri_plane(t, 1));
                        double4 C64 = plane64_of<K>(P, C, S, tri_plane(t, 2));
                        double x, y, z, D, kn;
                        solve_f64(A64, B64, C64, x, y, z, D, kn);
                        int side = side64(Q64, x, y, z, D, kn, P.g.tol_h);
                        if (!(D > 0.0)) side = 1;
                        out[s] = side == 2;
                        if (side == 1) anym = true;
                    }
                }
                if (__any_sync(kFull, anym)) C.marginal = true;
            }
        }
        Mask<K> Rm = ballot_mask<K>(out);
        if (!Rm.any()) return;
        if (Rm.equals(Vm)) {
            C.deleted = true;
            return;
        }
        C.pcut++;
        int p = alloc_plane();
        if (p < 0) {
            C.overflow = true;
            return;
        }
        const int j = S.cj[cb];
        if (lane == 0) {
            S.pl[p] = Q;
            S.pe[p] = make_float4(sqrtf(E.z), E.x, E.y, fabsf(Q.w));
            S.pid[p] = P.a.pid[j];
            S.psrc[p] = j;
            S.pshift[p] = S.cs[cb];
            if (MODE == VGPU_FP64) S.pl64[p] = S.u.c.cd64[cb];
        }
        cut(p, Rm);
    }

    // ---- remove the vertices in Rm and close the hole with the face of plane p
    __device__ void cut(int p, const Mask<K> &Rm) {
        // Phase A: boundary edges of the removed region
        unsigned be[3 * K];
        int nbe = 0;
        bool broken = false;
#pragma unroll
        for (int s = 0; s < K; s++) {
            int t = lane + 32 * s;
            if (Rm.test(t)) {
                unsigned T = V.tri[s];
                unsigned A3 = S.adj[t];
#pragma unroll
                for (int e = 0; e < 3; e++) {
                    int u = (A3 >> (8 * e)) & 255u;
                    if (u >= 32 * K) { broken = true; continue; }
                    if (!Rm.test(u)) {
                        int a = tri_plane(T, e), b = tri_plane(T, e == 2 ? 0 : e + 1);
                        be[nbe++] = (unsigned)a | ((unsigned)b << 8) | ((unsigned)u << 16);
                    }
                }
            }
        }
        // exclusive prefix of per-lane counts
        int incl = nbe;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += y;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        const int base = incl - nbe;
        if (__any_sync(kFull, broken)) {  // inconsistent adjacency: hand the cell to the large engine
            C.overflow = true;
            return;
        }
        Mask<K> Fm;
#pragma unroll
        for (int i = 0; i < Mask<K>::W; i++) Fm.w[i] = ~Vm.w[i] | Rm.w[i];
        if (total < 3) {  // not a closed boundary: inconsistent side decisions
            C.marginal = true;
            return;
        }
        if (Fm.popc() < total) {
            C.overflow = true;
            return;
        }
        __syncwarp();
        // Phase B: new triangles (a, b, p) in the first free slots
        int fslot[3 * K];
        for (int q = 0; q < nbe; q++) {
            unsigned E = be[q];
            int a = E & 255u, b = (E >> 8) & 255u, u = (E >> 16) & 255u;
            int f = Fm.nth(base + q);
            fslot[q] = f;
            S.tri[f] = (unsigned)a | ((unsigned)b << 8) | ((unsigned)p << 16);
            S.adj[f] = (unsigned)u;
            S.startN[a] = (unsigned char)f;
            S.endN[b] = (unsigned char)f;
            unsigned Tu = S.tri[u];
#pragma unroll
            for (int e = 0; e < 3; e++) {
                if (tri_plane(Tu, e) == b && tri_plane(Tu, e == 2 ? 0 : e + 1) == a)
                    reinterpret_cast<unsigned char *>(&S.adj[u])[e] = (unsigned char)f;
            }
        }
        __syncwarp();
        // Phase C: link the new triangles around the new face
        bool bad = false;
        for (int q = 0; q < nbe; q++) {
            unsigned E = be[q];
            int a = E & 255u, b = (E >> 8) & 255u;
            int f = fslot[q];
            if (S.startN[a] != f) bad = true;
            unsigned char *ab = reinterpret_cast<unsigned char *>(&S.adj[f]);
            ab[1] = S.startN[b];
            ab[2] = S.endN[a];
        }
        if (__any_sync(kFull, bad)) C.marginal = true;
        // new valid mask: removed slots cleared, first `total` free slots set
        Mask<K> Nm;
        Nm.clear();
        if (total > 0) {
            int last = Fm.nth(total - 1);
#pragma unroll
            for (int i = 0; i < Mask<K>::W; i++) {
                unsigned long long lim;
                if (last >= i * 64 + 63) lim = ~0ull;
                else if (last < i * 64) lim = 0ull;
                else lim = (2ull << (last - i * 64)) - 1ull;
                Nm.w[i] = Fm.w[i] & lim;
            }
        }
#pragma unroll
        for (int i = 0; i < Mask<K>::W; i++) Vm.w[i] = (Vm.w[i] & ~Rm.w[i]) | Nm.w[i];
        __syncwarp();
        // Phase D: positions of the new vertices
#pragma unroll
        for (int s = 0; s < K; s++) {
            int t = lane + 32 * s;
            if (Nm.test(t)) {
                V.tri[s] = S.tri[t];
                compute_vertex(s);
            }
        }
        update_radius();
    }

    // ---- candidate buffer: sort by (power) distance and test in order
    __device__ void flush() {
        const int n = C.ncand;
        if (n == 0) return;
        __syncwarp();
        unsigned k0 = lane < n ? S.ck[lane] : 0xffffffffu;
        unsigned k1 = lane + 32 < n ? S.ck[lane + 32] : 0xffffffffu;
        if (n > 32) bitonic64(k0, k1, lane);
        else bitonic32(k0, lane);
        for (int i = 0; i < n; i++) {
            unsigned key = __shfl_sync(kFull, i < 32 ? k0 : k1, i & 31);
            int cb = key & 63u;
            float4 E = S.u.c.ce[cb];
            if (P.g.poly) {
                float rs = E.w;
                if (!(rs <= 0.0f || rs * rs < 4.0f * C.R2 * E.z * (1.0f + 16.0f * kU32))) continue;
            } else {
                if (E.z >= C.cutoff2 * (1.0f + 1e-4f)) break;
            }
            test_and_cut(cb);
            if (C.deleted || C.overflow) break;
        }
        C.ncand = 0;
        __syncwarp();
    }

    // ---- evaluate one block offset for this lane: wrap/skip, block distance
    __device__ void gather_offsets(int e_begin, int e_end, bool from_table, int shell_r) {
        const float l[3] = {C.me32.x, C.me32.y, C.me32.z};
        for (int base = e_begin; base < e_end; base += 32) {
            int e = base + lane;
            int di = 0, dj = 0, dk = 0;
            bool ok = e < e_end;
            if (ok) {
                if (from_table) {
                    int code = offsets[e];
                    di = (code & 31) - 16;
                    dj = ((code >> 5) & 31) - 16;
                    dk = ((code >> 10) & 31) - 16;
                } else {
                    int w = 2 * shell_r + 1;
                    di = e % w - shell_r;
                    dj = (e / w) % w - shell_r;
                    dk = e / (w * w) - shell_r;
                    int m = max(abs(di), max(abs(dj), abs(dk)));
                    int l2 = max(abs(di) - 1, 0) * max(abs(di) - 1, 0) + max(abs(dj) - 1, 0) * max(abs(dj) - 1, 0) +
                             max(abs(dk) - 1, 0) * max(abs(dk) - 1, 0);
                    ok = (m == shell_r) && (l2 > kTableLb2Max);
                }
            }
            int d[3] = {di, dj, dk};
            int cb[3] = {C.bi + di, C.bj + dj, C.bk + dk};
            int wrapped[3], img[3];
            float md2 = 0.0f;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                int n = P.g.gn[a];
                int c = cb[a];
                if (P.g.per[a]) {
                    int w = c % n;
                    if (w < 0) w += n;
                    img[a] = (c - w) / n;
                    wrapped[a] = w;
                } else {
                    img[a] = 0;
                    wrapped[a] = c;
                    if (c < 0 || c >= n) ok = false;
                }
                float bs = P.g.gbs32[a];
                float t = d[a] > 0 ? (float)d[a] * bs - l[a] : (d[a] < 0 ? l[a] - (float)(d[a] + 1) * bs : 0.0f);
                t = fmaxf(t, 0.0f);
                md2 = fmaf(t, t, md2);
            }
            if (ok && md2 * (1.0f - 1e-5f) >= C.cutoff2) ok = false;
            int cnt = 0, st = 0, code = 0;
            if (ok) {
                int b = wrapped[0] + P.g.gn[0] * (wrapped[1] + P.g.gn[1] * wrapped[2]);
                st = P.a.bstart[b];
                cnt = P.a.bstart[b + 1] - st;
                code = (img[0] + 128) | ((img[1] + 128) << 8) | ((img[2] + 128) << 16);
            }
            int incl = cnt;
#pragma unroll
            for (int q = 1; q < 32; q <<= 1) {
                int y = __shfl_up_sync(kFull, incl, q);
                if (lane >= q) incl += y;
            }
            const int tot = __shfl_sync(kFull, incl, 31);
            const int packed_d = (di + 16) | ((dj + 16) << 5) | ((dk + 16) << 10);
            for (int c0 = 0; c0 < tot; c0 += 32) {
                if (C.ncand > kCandBuf - 32) flush();
                if (C.deleted || C.overflow) return;
                int c = c0 + lane;
                bool has = c < tot;
                // owner lane: number of lanes whose inclusive prefix is <= c
                int pos = 0;
#pragma unroll
                for (int w = 16; w >= 1; w >>= 1) {
                    int v = __shfl_sync(kFull, incl, pos + w - 1);
                    if (v <= c) pos += w;
                }
                pos = min(pos, 31);
                int o_incl = __shfl_sync(kFull, incl, pos);
                int o_cnt = __shfl_sync(kFull, cnt, pos);
                int o_st = __shfl_sync(kFull, st, pos);
                int o_code = __shfl_sync(kFull, code, pos);
                int o_d = __shfl_sync(kFull, packed_d, pos);
                bool pass = false;
                unsigned key = 0;
                float4 cd = make_float4(0, 0, 0, 0), ce = make_float4(0, 0, 0, 0);
                int j = 0;
                if (has) {
                    j = o_st + (c - (o_incl - o_cnt));
                    int ddi = (o_d & 31) - 16, ddj = ((o_d >> 5) & 31) - 16, ddk = ((o_d >> 10) & 31) - 16;
                    bool self = (j == C.k) && ddi == 0 && ddj == 0 && ddk == 0;
                    if (!self) {
                        float4 lj = P.a.l32[j];
                        float dx = fmaf((float)ddi, P.g.gbs32[0], lj.x - C.me32.x);
                        float dy = fmaf((float)ddj, P.g.gbs32[1], lj.y - C.me32.y);
                        float dz = fmaf((float)ddk, P.g.gbs32[2], lj.z - C.me32.z);
                        float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        float rs = d2;
                        float rr = 0.0f;
                        if (P.g.poly) {
                            rr = C.ri2 + lj.w * lj.w;
                            rs = d2 + (C.ri2 - lj.w * lj.w);
                            pass = rs <= 0.0f || rs * rs < 4.0f * C.R2 * d2 * (1.0f + 16.0f * kU32);
                        } else {
                            pass = d2 < C.cutoff2 * (1.0f + 1e-5f);
                        }
                        int M = max(abs(ddi), max(abs(ddj), abs(ddk)));
                        float bsmax = fmaxf(P.g.gbs32[0], fmaxf(P.g.gbs32[1], P.g.gbs32[2]));
                        float dn = sqrtf(d2);
                        float en = kU32 * (1.75f * (float)(M + 3) * bsmax + 1.01f * dn) + 1e-12f * bsmax;
                        float eh = dn * en + 2.0f * kU32 * (d2 + rr) + 0.5f * en * en;
                        cd = make_float4(dx, dy, dz, 0.5f * rs);
                        ce = make_float4(en, eh, d2, rs);
                        key = float_key(P.g.poly ? rs : d2);
                    }
                }
                unsigned bal = __ballot_sync(kFull, pass);
                if (pass) {
                    int slot = C.ncand + __popc(bal & ((1u << lane) - 1u));
                    S.ck[slot] = (key & ~63u) | (unsigned)slot;
                    S.cj[slot] = j;
                    S.cs[slot] = o_code;
                    S.u.c.cd[slot] = cd;
                    S.u.c.ce[slot] = ce;
                    if (MODE == VGPU_FP64) S.u.c.cd64[slot] = plane64_from(P, C, j, o_code);
                }
                C.ncand += __popc(bal);
            }
        }
    }

    // ---- the search: blocks in order of lower-bound distance (src/v_compute.cc:289-621
    //      does the same with its 64 worklists, mrad cut-offs and the block queue)
    __device__ void search() {
        const float bmin2 = P.g.gbs_min * P.g.gbs_min;
        bool done = false;
        for (int g = 0; g < P.ngroups && !done; g++) {
            if ((float)P.group_lb2[g] * bmin2 >= C.cutoff2 * (1.0f + 1e-5f)) { done = true; break; }
            gather_offsets(P.group_start[g], P.group_start[g + 1], true, 0);
            if (C.deleted || C.overflow) return;
            flush();
            if (C.deleted || C.overflow) return;
        }
        if (done) return;
        // beyond the table: Chebyshev shells, skipping what the table covered
        int rmax_grid = max(P.g.gn[0], max(P.g.gn[1], P.g.gn[2]));
        for (int r = 2; r < 4 * rmax_grid + 8; r++) {
            float lb = (float)(r - 1) * P.g.gbs_min;
            if (lb * lb >= C.cutoff2 * (1.0f + 1e-5f)) return;
            bool any_periodic = P.g.per[0] || P.g.per[1] || P.g.per[2];
            if (!any_periodic && r > rmax_grid + 1) return;
            int w = 2 * r + 1;
            gather_offsets(0, w * w * w, false, r);
            if (C.deleted || C.overflow) return;
            flush();
            if (C.deleted || C.overflow) return;
        }
        C.overflow = true;  // search did not terminate
    }

    // ---- reductions: vertex/face counts, neighbours, FP64 volume and centroid
    __device__ void finish() {
        const int out = P.a.outpos[C.k];
        if (C.overflow) return;
        if (C.deleted) {
            if (lane == 0) {
                P.r.vol[out] = 0.0;
                P.r.cen[3 * out] = P.r.cen[3 * out + 1] = P.r.cen[3 * out + 2] = 0.0;
                P.r.nf[out] = 0;
                P.r.nv[out] = 0;
                P.r.maxr2[out] = 0.0;
                P.r.flags[out] = (C.marginal ? VGPU_CELL_MARGINAL : 0) | (C.repaired ? VGPU_CELL_REPAIRED : 0);
            }
            return;
        }
        unsigned long long live = 0ull;
#pragma unroll
        for (int s = 0; s < K; s++)
            if (Vm.test(lane + 32 * s)) {
                unsigned t = V.tri[s];
                live |= (1ull << tri_plane(t, 0)) | (1ull << tri_plane(t, 1)) | (1ull << tri_plane(t, 2));
            }
        live = warp_or64(live);
        const int nf = __popcll(live);
        const int nv = Vm.popc();
        // neighbours, ascending plane order; FP64 planes of the live faces
        for (int q = lane; q < nf; q += 32) {
            unsigned long long x = live;
            for (int i = 0; i < q; i++) x &= x - 1ull;
            int p = __ffsll((long long)x) - 1;
            P.r.nb[(size_t)out * kMaxNb + q] = S.pid[p];
            S.pl64[p] = plane64_of<K>(P, C, S, p);
        }
        __syncwarp();
        // FP64 vertices, rebuilt from their three planes
        double mr2 = 0.0;
#pragma unroll
        for (int s = 0; s < K; s++) {
            int t = lane + 32 * s;
            if (Vm.test(t)) {
                double x, y, z;
                if (MODE == VGPU_FP64) {
                    x = V.dx[s]; y = V.dy[s]; z = V.dz[s];
                } else {
                    unsigned T = V.tri[s];
                    double D, kn;
                    solve_f64(S.pl64[tri_plane(T, 0)], S.pl64[tri_plane(T, 1)], S.pl64[tri_plane(T, 2)], x, y, z, D, kn);
                }
                S.u.f.vtx[t] = make_double4(x, y, z, 0.0);
                mr2 = fmax(mr2, x * x + y * y + z * z);
            }
        }
        __syncwarp();
        // Origin for the volume sums: one vertex of the cell, so that every term
        // scales with the cell size rather than its distance from the particle.
        const double4 c0 = S.u.f.vtx[Vm.nth(0)];
        for (int q = lane; q < nf; q += 32) {
            unsigned long long x = live;
            for (int i = 0; i < q; i++) x &= x - 1ull;
            int p = __ffsll((long long)x) - 1;
            double4 pl = S.pl64[p];
            double nn = pl.x * pl.x + pl.y * pl.y + pl.z * pl.z;
            double f = (pl.w - (pl.x * c0.x + pl.y * c0.y + pl.z * c0.z)) / nn;
            S.foot[p] = make_double4(pl.x * f, pl.y * f, pl.z * f, 0.0);  // closest point of face p to c0, relative to c0
        }
        __syncwarp();
        // volume and centroid over edges (t,u) owned by the lower slot:
        // sum over edges of (p_y - p_x).(v_t x v_u), p_f a point of face f
        double vs = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
#pragma unroll
        for (int s = 0; s < K; s++) {
            int t = lane + 32 * s;
            if (Vm.test(t)) {
                unsigned T = V.tri[s];
                unsigned A3 = S.adj[t];
                double4 vt = S.u.f.vtx[t];
                vt.x -= c0.x; vt.y -= c0.y; vt.z -= c0.z;
#pragma unroll
                for (int e = 0; e < 3; e++) {
                    int u = (A3 >> (8 * e)) & 255u;
                    if (u > t && u < 32 * K) {
                        double4 vu = S.u.f.vtx[u];
                        vu.x -= c0.x; vu.y -= c0.y; vu.z -= c0.z;
                        double4 px = S.foot[tri_plane(T, e)];
                        double4 py = S.foot[tri_plane(T, e == 2 ? 0 : e + 1)];
                        double wx = vt.y * vu.z - vt.z * vu.y;
                        double wy = vt.z * vu.x - vt.x * vu.z;
                        double wz = vt.x * vu.y - vt.y * vu.x;
                        double ty = py.x * wx + py.y * wy + py.z * wz;
                        double tx = px.x * wx + px.y * wy + px.z * wz;
                        double dd = ty - tx;
                        vs += dd;
                        cx += dd * (vt.x + vu.x) + ty * py.x - tx * px.x;
                        cy += dd * (vt.y + vu.y) + ty * py.y - tx * px.y;
                        cz += dd * (vt.z + vu.z) + ty * py.z - tx * px.z;
                    }
                }
            }
        }
        vs = warp_sumd(vs);
        cx = warp_sumd(cx);
        cy = warp_sumd(cy);
        cz = warp_sumd(cz);
        mr2 = warp_maxd(mr2);
        if (lane == 0) {
            double vol = vs / 6.0;
            P.r.vol[out] = vol;
            // centroid threshold as src/cell.cc:1895 (raw doubled-coordinate sum = 48*volume)
            if (48.0 * vol > P.g.tol_cu) {
                double f = 1.0 / (4.0 * vs);
                P.r.cen[3 * out] = c0.x + cx * f;
                P.r.cen[3 * out + 1] = c0.y + cy * f;
                P.r.cen[3 * out + 2] = c0.z + cz * f;
            } else {
                P.r.cen[3 * out] = P.r.cen[3 * out + 1] = P.r.cen[3 * out + 2] = 0.0;
            }
            P.r.nf[out] = nf;
            P.r.nv[out] = nv;
            P.r.maxr2[out] = mr2;
            P.r.flags[out] = VGPU_CELL_OK | (C.marginal ? VGPU_CELL_MARGINAL : 0) | (C.repaired ? VGPU_CELL_REPAIRED : 0);
        }
    }

    __device__ void run(int k) {
        init_cell(k);
        search();
        finish();
    }
};

template <int MODE, int K>
__global__ void __launch_bounds__(128) cell_kernel(CellParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warps = blockDim.x >> 5;
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *offsets = reinterpret_cast<int *>(smem_raw);
    size_t off_bytes = ((size_t)P.noffsets * sizeof(int) + 15) & ~(size_t)15;
    WarpShared<K> *ws = reinterpret_cast<WarpShared<K> *>(smem_raw + off_bytes);
    for (int i = threadIdx.x; i < P.noffsets; i += blockDim.x) offsets[i] = P.offsets[i];
    __syncthreads();
    (void)warps;
    WarpShared<K> &S = ws[wid];
    unsigned long long tests = 0, repairs = 0, ptested = 0, pcut = 0, deleted = 0, marginal = 0, overflow = 0;
    unsigned long long *work = P.cell_list ? &P.cnt->overflow_work : &P.cnt->work;
    for (;;) {
        int w = 0;
        if (lane == 0) w = (int)atomicAdd(work, 1ull);
        w = __shfl_sync(kFull, w, 0);
        if (w >= P.ncells) break;
        int k = P.cell_list ? P.cell_list[w] : w;
        Engine<MODE, K> eng(P, S, offsets, lane);
        eng.run(k);
        tests += eng.C.tests;
        repairs += eng.C.repairs;
        ptested += eng.C.ptested;
        pcut += eng.C.pcut;
        if (eng.C.overflow) {
            overflow++;
            if (lane == 0) {
                unsigned long long slot = atomicAdd(&P.cnt->overflow, 1ull);
                if (P.overflow_list) P.overflow_list[slot] = k;
            }
        } else {
            deleted += eng.C.deleted ? 1 : 0;
            marginal += eng.C.marginal ? 1 : 0;
        }
        __syncwarp();
    }
    if (lane == 0) {
        atomicAdd(&P.cnt->side_tests, tests);
        atomicAdd(&P.cnt->fp64_repairs, repairs);
        atomicAdd(&P.cnt->planes_tested, ptested);
        atomicAdd(&P.cnt->planes_cut, pcut);
        atomicAdd(&P.cnt->deleted, deleted);
        atomicAdd(&P.cnt->marginal, marginal);
    }
}

__global__ void nf_to_ll_kernel(const int *nf, long long *out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = nf[i];
}

__global__ void compact_nb_kernel(const int *nf, const int *nb, const long long *off, int n, int *out) {
    int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int lane = threadIdx.x & 31;
    if (i >= n) return;
    int m = nf[i];
    long long o = off[i];
    // ascending order of neighbour IDs
    for (int q = lane; q < m; q += 32) {
        int v = nb[(size_t)i * kMaxNb + q];
        int rank = 0;
        for (int r = 0; r < m; r++) {
            int w = nb[(size_t)i * kMaxNb + r];
            rank += (w < v) || (w == v && r < q);
        }
        out[o + rank] = v;
    }
}

__global__ void sum_volumes_kernel(const double *vol, const int *flags, int n, double *out) {
    __shared__ double part[32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flags[i] & VGPU_CELL_OK) s += vol[i];
    s = warp_sumd(s);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
        t = warp_sumd(t);
        if (threadIdx.x == 0) out[blockIdx.x] = t;
    }
}

template <int MODE, int K>
cudaError_t launch_one(const CellParams &cp, int sms, cudaStream_t s) {
    const int warps = 4;
    size_t off_bytes = ((size_t)cp.noffsets * sizeof(int) + 15) & ~(size_t)15;
    size_t smem = off_bytes + warps * sizeof(WarpShared<K>);
    cudaError_t e = cudaFuncSetAttribute(cell_kernel<MODE, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cell_kernel<MODE, K>, warps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    long long want = (long long)sms * per_sm;
    long long need = (cp.ncells + warps - 1) / warps;
    int grid = (int)(want < need ? want : need);
    if (grid < 1) grid = 1;
    cell_kernel<MODE, K><<<grid, warps * 32, smem, s>>>(cp);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

// Box tables: corner (sx,sy,sz) uses faces x:(sx>0), y:2+(sy>0), z:4+(sz>0),
// ordered so that det(n_a,n_b,n_c) > 0; neighbours across each edge found by
// matching plane pairs.
static void build_box_tables(unsigned tri[8], unsigned adj[8]) {
    int fa[8][3];
    for (int c = 0; c < 8; c++) {
        int sx = (c & 1) ? 1 : -1, sy = (c & 2) ? 1 : -1, sz = (c & 4) ? 1 : -1;
        int fx = sx > 0 ? 1 : 0, fy = 2 + (sy > 0 ? 1 : 0), fz = 4 + (sz > 0 ? 1 : 0);
        if (sx * sy * sz > 0) { fa[c][0] = fx; fa[c][1] = fy; fa[c][2] = fz; }
        else { fa[c][0] = fx; fa[c][1] = fz; fa[c][2] = fy; }
        tri[c] = (unsigned)fa[c][0] | ((unsigned)fa[c][1] << 8) | ((unsigned)fa[c][2] << 16);
    }
    for (int c = 0; c < 8; c++) {
        unsigned a3 = 0;
        for (int e = 0; e < 3; e++) {
            int a = fa[c][e], b = fa[c][(e + 1) % 3];
            int found = -1;
            for (int u = 0; u < 8; u++) {
                if (u == c) continue;
                for (int q = 0; q < 3; q++)
                    if (fa[u][q] == b && fa[u][(q + 1) % 3] == a) found = u;
            }
            a3 |= (unsigned)(found < 0 ? 0 : found) << (8 * e);
        }
        adj[c] = a3;
    }
}

cudaError_t upload_box_tables() {
    unsigned tri[8], adj[8];
    build_box_tables(tri, adj);
    cudaError_t e = cudaMemcpyToSymbol(c_box_tri, tri, sizeof(tri));
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_box_adj, adj, sizeof(adj));
}

cudaError_t launch_cells(const CellParams &cp, int mode, int big, int sms, cudaStream_t s) {
    if (cp.ncells <= 0) return cudaSuccess;
    if (mode == VGPU_FP64) {
        return big ? launch_one<VGPU_FP64, 4>(cp, sms, s) : launch_one<VGPU_FP64, 2>(cp, sms, s);
    }
    return big ? launch_one<VGPU_MIXED, 4>(cp, sms, s) : launch_one<VGPU_MIXED, 2>(cp, sms, s);
}

cudaError_t launch_nf_to_ll(const int *nf, long long *out, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    nf_to_ll_kernel<<<(n + 255) / 256, 256, 0, s>>>(nf, out, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_compact_neighbors(const int *nf, const int *nb, const long long *off, int n, int *out,
                                     cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    compact_nb_kernel<<<(n + 7) / 8, 256, 0, s>>>(nf, nb, off, n, out);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_sum_volumes(const double *vol, const int *flags, int n, double *out, cudaStream_t s) {
    sum_volumes_kernel<<<64, 256, 0, s>>>(vol, flags, n, out);
    note_launch();
    return cudaGetLastError();
}

}  // namespace vgpu
