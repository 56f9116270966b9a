#pragma once
// The warp-per-cell clipping engine, included by the translation unit of
// each precision (vgpu_clip_mixed.cu, vgpu_clip_fp64.cu).
//
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
//    its three edges.  Lane l owns vertex slots l, l+32, ... in registers;
//    an empty slot holds a NaN position, so it never tests outside a plane.
//  * A candidate plane is tested against all vertices at once (one side test
//    per lane and slot, then a ballot).  The common case — the plane misses —
//    costs a handful of instructions.  A cut removes the vertices outside,
//    stages the boundary of the removed region (a cycle of edges) in shared
//    memory, and every free slot of rank r builds the new vertex for boundary
//    edge r, so slot assignment needs only a population count.
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
//  * A finished cell is written as a compact polytope record; the FP64
//    reductions run in the finish kernel (vgpu_finish.cu).
#include <cfloat>
#include <cstdio>
#include "vgpu_dev.cuh"

namespace vgpu {

namespace {

// How the clipping kernels store the polytope records: plain stores by
// default; -DVGPU_STREAMING_RECORD_STORES=1 builds streaming stores (st.cs,
// meant to keep the once-read records from pushing the particles and block
// starts out of the L2).  Measured on the 4M periodic box, clipping passes:
// plain 76.2 ms, streaming 80.1 ms (the streaming form also costs the lean
// pass registers: 100/160 spilled bytes against 56/80).
#if VGPU_STREAMING_RECORD_STORES
#define VGPU_RECORD_STORE(p, v) __stcs((p), (unsigned)(v))
#else
#define VGPU_RECORD_STORE(p, v) (*(p) = (unsigned)(v))
#endif

// ------------------------------------------------------------------ masks
// Slot l+32s (lane l, slot row s) is bit l of row word r[s]: one 32-bit word
// per row, as a ballot returns it, so that a lane's test of its own slot is
// one shift of a known word (a 64-bit word per two rows cost a wide shift).
template <int K>
struct Mask {
    unsigned r[K];
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int i = 0; i < K; i++) r[i] = 0u;
    }
    __device__ __forceinline__ unsigned row(int t) const {
        unsigned w = r[0];
#pragma unroll
        for (int i = 1; i < K; i++)
            if ((t >> 5) == i) w = r[i];
        return w;
    }
    __device__ __forceinline__ bool test(int t) const { return (row(t) >> (t & 31)) & 1u; }
    __device__ __forceinline__ int popc() const {
        int c = 0;
#pragma unroll
        for (int i = 0; i < K; i++) c += __popc(r[i]);
        return c;
    }
    __device__ __forceinline__ bool any() const {
        unsigned o = 0u;
#pragma unroll
        for (int i = 0; i < K; i++) o |= r[i];
        return o != 0u;
    }
    __device__ __forceinline__ bool equals(const Mask &o) const {
        bool e = true;
#pragma unroll
        for (int i = 0; i < K; i++) e = e && (r[i] == o.r[i]);
        return e;
    }
    // number of set bits below bit t
    __device__ __forceinline__ int rank(int t) const {
        int c = 0;
        const int wi = t >> 5;
#pragma unroll
        for (int i = 0; i < K; i++) {
            if (i < wi) c += __popc(r[i]);
            else if (i == wi) c += __popc(r[i] & ((1u << (t & 31)) - 1u));
        }
        return c;
    }
    // lowest set bit, or -1
    __device__ __forceinline__ int first() const {
#pragma unroll
        for (int i = 0; i < K; i++)
            if (r[i]) return i * 32 + __ffs((int)r[i]) - 1;
        return -1;
    }
};

template <int K>
__device__ __forceinline__ Mask<K> ballot_mask(const bool (&pred)[K]) {
    Mask<K> m;
#pragma unroll
    for (int s = 0; s < K; s++) m.r[s] = __ballot_sync(kFull, pred[s]);
    return m;
}

// ------------------------------------------------------------------ shared memory per warp
// plane slots of an engine with K vertex slot rows: 64, or 128 for the
// 128-vertex engines (a cell that outgrows 64 vertices can also hold more
// than 64 live planes at once: a radical cell of a large particle among
// small ones)
template <int K>
struct PlaneSlots {
    static constexpr int N = K >= 4 ? kMaxPlanesWide : kMaxPlanes;
    static constexpr int W = N / 32;   // 32-bit words of a set of planes
};

// set bit p of a set of planes held as 32-bit words
template <int NW>
__device__ __forceinline__ void plane_set_add(unsigned (&m)[NW], int p) {
#pragma unroll
    for (int i = 0; i < NW; i++)
        if ((p >> 5) == i) m[i] |= 1u << (p & 31);
}

template <int MODE, int K>
struct WarpShared {
#if VGPU_GATHER_TMA
    float4 cstage[kStageEntries];   // staged particle runs (bulk copies)
    unsigned long long cbar;        // their mbarrier
    unsigned cbar_phase;            // its current phase parity; bit 31: staging off
    unsigned cbar_pad;
#endif
    float4 pl[PlaneSlots<K>::N];   // plane n.x, n.y, n.z, h  (n.v <= h inside)
    float4 pe[PlaneSlots<K>::N];   // |n|, en (abs error of n), eh (abs error of h), |h|
    // (pl and pe are contiguous: at the end of a cell they hold the FP64 planes)
    double4 pl64x[MODE == VGPU_FP64 ? PlaneSlots<K>::N : 1];   // FP64 planes (FP64 engine, during the search)
    int pid[PlaneSlots<K>::N];     // neighbour ID of the plane
    int psrc[PlaneSlots<K>::N];    // engine index of the generating particle, -1 for initial faces
    int pshift[PlaneSlots<K>::N];  // packed periodic image counts (initial faces: face index)
    unsigned tri[32 * K];
    unsigned adj[32 * K];
    unsigned stage[48 * K];  // boundary edges of a cut (a | b<<8 | u<<16); final stage: edge list
    unsigned char vmap[32 * K];   // finished cell: vertex slot -> compact index
    unsigned char startN[PlaneSlots<K>::N];
    unsigned char endN[PlaneSlots<K>::N];
    // the warp's counters over its cells (side tests, repairs, planes tested,
    // planes cut, deleted, marginal): kept here rather than in registers,
    // which the clipping loop needs more
    unsigned long long stat[6];
    union {
        struct {
            unsigned ck[kCandBuf];    // sort keys
            int cj[kCandBuf];         // engine index
            int cs[kCandBuf];         // packed periodic image counts
            int cpid[kCandBuf];       // neighbour ID
            float4 cd[kCandBuf];      // plane (FP32): n, h
            float4 ce[kCandBuf];      // en, eh, |n|, rs
            double4 cd64[MODE == VGPU_FP64 ? kCandBuf : 1];  // plane (FP64), FP64 engine
        } c;
        struct {
            double vx[32 * K], vy[32 * K], vz[32 * K];   // FP64 vertices relative to c0
            double fx[PlaneSlots<K>::N], fy[PlaneSlots<K>::N], fz[PlaneSlots<K>::N];  // face points relative to c0
        } f;
    } u;
};

// ------------------------------------------------------------------ per-lane vertex registers
template <int MODE, int K>
struct Verts {
    unsigned tri[K];
    float x[K], y[K], z[K];   // FP32 position (NaN = empty slot)
    float a[K], e[K];         // |v| and the forward error bound of the position
    float r2[K];              // bound on |v|^2 (0 for empty)
    double dx[K], dy[K], dz[K];   // FP64 engine positions (NaN = empty)
};

struct CellCtx {
    double4 me64;     // particle (remapped position, radius)
    float4 me32;      // local coords, radius
    int bi, bj, bk;   // engine block coordinates
    int k;            // engine index
    float R2;         // upper bound of max |v|^2
    float cutoff2;    // squared distance bound for candidates / blocks
    float ri2;        // particle radius squared (poly)
    bool deleted, overflow, marginal, repaired;
    bool needs_fp64;  // this lane's vertex solve was ill-conditioned (first pass: the cell is rerun)
    int fail_reason;  // why overflow was set (VGPU_FAIL_*)
    unsigned freeplanes[2];   // plane slots not in use: slots 0-31, 32-63 (128-vertex engines: also fp_hi)
    int ncand;
    unsigned tests, repairs, ptested, pcut;
#ifdef VGPU_PHASE_TIMING
    unsigned long long phase[16];   // 8 clock totals, 8 event counts
#endif
};

// ------------------------------------------------------------------ out-of-line helpers
// The vertex solve, its FP64 refinement and the key sorts.  They are inlined by
// default (measured faster on the 4M periodic box: 16.9M vs 15.3M cells/s);
// -DVGPU_OUTLINE=1 keeps one out-of-line copy of each instead, which shrinks
// the kernel's code at the price of spills around the calls.
#ifndef VGPU_OUTLINE
#define VGPU_OUTLINE 0
#endif
#if VGPU_OUTLINE
#define VGPU_HELPER __device__ __noinline__
#else
#define VGPU_HELPER __device__ __forceinline__
#endif
struct VertexF32 {
    float x, y, z, a, e, r2;
    bool good;
};

// Vertex of planes (a,b,c) of triangle t in FP32, with a forward error bound e
// covering the planes' own storage error (pe: |n|, en, eh, |h|) and the
// rounding of this Cramer solve: |adj(A)| <= |n_b||n_c| + |n_c||n_a| + |n_a||n_b|
// and every row's error is at most rho.
// The reciprocal of D and |v| use the approximate hardware operations, whose
// documented errors (__fdividef: 2 ulp for 2^-126 <= |D| <= 2^126; rsqrtf:
// 2 ulp) are covered by widening the bound: 4u|v| more for the reciprocal's
// relative error in every coordinate, (1 + 8u) on 1/|D| in the first term,
// and |v| rounded up by 8u so that it stays an upper bound of the root.
VGPU_HELPER VertexF32 solve_vertex_f32(const float4 *pl, const float4 *pe, unsigned t) {
    const int a = tri_plane(t, 0), b = tri_plane(t, 1), c = tri_plane(t, 2);
    const float4 A = pl[a], B = pl[b], Cc = pl[c];
    const float4 EA = pe[a], EB = pe[b], EC = pe[c];
    const float bcx = B.y * Cc.z - B.z * Cc.y, bcy = B.z * Cc.x - B.x * Cc.z, bcz = B.x * Cc.y - B.y * Cc.x;
    const float cax = Cc.y * A.z - Cc.z * A.y, cay = Cc.z * A.x - Cc.x * A.z, caz = Cc.x * A.y - Cc.y * A.x;
    const float abx = A.y * B.z - A.z * B.y, aby = A.z * B.x - A.x * B.z, abz = A.x * B.y - A.y * B.x;
    const float D = A.x * bcx + A.y * bcy + A.z * bcz;
    const float inv = __fdividef(1.0f, D);
    VertexF32 o;
    o.x = (A.w * bcx + B.w * cax + Cc.w * abx) * inv;
    o.y = (A.w * bcy + B.w * cay + Cc.w * aby) * inv;
    o.z = (A.w * bcz + B.w * caz + Cc.w * abz) * inv;
    const float s2 = o.x * o.x + o.y * o.y + o.z * o.z;
    o.a = s2 * rsqrtf(s2) * (1.0f + 8.0f * kU32);   // NaN for s2 = 0 or inf: not good
    const float cof = fmaf(EB.x, EC.x, fmaf(EC.x, EA.x, EA.x * EB.x));
    const float r8 = 8.0f * kU32;
    const float ra = fmaf(EA.y, o.a, EA.z) + r8 * fmaf(EA.x, o.a, EA.w);
    const float rb = fmaf(EB.y, o.a, EB.z) + r8 * fmaf(EB.x, o.a, EB.w);
    const float rc = fmaf(EC.y, o.a, EC.z) + r8 * fmaf(EC.x, o.a, EC.w);
    o.e = 2.0f * cof * fmaxf(ra, fmaxf(rb, rc)) * (fabsf(inv) * (1.0f + 8.0f * kU32)) + (12.0f * kU32) * o.a;
    o.good = D >= FLT_MIN && D <= 8.5e37f && isfinite(o.e) && isfinite(o.a);
    if (!o.good) o.e = 3.0e38f;  // every test on it is repaired in FP64
    const float r = fminf((o.a + o.e) * (1.0f + 4.0f * kU32), 1.0e18f);
    o.r2 = r * r;
    return o;
}

// ------------------------------------------------------------------ warp sort of candidate keys
VGPU_HELPER unsigned bitonic32(unsigned x, int lane) {
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
    return x;
}
VGPU_HELPER uint2 bitonic64(unsigned x0, unsigned x1, int lane) {
#pragma unroll 1
    for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll 1
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j == 32) {
                unsigned a = min(x0, x1), b = max(x0, x1);
                x0 = a;
                x1 = b;
            } else {
                unsigned y0 = __shfl_xor_sync(kFull, x0, j);
                unsigned y1 = __shfl_xor_sync(kFull, x1, j);
                bool lower = (lane & j) == 0;
                bool up0 = (lane & k) == 0;
                bool up1 = ((lane + 32) & k) == 0;
                x0 = (lower == up0) ? min(x0, y0) : max(x0, y0);
                x1 = (lower == up1) ? min(x1, y1) : max(x1, y1);
            }
        }
    }
    return make_uint2(x0, x1);
}

// FP64 plane of an existing plane slot of a cell
template <int MODE, int K>
__device__ __forceinline__ double4 plane64_slot(const CellParams &P, const WarpShared<MODE, K> &S, double4 me, int p) {
    const int src = S.psrc[p];
    if (src >= 0) return plane64_from(P, me, src, S.pshift[p]);
    return initial64(P, me, S.pshift[p]);
}

// FP64 re-test of the vertices whose FP32 test against candidate cb was
// uncertain (bit s of uncbits: slot s of this lane, vertex planes tri_s).
// Returns the outside bits; *marginal is set for tolerance-band hits.
template <int MODE, int K>
__device__ __noinline__ unsigned repair_tests(const CellParams &P, const WarpShared<MODE, K> &S, double4 me, int cb,
                                              unsigned uncbits, unsigned tri0, unsigned tri1, unsigned tri2,
                                              unsigned tri3, unsigned *bandbits) {
    unsigned outbits = 0, band = 0;
    if (uncbits) {
        const int cj = S.u.c.cj[cb];   // (a wall: -1, with its face index in cs)
        const double4 Q = cj >= 0 ? plane64_from(P, me, cj, S.u.c.cs[cb]) : initial64(P, me, S.u.c.cs[cb]);
        for (int s = 0; s < K; s++) {
            if (!((uncbits >> s) & 1u)) continue;
            const unsigned t = s == 0 ? tri0 : (s == 1 ? tri1 : (s == 2 ? tri2 : tri3));
            const double4 A = plane64_slot<MODE, K>(P, S, me, tri_plane(t, 0));
            const double4 B = plane64_slot<MODE, K>(P, S, me, tri_plane(t, 1));
            const double4 Cq = plane64_slot<MODE, K>(P, S, me, tri_plane(t, 2));
            double x, y, z, D;
            float kn;
            solve_f64(A, B, Cq, x, y, z, D, kn);
            const double v = fma(Q.x, x, fma(Q.y, y, fma(Q.z, z, -Q.w)));
            const double vv = sqrt(x * x + y * y + z * z);
            const double nq = fabs(Q.x) + fabs(Q.y) + fabs(Q.z);
            const double verr = 16.0 * kU64 * (double)kn / fabs(D) + 64.0 * kU64 * vv;
            const double bnd = nq * verr + 8.0 * kU64 * (nq * vv + fabs(Q.w)) + P.g.tol_h;
            if (!(D > 0.0)) band |= 1u << s;
            else if (v > bnd) outbits |= 1u << s;
            else if (v >= -bnd) band |= 1u << s;
        }
    }
    *bandbits = band;
    return outbits;
}

// A vertex whose FP32 solve is ill-conditioned (error bound above
// kVertexTrust of its distance, or the determinant's sign lost) is solved in
// FP64 from the planes' double-precision source instead and rounded to FP32;
// its error bound is then the FP64 solve's plus that rounding.  Only nearly
// degenerate plane triples (as in jittered lattices) get here: FP64 runs at a
// small fraction of the FP32 rate, so the threshold is high and the code is
// kept out of line.  (At 1e-4 about 1 % of vertices came here and the 4M
// periodic box ran 1.8x slower.)
constexpr float kVertexTrust = 1e-2f;

template <int MODE, int K>
__device__ __noinline__ VertexF32 vertex_f64_fallback(const CellParams &P, const WarpShared<MODE, K> &S, double4 me,
                                                      unsigned t) {
    const double4 A = plane64_slot<MODE, K>(P, S, me, tri_plane(t, 0));
    const double4 B = plane64_slot<MODE, K>(P, S, me, tri_plane(t, 1));
    const double4 Cq = plane64_slot<MODE, K>(P, S, me, tri_plane(t, 2));
    double x, y, z, D;
    float kn;
    solve_f64(A, B, Cq, x, y, z, D, kn);
    VertexF32 o;
    const double vv = sqrt(x * x + y * y + z * z);
    o.x = (float)x;
    o.y = (float)y;
    o.z = (float)z;
    o.a = (float)vv;
    const double verr = 16.0 * kU64 * (double)kn / fabs(D) + 64.0 * kU64 * vv;
    o.e = (float)(verr * (1.0 + 1e-6)) + 4.0f * kU32 * o.a;
    o.good = D > 0.0 && isfinite(o.e) && isfinite(o.a);
    if (!o.good) o.e = 3.0e38f;   // every test on it is repaired in FP64
    const float r = fminf((o.a + o.e) * (1.0f + 4.0f * kU32), 1.0e18f);
    o.r2 = r * r;
    return o;
}

// Optional per-phase clock accounting (diagnostics builds: -DVGPU_PHASE_TIMING).
// Phases: 0 init, 1 block/candidate gather, 2 sort, 3 side tests, 4 cuts, 5 finish.
#ifdef VGPU_PHASE_TIMING
#define PHASE_BEGIN(v) const long long v = clock64()
#define PHASE_END(v, ph) C.phase[ph] += (unsigned long long)(clock64() - (v))
#define PHASE_COUNT(i, n) C.phase[8 + (i)] += (unsigned long long)(n)
#else
#define PHASE_BEGIN(v)
#define PHASE_END(v, ph)
#define PHASE_COUNT(i, n)
#endif

// ------------------------------------------------------------------ the engine
template <int MODE, int K, bool LEAN = false>
struct Engine {
    // LEAN (the mixed engine's first pass) carries no FP64 code: a cell that
    // needs an FP64 repair or vertex goes, like one that outgrows the slots,
    // to the rerun (the full 64-slot engine, then the 128-slot one).  Without
    // the two FP64 calls the kernel needs 80 registers instead of 168 (6 CTAs
    // per SM instead of 3).
    static constexpr bool kLean = LEAN && MODE == VGPU_MIXED;
    // The 64-slot engines walk each shell beyond the table as its whole cube
    // (no branches: the fastest at the small radii nearly every search ends
    // at) up to kNarrowShellRadius, and hand on a cell that searches further;
    // the 128-slot engines walk only the cubes' faces, up to kMaxShellRadius.
    // (The face walk in the 64-slot engines cost 1.2 ms of 66.4 on the 4M
    // periodic box, a branching one 7 ms.)
    static constexpr bool kWideSearch = K >= 4;
    const CellParams &P;
    WarpShared<MODE, K> &S;
    const int *offsets;   // shared copy of the offset table
    const int lane;
    Verts<MODE, K> V;
    Mask<K> Vm;           // valid vertex slots
    CellCtx C;
    unsigned fp_hi[PlaneSlots<K>::W > 2 ? 2 : 1];   // free plane slots 64-127 (128-vertex engines)

    __device__ Engine(const CellParams &p, WarpShared<MODE, K> &s, const int *off, int l)
        : P(p), S(s), offsets(off), lane(l) {}

    __device__ __forceinline__ void clear_slot(int s) {
        V.x[s] = V.y[s] = V.z[s] = __int_as_float(0x7fffffff);
        V.a[s] = V.e[s] = 0.0f;
        V.r2[s] = 0.0f;
        V.tri[s] = 0;
        if (MODE == VGPU_FP64) V.dx[s] = V.dy[s] = V.dz[s] = __longlong_as_double(0x7ff8000000000000ll);
    }

    // ---- bound of max |v|^2 and the candidate cut-off
    __device__ __forceinline__ void update_radius() {
        float m = 0.0f;   // r2 >= 0; fmaxf drops a NaN
#pragma unroll
        for (int s = 0; s < K; s++) m = fmaxf(m, V.r2[s]);
        C.R2 = warp_max_nonneg(m);
        if (P.g.poly) {
            float R = sqrtf(C.R2);
            float q = C.R2 + P.g.rmax32 * P.g.rmax32 - C.ri2;
            float D = R + sqrtf(fmaxf(q, 0.0f));
            C.cutoff2 = D * D * (1.0f + 8.0f * kU32);
        } else {
            C.cutoff2 = 4.0f * C.R2;
        }
    }

    // ---- vertex of slot s from the three planes of V.tri[s]
    __device__ __forceinline__ void compute_vertex(int s) {
        const unsigned t = V.tri[s];
        const int a = tri_plane(t, 0), b = tri_plane(t, 1), c = tri_plane(t, 2);
        if (MODE == VGPU_FP64) {
            double D;
            float kn;
            solve_f64(S.pl64x[a], S.pl64x[b], S.pl64x[c], V.dx[s], V.dy[s], V.dz[s], D, kn);
            const float vv = sqrtf((float)(V.dx[s] * V.dx[s] + V.dy[s] * V.dy[s] + V.dz[s] * V.dz[s]));
            V.e[s] = (float)(16.0 * kU64 * (double)kn / fabs(D)) + (float)(64.0 * kU64) * vv;
            V.a[s] = vv;
            if (!(D > 0.0)) C.marginal = true;
            const float r = vv * (1.0f + 4.0f * kU32) + V.e[s];
            V.r2[s] = r * r;
            return;
        }
        VertexF32 o = solve_vertex_f32(S.pl, S.pe, t);
        if (!(o.e <= kVertexTrust * o.a)) {
            if (kLean) C.needs_fp64 = true;   // the first pass hands the cell to the rerun
            else o = vertex_f64_fallback<MODE, K>(P, S, C.me64, t);
        }
        V.x[s] = o.x;
        V.y[s] = o.y;
        V.z[s] = o.z;
        V.a[s] = o.a;
        V.e[s] = o.e;
        V.r2[s] = o.r2;
    }

    // ---- initial cell: container box (src/container.hh:191-203, src/cell.cc:294-318,2567-2580)
    //      or the periodic unit cell (src/container_prd.hh:124-131)
    __device__ void init_cell(int k) {
        C.k = k;
        C.me64 = P.a.p64[k];
        C.me32 = P.a.l32[k];
        const int b = P.a.gblock[k];
        C.bi = b % P.g.gn[0];
        C.bj = (b / P.g.gn[0]) % P.g.gn[1];
        C.bk = b / (P.g.gn[0] * P.g.gn[1]);
        C.ri2 = C.me32.w * C.me32.w;
        C.deleted = C.overflow = C.marginal = C.repaired = C.needs_fp64 = false;
        C.fail_reason = 0;
        C.freeplanes[0] = ~0x3fu;
        C.freeplanes[1] = ~0u;
        if constexpr (PlaneSlots<K>::W > 2) fp_hi[0] = fp_hi[1] = ~0u;
        C.ncand = 0;
        C.tests = C.repairs = C.ptested = C.pcut = 0;
        if (lane < 6) {
            const double4 q = face64(P, C.me64, lane);
            if (MODE == VGPU_FP64) S.pl64x[lane] = q;
            S.pl[lane] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
            const float hf = fabsf((float)q.w);
            S.pe[lane] = make_float4(1.0f, 0.0f, 2.0f * kU32 * hf, hf);
            S.pid[lane] = P.g.unit_cell ? 0 : -(lane + 1);
            S.psrc[lane] = -1;
            S.pshift[lane] = lane;
        }
        Vm.clear();
        Vm.r[0] = 0xffu;
#pragma unroll
        for (int s = 0; s < K; s++) clear_slot(s);
        if (lane < 8) {
            S.tri[lane] = P.box_tri[lane];
            S.adj[lane] = P.box_adj[lane];
            V.tri[0] = P.box_tri[lane];
        }
        __syncwarp();
        if (lane < 8) compute_vertex(0);
        if (kLean && __any_sync(kFull, C.needs_fp64)) {
            C.overflow = true;
            C.fail_reason = 0;
            return;
        }
        update_radius();
        apply_walls();
    }

    // ---- the walls cut the initial cell in order (apply_walls,
    //      src/container.hh:86-89): lane w builds wall w's plane and adds it
    //      to the candidate buffer with distance 0 as source -1, face index
    //      6 + w; the search's first flush, which sorts them ahead of every
    //      particle candidate and in wall order, cuts with them through the
    //      one copy of the cutting code.  A wall that cuts the whole cell
    //      deletes it (compute_cell false).  A sheared periodic box binned
    //      at the reference's depth adds the unit cell's face planes here
    //      (type kWallLattice), sorted among the particle candidates.
    __device__ void apply_walls() {
        if (P.nwalls == 0) return;
        bool valid = false;
        float4 cd = make_float4(0, 0, 0, 0), ce = make_float4(0, 0, 0, 0);
        double4 q = make_double4(0, 0, 0, 0);
        if (lane < P.nwalls) {
            q = wall64_call(P.walls[lane], C.me64);
            valid = !isnan(q.w);   // NaN: no plane for this particle
            // the FP32 plane and its rounding: each component and h within
            // one unit in the last place
            const float nx = (float)q.x, ny = (float)q.y, nz = (float)q.z, h = (float)q.w;
            const float an = fabsf(nx) + fabsf(ny) + fabsf(nz);
            cd = make_float4(nx, ny, nz, h);
            // rs (w): 0 for a wall, which every flush tests; a unit-cell face
            // plane's |d|^2 (rounded down), so that a flush stops at it once
            // the cell no longer reaches it, as at a particle
            const float rs = P.walls[lane].type == kWallLattice ? 0.999f * (float)P.walls[lane].r : 0.0f;
            ce = make_float4(2.0f * kU32 * an, 2.0f * kU32 * fabsf(h),
                             sqrtf(nx * nx + ny * ny + nz * nz) * (1.0f + 8.0f * kU32) + 2.0f * kU32 * an, rs);
        }
        const unsigned bal = __ballot_sync(kFull, valid);
        if (valid) {
            const int slot = __popc(bal & ((1u << lane) - 1u));
            // walls first; a unit-cell face plane among the neighbours at its
            // lattice vector's distance, just ahead of the particle's own
            // image there (whose plane is the same: the face keeps ID 0, as
            // the unit cell's faces do in the reference)
            S.u.c.ck[slot] = (float_key(ce.w) & ~63u) | (unsigned)slot;
            S.u.c.cj[slot] = -1;
            S.u.c.cs[slot] = 6 + lane;
            S.u.c.cpid[slot] = P.walls[lane].id;
            S.u.c.cd[slot] = cd;
            S.u.c.ce[slot] = ce;
            if (MODE == VGPU_FP64) S.u.c.cd64[slot] = q;
        }
        C.ncand = __popc(bal);
    }

    // ---- plane slot allocation with recycling of dead planes
    //      (32-bit halves: the lowest free slot and its removal are single
    //      32-bit operations)
    __device__ __forceinline__ int alloc_plane() {
        if constexpr (PlaneSlots<K>::W == 2) {
            if ((C.freeplanes[0] | C.freeplanes[1]) == 0u) {
                unsigned long long live = 0ull;
#pragma unroll
                for (int s = 0; s < K; s++)
                    if (Vm.test(lane + 32 * s)) {
                        const unsigned t = V.tri[s];
                        live |= (1ull << tri_plane(t, 0)) | (1ull << tri_plane(t, 1)) | (1ull << tri_plane(t, 2));
                    }
                const unsigned long long fr = ~warp_or64(live);
                C.freeplanes[0] = (unsigned)fr;
                C.freeplanes[1] = (unsigned)(fr >> 32);
                if (fr == 0ull) return -1;
            }
            if (C.freeplanes[0]) {
                const int p = __ffs((int)C.freeplanes[0]) - 1;
                C.freeplanes[0] &= C.freeplanes[0] - 1u;
                return p;
            }
            const int p = 32 + __ffs((int)C.freeplanes[1]) - 1;
            C.freeplanes[1] &= C.freeplanes[1] - 1u;
            return p;
        } else {
            // 128 slots: words 0-1 in C.freeplanes, 2-3 in fp_hi
            unsigned *fw[4] = {&C.freeplanes[0], &C.freeplanes[1], &fp_hi[0], &fp_hi[1]};
            if ((C.freeplanes[0] | C.freeplanes[1] | fp_hi[0] | fp_hi[1]) == 0u) {
                unsigned live[4] = {0u, 0u, 0u, 0u};
#pragma unroll
                for (int s = 0; s < K; s++)
                    if (Vm.test(lane + 32 * s)) {
                        const unsigned t = V.tri[s];
#pragma unroll
                        for (int e = 0; e < 3; e++) plane_set_add(live, tri_plane(t, e));
                    }
                unsigned any = 0u;
#pragma unroll
                for (int w = 0; w < 4; w++) {
                    *fw[w] = ~__reduce_or_sync(kFull, live[w]);
                    any |= *fw[w];
                }
                if (any == 0u) return -1;
            }
#pragma unroll
            for (int w = 0; w < 4; w++)
                if (*fw[w]) {
                    const int p = 32 * w + __ffs((int)*fw[w]) - 1;
                    *fw[w] &= *fw[w] - 1u;
                    return p;
                }
            return -1;
        }
    }

    // ---- a candidate plane that cuts nothing but holds every vertex of a
    //      face within the tolerance band is that face's plane (a periodic
    //      box so sparse that a unit-cell face survives until the bisector of
    //      the particle's own image, the same plane, is tested): the face
    //      takes the candidate's ID, as the reference's facet construction
    //      through vertices on the plane relabels it (src/cell.cc:1166-1355).
    //      band: this lane's slots in the band.
    __device__ void relabel_coplanar(int cb, unsigned band) {
        constexpr int NW = PlaneSlots<K>::W;
        if constexpr (NW == 2) {
            unsigned long long on = 0ull, off = 0ull;
#pragma unroll
            for (int s = 0; s < K; s++)
                if (Vm.test(lane + 32 * s)) {
                    const unsigned t = V.tri[s];
                    const unsigned long long f =
                        (1ull << tri_plane(t, 0)) | (1ull << tri_plane(t, 1)) | (1ull << tri_plane(t, 2));
                    if ((band >> s) & 1u) on |= f;
                    else off |= f;
                }
            const unsigned long long faces = warp_or64(on) & ~warp_or64(off);
            if (lane == 0 && faces) {
                const int id = S.u.c.cpid[cb];
                for (unsigned long long m = faces; m; m &= m - 1ull) S.pid[__ffsll((long long)m) - 1] = id;
            }
        } else {
            unsigned on[NW], off[NW];
#pragma unroll
            for (int w = 0; w < NW; w++) on[w] = off[w] = 0u;
#pragma unroll
            for (int s = 0; s < K; s++)
                if (Vm.test(lane + 32 * s)) {
                    const unsigned t = V.tri[s];
#pragma unroll
                    for (int e = 0; e < 3; e++) {
                        if ((band >> s) & 1u) plane_set_add(on, tri_plane(t, e));
                        else plane_set_add(off, tri_plane(t, e));
                    }
                }
            const int id = S.u.c.cpid[cb];
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const unsigned faces = __reduce_or_sync(kFull, on[w]) & ~__reduce_or_sync(kFull, off[w]);
                if (lane == 0)
                    for (unsigned m = faces; m; m &= m - 1u) S.pid[32 * w + __ffs((int)m) - 1] = id;
            }
        }
        __syncwarp();
    }

    // ---- test candidate (buffer slot cb) and cut the cell if it intersects.
    __device__ __forceinline__ void test_and_cut(int cb) {
        PHASE_BEGIN(t_test);
        C.ptested++;
        C.tests += (unsigned)Vm.popc();
        bool out[K];
        unsigned uncbits = 0, band = 0;
        if (MODE == VGPU_FP64) {
            const double4 Q = S.u.c.cd64[cb];
            const double nq = fabs(Q.x) + fabs(Q.y) + fabs(Q.z);
#pragma unroll
            for (int s = 0; s < K; s++) {
                const double v = fma(Q.x, V.dx[s], fma(Q.y, V.dy[s], fma(Q.z, V.dz[s], -Q.w)));
                const double bnd = nq * (double)V.e[s] + 8.0 * kU64 * (nq * (double)V.a[s] + fabs(Q.w)) + P.g.tol_h;
                out[s] = v > bnd;
                if (!out[s] && v >= -bnd) uncbits |= 1u << s;
            }
            band = uncbits;   // tolerance band: kept, cell flagged
            if (__any_sync(kFull, uncbits != 0)) C.marginal = true;
        } else {
            const float4 Q = S.u.c.cd[cb];
            const float4 E = S.u.c.ce[cb];
            const float A = fmaf(3.0f * kU32, E.z, E.x);
            const float Cq = fmaf(3.0f * kU32, fabsf(Q.w), E.y) + P.g.tol_h32;
#pragma unroll
            for (int s = 0; s < K; s++) {
                out[s] = false;
                // a slot row with no vertex is skipped (the branch is the
                // warp's: Vm is the same in every lane); row 0 always holds some
                if (s > 0 && Vm.r[s] == 0u) continue;
                const float v = fmaf(Q.x, V.x[s], fmaf(Q.y, V.y[s], fmaf(Q.z, V.z[s], -Q.w)));
                const float bnd = 1.5f * fmaf(A, V.a[s], fmaf(E.z, V.e[s], Cq));
                out[s] = v > bnd;
                if (!(v > bnd) && v >= -bnd) uncbits |= 1u << s;
            }
            const unsigned ub = __ballot_sync(kFull, uncbits != 0);
            if (ub) {
                if (kLean) {   // the first pass hands the cell to the rerun, which repairs in FP64
                    C.overflow = true;
                    C.fail_reason = 0;
                    return;
                }
                C.repaired = true;
                C.repairs += __popc(ub);
                const unsigned ob = repair_tests<MODE, K>(P, S, C.me64, cb, uncbits, V.tri[0], K > 1 ? V.tri[K > 1 ? 1 : 0] : 0u,
                                                          K > 2 ? V.tri[K > 2 ? 2 : 0] : 0u, K > 3 ? V.tri[K > 3 ? 3 : 0] : 0u, &band);
                if (__any_sync(kFull, band != 0)) C.marginal = true;
#pragma unroll
                for (int s = 0; s < K; s++)
                    if ((uncbits >> s) & 1u) out[s] = (ob >> s) & 1u;
            }
        }
        const Mask<K> Rm = ballot_mask<K>(out);
        PHASE_END(t_test, 3);
        if (!Rm.any()) {
            if (!kLean && __any_sync(kFull, band != 0)) relabel_coplanar(cb, band);
            return;
        }
        if (Rm.equals(Vm)) {
            C.deleted = true;
            return;
        }
        PHASE_BEGIN(t_cut);
        C.pcut++;
        const int p = alloc_plane();
        if (p < 0) {
            C.overflow = true;
            C.fail_reason = VGPU_FAIL_PLANES;
            return;
        }
        if (lane == 0) {
            const float4 Q = S.u.c.cd[cb];
            const float4 E = S.u.c.ce[cb];
            const int j = S.u.c.cj[cb];
            S.pl[p] = Q;
            S.pe[p] = make_float4(E.z, E.x, E.y, fabsf(Q.w));
            S.pid[p] = S.u.c.cpid[cb];
            S.psrc[p] = j;
            S.pshift[p] = S.u.c.cs[cb];
            if (MODE == VGPU_FP64) S.pl64x[p] = S.u.c.cd64[cb];
        }
        cut(p, Rm, out);
        PHASE_END(t_cut, 4);
    }

    // ---- remove the vertices in Rm and close the hole with the face of plane p
    // (out: this lane's slots in Rm, the side test's own predicates)
    __device__ __forceinline__ void cut(int p, const Mask<K> &Rm, const bool (&out)[K]) {
        // Phase A: count boundary edges (edges from a removed vertex to a kept one)
        unsigned bnd[K], adj3[K];
        int nbe = 0;
        bool broken = false;
#pragma unroll
        for (int s = 0; s < K; s++) {
            bnd[s] = 0;
            adj3[s] = 0;
            if (out[s]) {
                const unsigned A3 = S.adj[lane + 32 * s];
                adj3[s] = A3;
#pragma unroll
                for (int e = 0; e < 3; e++) {
                    const int u = (A3 >> (8 * e)) & 255u;
                    if (u >= 32 * K) broken = true;
                    else if (!Rm.test(u)) bnd[s] |= 1u << e;
                }
                nbe += __popc(bnd[s]);
            }
        }
        int total;
        const int excl = warp_excl_scan_small<(3 * K < 8 ? 3 : (3 * K < 16 ? 4 : 5))>(nbe, lane, total);
        if (__any_sync(kFull, broken)) {  // inconsistent adjacency: hand the cell to the large engine
            C.overflow = true;
            C.fail_reason = VGPU_FAIL_ADJACENCY;
            return;
        }
        if (total < 3) {  // not a closed boundary: inconsistent side decisions
            C.marginal = true;
            return;
        }
        PHASE_COUNT(5, total);
        Mask<K> Fm;
#pragma unroll
        for (int i = 0; i < K; i++) Fm.r[i] = ~Vm.r[i] | Rm.r[i];
        if (Fm.popc() < total) {
            C.overflow = true;
            C.fail_reason = VGPU_FAIL_VERTICES;
            return;
        }
        // stage the boundary edges (a -> b, kept neighbour u) in lane order
        {
            int q = excl;
#pragma unroll
            for (int s = 0; s < K; s++) {
                if (bnd[s]) {
                    const unsigned T = V.tri[s];
                    const unsigned A3 = adj3[s];
#pragma unroll
                    for (int e = 0; e < 3; e++)
                        if ((bnd[s] >> e) & 1u) {
                            // bytes e and e+1 (mod 3) of T, byte e of A3, and T's
                            // zero top byte, in one byte permutation; the planes
                            // masked to their 7 bits as tri_plane does
                            constexpr unsigned kSel[3] = {0x3410u, 0x3521u, 0x3602u};
                            S.stage[q++] = __byte_perm(T, A3, kSel[e]) & 0x00ff7f7fu;
                        }
                }
            }
        }
        __syncwarp();
        // Phase B: the free slot of rank r hosts the new vertex (a, b, p) of boundary
        // edge r and solves its position.  Ranks count within the first slot row s
        // (lanes' s-th slots) that has room for all the new vertices, so that their
        // solves run in one pass; across all free slots only when no row has room.
        unsigned fw[K];   // free lanes of each slot row
#pragma unroll
        for (int s = 0; s < K; s++) fw[s] = Fm.r[s];
        int hs = -1;
#pragma unroll
        for (int s = K - 1; s >= 0; s--)
            if (__popc(fw[s]) >= total) hs = s;
        const unsigned lt = (1u << lane) - 1u;
        int before = 0;   // free slots ranked in the rows before s
        bool host[K];
#pragma unroll
        for (int s = 0; s < K; s++) {
            const int t = lane + 32 * s;
            const unsigned row = (hs < 0 || hs == s) ? fw[s] : 0u;
            const int r = before + __popc(row & lt);
            before += __popc(row);
            host[s] = false;
            if ((row >> lane) & 1u) {
                if (r < total) {
                    host[s] = true;
                    const unsigned E = S.stage[r];
                    const int a = E & 255u, b = (E >> 8) & 255u, u = E >> 16;   // (E's top byte is 0)
                    const unsigned T = __byte_perm(E, (unsigned)p, 0x5410u);   // a | b << 8 | p << 16
                    V.tri[s] = T;
                    S.tri[t] = T;
                    S.adj[t] = (unsigned)u;
                    S.startN[a] = (unsigned char)t;
                    S.endN[b] = (unsigned char)t;
                    const unsigned Tu = S.tri[u];
#pragma unroll
                    for (int e = 0; e < 3; e++)
                        if (tri_plane(Tu, e) == b && tri_plane(Tu, e == 2 ? 0 : e + 1) == a)
                            reinterpret_cast<unsigned char *>(&S.adj[u])[e] = (unsigned char)t;
                    // its position: independent of the linking, so the solve's
                    // arithmetic fills the shared-memory latencies around it
                    compute_vertex(s);
                }
            }
        }
        __syncwarp();
        if (kLean && __any_sync(kFull, C.needs_fp64)) {
            C.overflow = true;
            C.fail_reason = 0;
            return;
        }
        // Phase C: link the new vertices around the new face; clear freed slots
        bool bad = false;
#pragma unroll
        for (int s = 0; s < K; s++) {
            if (host[s]) {
                const int t = lane + 32 * s;
                const unsigned T = V.tri[s];
                const int a = T & 255u, b = (T >> 8) & 255u;
                if (S.startN[a] != t) bad = true;
                unsigned char *ab = reinterpret_cast<unsigned char *>(&S.adj[t]);
                ab[1] = S.startN[b];
                ab[2] = S.endN[a];
            } else if (Rm.test(lane + 32 * s)) {
                clear_slot(s);
            }
        }
        if (__any_sync(kFull, bad)) C.marginal = true;
        const Mask<K> Nm = ballot_mask<K>(host);
#pragma unroll
        for (int i = 0; i < K; i++) Vm.r[i] = (Vm.r[i] & ~Rm.r[i]) | Nm.r[i];
        __syncwarp();
        update_radius();
    }

    // ---- candidate buffer: sort by (power) distance and test in order
    __device__ void flush() {
        const int n = C.ncand;
        if (n == 0) return;
        PHASE_COUNT(0, 1);
        PHASE_COUNT(1, n > 32 ? 1 : 0);
        PHASE_BEGIN(t_sort);
        __syncwarp();
        unsigned k0 = lane < n ? S.u.c.ck[lane] : 0xffffffffu;
        unsigned k1 = lane + 32 < n ? S.u.c.ck[lane + 32] : 0xffffffffu;
        if (n > 32) {
            const uint2 kk = bitonic64(k0, k1, lane);
            k0 = kk.x;
            k1 = kk.y;
        } else {
            k0 = bitonic32(k0, lane);
        }
        PHASE_END(t_sort, 2);
        for (int i = 0; i < n; i++) {
            const unsigned key = __shfl_sync(kFull, i < 32 ? k0 : k1, i & 31);
            const int cb = key & 63u;
            const float4 E = S.u.c.ce[cb];
            if (P.g.poly) {
                const float rs = E.w;
                if (!(rs <= 0.0f || rs * rs < 4.0f * C.R2 * E.z * E.z * (1.0f + 16.0f * kU32))) continue;
            } else {
                if (E.w >= C.cutoff2 * (1.0f + 1e-4f)) break;
            }
            test_and_cut(cb);
            if (C.deleted || C.overflow) break;
        }
        C.ncand = 0;
        __syncwarp();
    }

#if VGPU_GATHER_TMA
    // ---- candidates w0 .. w0+kStageEntries-1 of a block pass into S.cstage:
    //      each lane copies the part of its block's run (16-byte particles,
    //      contiguous in engine order) that falls in the window.  False (the
    //      caller reads global memory) when staging is off for this warp; a
    //      wait that runs out turns staging off for the rest of the launch.
    __device__ bool stage_runs(int w0, int tot, int incl, int cnt, int st) {
        const unsigned ph = S.cbar_phase;
        if (ph & 0x80000000u) return false;
        const int W = min(kStageEntries, tot - w0);
        fence_proxy_async_smem();   // earlier reads of the window before the copies' writes
        __syncwarp();
        if (lane == 0) mbar_expect_tx(&S.cbar, (unsigned)W * 16u);
        __syncwarp();
        const int r0 = incl - cnt;
        const int a = max(r0, w0), b = min(incl, w0 + W);
        if (b > a) bulk_g2s(&S.cstage[a - w0], P.a.l32 + st + (a - r0), (unsigned)(b - a) * 16u, &S.cbar);
        const bool ok = __all_sync(kFull, mbar_wait_bounded(&S.cbar, ph & 1u));
        __syncwarp();
        if (lane == 0) S.cbar_phase = ok ? (ph ^ 1u) : 0x80000000u;
        __syncwarp();
        return ok;
    }
#endif

    // a block offset in one word: 10 bits per axis (|offset| <= kMaxShellRadius)
    __device__ __forceinline__ static int pack_offset(int di, int dj, int dk) {
        return (di + kShellPack) | ((dj + kShellPack) << 10) | ((dk + kShellPack) << 20);
    }

    // ---- candidates from a range of block offsets: wrap/skip, block distance,
    //      then one lane per candidate particle
    __device__ void gather_offsets(int e_begin, int e_end, bool from_table, int shell_r) {
        const float l0 = C.me32.x, l1 = C.me32.y, l2 = C.me32.z;
        for (int base = e_begin; base < e_end; base += 32) {
            PHASE_COUNT(2, 1);
            const int e = base + lane;
            int di = 0, dj = 0, dk = 0;
            bool ok = e < e_end;
            if (ok) {
                if (from_table) {
                    const int code = offsets[e];
                    di = (code & 31) - 16;
                    dj = ((code >> 5) & 31) - 16;
                    dk = ((code >> 10) & 31) - 16;
                } else {
                    // (at radius kOffsetRadius the table already holds the
                    // offsets of lower bound <= kTableLb2Max)
                    if constexpr (kWideSearch) {
                        ok = shell_offset(e, shell_r, di, dj, dk);   // the cube's faces
                    } else {   // the whole cube, without branches
                        const int w = 2 * shell_r + 1;
                        di = e % w - shell_r;
                        dj = (e / w) % w - shell_r;
                        dk = e / (w * w) - shell_r;
                        ok = max(abs(di), max(abs(dj), abs(dk))) == shell_r;
                    }
                    const int a = max(abs(di) - 1, 0), b = max(abs(dj) - 1, 0), c = max(abs(dk) - 1, 0);
                    ok = ok && (a * a + b * b + c * c > kTableLb2Max);
                }
            }
            int cnt = 0, st = 0, code = 0;
            {
                const int d[3] = {di, dj, dk};
                const int cb[3] = {C.bi + di, C.bj + dj, C.bk + dk};
                const float l[3] = {l0, l1, l2};
                int wr[3], img[3];
                float md2 = 0.0f;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const int n = P.g.gn[a];
                    int c = cb[a];
                    img[a] = 0;
                    if (P.g.per[a]) {
                        if (from_table && n > 2 * kOffsetRadius) {
                            if (c < 0) { c += n; img[a] = -1; }
                            else if (c >= n) { c -= n; img[a] = 1; }
                        } else {
                            int w = c % n;
                            if (w < 0) w += n;
                            img[a] = (c - w) / n;
                            c = w;
                        }
                    } else if (c < 0 || c >= n) {
                        ok = false;
                    }
                    wr[a] = c;
                    const float bs = P.g.gbs32[a];
                    float t = d[a] > 0 ? (float)d[a] * bs - l[a] : (d[a] < 0 ? l[a] - (float)(d[a] + 1) * bs : 0.0f);
                    t = fmaxf(t, 0.0f);
                    md2 = fmaf(t, t, md2);
                }
                if (ok && md2 * (1.0f - 1e-5f) >= C.cutoff2) ok = false;
                if (ok) {
                    const int b = wr[0] + P.g.gn[0] * (wr[1] + P.g.gn[1] * wr[2]);
                    st = P.a.bstart[b];
                    cnt = P.a.bstart[b + 1] - st;
                    code = (img[0] + 128) | ((img[1] + 128) << 8) | ((img[2] + 128) << 16);
                }
            }
            const int incl = warp_incl_scan(cnt, lane);
            const int tot = __shfl_sync(kFull, incl, 31);
            const int packed_d = pack_offset(di, dj, dk);
#if VGPU_GATHER_TMA
            int w0 = 0;
            bool staged = false;
#endif
            for (int c0 = 0; c0 < tot; c0 += 32) {
                PHASE_COUNT(3, 1);
                if (C.ncand > kCandBuf - 32) {
                    PHASE_BEGIN(t_nested);
                    flush();
                    PHASE_END(t_nested, 6);
                }
                if (C.deleted || C.overflow) return;
#if VGPU_GATHER_TMA
                if ((c0 & (kStageEntries - 1)) == 0) {
                    w0 = c0;
                    staged = stage_runs(c0, tot, incl, cnt, st);
                }
#endif
                const int c = c0 + lane;
                // owner lane: number of lanes whose inclusive prefix is <= c
                int pos = 0;
#pragma unroll
                for (int w = 16; w >= 1; w >>= 1) {
                    const int v = __shfl_sync(kFull, incl, pos + w - 1);
                    if (v <= c) pos += w;
                }
                pos = min(pos, 31);
                const int o_incl = __shfl_sync(kFull, incl, pos);
                const int o_cnt = __shfl_sync(kFull, cnt, pos);
                const int o_st = __shfl_sync(kFull, st, pos);
                const int o_code = __shfl_sync(kFull, code, pos);
                const int o_d = __shfl_sync(kFull, packed_d, pos);
                bool pass = false;
                unsigned key = 0;
                float4 cd = make_float4(0, 0, 0, 0), ce = make_float4(0, 0, 0, 0);
                const int j = o_st + (c - (o_incl - o_cnt));
                if (c < tot) {
                    const int ddi = (o_d & 1023) - kShellPack, ddj = ((o_d >> 10) & 1023) - kShellPack,
                              ddk = ((o_d >> 20) & 1023) - kShellPack;
                    const bool self = (j == C.k) && ddi == 0 && ddj == 0 && ddk == 0;
                    if (!self) {
#if VGPU_GATHER_TMA
                        const float4 lj = staged ? S.cstage[c - w0] : P.a.l32[j];
#else
                        const float4 lj = P.a.l32[j];
#endif
                        const float dx = fmaf((float)ddi, P.g.gbs32[0], lj.x - l0);
                        const float dy = fmaf((float)ddj, P.g.gbs32[1], lj.y - l1);
                        const float dz = fmaf((float)ddk, P.g.gbs32[2], lj.z - l2);
                        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        float rs = d2, rr = 0.0f;
                        if (P.g.poly) {
                            rr = C.ri2 + lj.w * lj.w;
                            rs = d2 + (C.ri2 - lj.w * lj.w);
                            pass = rs <= 0.0f || rs * rs < 4.0f * C.R2 * d2 * (1.0f + 16.0f * kU32);
                        } else {
                            pass = d2 < C.cutoff2 * (1.0f + 1e-5f);
                        }
                        // forward error of the FP32 plane: local coordinates and block
                        // offsets each carry at most u*bs; the sum one more rounding
                        const int M = max(abs(ddi), max(abs(ddj), abs(ddk)));
                        // |n| rounded up (rsqrtf: 2 ulp) as an upper bound of the root
                        const float dn = d2 > 0.0f ? d2 * rsqrtf(d2) * (1.0f + 8.0f * kU32) : 0.0f;
                        const float en = kU32 * (1.75f * (float)(M + 3) * P.g.gbs_max + 1.01f * dn) + 1e-12f * P.g.gbs_max;
                        const float eh = dn * en + 2.0f * kU32 * (d2 + rr) + 0.5f * en * en;
                        cd = make_float4(dx, dy, dz, 0.5f * rs);
                        ce = make_float4(en, eh, dn, rs);
                        key = float_key(rs);
                    }
                }
                const unsigned bal = __ballot_sync(kFull, pass);
                if (pass) {
                    const int slot = C.ncand + __popc(bal & ((1u << lane) - 1u));
                    S.u.c.ck[slot] = (key & ~63u) | (unsigned)slot;
                    S.u.c.cj[slot] = j;
                    S.u.c.cs[slot] = o_code;
                    S.u.c.cpid[slot] = P.a.pid[j];
                    S.u.c.cd[slot] = cd;
                    S.u.c.ce[slot] = ce;
                    if (MODE == VGPU_FP64) S.u.c.cd64[slot] = plane64_from(P, C.me64, j, o_code);
                }
                C.ncand += __popc(bal);
                PHASE_COUNT(4, __popc(bal));
            }
        }
    }

    // ---- the search: blocks in order of lower-bound distance (src/v_compute.cc:289-621
    //      does the same with its 64 worklists, mrad cut-offs and the block queue).
    //      Segments 0..ngroups-1 are the table's distance groups; after them come
    //      Chebyshev shells r = kOffsetRadius, ... with what the table covered skipped.
    __device__ void search() {
        const float bmin2 = P.g.gbs_min * P.g.gbs_min;
        const int rmax_grid = max(P.g.gn[0], max(P.g.gn[1], P.g.gn[2]));
        const bool any_periodic = P.g.per[0] || P.g.per[1] || P.g.per[2];
        const int rlim = min(4 * rmax_grid + 8, kWideSearch ? kMaxShellRadius : kNarrowShellRadius);
        for (int seg = 0;; seg++) {
            const bool table = seg < P.ngroups;
            int b0 = 0, b1 = 0, r = 0;
            float lb2;
            if (table) {
                lb2 = (float)P.group_lb2[seg] * bmin2;
                b0 = P.group_start[seg];
                b1 = P.group_start[seg + 1];
            } else {
                r = kOffsetRadius + (seg - P.ngroups);
                if (r >= rlim) {
                    C.overflow = true;  // search did not terminate
                    C.fail_reason = VGPU_FAIL_SEARCH;
                    return;
                }
                if (!any_periodic && r > rmax_grid + 1) return;
                lb2 = (float)((r - 1) * (r - 1)) * bmin2;
                b1 = kWideSearch ? 6 * (2 * r + 1) * (2 * r + 1) : (2 * r + 1) * (2 * r + 1) * (2 * r + 1);
            }
            if (lb2 >= C.cutoff2 * (1.0f + 1e-5f)) return;
            PHASE_COUNT(6, 1);
            PHASE_BEGIN(t_g);
            gather_offsets(b0, b1, table, r);
            PHASE_END(t_g, 1);
            if (C.deleted || C.overflow) return;
            flush();
            if (C.deleted || C.overflow) return;
        }
    }

    // ---- reductions: vertex/face counts, neighbours, FP64 volume and centroid
    // ---- results of a cell with no polytope: deleted (compute_cell false), or
    //      overflowed (a larger engine reruns it and overwrites this; if none
    //      does, it stays failed)
    __device__ __forceinline__ void write_empty() {
        const int out = P.a.outpos[C.k];
        if (lane == 0) {
            P.r.vol[out] = 0.0;
            P.r.cen[3 * out] = P.r.cen[3 * out + 1] = P.r.cen[3 * out + 2] = 0.0;
            P.r.nf[out] = 0;
            P.r.nv[out] = 0;
            P.r.maxr2[out] = 0.0;
            P.r.flags[out] = C.overflow ? (VGPU_CELL_FAILED | (C.fail_reason << 8))
                                        : ((C.marginal ? VGPU_CELL_MARGINAL : 0) | (C.repaired ? VGPU_CELL_REPAIRED : 0));
        }
    }

    __device__ void run(int k) {
#ifdef VGPU_PHASE_TIMING
        for (int i = 0; i < 16; i++) C.phase[i] = 0;
        PHASE_COUNT(7, 1);
#endif
        PHASE_BEGIN(t_init);
        init_cell(k);
        PHASE_END(t_init, 0);
        search();
        PHASE_BEGIN(t_fin);
        // no reductions here: the finish kernel completes the cell from its
        // record, which keeps the FP64 code out of this kernel's instruction
        // stream; a full record store fails the cell
        if (!C.overflow && !C.deleted) {
            if (emit_record()) {
                PHASE_END(t_fin, 5);
                return;
            }
            C.overflow = true;
            C.fail_reason = VGPU_FAIL_RECORDS;
        }
        write_empty();
        PHASE_END(t_fin, 5);
    }

    // ---- the finished polytope as a compact record for the finish kernel
    //      (stored by VGPU_RECORD_STORE)
    //      (layout in CellParams): valid vertices and live planes only, in
    //      slot order, with plane and vertex indices renumbered to match;
    //      false if the record store is full
    __device__ bool emit_record() {
        constexpr int VW = MODE == VGPU_FP64 ? 6 : 3;   // words per vertex position
        constexpr int NW = PlaneSlots<K>::W;
        // the live planes as NW 32-bit words (64 slots: built as one 64-bit word)
        unsigned live[NW];
        int nf = 0;
        if constexpr (NW == 2) {
            unsigned long long l64 = 0ull;
#pragma unroll
            for (int s = 0; s < K; s++)
                if (Vm.test(lane + 32 * s)) {
                    const unsigned t = V.tri[s];
                    l64 |= (1ull << tri_plane(t, 0)) | (1ull << tri_plane(t, 1)) | (1ull << tri_plane(t, 2));
                }
            l64 = warp_or64(l64);
            live[0] = (unsigned)l64;
            live[1] = (unsigned)(l64 >> 32);
            nf = __popcll(l64);
        } else {
#pragma unroll
            for (int w = 0; w < NW; w++) live[w] = 0u;
#pragma unroll
            for (int s = 0; s < K; s++)
                if (Vm.test(lane + 32 * s)) {
                    const unsigned t = V.tri[s];
#pragma unroll
                    for (int e = 0; e < 3; e++) plane_set_add(live, tri_plane(t, e));
                }
#pragma unroll
            for (int w = 0; w < NW; w++) {
                live[w] = __reduce_or_sync(kFull, live[w]);
                nf += __popc(live[w]);
            }
        }
        const int nv = Vm.popc();
        const unsigned words = (unsigned)(kRecHeader + (2 + VW) * nv + 3 * nf);
        unsigned long long off = 0;
        if (lane == 0) off = atomicAdd(P.rec_used, (unsigned long long)words);
        off = __shfl_sync(kFull, off, 0);
        if (off + words > P.rec_cap) return false;
        unsigned *R = P.rec + off;
        if (lane == 0) {
            VGPU_RECORD_STORE(&R[0], (unsigned)nv);
            VGPU_RECORD_STORE(&R[1], (unsigned)nf);
            VGPU_RECORD_STORE(&R[2], (C.marginal ? VGPU_CELL_MARGINAL : 0) | (C.repaired ? VGPU_CELL_REPAIRED : 0));
            VGPU_RECORD_STORE(&R[3], 0);
            VGPU_RECORD_STORE(&R[4], 0);
        }
        // compact indices: vertex slot -> rank among valid slots (vmap),
        // plane slot -> rank among live planes (endN, free once the cell is done)
#pragma unroll
        for (int s = 0; s < K; s++) {
            const int t = lane + 32 * s;
            if (Vm.test(t)) S.vmap[t] = (unsigned char)Vm.rank(t);
        }
        if constexpr (NW == 2) {
            const unsigned long long l64 = ((unsigned long long)live[1] << 32) | live[0];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int q = lane + 32 * h;
                if ((l64 >> q) & 1ull) S.endN[q] = (unsigned char)__popcll(l64 & ((1ull << q) - 1ull));
            }
        } else {
            const unsigned lt = (1u << lane) - 1u;
            int before = 0;
#pragma unroll
            for (int h = 0; h < NW; h++) {
                if ((live[h] >> lane) & 1u) S.endN[lane + 32 * h] = (unsigned char)(before + __popc(live[h] & lt));
                before += __popc(live[h]);
            }
        }
        __syncwarp();
        unsigned *rv = R + kRecHeader;
#pragma unroll
        for (int s = 0; s < K; s++) {
            const int t = lane + 32 * s;
            if (Vm.test(t)) {
                const int r = S.vmap[t];
                const unsigned T = V.tri[s];
                const unsigned A3 = S.adj[t];
                VGPU_RECORD_STORE(&rv[r], (unsigned)S.endN[tri_plane(T, 0)] | ((unsigned)S.endN[tri_plane(T, 1)] << 8) |
                        ((unsigned)S.endN[tri_plane(T, 2)] << 16));
                VGPU_RECORD_STORE(&rv[nv + r], (unsigned)S.vmap[A3 & 255u] | ((unsigned)S.vmap[(A3 >> 8) & 255u] << 8) |
                             ((unsigned)S.vmap[(A3 >> 16) & 255u] << 16));
                if (MODE == VGPU_FP64) {
                    const double c[3] = {V.dx[s], V.dy[s], V.dz[s]};
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        const unsigned long long b = (unsigned long long)__double_as_longlong(c[a]);
                        VGPU_RECORD_STORE(&rv[(2 + 2 * a) * nv + 2 * r], (unsigned)b);
                        VGPU_RECORD_STORE(&rv[(2 + 2 * a) * nv + 2 * r + 1], (unsigned)(b >> 32));
                    }
                } else {
                    VGPU_RECORD_STORE(&rv[2 * nv + r], __float_as_uint(V.x[s]));
                    VGPU_RECORD_STORE(&rv[3 * nv + r], __float_as_uint(V.y[s]));
                    VGPU_RECORD_STORE(&rv[4 * nv + r], __float_as_uint(V.z[s]));
                }
            }
        }
        unsigned *rp = rv + (2 + VW) * nv;
#pragma unroll
        for (int h = 0; h < NW; h++) {
            const int q = lane + 32 * h;
            if ((live[h] >> lane) & 1u) {
                const int r = S.endN[q];
                VGPU_RECORD_STORE(&rp[r], (unsigned)S.psrc[q]);
                VGPU_RECORD_STORE(&rp[nf + r], (unsigned)S.pshift[q]);
                VGPU_RECORD_STORE(&rp[2 * nf + r], (unsigned)S.pid[q]);
            }
        }
        if (lane == 0) P.rec_off[C.k] = off;
        return true;
    }
};

// CTAs of 4 warps kept resident per SM by the main (mixed, 64-slot, FP64-free)
// engine; it fixes the register budget (65536 / (128 * blocks)).  Measured on
// the 4M periodic box (both clipping passes): with the slot masks as 64-bit
// words 6 (80 registers, 24 warps per SM) 82.2 ms, 5 (96) 83.5 ms, 7 (72)
// 84.2 ms, 4 (103, no spills) 88.9 ms, 3 (118) 86.8 ms; with one 32-bit word
// per slot row (no spills at 80 registers) 6: 66.49 ms, 7: 66.34 ms (72
// registers, 44 bytes spilled); shared memory allows no more than 7.  (With
// the FP64 repair and vertex calls in this engine it needed 224 registers:
// 3 CTAs at 168 registers, 102 ms.)
#ifndef VGPU_MIN_BLOCKS
#define VGPU_MIN_BLOCKS 7
#endif
// Largest CTA the clipping kernels are built for (VGPU_CTA_THREADS, in
// vgpu_internal.cuh); the default launch uses 4 warps.
constexpr int kMaxCtaWarps = kBuiltCtaWarps;
// CTAs per SM of the other engines: the full mixed 64-slot engine keeps
// VGPU_FULL_MIN_BLOCKS (3: 168 registers), the 128-slot and FP64 engines 2.
// The full engine reruns the cells the first pass hands on (2.3 % on the 4M
// periodic box); its clipping there took 66.4 ms at 3, 66.9 ms at 2 (no
// spills) and 67.0 ms at 4 (128 registers, 484 bytes spilled).
#ifndef VGPU_FULL_MIN_BLOCKS
#define VGPU_FULL_MIN_BLOCKS 3
#endif
template <int MODE, int K, bool LEAN>
constexpr int min_blocks() {
    return (MODE == VGPU_MIXED && K == 2) ? (LEAN ? VGPU_MIN_BLOCKS : VGPU_FULL_MIN_BLOCKS) : 2;
}
// Cells a warp takes from the work queue at a time (at most; fewer when the
// launch has under four chunks per warp, so that small containers still
// spread over all warps).  Consecutive cells (engine order: neighbouring
// blocks) search nearly the same blocks, so a warp that runs them back to
// back finds their block starts and particles in its SM's L1.  On the 4M
// periodic box the clipping passes take 77.9 / 78.1 / 78.4 ms with chunks
// of 4 / 8 / 16: within the run-to-run spread.  (VGPU_CELL_CHUNK, in
// vgpu_internal.cuh; per container: vgpu_tuning.cells_per_chunk.)

template <int MODE, int K, bool LEAN>
__global__ void __launch_bounds__(VGPU_CTA_THREADS, min_blocks<MODE, K, LEAN>()) cell_kernel(const __grid_constant__ CellParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *offsets = reinterpret_cast<int *>(smem_raw);
    const size_t off_bytes = ((size_t)P.noffsets * sizeof(int) + 15) & ~(size_t)15;
    WarpShared<MODE, K> *ws = reinterpret_cast<WarpShared<MODE, K> *>(smem_raw + off_bytes);
    for (int i = threadIdx.x; i < P.noffsets; i += blockDim.x) offsets[i] = P.offsets[i];
    __syncthreads();
    WarpShared<MODE, K> &S = ws[wid];
    if (lane < 6) S.stat[lane] = 0ull;
#if VGPU_GATHER_TMA
    if (lane == 0) {
        mbar_init(&S.cbar, 1);
        S.cbar_phase = 0;
    }
    __syncwarp();
#endif
#ifdef VGPU_PHASE_TIMING
    unsigned long long ph[16] = {};
    const long long t_kernel0 = clock64();
#endif
    unsigned long long *work = P.cell_list ? &P.cnt->overflow_work : &P.cnt->work;
    const int chunk = max(1, min(P.cell_chunk > 0 ? P.cell_chunk : VGPU_CELL_CHUNK,
                                 P.ncells / (int)(4 * gridDim.x * (blockDim.x >> 5))));
    int w = 0, wend = 0;
    for (;;) {
        if (w == wend) {
            if (lane == 0) w = (int)atomicAdd(work, (unsigned long long)chunk);
            w = __shfl_sync(kFull, w, 0);
            if (w >= P.ncells) break;
            wend = min(w + chunk, P.ncells);
        }
        const int k = P.cell_list ? P.cell_list[w] : P.cell_begin + w;
        w++;
        Engine<MODE, K, LEAN> eng(P, S, offsets, lane);
        eng.run(k);
#ifdef VGPU_PHASE_TIMING
        for (int i = 0; i < 16; i++) ph[i] += eng.C.phase[i];
#endif
        if (lane == 0) {
            S.stat[0] += eng.C.tests;
            S.stat[1] += eng.C.repairs;
            S.stat[2] += eng.C.ptested;
            S.stat[3] += eng.C.pcut;
            if (eng.C.overflow) {
                const unsigned long long slot = atomicAdd(&P.cnt->overflow, 1ull);
                if (P.overflow_list) P.overflow_list[slot] = k;
            } else {
                S.stat[4] += eng.C.deleted ? 1 : 0;
                S.stat[5] += eng.C.marginal ? 1 : 0;
            }
        }
        __syncwarp();
    }
    if (lane == 0) {
        atomicAdd(&P.cnt->side_tests, S.stat[0]);
        atomicAdd(&P.cnt->fp64_repairs, S.stat[1]);
        atomicAdd(&P.cnt->planes_tested, S.stat[2]);
        atomicAdd(&P.cnt->planes_cut, S.stat[3]);
        atomicAdd(&P.cnt->deleted, S.stat[4]);
        atomicAdd(&P.cnt->marginal, S.stat[5]);
#ifdef VGPU_PHASE_TIMING
        ph[7] = (unsigned long long)(clock64() - t_kernel0);
        for (int i = 0; i < 16; i++) atomicAdd(&P.cnt->phase_cycles[i], ph[i]);
#endif
    }
}

// Many containers in one persistent launch.  A warp takes global cell indices
// from one queue (container-major, so neighbouring warps share blocks); when
// a cell belongs to another container than the warp's previous one, the warp
// copies that container's parameters into its shared slot and flushes its
// counters to the previous container's.
template <int MODE, int K, bool LEAN>
__global__ void __launch_bounds__(VGPU_CTA_THREADS, min_blocks<MODE, K, LEAN>()) cell_batch_kernel(const __grid_constant__ BatchParams B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int warps = blockDim.x >> 5;
    int *offsets = reinterpret_cast<int *>(smem_raw);
    const size_t off_bytes = ((size_t)B.noffsets * sizeof(int) + 15) & ~(size_t)15;
    constexpr size_t cp_slot = (sizeof(CellParams) + 15) & ~(size_t)15;
    CellParams *cps = reinterpret_cast<CellParams *>(smem_raw + off_bytes);
    WarpShared<MODE, K> *ws = reinterpret_cast<WarpShared<MODE, K> *>(smem_raw + off_bytes + cp_slot * warps);
    for (int i = threadIdx.x; i < B.noffsets; i += blockDim.x) offsets[i] = B.offsets[i];
    __syncthreads();
    CellParams &P = *reinterpret_cast<CellParams *>(reinterpret_cast<unsigned char *>(cps) + cp_slot * wid);
    WarpShared<MODE, K> &S = ws[wid];
#if VGPU_GATHER_TMA
    if (lane == 0) {
        mbar_init(&S.cbar, 1);
        S.cbar_phase = 0;
    }
    __syncwarp();
#endif
    int cur = -1;
    long long cbeg = 0, cend = 0;
    unsigned long long tests = 0, repairs = 0, ptested = 0, pcut = 0, deleted = 0, marginal = 0, ovf = 0;
    auto flush = [&]() {
        if (cur >= 0 && lane == 0) {
            Counters *c = B.cps[cur].cnt;
            atomicAdd(&c->side_tests, tests);
            atomicAdd(&c->fp64_repairs, repairs);
            atomicAdd(&c->planes_tested, ptested);
            atomicAdd(&c->planes_cut, pcut);
            atomicAdd(&c->deleted, deleted);
            atomicAdd(&c->marginal, marginal);
            if (ovf) atomicAdd(B.overflow_list ? &c->overflow : &c->failed, ovf);
        }
        tests = repairs = ptested = pcut = deleted = marginal = ovf = 0;
    };
    const long long chunk =
        max(1ll, min((long long)VGPU_CELL_CHUNK, B.ncells / (long long)(4 * gridDim.x * (blockDim.x >> 5))));
    long long w = 0, wend = 0;
    for (;;) {
        if (w == wend) {
            if (lane == 0) w = (long long)atomicAdd(B.work, (unsigned long long)chunk);
            w = __shfl_sync(kFull, w, 0);
            if (w >= B.ncells) break;
            wend = min(w + chunk, B.ncells);
        }
        const long long gidx = B.cell_list ? B.cell_list[w] : B.cell_begin + w;
        w++;
        if (gidx < cbeg || gidx >= cend) {
            flush();
            // the container c with cell_start[c] <= gidx < cell_start[c+1]
            int lo = 0, hi = B.ncont;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (B.cell_start[mid] <= gidx) lo = mid;
                else hi = mid;
            }
            cur = lo;
            cbeg = B.cell_start[lo];
            cend = B.cell_start[lo + 1];
            __syncwarp();
            const unsigned *src = reinterpret_cast<const unsigned *>(B.cps + cur);
            unsigned *dst = reinterpret_cast<unsigned *>(&P);
            for (int i = lane; i < (int)(sizeof(CellParams) / 4); i += 32) dst[i] = src[i];
            __syncwarp();
        }
        // a sheared box's cells are its particles, not the images it stores
        const int k = P.cell_list ? P.cell_list[gidx - cbeg] : (int)(gidx - cbeg);
        Engine<MODE, K, LEAN> eng(P, S, offsets, lane);
        eng.run(k);
        tests += eng.C.tests;
        repairs += eng.C.repairs;
        ptested += eng.C.ptested;
        pcut += eng.C.pcut;
        if (eng.C.overflow) {
            ovf++;
            if (lane == 0 && B.overflow_list) {
                const unsigned long long slot = atomicAdd(B.overflow_count, 1ull);
                B.overflow_list[slot] = gidx;
            }
        } else {
            deleted += eng.C.deleted ? 1 : 0;
            marginal += eng.C.marginal ? 1 : 0;
        }
        __syncwarp();
    }
    flush();
}

template <int MODE, int K, bool LEAN>
cudaError_t launch_one(const CellParams &cp, int warps, int sms, cudaStream_t s) {
    const size_t off_bytes = ((size_t)cp.noffsets * sizeof(int) + 15) & ~(size_t)15;
    const size_t smem = off_bytes + warps * sizeof(WarpShared<MODE, K>);
    cudaError_t e = cudaFuncSetAttribute(cell_kernel<MODE, K, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cell_kernel<MODE, K, LEAN>, warps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sms * per_sm;
    const long long need = (cp.ncells + warps - 1) / warps;
    int grid = (int)(want < need ? want : need);
    if (grid < 1) grid = 1;
    cell_kernel<MODE, K, LEAN><<<grid, warps * 32, smem, s>>>(cp);
    note_launch();
    return cudaGetLastError();
}

template <int MODE, int K, bool LEAN>
cudaError_t launch_batch_one(const BatchParams &bp, int sms, cudaStream_t s) {
    const int warps = 4;
    const size_t off_bytes = ((size_t)bp.noffsets * sizeof(int) + 15) & ~(size_t)15;
    const size_t cp_slot = (sizeof(CellParams) + 15) & ~(size_t)15;
    const size_t smem = off_bytes + warps * (cp_slot + sizeof(WarpShared<MODE, K>));
    cudaError_t e =
        cudaFuncSetAttribute(cell_batch_kernel<MODE, K, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cell_batch_kernel<MODE, K, LEAN>, warps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sms * per_sm;
    const long long need = (bp.ncells + warps - 1) / warps;
    int grid = (int)(want < need ? want : need);
    if (grid < 1) grid = 1;
    cell_batch_kernel<MODE, K, LEAN><<<grid, warps * 32, smem, s>>>(bp);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

}  // namespace vgpu
