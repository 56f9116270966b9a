// The finish kernel: volume, centroid, neighbours and the optional polytope
// of every cell from the records the clipping kernels write.
#include "vgpu_dev.cuh"

namespace vgpu {

namespace {

// ------------------------------------------------------------------ finish
// The reductions of every cell from the compact record its clipping kernel
// wrote (layout in CellParams).  They run as a separate kernel so that the
// clipping loop keeps the instruction cache to itself.  Planes are rebuilt
// in FP64 from the particles (the reference's arithmetic).  Vertices: the
// FP64 engine's are used as they are; the MIXED engine's FP32 vertices get
// one residual correction against their three planes (refine_vertex_ff).
// Volume and centroid: sums over edges relative to vertex 0 with each face's
// reference point one of its own vertices (the edge formula holds for any
// point of the face), in FP64 for the FP64 engine and in float pairs for the
// MIXED engine.  Optionally the polytope itself is written out.
constexpr int kFinMaxV = 128;   // vertices (the 128-slot engine's capacity)

// One cell's shared arrays for cells of at most NV vertices (a whole warp:
// 128; a 16-lane half: 64).  Planes (the record's, numbered compactly): 128
// for a whole warp, as the 128-vertex engines allow; 64 for a half, whose
// cell of at most 64 vertices has at most 34 faces.  (The two halves' space
// is the larger: the whole warp's extra planes cost no shared memory.)
template <int NV>
struct FinishShared {
    static constexpr int kNV = NV;
    static constexpr int kNP = NV >= 128 ? kMaxPlanesWide : kMaxPlanes;
    unsigned tri[NV];
    unsigned adj[NV];
    int psrc[kNP], pshift[kNP];
    int rep[kNP];             // per face: its lowest vertex
    int ford[kNP];            // per face: its vertex count
    float4 plh[kNP], pll[kNP];   // the FP64 planes as float pairs (MIXED engine)
    // vertices relative to c0: FP64 (FP64 engine) or scaled float pairs
    // (MIXED engine: vh + vl, see the edge sums)
    union {
        struct {
            double vx[NV], vy[NV], vz[NV];
        } d;
        struct {
            float vh[3][NV], vl[3][NV];
        } f;
    } v;
    unsigned stage[3 * NV / 2];      // owned edges (t < u)
};

// A warp's shared arrays: one cell of up to 128 vertices, or two of up to 64
// (one per 16-lane half) in the same space.
union FinishWarp {
    FinishShared<128> whole;
    FinishShared<64> half[2];
};

// ------------------------------------------------------------------ float-pair arithmetic
// A value is the unevaluated sum h + l of two floats (|l| <= ulp(h)/2): about
// 48 significant bits.  GB300 issues FP32 at 64 times its FP64 rate, so the
// MIXED engine's vertex corrections and edge sums run on pairs: Knuth's
// two-sum and the FMA two-product (exact error terms; every operation is an
// explicitly rounded intrinsic that the compiler may neither contract nor
// reorder).  Addition and multiplication have relative errors of a few
// 2^-46 (of |a| + |b| for a sum), so the sums keep about 1e-13 of the cell's
// scale: far inside the 1e-10 tolerance of the MIXED engine.
struct FF {
    float h, l;
};
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {   // |a| >= |b| or a = 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float v = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const FF s = ff_two_sum(a.h, b.h);
    return ff_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.h, -a.l}; }
__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ FF ff_mulf(FF a, float b) {   // pair times float
    const float p = __fmul_rn(a.h, b);
    return ff_fast_two_sum(p, __fmaf_rn(a.l, b, __fmaf_rn(a.h, b, -p)));
}
__device__ __forceinline__ FF ff_scale(FF a, float pow2) { return {__fmul_rn(a.h, pow2), __fmul_rn(a.l, pow2)}; }
__device__ __forceinline__ bool ff_less(FF a, FF b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.h + (double)a.l; }
// a / b: the float quotient, corrected by the pair remainder (long division)
__device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q1 = __fdiv_rn(a.h, b.h);
    const FF r = ff_sub(a, ff_mulf(b, q1));
    return ff_fast_two_sum(q1, __fdiv_rn(r.h, b.h));
}
__device__ __forceinline__ FF ff_shfl_xor(FF a, int d, int w) {
    return {__shfl_xor_sync(kFull, a.h, d, w), __shfl_xor_sync(kFull, a.l, d, w)};
}
__device__ __forceinline__ FF ff_shfl(FF a, int src, int w) {
    return {__shfl_sync(kFull, a.h, src, w), __shfl_sync(kFull, a.l, src, w)};
}
__device__ __forceinline__ FF ff_from_double(double d) {
    const float h = __double2float_rn(d);
    return {h, __double2float_rn(d - (double)h)};
}
// 2^k as a float (|k| <= 126) and as a double (|k| <= 1022): exact
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }
__device__ __forceinline__ double pow2d(int k) { return __hiloint2double((1023 + k) << 20, 0); }

template <class FS>
__device__ __forceinline__ double4 plane64_rec(const CellParams &P, const FS &F, double4 me, int p) {
    const int src = F.psrc[p];
    if (src >= 0) return plane64_from(P, me, src, F.pshift[p]);
    return initial64(P, me, F.pshift[p]);
}

// The plane of candidate j (image code) of the cell of particle k as float
// pairs, without FP64 arithmetic: the difference of the two particles is
// their engine-block offset times the block size plus the difference of
// their block-local positions (both stored as float pairs by the binning),
// h = |d|^2 / 2 [+ (r_k^2 - r_j^2) / 2].  Its error is a few 2^-46 of the
// cell's scale, against the reference's own rounding of p_j - p_k.
struct PlaneFF {
    FF x, y, z, w;
};
__device__ __forceinline__ PlaneFF plane_ff(const CellParams &P, int bk[3], float4 mh, float4 ml, int j, int code) {
    const int b = P.a.gblock[j];
    const int bj[3] = {b % P.g.gn[0], (b / P.g.gn[0]) % P.g.gn[1], b / (P.g.gn[0] * P.g.gn[1])};
    const float4 qh = P.a.lffh[j], ql = P.a.lffl[j];
    const float lq[3] = {qh.x, qh.y, qh.z}, lqe[3] = {ql.x, ql.y, ql.z};
    const float lm[3] = {mh.x, mh.y, mh.z}, lme[3] = {ml.x, ml.y, ml.z};
    FF d[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int db = bj[a] - bk[a] + unpack_shift(code, a) * P.g.gn[a];
        d[a] = ff_add(ff_mulf({P.g.gbs_h[a], P.g.gbs_l[a]}, (float)db), ff_sub({lq[a], lqe[a]}, {lm[a], lme[a]}));
    }
    FF rs = ff_add(ff_add(ff_mul(d[0], d[0]), ff_mul(d[1], d[1])), ff_mul(d[2], d[2]));
    if (P.g.poly) rs = ff_add(rs, ff_sub(ff_mul({mh.w, ml.w}, {mh.w, ml.w}), ff_mul({qh.w, ql.w}, {qh.w, ql.w})));
    return {d[0], d[1], d[2], ff_scale(rs, 0.5f)};
}

// The FP32 vertex (fx, fy, fz) of planes t corrected by residual steps:
// residuals r = h - n.v against the planes' float pairs (pair products and
// sums), the correction A^-1 r solved in FP32 with the planes' FP32 normals,
// and the vertex returned as the pair v + correction.  Each step multiplies
// the vertex's error by about kappa u (kappa = |A| |A^-1|, u = 2^-24), and the
// FP32 vertex starts with an error of about kappa u |v|, so one step leaves
// (kappa u)^2 |v|: enough for kappa up to about 1 / kOneStepDet (the volume
// then agrees with the FP64 engine's to ~1e-12); up to 1 / kFp64Det a second
// step starts from the pair vertex.  A nearly singular FP32 system (|D| <=
// kFp64Det of the product of the normals' norms), or force64, is solved in
// FP64 from the FP64 planes instead, rebuilt for it.  (With one step up to
// kappa = 1000 a cell of the 2M radical box differed from the FP64 engine by
// 6.5e-9.)
constexpr float kFp64Det = 1e-3f;
constexpr float kOneStepDet = 3e-2f;
// cells smaller than this fraction of R^3 (R: largest vertex distance from
// the particle) get FP64 vertices (finish_record)
constexpr double kTinyRel = 1e-4;
template <class FS>
__device__ __forceinline__ void refine_vertex_ff(const CellParams &P, const FS &F, double4 me, unsigned t,
                                                 float fx, float fy, float fz, bool force64, FF &vx, FF &vy, FF &vz) {
    const int ia = tri_plane(t, 0), ib = tri_plane(t, 1), ic = tri_plane(t, 2);
    const float4 a = F.plh[ia], b = F.plh[ib], c = F.plh[ic];
    const float bcx = b.y * c.z - b.z * c.y, bcy = b.z * c.x - b.x * c.z, bcz = b.x * c.y - b.y * c.x;
    const float cax = c.y * a.z - c.z * a.y, cay = c.z * a.x - c.x * a.z, caz = c.x * a.y - c.y * a.x;
    const float abx = a.y * b.z - a.z * b.y, aby = a.z * b.x - a.x * b.z, abz = a.x * b.y - a.y * b.x;
    const float D = a.x * bcx + a.y * bcy + a.z * bcz;
    const float scale = (fabsf(a.x) + fabsf(a.y) + fabsf(a.z)) * (fabsf(b.x) + fabsf(b.y) + fabsf(b.z)) *
                        (fabsf(c.x) + fabsf(c.y) + fabsf(c.z));
    if (!force64 && fabsf(D) > kFp64Det * scale) {
        float r[3];
        const int ip[3] = {ia, ib, ic};
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const float4 h = F.plh[ip[q]], l = F.pll[ip[q]];
            FF acc = ff_mulf({h.x, l.x}, fx);
            acc = ff_add(acc, ff_mulf({h.y, l.y}, fy));
            acc = ff_add(acc, ff_mulf({h.z, l.z}, fz));
            r[q] = ff_sub({h.w, l.w}, acc).h;
        }
        const float inv = 1.0f / D;
        vx = ff_two_sum(fx, (r[0] * bcx + r[1] * cax + r[2] * abx) * inv);
        vy = ff_two_sum(fy, (r[0] * bcy + r[1] * cay + r[2] * aby) * inv);
        vz = ff_two_sum(fz, (r[0] * bcz + r[1] * caz + r[2] * abz) * inv);
        if (fabsf(D) <= kOneStepDet * scale) {   // a second step from the pair vertex
#pragma unroll
            for (int q = 0; q < 3; q++) {
                const float4 h = F.plh[ip[q]], l = F.pll[ip[q]];
                FF acc = ff_mul({h.x, l.x}, vx);
                acc = ff_add(acc, ff_mul({h.y, l.y}, vy));
                acc = ff_add(acc, ff_mul({h.z, l.z}, vz));
                r[q] = ff_sub({h.w, l.w}, acc).h;
            }
            vx = ff_add(vx, {(r[0] * bcx + r[1] * cax + r[2] * abx) * inv, 0.0f});
            vy = ff_add(vy, {(r[0] * bcy + r[1] * cay + r[2] * aby) * inv, 0.0f});
            vz = ff_add(vz, {(r[0] * bcz + r[1] * caz + r[2] * abz) * inv, 0.0f});
        }
    } else {
        double x, y, z, DD;
        float kn;
        solve_f64(plane64_rec(P, F, me, ia), plane64_rec(P, F, me, ib), plane64_rec(P, F, me, ic), x, y, z, DD, kn);
        vx = ff_from_double(x);
        vy = ff_from_double(y);
        vz = ff_from_double(z);
    }
}

template <int G>
__device__ __forceinline__ void group_sum4(double &a, double &b, double &c, double &d, int gl) {
    const bool lo = gl < G / 2;
    double k0 = lo ? a : c, k1 = lo ? b : d;
    const double s0 = lo ? c : a, s1 = lo ? d : b;
    k0 += __shfl_xor_sync(kFull, s0, G / 2, G);
    k1 += __shfl_xor_sync(kFull, s1, G / 2, G);
    const bool lo4 = (gl & (G / 4)) == 0;
    double k = lo4 ? k0 : k1;
    k += __shfl_xor_sync(kFull, lo4 ? k1 : k0, G / 4, G);
#pragma unroll
    for (int dd = G / 8; dd >= 1; dd >>= 1) k += __shfl_xor_sync(kFull, k, dd, G);
    a = __shfl_sync(kFull, k, 0, G);
    b = __shfl_sync(kFull, k, G / 4, G);
    c = __shfl_sync(kFull, k, G / 2, G);
    d = __shfl_sync(kFull, k, 3 * G / 4, G);
}

// Maximum of non-negative doubles over a group of G lanes by their bit
// patterns (ordered like the values), on integer units instead of the FP64 pipe.
// group_sum4 on float pairs (the same transposed folding, FP32 pipe only)
template <int G>
__device__ __forceinline__ void group_sum4_ff(FF &a, FF &b, FF &c, FF &d, int gl) {
    const bool lo = gl < G / 2;
    FF k0 = lo ? a : c, k1 = lo ? b : d;
    const FF s0 = lo ? c : a, s1 = lo ? d : b;
    k0 = ff_add(k0, ff_shfl_xor(s0, G / 2, G));
    k1 = ff_add(k1, ff_shfl_xor(s1, G / 2, G));
    const bool lo4 = (gl & (G / 4)) == 0;
    FF k = lo4 ? k0 : k1;
    k = ff_add(k, ff_shfl_xor(lo4 ? k1 : k0, G / 4, G));
#pragma unroll
    for (int dd = G / 8; dd >= 1; dd >>= 1) k = ff_add(k, ff_shfl_xor(k, dd, G));
    a = ff_shfl(k, 0, G);
    b = ff_shfl(k, G / 4, G);
    c = ff_shfl(k, G / 2, G);
    d = ff_shfl(k, 3 * G / 4, G);
}

template <int G>
__device__ __forceinline__ double group_max_nonneg(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
#pragma unroll
    for (int dd = G / 2; dd >= 1; dd >>= 1) {
        const unsigned long long o = __shfl_xor_sync(kFull, b, dd, G);
        b = o > b ? o : b;
    }
    return __longlong_as_double((long long)b);
}

template <int G>
__device__ __forceinline__ int group_incl_scan(int x, int gl) {
#pragma unroll
    for (int dd = 1; dd < G; dd <<= 1) {
        const int y = __shfl_up_sync(kFull, x, dd, G);
        if (gl >= dd) x += y;
    }
    return x;
}

__device__ __forceinline__ double rec_double(const unsigned *w) {
    return __longlong_as_double((long long)((unsigned long long)w[0] | ((unsigned long long)w[1] << 32)));
}

// The reductions of cell k (engine order, k < 0: none) from its record, if it
// has one, by a group of G lanes: G = 32 for any cell, G = 16 (two cells per
// warp, one per half) for cells of at most 64 vertices.  Every collective is
// reached by both halves of the warp whatever their cells.
template <int MODE, int G>
__device__ __forceinline__ void finish_record(const CellParams &P, FinishShared<4 * G> &F, int k, int gl) {
    constexpr bool kFF = MODE == VGPU_MIXED;   // float-pair vertices and sums
    constexpr int VW = kFF ? 3 : 6;
    constexpr int SL = 4;   // vertex slots per lane: 128 vertices (G = 32) or 64 (G = 16)
    static_assert(SL * 32 == kFinMaxV, "slot count");
    const unsigned long long off = k >= 0 ? P.rec_off[k] : kNoRecord;
    const bool have = off != kNoRecord;
    const unsigned *R = P.rec + (have ? off : 0);
    const int nv = have ? (int)R[0] : 0, nf = have ? (int)R[1] : 0;
    const unsigned fl = have ? R[2] : 0u;
    const unsigned *rv = R + kRecHeader;
    const unsigned *rp = rv + (2 + VW) * nv;
    const double4 me = have ? P.a.p64[k] : make_double4(0, 0, 0, 0);
    const int out = have ? P.a.outpos[k] : 0;
    int bk[3] = {0, 0, 0};
    float4 mh = make_float4(0, 0, 0, 0), ml = mh;
    if (kFF && have) {
        const int b = P.a.gblock[k];
        bk[0] = b % P.g.gn[0];
        bk[1] = (b / P.g.gn[0]) % P.g.gn[1];
        bk[2] = b / (P.g.gn[0] * P.g.gn[1]);
        mh = P.a.lffh[k];
        ml = P.a.lffl[k];
    }
    // neighbour IDs: the cell's row of kNbStride, or with more faces its
    // first kNbStride-1 there and the rest in the overflow store
    int *row = P.r.nb + (size_t)out * kNbStride;
    long long ovf = 0;
    if (have && nf > kNbStride && gl == 0) {
        const unsigned long long need = (unsigned long long)(nf - (kNbStride - 1));
        const unsigned long long o = atomicAdd(&P.cnt->nb_ovf_used, need);
        ovf = o + need <= P.r.nb_ovf_cap ? (long long)o : -1;
        if (ovf >= 0) row[kNbStride - 1] = (int)ovf;
    }
    ovf = __shfl_sync(kFull, ovf, 0, G);
    const bool nb_full = ovf < 0;
    // planes: neighbour IDs (plane order), sources, planes as float pairs
    for (int q = gl; q < nf; q += G) {
        F.psrc[q] = (int)rp[q];
        F.pshift[q] = (int)rp[nf + q];
        F.rep[q] = 0x7fffffff;
        F.ford[q] = 0;
        const int id = (int)rp[2 * nf + q];
        if (nf <= kNbStride || q < kNbStride - 1) row[q] = id;
        else if (!nb_full) P.r.nb_ovf[ovf + q - (kNbStride - 1)] = id;
        if (kFF) {   // (the FP64 engine's vertices need no planes)
            PlaneFF pl;
            if (F.psrc[q] >= 0) {
                pl = plane_ff(P, bk, mh, ml, F.psrc[q], F.pshift[q]);
            } else {   // a wall of the container (FP64, rare)
                const double4 w = initial64(P, me, F.pshift[q]);
                pl = {ff_from_double(w.x), ff_from_double(w.y), ff_from_double(w.z), ff_from_double(w.w)};
            }
            F.plh[q] = make_float4(pl.x.h, pl.y.h, pl.z.h, pl.w.h);
            F.pll[q] = make_float4(pl.x.l, pl.y.l, pl.z.l, pl.w.l);
        }
    }
    __syncwarp();
    // vertices (particle-relative): FP64 (vd) or float pairs (vf).  Float-pair
    // vertices are within about 2^-46 of their distance from the particle,
    // which is far inside the tolerance for every cell but a tiny one far
    // from its particle (a radical cell squeezed between large neighbours:
    // volume 1e-11 at distance 2 in the 2M radical box, where it made a
    // relative error of 4e-10).  A cell whose volume is below kTinyRel of
    // the cube of its largest vertex distance is therefore done again with
    // every vertex solved in FP64 from the FP64 planes (force64): both halves
    // of the warp run a second pass when either needs it, the other half
    // repeating its float-pair one.  A cell that met
    // the tolerance band (marginal) gets FP64 vertices from the start: its
    // coincident vertices are merged below by their distance.
    unsigned tri[SL];
    double vd[SL][3];
    FF vf[SL][3];
    double mr2 = 0.0;
    FF mf = {0.0f, 0.0f};
    int sc = 0;
    double c0[3];
    FF c0f[3];
    double vol_out = 0.0, cen_out[3] = {0.0, 0.0, 0.0};
    const bool marg = have && (fl & VGPU_CELL_MARGINAL) != 0u;
    bool redo64 = false;   // this group's cell is tiny: its second pass is in FP64
    for (int pass = 0;; pass++) {
        const bool force64 = redo64 || marg;
        mr2 = 0.0;
        mf = {0.0f, 0.0f};
    #pragma unroll
        for (int s = 0; s < SL; s++) {
            const int t = gl + G * s;
            tri[s] = 0;
    #pragma unroll
            for (int a = 0; a < 3; a++) {
                vd[s][a] = 0.0;
                vf[s][a] = {0.0f, 0.0f};
            }
            if (t < nv) {
                tri[s] = rv[t];
                F.tri[t] = tri[s];
                F.adj[t] = rv[nv + t];
                if (kFF) {
                    refine_vertex_ff(P, F, me, tri[s], __uint_as_float(rv[2 * nv + t]), __uint_as_float(rv[3 * nv + t]),
                                     __uint_as_float(rv[4 * nv + t]), force64, vf[s][0], vf[s][1], vf[s][2]);
                    const FF q = ff_add(ff_add(ff_mul(vf[s][0], vf[s][0]), ff_mul(vf[s][1], vf[s][1])),
                                        ff_mul(vf[s][2], vf[s][2]));
                    if (ff_less(mf, q)) mf = q;
                } else {
    #pragma unroll
                    for (int a = 0; a < 3; a++) vd[s][a] = rec_double(rv + (2 + 2 * a) * nv + 2 * t);
                    mr2 = fmax(mr2, vd[s][0] * vd[s][0] + vd[s][1] * vd[s][1] + vd[s][2] * vd[s][2]);
                }
                if (pass == 0)
    #pragma unroll
                    for (int e = 0; e < 3; e++) {
                        atomicMin(&F.rep[tri_plane(tri[s], e)], t);
                        atomicAdd(&F.ford[tri_plane(tri[s], e)], 1);
                    }
            }
        }
        // the largest |v|^2 over the group and, for the pairs, the power of two
        // 2^sc (about 2 sqrt(max |v|^2) >= |v - c0|) that scales the relative
        // coordinates to magnitude about 1, so that their products neither
        // underflow nor overflow
        sc = 0;
        if (kFF) {
    #pragma unroll
            for (int dd = G / 2; dd >= 1; dd >>= 1) {
                const FF o = {__shfl_xor_sync(kFull, mf.h, dd, G), __shfl_xor_sync(kFull, mf.l, dd, G)};
                if (ff_less(mf, o)) mf = o;
            }
            if (mf.h > 0.0f && mf.h < 3.0e38f) sc = (ilogbf(mf.h) + 2) / 2 + 1;
        } else {
            mr2 = group_max_nonneg<G>(mr2);
        }
        // origin of the sums: vertex 0
    #pragma unroll
        for (int a = 0; a < 3; a++) {
            if (kFF) {
                c0f[a] = {__shfl_sync(kFull, vf[0][a].h, 0, G), __shfl_sync(kFull, vf[0][a].l, 0, G)};
                c0[a] = ff_to_double(c0f[a]);
            } else {
                c0[a] = __shfl_sync(kFull, vd[0][a], 0, G);
            }
        }
        const float down = pow2f(-sc);
        int ne = 0;
        unsigned own[SL];
    #pragma unroll
        for (int s = 0; s < SL; s++) {
            own[s] = 0;
            const int t = gl + G * s;
            if (t < nv) {
    #pragma unroll
                for (int a = 0; a < 3; a++) {
                    if (kFF) {
                        const FF q = ff_scale(ff_sub(vf[s][a], c0f[a]), down);
                        F.v.f.vh[a][t] = q.h;
                        F.v.f.vl[a][t] = q.l;
                    } else {
                        (a == 0 ? F.v.d.vx : (a == 1 ? F.v.d.vy : F.v.d.vz))[t] = vd[s][a] - c0[a];
                    }
                }
                const unsigned A3 = F.adj[t];
    #pragma unroll
                for (int e = 0; e < 3; e++)
                    if ((int)((A3 >> (8 * e)) & 255u) > t) own[s] |= 1u << e;
                ne += __popc(own[s]);
            }
        }
        const int eincl = group_incl_scan<G>(ne, gl);
        const int etot = __shfl_sync(kFull, eincl, G - 1, G);
        {
            int q = eincl - ne;
    #pragma unroll
            for (int s = 0; s < SL; s++)
    #pragma unroll
                for (int e = 0; e < 3; e++)
                    if ((own[s] >> e) & 1u) F.stage[q++] = (unsigned)(gl + G * s) | ((unsigned)e << 8);
        }
        __syncwarp();
        // sum over edges (t,u) of (p_y - p_x).(v_t x v_u), p_f a vertex of face f
        double vs = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
        if (kFF) {
            FF s0 = {0.0f, 0.0f}, s1 = s0, s2 = s0, s3 = s0;
            for (int i = gl; i < etot; i += G) {
                const unsigned E = F.stage[i];
                const int t = E & 255u, e = E >> 8;
                const unsigned T = F.tri[t];
                const int u = (F.adj[t] >> (8 * e)) & 255u;
                const int rx = F.rep[tri_plane(T, e)], ry = F.rep[tri_plane(T, e == 2 ? 0 : e + 1)];
                FF tv[3], uv[3], av[3], bv[3];
    #pragma unroll
                for (int c = 0; c < 3; c++) {
                    tv[c] = {F.v.f.vh[c][t], F.v.f.vl[c][t]};
                    uv[c] = {F.v.f.vh[c][u], F.v.f.vl[c][u]};
                    av[c] = {F.v.f.vh[c][rx], F.v.f.vl[c][rx]};
                    bv[c] = {F.v.f.vh[c][ry], F.v.f.vl[c][ry]};
                }
                const FF w[3] = {ff_sub(ff_mul(tv[1], uv[2]), ff_mul(tv[2], uv[1])),
                                 ff_sub(ff_mul(tv[2], uv[0]), ff_mul(tv[0], uv[2])),
                                 ff_sub(ff_mul(tv[0], uv[1]), ff_mul(tv[1], uv[0]))};
                const FF dy = ff_add(ff_add(ff_mul(bv[0], w[0]), ff_mul(bv[1], w[1])), ff_mul(bv[2], w[2]));
                const FF dx = ff_add(ff_add(ff_mul(av[0], w[0]), ff_mul(av[1], w[1])), ff_mul(av[2], w[2]));
                const FF dd = ff_sub(dy, dx);
                s0 = ff_add(s0, dd);
                s1 = ff_add(s1, ff_sub(ff_add(ff_mul(dd, ff_add(tv[0], uv[0])), ff_mul(dy, bv[0])), ff_mul(dx, av[0])));
                s2 = ff_add(s2, ff_sub(ff_add(ff_mul(dd, ff_add(tv[1], uv[1])), ff_mul(dy, bv[1])), ff_mul(dx, av[1])));
                s3 = ff_add(s3, ff_sub(ff_add(ff_mul(dd, ff_add(tv[2], uv[2])), ff_mul(dy, bv[2])), ff_mul(dx, av[2])));
            }
            // the group's sums, then the outputs from pairs with few FP64
            // operations: vol = s0 / 6 * 2^(3 sc); centroid = c0 + 2^sc C / (4 s0)
            group_sum4_ff<G>(s0, s1, s2, s3, gl);
            if (have && gl == 0) {
                constexpr float kSixthH = (float)(1.0 / 6.0);
                constexpr float kSixthL = (float)(1.0 / 6.0 - (double)(float)(1.0 / 6.0));
                vol_out = ff_to_double(ff_mul(s0, {kSixthH, kSixthL})) * pow2d(3 * sc);
                if (48.0 * vol_out > P.g.tol_cu) {   // src/cell.cc:1895
                    const FF inv = ff_div({1.0f, 0.0f}, ff_scale(s0, 4.0f));
                    const float up = pow2f(sc);
                    const FF sc3[3] = {s1, s2, s3};
    #pragma unroll
                    for (int a = 0; a < 3; a++) cen_out[a] = ff_to_double(ff_add(c0f[a], ff_scale(ff_mul(sc3[a], inv), up)));
                } else {
                    cen_out[0] = cen_out[1] = cen_out[2] = 0.0;
                }
            }
        } else {
            for (int i = gl; i < etot; i += G) {
                const unsigned E = F.stage[i];
                const int t = E & 255u, e = E >> 8;
                const unsigned T = F.tri[t];
                const int u = (F.adj[t] >> (8 * e)) & 255u;
                const int rx = F.rep[tri_plane(T, e)], ry = F.rep[tri_plane(T, e == 2 ? 0 : e + 1)];
                const double tx = F.v.d.vx[t], ty = F.v.d.vy[t], tz = F.v.d.vz[t];
                const double ux = F.v.d.vx[u], uy = F.v.d.vy[u], uz = F.v.d.vz[u];
                const double wx = ty * uz - tz * uy;
                const double wy = tz * ux - tx * uz;
                const double wz = tx * uy - ty * ux;
                const double ax = F.v.d.vx[rx], ay = F.v.d.vy[rx], az = F.v.d.vz[rx];
                const double bx = F.v.d.vx[ry], by = F.v.d.vy[ry], bz = F.v.d.vz[ry];
                const double dy = bx * wx + by * wy + bz * wz;
                const double dx = ax * wx + ay * wy + az * wz;
                const double dd = dy - dx;
                vs += dd;
                cx += dd * (tx + ux) + dy * bx - dx * ax;
                cy += dd * (ty + uy) + dy * by - dx * ay;
                cz += dd * (tz + uz) + dy * bz - dx * az;
            }
            group_sum4<G>(vs, cx, cy, cz, gl);
            if (have && gl == 0) {
                vol_out = vs / 6.0;
                if (48.0 * vol_out > P.g.tol_cu) {   // src/cell.cc:1895
                    const double f = 1.0 / (4.0 * vs);
                    cen_out[0] = c0[0] + cx * f;
                    cen_out[1] = c0[1] + cy * f;
                    cen_out[2] = c0[2] + cz * f;
                } else {
                    cen_out[0] = cen_out[1] = cen_out[2] = 0.0;
                }
            }
        }
        const double r2 = kFF ? ff_to_double(mf) : mr2;
        const bool tiny = kFF && !force64 && have && gl == 0 && vol_out < kTinyRel * r2 * sqrt(r2);
        if (!__any_sync(kFull, tiny)) break;
        // the other half of the warp repeats its own pass unchanged, so a
        // cell's result never depends on the cell that shares its warp
        redo64 = __shfl_sync(kFull, tiny, 0, G);
        __syncwarp();
    }
    if (have && gl == 0) {
        P.r.vol[out] = vol_out;
#pragma unroll
        for (int a = 0; a < 3; a++) P.r.cen[3 * out + a] = cen_out[a];
    }
    // Coincident vertices.  Where a cut plane passes through an existing
    // vertex within the reference's tolerance band, the reference makes that
    // vertex a vertex of the new face, of higher order (create_facet and the
    // marginal-vertex handling of nplane, src/cell.cc:1166-1355), while the
    // engine keeps every vertex of order 3: its cut leaves new vertices at
    // the same point, joined to the old one by edges of zero length.  Only a
    // cell that met the band (VGPU_CELL_MARGINAL) can hold such edges; there
    // every edge shorter than the band's width as a distance, tol / 2 over
    // the cell's largest vertex distance R (a plane of the cell is at most 2R
    // from the particle, and its band is tol_h / |d| wide, |d| <= 2R), is
    // contracted (label propagation over the contracted edges): two vertices
    // that close lie within the reference's band of each other's planes, so
    // nothing the reference keeps apart is merged.  This gives the
    // reference's vertex count and, in the polytope, its vertices of higher
    // order; a face that the merge reduces to an edge or a point (a plane that
    // touched the cell only there) is no face of the reference's cell and is
    // dropped.  Both halves of a warp run this when either needs it (it holds
    // collectives).  lab[t]: after the propagation, the lowest vertex of t's
    // class; then a class's lowest vertex holds -(1 + its rank).
    int nvm = nv, nfm = nf;
    const bool any_marg = __any_sync(kFull, marg);
    int *lab = reinterpret_cast<int *>(F.stage);   // (free once the sums are done)
    if (any_marg) {
        __syncwarp();
        unsigned zero[SL];
        const double r2 = kFF ? ff_to_double(mf) : mr2;
        // contraction length squared in the units of the staged coordinates
        // (float pairs: scaled by 2^-sc)
        const double eps = P.g.tol_h / (2.0 * sqrt(r2));
        const double eps2 = eps * eps * (kFF ? (double)pow2f(-2 * sc) : 1.0);
#pragma unroll
        for (int s = 0; s < SL; s++) {
            const int t = gl + G * s;
            zero[s] = 0;
            if (t < nv) {
                lab[t] = t;
                if (marg) {
                    const unsigned A3 = F.adj[t];
#pragma unroll
                    for (int e = 0; e < 3; e++) {
                        const int u = (A3 >> (8 * e)) & 255u;
                        if (u <= t || u >= nv) continue;
                        double d2 = 0.0;
#pragma unroll
                        for (int a = 0; a < 3; a++) {
                            double d;
                            if (kFF) d = ((double)F.v.f.vh[a][t] - (double)F.v.f.vh[a][u]) +
                                         ((double)F.v.f.vl[a][t] - (double)F.v.f.vl[a][u]);
                            else d = (a == 0 ? F.v.d.vx : (a == 1 ? F.v.d.vy : F.v.d.vz))[t] -
                                     (a == 0 ? F.v.d.vx : (a == 1 ? F.v.d.vy : F.v.d.vz))[u];
                            d2 += d * d;
                        }
                        if (d2 <= eps2) zero[s] |= 1u << e;
                    }
                }
            }
        }
        __syncwarp();
        // propagate the smallest label along contracted edges (classes hold a
        // few vertices: a vertex of order k splits into k - 2)
        for (int it = 0; it < 4 * kFinMaxV; it++) {
            bool changed = false;
#pragma unroll
            for (int s = 0; s < SL; s++) {
                const int t = gl + G * s;
#pragma unroll
                for (int e = 0; e < 3; e++) {
                    if (!((zero[s] >> e) & 1u)) continue;
                    const int u = (F.adj[t] >> (8 * e)) & 255u;
                    const int a = lab[t], b = lab[u];
                    if (a < b) {
                        atomicMin(&lab[u], a);
                        changed = true;
                    } else if (b < a) {
                        atomicMin(&lab[t], b);
                        changed = true;
                    }
                }
            }
            __syncwarp();
            if (!__any_sync(kFull, changed)) break;
        }
        // the classes' lowest vertices, ranked in vertex order
        const int lane = threadIdx.x & 31;   // (the kernels' CTAs are one-dimensional)
        const unsigned gmask = G == 32 ? kFull : (0xffffu << (lane & 16));
        const unsigned below = (1u << lane) - 1u;
        int before = 0;
        int rank[SL];
#pragma unroll
        for (int s = 0; s < SL; s++) {
            const int t = gl + G * s;
            const bool rep = t < nv && lab[t] == t;
            const unsigned b = __ballot_sync(kFull, rep) & gmask;
            rank[s] = before + __popc(b & below);
            before += __popc(b);
        }
        nvm = before;
        __syncwarp();
#pragma unroll
        for (int s = 0; s < SL; s++) {
            const int t = gl + G * s;
            if (t < nv && lab[t] == t) lab[t] = -1 - rank[s];
        }
        __syncwarp();
        // each face's loop without repeats of a merged vertex (consecutive
        // equal indices, and the last equal to the first): its new order
        for (int q = gl; q < nf; q += G) {
            if (!marg) continue;
            int t = F.rep[q], cnt = 0, first = -1, last = -1;
            for (int j = 0; j < F.ford[q]; j++) {
                const int l = lab[t];
                const int o = l < 0 ? -1 - l : -1 - lab[l];
                if (o != last) {
                    cnt++;
                    if (first < 0) first = o;
                    last = o;
                }
                const unsigned T = F.tri[t];
                const int e = tri_plane(T, 0) == q ? 0 : (tri_plane(T, 1) == q ? 1 : 2);
                t = (F.adj[t] >> (8 * e)) & 255u;
            }
            if (cnt > 1 && last == first) cnt--;
            F.ford[q] = cnt;
        }
        __syncwarp();
        // the neighbour IDs of the faces that remain, compacted (rare: one lane)
        if (marg && gl == 0 && !nb_full) {
            nfm = 0;
            for (int q = 0; q < nf; q++) nfm += F.ford[q] >= 3 ? 1 : 0;
            if (nfm < nf) {
                for (int q = 0, j = 0; q < nf; q++) {
                    if (F.ford[q] < 3) continue;
                    const int id = (int)rp[2 * nf + q];
                    if (nfm <= kNbStride || j < kNbStride - 1) row[j] = id;
                    else P.r.nb_ovf[ovf + j - (kNbStride - 1)] = id;
                    j++;
                }
            }
        }
        nfm = __shfl_sync(kFull, nfm, 0, G);
        __syncwarp();
    }
    // vertex t's index in the output (its class's rank where merged)
    auto vmap = [&](int t) -> int {
        if (!any_marg) return t;
        const int l = lab[t];
        return l < 0 ? -1 - l : -1 - lab[l];
    };
    if (have && gl == 0) {
        P.r.nf[out] = nb_full ? 0 : nfm;
        P.r.nv[out] = nvm;
        P.r.maxr2[out] = kFF ? ff_to_double(mf) : mr2;
        P.r.flags[out] = nb_full ? (VGPU_CELL_FAILED | (VGPU_FAIL_RECORDS << 8)) : (VGPU_CELL_OK | (int)fl);
        if (nb_full) atomicAdd(&P.cnt->nb_failed, 1ull);
    }
    if (P.poly != nullptr) {   // (uniform: P is the same for both halves of a warp)
        // the polytope: [nv, nf, vertices (3 nv, particle-relative), then per
        // face (plane order): neighbour ID, vertex count, vertex loop]; each
        // loop walks the face by the edges that start on it, which orders the
        // vertices clockwise seen from outside, as the reference's
        // face_vertices does (src/cell.cc:2285-2308)
        // (an upper bound where vertices were merged: the stream is then shorter)
        const unsigned long long need = 2ull + 6ull * (unsigned long long)nv + 2ull * (unsigned long long)nf;
        unsigned long long po = 0;
        if (have && gl == 0) po = atomicAdd(P.poly_used, need);
        po = __shfl_sync(kFull, po, 0, G);
        const bool fits = have && po + need <= P.poly_cap;
        double *D = P.poly + (fits ? po : 0);
        if (fits) {
            if (gl == 0) {
                D[0] = (double)nvm;
                D[1] = (double)nfm;
            }
#pragma unroll
            for (int s = 0; s < SL; s++) {
                const int t = gl + G * s;
                if (t < nv && (!any_marg || lab[t] < 0)) {   // a merged class: its lowest vertex
                    const int o = vmap(t);
#pragma unroll
                    for (int a = 0; a < 3; a++) D[2 + 3 * o + a] = kFF ? ff_to_double(vf[s][a]) : vd[s][a];
                }
            }
        }
        // face loops; the loop over face chunks runs the same number of times
        // in both halves, because it holds a group scan.  A merged cell
        // (marg: its faces' orders are the merged ones, F.ford) is written by
        // one lane below instead, skipping the faces the merge removed.
        double *DF = D + 2 + 3 * nvm;
        const int nfmax = __reduce_max_sync(kFull, fits ? nf : 0);
        for (int q0 = 0; q0 < nfmax; q0 += G) {
            const int q = q0 + gl;
            const bool mine = fits && !marg && q < nf;
            const int ord = mine ? F.ford[q] : 0;
            // faces before q: q * 2 header words plus their orders
            int before = 0;
            if (fits && !marg)
                for (int j = 0; j < q0 && j < nf; j++) before += F.ford[j];
            const int incl = group_incl_scan<G>(ord, gl);
            if (mine) {
                double *df = DF + 2 * q + before + (incl - ord);
                df[0] = (double)(int)rp[2 * nf + q];
                df[1] = (double)ord;
                int t = F.rep[q];
                for (int j = 0; j < ord; j++) {
                    df[2 + j] = (double)t;
                    const unsigned T = F.tri[t];
                    const int e = tri_plane(T, 0) == q ? 0 : (tri_plane(T, 1) == q ? 1 : 2);
                    t = (F.adj[t] >> (8 * e)) & 255u;
                }
            }
        }
        if (fits && marg && gl == 0) {   // merged vertices (rare): the walks of the count above
            double *df = DF;
            for (int q = 0; q < nf; q++) {
                const int ord = F.ford[q];
                if (ord < 3) continue;   // removed by the merge
                df[0] = (double)(int)rp[2 * nf + q];
                df[1] = (double)ord;
                int t = F.rep[q], w = 0, last = -1;
                for (int j = 0; w < ord && j < kFinMaxV; j++) {
                    const int o = vmap(t);
                    if (o != last) {
                        df[2 + w++] = (double)o;
                        last = o;
                    }
                    const unsigned T = F.tri[t];
                    const int e = tri_plane(T, 0) == q ? 0 : (tri_plane(T, 1) == q ? 1 : 2);
                    t = (F.adj[t] >> (8 * e)) & 255u;
                }
                df += 2 + ord;
            }
        }
        if (fits) {
            if (gl == 0) P.poly_off[out] = (long long)po;
        } else if (have && gl == 0) {
            P.poly_off[out] = -2;   // store full
        }
    }
    __syncwarp();
}

constexpr int kFinWarps = 2;   // warps per CTA (two cell slots per warp)
// CTAs kept resident per SM (the register bound of the launch).  With 22 KB
// of shared memory per CTA (a warp's two 16-lane cells share the space of
// one 128-vertex cell) registers decide.  Measured on the 4M periodic box,
// finish kernel: 6 (148 registers, so 6 CTAs resident) 14.1 ms; 7 (128
// registers, a few spilled bytes, 8 CTAs resident) 12.3 ms; 9 (96 registers,
// 468 bytes spilled, 10 CTAs resident) 15.1 ms against 12.2.  (Before the
// coincident-vertex merge and the second correction step the kernel fitted
// 124 registers: 8 CTAs, 11.0 ms.)
#ifndef VGPU_FIN_MIN_BLOCKS
#define VGPU_FIN_MIN_BLOCKS 7
#endif

// A record is checked before finish_record indexes the shared arrays by it:
// its face count within the planes held there and, for a cell that met the
// tolerance band (where a cut can leave links that do not return), every
// vertex's planes below the face count, its neighbours below the vertex
// count and its edges (links to a higher vertex) within the edge list's
// room.  A record that fails is a failed cell (VGPU_FAIL_ADJACENCY),
// written here; the caller then passes no cell (-1).  Every lane of the
// G-lane group calls it (group collectives).
template <int G>
__device__ __forceinline__ int checked_cell(const CellParams &P, int k, int gl, int lane) {
    const unsigned long long off = k >= 0 ? P.rec_off[k] : kNoRecord;
    bool bad = false;
    int owned = 0;
    if (off != kNoRecord) {
        const unsigned *R = P.rec + off;
        const int nv = (int)R[0], nf = (int)R[1];
        const unsigned *rv = R + kRecHeader;
        if (nf > FinishShared<4 * G>::kNP || nf < 0 || nv < 0) {
            bad = true;
        } else if ((R[2] & VGPU_CELL_MARGINAL) != 0u) {
            for (int t = gl; t < nv; t += G) {
                const unsigned T = rv[t], A3 = rv[nv + t];
                for (int e = 0; e < 3; e++) {
                    const int q = (int)tri_plane(T, e), u = (int)((A3 >> (8 * e)) & 255u);
                    if (q >= nf || u >= nv) bad = true;
                    owned += u > t ? 1 : 0;
                }
            }
        }
    }
    for (int dd = G / 2; dd >= 1; dd >>= 1) owned += __shfl_xor_sync(kFull, owned, dd, G);
    if (owned > 3 * (4 * G) / 2) bad = true;   // FinishShared::stage
    const unsigned gm = G == 32 ? kFull : (0xffffu << (lane & 16));
    bad = (__ballot_sync(kFull, bad) & gm) != 0u;
    if (!bad) return k;
    if (gl == 0) {
        const int o = P.a.outpos[k];
        P.r.vol[o] = 0.0;
        P.r.cen[3 * o] = P.r.cen[3 * o + 1] = P.r.cen[3 * o + 2] = 0.0;
        P.r.nf[o] = 0;
        P.r.nv[o] = 0;
        P.r.maxr2[o] = 0.0;
        P.r.flags[o] = VGPU_CELL_FAILED | (VGPU_FAIL_ADJACENCY << 8);
        atomicAdd(&P.cnt->nb_failed, 1ull);
    }
    return -1;
}

// Two cells per warp, one per 16-lane half, when both have at most 64
// vertices (nearly always: their FP64 work then fills the lanes better);
// otherwise the whole warp does one cell after the other.
template <int MODE>
__device__ __forceinline__ void finish_pair(const CellParams &P, FinishWarp &W, int k0, int k1, int lane) {
    const int half = lane >> 4, gl = lane & 15;
    const int mine = half ? k1 : k0;
    // (a record's vertices all have order 3, so a cell of at most 64
    // vertices has at most 34 faces: within a half's 64 planes)
    int nv = 0;
    if (mine >= 0) {
        const unsigned long long off = P.rec_off[mine];
        if (off != kNoRecord) nv = (int)P.rec[off];
    }
    if (!__any_sync(kFull, nv > 64)) {
        finish_record<MODE, 16>(P, W.half[half], checked_cell<16>(P, mine, gl, lane), gl);
    } else {
        finish_record<MODE, 32>(P, W.whole, checked_cell<32>(P, k0, lane, lane), lane);
        finish_record<MODE, 32>(P, W.whole, checked_cell<32>(P, k1, lane, lane), lane);
    }
}

template <int MODE>
__global__ void __launch_bounds__(32 * kFinWarps, VGPU_FIN_MIN_BLOCKS) finish_kernel(const __grid_constant__ CellParams P) {
    __shared__ FinishWarp fsh[kFinWarps];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int npairs = (P.ncells + 1) / 2;
    const int stride = gridDim.x * kFinWarps;
    // The records come from DRAM (the clipping kernels wrote gigabytes since):
    // each half-warp pulls the first 1 KB of its cell's record in the pair
    // after this one toward the L2 while this pair is finished, from the
    // offset it loaded a pair earlier (so that no prefetch waits on a load).
    // Measured on the 4M periodic box: 12.19 ms against 12.32 ms without.
    const int half = lane >> 4, gl = lane & 15;
    auto rec_of = [&](int pi) -> unsigned long long {
        const int i = 2 * pi + half;
        if (pi >= npairs || i >= P.ncells) return kNoRecord;
        return P.rec_off[P.cell_list ? P.cell_list[i] : i];
    };
    int pi = blockIdx.x * kFinWarps + wid;
    unsigned long long ahead = rec_of(pi + stride);
    for (; pi < npairs; pi += stride) {
        if (ahead != kNoRecord && gl < 8 && ahead + 32ull * gl < P.rec_cap)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(P.rec + ahead + 32ull * gl));
        const unsigned long long next = rec_of(pi + 2 * stride);
        const int i0 = 2 * pi, i1 = 2 * pi + 1;
        const int k0 = P.cell_list ? P.cell_list[i0] : i0;
        const int k1 = i1 < P.ncells ? (P.cell_list ? P.cell_list[i1] : i1) : -1;
        finish_pair<MODE>(P, fsh[wid], k0, k1, lane);
        ahead = next;
    }
}

// The same over the cells cell_begin .. cell_begin+ncells-1 of a batch
// (global numbering as cell_batch_kernel); a pair never straddles two
// containers.
template <int MODE>
__global__ void __launch_bounds__(32 * kFinWarps, VGPU_FIN_MIN_BLOCKS) finish_batch_kernel(const __grid_constant__ BatchParams B) {
    __shared__ FinishWarp fsh[kFinWarps];
    __shared__ __align__(16) unsigned char cpw[kFinWarps][(sizeof(CellParams) + 15) & ~(size_t)15];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    CellParams &P = *reinterpret_cast<CellParams *>(cpw[wid]);
    const long long nwarps = (long long)gridDim.x * kFinWarps;
    long long cbeg = 0, cend = 0;
    const long long gend = B.cell_begin + B.ncells;
    for (long long g = B.cell_begin + 2 * ((long long)blockIdx.x * kFinWarps + wid); g < gend; g += 2 * nwarps) {
        if (g < cbeg || g >= cend) {
            int lo = 0, hi = B.ncont;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (B.cell_start[mid] <= g) lo = mid;
                else hi = mid;
            }
            cbeg = B.cell_start[lo];
            cend = B.cell_start[lo + 1];
            __syncwarp();
            const unsigned *src = reinterpret_cast<const unsigned *>(B.cps + lo);
            unsigned *dst = reinterpret_cast<unsigned *>(&P);
            for (int i = lane; i < (int)(sizeof(CellParams) / 4); i += 32) dst[i] = src[i];
            __syncwarp();
        }
        // the pair (g, g+1); its second cell may belong to the next container
        // (a sheared box's cells: its particles, listed in cell_list)
        const int i0 = (int)(g - cbeg);
        const int k0 = P.cell_list ? P.cell_list[i0] : i0;
        const int k1 = g + 1 < cend && g + 1 < gend ? (P.cell_list ? P.cell_list[i0 + 1] : i0 + 1) : -1;
        finish_pair<MODE>(P, fsh[wid], k0, k1, lane);
        if (k1 < 0 && g + 1 < gend) {
            // g + 1 starts the next container: finish it with that container's parameters
            const long long g1 = g + 1;
            int lo = 0, hi = B.ncont;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (B.cell_start[mid] <= g1) lo = mid;
                else hi = mid;
            }
            cbeg = B.cell_start[lo];
            cend = B.cell_start[lo + 1];
            __syncwarp();
            const unsigned *src = reinterpret_cast<const unsigned *>(B.cps + lo);
            unsigned *dst = reinterpret_cast<unsigned *>(&P);
            for (int i = lane; i < (int)(sizeof(CellParams) / 4); i += 32) dst[i] = src[i];
            __syncwarp();
            const int j0 = (int)(g1 - cbeg);
            finish_pair<MODE>(P, fsh[wid], P.cell_list ? P.cell_list[j0] : j0, -1, lane);
        }
    }
}

}  // namespace

template <int MODE>
cudaError_t launch_finish_t(const CellParams &cp, int sms, cudaStream_t s) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, finish_kernel<MODE>, 32 * kFinWarps, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sms * per_sm;
    const long long need = ((cp.ncells + 1) / 2 + kFinWarps - 1) / kFinWarps;
    const int grid = (int)(want < need ? want : need);
    finish_kernel<MODE><<<grid, 32 * kFinWarps, 0, s>>>(cp);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_finish(const CellParams &cp, int mode, int sms, cudaStream_t s) {
    if (cp.ncells <= 0 || cp.rec == nullptr) return cudaSuccess;
    return mode == VGPU_FP64 ? launch_finish_t<VGPU_FP64>(cp, sms, s) : launch_finish_t<VGPU_MIXED>(cp, sms, s);
}

template <int MODE>
cudaError_t launch_finish_batch_t(const BatchParams &bp, int sms, cudaStream_t s) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, finish_batch_kernel<MODE>, 32 * kFinWarps, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sms * per_sm;
    const long long need = ((bp.ncells + 1) / 2 + kFinWarps - 1) / kFinWarps;
    const int grid = (int)(want < need ? want : need);
    finish_batch_kernel<MODE><<<grid, 32 * kFinWarps, 0, s>>>(bp);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_finish_batch(const BatchParams &bp, int mode, int sms, cudaStream_t s) {
    if (bp.ncells <= 0) return cudaSuccess;
    return mode == VGPU_FP64 ? launch_finish_batch_t<VGPU_FP64>(bp, sms, s)
                             : launch_finish_batch_t<VGPU_MIXED>(bp, sms, s);
}

}  // namespace vgpu
