// Device helpers shared by the engine's cell kernels.
#pragma once
#include "vgpu_internal.cuh"
#include "../../include/vorogpu.h"

namespace vgpu {

// Block offset e (0 <= e < 6 (2r+1)^2) on the surface of the cube of
// Chebyshev radius r, walked face by face (face e / (2r+1)^2: axis f >> 1,
// side f & 1) without branches.  Returns false for the copies of an edge or
// corner block: each surface block is taken once, by the face of its lowest
// axis.
__device__ __forceinline__ bool shell_offset(int e, int r, int &di, int &dj, int &dk) {
    const int A = 2 * r + 1, AA = A * A;
    const int f = e / AA, q = e - f * AA;
    const int u = q % A - r, v = q / A - r;
    const int ax = f >> 1, s = (f & 1) ? r : -r;
    di = ax == 0 ? s : u;
    dj = ax == 1 ? s : (ax == 0 ? u : v);
    dk = ax == 2 ? s : v;
    return !(ax > 0 && abs(di) == r) && !(ax > 1 && abs(dj) == r);
}


static constexpr float kU32 = 5.9604645e-08f;          // 2^-24
static constexpr double kU64 = 1.1102230246251565e-16; // 2^-53
static constexpr unsigned kFull = 0xffffffffu;

#if VGPU_GATHER_TMA
// Bulk copies of candidate particle runs into shared memory, completed on a
// per-warp mbarrier (cp.async.bulk, mbarrier.try_wait).  Every wait is bounded.
static __device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
static __device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
static __device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
static __device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
static __device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
static __device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity) {
    const unsigned a = smem_addr(bar);
    for (int i = 0; i < (1 << 20); i++) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}
#endif

// plane indices are always below the engine's plane slots (64 or 128); the
// mask (to the larger) keeps every shared-memory
// index in bounds even if a slot held inconsistent data
static __device__ __forceinline__ int tri_plane(unsigned t, int e) { return (t >> (8 * e)) & (kMaxPlanesWide - 1); }

// Sortable key of a float (total order as unsigned)
static __device__ __forceinline__ unsigned float_key(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

static __device__ __forceinline__ int unpack_shift(int code, int a) { return ((code >> (8 * a)) & 255) - 128; }

// step_int, step_mod, step_div: src/v_base.hh:61-80
static __device__ __forceinline__ int step_int(double a) {
    return a < 0 ? __double2int_rz(a) - 1 : __double2int_rz(a);
}
static __device__ __forceinline__ int step_mod(int a, int b) { return a >= 0 ? a % b : b - 1 - (b - 1 - a) % b; }
static __device__ __forceinline__ int step_div(int a, int b) { return a >= 0 ? a / b : -1 + (a + 1) / b; }

// FP64 plane of a candidate (engine index j, image counts) relative to the
// particle, with the reference's own arithmetic: x1 = p_j - (x - qx)
// (src/v_compute.cc:383-397) and rs = x1*x1+y1*y1+z1*z1 [+ r_i^2 - r_j^2]
// (r_scale, src/rad_option.hh:414-416).  h = rs/2 (the reference works in
// doubled coordinates; halving is exact).
static __device__ __noinline__ double4 plane64_from(const CellParams &P, double4 me, int j, int code) {
    double4 q = P.a.p64[j];
    double sx = unpack_shift(code, 0) * P.g.len[0];
    double sy = unpack_shift(code, 1) * P.g.len[1];
    double sz = unpack_shift(code, 2) * P.g.len[2];
    double x1 = __dsub_rn(q.x, __dsub_rn(me.x, sx));
    double y1 = __dsub_rn(q.y, __dsub_rn(me.y, sy));
    double z1 = __dsub_rn(q.z, __dsub_rn(me.z, sz));
    double rs = __dadd_rn(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)), __dmul_rn(z1, z1));
    if (P.g.poly) rs = __dsub_rn(__dadd_rn(rs, __dmul_rn(me.w, me.w)), __dmul_rn(q.w, q.w));
    return make_double4(x1, y1, z1, 0.5 * rs);
}

// FP64 plane (n, h: n.v <= h inside, v relative to the particle) of wall W for
// the particle me, with the reference's arithmetic (cut_cell_base,
// src/wall.cc:29-120; its nplane(x, y, z, rsq) is n = (x, y, z), h = rsq/2).
// h = NaN: the reference adds no plane (a curved wall through the particle).
static __device__ __forceinline__ double4 wall64(const WallSpec &W, double4 me) {
    // a unit-cell face plane: the bisector of a lattice vector, the same for
    // every particle (unitcell::unit_voro_apply, src/unitcell.cc:90-94)
    if (W.type == kWallLattice) return make_double4(W.c[0], W.c[1], W.c[2], 0.5 * W.r);
    const double x = me.x, y = me.y, z = me.z;
    if (W.type == VGPU_WALL_PLANE) {
        const double dq = __dmul_rn(2.0, __dsub_rn(__dsub_rn(__dsub_rn(W.r, __dmul_rn(x, W.c[0])), __dmul_rn(y, W.c[1])),
                                                   __dmul_rn(z, W.c[2])));
        return make_double4(W.c[0], W.c[1], W.c[2], 0.5 * dq);
    }
    double xd = __dsub_rn(x, W.c[0]), yd = __dsub_rn(y, W.c[1]), zd = __dsub_rn(z, W.c[2]);
    if (W.type == VGPU_WALL_SPHERE) {
        double dq = __dadd_rn(__dadd_rn(__dmul_rn(xd, xd), __dmul_rn(yd, yd)), __dmul_rn(zd, zd));
        if (!(dq > 1e-5)) return make_double4(0, 0, 0, __longlong_as_double(0x7ff8000000000000ll));
        dq = __dmul_rn(2.0, __dsub_rn(__dmul_rn(__dsqrt_rn(dq), W.r), dq));
        return make_double4(xd, yd, zd, 0.5 * dq);
    }
    double pa = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(xd, W.a[0]), __dmul_rn(yd, W.a[1])), __dmul_rn(zd, W.a[2])), W.asi);
    xd = __dsub_rn(xd, __dmul_rn(W.a[0], pa));
    yd = __dsub_rn(yd, __dmul_rn(W.a[1], pa));
    zd = __dsub_rn(zd, __dmul_rn(W.a[2], pa));
    pa = __dadd_rn(__dadd_rn(__dmul_rn(xd, xd), __dmul_rn(yd, yd)), __dmul_rn(zd, zd));
    if (!(pa > 1e-5)) return make_double4(0, 0, 0, __longlong_as_double(0x7ff8000000000000ll));
    if (W.type == VGPU_WALL_CYLINDER) {
        pa = __dmul_rn(2.0, __dsub_rn(__dmul_rn(__dsqrt_rn(pa), W.r), pa));
        return make_double4(xd, yd, zd, 0.5 * pa);
    }
    // cone
    pa = __ddiv_rn(1.0, __dsqrt_rn(pa));
    const double q = __dsqrt_rn(W.asi);
    const double sq = __dmul_rn(W.sang, q), cp = __dmul_rn(W.cang, pa);
    const double xf = __dadd_rn(__dmul_rn(-sq, W.a[0]), __dmul_rn(cp, xd));
    const double yf = __dadd_rn(__dmul_rn(-sq, W.a[1]), __dmul_rn(cp, yd));
    const double zf = __dadd_rn(__dmul_rn(-sq, W.a[2]), __dmul_rn(cp, zd));
    pa = __dmul_rn(2.0, __dadd_rn(__dadd_rn(__dmul_rn(xf, __dsub_rn(W.c[0], x)), __dmul_rn(yf, __dsub_rn(W.c[1], y))),
                                  __dmul_rn(zf, __dsub_rn(W.c[2], z))));
    return make_double4(xf, yf, zf, 0.5 * pa);
}

// wall64 out of line, for code that runs once per cell
static __device__ __noinline__ double4 wall64_call(const WallSpec &W, double4 me) { return wall64(W, me); }

// FP64 plane of an initial face (f = 2*axis + side) of the particle's cell
static __device__ __forceinline__ double4 face64(const CellParams &P, double4 me, int f) {
    const int ax = f >> 1;
    const bool hiside = f & 1;
    const double xa = ax == 0 ? me.x : (ax == 1 ? me.y : me.z);
    double h;
    if (P.g.unit_cell) h = P.g.half[ax];
    else if (P.g.per[ax]) h = 0.5 * P.g.len[ax];
    else h = hiside ? __dsub_rn(P.g.hi[ax], xa) : -__dsub_rn(P.g.lo[ax], xa);
    const double n = hiside ? 1.0 : -1.0;
    return make_double4(ax == 0 ? n : 0.0, ax == 1 ? n : 0.0, ax == 2 ? n : 0.0, h);
}

// FP64 plane of a plane slot without a source particle: initial face f < 6,
// or wall f - 6
static __device__ __forceinline__ double4 initial64(const CellParams &P, double4 me, int f) {
    return f < 6 ? face64(P, me, f) : wall64(P.walls[f - 6], me);
}

// Vertex of three FP64 planes by Cramer's rule; kn = sum over rows of
// |cofactor row| * (|h| + |n||v|), the scale of its rounding error.
static __device__ __forceinline__ void solve_f64(const double4 A, const double4 B, const double4 C, double &x, double &y,
                                          double &z, double &D, float &kn) {
    double bcx = B.y * C.z - B.z * C.y, bcy = B.z * C.x - B.x * C.z, bcz = B.x * C.y - B.y * C.x;
    double cax = C.y * A.z - C.z * A.y, cay = C.z * A.x - C.x * A.z, caz = C.x * A.y - C.y * A.x;
    double abx = A.y * B.z - A.z * B.y, aby = A.z * B.x - A.x * B.z, abz = A.x * B.y - A.y * B.x;
    D = A.x * bcx + A.y * bcy + A.z * bcz;
    double inv = 1.0 / D;
    x = (A.w * bcx + B.w * cax + C.w * abx) * inv;
    y = (A.w * bcy + B.w * cay + C.w * aby) * inv;
    z = (A.w * bcz + B.w * caz + C.w * abz) * inv;
    float vv = sqrtf((float)(x * x + y * y + z * z));
    float nbc = fabsf((float)bcx) + fabsf((float)bcy) + fabsf((float)bcz);
    float nca = fabsf((float)cax) + fabsf((float)cay) + fabsf((float)caz);
    float nab = fabsf((float)abx) + fabsf((float)aby) + fabsf((float)abz);
    float na = fabsf((float)A.x) + fabsf((float)A.y) + fabsf((float)A.z);
    float nb = fabsf((float)B.x) + fabsf((float)B.y) + fabsf((float)B.z);
    float nc = fabsf((float)C.x) + fabsf((float)C.y) + fabsf((float)C.z);
    kn = nbc * (fabsf((float)A.w) + na * vv) + nca * (fabsf((float)B.w) + nb * vv) + nab * (fabsf((float)C.w) + nc * vv);
}


// ------------------------------------------------------------------ warp helpers
static __device__ __forceinline__ unsigned long long warp_or64(unsigned long long x) {
    unsigned lo = __reduce_or_sync(kFull, (unsigned)x);
    unsigned hi = __reduce_or_sync(kFull, (unsigned)(x >> 32));
    return ((unsigned long long)hi << 32) | lo;
}
// Largest of the lanes' values, for values that are +0 or positive (their
// bit patterns order like unsigned integers): one redux instead of a
// shuffle tree.
static __device__ __forceinline__ float warp_max_nonneg(float x) {
    return __uint_as_float(__reduce_max_sync(kFull, __float_as_uint(x)));
}
static __device__ __forceinline__ double warp_sumd(double x) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(kFull, x, d);
    return x;
}
// Exclusive prefix sum and total of small non-negative lane values
// (x < 2^BITS) from one ballot per bit: the ballots are independent, so the
// latency is that of one ballot rather than of a chain of shuffles.
template <int BITS>
static __device__ __forceinline__ int warp_excl_scan_small(int x, int lane, int &total) {
    const unsigned lt = (1u << lane) - 1u;
    int ex = 0, tot = 0;
#pragma unroll
    for (int b = 0; b < BITS; b++) {
        const unsigned m = __ballot_sync(kFull, (x >> b) & 1);
        ex += __popc(m & lt) << b;
        tot += __popc(m) << b;
    }
    total = tot;
    return ex;
}
static __device__ __forceinline__ int warp_incl_scan(int x, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
    }
    return x;
}

}  // namespace vgpu
