// Binning: the device side of put().
//
// remap_kernel reproduces the reference's placement arithmetic exactly (same
// IEEE double operations, no contraction):
//   container:          put_remap          src/container.cc:174-191
//   container_periodic: put_locate_block   src/container_prd.cc:189-216
// and computes two keys per particle: the reference block (which fixes the
// loop order of results) and the engine block (which fixes the search grid).
#include <algorithm>
#include "vgpu_dev.cuh"

namespace vgpu {

namespace {

// The engine block of position c (clamped into the grid).
__device__ __forceinline__ unsigned engine_key(const Geometry &g, const double c[3]) {
    int e[3];
    for (int a = 0; a < 3; a++) {
        double t = (c[a] - g.lo[a]) / g.gbs[a];
        int v = (int)floor(t);
        e[a] = v < 0 ? 0 : (v >= g.gn[a] ? g.gn[a] - 1 : v);
    }
    return (unsigned)(e[0] + g.gn[0] * (e[1] + g.gn[1] * e[2]));
}

// A particle whose position (or, in a radical container, radius) is not
// finite cannot be placed: the remap would turn it into a block index it has
// no business in.  Both binning paths count such particles and the host
// fails the compute with VGPU_ERR_ARG before any cell is computed.
__device__ __forceinline__ bool finite_input(const Geometry &g, double4 q) {
    return isfinite(q.x) && isfinite(q.y) && isfinite(q.z) && (!g.poly || isfinite(q.w));
}

// The reference's placement of one particle: remapped position c, its
// reference block key uk (nub if put() drops it) and engine block key gk.
__device__ __forceinline__ bool remap_one(const Geometry &g, double4 q, int nub, int nblocks, double4 &out,
                                          unsigned &uk, unsigned &gk) {
    double c[3] = {q.x, q.y, q.z};
    int b[3];
    bool ok = true;
    if (g.kind == VGPU_CONTAINER || g.kind == VGPU_CONTAINER_POLY) {
        for (int a = 0; a < 3; a++) {
            int ijk = step_int(__dmul_rn(__dsub_rn(c[a], g.lo[a]), g.usp[a]));
            if (g.per[a]) {
                int l = step_mod(ijk, g.un[a]);
                c[a] = __dadd_rn(c[a], __dmul_rn(g.ubox[a], (double)(l - ijk)));
                ijk = l;
            } else if (ijk < 0 || ijk >= g.un[a]) {
                ok = false;
            }
            b[a] = ijk;
        }
    } else {
        // container_periodic: z, then y, then x, each remapped along its
        // lattice vector (c = (bxz, byz, bz), b = (bxy, by, 0), a = (bx, 0, 0))
        int k = step_int(__dmul_rn(c[2], g.usp[2]));
        if (k < 0 || k >= g.un[2]) {
            const int ak = step_div(k, g.un[2]);
            c[2] = __dsub_rn(c[2], __dmul_rn((double)ak, g.len[2]));
            c[1] = __dsub_rn(c[1], __dmul_rn((double)ak, g.shear[2]));
            c[0] = __dsub_rn(c[0], __dmul_rn((double)ak, g.shear[1]));
            k -= ak * g.un[2];
        }
        int j = step_int(__dmul_rn(c[1], g.usp[1]));
        if (j < 0 || j >= g.un[1]) {
            const int aj = step_div(j, g.un[1]);
            c[1] = __dsub_rn(c[1], __dmul_rn((double)aj, g.len[1]));
            c[0] = __dsub_rn(c[0], __dmul_rn((double)aj, g.shear[0]));
            j -= aj * g.un[1];
        }
        int i = step_int(__dmul_rn(c[0], g.usp[0]));
        if (i < 0 || i >= g.un[0]) {
            const int ai = step_div(i, g.un[0]);
            c[0] = __dsub_rn(c[0], __dmul_rn((double)ai, g.len[0]));
            i -= ai * g.un[0];
        }
        b[0] = i;
        b[1] = j;
        b[2] = k;
    }
    if (ok) {
        uk = (unsigned)(b[0] + g.un[0] * (b[1] + g.un[1] * b[2]));
        gk = engine_key(g, c);
    } else {
        uk = (unsigned)nub;
        gk = (unsigned)nblocks;
    }
    out = make_double4(c[0], c[1], c[2], q.w);
    return ok;
}

// The engine-order record of particle i (input order) placed at engine index k:
// its position, and its position relative to its engine block's origin as a
// float pair h + l (h: the clipping kernels' FP32 position; h + l: the
// finish kernel's planes).
__device__ __forceinline__ void gather_one(const Geometry &g, int k, int b, double4 p, int id, int outpos_i,
                                           double4 *p64, float4 *lffh, float4 *lffl, int *pid,
                                           int *outpos, int *gblock) {
    int bx = b % g.gn[0];
    int by = (b / g.gn[0]) % g.gn[1];
    int bz = b / (g.gn[0] * g.gn[1]);
    p64[k] = p;
    // (p - lo) - b * bs rather than p - (lo + b * bs): the block origin
    // rounded at the magnitude of lo would put an error of ulp(lo) into the
    // local positions (a box near 1e5 lost 1e-10 of its cells' volumes in
    // the float-pair planes); p - lo is exact within a container far from
    // the origin (p and lo within a factor two) and otherwise errs by an ulp
    // of the box's size, and it is the same difference the engine key uses
    const double d[4] = {(p.x - g.lo[0]) - bx * g.gbs[0], (p.y - g.lo[1]) - by * g.gbs[1],
                         (p.z - g.lo[2]) - bz * g.gbs[2], p.w};
    float h[4], l[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        h[a] = __double2float_rn(d[a]);
        l[a] = __double2float_rn(d[a] - (double)h[a]);
    }
    lffh[k] = make_float4(h[0], h[1], h[2], h[3]);
    lffl[k] = make_float4(l[0], l[1], l[2], l[3]);
    pid[k] = id;
    outpos[k] = outpos_i;
    gblock[k] = b;
}

__global__ void remap_kernel(BinParams bp, int nub, int nblocks, int *kept, unsigned long long *rmax_bits) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bp.n) return;
    const Geometry &g = bp.g;
    const double4 q = bp.xyzr_in[i];
    if (!finite_input(g, q)) atomicAdd(kept + 1, 1);   // counted; the host rejects the compute
    double4 r;
    unsigned uk, gk;
    if (remap_one(g, q, nub, nblocks, r, uk, gk)) {
        atomicAdd(kept, 1);
        // radius_poly::max_radius over stored particles (src/container.cc:108)
        if (g.poly) atomicMax(rmax_bits, (unsigned long long)__double_as_longlong(fmax(q.w, 0.0)));
    }
    bp.rem[i] = r;
    bp.ukey[i] = uk;
    bp.gkey[i] = gk;
    bp.idx[i] = i;
}

__global__ void loop_order_kernel(const int *uorder, int nkept, const int *ids_in, const double4 *rem,
                                  int *outpos_by_input, int *res_ids, double *res_pos, double *res_rad) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nkept) return;
    int i = uorder[m];
    outpos_by_input[i] = m;
    res_ids[m] = ids_in[i];
    double4 p = rem[i];
    res_pos[3 * m] = p.x;
    res_pos[3 * m + 1] = p.y;
    res_pos[3 * m + 2] = p.z;
    res_rad[m] = p.w;
}

// Engine entry k: input particle i = gorder[k] (i < nin), or the image
// i - nin of particle img_src[i - nin], which has no result slot (-1).
__global__ void gather_kernel(Geometry g, int nengine, int nin, const int *img_src, const int *gorder,
                              const unsigned *gkey_sorted, const double4 *rem, const int *ids_in,
                              const int *outpos_by_input, double4 *p64, float4 *lffh, float4 *lffl, int *pid,
                              int *outpos, int *gblock, int *bstart, int nblocks) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nengine) return;
    int i = gorder[k];
    int b = (int)gkey_sorted[k];
    const bool particle = i < nin;
    const int id = particle ? ids_in[i] : ids_in[img_src[i - nin]];
    gather_one(g, k, b, rem[i], id, particle ? outpos_by_input[i] : -1, p64, lffh, lffl, pid, outpos, gblock);
    int prev = k == 0 ? -1 : (int)gkey_sorted[k - 1];
    for (int q = prev + 1; q <= b; q++) bstart[q] = k;
    if (k == nengine - 1)
        for (int q = b + 1; q <= nblocks; q++) bstart[q] = nengine;
}

// The images of particle p (remapped into the primary domain) in the ghost
// layers of a sheared periodic box: p + ic*c + ib*b + ia*a for every
// (ib, ic) != (0, 0) whose y and z lie in the engine region, ia taking x into
// the primary range as put_locate_block would.  Displacements as the
// reference's image blocks build them (create_side_image and
// create_vertical_image, src/container_prd.cc:583-758; put_image, 766-774):
// x ic*bxz + ib*bxy + ia*bx, y ic*byz + ib*by, z ic*bz, each added to p.
// WRITE: stored from slot nin + base on; returns the count.
template <bool WRITE>
__device__ int images_of(const Geometry &g, double4 p, int src, int nin, int base, double4 *rem_out,
                         unsigned *gkey_out, int *idx_out, int *img_src) {
    const double zlo = g.lo[2], zhi = g.lo[2] + g.ext[2];
    const double ylo = g.lo[1], yhi = g.lo[1] + g.ext[1];
    // a remapped particle lies in the primary domain, so its image counts
    // span a few box lengths; the bounds also keep a non-finite input from
    // looping
    if (!(fabs(p.x) < 1e300 && fabs(p.y) < 1e300 && fabs(p.z) < 1e300)) return 0;
    const double fz = floor((zlo - p.z) / g.len[2]);
    if (!(fabs(fz) < 1e6)) return 0;
    const int c0 = (int)fz - 1;
    const int c1 = min((int)ceil((zhi - p.z) / g.len[2]) + 1, c0 + 64);
    int cnt = 0;
    for (int ic = c0; ic <= c1; ic++) {
        const double z = __dadd_rn(p.z, __dmul_rn((double)ic, g.len[2]));
        if (!(z >= zlo && z < zhi)) continue;
        const double yc = p.y + (double)ic * g.shear[2];
        const double fy = floor((ylo - yc) / g.len[1]);
        if (!(fabs(fy) < 1e6)) continue;
        const int b0 = (int)fy - 1;
        const int b1 = min((int)ceil((yhi - yc) / g.len[1]) + 1, b0 + 64);
        for (int ib = b0; ib <= b1; ib++) {
            if (ib == 0 && ic == 0) continue;
            const double dy = __dadd_rn(__dmul_rn((double)ic, g.shear[2]), __dmul_rn((double)ib, g.len[1]));
            const double y = __dadd_rn(p.y, dy);
            if (!(y >= ylo && y < yhi)) continue;
            if (WRITE) {
                const double dx0 = __dadd_rn(__dmul_rn((double)ic, g.shear[1]), __dmul_rn((double)ib, g.shear[0]));
                const int i = step_int(__dmul_rn(__dadd_rn(p.x, dx0), g.usp[0]));
                const int ia = (i < 0 || i >= g.un[0]) ? -step_div(i, g.un[0]) : 0;
                const double dx = __dadd_rn(dx0, __dmul_rn((double)ia, g.len[0]));
                const double c[3] = {__dadd_rn(p.x, dx), y, z};
                const int t = nin + base + cnt;
                rem_out[t] = make_double4(c[0], c[1], c[2], p.w);
                gkey_out[t] = engine_key(g, c);
                idx_out[t] = t;
                img_src[base + cnt] = src;
            }
            cnt++;
        }
    }
    return cnt;
}

__global__ void image_count_kernel(Geometry g, int n, const double4 *rem, int *count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    count[i] = images_of<false>(g, rem[i], i, 0, 0, nullptr, nullptr, nullptr, nullptr);
}

__global__ void image_write_kernel(Geometry g, int n, const double4 *rem, const int *offset, int nin,
                                   double4 *rem_out, unsigned *gkey_out, int *idx_out, int *img_src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    images_of<true>(g, rem[i], i, nin, offset[i], rem_out, gkey_out, idx_out, img_src);
}

__global__ void particle_flag_kernel(const int *outpos, int nengine, int *flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nengine) flag[k] = outpos[k] >= 0 ? 1 : 0;
}

__global__ void cell_list_kernel(const int *outpos, const int *slot, int nengine, int *list) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nengine && outpos[k] >= 0) list[slot[k]] = k;
}

// The whole of put()'s binning for one small container in one CTA: remap,
// the stable sort into loop order (reference block, then insertion order),
// the duplicate check, the stable sort into engine order and the gather, with
// the keys sorted in shared memory (bitonic, over 64-bit keys whose low half
// is the input index: stable).  A batch bins all its small members with one
// launch of this kernel instead of a dozen launches each.
__device__ __forceinline__ void cta_bitonic(unsigned long long *key, int n2) {
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int t = threadIdx.x; t < n2 / 2; t += blockDim.x) {
                const int i = 2 * j * (t / j) + (t % j);
                const int l = i + j;
                const bool up = (i & k) == 0;
                const unsigned long long a = key[i], b = key[l];
                if ((a > b) == up) {
                    key[i] = b;
                    key[l] = a;
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kSmallBinThreads) small_bin_kernel(const SmallBinJob *jobs, int cap) {
    extern __shared__ unsigned long long sbin[];
    __shared__ int s_kept, s_dup, s_bad;
    __shared__ unsigned long long s_rmax;
    const SmallBinJob &J = jobs[blockIdx.x];
    const Geometry &g = J.g;
    const int n = J.n;
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    unsigned long long *key = sbin;                                  // n2 keys
    unsigned *gk_in = reinterpret_cast<unsigned *>(sbin + cap);   // engine key per input index
    if (threadIdx.x == 0) {
        s_kept = 0;
        s_dup = 0;
        s_bad = 0;
        s_rmax = 0ull;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        if (i < n) {
            const double4 q = J.xyzr_in[i];
            if (!finite_input(g, q)) s_bad = 1;
            double4 r;
            unsigned uk, gk;
            if (remap_one(g, q, J.nub, J.nblocks, r, uk, gk)) {
                atomicAdd(&s_kept, 1);
                if (g.poly) atomicMax(&s_rmax, (unsigned long long)__double_as_longlong(fmax(q.w, 0.0)));
            }
            J.rem[i] = r;
            J.outpos_in[i] = -1;   // a dropped particle keeps -1 (kept ones: set below)
            key[i] = ((unsigned long long)uk << 32) | (unsigned)i;
            gk_in[i] = gk;
        } else {
            key[i] = ~0ull;
        }
    }
    __syncthreads();
    cta_bitonic(key, n2);
    const int nkept = s_kept;
    // loop order (c_loop_all): stored ids, positions, radii; input -> result slot
    for (int m = threadIdx.x; m < nkept; m += blockDim.x) {
        const int i = (int)(key[m] & 0xffffffffu);
        J.outpos_in[i] = m;
        J.res_ids[m] = J.ids_in[i];
        const double4 p = J.rem[i];
        J.res_pos[3 * m] = p.x;
        J.res_pos[3 * m + 1] = p.y;
        J.res_pos[3 * m + 2] = p.z;
        J.res_rad[m] = p.w;
        // check_duplicate within the reference block (src/common.cc:14-20)
        if (g.unit_cell) {
            const unsigned blk = (unsigned)(key[m] >> 32);
            for (int q = m + 1; q < nkept && (unsigned)(key[q] >> 32) == blk; q++) {
                const double4 o = J.rem[(int)(key[q] & 0xffffffffu)];
                const double dx = o.x - p.x, dy = o.y - p.y, dz = o.z - p.z;
                if (dx * dx + dy * dy + dz * dz < 1e-10) s_dup = 1;
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n2; i += blockDim.x)
        key[i] = i < n ? (((unsigned long long)gk_in[i] << 32) | (unsigned)i) : ~0ull;
    __syncthreads();
    cta_bitonic(key, n2);
    // engine order and the block starts
    for (int k = threadIdx.x; k < nkept; k += blockDim.x) {
        const int i = (int)(key[k] & 0xffffffffu);
        const int b = (int)(key[k] >> 32);
        gather_one(g, k, b, J.rem[i], J.ids_in[i], J.outpos_in[i], J.p64, J.lffh, J.lffl, J.pid, J.outpos,
                   J.gblock);
        const int prev = k == 0 ? -1 : (int)(key[k - 1] >> 32);
        for (int q = prev + 1; q <= b; q++) J.bstart[q] = k;
        if (k == nkept - 1)
            for (int q = b + 1; q <= J.nblocks; q++) J.bstart[q] = nkept;
    }
    if (nkept == 0)
        for (int q = threadIdx.x; q <= J.nblocks; q += blockDim.x) J.bstart[q] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        J.result[0] = (unsigned long long)nkept | ((unsigned long long)s_dup << 32) |
                      ((unsigned long long)s_bad << 33);
        J.result[1] = s_rmax;
    }
}

__global__ void empty_bstart_kernel(int *bstart, int nblocks) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q <= nblocks) bstart[q] = 0;
}

// check_duplicate (src/common.cc:14-20), applied within each reference block
// as container_periodic::put does (src/container_prd.cc:94-101).
__global__ void duplicate_kernel(const unsigned *ukey_sorted, const int *uorder, const double4 *rem, int nkept,
                                 int *dup_flag) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nkept) return;
    unsigned key = ukey_sorted[m];
    double4 a = rem[uorder[m]];
    for (int q = m + 1; q < nkept && ukey_sorted[q] == key; q++) {
        double4 b = rem[uorder[q]];
        double dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
        if (dx * dx + dy * dy + dz * dz < 1e-10) atomicExch(dup_flag, 1);
    }
}

}  // namespace

// The lowest index among n staged particles whose x, y or z (or r, when poly)
// is an infinity or a NaN, by atomicMin into *first (left as it was when all
// are finite).  put() runs it on the particles it has just copied, before it
// counts them as staged.
__global__ void first_nonfinite_kernel(const double4 *xyzr, long long n, int poly, unsigned long long *first) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const double4 q = xyzr[i];
        if (!(isfinite(q.x) && isfinite(q.y) && isfinite(q.z) && (!poly || isfinite(q.w))))
            atomicMin(first, (unsigned long long)i);
    }
}

cudaError_t launch_first_nonfinite(const double *xyzr, long long n, bool poly, unsigned long long *first,
                                   cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const long long blocks = std::min<long long>((n + 255) / 256, 4096);
    first_nonfinite_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const double4 *>(xyzr), n, poly ? 1 : 0,
                                                             first);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_remap(const BinParams &bp, int *kept, unsigned long long *rmax_bits, cudaStream_t s) {
    int nub = bp.g.un[0] * bp.g.un[1] * bp.g.un[2];
    int nblocks = bp.g.gn[0] * bp.g.gn[1] * bp.g.gn[2];
    int threads = 256, blocks = (bp.n + threads - 1) / threads;
    if (blocks > 0) {
        remap_kernel<<<blocks, threads, 0, s>>>(bp, nub, nblocks, kept, rmax_bits);
        note_launch();
    }
    return cudaGetLastError();
}

namespace {

// Ghost particles (compute_ghost_cell, src/container.hh:487-498 and 710-721,
// src/container_prd.hh:414-422 and 635-644): each is located like a put()
// (put_locate_block: the same remap, a point outside a non-periodic wall is
// rejected) and written as engine entry base + i, in no block's particle
// range, so that no cell sees it as a neighbour; its result slot is i.
__global__ void ghost_setup_kernel(Geometry g, int n, int nub, int nblocks, const double4 *q, int base,
                                   double4 *p64, float4 *lffh, float4 *lffl, int *pid, int *outpos, int *gblock,
                                   int *keep) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4 r;
    unsigned uk, gk;
    const bool ok = remap_one(g, q[i], nub, nblocks, r, uk, gk);
    keep[i] = ok ? 1 : 0;
    if (ok) gather_one(g, base + i, (int)gk, r, -1, i, p64, lffh, lffl, pid, outpos, gblock);
}

}  // namespace

cudaError_t launch_ghost_setup(const Geometry &g, int n, const double4 *q, int base, double4 *p64, float4 *lffh,
                               float4 *lffl, int *pid, int *outpos, int *gblock, int *keep, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    ghost_setup_kernel<<<(n + threads - 1) / threads, threads, 0, s>>>(
        g, n, g.un[0] * g.un[1] * g.un[2], g.gn[0] * g.gn[1] * g.gn[2], q, base, p64, lffh, lffl, pid, outpos, gblock,
        keep);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_gather(const Geometry &g, int nkept, int nengine, int nin, const int *img_src,
                          const int *uorder, const int *gorder,
                          const unsigned *gkey_sorted, const double4 *rem, const int *ids_in,
                          int *outpos_by_input, double4 *p64, float4 *lffh, float4 *lffl,
                          int *pid, int *outpos,
                          int *gblock, int *bstart, int nblocks, int *res_ids, double *res_pos,
                          double *res_rad, cudaStream_t s) {
    int threads = 256;
    if (nengine == 0) {
        empty_bstart_kernel<<<(nblocks + 1 + threads - 1) / threads, threads, 0, s>>>(bstart, nblocks);
        note_launch();
        return cudaGetLastError();
    }
    if (nkept > 0) {
        loop_order_kernel<<<(nkept + threads - 1) / threads, threads, 0, s>>>(uorder, nkept, ids_in, rem,
                                                                              outpos_by_input, res_ids, res_pos,
                                                                              res_rad);
        note_launch();
    }
    gather_kernel<<<(nengine + threads - 1) / threads, threads, 0, s>>>(g, nengine, nin, img_src, gorder,
                                                                        gkey_sorted, rem, ids_in, outpos_by_input,
                                                                        p64, lffh, lffl, pid, outpos, gblock,
                                                                        bstart, nblocks);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_image_count(const Geometry &g, int n, const double4 *rem, int *count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    image_count_kernel<<<(n + threads - 1) / threads, threads, 0, s>>>(g, n, rem, count);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_image_write(const Geometry &g, int n, const double4 *rem, const int *offset, int nin,
                               double4 *rem_out, unsigned *gkey_out, int *idx_out, int *img_src, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    image_write_kernel<<<(n + threads - 1) / threads, threads, 0, s>>>(g, n, rem, offset, nin, rem_out, gkey_out,
                                                                       idx_out, img_src);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_cell_list(const int *outpos, int nengine, int *list, int *flag, int *slot, int *scan_tmp,
                             size_t scan_tmp_ints_avail, cudaStream_t s) {
    if (nengine <= 0) return cudaSuccess;
    const int threads = 256, blocks = (nengine + threads - 1) / threads;
    particle_flag_kernel<<<blocks, threads, 0, s>>>(outpos, nengine, flag);
    note_launch();
    cudaError_t e = exclusive_scan_int(flag, slot, nengine, scan_tmp, scan_tmp_ints_avail, s);
    if (e != cudaSuccess) return e;
    cell_list_kernel<<<blocks, threads, 0, s>>>(outpos, slot, nengine, list);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_small_bin(const SmallBinJob *jobs, int njobs, int cap, cudaStream_t s) {
    if (njobs <= 0) return cudaSuccess;
    if (cap <= 0 || cap > kSmallBinMax || (cap & (cap - 1)) != 0) return cudaErrorInvalidValue;
    const size_t smem = (size_t)cap * 8 + (size_t)cap * 4;
    cudaError_t e = cudaFuncSetAttribute(small_bin_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    small_bin_kernel<<<njobs, kSmallBinThreads, smem, s>>>(jobs, cap);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_duplicate_check(const unsigned *ukey_sorted, const int *uorder, const double4 *rem,
                                   int nkept, int *dup_flag, cudaStream_t s) {
    if (nkept == 0) return cudaSuccess;
    int threads = 256, blocks = (nkept + threads - 1) / threads;
    duplicate_kernel<<<blocks, threads, 0, s>>>(ukey_sorted, uorder, rem, nkept, dup_flag);
    note_launch();
    return cudaGetLastError();
}

}  // namespace vgpu
