// Point location: the particle whose Voronoi cell contains a point, for
// many points at once (one thread per point).
//
// It replaces container::find_voronoi_cell (src/container.cc:237-301),
// container_periodic::find_voronoi_cell (src/container_prd.cc:303-359) and
// voro_compute::find_voronoi_cell (src/v_compute.cc:70-228): the point is
// remapped into the domain with the reference's own arithmetic (remap,
// src/container.cc:203-224 and src/container_prd.cc:266-291; a point outside
// a non-periodic wall is not found), then the particle of smallest
// x1*x1+y1*y1+z1*z1 [- r^2] with x1 = p - (x - shift) (scan_all,
// src/v_compute.cc:47-57) over the particles and their periodic images is
// searched on the engine's block grid, in order of the blocks' lower-bound
// distance (the offset table of the cell engine, then Chebyshev shells),
// until no unsearched block can hold a smaller value (r_max_add,
// src/rad_option.hh:123).  The returned position is the particle's stored
// position plus the image counts of the point and of the block times the box
// lengths, as the reference assembles it.  container_periodic keeps y and z
// images as stored particles of its ghost blocks (put_image,
// src/container_prd.cc:766-774: p + image * length), so along y and z the
// distance and the returned position start from that image position; x is
// wrapped by shifting the point, as for the flag-periodic container.  A
// sheared box stores its y and z images as engine entries (the ghost layers),
// so only x wraps; the answer is the stored image plus the point's image
// displacement ak*c + aj*b + ai*a in the reference's order.  Exact ties keep
// the first value found in this search order, which may differ from the
// reference's.
#include "vgpu_dev.cuh"

namespace vgpu {

namespace {

struct Best {
    double d;
    int j;
    int img[3];
};

// The particles of the engine block at offset (di,dj,dk) from block eb of the
// point c (local position loc in its block); skipped when wrapped off a
// non-periodic wall or when the block's lower bound exceeds the best so far.
__device__ __forceinline__ void scan_block(const CellParams &P, const int eb[3], const double c[3],
                                           const double loc[3], int di, int dj, int dk, double rmax2, Best &B) {
    const Geometry &g = P.g;
    const int d[3] = {di, dj, dk};
    int wr[3], img[3];
    double md2 = 0.0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int n = g.gn[a];
        int cb = eb[a] + d[a];
        img[a] = 0;
        if (g.per[a]) {
            int w = cb % n;
            if (w < 0) w += n;
            img[a] = (cb - w) / n;
            cb = w;
        } else if (cb < 0 || cb >= n) {
            return;
        }
        wr[a] = cb;
        double t = d[a] > 0 ? d[a] * g.gbs[a] - loc[a] : (d[a] < 0 ? loc[a] - (d[a] + 1) * g.gbs[a] : 0.0);
        t = fmax(t, 0.0);
        md2 += t * t;
    }
    if (md2 * (1.0 - 1e-12) > B.d + rmax2) return;
    const int b = wr[0] + g.gn[0] * (wr[1] + g.gn[1] * wr[2]);
    const int s0 = P.a.bstart[b], s1 = P.a.bstart[b + 1];
    // the point shifted by the image (or, for container_periodic's y and z,
    // the particle's image built as the reference stores it)
    const bool ghost = (g.kind == VGPU_CONTAINER_PERIODIC || g.kind == VGPU_CONTAINER_PERIODIC_POLY) && !g.tric;
    double q[3], sh[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool img_on_p = ghost && a > 0;
        q[a] = (img[a] && !img_on_p) ? __dsub_rn(c[a], __dmul_rn((double)img[a], g.len[a])) : c[a];
        sh[a] = (img[a] && img_on_p) ? __dmul_rn((double)img[a], g.len[a]) : 0.0;
    }
    for (int j = s0; j < s1; j++) {
        const double4 p = P.a.p64[j];
        const double py = sh[1] != 0.0 ? __dadd_rn(p.y, sh[1]) : p.y;
        const double pz = sh[2] != 0.0 ? __dadd_rn(p.z, sh[2]) : p.z;
        const double x1 = __dsub_rn(p.x, q[0]), y1 = __dsub_rn(py, q[1]), z1 = __dsub_rn(pz, q[2]);
        double rs = __dadd_rn(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)), __dmul_rn(z1, z1));
        if (g.poly) rs = __dsub_rn(rs, __dmul_rn(p.w, p.w));
        if (rs < B.d) {
            B.d = rs;
            B.j = j;
            B.img[0] = img[0];
            B.img[1] = img[1];
            B.img[2] = img[2];
        }
    }
}

__global__ void locate_kernel(const __grid_constant__ CellParams P, int n, const double *qxyz, int *found, int *pid,
                              double *rxyz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Geometry &g = P.g;
    double c[3] = {qxyz[3 * i], qxyz[3 * i + 1], qxyz[3 * i + 2]};
    int a[3] = {0, 0, 0};
    bool inside = true;
    if (g.kind == VGPU_CONTAINER || g.kind == VGPU_CONTAINER_POLY) {
        for (int ax = 0; ax < 3; ax++) {
            const int ci = step_int(__dmul_rn(__dsub_rn(c[ax], g.lo[ax]), g.usp[ax]));
            if (ci < 0 || ci >= g.un[ax]) {
                if (g.per[ax]) {
                    a[ax] = step_div(ci, g.un[ax]);
                    c[ax] = __dsub_rn(c[ax], __dmul_rn((double)a[ax], g.len[ax]));
                } else {
                    inside = false;
                }
            }
        }
    } else {   // container_periodic: z, then y, then x, along the lattice vectors
        int ci = step_int(__dmul_rn(c[2], g.usp[2]));
        if (ci < 0 || ci >= g.un[2]) {
            a[2] = step_div(ci, g.un[2]);
            c[2] = __dsub_rn(c[2], __dmul_rn((double)a[2], g.len[2]));
            c[1] = __dsub_rn(c[1], __dmul_rn((double)a[2], g.shear[2]));
            c[0] = __dsub_rn(c[0], __dmul_rn((double)a[2], g.shear[1]));
        }
        ci = step_int(__dmul_rn(c[1], g.usp[1]));
        if (ci < 0 || ci >= g.un[1]) {
            a[1] = step_div(ci, g.un[1]);
            c[1] = __dsub_rn(c[1], __dmul_rn((double)a[1], g.len[1]));
            c[0] = __dsub_rn(c[0], __dmul_rn((double)a[1], g.shear[0]));
        }
        ci = step_int(__dmul_rn(c[0], g.usp[0]));
        if (ci < 0 || ci >= g.un[0]) {
            a[0] = step_div(ci, g.un[0]);
            c[0] = __dsub_rn(c[0], __dmul_rn((double)a[0], g.len[0]));
        }
    }
    Best B;
    B.d = 3.0e300;
    B.j = -1;
    B.img[0] = B.img[1] = B.img[2] = 0;
    if (inside && P.ncells > 0) {
        int eb[3];
        double loc[3];
        for (int ax = 0; ax < 3; ax++) {
            int v = (int)floor((c[ax] - g.lo[ax]) / g.gbs[ax]);
            v = v < 0 ? 0 : (v >= g.gn[ax] ? g.gn[ax] - 1 : v);
            eb[ax] = v;
            loc[ax] = c[ax] - (g.lo[ax] + v * g.gbs[ax]);
        }
        const double rmax2 = g.poly ? g.rmax * g.rmax : 0.0;
        const double bmin2 = (double)g.gbs_min * (double)g.gbs_min;
        bool done = false;
        for (int seg = 0; seg < P.ngroups && !done; seg++) {
            if (P.group_lb2[seg] * bmin2 * (1.0 - 1e-12) > B.d + rmax2) {
                done = true;
                break;
            }
            for (int e = P.group_start[seg]; e < P.group_start[seg + 1]; e++) {
                const int code = P.offsets[e];
                scan_block(P, eb, c, loc, (code & 31) - 16, ((code >> 5) & 31) - 16, ((code >> 10) & 31) - 16, rmax2,
                           B);
            }
        }
        // Chebyshev shells beyond the table (at radius kOffsetRadius only the
        // offsets the table leaves out)
        const int rmax_grid = max(g.gn[0], max(g.gn[1], g.gn[2]));
        const bool any_periodic = g.per[0] || g.per[1] || g.per[2];
        const int rlim = min(4 * rmax_grid + 8, kMaxShellRadius);
        for (int r = kOffsetRadius; !done && r < rlim; r++) {
            if (!any_periodic && r > rmax_grid + 1) break;
            if ((double)((r - 1) * (r - 1)) * bmin2 * (1.0 - 1e-12) > B.d + rmax2) break;
            for (int e = 0; e < 6 * (2 * r + 1) * (2 * r + 1); e++) {
                int di, dj, dk;
                if (!shell_offset(e, r, di, dj, dk)) continue;
                const int x = max(abs(di) - 1, 0), y = max(abs(dj) - 1, 0), z = max(abs(dk) - 1, 0);
                if (r == kOffsetRadius && x * x + y * y + z * z <= kTableLb2Max) continue;
                scan_block(P, eb, c, loc, di, dj, dk, rmax2, B);
            }
        }
    }
    if (B.j < 0) {
        found[i] = 0;
        pid[i] = -1;
        rxyz[3 * i] = rxyz[3 * i + 1] = rxyz[3 * i + 2] = 0.0;
        return;
    }
    const double4 p = P.a.p64[B.j];
    const double pv[3] = {p.x, p.y, p.z};
    found[i] = 1;
    pid[i] = P.a.pid[B.j];
    if (g.tric) {   // a stored image, x wrapped by the block search; then the point's images
        rxyz[3 * i] = __dadd_rn(__dadd_rn(__dadd_rn(p.x, __dmul_rn((double)a[2], g.shear[1])),
                                          __dmul_rn((double)a[1], g.shear[0])),
                                __dmul_rn((double)(a[0] + B.img[0]), g.len[0]));
        rxyz[3 * i + 1] = __dadd_rn(__dadd_rn(p.y, __dmul_rn((double)a[2], g.shear[2])),
                                    __dmul_rn((double)a[1], g.len[1]));
        rxyz[3 * i + 2] = __dadd_rn(p.z, __dmul_rn((double)a[2], g.len[2]));
        return;
    }
    const bool ghost = g.kind == VGPU_CONTAINER_PERIODIC || g.kind == VGPU_CONTAINER_PERIODIC_POLY;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        if (ghost && ax > 0) {   // the stored image, then the point's own image count
            const double pi = B.img[ax] ? __dadd_rn(pv[ax], __dmul_rn((double)B.img[ax], g.len[ax])) : pv[ax];
            rxyz[3 * i + ax] = __dadd_rn(pi, __dmul_rn((double)a[ax], g.len[ax]));
        } else {
            rxyz[3 * i + ax] = __dadd_rn(pv[ax], __dmul_rn((double)(a[ax] + B.img[ax]), g.len[ax]));
        }
    }
}

}  // namespace

cudaError_t launch_locate(const CellParams &cp, int n, const double *qxyz, int *found, int *pid, double *rxyz,
                          cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int threads = 128;
    locate_kernel<<<(n + threads - 1) / threads, threads, 0, s>>>(cp, n, qxyz, found, pid, rxyz);
    note_launch();
    return cudaGetLastError();
}

}  // namespace vgpu
