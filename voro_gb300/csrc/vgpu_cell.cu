// Dispatch of the cell engine's kernels and the small kernels over its
// results (CSR neighbour lists, volume sums).
#include "vgpu_dev.cuh"

namespace vgpu {

namespace {

__global__ void nf_to_ll_kernel(const int *nf, long long *out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = nf[i];
}

// neighbour q of cell i (m faces): its row, or the overflow store
__device__ __forceinline__ int nb_get(const int *nb, const int *ovf, int i, int m, int q) {
    const int *row = nb + (size_t)i * kNbStride;
    if (m <= kNbStride || q < kNbStride - 1) return row[q];
    return ovf[(size_t)row[kNbStride - 1] + (q - (kNbStride - 1))];
}

__global__ void compact_nb_kernel(const int *nf, const int *nb, const int *ovf, const long long *off, int n,
                                  int *out) {
    int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int lane = threadIdx.x & 31;
    if (i >= n) return;
    int m = nf[i];
    long long o = off[i];
    // ascending order of neighbour IDs: a cell of at most 32 faces (nearly
    // all) by a bitonic sort across the warp's lanes, a larger one by ranks
    if (m <= 32) {
        // signed order as unsigned: flip the sign bit; the pads sort last
        unsigned x = lane < m ? (unsigned)nb_get(nb, ovf, i, m, lane) ^ 0x80000000u : 0xffffffffu;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const unsigned y = __shfl_xor_sync(0xffffffffu, x, j);
                const bool up = (lane & k) == 0, lower = (lane & j) == 0;
                x = (lower == up) ? min(x, y) : max(x, y);
            }
        }
        if (lane < m) out[o + lane] = (int)(x ^ 0x80000000u);
        return;
    }
    for (int q = lane; q < m; q += 32) {
        int v = nb_get(nb, ovf, i, m, q);
        int rank = 0;
        for (int r = 0; r < m; r++) {
            int w = nb_get(nb, ovf, i, m, r);
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

void box_tables(unsigned tri[8], unsigned adj[8]) { build_box_tables(tri, adj); }

cudaError_t launch_cells(const CellParams &cp, int mode, int pass, int sms, cudaStream_t s, int warps) {
    if (cp.ncells <= 0) return cudaSuccess;
    warps = warps < 1 ? 4 : (warps > 8 ? 8 : warps);   // the clipping translation units clamp further
    return mode == VGPU_FP64 ? launch_cells_fp64(cp, pass, sms, s, warps) : launch_cells_mixed(cp, pass, sms, s, warps);
}

cudaError_t launch_cells_batch(const BatchParams &bp, int mode, int pass, int sms, cudaStream_t s) {
    if (bp.ncells <= 0) return cudaSuccess;
    return mode == VGPU_FP64 ? launch_cells_batch_fp64(bp, pass, sms, s) : launch_cells_batch_mixed(bp, pass, sms, s);
}

cudaError_t launch_nf_to_ll(const int *nf, long long *out, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    nf_to_ll_kernel<<<(n + 255) / 256, 256, 0, s>>>(nf, out, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_compact_neighbors(const int *nf, const int *nb, const int *ovf, const long long *off, int n,
                                     int *out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    compact_nb_kernel<<<(n + 7) / 8, 256, 0, s>>>(nf, nb, ovf, off, n, out);
    note_launch();
    return cudaGetLastError();
}

namespace {

// A cell of max vertex distance R can be cut only by particles within its
// reach, 2R (R + sqrt(R^2 + rmax^2) for radical cells: a cutting particle j
// has |v - q_j|^2 < R^2 + r_j^2 at some vertex v); all of those are stored
// when the reach stays inside the ghost layers along y and z (x wraps).
__global__ void reach_check_kernel(Geometry g, int n, const double *pos, const double *mr2, const int *flags,
                                   int *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(flags[i] & VGPU_CELL_OK)) return;
    const double R = sqrt(mr2[i]);
    const double reach = (g.poly ? R + sqrt(R * R + g.rmax * g.rmax) : 2.0 * R) * (1.0 + 1e-9) +
                         1e-12 * (g.len[1] + g.len[2]);
    bool inside = true;
    for (int a = 1; a < 3; a++) {
        const double p = pos[3 * i + a];
        inside = inside && p - reach >= g.lo[a] && p + reach <= g.lo[a] + g.ext[a];
    }
    if (!inside) atomicExch(out, 1);
}

}  // namespace

cudaError_t launch_reach_check(const Geometry &g, int n, const double *pos, const double *mr2, const int *flags,
                               int *out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    reach_check_kernel<<<(n + 255) / 256, 256, 0, s>>>(g, n, pos, mr2, flags, out);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_sum_volumes(const double *vol, const int *flags, int n, double *out, cudaStream_t s) {
    sum_volumes_kernel<<<64, 256, 0, s>>>(vol, flags, n, out);
    note_launch();
    return cudaGetLastError();
}

}  // namespace vgpu
