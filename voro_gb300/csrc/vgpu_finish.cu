// The FP64 finish kernel: volume, centroid, neighbours and the optional
// polytope of every cell from the records the clipping kernels write.
#include "vgpu_dev.cuh"

namespace vgpu {

namespace {

// ------------------------------------------------------------------ finish
// The FP64 reductions of every cell from the compact record its clipping
// kernel wrote (layout in CellParams).  They run as a separate kernel so that
// the clipping loop keeps the instruction cache to itself.  Vertices: the
// MIXED engine's FP32 vertices get one FP64 residual correction against their
// three FP64 planes (refine_vertex_rec); the FP64 engine's are used as they
// are.  Volume and centroid: FP64 sums over edges relative to vertex 0 with
// each face's reference point one of its own vertices (the edge formula holds
// for any point of the face).  Optionally the polytope itself is written out.
constexpr int kFinMaxV = 128;   // vertices (the 128-slot engine's capacity)
constexpr int kFinMaxE = 192;   // edges (3 * kFinMaxV / 2)

struct FinishShared {
    unsigned tri[kFinMaxV];
    unsigned adj[kFinMaxV];
    int psrc[kMaxPlanes], pshift[kMaxPlanes];
    int rep[kMaxPlanes];             // per face: its lowest vertex
    int ford[kMaxPlanes];            // per face: its vertex count
    double4 pl64[kMaxPlanes];
    float4 pn[kMaxPlanes];           // the FP64 plane normals rounded to FP32
    double vx[kFinMaxV], vy[kFinMaxV], vz[kFinMaxV];   // FP64 vertices relative to c0
    unsigned stage[kFinMaxE];        // owned edges (t < u)
};

__device__ __forceinline__ double4 plane64_rec(const CellParams &P, const FinishShared &F, double4 me, int p) {
    const int src = F.psrc[p];
    if (src >= 0) return plane64_from(P, me, src, F.pshift[p]);
    return face64(P, me, F.pshift[p]);
}

// refine_vertex_f64 with the planes' FP32 normals taken from F.pn (rounded
// once per plane rather than once per vertex and plane).
__device__ __forceinline__ double3 refine_vertex_rec(const FinishShared &F, unsigned t, float fx, float fy, float fz) {
    const int ia = tri_plane(t, 0), ib = tri_plane(t, 1), ic = tri_plane(t, 2);
    const double4 A = F.pl64[ia], B = F.pl64[ib], Cq = F.pl64[ic];
    const float4 a = F.pn[ia], b = F.pn[ib], c = F.pn[ic];
    const double x = fx, y = fy, z = fz;
    const double ra = A.w - fma(A.x, x, fma(A.y, y, A.z * z));
    const double rb = B.w - fma(B.x, x, fma(B.y, y, B.z * z));
    const double rc = Cq.w - fma(Cq.x, x, fma(Cq.y, y, Cq.z * z));
    const float bcx = b.y * c.z - b.z * c.y, bcy = b.z * c.x - b.x * c.z, bcz = b.x * c.y - b.y * c.x;
    const float cax = c.y * a.z - c.z * a.y, cay = c.z * a.x - c.x * a.z, caz = c.x * a.y - c.y * a.x;
    const float abx = a.y * b.z - a.z * b.y, aby = a.z * b.x - a.x * b.z, abz = a.x * b.y - a.y * b.x;
    const float D = a.x * bcx + a.y * bcy + a.z * bcz;
    const float scale = (fabsf(a.x) + fabsf(a.y) + fabsf(a.z)) * (fabsf(b.x) + fabsf(b.y) + fabsf(b.z)) *
                        (fabsf(c.x) + fabsf(c.y) + fabsf(c.z));
    double3 v;
    if (fabsf(D) > 1e-3f * scale) {
        const float fra = (float)ra, frb = (float)rb, frc = (float)rc;
        const float inv = 1.0f / D;
        v.x = x + (double)((fra * bcx + frb * cax + frc * abx) * inv);
        v.y = y + (double)((fra * bcy + frb * cay + frc * aby) * inv);
        v.z = z + (double)((fra * bcz + frb * caz + frc * abz) * inv);
    } else {
        double DD;
        float kn;
        solve_f64(A, B, Cq, v.x, v.y, v.z, DD, kn);
    }
    return v;
}

// Sums of four values over a group of G lanes (G = 32 or 16) with few FP64
// additions (the FP64 pipe bounds the finish kernel): halves of the group
// first fold different pairs, then quarters different singles, then each
// quarter folds its own; the four sums end in the group's lanes 0, G/4, G/2,
// 3G/4 and are broadcast.  Fixed order: deterministic.
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
__device__ __forceinline__ void finish_record(const CellParams &P, FinishShared &F, int k, int gl) {
    constexpr int VW = MODE == VGPU_FP64 ? 6 : 3;
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
    // planes: neighbour IDs (plane order), sources, FP64 planes
    for (int q = gl; q < nf; q += G) {
        F.psrc[q] = (int)rp[q];
        F.pshift[q] = (int)rp[nf + q];
        F.rep[q] = 0x7fffffff;
        F.ford[q] = 0;
        P.r.nb[(size_t)out * kMaxNb + q] = (int)rp[2 * nf + q];
        const double4 pl = plane64_rec(P, F, me, q);
        F.pl64[q] = pl;
        F.pn[q] = make_float4((float)pl.x, (float)pl.y, (float)pl.z, 0.0f);
    }
    __syncwarp();
    unsigned tri[SL];
    double vx[SL], vy[SL], vz[SL];
    double mr2 = 0.0;
#pragma unroll
    for (int s = 0; s < SL; s++) {
        const int t = gl + G * s;
        tri[s] = 0;
        vx[s] = vy[s] = vz[s] = 0.0;
        if (t < nv) {
            tri[s] = rv[t];
            F.tri[t] = tri[s];
            F.adj[t] = rv[nv + t];
            if (MODE == VGPU_FP64) {
                vx[s] = rec_double(rv + 2 * nv + 2 * t);
                vy[s] = rec_double(rv + 4 * nv + 2 * t);
                vz[s] = rec_double(rv + 6 * nv + 2 * t);
            } else {
                const double3 r = refine_vertex_rec(F, tri[s], __uint_as_float(rv[2 * nv + t]),
                                                    __uint_as_float(rv[3 * nv + t]), __uint_as_float(rv[4 * nv + t]));
                vx[s] = r.x;
                vy[s] = r.y;
                vz[s] = r.z;
            }
            mr2 = fmax(mr2, vx[s] * vx[s] + vy[s] * vy[s] + vz[s] * vz[s]);
#pragma unroll
            for (int e = 0; e < 3; e++) {
                atomicMin(&F.rep[tri_plane(tri[s], e)], t);
                atomicAdd(&F.ford[tri_plane(tri[s], e)], 1);
            }
        }
    }
    // origin of the sums: vertex 0
    const double c0x = __shfl_sync(kFull, vx[0], 0, G);
    const double c0y = __shfl_sync(kFull, vy[0], 0, G);
    const double c0z = __shfl_sync(kFull, vz[0], 0, G);
    int ne = 0;
    unsigned own[SL];
#pragma unroll
    for (int s = 0; s < SL; s++) {
        own[s] = 0;
        const int t = gl + G * s;
        if (t < nv) {
            F.vx[t] = vx[s] - c0x;
            F.vy[t] = vy[s] - c0y;
            F.vz[t] = vz[s] - c0z;
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
    for (int i = gl; i < etot; i += G) {
        const unsigned E = F.stage[i];
        const int t = E & 255u, e = E >> 8;
        const unsigned T = F.tri[t];
        const int u = (F.adj[t] >> (8 * e)) & 255u;
        const int rx = F.rep[tri_plane(T, e)], ry = F.rep[tri_plane(T, e == 2 ? 0 : e + 1)];
        const double tx = F.vx[t], ty = F.vy[t], tz = F.vz[t];
        const double ux = F.vx[u], uy = F.vy[u], uz = F.vz[u];
        const double wx = ty * uz - tz * uy;
        const double wy = tz * ux - tx * uz;
        const double wz = tx * uy - ty * ux;
        const double ax = F.vx[rx], ay = F.vy[rx], az = F.vz[rx];
        const double bx = F.vx[ry], by = F.vy[ry], bz = F.vz[ry];
        const double dy = bx * wx + by * wy + bz * wz;
        const double dx = ax * wx + ay * wy + az * wz;
        const double dd = dy - dx;
        vs += dd;
        cx += dd * (tx + ux) + dy * bx - dx * ax;
        cy += dd * (ty + uy) + dy * by - dx * ay;
        cz += dd * (tz + uz) + dy * bz - dx * az;
    }
    group_sum4<G>(vs, cx, cy, cz, gl);
    mr2 = group_max_nonneg<G>(mr2);
    if (have && gl == 0) {
        const double vol = vs / 6.0;
        P.r.vol[out] = vol;
        if (48.0 * vol > P.g.tol_cu) {   // src/cell.cc:1895
            const double f = 1.0 / (4.0 * vs);
            P.r.cen[3 * out] = c0x + cx * f;
            P.r.cen[3 * out + 1] = c0y + cy * f;
            P.r.cen[3 * out + 2] = c0z + cz * f;
        } else {
            P.r.cen[3 * out] = P.r.cen[3 * out + 1] = P.r.cen[3 * out + 2] = 0.0;
        }
        P.r.nf[out] = nf;
        P.r.nv[out] = nv;
        P.r.maxr2[out] = mr2;
        P.r.flags[out] = VGPU_CELL_OK | (int)fl;
    }
    if (P.poly != nullptr) {   // (uniform: P is the same for both halves of a warp)
        // the polytope: [nv, nf, vertices (3 nv, particle-relative), then per
        // face (plane order): neighbour ID, vertex count, vertex loop]; each
        // loop walks the face by the edges that start on it, which orders the
        // vertices clockwise seen from outside, as the reference's
        // face_vertices does (src/cell.cc:2285-2308)
        const unsigned long long need = 2ull + 6ull * (unsigned long long)nv + 2ull * (unsigned long long)nf;
        unsigned long long po = 0;
        if (have && gl == 0) po = atomicAdd(P.poly_used, need);
        po = __shfl_sync(kFull, po, 0, G);
        const bool fits = have && po + need <= P.poly_cap;
        double *D = P.poly + (fits ? po : 0);
        if (fits) {
            if (gl == 0) {
                D[0] = (double)nv;
                D[1] = (double)nf;
            }
#pragma unroll
            for (int s = 0; s < SL; s++) {
                const int t = gl + G * s;
                if (t < nv) {
                    D[2 + 3 * t] = vx[s];
                    D[3 + 3 * t] = vy[s];
                    D[4 + 3 * t] = vz[s];
                }
            }
        }
        // face loops; the loop over face chunks runs the same number of times
        // in both halves, because it holds a group scan
        double *DF = D + 2 + 3 * nv;
        const int nfmax = __reduce_max_sync(kFull, fits ? nf : 0);
        for (int q0 = 0; q0 < nfmax; q0 += G) {
            const int q = q0 + gl;
            const bool mine = fits && q < nf;
            const int ord = mine ? F.ford[q] : 0;
            // faces before q: q * 2 header words plus their orders
            int before = 0;
            if (fits)
                for (int j = 0; j < q0 && j < nf; j++) before += F.ford[j];
            const int incl = group_incl_scan<G>(ord, gl);
            if (mine) {
                double *df = DF + 2 * q + before + (incl - ord);
                df[0] = (double)P.r.nb[(size_t)out * kMaxNb + q];
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
        if (fits) {
            if (gl == 0) P.poly_off[out] = (long long)po;
        } else if (have && gl == 0) {
            P.poly_off[out] = -2;   // store full
        }
    }
    __syncwarp();
}

constexpr int kFinWarps = 2;   // warps per CTA (two cell slots per warp)

// Two cells per warp, one per 16-lane half, when both have at most 64
// vertices (nearly always: their FP64 work then fills the lanes better);
// otherwise the whole warp does one cell after the other.
template <int MODE>
__device__ __forceinline__ void finish_pair(const CellParams &P, FinishShared *F2, int k0, int k1, int lane) {
    const int half = lane >> 4, gl = lane & 15;
    const int mine = half ? k1 : k0;
    int nv = 0;
    if (mine >= 0) {
        const unsigned long long off = P.rec_off[mine];
        if (off != kNoRecord) nv = (int)P.rec[off];
    }
    if (!__any_sync(kFull, nv > 64)) {
        finish_record<MODE, 16>(P, F2[half], mine, gl);
    } else {
        finish_record<MODE, 32>(P, F2[0], k0, lane);
        finish_record<MODE, 32>(P, F2[0], k1, lane);
    }
}

template <int MODE>
__global__ void __launch_bounds__(32 * kFinWarps) finish_kernel(const __grid_constant__ CellParams P) {
    __shared__ FinishShared fsh[kFinWarps][2];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int npairs = (P.ncells + 1) / 2;
    for (int pi = blockIdx.x * kFinWarps + wid; pi < npairs; pi += gridDim.x * kFinWarps) {
        const int i0 = 2 * pi, i1 = 2 * pi + 1;
        const int k0 = P.cell_list ? P.cell_list[i0] : i0;
        const int k1 = i1 < P.ncells ? (P.cell_list ? P.cell_list[i1] : i1) : -1;
        finish_pair<MODE>(P, fsh[wid], k0, k1, lane);
    }
}

// The same over the cells of a batch (global numbering as cell_batch_kernel);
// a pair never straddles two containers.
template <int MODE>
__global__ void __launch_bounds__(32 * kFinWarps) finish_batch_kernel(const __grid_constant__ BatchParams B) {
    __shared__ FinishShared fsh[kFinWarps][2];
    __shared__ __align__(16) unsigned char cpw[kFinWarps][(sizeof(CellParams) + 15) & ~(size_t)15];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    CellParams &P = *reinterpret_cast<CellParams *>(cpw[wid]);
    const long long nwarps = (long long)gridDim.x * kFinWarps;
    long long cbeg = 0, cend = 0;
    for (long long g = 2 * ((long long)blockIdx.x * kFinWarps + wid); g < B.ncells; g += 2 * nwarps) {
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
        const int k0 = (int)(g - cbeg);
        const int k1 = g + 1 < cend ? (int)(g + 1 - cbeg) : -1;
        finish_pair<MODE>(P, fsh[wid], k0, k1, lane);
        if (k1 < 0 && g + 1 < B.ncells) {
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
            finish_pair<MODE>(P, fsh[wid], (int)(g1 - cbeg), -1, lane);
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
