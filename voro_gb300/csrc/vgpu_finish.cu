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

// Warp sums of four values with few FP64 additions (the FP64 pipe bounds the
// finish kernel): halves of the warp first fold different pairs, then
// quarters different singles, then each quarter folds its own; the four sums
// end in lanes 0, 8, 16, 24 and are broadcast.  Fixed order: deterministic.
__device__ __forceinline__ void warp_sum4(double &a, double &b, double &c, double &d, int lane) {
    const bool lo = lane < 16;
    double k0 = lo ? a : c, k1 = lo ? b : d;
    const double s0 = lo ? c : a, s1 = lo ? d : b;
    k0 += __shfl_xor_sync(kFull, s0, 16);
    k1 += __shfl_xor_sync(kFull, s1, 16);
    const bool lo8 = (lane & 8) == 0;
    double k = lo8 ? k0 : k1;
    k += __shfl_xor_sync(kFull, lo8 ? k1 : k0, 8);
    k += __shfl_xor_sync(kFull, k, 4);
    k += __shfl_xor_sync(kFull, k, 2);
    k += __shfl_xor_sync(kFull, k, 1);
    a = __shfl_sync(kFull, k, 0);
    b = __shfl_sync(kFull, k, 8);
    c = __shfl_sync(kFull, k, 16);
    d = __shfl_sync(kFull, k, 24);
}

// Warp maximum of non-negative doubles by their bit patterns (ordered like
// the values), on the integer reduction unit instead of the FP64 pipe.
__device__ __forceinline__ double warp_max_nonneg(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned mhi = __reduce_max_sync(kFull, hi);
    const unsigned mlo = __reduce_max_sync(kFull, hi == mhi ? lo : 0u);
    return __longlong_as_double((long long)(((unsigned long long)mhi << 32) | mlo));
}

__device__ __forceinline__ double rec_double(const unsigned *w) {
    return __longlong_as_double((long long)((unsigned long long)w[0] | ((unsigned long long)w[1] << 32)));
}

// The reductions of cell k (engine order) from its record, if it has one.
template <int MODE>
__device__ __forceinline__ void finish_record(const CellParams &P, FinishShared &F, int k, int lane) {
    constexpr int VW = MODE == VGPU_FP64 ? 6 : 3;
    constexpr int SL = kFinMaxV / 32;
    const unsigned long long off = P.rec_off[k];
    if (off == kNoRecord) return;
    const unsigned *R = P.rec + off;
    const int nv = (int)R[0], nf = (int)R[1];
    const unsigned fl = R[2];
    const unsigned *rv = R + kRecHeader;
    const unsigned *rp = rv + (2 + VW) * nv;
    const double4 me = P.a.p64[k];
    const int out = P.a.outpos[k];
    // planes: neighbour IDs (plane order), sources, FP64 planes
    for (int q = lane; q < nf; q += 32) {
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
        const int t = lane + 32 * s;
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
    const double c0x = __shfl_sync(kFull, vx[0], 0);
    const double c0y = __shfl_sync(kFull, vy[0], 0);
    const double c0z = __shfl_sync(kFull, vz[0], 0);
    int ne = 0;
    unsigned own[SL];
#pragma unroll
    for (int s = 0; s < SL; s++) {
        own[s] = 0;
        const int t = lane + 32 * s;
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
    const int eincl = warp_incl_scan(ne, lane);
    const int etot = __shfl_sync(kFull, eincl, 31);
    {
        int q = eincl - ne;
#pragma unroll
        for (int s = 0; s < SL; s++)
#pragma unroll
            for (int e = 0; e < 3; e++)
                if ((own[s] >> e) & 1u) F.stage[q++] = (unsigned)(lane + 32 * s) | ((unsigned)e << 8);
    }
    __syncwarp();
    // sum over edges (t,u) of (p_y - p_x).(v_t x v_u), p_f a vertex of face f
    double vs = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
    for (int i = lane; i < etot; i += 32) {
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
    warp_sum4(vs, cx, cy, cz, lane);
    mr2 = warp_max_nonneg(mr2);
    if (lane == 0) {
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
    if (P.poly != nullptr) {
        // the polytope: [nv, nf, vertices (3 nv, particle-relative), then per
        // face (plane order): neighbour ID, vertex count, vertex loop]; each
        // loop walks the face by the edges that start on it, which orders the
        // vertices clockwise seen from outside, as the reference's
        // face_vertices does (src/cell.cc:2285-2308)
        const unsigned long long need = 2ull + 6ull * (unsigned long long)nv + 2ull * (unsigned long long)nf;
        unsigned long long po = 0;
        if (lane == 0) po = atomicAdd(P.poly_used, need);
        po = __shfl_sync(kFull, po, 0);
        if (po + need <= P.poly_cap) {
            double *D = P.poly + po;
            if (lane == 0) {
                D[0] = (double)nv;
                D[1] = (double)nf;
            }
#pragma unroll
            for (int s = 0; s < SL; s++) {
                const int t = lane + 32 * s;
                if (t < nv) {
                    D[2 + 3 * t] = vx[s];
                    D[3 + 3 * t] = vy[s];
                    D[4 + 3 * t] = vz[s];
                }
            }
            double *DF = D + 2 + 3 * nv;
            for (int q0 = 0; q0 < nf; q0 += 32) {
                const int q = q0 + lane;
                const int ord = q < nf ? F.ford[q] : 0;
                // faces before q: q0 * 2 header words plus their orders
                int before = 0;
                for (int j = 0; j < q0; j++) before += F.ford[j];
                const int incl = warp_incl_scan(ord, lane);
                if (q < nf) {
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
            if (lane == 0) P.poly_off[out] = (long long)po;
        } else if (lane == 0) {
            P.poly_off[out] = -2;   // store full
        }
    }
    __syncwarp();
}

template <int MODE>
__global__ void __launch_bounds__(128) finish_kernel(const __grid_constant__ CellParams P) {
    __shared__ FinishShared fsh[4];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * 4;
    for (int k = blockIdx.x * 4 + wid; k < P.ncells; k += nwarps) finish_record<MODE>(P, fsh[wid], k, lane);
}

// The same over the cells of a batch (global numbering as cell_batch_kernel).
template <int MODE>
__global__ void __launch_bounds__(128) finish_batch_kernel(const __grid_constant__ BatchParams B) {
    __shared__ FinishShared fsh[4];
    __shared__ __align__(16) unsigned char cpw[4][(sizeof(CellParams) + 15) & ~(size_t)15];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    CellParams &P = *reinterpret_cast<CellParams *>(cpw[wid]);
    const long long nwarps = (long long)gridDim.x * 4;
    long long cbeg = 0, cend = 0;
    for (long long g = (long long)blockIdx.x * 4 + wid; g < B.ncells; g += nwarps) {
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
        finish_record<MODE>(P, fsh[wid], (int)(g - cbeg), lane);
    }
}

}  // namespace

template <int MODE>
cudaError_t launch_finish_t(const CellParams &cp, int sms, cudaStream_t s) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, finish_kernel<MODE>, 128, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sms * per_sm;
    const long long need = (cp.ncells + 3) / 4;
    const int grid = (int)(want < need ? want : need);
    finish_kernel<MODE><<<grid, 128, 0, s>>>(cp);
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
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, finish_batch_kernel<MODE>, 128, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sms * per_sm;
    const long long need = (bp.ncells + 3) / 4;
    const int grid = (int)(want < need ? want : need);
    finish_batch_kernel<MODE><<<grid, 128, 0, s>>>(bp);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_finish_batch(const BatchParams &bp, int mode, int sms, cudaStream_t s) {
    if (bp.ncells <= 0) return cudaSuccess;
    return mode == VGPU_FP64 ? launch_finish_batch_t<VGPU_FP64>(bp, sms, s)
                             : launch_finish_batch_t<VGPU_MIXED>(bp, sms, s);
}

}  // namespace vgpu
