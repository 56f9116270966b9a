// Device scan and stable LSD radix sort used by binning (put() into blocks).
//
// The reference appends particles to per-block arrays in put() order
// (src/container.cc:90-111, add_particle_memory 305-326); its loop order is
// block-major, insertion order inside a block (src/c_loops.hh:165-210).  A
// stable sort by block index reproduces exactly that order.
#include "vgpu_internal.cuh"

namespace vgpu {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__global__ void scan_tiles_kernel(const T *in, T *out, T *tile_sums, int n) {
    __shared__ T warp_tot[kScanThreads / 32];
    const int tile0 = blockIdx.x * kScanTile;
    T v[kScanItems];
    T run = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        int idx = tile0 + threadIdx.x * kScanItems + i;
        T x = idx < n ? in[idx] : T(0);
        v[i] = run;
        run += x;
    }
    // warp inclusive scan of per-thread totals
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T w = lane < kScanThreads / 32 ? warp_tot[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = wi - w;  // exclusive
        if (lane == kScanThreads / 32 - 1 && tile_sums) tile_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    T base = warp_tot[wid] + incl - run;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        int idx = tile0 + threadIdx.x * kScanItems + i;
        if (idx < n) out[idx] = base + v[i];
    }
}

template <typename T>
__global__ void scan_add_kernel(T *out, const T *tile_offsets, int n) {
    int tile = blockIdx.x;
    T add = tile_offsets[tile];
    int tile0 = tile * kScanTile;
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
        int idx = tile0 + i;
        if (idx < n) out[idx] += add;
    }
}

template <typename T>
cudaError_t scan_rec(const T *in, T *out, int n, T *tmp, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 1) {
        scan_tiles_kernel<T><<<1, kScanThreads, 0, s>>>(in, out, nullptr, n);
        note_launch();
        return cudaGetLastError();
    }
    T *sums = tmp;
    T *sums_scanned = tmp + tiles;
    scan_tiles_kernel<T><<<tiles, kScanThreads, 0, s>>>(in, out, sums, n);
    note_launch();
    cudaError_t e = scan_rec<T>(sums, sums_scanned, tiles, tmp + 2 * tiles, s);
    if (e != cudaSuccess) return e;
    scan_add_kernel<T><<<tiles, kScanThreads, 0, s>>>(out, sums_scanned, n);
    note_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------- radix sort
constexpr int kSortWarps = 8;
constexpr int kSortPerWarp = 256;
constexpr int kSortTile = kSortWarps * kSortPerWarp;  // 2048

__global__ void radix_hist_kernel(const unsigned *keys, int n, int shift, int *hist, int ntiles) {
    __shared__ int h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    int tile0 = blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        int idx = tile0 + i;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d * ntiles + blockIdx.x] = h[d];
}

__global__ void radix_scatter_kernel(const unsigned *keys, const int *vals, unsigned *okeys, int *ovals,
                                     int n, int shift, const int *hist_scanned, int ntiles) {
    __shared__ int cnt[kSortWarps][256];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSortWarps * 256; i += blockDim.x) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile + wid * kSortPerWarp;
    const unsigned lt = (1u << lane) - 1u;
    // pass 1: per-warp digit counts, in order
    for (int c = 0; c < kSortPerWarp; c += 32) {
        int idx = base + c + lane;
        bool ok = idx < n;
        unsigned act = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            unsigned d = (keys[idx] >> shift) & 255u;
            unsigned peers = __match_any_sync(act, d);
            int leader = 31 - __clz(peers);
            if (lane == leader) cnt[wid][d] += __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // per digit: turn counts into global bases, warps in order
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        int run = hist_scanned[d * ntiles + blockIdx.x];
        for (int w = 0; w < kSortWarps; w++) {
            int t = cnt[w][d];
            cnt[w][d] = run;
            run += t;
        }
    }
    __syncthreads();
    // pass 2: stable scatter
    for (int c = 0; c < kSortPerWarp; c += 32) {
        int idx = base + c + lane;
        bool ok = idx < n;
        unsigned act = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            unsigned k = keys[idx];
            unsigned d = (k >> shift) & 255u;
            unsigned peers = __match_any_sync(act, d);
            int pos = cnt[wid][d] + __popc(peers & lt);
            okeys[pos] = k;
            ovals[pos] = vals[idx];
            __syncwarp(act);
            int leader = 31 - __clz(peers);
            if (lane == leader) cnt[wid][d] += __popc(peers);
        }
        __syncwarp();
    }
}

}  // namespace

size_t scan_tmp_ints(int n) {
    size_t total = 0;
    int m = n;
    while (m > kScanTile) {
        int tiles = (m + kScanTile - 1) / kScanTile;
        total += 2 * (size_t)tiles;
        m = tiles;
    }
    return total + 16;
}

cudaError_t exclusive_scan_int(const int *in, int *out, int n, int *tmp, size_t tmp_ints, cudaStream_t s) {
    if (tmp_ints < scan_tmp_ints(n)) return cudaErrorInvalidValue;
    return scan_rec<int>(in, out, n, tmp, s);
}

cudaError_t exclusive_scan_ll(const long long *in, long long *out, int n, long long *tmp, cudaStream_t s) {
    return scan_rec<long long>(in, out, n, tmp, s);
}

size_t radix_hist_ints(int n) {
    int ntiles = (n + kSortTile - 1) / kSortTile;
    return (size_t)256 * (ntiles > 0 ? ntiles : 1);
}

cudaError_t radix_sort_pairs(unsigned *keys, int *vals, unsigned *keys_alt, int *vals_alt, int n,
                             int key_bits, int *hist, size_t hist_ints, int *scan_tmp, size_t scan_tmp_n,
                             cudaStream_t s, bool *result_in_alt) {
    *result_in_alt = false;
    if (n <= 1) return cudaSuccess;
    int ntiles = (n + kSortTile - 1) / kSortTile;
    if (hist_ints < (size_t)256 * ntiles) return cudaErrorInvalidValue;
    unsigned *k0 = keys, *k1 = keys_alt;
    int *v0 = vals, *v1 = vals_alt;
    bool alt = false;
    for (int shift = 0; shift < key_bits; shift += 8) {
        radix_hist_kernel<<<ntiles, 256, 0, s>>>(k0, n, shift, hist, ntiles);
        note_launch();
        cudaError_t e = exclusive_scan_int(hist, hist, 256 * ntiles, scan_tmp, scan_tmp_n, s);
        if (e != cudaSuccess) return e;
        radix_scatter_kernel<<<ntiles, kSortWarps * 32, 0, s>>>(k0, v0, k1, v1, n, shift, hist, ntiles);
        note_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        unsigned *tk = k0; k0 = k1; k1 = tk;
        int *tv = v0; v0 = v1; v1 = tv;
        alt = !alt;
    }
    *result_in_alt = alt;
    return cudaSuccess;
}

}  // namespace vgpu
