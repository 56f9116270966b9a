// Internal types shared by the engine's translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace vgpu {

constexpr int kWarp = 32;
// Cells a warp of the clipping kernels takes from the work queue at a time by
// default, and the largest CTA they are built for (threads); both can be
// changed at build time (-D), the first also per container (vgpu_tuning).
#ifndef VGPU_CELL_CHUNK
#define VGPU_CELL_CHUNK 8
#endif
#ifndef VGPU_CTA_THREADS
#define VGPU_CTA_THREADS 128
#endif
constexpr int kDefaultCellChunk = VGPU_CELL_CHUNK;
constexpr int kBuiltCtaWarps = VGPU_CTA_THREADS / 32;
constexpr int kMaxPlanes = 64;       // plane slots per cell of the 64-vertex engines
constexpr int kMaxPlanesWide = 128;  // ... of the 128-vertex engines (cells of up to 128 live planes)
constexpr int kCandBuf = 64;
// VGPU_GATHER_TMA=1 builds the candidate gather with the block runs of each
// 64-candidate window bulk-copied (cp.async.bulk, one copy per block run,
// completed on a per-warp mbarrier) into shared memory instead of one
// float4 load per lane.  Results are identical; measured on the 4M periodic
// box the clipping passes took 103.4 ms against 80.1 ms for the per-lane
// loads: a window's copies are a round trip the warp waits out whole, while
// the loads overlap the distance arithmetic and the other warps.  Off.
#ifndef VGPU_GATHER_TMA
#define VGPU_GATHER_TMA 0
#endif
constexpr int kStageEntries = 64;   // staged candidate particles per warp (VGPU_GATHER_TMA)       // candidate buffer entries per warp
// Neighbour IDs: kNbStride slots per cell in a fixed-stride array; a cell with
// more faces keeps kNbStride-1 there and the rest in an overflow store, whose
// offset takes the row's last slot.
constexpr int kNbStride = 32;
constexpr int kOffsetRadius = 4;   // engine search table covers Chebyshev radius <= 4
constexpr int kTableLb2Max = 15;   // ... and lower-bound shells lb2 <= 15 (complete there)
// Beyond the table the search walks Chebyshev shells of blocks: the 64-slot
// engines up to kNarrowShellRadius (they hand a cell that reaches further to
// the next engine), the 128-slot engines up to kMaxShellRadius (a cell
// reaching further fails with VGPU_FAIL_SEARCH).  A candidate's block offset
// travels packed in 10 bits per axis, offset by kShellPack.
constexpr int kNarrowShellRadius = 40;
constexpr int kMaxShellRadius = 500;
constexpr int kShellPack = 512;
constexpr int kMaxGroups = 16;

// Geometry of one container, in the reference's own terms plus the engine's
// private block grid.
struct Geometry {
    int kind;           // VGPU_CONTAINER .. VGPU_CONTAINER_PERIODIC_POLY
    int poly;           // radical (power) tessellation
    int unit_cell;      // periodic kinds: initial cell is the unit Voronoi cell
    // Sheared container_periodic (bxy, bxz or byz != 0): the y and z images
    // are stored as particles of ghost layers below and above the primary
    // domain (as container_periodic_base keeps them), so the engine grid
    // is periodic in x only and open in y and z; the initial cell is the
    // box of half extents half[] cut by the unit cell's face planes.
    int tric;
    int per[3];         // periodic flags per axis (of the engine grid)
    double lo[3];       // engine region lower corner (container: ax,ay,az; periodic kinds: 0, or the ghost layers' lower corner)
    double len[3];      // domain lengths (bx-ax, ...); periodic kinds: bx, by, bz
    double hi[3];       // domain upper corner as given (bx, by, bz)
    double ext[3];      // engine region extents from lo (len, or with the ghost layers)
    double shear[3];    // bxy, bxz, byz (periodic kinds)
    double half[3];     // unit_cell kinds: half extents of the initial box
    // reference block grid: loop order and put_remap semantics
    int un[3];          // nx, ny, nz
    double ubox[3];     // boxx = (bx-ax)/nx  (src/container.cc:31)
    double usp[3];      // xsp = 1/boxx       (src/v_base.cc:26)
    // engine block grid
    int gn[3];
    double gbs[3];      // engine block sizes
    float gbs32[3];
    float gbs_h[3], gbs_l[3];   // engine block sizes as float pairs (h + l)
    float gbs_min;
    float gbs_max;
    double tol_h;       // half the reference tolerance: 0.5*10*DBL_EPSILON*max_len_sq
    float tol_h32;      // the same rounded up to FP32 (the FP32 side tests' band)
    double tol_cu;      // reference tol_cu (centroid threshold, src/cell.cc:25)
    double rmax;        // largest radius (poly kinds)
    float rmax32;
};

// Particles in engine order (sorted by engine block).
struct EngineArrays {
    const double4 *p64;   // remapped position + radius (double)
    const float4 *l32;    // position local to its engine block + radius (float)
    const float4 *lffh;   // the same as float pairs: high parts (the same array as l32)
    const float4 *lffl;   // ... and low parts (finish kernel)
    const int *pid;       // particle id
    const int *outpos;    // slot of this particle in the loop-order result arrays
    const int *gblock;    // engine block index of this particle
    const int *bstart;    // engine block start offsets, size nblocks+1
};

struct Results {
    double *vol;
    double *cen;      // 3 per cell
    int *nf;
    int *nv;
    double *maxr2;
    int *flags;
    int *nb;          // kNbStride per cell
    int *nb_ovf;      // overflow store of the neighbour IDs (use: Counters::nb_ovf_used)
    unsigned long long nb_ovf_cap;     // its capacity (ints, < 2^31)
};

struct Counters {
    unsigned long long side_tests;
    unsigned long long fp64_repairs;
    unsigned long long planes_tested;
    unsigned long long planes_cut;
    unsigned long long deleted;
    unsigned long long marginal;
    unsigned long long overflow;   // cells appended to the overflow list
    unsigned long long work;       // work-queue counter
    unsigned long long overflow_work;
    unsigned long long failed;     // batched launches: cells that overflowed every capacity
    unsigned long long rec_used;   // words of the polytope record store in use
    unsigned long long poly_used;  // doubles of the polytope output in use
    unsigned long long nb_ovf_used;  // ints of the neighbour overflow store in use
    unsigned long long nb_failed;    // finish kernel: cells whose neighbours found it full
    unsigned long long phase_cycles[16];  // diagnostics build only (VGPU_PHASE_TIMING): 8 clocks, 8 counts
};

// A wall (src/wall.hh:25-130): the parameters as the reference's classes hold
// them, including its precomputed asi = 1/|a|^2 and the cone's tan, sin and
// cos of the angle.  Type: VGPU_WALL_* (include/vorogpu.h).
struct WallSpec {
    int type;
    int id;                 // neighbour ID of the wall's faces
    double c[3];            // centre / normal (plane: xc, yc, zc)
    double a[3];            // axis (cylinder, cone)
    double r;               // radius (sphere, cylinder), ac (plane)
    double asi, gra, sang, cang;
};
constexpr int kMaxWalls = 32;   // one lane each when they are applied
// Internal wall type: a face plane of the unit Voronoi cell of a sheared
// periodic box, n = c (the lattice vector), h = r/2 (r = |c|^2), relative to
// the particle; staged with the neighbour candidates at distance r.
constexpr int kWallLattice = 100;

struct CellParams {
    Geometry g;
    EngineArrays a;
    Results r;
    Counters *cnt;
    int ncells;             // cells to compute (engine order), or overflow list length
    const int *cell_list;   // NULL: cells cell_begin..cell_begin+ncells-1; else the list of engine indices
    int cell_begin;
    int cell_chunk;         // consecutive cells a warp takes from the queue at once (0: the built-in default)
    int *overflow_list;     // cells that overflowed this engine's capacity
    const int *offsets;     // packed search offsets (engine table), sorted by lb2
    int noffsets;
    int ngroups;
    int group_start[kMaxGroups + 1];
    int group_lb2[kMaxGroups];
    unsigned box_tri[8];    // initial box: corner triangles and neighbours
    unsigned box_adj[8];
    // The clipping kernels write each finished polytope as a record here and
    // the finish kernel does the FP64 reductions.  Record layout (32-bit words):
    // [nv, nf, flags, 0, 0, tri[nv], adj[nv], positions, psrc[nf], pshift[nf],
    //  pid[nf]] over the cell's valid vertices and live planes, renumbered
    // compactly; positions are x[nv], y[nv], z[nv] as FP32 (MIXED engine) or
    // as FP64 word pairs (FP64 engine).
    unsigned *rec;
    unsigned long long rec_cap;     // words
    unsigned long long *rec_used;   // bump allocator (words)
    unsigned long long *rec_off;    // per engine index: record offset (words), kNoRecord if none
    // Optional polytope output (written by the finish kernel), NULL: none.
    // Per cell [nv, nf, vertices (3 nv), per face: neighbour, count, loop].
    double *poly;
    unsigned long long poly_cap;    // doubles
    unsigned long long *poly_used;  // bump allocator (doubles)
    long long *poly_off;            // per loop-order cell: offset, -1 none, -2 store full
    // Walls cut every cell after its initial box, in order (apply_walls,
    // src/container.hh:86-89); as planes their slots have source -1 and
    // shift 6 + wall index.
    const WallSpec *walls;
    int nwalls;
};
constexpr unsigned long long kNoRecord = ~0ull;

constexpr int kRecHeader = 5;

// Many containers in one persistent launch: cells are numbered globally,
// container c owning [cell_start[c], cell_start[c+1]).
struct BatchParams {
    const CellParams *cps;          // per-container parameters (device array)
    const long long *cell_start;    // ncont + 1 prefix sums of cells
    int ncont;
    long long ncells;               // cells in this pass
    long long cell_begin;           // cell_list NULL: global cells cell_begin .. cell_begin+ncells-1
    const long long *cell_list;     // else their global indices
    long long *overflow_list;       // first pass: cells that need the larger engine; NULL: rerun
    unsigned long long *overflow_count;
    unsigned long long *work;       // work-queue counter (starts at 0)
    const int *offsets;             // the engine's offset table (same for every container)
    int noffsets;
};

// launch accounting (vgpu_api.cu)
void note_launch(int n = 1);
long long launch_count();
// sets the message vgpu_last_error returns; returns code
int report_error(int code, const char *fmt, ...);

// vgpu_sort.cu
cudaError_t exclusive_scan_int(const int *in, int *out, int n, int *tmp, size_t tmp_ints, cudaStream_t s);
size_t scan_tmp_ints(int n);
cudaError_t radix_sort_pairs(unsigned *keys, int *vals, unsigned *keys_alt, int *vals_alt, int n,
                             int key_bits, int *hist, size_t hist_ints, int *scan_tmp, size_t scan_tmp_n,
                             cudaStream_t s, bool *result_in_alt);
size_t radix_hist_ints(int n);

// vgpu_bin.cu
struct BinParams {
    Geometry g;
    int n;
    const int *ids_in;
    const double4 *xyzr_in;
    double4 *rem;        // remapped positions (input order)
    unsigned *ukey;      // loop-order key (reference block, or 0xffffffff dropped)
    unsigned *gkey;      // engine block key
    int *idx;            // identity 0..n-1
};
cudaError_t launch_remap(const BinParams &bp, int *kept, unsigned long long *rmax_bits, cudaStream_t s);
cudaError_t launch_first_nonfinite(const double *xyzr, long long n, bool poly, unsigned long long *first,
                                   cudaStream_t s);
// nkept particles in loop order (uorder) and nengine engine entries in engine
// order (gorder; an index i >= nin is image i - nin of particle img_src[i - nin])
cudaError_t launch_gather(const Geometry &g, int nkept, int nengine, int nin, const int *img_src,
                          const int *uorder, const int *gorder,
                          const unsigned *gkey_sorted, const double4 *rem, const int *ids_in,
                          int *outpos_by_input, double4 *p64, float4 *lffh, float4 *lffl,
                          int *pid, int *outpos,
                          int *gblock, int *bstart, int nblocks, int *res_ids, double *res_pos,
                          double *res_rad, cudaStream_t s);
// Sheared periodic boxes: the images of the n particles (remapped positions
// rem) that lie in the ghost layers; count per particle, then written from
// their offsets (exclusive scan of the counts) to rem_out/gkey_out/idx_out at
// nin + offset, with their source particle in img_src.
cudaError_t launch_image_count(const Geometry &g, int n, const double4 *rem, int *count, cudaStream_t s);
cudaError_t launch_image_write(const Geometry &g, int n, const double4 *rem, const int *offset, int nin,
                               double4 *rem_out, unsigned *gkey_out, int *idx_out, int *img_src, cudaStream_t s);
// The engine indices of the particles (not images), in engine order (flag and
// slot: nengine ints of scratch each; scan_tmp: scratch of exclusive_scan_int).
cudaError_t launch_cell_list(const int *outpos, int nengine, int *list, int *flag, int *slot, int *scan_tmp,
                             size_t scan_tmp_ints_avail, cudaStream_t s);
// One small container's binning in one CTA (batches): at most kSmallBinMax
// particles, sorted in shared memory (12 bytes per particle, rounded up to a
// power of two).  Members of at most kSmallBinTier particles go in a launch
// of 48 KB CTAs, the larger ones in a launch of 192 KB CTAs.
constexpr int kSmallBinMax = 16384;
constexpr int kSmallBinTier = 4096;
constexpr int kSmallBinThreads = 512;
struct SmallBinJob {
    Geometry g;
    int n, nub, nblocks;
    const int *ids_in;
    const double4 *xyzr_in;
    double4 *rem;
    int *outpos_in;
    double4 *p64;
    float4 *lffh, *lffl;
    int *pid, *outpos, *gblock, *bstart;
    int *res_ids;
    double *res_pos, *res_rad;
    unsigned long long *result;   // [0] kept | duplicate << 32, [1] largest radius (bits)
};
// jobs of at most cap particles each (cap a power of two, <= kSmallBinMax)
cudaError_t launch_small_bin(const SmallBinJob *jobs, int njobs, int cap, cudaStream_t s);
cudaError_t launch_ghost_setup(const Geometry &g, int n, const double4 *q, int base, double4 *p64, float4 *lffh,
                               float4 *lffl, int *pid, int *outpos, int *gblock, int *keep, cudaStream_t s);
cudaError_t launch_duplicate_check(const unsigned *ukey_sorted, const int *uorder, const double4 *rem,
                                   int nkept, int *dup_flag, cudaStream_t s);

// vgpu_cell.cu, vgpu_finish.cu
cudaError_t launch_cells(const CellParams &cp, int mode, int pass, int sms, cudaStream_t s, int warps = 4);
// vgpu_clip_mixed.cu, vgpu_clip_fp64.cu
cudaError_t launch_cells_mixed(const CellParams &cp, int pass, int sms, cudaStream_t s, int warps);
cudaError_t launch_cells_fp64(const CellParams &cp, int pass, int sms, cudaStream_t s, int warps);
cudaError_t launch_cells_batch_mixed(const BatchParams &bp, int pass, int sms, cudaStream_t s);
cudaError_t launch_cells_batch_fp64(const BatchParams &bp, int pass, int sms, cudaStream_t s);
cudaError_t launch_cells_batch(const BatchParams &bp, int mode, int pass, int sms, cudaStream_t s);
cudaError_t launch_finish(const CellParams &cp, int mode, int sms, cudaStream_t s);
cudaError_t launch_finish_batch(const BatchParams &bp, int mode, int sms, cudaStream_t s);
cudaError_t launch_compact_neighbors(const int *nf, const int *nb, const int *ovf, const long long *off, int n,
                                     int *out, cudaStream_t s);
cudaError_t launch_nf_to_ll(const int *nf, long long *out, int n, cudaStream_t s);
cudaError_t exclusive_scan_ll(const long long *in, long long *out, int n, long long *tmp, cudaStream_t s);
cudaError_t launch_sum_volumes(const double *vol, const int *flags, int n, double *out, cudaStream_t s);
// Sheared boxes with thin ghost layers: *out = 1 if some kept cell (loop order:
// stored position pos, max_radius_squared mr2 in real units) reaches past them.
cudaError_t launch_reach_check(const Geometry &g, int n, const double *pos, const double *mr2, const int *flags,
                               int *out, cudaStream_t s);
void box_tables(unsigned tri[8], unsigned adj[8]);
// vgpu_locate.cu
cudaError_t launch_locate(const CellParams &cp, int n, const double *qxyz, int *found, int *pid, double *rxyz,
                          cudaStream_t s);


}  // namespace vgpu
