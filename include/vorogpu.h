/* vorogpu.h — C ABI of the GB300 per-cell Voronoi engine.
 *
 * This is the drop-in boundary for the reference's per-particle cell path
 * (Voro++).  Each entry point names the reference interface it replaces.
 * All functions return an int status (VGPU_OK = 0); nothing exits, traps or
 * prints.  Plain pointers and sizes only; host pointers unless a name says
 * "device".  One handle = one container = one CUDA stream; handles are
 * independent and may be used from different host threads.
 */
#ifndef VOROGPU_H
#define VOROGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: 1-4 mirror VOROPP_* exit codes (src/config.hh:105-119) -- */
#define VGPU_OK 0
#define VGPU_ERR_FILE 1          /* VOROPP_FILE_ERROR */
#define VGPU_ERR_MEMORY 2        /* VOROPP_MEMORY_ERROR (device allocation) */
#define VGPU_ERR_INTERNAL 3      /* VOROPP_INTERNAL_ERROR */
#define VGPU_ERR_ARG 16          /* bad argument / handle */
#define VGPU_ERR_CUDA 17         /* CUDA runtime error (see vgpu_last_error) */
#define VGPU_ERR_UNSUPPORTED 18  /* not supported (walls on a periodic box) */
#define VGPU_ERR_DUPLICATE 19    /* container_periodic put of a duplicate point
                                    (src/common.cc:14-20 exits; we return this) */
#define VGPU_ERR_NOT_COMPUTED 20 /* results requested before vgpu_compute */
#define VGPU_ERR_CAPACITY 21     /* a cell exceeded every engine capacity */
#define VGPU_ERR_NO_DEVICE 22    /* no CUDA device */

/* ---- container kinds (reference classes) ------------------------------- */
#define VGPU_CONTAINER 0               /* container, src/container.hh:289-291 */
#define VGPU_CONTAINER_POLY 1          /* container_poly, src/container.hh:511-513 */
#define VGPU_CONTAINER_PERIODIC 2      /* container_periodic, src/container_prd.hh:213-216 */
#define VGPU_CONTAINER_PERIODIC_POLY 3 /* container_periodic_poly, src/container_prd.hh:434-437 */

/* ---- precision modes ---------------------------------------------------- */
#define VGPU_FP64 0  /* every side test, vertex and reduction in FP64 */
#define VGPU_MIXED 1 /* FP32 side tests under a forward error filter; filter-band
                        hits redone in FP64 (topology as in FP64).  Final
                        vertices: the FP32 vertex corrected against its three
                        planes by residual steps in float pairs (about 48
                        bits; ill-conditioned triples, cells that met the
                        tolerance band and cells below 1e-4 of the cube of
                        their radius solved in FP64); volume and centroid
                        summed in float pairs.  Per-cell volume and centroid
                        within 1e-10 of the FP64 engine's.  Containers
                        whose FP32 filter band is saturated run on the FP64
                        engine (vgpu_set_fp64_fallback) */

/* ---- per-cell flag bits (vgpu_get_cells, out_flags) -------------------- */
#define VGPU_CELL_OK 1        /* compute_cell returned true (cell not deleted) */
#define VGPU_CELL_MARGINAL 2  /* a vertex fell inside the reference tolerance band
                                 (|plane value| <= tol): the reference would merge
                                 vertices there; topology may differ from it */
#define VGPU_CELL_REPAIRED 4  /* at least one FP32 test was redone in FP64 */
#define VGPU_CELL_FAILED 8    /* the cell exceeded every engine capacity; bits 8-11 give why: */
#define VGPU_FAIL_PLANES 1    /*   more live planes than the last engine's 128 slots */
#define VGPU_FAIL_ADJACENCY 2 /*   inconsistent vertex adjacency (after a cut, or in a
                                   cell record the finish kernel checks) */
#define VGPU_FAIL_VERTICES 3  /*   more vertices than the last engine's 128 slots */
#define VGPU_FAIL_SEARCH 4    /*   the neighbour search did not terminate */
#define VGPU_FAIL_RECORDS 5   /*   the polytope record store was full */

typedef struct vgpu_container vgpu_container;

/* Engine counters for the last vgpu_compute. */
typedef struct vgpu_stats {
    int64_t cells;            /* cells computed (stored particles) */
    int64_t deleted;          /* cells removed entirely (compute_cell == false) */
    int64_t marginal_cells;   /* cells flagged VGPU_CELL_MARGINAL */
    int64_t side_tests;       /* vertex-plane side tests evaluated */
    int64_t fp64_repairs;     /* FP32 tests redone in FP64 */
    int64_t planes_tested;    /* candidate planes tested against a cell */
    int64_t planes_cut;       /* candidate planes that cut a cell */
    int64_t overflow_reruns;  /* cells re-run by the large-capacity engine */
    int64_t failed_cells;     /* cells that overflowed every engine capacity */
    double kernel_ms;         /* device time of the cell kernel(s), last compute */
    double bin_ms;            /* device time of binning, last compute */
    double step_ms;           /* device time of the whole compute (events on the handle's stream) */
    int64_t kernel_launches;  /* engine kernels launched by the last compute */
    double clip_ms;           /* of kernel_ms: the main clipping kernel alone */
    double finish_ms;         /* of kernel_ms: the FP64 finish kernel (mixed engine) */
    int64_t fp64_engine_cells; /* mixed compute: cells the FP64 engine computed because the
                                  first pass (or its sample) showed the FP32 filter band
                                  saturated (0 or all of a container's) */
} vgpu_stats;

/* Library / device. */
const char *vgpu_version(void);
int vgpu_device_count(int *count);
/* Message for the last error on this thread. */
const char *vgpu_last_error(void);

/* Replaces the constructors container(ax,bx,ay,by,az,bz,nx,ny,nz,xper,yper,zper,
 * init_mem) (src/container.hh:290-291), container_poly(...) (src/container.hh:512-513),
 * container_periodic(bx,bxy,by,bxz,byz,bz,nx,ny,nz,init_mem) (src/container_prd.hh:215-216)
 * and container_periodic_poly (src/container_prd.hh:436-437).
 * geom: container kinds (ax,bx,ay,by,az,bz); periodic kinds (bx,bxy,by,bxz,byz,bz),
 * rectangular or sheared (the unit cell, src/unitcell.cc:26-79, is built
 * here; VGPU_ERR_MEMORY if it is not bounded within ten shells of images).
 * grid: (nx,ny,nz) as given to the reference (it fixes the loop order of results).
 * periodic: three flags, container kinds only (ignored for periodic kinds). */
int vgpu_container_create(vgpu_container **out, int kind, const double geom[6],
                          const int grid[3], const int periodic[3]);
int vgpu_container_destroy(vgpu_container *h);

/* Replaces container::put(n,x,y,z) (src/container.cc:90-97),
 * container_poly::put(n,x,y,z,r) (src/container.cc:103-111) and
 * container_periodic(_poly)::put (src/container_prd.cc:94-119), called n times:
 * appends ids[i] with xyzr[4i..4i+3] = (x,y,z,r) to the container's device
 * staging area; the copy completes before return, so the caller may reuse its
 * arrays (r ignored for mono kinds).  Out-of-range points in non-periodic directions
 * are dropped at compute time exactly as put_remap (src/container.cc:174-191).
 * A non-finite x, y or z (or r, radical kinds) fails the whole call with
 * VGPU_ERR_ARG and stages none of its particles (the reference has no check;
 * its remap would turn such a value into an arbitrary block index). */
int vgpu_put(vgpu_container *h, int64_t n, const int32_t *ids, const double *xyzr);
/* Same, from device memory already resident on the container's device; the
 * next vgpu_compute reads it in place (no host staging, no copy).  The input
 * is checked during the compute's binning instead: a non-finite x, y or z (or
 * r, radical kinds) makes vgpu_compute return VGPU_ERR_ARG before any cell
 * is computed. */
int vgpu_put_device(vgpu_container *h, int64_t n, const int32_t *dev_ids, const double *dev_xyzr);
/* Replaces container::clear() (src/container.cc:385-387). */
int vgpu_clear(vgpu_container *h);

/* Replaces compute_all_cells() (src/container.cc:438-453, src/container_prd.cc:514-529):
 * computes every cell and keeps per-cell results on the device.
 * mode: VGPU_FP64 or VGPU_MIXED.  Synchronous. */
int vgpu_compute(vgpu_container *h, int mode);
/* Replaces sum_cell_volumes() (src/container.cc:459-477, src/container_prd.cc:535-546):
 * sum of the volumes of the cells from the last compute (deleted cells add 0). */
int vgpu_sum_cell_volumes(vgpu_container *h, double *out);
int vgpu_get_stats(vgpu_container *h, vgpu_stats *out);

/* Number of stored particles (= result records) after the last compute, in the
 * reference's loop order (c_loop_all, src/c_loops.hh:165-210;
 * c_loop_all_periodic, src/c_loops.hh:325-393). */
int vgpu_num_cells(vgpu_container *h, int64_t *n);
/* Input order (particle_order with c_loop_order, src/c_loops.hh:268-317):
 * rows[i] = the loop-order result row of the i-th particle put since the last
 * vgpu_clear, or -1 if put() dropped it (outside a non-periodic wall).  One
 * entry per particle put; valid after a compute (or point location). */
int vgpu_get_input_rows(vgpu_container *h, int32_t *rows);
/* Total neighbour entries over all cells (sum of face counts). */
int vgpu_num_neighbors(vgpu_container *h, int64_t *total);

/* Per-cell results of the last compute, in loop order; any pointer may be NULL.
 * Replaces, per cell, the voronoicell queries the reference's callers make
 * after compute_cell (src/container.hh:462-478):
 *   ids      particle ID (c_loop_base::pid, src/c_loops.hh:149)
 *   pos      stored (remapped) position, 3 doubles (c_loop_base::pos, src/c_loops.hh:123-127)
 *   vol      voronoicell_base::volume (src/cell.cc:1584-1616)
 *   cen      voronoicell_base::centroid, particle-relative, 3 doubles (src/cell.cc:1861-1901)
 *   nfaces   voronoicell_base::number_of_faces (src/cell.cc:2168-2187)
 *   nverts   voronoicell_base::p (src/cell.hh:54)
 *   maxr2    max vertex distance squared from the particle, real units
 *            (0.25 * voronoicell_base::max_radius_squared, src/cell.cc:1907-1917)
 *   flags    VGPU_CELL_* bits */
int vgpu_get_cells(vgpu_container *h, int32_t *ids, double *pos, double *vol, double *cen,
                   int32_t *nfaces, int32_t *nverts, double *maxr2, int32_t *flags);
/* Autotuner (vgpu_autotune_ex without the cache), returning the chosen
 * engine-grid density.  No counterpart in the reference (a tuning choice of
 * this engine). */
int vgpu_autotune(vgpu_container *h, int mode, double *best_density, double *best_ms);

/* Optional outputs of vgpu_compute (flags; default 0).  VGPU_OUTPUT_POLYTOPES
 * keeps every cell's polytope — FP64 vertices and ordered face loops — for
 * the queries that need the cell itself (voronoicell_base::vertices,
 * face_vertices, face_areas, normals, ... src/cell.hh:132-184, and the
 * print_custom fields %p %P %o %g %E %e %F %A %a %f %t %l, src/cell.cc:
 * 2485-2558).  Applies from the next compute. */
#define VGPU_OUTPUT_POLYTOPES 1

/* Walls (src/wall.hh:25-130; container_base only: not for the
 * container_periodic kinds, VGPU_ERR_UNSUPPORTED).  Each cuts every cell
 * after its initial box, in the order added, with one plane computed from
 * the particle's position as the reference's cut_cell does (src/wall.cc);
 * its faces carry the wall's ID as neighbour.  params (7 doubles):
 *   VGPU_WALL_SPHERE   xc yc zc rc            (wall_sphere)
 *   VGPU_WALL_PLANE    xc yc zc ac            (wall_plane: x.c < ac inside)
 *   VGPU_WALL_CYLINDER xc yc zc xa ya za rc   (wall_cylinder)
 *   VGPU_WALL_CONE     xc yc zc xa ya za ang  (wall_cone)
 * Applies from the next compute.  point_inside_walls
 * (src/container.hh:75-78) is vgpu_point_inside_walls. */
#define VGPU_WALL_SPHERE 0
#define VGPU_WALL_PLANE 1
#define VGPU_WALL_CYLINDER 2
#define VGPU_WALL_CONE 3
int vgpu_set_output(vgpu_container *h, int flags);
/* The polytopes of the last compute in loop order, CSR: offsets[n+1] (int64,
 * in doubles) and data.  Cell k is data[offsets[k] .. offsets[k+1]):
 *   nv, nf, vertices (3 nv doubles, relative to the particle), then per face:
 *   neighbour ID, vertex count m, m vertex indices (a loop, clockwise seen
 *   from outside, as the reference's face_vertices).
 * Deleted and failed cells are empty.  data may be NULL to get the offsets. */
int vgpu_get_polytopes(vgpu_container *h, int64_t *offsets, double *data);
/* Stored radius of every cell's particle, in loop order (the r argument of
 * put; what container_poly::print_custom prints for %r, src/container.hh:
 * 660-671, reading p[ijk][4q+3]). */
int vgpu_get_radii(vgpu_container *h, double *radii);
/* Neighbour lists in CSR form: offsets[n+1] (int64) and ids[total].  Each
 * cell's list holds one ID per face, in ascending order (the reference's order,
 * voronoicell_neighbor::neighbors src/cell.cc:2660-2678, is an artefact of
 * plane insertion; the multiset is what is preserved).  Box walls are -1..-6
 * (src/cell.cc:2567-2580); unit-cell faces of periodic kinds are 0
 * (src/cell.cc:86-95). */
int vgpu_get_neighbors(vgpu_container *h, int64_t *offsets, int32_t *ids);

int vgpu_add_wall(vgpu_container *h, int type, const double params[7], int id);
int vgpu_clear_walls(vgpu_container *h);
int vgpu_point_inside_walls(vgpu_container *h, double x, double y, double z, int *inside);

/* Point location: for each of n points (xyz[3i..3i+2]) the particle whose
 * Voronoi cell contains it (container::find_voronoi_cell,
 * src/container.cc:237-301; container_periodic::find_voronoi_cell,
 * src/container_prd.cc:303-359): the particle of smallest squared distance
 * (power distance |x - p|^2 - r^2 for the radical kinds) over the periodic
 * images.  found[i] = 0 where the reference returns false (a point outside a
 * non-periodic wall, or no particles); else pid[i] = its ID and
 * rxyz[3i..3i+2] = its position, the periodic image nearest the point in
 * the point's own frame (stored position plus image counts times the box
 * lengths, as the reference assembles it).  Exact ties may pick another of
 * the tied particles than the reference.  Host arrays.  Bins the particles
 * first if no compute has since the last put. */
int vgpu_find_voronoi_cells(vgpu_container *h, int64_t n, const double *xyz, int32_t *pid, double *rxyz,
                            int32_t *found);

/* Ghost cells: the Voronoi cells of n ghost particles (xyzr[4i..4i+3], the
 * radius used by the radical kinds) among the container's particles, each
 * as if it alone were added (compute_ghost_cell, src/container.hh:487-498
 * and 710-721; src/container_prd.hh:414-422 and 635-644): a ghost is placed
 * like a put() (outside a non-periodic wall: no cell, flags 0), is no
 * neighbour of any other cell or ghost, and a radius above the container's
 * largest widens the search as the reference's max_radius does.  The
 * container's own results are untouched.  Results (ghost order):
 * vgpu_get_ghost_cells (as vgpu_get_cells; centroids relative to the
 * ghost's stored position), vgpu_get_ghost_neighbors (CSR, each list
 * ascending) and, with VGPU_OUTPUT_POLYTOPES set, vgpu_get_ghost_polytopes
 * (as vgpu_get_polytopes).  Bins the particles first if no compute has
 * since the last put. */
int vgpu_compute_ghost_cells(vgpu_container *h, int mode, int64_t n, const double *xyzr);
int vgpu_get_ghost_cells(vgpu_container *h, double *vol, double *cen, int32_t *nfaces, int32_t *nverts,
                         double *maxr2, int32_t *flags);
int vgpu_get_ghost_neighbors(vgpu_container *h, int64_t *offsets, int32_t *ids);
int vgpu_get_ghost_polytopes(vgpu_container *h, int64_t *offsets, double *data);

/* Diagnostics: per-phase SM clock totals of the last compute's cell kernel,
 * summed over warps (0 init, 1 candidate gather, 2 sort, 3 side tests,
 * 4 cuts, 5 record output, 6 the part of 1 spent in flushes the gather
 * starts when its candidate buffer fills, 7 whole kernel).  All zero unless
 * the library was built with -DVGPU_PHASE_TIMING. */
int vgpu_phase_cycles(vgpu_container *h, double out[8]);
/* Diagnostics, same build: event counts of the last compute's cell kernel
 * (0 candidate flushes, 1 of them sorting 64 keys, 2 block passes of the
 * gather, 3 candidate passes, 4 candidates kept, 5 vertices created by cuts,
 * 6 search segments, 7 cells run). */
int vgpu_phase_counts(vgpu_container *h, double out[8]);

/* Device-resident views of the results (valid until the next compute/destroy):
 * volumes (double[n]) and face counts (int32[n]). */
int vgpu_device_results(vgpu_container *h, const double **dev_vol, const int32_t **dev_nfaces);

/* Engine tuning: target particles per engine block (0 = default 0.6) and warps
 * (cells in flight) per CTA of the clipping kernel, 1-8, at most what the
 * library was built for (0 = default 4).
 * Applies from the next compute. */
int vgpu_set_tuning(vgpu_container *h, double particles_per_block, int warps_per_cta);

/* The engine's tuning of one container (no counterpart in the reference,
 * whose only knob is the block grid it is given):
 *   particles_per_block  target density of the engine's own search grid
 *   warps_per_cta        cells in flight per CTA of the clipping kernels
 *                        (1 to the build's maximum, 4 by default)
 *   cells_per_chunk      consecutive cells (neighbouring blocks) a warp
 *                        takes from the work queue at once (1-64, default 8)
 *   fp64_fallback        see vgpu_set_fp64_fallback
 * In vgpu_set_tuning_ex a zero field keeps the current value.  None of them
 * changes a cell's topology; volumes stay within the precision mode's bound. */
typedef struct vgpu_tuning {
    double particles_per_block;
    int warps_per_cta;
    int cells_per_chunk;
    double fp64_fallback;
} vgpu_tuning;
int vgpu_get_tuning(vgpu_container *h, vgpu_tuning *out);
int vgpu_set_tuning_ex(vgpu_container *h, const vgpu_tuning *t);

/* The autotuner: times computes of the container's own particles over the
 * engine-grid density, then warps per CTA, then cells per chunk (coordinate
 * search, best of two computes each), keeps the fastest tuple and leaves the
 * results of a compute with it.  Flags: VGPU_TUNE_USE_CACHE takes the tuple
 * a previous search stored for the same GPU and workload signature (device
 * name, container kind, precision, particle count to within a factor of two,
 * box aspect ratio, walls) instead of searching; VGPU_TUNE_WRITE_CACHE
 * stores the tuple it finds.  The cache is a text file:
 * $VORO_GB300_TUNE_CACHE, else $XDG_CACHE_HOME/voro_gb300/autotune.txt, else
 * ~/.cache/voro_gb300/autotune.txt.  *best_ms: the chosen tuple's step time. */
#define VGPU_TUNE_USE_CACHE 1
#define VGPU_TUNE_WRITE_CACHE 2
int vgpu_autotune_ex(vgpu_container *h, int mode, int flags, vgpu_tuning *chosen, double *best_ms);

/* Sheared container_periodic: depth of the ghost layers of images a compute
 * stores first, in mean particle spacings (0 = default 8; < 0: always the
 * reference's depth).  A compute whose cells reach past them is redone at the
 * reference's depth, so the results never depend on it; deeper layers cost
 * memory and binning time, shallower ones make the rerun likelier. */
int vgpu_set_ghost_depth(vgpu_container *h, double spacings);

/* Budget in bytes of the polytope-record store one compute of this container
 * may use (the scratch the clipping kernels write and the finish kernel reads;
 * about 0.75 KB per cell with the mixed engine), 0 = the default of 1 KB per
 * cell.  Where the reference meets an allocation limit it exits with
 * VOROPP_MEMORY_ERROR (max_vertices etc., src/config.hh:44-56;
 * src/cell.cc:130-288); here the cells whose records do not fit are flagged
 * VGPU_CELL_FAILED with reason VGPU_FAIL_RECORDS, the others complete, and
 * vgpu_compute returns VGPU_ERR_CAPACITY.  Applies from the next compute. */
int vgpu_set_record_budget(vgpu_container *h, int64_t bytes);

/* Mixed computes assess the FP32 engine's first pass: a large container (at
 * least 262,144 cells) runs it first on 1/64 of its cells, a smaller one on
 * all of them (and a batch member by its share of the batch's first pass).
 * If more than this fraction of those cells need FP64 (tests inside the
 * filter band or ill-conditioned vertices, as in jittered lattices where
 * three near-coplanar bisectors meet), the whole container is computed by the
 * FP64 engine instead, which is faster there, gives the same topology and
 * stays exact where a lattice is jittered at the tolerance's own scale;
 * vgpu_stats.fp64_engine_cells reports it.  Default 0.25; a value >= 1 never
 * switches.  No counterpart in the reference (it computes in FP64
 * throughout). */
int vgpu_set_fp64_fallback(vgpu_container *h, double fraction);
/* The container's length tolerance as the reference's cells hold it:
 * tol = 10 * DBL_EPSILON * max_len_sq (src/cell.cc:26, src/config.hh:80),
 * max_len_sq from the container's geometry (src/container.cc:34-35 for
 * container / container_poly, the unit cell's max_radius_squared for the
 * periodic kinds, src/container_prd.cc:32), in the reference's doubled
 * vertex coordinates.  It is the threshold of voronoicell_base::normals
 * (src/cell.cc:2108-2164), which the host-side polytope queries follow. */
int vgpu_get_tolerance(vgpu_container *h, double *tol);

/* ---- batches: many containers computed by one persistent launch ----
 * The reference computes containers one at a time (compute_all_cells per
 * container, src/container.cc:438-453).  A batch bins every member container
 * (each on its own stream) and then runs all their cells in one launch of the
 * cell engine with a single device work queue, so thousands of small and
 * large containers share the GPU.  Results land in each member container and
 * are read with the usual getters.  Containers stay owned by the caller and
 * must outlive the batch's computes.  A sheared container_periodic joins a
 * batch with its images stored at the reference's depth. */
typedef struct vgpu_batch vgpu_batch;
int vgpu_batch_create(vgpu_batch **out);
int vgpu_batch_add(vgpu_batch *b, vgpu_container *h);
int vgpu_batch_compute(vgpu_batch *b, int mode);
/* Sums over the members; kernel_ms = the batched launch(es), bin_ms = the
 * members' binning (host wall time), step_ms = the whole call (wall time). */
int vgpu_batch_get_stats(vgpu_batch *b, vgpu_stats *out);
/* Budget in bytes of the batch's polytope-record store (the scratch the
 * clipping kernels write and the finish kernel reads; about 1 KB per cell),
 * 0 = the default 8 GiB.  A batch whose records exceed it is processed in
 * waves of cells, each clipped and finished before the next; results are the
 * same.  *waves (vgpu_batch_waves) = the waves of the last compute. */
int vgpu_batch_set_record_budget(vgpu_batch *b, int64_t bytes);
int vgpu_batch_waves(vgpu_batch *b, int *waves);
int vgpu_batch_destroy(vgpu_batch *b);

/* Σ of n device-resident cell volumes (e.g. vgpu_device_results' dev_vol;
 * deleted cells hold volume 0) written to dev_out (one double, device memory),
 * launched on the caller's stream (a cudaStream_t; NULL = legacy default
 * stream) and not waited for.  No counterpart in the reference: it exists for
 * callers that must not allocate device memory — it calls no allocator and
 * keeps its partial sums in a fixed 64 KB static device array, so n is limited
 * to 33,554,432 (larger n: VGPU_ERR_ARG).  The first call on each device, with
 * that device current, does a one-time set-up (the scratch address lookup);
 * make it before any stream capture, and do not use the entry point after a
 * cudaDeviceReset in the same process (the cached address would be stale).
 * Every call runs on the current device, which must own dev_vol, dev_out and
 * the stream: a pointer of host memory or of another device is rejected with
 * VGPU_ERR_ARG before anything is launched.  Nothing has to be zeroed
 * beforehand.  Calls that overlap on one device share the scratch and race:
 * serialise them.  The summation order is fixed, so repeated calls give
 * identical results. */
int vgpu_sum_volumes_noalloc(const double *dev_vol, int64_t n, double *dev_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* VOROGPU_H */
