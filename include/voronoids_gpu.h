/* voronoids_gpu.h -- C ABI of the GB300 Delaunay build.
 *
 * Drop-in boundary for the `DelaunayTree` new / insert / parallel-insert path
 * of kazewong/Voronoids.  Each entry point names the reference interface it
 * replaces (file:line in the reference crate).  Plain pointers and sizes only;
 * every call returns a vd_status (no panics, no aborts).
 *
 * Conventions
 *  - Points are row-major doubles, `dim` per point (dim = 2 or 3), as the
 *    reference's Vec<[f64; N]>.  Host pointers unless the name says _device.
 *  - Vertices are numbered by input order across all insert calls on a tree
 *    (0, 1, 2, ...); the super-simplex vertices are not part of any output.
 *  - Edge lists are (u, v) pairs of those vertex numbers with u < v, sorted
 *    lexicographically.
 *  - One tree = one CUDA stream; a tree is not thread-safe, distinct trees are.
 *  - Exactness: conflict tests are exact; a point exactly on a circumsphere is
 *    resolved by a symbolic perturbation that reproduces the reference's
 *    strict `dist < r` rule for insertion in input order, so the output is the
 *    unique triangulation that rule yields, whatever the parallel order.
 */
#ifndef VORONOIDS_GPU_H
#define VORONOIDS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vd_tree vd_tree;

/* Status codes.  VD_ERR_DUPLICATE is not fatal: duplicates are skipped and the
 * tree holds the triangulation of the distinct points. */
enum vd_status {
  VD_OK = 0,
  VD_ERR_ARG = 1,          /* bad argument (dim, size, NULL pointer, capacity) */
  VD_ERR_CUDA = 2,         /* CUDA runtime error */
  VD_ERR_NOMEM = 3,        /* device allocation failed */
  VD_ERR_DUPLICATE = 4,    /* some points equal earlier ones and were skipped */
  VD_ERR_NONFINITE = 5,    /* NaN or infinite coordinate */
  VD_ERR_OUTSIDE = 6,      /* point not strictly inside the super simplex */
  VD_ERR_PRECISION = 7,    /* exact-arithmetic capacity exceeded */
  VD_ERR_ROUND_LIMIT = 8,  /* insertion rounds stopped making progress */
  VD_ERR_CAVITY = 9,       /* a conflict region exceeded the supported size */
  VD_ERR_WALK = 10,        /* point location did not terminate */
  VD_ERR_INTERNAL = 11,    /* inconsistent internal state */
  VD_ERR_DEGENERATE = 12,  /* super simplex degenerate (e.g. all points equal) */
  VD_ERR_RANGE = 13        /* |coordinate| outside [2^-150, 2^150] (and not 0) */
};

typedef struct vd_stats {
  int64_t rounds;            /* insertion rounds run on this tree */
  int64_t inserted;          /* vertices inserted */
  int64_t duplicates;        /* points skipped as duplicates */
  int64_t live_simplices;    /* simplices of the current triangulation (incl. super) */
  int64_t slots;             /* simplex slots in use (live + holes) */
  int64_t created;           /* simplices created over all insertions */
  int64_t killed;            /* simplices removed over all insertions */
  int64_t max_cavity;        /* largest conflict region (simplices) */
  int64_t max_facets;        /* largest conflict-region boundary (facets) */
  int64_t pred_f32;          /* predicates decided by the FP32 filter */
  int64_t pred_f64;          /* ... by the FP64 filter */
  int64_t pred_exact;        /* ... by exact expansion arithmetic */
  int64_t pred_sos;          /* ... of which resolved by symbolic perturbation */
  int64_t walk_steps;        /* point-relocation steps */
  int64_t cavity_tests;      /* conflict tests during cavity searches */
  int64_t deferred_overflow; /* candidate deferrals: cavity above per-warp capacity */
  int64_t deferred_pool;     /* candidate deferrals: cavity pool full */
  int64_t candidates;        /* nominations (one per simplex holding points, per round) */
  int64_t searched;          /* nominations that won the thinning claim and were searched */
  int64_t won_pass[3];       /* insertions decided in resolution pass 0, 1, 2 and later */
  int64_t spilled;           /* cavity searches that spilled to the pool */
  int64_t max_search_levels; /* longest conflict-region search in waves of 32 (simplex, face)
                                tests, when above 64 (0 otherwise) */
} vd_stats;

/* DelaunayTree::<3,4>::new / ::<2,3>::new
 * (src/delaunay_tree.rs:389-510, :544-640; bounding_sphere src/geometry.rs:99-142).
 * Sizes the super simplex from `pts` (n points); the points are NOT inserted.
 * Returns NULL only if allocation of the handle itself fails; otherwise check
 * *status. */
vd_tree* vd_tree_new(int dim, const double* pts, int64_t n, int* status);
/* Same, with all device work on the caller's CUDA stream (cudaStream_t). */
vd_tree* vd_tree_new_on_stream(int dim, const double* pts, int64_t n, void* stream, int* status);
void vd_tree_free(vd_tree* t);
/* `new` from points already in device memory (n * dim doubles).  The super
 * simplex is bit-identical to the host path's. */
vd_tree* vd_tree_new_device(int dim, const double* d_pts, int64_t n, void* stream, int* status);
/* Empties the tree and sizes its super simplex from new points (host /
 * device), keeping every device allocation for reuse. */
int vd_tree_reset(vd_tree* t, const double* pts, int64_t n);
int vd_tree_reset_device(vd_tree* t, const double* d_pts, int64_t n);

/* The super simplex `new` would build for `pts` (host computation only, no
 * device work): out[3*k + j] = coordinate j of super vertex k (z = 0 in 2D),
 * in the reference's vertex order, and *radius = 10 x bounding radius.
 * bounding_sphere src/geometry.rs:99-142; vertices src/delaunay_tree.rs:392-406,
 * :547-558. */
int vd_super_simplex(int dim, const double* pts, int64_t n, double* out, double* radius);

/* DelaunayTree::add_points_to_tree (src/delaunay_tree.rs:336-386), with the
 * queue/placement of src/scheduler.rs:6-55 replaced by GPU priority rounds.
 * `seed` fixes the random insertion priorities. */
int vd_insert_points(vd_tree* t, const double* pts, int64_t n, uint64_t seed);
/* Same with `d_pts` already in device memory (n * dim doubles). */
int vd_insert_points_device(vd_tree* t, const double* d_pts, int64_t n, uint64_t seed);
/* TreeUpdate::new + DelaunayTree::insert_point
 * (src/delaunay_tree.rs:709-740, :125-211): one point. */
int vd_insert_point(vd_tree* t, const double* p);

/* Conflict region of a query point (`locate`, src/delaunay_tree.rs:33-58):
 * ids of the simplices whose circumsphere strictly contains `p` (perturbed),
 * sorted ascending.  *n receives the count even when it exceeds `cap`. */
int vd_locate(vd_tree* t, const double* p, int64_t* out, int64_t cap, int64_t* n);
/* The same for nq query points at once (host arrays): the conflict region of
 * query i is ids[offsets[i] .. offsets[i+1]) (offsets: nq + 1 entries),
 * numbered as vd_simplices exports the simplices, each list sorted.  With
 * `ids` NULL only the offsets are filled.  VD_ERR_OUTSIDE if a query lies
 * outside the super simplex (its list is empty).  Single-set trees. */
int vd_locate_points(vd_tree* t, const double* pts, int64_t nq, int64_t* offsets, int64_t* ids, int64_t cap);

/* Vertices inserted so far (super vertices excluded). */
int vd_num_vertices(vd_tree* t, int64_t* n);
/* DelaunayTree::max_simplex_id (src/delaunay_tree.rs:29): id of the last
 * simplex created, counting the reference's initial 5 (3D) / 4 (2D). */
int vd_max_simplex_id(vd_tree* t, int64_t* id);

/* Live simplices, as the reference's simplex map (src/lib.rs:87-100):
 * verts[4*i + j] = vertex j of simplex i (super vertices are -(1+k), k = 0..dim;
 * in 2D verts[4*i+3] = -1); nbrs[4*i + j] = simplex across the face opposite
 * vertex j, or -1 on the hull.  *n receives the count. */
int vd_num_simplices(vd_tree* t, int64_t* n);
int vd_simplices(vd_tree* t, int32_t* verts, int32_t* nbrs, int64_t cap, int64_t* n);

/* Circumcentre and radius of every live simplex, in vd_simplices order
 * (PySimplex.center / .radius of the reference's dictionary view,
 * src/lib.rs:32-59; computed in FP64 on the GPU for the final simplices,
 * which the reference computes in floating point too, src/geometry.rs:2-56).
 * centers: 3 doubles per simplex (z = 0 in 2D).  *n receives the count. */
int vd_circumspheres(vd_tree* t, double* centers, double* radii, int64_t cap, int64_t* n);

/* Voronoi dual (the reference's stated purpose, README.md:2-4; the reference
 * keeps only the Voronoi vertices, Simplex::center / radius,
 * src/delaunay_tree.rs:10-17).  Voronoi vertices: vd_circumspheres.
 * Voronoi edges: one per interior facet, the (i, j) pair (i < j) of the two
 * live simplices sharing it, numbered as vd_simplices exports them, sorted;
 * pairs NULL to query the count (*n). */
int vd_voronoi_edges(vd_tree* t, int64_t* pairs, int64_t cap, int64_t* n);
/* Voronoi cells: the live simplices incident to input vertex v (the vertices
 * of its cell, vd_simplices numbering) are ids[offsets[v] .. offsets[v+1]),
 * sorted.  offsets: vd_num_vertices + 1 entries (always filled); ids NULL to
 * query the sizes.  A skipped duplicate has an empty cell. */
int vd_voronoi_cells(vd_tree* t, int64_t* offsets, int64_t* ids, int64_t cap);

/* Sorted Delaunay edge list among inserted points. */
int vd_num_edges(vd_tree* t, int64_t* n);
int vd_edges(vd_tree* t, int64_t* uv, int64_t cap, int64_t* n);
/* Same into device memory as uint32 pairs. */
int vd_edges_device(vd_tree* t, uint32_t* d_uv, int64_t cap, int64_t* n);
/* Same into host memory as uint32 pairs (one copy). */
int vd_edges_u32(vd_tree* t, uint32_t* uv, int64_t cap, int64_t* n);

/* DelaunayTree::check_delaunay (src/delaunay_tree.rs:512-541, :642-671),
 * exact: *ok = 1 iff every simplex is positively oriented, adjacency is
 * symmetric and every interior facet is locally Delaunay.  `violations`
 * (NULL or 6 entries): non-positive, asymmetric, not Delaunay, not
 * perturbed-Delaunay, hull facets, facets checked. */
int vd_check_delaunay(vd_tree* t, int* ok, int64_t* violations);

/* check_delaunay (src/delaunay_tree.rs:512-541, :642-671) on a caller's
 * triangulation rather than a tree's: the same exact device checks as
 * vd_check_delaunay, for simplices built anywhere (an exported and edited
 * tree, another library's output).
 *   pts      host, npts rows of `dim` doubles; vertex id i is row i (the
 *            caller includes any super vertices)
 *   verts    host, ns rows of 4 int32 vertex ids, positively oriented as
 *            vd_simplices exports them (2D: the 4th id is ignored)
 *   nbrs     host, ns rows of 4 int32: the simplex across the face opposite
 *            vertex j, or -1 on the hull
 * *ok = 1 iff no simplex is non-positive, no link is one-sided or out of
 * range, and every interior facet is locally Delaunay (exact and perturbed by
 * vertex id).  `violations` (NULL or 6 entries) as vd_check_delaunay; a vertex
 * id outside [0, npts) counts as a structural (asymmetric) fault.  Allocates
 * and frees its own device buffers; synchronous. */
int vd_check_triangulation(int dim, const double* pts, int64_t npts, const int32_t* verts, const int32_t* nbrs,
                           int64_t ns, int* ok, int64_t* violations);

/* Duplicates skipped so far: pairs (skipped vertex, vertex it equals). */
int vd_duplicates(vd_tree* t, int64_t* pairs, int64_t cap, int64_t* n);

int vd_get_stats(vd_tree* t, vd_stats* s);
const char* vd_status_str(int status);

/* Diagnostics (no reference counterpart; the reference prints timings with
 * println!, src/delaunay_tree.rs:337-368).  Profiling records CUDA events
 * around every kernel of every round on the tree's stream; vd_profile returns
 * the summed milliseconds and launch counts per kernel (names from
 * vd_profile_name; "edges" is the edge extraction).  Turning it on
 * resets the sums.  The trace synchronises after every round and keeps one
 * row per round: round, active points at start, cumulative nominations,
 * cumulative searches, cumulative insertions, cumulative conflict tests,
 * GPU microseconds of the round (-1 unless profiling is on), active points
 * after the round. */
int vd_set_profiling(vd_tree* t, int on);
/* Insertion schedule (no reference counterpart: the reference places all
 * points of a batch in rounds up front, src/scheduler.rs:6-55).  The points
 * of a call are split by priority into levels of `first_prefix` points, then
 * growing by `growth` (1 < growth <= 16); a round activates further levels
 * while fewer than `ratio` (0 < ratio <= 64) times the inserted points are
 * active.  Defaults 64, 1.25 and 0.12. */
int vd_set_schedule(vd_tree* t, int64_t first_prefix, double growth, double ratio);
/* Round tuning: resolution passes per round (1..6) and the thinning radius
 * (0 = every nominee is searched, 1 = a nominee must hold its simplex and
 * face neighbours, 2 = and no lower nominee two faces away).  Defaults: 3D 2 passes / radius 2, 2D 2 / 1. */
int vd_set_tuning(vd_tree* t, int passes, int thin);
/* Round mode (no reference counterpart).  0: winners of a pass have
 * disjoint cavities and no cavity touches another's outer shell, the
 * reference's 2-ring independence (src/scheduler.rs:30-55).  1 (default):
 * cavities only need to be disjoint; a cavity next to a lower-priority cavity
 * wins if the shared facets stay locally Delaunay (exact test), and the two
 * stars are stitched after the pass.  Same triangulation either way. */
int vd_set_adjacent(vd_tree* t, int on);
/* While the next round would have fewer than `max_active` active points
 * (default 0 = never), rounds run in one cooperative launch with a
 * grid barrier between their phases instead of one kernel launch per phase
 * (the first rounds of a build are latency chains of small kernels).  No
 * reference counterpart; the triangulation is the same. */
int vd_set_small_rounds(vd_tree* t, int max_active);
/* Early phase of a call: until `until_inserted` points of the tree are
 * inserted, rounds use thinning radius `thin` and a feed ratio of at least
 * `ratio` (the device is far from busy while the triangulation is small, so
 * more searches per round cost little and save rounds).  Defaults 10000
 * points, radius 0, ratio 0.5; until_inserted = 0 turns it off.  No
 * reference counterpart; the triangulation is the same. */
int vd_set_early_phase(vd_tree* t, int64_t until_inserted, int thin, double ratio);
/* Exact tier of the conflict tests (the insphere sign when the FP32 and FP64
 * filters cannot decide).  mode 1: floating-point expansions only; mode 2:
 * an integer evaluation first (every coordinate a multiple of a common power
 * of two within 126 bits, 32-bit limbs), the expansions beyond that; mode 0
 * (default): expansions until a call has made `switch_after` exact tests
 * (default 32), then the integer form for the rest of the call.  The kernels
 * of each form are compiled separately: the integer form needs far more
 * registers, which slows inputs that never reach the exact tier, while on
 * near-degenerate inputs it is several times faster than the expansions.
 * Every mode gives the same signs, so the same triangulation.  The
 * reference's conflict test (circumsphere centre and radius, then a distance
 * comparison in f64, src/geometry.rs:58-97) has no exact tier. */
int vd_set_exact_tier(vd_tree* t, int mode, int64_t switch_after);
/* First points of a fresh single-set call (no reference counterpart; the
 * reference inserts the first 1e5 points one at a time, src/lib.rs:108-114).
 * While the triangulation is small, a device-wide round inserts only one or a
 * few points, so the first whole priority levels, at most `max_points` points
 * and at most the block's capacity (320 in 3D, 641 in 2D), are inserted one
 * after another by one thread block holding the triangulation in shared
 * memory; the rounds continue from there.  The triangulation is the same.
 * Default: 150 points (the block's time per point grows with the
 * triangulation, so past a few hundred points the rounds are faster); 0
 * turns it off. */
int vd_set_first_block(vd_tree* t, int64_t max_points);
/* Rounds are launched in chunks captured once as CUDA graphs and replayed
 * (default on; profiling and tracing launch kernel by kernel).  No reference
 * counterpart. */
int vd_set_graphs(vd_tree* t, int on);
int vd_profile(vd_tree* t, double* ms, int64_t* launches, int cap, int* n);
const char* vd_profile_name(int i);
int vd_set_trace(vd_tree* t, int on);
/* Kernels launched by this library in this process so far. */
int64_t vd_kernel_launches(void);
int vd_trace(vd_tree* t, int64_t* rows, int64_t cap, int64_t* n);

/* voronoids.delaunay(points) (src/lib.rs:104-125) in one call: new + insert
 * all points + sorted edge list.  `uv` may be NULL to query the count. */
int vd_delaunay(int dim, const double* pts, int64_t n, uint64_t seed, int64_t* uv, int64_t cap,
                int64_t* n_edges);
/* The same on a reusable tree (its dimension is kept; allocations are
 * reused): host points in, host uint32 edge pairs out (pinned buffers give
 * full-speed copies). */
int vd_delaunay_tree(vd_tree* t, const double* pts, int64_t n, uint64_t seed, uint32_t* uv, int64_t cap,
                     int64_t* n_edges);
/* The same with device points in and device uint32 edge pairs out. */
int vd_delaunay_device(vd_tree* t, const double* d_pts, int64_t n, uint64_t seed, uint32_t* d_uv,
                       int64_t cap, int64_t* n_edges);

/* Batched build (no reference counterpart: the reference builds one tree per
 * call, src/lib.rs:104-125).  `nsets` independent point sets, set s being the
 * points offsets[s] .. offsets[s+1]-1 of `pts` (offsets: nsets + 1 host
 * entries, offsets[0] = 0, every set non-empty), are triangulated together in
 * one pass of insertion rounds; each set's triangulation is exactly the one
 * vd_delaunay builds for it alone with the same seed.  Edges are written set
 * after set as uint32 pairs of point numbers within the set (u < v, sorted);
 * edge_offsets (nsets + 1 host entries) bounds each set's edges.  The tree is
 * reset to the batch (any earlier content is dropped); vd_check_delaunay,
 * vd_get_stats and vd_num_edges (global numbering) then apply to all sets.
 * Host points in, host pairs out: */
int vd_batch_delaunay(vd_tree* t, const double* pts, const int64_t* offsets, int nsets, uint64_t seed,
                      uint32_t* uv, int64_t cap, int64_t* edge_offsets);
/* Device points in, device pairs out (`offsets` and `edge_offsets` on the host). */
int vd_batch_delaunay_device(vd_tree* t, const double* d_pts, const int64_t* offsets, int nsets, uint64_t seed,
                             uint32_t* d_uv, int64_t cap, int64_t* edge_offsets);
/* Launch shape of the round kernels: warps per SM for the candidate-per-warp
 * kernels (4..32, multiple of 4; default 20) and 256-thread blocks per SM for
 * the point-per-thread kernels (1..32; default 8).  No reference counterpart. */
int vd_set_launch(vd_tree* t, int warps_per_sm, int blocks_per_sm);
/* Autotuner for batched builds (no reference counterpart).  Times batched
 * builds of a sample of the sets (every k-th set, about `sample_points`
 * points: the batch's size mix) with CUDA events, sweeping in turn the round
 * mode, feed ratio, resolution passes, thinning radius, warps per SM and
 * blocks per SM,
 * and keeps the fastest setting on the tree.  out (NULL or 9 entries): warps
 * per SM, blocks per SM, passes, thinning radius, ratio x 1000, best sample
 * microseconds, sample points, sample sets, round mode.  The tree is left
 * reset to the sample. */
int vd_autotune_batch(vd_tree* t, const double* d_pts, const int64_t* offsets, int nsets, int64_t sample_points,
                      int64_t* out);
/* Point sets of the tree (1 unless built by vd_batch_*). */
int vd_num_sets(vd_tree* t, int* nsets);
/* An empty tree (no super simplex yet) for the batched calls, vd_tree_reset
 * or vd_delaunay_tree / vd_delaunay_device. */
vd_tree* vd_tree_create(int dim, void* stream, int* status);

/* Serving loop (no reference counterpart: the reference triangulates one set
 * per blocking call, src/lib.rs:104-125).  Requests of mixed size and
 * dimension are queued by vd_server_submit (points copied).  `slots` workers,
 * each with its own host thread, CUDA stream and reusable trees, form batches
 * from the queue of the dimension whose oldest request waited longest and run
 * them as batched builds, so that requests arriving while others run are
 * admitted as slots and budget free up, and batches of different slots
 * overlap on the device.  Admission: the estimated device bytes of the
 * requests in flight (3D 1850 B/point, 2D 700 B/point, 1.5x slack included)
 * stay within `pool_bytes`; a request larger than the budget finishes with
 * VD_ERR_NOMEM.  `max_batch_points` caps a batch (0 = only the budget).
 * Each result is the triangulation of the request alone. */
typedef struct vd_server vd_server;
vd_server* vd_server_new(uint64_t pool_bytes, int slots, int64_t max_batch_points, uint64_t seed, int* status);
int vd_server_submit(vd_server* s, int dim, const double* pts, int64_t n, int64_t* id);
/* Ids of requests finished since the last call (at most `cap`); waits up to
 * `timeout_ms` for one when none is ready. */
int vd_server_poll(vd_server* s, int64_t* ids, int64_t cap, int64_t* n, int timeout_ms);
/* Result of a finished request: its status and edges (uint32 pairs numbered
 * within the request, sorted).  With `uv` NULL only the count and status are
 * returned; otherwise the result is copied out and released. */
int vd_server_result(vd_server* s, int64_t id, uint32_t* uv, int64_t cap, int64_t* n_edges, int* req_status);
/* out[0..7]: submitted, finished, batches, bytes in flight, peak bytes in
 * flight, queued, requests re-run alone after a failed batch, budget. */
int vd_server_stats(vd_server* s, int64_t* out);
/* Finishes every queued request, then stops the workers. */
void vd_server_free(vd_server* s);

/* Sorted edge list of a caller-owned simplex list, for callers that may not
 * allocate GPU memory (for example an application whose memory manager owns
 * the whole device, or a loop that cannot afford the synchronisation of a
 * cudaMalloc).  No counterpart in the reference.  It allocates nothing: its
 * scratch is one statically sized device array (about 10.5 MB) that every GPU
 * loading this library holds until the process exits.
 *   d_simp  device array of ns rows of 4 int32 vertex ids (16-byte aligned);
 *           negative ids (super vertices, the unused 4th id in 2D) are skipped
 *   ns <= 131072 simplices, vertex ids < nverts <= 65536; larger inputs are
 *           rejected with VD_ERR_ARG
 *   d_uv    device output, (u, v) uint32 pairs, u < v, sorted; *n_edges gets
 *           the count (VD_ERR_ARG if it exceeds cap)
 *   stream  cudaStream_t (NULL = default stream); the call is synchronous:
 *           it returns after its work on that stream has finished.
 * All calls on a device share the scratch array and leave their data in it;
 * calls whose GPU work overlaps race and give wrong results.  The first call
 * on a device looks up the array's address (cudaGetSymbolAddress) with that
 * device current, and looks it up again once the device's context has been
 * recreated (e.g. after cudaDeviceReset); make that first call before starting
 * any stream capture. */
int vd_edges_from_simplices_noalloc(int dim, const int32_t* d_simp, int64_t ns, int64_t nverts,
                                    uint32_t* d_uv, int64_t cap, int64_t* n_edges, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VORONOIDS_GPU_H */
