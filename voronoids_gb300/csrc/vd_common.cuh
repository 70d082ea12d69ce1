// Device-side data layout of a Delaunay tree on one GPU.
//
// The reference keeps simplices in a DashMap<usize, Simplex> with a
// Vec<usize> of neighbours each and a kd-tree of vertices
// (src/delaunay_tree.rs:10-30).  Here everything is a flat, device-resident
// pool addressed by 32-bit indices:
//
//   pts[v]        vertex v: (x, y, z | 0, pad) f64, 32 B, one sector per gather;
//                 ids 0..D are the super-simplex vertices, D+1+i is input point i
//   simp[s]       simplex slot s: v[0..D] vertex ids (positively oriented),
//                 n[f] = (neighbour << 2) | face-in-neighbour across the face
//                 opposite v[f], or -1 on the super-simplex hull; a dead slot
//                 has v[0] = -1 and n[0] pointing at a simplex of the star that
//                 replaced it.  32 B = one sector.
//   vote[s]       epoch|priority of the lowest-priority uninserted point inside s
//   thin[s]       epoch|priority of the lowest candidate whose simplex is s or
//                 a face neighbour of s (cheap pre-selection before any search)
//   claim_c[s]    epoch|priority of the lowest candidate whose cavity holds s
//   claim_n[s]    epoch|priority of the lowest candidate that rewrites a face of s
//   killed[s]     (round, vertex) of the insertion that removed s
//   touched[s]    round in which an insertion repointed a face of s
//
// Epoch-tagged 64-bit keys ((2^32 - 1 - round) << 32 | priority) make stale
// values from earlier rounds compare larger, so none of these arrays is ever
// cleared between rounds.
#pragma once
#include <stdint.h>

#include "vd_predicates.cuh"

namespace vd {

struct alignas(32) Simplex {
  int v[4];
  int n[4];
};

// Per-round statuses of a candidate.
// ST_BIG: the search outgrew a warp's shared memory and waits for k_cavity_big.
enum : int { ST_OK = 0, ST_DUP = 1, ST_OVERFLOW = 2, ST_POOL = 3, ST_LOST = 4, ST_DONE = 5, ST_WIN = 6, ST_BIG = 7 };

// Resolution passes per round (independent-set refinement), see vd_build.cu.
constexpr int kPassesMax = 6;
// Work-list stages of a round: 0 = searched nominees, then per pass the
// losers (odd) and the re-claimers (even).
constexpr int kStages = 2 * kPassesMax;

// Error codes (mirrored by the C ABI's vd_status).
enum : int {
  E_OK = 0,
  E_ARG = 1,
  E_CUDA = 2,
  E_NOMEM = 3,
  E_DUPLICATE = 4,
  E_NONFINITE = 5,
  E_OUTSIDE = 6,
  E_PRECISION = 7,
  E_ROUND_LIMIT = 8,
  E_CAVITY = 9,
  E_WALK = 10,
  E_INTERNAL = 11,
  E_DEGENERATE = 12,
  E_RANGE = 13,
};

// Statistics counters kept in stripes (see Counters::stat).
constexpr int kStatStripes = 32;
constexpr int kStatPad = 16;  // one 128-byte line per stripe
enum : int { STAT_F32 = 0, STAT_F64 = 1, STAT_EXACT = 2, STAT_SOS = 3, STAT_TESTS = 4, STAT_WALK = 5, STAT_COUNT = 6 };

struct Counters {
  int nact[2];        // active (uninserted) points, by round parity
  int ncand;          // candidates of the current round
  int nbig;           // searches of the round deferred to k_cavity_big
  int nbigw;          // stars of the pass deferred to k_commit_big
  int pool_used;      // ints of the cavity pool used in the current round
  int nsimp;          // simplex slots handed out (high-water mark)
  int wasted;         // slots reserved by allocations that did not fit
  int err;            // first error code
  int ndup;           // duplicates dropped
  int overflow;       // candidates deferred: cavity larger than a warp holds
  int pool_overflow;  // candidates deferred: cavity pool full
  int simp_overflow;  // winners deferred: simplex pool full
  int ninserted;      // vertices inserted (total)
  int winners;        // winners (total)
  int max_cav, max_fac;
  int holes;          // dead slots left when a cavity had more simplices than facets
  unsigned long long created;  // simplices created (total)
  unsigned long long killed;   // simplices removed (total)
  // statistics in kStatStripes copies, added to by warps in turn (one
  // counter for a whole launch's warps would serialise their atomics):
  // predicate decisions (f32, f64, exact, sos), conflict tests in cavity
  // searches, walk steps; stat_total() sums the copies
  unsigned long long stat[kStatStripes][kStatPad];
  unsigned long long candidates;    // nominated points (all rounds)
  unsigned long long searched;      // candidates that passed the thinning claim
  unsigned long long won[kPassesMax];  // winners per resolution pass
  unsigned long long spilled;       // searches that used the pool spill path
  int nwl[kStages];                 // work-list lengths of the current round
  // continuous feed of priority levels (see k_plan in vd_build.cu)
  int lev_next;                     // first level not yet activated
  int nlev;                         // levels of the current call
  int feed_lo, feed_hi;             // range of `order` activated this round
  int round;                        // round being run (advanced by k_plan)
  int nwin, win_lo;                 // winners of the round (adjacent mode), first of the pass
  int max_levels;                   // deepest cavity search (breadth-first levels)
  // grid barrier and loop decision of the small-round kernel
  unsigned bar_count, bar_gen;
  int bar_abort, coop_go;
  int single;                       // outcome of the last one-point insertion (k_insert_one)
};

// Sum of a striped statistics counter (host or device).
__host__ __device__ inline unsigned long long stat_total(const Counters& c, int k) {
  unsigned long long s = 0;
  for (int i = 0; i < kStatStripes; ++i) s += c.stat[i][k];
  return s;
}

// Points of one insertion call are split into priority levels of
// geometrically growing size; at most this many.
constexpr int kMaxLevels = 96;

// One point set of a tree.  A tree holds a single set (the reference's
// DelaunayTree) or many independent sets triangulated together (batched
// build).  Vertex ids: the super-simplex vertices of all sets come first,
// D + 1 per set, then the input points of all sets in input order; set s
// starts with simplex slot s, its super simplex.
struct alignas(16) SetGeo {
  double org[3];    // location-hint grid origin (centre - bounding radius)
  double scale;     // 1 / grid extent
  int hint_off;     // first hint cell of the set
  int hint_levels;  // finest hint level (2^l cells per axis)
  int root;         // slot of the set's super simplex
  int n;            // input points of the set (batched build)
  int sup[4];       // super-simplex vertex ids, positively oriented (-1 pads 2D)
  float orgf[3];    // org and scale rounded to f32: hint cells are mapped in FP32
  float scalef;
};

// Hint cells of levels 0..levels.
__host__ __device__ inline long long hint_cells(int dim, int levels) {
  return dim == 3 ? ((1LL << (3 * (levels + 1))) - 1) / 7 : ((1LL << (2 * (levels + 1))) - 1) / 3;
}

struct DevTree {
  vdp::VPt* pts;
  vdp::FPt* ptf;      // the same coordinates split into f32 hi/lo pairs
  Simplex* simp;
  unsigned long long* vote;
  unsigned long long* thin;
  unsigned long long* claim_c;
  unsigned long long* claim_n;
  int2* killed;
  int* touched;
  int4* act[2];   // (vid, loc, priority, 0)
  int4* cand;     // (vid, loc, priority, active slot)
  int4* cinfo;    // (ncav, nfac, pool offset, status)
  int* wl[2];     // work lists (candidate indices), stage s in wl[s & 1]
  int* win;       // winners of the round (adjacent mode)
  int* bigc;      // candidates whose search k_cavity_big finishes (nbig of them)
  int* bigw;      // winners whose star k_commit_big writes (nbigw of them)
  int* repl;      // per (slot << 2 | face): new simplex code on that face (adjacent mode)
  int* pool;
  int2* dups;     // (dropped vid, vid it equals)
  Counters* ctr;
  int2* wchunk;       // per-warp fresh-slot chunk (base, left) of k_check
  int cap_wchunk;
  int* order;         // vertex ids of the current call grouped by priority level
  int* lev_off;       // kMaxLevels + 1 offsets of the levels in `order`
  int* hint;          // location hints of all sets (see vd_build.cu)
  SetGeo* sets;       // nsets entries
  int* set_of;        // set of input point (vid - nsuper); unused when nsets == 1
  int nsets;
  int nsuper;         // vertex ids below this are super-simplex vertices
  int cap_simp;
  int cap_verts;
  int cap_pool;
  int cap_cand;
  int cap_dups;
  int hint_all_below;  // winners write every hint level while fewer points are inserted
};

__host__ __device__ inline unsigned long long epoch(int round) {
  return (unsigned long long)(0xFFFFFFFFu - (unsigned)round) << 32;
}
// Claim keys of resolution pass p of round r (later passes compare lower).
__host__ __device__ inline unsigned long long pass_epoch(int round, int pass) {
  return epoch(8 * round + pass);
}

// Insertion priority: a bijective mix of the 32-bit vertex id and the seed,
// so priorities are distinct and form a seeded random order.
__host__ __device__ inline uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
__host__ __device__ inline uint32_t priority(uint32_t vid, uint64_t seed) {
  uint32_t x = vid ^ (uint32_t)seed;
  x = mix32(x);
  x ^= (uint32_t)(seed >> 32);
  return mix32(x);
}
// Inverse of mix32: each xor-shift and odd multiplication is undone in
// reverse order (multiplicative inverses modulo 2^32 of the two constants).
__host__ __device__ inline uint32_t unmix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x43021123U;  // inverse of 0x846ca68b
  x ^= (x >> 15) ^ (x >> 30);
  x *= 0x1d69e2a5U;  // inverse of 0x7feb352d
  x ^= x >> 16;
  return x;
}
// The vertex id with priority `pr` under `seed`.
__host__ __device__ inline uint32_t vertex_of_priority(uint32_t pr, uint64_t seed) {
  return unmix32(unmix32(pr) ^ (uint32_t)(seed >> 32)) ^ (uint32_t)seed;
}

#if defined(__CUDACC__)
__device__ inline void set_error(Counters* c, int code) { atomicCAS(&c->err, 0, code); }
// Index guards: a corrupted structure must turn into an error status, never
// into an out-of-bounds access.
__device__ inline bool bad_simp(const DevTree& T, int s) { return (unsigned)s >= (unsigned)T.cap_simp; }
__device__ inline bool bad_vert(const DevTree& T, int v) { return (unsigned)v >= (unsigned)T.cap_verts; }
__device__ inline int set_index(const DevTree& T, int vid) {
  return T.nsets == 1 ? 0 : T.set_of[vid - T.nsuper];
}
#endif

// Kernels launched by this library in this process (diagnostics).
void note_launches(long long k);
long long launches_total();

// Host-side launchers (vd_build.cu, vd_edges.cu, vd_check.cu).
struct Launch {
  int blocks;      // persistent grid size for thread-per-item kernels
  int warps;       // persistent warp count for warp-per-item kernels (multiple of 4)
  cudaStream_t stream;
};

// Writes the points (and their split f32 form) as vertices base_vid.. and
// checks that each lies strictly inside its set's super simplex.
void launch_upload(const DevTree& T, const Launch& L, int dim, const double* d_xyz, int64_t n, int base_vid);
// Priority levels of the points base_vid .. base_vid + n - 1.  With one set,
// level k holds the priorities in [thr[k-1], thr[k]); with many, each set
// has its own levels, of `first` points growing by `growth`, sized by the
// set.  d_work holds 2 * kMaxLevels ints (counts, cursors) and must be zero
// on entry; on exit T.order lists the points level by level,
// T.lev_off[0..nlev] bounds the levels and the feed counters are reset.
void launch_levels(const DevTree& T, const Launch& L, int64_t n, int base_vid, uint64_t seed,
                   const unsigned long long* thr, int nlev, double first, double growth, int* d_work);
// Feed of one round: activate priority levels while the active points are
// fewer than `ratio` times the inserted ones (at least one level when none
// is active).
struct Feed {
  uint64_t seed;
  float ratio;
};
// Runtime tuning of a round: resolution passes (1..kPassesMax) and the
// thinning radius (1: face neighbours, 2: also their neighbours).
struct Tuning {
  int passes;
  int thin;
  int adjacent;  // 1: cavities of one pass may touch (see k_check in vd_build.cu)
  int exact_int;  // 1: conflict tests use the integer exact tier before the expansions
  int big_block;  // 1: oversized searches and stars go to whole-block kernels (k_cavity_big, k_commit_big)
};
// Kernel types for profiling.
enum {
  KT_PICK,
  KT_THIN,
  KT_CAVITY,
  KT_CHECK,
  KT_RECLAIM,
  KT_RELOCATE,
  KT_ACTIVATE,
  KT_EDGES,
  KT_DECIDE,
  KT_SMALL,
  KT_BIG,
  KT_BIGW,
  KT_SEED,
  KT_COUNT
};
extern const char* const kKernelTypeNames[KT_COUNT];
// Event log of one round: ev[0] before the first kernel, ev[i + 1] after
// kernel i, whose type is type[i].
struct Prof {
  static constexpr int kMax = 6 + 4 * kPassesMax;
  cudaEvent_t ev[kMax + 1];
  int type[kMax];
  int n;
};
// Kernel attributes the rounds need (shared-memory size); once per device
// before the first round or capture.
int prepare_round_kernels();
// One insertion round; its number is kept on the device (Counters::round,
// advanced by the round's first kernel), so a captured sequence of rounds
// can be replayed.
void launch_round(const DevTree& T, const Launch& L, int dim, const Tuning& tu, const Feed& fd, Prof* pf);
// One point inserted by a single warp (no rounds): its coordinates c[0..dim),
// its vertex id vid (the next one of the tree).  ctr->single receives the
// outcome (see k_insert_one in vd_build.cu).
void launch_insert_one(const DevTree& T, cudaStream_t stream, int dim, const double* c, int vid);
// The first `npts` points of `order` (the first `nlev` priority levels of a
// fresh single-set call, priorities under `seed`) inserted one after another
// by one block, the triangulation in shared memory (k_seed in vd_build.cu).
// On success the tree holds them, compacted, with their hints, and the level
// feed starts at level nlev; if a shared-memory capacity would be exceeded
// nothing is written and the rounds insert them.  npts <= seed_max_points(dim).
void launch_seed(const DevTree& T, cudaStream_t stream, int dim, int npts, int nlev, uint64_t seed);
int seed_max_points(int dim);
// Rounds while few points are active, in one cooperative launch (all blocks
// resident, grid barrier between phases): runs until the next round's active
// set reaches `max_active`, the call is done, `max_rounds` rounds ran, a pool
// overflowed or an error is flagged.  Returns E_CUDA if the launch is refused
// (then nothing ran).
int launch_small_rounds(const DevTree& T, cudaStream_t stream, int dim, const Tuning& tu, const Feed& fd,
                        int max_active, int max_rounds);

// Edges: counts / offsets / segment buffers are caller-provided device arrays.
struct EdgeScratch {
  int* cnt;        // n_in + 1
  int* off;        // n_in + 1
  int* buf;        // capacity cap_buf
  int* ucnt;       // n_in + 1
  int* uoff;       // n_in + 1
  int* big;        // list of vertices with long segments, capacity n_in
  int* nbig;       // 1 int
  int* scan_tmp;   // scan scratch (see scan_scratch_ints)
  int64_t cap_buf;
};
int64_t scan_scratch_ints(int64_t n);
// out[i] = sum(in[0..i)) for i < n, out[n] = total; tmp: scan_scratch_ints(n).
void scan_ints(const int* in, int* out, int64_t n, int* tmp, cudaStream_t st);
// Conflict regions of nq query points (vd_locate.cu): slots of query i in
// out[i * cap_per ..] numbered by rank[], count in counts[i] (-1: outside
// the super simplex; above cap_per: truncated).  rank[s] = position of live
// slot s among the
// live slots (nsimp + 1 entries, tmp: scan_scratch_ints(nsimp)).
void launch_locate(const DevTree& T, const Launch& L, int dim, const double* d_q, int nq, int cap_per,
                   const int* rank, int* out, int* counts);
void launch_live_rank(const DevTree& T, const Launch& L, int nsimp, int* flags, int* rank, int* tmp);
// Circumcentre (3 doubles, z = 0 in 2D) and radius of each live simplex,
// written at its rank.
void launch_circum(const DevTree& T, const Launch& L, int dim, int nsimp, const int* rank, double* centers,
                   double* radii);
void launch_edges(const DevTree& T, const Launch& L, int dim, int nsimp, int n_in,
                  const EdgeScratch& S, uint2* d_out);

// Device sizing of the super simplex (vd_size.cu).
void launch_bbox(const Launch& L, int dim, const double* d_xyz, int64_t n, unsigned long long* d_mm);
void launch_outside(const Launch& L, int dim, const double* d_xyz, int64_t n, const double* c, double r0,
                    int* d_flag);
void launch_close_chunks(const DevTree& T, const Launch& L);
// Batched build (vd_size.cu).  off[0..nsets] are the sets' first points
// (int64, device).  Per-set bounding box as order-preserving keys (mm[6 s +
// 0..2] minima, +3..5 maxima), the reference's "point not strictly inside"
// test against (cr[4 s + 0..2] centre, cr[4 s + 3] radius), and the set of
// every point.
void launch_set_bbox(const Launch& L, int dim, const double* d_xyz, const long long* off, int nsets,
                     unsigned long long* d_mm);
void launch_set_outside(const Launch& L, int dim, const double* d_xyz, const long long* off, int nsets,
                        const double* cr, int* d_flags);
void launch_set_fill(const Launch& L, const long long* off, int nsets, int* set_of);
// Edge pairs of global point numbers -> numbers within their set.
void launch_localize(const Launch& L, uint2* uv, int64_t m, const int* set_of, const long long* off);
// Edge offsets of the sets: eoff[s] = uoff[off[s]] (uoff: per-point edge
// offsets of the last extraction).
void launch_set_edge_offsets(const Launch& L, const int* uoff, const long long* off, int nsets,
                             long long* eoff);

// Sort and de-duplicate every bucket buf[off[u] .. off[u+1]) (u < n) in
// place (vd_edges.cu); ucnt[u] receives the unique count.  big (n ints) and
// nbig (1 int) are device scratch, h_pair pinned host scratch.  Synchronises;
// returns 0, or -1 on a CUDA error.  sort_big_buckets sorts the nbig long
// buckets listed in big[] (the warp pass leaves them to it).
int sort_buckets(const Launch& L, int n, const int* off, int* buf, int* ucnt, int* big, int* nbig, int* d_pair,
                 int* h_pair);
int sort_big_buckets(const Launch& L, int n, const int* off, int* buf, int* ucnt, const int* big, int nbig);
// Voronoi dual (vd_dual.cu).  Edges: with fill = false, cnt[rank] = interior
// facets each live slot owns and off = their exclusive scan over the nlive
// ranks; with fill = true, out[off[rank] ..] = (rank, partner rank) pairs.
void launch_dual_edges(const DevTree& T, const Launch& L, int dim, int nsimp, const int* rank, int* cnt, int* off,
                       int* tmp, int nlive, int2* out, bool fill);
// Cells: cnt (n_in + 1) = simplices incident to each input vertex, off = scan;
// fill scatters the live ranks into buf by vertex (cnt returns to zero).
void launch_cell_count(const DevTree& T, const Launch& L, int dim, int nsimp, int n_in, int* cnt, int* off,
                       int* tmp);
void launch_cell_fill(const DevTree& T, const Launch& L, int dim, int nsimp, int n_in, const int* rank, int* cnt,
                      const int* off, int* buf);

// Validator: out[0..5] = non-positive, asymmetric, not Delaunay (exact),
// not perturbed-Delaunay, hull facets, facets checked.
void launch_check(const DevTree& T, const Launch& L, int dim, int nsimp,
                  unsigned long long* d_out);

}  // namespace vd
