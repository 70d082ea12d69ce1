// Round-parallel Bowyer-Watson insertion on one GPU.
//
// One round replaces one `add_points_to_tree` batch of the reference
// (src/delaunay_tree.rs:336-386; queue + placement in src/scheduler.rs:6-55):
//
//   k_plan      one thread opens the round and activates priority levels.
//   k_activate  newly fed points walk from a location hint to the simplex
//               that contains them and vote.
//   k_pick      every simplex that holds uninserted points nominates the one
//               with the lowest priority (votes were cast by k_activate and
//               the previous k_relocate); a nominee claims its simplex and
//               the face neighbours (thinning) so that only locally lowest
//               nominees pay for a cavity search.
//   k_thin      nominees that lose a thinning claim, or duplicate a vertex of
//               their simplex, drop out (with thinning radius 0, k_pick does
//               the duplicate test and this kernel is not launched).
//   k_cavity    one warp per surviving nominee: search of the conflict region
//               from the simplex that contains it (`locate` +
//               `find_all_neighbors`, src/delaunay_tree.rs:33-75) with exact
//               perturbed in-sphere tests, collection of the boundary facets
//               (`get_new_simplices`, :77-123), then atomicMin claims with the
//               candidate's priority on the cavity (claim_c) and, in the
//               strict round mode, on every outer neighbour (claim_n).
//               Regions that outgrow a warp's shared memory are searched
//               again in the pool (by the warp, or by a block of
//               k_cavity_big once a call has had one).
//   k_check /   resolution passes, one warp per candidate: the independence
//   k_reclaim   test (see k_check), then winners write the star (killed slots
//               first, then fresh slots), link it internally by matching ridges
//               (`pair_simplices`, :674-695) and repoint the outer faces
//               (`insert_points_parallel`, :213-334).  In the default adjacent
//               mode a decide half and a commit half are separate kernels, and
//               the stars of winners that share a facet are stitched at the
//               start of k_relocate.  A round equals some sequential insertion
//               order.
//   k_relocate  one thread per uninserted point: points whose simplex was
//               removed walk inside the new star (faces through the new vertex
//               only) to the simplex that contains them; every point then votes
//               for the next round; survivors are compacted.
//
// A point is always located in a simplex that contains it, and a closed
// simplex meets its circumsphere only in its vertices, so the containing
// simplex is in conflict unless the point duplicates one of its vertices,
// which k_thin (or k_pick) detects and drops.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "vd_common.cuh"

namespace vd {
namespace {

constexpr unsigned FULL = 0xffffffffu;

template <int D>
struct Cap;
#ifndef VD_CAP3_C
#define VD_CAP3_C 128
#define VD_CAP3_F 192
#define VD_CAP3_H 256
#endif
#ifndef VD_CAVITY_MIN_BLOCKS
#define VD_CAVITY_MIN_BLOCKS 5
#endif
// resident 256-thread blocks per SM asked of the point-walk kernels (0: no bound)
#ifndef VD_WALK_MIN_BLOCKS
#define VD_WALK_MIN_BLOCKS 2
#endif
#if VD_WALK_MIN_BLOCKS > 0
#define VD_WALK_BOUNDS __launch_bounds__(256, VD_WALK_MIN_BLOCKS)
#else
#define VD_WALK_BOUNDS
#endif
template <>
struct Cap<3> {
  static constexpr int MAXC = VD_CAP3_C, MAXF = VD_CAP3_F, HS = VD_CAP3_H;
};
template <>
struct Cap<2> {
  static constexpr int MAXC = 64, MAXF = 96, HS = 128;
};

__device__ __forceinline__ int get4(const int4& a, int i) {
  return i == 0 ? a.x : (i == 1 ? a.y : (i == 2 ? a.z : a.w));
}
__device__ __forceinline__ int4 set4(int4 a, int i, int v) {
  if (i == 0) a.x = v;
  else if (i == 1) a.y = v;
  else if (i == 2) a.z = v;
  else a.w = v;
  return a;
}
__device__ __forceinline__ void load_simplex(const DevTree& T, int s, int4& v, int4& n) {
  if (bad_simp(T, s)) {
    set_error(T.ctr, E_INTERNAL);
    s = 0;
  }
  const int4* p = reinterpret_cast<const int4*>(T.simp + s);
  v = p[0];
  n = p[1];
}
__device__ __forceinline__ void store_simplex(const DevTree& T, int s, int4 v, int4 n) {
  if (bad_simp(T, s)) {
    set_error(T.ctr, E_INTERNAL);
    return;
  }
  int4* p = reinterpret_cast<int4*>(T.simp + s);
  p[0] = v;
  p[1] = n;
}
__device__ __forceinline__ vdp::VPt load_pt(const DevTree& T, int v) {
  if (bad_vert(T, v)) {
    set_error(T.ctr, E_INTERNAL);
    v = 0;
  }
  const double4_32a a = reinterpret_cast<const double4_32a*>(T.pts)[v];
  return vdp::VPt{a.x, a.y, a.z, a.w};
}

__device__ __forceinline__ vdp::FPt load_fpt(const DevTree& T, int v) {
  if (bad_vert(T, v)) {
    set_error(T.ctr, E_INTERNAL);
    v = 0;
  }
  const float4* p = reinterpret_cast<const float4*>(T.ptf + v);
  const float4 h = p[0], l = p[1];
  return vdp::FPt{h.x, h.y, h.z, h.w, l.x, l.y, l.z, l.w};
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(FULL, v, o);
  return v;
}
// Statistics: each warp adds its sums to one of kStatStripes copies of the
// counters, so that the warps of a launch, finishing together, do not all
// add to the same address (those atomics serialise in L2: about 3 % of a
// 1M-point build).  Counts that steer the build (winners, inserted) are
// summed per block instead (shared memory, one atomic per block).
__device__ void flush_tally(Counters* c, const vdp::Tally& t, unsigned tests, unsigned walk) {
  const unsigned long long v[STAT_COUNT] = {warp_sum(t.f32), warp_sum(t.f64), warp_sum(t.exact),
                                            warp_sum(t.sos), warp_sum(tests), warp_sum(walk)};
  if ((threadIdx.x & 31) == 0) {
    const unsigned stripe = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) % kStatStripes;
    for (int i = 0; i < STAT_COUNT; ++i)
      if (v[i]) atomicAdd(&c->stat[stripe][i], v[i]);
  }
}

// Warp-aggregated atomicMin of `val` into vote[loc] for all lanes with
// `active`; lanes that share a location are combined first.
__device__ __forceinline__ void vote_min(unsigned long long* vote, bool active, int loc,
                                         unsigned long long val) {
  unsigned am = __ballot_sync(FULL, active);
  if (!active) return;
  unsigned grp = __match_any_sync(am, loc);
  unsigned long long m = val;
  // min over the group: each lane pulls from every other member
  for (unsigned g = grp; g; g &= g - 1) {
    int src = __ffs(g) - 1;
    unsigned long long o = __shfl_sync(grp, val, src);
    m = o < m ? o : m;
  }
  if ((threadIdx.x & 31) == __ffs(grp) - 1) atomicMin(vote + loc, m);
}

// Warp-aggregated append; returns the slot for lanes with `flag`.
__device__ __forceinline__ int warp_append(int* counter, bool flag) {
  unsigned m = __ballot_sync(FULL, flag);
  if (!m) return -1;
  int lane = threadIdx.x & 31, leader = __ffs(m) - 1, base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(FULL, base, leader);
  return flag ? base + __popc(m & ((1u << lane) - 1)) : -1;
}

// ---------------------------------------------------------------------------
template <int D>
__global__ void k_upload(DevTree T, const double* xyz, long long n, int base) {
  constexpr int NV = D + 1;
  const double lo = 7.006492321624085e-46;  // 2^-150
  const double hi = 1.4272476927059599e45;  // 2^150
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  vdp::VPt sv[NV];
  int cur_set = -1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int set = set_index(T, base + (int)i);
    if (set != cur_set) {  // super simplex of the point's set
      cur_set = set;
      for (int j = 0; j < NV; ++j) sv[j] = load_pt(T, T.sets[set].sup[j]);
    }
    double c[3] = {xyz[i * D], xyz[i * D + 1], D == 3 ? xyz[i * D + 2] : 0.0};
    for (int k = 0; k < 3; ++k) {
      double a = fabs(c[k]);
      if (!(a <= 1.7976931348623157e308)) set_error(T.ctr, E_NONFINITE);
      else if (a != 0.0 && (a < lo || a > hi)) set_error(T.ctr, E_RANGE);
    }
    vdp::VPt p{c[0], c[1], c[2], 0.0};
    reinterpret_cast<double4_32a*>(T.pts)[base + i] = make_double4_32a(c[0], c[1], c[2], 0.0);
    T.ptf[base + i] = vdp::split_point(c[0], c[1], c[2]);
    if (vdp::exit_face<D, true>(sv, p, (1u << NV) - 1, tl, perr) >= 0) set_error(T.ctr, E_OUTSIDE);
  }
  if (perr) set_error(T.ctr, E_PRECISION);
}

// Multi-level grid of location hints, one per set.  Level l splits the
// set's sizing box (centre +- bounding radius) into 2^l cells per axis; each
// cell keeps the slot of a simplex created near it (written by every winner,
// races are harmless: any live simplex of the set is a valid walk start, a
// near one is a short walk).
//
// Cell of p at the finest level of set g, per axis, from the f32 high parts
// of its split coordinates (a hint cell need not be exact, and the FP64 pipe
// of this GPU is narrow); the cell of a coarser level l is this one shifted
// right by hint_levels - l, the same cell as floor(u * 2^l) gives directly.
// Most hint levels of a set (2D single set: 9).
constexpr int kHintLevelsMax = 9;
template <int D>
__device__ __forceinline__ void hint_cell(const SetGeo& g, const vdp::FPt& p, int* ic) {
  const int side = 1 << g.hint_levels;
  const float c[3] = {p.hx, p.hy, p.hz};
  for (int k = 0; k < D; ++k) {
    const float u = (c[k] - g.orgf[k]) * g.scalef;
    const int i = u > 0.0f ? (int)fminf(u * (float)side, (float)side) : 0;
    ic[k] = i >= side ? side - 1 : i;
  }
}
template <int D>
__device__ __forceinline__ int hint_at(const SetGeo& g, const int* ic, int level) {
  const int sh = g.hint_levels - level;
  int idx = 0;
  for (int k = D - 1; k >= 0; --k) idx = (idx << level) + (ic[k] >> sh);
  const int off = D == 3 ? ((1 << (3 * level)) - 1) / 7 : ((1 << (2 * level)) - 1) / 3;
  return g.hint_off + off + idx;
}

template <int D>
__device__ __forceinline__ void write_hints(const DevTree& T, int vid, const vdp::FPt& q, int slot) {
  const SetGeo& g = T.sets[set_index(T, vid)];
  int ic[3];
  hint_cell<D>(g, q, ic);
  for (int l = 0; l <= g.hint_levels; ++l) T.hint[hint_at<D>(g, ic, l)] = slot;
}

// The same with coarse levels sampled: a cell of level l covers 2^(D (L - l))
// cells of the finest level L, so it is written with probability
// 2^-(D (L - l)) (from the low bits of the point's priority).  Every cell
// then takes about as many writes as a finest cell, instead of every winner
// of a round storing to the one cell of level 0.  With `all` (while the
// tree is small and most fine cells are still empty) every level is written.
template <int D>
__device__ __forceinline__ void write_hints_sampled(const DevTree& T, int vid, const vdp::FPt& q, int slot,
                                                   unsigned pr, bool all) {
  const SetGeo& g = T.sets[set_index(T, vid)];
  int ic[3];
  hint_cell<D>(g, q, ic);
  for (int l = 0; l <= g.hint_levels; ++l) {
    const int sh = D * (g.hint_levels - l);
    if (all || sh == 0 || (sh < 32 && (pr & ((1u << sh) - 1u)) == 0)) T.hint[hint_at<D>(g, ic, l)] = slot;
  }
}

// Priority levels.  Level k holds the points with thr[k-1] <= priority <
// thr[k]; the thresholds grow geometrically, so level sizes do too (the
// biased randomized insertion order: every prefix of levels is a random
// sample of the input).
struct Thresholds {
  unsigned long long t[kMaxLevels];
  int n;
  double first;   // per-set levels (batched build): first level size
  double lgrow;   // and log of the growth factor
};

__device__ __forceinline__ int level_of(unsigned long long pr, const unsigned long long* t, int n) {
  int lo = 0, hi = n - 1;  // first k with pr < t[k]; t[n-1] = 2^32 holds every priority
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pr < t[mid]) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// Level of a point in a batched build: the set's own thresholds
// first * growth^k / n_set of the priority range.
__device__ __forceinline__ int set_level(const DevTree& T, int vid, unsigned long long pr, const Thresholds& th) {
  const double t0 = th.first / (double)T.sets[set_index(T, vid)].n * 4294967296.0;
  if ((double)pr < t0) return 0;
  const int k = 1 + (int)floor(log((double)pr / t0) / th.lgrow);
  return k < th.n - 1 ? k : th.n - 1;
}

__global__ void k_level_hist(DevTree T, long long n, int base, unsigned long long seed, Thresholds th,
                             int* counts) {
  __shared__ int sh[kMaxLevels];
  __shared__ unsigned long long st[kMaxLevels];
  for (int k = threadIdx.x; k < kMaxLevels; k += blockDim.x) {
    sh[k] = 0;
    st[k] = th.t[k];
  }
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
  {
    const unsigned long long pr = priority((uint32_t)(base + i), seed);
    atomicAdd(&sh[T.nsets == 1 ? level_of(pr, st, th.n) : set_level(T, base + (int)i, pr, th)], 1);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < th.n; k += blockDim.x)
    if (sh[k]) atomicAdd(counts + k, sh[k]);
}

// Level offsets (exclusive scan of the counts) and a fresh feed.
__global__ void k_level_init(DevTree T, const int* counts, int nlev) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int acc = 0;
  for (int k = 0; k < nlev; ++k) {
    T.lev_off[k] = acc;
    acc += counts[k];
  }
  for (int k = nlev; k <= kMaxLevels; ++k) T.lev_off[k] = acc;
  T.ctr->lev_next = 0;
  T.ctr->nlev = nlev;
  T.ctr->feed_lo = 0;
  T.ctr->feed_hi = 0;
}

// Scatter of the vertex ids into `order`, level by level.  Each tile of the
// block ranks its items per level in shared memory and reserves one range
// per level with a single global atomic.
__global__ void k_level_order(DevTree T, long long n, int base, unsigned long long seed, Thresholds th,
                              int* cursor) {
  __shared__ int cnt[kMaxLevels], gb[kMaxLevels];
  __shared__ unsigned long long st[kMaxLevels];
  for (int k = threadIdx.x; k < kMaxLevels; k += blockDim.x) {
    cnt[k] = 0;
    st[k] = th.t[k];
  }
  __syncthreads();
  for (long long b = blockIdx.x * (long long)blockDim.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    const long long i = b + threadIdx.x;
    int lev = -1, rank = 0;
    if (i < n) {
      const unsigned long long pr = priority((uint32_t)(base + i), seed);
      lev = T.nsets == 1 ? level_of(pr, st, th.n) : set_level(T, base + (int)i, pr, th);
      rank = atomicAdd(&cnt[lev], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < th.n; k += blockDim.x)
      if (cnt[k]) gb[k] = atomicAdd(cursor + k, cnt[k]);
    __syncthreads();
    if (lev >= 0) T.order[T.lev_off[lev] + gb[lev] + rank] = base + (int)i;
    __syncthreads();
    for (int k = threadIdx.x; k < th.n; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
  }
}

// Feed decision of a round (one thread): levels are activated while fewer
// than `ratio` x inserted points are active, and at least one level when no
// point is active.  Keeping the active set proportional to the triangulation
// keeps the share of points that win a round high, so few rounds are needed
// and each point is located and nominated only a few times.
__device__ __forceinline__ void plan_body(DevTree T, float ratio, int bid, int nblk) {
  if (threadIdx.x != 0 || bid != 0) return;
  Counters* c = T.ctr;
  const int round = c->round + 1;  // the round this launch opens
  c->round = round;
  long long a = c->nact[round & 1];
  const double target = (double)ratio * (double)c->ninserted;
  int lev = c->lev_next;
  const int first = lev;
  while (lev < c->nlev && (a == 0 || (double)a < target)) {
    a += T.lev_off[lev + 1] - T.lev_off[lev];
    ++lev;
  }
  c->feed_lo = T.lev_off[first];
  c->feed_hi = T.lev_off[lev];
  c->lev_next = lev;
}
__global__ void k_plan(DevTree T, float ratio) { plan_body(T, ratio, blockIdx.x, gridDim.x); }

// Activates the points planned for this round: each walks from the finest
// available grid hint to the simplex that contains it (visibility walk,
// exact orientation), joins the active list and votes for this round.
template <int D>
__device__ __forceinline__ void activate_body(DevTree T, unsigned long long seed, int bid, int nblk) {
  const int round = T.ctr->round;
  constexpr int NV = D + 1;
  const int par = round & 1;
  const unsigned long long ep = epoch(round);
  const int lo = T.ctr->feed_lo, n = T.ctr->feed_hi - lo;
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  unsigned walk = 0;
  const int cap = 1 << 16;
  for (int b = bid * blockDim.x; b < n; b += nblk * blockDim.x) {
    const int i = b + threadIdx.x;
    const bool act = i < n;
    int cur = 0, vid = 0;
    unsigned pr = 0;
    if (act) {
      vid = T.order[lo + i];
      if (bad_vert(T, vid)) {
        set_error(T.ctr, E_INTERNAL);
        vid = 0;
      }
      pr = priority((uint32_t)vid, seed);
      const vdp::FPt fp = load_fpt(T, vid);
      const SetGeo& g = T.sets[set_index(T, vid)];
      cur = -1;
      int ic[3];
      hint_cell<D>(g, fp, ic);
      // every level's hint in one round trip, then the finest that is set
      int hv[kHintLevelsMax + 1];
#pragma unroll
      for (int l = 0; l <= kHintLevelsMax; ++l) hv[l] = l <= g.hint_levels ? T.hint[hint_at<D>(g, ic, l)] : -1;
#pragma unroll
      for (int l = kHintLevelsMax; l >= 0; --l)
        if (cur < 0) cur = hv[l];
      if (cur < 0) cur = g.root;  // no insertion into the set yet: its super simplex
      int4 v, nn;
      load_simplex(T, cur, v, nn);
      for (int k = 0; k < 64 && v.x < 0; ++k) {  // dead slot: follow it into its star
        cur = nn.x >> 2;
        if (nn.x < 0 || bad_simp(T, cur)) {
          set_error(T.ctr, E_INTERNAL);
          cur = 0;
        }
        load_simplex(T, cur, v, nn);
      }
      int step = 0;
      for (; step < cap; ++step) {
        vdp::FPt fv[NV];
        for (int j = 0; j < NV; ++j) fv[j] = load_fpt(T, get4(v, j));
        auto load64 = [&](vdp::VPt* v64, vdp::VPt& p64) {
          for (int j = 0; j < NV; ++j) v64[j] = load_pt(T, get4(v, j));
          p64 = load_pt(T, vid);  // the f64 point only on the fallback path
        };
        const int f = vdp::exit_face_hl<D>(fv, fp, (1u << NV) - 1, tl, perr, load64);
        if (f < 0) break;
        const int code = get4(nn, f);
        if (code < 0 || bad_simp(T, code >> 2)) {
          set_error(T.ctr, code < 0 ? E_OUTSIDE : E_INTERNAL);
          break;
        }
        cur = code >> 2;
        load_simplex(T, cur, v, nn);
        ++walk;
      }
      if (step == cap) set_error(T.ctr, E_WALK);
    }
    vote_min(T.vote, act, cur, ep | pr);
    const int k = warp_append(&T.ctr->nact[par], act);
    if (act) T.act[par][k] = make_int4(vid, cur, (int)pr, 0);
  }
  if (perr) set_error(T.ctr, E_PRECISION);
  flush_tally(T.ctr, tl, 0, walk);
}
template <int D>
__global__ void VD_WALK_BOUNDS k_activate(DevTree T, unsigned long long seed) { activate_body<D>(T, seed, blockIdx.x, gridDim.x); }

// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ bool screen_nominee(const DevTree& T, int c, int4 e, int thin, int round);

// With thin == 0 the nominees are screened here (duplicates only; k_thin is
// not launched): the survivors go straight to work list stage 0, whose count
// k_relocate of the previous round set to 0.
template <int D>
__device__ __forceinline__ void pick_body(DevTree T, int thin, int bid, int nblk) {
  const int round = T.ctr->round;
  const int par = round & 1;
  if (bid == 0 && threadIdx.x == 0) {
    T.ctr->nact[par ^ 1] = 0;
    for (int k = 1; k < kStages; ++k) T.ctr->nwl[k] = 0;
    T.ctr->nwin = 0;
    T.ctr->win_lo = 0;
  }
  const int n = T.ctr->nact[par];
  const unsigned long long ep = epoch(round);
  unsigned long long ncand = 0;
  for (int b = bid * blockDim.x; b < n; b += nblk * blockDim.x) {
    int i = b + threadIdx.x;
    bool is = false;
    int4 e = make_int4(-1, 0, 0, 0);
    if (i < n) {
      e = T.act[par][i];
      is = e.x >= 0 && T.vote[e.y] == (ep | (unsigned)e.z);
    }
    int k = warp_append(&T.ctr->ncand, is);
    if (thin == 0) {
      const bool surv = is && k < T.cap_cand && screen_nominee<D>(T, k, make_int4(e.x, e.y, e.z, i), 0, round);
      const int w = warp_append(&T.ctr->nwl[0], surv);
      if (surv) T.wl[0][w] = k;
    }
    if (is) {
      ++ncand;
      if (k < T.cap_cand) T.cand[k] = make_int4(e.x, e.y, e.z, i);
      // thinning claim: the home simplex and its face neighbours
      const unsigned long long key = ep | (unsigned)e.z;
      int4 v, nn;
      if (thin == 0) continue;  // every nominee is searched
      load_simplex(T, e.y, v, nn);
      atomicMin(T.thin + e.y, key);
      const int nb[4] = {nn.x, nn.y, nn.z, nn.w};
      for (int f = 0; f < 4; ++f)
        if (nb[f] >= 0 && !bad_simp(T, nb[f] >> 2)) atomicMin(T.thin + (nb[f] >> 2), key);
    }
  }
  {
    __shared__ unsigned long long nb_acc;
    ncand = warp_sum(ncand);
    __syncthreads();
    if (threadIdx.x == 0) nb_acc = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && ncand) atomicAdd(&nb_acc, ncand);
    __syncthreads();
    if (threadIdx.x == 0 && nb_acc) atomicAdd(&T.ctr->candidates, nb_acc);
  }
}
template <int D>
__global__ void k_pick(DevTree T, int thin) { pick_body<D>(T, thin, blockIdx.x, gridDim.x); }

// Headers of a warp's items in a grid-stride loop over a candidate list,
// staged in shared memory: lane k loads item it0 + k * nw (its candidate,
// candidate record and state), one round trip for up to 32 items instead of
// three dependent loads per item.
struct HeadBuf {
  int c[32];
  int4 cd[32];
  int4 info[32];
};
__device__ __forceinline__ int load_heads(const DevTree& T, HeadBuf& H, const int* list, int it0, int nin, int nw,
                                          int lane) {
  const int n = min(32, (nin - it0 + nw - 1) / nw);
  __syncwarp();  // the previous batch is read
  if (lane < n) {
    const int c = list[it0 + lane * nw];
    H.c[lane] = c;
    H.cd[lane] = T.cand[c];
    H.info[lane] = T.cinfo[c];
  }
  __syncwarp();
  return n;
}

// Storage of one cavity search: shared memory for the common case, a
// reserved, 16-byte aligned stretch of the round's cavity pool when that
// overflows.  Generic pointers let the same code run on both.
struct CavStore {
  int* cav;     // simplex ids of the conflict region
  int4* cv;     // their vertex ids
  int4* cn;     // their neighbour codes
  int* hk;      // open-addressing set of cavity ids (hs slots, power of two)
  int2* fr;     // boundary facets: (outer code, (k << 2) | face); expanded to
                // 6-int records (new simplex vertices, outer code, (k << 2) | face)
                // when the lists are stored
  int maxc, maxf, hs;
};

// Spill stretch layout (ints): cavity ids | facet records | cv | cn | id set |
// ridge table (keys 2 ints + partners 2 ints per slot).  The search uses the
// first five parts, the commit of a large star the facets and the ridge table.
constexpr int kBigC = 8192, kBigF = 12288, kBigH = 32768, kBigR = 65536;
// Fresh simplex slots a warp takes at a time in k_check.
constexpr int kSlotChunk = 32;
constexpr int kOffF = kBigC;
constexpr int kOffCV = kOffF + 6 * kBigF;
constexpr int kOffCN = kOffCV + 4 * kBigC;
constexpr int kOffH = kOffCN + 4 * kBigC;
constexpr int kOffR = kOffH + kBigH;
constexpr int kBigInts = kOffR + 4 * kBigR;  // multiple of 4
// Dynamic shared memory of k_cavity_big: the id set (kBigH ints) and the
// ready marks (kBigC ints) of its block search.
constexpr int kBigSmem = (kBigH + kBigC) * (int)sizeof(int);
// Offset of the facet records after ncav cavity ids: even, so that records
// (6 ints) start on 8-byte boundaries in an even pool stretch.
__host__ __device__ constexpr int facets_at(int ncav) { return (ncav + 1) & ~1; }

__device__ bool hset_insert(int* hk, int hs, int key) {
  unsigned h = ((unsigned)key * 2654435761u) & (hs - 1);
  for (int probe = 0; probe < hs; ++probe) {
    int old = atomicCAS(&hk[h], -1, key);
    if (old == -1) return true;
    if (old == key) return false;
    h = (h + 1) & (hs - 1);
  }
  return false;
}
__device__ bool hset_find(const int* hk, int hs, int key) {
  unsigned h = ((unsigned)key * 2654435761u) & (hs - 1);
  for (int probe = 0; probe < hs; ++probe) {
    int k = *((volatile const int*)&hk[h]);
    if (k == key) return true;
    if (k == -1) return false;
    h = (h + 1) & (hs - 1);
  }
  return false;
}

struct WarpCtl {
  int ncav, nfac, flags, pad;
  int head, pend;  // block search: next item to hand out, items created and not finished
};

// Waits of one thread in the block search (cavity_search_dyn), at most:
// past it the search reports E_INTERNAL and ends instead of waiting on.
constexpr long long kDynWaitLimit = 1LL << 24;

// Block form of the search (k_cavity_big), without waves: threads take
// (simplex, face) items from a shared counter as soon as the simplex is
// stored, so a slow conflict test (FP64 or exact tier) holds up only the
// items behind it, not a whole wave at a barrier.  `pend` counts items
// created and not yet finished; a simplex adds its D + 1 items before its
// parent item finishes and before it is marked ready, so the count reaches
// zero only when the region is complete.  rdy[k] marks cavity entry k as
// stored (rdy: S.maxc ints, in shared memory).  Same region, facets
// and capacity flags as the wave form; only the order of the lists differs.
template <int D, int XT>
__device__ void cavity_search_dyn(const DevTree& T, const CavStore& S, WarpCtl& ctl, int* rdy, int rank,
                                  int start, int4 v0, int4 n0, int qv, const vdp::FPt& fq, vdp::Tally& tl,
                                  int& perr, unsigned& ntests) {
  constexpr int NV = D + 1;
  const int G = (int)blockDim.x;
  for (int i = rank; i < S.hs; i += G) S.hk[i] = -1;
  for (int i = rank; i < S.maxc; i += G) rdy[i] = 0;
  __syncthreads();
  if (rank == 0) {
    ctl.ncav = 1;
    ctl.nfac = 0;
    ctl.flags = 0;
    ctl.head = 0;
    ctl.pend = NV;
    S.cav[0] = start;
    S.cv[0] = v0;
    S.cn[0] = n0;
    hset_insert(S.hk, S.hs, start);
    rdy[0] = 1;
  }
  __syncthreads();
  long long waits = 0;
  while (true) {
    const int it = atomicAdd(&ctl.head, 1);
    const int k = it / NV, f = it - k * NV;
    bool ready = false;
    while (true) {
      if (k < S.maxc && k < *(volatile int*)&ctl.ncav && *(volatile int*)&rdy[k]) {
        ready = true;
        break;
      }
      if (*(volatile int*)&ctl.pend == 0 || *(volatile int*)&ctl.flags) break;
      if (++waits > kDynWaitLimit) {
        set_error(T.ctr, E_INTERNAL);
        atomicOr(&ctl.flags, 4);
        break;
      }
      __nanosleep(32);
    }
    if (!ready) break;
    __threadfence_block();  // the entry's records after its ready mark
    const int code = get4(__ldcg(&S.cn[k]), f);  // from L2: another thread stored it
    bool facet = code < 0;
    const bool broken = !facet && bad_simp(T, code >> 2);
    if (broken) set_error(T.ctr, E_INTERNAL);
    if (!facet && !broken) {
      const int nb = code >> 2;
      if (!hset_find(S.hk, S.hs, nb)) {
        int4 vv, nn;
        load_simplex(T, nb, vv, nn);
        vdp::FPt fv[NV];
        int kv[NV];
        for (int j = 0; j < NV; ++j) {
          kv[j] = get4(vv, j);
          fv[j] = load_fpt(T, kv[j]);
        }
        ++ntests;
        auto load64 = [&](vdp::VPt* v64, vdp::VPt& q64) {
          for (int j = 0; j < NV; ++j) v64[j] = load_pt(T, kv[j]);
          q64 = load_pt(T, qv);
        };
        if (vdp::in_conflict_hl<D, XT>(fv, kv, fq, qv, tl, perr, load64)) {
          if (hset_insert(S.hk, S.hs, nb)) {
            const int s = atomicAdd(&ctl.ncav, 1);
            if (s < S.maxc) {
              S.cav[s] = nb;
              S.cv[s] = vv;
              S.cn[s] = nn;
              atomicAdd(&ctl.pend, NV);  // before the mark: the parent item is still counted
              __threadfence_block();
              *(volatile int*)&rdy[s] = 1;
            } else {
              atomicOr(&ctl.flags, 1);
            }
          }
        } else {
          facet = true;
        }
      }
    }
    if (facet) {
      const int s = atomicAdd(&ctl.nfac, 1);
      if (s < S.maxf) S.fr[s] = make_int2(code, (k << 2) | f);
      else atomicOr(&ctl.flags, 2);
    }
    atomicSub(&ctl.pend, 1);
  }
  __syncthreads();
}

// Breadth-first search of the conflict region of candidate q from the
// simplex that contains it; all 32 lanes of the warp call this.  Returns
// with ctl.flags != 0 if a capacity was exceeded.
//
// BLOCK: the whole block searches (k_cavity_big, lane = thread index, waves
// of blockDim.x items); ctl.pad carries the wave's item count, published by
// thread 0 so that every thread leaves the loop after the same barrier.
template <int D, int XT, bool BLOCK = false>
__device__ void cavity_search(const DevTree& T, const CavStore& S, WarpCtl& ctl, int lane, int start,
                              int4 v0, int4 n0, int qv, const vdp::FPt& fq, vdp::Tally& tl, int& perr,
                              unsigned& ntests) {
  constexpr int NV = D + 1;
  const int G = BLOCK ? (int)blockDim.x : 32;
  auto sync = [] {
    if (BLOCK)
      __syncthreads();
    else
      __syncwarp();
  };
  for (int i = lane; i < S.hs; i += G) S.hk[i] = -1;
  if (lane == 0) {
    ctl.ncav = 1;
    ctl.nfac = 0;
    ctl.flags = 0;
    S.cav[0] = start;
    S.cv[0] = v0;
    S.cn[0] = n0;
  }
  sync();
  if (lane == 0) hset_insert(S.hk, S.hs, start);
  sync();
  // (simplex, face) items are taken in waves of G in discovery order, not
  // level by level: a wave also takes the items of simplices the previous
  // wave appended, so a search needs about items / G dependent rounds of
  // gathers rather than one or more per level
  int head = 0, levels = 0;
  while (true) {
    int avail;
    if (BLOCK) {
      if (lane == 0) {
        const int a = min(*(volatile int*)&ctl.ncav, S.maxc) * NV;
        ctl.pad = (*(volatile int*)&ctl.flags || head >= a) ? -1 : a;
      }
      sync();
      avail = *(volatile int*)&ctl.pad;
      if (avail < 0) break;
    } else {
      avail = min(*(volatile int*)&ctl.ncav, S.maxc) * NV;
      if (*(volatile int*)&ctl.flags || head >= avail) break;
    }
    ++levels;
    const int it = head + lane;
    if (it < avail) {
      const int k = it / NV, f = it - k * NV;
      const int code = get4(S.cn[k], f);
      bool facet = code < 0;
      const bool broken = !facet && bad_simp(T, code >> 2);
      if (broken) set_error(T.ctr, E_INTERNAL);
      if (!facet && !broken) {
        const int nb = code >> 2;
        if (!hset_find(S.hk, S.hs, nb)) {
          int4 vv, nn;
          load_simplex(T, nb, vv, nn);
          vdp::FPt fv[NV];
          int kv[NV];
          for (int j = 0; j < NV; ++j) {
            kv[j] = get4(vv, j);
            fv[j] = load_fpt(T, kv[j]);
          }
          ++ntests;
          auto load64 = [&](vdp::VPt* v64, vdp::VPt& q64) {
            for (int j = 0; j < NV; ++j) v64[j] = load_pt(T, kv[j]);
            q64 = load_pt(T, qv);  // reloaded: the rare FP64 path need not hold q in registers
          };
          if (vdp::in_conflict_hl<D, XT>(fv, kv, fq, qv, tl, perr, load64)) {
            if (hset_insert(S.hk, S.hs, nb)) {
              int s = atomicAdd(&ctl.ncav, 1);
              if (s < S.maxc) {
                S.cav[s] = nb;
                S.cv[s] = vv;
                S.cn[s] = nn;
              } else {
                atomicOr(&ctl.flags, 1);
              }
            }
          } else {
            facet = true;
          }
        }
      }
      if (facet) {
        int s = atomicAdd(&ctl.nfac, 1);
        if (s < S.maxf) {
          S.fr[s] = make_int2(code, (k << 2) | f);
        } else {
          atomicOr(&ctl.flags, 2);
        }
      }
    }
    sync();
    head += min(G, avail - head);
  }
  sync();
  if (lane == 0 && levels > 64) atomicMax(&T.ctr->max_levels, levels);
}

// Thinning test of one nominee (one thread): it must hold the thinning claim
// on its simplex and on every face neighbour; with `thin` >= 2 no lower
// nominee may claim a simplex two faces away either.
// Exact coordinate equality (as vdp::same_point) on the bit patterns, with
// +0 and -0 equal: integer compares instead of FP64 ones.
__device__ __forceinline__ bool same_bits(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a);
  const unsigned long long y = (unsigned long long)__double_as_longlong(b);
  return x == y || ((x | y) << 1) == 0ull;
}
__device__ __forceinline__ bool same_point_bits(const vdp::VPt& a, const vdp::VPt& b) {
  return same_bits(a.x, b.x) && same_bits(a.y, b.y) && same_bits(a.z, b.z);
}

template <int D>
__device__ bool thin_lost1(const DevTree& T, int home, int4 n0, unsigned long long key, int thin) {
  constexpr int NV = D + 1;
  if (thin == 0) return false;
  // every load is issued before any test decides, so that the claims of the
  // home simplex, its face neighbours and (thin >= 2) their neighbours
  // arrive in two round trips
  int nb[NV];
  for (int f = 0; f < NV; ++f) {
    const int x = get4(n0, f);
    nb[f] = (x < 0 || bad_simp(T, x >> 2)) ? -1 : x >> 2;
  }
  unsigned long long th[NV];
  int4 n2[NV];
  const unsigned long long own = T.thin[home];
  for (int f = 0; f < NV; ++f) {
    th[f] = nb[f] >= 0 ? T.thin[nb[f]] : key;
    n2[f] = make_int4(-1, -1, -1, -1);
    if (thin >= 2 && nb[f] >= 0) {
      int4 v2;
      load_simplex(T, nb[f], v2, n2[f]);
    }
  }
  bool lost = own != key;
  for (int f = 0; f < NV; ++f) lost |= th[f] != key;
  if (thin >= 2) {
    for (int f = 0; f < NV; ++f)
      for (int g = 0; g < NV; ++g) {
        const int x = get4(n2[f], g);
        if (x >= 0 && !bad_simp(T, x >> 2)) lost |= T.thin[x >> 2] < key;
      }
  }
  return lost;
}

// One nominee c (record e): duplicate test against the vertices of its
// simplex, then the thinning test.  Returns whether it goes on to the search.
template <int D>
__device__ __forceinline__ bool screen_nominee(const DevTree& T, int c, int4 e, int thin, int round) {
  constexpr int NV = D + 1;
  const int par = round & 1;
  int4 v, n;
  load_simplex(T, e.y, v, n);
  const vdp::VPt q = load_pt(T, e.x);
  int dup = -1;
  for (int j = 0; j < NV; ++j) {
    const int vid = get4(v, j);
    if (same_point_bits(load_pt(T, vid), q)) dup = vid;
  }
  if (dup >= 0) {
    T.act[par][e.w].x = -1;
    const int k = atomicAdd(&T.ctr->ndup, 1);
    if (k < T.cap_dups) T.dups[k] = make_int2(e.x, dup);
    T.cinfo[c] = make_int4(0, 0, 0, ST_DUP);
    return false;
  }
  if (thin_lost1<D>(T, e.y, n, epoch(round) | (unsigned)e.z, thin)) {
    T.cinfo[c] = make_int4(0, 0, 0, ST_LOST);
    return false;
  }
  return true;
}

// Per nominee (one thread): duplicate test against the vertices of its
// simplex and the thinning test; survivors go to work list stage 0.
template <int D>
__device__ __forceinline__ void thin_body(DevTree T, int thin, int bid, int nblk) {
  const int round = T.ctr->round;
  const int nc = min(T.ctr->ncand, T.cap_cand);
  for (int b = bid * blockDim.x; b < nc; b += nblk * blockDim.x) {
    const int c = b + threadIdx.x;
    const bool survive = c < nc && screen_nominee<D>(T, c, T.cand[c], thin, round);
    const int k = warp_append(&T.ctr->nwl[0], survive);
    if (survive) T.wl[0][k] = c;
  }
}
template <int D>
__global__ void k_thin(DevTree T, int thin) { thin_body<D>(T, thin, blockIdx.x, gridDim.x); }

template <int D>
struct WarpCav {
  WarpCtl ctl;
  int cav[Cap<D>::MAXC];
  int4 cv[Cap<D>::MAXC];
  int4 cn[Cap<D>::MAXC];
  int hkey[Cap<D>::HS];
  int2 fr[Cap<D>::MAXF];
};

// Claims of a candidate for one resolution pass: its cavity in claim_c, every
// outer neighbour in claim_n (not in adjacent mode, where cavities may touch).
// P = cavity ids, F = facet records.
// Facet records of a search, expanded for the later kernels: the new
// simplex on facet (k, f) has the vertices of cavity simplex k with v[f]
// replaced by the candidate's point qv.
__device__ __forceinline__ void expand_facets(const int2* fr, const int4* cv, int nfac, int qv, int* F, int lane) {
  for (int j = lane; j < nfac; j += 32) {
    const int2 e = fr[j];
    const int4 nv4 = set4(cv[e.y >> 2], e.y & 3, qv);
    int2* r = reinterpret_cast<int2*>(F + 6 * j);  // records start on 8-byte boundaries
    r[0] = make_int2(nv4.x, nv4.y);
    r[1] = make_int2(nv4.z, nv4.w);
    r[2] = e;
  }
}

__device__ __forceinline__ void claim_region(const DevTree& T, const int* P, int ncav, const int* F,
                                             int nfac, unsigned long long key, int lane, int adjacent) {
  for (int i = lane; i < ncav; i += 32) atomicMin(T.claim_c + P[i], key);
  if (adjacent) return;
  for (int j = lane; j < nfac; j += 32) {
    const int o = F[6 * j + 4];
    if (o >= 0 && !bad_simp(T, o >> 2)) atomicMin(T.claim_n + (o >> 2), key);
  }
}

// Search of a conflict region too large for a warp's shared memory, with
// its lists in a reserved stretch of the round's pool (global memory); a
// warp (BLOCK = false) or the whole block (k_cavity_big) runs it.  The
// stretch offset is broadcast through ctl.pad.
template <int D, int XT, bool BLOCK>
__device__ void big_search(const DevTree& T, WarpCtl& ctl, int* bsm, int rank, int c, int4 cd, int4 v0, int4 n0,
                           const vdp::FPt& fq, unsigned long long key, int adjacent, vdp::Tally& tl, int& perr,
                           unsigned& ntests, int& mcav, int& mfac) {
  auto sync = [] {
    if (BLOCK)
      __syncthreads();
    else
      __syncwarp();
  };
  if (rank == 0) {
    const int o = atomicAdd(&T.ctr->pool_used, kBigInts + 4);
    ctl.pad = (o + 3) & ~3;  // int4 alignment of cv / cn
  }
  sync();
  const int off = *(volatile int*)&ctl.pad;
  sync();
  if (off + kBigInts > T.cap_pool) {
    if (rank == 0) {
      T.cinfo[c] = make_int4(0, 0, 0, ST_POOL);
      atomicAdd(&T.ctr->pool_overflow, 1);
    }
    sync();
    return;
  }
  int* P = T.pool + off;
  // the search's 2-int facet records go to the ridge-table area (unused
  // until the commit) and are expanded to P + kOffF afterwards
  // the block search keeps its id set and ready marks in shared memory (bsm)
  const CavStore big{P, reinterpret_cast<int4*>(P + kOffCV), reinterpret_cast<int4*>(P + kOffCN),
                     BLOCK ? bsm : P + kOffH, reinterpret_cast<int2*>(P + kOffR), kBigC, kBigF, kBigH};
  if constexpr (BLOCK)
    cavity_search_dyn<D, XT>(T, big, ctl, bsm + kBigH, rank, cd.y, v0, n0, cd.x, fq, tl, perr, ntests);
  else
    cavity_search<D, XT, false>(T, big, ctl, rank, cd.y, v0, n0, cd.x, fq, tl, perr, ntests);
  const int ncav = min(*(volatile int*)&ctl.ncav, kBigC), nfac = min(*(volatile int*)&ctl.nfac, kBigF);
  const int flags = *(volatile int*)&ctl.flags;
  sync();
  if (flags) {
    if (rank == 0) {
      T.cinfo[c] = make_int4(ncav, nfac, 0, ST_OVERFLOW);
      atomicAdd(&T.ctr->overflow, 1);
    }
    sync();
    return;
  }
  // the facets stay at P + kOffF; cinfo.y carries the flag (see cand_lists)
  const int G = BLOCK ? (int)blockDim.x : 32;
  for (int j = rank; j < nfac; j += G) {
    const int2 e = big.fr[j];
    const int4 nv4 = set4(big.cv[e.y >> 2], e.y & 3, cd.x);
    int2* r = reinterpret_cast<int2*>(P + kOffF + 6 * j);
    r[0] = make_int2(nv4.x, nv4.y);
    r[1] = make_int2(nv4.z, nv4.w);
    r[2] = e;
  }
  sync();
  for (int i = rank; i < ncav; i += G) atomicMin(T.claim_c + P[i], key);
  if (!adjacent)
    for (int j = rank; j < nfac; j += G) {
      const int o = P[kOffF + 6 * j + 4];
      if (o >= 0 && !bad_simp(T, o >> 2)) atomicMin(T.claim_n + (o >> 2), key);
    }
  if (rank == 0) T.cinfo[c] = make_int4(ncav, nfac | (1 << 30), off, ST_OK);
  mcav = max(mcav, ncav);
  mfac = max(mfac, nfac);
  sync();
}

template <int D, int XT>
__device__ __forceinline__ void cavity_body(DevTree T, int adjacent, int bid, int nblk, WarpCav<D>* smem,
                                            bool defer_big) {
  const int round = T.ctr->round;
  constexpr int MAXC = Cap<D>::MAXC, MAXF = Cap<D>::MAXF, HS = Cap<D>::HS;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpCav<D>& W = smem[wib];
  const unsigned long long pe = pass_epoch(round, 0);
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  unsigned ntests = 0;
  unsigned long long nsearched = 0, nspill = 0;
  int mcav = 0, mfac = 0;
  // pool space is taken in per-warp chunks (one atomic per chunk, not per
  // candidate); what a warp leaves unused is dropped with the round's pool
  const int pchunk = max(256, min(8192, T.cap_pool / (nblk * 16))) & ~1;  // offsets stay even
  int pbase = 0, pleft = 0;
  const CavStore fast{W.cav, W.cv, W.cn, W.hkey, W.fr, MAXC, MAXF, HS};
  const int nw = nblk * 4;
  const int nsurv = T.ctr->nwl[0];
  // the list entry and candidate record of the warp's next item are read one
  // search ahead, so that a search starts with one round trip (its point and
  // start simplex) instead of three
  int it = bid * 4 + wib;
  int c_next = it < nsurv ? T.wl[0][it] : 0;
  int4 cd_next = it < nsurv ? T.cand[c_next] : make_int4(0, 0, 0, 0);
  int c_after = it + nw < nsurv ? T.wl[0][it + nw] : 0;
  for (; it < nsurv; it += nw) {
    const int c = c_next;
    const int4 cd = cd_next;
    const vdp::FPt fq = load_fpt(T, cd.x);
    int4 v0, n0;
    load_simplex(T, cd.y, v0, n0);
    if (it + nw < nsurv) {
      c_next = c_after;
      cd_next = T.cand[c_after];
    }
    if (it + 2 * nw < nsurv) c_after = T.wl[0][it + 2 * nw];
    if (lane == 0) ++nsearched;
    const unsigned long long key = pe | (unsigned)cd.z;
    cavity_search<D, XT>(T, fast, W.ctl, lane, cd.y, v0, n0, cd.x, fq, tl, perr, ntests);
    int ncav = min(W.ctl.ncav, MAXC), nfac = min(W.ctl.nfac, MAXF);
    int off = 0;
    if (W.ctl.flags) {
      // spill: the region outgrew shared memory; the search is redone in a
      // reserved pool stretch, by the whole block of k_cavity_big or here
      if (lane == 0) ++nspill;
      if (defer_big) {
        if (lane == 0) {
          T.bigc[atomicAdd(&T.ctr->nbig, 1)] = c;
          T.cinfo[c] = make_int4(0, 0, 0, ST_BIG);
        }
      } else {
        big_search<D, XT, false>(T, W.ctl, nullptr, lane, c, cd, v0, n0, fq, key, adjacent, tl, perr, ntests, mcav,
                                 mfac);
      }
      __syncwarp();
      continue;
    }
    const int need = facets_at(ncav) + nfac * 6;
    if (need > pleft) {
      const int take = max(need, pchunk);
      if (lane == 0) pbase = atomicAdd(&T.ctr->pool_used, take);
      pbase = __shfl_sync(FULL, pbase, 0);
      pleft = take;
      if (pbase + take > T.cap_pool) pleft = 0;
    }
    if (need > pleft) {
      if (lane == 0) {
        T.cinfo[c] = make_int4(ncav, nfac, 0, ST_POOL);
        atomicAdd(&T.ctr->pool_overflow, 1);
      }
      __syncwarp();
      continue;
    }
    off = pbase;
    pbase += need;
    pleft -= need;
    int* P = T.pool + off;
    for (int i = lane; i < ncav; i += 32) P[i] = W.cav[i];
    int* F = P + facets_at(ncav);
    expand_facets(W.fr, W.cv, nfac, cd.x, F, lane);
    __syncwarp();
    claim_region(T, W.cav, ncav, F, nfac, key, lane, adjacent);
    if (lane == 0) T.cinfo[c] = make_int4(ncav, nfac, off, ST_OK);
    mcav = max(mcav, ncav);
    mfac = max(mfac, nfac);
    __syncwarp();
  }
  if (perr) set_error(T.ctr, E_PRECISION);
  flush_tally(T.ctr, tl, ntests, 0);
  {
    __shared__ unsigned long long cs[2];
    __shared__ int cm[2];
    nsearched = warp_sum(nsearched);
    nspill = warp_sum(nspill);
    __syncthreads();
    if (threadIdx.x == 0) cs[0] = cs[1] = 0, cm[0] = cm[1] = 0;
    __syncthreads();
    if (lane == 0) {
      if (nsearched) atomicAdd(&cs[0], nsearched);
      if (nspill) atomicAdd(&cs[1], nspill);
      if (mcav) atomicMax(&cm[0], mcav);
      if (mfac) atomicMax(&cm[1], mfac);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (cs[0]) atomicAdd(&T.ctr->searched, cs[0]);
      if (cs[1]) atomicAdd(&T.ctr->spilled, cs[1]);
      if (cm[0]) atomicMax(&T.ctr->max_cav, cm[0]);
      if (cm[1]) atomicMax(&T.ctr->max_fac, cm[1]);
    }
  }
}
template <int D, int XT>
__global__ void __launch_bounds__(128, VD_CAVITY_MIN_BLOCKS) k_cavity(DevTree T, int adjacent, int defer_big) {
  __shared__ WarpCav<D> smem[4];
  cavity_body<D, XT>(T, adjacent, blockIdx.x, gridDim.x, smem, defer_big != 0);
}

// The searches k_cavity deferred (ST_BIG): one block per search, waves of
// 512 (simplex, face) items.
template <int D, int XT>
__global__ void __launch_bounds__(512, 1) k_cavity_big(DevTree T, int adjacent) {
  __shared__ WarpCtl ctl;
  extern __shared__ int bsm[];  // kBigSmem bytes: the search's id set, then its ready marks
  const int n = T.ctr->nbig;
  if (n == 0) return;
  const unsigned long long pe = pass_epoch(T.ctr->round, 0);
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0, mcav = 0, mfac = 0;
  unsigned ntests = 0;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const int c = T.bigc[i];
    const int4 cd = T.cand[c];
    const vdp::FPt fq = load_fpt(T, cd.x);
    int4 v0, n0;
    load_simplex(T, cd.y, v0, n0);
    big_search<D, XT, true>(T, ctl, bsm, threadIdx.x, c, cd, v0, n0, fq, pe | (unsigned)cd.z, adjacent, tl, perr, ntests,
                            mcav, mfac);
  }
  if (perr) set_error(T.ctr, E_PRECISION);
  flush_tally(T.ctr, tl, ntests, 0);
  if (threadIdx.x == 0) {
    if (mcav) atomicMax(&T.ctr->max_cav, mcav);
    if (mfac) atomicMax(&T.ctr->max_fac, mfac);
  }
}

// Pool layout of a searched candidate: cavity ids at P, facet records at
// P + facets_at(ncav) (8-byte aligned), or at P + kOffF for a spilled (large)
// search, flagged by bit 30
// of cinfo.y.
__device__ __forceinline__ void cand_lists(const DevTree& T, const int4& info, int*& P, int*& F, int& ncav,
                                           int& nfac, bool& big) {
  P = T.pool + info.z;
  ncav = info.x;
  big = (info.y >> 30) & 1;
  nfac = info.y & ((1 << 30) - 1);
  F = big ? P + kOffF : P + facets_at(ncav);
}

template <int D>
struct WarpCommit {
  // ridge table: a star of f facets has f D / 2 ridges; the table is paired
  // in sweeps of at most 2/3 HR ridges each (one sweep below 170 ridges in
  // 3D, 85 in 2D)
  static constexpr int HR = D == 3 ? 256 : 128;
  unsigned long long rk[HR];   // ridge key (r0 << 32 | r1)
  int ra[HR];                  // first half-ridge to arrive (facet << 2 | face), -2 once paired
  int id[Cap<D>::MAXF];
  int first[Cap<D>::MAXC];     // first facet index of each cavity simplex
  int freeslot[Cap<D>::MAXC];  // cavity slots without an own facet
  HeadBuf hb;
};

// Ridge of face g of new simplex r (vertices r[0..3], new vertex at qf): the
// vertices other than r[g] and the new vertex, smaller first (2D: one vertex).
template <int D>
__device__ __forceinline__ void ridge_of(const int* r, int g, int qf, int& r0, int& r1) {
  r0 = -1;
  r1 = -1;
  for (int i = 0; i < D + 1; ++i) {
    if (i == g || i == qf) continue;
    if (r0 < 0) r0 = r[i];
    else r1 = r[i];
  }
  if (D == 3 && r1 < r0) {
    const int t = r0;
    r0 = r1;
    r1 = t;
  }
}

// Writes one new simplex and repoints its outer neighbour.  An outer
// neighbour that another winner of this round removed (adjacent mode) is left
// alone: the two new simplices on that facet are linked at the start of
// k_relocate (fix_body).
__device__ __forceinline__ bool emit_simplex(const DevTree& T, const int* r, int myid, int4 nn, int round) {
  const int4 v = make_int4(r[0], r[1], r[2], r[3]);
  const int qf = r[5] & 3, o = r[4];
  store_simplex(T, myid, v, nn);
  if (o < 0 || bad_simp(T, o >> 2)) return false;
  if (T.killed[o >> 2].x == round) return true;  // another winner's cavity: linked by fix_body
  reinterpret_cast<int*>(T.simp + (o >> 2))[4 + (o & 3)] = (myid << 2) | qf;
  T.touched[o >> 2] = round;
  return false;
}

// Star of one winner, small case.  The new simplices are written first, each
// with its outer neighbour; then their faces through the new vertex are
// paired.  Such a face is determined by its ridge (its vertices other than
// the new vertex), and every ridge of the star belongs to exactly two new
// simplices.  The half-ridges go into a shared-memory table keyed by the
// ridge; the second half of a ridge to arrive finds the first and writes the
// two links.  A star with more ridges than 2/3 of the table is paired in
// several sweeps, each over the ridges of one residue of the key hash.
__device__ __forceinline__ unsigned ridge_hash(int r0, int r1) {
  return ((unsigned)r0 * 0x9E3779B1u) ^ ((unsigned)r1 * 0x85EBCA77u);
}
// Returns, per lane, a bit for each of its facets (j = lane, lane + 32, ...)
// whose outer neighbour another winner of this round removed.
template <int D>
__device__ unsigned write_star(const DevTree& T, WarpCommit<D>& W, const int* __restrict__ FR, int nfac, int qv,
                               int round, int lane) {
  constexpr int NV = D + 1;
  constexpr int HR = WarpCommit<D>::HR;
  constexpr int LOG_HR = D == 3 ? 8 : 7;
  constexpr int PER_SWEEP = 2 * HR / 3;
  const unsigned long long EMPTY = ~0ull;
  unsigned dead = 0;
  for (int j = lane, bit = 0; j < nfac; j += 32, ++bit) {
    const int* r = FR + 6 * j;
    const int qf = r[5] & 3;
    if (emit_simplex(T, r, W.id[j], set4(make_int4(-1, -1, -1, -1), qf, r[4]), round)) dead |= 1u << bit;
  }
  const int sweeps = (nfac * D / 2 + PER_SWEEP - 1) / PER_SWEEP;
  // the table is empty on entry (cleared when the warp starts, and after
  // every sweep by the check below)
  for (int sw = 0; sw < sweeps; ++sw) {
    __syncwarp();  // also orders the record stores above before the link stores below
    for (int j = lane; j < nfac; j += 32) {
      // the facet record in three 8-byte loads (records are 8-byte aligned)
      const int2* r2 = reinterpret_cast<const int2*>(FR + 6 * j);
      const int2 a = r2[0], b = r2[1], c = r2[2];
      const int r[6] = {a.x, a.y, b.x, b.y, c.x, c.y};
      const int qf = r[5] & 3;
      const int idj = W.id[j];
#pragma unroll
      for (int g = 0; g < NV; ++g) {
        if (g == qf) continue;
        int r0, r1;
        ridge_of<D>(r, g, qf, r0, r1);
        const unsigned hv = ridge_hash(r0, r1);
        if (sweeps > 1 && (int)((hv & 0xffffu) % (unsigned)sweeps) != sw) continue;
        const unsigned long long key = ((unsigned long long)(unsigned)r0 << 32) | (unsigned)r1;
        const int mine = (j << 2) | g;
        unsigned h = hv >> (32 - LOG_HR);
        for (int probe = 0; probe < HR; ++probe, h = (h + 1) & (HR - 1)) {
          const unsigned long long old = atomicCAS(&W.rk[h], EMPTY, key);
          if (old != EMPTY && old != key) continue;
          const int other = atomicCAS(&W.ra[h], -1, mine);
          if (other >= 0) {
            // second half: link both new simplices across the ridge
            W.ra[h] = -2;
            const int m = other >> 2, gm = other & 3;
            reinterpret_cast<int*>(T.simp + idj)[4 + g] = (W.id[m] << 2) | gm;
            reinterpret_cast<int*>(T.simp + W.id[m])[4 + gm] = (idj << 2) | g;
          }
          break;
        }
      }
    }
    __syncwarp();
    // a ridge with one half would be a broken star; the table is emptied
    // for the next sweep or star
    for (int i = lane; i < HR; i += 32) {
      if (W.ra[i] >= 0) set_error(T.ctr, E_INTERNAL);
      W.rk[i] = EMPTY;
      W.ra[i] = -1;
    }
    __syncwarp();
  }
  return dead;
}

// Star of one winner, large case: every (facet, face) inserts its ridge into
// an open-addressing table (two halves per ridge), then reads its partner.
// A warp (BLOCK = false) or the whole block (k_commit_big) writes it.
template <int D, bool BLOCK = false>
__device__ void write_star_big(const DevTree& T, const int* FR, const int* ID, int nfac, int round,
                               int* R, int lane) {
  constexpr int NV = D + 1;
  const int G = BLOCK ? (int)blockDim.x : 32;
  auto sync = [] {
    if (BLOCK)
      __syncthreads();
    else
      __syncwarp();
  };
  const unsigned mask = kBigR - 1;
  for (int i = lane; i < 4 * kBigR; i += G) R[i] = -1;
  sync();
  // R[4h] = r0, R[4h+1] = r1 (key), R[4h+2], R[4h+3] = the two half-ridges
  for (int it = lane; it < nfac * NV; it += G) {
    const int j = it / NV, g = it - j * NV;
    const int* r = FR + 6 * j;
    const int qf = r[5] & 3;
    if (g == qf) continue;
    int r0, r1;
    ridge_of<D>(r, g, qf, r0, r1);
    unsigned h = ((unsigned)r0 * 2654435761u ^ (unsigned)(r1 + 1) * 40503u) & mask;
    for (int probe = 0; probe < kBigR; ++probe, h = (h + 1) & mask) {
      const int old = atomicCAS(&R[4 * h], -1, r0);
      if (old == -1 || old == r0) {
        // r0 matches or was just written: settle the second key word
        const int o1 = atomicCAS(&R[4 * h + 1], -1, r1);
        if (o1 == -1 || o1 == r1) {
          const int side = atomicCAS(&R[4 * h + 2], -1, (j << 2) | g) == -1 ? 2 : 3;
          if (side == 3) R[4 * h + 3] = (j << 2) | g;
          break;
        }
      }
    }
  }
  sync();
  for (int j = lane; j < nfac; j += G) {
    const int* r = FR + 6 * j;
    const int qf = r[5] & 3;
    int4 nn = make_int4(-1, -1, -1, -1);
    nn = set4(nn, qf, r[4]);
    for (int g = 0; g < NV; ++g) {
      if (g == qf) continue;
      int r0, r1;
      ridge_of<D>(r, g, qf, r0, r1);
      unsigned h = ((unsigned)r0 * 2654435761u ^ (unsigned)(r1 + 1) * 40503u) & mask;
      int other = -1;
      for (int probe = 0; probe < kBigR; ++probe, h = (h + 1) & mask) {
        if (R[4 * h] == -1) break;
        if (R[4 * h] == r0 && R[4 * h + 1] == r1) {
          const int a = R[4 * h + 2], b = R[4 * h + 3];
          other = a == ((j << 2) | g) ? b : a;
          break;
        }
      }
      if (other < 0) {
        set_error(T.ctr, E_INTERNAL);
        continue;
      }
      const int m = other >> 2;
      if (m >= nfac) {
        set_error(T.ctr, E_INTERNAL);
        continue;
      }
      nn = set4(nn, g, (ID[m] << 2) | (other & 3));
    }
    emit_simplex(T, r, ID[j], nn, round);
  }
  sync();
}

// Adjacent mode, commit half of a large star after its links: facets shared
// with another winner's cavity publish this side's new simplex and record
// where the other side's goes (fix_body).
template <bool BLOCK>
__device__ __forceinline__ void publish_shared_facets(const DevTree& T, int* F, const int* P, const int* IDS,
                                                      int nfac, int round, int lane) {
  const int G = BLOCK ? (int)blockDim.x : 32;
  for (int j = lane; j < nfac; j += G) {
    const int o = F[6 * j + 4];
    if (o < 0 || bad_simp(T, o >> 2) || T.killed[o >> 2].x != round) continue;
    const int kf = F[6 * j + 5], k = kf >> 2;
    const int inner = (P[k] << 2) | (kf & 3);  // the removed simplex and its face on this facet
    T.repl[inner] = (IDS[j] << 2) | (kf & 3);
    F[6 * j] = IDS[j];
    F[6 * j + 1] = kf & 3;
    F[6 * j + 2] = -2;
  }
}

// The same for a small star, from the facets write_star marked (no second
// read of the kill marks).
__device__ __forceinline__ void publish_marked(const DevTree& T, int* F, const int* P, const int* IDS, int nfac,
                                               unsigned dead, int lane) {
  for (int j = lane, bit = 0; j < nfac; j += 32, ++bit) {
    if (!((dead >> bit) & 1u)) continue;
    const int kf = F[6 * j + 5], k = kf >> 2;
    const int inner = (P[k] << 2) | (kf & 3);
    T.repl[inner] = (IDS[j] << 2) | (kf & 3);
    F[6 * j] = IDS[j];
    F[6 * j + 1] = kf & 3;
    F[6 * j + 2] = -2;
  }
}

// Resolution pass `pass` of a round, check half.  A candidate wins iff it
// holds every claim on its cavity, no lower candidate rewrites a face of its
// cavity (claim_n), and no lower candidate's cavity holds one of its outer
// neighbours.  Winners are pairwise independent (disjoint cavities, no
// cavity meets another's outer shell), so a pass equals inserting its
// winners one after the other.  Losers stay pending; k_reclaim lets those
// whose region no winner of this round touched claim again, so candidates
// that lost only to other losers still get in (winners grow toward a
// maximal independent set).
//
// Slots: the new simplex built on a boundary facet of cavity simplex k reuses
// the slot of k when it is the first facet of k, so a point that was inside
// k usually finds itself in (or next to) the simplex now in k's slot.
//
// Adjacent mode (MODE 1 + 2) relaxes independence to disjoint cavities.  A
// candidate whose boundary facet touches the cavity of a lower candidate X
// (claim_c of the outer simplex holds X's key; X is recovered from its
// priority) wins only if X's point is outside the new simplex it would build
// on that facet: then the two new simplices on the facet are locally
// Delaunay and inserting both equals inserting them one after the other.
// MODE 1 decides (claims, facet tests, fresh slots, kill marks) for all
// candidates of the pass, so that MODE 2, which writes the stars, knows every
// simplex removed in the pass and leaves links into them to fix_body.
template <int D, int MODE, int XT>
__device__ __forceinline__ void check_body(DevTree T, int pass, int last, unsigned long long seed, int bid, int nblk,
                                           unsigned char* dsm, bool defer_big = false) {
  constexpr int NV = D + 1;
  const int round = T.ctr->round;
  if (MODE == 1 && bid == 0 && threadIdx.x == 0) T.ctr->nbigw = 0;  // stars deferred by this pass's commit
  const int sin = 2 * pass, sout = 2 * pass + 1;
  constexpr int MAXF = Cap<D>::MAXF, MAXC = Cap<D>::MAXC;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // MODE 1 gets only the item headers in shared memory, the others a WarpCommit each
  WarpCommit<D>& W = reinterpret_cast<WarpCommit<D>*>(dsm)[wib];
  HeadBuf& H = MODE == 1 ? reinterpret_cast<HeadBuf*>(dsm)[wib] : W.hb;
  if (MODE != 1) {
    // empty ridge table for write_star (which leaves it empty after each star)
    for (int i = lane; i < WarpCommit<D>::HR; i += 32) {
      W.rk[i] = ~0ull;
      W.ra[i] = -1;
    }
    __syncwarp();
  }
  const unsigned long long pe = pass_epoch(round, pass);
  const int par = round & 1;
  const bool hint_all = T.ctr->ninserted < T.hint_all_below;
  unsigned long long nwon = 0, ncreated = 0, nkilled = 0;
  int nholes = 0;
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  // fresh simplex slots come from a per-warp chunk kept across launches
  const int gw = bid * 4 + wib;
  int2 chunk = (MODE != 2 && gw < T.cap_wchunk) ? T.wchunk[gw] : make_int2(0, 0);
  const int nw = nblk * 4;
  const int lo = MODE == 2 ? T.ctr->win_lo : 0;
  const int nin = MODE == 2 ? T.ctr->nwin : T.ctr->nwl[sin];
  const int* list = MODE == 2 ? T.win : T.wl[sin & 1];
  for (int it0 = lo + bid * 4 + wib; it0 < nin; it0 += 32 * nw) {
    // lane k loads the list entry, state and candidate record of the warp's
    // k-th next item: one round trip for up to 32 items instead of three each
    const int nh = load_heads(T, H, list, it0, nin, nw, lane);
    for (int k = 0; k < nh; ++k) {
      const int c = H.c[k];
      const int4 info = H.info[k];
      if (info.w != (MODE == 2 ? ST_WIN : ST_OK)) continue;
      const int4 cd = H.cd[k];
      const unsigned long long key = pe | (unsigned)cd.z;
      int *P, *F, ncav, nfac;
      bool big;
      cand_lists(T, info, P, F, ncav, nfac, big);
      // the winner's point for its hints, read now so that it arrives while the star is written
      vdp::FPt fq{};
      if (MODE != 1 && lane == 0) fq = load_fpt(T, cd.x);
      int base;
      if (MODE != 2) {
        // the cavity's and the outer simplices' claims are read together:
        // pool entries in one round trip, all their claims in the next, and
        // only then decided (a verdict needs every one of them anyway)
        bool ok = true;
        const int nrun = max(ncav, nfac);
        for (int t = lane; t < nrun; t += 32) {
          const bool hs = t < ncav, hf = t < nfac;
          const int s = hs ? P[t] : 0;
          const int o = hf ? F[6 * t + 4] : -1;
          const bool sbad = hs && bad_simp(T, s);
          const bool obad = o >= 0 && bad_simp(T, o >> 2);
          const unsigned long long kc = (hs && !sbad) ? T.claim_c[s] : key;
          const unsigned long long kn = (MODE == 0 && hs && !sbad) ? T.claim_n[s] : ~0ull;
          const unsigned long long ko = (o >= 0 && !obad) ? T.claim_c[o >> 2] : ~0ull;
          ok = ok && !sbad && !obad && kc == key && (MODE == 1 || kn > key);
          if (!ok || o < 0) continue;
          if (MODE == 0) {
            ok = ko > key;
          } else if (ko < key) {
            // the lower candidate X whose cavity holds the outer simplex
            const int xv = (int)vertex_of_priority((uint32_t)ko, seed);
            if (bad_vert(T, xv)) {
              ok = false;
              continue;
            }
            const int* r = F + 6 * t;
            vdp::FPt fv[NV];
            for (int i = 0; i < NV; ++i) fv[i] = load_fpt(T, r[i]);
            const vdp::FPt fx = load_fpt(T, xv);
            auto load64 = [&](vdp::VPt* v64, vdp::VPt& p64) {
              for (int i = 0; i < NV; ++i) v64[i] = load_pt(T, r[i]);
              p64 = load_pt(T, xv);
            };
            ok = !vdp::in_conflict_hl<D, XT>(fv, r, fx, xv, tl, perr, load64);
          }
        }
        if (!__all_sync(FULL, ok)) {
          if (lane == 0) {
            if (last) {
              T.cinfo[c].w = ST_LOST;
            } else {
              const int k = atomicAdd(&T.ctr->nwl[sout], 1);
              T.wl[sout & 1][k] = c;
            }
          }
          continue;
        }
        const int fresh = max(0, nfac - ncav);
        if (fresh > chunk.y) {
          const int take = max(fresh, kSlotChunk);
          int b0 = 0;
          if (lane == 0) b0 = atomicAdd(&T.ctr->nsimp, take);
          b0 = __shfl_sync(FULL, b0, 0);
          chunk = make_int2(b0, take);
          if (b0 + take > T.cap_simp) {
            if (lane == 0) {
              atomicAdd(&T.ctr->wasted, take);
              atomicExch(&T.ctr->simp_overflow, 1);
            }
            chunk = make_int2(0, 0);
          }
        }
        if (fresh > chunk.y) {
          if (lane == 0) T.cinfo[c].w = ST_LOST;
          continue;
        }
        base = chunk.x;
        chunk.x += fresh;
        chunk.y -= fresh;
        for (int i = lane; i < ncav; i += 32) T.killed[P[i]] = make_int2(round, cd.x);
        ++nwon;
        if (MODE == 1) {
          if (lane == 0) {
            T.cand[c].y = base;  // the home simplex is not needed any more
            T.cinfo[c].w = ST_WIN;
            T.win[atomicAdd(&T.ctr->nwin, 1)] = c;
          }
          __syncwarp();
          continue;
        }
      } else {
        base = cd.y;
      }
      int id0;
      const int* IDS;
      unsigned dead = 0;
      bool small_star = false;
      if (!big && nfac <= MAXF && ncav <= MAXC) {
        // slot assignment: first facet of cavity simplex k takes k's slot;
        // the other facets take the remaining cavity slots, then fresh ones
        for (int i = lane; i < ncav; i += 32) W.first[i] = 0x7fffffff;
        __syncwarp();
        for (int j = lane; j < nfac; j += 32) atomicMin(&W.first[__ldg(F + 6 * j + 5) >> 2], j);
        __syncwarp();
        int nfree = 0;  // cavity slots without an own facet, ranked
        for (int i0 = 0; i0 < ncav; i0 += 32) {
          const int i = i0 + lane;
          const bool fr = i < ncav && W.first[i] == 0x7fffffff;
          const unsigned m = __ballot_sync(FULL, fr);
          if (fr) W.freeslot[nfree + __popc(m & ((1u << lane) - 1))] = P[i];
          nfree += __popc(m);
        }
        int nsec = 0;  // facets that are not the first of their cavity simplex
        for (int j0 = 0; j0 < nfac; j0 += 32) {
          const int j = j0 + lane;
          int id = 0;
          bool sec = false;
          if (j < nfac) {
            const int k = __ldg(F + 6 * j + 5) >> 2;
            sec = W.first[k] != j;
            if (!sec) id = P[k];
          }
          const unsigned m = __ballot_sync(FULL, sec);
          if (sec) {
            const int t = nsec + __popc(m & ((1u << lane) - 1));
            id = t < nfree ? W.freeslot[t] : base + (t - nfree);
          }
          if (j < nfac) W.id[j] = id;
          nsec += __popc(m);
        }
        __syncwarp();
        id0 = W.id[0];
        IDS = W.id;
        // leftover cavity slots become holes pointing into the star
        for (int t = nsec + lane; t < nfree; t += 32)
          store_simplex(T, W.freeslot[t], make_int4(-1, -1, -1, -1), make_int4(id0 << 2, -1, -1, -1));
        dead = write_star<D>(T, W, F, nfac, cd.x, round, lane);
        small_star = true;
      } else {
        // large star (spilled search): plain slot assignment, ids in the
        // stretch's vertex-list area (free after the search), ridge table in
        // its own area; with defer_big the whole block of k_commit_big
        // writes it (and the rest of this winner's commit)
        if (MODE == 2 && defer_big) {
          if (lane == 0) T.bigw[atomicAdd(&T.ctr->nbigw, 1)] = c;
          __syncwarp();
          continue;
        }
        int* ID = P + kOffCV;
        for (int j = lane; j < nfac; j += 32) ID[j] = j < ncav ? P[j] : base + (j - ncav);
        __syncwarp();
        id0 = ID[0];
        IDS = ID;
        for (int i = nfac + lane; i < ncav; i += 32)
          store_simplex(T, P[i], make_int4(-1, -1, -1, -1), make_int4(id0 << 2, -1, -1, -1));
        write_star_big<D>(T, F, ID, nfac, round, P + kOffR, lane);
      }
      if (MODE == 2) {
        // facets shared with another winner's cavity: publish this side's new
        // simplex and remember where the other side's goes (fix_body)
        __syncwarp();
        if (small_star)
          publish_marked(T, F, P, IDS, nfac, dead, lane);
        else
          publish_shared_facets<false>(T, F, P, IDS, nfac, round, lane);
      }
      if (lane == 0) {
        write_hints_sampled<D>(T, cd.x, fq, id0, (unsigned)cd.z, hint_all);
        T.cinfo[c].w = ST_DONE;
        T.act[par][cd.w].x = -1;
      }
      ncreated += nfac;
      nkilled += ncav;
      nholes += max(0, ncav - nfac);
      __syncwarp();
    }
  }
  if (perr) set_error(T.ctr, E_PRECISION);
  if (MODE == 1) flush_tally(T.ctr, tl, 0, 0);
  if (lane == 0 && MODE != 2 && gw < T.cap_wchunk) T.wchunk[gw] = chunk;
  {
    // per-warp counts (the same in every lane) summed over the block
    __shared__ unsigned long long ks[4];  // won, created, killed, holes
    __syncthreads();
    if (threadIdx.x < 4) ks[threadIdx.x] = 0;
    __syncthreads();
    if (lane == 0) {
      if (nwon) atomicAdd(&ks[0], nwon);
      if (ncreated) atomicAdd(&ks[1], ncreated);
      if (nkilled) atomicAdd(&ks[2], nkilled);
      if (nholes) atomicAdd(&ks[3], (unsigned long long)nholes);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (ks[0]) {
        atomicAdd(&T.ctr->won[min(pass, kPassesMax - 1)], ks[0]);
        atomicAdd(&T.ctr->winners, (int)ks[0]);
        atomicAdd(&T.ctr->ninserted, (int)ks[0]);
      }
      if (ks[1]) atomicAdd(&T.ctr->created, ks[1]);
      if (ks[2]) atomicAdd(&T.ctr->killed, ks[2]);
      if (ks[3]) atomicAdd(&T.ctr->holes, (int)ks[3]);
    }
  }
}
// resident 128-thread blocks per SM asked of the decide / commit kernels (0:
// no bound).  Without one the compiler keeps them at 48-56 registers and
// spills; with 6 (at most 85 registers) the commit half has none and the
// 1M-point build is 1.6 % faster than with no bound (4 and 8 measured too).
#ifndef VD_CHECK_MIN_BLOCKS
#define VD_CHECK_MIN_BLOCKS 6
#endif
#if VD_CHECK_MIN_BLOCKS > 0
#define VD_CHECK_BOUNDS __launch_bounds__(128, VD_CHECK_MIN_BLOCKS)
#else
#define VD_CHECK_BOUNDS __launch_bounds__(128)
#endif
template <int D, int MODE, int XT>
__global__ void VD_CHECK_BOUNDS k_check(DevTree T, int pass, int last, unsigned long long seed, int defer_big) {
  extern __shared__ __align__(16) unsigned char dsm[];
  check_body<D, MODE, XT>(T, pass, last, seed, blockIdx.x, gridDim.x, dsm, defer_big != 0);
}

// The large stars the commit half deferred: one block per winner writes its
// star, publishes its shared facets and its hints.
template <int D>
__global__ void __launch_bounds__(512, 1) k_commit_big(DevTree T) {
  const int n = T.ctr->nbigw;
  if (n == 0) return;
  const int round = T.ctr->round;
  const int par = round & 1;
  unsigned long long ncreated = 0, nkilled = 0;
  int nholes = 0;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const int c = T.bigw[i];
    const int4 info = T.cinfo[c];
    const int4 cd = T.cand[c];
    int *P, *F, ncav, nfac;
    bool big;
    cand_lists(T, info, P, F, ncav, nfac, big);
    const int base = cd.y;
    int* ID = P + kOffCV;
    for (int j = threadIdx.x; j < nfac; j += blockDim.x) ID[j] = j < ncav ? P[j] : base + (j - ncav);
    __syncthreads();
    const int id0 = ID[0];
    for (int k = nfac + threadIdx.x; k < ncav; k += blockDim.x)
      store_simplex(T, P[k], make_int4(-1, -1, -1, -1), make_int4(id0 << 2, -1, -1, -1));
    write_star_big<D, true>(T, F, ID, nfac, round, P + kOffR, threadIdx.x);
    publish_shared_facets<true>(T, F, P, ID, nfac, round, threadIdx.x);
    if (threadIdx.x == 0) {
      write_hints<D>(T, cd.x, load_fpt(T, cd.x), id0);
      T.cinfo[c].w = ST_DONE;
      T.act[par][cd.w].x = -1;
    }
    ncreated += nfac;
    nkilled += ncav;
    nholes += max(0, ncav - nfac);
    __syncthreads();
  }
  if (threadIdx.x == 0 && ncreated) {
    atomicAdd(&T.ctr->created, ncreated);
    atomicAdd(&T.ctr->killed, nkilled);
    if (nholes) atomicAdd(&T.ctr->holes, nholes);
  }
}

// Adjacent mode, end of a round: a new simplex whose outer neighbour another
// winner removed takes, as that neighbour, the other winner's new simplex on
// the same facet.
__device__ __forceinline__ void fix_body(DevTree T, int bid, int nblk) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = nblk * (blockDim.x >> 5);
  const int n = T.ctr->nwin;
  const long long nrepl = 4LL * T.cap_simp;
  // the last warps of the grid take the winners, so that in a small round the
  // first warps, which relocate the points, do not wait for this chain first
  for (int it = nw - 1 - (bid * (blockDim.x >> 5) + wib); it < n; it += nw) {
    const int c = T.win[it];
    const int4 info = T.cinfo[c];
    if (info.w != ST_DONE) continue;
    int *P, *F, ncav, nfac;
    bool big;
    cand_lists(T, info, P, F, ncav, nfac, big);
    for (int j = lane; j < nfac; j += 32) {
      if (F[6 * j + 2] != -2) continue;
      const int id = F[6 * j], g = F[6 * j + 1], o = F[6 * j + 4];
      if (bad_simp(T, id) || o < 0 || o >= nrepl) {
        set_error(T.ctr, E_INTERNAL);
        continue;
      }
      reinterpret_cast<int*>(T.simp + id)[4 + g] = T.repl[o];
    }
  }
}

// Resolution pass `pass` >= 1, claim half: a pending loser whose cavity holds
// a simplex that a winner of this round removed or repointed, or whose outer
// neighbour a winner removed, drops out for this round; the others claim
// again with this pass's key (smaller than every earlier key of the round).
template <int D>
__device__ __forceinline__ void reclaim_body(DevTree T, int pass, int adjacent, int bid, int nblk) {
  const int round = T.ctr->round;
  if (bid == 0 && threadIdx.x == 0) T.ctr->win_lo = T.ctr->nwin;  // winners of this pass start here
  const int sin = 2 * pass - 1, sout = 2 * pass;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nc = min(T.ctr->ncand, T.cap_cand);
  const unsigned long long pe = pass_epoch(round, pass);
  const int nw = nblk * 4;
  const int nin = T.ctr->nwl[sin];
  for (int it = bid * 4 + wib; it < nin; it += nw) {
    const int c = T.wl[sin & 1][it];
    const int4 info = T.cinfo[c];
    if (info.w != ST_OK) continue;
    const int4 cd = T.cand[c];
    int *P, *F, ncav, nfac;
    bool big;
    cand_lists(T, info, P, F, ncav, nfac, big);
    // bitwise ors: every mark is loaded, none waits for an earlier verdict
    bool blocked = false;
    for (int i = lane; i < ncav; i += 32) {
      const int s = P[i];
      blocked |= (T.killed[s].x == round) | (T.touched[s] == round);
    }
    for (int j = lane; j < nfac; j += 32) {
      const int o = F[6 * j + 4];
      if (o >= 0) blocked |= T.killed[o >> 2].x == round;
    }
    if (__any_sync(FULL, blocked)) {
      if (lane == 0) T.cinfo[c].w = ST_LOST;
      continue;
    }
    claim_region(T, P, ncav, F, nfac, pe | (unsigned)cd.z, lane, adjacent);
    if (lane == 0) {
      const int k = atomicAdd(&T.ctr->nwl[sout], 1);
      T.wl[sout & 1][k] = c;
    }
  }
}
template <int D>
__global__ void __launch_bounds__(128) k_reclaim(DevTree T, int pass, int adjacent) { reclaim_body<D>(T, pass, adjacent, blockIdx.x, gridDim.x); }

template <int D>
__device__ __forceinline__ void relocate_body(DevTree T, int bid, int nblk) {
  // adjacent mode: first link the stars of winners that share facets (the
  // walks below stay inside stars, so they do not need those links)
  fix_body(T, bid, nblk);
  const int round = T.ctr->round;
  constexpr int NV = D + 1;
  const int par = round & 1;
  if (bid == 0 && threadIdx.x == 0) {
    T.ctr->ncand = 0;
    T.ctr->nwl[0] = 0;  // k_pick may append to stage 0 (thin == 0)
    T.ctr->pool_used = 0;
    T.ctr->nbig = 0;
  }
  const int n = T.ctr->nact[par];
  const unsigned long long ep1 = epoch(round + 1);
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  unsigned walk = 0;
  const int cap = 4096;
  for (int b = bid * blockDim.x; b < n; b += nblk * blockDim.x) {
    const int i = b + threadIdx.x;
    bool keep = false;
    int4 e = make_int4(-1, -1, 0, 0);
    if (i < n) {
      e = T.act[par][i];
      if (e.x >= 0) {
        keep = true;
        if (bad_simp(T, e.y)) {
          set_error(T.ctr, E_INTERNAL);
          e.y = 0;
        }
        const int2 kr = T.killed[e.y];
        if (kr.x == round) {
          int cur = e.y;
          int4 v, nn;
          load_simplex(T, cur, v, nn);
          if (v.x < 0) {
            cur = nn.x >> 2;
            if (nn.x < 0 || bad_simp(T, cur)) {
              set_error(T.ctr, E_INTERNAL);
              cur = e.y;
            }
            load_simplex(T, cur, v, nn);
          }
          const vdp::FPt fp = load_fpt(T, e.x);
          int step = 0;
          for (; step < cap; ++step) {
            int qpos = 0;
            for (int j = 0; j < NV; ++j)
              if (get4(v, j) == kr.y) qpos = j;
            vdp::FPt fv[NV];
            for (int j = 0; j < NV; ++j) fv[j] = load_fpt(T, get4(v, j));
            const unsigned mask = ((1u << NV) - 1) & ~(1u << qpos);
            auto load64 = [&](vdp::VPt* v64, vdp::VPt& p64) {
              for (int j = 0; j < NV; ++j) v64[j] = load_pt(T, get4(v, j));
              p64 = load_pt(T, e.x);
            };
            const int f = vdp::exit_face_hl<D>(fv, fp, mask, tl, perr, load64);
            if (f < 0) break;
            cur = get4(nn, f) >> 2;
            if (get4(nn, f) < 0 || bad_simp(T, cur)) {
              set_error(T.ctr, E_INTERNAL);
              cur = e.y;
              break;
            }
            load_simplex(T, cur, v, nn);
            ++walk;
          }
          if (step == cap) set_error(T.ctr, E_WALK);
          e.y = cur;
        }
      }
    }
    vote_min(T.vote, keep, e.y, ep1 | (unsigned)e.z);
    const int k = warp_append(&T.ctr->nact[par ^ 1], keep);
    if (keep) T.act[par ^ 1][k] = e;
  }
  if (perr) set_error(T.ctr, E_PRECISION);
  flush_tally(T.ctr, tl, 0, walk);
}
template <int D>
__global__ void VD_WALK_BOUNDS k_relocate(DevTree T) { relocate_body<D>(T, blockIdx.x, gridDim.x); }

// ---------------------------------------------------------------------------
// Small rounds in one launch.  While few points are active a round is a
// latency chain of about ten short kernels; here whole rounds run in one
// cooperative launch (every block resident) with a grid barrier between the
// phases.  The barrier's waits are bounded: a block that waits more than about
// a second flags an error and the launch ends, so a fault in the protocol
// cannot hang the device.
__device__ __forceinline__ bool grid_sync(Counters* c, int nblk) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = &c->bar_gen;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(&c->bar_count, 1u) == (unsigned)nblk - 1) {
      c->bar_count = 0;
      __threadfence();
      atomicAdd(&c->bar_gen, 1u);
    } else {
      long long spin = 0;
      while (*gen == g) {
        if (++spin > (1LL << 24)) {
          atomicExch(&c->bar_abort, 1);
          set_error(c, E_INTERNAL);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int*)&c->bar_abort == 0;
}

template <int D>
__global__ void __launch_bounds__(128) k_rounds_small(DevTree T, Tuning tu, unsigned long long seed, float ratio,
                                                      int max_active, int max_rounds) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int bid = blockIdx.x, nblk = gridDim.x;
  Counters* c = T.ctr;
  for (int r = 0; r < max_rounds; ++r) {
    plan_body(T, ratio, bid, nblk);
    if (!grid_sync(c, nblk)) return;
    activate_body<D>(T, seed, bid, nblk);
    if (!grid_sync(c, nblk)) return;
    pick_body<D>(T, tu.thin, bid, nblk);
    if (!grid_sync(c, nblk)) return;
    if (tu.thin > 0) {
      thin_body<D>(T, tu.thin, bid, nblk);
      if (!grid_sync(c, nblk)) return;
    }
    cavity_body<D, 0>(T, tu.adjacent, bid, nblk, reinterpret_cast<WarpCav<D>*>(dsm), false);
    if (!grid_sync(c, nblk)) return;
    for (int p = 0; p < tu.passes; ++p) {
      const int last = p == tu.passes - 1;
      if (p > 0) {
        reclaim_body<D>(T, p, tu.adjacent, bid, nblk);
        if (!grid_sync(c, nblk)) return;
      }
      if (tu.adjacent) {
        check_body<D, 1, 0>(T, p, last, seed, bid, nblk, dsm);
        if (!grid_sync(c, nblk)) return;
        check_body<D, 2, 0>(T, p, last, seed, bid, nblk, dsm);
      } else {
        check_body<D, 0, 0>(T, p, last, seed, bid, nblk, dsm);
      }
      if (!grid_sync(c, nblk)) return;
    }
    relocate_body<D>(T, bid, nblk);
    if (!grid_sync(c, nblk)) return;
    if (bid == 0 && threadIdx.x == 0) {
      const int next = c->nact[(c->round & 1) ^ 1];
      const bool done = c->lev_next >= c->nlev && next == 0;
      const bool grow = c->simp_overflow || c->pool_overflow || c->overflow ||
                        (double)c->nsimp > 0.85 * (double)T.cap_simp;
      c->coop_go = (!done && !grow && c->err == 0 && next < max_active) ? 1 : 0;
    }
    if (!grid_sync(c, nblk)) return;
    if (*(volatile int*)&c->coop_go == 0) return;
  }
}

// ---------------------------------------------------------------------------
// One point, one warp: TreeUpdate::new + insert_point (src/delaunay_tree.rs:
// 709-740, :125-211), the reference's sequential path (src/lib.rs:108-114),
// without the round machinery.  The warp checks and stores the point, walks
// to the simplex that contains it, searches the conflict region in shared
// memory, writes the star into the removed slots (then fresh ones) and links
// it, all in one launch.  No other insertion runs at the same time, so no
// claims are needed, and no point is waiting to be relocated.  The outcome
// goes to ctr->single: 0 inserted, E_DUPLICATE (skipped and recorded),
// another error code, or -1 when the region outgrew the warp's shared memory
// and nothing but the point record was written (the caller then inserts it
// through the rounds).
template <int D>
__global__ void __launch_bounds__(32) k_insert_one(DevTree T, double x, double y, double z, int vid) {
  constexpr int NV = D + 1;
  constexpr int MAXC = Cap<D>::MAXC, MAXF = Cap<D>::MAXF, HS = Cap<D>::HS;
  constexpr int HR = WarpCommit<D>::HR;
  __shared__ WarpCav<D> C;
  __shared__ WarpCommit<D> W;
  __shared__ __align__(16) int F[6 * MAXF];
  __shared__ int s_start, s_status;
  const int lane = threadIdx.x;
  Counters* ctr = T.ctr;
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  const double c[3] = {x, y, D == 3 ? z : 0.0};
  const vdp::FPt fq = vdp::split_point(c[0], c[1], c[2]);
  if (lane == 0) {
    s_status = 0;
    s_start = -1;
    const double lo = 7.006492321624085e-46;  // 2^-150
    const double hi = 1.4272476927059599e45;  // 2^150
    for (int k = 0; k < 3; ++k) {
      const double a = fabs(c[k]);
      if (!(a <= 1.7976931348623157e308)) s_status = E_NONFINITE;
      else if (s_status == 0 && a != 0.0 && (a < lo || a > hi)) s_status = E_RANGE;
    }
    if (s_status == 0 && bad_vert(T, vid)) s_status = E_INTERNAL;
    if (s_status == 0) {
      reinterpret_cast<double4_32a*>(T.pts)[vid] = make_double4_32a(c[0], c[1], c[2], 0.0);
      T.ptf[vid] = fq;
      const SetGeo& g = T.sets[0];
      vdp::VPt sv[NV];
      for (int j = 0; j < NV; ++j) sv[j] = load_pt(T, g.sup[j]);
      const vdp::VPt p{c[0], c[1], c[2], 0.0};
      if (vdp::exit_face<D, true>(sv, p, (1u << NV) - 1, tl, perr) >= 0) s_status = E_OUTSIDE;
    }
    if (s_status == 0) {
      // walk from the finest hint of the point's cell (as k_activate)
      const SetGeo& g = T.sets[0];
      int ic[3];
      hint_cell<D>(g, fq, ic);
      int cur = -1;
      for (int l = g.hint_levels; l >= 0 && cur < 0; --l) cur = T.hint[hint_at<D>(g, ic, l)];
      if (cur < 0) cur = g.root;
      int4 v, nn;
      load_simplex(T, cur, v, nn);
      for (int k = 0; k < 64 && v.x < 0; ++k) {  // dead slot: into the star that replaced it
        cur = nn.x >> 2;
        if (nn.x < 0 || bad_simp(T, cur)) {
          s_status = E_INTERNAL;
          break;
        }
        load_simplex(T, cur, v, nn);
      }
      int step = 0;
      const int cap = 1 << 16;
      for (; s_status == 0 && step < cap; ++step) {
        vdp::FPt fv[NV];
        for (int j = 0; j < NV; ++j) fv[j] = load_fpt(T, get4(v, j));
        auto load64 = [&](vdp::VPt* v64, vdp::VPt& p64) {
          for (int j = 0; j < NV; ++j) v64[j] = load_pt(T, get4(v, j));
          p64 = vdp::VPt{c[0], c[1], c[2], 0.0};
        };
        const int f = vdp::exit_face_hl<D>(fv, fq, (1u << NV) - 1, tl, perr, load64);
        if (f < 0) break;
        const int code = get4(nn, f);
        if (code < 0 || bad_simp(T, code >> 2)) {
          s_status = code < 0 ? E_OUTSIDE : E_INTERNAL;
          break;
        }
        cur = code >> 2;
        load_simplex(T, cur, v, nn);
      }
      if (step == cap) s_status = E_WALK;
      if (s_status == 0) {
        // a duplicate of a vertex of its simplex is skipped and recorded
        const vdp::VPt q{c[0], c[1], c[2], 0.0};
        int dup = -1;
        for (int j = 0; j < NV; ++j) {
          const int w = get4(v, j);
          if (same_point_bits(load_pt(T, w), q)) dup = w;
        }
        if (dup >= 0) {
          const int k = atomicAdd(&ctr->ndup, 1);
          if (k < T.cap_dups) T.dups[k] = make_int2(vid, dup);
          s_status = E_DUPLICATE;
        }
      }
      s_start = cur;
    }
    if (s_status != 0 && s_status != E_DUPLICATE) set_error(ctr, s_status);
  }
  __syncwarp();
  if (s_status != 0) {
    if (lane == 0) ctr->single = s_status;
    return;
  }
  const int start = s_start;
  int4 v0, n0;
  load_simplex(T, start, v0, n0);
  unsigned ntests = 0;
  const CavStore S{C.cav, C.cv, C.cn, C.hkey, C.fr, MAXC, MAXF, HS};
  cavity_search<D, 0>(T, S, C.ctl, lane, start, v0, n0, vid, fq, tl, perr, ntests);
  if (C.ctl.flags) {  // too large for the warp: the rounds insert it
    if (lane == 0) ctr->single = -1;
    return;
  }
  const int ncav = C.ctl.ncav, nfac = C.ctl.nfac;
  expand_facets(C.fr, C.cv, nfac, vid, F, lane);
  for (int i = lane; i < HR; i += 32) {
    W.rk[i] = ~0ull;
    W.ra[i] = -1;
  }
  for (int i = lane; i < ncav; i += 32) W.first[i] = 0x7fffffff;
  __syncwarp();
  // slots: the first facet of cavity simplex k takes k's slot, the others
  // the cavity slots left over, then fresh ones
  for (int j = lane; j < nfac; j += 32) atomicMin(&W.first[F[6 * j + 5] >> 2], j);
  __syncwarp();
  int nfree = 0;
  for (int i0 = 0; i0 < ncav; i0 += 32) {
    const int i = i0 + lane;
    const bool fr = i < ncav && W.first[i] == 0x7fffffff;
    const unsigned m = __ballot_sync(FULL, fr);
    if (fr) W.freeslot[nfree + __popc(m & ((1u << lane) - 1))] = C.cav[i];
    nfree += __popc(m);
  }
  const int fresh = max(0, nfac - ncav);
  int base = 0;
  if (lane == 0 && fresh > 0) base = atomicAdd(&ctr->nsimp, fresh);
  base = __shfl_sync(FULL, base, 0);
  if (base + fresh > T.cap_simp) {  // the caller keeps spare slots: cannot happen
    if (lane == 0) {
      set_error(ctr, E_INTERNAL);
      ctr->single = E_INTERNAL;
    }
    return;
  }
  int nsec = 0;
  for (int j0 = 0; j0 < nfac; j0 += 32) {
    const int j = j0 + lane;
    int id = 0;
    bool sec = false;
    if (j < nfac) {
      const int k = F[6 * j + 5] >> 2;
      sec = W.first[k] != j;
      if (!sec) id = C.cav[k];
    }
    const unsigned m = __ballot_sync(FULL, sec);
    if (sec) {
      const int t = nsec + __popc(m & ((1u << lane) - 1));
      id = t < nfree ? W.freeslot[t] : base + (t - nfree);
    }
    if (j < nfac) W.id[j] = id;
    nsec += __popc(m);
  }
  __syncwarp();
  const int id0 = W.id[0];
  for (int t = nsec + lane; t < nfree; t += 32)
    store_simplex(T, W.freeslot[t], make_int4(-1, -1, -1, -1), make_int4(id0 << 2, -1, -1, -1));
  // no slot carries round -2 in `killed`, so every outer neighbour is repointed
  write_star<D>(T, W, F, nfac, vid, -2, lane);
  if (perr) set_error(ctr, E_PRECISION);
  flush_tally(ctr, tl, ntests, 0);
  if (lane == 0) {
    write_hints<D>(T, vid, fq, id0);
    ctr->ninserted += 1;
    ctr->winners += 1;
    ctr->created += nfac;
    ctr->killed += ncav;
    ctr->holes += max(0, ncav - nfac);
    ctr->max_cav = max(ctr->max_cav, ncav);
    ctr->max_fac = max(ctr->max_fac, nfac);
    ctr->single = 0;
  }
}

// ---------------------------------------------------------------------------
// The first points of a fresh single-set build, one after another in one
// block, with the whole triangulation in shared memory.
//
// While the triangulation is small, nearly every conflict region holds part of
// the super simplex's star, so a device-wide round inserts one or a few points
// for about ten dependent kernel launches.  Here one 512-thread block inserts
// the first priority levels (Bowyer-Watson in the reference's sense,
// src/delaunay_tree.rs:125-211, one point at a time):
//   1. every live simplex is tested against the point (exact, perturbed
//      conflict test keyed by the global vertex ids, as in the rounds), so no
//      point location is needed;
//   2. the faces of the conflict region whose neighbour is outside it are the
//      boundary facets; no conflict region means the point duplicates a vertex;
//   3. each facet gets a new simplex (a region slot first, then a fresh slot)
//      with its outer link, and the faces through the new point are paired
//      through a ridge table.
// The triangulation is unique, so any insertion order gives the one the
// rounds would build.  The tree in global memory is written only at the end,
// compacted (live simplices in slots 0..m-1) with the location hints of every
// point; when any capacity below would be exceeded the kernel writes nothing
// and the rounds insert these points as usual.
constexpr int kSeedThreads = 512;
template <int D>
struct SeedCap;
template <>
struct SeedCap<3> {
  static constexpr int S = 2560, P = 324, C = 1024, F = 1024, H = 4096, DUP = 64;
};
template <>
struct SeedCap<2> {
  static constexpr int S = 2560, P = 644, C = 1024, F = 1024, H = 4096, DUP = 64;
};
// Shared-memory layout of k_seed (bytes), in this order: simplex vertices and
// neighbour codes (local ids), point records and global ids, cavity marks,
// cavity, facets (new vertices, outer code, position of the new point), ridge
// table (keys, first and second half), flags of inserted points, duplicates.
template <int D>
constexpr size_t seed_smem() {
  using C = SeedCap<D>;
  return (size_t)C::S * 32 + (size_t)C::P * (sizeof(vdp::FPt) + 4) + (size_t)C::S * 4 + (size_t)C::C * 4 +
         (size_t)C::F * 24 + (size_t)C::H * 16 + (size_t)C::P * 4 + (size_t)C::DUP * 8;
}
__device__ __forceinline__ unsigned seed_hash(int r0, int r1, int H) {
  return ((((unsigned)r0 * 0x9E3779B1u) ^ ((unsigned)r1 * 0x85EBCA77u)) >> 12) & (unsigned)(H - 1);
}
// Slot of the key (epoch, r0, r1) in the ridge table, -1 if absent.
__device__ __forceinline__ int seed_find(const unsigned long long* hk, int H, unsigned long long key, int r0, int r1) {
  unsigned h = seed_hash(r0, r1, H);
  for (int probe = 0; probe < H; ++probe, h = (h + 1) & (unsigned)(H - 1)) {
    const unsigned long long k = hk[h];
    if (k == key) return (int)h;
    if ((k >> 32) != (key >> 32)) return -1;  // an entry of an earlier point: the key is not there
  }
  return -1;
}

template <int D>
__global__ void __launch_bounds__(kSeedThreads, 1) k_seed(DevTree T, int npts, int nlev, unsigned long long seed) {
  using C = SeedCap<D>;
  constexpr int NV = D + 1;
  extern __shared__ __align__(16) unsigned char seed_sm[];
  int4* sv = reinterpret_cast<int4*>(seed_sm);
  int4* sn = sv + C::S;
  vdp::FPt* fp = reinterpret_cast<vdp::FPt*>(sn + C::S);
  int* gid = reinterpret_cast<int*>(fp + C::P);
  int* mark = gid + C::P;
  int* cav = mark + C::S;
  int4* fnv = reinterpret_cast<int4*>(cav + C::C);
  int* fcode = reinterpret_cast<int*>(fnv + C::F);
  int* fqf = fcode + C::F;
  unsigned long long* hk = reinterpret_cast<unsigned long long*>(fqf + C::F);
  int* ha = reinterpret_cast<int*>(hk + C::H);
  int* hb = ha + C::H;
  int* ins = hb + C::H;
  int2* dl = reinterpret_cast<int2*>(ins + C::P);
  __shared__ int s_ns, s_ncav, s_nfac, s_abort, s_ndup, s_dupof, s_nins;
  __shared__ unsigned long long s_created, s_killed;
  __shared__ int s_maxc, s_maxf, s_holes;
  const int tid = threadIdx.x;
  const SetGeo& g = T.sets[0];
  if (T.nsets != 1 || npts < 1 || npts + NV > C::P || npts > C::C || npts > C::S) return;
  // start: the super simplex (local vertices 0..D) and the points of the
  // levels in priority order (local vertex NV + k is the k-th lowest), so that
  // of equal points the one with the lowest priority is inserted and the
  // others are its duplicates, as in the rounds
  for (int i = tid; i < npts; i += kSeedThreads) {
    const int v = T.order[i];
    mark[i] = v;
    cav[i] = (int)priority((uint32_t)v, seed);
  }
  for (int i = tid; i < C::H; i += kSeedThreads) hk[i] = 0ull;
  __syncthreads();
  for (int i = tid; i < npts; i += kSeedThreads) {
    const unsigned pr = (unsigned)cav[i];
    int rank = 0;
    for (int j = 0; j < npts; ++j) rank += (unsigned)cav[j] < pr ? 1 : 0;
    const int v = mark[i];
    const bool bad = bad_vert(T, v);
    if (bad) set_error(T.ctr, E_INTERNAL);
    gid[NV + rank] = bad ? 0 : v;
    fp[NV + rank] = load_fpt(T, bad ? 0 : v);
    ins[NV + rank] = 0;
  }
  for (int l = tid; l < NV; l += kSeedThreads) {
    const int v = g.sup[l];
    const bool bad = bad_vert(T, v);
    if (bad) set_error(T.ctr, E_INTERNAL);
    gid[l] = bad ? 0 : v;
    fp[l] = load_fpt(T, bad ? 0 : v);
    ins[l] = 1;
  }
  __syncthreads();
  for (int i = tid; i < C::S; i += kSeedThreads) mark[i] = 0;
  if (tid == 0) {
    sv[0] = D == 3 ? make_int4(0, 1, 2, 3) : make_int4(0, 1, 2, -1);
    sn[0] = make_int4(-1, -1, -1, -1);
    s_ns = 1;
    s_ncav = s_nfac = s_abort = s_ndup = s_nins = 0;
    s_created = s_killed = 0ull;
    s_maxc = s_maxf = s_holes = 0;
  }
  __syncthreads();
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  unsigned ntests = 0;
  for (int p = 0; p < npts; ++p) {
    const int ql = NV + p, qv = gid[ql];
    const vdp::FPt fq = fp[ql];
    const int ns = s_ns;
    // 0. a point equal to an inserted vertex is skipped and recorded, as the
    // rounds do before any search (its conflict region need not be empty:
    // the perturbation of an equal vertex with a larger id puts it inside)
    if (tid == 0) s_dupof = -1;
    __syncthreads();
    for (int l = tid; l < ql; l += kSeedThreads) {
      if (!ins[l]) continue;
      const vdp::FPt& a = fp[l];
      if (a.hx == fq.hx && a.hy == fq.hy && a.hz == fq.hz && a.lx == fq.lx && a.ly == fq.ly && a.lz == fq.lz &&
          same_point_bits(load_pt(T, gid[l]), load_pt(T, qv)))
        s_dupof = gid[l];
    }
    __syncthreads();
    if (s_dupof >= 0) {
      if (tid == 0) {
        if (s_ndup >= C::DUP) s_abort = 1;
        else dl[s_ndup++] = make_int2(qv, s_dupof);
      }
      __syncthreads();
      if (s_abort) break;
      continue;
    }
    // 1. conflict region: every live simplex, exact perturbed test
    for (int s = tid; s < ns; s += kSeedThreads) {
      const int4 v = sv[s];
      if (v.x < 0) continue;
      vdp::FPt fv[NV];
      int kv[NV];
      for (int j = 0; j < NV; ++j) {
        const int l = get4(v, j);
        kv[j] = gid[l];
        fv[j] = fp[l];
      }
      ++ntests;
      auto load64 = [&](vdp::VPt* v64, vdp::VPt& q64) {
        for (int j = 0; j < NV; ++j) v64[j] = load_pt(T, kv[j]);
        q64 = load_pt(T, qv);
      };
      if (vdp::in_conflict_hl<D, 1>(fv, kv, fq, qv, tl, perr, load64)) {
        const int k = atomicAdd(&s_ncav, 1);
        if (k < C::C) cav[k] = s;
        mark[s] = p + 1;
      }
    }
    __syncthreads();
    const int ncav = s_ncav;
    if (ncav > C::C) break;  // s_abort is set below, by thread 0
    if (ncav == 0) {
      // a point that is no vertex lies in the closed simplex that contains
      // it, and so inside its circumsphere: an empty region is a fault
      if (tid == 0) {
        set_error(T.ctr, E_INTERNAL);
        s_abort = 1;
      }
      __syncthreads();
      break;
    }
    // 2. boundary facets: faces of the region whose neighbour is outside it
    // (the ridge table's halves are emptied meanwhile)
    for (int i = tid; i < C::H; i += kSeedThreads) {
      ha[i] = -1;
      hb[i] = -1;
    }
    for (int it = tid; it < ncav * NV; it += kSeedThreads) {
      const int k = it / NV, f = it - k * NV;
      const int s = cav[k];
      const int code = get4(sn[s], f);
      if (code >= 0 && mark[code >> 2] == p + 1) continue;
      const int j = atomicAdd(&s_nfac, 1);
      if (j < C::F) {
        fnv[j] = set4(sv[s], f, ql);
        fcode[j] = code;
        fqf[j] = f;
      }
    }
    __syncthreads();
    const int nfac = s_nfac;
    if (nfac > C::F || ns + max(0, nfac - ncav) > C::S) break;
    // 3a. ridge table: each face through the new point, keyed by its other
    // old vertices (3D: two, 2D: one), takes the first or the second half
    const unsigned long long ep = (unsigned long long)(p + 1) << 32;
    for (int it = tid; it < nfac * NV; it += kSeedThreads) {
      const int j = it / NV, gf = it - j * NV, qf = fqf[j];
      if (gf == qf) continue;
      int r[4] = {fnv[j].x, fnv[j].y, fnv[j].z, fnv[j].w};
      int r0, r1;
      ridge_of<D>(r, gf, qf, r0, r1);
      const unsigned long long key = ep | ((unsigned long long)(unsigned)(r0 & 0xffff) << 16) | (unsigned)(r1 & 0xffff);
      unsigned h = seed_hash(r0, r1, C::H);
      for (int probe = 0; probe < C::H; ++probe, h = (h + 1) & (unsigned)(C::H - 1)) {
        unsigned long long cur = hk[h];
        if ((cur >> 32) != (unsigned long long)(p + 1)) {
          const unsigned long long old = atomicCAS(&hk[h], cur, key);
          if (old == cur) {
            ha[h] = (j << 2) | gf;
            break;
          }
          cur = old;
        }
        if (cur == key) {
          hb[h] = (j << 2) | gf;
          break;
        }
      }
    }
    __syncthreads();
    // 3b. new simplices: facet j takes region slot cav[j], or a fresh slot
    for (int j = tid; j < nfac; j += kSeedThreads) {
      const int slot = j < ncav ? cav[j] : ns + (j - ncav);
      const int qf = fqf[j];
      const int4 nv = fnv[j];
      int r[4] = {nv.x, nv.y, nv.z, nv.w};
      int4 nn = make_int4(-1, -1, -1, -1);
      for (int gf = 0; gf < NV; ++gf) {
        if (gf == qf) {
          nn = set4(nn, gf, fcode[j]);
          continue;
        }
        int r0, r1;
        ridge_of<D>(r, gf, qf, r0, r1);
        const unsigned long long key = ep | ((unsigned long long)(unsigned)(r0 & 0xffff) << 16) | (unsigned)(r1 & 0xffff);
        const int h = seed_find(hk, C::H, key, r0, r1);
        const int mine = (j << 2) | gf;
        const int other = h < 0 ? -1 : (ha[h] == mine ? hb[h] : ha[h]);
        if (other < 0 || (other >> 2) >= nfac) {
          set_error(T.ctr, E_INTERNAL);  // a ridge with one half: not a closed star
          s_abort = 1;
          continue;
        }
        const int oj = other >> 2;
        const int oslot = oj < ncav ? cav[oj] : ns + (oj - ncav);
        nn = set4(nn, gf, (oslot << 2) | (other & 3));
      }
      sv[slot] = nv;
      sn[slot] = nn;
    }
    __syncthreads();
    // 3c. outer neighbours point at the new simplices; region slots without a
    // facet die (their records are not read again)
    for (int j = tid; j < nfac; j += kSeedThreads) {
      const int code = fcode[j];
      if (code < 0) continue;
      const int slot = j < ncav ? cav[j] : ns + (j - ncav);
      reinterpret_cast<int*>(sn + (code >> 2))[code & 3] = (slot << 2) | fqf[j];
    }
    for (int k = nfac + tid; k < ncav; k += kSeedThreads) sv[cav[k]].x = -1;
    __syncthreads();
    if (tid == 0) {
      s_ns = ns + max(0, nfac - ncav);
      s_ncav = 0;
      s_nfac = 0;
      s_nins += 1;
      s_created += nfac;
      s_killed += ncav;
      s_maxc = max(s_maxc, ncav);
      s_maxf = max(s_maxf, nfac);
      s_holes += max(0, ncav - nfac);
      ins[ql] = 1;
    }
    __syncthreads();
    if (s_abort) break;
  }
  // a loop left early (capacity) has not finished its point
  if (tid == 0 && (s_ncav > C::C || s_nfac > C::F || s_ncav != 0 || s_nfac != 0)) s_abort = 1;
  __syncthreads();
  if (perr) set_error(T.ctr, E_PRECISION);
  if (s_abort) return;  // nothing written: the rounds insert these points
  // write-out: live slots are ranked (mark[] holds the ranks) and stored
  // compacted with global vertex ids and neighbour codes
  const int ns = s_ns;
  __shared__ int wsum[kSeedThreads / 32];
  constexpr int PER = (C::S + kSeedThreads - 1) / kSeedThreads;
  int cnt = 0;
  for (int k = 0; k < PER; ++k) {
    const int s = tid * PER + k;
    cnt += (s < ns && sv[s].x >= 0) ? 1 : 0;
  }
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(FULL, incl, o);
    if ((tid & 31) >= o) incl += y;
  }
  if ((tid & 31) == 31) wsum[tid >> 5] = incl;
  __syncthreads();
  int base = 0;
  for (int w = 0; w < (tid >> 5); ++w) base += wsum[w];
  base += incl - cnt;
  for (int k = 0; k < PER; ++k) {
    const int s = tid * PER + k;
    if (s < ns && sv[s].x >= 0) mark[s] = base++;
  }
  __syncthreads();
  int nlive = 0;
  for (int w = 0; w < kSeedThreads / 32; ++w) nlive += wsum[w];
  if (nlive > T.cap_simp) {
    if (tid == 0) set_error(T.ctr, E_INTERNAL);
    return;
  }
  for (int s = tid; s < ns; s += kSeedThreads) {
    const int4 v = sv[s];
    if (v.x < 0) continue;
    const int4 n = sn[s];
    int4 gv = make_int4(-1, -1, -1, -1), gn = make_int4(-1, -1, -1, -1);
    for (int j = 0; j < NV; ++j) {
      gv = set4(gv, j, gid[get4(v, j)]);
      const int c = get4(n, j);
      gn = set4(gn, j, c < 0 ? -1 : (mark[c >> 2] << 2) | (c & 3));
    }
    store_simplex(T, mark[s], gv, gn);
    for (int j = 0; j < NV; ++j) {
      const int l = get4(v, j);
      if (l >= NV) write_hints<D>(T, gid[l], fp[l], mark[s]);
    }
  }
  flush_tally(T.ctr, tl, ntests, 0);
  if (tid == 0) {
    Counters* c = T.ctr;
    c->nsimp = nlive;
    c->ninserted += s_nins;
    c->winners += s_nins;
    c->created += s_created;
    c->killed += s_killed;
    c->holes += s_holes;
    c->max_cav = max(c->max_cav, s_maxc);
    c->max_fac = max(c->max_fac, s_maxf);
    const int d0 = c->ndup;
    for (int k = 0; k < s_ndup; ++k)
      if (d0 + k < T.cap_dups) T.dups[d0 + k] = dl[k];
    c->ndup = d0 + s_ndup;
    c->lev_next = nlev;
  }
}

template <int D>
constexpr size_t small_rounds_smem() {
  return 4 * sizeof(WarpCav<D>) > 4 * sizeof(WarpCommit<D>) ? 4 * sizeof(WarpCav<D>) : 4 * sizeof(WarpCommit<D>);
}

// Blocks of the small-round kernel (0: one per SM).
#ifndef VD_SMALL_GRID
#define VD_SMALL_GRID 0
#endif
// Resident blocks on the whole GPU of the strict-mode k_check (MODE 0) and
// of the commit half (MODE 2), 2D and 3D.
int g_check_wave[2] = {1 << 20, 1 << 20};
int g_commit_wave[2] = {1 << 20, 1 << 20};
// Resident blocks of the decide half (XT = 1 form, the larger), 2D and 3D.
int g_decide_wave[2] = {1 << 20, 1 << 20};
#ifndef VD_DECIDE_WIDE
#define VD_DECIDE_WIDE 1
#endif
// Grid of k_cavity_big: one 512-thread block per SM.
int g_big_grid = 1;
// Grid of the small-round kernel (0: not available).
int g_small_grid[2] = {0, 0};

template <int D>
void round_impl(const DevTree& T, const Launch& L, const Tuning& tu, const Feed& fd, Prof* pf) {
  auto mark = [&](int type) {
    if (pf && pf->n < Prof::kMax) {
      cudaEventRecord(pf->ev[pf->n + 1], L.stream);
      pf->type[pf->n++] = type;
    }
  };
  if (pf && pf->n == 0) cudaEventRecord(pf->ev[0], L.stream);
  note_launches((tu.adjacent ? 6 + 3 * tu.passes - 1 : 6 + 2 * tu.passes - 1) - (tu.thin > 0 ? 0 : 1) +
                (tu.big_block ? 1 + (tu.adjacent ? tu.passes : 0) : 0));
  k_plan<<<1, 32, 0, L.stream>>>(T, fd.ratio);
  k_activate<D><<<L.blocks, 256, 0, L.stream>>>(T, fd.seed);
  mark(KT_ACTIVATE);
  k_pick<D><<<L.blocks, 256, 0, L.stream>>>(T, tu.thin);
  mark(KT_PICK);
  if (tu.thin > 0) {
    k_thin<D><<<L.blocks, 256, 0, L.stream>>>(T, tu.thin);
    mark(KT_THIN);
  }
  // kernels with conflict tests come in two forms: exact tier on expansions
  // alone (small register allocation) or integer tier first (tu.exact_int)
  if (tu.exact_int)
    k_cavity<D, 1><<<L.warps / 4, 128, 0, L.stream>>>(T, tu.adjacent, tu.big_block);
  else
    k_cavity<D, 0><<<L.warps / 4, 128, 0, L.stream>>>(T, tu.adjacent, tu.big_block);
  mark(KT_CAVITY);
  // with big_block, searches that outgrew a warp's shared memory are redone
  // by whole blocks (the host turns it on once a call has spilled searches)
  if (tu.big_block) {
    if (tu.exact_int)
      k_cavity_big<D, 1><<<g_big_grid, 512, kBigSmem, L.stream>>>(T, tu.adjacent);
    else
      k_cavity_big<D, 0><<<g_big_grid, 512, kBigSmem, L.stream>>>(T, tu.adjacent);
    mark(KT_BIG);
  }
  // the commit half needs little shared memory per warp and few registers,
  // so it runs up to twice the warps of the search (one resident wave)
  const int commit_grid = std::min(L.warps / 2, g_commit_wave[D - 2]);
  // the decide half (56 registers, 1 KB of shared memory per warp) likewise
  const int decide_grid = VD_DECIDE_WIDE ? std::min(L.warps / 2, g_decide_wave[D - 2]) : L.warps / 4;
  const int strict_grid = std::min(L.warps / 4, g_check_wave[D - 2]);
  for (int p = 0; p < tu.passes; ++p) {
    const int last = p == tu.passes - 1;
    if (p > 0) {
      // reclaim (40 registers, no shared memory) runs twice the search's warps
      k_reclaim<D><<<L.warps / 2, 128, 0, L.stream>>>(T, p, tu.adjacent);
      mark(KT_RECLAIM);
    }
    if (tu.adjacent) {
      if (tu.exact_int)
        k_check<D, 1, 1><<<decide_grid, 128, 4 * sizeof(HeadBuf), L.stream>>>(T, p, last, fd.seed, 0);
      else
        k_check<D, 1, 0><<<decide_grid, 128, 4 * sizeof(HeadBuf), L.stream>>>(T, p, last, fd.seed, 0);
      mark(KT_DECIDE);
      k_check<D, 2, 0><<<commit_grid, 128, 4 * sizeof(WarpCommit<D>), L.stream>>>(T, p, last, fd.seed,
                                                                                  tu.big_block);
      mark(KT_CHECK);
      if (tu.big_block) {
        k_commit_big<D><<<g_big_grid, 512, 0, L.stream>>>(T);
        mark(KT_BIGW);
      }
    } else {
      if (tu.exact_int)
        k_check<D, 0, 1><<<strict_grid, 128, 4 * sizeof(WarpCommit<D>), L.stream>>>(T, p, last, fd.seed, 0);
      else
        k_check<D, 0, 0><<<strict_grid, 128, 4 * sizeof(WarpCommit<D>), L.stream>>>(T, p, last, fd.seed, 0);
      mark(KT_CHECK);
    }
  }
  k_relocate<D><<<L.blocks, 256, 0, L.stream>>>(T);
  mark(KT_RELOCATE);
}

}  // namespace

void launch_upload(const DevTree& T, const Launch& L, int dim, const double* d_xyz, int64_t n, int base_vid) {
  note_launches(1);
  if (dim == 3)
    k_upload<3><<<L.blocks, 256, 0, L.stream>>>(T, d_xyz, n, base_vid);
  else
    k_upload<2><<<L.blocks, 256, 0, L.stream>>>(T, d_xyz, n, base_vid);
}

void launch_levels(const DevTree& T, const Launch& L, int64_t n, int base_vid, uint64_t seed,
                   const unsigned long long* thr, int nlev, double first, double growth, int* d_work) {
  note_launches(3);
  Thresholds th;
  th.n = nlev;
  th.first = first;
  th.lgrow = log(growth);
  for (int k = 0; k < kMaxLevels; ++k) th.t[k] = k < nlev ? thr[k] : ~0ull;
  k_level_hist<<<L.blocks, 256, 0, L.stream>>>(T, n, base_vid, seed, th, d_work);
  k_level_init<<<1, 32, 0, L.stream>>>(T, d_work, nlev);
  k_level_order<<<L.blocks, 256, 0, L.stream>>>(T, n, base_vid, seed, th, d_work + kMaxLevels);
}

namespace {
int prepare_once() {
  cudaError_t e = cudaSuccess;
  auto attr = [&](const void* f, int bytes) {
    const cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (r != cudaSuccess) e = r;
  };
  attr((const void*)k_check<3, 0, 0>, 4 * (int)sizeof(WarpCommit<3>));
  attr((const void*)k_check<3, 0, 1>, 4 * (int)sizeof(WarpCommit<3>));
  attr((const void*)k_check<3, 2, 0>, 4 * (int)sizeof(WarpCommit<3>));
  attr((const void*)k_check<2, 0, 0>, 4 * (int)sizeof(WarpCommit<2>));
  attr((const void*)k_check<2, 0, 1>, 4 * (int)sizeof(WarpCommit<2>));
  attr((const void*)k_check<2, 2, 0>, 4 * (int)sizeof(WarpCommit<2>));
  attr((const void*)k_cavity_big<3, 0>, kBigSmem);
  attr((const void*)k_cavity_big<3, 1>, kBigSmem);
  attr((const void*)k_cavity_big<2, 0>, kBigSmem);
  attr((const void*)k_cavity_big<2, 1>, kBigSmem);
  attr((const void*)k_seed<3>, (int)seed_smem<3>());
  attr((const void*)k_seed<2>, (int)seed_smem<2>());
  if (e != cudaSuccess) return E_CUDA;
  // k_check is a grid-stride loop: one resident wave avoids a ragged second
  int dev = 0, sms = 0, b3 = 0, b2 = 0, c3 = 0, c2 = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, k_check<3, 0, 1>, 128, 4 * sizeof(WarpCommit<3>)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_check<2, 0, 1>, 128, 4 * sizeof(WarpCommit<2>)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c3, k_check<3, 2, 0>, 128, 4 * sizeof(WarpCommit<3>)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c2, k_check<2, 2, 0>, 128, 4 * sizeof(WarpCommit<2>)) != cudaSuccess)
    return E_CUDA;
  g_check_wave[1] = std::max(1, sms * b3);
  g_check_wave[0] = std::max(1, sms * b2);
  g_big_grid = std::max(1, sms);
  g_commit_wave[1] = std::max(1, sms * c3);
  g_commit_wave[0] = std::max(1, sms * c2);
  int d3 = 0, d2 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d3, k_check<3, 1, 1>, 128, 4 * sizeof(HeadBuf)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d2, k_check<2, 1, 1>, 128, 4 * sizeof(HeadBuf)) != cudaSuccess)
    return E_CUDA;
  g_decide_wave[1] = std::max(1, sms * d3);
  g_decide_wave[0] = std::max(1, sms * d2);
  // small-round kernel: one block per SM when a block fits
  int s3 = 0, s2 = 0;
  cudaFuncSetAttribute((const void*)k_rounds_small<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)small_rounds_smem<3>());
  cudaFuncSetAttribute((const void*)k_rounds_small<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)small_rounds_smem<2>());
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s3, k_rounds_small<3>, 128, small_rounds_smem<3>()) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s2, k_rounds_small<2>, 128, small_rounds_smem<2>()) !=
          cudaSuccess) {
    cudaGetLastError();
    s3 = s2 = 0;
  }
  // a small grid keeps the grid barrier short (the rounds it runs are small)
  const int cap3 = sms * s3, cap2 = sms * s2;
  g_small_grid[1] = s3 > 0 ? (VD_SMALL_GRID > 0 ? std::min(VD_SMALL_GRID, cap3) : sms) : 0;
  g_small_grid[0] = s2 > 0 ? (VD_SMALL_GRID > 0 ? std::min(VD_SMALL_GRID, cap2) : sms) : 0;
  return E_OK;
}
}  // namespace

// Once per process (trees may be created from several host threads).
// Function attributes (dynamic shared memory above 48 KB) belong to a device's
// context, so they are set once per device the process uses.
int prepare_round_kernels() {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static int state[kMaxDevices] = {};  // 0 not yet, 1 ready, -1 failed
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return E_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if (state[dev] == 0) state[dev] = prepare_once() == E_OK ? 1 : -1;
  return state[dev] == 1 ? E_OK : E_CUDA;
}

int launch_small_rounds(const DevTree& T, cudaStream_t stream, int dim, const Tuning& tu, const Feed& fd,
                        int max_active, int max_rounds) {
  const int grid = g_small_grid[dim - 2];
  if (grid <= 0) return E_CUDA;
  DevTree t = T;
  Tuning tuc = tu;
  unsigned long long seed = fd.seed;
  float ratio = fd.ratio;
  void* args[] = {&t, &tuc, &seed, &ratio, &max_active, &max_rounds};
  const void* fn = dim == 3 ? (const void*)k_rounds_small<3> : (const void*)k_rounds_small<2>;
  const size_t smem = dim == 3 ? small_rounds_smem<3>() : small_rounds_smem<2>();
  const cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(128), args, smem, stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return E_CUDA;
  }
  note_launches(1);
  return E_OK;
}

int seed_max_points(int dim) { return dim == 3 ? SeedCap<3>::P - 4 : SeedCap<2>::P - 3; }

void launch_seed(const DevTree& T, cudaStream_t stream, int dim, int npts, int nlev, uint64_t seed) {
  note_launches(1);
  if (dim == 3)
    k_seed<3><<<1, kSeedThreads, seed_smem<3>(), stream>>>(T, npts, nlev, seed);
  else
    k_seed<2><<<1, kSeedThreads, seed_smem<2>(), stream>>>(T, npts, nlev, seed);
}

void launch_insert_one(const DevTree& T, cudaStream_t stream, int dim, const double* c, int vid) {
  note_launches(1);
  if (dim == 3)
    k_insert_one<3><<<1, 32, 0, stream>>>(T, c[0], c[1], c[2], vid);
  else
    k_insert_one<2><<<1, 32, 0, stream>>>(T, c[0], c[1], 0.0, vid);
}

void launch_round(const DevTree& T, const Launch& L, int dim, const Tuning& tu, const Feed& fd, Prof* pf) {
  if (dim == 3)
    round_impl<3>(T, L, tu, fd, pf);
  else
    round_impl<2>(T, L, tu, fd, pf);
}

const char* const kKernelTypeNames[KT_COUNT] = {"k_pick",     "k_thin",         "k_cavity",     "k_check",
                                                "k_reclaim",  "k_relocate",     "k_activate",   "edges",
                                                "k_decide",   "k_rounds_small", "k_cavity_big", "k_commit_big",
                                                "k_seed"};

}  // namespace vd
