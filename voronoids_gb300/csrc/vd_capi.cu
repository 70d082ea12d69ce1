// Host runtime behind the C ABI (include/voronoids_gpu.h).
//
// Owns the device pools of one tree, sizes them, drives the insertion rounds
// on the tree's stream and converts results to the reference's shapes.  The
// only host<->device synchronisations during a build are one counter read
// every few rounds (to stop, to grow a pool, or to report an error).
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "../../include/voronoids_gpu.h"
#include "vd_common.cuh"

namespace vd {
static std::atomic<long long> g_launches{0};
void note_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launches_total() { return g_launches.load(std::memory_order_relaxed); }
int64_t run_edges(const DevTree& T, const Launch& L, int dim, int nsimp, int n_in,
                  const EdgeScratch& S, uint2* d_out, int64_t cap_out, int* d_total_pair, int* h_total_pair);
}

namespace {

using vd::Counters;
using vd::DevTree;

// ---------------------------------------------------------------------------
// Reference super simplex, restated bit for bit (host code is compiled with
// -ffp-contract=off so each operation rounds as in Rust).
//   bounding_sphere: src/geometry.rs:99-142
//   3D vertices:     src/delaunay_tree.rs:392-406
//   2D vertices:     src/delaunay_tree.rs:547-558
// ---------------------------------------------------------------------------
bool ref_in_sphere(const double* v, const double* c, double r, int dim) {
  double d = 0.0;
  for (int i = 0; i < dim; ++i) d += (c[i] - v[i]) * (c[i] - v[i]);
  return d < r * r;
}

void ref_bounding_sphere(int dim, const double* pts, int64_t n, double* center, double* radius) {
  double lo[3], hi[3];
  for (int i = 0; i < dim; ++i) {
    double l = INFINITY, h = -INFINITY;
    for (int64_t k = 0; k < n; ++k) {
      const double v = pts[k * dim + i];
      l = fmin(l, v);
      h = fmax(h, v);
    }
    lo[i] = l;
    hi[i] = h;
    center[i] = (h + l) / 2.0;
  }
  double su = 0.0, sl = 0.0;
  for (int i = 0; i < dim; ++i) su += (hi[i] - center[i]) * (hi[i] - center[i]);
  for (int i = 0; i < dim; ++i) sl += (lo[i] - center[i]) * (lo[i] - center[i]);
  const double ud = sqrt(su), ld = sqrt(sl);
  double r = ud > ld ? ud : ld;
  for (int64_t k = 0; k < n; ++k)
    if (!ref_in_sphere(pts + k * dim, center, r, dim)) r = r * 1.5;
  *radius = r;
}

// Super vertices for bounding centre c and radius r (src/delaunay_tree.rs:392-406, :547-558).
void ref_super_from_sphere(int dim, const double* c, double r, double out[4][3], double* R) {
  r *= 10.0;
  *R = r;
  const double pi = 3.141592653589793;
  const double c1 = cos(2. * pi / 3.), s1 = sin(2. * pi / 3.);
  const double c2 = cos(4. * pi / 3.), s2 = sin(4. * pi / 3.);
  if (dim == 3) {
    const double v[4][3] = {{c[0], c[1], c[2] + r},
                            {c[0] + r, c[1], c[2] - r},
                            {c[0] + r * c1, c[1] + r * s1, c[2] - r},
                            {c[0] + r * c2, c[1] + r * s2, c[2] - r}};
    memcpy(out, v, sizeof(v));
  } else {
    const double v[3][3] = {
        {c[0] + r, c[1], 0.0}, {c[0] + r * c1, c[1] + r * s1, 0.0}, {c[0] + r * c2, c[1] + r * s2, 0.0}};
    memcpy(out, v, sizeof(v));
    out[3][0] = out[3][1] = out[3][2] = 0.0;
  }
}

void ref_super_vertices(int dim, const double* pts, int64_t n, double out[4][3], double* R) {
  double c[3] = {0, 0, 0}, r;
  ref_bounding_sphere(dim, pts, n, c, &r);
  ref_super_from_sphere(dim, c, r, out, R);
}

bool coord_ok(double a) {
  a = fabs(a);
  return a == 0.0 || (a >= 7.006492321624085e-46 && a <= 1.4272476927059599e45);
}

template <class T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void**)p, sizeof(T) * count) == cudaSuccess ? vd::E_OK : vd::E_NOMEM;
}

template <class T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

}  // namespace

struct vd_tree {
  int dim = 3;
  int ns = 4;
  int device = 0;
  int sms = 1;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double sup[4][3] = {};
  double R = 0;
  int sup_order[4] = {0, 1, 2, 3};
  int64_t nverts = 0;     // super + inserted/pending vertices
  int64_t cap_verts = 0;
  int64_t cap_act = 0;
  int round = 0;
  int round_base = 0;  // first round of the current triangulation
  int64_t inserted = 0;   // vertices inserted (from counters)
  int64_t calls = 0;
  DevTree T = {};
  Counters* hctr = nullptr;   // pinned host mirror
  // edges
  bool edges_valid = false;
  int64_t nedges = 0;
  uint2* d_edges = nullptr;
  int64_t cap_edges = 0;
  vd::EdgeScratch es = {};
  int64_t es_n = -1;
  int* d_pair = nullptr;
  int* h_pair = nullptr;
  unsigned long long* d_check = nullptr;
  int* d_misc = nullptr;      // small device scratch (live-slot search, locate)
  int64_t* d_loc = nullptr;
  int64_t cap_loc = 0;
  int64_t ncells = 0;
  // pinned staging for small host<->device copies
  unsigned long long* h_mm = nullptr;
  // device staging of host input points (one-shot host path)
  double* d_in = nullptr;
  int64_t cap_in = 0;
  // insertion schedule: priority levels from `first_prefix` points growing
  // by `growth`, fed while fewer than `ratio` x inserted points are active
  int64_t first_prefix = 64;
  double growth = 1.25;
  double ratio = 0.12;
  int* d_counts = nullptr;     // 2 * kMaxLevels ints: level counts, cursors
  // profiling: per-kernel time from CUDA events on the tree's stream
  bool prof = false;
  std::vector<vd::Prof> profs;   // one event log per round of a chunk
  double kms[vd::KT_COUNT] = {};
  int64_t kcnt[vd::KT_COUNT] = {};
  vd::Tuning tuning = {2, 2, 1};
  // per-round trace (diagnostics; syncs after every round)
  bool trace = false;
  std::vector<int64_t> trace_rows;
  // chunks of rounds captured as CUDA graphs, keyed by everything a launch
  // bakes in (the device tree by value, grid, tuning and feed)
  struct ChunkGraph {
    vd::DevTree T;
    int chunk, blocks, warps, passes, thin, adjacent, exact_int, big_block;
    uint64_t seed;
    float ratio;
    long long launches;
    cudaGraphExec_t exec;
  };
  std::vector<ChunkGraph> graphs;
  bool use_graphs = true;
  bool has_geometry = false;  // a super simplex exists (vd_tree_create leaves none)
  // sets (one unless built by vd_batch_*): first input point of each set
  int nsets = 1;
  std::vector<long long> set_off;   // nsets + 1 (batched build)
  int64_t cap_sets = 0;              // capacity of T.sets and the per-set scratch
  long long* d_setoff = nullptr;     // nsets + 1
  long long* d_eoff = nullptr;       // nsets + 1 edge offsets
  double* d_cr = nullptr;            // 4 per set: sizing centre and radius
  int* d_flags = nullptr;            // per set: some point not strictly inside
  unsigned long long* d_mm = nullptr;  // 6 per set: bounding-box keys
  int64_t cap_setof = 0;
  // highest simplex slot handed out since the last reset: slots below it
  // may hold simplices of an earlier build and are cleared on reset
  int64_t simp_hwm = 0;
  // launch shape: blocks of 256 threads per SM for point-per-thread kernels,
  // warps per SM for candidate-per-warp kernels (see vd_autotune_batch)
  int blocks_per_sm = 8;
  int warps_per_sm = 20;
  // rounds run in one cooperative launch while fewer points are active
  int small_rounds_max = 0;
  // early phase: until `early_until` points are inserted, rounds use thinning
  // radius `early_thin` and feed ratio `early_ratio` (the device is mostly
  // idle then, so extra searches are nearly free and fewer rounds pay off)
  int64_t early_until = 10000;
  int early_thin = 0;
  double early_ratio = 0.5;
  // exact tier of the conflict tests: 0 automatic (expansions until a build
  // has made `exact_switch` exact tests, then the integer tier first),
  // 1 expansions only, 2 integer tier first from the start
  int exact_mode = 0;
  int64_t exact_switch = 32;
  // most points a fresh single-set call inserts in one block before its
  // rounds (whole priority levels, up to the block's capacity; 0: none; -1:
  // the dimension's default, 150 points in 2D and 3D)
  int64_t first_block = -1;
};

namespace {

constexpr int kMaxWarpsPerSm = 32;
// per-warp fresh-slot chunks: room for the widest k_check grid per SM
constexpr int kChunkWarpsPerSm = 64;

vd::Launch launch_of(const vd_tree* t) {
  vd::Launch L;
  L.blocks = t->sms * t->blocks_per_sm;
  L.warps = t->sms * t->warps_per_sm;
  L.stream = t->stream;
  return L;
}

int cuda_status(cudaError_t e) { return e == cudaSuccess ? vd::E_OK : vd::E_CUDA; }

constexpr int kChunkMax = 8;

vd::Prof* round_prof(vd_tree* t, int k) {
  if (!t->prof) return nullptr;
  if (t->profs.empty()) {
    t->profs.resize(kChunkMax + 1);
    for (auto& p : t->profs)
      for (auto& e : p.ev) cudaEventCreate(&e);
  }
  t->profs[k].n = 0;
  return &t->profs[k];
}

void accumulate_events(vd_tree* t, int rounds) {
  if (!t->prof) return;
  for (int r = 0; r < rounds; ++r) {
    const vd::Prof& p = t->profs[r];
    for (int i = 0; i < p.n; ++i) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, p.ev[i], p.ev[i + 1]) == cudaSuccess) {
        t->kms[p.type[i]] += ms;
        t->kcnt[p.type[i]] += 1;
      }
    }
  }
}

// Times one non-round kernel sequence (activation, edges) into type `kt`.
struct ScopedProf {
  vd_tree* t;
  int kt;
  vd::Prof* p;
  ScopedProf(vd_tree* t_, int kt_) : t(t_), kt(kt_), p(round_prof(t_, kChunkMax)) {
    if (p) cudaEventRecord(p->ev[0], t->stream);
  }
  ~ScopedProf() {
    if (!p) return;
    cudaEventRecord(p->ev[1], t->stream);
    cudaEventSynchronize(p->ev[1]);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p->ev[0], p->ev[1]) == cudaSuccess) {
      t->kms[kt] += ms;
      t->kcnt[kt] += 1;
    }
  }
};

int sync_counters(vd_tree* t) {
  cudaMemcpyAsync(t->hctr, t->T.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, t->stream);
  const int rc = cuda_status(cudaStreamSynchronize(t->stream));
  t->simp_hwm = std::max<int64_t>(t->simp_hwm, t->hctr->nsimp);
  return rc;
}

// Grow a device array to `want` elements, keeping the first `keep` elements,
// filling the new tail with `fill` bytes (-1 = leave uninitialised).
template <class T>
int grow(T** p, int64_t* cap, int64_t want, int64_t keep, int fill, cudaStream_t st) {
  if (want <= *cap) return vd::E_OK;
  T* np = nullptr;
  if (dalloc(&np, (size_t)want) != vd::E_OK) return vd::E_NOMEM;
  if ((*p && keep > 0 &&
       cudaMemcpyAsync(np, *p, sizeof(T) * keep, cudaMemcpyDeviceToDevice, st) != cudaSuccess) ||
      (fill >= 0 && cudaMemsetAsync(np + keep, fill, sizeof(T) * (want - keep), st) != cudaSuccess) ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaFree(np);  // the old array and its capacity stay as they were
    return vd::E_CUDA;
  }
  if (*p) cudaFree(*p);
  *p = np;
  *cap = want;
  return vd::E_OK;
}

int ensure_simplices(vd_tree* t, int64_t want) {
  int64_t cap = t->T.cap_simp;
  if (want <= cap) return vd::E_OK;
  want = std::max(want, cap + cap / 2);
  if (want > (int64_t(1) << 29)) return vd::E_NOMEM;  // neighbour codes use 30 bits
  int64_t used = t->hctr->nsimp;
  int64_t c[7] = {cap, cap, cap, cap, cap, cap, cap};
  int rc = vd::E_OK;
  rc |= grow(&t->T.simp, &c[0], want, used, 0xff, t->stream);
  rc |= grow(&t->T.vote, &c[1], want, used, 0xff, t->stream);
  rc |= grow(&t->T.thin, &c[2], want, used, 0xff, t->stream);
  rc |= grow(&t->T.claim_c, &c[3], want, used, 0xff, t->stream);
  rc |= grow(&t->T.claim_n, &c[4], want, used, 0xff, t->stream);
  rc |= grow(&t->T.killed, &c[5], want, used, 0xff, t->stream);
  rc |= grow(&t->T.touched, &c[6], want, used, 0xff, t->stream);
  int64_t cr = 4 * cap;  // read only where written in the same round
  rc |= grow(&t->T.repl, &cr, 4 * want, 0, -1, t->stream);
  if (rc) return vd::E_NOMEM;
  t->T.cap_simp = (int)want;
  return vd::E_OK;
}

int ensure_points(vd_tree* t, int64_t n_new) {
  int64_t want = t->nverts + n_new;
  if (want > 0x7ffffff0LL) return vd::E_ARG;
  int64_t cap = t->cap_verts;
  if (want > cap) {
    int64_t target = std::max(want, cap + cap / 2);
    int64_t cap2 = t->cap_verts;
    if (grow(&t->T.pts, &cap, target, t->nverts, -1, t->stream)) return vd::E_NOMEM;
    if (grow(&t->T.ptf, &cap2, target, t->nverts, -1, t->stream)) return vd::E_NOMEM;
    t->cap_verts = cap;
    t->T.cap_verts = (int)cap;
  }
  if (n_new > t->cap_act) {
    int64_t c = std::max<int64_t>(n_new, 1024);
    dfree(t->T.act[0]);
    dfree(t->T.act[1]);
    dfree(t->T.cand);
    dfree(t->T.cinfo);
    dfree(t->T.wl[0]);
    dfree(t->T.wl[1]);
    dfree(t->T.order);
    dfree(t->T.win);
    dfree(t->T.bigc);
    dfree(t->T.bigw);
    // capacities read as empty until every array is back: a failed
    // allocation must not leave a later, smaller call on freed arrays
    t->cap_act = 0;
    t->T.cap_cand = 0;
    if (dalloc(&t->T.act[0], c) || dalloc(&t->T.act[1], c) || dalloc(&t->T.cand, c) ||
        dalloc(&t->T.cinfo, c) || dalloc(&t->T.wl[0], c) || dalloc(&t->T.wl[1], c) ||
        dalloc(&t->T.order, c) || dalloc(&t->T.win, c) || dalloc(&t->T.bigc, c) || dalloc(&t->T.bigw, c))
      return vd::E_NOMEM;
    t->cap_act = c;
    t->T.cap_cand = (int)c;
  }
  const int64_t pool_want = std::min<int64_t>(
      std::max<int64_t>((t->dim == 3 ? 48 : 24) * std::max<int64_t>(n_new, 1024), 8 * 360448 + 64),
      0x7fffffffLL);
  if (pool_want > t->T.cap_pool) {
    dfree(t->T.pool);
    t->T.cap_pool = 0;
    if (dalloc(&t->T.pool, pool_want)) return vd::E_NOMEM;
    t->T.cap_pool = (int)pool_want;
  }
  const int64_t dup_want = t->hctr->ndup + n_new;
  if (dup_want > t->T.cap_dups) {
    int64_t cap_d = t->T.cap_dups;
    if (grow(&t->T.dups, &cap_d, std::max(dup_want, cap_d * 2), std::min<int64_t>(t->hctr->ndup, cap_d),
             -1, t->stream))
      return vd::E_NOMEM;
    t->T.cap_dups = (int)cap_d;
  }
  return vd::E_OK;
}

void drop_graphs(vd_tree* t) {
  for (auto& g : t->graphs) cudaGraphExecDestroy(g.exec);
  t->graphs.clear();
}

void release(vd_tree* t) {
  if (!t) return;
  if (t->stream) cudaStreamSynchronize(t->stream);
  drop_graphs(t);
  dfree(t->T.sets);
  dfree(t->T.set_of);
  dfree(t->d_setoff);
  dfree(t->d_eoff);
  dfree(t->d_cr);
  dfree(t->d_flags);
  dfree(t->d_mm);
  dfree(t->T.pts);
  dfree(t->T.ptf);
  dfree(t->T.simp);
  dfree(t->T.vote);
  dfree(t->T.thin);
  dfree(t->T.claim_c);
  dfree(t->T.claim_n);
  dfree(t->T.touched);
  dfree(t->T.killed);
  dfree(t->T.act[0]);
  dfree(t->T.act[1]);
  dfree(t->T.order);
  dfree(t->T.win);
  dfree(t->T.bigc);
  dfree(t->T.bigw);
  dfree(t->T.repl);
  dfree(t->T.cand);
  dfree(t->T.cinfo);
  dfree(t->T.wl[0]);
  dfree(t->T.wl[1]);
  dfree(t->T.pool);
  dfree(t->T.dups);
  dfree(t->T.ctr);
  dfree(t->d_edges);
  dfree(t->es.cnt);
  dfree(t->es.off);
  dfree(t->es.buf);
  dfree(t->es.ucnt);
  dfree(t->es.uoff);
  dfree(t->es.big);
  dfree(t->es.nbig);
  dfree(t->es.scan_tmp);
  dfree(t->d_pair);
  dfree(t->d_check);
  dfree(t->d_misc);
  dfree(t->d_loc);
  dfree(t->d_counts);
  dfree(t->T.lev_off);
  dfree(t->T.hint);
  dfree(t->T.wchunk);
  if (t->h_mm) cudaFreeHost(t->h_mm);
  t->h_mm = nullptr;
  dfree(t->d_in);
  if (t->hctr) cudaFreeHost(t->hctr);
  if (t->h_pair) cudaFreeHost(t->h_pair);
  t->hctr = nullptr;
  t->h_pair = nullptr;
  for (auto& p : t->profs)
    for (auto& e : p.ev) cudaEventDestroy(e);
  t->profs.clear();
  if (t->own_stream && t->stream) cudaStreamDestroy(t->stream);
  t->stream = nullptr;
}

// Device, stream and pools of an empty tree of dimension `dim`.
// Finest location-hint level of a single-set tree (its size is not known
// when it is created) and of a set of n points in a batched build (about two
// points per finest cell).
#ifndef VD_HINT_LEVELS_3D
#define VD_HINT_LEVELS_3D 5
#endif
int single_hint_levels(int dim) { return dim == 3 ? VD_HINT_LEVELS_3D : 9; }
int set_hint_levels(int dim, int64_t n) {
  int l = 0;
  const int per = dim == 3 ? 8 : 4;
  for (int64_t cells = per; cells * 2 <= n && l < single_hint_levels(dim); cells *= per) ++l;
  return l;
}

int ensure_sets(vd_tree* t, int64_t nsets) {
  if (nsets <= t->cap_sets) return vd::E_OK;
  const int64_t c = std::max<int64_t>(nsets, 2 * t->cap_sets);
  dfree(t->T.sets);
  dfree(t->d_setoff);
  dfree(t->d_eoff);
  dfree(t->d_cr);
  dfree(t->d_flags);
  dfree(t->d_mm);
  t->cap_sets = 0;
  if (dalloc(&t->T.sets, c) || dalloc(&t->d_setoff, c + 1) || dalloc(&t->d_eoff, c + 1) ||
      dalloc(&t->d_cr, 4 * c) || dalloc(&t->d_flags, c) || dalloc(&t->d_mm, 6 * c))
    return vd::E_NOMEM;
  t->cap_sets = c;
  return vd::E_OK;
}

int alloc_tree(vd_tree* t, int dim, void* stream) {
  t->dim = dim;
  t->ns = dim + 1;
  t->tuning = dim == 3 ? vd::Tuning{2, 2, 1} : vd::Tuning{2, 1, 1};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return vd::E_CUDA;
  t->device = dev;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  t->sms = std::max(sms, 1);
  if (vd::prepare_round_kernels() != vd::E_OK) return vd::E_CUDA;
  if (stream) {
    t->stream = (cudaStream_t)stream;
    t->own_stream = false;
  } else {
    if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) return vd::E_CUDA;
    t->own_stream = true;
  }
  if (cudaMallocHost((void**)&t->hctr, sizeof(Counters)) != cudaSuccess) return vd::E_NOMEM;
  if (cudaMallocHost((void**)&t->h_pair, 16 * sizeof(int)) != cudaSuccess) return vd::E_NOMEM;
  memset(t->hctr, 0, sizeof(Counters));
  if (dalloc(&t->T.ctr, 1) || dalloc(&t->d_pair, 4) || dalloc(&t->d_check, 8) ||
      dalloc(&t->d_misc, 16) || dalloc(&t->d_counts, 2 * vd::kMaxLevels) ||
      dalloc(&t->T.lev_off, vd::kMaxLevels + 1))
    return vd::E_NOMEM;
  if (cudaMallocHost((void**)&t->h_mm, 8 * sizeof(unsigned long long)) != cudaSuccess) return vd::E_NOMEM;
  t->T.cap_wchunk = t->sms * kChunkWarpsPerSm;
  if (dalloc(&t->T.wchunk, t->T.cap_wchunk)) return vd::E_NOMEM;
  t->ncells = vd::hint_cells(dim, single_hint_levels(dim));
  if (dalloc(&t->T.hint, t->ncells)) return vd::E_NOMEM;
  if (ensure_sets(t, 1)) return vd::E_NOMEM;
  t->T.nsets = 1;
  t->T.nsuper = t->ns;
  t->cap_verts = t->ns + 16;
  if (dalloc(&t->T.pts, t->cap_verts) || dalloc(&t->T.ptf, t->cap_verts)) return vd::E_NOMEM;
  t->T.cap_verts = (int)t->cap_verts;
  t->T.cap_simp = 0;
  t->hctr->nsimp = 0;
  if (ensure_simplices(t, 1024)) return vd::E_NOMEM;
  return vd::E_OK;
}

// Super simplex of one set for its bounding sphere (centre c, radius rb):
// the reference's vertices and the vertex order that orients it positively.
int set_super(int dim, const double* c, double rb, double sup[4][3], double* R, int order[4]) {
  ref_super_from_sphere(dim, c, rb, sup, R);
  if (!(*R > 0.0) || !isfinite(*R)) return vd::E_DEGENERATE;
  for (int i = 0; i <= dim; ++i)
    for (int j = 0; j < 3; ++j)
      if (!isfinite(sup[i][j]) || !coord_ok(sup[i][j])) return vd::E_RANGE;
  order[0] = 0;
  order[1] = 1;
  order[2] = 2;
  order[3] = dim == 3 ? 3 : -1;
  vdp::VPt v[4];
  for (int i = 0; i < 4; ++i) v[i] = vdp::VPt{sup[i][0], sup[i][1], sup[i][2], 0.0};
  vdp::Tally tl = {0, 0, 0, 0};
  int err = 0;
  const int neg = dim == 3 ? vdp::exit_face<3, true>(v, v[3], 1u << 3, tl, err)
                           : vdp::exit_face<2, true>(v, v[2], 1u << 2, tl, err);
  if (neg >= 0) {
    std::swap(order[0], order[1]);
    vdp::VPt w[4] = {v[1], v[0], v[2], v[3]};
    const int neg2 = dim == 3 ? vdp::exit_face<3, true>(w, w[3], 1u << 3, tl, err)
                              : vdp::exit_face<2, true>(w, w[2], 1u << 2, tl, err);
    if (neg2 >= 0) return vd::E_DEGENERATE;
  }
  return vd::E_OK;
}

// (Re)starts the tree as `nsets` super simplices, one per set, for the
// bounding spheres (centre c[3 s ..], radius rb[s]) of the sets' points;
// `sizes` (batched build) gives the points of each set.  Pools keep their
// capacity.
int set_geometry_sets(vd_tree* t, int nsets, const double* c, const double* rb, const int64_t* sizes) {
  const int dim = t->dim, nv = dim + 1;
  if (nsets < 1 || (int64_t)nsets * nv > 0x40000000LL) return vd::E_ARG;
  int rc = ensure_sets(t, nsets);
  if (rc) return rc;
  const int64_t ns = (int64_t)nsets * nv;
  if (ns + 16 > t->cap_verts) {
    int64_t cap = t->cap_verts, cap2 = t->cap_verts;
    if (grow(&t->T.pts, &cap, ns + 16, 0, -1, t->stream)) return vd::E_NOMEM;
    if (grow(&t->T.ptf, &cap2, ns + 16, 0, -1, t->stream)) return vd::E_NOMEM;
    t->cap_verts = cap;
    t->T.cap_verts = (int)cap;
  }
  rc = ensure_simplices(t, nsets + 1024);
  if (rc) return rc;
  std::vector<vdp::VPt> sv(ns);
  std::vector<vdp::FPt> sf(ns);
  std::vector<vd::Simplex> roots(nsets);
  std::vector<vd::SetGeo> geo(nsets);
  int64_t cells = 0;
  for (int s = 0; s < nsets; ++s) {
    double sup[4][3], R;
    int order[4];
    rc = set_super(dim, c + 3 * s, rb[s], sup, &R, order);
    if (rc) return rc;
    if (s == 0) {
      memcpy(t->sup, sup, sizeof(sup));
      t->R = R;
      memcpy(t->sup_order, order, sizeof(order));
    }
    for (int k = 0; k < nv; ++k) {
      sv[(int64_t)s * nv + k] = vdp::VPt{sup[k][0], sup[k][1], sup[k][2], 0.0};
      sf[(int64_t)s * nv + k] = vdp::split_point(sup[k][0], sup[k][1], sup[k][2]);
    }
    vd::SetGeo& g = geo[s];
    for (int k = 0; k < 3; ++k) g.org[k] = (k < dim ? c[3 * s + k] : 0.0) - rb[s];
    g.scale = rb[s] > 0 ? 1.0 / (2.0 * rb[s]) : 1.0;
    for (int k = 0; k < 3; ++k) g.orgf[k] = (float)g.org[k];
    g.scalef = (float)g.scale;
    g.hint_levels = sizes ? set_hint_levels(dim, sizes[s]) : single_hint_levels(dim);
    g.hint_off = (int)cells;
    g.root = s;
    g.n = sizes ? (int)sizes[s] : 0;
    for (int k = 0; k < 4; ++k) {
      g.sup[k] = order[k] < 0 ? -1 : s * nv + order[k];
      roots[s].v[k] = g.sup[k];
      roots[s].n[k] = -1;
    }
    cells += vd::hint_cells(dim, g.hint_levels);
    if (cells > 0x7fffffffLL) return vd::E_NOMEM;
  }
  if (cells > t->ncells) {
    dfree(t->T.hint);
    t->ncells = 0;
    if (dalloc(&t->T.hint, cells)) return vd::E_NOMEM;
    t->ncells = cells;
  }
  t->has_geometry = true;
  t->nsets = nsets;
  t->ns = (int)ns;
  t->T.nsets = nsets;
  t->T.nsuper = (int)ns;
  cudaMemsetAsync(t->T.hint, 0xff, sizeof(int) * cells, t->stream);
  cudaMemsetAsync(t->T.wchunk, 0, sizeof(int2) * t->T.cap_wchunk, t->stream);
  cudaMemcpyAsync(t->T.sets, geo.data(), sizeof(vd::SetGeo) * nsets, cudaMemcpyHostToDevice, t->stream);
  cudaMemcpyAsync(t->T.pts, sv.data(), sizeof(vdp::VPt) * ns, cudaMemcpyHostToDevice, t->stream);
  cudaMemcpyAsync(t->T.ptf, sf.data(), sizeof(vdp::FPt) * ns, cudaMemcpyHostToDevice, t->stream);
  // Slots of an earlier build read as dead: a warp that takes a new chunk
  // of fresh slots leaves the rest of its old chunk unwritten, and such
  // slots must not show an old simplex.
  const int64_t used = std::min<int64_t>(std::max<int64_t>(t->simp_hwm, t->hctr->nsimp), t->T.cap_simp);
  if (used > 0) cudaMemsetAsync(t->T.simp, 0xff, sizeof(vd::Simplex) * used, t->stream);
  t->simp_hwm = nsets;
  cudaMemcpyAsync(t->T.simp, roots.data(), sizeof(vd::Simplex) * nsets, cudaMemcpyHostToDevice, t->stream);
  t->nverts = ns;
  t->inserted = 0;
  t->round_base = t->round;
  t->edges_valid = false;
  memset(t->hctr, 0, sizeof(Counters));
  t->hctr->nsimp = nsets;
  t->hctr->round = t->round - 1;  // the next k_plan opens round t->round
  cudaMemcpyAsync(t->T.ctr, t->hctr, sizeof(Counters), cudaMemcpyHostToDevice, t->stream);
  return cuda_status(cudaStreamSynchronize(t->stream));
}

// Single-set tree: the reference's DelaunayTree.
int set_geometry(vd_tree* t, const double* c, double rb) {
  t->set_off.clear();
  return set_geometry_sets(t, 1, c, &rb, nullptr);
}

int check_host_points(int dim, const double* pts, int64_t n) {
  if ((dim != 2 && dim != 3) || n < 1 || !pts) return vd::E_ARG;
  for (int64_t i = 0; i < n * dim; ++i) {
    if (!isfinite(pts[i])) return vd::E_NONFINITE;
    if (!coord_ok(pts[i])) return vd::E_RANGE;
  }
  return vd::E_OK;
}

int init_tree(vd_tree* t, int dim, const double* pts, int64_t n, void* stream) {
  int rc = check_host_points(dim, pts, n);
  if (rc) return rc;
  double c[3] = {0, 0, 0}, rb = 0;
  ref_bounding_sphere(dim, pts, n, c, &rb);
  rc = alloc_tree(t, dim, stream);
  if (rc) return rc;
  return set_geometry(t, c, rb);
}

// Bounding sphere of n device points (same result as the reference's loop).
int size_from_device(vd_tree* t, const double* d_pts, int64_t n, double* c, double* rb) {
  if (n < 1 || !d_pts) return vd::E_ARG;
  const int dim = t->dim;
  const vd::Launch L = launch_of(t);
  unsigned long long init[6] = {~0ull, ~0ull, ~0ull, 0, 0, 0};
  memcpy(t->h_mm, init, sizeof(init));
  unsigned long long* d_mm = reinterpret_cast<unsigned long long*>(t->d_misc);
  cudaMemcpyAsync(d_mm, t->h_mm, sizeof(init), cudaMemcpyHostToDevice, t->stream);
  vd::launch_bbox(L, dim, d_pts, n, d_mm);
  cudaMemcpyAsync(t->h_mm, d_mm, sizeof(init), cudaMemcpyDeviceToHost, t->stream);
  if (cudaStreamSynchronize(t->stream) != cudaSuccess) return vd::E_CUDA;
  double lo[3], hi[3];
  for (int k = 0; k < dim; ++k) {
    auto dec = [](unsigned long long key) {
      const unsigned long long b = (key >> 63) ? (key & 0x7fffffffffffffffull) : ~key;
      double x;
      memcpy(&x, &b, 8);
      return x;
    };
    lo[k] = dec(t->h_mm[k]);
    hi[k] = dec(t->h_mm[3 + k]);
    if (!isfinite(lo[k]) || !isfinite(hi[k])) return vd::E_NONFINITE;
    c[k] = (hi[k] + lo[k]) / 2.0;
  }
  for (int k = dim; k < 3; ++k) c[k] = 0.0;
  double su = 0.0, sl = 0.0;
  for (int i = 0; i < dim; ++i) su += (hi[i] - c[i]) * (hi[i] - c[i]);
  for (int i = 0; i < dim; ++i) sl += (lo[i] - c[i]) * (lo[i] - c[i]);
  const double ud = sqrt(su), ld = sqrt(sl);
  const double r0 = ud > ld ? ud : ld;
  int* d_flag = t->d_misc + 12;
  cudaMemsetAsync(d_flag, 0, sizeof(int), t->stream);
  vd::launch_outside(L, dim, d_pts, n, c, r0, d_flag);
  cudaMemcpyAsync(t->h_pair + 8, d_flag, sizeof(int), cudaMemcpyDeviceToHost, t->stream);
  if (cudaStreamSynchronize(t->stream) != cudaSuccess) return vd::E_CUDA;
  *rb = t->h_pair[8] ? r0 * 1.5 : r0;
  return vd::E_OK;
}

vd::Launch sized_launch(const vd_tree* t, int64_t items) {
  vd::Launch L = launch_of(t);
  int64_t p2 = 128;  // powers of two keep the set of captured grids small
  while (p2 < items) p2 <<= 1;
  items = p2;
  const int64_t blocks = (items + 255) / 256;
  L.blocks = (int)std::max<int64_t>(1, std::min<int64_t>(blocks, L.blocks));
  const int64_t warps = ((items + 3) / 4) * 4;
  L.warps = (int)std::max<int64_t>(4, std::min<int64_t>(warps, L.warps));
  return L;
}

// Launches `chunk` rounds as one CUDA graph, capturing it on first use.
// Returns false (nothing launched) when graphs are off for this tree:
// profiling and tracing need per-kernel events, and a failed capture turns
// graphs off.
bool launch_chunk_graph(vd_tree* t, const vd::Launch& L, int chunk, const vd::Feed& fd) {
  if (!t->use_graphs || t->prof || t->trace) return false;
  vd_tree::ChunkGraph* hit = nullptr;
  for (auto& g : t->graphs)
    if (g.chunk == chunk && g.blocks == L.blocks && g.warps == L.warps && g.passes == t->tuning.passes &&
        g.thin == t->tuning.thin && g.adjacent == t->tuning.adjacent && g.exact_int == t->tuning.exact_int &&
        g.big_block == t->tuning.big_block &&
        g.seed == fd.seed && g.ratio == fd.ratio &&
        memcmp(&g.T, &t->T, sizeof(vd::DevTree)) == 0) {
      hit = &g;
      break;
    }
  if (!hit) {
    if (t->graphs.size() >= 24) drop_graphs(t);
    const long long before = vd::launches_total();
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool ok = cudaStreamBeginCapture(t->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      for (int k = 0; k < chunk; ++k) vd::launch_round(t->T, L, t->dim, t->tuning, fd, nullptr);
      ok = cudaStreamEndCapture(t->stream, &graph) == cudaSuccess && graph;
    }
    if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    const long long launches = vd::launches_total() - before;
    vd::note_launches(-launches);  // counted when replayed
    if (!ok) {
      cudaGetLastError();
      t->use_graphs = false;
      return false;
    }
    vd_tree::ChunkGraph g;
    memcpy(&g.T, &t->T, sizeof(vd::DevTree));
    g.chunk = chunk;
    g.blocks = L.blocks;
    g.warps = L.warps;
    g.passes = t->tuning.passes;
    g.thin = t->tuning.thin;
    g.adjacent = t->tuning.adjacent;
    g.exact_int = t->tuning.exact_int;
    g.big_block = t->tuning.big_block;
    g.seed = fd.seed;
    g.ratio = fd.ratio;
    g.launches = launches;
    g.exec = exec;
    t->graphs.push_back(g);
    hit = &t->graphs.back();
  }
  if (cudaGraphLaunch(hit->exec, t->stream) != cudaSuccess) {
    cudaGetLastError();
    t->use_graphs = false;
    return false;
  }
  vd::note_launches(hit->launches);
  return true;
}

// Runs insertion rounds until every priority level of the current call has
// been fed and no point is active.  The host only reads the counters between
// chunks of rounds (to grow pools and to stop); within a chunk the feed is
// decided on the device.
int run_rounds(vd_tree* t, int& r, int64_t n_call, uint64_t seed) {
  const vd::Feed fd_main{seed, (float)t->ratio};
  const vd::Feed fd_early{seed, (float)std::max(t->ratio, t->early_ratio)};
  // winners refresh every level of the location hints during the early phase
  t->T.hint_all_below = (int)std::min<int64_t>(t->early_until, 0x7fffffff);
  const vd::Tuning tu_main = t->tuning;
  vd::Tuning tu_early = t->tuning;
  tu_early.thin = t->early_thin;
  int chunk = 1;
  int64_t last_progress = -1;
  int stalled = 0;
  int rc = vd::E_OK;
  Counters& h = *t->hctr;
  int64_t active = 0, fed = 0, done = t->hctr->ninserted;
  // exact tests of this call so far decide the form of the conflict-test kernels
  const unsigned long long exact0 = vd::stat_total(h, vd::STAT_EXACT);
  bool exact_int = t->exact_mode == 2;
  // oversized searches and stars go to whole-block kernels once the call has
  // had one (until then a warp redoes them, and the extra kernels are not run)
  const unsigned long long spilled0 = h.spilled;
  bool big_block = false;
  // the first rounds, while few points are active, run in one cooperative
  // launch (k_rounds_small); the rest as chunks of captured rounds
  bool small = t->small_rounds_max > 0 && !t->trace;
  while (true) {
    if (t->trace) chunk = 1;
    // early phase or main phase for this chunk (the host knows the inserted count)
    const bool early = done < t->early_until;
    const vd::Feed& fd = early ? fd_early : fd_main;
    t->tuning = early ? tu_early : tu_main;
    t->tuning.exact_int = exact_int ? 1 : 0;
    t->tuning.big_block = big_block ? 1 : 0;
    bool ran_small = false;
    if (small) {
      small = false;
      ScopedProf sp(t, vd::KT_SMALL);
      ran_small = vd::launch_small_rounds(t->T, t->stream, t->dim, t->tuning, fd, t->small_rounds_max, 1 << 20) ==
                  vd::E_OK;
    }
    if (!ran_small) {
      // grid sized for the most points that can be active during the chunk
      const double grow = std::pow(1.4, chunk);
      const int64_t est = std::min<int64_t>(n_call - fed + active,
                                            (int64_t)((double)(done + active + 256) * grow));
      const vd::Launch L = sized_launch(t, est);
      if (!launch_chunk_graph(t, L, chunk, fd))
        for (int k = 0; k < chunk; ++k) vd::launch_round(t->T, L, t->dim, t->tuning, fd, round_prof(t, k));
      r += chunk;
    }
    rc = sync_counters(t);
    if (rc) break;
    if (ran_small)
      r = h.round + 1;  // the kernel decided how many rounds it ran
    else
      accumulate_events(t, chunk);
    if (t->trace) {
      // GPU time of the round in microseconds when profiling is on
      int64_t us = -1;
      if (t->prof && !t->profs.empty() && t->profs[0].n > 0) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, t->profs[0].ev[0], t->profs[0].ev[t->profs[0].n]) == cudaSuccess)
          us = (int64_t)(ms * 1000.0f);
      }
      const int64_t row[8] = {r - 1,
                              (int64_t)h.nact[(r - 1) & 1],
                              (int64_t)h.candidates,
                              (int64_t)h.searched,
                              (int64_t)h.ninserted,
                              (int64_t)vd::stat_total(h, vd::STAT_TESTS),
                              us,
                              (int64_t)h.nact[r & 1]};
      t->trace_rows.insert(t->trace_rows.end(), row, row + 8);
    }
    if (h.err) {
      rc = h.err;
      break;
    }
    if (t->exact_mode == 0 && (int64_t)(vd::stat_total(h, vd::STAT_EXACT) - exact0) >= t->exact_switch)
      exact_int = true;
    if (h.spilled > spilled0) big_block = true;
    active = h.nact[r & 1];
    fed = h.feed_hi;
    done = h.ninserted;
    const bool all_fed = h.lev_next >= h.nlev;
    if (all_fed && active == 0) break;
    // grow pools when a round had to defer work
    bool fix = false;
    if (h.simp_overflow || (double)h.nsimp > 0.85 * t->T.cap_simp) {
      h.nsimp -= h.wasted;
      h.wasted = 0;
      h.simp_overflow = 0;
      int64_t want = (int64_t)t->T.cap_simp + std::max<int64_t>(t->T.cap_simp / 2, 4096);
      rc = ensure_simplices(t, want);
      if (rc) break;
      fix = true;
    }
    if (h.pool_overflow) {
      int64_t want = std::min<int64_t>((int64_t)t->T.cap_pool * 2, 0x7fffffffLL);
      dfree(t->T.pool);
      t->T.cap_pool = 0;
      if (dalloc(&t->T.pool, want)) {
        rc = vd::E_NOMEM;
        break;
      }
      t->T.cap_pool = (int)want;
      h.pool_overflow = 0;
      fix = true;
    }
    if (fix) cudaMemcpyAsync(t->T.ctr, &h, sizeof(Counters), cudaMemcpyHostToDevice, t->stream);
    const int64_t progress = (int64_t)h.ninserted + h.ndup;
    if (progress == last_progress) {
      if (++stalled >= 8) {
        rc = h.overflow ? vd::E_CAVITY : vd::E_ROUND_LIMIT;
        break;
      }
    } else {
      stalled = 0;
      last_progress = progress;
    }
    // once everything is fed the active set drains in a few rounds
    chunk = all_fed ? 2 : std::min(chunk * 2, kChunkMax);
  }
  t->tuning = tu_main;
  return rc;
}

// Insertion of n points already in device memory.  The points are split into
// priority levels (the first `first_prefix` points, then growing by
// `growth`); rounds activate levels as the triangulation grows (k_plan), so
// early rounds, which can only insert a few points into a small
// triangulation, do not locate, relocate or nominate the whole input.
int insert_device(vd_tree* t, const double* d_xyz, int64_t n, uint64_t seed) {
  if (n < 0 || (n > 0 && !d_xyz) || !t->has_geometry) return vd::E_ARG;
  if (n == 0) return vd::E_OK;
  int rc = ensure_points(t, n);
  if (rc) return rc;
  const double per = t->dim == 3 ? 7.6 : 2.3;
  rc = ensure_simplices(t, t->hctr->nsimp + (int64_t)(per * (double)n) + 4096 + 32LL * t->T.cap_wchunk);
  if (rc) return rc;
  t->edges_valid = false;
  const vd::Launch L = launch_of(t);
  const int base = (int)t->nverts;
  vd::launch_upload(t->T, L, t->dim, d_xyz, n, base);
  // priority levels: thresholds of the one set, or a level count covering
  // the largest set of a batched build (each set computes its own)
  std::vector<unsigned long long> thr;
  const double first = (double)std::max<int64_t>(t->first_prefix, 1);
  if (t->nsets == 1) {
    double m = std::min<double>(first, (double)n);
    while ((int)thr.size() < vd::kMaxLevels - 1) {
      const double f = m / (double)n;
      if (f >= 1.0) break;
      thr.push_back((unsigned long long)(f * 4294967296.0));
      m = std::max(m * t->growth, m + 1.0);
    }
    thr.push_back(1ull << 32);
  } else {
    long long big = 1;
    for (int s = 0; s < t->nsets; ++s) big = std::max(big, t->set_off[s + 1] - t->set_off[s]);
    int nlev = 1;
    for (double m = first; m < (double)big && nlev < vd::kMaxLevels; m *= t->growth) ++nlev;
    thr.assign(nlev, 1ull << 32);
  }
  cudaMemsetAsync(t->d_counts, 0, sizeof(int) * 2 * vd::kMaxLevels, t->stream);
  vd::launch_levels(t->T, L, n, base, seed, thr.data(), (int)thr.size(), first, t->growth, t->d_counts);
  // a fresh single-set call starts with its first levels in one block
  const int64_t fb_max = t->first_block >= 0 ? t->first_block : 150;
  const bool first_block = fb_max > 0 && t->nsets == 1 && t->hctr->ninserted == 0 && t->hctr->ndup == 0;
  std::vector<int> lev_counts(thr.size(), 0);
  if (first_block)
    cudaMemcpyAsync(lev_counts.data(), t->d_counts, sizeof(int) * lev_counts.size(), cudaMemcpyDeviceToHost,
                    t->stream);
  rc = sync_counters(t);
  if (rc) return rc;
  if (t->hctr->err) return t->hctr->err;
  t->nverts += n;
  t->calls++;
  if (first_block) {
    const int64_t cap = std::min<int64_t>(fb_max, vd::seed_max_points(t->dim));
    int64_t pts = 0;
    int levs = 0;
    for (size_t k = 0; k < lev_counts.size() && pts + lev_counts[k] <= cap; ++k) {
      pts += lev_counts[k];
      levs = (int)k + 1;
    }
    if (levs > 0 && pts > 0) {
      ScopedProf sp(t, vd::KT_SEED);
      vd::launch_seed(t->T, t->stream, t->dim, (int)pts, levs, seed);
    }
  }
  int r = t->round;
  rc = run_rounds(t, r, n, seed);
  t->round = r;
  vd::launch_close_chunks(t->T, L);
  if (!rc) rc = sync_counters(t);
  t->inserted = t->hctr->ninserted;
  if (rc) return rc;
  if (t->hctr->err) return t->hctr->err;
  return vd::E_OK;
}

int insert_host(vd_tree* t, const double* pts, int64_t n, uint64_t seed) {
  if (n < 0 || (n > 0 && !pts)) return vd::E_ARG;
  if (n == 0) return vd::E_OK;
  double* d = nullptr;
  if (dalloc(&d, (size_t)n * t->dim)) return vd::E_NOMEM;
  cudaMemcpyAsync(d, pts, sizeof(double) * n * t->dim, cudaMemcpyHostToDevice, t->stream);
  int rc = insert_device(t, d, n, seed);
  cudaStreamSynchronize(t->stream);
  cudaFree(d);
  return rc;
}

int ensure_edge_scratch(vd_tree* t, int64_t n_in, int64_t nsimp) {
  const int64_t buf_want = (t->dim == 3 ? 6 : 3) * nsimp + 64;
  if (t->es_n < n_in) {
    dfree(t->es.cnt);
    dfree(t->es.off);
    dfree(t->es.ucnt);
    dfree(t->es.uoff);
    dfree(t->es.big);
    dfree(t->es.nbig);
    dfree(t->es.scan_tmp);
    t->es_n = -1;  // empty until every array is back (see ensure_points)
    const int64_t m = n_in + 2;
    if (dalloc(&t->es.cnt, m) || dalloc(&t->es.off, m) || dalloc(&t->es.ucnt, m) ||
        dalloc(&t->es.uoff, m) || dalloc(&t->es.big, m) || dalloc(&t->es.nbig, 1) ||
        dalloc(&t->es.scan_tmp, vd::scan_scratch_ints(m)))
      return vd::E_NOMEM;
    t->es_n = n_in;
  }
  if (t->es.cap_buf < buf_want) {
    dfree(t->es.buf);
    t->es.cap_buf = 0;
    if (dalloc(&t->es.buf, buf_want)) return vd::E_NOMEM;
    t->es.cap_buf = buf_want;
  }
  if (t->cap_edges < buf_want) {
    dfree(t->d_edges);
    t->cap_edges = 0;
    if (dalloc(&t->d_edges, buf_want)) return vd::E_NOMEM;
    t->cap_edges = buf_want;
  }
  return vd::E_OK;
}

// Edge list into `out` (device, capacity `cap`), or into the tree's own
// buffer when out is null.  *m receives the count (which may exceed cap).
int compute_edges(vd_tree* t, uint2* out = nullptr, int64_t cap = 0, int64_t* m = nullptr) {
  if (t->edges_valid && !out) {
    if (m) *m = t->nedges;
    return vd::E_OK;
  }
  int rc = sync_counters(t);
  if (rc) return rc;
  const int64_t n_in = t->nverts - t->ns;
  const int64_t nsimp = t->hctr->nsimp;
  if ((t->dim == 3 ? 6 : 3) * nsimp > 0x7fffff00LL) return vd::E_NOMEM;
  rc = ensure_edge_scratch(t, n_in, nsimp);
  if (rc) return rc;
  int64_t got;
  {
    ScopedProf sp(t, vd::KT_EDGES);
    got = vd::run_edges(t->T, launch_of(t), t->dim, (int)nsimp, (int)n_in, t->es, out ? out : t->d_edges,
                        out ? cap : t->cap_edges, t->d_pair, t->h_pair);
  }
  if (got < 0) return vd::E_CUDA;
  if (m) *m = got;
  if (!out) {
    t->nedges = got;
    t->edges_valid = true;
  }
  return vd::E_OK;
}

// Bounding sphere (centre, radius before the reference's 1.5 growth) from
// the order-preserving bounding-box keys of k_bbox / k_set_bbox; the same
// arithmetic as src/geometry.rs:99-131.
int sphere_from_keys(int dim, const unsigned long long* mm, double* c, double* r0) {
  auto dec = [](unsigned long long key) {
    const unsigned long long b = (key >> 63) ? (key & 0x7fffffffffffffffull) : ~key;
    double x;
    memcpy(&x, &b, 8);
    return x;
  };
  double lo[3], hi[3];
  for (int k = 0; k < dim; ++k) {
    lo[k] = dec(mm[k]);
    hi[k] = dec(mm[3 + k]);
    if (!isfinite(lo[k]) || !isfinite(hi[k])) return vd::E_NONFINITE;
    c[k] = (hi[k] + lo[k]) / 2.0;
  }
  for (int k = dim; k < 3; ++k) c[k] = 0.0;
  double su = 0.0, sl = 0.0;
  for (int i = 0; i < dim; ++i) su += (hi[i] - c[i]) * (hi[i] - c[i]);
  for (int i = 0; i < dim; ++i) sl += (lo[i] - c[i]) * (lo[i] - c[i]);
  const double ud = sqrt(su), ld = sqrt(sl);
  *r0 = ud > ld ? ud : ld;
  return vd::E_OK;
}

// Batched build: sizes every set's super simplex from its points (device
// reductions, one block per set), then restarts the tree with one super
// simplex per set.
int batch_reset_device(vd_tree* t, const double* d_pts, const int64_t* offsets, int nsets) {
  if (!d_pts || !offsets || nsets < 1 || offsets[0] != 0) return vd::E_ARG;
  for (int s = 0; s < nsets; ++s)
    if (offsets[s + 1] <= offsets[s]) return vd::E_ARG;  // every set needs a point
  const int64_t n = offsets[nsets];
  if (n + (int64_t)nsets * (t->dim + 1) > 0x7ffffff0LL) return vd::E_ARG;
  int rc = ensure_sets(t, nsets);
  if (rc) return rc;
  const vd::Launch L = launch_of(t);
  t->set_off.assign(offsets, offsets + nsets + 1);
  cudaMemcpyAsync(t->d_setoff, t->set_off.data(), sizeof(long long) * (nsets + 1), cudaMemcpyHostToDevice,
                  t->stream);
  std::vector<unsigned long long> mm(6 * (size_t)nsets);
  vd::launch_set_bbox(L, t->dim, d_pts, t->d_setoff, nsets, t->d_mm);
  cudaMemcpyAsync(mm.data(), t->d_mm, sizeof(unsigned long long) * mm.size(), cudaMemcpyDeviceToHost, t->stream);
  if (cudaStreamSynchronize(t->stream) != cudaSuccess) return vd::E_CUDA;
  std::vector<double> c(3 * (size_t)nsets), cr(4 * (size_t)nsets), rb(nsets);
  std::vector<int64_t> sizes(nsets);
  for (int s = 0; s < nsets; ++s) {
    rc = sphere_from_keys(t->dim, &mm[6 * (size_t)s], &c[3 * (size_t)s], &rb[s]);
    if (rc) return rc;
    for (int k = 0; k < 3; ++k) cr[4 * (size_t)s + k] = c[3 * (size_t)s + k];
    cr[4 * (size_t)s + 3] = rb[s];
    sizes[s] = offsets[s + 1] - offsets[s];
  }
  std::vector<int> flags(nsets);
  cudaMemcpyAsync(t->d_cr, cr.data(), sizeof(double) * cr.size(), cudaMemcpyHostToDevice, t->stream);
  vd::launch_set_outside(L, t->dim, d_pts, t->d_setoff, nsets, t->d_cr, t->d_flags);
  cudaMemcpyAsync(flags.data(), t->d_flags, sizeof(int) * nsets, cudaMemcpyDeviceToHost, t->stream);
  if (cudaStreamSynchronize(t->stream) != cudaSuccess) return vd::E_CUDA;
  for (int s = 0; s < nsets; ++s)
    if (flags[s]) rb[s] *= 1.5;
  rc = set_geometry_sets(t, nsets, c.data(), rb.data(), sizes.data());
  if (rc) return rc;
  t->set_off.assign(offsets, offsets + nsets + 1);
  if (n > t->cap_setof) {
    dfree(t->T.set_of);
    t->cap_setof = 0;
    if (dalloc(&t->T.set_of, n)) return vd::E_NOMEM;
    t->cap_setof = n;
  }
  vd::launch_set_fill(L, t->d_setoff, nsets, t->T.set_of);
  return vd::E_OK;
}

// Edges of a batched build into d_uv (numbers within each set) and the
// host edge offsets of the sets.
int batch_edges(vd_tree* t, uint2* d_uv, int64_t cap, int64_t* edge_offsets, int64_t* n_edges) {
  int64_t m = 0;
  int rc = compute_edges(t, d_uv, cap, &m);
  if (n_edges) *n_edges = m;
  if (rc) return rc;
  const vd::Launch L = launch_of(t);
  vd::launch_set_edge_offsets(L, t->es.uoff, t->d_setoff, t->nsets, t->d_eoff);
  cudaMemcpyAsync(edge_offsets, t->d_eoff, sizeof(long long) * (t->nsets + 1), cudaMemcpyDeviceToHost, t->stream);
  if (m > cap) {
    if (cudaStreamSynchronize(t->stream) != cudaSuccess) return vd::E_CUDA;
    return vd::E_ARG;
  }
  vd::launch_localize(L, d_uv, m, t->T.set_of, t->d_setoff);
  return cuda_status(cudaStreamSynchronize(t->stream));
}

}  // namespace

// ===========================================================================
extern "C" {

const char* vd_status_str(int s) {
  switch (s) {
    case VD_OK: return "ok";
    case VD_ERR_ARG: return "invalid argument";
    case VD_ERR_CUDA: return "CUDA runtime error";
    case VD_ERR_NOMEM: return "device allocation failed";
    case VD_ERR_DUPLICATE: return "duplicate points were skipped";
    case VD_ERR_NONFINITE: return "non-finite coordinate";
    case VD_ERR_OUTSIDE: return "point not strictly inside the super simplex";
    case VD_ERR_PRECISION: return "exact arithmetic capacity exceeded";
    case VD_ERR_ROUND_LIMIT: return "insertion rounds made no progress";
    case VD_ERR_CAVITY: return "conflict region too large";
    case VD_ERR_WALK: return "point location did not terminate";
    case VD_ERR_INTERNAL: return "internal inconsistency";
    case VD_ERR_DEGENERATE: return "degenerate super simplex";
    case VD_ERR_RANGE: return "coordinate magnitude out of range";
    default: return "unknown status";
  }
}

vd_tree* vd_tree_new_on_stream(int dim, const double* pts, int64_t n, void* stream, int* status) {
  vd_tree* t = new (std::nothrow) vd_tree();
  if (!t) {
    if (status) *status = VD_ERR_NOMEM;
    return nullptr;
  }
  int rc = init_tree(t, dim, pts, n, stream);
  if (status) *status = rc;
  return t;
}

vd_tree* vd_tree_new(int dim, const double* pts, int64_t n, int* status) {
  return vd_tree_new_on_stream(dim, pts, n, nullptr, status);
}

int vd_super_simplex(int dim, const double* pts, int64_t n, double* out, double* radius) {
  if ((dim != 2 && dim != 3) || n < 1 || !pts || !out || !radius) return VD_ERR_ARG;
  for (int64_t i = 0; i < n * dim; ++i)
    if (!isfinite(pts[i])) return VD_ERR_NONFINITE;
  double sv[4][3];
  ref_super_vertices(dim, pts, n, sv, radius);
  for (int k = 0; k <= dim; ++k)
    for (int j = 0; j < 3; ++j) out[3 * k + j] = sv[k][j];
  return VD_OK;
}

vd_tree* vd_tree_new_device(int dim, const double* d_pts, int64_t n, void* stream, int* status) {
  vd_tree* t = new (std::nothrow) vd_tree();
  if (!t) {
    if (status) *status = VD_ERR_NOMEM;
    return nullptr;
  }
  int rc = (dim == 2 || dim == 3) && n >= 1 && d_pts ? alloc_tree(t, dim, stream) : VD_ERR_ARG;
  double c[3], rb;
  if (!rc) rc = size_from_device(t, d_pts, n, c, &rb);
  if (!rc) rc = set_geometry(t, c, rb);
  if (status) *status = rc;
  return t;
}

int vd_tree_reset(vd_tree* t, const double* pts, int64_t n) {
  if (!t || !t->hctr) return VD_ERR_ARG;
  int rc = check_host_points(t->dim, pts, n);
  if (rc) return rc;
  double c[3] = {0, 0, 0}, rb = 0;
  ref_bounding_sphere(t->dim, pts, n, c, &rb);
  return set_geometry(t, c, rb);
}

int vd_tree_reset_device(vd_tree* t, const double* d_pts, int64_t n) {
  if (!t || !t->hctr) return VD_ERR_ARG;
  double c[3], rb;
  int rc = size_from_device(t, d_pts, n, c, &rb);
  if (rc) return rc;
  return set_geometry(t, c, rb);
}

int vd_delaunay_device(vd_tree* t, const double* d_pts, int64_t n, uint64_t seed, uint32_t* d_uv, int64_t cap,
                       int64_t* n_edges) {
  if (!t || !t->hctr || (t->dim != 2 && t->dim != 3)) return VD_ERR_ARG;
  int rc = vd_tree_reset_device(t, d_pts, n);
  if (rc) return rc;
  rc = insert_device(t, d_pts, n, seed);
  if (rc == VD_OK && t->hctr->ndup > 0) rc = VD_ERR_DUPLICATE;
  if (rc && rc != VD_ERR_DUPLICATE) return rc;
  const int rc2 = vd_edges_device(t, d_uv, cap, n_edges);
  return rc2 ? rc2 : rc;
}

int vd_delaunay_tree(vd_tree* t, const double* pts, int64_t n, uint64_t seed, uint32_t* uv, int64_t cap,
                     int64_t* n_edges) {
  if (!t || !t->hctr || !pts || n < 1) return VD_ERR_ARG;
  if (n * t->dim > t->cap_in) {
    dfree(t->d_in);
    t->cap_in = 0;
    if (dalloc(&t->d_in, (size_t)(n * t->dim))) return VD_ERR_NOMEM;
    t->cap_in = n * t->dim;
  }
  cudaMemcpyAsync(t->d_in, pts, sizeof(double) * n * t->dim, cudaMemcpyHostToDevice, t->stream);
  int rc = vd_tree_reset_device(t, t->d_in, n);
  if (rc) return rc;
  rc = insert_device(t, t->d_in, n, seed);
  if (rc == VD_OK && t->hctr->ndup > 0) rc = VD_ERR_DUPLICATE;
  if (rc && rc != VD_ERR_DUPLICATE) return rc;
  const int rc2 = vd_edges_u32(t, uv, cap, n_edges);
  return rc2 ? rc2 : rc;
}

void vd_tree_free(vd_tree* t) {
  if (!t) return;
  release(t);
  delete t;
}

static int ready(vd_tree* t) { return (t && t->hctr && t->T.ctr) ? VD_OK : VD_ERR_ARG; }

int vd_insert_points_device(vd_tree* t, const double* d_pts, int64_t n, uint64_t seed) {
  if (ready(t) || t->nsets != 1) return VD_ERR_ARG;  // batched trees take no further points
  int rc = insert_device(t, d_pts, n, seed);
  if (rc == VD_OK && t->hctr->ndup > 0) rc = VD_ERR_DUPLICATE;
  return rc;
}

int vd_insert_points(vd_tree* t, const double* pts, int64_t n, uint64_t seed) {
  if (ready(t) || t->nsets != 1) return VD_ERR_ARG;  // batched trees take no further points
  int rc = insert_host(t, pts, n, seed);
  if (rc == VD_OK && t->hctr->ndup > 0) rc = VD_ERR_DUPLICATE;
  return rc;
}

// One point: a single-warp kernel (k_insert_one) does the whole insertion in
// one launch, the way the reference's insert_point applies one TreeUpdate;
// only a conflict region too large for the warp's shared memory (or a batched
// tree) goes through the insertion rounds instead.
int vd_insert_point(vd_tree* t, const double* p) {
  if (ready(t) || !p) return VD_ERR_ARG;
  if (!t->has_geometry || t->nsets != 1) return vd_insert_points(t, p, 1, 0);
  int rc = ensure_points(t, 1);
  if (rc) return rc;
  rc = ensure_simplices(t, (int64_t)t->hctr->nsimp + 4096);  // above any star a warp can write
  if (rc) return rc;
  const double c[3] = {p[0], p[1], t->dim == 3 ? p[2] : 0.0};
  t->edges_valid = false;
  vd::launch_insert_one(t->T, t->stream, t->dim, c, (int)t->nverts);
  rc = sync_counters(t);
  if (rc) return rc;
  const int out = t->hctr->single;
  if (out == -1) return vd_insert_points(t, p, 1, 0);
  if (out == VD_OK || out == VD_ERR_DUPLICATE) {
    t->nverts += 1;
    t->calls++;
    t->inserted = t->hctr->ninserted;
  }
  return out;
}

int vd_num_vertices(vd_tree* t, int64_t* n) {
  if (ready(t) || !n) return VD_ERR_ARG;
  *n = t->nverts - t->ns;
  return VD_OK;
}

int vd_max_simplex_id(vd_tree* t, int64_t* id) {
  if (ready(t) || !id) return VD_ERR_ARG;
  int rc = sync_counters(t);
  if (rc) return rc;
  *id = (int64_t)t->ns + (int64_t)t->hctr->created;
  return VD_OK;
}

int vd_num_simplices(vd_tree* t, int64_t* n) {
  if (ready(t) || !n) return VD_ERR_ARG;
  int rc = sync_counters(t);
  if (rc) return rc;
  *n = 1 + (int64_t)t->hctr->created - (int64_t)t->hctr->killed;
  return VD_OK;
}

int vd_simplices(vd_tree* t, int32_t* verts, int32_t* nbrs, int64_t cap, int64_t* n) {
  if (ready(t) || !n) return VD_ERR_ARG;
  int rc = sync_counters(t);
  if (rc) return rc;
  const int64_t ns = t->hctr->nsimp;
  std::vector<vd::Simplex> h(ns);
  cudaMemcpyAsync(h.data(), t->T.simp, sizeof(vd::Simplex) * ns, cudaMemcpyDeviceToHost, t->stream);
  if (cudaStreamSynchronize(t->stream) != cudaSuccess) return VD_ERR_CUDA;
  std::vector<int32_t> remap(ns, -1);
  int64_t k = 0;
  for (int64_t i = 0; i < ns; ++i)
    if (h[i].v[0] >= 0) remap[i] = (int32_t)k++;
  *n = k;
  if (!verts && !nbrs) return VD_OK;
  if (cap < k) return VD_ERR_ARG;
  const int nv = t->dim + 1;
  int64_t r = 0;
  for (int64_t i = 0; i < ns; ++i) {
    if (h[i].v[0] < 0) continue;
    for (int j = 0; j < 4; ++j) {
      int v = j < nv ? h[i].v[j] : -1;
      if (verts) verts[4 * r + j] = j < nv ? (v < t->ns ? -(1 + v) : v - t->ns) : -1;
      int c = j < nv ? h[i].n[j] : -1;
      if (nbrs) nbrs[4 * r + j] = c < 0 ? -1 : remap[c >> 2];
    }
    ++r;
  }
  return VD_OK;
}

int vd_num_edges(vd_tree* t, int64_t* n) {
  if (ready(t) || !n) return VD_ERR_ARG;
  int rc = compute_edges(t, nullptr, 0, nullptr);
  if (rc) return rc;
  *n = t->nedges;
  return VD_OK;
}

int vd_edges(vd_tree* t, int64_t* uv, int64_t cap, int64_t* n) {
  if (ready(t)) return VD_ERR_ARG;
  int rc = compute_edges(t, nullptr, 0, nullptr);
  if (rc) return rc;
  if (n) *n = t->nedges;
  if (!uv) return VD_OK;
  if (cap < t->nedges) return VD_ERR_ARG;
  std::vector<uint2> h(t->nedges);
  cudaMemcpyAsync(h.data(), t->d_edges, sizeof(uint2) * t->nedges, cudaMemcpyDeviceToHost, t->stream);
  if (cudaStreamSynchronize(t->stream) != cudaSuccess) return VD_ERR_CUDA;
  for (int64_t i = 0; i < t->nedges; ++i) {
    uv[2 * i] = h[i].x;
    uv[2 * i + 1] = h[i].y;
  }
  return VD_OK;
}

int vd_edges_device(vd_tree* t, uint32_t* d_uv, int64_t cap, int64_t* n) {
  if (ready(t)) return VD_ERR_ARG;
  int64_t m = 0;
  int rc = d_uv ? compute_edges(t, reinterpret_cast<uint2*>(d_uv), cap, &m) : compute_edges(t, nullptr, 0, &m);
  if (rc) return rc;
  if (n) *n = m;
  return (d_uv && m > cap) ? VD_ERR_ARG : VD_OK;
}

int vd_edges_u32(vd_tree* t, uint32_t* uv, int64_t cap, int64_t* n) {
  if (ready(t)) return VD_ERR_ARG;
  int rc = compute_edges(t, nullptr, 0, nullptr);
  if (rc) return rc;
  if (n) *n = t->nedges;
  if (!uv) return VD_OK;
  if (cap < t->nedges) return VD_ERR_ARG;
  cudaMemcpyAsync(uv, t->d_edges, sizeof(uint2) * t->nedges, cudaMemcpyDeviceToHost, t->stream);
  return cuda_status(cudaStreamSynchronize(t->stream));
}

int vd_check_delaunay(vd_tree* t, int* ok, int64_t* violations) {
  if (ready(t) || !ok) return VD_ERR_ARG;
  int rc = sync_counters(t);
  if (rc) return rc;
  vd::launch_check(t->T, launch_of(t), t->dim, t->hctr->nsimp, t->d_check);
  unsigned long long h[6];
  cudaMemcpyAsync(h, t->d_check, sizeof(h), cudaMemcpyDeviceToHost, t->stream);
  rc = sync_counters(t);
  if (rc) return rc;
  if (violations)
    for (int k = 0; k < 6; ++k) violations[k] = (int64_t)h[k];
  const unsigned long long hull = (unsigned long long)t->nsets * (t->dim + 1);  // the super simplices' faces
  *ok = (h[0] == 0 && h[1] == 0 && h[2] == 0 && h[3] == 0 && h[4] == hull) ? 1 : 0;
  return t->hctr->err ? t->hctr->err : VD_OK;
}

int vd_duplicates(vd_tree* t, int64_t* pairs, int64_t cap, int64_t* n) {
  if (ready(t) || !n) return VD_ERR_ARG;
  int rc = sync_counters(t);
  if (rc) return rc;
  const int64_t m = std::min<int64_t>(t->hctr->ndup, t->T.cap_dups);
  *n = m;
  if (!pairs) return VD_OK;
  if (cap < m) return VD_ERR_ARG;
  std::vector<int2> h(m);
  if (m) {
    cudaMemcpyAsync(h.data(), t->T.dups, sizeof(int2) * m, cudaMemcpyDeviceToHost, t->stream);
    if (cudaStreamSynchronize(t->stream) != cudaSuccess) return VD_ERR_CUDA;
  }
  std::sort(h.begin(), h.end(), [](const int2& a, const int2& b) { return a.x < b.x; });
  for (int64_t i = 0; i < m; ++i) {
    pairs[2 * i] = h[i].x - t->ns;
    pairs[2 * i + 1] = h[i].y - t->ns;
  }
  return VD_OK;
}

int vd_get_stats(vd_tree* t, vd_stats* s) {
  if (ready(t) || !s) return VD_ERR_ARG;
  int rc = sync_counters(t);
  if (rc) return rc;
  const Counters& h = *t->hctr;
  s->rounds = t->round - t->round_base;
  s->inserted = h.ninserted;
  s->duplicates = h.ndup;
  s->live_simplices = 1 + (int64_t)h.created - (int64_t)h.killed;
  s->slots = h.nsimp;
  s->created = (int64_t)h.created;
  s->killed = (int64_t)h.killed;
  s->max_cavity = h.max_cav;
  s->max_facets = h.max_fac;
  s->pred_f32 = (int64_t)vd::stat_total(h, vd::STAT_F32);
  s->pred_f64 = (int64_t)vd::stat_total(h, vd::STAT_F64);
  s->pred_exact = (int64_t)vd::stat_total(h, vd::STAT_EXACT);
  s->pred_sos = (int64_t)vd::stat_total(h, vd::STAT_SOS);
  s->walk_steps = (int64_t)vd::stat_total(h, vd::STAT_WALK);
  s->cavity_tests = (int64_t)vd::stat_total(h, vd::STAT_TESTS);
  s->deferred_overflow = h.overflow;
  s->deferred_pool = h.pool_overflow;
  s->candidates = (int64_t)h.candidates;
  s->searched = (int64_t)h.searched;
  for (int p = 0; p < 3; ++p) s->won_pass[p] = (int64_t)h.won[p];
  for (int p = 3; p < vd::kPassesMax; ++p) s->won_pass[2] += (int64_t)h.won[p];
  s->spilled = (int64_t)h.spilled;
  s->max_search_levels = h.max_levels;
  return VD_OK;
}

int vd_delaunay(int dim, const double* pts, int64_t n, uint64_t seed, int64_t* uv, int64_t cap,
                int64_t* n_edges) {
  int st = 0;
  vd_tree* t = vd_tree_new(dim, pts, n, &st);
  if (!t) return VD_ERR_NOMEM;
  if (st) {
    vd_tree_free(t);
    return st;
  }
  int rc = vd_insert_points(t, pts, n, seed);
  if (rc && rc != VD_ERR_DUPLICATE) {
    vd_tree_free(t);
    return rc;
  }
  int rc2 = vd_edges(t, uv, cap, n_edges);
  vd_tree_free(t);
  return rc2 ? rc2 : rc;
}

int vd_set_profiling(vd_tree* t, int on) {
  if (ready(t)) return VD_ERR_ARG;
  t->prof = on != 0;
  for (int k = 0; k < vd::KT_COUNT; ++k) {
    t->kms[k] = 0.0;
    t->kcnt[k] = 0;
  }
  return VD_OK;
}

int vd_profile(vd_tree* t, double* ms, int64_t* launches, int cap, int* n) {
  if (ready(t) || !n) return VD_ERR_ARG;
  *n = vd::KT_COUNT;
  if (!ms && !launches) return VD_OK;
  if (cap < *n) return VD_ERR_ARG;
  for (int k = 0; k < vd::KT_COUNT; ++k) {
    if (ms) ms[k] = t->kms[k];
    if (launches) launches[k] = t->kcnt[k];
  }
  return VD_OK;
}

int64_t vd_kernel_launches(void) { return (int64_t)vd::launches_total(); }

const char* vd_profile_name(int i) {
  if (i >= 0 && i < vd::KT_COUNT) return vd::kKernelTypeNames[i];
  return "";
}

int vd_set_schedule(vd_tree* t, int64_t first_prefix, double growth, double ratio) {
  if (ready(t) || first_prefix < 1 || !(growth > 1.0 && growth <= 16.0) || !(ratio > 0.0 && ratio <= 64.0))
    return VD_ERR_ARG;
  t->first_prefix = first_prefix;
  t->growth = growth;
  t->ratio = ratio;
  return VD_OK;
}

int vd_set_tuning(vd_tree* t, int passes, int thin) {
  if (ready(t) || passes < 1 || passes > vd::kPassesMax || thin < 0 || thin > 2) return VD_ERR_ARG;
  t->tuning.passes = passes;
  t->tuning.thin = thin;
  return VD_OK;
}

int vd_set_early_phase(vd_tree* t, int64_t until_inserted, int thin, double ratio) {
  if (ready(t) || until_inserted < 0 || thin < 0 || thin > 2 || !(ratio > 0.0 && ratio <= 64.0)) return VD_ERR_ARG;
  t->early_until = until_inserted;
  t->early_thin = thin;
  t->early_ratio = ratio;
  return VD_OK;
}

int vd_set_first_block(vd_tree* t, int64_t max_points) {
  if (ready(t) || max_points < 0) return VD_ERR_ARG;
  t->first_block = max_points;
  return VD_OK;
}

int vd_set_exact_tier(vd_tree* t, int mode, int64_t switch_after) {
  if (ready(t) || mode < 0 || mode > 2 || switch_after < 0) return VD_ERR_ARG;
  t->exact_mode = mode;
  t->exact_switch = switch_after;
  return VD_OK;
}

int vd_set_small_rounds(vd_tree* t, int max_active) {
  if (ready(t) || max_active < 0) return VD_ERR_ARG;
  t->small_rounds_max = max_active;
  return VD_OK;
}

int vd_set_adjacent(vd_tree* t, int on) {
  if (ready(t)) return VD_ERR_ARG;
  t->tuning.adjacent = on ? 1 : 0;
  return VD_OK;
}

int vd_set_graphs(vd_tree* t, int on) {
  if (ready(t)) return VD_ERR_ARG;
  t->use_graphs = on != 0;
  if (!on) drop_graphs(t);
  return VD_OK;
}

int vd_set_trace(vd_tree* t, int on) {
  if (ready(t)) return VD_ERR_ARG;
  t->trace = on != 0;
  t->trace_rows.clear();
  return VD_OK;
}

int vd_trace(vd_tree* t, int64_t* rows, int64_t cap, int64_t* n) {
  if (ready(t) || !n) return VD_ERR_ARG;
  *n = (int64_t)t->trace_rows.size() / 8;
  if (!rows) return VD_OK;
  if (cap < *n) return VD_ERR_ARG;
  std::copy(t->trace_rows.begin(), t->trace_rows.end(), rows);
  return VD_OK;
}

vd_tree* vd_tree_create(int dim, void* stream, int* status) {
  vd_tree* t = new (std::nothrow) vd_tree();
  if (!t) {
    if (status) *status = VD_ERR_NOMEM;
    return nullptr;
  }
  const int rc = (dim == 2 || dim == 3) ? alloc_tree(t, dim, stream) : VD_ERR_ARG;
  if (status) *status = rc;
  return t;
}

int vd_batch_delaunay_device(vd_tree* t, const double* d_pts, const int64_t* offsets, int nsets, uint64_t seed,
                             uint32_t* d_uv, int64_t cap, int64_t* edge_offsets) {
  if (ready(t) || !edge_offsets || (!d_uv && cap > 0)) return VD_ERR_ARG;
  int rc = batch_reset_device(t, d_pts, offsets, nsets);
  if (rc) return rc;
  rc = insert_device(t, d_pts, offsets[nsets], seed);
  if (rc == VD_OK && t->hctr->ndup > 0) rc = VD_ERR_DUPLICATE;
  if (rc && rc != VD_ERR_DUPLICATE) return rc;
  const int rc2 = batch_edges(t, reinterpret_cast<uint2*>(d_uv), cap, edge_offsets, nullptr);
  return rc2 ? rc2 : rc;
}

int vd_batch_delaunay(vd_tree* t, const double* pts, const int64_t* offsets, int nsets, uint64_t seed,
                      uint32_t* uv, int64_t cap, int64_t* edge_offsets) {
  if (ready(t) || !pts || !offsets || nsets < 1 || !edge_offsets || (!uv && cap > 0)) return VD_ERR_ARG;
  const int64_t n = offsets[nsets];
  if (n < 1) return VD_ERR_ARG;
  int rc = check_host_points(t->dim, pts, n);
  if (rc) return rc;
  if (n * t->dim > t->cap_in) {
    dfree(t->d_in);
    t->cap_in = 0;
    if (dalloc(&t->d_in, (size_t)(n * t->dim))) return VD_ERR_NOMEM;
    t->cap_in = n * t->dim;
  }
  cudaMemcpyAsync(t->d_in, pts, sizeof(double) * n * t->dim, cudaMemcpyHostToDevice, t->stream);
  rc = batch_reset_device(t, t->d_in, offsets, nsets);
  if (rc) return rc;
  rc = insert_device(t, t->d_in, n, seed);
  if (rc == VD_OK && t->hctr->ndup > 0) rc = VD_ERR_DUPLICATE;
  if (rc && rc != VD_ERR_DUPLICATE) return rc;
  // edges into the tree's own buffer, numbered within their sets, then out
  int64_t m = 0;
  int rc2 = sync_counters(t);
  if (!rc2) rc2 = ensure_edge_scratch(t, t->nverts - t->ns, t->hctr->nsimp);
  if (!rc2) {
    t->edges_valid = false;  // the buffer holds set-local numbers
    rc2 = batch_edges(t, t->d_edges, t->cap_edges, edge_offsets, &m);
  }
  if (!rc2 && uv) {
    if (cap < m) return VD_ERR_ARG;
    cudaMemcpyAsync(uv, t->d_edges, sizeof(uint2) * m, cudaMemcpyDeviceToHost, t->stream);
    rc2 = cuda_status(cudaStreamSynchronize(t->stream));
  }
  return rc2 ? rc2 : rc;
}

int vd_num_sets(vd_tree* t, int* nsets) {
  if (ready(t) || !nsets) return VD_ERR_ARG;
  *nsets = t->nsets;
  return VD_OK;
}

int vd_set_launch(vd_tree* t, int warps_per_sm, int blocks_per_sm) {
  if (ready(t) || warps_per_sm < 4 || warps_per_sm > kMaxWarpsPerSm || (warps_per_sm & 3) || blocks_per_sm < 1 ||
      blocks_per_sm > 32)
    return VD_ERR_ARG;
  t->warps_per_sm = warps_per_sm;
  t->blocks_per_sm = blocks_per_sm;
  return VD_OK;
}

int vd_autotune_batch(vd_tree* t, const double* d_pts, const int64_t* offsets, int nsets, int64_t sample_points,
                      int64_t* out) {
  if (ready(t) || !d_pts || !offsets || nsets < 1 || offsets[0] != 0) return VD_ERR_ARG;
  for (int s = 0; s < nsets; ++s)
    if (offsets[s + 1] <= offsets[s]) return VD_ERR_ARG;
  const int dim = t->dim;
  // sample: every stride-th set (the size mix of the batch), up to sample_points
  const int64_t total = offsets[nsets];
  const int64_t want = std::max<int64_t>(1, std::min(sample_points, total));
  const int stride = (int)std::max<int64_t>(1, total / want);
  std::vector<int64_t> soff(1, 0);
  std::vector<int> pick;
  for (int s = 0; s < nsets && soff.back() < want; s += stride) {
    pick.push_back(s);
    soff.push_back(soff.back() + offsets[s + 1] - offsets[s]);
  }
  const int ns = (int)pick.size();
  const int64_t npts = soff.back();
  double* d_sample = nullptr;
  uint2* d_uv = nullptr;
  const int64_t cap = (dim == 3 ? 10 : 4) * npts + 64;
  if (dalloc(&d_sample, (size_t)(npts * dim)) || dalloc(&d_uv, (size_t)cap)) {
    dfree(d_sample);
    return VD_ERR_NOMEM;
  }
  for (int i = 0; i < ns; ++i)
    cudaMemcpyAsync(d_sample + soff[i] * dim, d_pts + offsets[pick[i]] * dim,
                    sizeof(double) * (offsets[pick[i] + 1] - offsets[pick[i]]) * dim, cudaMemcpyDeviceToDevice,
                    t->stream);
  struct Cfg {
    int wps, bps, passes, thin, adjacent;
    double ratio;
  };
  std::vector<int64_t> eoff(ns + 1);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = VD_OK;
  auto apply = [&](const Cfg& c) {
    t->warps_per_sm = c.wps;
    t->blocks_per_sm = c.bps;
    t->tuning.passes = c.passes;
    t->tuning.thin = c.thin;
    t->tuning.adjacent = c.adjacent;
    t->ratio = c.ratio;
  };
  auto time_cfg = [&](const Cfg& c) -> double {
    apply(c);
    double best = 1e30;
    for (int rep = 0; rep < 2 && !rc; ++rep) {
      cudaEventRecord(e0, t->stream);
      int r = batch_reset_device(t, d_sample, soff.data(), ns);
      if (!r) r = insert_device(t, d_sample, npts, 0x5eedULL);  // one seed: the second run replays graphs
      if (r == VD_ERR_DUPLICATE) r = VD_OK;
      if (!r) r = batch_edges(t, d_uv, cap, eoff.data(), nullptr);
      cudaEventRecord(e1, t->stream);
      if (r) {
        rc = r;
        break;
      }
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, (double)ms);
    }
    return best;
  };
  Cfg best{t->warps_per_sm, t->blocks_per_sm, t->tuning.passes, t->tuning.thin, t->tuning.adjacent, t->ratio};
  double best_ms = time_cfg(best);
  // coordinate descent, one sweep per coordinate
  const int wps_c[] = {8, 12, 16, 20, 24, 28, 32};
  const int bps_c[] = {4, 8, 16};
  const int pass_c[] = {1, 2, 3};
  const int thin_c[] = {0, 1, 2};
  const double ratio_c[] = {0.06, 0.12, 0.25, 0.5};
  const int adj_c[] = {0, 1};
  auto sweep = [&](auto field, const auto& values) {
    for (const auto& v : values) {
      if (rc) return;
      Cfg c = best;
      field(c, v);
      const double ms = time_cfg(c);
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
  };
  sweep([](Cfg& c, int v) { c.adjacent = v; }, adj_c);
  sweep([](Cfg& c, double v) { c.ratio = v; }, ratio_c);
  sweep([](Cfg& c, int v) { c.passes = v; }, pass_c);
  sweep([](Cfg& c, int v) { c.thin = v; }, thin_c);
  sweep([](Cfg& c, int v) { c.wps = v; }, wps_c);
  sweep([](Cfg& c, int v) { c.bps = v; }, bps_c);
  apply(best);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(t->stream);
  dfree(d_sample);
  dfree(d_uv);
  if (out) {
    out[0] = best.wps;
    out[1] = best.bps;
    out[2] = best.passes;
    out[3] = best.thin;
    out[4] = (int64_t)(best.ratio * 1000.0 + 0.5);
    out[5] = (int64_t)(best_ms * 1000.0);
    out[6] = npts;
    out[7] = ns;
    out[8] = best.adjacent;
  }
  return rc;
}

int vd_locate_points(vd_tree* t, const double* pts, int64_t nq, int64_t* offsets, int64_t* ids, int64_t cap) {
  if (ready(t) || !t->has_geometry || t->nsets != 1 || nq < 0 || (nq > 0 && !pts) || !offsets) return VD_ERR_ARG;
  offsets[0] = 0;
  if (nq == 0) return VD_OK;
  int rc = sync_counters(t);
  if (rc) return rc;
  const int dim = t->dim;
  const int nsimp = t->hctr->nsimp;
  const vd::Launch L = launch_of(t);
  int *flags = nullptr, *rank = nullptr, *tmp = nullptr, *out = nullptr, *cnt = nullptr;
  double* dq = nullptr;
  const int64_t chunk = std::min<int64_t>(nq, 1 << 16);
  int cap_per = 256;
  if (dalloc(&flags, nsimp + 1) || dalloc(&rank, nsimp + 1) || dalloc(&tmp, vd::scan_scratch_ints(nsimp + 1)) ||
      dalloc(&dq, (size_t)(chunk * dim)) || dalloc(&cnt, chunk) || dalloc(&out, (size_t)(chunk * cap_per))) {
    rc = vd::E_NOMEM;
  }
  if (!rc) vd::launch_live_rank(t->T, L, nsimp, flags, rank, tmp);
  std::vector<int> hc(chunk), ho;
  bool outside = false;
  int64_t total = 0;
  for (int64_t q0 = 0; q0 < nq && !rc; q0 += chunk) {
    const int m = (int)std::min<int64_t>(chunk, nq - q0);
    cudaMemcpyAsync(dq, pts + q0 * dim, sizeof(double) * m * dim, cudaMemcpyHostToDevice, t->stream);
    vd::launch_locate(t->T, L, dim, dq, m, cap_per, rank, out, cnt);
    cudaMemcpyAsync(hc.data(), cnt, sizeof(int) * m, cudaMemcpyDeviceToHost, t->stream);
    if (cudaStreamSynchronize(t->stream) != cudaSuccess) {
      rc = vd::E_CUDA;
      break;
    }
    int need = 0;
    for (int i = 0; i < m; ++i) need = std::max(need, hc[i]);
    if (need > cap_per) {  // a region larger than the per-query room: rerun this chunk with enough
      cap_per = need;
      dfree(out);
      if (dalloc(&out, (size_t)m * cap_per)) {
        rc = vd::E_NOMEM;
        break;
      }
      vd::launch_locate(t->T, L, dim, dq, m, cap_per, rank, out, cnt);
      cudaMemcpyAsync(hc.data(), cnt, sizeof(int) * m, cudaMemcpyDeviceToHost, t->stream);
    }
    ho.resize((size_t)m * cap_per);
    cudaMemcpyAsync(ho.data(), out, sizeof(int) * ho.size(), cudaMemcpyDeviceToHost, t->stream);
    if (cudaStreamSynchronize(t->stream) != cudaSuccess) {
      rc = vd::E_CUDA;
      break;
    }
    for (int i = 0; i < m; ++i) {
      const int c = std::max(hc[i], 0);
      outside = outside || hc[i] < 0;
      offsets[q0 + i + 1] = offsets[q0 + i] + c;
      if (ids && total + c <= cap) {
        int64_t* dst = ids + total;
        for (int k = 0; k < c; ++k) dst[k] = ho[(size_t)i * cap_per + k];
        std::sort(dst, dst + c);
      }
      total += c;
    }
  }
  dfree(flags);
  dfree(rank);
  dfree(tmp);
  dfree(dq);
  dfree(cnt);
  dfree(out);
  if (rc) return rc;
  if (t->hctr->err) return t->hctr->err;
  if (ids && total > cap) return VD_ERR_ARG;
  return outside ? VD_ERR_OUTSIDE : VD_OK;
}

int vd_circumspheres(vd_tree* t, double* centers, double* radii, int64_t cap, int64_t* n) {
  if (ready(t) || !t->has_geometry || !n) return VD_ERR_ARG;
  int rc = sync_counters(t);
  if (rc) return rc;
  const int nsimp = t->hctr->nsimp;
  const vd::Launch L = launch_of(t);
  int *flags = nullptr, *rank = nullptr, *tmp = nullptr;
  if (dalloc(&flags, nsimp + 1) || dalloc(&rank, nsimp + 1) || dalloc(&tmp, vd::scan_scratch_ints(nsimp + 1))) {
    dfree(flags);
    dfree(rank);
    return VD_ERR_NOMEM;
  }
  vd::launch_live_rank(t->T, L, nsimp, flags, rank, tmp);
  int live = 0;
  cudaMemcpyAsync(&live, rank + nsimp, sizeof(int), cudaMemcpyDeviceToHost, t->stream);
  rc = cuda_status(cudaStreamSynchronize(t->stream));
  *n = live;
  if (!rc && (centers || radii)) {
    double *dc = nullptr, *dr = nullptr;
    if (cap < live || !centers || !radii) {
      rc = VD_ERR_ARG;
    } else if (dalloc(&dc, 3 * (size_t)live + 3) || dalloc(&dr, (size_t)live + 1)) {
      rc = VD_ERR_NOMEM;
    } else {
      vd::launch_circum(t->T, L, t->dim, nsimp, rank, dc, dr);
      cudaMemcpyAsync(centers, dc, sizeof(double) * 3 * live, cudaMemcpyDeviceToHost, t->stream);
      cudaMemcpyAsync(radii, dr, sizeof(double) * live, cudaMemcpyDeviceToHost, t->stream);
      rc = cuda_status(cudaStreamSynchronize(t->stream));
    }
    dfree(dc);
    dfree(dr);
  }
  dfree(flags);
  dfree(rank);
  dfree(tmp);
  return rc;
}

// Live ranks of the tree's slots (vd_simplices numbering): rank[s], and the
// live count.  The caller frees flags, rank and tmp.
int live_ranks(vd_tree* t, int** flags, int** rank, int** tmp, int* nsimp, int* live) {
  *flags = *rank = *tmp = nullptr;
  int rc = sync_counters(t);
  if (rc) return rc;
  *nsimp = t->hctr->nsimp;
  if (dalloc(flags, *nsimp + 1) || dalloc(rank, *nsimp + 1) || dalloc(tmp, vd::scan_scratch_ints(*nsimp + 1)))
    return VD_ERR_NOMEM;
  vd::launch_live_rank(t->T, launch_of(t), *nsimp, *flags, *rank, *tmp);
  cudaMemcpyAsync(t->h_pair, *rank + *nsimp, sizeof(int), cudaMemcpyDeviceToHost, t->stream);
  rc = cuda_status(cudaStreamSynchronize(t->stream));
  *live = t->h_pair[0];
  return rc;
}

int vd_voronoi_edges(vd_tree* t, int64_t* pairs, int64_t cap, int64_t* n) {
  if (ready(t) || !t->has_geometry || !n) return VD_ERR_ARG;
  int *flags, *rank, *tmp, nsimp = 0, live = 0;
  int rc = live_ranks(t, &flags, &rank, &tmp, &nsimp, &live);
  int *cnt = nullptr, *off = nullptr, *tmp2 = nullptr;
  int2* d_out = nullptr;
  const vd::Launch L = launch_of(t);
  if (!rc && (dalloc(&cnt, live + 1) || dalloc(&off, live + 1) || dalloc(&tmp2, vd::scan_scratch_ints(live + 1))))
    rc = VD_ERR_NOMEM;
  int total = 0;
  if (!rc) {
    vd::launch_dual_edges(t->T, L, t->dim, nsimp, rank, cnt, off, tmp2, live, nullptr, false);
    cudaMemcpyAsync(t->h_pair, off + live, sizeof(int), cudaMemcpyDeviceToHost, t->stream);
    rc = cuda_status(cudaStreamSynchronize(t->stream));
    total = t->h_pair[0];
    *n = total;
  }
  if (!rc && pairs) {
    if (cap < total) {
      rc = VD_ERR_ARG;
    } else if (dalloc(&d_out, (size_t)total + 1)) {
      rc = VD_ERR_NOMEM;
    } else {
      vd::launch_dual_edges(t->T, L, t->dim, nsimp, rank, cnt, off, tmp2, live, d_out, true);
      std::vector<int2> h(total);
      cudaMemcpyAsync(h.data(), d_out, sizeof(int2) * total, cudaMemcpyDeviceToHost, t->stream);
      rc = cuda_status(cudaStreamSynchronize(t->stream));
      for (int64_t i = 0; i < total && !rc; ++i) {
        pairs[2 * i] = h[i].x;
        pairs[2 * i + 1] = h[i].y;
      }
    }
  }
  dfree(d_out);
  dfree(cnt);
  dfree(off);
  dfree(tmp2);
  dfree(flags);
  dfree(rank);
  dfree(tmp);
  if (!rc && t->hctr->err) rc = t->hctr->err;
  return rc;
}

int vd_voronoi_cells(vd_tree* t, int64_t* offsets, int64_t* ids, int64_t cap) {
  if (ready(t) || !t->has_geometry || !offsets) return VD_ERR_ARG;
  int *flags, *rank, *tmp, nsimp = 0, live = 0;
  int rc = live_ranks(t, &flags, &rank, &tmp, &nsimp, &live);
  const int n_in = (int)(t->nverts - t->ns);
  int *cnt = nullptr, *off = nullptr, *tmp2 = nullptr, *buf = nullptr, *ucnt = nullptr, *big = nullptr,
      *nbig = nullptr;
  const vd::Launch L = launch_of(t);
  if (!rc && (dalloc(&cnt, n_in + 2) || dalloc(&off, n_in + 2) || dalloc(&tmp2, vd::scan_scratch_ints(n_in + 2))))
    rc = VD_ERR_NOMEM;
  int total = 0;
  std::vector<int> hoff;
  if (!rc) {
    vd::launch_cell_count(t->T, L, t->dim, nsimp, n_in, cnt, off, tmp2);
    hoff.resize(n_in + 1);
    cudaMemcpyAsync(hoff.data(), off, sizeof(int) * (n_in + 1), cudaMemcpyDeviceToHost, t->stream);
    rc = cuda_status(cudaStreamSynchronize(t->stream));
    total = hoff[n_in];
    for (int i = 0; i <= n_in; ++i) offsets[i] = hoff[i];
  }
  if (!rc && ids) {
    if (cap < total) {
      rc = VD_ERR_ARG;
    } else if (dalloc(&buf, (size_t)total + 1) || dalloc(&ucnt, n_in + 1) || dalloc(&big, n_in + 1) ||
               dalloc(&nbig, 1)) {
      rc = VD_ERR_NOMEM;
    } else {
      vd::launch_cell_fill(t->T, L, t->dim, nsimp, n_in, rank, cnt, off, buf);
      if (vd::sort_buckets(L, n_in, off, buf, ucnt, big, nbig, t->d_pair, t->h_pair) != 0) rc = VD_ERR_CUDA;
      if (!rc) {
        std::vector<int> h(total);
        cudaMemcpyAsync(h.data(), buf, sizeof(int) * total, cudaMemcpyDeviceToHost, t->stream);
        rc = cuda_status(cudaStreamSynchronize(t->stream));
        for (int64_t i = 0; i < total && !rc; ++i) ids[i] = h[i];
      }
    }
  }
  dfree(buf);
  dfree(ucnt);
  dfree(big);
  dfree(nbig);
  dfree(cnt);
  dfree(off);
  dfree(tmp2);
  dfree(flags);
  dfree(rank);
  dfree(tmp);
  if (!rc && t->hctr->err) rc = t->hctr->err;
  return rc;
}

int vd_locate(vd_tree* t, const double* p, int64_t* out, int64_t cap, int64_t* n) {
  if (!n) return VD_ERR_ARG;
  int64_t off[2] = {0, 0};
  int rc = vd_locate_points(t, p, 1, off, nullptr, 0);
  *n = off[1];
  if (rc || !out) return rc;
  if (cap < off[1]) return VD_ERR_ARG;
  return vd_locate_points(t, p, 1, off, out, cap);
}

}  // extern "C"
