// Serving loop: continuous batching of triangulation requests.
//
// No counterpart in the reference (it triangulates one point set per call,
// src/lib.rs:104-125).  Requests of mixed size and dimension are queued on
// submission; each of `slots` workers (one host thread, one CUDA stream and
// one reusable tree per dimension each) repeatedly forms a batch from the
// queue of the dimension whose oldest request waited longest, admits it
// against the device-memory budget by estimated pool bytes, and runs it as one
// batched build (vd_batch_delaunay).  Requests that arrive while batches run
// are admitted as soon as a slot and budget free up, and the batches of
// different slots overlap on the device.  Every result is the triangulation
// of the request alone (batched builds are exact per set).
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/voronoids_gpu.h"

namespace {

// Estimated device bytes of a request, with 1.5x slack: simplex slots (3D
// 7.6, 2D 2.3 per point, 92 B each: record, claims, marks, star links) and
// per-point records, work lists and edge scratch (about 520 B in 3D, 250 B
// in 2D).
int64_t estimate_bytes(int dim, int64_t n) { return (dim == 3 ? 1850 : 700) * std::max<int64_t>(n, 1) + 4096; }

struct Request {
  int64_t id;
  int dim;
  std::vector<double> pts;
  int64_t n;
  int64_t bytes;
  int status = VD_OK;
  std::vector<uint32_t> uv;  // 2 per edge
};

}  // namespace

struct vd_server {
  uint64_t budget = 0;
  int64_t max_batch_points = 0;
  uint64_t seed = 0;
  std::mutex mu;
  std::condition_variable cv_work;   // workers: new requests or freed budget
  std::condition_variable cv_done;   // pollers: finished requests
  std::deque<std::unique_ptr<Request>> queue[2];  // by dimension (2D, 3D)
  std::unordered_map<int64_t, std::unique_ptr<Request>> finished;
  std::vector<int64_t> done_ids;
  uint64_t reserved = 0;
  int64_t next_id = 0;
  bool stop = false;
  int64_t n_batches = 0, n_done = 0, n_submitted = 0, n_isolated = 0;
  uint64_t peak_reserved = 0;
  std::vector<std::thread> workers;
  int device = 0;
};

namespace {

struct Slot {
  cudaStream_t stream = nullptr;
  vd_tree* tree[2] = {nullptr, nullptr};
  std::vector<double> pts;
  std::vector<int64_t> off, eoff;
  std::vector<uint32_t> uv;
};

// Runs one batch on the slot; fills each request's result.
void run_batch(vd_server* s, Slot& sl, int dim, std::vector<std::unique_ptr<Request>>& batch) {
  vd_tree*& t = sl.tree[dim - 2];
  if (!t) {
    int st = VD_OK;
    t = vd_tree_create(dim, sl.stream, &st);
    if (!t || st != VD_OK) {
      for (auto& r : batch) r->status = t ? st : VD_ERR_NOMEM;
      return;
    }
  }
  const int nsets = (int)batch.size();
  sl.off.assign(nsets + 1, 0);
  for (int i = 0; i < nsets; ++i) sl.off[i + 1] = sl.off[i] + batch[i]->n;
  sl.pts.resize((size_t)sl.off[nsets] * dim);
  for (int i = 0; i < nsets; ++i)
    memcpy(sl.pts.data() + (size_t)sl.off[i] * dim, batch[i]->pts.data(), sizeof(double) * batch[i]->n * dim);
  sl.eoff.assign(nsets + 1, 0);
  int64_t cap = (dim == 3 ? 10 : 4) * sl.off[nsets] + 64;
  int rc = VD_OK;
  for (int attempt = 0; attempt < 2; ++attempt) {
    sl.uv.resize((size_t)cap * 2);
    rc = vd_batch_delaunay(t, sl.pts.data(), sl.off.data(), nsets, s->seed, sl.uv.data(), cap, sl.eoff.data());
    if (rc == VD_ERR_ARG && sl.eoff[nsets] > cap) {  // more edges than the first guess
      cap = sl.eoff[nsets];
      continue;
    }
    break;
  }
  if (rc == VD_OK || rc == VD_ERR_DUPLICATE) {
    for (int i = 0; i < nsets; ++i) {
      batch[i]->uv.assign(sl.uv.begin() + 2 * sl.eoff[i], sl.uv.begin() + 2 * sl.eoff[i + 1]);
      batch[i]->status = VD_OK;
    }
    return;
  }
  if (nsets == 1) {
    batch[0]->status = rc;
    return;
  }
  // one request broke the batch (a degenerate set, a bad coordinate): run
  // each alone so that the others still get their results
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->n_isolated += nsets;
  }
  for (auto& r : batch) {
    std::vector<std::unique_ptr<Request>> one;
    one.push_back(std::move(r));
    run_batch(s, sl, dim, one);
    r = std::move(one[0]);
  }
}

void worker(vd_server* s) {
  cudaSetDevice(s->device);
  Slot sl;
  if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess) sl.stream = nullptr;
  while (true) {
    std::vector<std::unique_ptr<Request>> batch;
    int dim = 3;
    uint64_t bytes = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      while (true) {
        if (s->stop && s->queue[0].empty() && s->queue[1].empty()) break;
        // dimension of the oldest waiting request
        int q = -1;
        for (int k = 0; k < 2; ++k)
          if (!s->queue[k].empty() && (q < 0 || s->queue[k].front()->id < s->queue[q].front()->id)) q = k;
        if (q >= 0) {
          auto& Q = s->queue[q];
          const uint64_t head = (uint64_t)Q.front()->bytes;
          if (head > s->budget) {  // can never be admitted
            auto r = std::move(Q.front());
            Q.pop_front();
            r->status = VD_ERR_NOMEM;
            s->done_ids.push_back(r->id);
            s->finished.emplace(r->id, std::move(r));
            ++s->n_done;
            s->cv_done.notify_all();
            continue;
          }
          if (s->reserved + head <= s->budget) {
            int64_t pts = 0;
            while (!Q.empty()) {
              Request* r = Q.front().get();
              const bool room = s->reserved + bytes + (uint64_t)r->bytes <= s->budget;
              const bool fits = batch.empty() || s->max_batch_points <= 0 || pts + r->n <= s->max_batch_points;
              if (!room || !fits) break;
              pts += r->n;
              bytes += (uint64_t)r->bytes;
              batch.push_back(std::move(Q.front()));
              Q.pop_front();
            }
            dim = q + 2;
            s->reserved += bytes;
            s->peak_reserved = std::max(s->peak_reserved, s->reserved);
            ++s->n_batches;
            break;
          }
        }
        s->cv_work.wait(lk);
      }
      if (batch.empty()) break;  // stopping, nothing left
    }
    run_batch(s, sl, dim, batch);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->reserved -= bytes;
      for (auto& r : batch) {
        s->done_ids.push_back(r->id);
        ++s->n_done;
        r->pts.clear();
        r->pts.shrink_to_fit();
        s->finished.emplace(r->id, std::move(r));
      }
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
  for (auto*& t : sl.tree)
    if (t) vd_tree_free(t);
  if (sl.stream) cudaStreamDestroy(sl.stream);
}

}  // namespace

extern "C" {

vd_server* vd_server_new(uint64_t pool_bytes, int slots, int64_t max_batch_points, uint64_t seed, int* status) {
  if (slots < 1 || slots > 64 || pool_bytes == 0) {
    if (status) *status = VD_ERR_ARG;
    return nullptr;
  }
  vd_server* s = new (std::nothrow) vd_server();
  if (!s) {
    if (status) *status = VD_ERR_NOMEM;
    return nullptr;
  }
  s->budget = pool_bytes;
  s->max_batch_points = max_batch_points;
  s->seed = seed;
  if (cudaGetDevice(&s->device) != cudaSuccess) {
    delete s;
    if (status) *status = VD_ERR_CUDA;
    return nullptr;
  }
  for (int i = 0; i < slots; ++i) s->workers.emplace_back(worker, s);
  if (status) *status = VD_OK;
  return s;
}

int vd_server_submit(vd_server* s, int dim, const double* pts, int64_t n, int64_t* id) {
  if (!s || (dim != 2 && dim != 3) || n < 1 || !pts || !id) return VD_ERR_ARG;
  auto r = std::unique_ptr<Request>(new (std::nothrow) Request());
  if (!r) return VD_ERR_NOMEM;
  r->dim = dim;
  r->n = n;
  r->bytes = estimate_bytes(dim, n);
  r->pts.assign(pts, pts + n * dim);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return VD_ERR_ARG;
    r->id = s->next_id++;
    *id = r->id;
    ++s->n_submitted;
    s->queue[dim - 2].push_back(std::move(r));
  }
  s->cv_work.notify_one();
  return VD_OK;
}

int vd_server_poll(vd_server* s, int64_t* ids, int64_t cap, int64_t* n, int timeout_ms) {
  if (!s || !n || (cap > 0 && !ids)) return VD_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done_ids.empty() && timeout_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !s->done_ids.empty(); });
  const int64_t k = std::min<int64_t>(cap, (int64_t)s->done_ids.size());
  for (int64_t i = 0; i < k; ++i) ids[i] = s->done_ids[i];
  s->done_ids.erase(s->done_ids.begin(), s->done_ids.begin() + k);
  *n = k;
  return VD_OK;
}

int vd_server_result(vd_server* s, int64_t id, uint32_t* uv, int64_t cap, int64_t* n_edges, int* req_status) {
  if (!s || !n_edges) return VD_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->finished.find(id);
  if (it == s->finished.end()) return VD_ERR_ARG;
  Request& r = *it->second;
  *n_edges = (int64_t)r.uv.size() / 2;
  if (req_status) *req_status = r.status;
  if (!uv) return VD_OK;
  if (cap < *n_edges) return VD_ERR_ARG;
  memcpy(uv, r.uv.data(), sizeof(uint32_t) * r.uv.size());
  s->finished.erase(it);
  return VD_OK;
}

int vd_server_stats(vd_server* s, int64_t* out) {
  if (!s || !out) return VD_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  out[0] = s->n_submitted;
  out[1] = s->n_done;
  out[2] = s->n_batches;
  out[3] = (int64_t)s->reserved;
  out[4] = (int64_t)s->peak_reserved;
  out[5] = (int64_t)(s->queue[0].size() + s->queue[1].size());
  out[6] = s->n_isolated;
  out[7] = (int64_t)s->budget;
  return VD_OK;
}

void vd_server_free(vd_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& w : s->workers) w.join();
  delete s;
}

}  // extern "C"
