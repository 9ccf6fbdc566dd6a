// serve.cpp -- the ZI serving loop of libmczi_gpu (mczi_serve_* in mczi_gpu.h).
//
// No counterpart exists in the reference (ZI answers one query set per process,
// src/zi.rs:64-101).  Host threads only: every device step goes through the
// public entry points of this library (mczi_zi_build, mczi_zi_query_per_input,
// mczi_zi_batch_split), one context per worker.
#include "mczi_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

// device bytes per query byte during a batch: text, 2-bit stream, fragment
// bits, superkmer descriptors (double-buffered) and keys, absent runs
constexpr double HBM_BYTES_PER_QUERY_BYTE = 8.0;

// Pinned host blocks for batch results, reused across batches: the absent
// sets of a batch (hundreds of MB at full load) reach the host at the link's
// speed only in pinned memory, and a fresh pageable allocation per batch
// costs a page fault per 4 KiB on first touch.  A block returns to the pool
// when the last request of its batch has been copied out; the pool keeps at
// most POOL_MAX_BYTES of free blocks.
class PinnedPool {
 public:
  static constexpr size_t POOL_MAX_BYTES = 16ull << 30;
  ~PinnedPool() {
    for (auto& b : free_) cudaFreeHost(b.first);
  }
  // a block of at least `bytes`, or nullptr when pinned memory is exhausted
  void* get(size_t bytes, size_t* cap) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      size_t best = free_.size();
      for (size_t i = 0; i < free_.size(); i++)
        if (free_[i].second >= bytes && (best == free_.size() || free_[i].second < free_[best].second)) best = i;
      if (best < free_.size()) {
        void* p = free_[best].first;
        *cap = free_[best].second;
        cached_ -= *cap;
        free_.erase(free_.begin() + (long)best);
        return p;
      }
    }
    const size_t want = bytes + bytes / 4;  // room for a slightly larger batch next time
    void* p = nullptr;
    if (cudaHostAlloc(&p, want, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    *cap = want;
    return p;
  }
  void put(void* p, size_t cap) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (cached_ + cap <= POOL_MAX_BYTES) {
        free_.emplace_back(p, cap);
        cached_ += cap;
        return;
      }
    }
    cudaFreeHost(p);
  }

 private:
  std::mutex mu_;
  std::vector<std::pair<void*, size_t>> free_;
  size_t cached_ = 0;
};

// one batch's absent sets, split per request on the device and copied to
// the host once into a pinned block; requests keep a range of it
struct BatchResult {
  std::shared_ptr<PinnedPool> pool;
  void* block = nullptr;
  size_t cap = 0;
  uint64_t* lo = nullptr;
  uint64_t* hi = nullptr;
  std::unique_ptr<uint64_t[]> heap;  // when pinned memory ran out
  ~BatchResult() {
    if (block) pool->put(block, cap);
  }
};

struct ServeRequest {
  uint64_t id = 0;
  const uint8_t* data = nullptr;
  uint64_t len = 0;
  Clock::time_point arrival, started, finished;
  int32_t status = MCZI_OK;
  std::string error;
  std::shared_ptr<BatchResult> res;
  uint64_t off = 0, cnt = 0;
};

thread_local std::string open_error;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct mczi_server {
  int32_t device = 0;
  uint32_t k = 0;
  int32_t max_batch = 1;
  uint64_t per_worker_bytes = 0;
  std::vector<mczi_ctx*> ctxs;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ServeRequest*> queue;
  std::deque<uint64_t> done;
  std::unordered_map<uint64_t, std::unique_ptr<ServeRequest>> reqs;
  uint64_t next_id = 1;
  bool stop = false;
  uint64_t batches = 0, answered = 0, largest = 0;
  double t_query = 0.0, t_results = 0.0;
  std::shared_ptr<PinnedPool> pool = std::make_shared<PinnedPool>();
};

namespace {

// every waiting request that fits: at most max_batch of them and at most the
// worker's share of device memory (the first one is taken whatever its size)
std::vector<ServeRequest*> take_batch(mczi_server* S) {
  std::vector<ServeRequest*> batch;
  uint64_t bytes = 0;
  while (!S->queue.empty() && (int32_t)batch.size() < S->max_batch) {
    const uint64_t n = S->queue.front()->len;
    if (!batch.empty() && bytes + n > S->per_worker_bytes) break;
    batch.push_back(S->queue.front());
    S->queue.pop_front();
    bytes += n;
  }
  return batch;
}

void answer(mczi_server* S, mczi_ctx* ctx, const std::vector<ServeRequest*>& batch) {
  const size_t n = batch.size();
  std::vector<mczi_input> in(n);
  for (size_t i = 0; i < n; i++) in[i] = mczi_input{batch[i]->data, batch[i]->len};
  const Clock::time_point t0 = Clock::now();
  uint64_t records = 0, total = 0;
  std::vector<uint64_t> offs(n + 1, 0);
  auto br = std::make_shared<BatchResult>();
  br->pool = S->pool;
  int32_t rc = mczi_zi_query_per_input(ctx, in.data(), n, &records);
  const Clock::time_point tq = Clock::now();
  if (rc == MCZI_OK) rc = mczi_zi_batch_split(ctx, nullptr, nullptr, offs.data(), 0, &total);
  if (rc == MCZI_OK && total > 0) {
    const size_t words = (size_t)total * (S->k > 32 ? 2 : 1);
    br->block = S->pool->get(words * 8, &br->cap);
    if (br->block) {
      br->lo = static_cast<uint64_t*>(br->block);
    } else {
      br->heap.reset(new uint64_t[words]);
      br->lo = br->heap.get();
    }
    if (S->k > 32) br->hi = br->lo + total;
    rc = mczi_zi_batch_split(ctx, br->lo, br->hi, offs.data(), total, &total);
  }
  const std::string err = rc == MCZI_OK ? std::string() : std::string(mczi_last_error(ctx));
  for (size_t i = 0; i < n; i++) {
    ServeRequest* r = batch[i];
    r->status = rc;
    if (rc != MCZI_OK) {
      r->error = err;
      continue;
    }
    r->res = br;
    r->off = offs[i];
    r->cnt = offs[i + 1] - offs[i];
  }
  const Clock::time_point t1 = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->batches++;
    S->answered += n;
    S->largest = std::max<uint64_t>(S->largest, n);
    S->t_query += std::chrono::duration<double>(tq - t0).count();
    S->t_results += std::chrono::duration<double>(t1 - tq).count();
    for (ServeRequest* r : batch) {
      r->finished = t1;
      S->done.push_back(r->id);
    }
  }
  S->cv_done.notify_all();
}

void worker(mczi_server* S, mczi_ctx* ctx) {
  for (;;) {
    std::vector<ServeRequest*> batch;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [S] { return S->stop || !S->queue.empty(); });
      if (S->queue.empty()) return;  // stopping, nothing left
      batch = take_batch(S);
    }
    const Clock::time_point t = Clock::now();
    for (ServeRequest* r : batch) r->started = t;
    answer(S, ctx, batch);
  }
}

void destroy(mczi_server* S) {
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (std::thread& t : S->threads) t.join();
  for (mczi_ctx* c : S->ctxs) mczi_close(c);
  delete S;
}

}  // namespace

extern "C" {

int32_t mczi_serve_open(int32_t device, const uint8_t* index_fasta, uint64_t len, uint32_t k, uint32_t m,
                        int32_t workers, int32_t max_batch, uint64_t hbm_budget, mczi_server** out) {
  if (!out) return MCZI_ERR_STATE;
  *out = nullptr;
  open_error.clear();
  if (workers < 1 || workers > 64) {
    open_error = "workers must be in [1, 64]";
    return MCZI_ERR_INVALID_CONFIG;
  }
  if (max_batch < 1 || max_batch > 4096) {
    open_error = "max_batch must be in [1, 4096]";
    return MCZI_ERR_INVALID_CONFIG;
  }
  mczi_server* S = new mczi_server();
  S->device = device;
  S->k = k;
  S->max_batch = max_batch;
  for (int32_t w = 0; w < workers; w++) {
    mczi_ctx* c = nullptr;
    int32_t rc = mczi_open(device, &c);
    if (rc == MCZI_OK) {
      S->ctxs.push_back(c);
      rc = mczi_zi_build(c, index_fasta, len, k, m);
      if (rc != MCZI_OK) open_error = mczi_last_error(c);
    } else {
      open_error = "no usable CUDA device";
    }
    if (rc != MCZI_OK) {
      destroy(S);
      return rc;
    }
  }
  if (hbm_budget == 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaSetDevice(device) != cudaSuccess || cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      free_b = 8ull << 30;
    }
    hbm_budget = (uint64_t)(0.6 * (double)free_b);
  }
  S->per_worker_bytes =
      std::max<uint64_t>(1ull << 20, (uint64_t)((double)hbm_budget / workers / HBM_BYTES_PER_QUERY_BYTE));
  for (mczi_ctx* c : S->ctxs) S->threads.emplace_back(worker, S, c);
  *out = S;
  return MCZI_OK;
}

int32_t mczi_serve_submit(mczi_server* S, const uint8_t* query_fasta, uint64_t len, uint64_t* request_id) {
  if (!S || !request_id) return MCZI_ERR_STATE;
  auto r = std::make_unique<ServeRequest>();
  r->data = query_fasta;
  r->len = query_fasta ? len : 0;
  r->arrival = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return MCZI_ERR_STATE;
    r->id = S->next_id++;
    *request_id = r->id;
    S->queue.push_back(r.get());
    S->reqs.emplace(r->id, std::move(r));
  }
  S->cv_work.notify_one();
  return MCZI_OK;
}

int32_t mczi_serve_next(mczi_server* S, int32_t timeout_ms, uint64_t* request_id, int32_t* status,
                        uint64_t* n_kmers, double* latency_ms, double* queue_ms) {
  if (!S || !request_id) return MCZI_ERR_STATE;
  std::unique_lock<std::mutex> lk(S->mu);
  auto ready = [S] { return !S->done.empty(); };
  if (timeout_ms < 0) S->cv_done.wait(lk, ready);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return MCZI_ERR_TIMEOUT;
  const uint64_t id = S->done.front();
  S->done.pop_front();
  const ServeRequest* r = S->reqs.at(id).get();
  *request_id = id;
  if (status) *status = r->status;
  if (n_kmers) *n_kmers = r->cnt;
  if (latency_ms) *latency_ms = ms_between(r->arrival, r->finished);
  if (queue_ms) *queue_ms = ms_between(r->arrival, r->started);
  return MCZI_OK;
}

int32_t mczi_serve_result(mczi_server* S, uint64_t request_id, uint64_t* key_lo, uint64_t* key_hi, uint64_t cap,
                          uint64_t* n) {
  if (!S) return MCZI_ERR_STATE;
  std::unique_ptr<ServeRequest> r;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(request_id);
    if (it == S->reqs.end() || it->second->finished == Clock::time_point()) return MCZI_ERR_STATE;
    const ServeRequest* q = it->second.get();
    if (q->status != MCZI_OK) {
      const int32_t st = q->status;
      if (key_lo) S->reqs.erase(it);
      return st;
    }
    if (n) *n = q->cnt;
    if (!key_lo) return MCZI_OK;
    if (cap < q->cnt) return MCZI_ERR_INVALID_CONFIG;
    r = std::move(it->second);  // released here; copied below without the lock
    S->reqs.erase(it);
  }
  const uint64_t cnt = r->cnt;
  if (cnt) std::memcpy(key_lo, r->res->lo + r->off, cnt * 8);
  if (key_hi && cnt) {
    if (!r->res->hi) std::memset(key_hi, 0, cnt * 8);
    else std::memcpy(key_hi, r->res->hi + r->off, cnt * 8);
  }
  return MCZI_OK;  // the batch's buffer goes with its last request
}

int32_t mczi_serve_release(mczi_server* S, uint64_t request_id) {
  if (!S) return MCZI_ERR_STATE;
  std::unique_ptr<ServeRequest> r;  // destroyed after the lock is dropped
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(request_id);
  if (it == S->reqs.end() || it->second->finished == Clock::time_point()) return MCZI_ERR_STATE;
  const int32_t st = it->second->status;
  r = std::move(it->second);
  S->reqs.erase(it);
  return st;
}

const char* mczi_serve_error(mczi_server* S, uint64_t request_id) {
  if (!S) return open_error.c_str();
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(request_id);
  if (it == S->reqs.end()) return "no such request";
  return it->second->error.c_str();
}

int32_t mczi_serve_stats(mczi_server* S, double* out, int32_t cap) {
  if (!S || !out) return MCZI_ERR_STATE;
  std::lock_guard<std::mutex> lk(S->mu);
  const double v[7] = {(double)S->batches, (double)S->answered, (double)S->largest, S->t_query, S->t_results,
                       (double)S->queue.size(), (double)S->per_worker_bytes};
  const int32_t n = std::min<int32_t>(cap, 7);
  for (int32_t i = 0; i < n; i++) out[i] = v[i];
  return n;
}

int32_t mczi_serve_close(mczi_server* S) {
  if (!S) return MCZI_ERR_STATE;
  destroy(S);
  return MCZI_OK;
}

}  // extern "C"
