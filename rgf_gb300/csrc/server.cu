// Request loop: continuous batching of factorize / solve / RGFdiag requests
// on one GPU with factors kept resident.
//
// `slots` worker threads each own a CUDA stream (through the handles they
// drive); a request is admitted as soon as a worker is free and, for a new
// factorization, its HBM footprint fits the budget (least-recently-used idle
// factors are evicted to make room).  Admitted requests run concurrently on
// their own streams, so work that arrives while other requests are on the GPU
// overlaps with them.  Every kernel is the same as in the one-instance API,
// so a result does not depend on what else runs at the same time.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/rgf.h"
#include "rgf_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Factor {
  rgf_handle* h = nullptr;
  size_t bytes = 0;
  bool busy = false;
  int pending = 0;  // queued solve / diag requests that name this factor
  Clock::time_point last_use;
};

struct Pending {
  rgf_request* req;
  long long ticket;
  Clock::time_point t_submit;
  bool pinned;  // holds one `pending` reference on its factor
};

size_t estimate_bytes(const rgf_opts& o, size_t ns, size_t nt, size_t nd, size_t nnz) {
  const size_t n = ns * nt + nd;
  const size_t mf = 2 * (nt - 1) * ns * ns + ns * ns + n * nd;
  size_t b = 16 * nnz + 8 * (n + 1) + 8 * mf;       // CSC + factor
  b += 8 * mf + 8 * (nt * ns * ns + nd * nd) + 8 * (2 * ns * ns + nd * ns);  // selected inverse
  // split-K workspaces of the main and side streams
  b += 2 * 8 * std::min<size_t>(20u << 20, 8 * (2 * ns + nd) * std::max(ns, nd));
  if (o.precision == RGF_PREC_SPLIT) {  // slice workspaces of the main and side streams
    const size_t r = (2 * ns + nd + 127) / 128 * 128, k = (ns + nd + 63) / 64 * 64;
    const size_t one = 2 * 8 * r * k * 2;
    b += std::max(one, std::min<size_t>((size_t)1 << 30, nt * one / 4)) + (1 << 20);
    const size_t r2 = (ns + nd + 127) / 128 * 128;
    b += 2 * 8 * r2 * k * 2 + (1 << 20);
    b += 2 * (80 * 128 * 128 * 8 + 4096);  // split-K partial sums of both engines
  }
  return b + (8u << 20);
}

}  // namespace

struct rgf_server {
  rgf_opts opts{};
  size_t budget = 0, used = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> queue;
  std::map<long long, Factor> factors;
  std::map<long long, int> done;  // ticket -> status (completed, not yet waited)
  long long next_ticket = 1, next_factor = 1;
  bool stop = false;
  std::vector<std::thread> workers;
  rgf_server_stats_t stats{};
  rgf::DeviceArena* arena = nullptr;  // the HBM budget, reserved once
  int device = 0;
};

namespace {

// Evict least-recently-used idle factors until `need` more bytes fit.  A
// factor that a queued request names is not idle: it stays resident until
// that request has run.
bool make_room(rgf_server* s, size_t need) {
  while (s->used + need > s->budget) {
    long long victim = 0;
    Clock::time_point oldest = Clock::time_point::max();
    for (auto& kv : s->factors)
      if (!kv.second.busy && kv.second.pending == 0 && kv.second.last_use < oldest) {
        oldest = kv.second.last_use;
        victim = kv.first;
      }
    if (!victim) return false;
    Factor f = s->factors[victim];
    s->factors.erase(victim);
    s->used -= f.bytes;
    s->stats.evicted++;
    rgf_destroy(f.h);
  }
  return true;
}

// Index in the queue of the first request that can start now (FIFO among the
// admissible ones), or -1.  Reserves what it needs.
long admit(rgf_server* s) {
  for (size_t i = 0; i < s->queue.size(); ++i) {
    rgf_request* r = s->queue[i].req;
    if (r->kind == RGF_REQ_FACTOR) {
      const size_t n = r->ns * r->nt + r->nd;
      const size_t need = estimate_bytes(s->opts, r->ns, r->nt, r->nd, r->ia ? r->ia[n] : 0);
      if (need > s->budget) return (long)i;  // can never fit: fail it
      if (!make_room(s, need)) continue;
      s->used += need;
      r->reserved_bytes = need;
      return (long)i;
    }
    auto it = s->factors.find(r->factor_id);
    if (it == s->factors.end()) return (long)i;  // unknown or evicted: fail it
    if (it->second.busy) continue;
    it->second.busy = true;
    return (long)i;
  }
  return -1;
}

void run_request(rgf_server* s, Pending p) {
  rgf_request* r = p.req;
  int st = RGF_OK;
  if (r->kind == RGF_REQ_FACTOR) {
    const size_t n = r->ns * r->nt + r->nd;
    if (!r->ia || r->reserved_bytes == 0 || r->reserved_bytes > s->budget) {
      st = r->ia ? RGF_ENOMEM : RGF_EINVAL;
    } else {
      rgf_handle* h = nullptr;
      // The server's opts decide the upload (synchronous by default).  The
      // request's arrays stay valid until it is done, so async_upload is
      // allowed, but it measured slower here: 8 slots of concurrent requests
      // from pageable host arrays, ns up to 1500, served 17 req/s with the
      // block-column chunked upload against 47 req/s with one copy each.
      st = rgf_create(r->ia, r->ja, r->a, r->ns, r->nt, r->nd, &s->opts, &h);
      if (!st) st = rgf_factorize(h);
      if (!st) st = rgf_logdet(h, &r->logdet);
      std::lock_guard<std::mutex> lk(s->mu);
      if (!st) {
        Factor f;
        f.h = h;
        f.bytes = r->reserved_bytes;
        f.last_use = Clock::now();
        r->factor_id = s->next_factor++;
        s->factors[r->factor_id] = f;
      } else {
        if (h) rgf_destroy(h);
        s->used -= r->reserved_bytes;
      }
      (void)n;
    }
  } else {
    rgf_handle* h = nullptr;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      auto it = s->factors.find(r->factor_id);
      if (it == s->factors.end() || !it->second.busy) st = RGF_EINVAL;
      else h = it->second.h;
    }
    if (!st) {
      if (r->kind == RGF_REQ_SOLVE) st = rgf_solve(h, r->x, r->b, r->nrhs);
      else if (r->kind == RGF_REQ_DIAG) st = rgf_diag(h, r->diag);
      else if (r->kind == RGF_REQ_RELEASE) st = RGF_OK;
      else st = RGF_EINVAL;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->factors.find(r->factor_id);
    if (it != s->factors.end()) {
      if (p.pinned) it->second.pending--;
      if (r->kind == RGF_REQ_RELEASE && !st) {
        s->used -= it->second.bytes;
        rgf_destroy(it->second.h);
        s->factors.erase(it);
      } else {
        it->second.busy = false;
        it->second.last_use = Clock::now();
      }
    }
  }
  const double ms =
      std::chrono::duration<double, std::milli>(Clock::now() - p.t_submit).count();
  std::lock_guard<std::mutex> lk(s->mu);
  r->status = st;
  r->latency_ms = ms;
  s->stats.completed++;
  if (st) s->stats.failed++;
  s->done[p.ticket] = st;
  s->cv_done.notify_all();
  s->cv_work.notify_all();  // a factor became idle or memory was freed
}

void worker(rgf_server* s) {
  cudaSetDevice(s->device);
  rgf::set_thread_arena(s->arena);  // this thread's device memory comes from the arena
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    long i = -1;
    while (!s->stop && (i = admit(s)) < 0) s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
    if (s->stop && i < 0) return;
    Pending p = s->queue[i];
    s->queue.erase(s->queue.begin() + i);
    s->stats.admitted++;
    if (p.pinned && p.req->kind != RGF_REQ_FACTOR && !s->factors.count(p.req->factor_id))
      p.pinned = false;  // released before this request ran
    lk.unlock();
    run_request(s, p);
    lk.lock();
  }
}

}  // namespace

extern "C" {

int rgf_server_create(const rgf_opts* opts, size_t hbm_budget_bytes, int slots,
                      rgf_server** out) {
  if (!out || slots < 1 || slots > 256 || hbm_budget_bytes == 0) return RGF_EINVAL;
  rgf_server* s = new (std::nothrow) rgf_server();
  if (!s) return RGF_ENOMEM;
  rgf_default_opts(&s->opts);
  if (opts) s->opts = *opts;
  s->budget = hbm_budget_bytes;
  int dev = s->opts.device;
  if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) {
    delete s;
    return RGF_ECUDA;
  }
  if (cudaSetDevice(dev) != cudaSuccess) {
    delete s;
    return RGF_ECUDA;
  }
  s->device = dev;
  int st = RGF_OK;
  s->arena = rgf::arena_create(hbm_budget_bytes, &st);
  if (st) {
    delete s;
    return st;
  }
  for (int i = 0; i < slots; ++i) s->workers.emplace_back(worker, s);
  *out = s;
  return RGF_OK;
}

int rgf_server_submit(rgf_server* s, rgf_request* r, long long* ticket) {
  if (!s || !r || !ticket) return RGF_EINVAL;
  if (r->kind < RGF_REQ_FACTOR || r->kind > RGF_REQ_RELEASE) return RGF_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  r->status = -1;
  r->latency_ms = 0.0;
  r->reserved_bytes = 0;
  *ticket = s->next_ticket++;
  bool pinned = false;
  if (r->kind != RGF_REQ_FACTOR) {
    auto it = s->factors.find(r->factor_id);
    if (it != s->factors.end()) {
      it->second.pending++;
      pinned = true;
    }
  }
  s->queue.push_back({r, *ticket, Clock::now(), pinned});
  s->stats.submitted++;
  s->cv_work.notify_one();
  return RGF_OK;
}

int rgf_server_wait(rgf_server* s, long long ticket, double timeout_s, int* status) {
  if (!s) return RGF_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                           std::chrono::duration<double>(timeout_s));
  while (s->done.find(ticket) == s->done.end()) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout &&
        s->done.find(ticket) == s->done.end())
      return RGF_ETIMEOUT;
  }
  if (status) *status = s->done[ticket];
  s->done.erase(ticket);
  return RGF_OK;
}

int rgf_server_stats(rgf_server* s, rgf_server_stats_t* out) {
  if (!s || !out) return RGF_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->resident_factors = (long long)s->factors.size();
  out->used_bytes = s->used;
  out->queued = (long long)s->queue.size();
  out->arena_bytes = s->budget;
  out->arena_in_use = rgf::arena_in_use(s->arena);
  out->arena_fallbacks = rgf::arena_fallbacks(s->arena);
  return RGF_OK;
}

int rgf_server_destroy(rgf_server* s) {
  if (!s) return RGF_EINVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  for (auto& t : s->workers) t.join();
  for (auto& kv : s->factors) rgf_destroy(kv.second.h);
  rgf::arena_destroy(s->arena);
  delete s;
  return RGF_OK;
}

}  // extern "C"
