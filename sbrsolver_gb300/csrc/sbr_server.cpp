// Request server: continuous batching of propagation solves on resident
// scenes (no reference counterpart; the reference solves one transmitter per
// call from main()).
//
// A server owns `slots` worker threads.  Submitted requests (copied, with
// their receivers) wait in one queue.  A free worker takes the queued request
// with the least remaining priority cost that fits in the HBM budget next to
// the requests already running: cost = its device-memory estimate (which
// scales with its ray-tree bound, i.e. its work) minus kAgingBytesPerSec per
// second it has waited, so short requests go first and every request is
// served within about a second of becoming the oldest.  The policy may cap
// how many requests too large to batch run at once (small batches still run
// beside them); by default only the slots bound it, since one large solve at
// a time lowered the saturated throughput of a mixed stream by 2-5 % without
// lowering its tail latency.  If the chosen request is small, the worker also
// takes the queued small requests on the same scene (up to kMaxBatch, within
// the budget) and solves them together in one device pass (sbr_solve_batch),
// which fills the GPU far better than small requests one by one.  Every solve checks a workspace (buffers + CUDA
// stream) out of the process-wide pool, so work admitted while other work is
// on the GPU runs on its own stream and overlaps with it.  Each result is
// exactly what sbr_solve returns for that request alone: requests share only
// read-only scene data, and batch results are split per request.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sbr.h"

namespace sbr {
void set_error_message(const std::string& s);
double request_bytes(const sbr_request& q);  // device bytes a request may need
std::vector<sbr_result*> split_result(const sbr_result& batch);
}
// The result type is defined with the solver; the server only needs a
// reference to hand to split_result.
struct sbr_result;

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  long long tag;
  int scene;
  sbr_request req;
  std::vector<double> rx;
  long long est_bytes;
  Clock::time_point submitted;
};

// Device memory one request may need (node records at the ray-tree bound,
// queues, receivers, plus tables); it only gates admission.
long long estimate_bytes(const sbr_request& q) {
  return (long long)sbr::request_bytes(q) + (64LL << 20);
}

// Default policy (sbr_server_set_policy changes it): requests at most 2 GiB
// large (device-memory estimate) are batched, up to 64 in one pass; waiting
// time converted to priority at 16 GB per second (a request that has waited
// one second ranks like one whose estimate is 16 GB smaller); no cap on the
// larger requests running at once beyond the slots.
constexpr long long kDefaultBatchBytes = 2LL << 30;
constexpr int kDefaultMaxBatch = 64;
constexpr double kDefaultAging = 16e9;
constexpr int kDefaultMaxLarge = 0;

}  // namespace

struct sbr_server {
  std::vector<sbr_scene*> scenes;
  long long budget = 0;
  long long in_flight = 0;
  bool stopping = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job> queue;
  std::deque<sbr_completion> done;
  std::vector<std::thread> workers;
  int device = 0;
  long long batch_bytes = kDefaultBatchBytes;  // requests at most this large are batched
  size_t max_batch = size_t(kDefaultMaxBatch);
  double aging = kDefaultAging;  // priority bytes per second waited
  int max_large = kDefaultMaxLarge;  // larger-than-batch_bytes solves at once (0 = no limit)
  int large_running = 0;

  // Index of the queued request to run next (least aged cost among those
  // that fit the budget and the limit on large solves), or -1.  Caller holds mu.
  long pick() const {
    const Clock::time_point now = Clock::now();
    const bool large_full = max_large > 0 && large_running >= max_large;
    long best = -1;
    double best_cost = 0;
    for (size_t k = 0; k < queue.size(); ++k) {
      const Job& j = queue[k];
      if (large_full && j.est_bytes > batch_bytes) continue;
      const long long need = std::min(j.est_bytes, budget);
      if (!(in_flight == 0 || in_flight + need <= budget)) continue;
      const double waited = std::chrono::duration<double>(now - j.submitted).count();
      const double cost = double(j.est_bytes) - aging * waited;
      if (best < 0 || cost < best_cost) {
        best = long(k);
        best_cost = cost;
      }
    }
    return best;
  }

  void worker() {
    cudaSetDevice(device);
    for (;;) {
      std::vector<Job> batch;
      long long est = 0;
      bool large = false;
      {
        std::unique_lock<std::mutex> lock(mu);
        long sel = -1;
        cv_work.wait(lock, [&] {
          if (stopping && queue.empty()) return true;
          sel = pick();
          return sel >= 0;
        });
        if (queue.empty()) return;
        batch.push_back(std::move(queue[size_t(sel)]));
        queue.erase(queue.begin() + sel);
        est = std::min(batch[0].est_bytes, budget);
        large = batch[0].est_bytes > batch_bytes;
        if (large) {
          ++large_running;
        } else {
          for (auto it = queue.begin(); it != queue.end() && batch.size() < max_batch;) {
            if (it->scene == batch[0].scene && it->est_bytes <= batch_bytes &&
                in_flight + est + it->est_bytes <= budget) {
              est += it->est_bytes;
              batch.push_back(std::move(*it));
              it = queue.erase(it);
            } else {
              ++it;
            }
          }
        }
        in_flight += est;
      }
      cv_work.notify_all();
      const Clock::time_point start = Clock::now();
      std::vector<sbr_request> reqs(batch.size());
      for (size_t i = 0; i < batch.size(); ++i) {
        reqs[i] = batch[i].req;
        reqs[i].rx = batch[i].rx.empty() ? nullptr : batch[i].rx.data();
        reqs[i].rx_on_device = 0;
      }
      sbr_result* res = nullptr;
      const sbr_status st =
          sbr_solve_batch(scenes[batch[0].scene], reqs.data(), int(reqs.size()), &res);
      const Clock::time_point end = Clock::now();
      std::vector<sbr_result*> parts;
      if (res && batch.size() > 1) {
        parts = sbr::split_result(*res);
        sbr_result_destroy(res);
      } else {
        parts.assign(batch.size(), nullptr);
        if (res) parts[0] = res;
      }
      std::vector<sbr_completion> out;
      for (size_t i = 0; i < batch.size(); ++i) {
        sbr_completion c;
        std::memset(&c, 0, sizeof c);
        c.tag = batch[i].tag;
        c.scene = batch[i].scene;
        c.status = st;
        c.queue_ms = std::chrono::duration<double, std::milli>(start - batch[i].submitted).count();
        c.latency_ms = std::chrono::duration<double, std::milli>(end - batch[i].submitted).count();
        c.result = i < parts.size() ? parts[i] : nullptr;
        if (c.result) {
          sbr_timing t;
          sbr_result_timing(c.result, &t);
          c.device_ms = t.device_ms;
          sbr_result_counts(c.result, &c.counts);
        }
        out.push_back(c);
      }
      {
        std::lock_guard<std::mutex> lock(mu);
        in_flight -= est;
        if (large) --large_running;
        for (auto& c : out) done.push_back(c);
      }
      cv_work.notify_all();
      cv_done.notify_all();
    }
  }
};

extern "C" {

sbr_status sbr_server_create(sbr_scene* const* scenes, int n_scenes, int slots,
                             long long hbm_budget_bytes, sbr_server** out) {
  if (!scenes || n_scenes <= 0 || slots <= 0 || slots > 64 || !out) {
    sbr::set_error_message("sbr_server_create: need scenes, 1..64 slots and an output pointer");
    return SBR_ERR_INVALID_ARG;
  }
  for (int i = 0; i < n_scenes; ++i)
    if (!scenes[i]) {
      sbr::set_error_message("sbr_server_create: NULL scene");
      return SBR_ERR_INVALID_ARG;
    }
  auto srv = std::make_unique<sbr_server>();
  srv->scenes.assign(scenes, scenes + n_scenes);
  cudaGetDevice(&srv->device);
  if (hbm_budget_bytes <= 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      sbr::set_error_message("sbr_server_create: cudaMemGetInfo failed");
      return SBR_ERR_CUDA;
    }
    hbm_budget_bytes = (long long)(0.6 * double(free_b));
  }
  srv->budget = hbm_budget_bytes;
  for (int i = 0; i < slots; ++i) srv->workers.emplace_back(&sbr_server::worker, srv.get());
  *out = srv.release();
  return SBR_OK;
}

sbr_status sbr_server_submit(sbr_server* srv, int scene, const sbr_request* req, long long tag) {
  if (!srv || !req || scene < 0 || scene >= int(srv->scenes.size()) || req->n_rx < 0 ||
      (req->n_rx > 0 && !req->rx) || req->rx_on_device) {
    sbr::set_error_message("sbr_server_submit: bad arguments (receivers must be host memory)");
    return SBR_ERR_INVALID_ARG;
  }
  Job job;
  job.tag = tag;
  job.scene = scene;
  job.req = *req;
  job.rx.assign(req->rx, req->rx + 3 * size_t(req->n_rx));
  job.est_bytes = estimate_bytes(*req);
  job.submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    if (srv->stopping) {
      sbr::set_error_message("sbr_server_submit: server is shutting down");
      return SBR_ERR_NOT_READY;
    }
    srv->queue.push_back(std::move(job));
  }
  srv->cv_work.notify_one();
  return SBR_OK;
}

sbr_status sbr_server_poll(sbr_server* srv, sbr_completion* out, int max, int* n_out,
                           int timeout_ms) {
  if (!srv || !out || max <= 0 || !n_out) {
    sbr::set_error_message("sbr_server_poll: bad arguments");
    return SBR_ERR_INVALID_ARG;
  }
  std::unique_lock<std::mutex> lock(srv->mu);
  if (srv->done.empty() && timeout_ms > 0)
    srv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                          [&] { return !srv->done.empty(); });
  int n = 0;
  while (n < max && !srv->done.empty()) {
    out[n++] = srv->done.front();
    srv->done.pop_front();
  }
  *n_out = n;
  return SBR_OK;
}

sbr_status sbr_server_pending(sbr_server* srv, int* queued, long long* in_flight_bytes) {
  if (!srv) {
    sbr::set_error_message("sbr_server_pending: NULL server");
    return SBR_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(srv->mu);
  if (queued) *queued = int(srv->queue.size());
  if (in_flight_bytes) *in_flight_bytes = srv->in_flight;
  return SBR_OK;
}

sbr_status sbr_server_set_policy(sbr_server* server, long long batch_bytes, int max_batch,
                                double aging_bytes_per_s, int max_large) {
  if (!server || batch_bytes < 0 || max_batch < 1 || max_batch > 4096 ||
      !(aging_bytes_per_s >= 0.0) || max_large < 0) {
    sbr::set_error_message("sbr_server_set_policy: need a server, batch_bytes >= 0, "
                           "1 <= max_batch <= 4096, aging_bytes_per_s >= 0 and "
                           "max_large >= 0");
    return SBR_ERR_INVALID_ARG;
  }
  {
    std::lock_guard<std::mutex> lock(server->mu);
    server->batch_bytes = batch_bytes;
    server->max_batch = size_t(max_batch);
    server->aging = aging_bytes_per_s;
    server->max_large = max_large;
  }
  server->cv_work.notify_all();  // a looser limit may admit a queued request now
  return SBR_OK;
}

sbr_status sbr_server_destroy(sbr_server* srv) {
  if (!srv) return SBR_OK;
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->stopping = true;
  }
  srv->cv_work.notify_all();
  for (auto& t : srv->workers) t.join();
  for (auto& c : srv->done)
    if (c.result) sbr_result_destroy(c.result);
  delete srv;
  return SBR_OK;
}

}  // extern "C"
