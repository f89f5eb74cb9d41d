// Request server with continuous batching over the exo_* entry points.
//
// Requests (gemm / gemv / trsv / syrk in single or double precision, every
// operand resident in device memory) are submitted as they arrive.  Each of
// W worker threads owns one CUDA stream and its own workspace (the
// library's per-thread context), pre-grown at start so no worker ever frees
// device memory while others run.  A request is admitted when a worker slot
// is free AND its estimated device-memory footprint fits in the admission
// budget together with everything in flight; admitted requests from
// different workers run concurrently on the device.  Requests that arrive
// while others are executing wait in a bounded queue (arrivals beyond its
// capacity are rejected and counted, so overload degrades gracefully).
// Single-precision gemm / syrk run the split-BF16 tensor-core path,
// double-precision gemm / syrk the Ozaki path; gemv and trsv their native
// kernels.
// Latency = completion - arrival, measured on the host clock.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace sv {

using Clock = std::chrono::steady_clock;

static double now_s() {
  return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

struct Item {
  exoblas_request r;
  double arrival;
  size_t footprint;
};

static size_t footprint(const exoblas_request &r) {
  const size_t es = r.precision == 2 ? 8 : 4;
  auto rnd = [](long v, long m) { return size_t((v + m - 1) / m * m); };
  switch (r.op) {
    case EXOBLAS_REQ_GEMM:
    case EXOBLAS_REQ_SYRK: {
      const long m = r.m, n = r.op == EXOBLAS_REQ_SYRK ? r.m : r.n, k = r.k;
      if (r.precision == 2)  // Ozaki: 8 digit planes of both operands
        return 8 * (rnd(m, 128) + rnd(n, 64)) * rnd(k, 256) * 2 + size_t(m) * n * es;
      return 3 * (rnd(m, 128) + rnd(n, 128)) * rnd(k, 64) * 2 + size_t(m) * n * es;
    }
    case EXOBLAS_REQ_GEMV:
      return size_t(r.m + r.n) * es * 8;
    default:  // trsv: inverses + slots
      return size_t(r.m) * 64 * es + size_t(r.m) * es * 64;
  }
}

struct Server {
  int device = 0;
  int workers = 1;
  size_t budget = 0, inflight_bytes = 0, queue_cap = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_idle;
  std::deque<Item> queue;
  bool stop = false;
  int busy = 0;
  std::vector<std::thread> threads;
  std::vector<double> latencies;  // seconds, completion order
  std::atomic<long> completed{0}, rejected{0}, failed{0};
  double first_arrival = -1, last_completion = 0;
  size_t scratch_reserve = 0;

  void run_worker(int wid) {
    cudaSetDevice(device);
    // private stream + workspace for this worker thread
    exoblas_set_stream(nullptr);
    exoblas_set_blocking(0);
    if (scratch_reserve) scratch(scratch_reserve);
    for (;;) {
      Item it;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] {
          return stop || (!queue.empty() && inflight_bytes + queue.front().footprint <= budget);
        });
        if (stop && queue.empty()) return;
        if (queue.empty()) continue;
        it = queue.front();
        queue.pop_front();
        inflight_bytes += it.footprint;
        ++busy;
      }
      const bool ok = execute(it.r);
      const double done = now_s();
      {
        std::lock_guard<std::mutex> lk(mu);
        inflight_bytes -= it.footprint;
        --busy;
        latencies.push_back(done - it.arrival);
        last_completion = std::max(last_completion, done);
        if (ok)
          completed.fetch_add(1);
        else
          failed.fetch_add(1);
      }
      cv_work.notify_all();
      cv_idle.notify_all();
      (void)wid;
    }
  }

  // Runs one request on this worker's stream and waits for it.
  bool execute(const exoblas_request &r) {
    const int RM = CblasRowMajor;
    const bool dbl = r.precision == 2;
    switch (r.op) {
      case EXOBLAS_REQ_GEMM:
        exoblas_set_precision(dbl ? EXOBLAS_PRECISION_OZAKI : EXOBLAS_PRECISION_SPLIT_BF16);
        if (dbl)
          exo_dgemm(CBLAS_ORDER(RM), CBLAS_TRANSPOSE(r.flags[0]), CBLAS_TRANSPOSE(r.flags[1]), r.m, r.n, r.k, r.alpha,
                    static_cast<const double *>(r.A), r.lda, static_cast<const double *>(r.B), r.ldb, r.beta,
                    static_cast<double *>(r.C), r.ldc);
        else
          exo_sgemm(CBLAS_ORDER(RM), CBLAS_TRANSPOSE(r.flags[0]), CBLAS_TRANSPOSE(r.flags[1]), r.m, r.n, r.k,
                    float(r.alpha), static_cast<const float *>(r.A), r.lda, static_cast<const float *>(r.B), r.ldb,
                    float(r.beta), static_cast<float *>(r.C), r.ldc);
        break;
      case EXOBLAS_REQ_SYRK:
        exoblas_set_precision(dbl ? EXOBLAS_PRECISION_OZAKI : EXOBLAS_PRECISION_SPLIT_BF16);
        if (dbl)
          exo_dsyrk(CBLAS_ORDER(RM), CBLAS_UPLO(r.flags[0]), CBLAS_TRANSPOSE(r.flags[1]), r.m, r.k, r.alpha,
                    static_cast<const double *>(r.A), r.lda, r.beta, static_cast<double *>(r.C), r.ldc);
        else
          exo_ssyrk(CBLAS_ORDER(RM), CBLAS_UPLO(r.flags[0]), CBLAS_TRANSPOSE(r.flags[1]), r.m, r.k, float(r.alpha),
                    static_cast<const float *>(r.A), r.lda, float(r.beta), static_cast<float *>(r.C), r.ldc);
        break;
      case EXOBLAS_REQ_GEMV:
        if (dbl)
          exo_dgemv(CBLAS_ORDER(RM), CBLAS_TRANSPOSE(r.flags[0]), r.m, r.n, r.alpha, static_cast<const double *>(r.A),
                    r.lda, static_cast<const double *>(r.B), r.ldb, r.beta, static_cast<double *>(r.C), r.ldc);
        else
          exo_sgemv(CBLAS_ORDER(RM), CBLAS_TRANSPOSE(r.flags[0]), r.m, r.n, float(r.alpha),
                    static_cast<const float *>(r.A), r.lda, static_cast<const float *>(r.B), r.ldb, float(r.beta),
                    static_cast<float *>(r.C), r.ldc);
        break;
      default:
        if (dbl)
          exo_dtrsv(CBLAS_ORDER(RM), CBLAS_UPLO(r.flags[0]), CBLAS_TRANSPOSE(r.flags[1]), CBLAS_DIAG(r.flags[2]), r.m,
                    static_cast<const double *>(r.A), r.lda, static_cast<double *>(r.C), r.ldc);
        else
          exo_strsv(CBLAS_ORDER(RM), CBLAS_UPLO(r.flags[0]), CBLAS_TRANSPOSE(r.flags[1]), CBLAS_DIAG(r.flags[2]), r.m,
                    static_cast<const float *>(r.A), r.lda, static_cast<float *>(r.C), r.ldc);
        break;
    }
    int st = exoblas_get_status();
    if (st == EXOBLAS_SUCCESS) st = exoblas_synchronize();
    return st == EXOBLAS_SUCCESS;
  }
};

}  // namespace sv
}  // namespace exb

using namespace exb;

extern "C" {

int exoblas_server_create(int workers, size_t hbm_budget_bytes, size_t queue_capacity, size_t scratch_reserve_bytes,
                          exoblas_server *out) {
  return guarded("exoblas_server_create", [&] {
    if (!out || workers < 1) fail(EXOBLAS_INVALID_VALUE, "bad server arguments");
    Context &c = ctx();
    auto *s = new sv::Server();
    s->device = c.device;
    s->workers = workers;
    size_t freeb = 0, total = 0;
    EXB_CUDA(cudaMemGetInfo(&freeb, &total));
    const size_t auto_budget = freeb / 10 * 7;
    s->budget = hbm_budget_bytes ? std::min(hbm_budget_bytes, auto_budget) : auto_budget;
    s->queue_cap = queue_capacity ? queue_capacity : ~size_t(0);
    s->scratch_reserve = scratch_reserve_bytes;
    for (int w = 0; w < workers; ++w) s->threads.emplace_back([s, w] { s->run_worker(w); });
    *out = reinterpret_cast<exoblas_server>(s);
  });
}

// arrival_s: host steady-clock seconds (exoblas_server_now()); < 0 means now
int exoblas_server_submit(exoblas_server server, const exoblas_request *req, double arrival_s) {
  return guarded("exoblas_server_submit", [&] {
    auto *s = reinterpret_cast<sv::Server *>(server);
    if (!s || !req) fail(EXOBLAS_INVALID_VALUE, "NULL server or request");
    sv::Item it{*req, arrival_s < 0 ? sv::now_s() : arrival_s, sv::footprint(*req)};
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->first_arrival < 0) s->first_arrival = it.arrival;
      if (s->queue.size() >= s->queue_cap || it.footprint > s->budget) {
        s->rejected.fetch_add(1);
        return;
      }
      s->queue.push_back(it);
    }
    s->cv_work.notify_one();
  });
}

double exoblas_server_now(void) { return sv::now_s(); }

// Submits reqs[i] at t0 + offsets_s[i] (t0 = this call's start), sleeping
// until shortly before each arrival and spinning the rest, so a recorded
// arrival process is replayed on the host clock.  *t0_out (if not NULL)
// receives t0.
int exoblas_server_replay(exoblas_server server, const exoblas_request *reqs, const double *offsets_s, size_t count,
                          double *t0_out) {
  return guarded("exoblas_server_replay", [&] {
    auto *s = reinterpret_cast<sv::Server *>(server);
    if (!s || (count && (!reqs || !offsets_s))) fail(EXOBLAS_INVALID_VALUE, "NULL argument");
    const double t0 = sv::now_s();
    if (t0_out) *t0_out = t0;
    for (size_t i = 0; i < count; ++i) {
      const double at = t0 + offsets_s[i];
      double wait = at - sv::now_s();
      if (wait > 200e-6) std::this_thread::sleep_for(std::chrono::duration<double>(wait - 100e-6));
      while (sv::now_s() < at) {
      }
      const int st = exoblas_server_submit(server, &reqs[i], at);
      if (st != EXOBLAS_SUCCESS) fail(st, "submit failed");
    }
  });
}

// Waits until every submitted request has finished.
int exoblas_server_drain(exoblas_server server) {
  return guarded("exoblas_server_drain", [&] {
    auto *s = reinterpret_cast<sv::Server *>(server);
    if (!s) fail(EXOBLAS_INVALID_VALUE, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_idle.wait(lk, [&] { return s->queue.empty() && s->busy == 0; });
  });
}

// stats[0..7]: completed, rejected, failed, p50 s, p99 s, mean s, max s,
// solves per second (completed / (last completion - first arrival))
int exoblas_server_stats(exoblas_server server, double *stats) {
  return guarded("exoblas_server_stats", [&] {
    auto *s = reinterpret_cast<sv::Server *>(server);
    if (!s || !stats) fail(EXOBLAS_INVALID_VALUE, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, size_t(p * (l.size() - 1) + 0.5))]; };
    double mean = 0;
    for (double v : l) mean += v;
    stats[0] = double(s->completed.load());
    stats[1] = double(s->rejected.load());
    stats[2] = double(s->failed.load());
    stats[3] = pct(0.50);
    stats[4] = pct(0.99);
    stats[5] = l.empty() ? 0 : mean / double(l.size());
    stats[6] = l.empty() ? 0 : l.back();
    const double span = s->last_completion - s->first_arrival;
    stats[7] = span > 0 ? double(s->completed.load()) / span : 0;
  });
}

int exoblas_server_destroy(exoblas_server server) {
  return guarded("exoblas_server_destroy", [&] {
    auto *s = reinterpret_cast<sv::Server *>(server);
    if (!s) return;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->threads) t.join();
    delete s;
  });
}

int exoblas_reserve_scratch(size_t bytes) {
  return guarded("exoblas_reserve_scratch", [&] { scratch(bytes); });
}

}  // extern "C"
