// Request server with continuous batching over the exo_* entry points.
//
// Requests (gemm / gemv / trsv / syrk in single or double precision, every
// operand resident in device memory) are submitted as they arrive, and take
// one of two paths by size:
//  * small requests (gemm / syrk with m n k <= 2^24, gemv with m n <= 2^22,
//    trsv with n <= 512) go to a batcher thread.  Every tick it takes all
//    small requests that arrived since the previous tick and runs them as
//    one device batch (batch.cu: one launch whose CTAs claim the requests'
//    tiles, row blocks and solves from a ticket) on its own stream; requests
//    arriving meanwhile join the next tick.  gemm / syrk run FFMA / DFMA
//    tiles there.
//  * larger requests go to W worker threads, each owning one CUDA stream and
//    its own workspace (the library's per-thread context), pre-grown at
//    start so no worker ever frees device memory while others run.  A
//    request is admitted when a worker slot is free AND its estimated
//    device-memory footprint fits in the admission budget together with
//    everything in flight.  Single-precision gemm / syrk run the split-BF16
//    tensor-core path, double-precision gemm / syrk the Ozaki path; gemv and
//    trsv their native kernels.
// Device batches and worker requests run concurrently on the device.
// Requests that arrive while others are executing wait in bounded queues
// (arrivals beyond capacity are rejected and counted, so overload degrades
// gracefully).  Every path is deterministic and the path depends on the
// request's size only, so a request gives the same bits alone and in a mix.
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

#include "batch.h"
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

// Requests the device batcher takes (sizes where one batch launch beats a
// call of its own; larger ones keep the full-device kernels).
static bool batchable(const exoblas_request &r) {
  switch (r.op) {
    case EXOBLAS_REQ_GEMM:
    case EXOBLAS_REQ_SYRK: {
      const double n = r.op == EXOBLAS_REQ_SYRK ? r.m : r.n;
      return double(r.m) * n * r.k <= double(1 << 24);
    }
    case EXOBLAS_REQ_GEMV:
      return double(r.m) * r.n <= double(1 << 22) && r.ldb != 0 && r.ldc != 0;
    default:
      return r.m <= 512 && r.ldc != 0;
  }
}

// The device-batch description of a request.
static bt::Op batch_op(const exoblas_request &r) {
  bt::Op o{};
  const bool dbl = r.precision == 2;
  o.m = r.m;
  o.n = r.n;
  o.k = r.k;
  o.alpha = r.alpha;
  o.beta = r.beta;
  o.A = r.A;
  o.lda = r.lda;
  o.B = r.B;
  o.ldb = r.ldb;
  o.C = r.C;
  o.ldc = r.ldc;
  switch (r.op) {
    case EXOBLAS_REQ_GEMM:
      o.op = dbl ? bt::kOpDGemm : EXOBLAS_BATCH_SGEMM;
      o.f0 = r.flags[0];
      o.f1 = r.flags[1];
      break;
    case EXOBLAS_REQ_SYRK: {
      // C_tri = alpha op(A) op(A)^T + beta C_tri: a gemm of op(A) (n x k)
      // with op(A)^T, on the stored triangle only
      const bool trans = r.flags[1] != CblasNoTrans;
      o.op = dbl ? bt::kOpDSyrk : bt::kOpSSyrk;
      o.n = r.m;
      o.f0 = trans ? CblasTrans : CblasNoTrans;
      o.f1 = trans ? CblasNoTrans : CblasTrans;
      o.B = r.A;
      o.ldb = r.lda;
      o.tri = r.flags[0] == CblasUpper ? 2 : 1;
      break;
    }
    case EXOBLAS_REQ_GEMV:
      o.op = dbl ? EXOBLAS_BATCH_DGEMV : bt::kOpSGemv;
      o.f0 = r.flags[0];
      break;
    default:
      o.op = dbl ? bt::kOpDTrsv : EXOBLAS_BATCH_STRSV;
      o.f0 = r.flags[0];
      o.f1 = r.flags[1];
      o.f2 = r.flags[2];
      break;
  }
  return o;
}

struct Server {
  int device = 0;
  int workers = 1;
  int sm_count = 0;
  // device batcher: small requests waiting for the next tick
  std::deque<Item> small;
  std::condition_variable cv_batch;
  std::thread batcher;
  bool batch_busy = false;
  std::atomic<long> batched{0}, ticks{0};

  void run_batcher() {
    cudaSetDevice(device);
    bt::TickRunner *tr = nullptr;
    try {
      tr = bt::tick_create();
    } catch (const Error &) {
    }
    for (;;) {
      std::vector<Item> tick;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_batch.wait(lk, [&] { return stop || !small.empty(); });
        if (stop && small.empty()) break;
        tick.assign(small.begin(), small.end());
        small.clear();
        batch_busy = true;
      }
      std::vector<bt::Op> ops;
      ops.reserve(tick.size());
      for (const Item &it : tick) ops.push_back(batch_op(it.r));
      bool ok = tr != nullptr;
      if (ok) {
        try {
          ok = bt::tick_run(tr, ops, sm_count);
        } catch (const Error &) {
          ok = false;
        }
      }
      const double done = now_s();
      {
        std::lock_guard<std::mutex> lk(mu);
        for (const Item &it : tick) latencies.push_back(done - it.arrival);
        last_completion = std::max(last_completion, done);
        (ok ? completed : failed).fetch_add(long(tick.size()));
        batched.fetch_add(long(tick.size()));
        ticks.fetch_add(1);
        batch_busy = false;
      }
      cv_idle.notify_all();
    }
    bt::tick_destroy(tr);
  }
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
    s->sm_count = c.sm_count;
    for (int w = 0; w < workers; ++w) s->threads.emplace_back([s, w] { s->run_worker(w); });
    s->batcher = std::thread([s] { s->run_batcher(); });
    *out = reinterpret_cast<exoblas_server>(s);
  });
}

// arrival_s: host steady-clock seconds (exoblas_server_now()); < 0 means now
int exoblas_server_submit(exoblas_server server, const exoblas_request *req, double arrival_s) {
  return guarded("exoblas_server_submit", [&] {
    auto *s = reinterpret_cast<sv::Server *>(server);
    if (!s || !req) fail(EXOBLAS_INVALID_VALUE, "NULL server or request");
    sv::Item it{*req, arrival_s < 0 ? sv::now_s() : arrival_s, sv::footprint(*req)};
    const bool small = sv::batchable(*req);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->first_arrival < 0) s->first_arrival = it.arrival;
      if (small) {
        if (s->small.size() >= s->queue_cap) {
          s->rejected.fetch_add(1);
          return;
        }
        s->small.push_back(it);
      } else {
        if (s->queue.size() >= s->queue_cap || it.footprint > s->budget) {
          s->rejected.fetch_add(1);
          return;
        }
        s->queue.push_back(it);
      }
    }
    if (small)
      s->cv_batch.notify_one();
    else
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
    s->cv_idle.wait(lk, [&] { return s->queue.empty() && s->busy == 0 && s->small.empty() && !s->batch_busy; });
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

// stats[0..2]: requests served by device batches, device batches run, mean
// requests per batch
int exoblas_server_batch_stats(exoblas_server server, double *stats) {
  return guarded("exoblas_server_batch_stats", [&] {
    auto *s = reinterpret_cast<sv::Server *>(server);
    if (!s || !stats) fail(EXOBLAS_INVALID_VALUE, "NULL argument");
    const double b = double(s->batched.load()), t = double(s->ticks.load());
    stats[0] = b;
    stats[1] = t;
    stats[2] = t > 0 ? b / t : 0;
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
    s->cv_batch.notify_all();
    for (auto &t : s->threads) t.join();
    if (s->batcher.joinable()) s->batcher.join();
    delete s;
  });
}

int exoblas_reserve_scratch(size_t bytes) {
  return guarded("exoblas_reserve_scratch", [&] { scratch(bytes); });
}

}  // extern "C"
