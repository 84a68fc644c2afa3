// Serving loop: hydro runs arrive as requests, are admitted against an HBM
// budget and a slot limit, advance together in batched ticks (one launch per
// phase for every resident run), and retire independently at their own end
// (no counterpart in the reference, which runs one deck per process).
//
// Continuous batching.  A worker thread owned by the context repeats:
//   1. queue a tick: K cycles of the batch of resident runs (asynchronous);
//   2. while the GPU works, build the initial state of waiting requests that
//      fit the budget on a few host threads (prepare_run);
//   3. wait for the tick, read every run's done flag, retire finished runs
//      (stamp the completion, free or keep their HBM);
//   4. place the prepared runs on the device (upload + prologue), so they
//      join the next tick.
// A request's latency is retirement time minus submission time.  The batch
// kernels compute each run exactly as it would be computed alone, so a
// result does not depend on what it was served with.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <future>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "runtime.h"

namespace hydro {

int batch_enqueue(hydro_ctx* ctx, hydro_run* const* runs, int n, int ncycles);
int batch_done_flags(hydro_ctx* ctx, std::vector<int>* done);

namespace {
using Clock = std::chrono::steady_clock;
double secs(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}
}  // namespace

struct ServeRequest {
  long id = 0;
  hydro_spec spec{};
  int keep = 0;
  Clock::time_point submitted, admitted, placed;
  // placed run (while resident / kept)
  hydro_run* run = nullptr;
  long long cycles_enqueued = 0;
  size_t bytes = 0;
};

struct ServeState {
  hydro_ctx* ctx = nullptr;
  std::mutex mu;
  std::condition_variable cv;       // completions / new requests
  std::deque<ServeRequest> waiting;  // submitted, not admitted
  std::vector<ServeRequest> resident;
  std::map<long, ServeRequest> kept;  // finished, held for fetch
  std::vector<hydro_run*> to_free;    // released by the user, freed by the worker
  std::deque<hydro_serve_done> done;  // completions not yet polled
  long next_id = 1;
  bool stop = false;
  bool running = false;
  std::thread worker;
  // configuration
  size_t budget = 0;        // bytes; 0 = the context's budget (or none)
  int max_resident = 256;
  int tick_cycles = 8;
  int prep_threads = 4;
  // statistics
  hydro_serve_stats st{};
  Clock::time_point t_first{}, t_last{};
  bool any = false;
  int error = 0;
  std::string error_msg;
};

namespace {

size_t budget_of(const ServeState* S) {
  return S->budget ? S->budget : S->ctx->budget;
}

// HBM of a request: its run's arena (sizes only, no state is built).
size_t arena_of(const hydro_spec& s) { return run_arena_bytes(s); }

void worker_main(ServeState* S) {
  hydro_ctx* ctx = S->ctx;
  cudaSetDevice(ctx->device);
  std::vector<std::future<std::pair<int, PreparedRun*>>> prep;
  std::vector<ServeRequest> preparing;
  size_t reserved = 0;  // bytes of admitted requests not yet placed
  for (;;) {
    // ---- 1. tick
    std::vector<hydro_run*> runs;
    int K = S->tick_cycles;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      if (S->stop) break;
      for (auto& r : S->resident) {
        runs.push_back(r.run);
        const long long left = (r.spec.max_cycles > 0 ? r.spec.max_cycles : 1LL << 40) -
                               r.cycles_enqueued;
        if (left > 0 && left < K) K = (int)left;
      }
    }
    if (K < 1) K = 1;
    int rc = 0;
    if (!runs.empty()) {
      rc = batch_enqueue(ctx, runs.data(), (int)runs.size(), K);
      std::lock_guard<std::mutex> lk(S->mu);
      for (auto& r : S->resident) r.cycles_enqueued += K;
      S->st.ticks += 1;
      S->st.cycles += K;
    }
    // ---- 2. admit and prepare while the GPU works
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (runs.empty() && S->waiting.empty() && preparing.empty()) {
        S->cv.wait(lk, [&] {
          return S->stop || !S->waiting.empty() || !S->to_free.empty();
        });
        if (S->stop) break;
      }
      const size_t B = budget_of(S);
      size_t in_use = reserved;
      for (auto& r : S->resident) in_use += r.bytes;
      for (auto& k : S->kept) in_use += k.second.bytes;
      while (!S->waiting.empty() &&
             (int)(S->resident.size() + preparing.size()) < S->max_resident &&
             (int)preparing.size() < 2 * S->prep_threads) {
        ServeRequest& q = S->waiting.front();
        const size_t need = arena_of(q.spec);
        if (B && in_use + need > B) break;  // first-come first-served
        in_use += need;
        reserved += need;
        q.bytes = need;
        q.admitted = Clock::now();
        preparing.push_back(q);
        S->waiting.pop_front();
        const hydro_spec sp = preparing.back().spec;
        prep.push_back(std::async(std::launch::async, [sp]() {
          auto* pr = new PreparedRun();
          int r = prepare_run(sp, *pr);
          return std::make_pair(r, pr);
        }));
      }
    }
    // ---- 3. wait for the tick, retire finished runs
    std::vector<int> done;
    std::vector<hydro_run*> frees;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      frees.swap(S->to_free);
    }
    if (!runs.empty() && !rc) rc = batch_done_flags(ctx, &done);
    if (rc) {
      // runs released by the user are no longer listed anywhere: free them
      // here; requests still being prepared or on the device will never
      // finish, so their pollers get a failed completion (the resident runs
      // stay listed and are freed with the server)
      for (auto* r : frees) hydro_run_destroy(r);
      std::lock_guard<std::mutex> lk(S->mu);
      S->error = rc;
      S->error_msg = hydro_last_error();
      const auto now = Clock::now();
      auto post_failed = [&](const ServeRequest& q) {
        hydro_serve_done d{};
        d.req_id = q.id;
        d.status = -1;
        d.latency_s = secs(q.submitted, now);
        S->done.push_back(d);
        S->st.failed += 1;
      };
      for (const auto& q : preparing) post_failed(q);
      for (const auto& q : S->resident) post_failed(q);
      S->stop = true;
      S->cv.notify_all();
      break;
    }
    for (auto* r : frees) hydro_run_destroy(r);
    const auto now = Clock::now();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      std::vector<ServeRequest> still;
      for (size_t k = 0; k < S->resident.size(); ++k) {
        ServeRequest& r = S->resident[k];
        if (k < done.size() && done[k]) {
          unsigned code = 0;
          long cell = 0;
          hydro_run_error(r.run, &code, &cell);
          long cyc = 0;
          hydro_run_time(r.run, nullptr, nullptr, &cyc);
          hydro_serve_done d{};
          d.req_id = r.id;
          d.status = (int)code;
          d.latency_s = secs(r.submitted, now);
          d.wait_s = secs(r.submitted, r.admitted);
          d.resident_s = secs(r.placed, now);
          d.cycles = cyc;
          d.cells = (long)r.spec.nx * r.spec.ny;
          S->done.push_back(d);
          S->st.completed += 1;
          S->st.cell_updates += (double)d.cells * (double)cyc;
          S->t_last = now;
          if (r.keep) {
            S->kept[r.id] = r;
          } else {
            hydro_run_destroy(r.run);
          }
        } else {
          still.push_back(r);
        }
      }
      S->resident.swap(still);
      S->cv.notify_all();
    }
    // ---- 4. place prepared runs (their uploads join the stream after the
    // tick, so they are in HBM before the next one)
    for (size_t k = 0; k < prep.size();) {
      const bool ready =
          prep[k].wait_for(std::chrono::seconds(0)) == std::future_status::ready ||
          runs.empty();
      if (!ready) {
        ++k;
        continue;
      }
      auto res = prep[k].get();
      ServeRequest q = preparing[k];
      prep.erase(prep.begin() + k);
      preparing.erase(preparing.begin() + k);
      reserved -= q.bytes;
      PreparedRun* pr = res.second;
      int prc = res.first;
      hydro_run* run = nullptr;
      if (!prc) {
        q.bytes = pr->bytes;
        prc = place_run(ctx, *pr, &run, false);
      }
      delete pr;
      std::lock_guard<std::mutex> lk(S->mu);
      if (prc) {
        hydro_serve_done d{};
        d.req_id = q.id;
        d.status = -1;
        d.latency_s = secs(q.submitted, Clock::now());
        d.wait_s = secs(q.submitted, q.admitted);
        S->done.push_back(d);
        S->st.failed += 1;
        S->cv.notify_all();
        continue;
      }
      q.run = run;
      q.placed = Clock::now();
      q.cycles_enqueued = 0;
      if (!S->any) {
        S->any = true;
        S->t_first = Clock::now();
      }
      S->st.admitted += 1;
      S->resident.push_back(q);
    }
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->resident.empty() && preparing.empty() && !S->waiting.empty())
        // nothing resident and the head request does not fit: wait for a
        // release (kept runs hold the budget) or a stop
        S->cv.wait_for(lk, std::chrono::milliseconds(50),
                       [&] { return S->stop || !S->to_free.empty(); });
      S->st.resident = (long)S->resident.size();
      S->st.waiting = (long)(S->waiting.size() + preparing.size());
      size_t in_use = 0;
      for (auto& r : S->resident) in_use += r.bytes;
      for (auto& k : S->kept) in_use += k.second.bytes;
      S->st.bytes_in_use = in_use;
      if (in_use > S->st.peak_bytes) S->st.peak_bytes = in_use;
      if ((long)S->resident.size() > S->st.peak_resident)
        S->st.peak_resident = (long)S->resident.size();
    }
  }
  for (auto& f : prep) {
    auto res = f.get();
    delete res.second;
  }
}

ServeState* get_serve(hydro_ctx* ctx) {
  if (!ctx->serve) {
    auto* S = new ServeState();
    S->ctx = ctx;
    ctx->serve = S;
  }
  return ctx->serve;
}

void start_worker(ServeState* S) {
  if (!S->running) {
    S->stop = false;
    S->running = true;
    S->worker = std::thread(worker_main, S);
  }
}

void stop_worker(ServeState* S) {
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  S->running = false;
}

}  // namespace

void destroy_serve(ServeState* S) {
  if (!S) return;
  stop_worker(S);
  for (auto& r : S->resident) hydro_run_destroy(r.run);
  for (auto& k : S->kept) hydro_run_destroy(k.second.run);
  for (auto* r : S->to_free) hydro_run_destroy(r);
  delete S;
}

}  // namespace hydro

using namespace hydro;

extern "C" {

int hydro_serve_config(hydro_ctx* ctx, size_t budget_bytes, int max_resident,
                       int tick_cycles, int prep_threads) {
  if (!ctx) return fail(-1, "hydro_serve_config: null context");
  ServeState* S = get_serve(ctx);
  std::lock_guard<std::mutex> lk(S->mu);
  S->budget = budget_bytes;
  if (max_resident > 0) S->max_resident = max_resident;
  if (tick_cycles > 0) S->tick_cycles = tick_cycles;
  if (prep_threads > 0) S->prep_threads = prep_threads;
  return 0;
}

int hydro_serve_submit(hydro_ctx* ctx, const hydro_spec* spec, int keep,
                       long* req_id) {
  if (!ctx || !spec) return fail(-1, "hydro_serve_submit: null argument");
  if (spec->scheme != HYDRO_SCHEME_VNR && spec->scheme != HYDRO_SCHEME_EUCCLHYD)
    return fail(-4, "hydro_serve_submit: unknown scheme");
  if (spec->projection != 1)
    return fail(-5, "hydro_serve_submit: the serving loop advances runs with the remap");
  ServeState* S = get_serve(ctx);
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->error) return fail(-2, "serving stopped: " + S->error_msg);
  ServeRequest q;
  q.id = S->next_id++;
  q.spec = *spec;
  q.keep = keep ? 1 : 0;
  q.submitted = Clock::now();
  const size_t B = budget_of(S);
  if (B && arena_of(*spec) > B)
    return fail(-3, "hydro_serve_submit: the run alone exceeds the HBM budget");
  S->waiting.push_back(q);
  S->st.submitted += 1;
  if (req_id) *req_id = q.id;
  start_worker(S);
  S->cv.notify_all();
  return 0;
}

// Pops one completion (1), or returns 0 when none is ready within
// timeout_s seconds (0: do not wait).
int hydro_serve_poll(hydro_ctx* ctx, double timeout_s, hydro_serve_done* out) {
  if (!ctx || !out) return fail(-1, "hydro_serve_poll: null argument");
  ServeState* S = get_serve(ctx);
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->done.empty() && timeout_s > 0)
    S->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                   [&] { return !S->done.empty() || S->error; });
  if (S->done.empty()) {
    if (S->error) return fail(-2, "serving stopped: " + S->error_msg);
    return 0;
  }
  *out = S->done.front();
  S->done.pop_front();
  return 1;
}

// The run of a finished request submitted with keep = 1 (owned by the
// server until hydro_serve_release); NULL otherwise.
hydro_run* hydro_serve_result(hydro_ctx* ctx, long req_id) {
  if (!ctx || !ctx->serve) return nullptr;
  ServeState* S = ctx->serve;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->kept.find(req_id);
  return it == S->kept.end() ? nullptr : it->second.run;
}

int hydro_serve_release(hydro_ctx* ctx, long req_id) {
  if (!ctx || !ctx->serve) return fail(-1, "hydro_serve_release: nothing served");
  ServeState* S = ctx->serve;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->kept.find(req_id);
  if (it == S->kept.end()) return fail(-2, "hydro_serve_release: unknown request");
  // the worker frees it between ticks (it owns the batch plan)
  if (S->running)
    S->to_free.push_back(it->second.run);
  else
    hydro_run_destroy(it->second.run);
  S->kept.erase(it);
  S->cv.notify_all();
  return 0;
}

int hydro_serve_stats_get(hydro_ctx* ctx, hydro_serve_stats* out) {
  if (!ctx || !out) return fail(-1, "hydro_serve_stats_get: null argument");
  ServeState* S = get_serve(ctx);
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->st;
  out->busy_s = S->any ? secs(S->t_first, S->t_last) : 0.0;
  return 0;
}

// Stops the worker after the resident runs and waiting requests are done
// (drain = 1) or at once (drain = 0; unfinished runs are dropped).
int hydro_serve_stop(hydro_ctx* ctx, int drain) {
  if (!ctx || !ctx->serve) return 0;
  ServeState* S = ctx->serve;
  if (drain) {
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv.wait(lk, [&] {
      return S->error || (S->waiting.empty() && S->resident.empty() &&
                          S->st.admitted + S->st.failed >= S->st.submitted);
    });
  }
  stop_worker(S);
  std::lock_guard<std::mutex> lk(S->mu);
  for (auto& r : S->resident) hydro_run_destroy(r.run);
  for (auto* r : S->to_free) hydro_run_destroy(r);
  S->to_free.clear();
  S->resident.clear();
  S->waiting.clear();
  return S->error ? fail(-2, "serving stopped: " + S->error_msg) : 0;
}

}  // extern "C"
