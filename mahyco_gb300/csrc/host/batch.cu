// Batch engine: advances many independent runs together, one persistent
// launch per phase for all of them (no counterpart in the reference, whose
// scheme object advances one mesh).
//
// Layout.  Each run keeps its own HBM arena (runner.cu); the batch adds one
// device block holding the runs' RunViews, a done flag per run, and for each
// item domain (cells, nodes) and tile shape (kTileShapes) a table of tiles:
// {run, first row, first column}.  Tables are
// run-major, so consecutive blocks of a persistent grid work on neighbouring
// tiles of the same mesh.  Counts live on the device, so the CUDA graph that
// holds a cycle's launches stays valid when the membership changes, as long
// as the block does not have to grow.
//
// Tuning.  The tile shape and the grid size of each phase are chosen by
// timing real cycles of the batch, one candidate configuration per cycle.
// The mapping of items to threads does not change any result (each item is
// computed by one thread with the same arithmetic, and the cycle's dt / max
// pressure reductions are exact min / max), so tuning cycles are ordinary
// cycles of the runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "runtime.h"

namespace hydro {

namespace {
// Candidate grid modes: persistent (resident blocks x SMs) or one block per
// tile.
constexpr int kGridModes = 2;
constexpr int kNumCandidates = kNumTileShapes * kGridModes;
// cycle kernel kind (launch hook id) -> phase, -1 for control kernels
int phase_of_kind(int kind) {
  switch (kind) {
    case 2: return kPhLagNodes;
    case 3: return kPhLagCells;
    case 11: return kPhFaceGrad;
    case 4: return kPhSweepGrad;
    case 5: return kPhSweepFace;
    case 6: return kPhSweepUpdate;
    case 7: return kPhDualGrad;
    case 8: return kPhDualUpdate;
    case 9: return kPhFinal;
    case 12: return kPhEucCellPre;
    case 13: return kPhEucNodes;
    case 14: return kPhEucCells;
    case 15: return kPhEucFinal;
    default: return -1;
  }
}
}  // namespace

struct BatchPlan {
  hydro_ctx* ctx = nullptr;
  std::vector<hydro_run*> runs;
  // device block
  char* dmem = nullptr;
  size_t dbytes = 0;
  int cap_inst = 0;
  long long cap_tiles[2][kNumTileShapes] = {};
  RunView* d_views = nullptr;
  int* d_ninst = nullptr;
  int* d_done = nullptr;
  int* d_ntiles = nullptr;
  Tile* d_tiles[2][kNumTileShapes] = {};
  long long h_ntiles[2][kNumTileShapes] = {};
  std::vector<int> h_done;
  int blocks_per_sm[kNumPhases] = {};
  int occ_variant = 0;  // the kernel variant blocks_per_sm was measured for
  // chosen configuration
  int shape[kNumPhases] = {};
  int mode[kNumPhases] = {};
  int tune_next = 0;  // next candidate to time; kNumCandidates + 1 when done
  int tuned = 0;      // a timed tuning pass chose the configuration
  double tune_ms[kNumPhases][kNumCandidates] = {};
  BatchLaunch L{};
  cudaGraphExec_t graph = nullptr;
  int graph_cycles = 0;
  int kernels_per_cycle = 0;
  long long kernels_launched = 0;
  long long cells = 0;
};

void destroy_plan(BatchPlan* p) {
  if (!p) return;
  if (p->graph) cudaGraphExecDestroy(p->graph);
  if (p->dmem) cudaFree(p->dmem);
  delete p;
}

// A run that is destroyed leaves the batch: the next batched call rebuilds
// the tables without it.
void plan_forget_run(BatchPlan* p, const hydro_run* r) {
  if (!p) return;
  auto it = std::find(p->runs.begin(), p->runs.end(), r);
  if (it != p->runs.end()) p->runs.clear();
}

namespace {

void drop_graph(BatchPlan* p) {
  if (p->graph) cudaGraphExecDestroy(p->graph);
  p->graph = nullptr;
  p->graph_cycles = 0;
}

int grid_for(const BatchPlan* p, int ph, int w, int mode) {
  const int on = phase_on_nodes(ph) ? 1 : 0;
  if (mode == 1) return (int)std::max<long long>(1, std::min<long long>(p->h_ntiles[on][w], 1 << 30));
  const int per_sm = std::max(1, p->blocks_per_sm[ph]);
  return std::max(1, per_sm * p->ctx->num_sms);
}

void fill_launch(BatchPlan* p) {
  BatchLaunch& L = p->L;
  L.views = p->d_views;
  L.ninst = p->d_ninst;
  L.max_inst = p->cap_inst;
  L.done = p->d_done;
  for (int on = 0; on < 2; ++on)
    for (int w = 0; w < kNumTileShapes; ++w) {
      L.tiles[on][w] = p->d_tiles[on][w];
      L.ntiles[on][w] = p->d_ntiles + on * kNumTileShapes + w;
    }
  L.any_order2 = 0;
  L.any_face = 0;
  L.any_face_grad = 0;
  L.variant = kBatchNoOrder3 | kBatchNoPB;
  L.any_vnr = 0;
  L.any_euc = 0;
  for (auto* r : p->runs) {
    if (r->v.scheme == HYDRO_SCHEME_EUCCLHYD) L.any_euc = 1;
    else L.any_vnr = 1;
    if (r->v.order > 1) L.any_order2 = 1;
    // the face phase serves order-3 runs and order-1 runs without PenteBorne
    if (r->v.order == 3 || (r->v.order == 1 && r->v.pb == 0)) L.any_face = 1;
    if (r->v.order == 2 && r->v.pb == 0) L.any_face_grad = 1;
    if (r->v.order == 3) L.variant &= ~kBatchNoOrder3;
    if (r->v.pb == 1) L.variant &= ~kBatchNoPB;
  }
  if (L.variant != p->occ_variant && batch_occupancy(p->blocks_per_sm, L.variant) == 0)
    p->occ_variant = L.variant;
  for (int ph = 0; ph < kNumPhases; ++ph) {
    L.shape[ph] = p->shape[ph];
    L.grid[ph] = grid_for(p, ph, p->shape[ph], p->mode[ph]);
  }
}

void make_tiles(const std::vector<hydro_run*>& runs, int on_nodes, int w,
                std::vector<Tile>& out) {
  const int twl = kTileShapes[w].tw_log2;
  const int tw = 1 << twl, th = (kBatchThreads >> twl) * kTileShapes[w].rows;
  out.clear();
  for (size_t r = 0; r < runs.size(); ++r) {
    const int H = runs[r]->v.ny + on_nodes, W = runs[r]->v.nx + on_nodes;
    for (int i0 = 0; i0 < H; i0 += th)
      for (int j0 = 0; j0 < W; j0 += tw) out.push_back(Tile{(int)r, i0, j0, 0});
  }
}

// Sets the plan's members; grows the device block when needed (which drops
// the captured graph, whose launches hold its addresses).
int set_members(BatchPlan* p, hydro_run* const* runs, int n) {
  std::vector<Tile> tiles[2][kNumTileShapes];
  std::vector<hydro_run*> rv(runs, runs + n);
  long long cells = 0;
  for (auto* r : rv) cells += r->v.nc;
  bool grow = n > p->cap_inst;
  for (int on = 0; on < 2; ++on)
    for (int w = 0; w < kNumTileShapes; ++w) {
      make_tiles(rv, on, w, tiles[on][w]);
      if ((long long)tiles[on][w].size() > p->cap_tiles[on][w]) grow = true;
    }
  cudaStream_t s = p->ctx->stream;
  if (grow) {
    drop_graph(p);
    if (p->dmem) {
      CUDA_TRY(cudaStreamSynchronize(s));
      CUDA_TRY(cudaFree(p->dmem));
      p->dmem = nullptr;
    }
    // room for 25% more runs / tiles than asked, so a serving loop whose
    // membership drifts does not re-allocate every time
    p->cap_inst = std::max(n + n / 4, 64);
    size_t bytes = 0;
    auto take = [&](size_t b) {
      size_t at = (bytes + 255) & ~(size_t)255;
      bytes = at + b;
      return at;
    };
    const size_t o_views = take(sizeof(RunView) * p->cap_inst);
    const size_t o_ninst = take(sizeof(int));
    const size_t o_done = take(sizeof(int) * p->cap_inst);
    const size_t o_nt = take(sizeof(int) * 2 * kNumTileShapes);
    size_t o_t[2][kNumTileShapes];
    for (int on = 0; on < 2; ++on)
      for (int w = 0; w < kNumTileShapes; ++w) {
        const long long need = (long long)tiles[on][w].size();
        p->cap_tiles[on][w] = std::max<long long>(need + need / 4, 1024);
        o_t[on][w] = take(sizeof(Tile) * p->cap_tiles[on][w]);
      }
    CUDA_TRY(cudaMalloc(&p->dmem, bytes));
    p->dbytes = bytes;
    p->d_views = reinterpret_cast<RunView*>(p->dmem + o_views);
    p->d_ninst = reinterpret_cast<int*>(p->dmem + o_ninst);
    p->d_done = reinterpret_cast<int*>(p->dmem + o_done);
    p->d_ntiles = reinterpret_cast<int*>(p->dmem + o_nt);
    for (int on = 0; on < 2; ++on)
      for (int w = 0; w < kNumTileShapes; ++w)
        p->d_tiles[on][w] = reinterpret_cast<Tile*>(p->dmem + o_t[on][w]);
  }
  std::vector<RunView> views(n);
  for (int r = 0; r < n; ++r) {
    views[r] = rv[r]->v;
    views[r].o3g = views[r].o3y = nullptr;  // order-3 values per face
  }
  int nt[2 * kNumTileShapes];
  for (int on = 0; on < 2; ++on)
    for (int w = 0; w < kNumTileShapes; ++w) {
      p->h_ntiles[on][w] = (long long)tiles[on][w].size();
      nt[on * kNumTileShapes + w] = (int)tiles[on][w].size();
    }
  // pageable sources: each copy returns once its data is staged, so the
  // host vectors may go out of scope; the copies stay ordered after the
  // launches already queued on the stream
  if (n)
    CUDA_TRY(cudaMemcpyAsync(p->d_views, views.data(), sizeof(RunView) * n,
                             cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(p->d_ninst, &n, sizeof(int), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(p->d_ntiles, nt, sizeof(nt), cudaMemcpyHostToDevice, s));
  for (int on = 0; on < 2; ++on)
    for (int w = 0; w < kNumTileShapes; ++w)
      if (!tiles[on][w].empty())
        CUDA_TRY(cudaMemcpyAsync(p->d_tiles[on][w], tiles[on][w].data(),
                                 sizeof(Tile) * tiles[on][w].size(),
                                 cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  // the flags that decide which kernels a cycle launches
  const int old_flags[6] = {p->L.any_order2, p->L.variant, p->L.any_face,
                            p->L.any_face_grad, p->L.any_vnr, p->L.any_euc};
  p->runs = rv;
  p->cells = cells;
  p->h_done.assign(n, 0);
  int old_grid[kNumPhases];
  memcpy(old_grid, p->L.grid, sizeof(old_grid));
  fill_launch(p);
  // the persistent grids do not depend on the membership; one-block-per-tile
  // grids and the slope phases do
  const int new_flags[6] = {p->L.any_order2, p->L.variant, p->L.any_face,
                            p->L.any_face_grad, p->L.any_vnr, p->L.any_euc};
  if (memcmp(old_grid, p->L.grid, sizeof(old_grid)) ||
      memcmp(old_flags, new_flags, sizeof(old_flags)))
    drop_graph(p);
  return 0;
}

int get_plan(hydro_ctx* ctx, hydro_run* const* runs, int n, BatchPlan** out) {
  if (n < 1) return fail(-1, "batch: no runs");
  for (int r = 0; r < n; ++r) {
    if (!runs[r]) return fail(-1, "batch: null run");
    if (runs[r]->ctx != ctx) return fail(-2, "batch: run belongs to another context");
    if (runs[r]->v.scheme != HYDRO_SCHEME_VNR && runs[r]->v.scheme != HYDRO_SCHEME_EUCCLHYD)
      return fail(-4, "batch: unknown scheme");
    if (runs[r]->v.projection != 1)
      return fail(-5, "batch: the batched form advances runs with the remap");
  }
  if (!ctx->plan) {
    auto* p = new BatchPlan();
    p->ctx = ctx;
    if (batch_occupancy(p->blocks_per_sm, 0)) {
      delete p;
      return fail(-3, "batch: occupancy query failed");
    }
    // defaults until (or without) tuning: the narrowest tile shape, one
    // block per tile
    for (int ph = 0; ph < kNumPhases; ++ph) p->mode[ph] = 1;
    if (!ctx->batch_tuning) p->tune_next = kNumCandidates + 1;
    ctx->plan = p;
  }
  BatchPlan* p = ctx->plan;
  const bool same = (int)p->runs.size() == n &&
                    std::equal(p->runs.begin(), p->runs.end(), runs);
  if (!same)
    if (int rc = set_members(p, runs, n)) return rc;
  *out = p;
  return 0;
}

int capture_graph(BatchPlan* p, int cycles) {
  cudaStream_t s = p->ctx->stream;
  drop_graph(p);
  cudaGraph_t g;
  CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int nk = 0;
  for (int k = 0; k < cycles; ++k) nk = launch_batch_cycle(p->L, s, nullptr);
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess)
    return fail(-40, std::string("batch graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&p->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return fail(-41, std::string("batch graph instantiate: ") + cudaGetErrorString(e));
  p->graph_cycles = cycles;
  p->kernels_per_cycle = nk;
  return 0;
}

// Runs one cycle with every phase in candidate configuration `cand` and
// records per-phase device times.  Candidate -1 is the untimed warm-up.
int tune_cycle(BatchPlan* p, int cand) {
  cudaStream_t s = p->ctx->stream;
  const int c = cand < 0 ? 0 : cand;
  for (int ph = 0; ph < kNumPhases; ++ph) {
    p->shape[ph] = c / kGridModes;
    p->mode[ph] = c % kGridModes;
  }
  fill_launch(p);
  std::vector<cudaEvent_t> ev;
  std::vector<int> kinds;
  LaunchHook hook = [&](int kind) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    ev.push_back(e);
    kinds.push_back(kind);
  };
  p->kernels_launched += launch_batch_cycle(p->L, s, &hook);
  CUDA_TRY(cudaStreamSynchronize(s));
  for (size_t i = 0; i + 1 < ev.size(); ++i) {
    const int ph = phase_of_kind(kinds[i]);
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
    if (ph >= 0 && cand >= 0) p->tune_ms[ph][cand] += t;
  }
  for (auto e : ev) cudaEventDestroy(e);
  return 0;
}

void finish_tuning(BatchPlan* p) {
  p->tuned = 1;
  for (int ph = 0; ph < kNumPhases; ++ph) {
    int best = 0;
    for (int c = 1; c < kNumCandidates; ++c)
      if (p->tune_ms[ph][c] < p->tune_ms[ph][best]) best = c;
    p->shape[ph] = best / kGridModes;
    p->mode[ph] = best % kGridModes;
  }
  fill_launch(p);
  drop_graph(p);
}

// Enqueues ncycles cycles of the plan (tuning cycles first while tuning is
// unfinished, then replays of a captured graph).
int enqueue_cycles(BatchPlan* p, int ncycles) {
  cudaStream_t s = p->ctx->stream;
  int left = ncycles;
  while (left > 0 && p->tune_next <= kNumCandidates) {
    if (int rc = tune_cycle(p, p->tune_next - 1)) return rc;
    ++p->tune_next;
    --left;
    if (p->tune_next == kNumCandidates + 1) finish_tuning(p);
  }
  if (left <= 0) return 0;
  const int G = 4;
  if (!p->graph && left >= G)
    if (int rc = capture_graph(p, G)) return rc;
  while (p->graph && left >= p->graph_cycles) {
    CUDA_TRY(cudaGraphLaunch(p->graph, s));
    left -= p->graph_cycles;
    p->kernels_launched += (long long)p->graph_cycles * p->kernels_per_cycle;
  }
  for (; left > 0; --left) p->kernels_launched += launch_batch_cycle(p->L, s, nullptr);
  CUDA_TRY(cudaGetLastError());
  return 0;
}

int read_done(BatchPlan* p, int* nactive) {
  cudaStream_t s = p->ctx->stream;
  const int n = (int)p->runs.size();
  CUDA_TRY(cudaMemcpyAsync(p->h_done.data(), p->d_done, sizeof(int) * n,
                           cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  int a = 0;
  for (int r = 0; r < n; ++r) a += p->h_done[r] ? 0 : 1;
  if (nactive) *nactive = a;
  return 0;
}

}  // namespace

// Used by the serving loop.
int batch_enqueue(hydro_ctx* ctx, hydro_run* const* runs, int n, int ncycles) {
  BatchPlan* p = nullptr;
  if (int rc = get_plan(ctx, runs, n, &p)) return rc;
  return enqueue_cycles(p, ncycles);
}

int batch_done_flags(hydro_ctx* ctx, std::vector<int>* done) {
  BatchPlan* p = ctx->plan;
  if (!p) return fail(-1, "batch: no plan");
  if (int rc = read_done(p, nullptr)) return rc;
  *done = p->h_done;
  return 0;
}

}  // namespace hydro

using namespace hydro;

extern "C" {

int hydro_batch_enqueue(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                        int ncycles) {
  if (!ctx || !runs) return fail(-1, "hydro_batch_enqueue: null argument");
  CUDA_TRY(cudaSetDevice(ctx->device));
  return batch_enqueue(ctx, runs, nruns, ncycles);
}

int hydro_batch_step(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                     int ncycles, int* nactive) {
  if (!ctx || !runs) return fail(-1, "hydro_batch_step: null argument");
  CUDA_TRY(cudaSetDevice(ctx->device));
  if (int rc = batch_enqueue(ctx, runs, nruns, ncycles)) return rc;
  return read_done(ctx->plan, nactive);
}

// Device time of ncycles batched cycles (CUDA events on the context's
// stream around the enqueued work).  Tuning cycles still pending run first,
// untimed.  Benchmark helper.
int hydro_batch_timed(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                      int ncycles, float* ms) {
  if (!ctx || !runs || !ms) return fail(-1, "hydro_batch_timed: null argument");
  CUDA_TRY(cudaSetDevice(ctx->device));
  BatchPlan* p = nullptr;
  if (int rc = get_plan(ctx, runs, nruns, &p)) return rc;
  if (p->tune_next <= kNumCandidates)
    if (int rc = enqueue_cycles(p, kNumCandidates + 1 - p->tune_next)) return rc;
  if (!p->graph)
    if (int rc = capture_graph(p, 4)) return rc;
  cudaStream_t s = ctx->stream;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  CUDA_TRY(cudaStreamSynchronize(s));
  CUDA_TRY(cudaEventRecord(e0, s));
  if (int rc = enqueue_cycles(p, ncycles)) return rc;
  CUDA_TRY(cudaEventRecord(e1, s));
  CUDA_TRY(cudaEventSynchronize(e1));
  CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return read_done(p, nullptr);
}

// Per-kernel-kind device times of ncycles batched cycles launched one by one
// with events between launches (same kind ids as hydro_run_profile).
int hydro_batch_profile(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                        int ncycles, double* ms, long long* launches, int nkinds) {
  if (!ctx || !runs || !ms || !launches || nkinds < kNumKernelKinds)
    return fail(-1, "hydro_batch_profile: bad arguments");
  CUDA_TRY(cudaSetDevice(ctx->device));
  BatchPlan* p = nullptr;
  if (int rc = get_plan(ctx, runs, nruns, &p)) return rc;
  cudaStream_t s = ctx->stream;
  for (int k = 0; k < nkinds; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  for (int c = 0; c < ncycles; ++c) {
    std::vector<cudaEvent_t> ev;
    std::vector<int> kinds;
    LaunchHook hook = [&](int kind) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      cudaEventRecord(e, s);
      ev.push_back(e);
      kinds.push_back(kind);
    };
    p->kernels_launched += launch_batch_cycle(p->L, s, &hook);
    CUDA_TRY(cudaStreamSynchronize(s));
    for (size_t i = 0; i + 1 < ev.size(); ++i) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      ms[kinds[i]] += t;
      launches[kinds[i]] += 1;
    }
    for (auto e : ev) cudaEventDestroy(e);
  }
  return read_done(p, nullptr);
}

// Chosen tile width and height (items) and grid size (blocks) per batched
// phase, in BatchPhase order; returns 1 when a timed tuning pass chose them,
// 0 for the defaults (tuning off or unfinished).
int hydro_batch_config(hydro_ctx* ctx, int* width, int* height, int* grid,
                       int nphases) {
  if (!ctx || !width || !height || !grid || nphases < kNumPhases)
    return fail(-1, "hydro_batch_config: bad arguments");
  BatchPlan* p = ctx->plan;
  if (!p) return fail(-2, "hydro_batch_config: no batch has run");
  for (int ph = 0; ph < kNumPhases; ++ph) {
    const TileShape& t = kTileShapes[p->L.shape[ph]];
    width[ph] = 1 << t.tw_log2;
    height[ph] = (kBatchThreads >> t.tw_log2) * t.rows;
    grid[ph] = p->L.grid[ph];
  }
  return p->tuned;
}

// Turns the batch autotuner on (default) or off (32 x 4 tiles, one block
// per tile) for plans created afterwards.
int hydro_batch_set_tuning(hydro_ctx* ctx, int enable) {
  if (!ctx) return fail(-1, "hydro_batch_set_tuning: null context");
  ctx->batch_tuning = enable ? 1 : 0;
  if (ctx->plan) {
    destroy_plan(ctx->plan);
    ctx->plan = nullptr;
  }
  return 0;
}

long long hydro_batch_kernel_launches(hydro_ctx* ctx) {
  return (ctx && ctx->plan) ? ctx->plan->kernels_launched : 0;
}

}  // extern "C"
