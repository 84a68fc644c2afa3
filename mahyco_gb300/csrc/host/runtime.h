// Host runtime objects shared by the plain runner, the batch engine and the
// serving loop (CUDA translation units only).
#ifndef MAHYCO_GB300_RUNTIME_H
#define MAHYCO_GB300_RUNTIME_H

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../internal.h"
#include "init.h"

namespace hydro {

void launch_prologue(const RunView& v, cudaStream_t s);
int launch_device_init(const RunView& v, int test_case, int init_variant, cudaStream_t s);
int launch_cycle(const RunView& v, cudaStream_t s, const LaunchHook* hook);
void launch_node_mass(const RunView& v, cudaStream_t s);
int launch_euc_out_pressure(const RunView& v, double* out, cudaStream_t s);
int launch_batch_cycle(const BatchLaunch& L, cudaStream_t s, const LaunchHook* hook);
int batch_occupancy(int* blocks_per_sm, int variant);
int measure_fp64_peak(int device, double* tflops);

#define CUDA_TRY(expr)                                                       \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return ::hydro::fail(-100, std::string(#expr) + ": " +                 \
                                     cudaGetErrorString(e_));                \
  } while (0)

// A run whose initial state is built on the host but not yet placed on the
// device (run creation split in two so that a serving loop can prepare runs
// on worker threads while the GPU is busy).
struct PreparedRun {
  hydro_spec spec{};
  HostInit h;
  RunView v{};
  size_t bytes = 0;
};
int prepare_run(const hydro_spec& spec, PreparedRun& out);
// build_state = false leaves the cleared arena for the caller to fill (a
// restart from a checkpoint)
int place_run(hydro_ctx* ctx, PreparedRun& pr, hydro_run** out, bool wait,
              bool build_state = true);
size_t run_arena_bytes(const hydro_spec& spec);

struct BatchPlan;
struct ServeState;
struct FetchStage;
int create_fetch_stage(int num_sms, FetchStage** out);
void destroy_fetch_stage(FetchStage* st);
void destroy_plan(BatchPlan* p);
void plan_forget_run(BatchPlan* p, const struct ::hydro_run* r);
void destroy_serve(ServeState* s);

}  // namespace hydro

struct hydro_ctx {
  int device = 0;
  int num_sms = 0;
  size_t budget = 0;       // bytes of run state the context may hold (0: no cap)
  size_t used = 0;         // bytes of run state held
  cudaStream_t stream = nullptr;
  std::mutex mu;
  hydro::BatchPlan* plan = nullptr;   // batch engine (lazily created)
  hydro::ServeState* serve = nullptr; // serving loop (lazily created)
  hydro::FetchStage* fetch = nullptr; // pinned staging of hydro_run_fetch
  int batch_tuning = 1;               // autotune the batched launches
};

struct hydro_run {
  hydro_ctx* ctx = nullptr;
  hydro_spec spec{};
  hydro::RunView v{};
  double dt_init = 0.0;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  hydro::Ctrl* d_ctrl = nullptr;
  hydro::Ctrl h_ctrl{};
  cudaGraphExec_t graph = nullptr;
  int graph_cycles = 0;
  int kernels_per_cycle = 0;
  long long kernels_launched = 0;
};

#endif
