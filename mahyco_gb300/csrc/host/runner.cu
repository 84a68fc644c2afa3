// Host runtime of the GB300 hydro path: context, per-run HBM arena, cycle
// loop (CUDA-graph replay), field fetch and the public C ABI of
// include/hydro_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fetch.h"
#include "init.h"
#include "runtime.h"

namespace hydro {

static thread_local std::string g_last_error;

int fail(int rc, const std::string& msg) {
  g_last_error = msg;
  return rc;
}

}  // namespace hydro

using namespace hydro;

namespace {

long long round_up(long long n, long long a) { return (n + a - 1) / a * a; }

// Bump allocator over one device allocation.
struct Carve {
  char* base;
  size_t off = 0;
  template <class T>
  T* take(long long count) {
    size_t bytes = (size_t)count * sizeof(T);
    size_t at = (off + 255) & ~(size_t)255;
    off = at + bytes;
    return base ? reinterpret_cast<T*>(base + at) : nullptr;
  }
};

// The fused remap sweeps measured slower than the separate slope and update
// kernels on GB300 (the kernels are latency-bound; a tile's barrier between
// its slope and update phases idles warps), so they run only on request.
bool fused_sweeps_requested() {
  const char* e = std::getenv("MAHYCO_GB300_FUSED_SWEEPS");
  return e && e[0] == '1';
}

// Lays out every device array of a run; with base == nullptr it only sizes.
size_t layout(RunView& v, char* base) {
  Carve a{base};
  const long long P = v.pitch, NP = v.npitch, FP = v.fpitch;
  const int nb = v.nbmat, nc = v.ncomp;
  v.rho = a.take<double>(P);
  v.p = a.take<double>(P);
  v.c = a.take<double>(P);
  v.e = a.take<double>(P);
  v.q = a.take<double>(P);
  v.divu = a.take<double>(P);
  v.cell_mass = a.take<double>(P);
  v.rhom = a.take<double>(nb * P);
  v.pm = a.take<double>(nb * P);
  v.cm = a.take<double>(nb * P);
  v.em = a.take<double>(nb * P);
  v.qm = a.take<double>(nb * P);
  v.fm = a.take<double>(nb * P);
  v.mfm = a.take<double>(nb * P);
  v.cmassm = a.take<double>(nb * P);
  v.mixte = a.take<int>(P);
  v.pure = a.take<int>(P);
  v.u = a.take<double>(2 * NP);
  v.node_mass = a.take<double>(NP);
  v.speed = a.take<double>(NP);
  v.XN = (v.projection == 0) ? a.take<double>(2 * NP) : nullptr;
  v.vout = (v.projection == 0) ? a.take<double>(2 * NP) : nullptr;
  v.XL = a.take<double>(2 * NP);
  v.vL = a.take<double>(P);
  v.rL = a.take<double>(P);
  v.XcL = a.take<double>(2 * P);
  v.Hx = a.take<double>(P);
  v.Hy = a.take<double>(P);
  v.UL = a.take<double>(nc * P);
  v.Phi = a.take<double>(nc * P);
  v.U1 = a.take<double>(nc * P);
  v.gP = a.take<double>(nc * P);
  v.dPAv = a.take<double>(nc * P);
  v.dPAr = a.take<double>(nc * P);
  v.pbz = a.take<unsigned char>(P);
  v.u1s = a.take<unsigned char>(P);
  v.DPF = a.take<double>(nb * P);
  // face gradients of runs without PenteBorne (the slope kernel reads them
  // while it writes face values into phiF): the plateau-slope integral
  // planes, which those runs never use (2 nc cell planes hold nc face
  // planes: FP <= 2 P for nx, ny >= 2)
  v.phiG = v.dPAv;
  // the fused sweeps (opt-in: MAHYCO_GB300_FUSED_SWEEPS=1 when the run is
  // created) keep the integrals on chip: dPAv holds the first sweep's Phi of
  // the cells it changes
  v.Phi2 = (fused_sweeps_ok(v) && fused_sweeps_requested()) ? v.dPAv : nullptr;
  v.phiF = a.take<double>(nc * FP);
  v.FFd = a.take<double>(nb * P);
  if (v.order == 3) {
    v.o3g = a.take<double>(nc * P);
    v.o3c = a.take<double>(16 * P);
    v.o3y = a.take<double>(nc * FP);
  } else {
    v.o3g = v.o3y = nullptr;
    v.o3c = nullptr;
  }
  v.DPv = a.take<double>(2 * NP);
  v.gD = a.take<double>(2 * NP);
  v.UD1 = a.take<double>(3 * NP);
  v.xs = a.take<double>(v.nx + 1);
  v.ys = a.take<double>(v.ny + 1);
  if (v.scheme == HYDRO_SCHEME_EUCCLHYD) {
    v.cqs = v.cflsq = v.s0 = v.sqs0 = nullptr;
    v.sarg = nullptr;
    v.nsym = nullptr;
    v.gL = nullptr;
    v.geo0 = a.take<double>(5 * P);
    v.uc = a.take<double>(2 * P);
    v.uco = a.take<double>(2 * P);
    v.vg = a.take<double>(4 * P);
    v.Fs = a.take<double>(2 * nb * P);
    v.pex = a.take<double>(4 * P);
    v.uex = a.take<double>(8 * P);
    v.peex = a.take<double>(4 * nb * P);
    v.lpc = a.take<double>(8 * P);
    v.cmat = a.take<double>(12 * P);
    v.xcc = a.take<double>(2 * P);
    v.perim = a.take<double>(P);
    v.evol = a.take<double>(P);
  } else {
    v.geo0 = a.take<double>(5 * P);
    v.gL = a.take<unsigned char>(P);
    v.sarg = a.take<double>(P);
    v.nsym = a.take<unsigned char>(NP);
    v.cqs = a.take<double>(8 * P);
    v.cflsq = a.take<double>(P);
    v.s0 = a.take<double>(P);
    v.sqs0 = a.take<double>(P);
  }
  v.nout = a.take<double>(4 * P);
  v.flv = a.take<double>(v.ny);
  v.flh = a.take<double>(v.nx);
  v.rho0_left = a.take<double>(v.ny);
  v.ctrl = a.take<Ctrl>(1);
  return a.off + 256;
}

int validate(const hydro_spec& s) {
  if (s.scheme != HYDRO_SCHEME_VNR && s.scheme != HYDRO_SCHEME_EUCCLHYD)
    return fail(-20, "unknown Lagrange scheme");
  if (s.projection != 1 &&
      !(s.projection == 0 && s.scheme == HYDRO_SCHEME_VNR && s.sans_lagrange == 0))
    return fail(-21, "without the remap (AvecProjection = non) the GPU path runs the "
                     "VNR scheme with its Lagrange phase only");
  if (s.nbmat < 1 || s.nbmat > 3) return fail(-22, "nbmat must be 1..3");
  if (s.projection_order < 1 || s.projection_order > 3)
    return fail(-23, "projection order must be 1, 2 or 3");
  if (s.nx < 2 || s.ny < 2) return fail(-24, "nx and ny must be >= 2");
  for (int m = 0; m < s.nbmat; ++m)
    if (s.eos[m] != HYDRO_EOS_PERFECT_GAS && s.eos[m] != HYDRO_EOS_VOID)
      return fail(-25, "only PerfectGas and Void equations of state exist in "
                       "the reference (others only print)");
  if (s.dual_mass_flux < 0 || s.dual_mass_flux > 2)
    return fail(-26, "dual mass-flux method must be A1, A2 or PB");
  if (s.scheme == HYDRO_SCHEME_VNR && s.dual_mass_flux == 2 &&
      !(s.pb == 1 && s.projection_order > 1))
    return fail(-27, "the PB dual mass flux needs PenteBorne and order > 1");
  if (s.scheme == HYDRO_SCHEME_EUCCLHYD && s.space_order != 1 && s.space_order != 2)
    return fail(-28, "the Eucclhyd space order must be 1 or 2");
  return 0;
}

}  // namespace

extern "C" {

const char* hydro_last_error(void) { return g_last_error.c_str(); }

int hydro_ctx_create(int device, size_t budget, hydro_ctx** out) {
  if (!out) return fail(-1, "hydro_ctx_create: null out");
  int n = 0;
  CUDA_TRY(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n)
    return fail(-2, "hydro_ctx_create: no CUDA device " + std::to_string(device));
  CUDA_TRY(cudaSetDevice(device));
  auto* c = new hydro_ctx();
  c->device = device;
  c->budget = budget;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(-3, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
  }
  // the pinned staging and host copy threads of hydro_run_fetch, set up
  // with the context rather than inside a run's first fetch
  if (int rc = create_fetch_stage(c->num_sms, &c->fetch)) {
    cudaStreamDestroy(c->stream);
    delete c;
    return rc;
  }
  *out = c;
  return 0;
}

void hydro_ctx_destroy(hydro_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  destroy_serve(c->serve);
  c->serve = nullptr;
  destroy_plan(c->plan);
  c->plan = nullptr;
  if (c->stream) cudaStreamSynchronize(c->stream);
  destroy_fetch_stage(c->fetch);
  c->fetch = nullptr;
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

}  // extern "C"

namespace hydro {

// Host part of run creation: validation, initial state, sizes and options
// of the device view (no CUDA call; safe on any thread).
int prepare_run(const hydro_spec& spec_in, PreparedRun& pr) {
  if (int rc = validate(spec_in)) return rc;
  pr.spec = spec_in;
  const hydro_spec* spec = &pr.spec;
  const bool euc = spec->scheme == HYDRO_SCHEME_EUCCLHYD;
  if (int rc = euc ? init_options_euc(*spec, pr.h) : init_options(*spec, pr.h)) return rc;
  const HostInit& h = pr.h;
  RunView& v = pr.v;
  v = RunView{};
  v.nx = spec->nx;
  v.ny = spec->ny;
  v.nc = h.nc;
  v.nn = h.nn;
  v.pitch = round_up(h.nc, 32);
  v.npitch = round_up(h.nn, 32);
  v.fpitch = round_up(std::max((long long)(spec->nx + 1) * spec->ny,
                               (long long)spec->nx * (spec->ny + 1)),
                      32);
  v.nbmat = spec->nbmat;
  v.scheme = spec->scheme;
  for (int k = 0; k < kMaxComp; ++k) v.comp_ref[k] = -1;
  if (euc) {
    // volumes, masses, energies, momentum x / y (+ kinetic energy)
    v.ncomp = 3 * spec->nbmat + 2 + (spec->projection_conservative == 1 ? 1 : 0);
    for (int k = 0; k < v.ncomp; ++k) v.comp_ref[k] = k;
  } else {
    v.ncomp = 3 * spec->nbmat + 1;
    for (int k = 0; k < 3 * spec->nbmat; ++k) v.comp_ref[k] = k;
    v.comp_ref[3 * spec->nbmat] = 3 * spec->nbmat + 3;
  }
  v.space_order = spec->space_order;
  v.euc_cfl = spec->cfl;
  v.order = spec->projection_order;
  v.pb = spec->pb;
  v.pb_mixte = spec->pb_mixte;
  v.pb_complet = spec->pb_complet;
  v.limiter = spec->limiter;
  v.limiter_pure = spec->limiter_pure;
  v.dual_method = spec->dual_mass_flux;
  v.pseudo_centree = spec->pseudo_centree;
  v.sans_lagrange = spec->sans_lagrange;
  v.projection = spec->projection;
  v.conservative = spec->projection_conservative;
  for (int m = 0; m < 3; ++m) {
    v.eos[m] = spec->eos[m];
    v.gamma[m] = spec->gamma[m];
  }
  v.threshold = spec->threshold;
  v.gamma_scalar = spec->gamma_scalar;
  for (int m = 0; m < 3; ++m) {
    v.gm1[m] = v.gamma[m] - 1.0;
    v.hgm1[m] = v.gm1[m] * 0.5;
  }
  v.g0gm1 = v.gamma[0] * v.gm1[0];
  v.hgs1 = (v.gamma_scalar + 1) * 0.5;
  v.energy_limit = spec->energy_limit;
  v.dx = spec->dx;
  v.dy = spec->dy;
  v.euler_volume = spec->dx * spec->dy;
  v.dt_min = spec->dt_min;
  v.final_time = spec->final_time;
  v.cfl = spec->cfl;
  v.max_iter = spec->max_cycles > 0 ? spec->max_cycles + 1 : 500000000LL;
  v.bc_left = h.bc_left;
  v.bc_right = h.bc_right;
  v.bc_bottom = h.bc_bottom;
  v.bc_top = h.bc_top;
  for (int d = 0; d < 2; ++d) {
    v.v_left[d] = h.v_left[d];
    v.v_right[d] = h.v_right[d];
    v.v_bottom[d] = h.v_bottom[d];
    v.v_top[d] = h.v_top[d];
  }
  v.periodic_x = h.periodic_x;
  v.flux_bc = h.flux_bc;
  pr.bytes = layout(v, nullptr);
  return 0;
}

// Bytes of a run's arena for spec (layout sizes only).
size_t run_arena_bytes(const hydro_spec& spec) {
  RunView v{};
  const long long nc = (long long)spec.nx * spec.ny;
  const long long nn = (long long)(spec.nx + 1) * (spec.ny + 1);
  v.nx = spec.nx;
  v.ny = spec.ny;
  v.pitch = round_up(nc, 32);
  v.npitch = round_up(nn, 32);
  v.fpitch = round_up(std::max((long long)(spec.nx + 1) * spec.ny,
                               (long long)spec.nx * (spec.ny + 1)),
                      32);
  v.nbmat = spec.nbmat;
  v.scheme = spec.scheme;
  v.order = spec.projection_order;
  v.ncomp = spec.scheme == HYDRO_SCHEME_EUCCLHYD
                ? 3 * spec.nbmat + 2 + (spec.projection_conservative == 1 ? 1 : 0)
                : 3 * spec.nbmat + 1;
  return layout(v, nullptr);
}

// Device part: allocates the run's arena and queues, on the context's
// stream, its clearing, the control block's upload, the device kernels that
// build the initial state and geometry, and the prologue.  With wait,
// returns once they have run; without, the caller orders later work on the
// same stream (the control block is staged before this returns, so `pr` may
// be released at once).
int place_run(hydro_ctx* ctx, PreparedRun& pr, hydro_run** out, bool wait, bool build_state) {
  CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t bytes = pr.bytes;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->budget && ctx->used + bytes > ctx->budget)
      return fail(-30, "HBM budget exceeded");
    ctx->used += bytes;
  }
  auto* r = new hydro_run();
  r->ctx = ctx;
  r->spec = pr.spec;
  r->v = pr.v;
  r->dt_init = pr.h.dt_init;
  RunView& v = r->v;
  const HostInit& h = pr.h;
  cudaError_t e = cudaMalloc(&r->arena, bytes);
  if (e != cudaSuccess) {
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      ctx->used -= bytes;
    }
    delete r;
    return fail(-31, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  r->arena_bytes = bytes;
  layout(v, (char*)r->arena);
  r->d_ctrl = v.ctrl;
  cudaStream_t s = ctx->stream;
  int rc = 0;
  if (cudaMemsetAsync(r->arena, 0, bytes, s) != cudaSuccess)
    rc = fail(-32, "arena clear");
  Ctrl c0{};
  c0.t_n = 0.0;
  c0.dt_n = h.dt_init;
  c0.n = 0;
  c0.done = 0;
  c0.active = 0;
  c0.x_then_y = 1;
  c0.err = 0;
  c0.err_cell = LLONG_MAX;
  c0.dt_min_bits = 0xFFEFFFFFFFFFFFFFull;  // ordered encoding of +DBL_MAX
  c0.pmax_bits = 0x0010000000000000ull;    // ordered encoding of -DBL_MAX
  r->h_ctrl = c0;
  // the control block is the only host -> device copy (pageable, staged at
  // once); the initial state is built in place by the device
  if (!rc && build_state &&
      cudaMemcpyAsync(r->d_ctrl, &r->h_ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
    rc = fail(-33, "ctrl upload");
  if (!rc && build_state) launch_device_init(v, pr.spec.test_case, pr.spec.init_variant, s);
  if (!rc && build_state && v.scheme == HYDRO_SCHEME_VNR) launch_prologue(v, s);
  if (!rc && cudaGetLastError() != cudaSuccess) rc = fail(-34, "prologue launch");
  if (!rc && wait && cudaStreamSynchronize(s) != cudaSuccess)
    rc = fail(-34, std::string("initial upload: ") +
                       cudaGetErrorString(cudaGetLastError()));
  if (rc) {
    cudaStreamSynchronize(s);
    cudaFree(r->arena);
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      ctx->used -= bytes;
    }
    delete r;
    return rc;
  }
  *out = r;
  return 0;
}

}  // namespace hydro

extern "C" {

int hydro_run_create(hydro_ctx* ctx, const hydro_spec* spec, hydro_run** out) {
  if (!ctx || !spec || !out) return fail(-1, "hydro_run_create: null argument");
  PreparedRun pr;
  if (int rc = prepare_run(*spec, pr)) return rc;
  return place_run(ctx, pr, out, true);
}

int hydro_run_destroy(hydro_run* r) {
  if (!r) return 0;
  cudaSetDevice(r->ctx->device);
  plan_forget_run(r->ctx->plan, r);
  if (r->graph) cudaGraphExecDestroy(r->graph);
  if (r->arena) cudaFree(r->arena);
  {
    std::lock_guard<std::mutex> lk(r->ctx->mu);
    r->ctx->used -= r->arena_bytes;
  }
  delete r;
  return 0;
}

}  // extern "C"

namespace {

// Captures `cycles` consecutive cycles of one run into a CUDA graph.
int build_graph(hydro_run* r, int cycles) {
  cudaStream_t s = r->ctx->stream;
  if (r->graph) {
    cudaGraphExecDestroy(r->graph);
    r->graph = nullptr;
  }
  cudaGraph_t g;
  CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int nk = 0;
  for (int k = 0; k < cycles; ++k) nk = launch_cycle(r->v, s, nullptr);
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess) return fail(-40, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&r->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(-41, std::string("graph instantiate: ") + cudaGetErrorString(e));
  r->graph_cycles = cycles;
  r->kernels_per_cycle = nk;
  return 0;
}

int sync_ctrl(hydro_run* r) {
  cudaStream_t s = r->ctx->stream;
  CUDA_TRY(cudaMemcpyAsync(&r->h_ctrl, r->d_ctrl, sizeof(Ctrl),
                           cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return 0;
}

}  // namespace

extern "C" {

// Enqueues ncycles cycles without waiting (graph replays of 8 cycles plus
// single-cycle launches for the remainder).
int hydro_run_enqueue(hydro_run* r, int ncycles) {
  if (!r) return fail(-1, "null run");
  CUDA_TRY(cudaSetDevice(r->ctx->device));
  const int G = 8;
  if (!r->graph) {
    if (int rc = build_graph(r, G)) return rc;
  }
  cudaStream_t s = r->ctx->stream;
  int left = ncycles;
  while (left >= r->graph_cycles) {
    CUDA_TRY(cudaGraphLaunch(r->graph, s));
    left -= r->graph_cycles;
    r->kernels_launched += (long long)r->graph_cycles * r->kernels_per_cycle;
  }
  for (int k = 0; k < left; ++k) {
    r->kernels_launched += launch_cycle(r->v, s, nullptr);
  }
  CUDA_TRY(cudaGetLastError());
  return 0;
}

int hydro_run_step(hydro_run* r, int ncycles, int* done) {
  if (!r) return fail(-1, "null run");
  if (int rc = hydro_run_enqueue(r, ncycles)) return rc;
  if (int rc = sync_ctrl(r)) return rc;
  if (done) *done = r->h_ctrl.done;
  return 0;
}

// Arms or disarms the output pause in the device control block (stream
// ordered, so it takes effect between cycles).
static int set_pause(hydro_run* r, int on, double t_out) {
  Ctrl& h = r->h_ctrl;
  h.t_out = t_out;
  h.pause = on;
  h.pause_skip = on;
  h.paused = 0;
  static_assert(offsetof(Ctrl, pad3) == offsetof(Ctrl, t_out) + sizeof(double) + 3 * sizeof(int),
                "pause fields are contiguous");
  CUDA_TRY(cudaMemcpyAsync(&r->d_ctrl->t_out, &h.t_out,
                           sizeof(double) + 3 * sizeof(int), cudaMemcpyHostToDevice,
                           r->ctx->stream));
  return 0;
}

int hydro_run_step_to_output(hydro_run* r, int ncycles, double t_out, int* done,
                             int* paused) {
  if (!r) return fail(-1, "null run");
  if (ncycles < 1) return fail(-1, "hydro_run_step_to_output: ncycles < 1");
  CUDA_TRY(cudaSetDevice(r->ctx->device));
  if (int rc = sync_ctrl(r)) return rc;
  if (done) *done = r->h_ctrl.done;
  if (paused) *paused = 0;
  if (r->h_ctrl.done) return 0;
  if (int rc = set_pause(r, 1, t_out)) return rc;
  int left = ncycles, rc = 0;
  while (left > 0 && !rc) {
    // cycles to the next output at the current time step (the step grows by
    // at most 5% a cycle), so that few cycles are enqueued past the pause
    const Ctrl& c = r->h_ctrl;
    double est = 64.0;
    if (c.dt_n > 0.0 && t_out > c.t_n) {
      const double e = (t_out - c.t_n) / c.dt_n + 1.0;
      if (e < est) est = e;
    }
    const int chunk = std::min(left, std::max(1, (int)est));
    rc = hydro_run_enqueue(r, chunk);
    if (!rc) rc = sync_ctrl(r);
    left -= chunk;
    if (!rc && (r->h_ctrl.done || r->h_ctrl.paused)) break;
  }
  const int was_paused = rc ? 0 : r->h_ctrl.paused;
  const int rc2 = set_pause(r, 0, 0.0);
  if (rc) return rc;
  if (rc2) return rc2;
  if (done) *done = r->h_ctrl.done;
  if (paused) *paused = was_paused;
  return 0;
}

int hydro_run_sync(hydro_run* r, int* done) {
  if (!r) return fail(-1, "null run");
  if (int rc = sync_ctrl(r)) return rc;
  if (done) *done = r->h_ctrl.done;
  return 0;
}

int hydro_run_time(hydro_run* r, double* t, double* dt, long* cycle) {
  if (!r) return fail(-1, "null run");
  if (int rc = sync_ctrl(r)) return rc;
  if (t) *t = r->h_ctrl.t_n;
  if (dt) *dt = r->h_ctrl.dt_n;
  if (cycle) *cycle = (long)r->h_ctrl.n;
  return 0;
}

int hydro_run_error(hydro_run* r, unsigned* code, long* cell) {
  if (!r) return fail(-1, "null run");
  if (int rc = sync_ctrl(r)) return rc;
  if (code) *code = r->h_ctrl.err;
  if (cell) *cell = r->h_ctrl.err_cell == LLONG_MAX ? -1 : (long)r->h_ctrl.err_cell;
  return 0;
}

long long hydro_run_kernel_launches(hydro_run* r) {
  return r ? r->kernels_launched : 0;
}

// The variables the reference's dumpVariables hands to its VTK writer, by
// the names it gives them (vnr_remap/VnrRemap.cc:264-278,
// eucclhyd_remap/EucclhydRemap.cc:43-50).  Returns the material / component
// index the name selects, -1 for other names.
static int dump_plane(hydro_run* r, const char* f) {
  static const char* common[] = {"Pressure", "Density", "Energy"};
  for (auto n : common)
    if (!strcmp(f, n)) return 0;
  if (r->v.scheme == HYDRO_SCHEME_EUCCLHYD) {
    static const char* euc[] = {"F1", "F2", "F3"};
    for (int m = 0; m < 3; ++m)
      if (!strcmp(f, euc[m])) return m;
    if (!strcmp(f, "VelocityX")) return 0;
    if (!strcmp(f, "VelocityY")) return 1;
    return -1;
  }
  if (!strcmp(f, "fracvol1")) return 0;
  if (!strcmp(f, "fracvol2")) return 1;
  if (!strcmp(f, "VitesseX")) return 0;
  if (!strcmp(f, "VitesseY")) return 1;
  return -1;
}
static bool dump_on_nodes(hydro_run* r, const char* f) {
  return r->v.scheme == HYDRO_SCHEME_VNR && (!strcmp(f, "VitesseX") || !strcmp(f, "VitesseY"));
}

// Copies one dump variable (see dump_plane) into dst.  Eucclhyd's Pressure
// is the mean pressure of the current state as computeEOS +
// computePressionMoyenne give it at the start of the next cycle, where the
// reference dumps it; its VelocityX/Y are the clamped output velocities the
// final remap kernel keeps.  Material slots beyond nbmat read as zero.
static int fetch_dump(hydro_run* r, const char* f, int k, double* dst, size_t n) {
  const RunView& v = r->v;
  cudaStream_t s = r->ctx->stream;
  const double* plane = nullptr;
  double* scratch = nullptr;
  const bool euc = v.scheme == HYDRO_SCHEME_EUCCLHYD;
  if (!strcmp(f, "Density")) plane = v.rho;
  else if (!strcmp(f, "Energy")) plane = v.e;
  else if (!strcmp(f, "Pressure")) {
    if (euc) {
      CUDA_TRY(cudaMalloc(&scratch, v.nc * sizeof(double)));
      launch_euc_out_pressure(v, scratch, s);
      r->kernels_launched += 1;
      plane = scratch;
    } else {
      plane = v.p;
    }
  } else if (!strcmp(f, "VelocityX") || !strcmp(f, "VelocityY")) {
    plane = v.uco + k * v.pitch;
  } else if (!strcmp(f, "VitesseX") || !strcmp(f, "VitesseY")) {
    // m_x/y_velocity: without the remap only the interior nodes' are
    // refreshed (updateVelocity), a separate plane (vout) keeps that
    plane = (v.vout ? v.vout : v.u) + k * v.npitch;
  } else if (k < v.nbmat) {
    plane = v.fm + k * v.pitch;
  }
  if (!plane) {
    for (size_t i = 0; i < n; ++i) dst[i] = 0.0;
    return 0;
  }
  const int rc = fetch_planes(r->ctx, FetchPlanes{{plane, nullptr, nullptr}, 1}, (long long)n,
                              dst, &r->kernels_launched);
  if (scratch) {
    const cudaError_t e = cudaFree(scratch);
    if (!rc && e != cudaSuccess)
      return fail(-100, std::string("fetch ") + f + ": " + cudaGetErrorString(e));
  }
  return rc;
}

size_t hydro_run_field_size(hydro_run* r, const char* f) {
  if (!r || !f) return 0;
  const size_t nc = (size_t)r->v.nc, nn = (size_t)r->v.nn;
  static const char* cell1[] = {"density", "pressure", "energy", "sound_speed",
                                "pseudo", "divu", "cell_mass"};
  for (auto n : cell1)
    if (!strcmp(f, n)) return nc;
  static const char* cell3[] = {"density_env", "energy_env", "pressure_env",
                                "fracvol_env", "mass_fraction_env"};
  for (auto n : cell3)
    if (!strcmp(f, n)) return 3 * nc;
  if (!strcmp(f, "node_velocity")) return 2 * nn;
  if (!strcmp(f, "node_coord")) return 2 * nn;
  if (dump_plane(r, f) >= 0) return dump_on_nodes(r, f) ? nn : nc;
  if (r->v.scheme == HYDRO_SCHEME_EUCCLHYD) {
    if (!strcmp(f, "cell_velocity")) return 2 * nc;
    return 0;
  }
  if (!strcmp(f, "node_mass")) return nn;
  return 0;
}

// Copies a field to host memory.  Per-material fields use the reference's
// layout (3 values per cell, zero for absent material slots); node_velocity
// is (u, v) per node.
int hydro_run_fetch(hydro_run* r, const char* f, double* dst, size_t n) {
  if (!r || !f || !dst) return fail(-1, "hydro_run_fetch: null argument");
  const size_t want = hydro_run_field_size(r, f);
  if (!want) return fail(-2, std::string("unknown field ") + f);
  if (n != want) return fail(-3, "hydro_run_fetch: wrong size for " + std::string(f));
  CUDA_TRY(cudaSetDevice(r->ctx->device));
  cudaStream_t s = r->ctx->stream;
  const RunView& v = r->v;
  const long long nn = v.nn;
  if (const int k = dump_plane(r, f); k >= 0) return fetch_dump(r, f, k, dst, n);
  FetchPlanes g{{nullptr, nullptr, nullptr}, 1};
  if (!strcmp(f, "density")) g.p[0] = v.rho;
  else if (!strcmp(f, "pressure")) g.p[0] = v.p;
  else if (!strcmp(f, "energy")) g.p[0] = v.e;
  else if (!strcmp(f, "sound_speed")) g.p[0] = v.c;
  else if (!strcmp(f, "pseudo")) g.p[0] = v.q;
  else if (!strcmp(f, "divu")) g.p[0] = v.divu;
  else if (!strcmp(f, "cell_mass")) g.p[0] = v.cell_mass;
  else if (!strcmp(f, "node_mass")) {
    launch_node_mass(v, s);
    g.p[0] = v.node_mass;
  }
  // per-material planes, three values per cell (zeros past the run's
  // materials)
  const double* planes = nullptr;
  if (!strcmp(f, "density_env")) planes = v.rhom;
  else if (!strcmp(f, "energy_env")) planes = v.em;
  else if (!strcmp(f, "pressure_env")) planes = v.pm;
  else if (!strcmp(f, "fracvol_env")) planes = v.fm;
  else if (!strcmp(f, "mass_fraction_env")) planes = v.mfm;
  if (planes) {
    g.k = 3;
    for (int m = 0; m < v.nbmat && m < 3; ++m) g.p[m] = planes + m * v.pitch;
  }
  if (!strcmp(f, "node_coord")) {
    // the mesh the next output shows: the moving positions of a run without
    // the remap, the Euler mesh (dx * j, dy * i) otherwise
    if (!v.XN) {
      for (long long p = 0; p < nn; ++p) {
        const long long i = p / (v.nx + 1), j = p - i * (v.nx + 1);
        dst[2 * p] = v.dx * (double)j;
        dst[2 * p + 1] = v.dy * (double)i;
      }
      return 0;
    }
    g = FetchPlanes{{v.XN, v.XN + v.npitch, nullptr}, 2};
  } else if (!strcmp(f, "node_velocity")) {
    g = FetchPlanes{{v.u, v.u + v.npitch, nullptr}, 2};
  } else if (!strcmp(f, "cell_velocity")) {
    g = FetchPlanes{{v.uc, v.uc + v.pitch, nullptr}, 2};
  }
  if (!g.p[0] && !planes) return fail(-2, std::string("unknown field ") + f);
  return fetch_planes(r->ctx, g, (long long)(n / g.k), dst, &r->kernels_launched);
}

// Times ncycles cycles (graph replays) between two CUDA events recorded on
// the run's stream; *ms is the device time.  Benchmark helper, no
// counterpart in the reference.
int hydro_run_timed(hydro_run* r, int ncycles, float* ms) {
  if (!r || !ms) return fail(-1, "hydro_run_timed: null argument");
  CUDA_TRY(cudaSetDevice(r->ctx->device));
  cudaStream_t s = r->ctx->stream;
  if (!r->graph)
    if (int rc = build_graph(r, 8)) return rc;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  CUDA_TRY(cudaStreamSynchronize(s));
  CUDA_TRY(cudaEventRecord(e0, s));
  if (int rc = hydro_run_enqueue(r, ncycles)) return rc;
  CUDA_TRY(cudaEventRecord(e1, s));
  CUDA_TRY(cudaEventSynchronize(e1));
  CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return sync_ctrl(r);
}

// Runs ncycles cycles kernel by kernel with CUDA events between launches and
// accumulates per kernel kind: ms[kind] (device time) and launches[kind].
// Benchmark helper, no counterpart in the reference.
int hydro_run_profile(hydro_run* r, int ncycles, double* ms, long long* launches,
                      int nkinds) {
  if (!r || !ms || !launches || nkinds < kNumKernelKinds)
    return fail(-1, "hydro_run_profile: bad arguments");
  CUDA_TRY(cudaSetDevice(r->ctx->device));
  cudaStream_t s = r->ctx->stream;
  for (int k = 0; k < nkinds; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  std::vector<cudaEvent_t> ev;
  std::vector<int> kinds;
  for (int c = 0; c < ncycles; ++c) {
    ev.clear();
    kinds.clear();
    LaunchHook hook = [&](int kind) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      cudaEventRecord(e, s);
      ev.push_back(e);
      kinds.push_back(kind);
    };
    launch_cycle(r->v, s, &hook);
    CUDA_TRY(cudaStreamSynchronize(s));
    for (size_t i = 0; i + 1 < ev.size(); ++i) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      ms[kinds[i]] += t;
      launches[kinds[i]] += 1;
    }
    for (auto e : ev) cudaEventDestroy(e);
  }
  r->kernels_launched += 0;
  CUDA_TRY(cudaGetLastError());
  return sync_ctrl(r);
}

const char* hydro_kernel_name(int kind) {
  return (kind >= 0 && kind < kNumKernelKinds) ? kKernelNames[kind] : "";
}

int hydro_kernel_kinds(void) { return kNumKernelKinds; }

int hydro_fp64_peak(int device, double* tflops) {
  if (!tflops) return fail(-1, "hydro_fp64_peak: null argument");
  return measure_fp64_peak(device, tflops);
}

// Stream of the context (for host code that records CUDA events around
// enqueued cycles).
void* hydro_ctx_stream(hydro_ctx* c) { return c ? (void*)c->stream : nullptr; }

size_t hydro_run_device_bytes(hydro_run* r) { return r ? r->arena_bytes : 0; }

}  // extern "C"
