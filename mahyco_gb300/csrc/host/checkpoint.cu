// Checkpoint / restart of a run (no counterpart in the reference, whose runs
// only end or abort).
//
// A checkpoint is the run's options and its whole device arena, taken
// between cycles: the SoA state, the control block (time, dt, cycle count,
// sweep direction, the dt / pressure reductions carried into the next cycle,
// the error word) and the constant geometry and scratch planes.  Restoring it
// rebuilds the same layout from the options and refills the arena, so the
// resumed run continues bit for bit as the original would have.  Copies go
// through two pinned staging buffers so that the device->host copy of one
// chunk overlaps the file write of the previous one (and the reverse on
// restore).
//
// File: header (magic, format version, sizeof(hydro_spec), arena bytes, a
// hash of the layout, a hash of the arena contents, a hash of the options),
// the hydro_spec, then the arena bytes.  The layout hash ties a file to the
// library's layout; the content and option hashes reject truncated or
// corrupted files (a damaged option would otherwise resume the run with
// another scheme, limiter or end time).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "runtime.h"

namespace hydro {
namespace {

constexpr char kMagic[8] = {'H', 'G', 'B', '3', 'C', 'K', 'P', 'T'};
constexpr uint32_t kVersion = 5;
constexpr size_t kChunk = 64u << 20;

struct Header {
  char magic[8];
  uint32_t version;
  uint32_t spec_bytes;
  uint64_t arena_bytes;
  uint64_t layout_hash;
  uint64_t data_hash;
  uint64_t spec_hash;
  uint64_t reserved[2];
};

// FNV-1a over 64-bit words (tail bytes zero-padded)
struct Hash {
  uint64_t h = 0xcbf29ce484222325ull;
  void add(const void* p, size_t n) {
    const unsigned char* b = (const unsigned char*)p;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
      uint64_t w;
      std::memcpy(&w, b + i, 8);
      h = (h ^ w) * 0x100000001b3ull;
    }
    if (i < n) {
      uint64_t w = 0;
      std::memcpy(&w, b + i, n - i);
      h = (h ^ w) * 0x100000001b3ull;
    }
  }
};

uint64_t layout_hash(const RunView& v, size_t bytes) {
  const long long f[] = {v.nx, v.ny, v.nc, v.nn, v.pitch, v.npitch, v.fpitch, v.nbmat,
                         v.ncomp, v.scheme, (long long)bytes, (long long)sizeof(Ctrl),
                         (long long)sizeof(RunView)};
  Hash h;
  h.add(f, sizeof f);
  return h.h;
}

// Two pinned staging buffers and their events.
struct Staging {
  void* buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~Staging() {
    for (int k = 0; k < 2; ++k) {
      if (ev[k]) cudaEventDestroy(ev[k]);
      if (buf[k]) cudaFreeHost(buf[k]);
    }
  }
  int init() {
    for (int k = 0; k < 2; ++k) {
      CUDA_TRY(cudaMallocHost(&buf[k], kChunk));
      CUDA_TRY(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
    }
    return 0;
  }
};

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

}  // namespace
}  // namespace hydro

using namespace hydro;

extern "C" {

int hydro_run_checkpoint(hydro_run* r, const char* path) {
  if (!r || !path) return fail(-1, "hydro_run_checkpoint: null argument");
  CUDA_TRY(cudaSetDevice(r->ctx->device));
  cudaStream_t s = r->ctx->stream;
  CUDA_TRY(cudaStreamSynchronize(s));  // between cycles
  Staging st;
  if (int rc = st.init()) return rc;
  File out;
  out.f = std::fopen(path, "wb");
  if (!out.f) return fail(-40, std::string("checkpoint: cannot open ") + path);
  Header h{};
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.spec_bytes = sizeof(hydro_spec);
  h.arena_bytes = r->arena_bytes;
  h.layout_hash = layout_hash(r->v, r->arena_bytes);
  {
    Hash hs;
    hs.add(&r->spec, sizeof(hydro_spec));
    h.spec_hash = hs.h;
  }
  if (std::fwrite(&h, sizeof h, 1, out.f) != 1 ||
      std::fwrite(&r->spec, sizeof(hydro_spec), 1, out.f) != 1)
    return fail(-41, "checkpoint: write failed");
  Hash hash;
  const char* src = (const char*)r->arena;
  const size_t total = r->arena_bytes;
  const size_t nchunks = (total + kChunk - 1) / kChunk;
  auto issue = [&](size_t k) -> int {
    const size_t off = k * kChunk, n = std::min(kChunk, total - off);
    CUDA_TRY(cudaMemcpyAsync(st.buf[k & 1], src + off, n, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaEventRecord(st.ev[k & 1], s));
    return 0;
  };
  if (nchunks)
    if (int rc = issue(0)) return rc;
  for (size_t k = 0; k < nchunks; ++k) {
    if (k + 1 < nchunks)
      if (int rc = issue(k + 1)) return rc;  // overlaps the write of chunk k
    CUDA_TRY(cudaEventSynchronize(st.ev[k & 1]));
    const size_t n = std::min(kChunk, total - k * kChunk);
    hash.add(st.buf[k & 1], n);
    if (std::fwrite(st.buf[k & 1], 1, n, out.f) != n) {
      cudaStreamSynchronize(s);
      return fail(-41, "checkpoint: write failed");
    }
  }
  h.data_hash = hash.h;
  if (std::fseek(out.f, 0, SEEK_SET) != 0 || std::fwrite(&h, sizeof h, 1, out.f) != 1)
    return fail(-41, "checkpoint: header rewrite failed");
  const int cl = std::fclose(out.f);
  out.f = nullptr;
  if (cl != 0) return fail(-41, "checkpoint: close failed");
  return 0;
}

int hydro_run_restore(hydro_ctx* ctx, const char* path, hydro_run** out) {
  if (!ctx || !path || !out) return fail(-1, "hydro_run_restore: null argument");
  File in;
  in.f = std::fopen(path, "rb");
  if (!in.f) return fail(-42, std::string("restore: cannot open ") + path);
  Header h{};
  hydro_spec spec{};
  if (std::fread(&h, sizeof h, 1, in.f) != 1 || std::memcmp(h.magic, kMagic, 8) != 0)
    return fail(-43, "restore: not a hydro checkpoint");
  if (h.version != kVersion || h.spec_bytes != sizeof(hydro_spec))
    return fail(-43, "restore: checkpoint format version not supported");
  if (std::fread(&spec, sizeof spec, 1, in.f) != 1)
    return fail(-43, "restore: truncated checkpoint");
  {
    Hash hs;
    hs.add(&spec, sizeof spec);
    if (hs.h != h.spec_hash) return fail(-46, "restore: checkpoint options corrupted");
  }
  PreparedRun pr;
  if (int rc = prepare_run(spec, pr)) return rc;
  if (pr.bytes != h.arena_bytes || layout_hash(pr.v, pr.bytes) != h.layout_hash)
    return fail(-44, "restore: the checkpoint's layout differs from this library's");
  hydro_run* r = nullptr;
  if (int rc = place_run(ctx, pr, &r, true, false)) return rc;
  int rc = 0;
  cudaStream_t s = ctx->stream;
  Staging st;
  rc = st.init();
  Hash hash;
  char* dst = (char*)r->arena;
  const size_t total = h.arena_bytes;
  const size_t nchunks = (total + kChunk - 1) / kChunk;
  for (size_t k = 0; k < nchunks && !rc; ++k) {
    const size_t n = std::min(kChunk, total - k * kChunk);
    if (k >= 2 && cudaEventSynchronize(st.ev[k & 1]) != cudaSuccess) {
      rc = fail(-45, "restore: copy failed");
      break;
    }
    if (std::fread(st.buf[k & 1], 1, n, in.f) != n) {
      rc = fail(-43, "restore: truncated checkpoint");
      break;
    }
    hash.add(st.buf[k & 1], n);
    if (cudaMemcpyAsync(dst + k * kChunk, st.buf[k & 1], n, cudaMemcpyHostToDevice, s) !=
            cudaSuccess ||
        cudaEventRecord(st.ev[k & 1], s) != cudaSuccess)
      rc = fail(-45, "restore: copy failed");
  }
  if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = fail(-45, "restore: copy failed");
  if (!rc && std::fgetc(in.f) != EOF) rc = fail(-43, "restore: trailing bytes in checkpoint");
  if (!rc && hash.h != h.data_hash) rc = fail(-46, "restore: checkpoint contents corrupted");
  if (!rc && cudaMemcpy(&r->h_ctrl, r->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost) !=
                 cudaSuccess)
    rc = fail(-45, "restore: control block read failed");
  if (rc) {
    hydro_run_destroy(r);
    return rc;
  }
  *out = r;
  return 0;
}

}  // extern "C"
