// Per-device runtime state shared by the C entry points: a stream, a
// grow-only device workspace, pinned staging for small metadata uploads and
// the device properties the launch planners need.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <mutex>

namespace mlcp {

struct Context {
  int device = -1;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;      // library-owned non-blocking stream
  // device workspace (grow-only; reused across calls on this device)
  void* ws = nullptr;
  size_t ws_bytes = 0;
  // pinned host staging for metadata uploads; `staged` orders reuse
  void* stage = nullptr;
  size_t stage_bytes = 0;
  cudaEvent_t staged = nullptr;
  // power-cycle workspace (separate from the ALS workspace, which the cycle
  // also uses for its vector updates)
  void* cyc = nullptr;
  size_t cyc_bytes = 0;
  // autotuner: saved F terms during trials
  void* tune = nullptr;
  size_t tune_bytes = 0;
  // device copies of caller host buffers (host-buffer entry points)
  void* io = nullptr;
  size_t io_bytes = 0;
  // the power cycle's launch sequence captured as a CUDA graph, with the
  // key (shape, buffers, operator table) it was captured for
  cudaGraph_t cyc_graph = nullptr;
  cudaGraphExec_t cyc_exec = nullptr;
  unsigned long long cyc_key[16] = {};
  // optional timing of the dominant kernel of the latest call
  bool timing = false;
  bool timed = false;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  std::mutex mu;                       // one entry-point call at a time per device
};

// Context of the current device (created on first use).
Context* get_context(int* status);

// Launch-shape searches on (mlcp_gb300_set_autotune, MLCP_GB300_AUTOTUNE).
bool autotune_on();

// Ensure the workspace holds at least `bytes`; returns its base pointer.
// The previous contents are not preserved.
int ensure_workspace(Context* ctx, size_t bytes, void** out);

// Ensure the pinned staging area holds `bytes` and that no earlier upload
// from it is still in flight.
int ensure_stage(Context* ctx, size_t bytes, void** out);

// Bump allocator over a workspace region: 256-byte aligned slices.
struct Carver {
  char* base;
  size_t used = 0;
  explicit Carver(void* b) : base(static_cast<char*>(b)) {}
  template <typename T>
  T* take(size_t count) {
    size_t off = (used + 255) & ~size_t(255);
    used = off + count * sizeof(T);
    return reinterpret_cast<T*>(base + off);
  }
  // Byte size that a sequence of takes requires (dry run with base = null).
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace mlcp
