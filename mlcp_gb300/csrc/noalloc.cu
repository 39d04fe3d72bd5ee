// Allocation-free explicit-target ALS: one reduction (the alscpp_ operation)
// on caller-provided device buffers, with every piece of scratch memory taken
// from a fixed array compiled into the library.
//
// Who needs it: callers that cannot call cudaMalloc at the moment they reduce
// a vector: hosts whose device memory is owned up front by another allocator
// or memory pool (a framework that reserves the card, an MPS client with a
// hard memory limit), and latency-critical loops that must not enter the
// driver's allocator (cudaFree synchronises the device).
//
// Contract:
//  * Scratch lives in g_noalloc_scratch (kNoAllocScratchBytes = 32 MiB).  Every
//    GPU that loads this library holds the array until the process exits.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current).  Calls are not for
//    stream capture: the metadata below is a pageable copy from the stack.
//  * All calls share the array and it keeps the previous call's contents.
//    Every scratch region is fully written before it is read.  Calls whose
//    work overlaps on the GPU (two streams, or two host threads) race on the
//    array and give wrong results; serialise them.
//  * The caller's status word (d_status, required) is cleared by every call and
//    receives the kernel's flags: bit 0 when a normal-equation matrix was not
//    positive definite, bit 1 when an internal pipeline wait timed out.  Either
//    bit means the reduced vector is not valid.
//  * Sizes whose scratch exceeds the array are rejected with kTooLarge and a
//    message naming the limit; nothing is truncated.  Arguments are checked
//    before anything else, also when nals = 0 (which then does nothing).
//  * No cudaMalloc, cudaFree, cudaMallocHost or other allocating routine is
//    called.  Metadata is copied from the caller's stack with cudaMemcpyAsync
//    (a pageable copy: the call returns once the runtime has staged it).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/mlcp_gb300.h"
#include "als.cuh"
#include "common.cuh"
#include "context.cuh"

namespace mlcp {

int finish_status(int status);

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once).
int scratch_address(void** out) {
  int dev = 0;
  MLCP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("mlcp_als_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
    return kBadArgument;
  }
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* ptr = nullptr;
    MLCP_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    g_addr[dev] = ptr;
  }
  *out = g_addr[dev];
  return kOk;
}

int run(int ndof, const int* nbas, int rF, int rG, double* d_coef, double* d_base, int nals, int* d_status,
        cudaStream_t st) {
  if (ndof < 2 || ndof > 1024 || rF < 1 || rF > 64 || rG < 1 || nals < 0 || !nbas || !d_coef || !d_base) {
    set_error("mlcp_als_noalloc: bad arguments (ndof=%d rF=%d rG=%d nals=%d)", ndof, rF, rG, nals);
    return kBadArgument;
  }
  if (!d_status) {
    set_error("mlcp_als_noalloc: d_status is required (a device int that reports an invalid result)");
    return kBadArgument;
  }
  int off[1025], offp[1025], offg[1025];
  off[0] = offp[0] = offg[0] = 0;
  int npmax = 4, gsmax = 4;
  for (int d = 0; d < ndof; ++d) {
    if (nbas[d] < 1 || nbas[d] > 64) {
      set_error("mlcp_als_noalloc: nbas[%d] = %d outside [1, 64]", d, nbas[d]);
      return kBadArgument;
    }
    off[d + 1] = off[d] + nbas[d];
    offp[d + 1] = offp[d] + round_up(nbas[d], 4);
    offg[d + 1] = offg[d] + als_gstride(nbas[d]);
    npmax = std::max(npmax, round_up(nbas[d], 4));
    gsmax = std::max(gsmax, als_gstride(nbas[d]));
  }
  if (nals == 0) return kOk;
  const int nD = off[ndof], nDp = offp[ndof], nDg = offg[ndof];

  // launch shape: a cluster of up to 16 CTAs owning slices of the target terms
  int dev = 0, nsm = 0, optin = 0;
  MLCP_CUDA_TRY(cudaGetDevice(&dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  AlsShape shape;
  if (!als_choose_shape(1, rG, rF, npmax, gsmax, nsm, (size_t)optin, &shape)) {
    set_error("mlcp_als_noalloc: rank-%d target with rank-%d F needs more shared memory per CTA than %d bytes",
              rG, rF, optin);
    return kTooLarge;
  }
  const int CL = shape.cluster;

  // scratch layout inside the fixed array
  const size_t n_int = (size_t)ndof + 3 * (ndof + 1) + 2;
  const size_t n_ll = 6;
  const size_t sq = (size_t)rF * rF * ndof;
  size_t bytes = 0;
  auto reserve = [&](size_t b) { size_t o = align256(bytes); bytes = o + b; return o; };
  const size_t o_int = reserve(sizeof(int) * n_int);
  const size_t o_ll = reserve(sizeof(long long) * n_ll);
  const size_t o_gm = reserve(sizeof(float) * (size_t)rG * nDg);
  const size_t o_gc = reserve(sizeof(float) * (size_t)rG);
  const size_t o_f32 = reserve(sizeof(float) * (size_t)rF * nDp);
  const size_t o_f32lo = reserve(sizeof(float) * (size_t)rF * nDp);
  const size_t o_fcta = reserve(sizeof(float) * (size_t)rF * CL * nDp);
  const size_t o_gram = reserve(sizeof(dw) * sq * CL);
  const size_t o_suf = reserve(sizeof(dw) * sq * CL);
  if (bytes > kNoAllocScratchBytes) {
    set_error("mlcp_als_noalloc: a rank-%d target over %d modes (%d padded basis functions) needs %zu bytes of "
              "scratch; the fixed scratch array holds %zu bytes (use mlcp_als_batched instead)",
              rG, ndof, nDg, bytes, kNoAllocScratchBytes);
    return kTooLarge;
  }

  void* base_ptr = nullptr;
  int rc = scratch_address(&base_ptr);
  if (rc) return rc;
  char* w = static_cast<char*>(base_ptr);

  // metadata from the stack (pageable copy: the call returns once it is staged)
  int hi[1024 + 3 * 1025 + 2];
  long long hl[6];
  std::memcpy(hi, nbas, sizeof(int) * ndof);
  std::memcpy(hi + ndof, off, sizeof(int) * (ndof + 1));
  std::memcpy(hi + 2 * ndof + 1, offp, sizeof(int) * (ndof + 1));
  std::memcpy(hi + 3 * ndof + 2, offg, sizeof(int) * (ndof + 1));
  hi[4 * ndof + 3] = rF;
  hi[4 * ndof + 4] = rG;
  hl[0] = 0;   // F terms start at term 0
  hl[1] = 0;   // first target row
  hl[2] = 0;   // first F row
  hl[3] = 0;   // target copy offset
  hl[4] = 0;   // Gram offset
  hl[5] = rF;  // target terms follow F
  MLCP_CUDA_TRY(cudaMemcpyAsync(w + o_int, hi, sizeof(int) * n_int, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaMemcpyAsync(w + o_ll, hl, sizeof(long long) * n_ll, cudaMemcpyHostToDevice, st));
  int* status = d_status;
  MLCP_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));

  const int* d_int = reinterpret_cast<const int*>(w + o_int);
  const long long* d_ll = reinterpret_cast<const long long*>(w + o_ll);
  AlsParams prm;
  prm.nvec = 1;
  prm.ndof = ndof;
  prm.nD = nD;
  prm.nDp = nDp;
  prm.nDg = nDg;
  prm.npmax = npmax;
  prm.rf_max = rF;
  prm.gsmax = gsmax;
  prm.nals = nals;
  prm.pen_factor = 1.0e-10;
  prm.cluster = CL;
  prm.stages = shape.stages;
  prm.tc = shape.tc;
  prm.rows_cta_max = shape.rows_cta;
  prm.total_rows = rG;
  prm.total_f_terms = rF;
  prm.nbas = d_int;
  prm.off = d_int + ndof;
  prm.offp = d_int + 2 * ndof + 1;
  prm.offg = d_int + 3 * ndof + 2;
  prm.rF = d_int + 4 * ndof + 3;
  prm.rG = d_int + 4 * ndof + 4;
  prm.term_off = d_ll;
  prm.g_row_off = d_ll + 1;
  prm.f_row_off = d_ll + 2;
  prm.gm_off = d_ll + 3;
  prm.sq_off = d_ll + 4;
  prm.g_term_off = d_ll + 5;
  prm.base = d_base;
  prm.coef = d_coef;
  prm.g_base = d_base;
  prm.g_coef = d_coef;
  prm.shared_target = 0;
  prm.g_host = 0;
  prm.shared_w = nullptr;
  prm.gm = reinterpret_cast<float*>(w + o_gm);
  prm.gc = reinterpret_cast<float*>(w + o_gc);
  prm.f32 = reinterpret_cast<float*>(w + o_f32);
  prm.f32lo = reinterpret_cast<float*>(w + o_f32lo);
  prm.fcta = reinterpret_cast<float*>(w + o_fcta);
  prm.gram = reinterpret_cast<dw*>(w + o_gram);
  prm.suf = reinterpret_cast<dw*>(w + o_suf);
  prm.status = status;
  return als_launch(prm, shape.smem, st);
}

}  // namespace

}  // namespace mlcp

extern "C" int mlcp_als_noalloc(int ndof, const int* nbas, int rF, int rG, double* d_coef, double* d_base, int nals,
                                int* d_status, void* stream) {
  return mlcp::finish_status(mlcp::run(ndof, nbas, rF, rG, d_coef, d_base, nals, d_status,
                                       static_cast<cudaStream_t>(stream)));
}
