// C entry points (drop-in for the reference's src/intertwining.cu) and the
// host-side planners of the batched ALS.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/mlcp_gb300.h"
#include "als.cuh"
#include "common.cuh"
#include "context.cuh"
#include "intertwine.cuh"

namespace mlcp {

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------

static thread_local std::string t_error;
static thread_local int t_status = 0;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_error = buf;
}
const char* last_error() { return t_error.c_str(); }

static int finish(int status) {
  t_status = status;
  if (status == kOk) t_error.clear();
  // a failed call leaves no stale runtime error behind (a refused allocation
  // would otherwise surface at the next call's launch check); errors that
  // poison the context persist whatever is read here
  if (status == kCudaError) (void)cudaGetLastError();
  return status;
}
int finish_status(int status) { return finish(status); }

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------

static std::mutex g_ctx_mu;
static std::map<int, Context*> g_ctx;

Context* get_context(int* status) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("cudaGetDevice failed: %s", cudaGetErrorString(e));
    *status = kCudaError;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  auto it = g_ctx.find(dev);
  if (it != g_ctx.end()) {
    *status = kOk;
    return it->second;
  }
  Context* c = new Context();
  c->device = dev;
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->staged, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&c->t0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->t1);
  if (e != cudaSuccess) {
    set_error("context creation failed: %s", cudaGetErrorString(e));
    delete c;
    *status = kCudaError;
    return nullptr;
  }
  c->num_sms = prop.multiProcessorCount;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  g_ctx[dev] = c;
  *status = kOk;
  return c;
}

int ensure_workspace(Context* ctx, size_t bytes, void** out) {
  if (bytes > ctx->ws_bytes) {
    if (ctx->ws) {
      MLCP_CUDA_TRY(cudaDeviceSynchronize());
      MLCP_CUDA_TRY(cudaFree(ctx->ws));
      ctx->ws = nullptr;
      ctx->ws_bytes = 0;
    }
    size_t want = std::max(bytes, ctx->ws_bytes + ctx->ws_bytes / 2);
    MLCP_CUDA_TRY(cudaMalloc(&ctx->ws, want));
    ctx->ws_bytes = want;
  }
  *out = ctx->ws;
  return kOk;
}

int ensure_stage(Context* ctx, size_t bytes, void** out) {
  MLCP_CUDA_TRY(cudaEventSynchronize(ctx->staged));
  if (bytes > ctx->stage_bytes) {
    if (ctx->stage) MLCP_CUDA_TRY(cudaFreeHost(ctx->stage));
    size_t want = std::max(bytes, size_t(1) << 16);
    MLCP_CUDA_TRY(cudaMallocHost(&ctx->stage, want));
    ctx->stage_bytes = want;
  }
  *out = ctx->stage;
  return kOk;
}

// ---------------------------------------------------------------------------
// Batched explicit-G ALS planner
// ---------------------------------------------------------------------------

namespace {

constexpr int kMaxRank = 64;
constexpr int kMaxBasis = 64;

struct AlsPlan {
  int D, nD, nDp, nDg, npmax, gsmax, rFmax;
  AlsShape shape;
  std::vector<int> off, offp, offg;
  std::vector<long long> g_row_off, f_row_off, gm_off, sq_off;
  long long total_rows, total_f, gm_floats, sq_total;
};

int plan_als(Context* ctx, int nvec, int ndof, const int* nbas, const int* rF, const int* rG, AlsPlan* P) {
  if (nvec < 1 || ndof < 2) {
    set_error("mlcp_als_batched: nvec (%d) must be positive and ndof (%d) at least 2", nvec, ndof);
    return kBadArgument;
  }
  P->D = ndof;
  P->off.assign(ndof + 1, 0);
  P->offp.assign(ndof + 1, 0);
  P->offg.assign(ndof + 1, 0);
  P->npmax = 4;
  P->gsmax = 4;
  for (int d = 0; d < ndof; ++d) {
    if (nbas[d] < 1 || nbas[d] > kMaxBasis) {
      set_error("mlcp_als_batched: nbas[%d] = %d outside [1, %d]", d, nbas[d], kMaxBasis);
      return nbas[d] < 1 ? kBadArgument : kTooLarge;
    }
    P->off[d + 1] = P->off[d] + nbas[d];
    P->offp[d + 1] = P->offp[d] + round_up(nbas[d], 4);
    P->offg[d + 1] = P->offg[d] + als_gstride(nbas[d]);
    P->npmax = std::max(P->npmax, round_up(nbas[d], 4));
    P->gsmax = std::max(P->gsmax, als_gstride(nbas[d]));
  }
  P->nD = P->off[ndof];
  P->nDp = P->offp[ndof];
  P->nDg = P->offg[ndof];
  P->g_row_off.resize(nvec);
  P->f_row_off.resize(nvec);
  P->gm_off.resize(nvec);
  P->sq_off.resize(nvec);
  long long gr = 0, fr = 0, gmo = 0, sq = 0;
  int rGmax = 0;
  P->rFmax = 0;
  for (int v = 0; v < nvec; ++v) {
    if (rF[v] < 1 || rG[v] < 1) {
      set_error("mlcp_als_batched: vector %d has rF=%d rG=%d (both must be positive)", v, rF[v], rG[v]);
      return kBadArgument;
    }
    if (rF[v] > kMaxRank) {
      set_error("mlcp_als_batched: vector %d has rF=%d > %d", v, rF[v], kMaxRank);
      return kTooLarge;
    }
    P->g_row_off[v] = gr;
    P->f_row_off[v] = fr;
    P->gm_off[v] = gmo;
    P->sq_off[v] = sq;
    gr += rG[v];
    fr += rF[v];
    gmo += (long long)rG[v] * P->nDg;
    sq += (long long)rF[v] * rF[v] * ndof;
    rGmax = std::max(rGmax, rG[v]);
    P->rFmax = std::max(P->rFmax, rF[v]);
  }
  P->total_rows = gr;
  P->total_f = fr;
  P->gm_floats = gmo;
  P->sq_total = sq;
  if (!als_choose_shape(nvec, rGmax, P->rFmax, P->npmax, P->gsmax, ctx->num_sms, ctx->smem_optin, &P->shape)) {
    set_error("mlcp_als_batched: rank-%d target with rank-%d F (padded basis %d) needs more than %zu bytes of "
              "shared memory per CTA even with 16-CTA clusters",
              rGmax, P->rFmax, P->gsmax, ctx->smem_optin);
    return kTooLarge;
  }
  return kOk;
}

// ---------------------------------------------------------------------------
// Launch-shape autotuner of the batched ALS
// ---------------------------------------------------------------------------
// The reference sizes its kernels' blocks by fixed rules on the ranks
// (PVVkernel::initnew, src/modvecvec.cu:27-94).  Here two shape parameters of
// the cluster kernel are measured instead: the cluster size (CTAs sharing one
// vector's target terms) and the depth of the target-tile ring.  The first
// call for a batch shape runs one sweep with every feasible (cluster, stages)
// pair on the caller's own data (the F terms are saved first and restored
// after every trial, so the call's result is unaffected), times each with CUDA
// events on the call's stream, and caches the fastest for the process, per
// device and shape.  Later calls with the same shape reuse it.  Disabled by
// mlcp_gb300_set_autotune(0) or MLCP_GB300_AUTOTUNE=0 (then the rule of
// als_choose_shape applies).

struct TuneKey {
  int device, nvec, ndof, nD, npmax, gsmax, rGmax, rFmax;
  long long total_rows;
  int engine;
  bool operator<(const TuneKey& o) const {
    return std::tie(device, nvec, ndof, nD, npmax, gsmax, rGmax, rFmax, total_rows, engine) <
           std::tie(o.device, o.nvec, o.ndof, o.nD, o.npmax, o.gsmax, o.rGmax, o.rFmax, o.total_rows, o.engine);
  }
};

struct TuneEntry {
  AlsShape shape;
  std::vector<std::pair<AlsShape, float>> trials;  // (shape, ms for one sweep)
};

std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;
int g_autotune = -1;  // -1: not yet read from the environment

int g_als_engine = -1;  // -1: not yet read from the environment

}  // namespace

int als_engine() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (g_als_engine < 0) {
    const char* e = getenv("MLCP_GB300_ALS_ENGINE");
    g_als_engine = (e && (e[0] == '1' || e[0] == '2')) ? e[0] - '0' : 0;
  }
  return g_als_engine;
}

void set_als_engine(int e) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_als_engine = (e == 1 || e == 2) ? e : 0;
}

namespace {

bool autotune_enabled() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (g_autotune < 0) {
    const char* e = getenv("MLCP_GB300_AUTOTUNE");
    g_autotune = (e && e[0] == '0') ? 0 : 1;
  }
  return g_autotune != 0;
}

// Feasible (cluster, stages, engine) triples: every power-of-two cluster up
// to 16 whose clusters fit on the GPU in at most two waves, every ring depth
// 2-6 whose shared memory fits, in the CUDA-core form and, where it fits
// (als_tc_fits), the tensor-core form, as the engine setting allows.
std::vector<AlsShape> als_candidates(int nvec, int rGmax, int rFmax, int npmax, int gsmax, int num_sms,
                                     size_t smem_limit) {
  std::vector<AlsShape> out;
  const int engine = als_engine();
  for (int cl = 1; cl <= 16; cl *= 2) {
    if (cl > 1 && (long long)cl * nvec > 2LL * num_sms) break;
    const int rows = (rGmax + cl - 1) / cl;
    for (int tc = 1; tc >= 0; --tc) {
      if (tc == 1 && (engine == 1 || !als_tc_fits(rows, rFmax, npmax))) continue;
      for (int ns = tc ? 3 : 2; ns <= 6; ++ns) {  // the tensor-core form refills one tile ahead
        const size_t b = als_smem_bytes(rows, rFmax, npmax, gsmax, ns, tc);
        if (b > smem_limit) continue;
        AlsShape s;
        s.cluster = cl;
        s.stages = ns;
        s.rows_cta = rows;
        s.tc = tc;
        s.smem = b;
        out.push_back(s);
      }
    }
  }
  // forced tensor cores: only the tensor-core shapes, unless none fits
  if (engine == 2) {
    std::vector<AlsShape> t;
    for (const AlsShape& s : out)
      if (s.tc) t.push_back(s);
    if (!t.empty()) out.swap(t);
  }
  return out;
}

}  // namespace

bool autotune_on() { return autotune_enabled(); }

int als_run_shape(Context* ctx, const AlsJob& job, cudaStream_t st, const AlsShape* forced);

// Runs one batched reduction; everything is enqueued on `st`.  The launch
// shape comes from the autotuner (measured once per batch shape) or, with
// tuning off or for shared-target and host-target jobs, from the rule.
int als_run(Context* ctx, const AlsJob& job, cudaStream_t st) {
  if (job.nals <= 0 || job.shared_w || !autotune_enabled()) return als_run_shape(ctx, job, st, nullptr);
  AlsPlan P;
  int rc = plan_als(ctx, job.nvec, job.ndof, job.nbas, job.rF, job.rG, &P);
  if (rc) return rc;
  TuneKey key{ctx->device, job.nvec, job.ndof, P.nD, P.npmax, P.gsmax, 0, P.rFmax, P.total_rows, als_engine()};
  for (int v = 0; v < job.nvec; ++v) key.rGmax = std::max(key.rGmax, job.rG[v]);
  {
    AlsShape cached;
    bool hit = false;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        cached = it->second.shape;
        hit = true;
      }
    }
    if (hit) return als_run_shape(ctx, job, st, &cached);  // (outside the lock: the run reads the engine setting)
  }
  if (job.g_host) return als_run_shape(ctx, job, st, nullptr);  // tuned by a device-resident call
  std::vector<AlsShape> cand = als_candidates(job.nvec, key.rGmax, P.rFmax, P.npmax, P.gsmax, ctx->num_sms,
                                              ctx->smem_optin);
  if (cand.size() <= 1) return als_run_shape(ctx, job, st, nullptr);
  // save the F terms (the trials overwrite them)
  const size_t fvals = (size_t)P.total_f * P.nD;
  const size_t bytes = sizeof(double) * (fvals + P.total_f);
  if (bytes > ctx->tune_bytes) {
    if (ctx->tune) {
      MLCP_CUDA_TRY(cudaStreamSynchronize(st));
      MLCP_CUDA_TRY(cudaFree(ctx->tune));
      ctx->tune = nullptr;
      ctx->tune_bytes = 0;
    }
    MLCP_CUDA_TRY(cudaMalloc(&ctx->tune, bytes));
    ctx->tune_bytes = bytes;
  }
  double* sb = static_cast<double*>(ctx->tune);
  double* sc = sb + fvals;
  auto copy_f = [&](bool save) -> int {
    size_t fo = 0;
    for (int v = 0; v < job.nvec; ++v) {
      double* b = job.d_base + (size_t)job.term_off[v] * P.nD;
      double* c = job.d_coef + job.term_off[v];
      const size_t nb = sizeof(double) * (size_t)job.rF[v] * P.nD, nc = sizeof(double) * job.rF[v];
      MLCP_CUDA_TRY(cudaMemcpyAsync(save ? sb + fo * P.nD : b, save ? b : sb + fo * P.nD, nb,
                                    cudaMemcpyDeviceToDevice, st));
      MLCP_CUDA_TRY(cudaMemcpyAsync(save ? sc + fo : c, save ? c : sc + fo, nc, cudaMemcpyDeviceToDevice, st));
      fo += job.rF[v];
    }
    return kOk;
  };
  if ((rc = copy_f(true))) return rc;
  cudaEvent_t e0, e1;
  MLCP_CUDA_TRY(cudaEventCreate(&e0));
  MLCP_CUDA_TRY(cudaEventCreate(&e1));
  AlsJob trial = job;
  trial.nals = 1;
  TuneEntry entry;
  float best = 0.f;
  for (const AlsShape& c : cand) {
    MLCP_CUDA_TRY(cudaEventRecord(e0, st));
    rc = als_run_shape(ctx, trial, st, &c);
    if (rc) break;
    MLCP_CUDA_TRY(cudaEventRecord(e1, st));
    MLCP_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    MLCP_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    entry.trials.push_back({c, ms});
    if (entry.trials.size() == 1 || ms < best) {
      best = ms;
      entry.shape = c;
    }
    if ((rc = copy_f(false))) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = entry;
  }
  const AlsShape s = entry.shape;
  return als_run_shape(ctx, job, st, &s);
}

int autotune_report(char* buf, int len) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::string out;
  char line[256];
  for (const auto& kv : g_tune) {
    const TuneKey& k = kv.first;
    snprintf(line, sizeof(line), "als nvec=%d ndof=%d nD=%d rG<=%d rF<=%d engine=%d: cluster %d stages %d %s;",
             k.nvec, k.ndof, k.nD, k.rGmax, k.rFmax, k.engine, kv.second.shape.cluster, kv.second.shape.stages,
             kv.second.shape.tc ? "tensor" : "cuda");
    out += line;
    for (const auto& t : kv.second.trials) {
      snprintf(line, sizeof(line), " %dx%d%s=%.3fms", t.first.cluster, t.first.stages, t.first.tc ? "t" : "c",
               t.second);
      out += line;
    }
    out += "\n";
  }
  gs_tune_report(out);
  if (buf && len > 0) {
    strncpy(buf, out.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)out.size();
}

void set_autotune(int on) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_autotune = on ? 1 : 0;
}

// One batched reduction with the given launch shape (null: the rule).
int als_run_shape(Context* ctx, const AlsJob& job, cudaStream_t st, const AlsShape* forced) {
  const int nvec = job.nvec, ndof = job.ndof, nals = job.nals;
  const int *nbas = job.nbas, *rF = job.rF, *rG = job.rG;
  const long long* term_off = job.term_off;
  double* d_coef = job.d_coef;
  double* d_base = job.d_base;
  int* d_status = job.d_status;
  if (nals == 0) return kOk;  // reference returns before touching the data (src/als.cu:1026)
  if (nals < 0) {
    set_error("mlcp_als_batched: nals = %d is negative", nals);
    return kBadArgument;
  }
  AlsPlan P;
  int rc = plan_als(ctx, nvec, ndof, nbas, rF, rG, &P);
  if (rc) return rc;
  if (forced) P.shape = *forced;
  const int CL = P.shape.cluster;

  // metadata block: ints then long longs (uploaded in one copy)
  const size_t n_int = (size_t)(ndof) + 3 * (ndof + 1) + 2 * nvec;
  const size_t n_ll = (size_t)6 * nvec;  // term, g_row, f_row, gm, sq, g_term offsets
  const size_t meta_bytes = align256(n_int * sizeof(int)) + n_ll * sizeof(long long);
  // workspace layout
  size_t bytes = 0;
  auto reserve = [&](size_t b) { size_t o = align256(bytes); bytes = o + b; return o; };
  const size_t o_meta = reserve(meta_bytes);
  const size_t o_gm = reserve(sizeof(float) * (job.shared_w ? (long long)rG[0] * P.nDg : P.gm_floats));
  const size_t o_gc = reserve(sizeof(float) * P.total_rows);
  const size_t o_f32 = reserve(sizeof(float) * P.total_f * P.nDp);
  const size_t o_f32lo = reserve(sizeof(float) * P.total_f * P.nDp);
  const size_t o_fcta = reserve(sizeof(float) * P.total_f * CL * P.nDp);
  const size_t o_gram = reserve(sizeof(dw) * P.sq_total * CL);
  const size_t o_suf = reserve(sizeof(dw) * P.sq_total * CL);
  const size_t o_status = reserve(sizeof(int) * nvec);
  void* ws = nullptr;
  rc = ensure_workspace(ctx, bytes, &ws);
  if (rc) return rc;
  char* w = static_cast<char*>(ws);

  void* stage = nullptr;
  rc = ensure_stage(ctx, meta_bytes, &stage);
  if (rc) return rc;
  int* hi = static_cast<int*>(stage);
  long long* hl = reinterpret_cast<long long*>(static_cast<char*>(stage) + align256(n_int * sizeof(int)));
  int* p_nbas = hi;
  int* p_off = p_nbas + ndof;
  int* p_offp = p_off + (ndof + 1);
  int* p_offg = p_offp + (ndof + 1);
  int* p_rF = p_offg + (ndof + 1);
  int* p_rG = p_rF + nvec;
  std::memcpy(p_nbas, nbas, sizeof(int) * ndof);
  std::memcpy(p_off, P.off.data(), sizeof(int) * (ndof + 1));
  std::memcpy(p_offp, P.offp.data(), sizeof(int) * (ndof + 1));
  std::memcpy(p_offg, P.offg.data(), sizeof(int) * (ndof + 1));
  std::memcpy(p_rF, rF, sizeof(int) * nvec);
  std::memcpy(p_rG, rG, sizeof(int) * nvec);
  long long* p_term = hl;
  long long* p_gro = p_term + nvec;
  long long* p_fro = p_gro + nvec;
  long long* p_gmo = p_fro + nvec;
  long long* p_sqo = p_gmo + nvec;
  long long* p_gto = p_sqo + nvec;
  std::memcpy(p_term, term_off, sizeof(long long) * nvec);
  std::memcpy(p_gro, P.g_row_off.data(), sizeof(long long) * nvec);
  std::memcpy(p_fro, P.f_row_off.data(), sizeof(long long) * nvec);
  std::memcpy(p_gmo, P.gm_off.data(), sizeof(long long) * nvec);
  std::memcpy(p_sqo, P.sq_off.data(), sizeof(long long) * nvec);
  for (int v = 0; v < nvec; ++v)
    p_gto[v] = job.shared_w ? 0 : (job.g_term_off ? job.g_term_off[v] : term_off[v] + rF[v]);
  if (job.shared_w) {
    // every vector reads vector 0's converted target
    for (int v = 0; v < nvec; ++v) p_gmo[v] = 0;
  }
  MLCP_CUDA_TRY(cudaMemcpyAsync(w + o_meta, stage, meta_bytes, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaEventRecord(ctx->staged, st));

  const char* dm = w + o_meta;
  const int* d_int = reinterpret_cast<const int*>(dm);
  const long long* d_ll = reinterpret_cast<const long long*>(dm + align256(n_int * sizeof(int)));
  AlsParams prm;
  prm.nvec = nvec;
  prm.ndof = ndof;
  prm.nD = P.nD;
  prm.nDp = P.nDp;
  prm.nDg = P.nDg;
  prm.npmax = P.npmax;
  prm.rf_max = P.rFmax;
  prm.gsmax = P.gsmax;
  prm.nals = nals;
  prm.pen_factor = job.pen_factor;
  prm.cluster = CL;
  prm.stages = P.shape.stages;
  prm.tc = P.shape.tc;
  prm.rows_cta_max = P.shape.rows_cta;
  prm.total_rows = P.total_rows;
  prm.total_f_terms = P.total_f;
  prm.nbas = d_int;
  prm.off = d_int + ndof;
  prm.offp = prm.off + (ndof + 1);
  prm.offg = prm.offp + (ndof + 1);
  prm.rF = prm.offg + (ndof + 1);
  prm.rG = prm.rF + nvec;
  prm.term_off = d_ll;
  prm.g_row_off = d_ll + nvec;
  prm.f_row_off = d_ll + 2 * nvec;
  prm.gm_off = d_ll + 3 * nvec;
  prm.sq_off = d_ll + 4 * nvec;
  prm.g_term_off = d_ll + 5 * nvec;
  prm.base = d_base;
  prm.coef = d_coef;
  prm.g_base = job.g_base ? job.g_base : d_base;
  prm.g_coef = job.g_coef ? job.g_coef : d_coef;
  prm.shared_target = job.shared_w ? 1 : 0;
  prm.g_host = job.g_host ? 1 : 0;
  prm.shared_w = job.shared_w;
  prm.gm = reinterpret_cast<float*>(w + o_gm);
  prm.gc = reinterpret_cast<float*>(w + o_gc);
  prm.f32 = reinterpret_cast<float*>(w + o_f32);
  prm.f32lo = reinterpret_cast<float*>(w + o_f32lo);
  prm.fcta = reinterpret_cast<float*>(w + o_fcta);
  prm.gram = reinterpret_cast<dw*>(w + o_gram);
  prm.suf = reinterpret_cast<dw*>(w + o_suf);
  prm.status = d_status ? d_status : reinterpret_cast<int*>(w + o_status);
  MLCP_CUDA_TRY(cudaMemsetAsync(prm.status, 0, sizeof(int) * nvec, st));

  ctx->timed = ctx->timing;
  return als_launch(prm, P.shape.smem, st, ctx->timing ? ctx->t0 : nullptr, ctx->timing ? ctx->t1 : nullptr);
}

// ---------------------------------------------------------------------------
// Full CP inner products (FP64), deterministic two-stage reduction
// ---------------------------------------------------------------------------

namespace {

struct DotParams {
  int nvec, ndof, nD, chunks;
  const int* nbas;
  const long long* x_off;
  const int* rx;
  const long long* y_off;
  const int* ry;
  const double* coef;
  const double* base;
  double* partial;  // [nvec][chunks]
};

__global__ void cp_dot_kernel(DotParams p) {
  const int v = blockIdx.y, chunk = blockIdx.x;
  const int rx = p.rx[v], ry = p.ry[v];
  const long long npairs = (long long)rx * ry;
  const long long per = (npairs + p.chunks - 1) / p.chunks;
  const long long e0 = chunk * per, e1 = min(npairs, e0 + per);
  double acc = 0.0;
  for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int i = (int)(e / ry), j = (int)(e % ry);
    const double* a = p.base + (p.x_off[v] + i) * (long long)p.nD;
    const double* b = p.base + (p.y_off[v] + j) * (long long)p.nD;
    double prod = p.coef[p.x_off[v] + i] * p.coef[p.y_off[v] + j];
    int s = 0;
    for (int d = 0; d < p.ndof; ++d) {
      const int n = p.nbas[d];
      double t = 0.0;
      for (int q = 0; q < n; ++q) t += a[s + q] * b[s + q];
      prod *= t;
      s += n;
    }
    acc += prod;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) p.partial[(long long)v * p.chunks + chunk] = red[0];
}

__global__ void cp_dot_finish(const double* partial, int chunks, int nvec, double* out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvec) return;
  double s = 0.0;
  for (int c = 0; c < chunks; ++c) s += partial[(long long)v * chunks + c];
  out[v] = s;
}

}  // namespace

int cp_dot_device(Context* ctx, int nvec, int ndof, const int* nbas, const long long* x_off, const int* rx,
                  const long long* y_off, const int* ry, const double* d_coef, const double* d_base, double* d_out,
                  cudaStream_t st) {
  if (nvec < 1 || ndof < 1) {
    set_error("mlcp_cp_dot_batched: nvec and ndof must be positive");
    return kBadArgument;
  }
  int nD = 0;
  for (int d = 0; d < ndof; ++d) nD += nbas[d];
  const int chunks = std::max(1, (2 * ctx->num_sms + nvec - 1) / nvec);
  const size_t n_int = (size_t)ndof + 2 * nvec;
  const size_t meta = align256(n_int * sizeof(int)) + 2 * nvec * sizeof(long long);
  void* ws = nullptr;
  int rc = ensure_workspace(ctx, align256(meta) + sizeof(double) * (size_t)nvec * chunks, &ws);
  if (rc) return rc;
  void* stage = nullptr;
  rc = ensure_stage(ctx, meta, &stage);
  if (rc) return rc;
  int* hi = static_cast<int*>(stage);
  std::memcpy(hi, nbas, sizeof(int) * ndof);
  std::memcpy(hi + ndof, rx, sizeof(int) * nvec);
  std::memcpy(hi + ndof + nvec, ry, sizeof(int) * nvec);
  long long* hl = reinterpret_cast<long long*>(static_cast<char*>(stage) + align256(n_int * sizeof(int)));
  std::memcpy(hl, x_off, sizeof(long long) * nvec);
  std::memcpy(hl + nvec, y_off, sizeof(long long) * nvec);
  char* w = static_cast<char*>(ws);
  MLCP_CUDA_TRY(cudaMemcpyAsync(w, stage, meta, cudaMemcpyHostToDevice, st));
  MLCP_CUDA_TRY(cudaEventRecord(ctx->staged, st));
  DotParams p;
  p.nvec = nvec;
  p.ndof = ndof;
  p.nD = nD;
  p.chunks = chunks;
  p.nbas = reinterpret_cast<const int*>(w);
  p.rx = p.nbas + ndof;
  p.ry = p.rx + nvec;
  p.x_off = reinterpret_cast<const long long*>(w + align256(n_int * sizeof(int)));
  p.y_off = p.x_off + nvec;
  p.coef = d_coef;
  p.base = d_base;
  p.partial = reinterpret_cast<double*>(w + align256(meta));
  cp_dot_kernel<<<dim3(chunks, nvec), 256, 0, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  cp_dot_finish<<<(nvec + 127) / 128, 128, 0, st>>>(p.partial, chunks, nvec, d_out);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp

// ---------------------------------------------------------------------------
// extern "C" layer
// ---------------------------------------------------------------------------

using namespace mlcp;

extern "C" const char* mlcp_gb300_last_error(void) { return last_error(); }

extern "C" int mlcp_gb300_wait_selftest(int* flags_out) {
  int rc = kOk;
  Context* ctx = get_context(&rc);
  if (!ctx) return finish(rc);
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!flags_out) {
    set_error("mlcp_gb300_wait_selftest: null output");
    return finish(kBadArgument);
  }
  return finish(als_wait_selftest(ctx->stream, flags_out));
}

extern "C" void mlcp_gb300_set_kernel_timing(int enable) {
  int rc = kOk;
  Context* ctx = get_context(&rc);
  if (!ctx) return;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->timing = enable != 0;
}

extern "C" double mlcp_gb300_last_kernel_ms(void) {
  int rc = kOk;
  Context* ctx = get_context(&rc);
  if (!ctx) return -1.0;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ctx->timed) return -1.0;
  if (cudaEventSynchronize(ctx->t1) != cudaSuccess) return -1.0;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ctx->t0, ctx->t1) != cudaSuccess) return -1.0;
  return ms;
}
extern "C" int mlcp_gb300_last_status(void) { return t_status; }

extern "C" void mlcp_gb300_set_autotune(int enable) { set_autotune(enable); }

extern "C" void mlcp_gb300_set_als_engine(int engine) { set_als_engine(engine); }

extern "C" int mlcp_gb300_als_engine(void) { return als_engine(); }

extern "C" int mlcp_gb300_autotune_report(char* buf, int len) { return autotune_report(buf, len); }

static cudaStream_t pick_stream(Context* ctx, void* stream) {
  return stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
}

extern "C" int mlcp_als_batched(int nvec, int ndof, const int* nbas, const int* rF, const int* rG,
                                const long long* term_off, double* d_coef, double* d_base, int nals, int* d_status,
                                void* stream) {
  int rc = kOk;
  Context* ctx = get_context(&rc);
  if (!ctx) return finish(rc);
  std::lock_guard<std::mutex> lk(ctx->mu);
  AlsJob job;
  job.nvec = nvec; job.ndof = ndof; job.nals = nals; job.nbas = nbas; job.rF = rF; job.rG = rG;
  job.term_off = term_off; job.d_base = d_base; job.d_coef = d_coef; job.d_status = d_status;
  rc = als_run(ctx, job, pick_stream(ctx, stream));
  return finish(rc);
}

extern "C" int mlcp_als_batched_host(int nvec, int ndof, const int* nbas, const int* rF, const int* rG,
                                     const long long* term_off, double* h_coef, double* h_base, int nals,
                                     void* stream) {
  int rc = kOk;
  Context* ctx = get_context(&rc);
  if (!ctx) return finish(rc);
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (nals == 0) return finish(kOk);
  if (nvec < 1 || ndof < 1) {
    set_error("mlcp_als_batched_host: nvec and ndof must be positive");
    return finish(kBadArgument);
  }
  cudaStream_t st = pick_stream(ctx, stream);
  int nD = 0;
  for (int d = 0; d < ndof; ++d) nD += nbas[d];
  long long nterms = 0, nf = 0;
  for (int v = 0; v < nvec; ++v) {
    if (rF[v] < 1 || rG[v] < 1) {
      set_error("mlcp_als_batched_host: vector %d has rF=%d rG=%d (both must be positive)", v, rF[v], rG[v]);
      return finish(kBadArgument);
    }
    nterms = std::max(nterms, term_off[v] + rF[v] + rG[v]);
    nf += rF[v];
  }
  // Page-locked, mapped caller arrays (cudaHostAlloc, cudaHostRegister,
  // pinned torch tensors): the conversion kernel reads the target terms
  // straight from host memory, so crossing the host link and the FP64 ->
  // FP32 conversion are one pass, and only the F terms go through a device
  // buffer.  Other host memory: one copy of the whole batch.
  cudaPointerAttributes ab{}, ac{};
  const bool mapped = cudaPointerGetAttributes(&ab, h_base) == cudaSuccess && ab.type == cudaMemoryTypeHost &&
                      ab.devicePointer && cudaPointerGetAttributes(&ac, h_coef) == cudaSuccess &&
                      ac.type == cudaMemoryTypeHost && ac.devicePointer;
  (void)cudaGetLastError();
  // device copies live in their own allocation so the ALS workspace can grow
  // independently: the F terms only (mapped) or the whole batch
  const size_t need = sizeof(double) * (size_t)(mapped ? nf : nterms) * (nD + 1);
  if (need > ctx->io_bytes) {
    if (ctx->io) {
      cudaError_t e0 = cudaStreamSynchronize(st);
      if (e0 == cudaSuccess) e0 = cudaFree(ctx->io);
      if (e0 != cudaSuccess) {
        set_error("releasing the I/O buffer failed: %s", cudaGetErrorString(e0));
        return finish(kCudaError);
      }
    }
    ctx->io = nullptr;
    ctx->io_bytes = 0;
    cudaError_t e = cudaMalloc(&ctx->io, need);
    if (e != cudaSuccess) {
      set_error("cudaMalloc(%zu) failed: %s", need, cudaGetErrorString(e));
      return finish(kCudaError);
    }
    ctx->io_bytes = need;
  }
  double* d_buf = static_cast<double*>(ctx->io);
  double* d_base = d_buf;
  double* d_coef = d_buf + (size_t)(mapped ? nf : nterms) * nD;
  // F terms of vector v: host terms term_off[v].., device terms doff[v]..
  std::vector<long long> doff(nvec), gto(nvec);
  {
    long long o = 0;
    for (int v = 0; v < nvec; ++v) {
      doff[v] = mapped ? o : term_off[v];
      gto[v] = term_off[v] + rF[v];
      o += rF[v];
    }
  }
  // the F terms between host and device: one strided copy per array when the
  // vectors are evenly spaced with equal rF (the usual batch), else one copy
  // per vector
  bool even = nvec > 1;
  for (int v = 1; v < nvec && even; ++v)
    even = rF[v] == rF[0] && term_off[v] - term_off[v - 1] == term_off[1] - term_off[0];
  const long long hstep = nvec > 1 ? term_off[1] - term_off[0] : 0;
  even = even && hstep >= rF[0];
  auto copy_f = [&](cudaMemcpyKind kind) -> int {
    const bool h2d = kind == cudaMemcpyHostToDevice;
    const long long dstep = mapped ? rF[0] : hstep;
    cudaError_t e = cudaSuccess;
    if (even) {
      const size_t t0 = (size_t)term_off[0], w = sizeof(double) * (size_t)rF[0];
      double* hb = h_base + t0 * nD;
      double* hc = h_coef + t0;
      double* db = d_base + (size_t)doff[0] * nD;
      double* dc = d_coef + (size_t)doff[0];
      const size_t hpb = sizeof(double) * (size_t)hstep * nD, dpb = sizeof(double) * (size_t)dstep * nD;
      const size_t hpc = sizeof(double) * (size_t)hstep, dpc = sizeof(double) * (size_t)dstep;
      e = h2d ? cudaMemcpy2DAsync(db, dpb, hb, hpb, w * nD, nvec, kind, st)
              : cudaMemcpy2DAsync(hb, hpb, db, dpb, w * nD, nvec, kind, st);
      if (e == cudaSuccess)
        e = h2d ? cudaMemcpy2DAsync(dc, dpc, hc, hpc, w, nvec, kind, st)
                : cudaMemcpy2DAsync(hc, hpc, dc, dpc, w, nvec, kind, st);
    } else {
      for (int v = 0; v < nvec && e == cudaSuccess; ++v) {
        double* hb = h_base + (size_t)term_off[v] * nD;
        double* db = d_base + (size_t)doff[v] * nD;
        const size_t bb = sizeof(double) * (size_t)rF[v] * nD, bc = sizeof(double) * (size_t)rF[v];
        e = h2d ? cudaMemcpyAsync(db, hb, bb, kind, st) : cudaMemcpyAsync(hb, db, bb, kind, st);
        if (e == cudaSuccess)
          e = h2d ? cudaMemcpyAsync(d_coef + doff[v], h_coef + term_off[v], bc, kind, st)
                  : cudaMemcpyAsync(h_coef + term_off[v], d_coef + doff[v], bc, kind, st);
      }
    }
    if (e != cudaSuccess) {
      set_error("copying the F terms failed: %s", cudaGetErrorString(e));
      return kCudaError;
    }
    return kOk;
  };
  AlsJob job;
  job.nvec = nvec; job.ndof = ndof; job.nals = nals; job.nbas = nbas; job.rF = rF; job.rG = rG;
  job.d_base = d_base; job.d_coef = d_coef;
  if (mapped) {
    if ((rc = copy_f(cudaMemcpyHostToDevice))) return finish(rc);
    job.term_off = doff.data();
    job.g_base = static_cast<const double*>(ab.devicePointer);
    job.g_coef = static_cast<const double*>(ac.devicePointer);
    job.g_term_off = gto.data();
    job.g_host = true;
  } else {
    cudaError_t e = cudaMemcpyAsync(d_base, h_base, sizeof(double) * (size_t)nterms * nD, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_coef, h_coef, sizeof(double) * (size_t)nterms, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      set_error("cudaMemcpyAsync failed: %s", cudaGetErrorString(e));
      return finish(kCudaError);
    }
    job.term_off = term_off;
  }
  rc = als_run(ctx, job, st);
  if (rc) return finish(rc);
  if ((rc = copy_f(cudaMemcpyDeviceToHost))) return finish(rc);
  if (!stream) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error("ALS failed: %s", cudaGetErrorString(e));
      return finish(kCudaError);
    }
  }
  return finish(kOk);
}

extern "C" int mlcp_cp_dot_batched(int nvec, int ndof, const int* nbas, const long long* x_off, const int* rx,
                                   const long long* y_off, const int* ry, const double* d_coef,
                                   const double* d_base, double* d_out, void* stream) {
  int rc = kOk;
  Context* ctx = get_context(&rc);
  if (!ctx) return finish(rc);
  std::lock_guard<std::mutex> lk(ctx->mu);
  rc = cp_dot_device(ctx, nvec, ndof, nbas, x_off, rx, y_off, ry, d_coef, d_base, d_out, pick_stream(ctx, stream));
  return finish(rc);
}

// Reference src/intertwining.cu:180.  Same argument meaning; the whole
// reduction runs in one cluster launch and the context is kept.
extern "C" void alscpp_(double* coef, double* base, int* nbas, const int& ndof, const int& rF, const int& rG,
                        const int& nals) {
  if (nals == 0) {
    finish(kOk);
    return;
  }
  // The reference walks the target in blocks of rF terms (nbloc = (rF+rG)/rF,
  // src/intertwining.cu:189, src/als.cu:1003), so only the first
  // (rG/rF)*rF target terms take part; callers pad G to a multiple of rF.
  const int rGe = (rG / rF) * rF;
  const long long term_off = 0;
  const int rc = mlcp_als_batched_host(1, ndof, nbas, &rF, &rGe, &term_off, coef, base, nals, nullptr);
  if (rc != kOk) fprintf(stderr, "alscpp_: %s\n", mlcp_gb300_last_error());
}
