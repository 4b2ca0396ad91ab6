// C-ABI of the GB300 Schur engine (declared in include/gschur_gb300.h).
//
// Host glue only: argument checks, a device workspace arena, host<->device
// staging, the fork/join of the size-bin kernels onto auxiliary streams and the
// optional CUDA-graph replay.  All arithmetic runs in the kernels.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gschur_gb300.h"
#include "gs_internal.h"

using namespace gsk;

static constexpr int kPipeChunks = 4;       // chunks of a pipelined host-buffer batched call
static constexpr int64_t kPipeMinCount = 2048;

struct gs_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t aux[kNumBins] = {};
  cudaStream_t cap = nullptr;
  cudaEvent_t fork = nullptr, join[kNumBins] = {};
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  bool timed = false;
  // mixed batched form: refinement counters (device) and events around the refinement
  unsigned long long* mix_stats = nullptr;
  cudaEvent_t mix_e0 = nullptr, mix_e1 = nullptr;
  bool mix_valid = false, mix_timed = false;
  char* dws = nullptr;
  size_t dws_cap = 0;
  std::string err;
  // cached graph of the batched launch sequence
  cudaGraphExec_t gexec = nullptr;
  std::vector<long long> gkey;
  // launch shapes of the batched kernels (gs_set_tuning); tun_gen changes with them
  BinTuning tun_real = default_tuning_real();
  BinTuning tun_cplx = default_tuning_cplx();
  BinTuning tun_mixed32 = default_tuning_mixed32();
  long long tun_gen = 0;
  std::string tun_source = "built-in defaults";
  // host-buffer batched calls: chunks whose copies overlap the other chunks' kernels
  bool pipe_ready = false;
  cudaStream_t pipe_s[kPipeChunks] = {}, pipe_aux[kPipeChunks][kNumBins] = {}, pipe_d2h = nullptr;
  cudaEvent_t pipe_h2d[kPipeChunks] = {}, pipe_fork[kPipeChunks] = {}, pipe_join[kPipeChunks][kNumBins] = {},
              pipe_done[kPipeChunks] = {}, pipe_out = nullptr;
};

namespace {

int set_err(gs_context* c, int code, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return code;
}

#define CK(...)                                                                           \
  do {                                                                                    \
    cudaError_t e_ = (__VA_ARGS__);                                                       \
    if (e_ != cudaSuccess)                                                                \
      return set_err(ctx, GS_CUDA, "%s failed: %s", #__VA_ARGS__, cudaGetErrorString(e_)); \
  } while (0)

// Bump allocator over the context's device arena.
struct Arena {
  size_t off = 0;
  template <class T> size_t take(size_t count) {
    off = (off + 255) & ~size_t(255);
    size_t at = off;
    off += count * sizeof(T);
    return at;
  }
};

int ensure_ws(gs_context* ctx, size_t bytes) {
  if (bytes <= ctx->dws_cap) return GS_OK;
  if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; ctx->gkey.clear(); }
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->dws) CK(cudaFree(ctx->dws));
  ctx->dws = nullptr;
  ctx->dws_cap = 0;
  size_t cap = std::max(bytes, (size_t)1 << 20);
  cap = cap + cap / 4;
  CK(cudaMalloc(&ctx->dws, cap));
  ctx->dws_cap = cap;
  return GS_OK;
}

// Fork the aux streams off `s`, run `body(aux)`, join back into `s`.
template <class F> int fork_join(gs_context* ctx, cudaStream_t s, F body) {
  CK(cudaEventRecord(ctx->fork, s));
  for (int i = 0; i < kNumBins; ++i) CK(cudaStreamWaitEvent(ctx->aux[i], ctx->fork, 0));
  cudaError_t e = body(ctx->aux);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  for (int i = 0; i < kNumBins; ++i) {
    CK(cudaEventRecord(ctx->join[i], ctx->aux[i]));
    CK(cudaStreamWaitEvent(s, ctx->join[i], 0));
  }
  return GS_OK;
}

}  // namespace

extern "C" {

int gs_version(void) { return 100; }

int gs_create(gs_context** out, int device) {
  if (!out) return GS_BADARG;
  *out = nullptr;
  gs_context* ctx = new gs_context();
  ctx->device = device;
  int rc = GS_OK;
  do {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { rc = set_err(ctx, GS_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e)); break; }
    e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) { rc = set_err(ctx, GS_CUDA, "device query: %s", cudaGetErrorString(e)); break; }
    if ((e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->cap, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreate(&ctx->t0)) != cudaSuccess || (e = cudaEventCreate(&ctx->t1)) != cudaSuccess) {
      rc = set_err(ctx, GS_CUDA, "stream/event create: %s", cudaGetErrorString(e));
      break;
    }
    for (int i = 0; i < kNumBins && e == cudaSuccess; ++i) {
      e = cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) { rc = set_err(ctx, GS_CUDA, "aux streams: %s", cudaGetErrorString(e)); break; }
    ctx->stream = ctx->own;
  } while (0);
  if (rc != GS_OK) {
    // keep the context so that gs_last_error can report; compute calls will fail
    *out = ctx;
    return rc;
  }
  *out = ctx;
  return GS_OK;
}

int gs_destroy(gs_context* ctx) {
  if (!ctx) return GS_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  if (ctx->dws) cudaFree(ctx->dws);
  for (int i = 0; i < kNumBins; ++i) {
    if (ctx->aux[i]) cudaStreamDestroy(ctx->aux[i]);
    if (ctx->join[i]) cudaEventDestroy(ctx->join[i]);
  }
  if (ctx->fork) cudaEventDestroy(ctx->fork);
  if (ctx->t0) cudaEventDestroy(ctx->t0);
  if (ctx->t1) cudaEventDestroy(ctx->t1);
  if (ctx->mix_stats) cudaFree(ctx->mix_stats);
  if (ctx->mix_e0) cudaEventDestroy(ctx->mix_e0);
  if (ctx->mix_e1) cudaEventDestroy(ctx->mix_e1);
  if (ctx->cap) cudaStreamDestroy(ctx->cap);
  if (ctx->pipe_ready) {
    for (int c = 0; c < kPipeChunks; ++c) {
      cudaStreamDestroy(ctx->pipe_s[c]);
      cudaEventDestroy(ctx->pipe_h2d[c]);
      cudaEventDestroy(ctx->pipe_fork[c]);
      cudaEventDestroy(ctx->pipe_done[c]);
      for (int i = 0; i < kNumBins; ++i) {
        cudaStreamDestroy(ctx->pipe_aux[c][i]);
        cudaEventDestroy(ctx->pipe_join[c][i]);
      }
    }
    cudaStreamDestroy(ctx->pipe_d2h);
    cudaEventDestroy(ctx->pipe_out);
  }
  if (ctx->own) cudaStreamDestroy(ctx->own);
  delete ctx;
  return GS_OK;
}

int gs_set_stream(gs_context* ctx, void* stream) {
  if (!ctx) return GS_BADARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
  return GS_OK;
}

const char* gs_last_error(const gs_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

float gs_last_kernel_ms(const gs_context* ctx) {
  if (!ctx || !ctx->timed) return -1.0f;
  float ms = -1.0f;
  if (cudaEventSynchronize(ctx->t1) != cudaSuccess) return -1.0f;
  if (cudaEventElapsedTime(&ms, ctx->t0, ctx->t1) != cudaSuccess) return -1.0f;
  return ms;
}

int gs_host_alloc(gs_context* ctx, void** ptr, size_t bytes) {
  if (!ctx || !ptr) return GS_BADARG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaHostAlloc(ptr, bytes, cudaHostAllocDefault));
  return GS_OK;
}

int gs_host_free(gs_context* ctx, void* ptr) {
  if (!ctx) return GS_BADARG;
  if (ptr) CK(cudaFreeHost(ptr));
  return GS_OK;
}

// ---------------------------------------------------------------------------
// tuning table of the batched kernels
// ---------------------------------------------------------------------------
static std::string tuning_text(const gs_context* ctx) {
  std::string t = "# gschur_gb300 batched tuning (" + ctx->tun_source + ")\n# kind bin nmax threads hsmem ctas_per_sm\n";
  char line[128];
  static const char* kinds[3] = {"real_f64", "complex_f64", "mixed_f32"};
  for (int k = 0; k < 3; ++k) {
    const BinTuning& b = k == kTuneReal ? ctx->tun_real : (k == kTuneCplx ? ctx->tun_cplx : ctx->tun_mixed32);
    for (int i = 0; i < kNumBins; ++i) {
      snprintf(line, sizeof(line), "%s %d %d %d %d %d\n", kinds[k], i, b.bounds[i], b.nt[i], b.hsmem[i], b.ctas[i]);
      t += line;
    }
  }
  return t;
}

int gs_set_tuning(gs_context* ctx, const char* path) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  BinTuning tr = default_tuning_real(), tc = default_tuning_cplx(), tm = default_tuning_mixed32();
  std::string source = "built-in defaults";
  if (path && path[0]) {
    FILE* f = fopen(path, "r");
    if (!f) return set_err(ctx, GS_BADARG, "tuning table %s: cannot open", path);
    char line[512];
    int lineno = 0, rc = GS_OK;
    while (rc == GS_OK && fgets(line, sizeof(line), f)) {
      ++lineno;
      char* p = line;
      while (*p == ' ' || *p == '\t') ++p;
      if (*p == '#' || *p == '\n' || *p == '\r' || *p == 0) continue;
      char kind[64];
      int bin, nmax, nt, hs, ctas;
      if (sscanf(p, "%63s %d %d %d %d %d", kind, &bin, &nmax, &nt, &hs, &ctas) != 6) {
        rc = set_err(ctx, GS_BADARG, "tuning table %s:%d: expected 'kind bin nmax threads hsmem ctas_per_sm'", path,
                     lineno);
        break;
      }
      const int k = !strcmp(kind, "real_f64")
                        ? kTuneReal
                        : (!strcmp(kind, "complex_f64") ? kTuneCplx : (!strcmp(kind, "mixed_f32") ? kTuneMixed32 : -1));
      if (k < 0 || bin < 0 || bin >= kNumBins || ctas < 0 || (hs != 0 && hs != 1) ||
          !tuning_shape_ok(k, nmax, nt, hs) || (k == kTuneMixed32 && nmax != bin_max(bin))) {
        rc = set_err(ctx, GS_BADARG, "tuning table %s:%d: unknown kind, bin, a shape that is not compiled or does "
                     "not fit in shared memory, or a mixed_f32 bound other than the default", path, lineno);
        break;
      }
      BinTuning& b = k == kTuneReal ? tr : (k == kTuneCplx ? tc : tm);
      b.bounds[bin] = nmax;
      b.nt[bin] = nt;
      b.hsmem[bin] = hs;
      b.ctas[bin] = ctas;
    }
    fclose(f);
    if (rc != GS_OK) return rc;
    for (int k = 0; k < 3; ++k) {
      const BinTuning& b = k == kTuneReal ? tr : (k == kTuneCplx ? tc : tm);
      for (int i = 0; i < kNumBins; ++i)
        if (b.bounds[i] < 1 || (i > 0 && b.bounds[i] <= b.bounds[i - 1]))
          return set_err(ctx, GS_BADARG, "tuning table %s: bin bounds must increase", path);
      if (b.bounds[kNumBins - 1] != kSmallMax)
        return set_err(ctx, GS_BADARG, "tuning table %s: the last bin must end at %d", path, kSmallMax);
      for (int i = 0; i < kNumBins; ++i)  // a bin whose bound moved must still fit its shape
        if (!tuning_shape_ok(k, b.bounds[i], b.nt[i], b.hsmem[i]))
          return set_err(ctx, GS_BADARG, "tuning table %s: bin %d shape does not fit", path, i);
    }
    source = path;
  }
  ctx->tun_real = tr;
  ctx->tun_cplx = tc;
  ctx->tun_mixed32 = tm;
  ctx->tun_source = source;
  ++ctx->tun_gen;
  return GS_OK;
}

int gs_get_tuning(const gs_context* ctx, char* buf, size_t len) {
  if (!ctx || !buf || len == 0) return GS_BADARG;
  const std::string t = tuning_text(ctx);
  const size_t m = std::min(len - 1, t.size());
  memcpy(buf, t.data(), m);
  buf[m] = 0;
  return t.size() < len ? GS_OK : GS_BADARG;
}

// ---------------------------------------------------------------------------
// batched real
// ---------------------------------------------------------------------------
}  // extern "C"
// Run `enqueue` on the context stream, or replay it as a CUDA graph cached under `key`
// (captured on the first call with that key).  Brackets the work with the timing events.
template <class F>
static int run_graph_or_direct(gs_context* ctx, bool use_graph, const std::vector<long long>& key, F enqueue) {
  CK(cudaEventRecord(ctx->t0, ctx->stream));
  if (use_graph) {
    if (!ctx->gexec || ctx->gkey != key) {
      if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
      CK(cudaStreamBeginCapture(ctx->cap, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue(ctx->cap);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(ctx->cap, &g);
      if (rc != GS_OK) { if (g) cudaGraphDestroy(g); return rc; }
      if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "graph capture: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&ctx->gexec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { ctx->gexec = nullptr; return set_err(ctx, GS_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
      ctx->gkey = key;
    }
    CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
  } else {
    int rc = enqueue(ctx->stream);
    if (rc != GS_OK) return rc;
  }
  CK(cudaEventRecord(ctx->t1, ctx->stream));
  ctx->timed = true;
  return GS_OK;
}

template <class T, class W>
static int run_batched_real(gs_context* ctx, const RealBatchT<T, W>& bt, int* order, int* sched, unsigned flags,
                            bool use_graph, const std::vector<long long>& key) {
  // FP64 runs the context's tuned shapes; the FP32 instances the defaults
  constexpr bool tuned = sizeof(T) == 8 && sizeof(W) == 8;
  BinBounds bounds;
  for (int i = 0; i < kNumBins; ++i) bounds.b[i] = tuned ? ctx->tun_real.bounds[i] : bin_max(i);
  auto enqueue = [&](cudaStream_t s) -> int {
    cudaError_t e = launch_bin_sort(bt.ns, bt.count, order, sched, bounds, s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "bin sort launch: %s", cudaGetErrorString(e));
    return fork_join(ctx, s, [&](cudaStream_t* aux) {
      if constexpr (tuned)
        return launch_schur_batched_real_tuned(bt, order, sched, ctx->num_sms, aux, kNumBins, ctx->tun_real);
      else
        return launch_schur_batched_real(bt, order, sched, ctx->num_sms, aux, kNumBins);
    });
  };
  return run_graph_or_direct(ctx, use_graph, key, enqueue);
}

static int pipe_setup(gs_context* ctx) {
  if (ctx->pipe_ready) return GS_OK;
  for (int c = 0; c < kPipeChunks; ++c) {
    CK(cudaStreamCreateWithFlags(&ctx->pipe_s[c], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->pipe_h2d[c], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->pipe_fork[c], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->pipe_done[c], cudaEventDisableTiming));
    for (int i = 0; i < kNumBins; ++i) {
      CK(cudaStreamCreateWithFlags(&ctx->pipe_aux[c][i], cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&ctx->pipe_join[c][i], cudaEventDisableTiming));
    }
  }
  CK(cudaStreamCreateWithFlags(&ctx->pipe_d2h, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->pipe_out, cudaEventDisableTiming));
  ctx->pipe_ready = true;
  return GS_OK;
}

// Host-buffer batched call as a pipeline: the batch is cut into kPipeChunks runs of
// consecutive matrices (the first and last small, so that little copying is exposed),
// each run's inputs are copied on the context stream, its compute (`launch_run(c, b0, b1,
// stream)`: bin sort and kernels of matrices [b0, b1), forked onto the run's own aux
// streams) runs on a stream of its own once its copy has landed, and its outputs are
// copied back on a separate stream once its kernels are done.  So the copies of one run
// overlap the kernels of the others, and the runs' kernels overlap each other's tails.
// Requires the matrices to be stored in order (offsets increasing, not overlapping), which
// makes each run one contiguous range of every buffer.  dA, dZ, dwr, dwi, dst: the device
// copies (dns, doffs, dwoffs the metadata); device layout as the unpipelined call.
template <class T, class F>
static int batched_pipelined(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                             const int64_t* woffs, T* A, T* Z, T* wr, T* wi, int32_t* status, int* dns,
                             long long* doffs, long long* dwoffs, T* dA, T* dZ, T* dwr, T* dwi, int* dst,
                             F launch_run) {
  int rc = pipe_setup(ctx);
  if (rc) return rc;
  // run boundaries by cumulative n^3 work: 10%, 40%, 40%, 10%
  double tot = 0.0;
  for (int64_t b = 0; b < count; ++b) tot += (double)ns[b] * ns[b] * ns[b];
  const double cut[kPipeChunks - 1] = {0.1, 0.5, 0.9};
  int64_t edge[kPipeChunks + 1];
  edge[0] = 0;
  edge[kPipeChunks] = count;
  {
    double run = 0.0;
    int k = 0;
    for (int64_t b = 0; b < count && k < kPipeChunks - 1; ++b) {
      run += (double)ns[b] * ns[b] * ns[b];
      while (k < kPipeChunks - 1 && run >= cut[k] * tot) edge[++k] = b + 1;
    }
    while (k < kPipeChunks - 1) edge[++k] = count;
  }
  cudaStream_t s = ctx->stream;
  // metadata for the whole batch first (small), then the runs' matrices in order
  CK(cudaMemcpyAsync(dns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(doffs, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dwoffs, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
  auto a_lo = [&](int64_t b) { return (long long)offs[b]; };
  auto a_hi = [&](int64_t b) { return (long long)offs[b - 1] + (long long)ns[b - 1] * ns[b - 1]; };
  auto w_lo = [&](int64_t b) { return (long long)woffs[b]; };
  auto w_hi = [&](int64_t b) { return (long long)woffs[b - 1] + ns[b - 1]; };
  for (int c = 0; c < kPipeChunks; ++c) {
    const int64_t b0 = edge[c], b1 = edge[c + 1];
    if (b1 > b0) {
      const long long lo = a_lo(b0), hi = a_hi(b1);
      CK(cudaMemcpyAsync(dA + lo, A + lo, sizeof(T) * (hi - lo), cudaMemcpyHostToDevice, s));
    }
    CK(cudaEventRecord(ctx->pipe_h2d[c], s));
  }
  bool timed = false;
  for (int c = 0; c < kPipeChunks; ++c) {
    const int64_t b0 = edge[c], b1 = edge[c + 1];
    cudaStream_t cs = ctx->pipe_s[c];
    CK(cudaStreamWaitEvent(cs, ctx->pipe_h2d[c], 0));
    if (b1 > b0) {
      if (!timed) { CK(cudaEventRecord(ctx->t0, cs)); timed = true; }
      rc = launch_run(c, b0, b1, cs);
      if (rc) return rc;
    }
    CK(cudaEventRecord(ctx->pipe_done[c], cs));
  }
  // kernel time: from the first run's start to the end of every run's kernels
  cudaStream_t last = ctx->pipe_s[kPipeChunks - 1];
  for (int c = 0; c < kPipeChunks - 1; ++c) CK(cudaStreamWaitEvent(last, ctx->pipe_done[c], 0));
  if (timed) {
    CK(cudaEventRecord(ctx->t1, last));
    ctx->timed = true;
  }
  cudaStream_t d = ctx->pipe_d2h;
  for (int c = 0; c < kPipeChunks; ++c) {
    const int64_t b0 = edge[c], b1 = edge[c + 1];
    CK(cudaStreamWaitEvent(d, ctx->pipe_done[c], 0));
    if (b1 <= b0) continue;
    const long long lo = a_lo(b0), hi = a_hi(b1), wlo = w_lo(b0), whi = w_hi(b1);
    CK(cudaMemcpyAsync(A + lo, dA + lo, sizeof(T) * (hi - lo), cudaMemcpyDeviceToHost, d));
    if (dZ) CK(cudaMemcpyAsync(Z + lo, dZ + lo, sizeof(T) * (hi - lo), cudaMemcpyDeviceToHost, d));
    if (whi > wlo) {
      CK(cudaMemcpyAsync(wr + wlo, dwr + wlo, sizeof(T) * (whi - wlo), cudaMemcpyDeviceToHost, d));
      CK(cudaMemcpyAsync(wi + wlo, dwi + wlo, sizeof(T) * (whi - wlo), cudaMemcpyDeviceToHost, d));
    }
    CK(cudaMemcpyAsync(status + b0, dst + b0, sizeof(int) * (b1 - b0), cudaMemcpyDeviceToHost, d));
  }
  CK(cudaEventRecord(ctx->pipe_out, d));
  CK(cudaStreamWaitEvent(s, ctx->pipe_out, 0));
  CK(cudaStreamSynchronize(s));
  for (int64_t b = 0; b < count; ++b)
    if (status[b] != GS_OK) return set_err(ctx, GS_UNCONVERGED, "matrix %lld: iteration limit reached", (long long)b);
  return GS_OK;
}

template <class T>
static int schur_batched_real_pipelined(gs_context* ctx, const RealBatchT<T, T>& bt, int64_t count,
                                        const int32_t* ns, const int64_t* offs, const int64_t* woffs, T* A, T* Z,
                                        T* wr, T* wi, int32_t* status, int* order, int* sched) {
  constexpr bool tuned = sizeof(T) == 8;
  BinBounds bounds;
  for (int i = 0; i < kNumBins; ++i) bounds.b[i] = tuned ? ctx->tun_real.bounds[i] : bin_max(i);
  return batched_pipelined<T>(
      ctx, count, ns, offs, woffs, A, Z, wr, wi, status, (int*)bt.ns, (long long*)bt.offs, (long long*)bt.woffs,
      bt.A, bt.Z, bt.wr, bt.wi, bt.status, [&](int c, int64_t b0, int64_t b1, cudaStream_t cs) -> int {
        RealBatchT<T, T> bc = bt;
        bc.count = (int)(b1 - b0);
        bc.ns = bt.ns + b0;
        bc.offs = bt.offs + b0;
        bc.woffs = bt.woffs + b0;
        bc.status = bt.status + b0;
        int* oc = order + b0;  // each run sorts its own slice of the order array
        int* sc = sched + 3 * kNumBins * c;
        cudaError_t e = launch_bin_sort(bc.ns, bc.count, oc, sc, bounds, cs);
        if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "bin sort launch: %s", cudaGetErrorString(e));
        CK(cudaEventRecord(ctx->pipe_fork[c], cs));
        for (int i = 0; i < kNumBins; ++i) CK(cudaStreamWaitEvent(ctx->pipe_aux[c][i], ctx->pipe_fork[c], 0));
        if constexpr (tuned)
          e = launch_schur_batched_real_tuned(bc, oc, sc, ctx->num_sms, ctx->pipe_aux[c], kNumBins, ctx->tun_real);
        else
          e = launch_schur_batched_real(bc, oc, sc, ctx->num_sms, ctx->pipe_aux[c], kNumBins);
        if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
        for (int i = 0; i < kNumBins; ++i) {
          CK(cudaEventRecord(ctx->pipe_join[c][i], ctx->pipe_aux[c][i]));
          CK(cudaStreamWaitEvent(cs, ctx->pipe_join[c][i], 0));
        }
        return GS_OK;
      });
}

template <class T>
static int schur_batched_real_impl(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                   const int64_t* woffs, T* A, T* Z, T* wr, T* wi, int32_t* status, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (count < 0 || count > (1LL << 30)) return set_err(ctx, GS_BADARG, "bad count %lld", (long long)count);
  if (count == 0) return GS_OK;
  const bool wantz = flags & GS_WANTZ;
  if (!ns || !offs || !woffs || !A || !wr || !wi || !status || (wantz && !Z))
    return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  RealBatchT<T, T> bt{};
  bt.count = (int)count;
  bt.wantz = wantz;
  bt.scale = (flags & GS_SCALE) ? 1 : 0;
  bt.maxiter_mult = 100;
  Arena ar;
  long long na = 0, nw = 0;
  bool in_order = true;  // matrices stored one after another (the pipelined copy needs it)
  if (!dev) {
    for (int64_t b = 0; b < count; ++b) {
      const int n = ns[b];
      if (n < 0 || n > kSmallMax)
        return set_err(ctx, GS_BADARG, "matrix %lld: order %d outside [0, %d]", (long long)b, n, kSmallMax);
      if (offs[b] < 0 || woffs[b] < 0) return set_err(ctx, GS_BADARG, "matrix %lld: negative offset", (long long)b);
      if (b > 0 && (offs[b] < offs[b - 1] + (long long)ns[b - 1] * ns[b - 1] || woffs[b] < woffs[b - 1] + ns[b - 1]))
        in_order = false;
      na = std::max(na, (long long)offs[b] + (long long)n * n);
      nw = std::max(nw, (long long)woffs[b] + n);
    }
  }
  const bool pipelined = !dev && !(flags & GS_GRAPH) && in_order && count >= kPipeMinCount;
  const size_t o_order = ar.take<int>(count);
  const size_t o_sched = ar.take<int>(3 * kNumBins * kPipeChunks);
  size_t o_A = 0, o_Z = 0, o_wr = 0, o_wi = 0, o_ns = 0, o_offs = 0, o_woffs = 0, o_st = 0;
  if (!dev) {
    o_A = ar.take<T>(na);
    o_Z = ar.take<T>(wantz ? na : 1);
    o_wr = ar.take<T>(nw);
    o_wi = ar.take<T>(nw);
    o_ns = ar.take<int>(count);
    o_offs = ar.take<long long>(count);
    o_woffs = ar.take<long long>(count);
    o_st = ar.take<int>(count);
  }
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  int* order = (int*)(base + o_order);
  int* sched = (int*)(base + o_sched);
  cudaStream_t s = ctx->stream;
  if (!dev) {
    bt.ns = (const int*)(base + o_ns);
    bt.offs = (const long long*)(base + o_offs);
    bt.woffs = (const long long*)(base + o_woffs);
    bt.A = (T*)(base + o_A);
    bt.Z = wantz ? (T*)(base + o_Z) : nullptr;
    bt.wr = (T*)(base + o_wr);
    bt.wi = (T*)(base + o_wi);
    bt.status = (int*)(base + o_st);
    if (pipelined)
      return schur_batched_real_pipelined<T>(ctx, bt, count, ns, offs, woffs, A, Z, wr, wi, status, order, sched);
    CK(cudaMemcpyAsync((void*)bt.ns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)bt.offs, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)bt.woffs, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(bt.A, A, sizeof(T) * na, cudaMemcpyHostToDevice, s));
  } else {
    bt.ns = ns;
    bt.offs = (const long long*)offs;
    bt.woffs = (const long long*)woffs;
    bt.A = A;
    bt.Z = wantz ? Z : nullptr;
    bt.wr = wr;
    bt.wi = wi;
    bt.status = status;
  }
  std::vector<long long> key = {(long long)sizeof(T), (long long)count, (long long)(uintptr_t)bt.A, (long long)(uintptr_t)bt.Z,
                                (long long)(uintptr_t)bt.ns, (long long)(uintptr_t)bt.wr,
                                (long long)(uintptr_t)order, (long long)flags, ctx->tun_gen};
  rc = run_batched_real(ctx, bt, order, sched, flags, (flags & GS_GRAPH) != 0, key);
  if (rc) return rc;
  if (dev) return GS_OK;
  CK(cudaMemcpyAsync(A, bt.A, sizeof(T) * na, cudaMemcpyDeviceToHost, s));
  if (wantz) CK(cudaMemcpyAsync(Z, bt.Z, sizeof(T) * na, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(wr, bt.wr, sizeof(T) * nw, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(wi, bt.wi, sizeof(T) * nw, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(status, bt.status, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int64_t b = 0; b < count; ++b)
    if (status[b] != GS_OK) return set_err(ctx, GS_UNCONVERGED, "matrix %lld: iteration limit reached", (long long)b);
  return GS_OK;
}

// GS_MIXED: FP32 Schur pairs refined to FP64 (refine_batched.cu).  Same arguments and
// results as the FP64 batched call; the workspace grows with the batch (five FP32 and
// two or three FP64 copies of A), so a device-pointer call first reads the batch's
// extents back from the device.
static int schur_batched_mixed_impl(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                                    const int64_t* woffs, double* A, double* Z, double* wr, double* wi,
                                    int32_t* status, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (count < 0 || count > (1LL << 30)) return set_err(ctx, GS_BADARG, "bad count %lld", (long long)count);
  if (count == 0) return GS_OK;
  const bool wantz = flags & GS_WANTZ;
  if (!ns || !offs || !woffs || !A || !wr || !wi || !status || (wantz && !Z))
    return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  cudaStream_t s = ctx->stream;
  long long na = 0, nw = 0;
  if (!dev) {
    for (int64_t b = 0; b < count; ++b) {
      const int n = ns[b];
      if (n < 0 || n > kSmallMax)
        return set_err(ctx, GS_BADARG, "matrix %lld: order %d outside [0, %d]", (long long)b, n, kSmallMax);
      if (offs[b] < 0 || woffs[b] < 0) return set_err(ctx, GS_BADARG, "matrix %lld: negative offset", (long long)b);
      na = std::max(na, (long long)offs[b] + (long long)n * n);
      nw = std::max(nw, (long long)woffs[b] + n);
    }
  } else {
    Arena ar0;
    const size_t o_ext = ar0.take<unsigned long long>(2);
    int rc = ensure_ws(ctx, ar0.off);
    if (rc) return rc;
    unsigned long long* dext = (unsigned long long*)(ctx->dws + o_ext);
    unsigned long long ext[2] = {0, 0};
    CK(cudaMemsetAsync(dext, 0, sizeof(ext), s));
    CK(launch_batch_extent(ns, (const long long*)offs, (const long long*)woffs, (int)count, dext, s));
    CK(cudaMemcpyAsync(ext, dext, sizeof(ext), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    na = (long long)ext[0];
    nw = (long long)ext[1];
  }
  Arena ar;
  const size_t o_order = ar.take<int>(count);
  const size_t o_sched = ar.take<int>(3 * kNumBins * kPipeChunks);
  size_t o_A = 0, o_Z = 0, o_wr = 0, o_wi = 0, o_ns = 0, o_offs = 0, o_woffs = 0, o_st = 0;
  if (!dev) {
    o_A = ar.take<double>(na);
    o_Z = ar.take<double>(wantz ? na : 1);
    o_wr = ar.take<double>(nw);
    o_wi = ar.take<double>(nw);
    o_ns = ar.take<int>(count);
    o_offs = ar.take<long long>(count);
    o_woffs = ar.take<long long>(count);
    o_st = ar.take<int>(count);
  }
  const size_t o_ws = ar.take<char>(mixed_batched_ws_bytes(na, nw, wantz));
  const size_t o_iws = ar.take<int>(mixed_batched_iws_ints(count));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  MixedBatch mb{};
  mb.count = (int)count;
  mb.order = (int*)(base + o_order);
  mb.sched = (int*)(base + o_sched);
  mb.ws = base + o_ws;
  mb.iws = (int*)(base + o_iws);
  if (!ctx->mix_stats) {
    CK(cudaMalloc(&ctx->mix_stats, 5 * sizeof(unsigned long long)));  // 4 counters, the error word
    CK(cudaEventCreate(&ctx->mix_e0));
    CK(cudaEventCreate(&ctx->mix_e1));
  }
  mb.stats = ctx->mix_stats;
  mb.tc_err = reinterpret_cast<int*>(ctx->mix_stats + 4);
  ctx->mix_valid = true;
  ctx->mix_timed = false;
  mb.na = na;
  mb.nw = nw;
  mb.scale = (flags & GS_SCALE) ? 1 : 0;
  mb.nofallback = (flags & GS_NOFALLBACK) ? 1 : 0;
  if (!dev) {
    mb.ns = (const int*)(base + o_ns);
    mb.offs = (const long long*)(base + o_offs);
    mb.woffs = (const long long*)(base + o_woffs);
    mb.A = (double*)(base + o_A);
    mb.Z = wantz ? (double*)(base + o_Z) : nullptr;
    mb.wr = (double*)(base + o_wr);
    mb.wi = (double*)(base + o_wi);
    mb.status = (int*)(base + o_st);
    CK(cudaMemcpyAsync((void*)mb.ns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)mb.offs, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)mb.woffs, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(mb.A, A, sizeof(double) * na, cudaMemcpyHostToDevice, s));
  } else {
    mb.ns = ns;
    mb.offs = (const long long*)offs;
    mb.woffs = (const long long*)woffs;
    mb.A = A;
    mb.Z = wantz ? Z : nullptr;
    mb.wr = wr;
    mb.wi = wi;
    mb.status = status;
  }
  std::vector<long long> key = {-1, (long long)count, (long long)(uintptr_t)mb.A, (long long)(uintptr_t)mb.Z,
                                (long long)(uintptr_t)mb.ns, (long long)(uintptr_t)mb.wr, (long long)(uintptr_t)mb.ws,
                                na, nw, (long long)flags, ctx->tun_gen};
  mb.ref0 = ctx->mix_e0;
  mb.ref1 = ctx->mix_e1;
  ctx->mix_timed = true;
  // Host-buffer calls: all inputs in, the whole sequence as one CUDA graph (captured on the
  // first call with these extents), all outputs out.  Runs of matrices whose copies overlap
  // the other runs' kernels (the FP64 form's pipeline) were measured slower here: each run
  // repeats the stages' tails (a large matrix's FP32 Schur and each Newton step), which
  // costs more than the 14 ms of copies it hides.
  const bool use_graph = (flags & GS_GRAPH) != 0 || !dev;
  rc = run_graph_or_direct(ctx, use_graph, key, [&](cudaStream_t st) -> int {
    CK(cudaMemsetAsync(mb.stats, 0, 5 * sizeof(unsigned long long), st));
    cudaError_t e = launch_mixed_batched(mb, ctx->num_sms, st, ctx->aux, kNumBins, ctx->fork, ctx->join, ctx->tun_real,
                                         ctx->tun_mixed32);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "mixed batched launch: %s", cudaGetErrorString(e));
    return GS_OK;
  });
  if (rc) return rc;
  if (dev) return GS_OK;
  CK(cudaMemcpyAsync(A, mb.A, sizeof(double) * na, cudaMemcpyDeviceToHost, s));
  if (wantz) CK(cudaMemcpyAsync(Z, mb.Z, sizeof(double) * na, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(wr, mb.wr, sizeof(double) * nw, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(wi, mb.wi, sizeof(double) * nw, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(status, mb.status, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int64_t b = 0; b < count; ++b)
    if (status[b] != GS_OK) return set_err(ctx, GS_UNCONVERGED, "matrix %lld: iteration limit reached", (long long)b);
  return GS_OK;
}

extern "C" {
int gs_schur_batched_f64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                         const int64_t* woffs, double* A, double* Z, double* wr, double* wi,
                         int32_t* status, unsigned flags) {
  if (flags & GS_MIXED) return schur_batched_mixed_impl(ctx, count, ns, offs, woffs, A, Z, wr, wi, status, flags);
  return schur_batched_real_impl<double>(ctx, count, ns, offs, woffs, A, Z, wr, wi, status, flags);
}

int gs_mixed_batched_info(gs_context* ctx, int64_t* info) {
  if (!ctx || !info) return GS_BADARG;
  ctx->err.clear();
  if (!ctx->mix_valid) return set_err(ctx, GS_BADARG, "no GS_MIXED batched call on this context yet");
  unsigned long long st[5] = {0, 0, 0, 0, 0};
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(st, ctx->mix_stats, sizeof(st), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; ++i) info[i] = (int64_t)st[i];
  info[4] = -1;
  info[5] = -1;
  float ms = 0.0f;
  if (ctx->mix_timed) {
    if (cudaEventElapsedTime(&ms, ctx->mix_e0, ctx->mix_e1) == cudaSuccess) info[4] = (int64_t)(1000.0 * ms);
    else (void)cudaGetLastError();  // not recorded: leave no error behind for the caller's next launch
    // the FP32 stage: from the start of the call's kernels to the start of the refinement
    if (ctx->timed && cudaEventElapsedTime(&ms, ctx->t0, ctx->mix_e0) == cudaSuccess) info[5] = (int64_t)(1000.0 * ms);
    else (void)cudaGetLastError();
  }
  // a tensor-core wait that timed out handed its matrix back to the FP64 kernel (results
  // stay correct); report it, with the counters filled
  if ((int)(st[4] & 0xffffffffu) != 0)
    return set_err(ctx, GS_CUDA, "a tensor-core wait of the refinement timed out (code %d)", (int)(st[4] & 0xffffffffu));
  return GS_OK;
}

int gs_schur_batched_f32(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                         const int64_t* woffs, float* A, float* Z, float* wr, float* wi,
                         int32_t* status, unsigned flags) {
  return schur_batched_real_impl<float>(ctx, count, ns, offs, woffs, A, Z, wr, wi, status, flags);
}

// ---------------------------------------------------------------------------
// large real matrix (n > 128): whole-GPU Hessenberg + multishift QR
// ---------------------------------------------------------------------------
}  // extern "C"
template <class T>
static int schur_large_impl(gs_context* ctx, int64_t n, T* A, int64_t lda, T* Z, int64_t ldz, T* wr, T* wi,
                            unsigned flags, int64_t maxiter) {
  if (n > (1 << 16)) return set_err(ctx, GS_BADARG, "order %lld too large", (long long)n);
  const bool wantz = flags & GS_WANTZ;
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  Arena ar;
  const size_t o_A = ar.take<T>(nn), o_Z = ar.take<T>(wantz ? nn : 1);
  const size_t o_wr = ar.take<double>(n), o_wi = ar.take<double>(n);
  const size_t o_w32 = ar.take<T>(2 * n);
  const size_t o_ws = ar.take<char>(schur_large_ws_bytes((int)n, sizeof(T)));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  T* dA = (T*)(base + o_A);
  CK(cudaMemcpy2DAsync(dA, n * sizeof(T), A, lda * sizeof(T), n * sizeof(T), n, in, s));
  LargeRun<T> r{};
  r.A = dA;
  r.Z = wantz ? (T*)(base + o_Z) : nullptr;
  r.wr = (double*)(base + o_wr);
  r.wi = (double*)(base + o_wi);
  r.n = (int)n;
  r.scale = (flags & GS_SCALE) ? 1 : 0;
  r.maxiter = maxiter > 0 ? maxiter : 0;
  r.ws = base + o_ws;
  r.num_sms = ctx->num_sms;
  r.stream = s;
  r.cuda_error = cudaSuccess;
  large_tuning((int)n, &r.bulges, &r.chunk, &r.aedw, sizeof(T));
  r.shift_fp32 = sizeof(T) == 8 ? large_shift_fp32() : 0;
  CK(cudaEventRecord(ctx->t0, s));
  const int st = schur_large_run<T>(r);
  if (st < 0) return set_err(ctx, GS_CUDA, "large Schur path: %s", cudaGetErrorString(r.cuda_error));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  CK(cudaMemcpy2DAsync(A, lda * sizeof(T), dA, n * sizeof(T), n * sizeof(T), n, out, s));
  if (wantz) CK(cudaMemcpy2DAsync(Z, ldz * sizeof(T), r.Z, n * sizeof(T), n * sizeof(T), n, out, s));
  // eigenvalues are produced in FP64; the element type's copy is made on the device
  T* w32 = (T*)(base + o_w32);
  CK(convert_array<double, T>(r.wr, w32, n, 1.0, s));
  CK(convert_array<double, T>(r.wi, w32 + n, n, 1.0, s));
  CK(cudaMemcpyAsync(wr, w32, n * sizeof(T), out, s));
  CK(cudaMemcpyAsync(wi, w32 + n, n * sizeof(T), out, s));
  CK(cudaStreamSynchronize(s));
  if (st != ST_OK) return set_err(ctx, GS_UNCONVERGED, "iteration limit reached");
  return GS_OK;
}

// ---------------------------------------------------------------------------
// single real matrix: n <= 128 runs as a batch of one
// ---------------------------------------------------------------------------
template <class T>
static int schur_real_impl(gs_context* ctx, int64_t n, T* A, int64_t lda, T* Z, int64_t ldz, T* wr, T* wi,
                           unsigned flags, int64_t maxiter) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  const bool wantz = flags & GS_WANTZ;
  if (n < 0) return set_err(ctx, GS_BADARG, "negative order");
  if (lda < std::max<int64_t>(n, 1) || (wantz && ldz < std::max<int64_t>(n, 1)))
    return set_err(ctx, GS_BADARG, "leading dimension smaller than n");
  if (n == 0) return GS_OK;
  if (!A || !wr || !wi || (wantz && !Z)) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  if (n > kSmallMax) return schur_large_impl<T>(ctx, n, A, lda, Z, ldz, wr, wi, flags, maxiter);
  const bool dev = flags & GS_DEVICE;
  Arena ar;
  const size_t o_A = ar.take<T>(n * n), o_Z = ar.take<T>(n * n);
  const size_t o_wr = ar.take<T>(n), o_wi = ar.take<T>(n);
  const size_t o_meta = ar.take<long long>(4), o_st = ar.take<int>(2);
  const size_t o_order = ar.take<int>(1), o_sched = ar.take<int>(3 * kNumBins);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  T* dA = (T*)(base + o_A);
  T* dZ = (T*)(base + o_Z);
  CK(cudaMemcpy2DAsync(dA, n * sizeof(T), A, lda * sizeof(T), n * sizeof(T), n, in, s));
  long long meta_h[4] = {0, 0, 0, 0};  // offs, woffs, n (as int in first half of [2])
  int n32 = (int)n;
  long long* meta = (long long*)(base + o_meta);
  CK(cudaMemcpyAsync(meta, meta_h, sizeof(meta_h), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(meta + 2, &n32, sizeof(int), cudaMemcpyHostToDevice, s));
  RealBatchT<T, T> bt{};
  bt.count = 1;
  bt.ns = (const int*)(meta + 2);
  bt.offs = meta;
  bt.woffs = meta + 1;
  bt.A = dA;
  bt.Z = wantz ? dZ : nullptr;
  bt.wr = (T*)(base + o_wr);
  bt.wi = (T*)(base + o_wi);
  bt.status = (int*)(base + o_st);
  bt.wantz = wantz;
  bt.scale = (flags & GS_SCALE) ? 1 : 0;
  long long mi = maxiter > 0 ? maxiter : 100 * n;
  bt.maxiter_mult = 100;
  bt.maxiter_abs = mi;
  rc = run_batched_real(ctx, bt, (int*)(base + o_order), (int*)(base + o_sched), flags, false, {});
  if (rc) return rc;
  CK(cudaMemcpy2DAsync(A, lda * sizeof(T), dA, n * sizeof(T), n * sizeof(T), n, out, s));
  if (wantz) CK(cudaMemcpy2DAsync(Z, ldz * sizeof(T), dZ, n * sizeof(T), n * sizeof(T), n, out, s));
  CK(cudaMemcpyAsync(wr, bt.wr, n * sizeof(T), out, s));
  CK(cudaMemcpyAsync(wi, bt.wi, n * sizeof(T), out, s));
  int st = 0;
  CK(cudaMemcpyAsync(&st, bt.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (st != GS_OK) return set_err(ctx, GS_UNCONVERGED, "iteration limit %lld reached", mi);
  return GS_OK;
}

extern "C" {
int gs_schur_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* Z, int64_t ldz, double* wr,
                 double* wi, unsigned flags, int64_t maxiter) {
  return schur_real_impl<double>(ctx, n, A, lda, Z, ldz, wr, wi, flags, maxiter);
}

int gs_schur_f32(gs_context* ctx, int64_t n, float* A, int64_t lda, float* Z, int64_t ldz, float* wr, float* wi,
                 unsigned flags, int64_t maxiter) {
  return schur_real_impl<float>(ctx, n, A, lda, Z, ldz, wr, wi, flags, maxiter);
}

// ---------------------------------------------------------------------------
// complex: batched and single
// ---------------------------------------------------------------------------
static int run_batched_cplx(gs_context* ctx, const CplxBatch& bt, int* order, int* sched, bool use_graph,
                            const std::vector<long long>& key) {
  BinBounds bounds;
  for (int i = 0; i < kNumBins; ++i) bounds.b[i] = ctx->tun_cplx.bounds[i];
  auto enqueue = [&](cudaStream_t s) -> int {
    cudaError_t e = launch_bin_sort(bt.ns, bt.count, order, sched, bounds, s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "bin sort launch: %s", cudaGetErrorString(e));
    return fork_join(ctx, s, [&](cudaStream_t* aux) {
      return launch_schur_batched_cplx_tuned(bt, order, sched, ctx->num_sms, aux, kNumBins, ctx->tun_cplx);
    });
  };
  CK(cudaEventRecord(ctx->t0, ctx->stream));
  if (use_graph) {
    if (!ctx->gexec || ctx->gkey != key) {
      if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
      CK(cudaStreamBeginCapture(ctx->cap, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue(ctx->cap);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(ctx->cap, &g);
      if (rc != GS_OK) { if (g) cudaGraphDestroy(g); return rc; }
      if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "graph capture: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&ctx->gexec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { ctx->gexec = nullptr; return set_err(ctx, GS_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
      ctx->gkey = key;
    }
    CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
  } else {
    int rc = enqueue(ctx->stream);
    if (rc != GS_OK) return rc;
  }
  CK(cudaEventRecord(ctx->t1, ctx->stream));
  ctx->timed = true;
  return GS_OK;
}

int gs_schur_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                         const int64_t* woffs, double* A, double* Z, double* w, int32_t* status, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (count < 0 || count > (1LL << 30)) return set_err(ctx, GS_BADARG, "bad count %lld", (long long)count);
  if (count == 0) return GS_OK;
  const bool wantz = flags & GS_WANTZ;
  if (!ns || !offs || !woffs || !A || !w || !status || (wantz && !Z))
    return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  CplxBatch bt{};
  bt.count = (int)count;
  bt.wantz = wantz;
  bt.scale = (flags & GS_SCALE) ? 1 : 0;
  bt.maxiter_mult = 100;
  bt.maxinner_mult = 30;
  Arena ar;
  long long na = 0, nw = 0;
  if (!dev) {
    for (int64_t b = 0; b < count; ++b) {
      const int n = ns[b];
      if (n < 0 || n > kSmallMax)
        return set_err(ctx, GS_BADARG, "matrix %lld: order %d outside [0, %d]", (long long)b, n, kSmallMax);
      if (offs[b] < 0 || woffs[b] < 0) return set_err(ctx, GS_BADARG, "matrix %lld: negative offset", (long long)b);
      na = std::max(na, (long long)offs[b] + (long long)n * n);
      nw = std::max(nw, (long long)woffs[b] + n);
    }
  }
  const size_t o_order = ar.take<int>(count);
  const size_t o_sched = ar.take<int>(3 * kNumBins);
  size_t o_A = 0, o_Z = 0, o_w = 0, o_ns = 0, o_offs = 0, o_woffs = 0, o_st = 0;
  if (!dev) {
    o_A = ar.take<double2>(na);
    o_Z = ar.take<double2>(wantz ? na : 1);
    o_w = ar.take<double2>(nw);
    o_ns = ar.take<int>(count);
    o_offs = ar.take<long long>(count);
    o_woffs = ar.take<long long>(count);
    o_st = ar.take<int>(count);
  }
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  int* order = (int*)(base + o_order);
  int* sched = (int*)(base + o_sched);
  cudaStream_t s = ctx->stream;
  if (!dev) {
    bt.ns = (const int*)(base + o_ns);
    bt.offs = (const long long*)(base + o_offs);
    bt.woffs = (const long long*)(base + o_woffs);
    bt.A = (double2*)(base + o_A);
    bt.Z = wantz ? (double2*)(base + o_Z) : nullptr;
    bt.w = (double2*)(base + o_w);
    bt.status = (int*)(base + o_st);
    CK(cudaMemcpyAsync((void*)bt.ns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)bt.offs, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync((void*)bt.woffs, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(bt.A, A, sizeof(double2) * na, cudaMemcpyHostToDevice, s));
  } else {
    bt.ns = ns;
    bt.offs = (const long long*)offs;
    bt.woffs = (const long long*)woffs;
    bt.A = (double2*)A;
    bt.Z = wantz ? (double2*)Z : nullptr;
    bt.w = (double2*)w;
    bt.status = status;
  }
  std::vector<long long> key = {2, (long long)count, (long long)(uintptr_t)bt.A, (long long)(uintptr_t)bt.Z,
                                (long long)(uintptr_t)bt.ns, (long long)(uintptr_t)bt.w,
                                (long long)(uintptr_t)order, (long long)flags, ctx->tun_gen};
  rc = run_batched_cplx(ctx, bt, order, sched, (flags & GS_GRAPH) != 0, key);
  if (rc) return rc;
  if (dev) return GS_OK;
  CK(cudaMemcpyAsync(A, bt.A, sizeof(double2) * na, cudaMemcpyDeviceToHost, s));
  if (wantz) CK(cudaMemcpyAsync(Z, bt.Z, sizeof(double2) * na, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(w, bt.w, sizeof(double2) * nw, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(status, bt.status, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int64_t b = 0; b < count; ++b)
    if (status[b] != GS_OK) return set_err(ctx, GS_UNCONVERGED, "matrix %lld: iteration limit reached", (long long)b);
  return GS_OK;
}

int gs_schur_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* Z, int64_t ldz, double* w,
                 unsigned flags, int64_t maxiter, int64_t maxinner) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  const bool wantz = flags & GS_WANTZ;
  if (n < 0) return set_err(ctx, GS_BADARG, "negative order");
  if (lda < std::max<int64_t>(n, 1) || (wantz && ldz < std::max<int64_t>(n, 1)))
    return set_err(ctx, GS_BADARG, "leading dimension smaller than n");
  if (n == 0) return GS_OK;
  if (!A || !w || (wantz && !Z)) return set_err(ctx, GS_BADARG, "null array argument");
  if (n > (1 << 20)) return set_err(ctx, GS_BADARG, "order %lld too large", (long long)n);
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const bool large = n > kSmallMax;
  Arena ar;
  const size_t o_A = ar.take<double2>(n * n), o_Z = ar.take<double2>(n * n), o_w = ar.take<double2>(n);
  const size_t o_h = ar.take<char>(large ? schur_large_cplx_ws_bytes((int)n) : 1);
  const size_t o_meta = ar.take<long long>(4), o_st = ar.take<int>(2);
  const size_t o_order = ar.take<int>(1), o_sched = ar.take<int>(3 * kNumBins);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  double2* dA = (double2*)(base + o_A);
  double2* dZ = (double2*)(base + o_Z);
  const size_t es = sizeof(double2);
  CK(cudaMemcpy2DAsync(dA, n * es, A, lda * es, n * es, n, in, s));
  long long meta_h[4] = {0, 0, 0, 0};
  int n32 = (int)n;
  long long* meta = (long long*)(base + o_meta);
  CK(cudaMemcpyAsync(meta, meta_h, sizeof(meta_h), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(meta + 2, &n32, sizeof(int), cudaMemcpyHostToDevice, s));
  CplxBatch bt{};
  bt.count = 1;
  bt.ns = (const int*)(meta + 2);
  bt.offs = meta;
  bt.woffs = meta + 1;
  bt.A = dA;
  bt.Z = wantz ? dZ : nullptr;
  bt.w = (double2*)(base + o_w);
  bt.status = (int*)(base + o_st);
  bt.wantz = wantz;
  bt.scale = (flags & GS_SCALE) ? 1 : 0;
  bt.maxiter_mult = 100;
  bt.maxinner_mult = 30;
  bt.maxiter_abs = maxiter > 0 ? maxiter : 0;
  bt.maxinner_abs = maxinner > 0 ? maxinner : 0;
  int st = 0;
  if (large) {
    // the whole GPU: Hessenberg reduction and multishift QR (schur_large_cplx.cu)
    CK(cudaEventRecord(ctx->t0, s));
    cudaError_t ce = cudaSuccess;
    st = schur_large_cplx_run(dA, wantz ? dZ : nullptr, bt.w, (int)n, bt.scale, maxiter > 0 ? maxiter : 0,
                              base + o_h, ctx->num_sms, s, &ce);
    if (st < 0) return set_err(ctx, GS_CUDA, "complex large path: %s", cudaGetErrorString(ce));
    CK(cudaEventRecord(ctx->t1, s));
    ctx->timed = true;
  } else {
    rc = run_batched_cplx(ctx, bt, (int*)(base + o_order), (int*)(base + o_sched), false, {});
    if (rc) return rc;
  }
  CK(cudaMemcpy2DAsync(A, lda * es, dA, n * es, n * es, n, out, s));
  if (wantz) CK(cudaMemcpy2DAsync(Z, ldz * es, dZ, n * es, n * es, n, out, s));
  CK(cudaMemcpyAsync(w, bt.w, n * es, out, s));
  if (!large) CK(cudaMemcpyAsync(&st, bt.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (st != GS_OK) return set_err(ctx, GS_UNCONVERGED, "iteration limit reached");
  return GS_OK;
}

// ---------------------------------------------------------------------------
// eigenvectors and triangularize
// ---------------------------------------------------------------------------
namespace {

// Everything on device pointers: T/Z complex (Zc may be null), outputs VR/VL complex.
int run_eigvecs(gs_context* ctx, int count, const int* ns, const long long* offs, const double2* T,
                const double2* Z, double2* VR, double2* VL, double2* scratch, const long long* woffs,
                const int* colmap, bool normalize) {
  EigBatch eb{};
  eb.count = count;
  eb.ns = ns;
  eb.offs = offs;
  eb.T = T;
  eb.Z = Z;
  eb.VR = VR;
  eb.VL = VL;
  eb.scratch = scratch;
  eb.normalize = normalize ? 1 : 0;
  eb.woffs = woffs;
  eb.colmap = colmap;
  cudaError_t e = launch_eigvecs_batched(eb, kSmallMax, ctx->num_sms, ctx->stream);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "eigvecs launch: %s", cudaGetErrorString(e));
  return GS_OK;
}

// Shared driver of the eigenvector entry points.  `real` selects real T/Z input
// (triangularized first).  Host or device pointers per GS_DEVICE.
int eigvecs_driver(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs, const int64_t* woffs,
                   int64_t packed_len, int64_t w_len, const double* T, const double* Z, double* VR, double* VL,
                   unsigned flags, bool real) {
  if (count < 0) return set_err(ctx, GS_BADARG, "bad count");
  if (count == 0) return GS_OK;
  if (!ns || !offs || !T || (!VR && !VL) || (real && !woffs)) return set_err(ctx, GS_BADARG, "null array argument");
  if (packed_len < 0 || w_len < 0) return set_err(ctx, GS_BADARG, "negative length");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  if (!dev) {
    for (int64_t b = 0; b < count; ++b) {
      const int n = ns[b];
      if (n < 0 || n > kSmallMax) return set_err(ctx, GS_BADARG, "matrix %lld: order %d outside [0, %d]", (long long)b, n, kSmallMax);
      if (offs[b] < 0 || offs[b] + (long long)n * n > packed_len) return set_err(ctx, GS_BADARG, "matrix %lld outside the packed buffer", (long long)b);
      if (real && (woffs[b] < 0 || woffs[b] + n > w_len)) return set_err(ctx, GS_BADARG, "matrix %lld: eigenvalue offset outside w_len", (long long)b);
    }
  }
  const size_t es = real ? sizeof(double) : sizeof(double2);
  Arena ar;
  size_t o_T = 0, o_Z = 0, o_ns = 0, o_offs = 0, o_woffs = 0, o_VR = 0, o_VL = 0;
  const size_t o_X = ar.take<double2>(packed_len);
  size_t o_Tc = 0, o_Zc = 0, o_map = 0;
  if (real) {
    o_Tc = ar.take<double2>(packed_len);
    o_Zc = ar.take<double2>(Z ? packed_len : 1);
    o_map = ar.take<int>(w_len);
  }
  if (!dev) {
    o_T = ar.take<char>(es * packed_len);
    o_Z = ar.take<char>(Z ? es * packed_len : 1);
    o_ns = ar.take<int>(count);
    o_offs = ar.take<long long>(count);
    o_woffs = ar.take<long long>(real ? count : 1);
    o_VR = ar.take<double2>(VR ? packed_len : 1);
    o_VL = ar.take<double2>(VL ? packed_len : 1);
  }
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const int* d_ns = (const int*)ns;
  const long long* d_offs = (const long long*)offs;
  const long long* d_woffs = (const long long*)woffs;
  const void* d_T = T;
  const void* d_Z = Z;
  double2* d_VR = (double2*)VR;
  double2* d_VL = (double2*)VL;
  if (!dev) {
    CK(cudaMemcpyAsync(base + o_ns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_offs, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    if (real) CK(cudaMemcpyAsync(base + o_woffs, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_T, T, es * packed_len, cudaMemcpyHostToDevice, s));
    if (Z) CK(cudaMemcpyAsync(base + o_Z, Z, es * packed_len, cudaMemcpyHostToDevice, s));
    d_ns = (const int*)(base + o_ns);
    d_offs = (const long long*)(base + o_offs);
    d_woffs = (const long long*)(base + o_woffs);
    d_T = base + o_T;
    d_Z = Z ? (const void*)(base + o_Z) : nullptr;
    d_VR = VR ? (double2*)(base + o_VR) : nullptr;
    d_VL = VL ? (double2*)(base + o_VL) : nullptr;
  }
  CK(cudaEventRecord(ctx->t0, s));
  const double2* cT = (const double2*)d_T;
  const double2* cZ = (const double2*)d_Z;
  const int* cmap = nullptr;
  if (real) {
    TriBatch tb{};
    tb.count = (int)count;
    tb.ns = d_ns;
    tb.offs = d_offs;
    tb.woffs = d_woffs;
    tb.Tr = (const double*)d_T;
    tb.Zr = (const double*)d_Z;
    tb.Tc = (double2*)(base + o_Tc);
    tb.Zc = d_Z ? (double2*)(base + o_Zc) : nullptr;
    tb.w = nullptr;
    tb.colmap = (int*)(base + o_map);
    cudaError_t e = launch_triangularize(tb, ctx->num_sms, s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "triangularize launch: %s", cudaGetErrorString(e));
    cT = tb.Tc;
    cZ = tb.Zc;
    cmap = tb.colmap;
  }
  rc = run_eigvecs(ctx, (int)count, d_ns, d_offs, cT, cZ, d_VR, d_VL, (double2*)(base + o_X), d_woffs, cmap,
                   !(flags & GS_RAW));
  if (rc) return rc;
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  if (dev) return GS_OK;
  if (VR) CK(cudaMemcpyAsync(VR, d_VR, sizeof(double2) * packed_len, cudaMemcpyDeviceToHost, s));
  if (VL) CK(cudaMemcpyAsync(VL, d_VL, sizeof(double2) * packed_len, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

}  // namespace

// One matrix of order > 128: tiled back-substitution (eigvecs_large.cu); real input is
// triangularised first.
static int eigvecs_large_driver(gs_context* ctx, int64_t n, const double* T, const double* Z, double* VR, double* VL,
                                unsigned flags, bool real) {
  if (!T || (!VR && !VL)) return set_err(ctx, GS_BADARG, "null array argument");
  if (n > (1 << 16)) return set_err(ctx, GS_BADARG, "order %lld too large", (long long)n);
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  const size_t es = real ? sizeof(double) : sizeof(double2);
  Arena ar;
  const size_t o_ws = ar.take<double2>(eigvecs_large_ws_elems((int)n));
  const size_t o_bad = ar.take<int>(4);
  size_t o_T = 0, o_Z = 0, o_VR = 0, o_VL = 0, o_Tc = 0, o_Zc = 0, o_map = 0, o_meta = 0;
  if (real) {
    o_Tc = ar.take<double2>(nn);
    o_Zc = ar.take<double2>(Z ? nn : 1);
    o_map = ar.take<int>(n);
    o_meta = ar.take<long long>(4);
  }
  if (!dev) {
    o_T = ar.take<char>(es * nn);
    o_Z = ar.take<char>(Z ? es * nn : 1);
    o_VR = ar.take<double2>(VR ? nn : 1);
    o_VL = ar.take<double2>(VL ? nn : 1);
  }
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const void* d_T = T;
  const void* d_Z = Z;
  double2* d_VR = (double2*)VR;
  double2* d_VL = (double2*)VL;
  if (!dev) {
    CK(cudaMemcpyAsync(base + o_T, T, es * nn, cudaMemcpyHostToDevice, s));
    if (Z) CK(cudaMemcpyAsync(base + o_Z, Z, es * nn, cudaMemcpyHostToDevice, s));
    d_T = base + o_T;
    d_Z = Z ? (const void*)(base + o_Z) : nullptr;
    d_VR = VR ? (double2*)(base + o_VR) : nullptr;
    d_VL = VL ? (double2*)(base + o_VL) : nullptr;
  }
  int* bad = (int*)(base + o_bad);
  CK(cudaMemsetAsync(bad, 0, sizeof(int), s));
  CK(cudaEventRecord(ctx->t0, s));
  const double2* cT = (const double2*)d_T;
  const double2* cZ = (const double2*)d_Z;
  const int* cmap = nullptr;
  if (real) {
    long long meta_h[4] = {0, 0, 0, 0};
    int n32 = (int)n;
    long long* meta = (long long*)(base + o_meta);
    CK(cudaMemcpyAsync(meta, meta_h, sizeof(meta_h), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(meta + 2, &n32, sizeof(int), cudaMemcpyHostToDevice, s));
    TriBatch tb{};
    tb.count = 1;
    tb.ns = (const int*)(meta + 2);
    tb.offs = meta;
    tb.woffs = meta + 1;
    tb.Tr = (const double*)d_T;
    tb.Zr = (const double*)d_Z;
    tb.Tc = (double2*)(base + o_Tc);
    tb.Zc = d_Z ? (double2*)(base + o_Zc) : nullptr;
    tb.w = nullptr;
    tb.colmap = (int*)(base + o_map);
    cudaError_t e = launch_triangularize(tb, ctx->num_sms, s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "triangularize launch: %s", cudaGetErrorString(e));
    cT = tb.Tc;
    cZ = tb.Zc;
    cmap = tb.colmap;
  }
  cudaError_t e = launch_eigvecs_large((int)n, cT, cZ, d_VR, d_VL, !(flags & GS_RAW), cmap,
                                       (double2*)(base + o_ws), bad, s);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "eigenvector kernels: %s", cudaGetErrorString(e));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  int nbad = 0;
  CK(cudaMemcpyAsync(&nbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (!dev) {
    if (VR) CK(cudaMemcpyAsync(VR, d_VR, sizeof(double2) * nn, cudaMemcpyDeviceToHost, s));
    if (VL) CK(cudaMemcpyAsync(VL, d_VL, sizeof(double2) * nn, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (nbad) return set_err(ctx, GS_UNCONVERGED, "%d eigenvector columns overflowed (no rescaling for n > %d)", nbad,
                           kSmallMax);
  return GS_OK;
}

int gs_eigvecs_c64(gs_context* ctx, int64_t n, const double* T, const double* Z, double* VR, double* VL,
                   unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n > kSmallMax) return eigvecs_large_driver(ctx, n, T, Z, VR, VL, flags, false);
  if (n < 0) return set_err(ctx, GS_BADARG, "negative order");
  if (n == 0) return GS_OK;
  if (flags & GS_DEVICE) return set_err(ctx, GS_BADARG, "gs_eigvecs_c64 with GS_DEVICE: use gs_eigvecs_batched_c64");
  const int32_t n32 = (int32_t)n;
  const int64_t zero = 0;
  return eigvecs_driver(ctx, 1, &n32, &zero, nullptr, n * n, 0, T, Z, VR, VL, flags, false);
}

int gs_eigvecs_f64(gs_context* ctx, int64_t n, const double* T, const double* Z, double* VR, double* VL,
                   unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n > kSmallMax) return eigvecs_large_driver(ctx, n, T, Z, VR, VL, flags, true);
  if (n < 0) return set_err(ctx, GS_BADARG, "negative order");
  if (n == 0) return GS_OK;
  if (flags & GS_DEVICE) return set_err(ctx, GS_BADARG, "gs_eigvecs_f64 with GS_DEVICE: use gs_eigvecs_batched_f64");
  const int32_t n32 = (int32_t)n;
  const int64_t zero = 0;
  return eigvecs_driver(ctx, 1, &n32, &zero, &zero, n * n, n, T, Z, VR, VL, flags, true);
}

int gs_eigvecs_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs, int64_t packed_len,
                           const double* T, const double* Z, double* VR, double* VL, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  return eigvecs_driver(ctx, count, ns, offs, nullptr, packed_len, 0, T, Z, VR, VL, flags, false);
}

int gs_eigvecs_batched_f64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                           const int64_t* woffs, int64_t packed_len, int64_t w_len, const double* T, const double* Z,
                           double* VR, double* VL, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  return eigvecs_driver(ctx, count, ns, offs, woffs, packed_len, w_len, T, Z, VR, VL, flags, true);
}

int gs_triangularize_f64(gs_context* ctx, int64_t n, const double* T, const double* Z, double* Tc, double* Zc,
                         double* w, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0) return set_err(ctx, GS_BADARG, "negative order");
  if (n == 0) return GS_OK;
  if (!T || !Tc || (Zc && !Z)) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  Arena ar;
  const size_t o_meta = ar.take<long long>(4);
  size_t o_T = 0, o_Z = 0, o_Tc = 0, o_Zc = 0, o_w = 0;
  if (!dev) {
    o_T = ar.take<double>(nn);
    o_Z = ar.take<double>(Z ? nn : 1);
    o_Tc = ar.take<double2>(nn);
    o_Zc = ar.take<double2>(Zc ? nn : 1);
    o_w = ar.take<double2>(n);
  }
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  long long meta_h[4] = {0, 0, 0, 0};
  int n32 = (int)n;
  long long* meta = (long long*)(base + o_meta);
  CK(cudaMemcpyAsync(meta, meta_h, sizeof(meta_h), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(meta + 2, &n32, sizeof(int), cudaMemcpyHostToDevice, s));
  TriBatch tb{};
  tb.count = 1;
  tb.ns = (const int*)(meta + 2);
  tb.offs = meta;
  tb.woffs = meta + 1;
  if (!dev) {
    CK(cudaMemcpyAsync(base + o_T, T, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    if (Z) CK(cudaMemcpyAsync(base + o_Z, Z, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    tb.Tr = (const double*)(base + o_T);
    tb.Zr = Z ? (const double*)(base + o_Z) : nullptr;
    tb.Tc = (double2*)(base + o_Tc);
    tb.Zc = Zc ? (double2*)(base + o_Zc) : nullptr;
    tb.w = w ? (double2*)(base + o_w) : nullptr;
  } else {
    tb.Tr = T;
    tb.Zr = Z;
    tb.Tc = (double2*)Tc;
    tb.Zc = (double2*)Zc;
    tb.w = (double2*)w;
  }
  tb.colmap = nullptr;
  cudaError_t e = launch_triangularize(tb, ctx->num_sms, s);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "triangularize launch: %s", cudaGetErrorString(e));
  if (dev) return GS_OK;
  CK(cudaMemcpyAsync(Tc, tb.Tc, nn * sizeof(double2), cudaMemcpyDeviceToHost, s));
  if (Zc) CK(cudaMemcpyAsync(Zc, tb.Zc, nn * sizeof(double2), cudaMemcpyDeviceToHost, s));
  if (w) CK(cudaMemcpyAsync(w, tb.w, n * sizeof(double2), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

// ---------------------------------------------------------------------------
// eigenvalue adjoint
// ---------------------------------------------------------------------------
int gs_eig_adjoint_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs,
                               const int64_t* woffs, int64_t packed_len, int64_t w_len, const double* T,
                               const double* Z, const double* gbar, double* grad, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (count < 0 || packed_len < 0 || w_len < 0) return set_err(ctx, GS_BADARG, "negative size");
  if (count == 0) return GS_OK;
  if (!ns || !offs || !woffs || !T || !Z || !gbar || !grad) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  if (!dev) {
    for (int64_t b = 0; b < count; ++b) {
      const int n = ns[b];
      if (n < 0 || n > kSmallMax) return set_err(ctx, GS_BADARG, "matrix %lld: order %d outside [0, %d]", (long long)b, n, kSmallMax);
      if (offs[b] < 0 || offs[b] + (long long)n * n > packed_len) return set_err(ctx, GS_BADARG, "matrix %lld outside the packed buffer", (long long)b);
      if (woffs[b] < 0 || woffs[b] + n > w_len) return set_err(ctx, GS_BADARG, "matrix %lld: eigenvalue offset outside w_len", (long long)b);
    }
  }
  Arena ar;
  const size_t o_X = ar.take<double2>(packed_len), o_VR = ar.take<double2>(packed_len), o_VL = ar.take<double2>(packed_len);
  size_t o_T = 0, o_Z = 0, o_g = 0, o_G = 0, o_ns = 0, o_offs = 0, o_woffs = 0;
  if (!dev) {
    o_T = ar.take<double2>(packed_len);
    o_Z = ar.take<double2>(packed_len);
    o_g = ar.take<double2>(w_len);
    o_G = ar.take<double2>(packed_len);
    o_ns = ar.take<int>(count);
    o_offs = ar.take<long long>(count);
    o_woffs = ar.take<long long>(count);
  }
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const int* d_ns = ns;
  const long long* d_offs = (const long long*)offs;
  const long long* d_woffs = (const long long*)woffs;
  const double2* d_T = (const double2*)T;
  const double2* d_Z = (const double2*)Z;
  const double2* d_g = (const double2*)gbar;
  double2* d_G = (double2*)grad;
  if (!dev) {
    CK(cudaMemcpyAsync(base + o_ns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_offs, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_woffs, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_T, T, sizeof(double2) * packed_len, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_Z, Z, sizeof(double2) * packed_len, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_g, gbar, sizeof(double2) * w_len, cudaMemcpyHostToDevice, s));
    d_ns = (const int*)(base + o_ns);
    d_offs = (const long long*)(base + o_offs);
    d_woffs = (const long long*)(base + o_woffs);
    d_T = (const double2*)(base + o_T);
    d_Z = (const double2*)(base + o_Z);
    d_g = (const double2*)(base + o_g);
    d_G = (double2*)(base + o_G);
  }
  CK(cudaEventRecord(ctx->t0, s));
  double2* VR = (double2*)(base + o_VR);
  double2* VL = (double2*)(base + o_VL);
  rc = run_eigvecs(ctx, (int)count, d_ns, d_offs, d_T, d_Z, VR, VL, (double2*)(base + o_X), nullptr, nullptr, false);
  if (rc) return rc;
  AdjBatch ab{};
  ab.count = (int)count;
  ab.ns = d_ns;
  ab.offs = d_offs;
  ab.woffs = d_woffs;
  ab.VR = VR;
  ab.VL = VL;
  ab.gbar = d_g;
  ab.grad = d_G;
  cudaError_t e = launch_eig_adjoint(ab, kSmallMax, ctx->num_sms, s);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "adjoint launch: %s", cudaGetErrorString(e));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  if (dev) return GS_OK;
  CK(cudaMemcpyAsync(grad, d_G, sizeof(double2) * packed_len, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

// ---------------------------------------------------------------------------
// Hessenberg reduction (hessenberg!, pirates.jl:232 -> _hessenberg!, hessenberg.jl:3-17)
// ---------------------------------------------------------------------------
int gs_hessenberg_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* tau, double* Q, int64_t ldq,
                      unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0) return set_err(ctx, GS_BADARG, "negative order");
  if (lda < std::max<int64_t>(n, 1) || (Q && ldq < std::max<int64_t>(n, 1)))
    return set_err(ctx, GS_BADARG, "leading dimension smaller than n");
  if (n == 0) return GS_OK;
  if (!A || (n > 1 && !tau)) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  Arena ar;
  const size_t o_A = ar.take<double>(nn), o_Q = ar.take<double>(Q ? nn : 1), o_tau = ar.take<double>(n);
  const size_t o_ws = ar.take<double>(std::max(hess_large_ws_elems((int)n), hess_blocked_ws_elems((int)n)));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  double* dA = (double*)(base + o_A);
  double* dQ = Q ? (double*)(base + o_Q) : nullptr;
  double* dtau = (double*)(base + o_tau);
  CK(cudaMemsetAsync(dtau, 0, n * sizeof(double), s));
  CK(cudaMemcpy2DAsync(dA, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n, in, s));
  int herr = 0;
  CK(cudaEventRecord(ctx->t0, s));
  cudaError_t e = (n >= hess_blocked_min(sizeof(double)))
                      ? hessenberg_blocked<double>((int)n, dA, (int)n, dQ, (int)n, dtau, (double*)(base + o_ws),
                                                   ctx->num_sms, &herr, s)
                      : hessenberg_large<double>((int)n, dA, (int)n, dQ, (int)n, dtau, (double*)(base + o_ws), s);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "hessenberg: %s", cudaGetErrorString(e));
  if (herr) return set_err(ctx, GS_CUDA, "hessenberg: grid barrier timed out");
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  CK(cudaMemcpy2DAsync(A, lda * sizeof(double), dA, n * sizeof(double), n * sizeof(double), n, out, s));
  if (Q) CK(cudaMemcpy2DAsync(Q, ldq * sizeof(double), dQ, n * sizeof(double), n * sizeof(double), n, out, s));
  if (n > 1) CK(cudaMemcpyAsync(tau, dtau, (n - 1) * sizeof(double), out, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

// ---------------------------------------------------------------------------
// eigenvectors of a complex generalized Schur pair (ggevc.cu)
// ---------------------------------------------------------------------------
int gs_ggeigvecs_c64(gs_context* ctx, int64_t n, const double* S, const double* T, const double* Q, const double* Z,
                     double* VR, double* VL, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 15)) return set_err(ctx, GS_BADARG, "bad order %lld", (long long)n);
  if (n == 0) return GS_OK;
  if (!S || !T) return set_err(ctx, GS_BADARG, "null array argument");
  if (!VR && !VL) return GS_OK;
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  const int N = (int)n;
  Arena ar;
  const size_t o_S = ar.take<double2>(dev ? 1 : nn), o_T = ar.take<double2>(dev ? 1 : nn);
  const size_t o_Q = ar.take<double2>(dev || !Q ? 1 : nn), o_Z = ar.take<double2>(dev || !Z ? 1 : nn);
  const size_t o_V = ar.take<double2>(dev ? 1 : nn), o_ws = ar.take<char>(ggevc_ws_bytes(N));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const double2 *dS = (const double2*)S, *dT = (const double2*)T, *dQ = (const double2*)Q, *dZ = (const double2*)Z;
  if (!dev) {
    CK(cudaMemcpyAsync(base + o_S, S, nn * sizeof(double2), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_T, T, nn * sizeof(double2), cudaMemcpyHostToDevice, s));
    if (Q) CK(cudaMemcpyAsync(base + o_Q, Q, nn * sizeof(double2), cudaMemcpyHostToDevice, s));
    if (Z) CK(cudaMemcpyAsync(base + o_Z, Z, nn * sizeof(double2), cudaMemcpyHostToDevice, s));
    dS = (const double2*)(base + o_S);
    dT = (const double2*)(base + o_T);
    dQ = Q ? (const double2*)(base + o_Q) : nullptr;
    dZ = Z ? (const double2*)(base + o_Z) : nullptr;
  }
  CK(cudaEventRecord(ctx->t0, s));
  for (int left = 0; left < 2; ++left) {
    double* out = left ? VL : VR;
    if (!out) continue;
    double2* dV = dev ? (double2*)out : (double2*)(base + o_V);
    cudaError_t e = launch_ggevc(N, dS, dT, left ? dQ : dZ, left, dV, base + o_ws, s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "generalized eigenvectors: %s", cudaGetErrorString(e));
    if (!dev) CK(cudaMemcpyAsync(out, dV, nn * sizeof(double2), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

int gs_ggordschur_c64(gs_context* ctx, int64_t n, double* S, double* T, double* Q, double* Z, const int32_t* select,
                      double* alpha, double* beta, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 15)) return set_err(ctx, GS_BADARG, "bad order %lld", (long long)n);
  if (n == 0) return GS_OK;
  if (!S || !T || !Q || !Z || !select || !alpha || !beta) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n, zb = sizeof(double2);
  Arena ar;
  const size_t o_S = ar.take<double2>(dev ? 1 : nn), o_T = ar.take<double2>(dev ? 1 : nn),
               o_Q = ar.take<double2>(dev ? 1 : nn), o_Z = ar.take<double2>(dev ? 1 : nn),
               o_al = ar.take<double2>(dev ? 1 : n), o_be = ar.take<double2>(dev ? 1 : n), o_sel = ar.take<int>(n),
               o_st = ar.take<int>(4);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  double2* dS = dev ? (double2*)S : (double2*)(base + o_S);
  double2* dT = dev ? (double2*)T : (double2*)(base + o_T);
  double2* dQ = dev ? (double2*)Q : (double2*)(base + o_Q);
  double2* dZ = dev ? (double2*)Z : (double2*)(base + o_Z);
  double2* dal = dev ? (double2*)alpha : (double2*)(base + o_al);
  double2* dbe = dev ? (double2*)beta : (double2*)(base + o_be);
  int* dsel = (int*)(base + o_sel);
  int* dst = (int*)(base + o_st);
  if (!dev) {
    CK(cudaMemcpyAsync(dS, S, zb * nn, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dT, T, zb * nn, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dQ, Q, zb * nn, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dZ, Z, zb * nn, cudaMemcpyHostToDevice, s));
  }
  CK(cudaMemcpyAsync(dsel, select, sizeof(int) * n, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  CK(cudaEventRecord(ctx->t0, s));
  CK(launch_ggordschur_cplx((int)n, dS, dT, dQ, dZ, dsel, (flags & GS_SCALE) ? 1 : 0, dal, dbe, dst, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  int st = 0;
  CK(cudaMemcpyAsync(&st, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (!dev) {
    CK(cudaMemcpyAsync(S, dS, zb * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(T, dT, zb * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(Q, dQ, zb * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(Z, dZ, zb * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(alpha, dal, zb * n, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(beta, dbe, zb * n, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (st) return set_err(ctx, GS_UNCONVERGED, "swap at %d rejected as ill-conditioned", st - 1);
  return GS_OK;
}

int gs_ggordschur_f64(gs_context* ctx, int64_t n, double* S, double* T, double* Q, double* Z, const int32_t* select,
                      double* alpha, double* beta, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 15)) return set_err(ctx, GS_BADARG, "bad order %lld", (long long)n);
  if (n == 0) return GS_OK;
  if (!S || !T || !select || !alpha || !beta) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n, db = sizeof(double);
  Arena ar;
  const size_t o_S = ar.take<double>(dev ? 1 : nn), o_T = ar.take<double>(dev ? 1 : nn),
               o_Q = ar.take<double>(dev || !Q ? 1 : nn), o_Z = ar.take<double>(dev || !Z ? 1 : nn),
               o_al = ar.take<double2>(dev ? 1 : n), o_be = ar.take<double>(dev ? 1 : n), o_sel = ar.take<int>(n),
               o_st = ar.take<int>(4);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  double* dS = dev ? S : (double*)(base + o_S);
  double* dT = dev ? T : (double*)(base + o_T);
  double* dQ = Q ? (dev ? Q : (double*)(base + o_Q)) : nullptr;
  double* dZ = Z ? (dev ? Z : (double*)(base + o_Z)) : nullptr;
  double2* dal = dev ? (double2*)alpha : (double2*)(base + o_al);
  double* dbe = dev ? beta : (double*)(base + o_be);
  int* dsel = (int*)(base + o_sel);
  int* dst = (int*)(base + o_st);
  if (!dev) {
    CK(cudaMemcpyAsync(dS, S, db * nn, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dT, T, db * nn, cudaMemcpyHostToDevice, s));
    if (Q) CK(cudaMemcpyAsync(dQ, Q, db * nn, cudaMemcpyHostToDevice, s));
    if (Z) CK(cudaMemcpyAsync(dZ, Z, db * nn, cudaMemcpyHostToDevice, s));
  }
  CK(cudaMemcpyAsync(dsel, select, sizeof(int) * n, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  CK(cudaEventRecord(ctx->t0, s));
  CK(launch_ggordschur_real((int)n, dS, dT, dQ, dZ, dsel, (flags & GS_SCALE) ? 1 : 0, dal, dbe, dst, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  int st = 0;
  CK(cudaMemcpyAsync(&st, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (!dev) {
    CK(cudaMemcpyAsync(S, dS, db * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(T, dT, db * nn, cudaMemcpyDeviceToHost, s));
    if (Q) CK(cudaMemcpyAsync(Q, dQ, db * nn, cudaMemcpyDeviceToHost, s));
    if (Z) CK(cudaMemcpyAsync(Z, dZ, db * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(alpha, dal, sizeof(double2) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(beta, dbe, db * n, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (st) return set_err(ctx, GS_UNCONVERGED, "the block at %d could not be moved (ill-conditioned swap)", st - 1);
  return GS_OK;
}

int gs_ggeigvecs_f64(gs_context* ctx, int64_t n, const double* S, const double* T, const double* Q, const double* Z,
                     double* VR, double* VL, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 15)) return set_err(ctx, GS_BADARG, "bad order %lld", (long long)n);
  if (n == 0) return GS_OK;
  if (!S || !T) return set_err(ctx, GS_BADARG, "null array argument");
  if (!VR && !VL) return GS_OK;
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  const int N = (int)n;
  Arena ar;
  const size_t o_S = ar.take<double>(dev ? 1 : nn), o_T = ar.take<double>(dev ? 1 : nn);
  const size_t o_Q = ar.take<double>(dev || !Q ? 1 : nn), o_Z = ar.take<double>(dev || !Z ? 1 : nn);
  const size_t o_V = ar.take<double2>(dev ? 1 : nn), o_ws = ar.take<char>(rgevc_ws_bytes(N));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const double *dS = S, *dT = T, *dQ = Q, *dZ = Z;
  if (!dev) {
    CK(cudaMemcpyAsync(base + o_S, S, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_T, T, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    if (Q) CK(cudaMemcpyAsync(base + o_Q, Q, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    if (Z) CK(cudaMemcpyAsync(base + o_Z, Z, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    dS = (const double*)(base + o_S);
    dT = (const double*)(base + o_T);
    dQ = Q ? (const double*)(base + o_Q) : nullptr;
    dZ = Z ? (const double*)(base + o_Z) : nullptr;
  }
  CK(cudaEventRecord(ctx->t0, s));
  for (int left = 0; left < 2; ++left) {
    double* out = left ? VL : VR;
    if (!out) continue;
    double2* dV = dev ? (double2*)out : (double2*)(base + o_V);
    cudaError_t e = launch_rgevc(N, dS, dT, left ? dQ : dZ, left, dV, base + o_ws, s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "generalized eigenvectors: %s", cudaGetErrorString(e));
    if (!dev) CK(cudaMemcpyAsync(out, dV, nn * sizeof(double2), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

// ---------------------------------------------------------------------------
// FP64 product on the BF16 tensor cores (gemm_f64_tc.cu)
// ---------------------------------------------------------------------------
int gs_gemm_f64_tc(gs_context* ctx, int64_t m, int64_t p, int64_t q, const double* A, int64_t lda, int transA,
                   const double* B, int64_t ldb, double* C, int64_t ldc, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (m < 0 || p < 0 || q < 0 || m > (1 << 20) || p > (1 << 20) || q > (1 << 20))
    return set_err(ctx, GS_BADARG, "bad dimensions");
  const int64_t ar_rows = transA ? q : m;
  if (lda < std::max<int64_t>(ar_rows, 1) || ldb < std::max<int64_t>(q, 1) || ldc < std::max<int64_t>(m, 1))
    return set_err(ctx, GS_BADARG, "leading dimension too small");
  if (m == 0 || p == 0) return GS_OK;
  if (!C || (q > 0 && (!A || !B))) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const int M = (int)m, P = (int)p, Q = (int)q;
  const int arows = (int)ar_rows, acols = transA ? M : Q;
  Arena ar;
  const size_t o_A = ar.take<double>(dev ? 1 : (size_t)arows * acols), o_B = ar.take<double>(dev ? 1 : (size_t)Q * P);
  const size_t o_C = ar.take<double>(dev ? 1 : (size_t)M * P), o_ws = ar.take<char>(gemm_tc_ws_bytes(M, P, Q));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const double* dA = A;
  const double* dB = B;
  double* dC = C;
  int la = (int)lda, lb = (int)ldb, lc = (int)ldc;
  if (!dev) {
    double* hA = (double*)(base + o_A);
    double* hB = (double*)(base + o_B);
    if (Q > 0) {
      CK(cudaMemcpy2DAsync(hA, arows * sizeof(double), A, lda * sizeof(double), arows * sizeof(double), acols,
                           cudaMemcpyHostToDevice, s));
      CK(cudaMemcpy2DAsync(hB, Q * sizeof(double), B, ldb * sizeof(double), Q * sizeof(double), P,
                           cudaMemcpyHostToDevice, s));
    }
    dA = hA; dB = hB; la = std::max(arows, 1); lb = std::max(Q, 1);
    dC = (double*)(base + o_C); lc = M;
  }
  void* ws = base + o_ws;
  CK(cudaMemsetAsync(gemm_tc_err_word(M, P, Q, ws), 0, sizeof(int), s));
  CK(cudaEventRecord(ctx->t0, s));
  cudaError_t e = launch_gemm_tc(M, P, Q, dA, la, transA ? 1 : 0, dB, lb, dC, lc, ws, s);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "gemm_tc: %s", cudaGetErrorString(e));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, gemm_tc_err_word(M, P, Q, ws), sizeof(int), cudaMemcpyDeviceToHost, s));
  if (!dev)
    CK(cudaMemcpy2DAsync(C, ldc * sizeof(double), dC, M * sizeof(double), M * sizeof(double), P,
                         cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (herr) return set_err(ctx, GS_CUDA, "gemm_tc: pipeline wait timed out (code %d)", herr);
  return GS_OK;
}

// ---------------------------------------------------------------------------
// mixed precision: FP32 Schur on the GPU + FP64 refinement of the Schur pair
// ---------------------------------------------------------------------------
int gs_schur_mixed_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, double* Z, int64_t ldz, double* wr,
                       double* wi, unsigned flags, int64_t maxiter, double* info) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 16)) return set_err(ctx, GS_BADARG, "bad order %lld", (long long)n);
  if (lda < std::max<int64_t>(n, 1) || ldz < std::max<int64_t>(n, 1)) return set_err(ctx, GS_BADARG, "leading dimension smaller than n");
  if (n == 0) return GS_OK;
  if (!A || !Z || !wr || !wi) return set_err(ctx, GS_BADARG, "null array argument (Z is required)");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  const int N32 = (int)n;
  Arena ar;
  const size_t o_A0 = ar.take<double>(nn), o_A32 = ar.take<float>(nn), o_Z32 = ar.take<float>(nn);
  const size_t o_Z = ar.take<double>(nn), o_T1 = ar.take<double>(nn), o_T2 = ar.take<double>(nn);
  const size_t o_T3 = ar.take<double>(nn), o_W = ar.take<double>(nn);
  const size_t o_wr = ar.take<double>(n), o_wi = ar.take<double>(n), o_sub = ar.take<float>(n);
  const size_t o_bs = ar.take<int>(n), o_bz = ar.take<int>(n), o_blk = ar.take<int>(n), o_cs = ar.take<double>(4 * n);
  const size_t o_ts = ar.take<int>(n + 1), o_tbk = ar.take<int>(n + 1);
  const size_t o_part = ar.take<double>(sylv_part_elems((int)((n + 30) / 31) + 1));
  const size_t o_nrm = ar.take<double>(4), o_max = ar.take<unsigned long long>(2);
  const size_t o_ws = ar.take<char>(schur_large_ws_bytes(N32, sizeof(float)));
  const size_t o_tc = ar.take<char>(gemm_tc_ws_bytes(N32, N32, N32));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  double* A0 = (double*)(base + o_A0);
  float* A32 = (float*)(base + o_A32);
  float* Z32 = (float*)(base + o_Z32);
  double* dZ = (double*)(base + o_Z);
  double* T1 = (double*)(base + o_T1);
  double* T2 = (double*)(base + o_T2);
  double* T3 = (double*)(base + o_T3);
  double* W = (double*)(base + o_W);
  double* dwr = (double*)(base + o_wr);
  double* dwi = (double*)(base + o_wi);
  double* nrm = (double*)(base + o_nrm);
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CK(cudaMemcpy2DAsync(A0, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n, in, s));
  cudaEvent_t e0, e1, e2;
  CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1)); CK(cudaEventCreate(&e2));
  CK(cudaEventRecord(e0, s));
  CK(cudaEventRecord(ctx->t0, s));
  // exact power-of-two prescale to max|a| in [0.5, 1): FP32 range safety, undone at the end
  double amax = 0.0;
  {
    unsigned long long* dmax = (unsigned long long*)(base + o_max);
    CK(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), s));
    cudaError_t e = launch_absmax(A0, nn, dmax, ctx->num_sms, s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "absmax: %s", cudaGetErrorString(e));
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::memcpy(&amax, &bits, sizeof(amax));
  }
  if (!(amax > 0.0) || !std::isfinite(amax)) {
    // zero or non-finite input: the plain FP64 path handles it with the reference's semantics
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
    return gs_schur_f64(ctx, n, A, lda, Z, ldz, wr, wi, flags | GS_WANTZ, maxiter);
  }
  int ex = 0;
  std::frexp(amax, &ex);
  const double pre = std::ldexp(1.0, -ex);   // A0 * pre has max in [0.5, 1)
  CK(convert_array<double, double>(A0, A0, nn, pre, s));
  CK(convert_array<double, float>(A0, A32, nn, 1.0, s));
  // ---- FP32 Schur
  LargeRun<float> r{};
  r.A = A32;
  r.Z = Z32;
  r.wr = dwr;
  r.wi = dwi;
  r.n = N32;
  r.scale = 0;
  r.maxiter = maxiter > 0 ? maxiter : 0;
  r.ws = base + o_ws;
  r.num_sms = ctx->num_sms;
  r.stream = s;
  r.cuda_error = cudaSuccess;
  large_tuning(N32, &r.bulges, &r.chunk, &r.aedw, sizeof(float));
  r.shift_fp32 = 0;
  const int st = schur_large_run<float>(r);
  if (st < 0) return set_err(ctx, GS_CUDA, "FP32 Schur stage: %s", cudaGetErrorString(r.cuda_error));
  if (st != ST_OK) return set_err(ctx, GS_UNCONVERGED, "FP32 Schur stage: iteration limit reached");
  CK(cudaEventRecord(e1, s));
  // ---- block structure from the FP32 quasi-triangular form
  std::vector<float> sub(n, 0.0f);
  {
    // subdiagonal T32[i+1, i] at element (i+1) + i*n
    CK(cudaMemcpy2DAsync(sub.data(), sizeof(float), A32 + 1, (n + 1) * sizeof(float), sizeof(float), n - 1,
                         cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  std::vector<int> bs, bz, blk(n);
  for (int i = 0; i < n;) {
    const int z = (i + 1 < n && sub[i] != 0.0f) ? 2 : 1;
    bs.push_back(i);
    bz.push_back(z);
    for (int q = 0; q < z; ++q) blk[i + q] = (int)bs.size() - 1;
    i += z;
  }
  const int NB = (int)bs.size();
  int* dbs = (int*)(base + o_bs);
  int* dbz = (int*)(base + o_bz);
  int* dblk = (int*)(base + o_blk);
  CK(cudaMemcpyAsync(dbs, bs.data(), sizeof(int) * NB, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dbz, bz.data(), sizeof(int) * NB, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dblk, blk.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  // tiles of the Sylvester solve (32 rows, never splitting a 2x2 block)
  std::vector<int> ts(n + 1), tbk(n + 1);
  const int nT = sylv_tiles(N32, blk.data(), ts.data(), tbk.data());
  int* dts = (int*)(base + o_ts);
  int* dtbk = (int*)(base + o_tbk);
  CK(cudaMemcpyAsync(dts, ts.data(), sizeof(int) * (nT + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dtbk, tbk.data(), sizeof(int) * (nT + 1), cudaMemcpyHostToDevice, s));
  // ---- FP64 refinement
  // FP64 products (Z^T A Z, Z^T Z) on the BF16 tensor cores by exact splitting: FP64
  // accuracy at tensor-core speed (gemm_f64_tc.cu).  Their timeout word is read at every
  // host synchronisation of the loop below.
  void* tcws = base + o_tc;
  int* tc_err = gemm_tc_err_word(N32, N32, N32, tcws);
  CK(cudaMemsetAsync(tc_err, 0, sizeof(int), s));
  auto gemm = [&](int m, int p, int q, const double* Am, int la, int tA, const double* Bm, int lb, double* Cm, int lc) {
    return launch_gemm_tc(m, p, q, Am, la, tA, Bm, lb, Cm, lc, tcws, s);
  };
  // Z <- Z + Z X for a small correction X (|X| <= ~1e-6): the product only needs first-order
  // accuracy, so it runs as an FP32 GEMM (Z and X rounded to FP32 into the FP32 stage's
  // buffers, the product into T2's storage) and is added to the FP64 Z.
  float* P32 = (float*)T2;
  auto add_product = [&](const double* X) -> cudaError_t {
    cudaError_t e = convert_array<double, float>(dZ, Z32, nn, 1.0, s);
    if (e == cudaSuccess) e = convert_array<double, float>(X, A32, nn, 1.0, s);
    if (e == cudaSuccess) e = launch_gemm<float>(N32, N32, N32, Z32, N32, 0, A32, N32, P32, N32, s);
    if (e == cudaSuccess) e = launch_add_f32(dZ, P32, nn, s);
    return e;
  };
  auto ns_step = [&]() -> cudaError_t {
    // Newton-Schulz: Z <- Z (1.5 I - 0.5 Z^T Z) = Z + Z E with E = (I - Z^T Z) / 2; Z^T Z in
    // FP64.  E is left in W (free between Sylvester solves).
    cudaError_t e = gemm(N32, N32, N32, dZ, N32, 1, dZ, N32, W, N32);
    if (e == cudaSuccess) e = launch_refine_elementwise(2, N32, nullptr, W, 0.0, s);
    if (e == cudaSuccess) e = add_product(W);
    return e;
  };
  auto form_At = [&]() -> cudaError_t {
    // T3 = A0 Z; T1 = Z^T T3
    cudaError_t e = gemm(N32, N32, N32, A0, N32, 0, dZ, N32, T3, N32);
    if (e == cudaSuccess) e = gemm(N32, N32, N32, dZ, N32, 1, T3, N32, T1, N32);
    return e;
  };
  CK(convert_array<float, double>(Z32, dZ, nn, 1.0, s));
  // one Newton-Schulz step takes the FP32 factor's orthogonality error e (~1e-6) to
  // ~e^2; the step after the first correction (always taken, |S| ~ 1e-6) finishes it
  cudaError_t e = ns_step();
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "orthonormalisation: %s", cudaGetErrorString(e));
  // Convergence: the residual reaches the rounding level of forming Z^T A Z, or it stops
  // shrinking (Newton converges quadratically, so a step that gains less than 4x is at
  // the noise floor) while below the acceptance bound.  NaN or a growing residual means
  // the FP32 eigenvalues were not separated enough for the Newton step.
  const double eps = 2.220446049250313e-16;
  const double tol = 4.0 * eps * std::sqrt((double)n);
  const double accept = eps * (double)n;
  const int maxit = 6;
  double res = 0.0, prev = 0.0;
  int its = 0;
  bool conv = false;
  bool have_At = false;  // T1 already holds Z^T A Z for the current Z (low-order update)
  // |S|_F bound for the low-order update of Z^T A Z (measured on GB300: at n = 4096 it
  // saves two FP64 GEMMs with the backward error unchanged at ~0.03 n eps)
  double cheap_at = 1e-5;
  if (const char* ev = std::getenv("GS_MIXED_CHEAP_AT")) cheap_at = std::atof(ev);
  for (;;) {
    e = have_At ? cudaSuccess : form_At();
    have_At = false;
    if (e == cudaSuccess) e = cudaMemsetAsync(nrm, 0, 4 * sizeof(double), s);
    if (e == cudaSuccess) e = launch_lower_norm(N32, T1, dblk, nrm, ctx->num_sms, s);
    double hn[2] = {0.0, 0.0};
    int htc = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(hn, nrm, sizeof(hn), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&htc, tc_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "refinement residual: %s", cudaGetErrorString(e));
    if (htc) return set_err(ctx, GS_CUDA, "refinement: tensor-core product timed out (code %d)", htc);
    res = std::sqrt(hn[0]) / std::max(std::sqrt(hn[1]), 1e-300);
    if (!(res == res)) break;
    if (res <= tol) { conv = true; break; }
    if (its > 0 && res > 0.25 * prev) { conv = res <= accept; break; }
    if (its >= maxit) break;
    prev = res;
    ++its;
    // block Sylvester solve for W, then Z <- Z (I + S), S = W - W^T
    e = cudaMemsetAsync(W, 0, nn * sizeof(double), s);
    const double floor = 1e-3 * std::sqrt(hn[1]) * eps;
    if (e == cudaSuccess)
      e = launch_sylv_tiled(N32, nT, T1, W, dbs, dbz, dblk, dts, dtbk, (double*)(base + o_part), floor, s);
    double wn[2] = {0.0, 0.0};
    if (e == cudaSuccess) e = launch_lower_norm(N32, W, dblk, nrm + 2, ctx->num_sms, s);
    if (e == cudaSuccess) e = launch_refine_elementwise(0, N32, W, T3, 0.0, s);  // T3 = S
    if (e == cudaSuccess) e = add_product(T3);                                     // Z <- Z (I + S)
    if (e == cudaSuccess) e = cudaMemcpyAsync(wn, nrm + 2, sizeof(wn), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // Z (I + S) departs from orthogonality by |S|^2: re-orthonormalise after the first
    // correction and while |S|_F > 1e-8.  From the second correction on, while
    // |S|_F <= cheap_at, Z^T A Z for the new Z is taken as At + At S - S At - S (At S)
    // with FP32 products instead of two FP64 GEMMs (after the first correction At must
    // be recomputed in FP64: the FP32 accumulation error times |S| ~ 1e-5 would stay in T).
    const double sf = std::sqrt(wn[1]);
    if (e == cudaSuccess && its >= 2 && sf <= cheap_at) {
      float* P1 = (float*)T2;
      float* P2 = P1 + nn;
      e = convert_array<double, float>(T1, A32, nn, 1.0, s);
      if (e == cudaSuccess) e = convert_array<double, float>(T3, Z32, nn, 1.0, s);
      if (e == cudaSuccess) e = launch_gemm<float>(N32, N32, N32, A32, N32, 0, Z32, N32, P1, N32, s);  // At S
      if (e == cudaSuccess) e = launch_gemm<float>(N32, N32, N32, Z32, N32, 0, A32, N32, P2, N32, s);  // S At
      if (e == cudaSuccess) e = launch_add_diff_f32(T1, P1, P2, nn, s);
      if (e == cudaSuccess) e = launch_gemm<float>(N32, N32, N32, Z32, N32, 0, P1, N32, P2, N32, s);  // S At S
      if (e == cudaSuccess) e = launch_sub_f32(T1, P2, nn, s);
      have_At = true;
      if (e == cudaSuccess && !(sf <= 1e-8)) {
        // orthogonality |S|^2 > eps: Newton-Schulz, and its effect on Z^T A Z to first
        // order, At <- At + E At + At E (E = (I - Z^T Z)/2 symmetric, |E| ~ |S|^2)
        e = ns_step();
        if (e == cudaSuccess) e = convert_array<double, float>(T1, A32, nn, 1.0, s);
        if (e == cudaSuccess) e = convert_array<double, float>(W, Z32, nn, 1.0, s);
        if (e == cudaSuccess) e = launch_gemm<float>(N32, N32, N32, Z32, N32, 0, A32, N32, P1, N32, s);  // E At
        if (e == cudaSuccess) e = launch_gemm<float>(N32, N32, N32, A32, N32, 0, Z32, N32, P2, N32, s);  // At E
        if (e == cudaSuccess) e = launch_add_f32(T1, P1, nn, s);
        if (e == cudaSuccess) e = launch_add_f32(T1, P2, nn, s);
      }
    } else if (e == cudaSuccess && (its == 1 || !(sf <= 1e-8))) {
      e = ns_step();
    }
    if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "refinement step: %s", cudaGetErrorString(e));
  }
  if (!conv) {
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
    if (flags & GS_NOFALLBACK)
      return set_err(ctx, GS_UNCONVERGED, "refinement did not converge (residual %.3g after %d steps)", res, its);
    // the FP32 eigenvalues were not separated enough: recompute in FP64 from the untouched input
    const int rc2 = gs_schur_f64(ctx, n, A, lda, Z, ldz, wr, wi, (flags & ~GS_NOFALLBACK) | GS_WANTZ, maxiter);
    if (info) {
      info[0] = -1.0;
      info[1] = res;
      info[2] = 0.0;
      info[3] = 0.0;
    }
    return rc2;
  }
  // ---- T = block-upper part of Z^T A Z (already in T1), standardise 2x2 blocks
  double* dT = T2;
  e = launch_block_triu(N32, T1, dblk, dT, s);
  if (e == cudaSuccess) e = launch_std_blocks(N32, NB, dbs, dbz, dT, dZ, (double*)(base + o_cs), dwr, dwi, s);
  // undo the prescale (exact power of two)
  if (e == cudaSuccess) e = convert_array<double, double>(dT, dT, nn, 1.0 / pre, s);
  if (e == cudaSuccess) e = convert_array<double, double>(dwr, dwr, n, 1.0 / pre, s);
  if (e == cudaSuccess) e = convert_array<double, double>(dwi, dwi, n, 1.0 / pre, s);
  if (e != cudaSuccess) return set_err(ctx, GS_CUDA, "final form: %s", cudaGetErrorString(e));
  CK(cudaEventRecord(e2, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  CK(cudaMemcpy2DAsync(A, lda * sizeof(double), dT, n * sizeof(double), n * sizeof(double), n, out, s));
  CK(cudaMemcpy2DAsync(Z, ldz * sizeof(double), dZ, n * sizeof(double), n * sizeof(double), n, out, s));
  CK(cudaMemcpyAsync(wr, dwr, n * sizeof(double), out, s));
  CK(cudaMemcpyAsync(wi, dwi, n * sizeof(double), out, s));
  CK(cudaStreamSynchronize(s));
  float ms1 = 0.f, ms2 = 0.f;
  cudaEventElapsedTime(&ms1, e0, e1);
  cudaEventElapsedTime(&ms2, e1, e2);
  cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
  if (info) {
    info[0] = its;
    info[1] = res;
    info[2] = ms1;
    info[3] = ms2;
  }
  return GS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// balancing (balance!, balance.jl:33-185) and the Balancer on eigenvectors
// ---------------------------------------------------------------------------
template <class S>
static int balance_impl(gs_context* ctx, int64_t n, S* A, int64_t lda, unsigned flags, int64_t* info, int64_t* sp,
                        double* D) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 16)) return set_err(ctx, GS_BADARG, "bad order %lld", (long long)n);
  if (lda < std::max<int64_t>(n, 1)) return set_err(ctx, GS_BADARG, "leading dimension smaller than n");
  if (!info || (n > 0 && (!A || !sp || !D))) return set_err(ctx, GS_BADARG, "null array argument");
  for (int64_t i = 0; i < n; ++i) { sp[i] = 0; D[i] = 1.0; }
  info[0] = 1; info[1] = n; info[2] = 1;
  if (n == 0) return GS_OK;
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const bool permute = flags & GS_BAL_PERMUTE, scale = flags & GS_SCALE;
  const size_t nn = (size_t)n * n;
  Arena ar;
  const size_t o_A = ar.take<S>(dev ? 1 : nn), o_flag = ar.take<int>(n + 2), o_pick = ar.take<int>(4),
               o_D = ar.take<double>(n), o_st = ar.take<int>(4);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  S* dA = dev ? A : (S*)(base + o_A);
  const int ld = dev ? (int)lda : (int)n;
  if (!dev)
    CK(cudaMemcpy2DAsync(dA, n * sizeof(S), A, lda * sizeof(S), n * sizeof(S), n, cudaMemcpyHostToDevice, s));
  int* flag = (int*)(base + o_flag);
  int* pick = (int*)(base + o_pick);
  const int N = (int)n;
  int ilo = 1, ihi = N;
  bool trivial = true;
  auto search = [&](int lo, int hi, int rows, int* out) -> int {
    CK(cudaMemsetAsync(flag, 0, sizeof(int) * (n + 2), s));
    CK(launch_bal_mark<S>(dA, ld, lo, hi, rows, flag, ctx->num_sms, s));
    CK(launch_bal_pick(flag, lo, hi, rows, pick, s));
    CK(cudaMemcpyAsync(out, pick, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return GS_OK;
  };
  if (permute) {
    // rows whose off-diagonal part inside the block vanishes go to the bottom (balance.jl:62-95)
    ihi = N + 1;
    while (ihi > 1) {
      ihi -= 1;
      int js = 0;
      if ((rc = search(1, ihi, 1, &js)) != GS_OK) return rc;
      if (js == 0) break;
      sp[ihi - 1] = js;
      if (js != ihi) {
        trivial = false;
        CK(launch_bal_swap<S>(dA, ld, N, js, ihi, ihi, ilo, s));
      }
    }
    // columns whose off-diagonal part vanishes go to the left (balance.jl:96-130)
    if (ihi > 1) {
      ilo = 0;
      while (ilo < N) {
        ilo += 1;
        int js = 0;
        if ((rc = search(ilo, ihi, 0, &js)) != GS_OK) return rc;
        if (js == 0) break;
        sp[ilo - 1] = js;
        if (js != ilo) {
          trivial = false;
          CK(launch_bal_swap<S>(dA, ld, N, js, ilo, ihi, ilo, s));
        }
      }
    }
  }
  if (scale) {
    double* dD = (double*)(base + o_D);
    int* st = (int*)(base + o_st);
    std::vector<double> ones(n, 1.0);
    CK(cudaMemcpyAsync(dD, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CK(launch_bal_scale<S>(dA, ld, N, ilo, ihi, dD, st, s));
    int hst[2] = {0, 0};
    CK(cudaMemcpyAsync(hst, st, sizeof(hst), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(D, dD, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (hst[0] == 2) return set_err(ctx, GS_BADARG, "NaN encountered while balancing");
    if (hst[0] == 3) return set_err(ctx, GS_UNCONVERGED, "balancing did not settle within the sweep limit");
    if (hst[1]) trivial = false;
  }
  if (!dev)
    CK(cudaMemcpy2DAsync(A, lda * sizeof(S), dA, n * sizeof(S), n * sizeof(S), n, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  info[0] = ilo;
  info[1] = ihi;
  info[2] = trivial ? 1 : 0;
  return GS_OK;
}

extern "C" {

int gs_balance_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, unsigned flags, int64_t* info, int64_t* sp,
                   double* D) {
  return balance_impl<double>(ctx, n, A, lda, flags, info, sp, D);
}

int gs_balance_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, unsigned flags, int64_t* info, int64_t* sp,
                   double* D) {
  return balance_impl<double2>(ctx, n, (double2*)A, lda, flags, info, sp, D);
}

int gs_balancer_apply_c64(gs_context* ctx, int64_t n, int64_t m, double* V, int64_t ldv, const int64_t* info,
                          const int64_t* sp, const double* D, int inverse, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || m < 0 || ldv < std::max<int64_t>(n, 1)) return set_err(ctx, GS_BADARG, "bad dimensions");
  if (!info || (n > 0 && m > 0 && (!V || !sp || !D))) return set_err(ctx, GS_BADARG, "null array argument");
  const int64_t ilo = info[0], ihi = info[1], trivial = info[2];
  if (n == 0 || m == 0 || trivial) return GS_OK;
  if (ilo < 1 || ihi > n || ilo > ihi + 1) return set_err(ctx, GS_BADARG, "bad ilo/ihi");
  // composed row permutation of the swaps (balance.jl:198-220), applied after the scaling
  std::vector<int> src(n);
  for (int64_t i = 0; i < n; ++i) src[i] = (int)i;
  for (int64_t j = ilo - 1; j >= 1; --j) {
    const int64_t mm = sp[j - 1];
    if (mm < 1 || mm > n) return set_err(ctx, GS_BADARG, "bad permutation record");
    if (mm != j) std::swap(src[j - 1], src[mm - 1]);
  }
  for (int64_t j = ihi + 1; j <= n; ++j) {
    const int64_t mm = sp[j - 1];
    if (mm < 1 || mm > n) return set_err(ctx, GS_BADARG, "bad permutation record");
    if (mm != j) std::swap(src[j - 1], src[mm - 1]);
  }
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nm = (size_t)n * m;
  Arena ar;
  const size_t o_V = ar.take<double2>(nm), o_W = ar.take<double2>(nm), o_src = ar.take<int>(n),
               o_D = ar.take<double>(n);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  double2* dV = (double2*)(base + o_V);
  double2* dW = (double2*)(base + o_W);
  int* dsrc = (int*)(base + o_src);
  double* dD = (double*)(base + o_D);
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CK(cudaMemcpy2DAsync(dV, n * sizeof(double2), V, ldv * sizeof(double2), n * sizeof(double2), m, in, s));
  CK(cudaMemcpyAsync(dsrc, src.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dD, D, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(launch_bal_apply((int)n, (int)m, dV, (int)n, dW, dsrc, dD, ilo != ihi, inverse, ctx->num_sms, s));
  CK(cudaMemcpy2DAsync(V, ldv * sizeof(double2), dW, n * sizeof(double2), n * sizeof(double2), m, out, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

int gs_enormalize_c64(gs_context* ctx, int64_t n, int64_t m, double* V, int64_t ldv, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || m < 0 || ldv < std::max<int64_t>(n, 1)) return set_err(ctx, GS_BADARG, "bad dimensions");
  if (n == 0 || m == 0) return GS_OK;
  if (!V) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nm = (size_t)n * m;
  Arena ar;
  const size_t o_V = ar.take<double2>(nm), o_bad = ar.take<int>(4);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  double2* dV = (double2*)(base + o_V);
  int* bad = (int*)(base + o_bad);
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CK(cudaMemsetAsync(bad, 0, sizeof(int), s));
  CK(cudaMemcpy2DAsync(dV, n * sizeof(double2), V, ldv * sizeof(double2), n * sizeof(double2), m, in, s));
  CK(launch_enormalize((int)n, (int)m, dV, !(flags & GS_RAW), bad, s));
  CK(cudaMemcpy2DAsync(V, ldv * sizeof(double2), dV, n * sizeof(double2), n * sizeof(double2), m, out, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

int gs_rconde_c64(gs_context* ctx, int64_t n, const double* VL, const double* VR, double* rconde, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0) return set_err(ctx, GS_BADARG, "negative order");
  if (n == 0) return GS_OK;
  if (!VL || !VR || !rconde) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  Arena ar;
  const size_t o_L = ar.take<double2>(dev ? 1 : nn), o_R = ar.take<double2>(dev ? 1 : nn), o_o = ar.take<double>(n);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const double2* dL = (const double2*)VL;
  const double2* dR = (const double2*)VR;
  double* dout = dev ? rconde : (double*)(base + o_o);
  if (!dev) {
    CK(cudaMemcpyAsync(base + o_L, VL, sizeof(double2) * nn, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_R, VR, sizeof(double2) * nn, cudaMemcpyHostToDevice, s));
    dL = (const double2*)(base + o_L);
    dR = (const double2*)(base + o_R);
  }
  CK(launch_rconde((int)n, (int)n, dL, dR, dout, s));
  if (!dev) CK(cudaMemcpyAsync(rconde, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

}  // extern "C"

// gordschur!(T, Z, select): real standard form (rordschur.jl:3-47) or complex triangular
// (ordschur.jl:24-74).  T, Z n x n, leading dimension n (in place); select n int32.
static int ordschur_impl(gs_context* ctx, int64_t n, double* T, double* Z, const int32_t* select, double* wr,
                         double* wi, unsigned flags, bool cplx) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 16)) return set_err(ctx, GS_BADARG, "bad order %lld", (long long)n);
  if (n == 0) return GS_OK;
  if (!T || !Z || !select || !wr || (!cplx && !wi)) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n, es = cplx ? sizeof(double2) : sizeof(double);
  Arena ar;
  const size_t o_T = ar.take<char>(dev ? 1 : es * nn), o_Z = ar.take<char>(dev ? 1 : es * nn),
               o_sel = ar.take<int>(n), o_w = ar.take<double>(2 * n), o_st = ar.take<int>(4);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  void* dT = dev ? (void*)T : (void*)(base + o_T);
  void* dZ = dev ? (void*)Z : (void*)(base + o_Z);
  int* dsel = (int*)(base + o_sel);
  double* dw = (double*)(base + o_w);
  int* dst = (int*)(base + o_st);
  if (!dev) {
    CK(cudaMemcpyAsync(dT, T, es * nn, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dZ, Z, es * nn, cudaMemcpyHostToDevice, s));
  }
  CK(cudaMemcpyAsync(dsel, select, sizeof(int) * n, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(dst, 0, sizeof(int), s));
  CK(cudaEventRecord(ctx->t0, s));
  if (cplx) CK(launch_ordschur_cplx((double2*)dT, (double2*)dZ, (int)n, dsel, (double2*)dw, s));
  else CK(launch_ordschur_real((double*)dT, (double*)dZ, (int)n, dsel, dw, dw + n, dst, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  int st = 0;
  CK(cudaMemcpyAsync(&st, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (!dev) {
    CK(cudaMemcpyAsync(T, dT, es * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(Z, dZ, es * nn, cudaMemcpyDeviceToHost, s));
  }
  if (cplx) {
    CK(cudaMemcpyAsync(wr, dw, sizeof(double2) * n, out, s));
  } else {
    CK(cudaMemcpyAsync(wr, dw, sizeof(double) * n, out, s));
    CK(cudaMemcpyAsync(wi, dw + n, sizeof(double) * n, out, s));
  }
  CK(cudaStreamSynchronize(s));
  if (st) return set_err(ctx, GS_UNCONVERGED, "IllConditionException: block %d could not be swapped", st);
  return GS_OK;
}

extern "C" {

int gs_ordschur_f64(gs_context* ctx, int64_t n, double* T, double* Z, const int32_t* select, double* wr, double* wi,
                    unsigned flags) {
  return ordschur_impl(ctx, n, T, Z, select, wr, wi, flags, false);
}

int gs_ordschur_c64(gs_context* ctx, int64_t n, double* T, double* Z, const int32_t* select, double* w,
                    unsigned flags) {
  return ordschur_impl(ctx, n, T, Z, select, w, nullptr, flags, true);
}

}  // extern "C"


// ---- condition estimators: eigvalscond / subspacesep (ordschur.jl:84-140) ----------
namespace {

// Julia's max / min propagate NaN
inline double jmax(double a, double b) { return (a != a || b != b) ? NAN : std::max(a, b); }

// Device workspace of one estimate for the leading m = nsub block of an n x n T.
struct CondLayout {
  size_t o_adjA, o_adjB, o_x, o_bak, o_flag, o_dbl, o_max, bytes;
};
template <class S> CondLayout cond_layout(int64_t n, int64_t m, size_t base) {
  const int64_t p = n - m;
  Arena ar;
  ar.off = base;
  CondLayout L;
  L.o_adjA = ar.take<S>((size_t)m * m);
  L.o_adjB = ar.take<S>((size_t)p * p);
  L.o_x = ar.take<S>((size_t)std::max<int64_t>(m * p, 1));
  L.o_bak = ar.take<S>((size_t)std::max<int64_t>(m * p, 1));
  L.o_flag = ar.take<int>(4);
  L.o_dbl = ar.take<double>(8);
  L.o_max = ar.take<unsigned long long>(2);
  L.bytes = ar.off;
  return L;
}

// norm1est! (norm1est.jl:21-74) on the host over an operator applied in place to the
// device vector x (N entries): apply(adjoint) runs the operator or its adjoint on x.
// work holds at least four doubles of device memory.
template <class S, class Apply>
int norm1est_host(gs_context* ctx, cudaStream_t s, S* x, long long N, double* work, Apply apply, double* est_out) {
  const double tiny = 2.2250738585072014e-308;
  double st[4];
  auto step = [&](int op, double arg) -> int {
    CK(launch_n1_step<S>(op, x, N, arg, ctx->num_sms, s));
    return GS_OK;
  };
  auto stats = [&](long long jlast) -> int {
    CK(launch_n1_stats<S>(x, N, jlast, work, s));
    CK(cudaMemcpyAsync(st, work, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return GS_OK;
  };
#define COND_TRY(expr) do { int rc_ = (expr); if (rc_) return rc_; } while (0)
  COND_TRY(step(N1_FILL, 1.0 / (double)N));
  COND_TRY(apply(false));
  COND_TRY(stats(-1));
  double est;
  if (N == 1) {
    est = st[0];
  } else {
    double gamma = st[0];
    COND_TRY(step(N1_SIGN, tiny));
    COND_TRY(apply(true));
    COND_TRY(stats(-1));
    long long j0 = (long long)st[2];
    for (int iter = 0; iter < 5; ++iter) {
      COND_TRY(step(N1_UNIT, (double)j0));
      COND_TRY(apply(false));
      COND_TRY(stats(-1));
      const double old = gamma;
      gamma = st[0];
      if (gamma <= old) break;
      COND_TRY(step(N1_SIGN, tiny));
      COND_TRY(apply(true));
      const long long jlast = j0;
      COND_TRY(stats(jlast));
      j0 = (long long)st[2];
      if (st[3] == st[1]) break;
    }
    COND_TRY(step(N1_ALT, 0.0));
    COND_TRY(apply(false));
    COND_TRY(stats(-1));
    const double t = 2.0 * st[0] / (double)(3 * N);
    est = jmax(t, gamma);
  }
#undef COND_TRY
  *est_out = est;
  return GS_OK;
}

template <class S> struct CondRun {
  gs_context* ctx;
  cudaStream_t s;
  const S* T;     // device, leading dimension ldt
  int ldt, m, p;
  char* base;
  CondLayout L;
  double smin = 0, bignum = 0;

  S* x() const { return (S*)(base + L.o_x); }
  int* flag() const { return (int*)(base + L.o_flag); }
  double* dbl() const { return (double*)(base + L.o_dbl); }

  // smin and bignum of trsylvester! (sylvester.jl:37-41) for T11 = T[1:m,1:m], T22.
  int prepare(bool adjoint) {
    unsigned long long* dmax = (unsigned long long*)(base + L.o_max);
    CK(cudaMemsetAsync(dmax, 0, 2 * sizeof(unsigned long long), s));
    CK(launch_cond_maxabs<S>(T, ldt, m, m, dmax, ctx->num_sms, s));
    CK(launch_cond_maxabs<S>(T + m + (size_t)m * ldt, ldt, p, p, dmax + 1, ctx->num_sms, s));
    if (adjoint) {
      CK(launch_adj_copy<S>(T, ldt, m, (S*)(base + L.o_adjA), ctx->num_sms, s));
      CK(launch_adj_copy<S>(T + m + (size_t)m * ldt, ldt, p, (S*)(base + L.o_adjB), ctx->num_sms, s));
    }
    unsigned long long bits[2];
    CK(cudaMemcpyAsync(bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    double na, nb;
    std::memcpy(&na, &bits[0], sizeof(double));
    std::memcpy(&nb, &bits[1], sizeof(double));
    const double tiny = 2.220446049250313e-16;
    const double small = 2.2250738585072014e-308 * m * p / tiny;
    bignum = 1.0 / small;
    smin = jmax(small, tiny * na * nb);
    return GS_OK;
  }

  // trsylvester! (adj = false) / adjtrsylvester! (adj = true) on C = x (m x p, ld m);
  // *scale receives sigma.
  int solve(bool adj, double* scale) {
    SylvArgs<S> P;
    P.A = adj ? (const S*)(base + L.o_adjA) : T;
    P.lda = adj ? m : ldt;
    P.B = adj ? (const S*)(base + L.o_adjB) : T + m + (size_t)m * ldt;
    P.ldb = adj ? p : ldt;
    P.C = x();
    P.ldc = m;
    P.m = m;
    P.p = p;
    P.mT = (m + 31) / 32;
    P.pT = (p + 31) / 32;
    P.flip = adj ? 1 : 0;
    P.le = adj ? 0 : 1;
    P.pos = 0;
    P.smin = smin;
    P.bignum = bignum;
    P.flag = flag();
    const size_t bytes = sizeof(S) * (size_t)m * p;
    CK(cudaMemcpyAsync(base + L.o_bak, x(), bytes, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(flag(), 0, sizeof(int), s));
    CK(launch_trsyl_levels<S>(P, s));
    int fl = 0;
    CK(cudaMemcpyAsync(&fl, flag(), sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *scale = 1.0;
    if (fl & 6) {
      // the overflow rescaling (or a non-finite entry): the reference's element order
      CK(cudaMemcpyAsync(x(), base + L.o_bak, bytes, cudaMemcpyDeviceToDevice, s));
      CK(launch_trsyl_exact<S>(P, dbl() + 7, s));
      CK(cudaMemcpyAsync(scale, dbl() + 7, sizeof(double), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
    return GS_OK;
  }

  // stats of x: {sum |x|, _findamax value, its index, |x[jlast]|}
  int stats(long long jlast, double out[4]) {
    CK(launch_n1_stats<S>(x(), (long long)m * p, jlast, dbl(), s));
    CK(cudaMemcpyAsync(out, dbl(), 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return GS_OK;
  }

  // eigvalscond (ordschur.jl:92-105)
  int eigvalscond(double* out) {
    if (m == 0 || p == 0) { *out = 1.0; return GS_OK; }
    int rc = prepare(false);
    if (rc) return rc;
    CK(cudaMemcpy2DAsync(x(), sizeof(S) * m, T + (size_t)m * ldt, sizeof(S) * ldt, sizeof(S) * m, p,
                         cudaMemcpyDeviceToDevice, s));
    double scale;
    rc = solve(false, &scale);
    if (rc) return rc;
    CK(launch_cond_fro<S>(x(), (long long)m * p, dbl() + 6, s));
    double rnorm;
    CK(cudaMemcpyAsync(&rnorm, dbl() + 6, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *out = rnorm > 0.0 ? scale / (std::sqrt(scale * scale / rnorm + rnorm) * std::sqrt(rnorm)) : 1.0;
    return GS_OK;
  }

  // subspacesep (ordschur.jl:118-140) through norm1est! (norm1est.jl:21-74)
  int subspacesep(double* out) {
    if (m == 0 || p == 0) return set_err(ctx, GS_BADARG, "subspacesep needs 0 < nsub < n");
    int rc = prepare(true);
    if (rc) return rc;
    double scale = 1.0, est = 0.0;
    rc = norm1est_host<S>(
        ctx, s, x(), (long long)m * p, dbl(), [&](bool adj) { return solve(adj, &scale); }, &est);
    if (rc) return rc;
    *out = scale / est;
    return GS_OK;
  }
};

// trsylvester!(A, B, C; possign) / adjtrsylvester! (sylvester.jl:11-139) for upper
// triangular A (m x m) and B (n x n) on C (m x n), through the tiled level solve of
// condition.cu (and the reference's element order when a rescaling or a non-finite entry
// is met).
template <class S>
int trsyl_std_impl(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B, int64_t ldb,
                   double* C, int64_t ldc, int adjoint, int possign, double* scale, int32_t* perturbed,
                   unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (m < 0 || n < 0 || lda < std::max<int64_t>(m, 1) || ldb < std::max<int64_t>(n, 1) ||
      ldc < std::max<int64_t>(m, 1))
    return set_err(ctx, GS_BADARG, "bad sizes");
  if (m > (1 << 16) || n > (1 << 16)) return set_err(ctx, GS_BADARG, "order too large");
  if (scale) *scale = 1.0;
  if (perturbed) *perturbed = 0;
  if (m == 0 || n == 0) return GS_OK;
  if (!A || !B || !C) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t mm = (size_t)m * m, nn = (size_t)n * n, mn = (size_t)m * n;
  Arena ar;
  const size_t o_A = ar.take<S>(mm), o_B = ar.take<S>(nn), o_C = ar.take<S>(mn), o_bak = ar.take<S>(mn),
               o_scr = ar.take<S>(adjoint ? std::max(mm, nn) : 1), o_max = ar.take<unsigned long long>(2),
               o_flag = ar.take<int>(4), o_dbl = ar.take<double>(2);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  S* dA = (S*)(base + o_A);
  S* dB = (S*)(base + o_B);
  S* dC = (S*)(base + o_C);
  CK(cudaMemcpy2DAsync(dA, sizeof(S) * m, A, sizeof(S) * lda, sizeof(S) * m, m, in, s));
  CK(cudaMemcpy2DAsync(dB, sizeof(S) * n, B, sizeof(S) * ldb, sizeof(S) * n, n, in, s));
  CK(cudaMemcpy2DAsync(dC, sizeof(S) * m, C, sizeof(S) * ldc, sizeof(S) * m, n, in, s));
  CK(cudaEventRecord(ctx->t0, s));
  unsigned long long* dmax = (unsigned long long*)(base + o_max);
  CK(cudaMemsetAsync(dmax, 0, 2 * sizeof(unsigned long long), s));
  CK(launch_cond_maxabs<S>(dA, (int)m, (int)m, (int)m, dmax, ctx->num_sms, s));
  CK(launch_cond_maxabs<S>(dB, (int)n, (int)n, (int)n, dmax + 1, ctx->num_sms, s));
  unsigned long long bits[2];
  CK(cudaMemcpyAsync(bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  double na, nb;
  std::memcpy(&na, &bits[0], sizeof(double));
  std::memcpy(&nb, &bits[1], sizeof(double));
  const double tiny = 2.220446049250313e-16;
  const double small = 2.2250738585072014e-308 * (double)m * (double)n / tiny;
  SylvArgs<S> P;
  if (adjoint) {
    // the forward solve on the reversed conjugate transposes; C through the index map
    S* Ap = (S*)(base + o_scr);
    CK(launch_adj_copy<S>(dA, (int)m, (int)m, Ap, ctx->num_sms, s));
    CK(cudaMemcpyAsync(dA, Ap, sizeof(S) * mm, cudaMemcpyDeviceToDevice, s));
    CK(launch_adj_copy<S>(dB, (int)n, (int)n, Ap, ctx->num_sms, s));
    CK(cudaMemcpyAsync(dB, Ap, sizeof(S) * nn, cudaMemcpyDeviceToDevice, s));
  }
  P.A = dA; P.lda = (int)m; P.B = dB; P.ldb = (int)n; P.C = dC; P.ldc = (int)m;
  P.m = (int)m; P.p = (int)n; P.mT = (int)((m + 31) / 32); P.pT = (int)((n + 31) / 32);
  P.flip = adjoint ? 1 : 0;
  P.le = adjoint ? 0 : 1;
  P.pos = possign ? 1 : 0;
  P.bignum = 1.0 / small;
  P.smin = jmax(small, tiny * na * nb);
  P.flag = (int*)(base + o_flag);
  CK(cudaMemcpyAsync(base + o_bak, dC, sizeof(S) * mn, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemsetAsync(P.flag, 0, sizeof(int), s));
  CK(launch_trsyl_levels<S>(P, s));
  int fl = 0;
  CK(cudaMemcpyAsync(&fl, P.flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  double sc = 1.0;
  if (fl & 6) {
    CK(cudaMemcpyAsync(dC, base + o_bak, sizeof(S) * mn, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(P.flag, 0, sizeof(int), s));
    CK(launch_trsyl_exact<S>(P, (double*)(base + o_dbl), s));
    CK(cudaMemcpyAsync(&sc, base + o_dbl, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&fl, P.flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  CK(cudaMemcpy2DAsync(C, sizeof(S) * ldc, dC, sizeof(S) * m, sizeof(S) * m, n,
                       dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (scale) *scale = sc;
  if (perturbed) *perturbed = (fl & 1) ? 1 : 0;
  return GS_OK;
}

template <class S>
int condition_impl(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* out, unsigned flags,
                   bool sep) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || nsub < 0 || nsub > n || ldt < std::max<int64_t>(n, 1)) return set_err(ctx, GS_BADARG, "bad sizes");
  if (!out || (n > 0 && !T)) return set_err(ctx, GS_BADARG, "null argument");
  if (n > (1 << 16)) return set_err(ctx, GS_BADARG, "order too large");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  Arena ar;
  const size_t o_T = ar.take<S>(dev ? 1 : (size_t)n * n);
  CondLayout L = cond_layout<S>(n, nsub, ar.off);
  int rc = ensure_ws(ctx, L.bytes);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;
  const S* dT = (const S*)T;
  int64_t ld = ldt;
  if (!dev && n > 0) {
    CK(cudaMemcpy2DAsync(ctx->dws + o_T, sizeof(S) * n, T, sizeof(S) * ldt, sizeof(S) * n, n,
                         cudaMemcpyHostToDevice, s));
    dT = (const S*)(ctx->dws + o_T);
    ld = n;
  }
  CondRun<S> r{ctx, s, dT, (int)ld, (int)nsub, (int)(n - nsub), ctx->dws, L};
  CK(cudaEventRecord(ctx->t0, s));
  rc = sep ? r.subspacesep(out) : r.eigvalscond(out);
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  return rc;
}

// eigen!(A; jcv = true) (pirates.jl:136-153): for each j, the eigenvalue moved to the
// front of a copy of T by ordschur!, then eigvalscond(., 1) and subspacesep(., 1).
template <class S>
int rcondv_impl(gs_context* ctx, int64_t n, const double* T, double* rconde, double* rcondv, unsigned flags) {
  constexpr bool cplx = sizeof(S) == sizeof(double2);
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 16)) return set_err(ctx, GS_BADARG, "bad order");
  if (n == 0) return GS_OK;
  if (!T || (!rconde && !rcondv)) return set_err(ctx, GS_BADARG, "null argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t nn = (size_t)n * n;
  Arena ar;
  const size_t o_T = ar.take<S>(nn), o_Tt = ar.take<S>(nn), o_Z = ar.take<S>(nn), o_sel = ar.take<int>(n),
               o_w = ar.take<double>(4 * n), o_st = ar.take<int>(4);
  CondLayout L = cond_layout<S>(n, 1, ar.off);
  int rc = ensure_ws(ctx, L.bytes);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  S* dT = (S*)(base + o_T);
  S* dTt = (S*)(base + o_Tt);
  S* dZ = (S*)(base + o_Z);
  int* dsel = (int*)(base + o_sel);
  double* dw = (double*)(base + o_w);
  int* dst = (int*)(base + o_st);
  CK(cudaMemcpyAsync(dT, T, sizeof(S) * nn, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(dZ, 0, sizeof(S) * nn, s));  // the reordering's Z is not wanted
  std::vector<int> sel((size_t)n, 0);
  std::vector<double> ec(rconde ? n : 0), vc(rcondv ? n : 0);
  CK(cudaEventRecord(ctx->t0, s));
  for (int64_t j = 0; j < n; ++j) {
    CK(cudaMemcpyAsync(dTt, dT, sizeof(S) * nn, cudaMemcpyDeviceToDevice, s));
    sel.assign((size_t)n, 0);
    sel[j] = 1;
    CK(cudaMemcpyAsync(dsel, sel.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(dst, 0, sizeof(int), s));
    if (cplx) CK(launch_ordschur_cplx((double2*)dTt, (double2*)dZ, (int)n, dsel, (double2*)dw, s));
    else CK(launch_ordschur_real((double*)dTt, (double*)dZ, (int)n, dsel, dw, dw + n, dst, s));
    int st = 0;
    CK(cudaMemcpyAsync(&st, dst, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (st) return set_err(ctx, GS_UNCONVERGED, "reordering rejected a block swap (eigenvalue %lld)", (long long)j + 1);
    CondRun<S> r{ctx, s, dTt, (int)n, 1, (int)(n - 1), base, L};
    if (rconde) {
      rc = r.eigvalscond(&ec[j]);
      if (rc) return rc;
    }
    if (rcondv) {
      if (n == 1) {
        return set_err(ctx, GS_BADARG, "subspacesep needs n > 1");
      }
      rc = r.subspacesep(&vc[j]);
      if (rc) return rc;
    }
  }
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  const cudaMemcpyKind k = dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
  if (rconde) CK(cudaMemcpyAsync(rconde, ec.data(), sizeof(double) * n, k, s));
  if (rcondv) CK(cudaMemcpyAsync(rcondv, vc.data(), sizeof(double) * n, k, s));
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

// Generalized Sylvester solves and condition estimates of a complex generalized Schur form
// (gsylvester.jl, gcondition.jl) over the wavefront solver of gcondition.cu.
struct GsylRun {
  gs_context* ctx;
  cudaStream_t s;
  int* flag;     // device, one int
  GsylBar* bar;  // device
  double* dbl;   // device, eight doubles

  // one solve; *pert receives the perturbed-pivot flag of the reference
  int run(int mode, int m, int n, const double2* A, int lda, const double2* B, int ldb, const double2* D, int ldd,
          const double2* E, int lde, double2* C, int ldc, double2* F, int ldf, bool* pert = nullptr) {
    if (pert) *pert = false;
    if (m == 0 || n == 0) return GS_OK;
    GsylArgs P{A, B, D, E, lda, ldb, ldd, lde, C, F, ldc, ldf, m, n, mode, flag, bar};
    CK(cudaMemsetAsync(flag, 0, sizeof(int), s));
    CK(cudaMemsetAsync(bar, 0, gsyl_bar_bytes(), s));
    CK(launch_gsyl(P, ctx->num_sms, s));
    int fl = 0;
    CK(cudaMemcpyAsync(&fl, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (fl & 8) return set_err(ctx, GS_CUDA, "generalized Sylvester solve: grid barrier timed out");
    if (fl & 2)
      return set_err(ctx, GS_BADARG,
                     "generalized Sylvester solve: a 2 x 2 system needed rescaling against overflow, where "
                     "the reference's trsylvester! calls lmul!(view, scale) and raises");
    if (fl & 4)
      return set_err(ctx, GS_BADARG, "singular 2 x 2 system in the separation estimate (lu raises SingularException)");
    if (pert) *pert = (fl & 1) != 0;
    return GS_OK;
  }

  double fro(const double2* x, long long N, int slot) {
    if (N == 0) return 0.0;
    if (launch_cond_fro<double2>(x, N, dbl + slot, s) != cudaSuccess) return -1.0;
    double v = -1.0;
    if (cudaMemcpyAsync(&v, dbl + slot, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1.0;
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1.0;
    return v;
  }
};

struct GCondLayout {
  size_t o_S, o_T, o_x, o_flag, o_bar, o_dbl, bytes;
};
GCondLayout gcond_layout(int64_t n, int64_t nsub, bool dev) {
  Arena ar;
  GCondLayout L;
  L.o_S = ar.take<double2>(dev ? 1 : (size_t)n * n);
  L.o_T = ar.take<double2>(dev ? 1 : (size_t)n * n);
  L.o_x = ar.take<double2>((size_t)std::max<int64_t>(2 * nsub * (n - nsub), 1));
  L.o_flag = ar.take<int>(4);
  L.o_bar = ar.take<char>(std::max<size_t>(gsyl_bar_bytes(), 16));
  L.o_dbl = ar.take<double>(8);
  L.bytes = ar.off;
  return L;
}

// eigvalscond (what = 0, gcondition.jl:121-165) and subspacesep (what = 1 with pnorm 0 for
// :F, 1 for the one-norm estimate; gcondition.jl:169-260) of the pencil's leading nsub block.
int gcond_impl(gs_context* ctx, int64_t n, const double* S, int64_t lds, const double* T, int64_t ldt, int64_t nsub,
               int what, int pnorm, double* out, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || nsub < 0 || nsub > n || lds < std::max<int64_t>(n, 1) || ldt < std::max<int64_t>(n, 1))
    return set_err(ctx, GS_BADARG, "bad sizes");
  if (n > (1 << 16)) return set_err(ctx, GS_BADARG, "order too large");
  if (!out || (n > 0 && (!S || !T))) return set_err(ctx, GS_BADARG, "null argument");
  if (what == 1 && pnorm != 0 && pnorm != 1) return set_err(ctx, GS_BADARG, "pnorm must be :Frobenius or 1");
  const int64_t n1 = nsub, n2 = n - nsub;
  if (what == 0 && (n1 == 0 || n2 == 0)) {
    out[0] = out[1] = 1.0;
    return GS_OK;
  }
  if (what == 1 && pnorm == 0 && (n1 == 0 || n2 == 0)) {
    out[0] = out[1] = 0.0;
    return GS_OK;
  }
  if (what == 1 && (n1 == 0 || n2 == 0)) return set_err(ctx, GS_BADARG, "subspacesep with pnorm = 1 needs 0 < nsub < n");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const GCondLayout L = gcond_layout(n, nsub, dev);
  int rc = ensure_ws(ctx, L.bytes);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const double2* dS = (const double2*)S;
  const double2* dT = (const double2*)T;
  int64_t ls = lds, lt = ldt;
  if (!dev) {
    CK(cudaMemcpy2DAsync(base + L.o_S, 16 * n, S, 16 * lds, 16 * n, n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpy2DAsync(base + L.o_T, 16 * n, T, 16 * ldt, 16 * n, n, cudaMemcpyHostToDevice, s));
    dS = (const double2*)(base + L.o_S);
    dT = (const double2*)(base + L.o_T);
    ls = lt = n;
  }
  GsylRun g{ctx, s, (int*)(base + L.o_flag), (GsylBar*)(base + L.o_bar), (double*)(base + L.o_dbl)};
  double2* x = (double2*)(base + L.o_x);
  const long long N1 = (long long)n1 * n2;
  const double2 *S11 = dS, *S22 = dS + n1 + (size_t)n1 * ls, *T11 = dT, *T22 = dT + n1 + (size_t)n1 * lt;
  CK(cudaEventRecord(ctx->t0, s));
  double res[2] = {0.0, 0.0};
  if (what == 0) {
    // S11 R - L S22 = s S12, T11 R - L T22 = s T12
    CK(cudaMemcpy2DAsync(x, 16 * n1, dS + (size_t)n1 * ls, 16 * ls, 16 * n1, n2, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpy2DAsync(x + N1, 16 * n1, dT + (size_t)n1 * lt, 16 * lt, 16 * n1, n2, cudaMemcpyDeviceToDevice, s));
    rc = g.run(0, (int)n1, (int)n2, S11, (int)ls, S22, (int)ls, T11, (int)lt, T22, (int)lt, x, (int)n1, x + N1, (int)n1);
    if (rc) return rc;
    for (int k = 0; k < 2; ++k) {
      const double p = g.fro(x + k * N1, N1, k);
      if (p < 0.0) return set_err(ctx, GS_CUDA, "CUDA error in the norm of the Sylvester solution");
      res[k] = p == 0.0 ? 1.0 : 1.0 / (std::sqrt(1.0 / p + p) * std::sqrt(p));
    }
  } else {
    for (int k = 0; k < 2; ++k) {
      // k = 0: (S11, S22, T11, T22), m = n1; k = 1: the blocks exchanged, m = n2
      const int m = (int)(k == 0 ? n1 : n2), q = (int)(k == 0 ? n2 : n1);
      const double2 *A = k == 0 ? S11 : S22, *B = k == 0 ? S22 : S11, *D = k == 0 ? T11 : T22, *E = k == 0 ? T22 : T11;
      if (pnorm == 0) {
        CK(cudaMemsetAsync(x, 0, 16 * (size_t)(2 * N1), s));
        rc = g.run(2, m, q, A, (int)ls, B, (int)ls, D, (int)lt, E, (int)lt, x, m, x + N1, m);
        if (rc) return rc;
        const double f = g.fro(x, 2 * N1, 2);
        if (f < 0.0) return set_err(ctx, GS_CUDA, "CUDA error in the norm of the look-ahead solution");
        res[k] = std::sqrt(2.0 * (double)m * (double)q) / f;
      } else {
        double est = 0.0;
        rc = norm1est_host<double2>(
            ctx, s, x, 2 * N1, g.dbl,
            [&](bool adj) {
              return g.run(adj ? 1 : 0, m, q, A, (int)ls, B, (int)ls, D, (int)lt, E, (int)lt, x, m, x + N1, m);
            },
            &est);
        if (rc) return rc;
        res[k] = 1.0 / est;
      }
    }
  }
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  out[0] = res[0];
  out[1] = res[1];
  return GS_OK;
}

// trsylvester!(A, B, C, D, E, F) / adjtrsylvester! (gsylvester.jl:23-155), complex.
int gtrsyl_impl(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B, int64_t ldb,
                double* C, int64_t ldc, const double* D, int64_t ldd, const double* E, int64_t lde, double* F,
                int64_t ldf, int adjoint, double* scale, int32_t* perturbed, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  const int64_t m1 = std::max<int64_t>(m, 1);
  if (m < 0 || n < 0 || lda < m1 || ldd < m1 || ldc < m1 || ldf < m1 || ldb < std::max<int64_t>(n, 1) ||
      lde < std::max<int64_t>(n, 1))
    return set_err(ctx, GS_BADARG, "bad sizes");
  if (m > (1 << 16) || n > (1 << 16)) return set_err(ctx, GS_BADARG, "order too large");
  if (scale) *scale = 1.0;
  if (perturbed) *perturbed = 0;
  if (m == 0 || n == 0) return GS_OK;
  if (!A || !B || !C || !D || !E || !F) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const size_t mm = (size_t)m * m, nn = (size_t)n * n, mn = (size_t)m * n;
  Arena ar;
  const size_t o_A = ar.take<double2>(dev ? 1 : mm), o_D = ar.take<double2>(dev ? 1 : mm),
               o_B = ar.take<double2>(dev ? 1 : nn), o_E = ar.take<double2>(dev ? 1 : nn),
               o_C = ar.take<double2>(dev ? 1 : mn), o_F = ar.take<double2>(dev ? 1 : mn), o_flag = ar.take<int>(4),
               o_bar = ar.take<char>(std::max<size_t>(gsyl_bar_bytes(), 16)), o_dbl = ar.take<double>(8);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const double2 *dA = (const double2*)A, *dB = (const double2*)B, *dD = (const double2*)D, *dE = (const double2*)E;
  double2 *dC = (double2*)C, *dF = (double2*)F;
  int64_t la = lda, lb = ldb, lc = ldc, ld = ldd, le = lde, lf = ldf;
  if (!dev) {
    auto up = [&](size_t off, const double* h, int64_t ldh, int64_t rows, int64_t cols) -> int {
      CK(cudaMemcpy2DAsync(base + off, 16 * rows, h, 16 * ldh, 16 * rows, cols, cudaMemcpyHostToDevice, s));
      return GS_OK;
    };
    if ((rc = up(o_A, A, lda, m, m)) || (rc = up(o_D, D, ldd, m, m)) || (rc = up(o_B, B, ldb, n, n)) ||
        (rc = up(o_E, E, lde, n, n)) || (rc = up(o_C, C, ldc, m, n)) || (rc = up(o_F, F, ldf, m, n)))
      return rc;
    dA = (const double2*)(base + o_A); dD = (const double2*)(base + o_D);
    dB = (const double2*)(base + o_B); dE = (const double2*)(base + o_E);
    dC = (double2*)(base + o_C); dF = (double2*)(base + o_F);
    la = ld = lc = lf = m;
    lb = le = n;
  }
  GsylRun g{ctx, s, (int*)(base + o_flag), (GsylBar*)(base + o_bar), (double*)(base + o_dbl)};
  CK(cudaEventRecord(ctx->t0, s));
  bool pert = false;
  rc = g.run(adjoint ? 1 : 0, (int)m, (int)n, dA, (int)la, dB, (int)lb, dD, (int)ld, dE, (int)le, dC, (int)lc, dF,
             (int)lf, &pert);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  if (!dev) {
    CK(cudaMemcpy2DAsync(C, 16 * ldc, dC, 16 * m, 16 * m, n, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpy2DAsync(F, 16 * ldf, dF, 16 * m, 16 * m, n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  if (perturbed) *perturbed = pert ? 1 : 0;
  return GS_OK;
}

}  // namespace

extern "C" {

int gs_eigvalscond_f64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* s,
                       unsigned flags) {
  return condition_impl<double>(ctx, n, T, ldt, nsub, s, flags, false);
}
int gs_eigvalscond_c64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* s,
                       unsigned flags) {
  return condition_impl<double2>(ctx, n, T, ldt, nsub, s, flags, false);
}
int gs_subspacesep_f64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* sep,
                       unsigned flags) {
  return condition_impl<double>(ctx, n, T, ldt, nsub, sep, flags, true);
}
int gs_subspacesep_c64(gs_context* ctx, int64_t n, const double* T, int64_t ldt, int64_t nsub, double* sep,
                       unsigned flags) {
  return condition_impl<double2>(ctx, n, T, ldt, nsub, sep, flags, true);
}
int gs_eigen_rcond_f64(gs_context* ctx, int64_t n, const double* T, double* rconde, double* rcondv, unsigned flags) {
  return rcondv_impl<double>(ctx, n, T, rconde, rcondv, flags);
}
int gs_eigen_rcond_c64(gs_context* ctx, int64_t n, const double* T, double* rconde, double* rcondv, unsigned flags) {
  return rcondv_impl<double2>(ctx, n, T, rconde, rcondv, flags);
}

int gs_trsylvester_f64(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B,
                       int64_t ldb, double* C, int64_t ldc, int32_t adjoint, int32_t possign, double* scale,
                       int32_t* perturbed, unsigned flags) {
  return trsyl_std_impl<double>(ctx, m, n, A, lda, B, ldb, C, ldc, adjoint, possign, scale, perturbed, flags);
}
int gs_trsylvester_c64(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B,
                       int64_t ldb, double* C, int64_t ldc, int32_t adjoint, int32_t possign, double* scale,
                       int32_t* perturbed, unsigned flags) {
  return trsyl_std_impl<double2>(ctx, m, n, A, lda, B, ldb, C, ldc, adjoint, possign, scale, perturbed, flags);
}
int gs_gtrsylvester_c64(gs_context* ctx, int64_t m, int64_t n, const double* A, int64_t lda, const double* B,
                        int64_t ldb, double* C, int64_t ldc, const double* D, int64_t ldd, const double* E,
                        int64_t lde, double* F, int64_t ldf, int32_t adjoint, double* scale, int32_t* perturbed,
                        unsigned flags) {
  return gtrsyl_impl(ctx, m, n, A, lda, B, ldb, C, ldc, D, ldd, E, lde, F, ldf, adjoint, scale, perturbed, flags);
}
int gs_geigvalscond_c64(gs_context* ctx, int64_t n, const double* S, int64_t lds, const double* T, int64_t ldt,
                        int64_t nsub, double* plpr, unsigned flags) {
  return gcond_impl(ctx, n, S, lds, T, ldt, nsub, 0, 0, plpr, flags);
}
int gs_gsubspacesep_c64(gs_context* ctx, int64_t n, const double* S, int64_t lds, const double* T, int64_t ldt,
                        int64_t nsub, int32_t pnorm, double* sep, unsigned flags) {
  return gcond_impl(ctx, n, S, lds, T, ldt, nsub, 1, pnorm, sep, flags);
}
}  // extern "C"

// ---- Hermitian path: geigen! / geigvals!, hessenberg!(Hermitian), _gschur!(SymTridiagonal) ----
namespace {

struct HeLayout {
  size_t o_A, o_B, o_W, o_part, o_ctl, o_tau, o_d, o_e, o_Q, o_rot, o_st, o_p, o_dc, bytes;
  int npart;
};
template <class S> HeLayout he_layout(int64_t n, bool host_a, bool wantq, int num_sms, bool dc = false) {
  HeLayout L;
  Arena ar;
  const size_t nn = (size_t)n * n;
  L.npart = std::max(1, 4 * num_sms);
  L.o_A = ar.take<S>(host_a ? nn : 1);
  L.o_B = ar.take<S>(std::max<size_t>(nn, 1));
  L.o_W = ar.take<S>(std::max<int64_t>(n, 1));
  L.o_part = ar.take<S>(L.npart);
  L.o_ctl = ar.take<HeCtlBuf>(1);
  L.o_tau = ar.take<S>(std::max<int64_t>(n, 1));
  L.o_d = ar.take<double>(std::max<int64_t>(n, 1));
  L.o_e = ar.take<double>(std::max<int64_t>(n, 1));
  L.o_Q = ar.take<S>(wantq ? nn : 1);
  L.o_rot = ar.take<double>(4 * std::max<int64_t>(n, 1));
  L.o_st = ar.take<char>(steqr_ctl_bytes());
  L.o_p = ar.take<int>(std::max<int64_t>(n, 1));
  L.o_dc = ar.take<char>(dc ? stedc_ws_bytes((int)n, sizeof(S) == sizeof(double2) ? 1 : 0) : 1);
  L.bytes = ar.off;
  return L;
}

// run_stedc's status as the library's error codes (the reference throws
// UnconvergedException when a secular equation fails, symtri_dc.jl:190-192)
int stedc_result(gs_context* ctx, int st) {
  if (st & 4) return set_err(ctx, GS_CUDA, "divide and conquer: a tensor-core GEMM wait timed out");
  if (st & 1) return set_err(ctx, GS_UNCONVERGED, "unable to solve secular equation accurately");
  if (st & 2) return set_err(ctx, GS_UNCONVERGED, "tridiagonal QR (divide-and-conquer leaf): sweep limit reached");
  return GS_OK;
}

// reads the sweep kernel's {err, status}
int steqr_result(gs_context* ctx, const char* st_dev, cudaStream_t s) {
  int words[5];
  CK(cudaMemcpyAsync(words, st_dev, sizeof(words), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (words[2]) return set_err(ctx, GS_CUDA, "tridiagonal QR: a grid barrier wait gave up");
  if (words[4]) return set_err(ctx, GS_UNCONVERGED, "tridiagonal QR: sweep limit reached");
  return GS_OK;
}

template <class S>
int heev_impl(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* w, double* V, int64_t ldv,
              unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 16) || lda < std::max<int64_t>(n, 1)) return set_err(ctx, GS_BADARG, "bad sizes");
  if (uplo != 'L' && uplo != 'U') return set_err(ctx, GS_BADARG, "uplo must be 'L' or 'U'");
  const bool wantz = flags & GS_WANTZ;
  if (n == 0) return GS_OK;
  if (!A || !w || (wantz && (!V || ldv < n))) return set_err(ctx, GS_BADARG, "null or short array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const bool dc = flags & GS_DC;
  if (dc && n > (1 << 15)) return set_err(ctx, GS_BADARG, "order too large for divide and conquer");
  const HeLayout L = he_layout<S>(n, !dev, wantz, ctx->num_sms, dc);
  int rc = ensure_ws(ctx, L.bytes);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  const S* dA = (const S*)A;
  int64_t ld = lda;
  if (!dev) {
    CK(cudaMemcpy2DAsync(base + L.o_A, sizeof(S) * n, A, sizeof(S) * lda, sizeof(S) * n, n, cudaMemcpyHostToDevice, s));
    dA = (const S*)(base + L.o_A);
    ld = n;
  }
  S* B = (S*)(base + L.o_B);
  S* tau = (S*)(base + L.o_tau);
  double* d = (double*)(base + L.o_d);
  double* e = (double*)(base + L.o_e);
  S* Q = (S*)(base + L.o_Q);
  const int upper = uplo == 'U';
  CK(cudaEventRecord(ctx->t0, s));
  CK(launch_he_tridiag<S>(dA, ld, (int)n, upper, B, (S*)(base + L.o_W), (S*)(base + L.o_part), L.npart,
                          (HeCtlBuf*)(base + L.o_ctl), tau, d, e, ctx->num_sms, s));
  if (wantz) CK(launch_he_formq<S>(B, (int)n, tau, Q, ctx->num_sms, s));
  if (dc) {
    // gschur!(H, V, DivideAndConquer()) (GenericSchur.jl:126-136, symtri_dc.jl:6-104)
    int st = 0;
    CK(run_stedc((int)n, d, e, wantz ? (double*)Q : nullptr, n, sizeof(S) == sizeof(double2) ? 1 : 0, base + L.o_dc,
                 ctx->num_sms, s, &st));
    CK(cudaEventRecord(ctx->t1, s));
    ctx->timed = true;
    rc = stedc_result(ctx, st);
  } else {
    CK(launch_steqr<S>((int)n, d, e, wantz ? Q : nullptr, n, wantz ? (int)n : 0, (double*)(base + L.o_rot),
                       base + L.o_st, 30LL * n, ctx->num_sms, s));
    CK(cudaEventRecord(ctx->t1, s));
    ctx->timed = true;
    rc = steqr_result(ctx, base + L.o_st, s);
  }
  if (rc == GS_CUDA) return rc;
  // sorteig!(w, V, eigsortby): stable ascending order
  std::vector<double> dh(n);
  CK(cudaMemcpyAsync(dh.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  std::vector<int> p(n);
  for (int64_t i = 0; i < n; ++i) p[i] = (int)i;
  std::stable_sort(p.begin(), p.end(), [&](int a, int b) { return dh[a] < dh[b]; });
  std::vector<double> ws(n);
  for (int64_t j = 0; j < n; ++j) ws[j] = dh[p[j]];
  CK(cudaMemcpyAsync(w, ws.data(), sizeof(double) * n, dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost, s));
  if (wantz) {
    int* dp = (int*)(base + L.o_p);
    CK(cudaMemcpyAsync(dp, p.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    if (dev) {
      CK(launch_he_gather<S>(Q, (int)n, dp, upper, (S*)V, ldv, s));
    } else {
      CK(launch_he_gather<S>(Q, (int)n, dp, upper, B, n, s));
      CK(cudaMemcpy2DAsync(V, sizeof(S) * ldv, B, sizeof(S) * n, sizeof(S) * n, n, cudaMemcpyDeviceToHost, s));
    }
  }
  CK(cudaStreamSynchronize(s));
  return rc;
}

template <class S>
int hetrd_impl(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* d, double* e, double* tau,
               unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 16) || lda < std::max<int64_t>(n, 1)) return set_err(ctx, GS_BADARG, "bad sizes");
  if (uplo != 'L' && uplo != 'U') return set_err(ctx, GS_BADARG, "uplo must be 'L' or 'U'");
  if (n == 0) return GS_OK;
  if (!A || !d || (n > 1 && (!e || !tau))) return set_err(ctx, GS_BADARG, "null array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  const HeLayout L = he_layout<S>(n, true, false, ctx->num_sms);
  int rc = ensure_ws(ctx, L.bytes);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  S* dA = (S*)(base + L.o_A);
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CK(cudaMemcpy2DAsync(dA, sizeof(S) * n, A, sizeof(S) * lda, sizeof(S) * n, n, in, s));
  S* B = (S*)(base + L.o_B);
  S* dtau = (S*)(base + L.o_tau);
  double* dd = (double*)(base + L.o_d);
  double* de = (double*)(base + L.o_e);
  const int upper = uplo == 'U';
  CK(cudaEventRecord(ctx->t0, s));
  CK(launch_he_tridiag<S>(dA, n, (int)n, upper, B, (S*)(base + L.o_W), (S*)(base + L.o_part), L.npart,
                          (HeCtlBuf*)(base + L.o_ctl), dtau, dd, de, ctx->num_sms, s));
  CK(launch_he_store<S>(B, (int)n, upper, dA, n, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  CK(cudaMemcpy2DAsync(A, sizeof(S) * lda, dA, sizeof(S) * n, sizeof(S) * n, n, out, s));
  // d, e, tau to the host (reversed for the upper form), then out
  std::vector<double> hd(n), he(n > 1 ? n - 1 : 1);
  std::vector<S> ht(n > 1 ? n - 1 : 1);
  CK(cudaMemcpyAsync(hd.data(), dd, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (n > 1) {
    CK(cudaMemcpyAsync(he.data(), de, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ht.data(), dtau, sizeof(S) * (n - 1), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (upper) {
    std::reverse(hd.begin(), hd.end());
    if (n > 1) {
      std::reverse(he.begin(), he.begin() + (n - 1));
      std::reverse(ht.begin(), ht.begin() + (n - 1));
    }
  }
  const cudaMemcpyKind hk = dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
  CK(cudaMemcpyAsync(d, hd.data(), sizeof(double) * n, hk, s));
  if (n > 1) {
    CK(cudaMemcpyAsync(e, he.data(), sizeof(double) * (n - 1), hk, s));
    CK(cudaMemcpyAsync(tau, ht.data(), sizeof(S) * (n - 1), hk, s));
  }
  CK(cudaStreamSynchronize(s));
  return GS_OK;
}

}  // namespace

extern "C" {

int gs_heev_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* w, double* V, int64_t ldv,
                unsigned flags) {
  return heev_impl<double>(ctx, n, A, lda, uplo, w, V, ldv, flags);
}
int gs_heev_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* w, double* V, int64_t ldv,
                unsigned flags) {
  return heev_impl<double2>(ctx, n, A, lda, uplo, w, V, ldv, flags);
}
int gs_hetrd_f64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* d, double* e, double* tau,
                 unsigned flags) {
  return hetrd_impl<double>(ctx, n, A, lda, uplo, d, e, tau, flags);
}
int gs_hetrd_c64(gs_context* ctx, int64_t n, double* A, int64_t lda, int uplo, double* d, double* e, double* tau,
                 unsigned flags) {
  return hetrd_impl<double2>(ctx, n, A, lda, uplo, d, e, tau, flags);
}

int gs_stedc_f64(gs_context* ctx, int64_t n, double* d, double* e, double* Z, int64_t ldz, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 15)) return set_err(ctx, GS_BADARG, "bad order");
  if (n == 0) return GS_OK;
  if (!d || (n > 1 && !e) || (Z && ldz < n)) return set_err(ctx, GS_BADARG, "null or short array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  Arena ar;
  const size_t o_d = ar.take<double>(n), o_e = ar.take<double>(n), o_Z = ar.take<double>(Z && !dev ? (size_t)n * n : 1),
               o_dc = ar.take<char>(stedc_ws_bytes((int)n, 0));
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  double* dd = (double*)(base + o_d);
  double* de = (double*)(base + o_e);
  double* dZ = Z ? (dev ? Z : (double*)(base + o_Z)) : nullptr;
  const long long ldd = dev ? ldz : n;
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CK(cudaMemcpyAsync(dd, d, sizeof(double) * n, in, s));
  CK(cudaMemsetAsync(de, 0, sizeof(double) * n, s));
  if (n > 1) CK(cudaMemcpyAsync(de, e, sizeof(double) * (n - 1), in, s));
  if (Z && !dev)
    CK(cudaMemcpy2DAsync(dZ, sizeof(double) * n, Z, sizeof(double) * ldz, sizeof(double) * n, n, in, s));
  CK(cudaEventRecord(ctx->t0, s));
  int st = 0;
  CK(run_stedc((int)n, dd, de, dZ, ldd, 0, base + o_dc, ctx->num_sms, s, &st));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  rc = stedc_result(ctx, st);
  if (rc == GS_CUDA) return rc;
  CK(cudaMemcpyAsync(d, dd, sizeof(double) * n, out, s));
  if (n > 1) CK(cudaMemcpyAsync(e, de, sizeof(double) * (n - 1), out, s));
  if (Z && !dev)
    CK(cudaMemcpy2DAsync(Z, sizeof(double) * ldz, dZ, sizeof(double) * n, sizeof(double) * n, n, out, s));
  CK(cudaStreamSynchronize(s));
  return rc;
}

int gs_steqr_f64(gs_context* ctx, int64_t n, double* d, double* e, double* Z, int64_t ldz, unsigned flags) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (n < 0 || n > (1 << 16)) return set_err(ctx, GS_BADARG, "bad order");
  if (n == 0) return GS_OK;
  if (!d || (n > 1 && !e) || (Z && ldz < n)) return set_err(ctx, GS_BADARG, "null or short array argument");
  CK(cudaSetDevice(ctx->device));
  const bool dev = flags & GS_DEVICE;
  Arena ar;
  const size_t o_d = ar.take<double>(n), o_e = ar.take<double>(n), o_Z = ar.take<double>(Z && !dev ? (size_t)n * n : 1),
               o_rot = ar.take<double>(4 * n), o_st = ar.take<char>(steqr_ctl_bytes());
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  double* dd = (double*)(base + o_d);
  double* de = (double*)(base + o_e);
  double* dZ = Z ? (dev ? Z : (double*)(base + o_Z)) : nullptr;
  const long long ldd = dev ? ldz : n;
  const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CK(cudaMemcpyAsync(dd, d, sizeof(double) * n, in, s));
  CK(cudaMemsetAsync(de, 0, sizeof(double) * n, s));
  if (n > 1) CK(cudaMemcpyAsync(de, e, sizeof(double) * (n - 1), in, s));
  if (Z && !dev)
    CK(cudaMemcpy2DAsync(dZ, sizeof(double) * n, Z, sizeof(double) * ldz, sizeof(double) * n, n, in, s));
  CK(cudaEventRecord(ctx->t0, s));
  CK(launch_steqr<double>((int)n, dd, de, dZ, ldd, Z ? (int)n : 0, (double*)(base + o_rot), base + o_st, 30LL * n,
                          ctx->num_sms, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  rc = steqr_result(ctx, base + o_st, s);
  if (rc == GS_CUDA) return rc;
  CK(cudaMemcpyAsync(d, dd, sizeof(double) * n, out, s));
  if (n > 1) CK(cudaMemcpyAsync(e, de, sizeof(double) * (n - 1), out, s));
  if (Z && !dev)
    CK(cudaMemcpy2DAsync(Z, sizeof(double) * ldz, dZ, sizeof(double) * n, sizeof(double) * n, n, out, s));
  CK(cudaStreamSynchronize(s));
  return rc;
}

}  // extern "C"

// ---- generalized Schur of complex pencils: ggschur!(A, B) (generalized.jl:21-80) ----
namespace {

// single > 0: one pencil of that order (ns, offs, woffs unused).
int ggschur_real_impl(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs, int64_t plen, double* A,
                      double* B, double* Q, double* Z, const int64_t* woffs, int64_t wlen, double* alpha, double* beta,
                      int32_t* status, unsigned flags, int single = 0) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (count < 0 || plen < 0 || wlen < 0) return set_err(ctx, GS_BADARG, "negative size");
  if (count == 0) return GS_OK;
  if ((!single && (!ns || !offs || !woffs)) || !A || !B || !alpha || !beta)
    return set_err(ctx, GS_BADARG, "null array argument");
  const bool dev = flags & GS_DEVICE;
  if (!dev && !single) {
    for (int64_t b = 0; b < count; ++b) {
      const int64_t n = ns[b];
      if (n < 0 || n > 4096 || offs[b] < 0 || offs[b] + n * n > plen || woffs[b] < 0 || woffs[b] + n > wlen)
        return set_err(ctx, GS_BADARG, "pencil %lld: order or offsets out of range", (long long)b);
    }
  }
  CK(cudaSetDevice(ctx->device));
  Arena ar;
  const size_t o_ns = ar.take<int>(dev ? 1 : count), o_off = ar.take<long long>(dev ? 1 : count),
               o_woff = ar.take<long long>(dev ? 1 : count), o_A = ar.take<double>(dev ? 1 : plen),
               o_B = ar.take<double>(dev ? 1 : plen), o_Q = ar.take<double>(dev || !Q ? 1 : plen),
               o_Z = ar.take<double>(dev || !Z ? 1 : plen), o_al = ar.take<double2>(dev ? 1 : wlen),
               o_be = ar.take<double>(dev ? 1 : wlen), o_st = ar.take<int>(count);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  QzrBatch bt;
  bt.count = (int)count;
  bt.scale = (flags & GS_SCALE) ? 1 : 0;
  bt.n1 = single;
  if (dev) {
    bt.ns = single ? nullptr : ns;
    bt.offs = (const long long*)offs;
    bt.woffs = (const long long*)woffs;
    bt.A = A; bt.B = B; bt.Q = Q; bt.Z = Z;
    bt.alpha = (double2*)alpha; bt.beta = beta;
    bt.status = status ? (int*)status : (int*)(base + o_st);
  } else {
    if (!single) {
      CK(cudaMemcpyAsync(base + o_ns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(base + o_off, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(base + o_woff, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(base + o_A, A, sizeof(double) * plen, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_B, B, sizeof(double) * plen, cudaMemcpyHostToDevice, s));
    bt.ns = single ? nullptr : (const int*)(base + o_ns);
    bt.offs = (const long long*)(base + o_off);
    bt.woffs = (const long long*)(base + o_woff);
    bt.A = (double*)(base + o_A); bt.B = (double*)(base + o_B);
    bt.Q = Q ? (double*)(base + o_Q) : nullptr; bt.Z = Z ? (double*)(base + o_Z) : nullptr;
    bt.alpha = (double2*)(base + o_al); bt.beta = (double*)(base + o_be);
    bt.status = (int*)(base + o_st);
  }
  CK(cudaEventRecord(ctx->t0, s));
  CK(launch_ggschur_real(bt, ctx->num_sms, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  std::vector<int> st(count);
  CK(cudaMemcpyAsync(st.data(), bt.status, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
  if (!dev) {
    CK(cudaMemcpyAsync(A, bt.A, sizeof(double) * plen, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(B, bt.B, sizeof(double) * plen, cudaMemcpyDeviceToHost, s));
    if (Q) CK(cudaMemcpyAsync(Q, bt.Q, sizeof(double) * plen, cudaMemcpyDeviceToHost, s));
    if (Z) CK(cudaMemcpyAsync(Z, bt.Z, sizeof(double) * plen, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(alpha, bt.alpha, sizeof(double2) * wlen, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(beta, bt.beta, sizeof(double) * wlen, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (status && !dev) std::memcpy(status, st.data(), sizeof(int) * count);
  for (int64_t b = 0; b < count; ++b)
    if (st[b]) return set_err(ctx, GS_UNCONVERGED, "pencil %lld: iteration limit reached", (long long)b);
  return GS_OK;
}

int ggschur_batched_impl(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs, int64_t plen,
                         double* A, double* B, double* Q, double* Z, const int64_t* woffs, int64_t wlen, double* alpha,
                         double* beta, int32_t* status, unsigned flags, int single = 0) {
  if (!ctx) return GS_BADARG;
  ctx->err.clear();
  if (count < 0 || plen < 0 || wlen < 0) return set_err(ctx, GS_BADARG, "negative size");
  if (count == 0) return GS_OK;
  if ((!single && (!ns || !offs || !woffs)) || !A || !B || !alpha || !beta)
    return set_err(ctx, GS_BADARG, "null array argument");
  const bool dev = flags & GS_DEVICE;
  if (!dev && !single) {
    for (int64_t b = 0; b < count; ++b) {
      const int64_t n = ns[b];
      if (n < 0 || n > 4096 || offs[b] < 0 || offs[b] + n * n > plen || woffs[b] < 0 || woffs[b] + n > wlen)
        return set_err(ctx, GS_BADARG, "pencil %lld: order or offsets out of range", (long long)b);
    }
  }
  CK(cudaSetDevice(ctx->device));
  const size_t zb = sizeof(double2);
  Arena ar;
  const size_t o_ns = ar.take<int>(dev ? 1 : count), o_off = ar.take<long long>(dev ? 1 : count),
               o_woff = ar.take<long long>(dev ? 1 : count), o_A = ar.take<double2>(dev ? 1 : plen),
               o_B = ar.take<double2>(dev ? 1 : plen), o_Q = ar.take<double2>(dev || !Q ? 1 : plen),
               o_Z = ar.take<double2>(dev || !Z ? 1 : plen), o_al = ar.take<double2>(dev ? 1 : wlen),
               o_be = ar.take<double2>(dev ? 1 : wlen), o_st = ar.take<int>(count);
  int rc = ensure_ws(ctx, ar.off);
  if (rc) return rc;
  char* base = ctx->dws;
  cudaStream_t s = ctx->stream;
  QzBatch bt;
  bt.count = (int)count;
  bt.scale = (flags & GS_SCALE) ? 1 : 0;
  bt.n1 = single;
  if (dev) {
    bt.ns = single ? nullptr : ns;
    bt.offs = (const long long*)offs;
    bt.woffs = (const long long*)woffs;
    bt.A = (double2*)A; bt.B = (double2*)B; bt.Q = (double2*)Q; bt.Z = (double2*)Z;
    bt.alpha = (double2*)alpha; bt.beta = (double2*)beta;
    bt.status = status ? (int*)status : (int*)(base + o_st);
  } else {
    if (!single) {
      CK(cudaMemcpyAsync(base + o_ns, ns, sizeof(int) * count, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(base + o_off, offs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(base + o_woff, woffs, sizeof(long long) * count, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(base + o_A, A, zb * plen, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_B, B, zb * plen, cudaMemcpyHostToDevice, s));
    bt.ns = single ? nullptr : (const int*)(base + o_ns);
    bt.offs = (const long long*)(base + o_off);
    bt.woffs = (const long long*)(base + o_woff);
    bt.A = (double2*)(base + o_A); bt.B = (double2*)(base + o_B);
    bt.Q = Q ? (double2*)(base + o_Q) : nullptr; bt.Z = Z ? (double2*)(base + o_Z) : nullptr;
    bt.alpha = (double2*)(base + o_al); bt.beta = (double2*)(base + o_be);
    bt.status = (int*)(base + o_st);
  }
  CK(cudaEventRecord(ctx->t0, s));
  CK(launch_ggschur(bt, ctx->num_sms, s));
  CK(cudaEventRecord(ctx->t1, s));
  ctx->timed = true;
  std::vector<int> st(count);
  CK(cudaMemcpyAsync(st.data(), bt.status, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
  if (!dev) {
    CK(cudaMemcpyAsync(A, bt.A, zb * plen, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(B, bt.B, zb * plen, cudaMemcpyDeviceToHost, s));
    if (Q) CK(cudaMemcpyAsync(Q, bt.Q, zb * plen, cudaMemcpyDeviceToHost, s));
    if (Z) CK(cudaMemcpyAsync(Z, bt.Z, zb * plen, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(alpha, bt.alpha, zb * wlen, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(beta, bt.beta, zb * wlen, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (status && !dev) std::memcpy(status, st.data(), sizeof(int) * count);
  for (int64_t b = 0; b < count; ++b)
    if (st[b]) return set_err(ctx, GS_UNCONVERGED, "pencil %lld: iteration limit reached", (long long)b);
  return GS_OK;
}

}  // namespace

extern "C" {

int gs_ggschur_batched_c64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs, int64_t packed_len,
                           double* A, double* B, double* Q, double* Z, const int64_t* woffs, int64_t wlen,
                           double* alpha, double* beta, int32_t* status, unsigned flags) {
  return ggschur_batched_impl(ctx, count, ns, offs, packed_len, A, B, Q, Z, woffs, wlen, alpha, beta, status, flags);
}

int gs_ggschur_f64(gs_context* ctx, int64_t n, double* A, double* B, double* Q, double* Z, double* alpha, double* beta,
                   unsigned flags) {
  if (!ctx) return GS_BADARG;
  if (n < 0 || n > 4096) return set_err(ctx, GS_BADARG, "bad order");
  if (n == 0) return GS_OK;
  return ggschur_real_impl(ctx, 1, nullptr, nullptr, n * n, A, B, Q, Z, nullptr, n, alpha, beta, nullptr, flags,
                           (int)n);
}

int gs_ggschur_batched_f64(gs_context* ctx, int64_t count, const int32_t* ns, const int64_t* offs, int64_t packed_len,
                           double* A, double* B, double* Q, double* Z, const int64_t* woffs, int64_t wlen,
                           double* alpha, double* beta, int32_t* status, unsigned flags) {
  const int rc = ggschur_real_impl(ctx, count, ns, offs, packed_len, A, B, Q, Z, woffs, wlen, alpha, beta, status,
                                   flags);
  return rc;
}

int gs_ggschur_c64(gs_context* ctx, int64_t n, double* A, double* B, double* Q, double* Z, double* alpha, double* beta,
                   unsigned flags) {
  if (!ctx) return GS_BADARG;
  if (n < 0 || n > 4096) return set_err(ctx, GS_BADARG, "bad order");
  if (n == 0) return GS_OK;
  return ggschur_batched_impl(ctx, 1, nullptr, nullptr, n * n, A, B, Q, Z, nullptr, n, alpha, beta, nullptr, flags,
                              (int)n);
}

}  // extern "C"
