// Runtime plumbing for the GB300 octree library: the per-handle context
// (stream, device error word, scratch counters), stream-ordered device
// buffers and error propagation.  Every C-ABI entry point runs on the
// context's stream; a context is used by one host thread at a time.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <exception>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "dg_common.cuh"

namespace dg {

// per-kernel timing (enabled by dg_ctx_profile): CUDA events around the
// launches on the context's stream, resolved when an API call completes
struct ProfStat {
  double ms = 0.0;
  uint64_t launches = 0;
  double bytes = 0.0;  // algorithmic bytes moved by those launches
};
struct ProfPending {
  std::string name;
  cudaEvent_t a, b;
  double bytes;
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // a second stream and two events for work that overlaps the main
  // stream's (the coarse inverse's look-ahead), created on first use
  cudaStream_t side = nullptr;
  cudaEvent_t side_ev[2] = {nullptr, nullptr};
  uint32_t *d_flags = nullptr;     // device error bitmask (DGF_*)
  unsigned long long *d_scratch = nullptr;  // small device counters
  unsigned long long *h_scratch = nullptr;  // pinned mirror of d_scratch
  int num_sms = 0;
  std::string last_error;
  // stencil tables (FP64 and FP32) on the device, created on first use
  double *d_sten64 = nullptr;
  float *d_sten32 = nullptr;
  uint8_t *d_etype_of = nullptr;   // [8][256] -> element type or 255
  uint8_t *d_etype_mask = nullptr; // [8][18] -> hanging mask
  double *d_csten64 = nullptr;     // canonical full stencils, 18 types (dg_elem.cuh)
  float *d_csten32 = nullptr;
  uint32_t *d_cperm = nullptr;     // [8][18] vertex relabelling, 3 bits each
  // combined stencils lapf 2^-l/2 L_t + massf 2^-3l/8 M_t per (type, level)
  // for the factors of the last element loop (dg_elem.cuh, comb_table)
  double *d_comb64 = nullptr;
  float *d_comb32 = nullptr;
  double comb64_f[2] = {0, 0}, comb32_f[2] = {0, 0};
  bool comb64_ok = false, comb32_ok = false;
  // the FP64 combined stencils as (hi, lo) FP32 pairs, two rows per float4
  // (double-single loop)
  float4 *d_comb_ds = nullptr;
  float *d_comb_rowabs = nullptr;  // per (type, level): largest row sum of |combined stencil entries|
  double comb_ds_f[2] = {0, 0};
  bool comb_ds_ok = false;
  bool prof = false;
  std::map<std::string, ProfStat> prof_stats;
  std::vector<ProfPending> prof_pending;
  std::vector<cudaEvent_t> prof_pool;
  // autotuner: the radix sort's launch shape per (key width: 0 = 8 bytes,
  // 1 = 16 bytes, log2 of the key count); items == 0: not tuned yet
  struct Tune {
    int items = 0;     // keys per thread of a onesweep tile
    int minb = 0;      // onesweep blocks per SM the kernel is compiled for
    int hist_mul = 0;  // digit-histogram blocks per SM
  } tune[2][64];
  std::string tune_log;  // one line per decision
  // order of octant records at the boundary (downloads, uploads, files):
  // 0 Morton, 1 Hilbert (the reference's HILBERT_ORDERING builds); the
  // octrees themselves are always kept in Morton order on the device
  int order = 0;
  // FP32 element loop form: 0 the run form where the mesh has its tables,
  // 1 the pair form (dg_ctx_set_matvec_form)
  int matvec_form = 0;
};

// thrown inside the library, converted to a status code at the C ABI
struct Error {
  int code;
  std::string msg;
};

[[noreturn]] inline void fail(int code, const std::string &msg) { throw Error{code, msg}; }

inline void check_cuda(cudaError_t e, const char *what, const char *file, int line) {
  if (e != cudaSuccess) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    fail(e == cudaErrorMemoryAllocation ? DG_ERR_OUT_OF_MEMORY : DG_ERR_CUDA, buf);
  }
}
#define DG_CUDA(call) ::dg::check_cuda((call), #call, __FILE__, __LINE__)
#define DG_LAUNCH_CHECK() ::dg::check_cuda(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

// Stream-ordered device buffer (cudaMallocAsync from the device's default
// pool; the pool keeps freed blocks for reuse by later calls).
template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(size_t count, cudaStream_t stream) { alloc(count, stream); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n), s(o.s) {
    o.p = nullptr;
    o.n = 0;
  }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      s = o.s;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  void alloc(size_t count, cudaStream_t stream) {
    release();
    s = stream;
    n = count;
    if (count) DG_CUDA(cudaMallocAsync((void **)&p, count * sizeof(T), stream));
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
  T *get() const { return p; }
  T *release_ptr() {
    T *q = p;
    p = nullptr;
    n = 0;
    return q;
  }
  // take ownership of a stream-ordered allocation
  void adopt(T *q, size_t count, cudaStream_t stream) {
    release();
    p = q;
    n = count;
    s = stream;
  }
};

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per (device,
// kernel): the attribute belongs to each device's context
template <typename F>
void ensure_smem_attr(const Context &ctx, F *kernel, int bytes) {
  static std::mutex mu;
  static std::set<std::pair<int, const void *>> done;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_pair(ctx.device, reinterpret_cast<const void *>(kernel));
  if (done.count(key)) return;
  DG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.insert(key);
}

inline unsigned grid_for(size_t n, unsigned block, unsigned max_blocks = 1u << 30) {
  size_t g = (n + block - 1) / block;
  if (g == 0) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (unsigned)g;
}

// synchronously read one small device value through the pinned mirror
template <typename T>
inline T read_scalar(Context &ctx, const T *dptr) {
  DG_CUDA(cudaMemcpyAsync(ctx.h_scratch, dptr, sizeof(T), cudaMemcpyDeviceToHost, ctx.stream));
  DG_CUDA(cudaStreamSynchronize(ctx.stream));
  T v;
  std::memcpy(&v, ctx.h_scratch, sizeof(T));
  return v;
}

inline cudaEvent_t prof_event(Context &c) {
  if (!c.prof_pool.empty()) {
    cudaEvent_t e = c.prof_pool.back();
    c.prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  DG_CUDA(cudaEventCreate(&e));
  return e;
}

// the context of the C-ABI call running on this thread (for primitives
// that only receive a stream)
inline Context *&current_context() {
  static thread_local Context *c = nullptr;
  return c;
}

// RAII timing scope around one kernel launch (no-op unless profiling)
struct ProfScope {
  Context *c = nullptr;
  cudaEvent_t a = nullptr;
  const char *name;
  double bytes;
  ProfScope(Context &ctx, const char *nm, double b) : name(nm), bytes(b) { start(&ctx); }
  ProfScope(const char *nm, double b) : name(nm), bytes(b) { start(current_context()); }
  void start(Context *ctx) {
    if (!ctx || !ctx->prof) return;
    c = ctx;
    a = prof_event(*ctx);
    cudaEventRecord(a, ctx->stream);
  }
  ~ProfScope() {
    if (!c) return;
    cudaEvent_t b = nullptr;
    try {
      b = prof_event(*c);
    } catch (...) {
      return;
    }
    cudaEventRecord(b, c->stream);
    c->prof_pending.push_back(ProfPending{name, a, b, bytes});
  }
};

// fold completed timing events into the statistics (stream must be idle)
inline void prof_resolve(Context &c) {
  for (auto &p : c.prof_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      ProfStat &st = c.prof_stats[p.name];
      st.ms += ms;
      st.launches += 1;
      st.bytes += p.bytes;
    }
    c.prof_pool.push_back(p.a);
    c.prof_pool.push_back(p.b);
  }
  c.prof_pending.clear();
}

// A CUDA graph captured from the launches a function makes on one stream,
// then replayed with cudaGraphLaunch.  capture() records in thread-local
// mode (other host threads keep launching on their own streams); a failure
// to capture or instantiate leaves exec null, and the caller launches the
// work directly instead.
struct CudaGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  CudaGraph() = default;
  CudaGraph(const CudaGraph &) = delete;
  CudaGraph &operator=(const CudaGraph &) = delete;
  ~CudaGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
  template <typename F>
  void capture(cudaStream_t s, F &&work) {
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    std::exception_ptr failed;
    try {
      work();
    } catch (...) {
      failed = std::current_exception();
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(s, &g) != cudaSuccess || failed) {
      cudaGetLastError();
      if (g) cudaGraphDestroy(g);
      if (failed) std::rethrow_exception(failed);  // the work itself failed: report it as the eager path would
      return;
    }
    graph = g;
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
      cudaGetLastError();
      exec = nullptr;
    }
  }
};

// read and clear the device error word; throw on any flag
void check_device_flags(Context &ctx, const char *where);

// Persistent autotuner decisions, shared by the contexts of a process and
// kept on disk between processes, keyed by the device (name, SM count,
// compute capability) and the size class.  The file is
// $DENDRO_GB300_TUNE_CACHE when set (an empty value turns the disk cache
// off), else $XDG_CACHE_HOME/dendro_gb300/autotune.tsv or
// $HOME/.cache/dendro_gb300/autotune.tsv.  I/O failures only lose the cache.
bool tune_cache_get(int device, int width, int bucket, Context::Tune *out);
void tune_cache_put(int device, int width, int bucket, const Context::Tune &t);
std::string tune_cache_path();

}  // namespace dg
