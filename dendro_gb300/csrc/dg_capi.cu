// C ABI (include/dendro_gb300.h) over the device pipelines.
#include <cuda_runtime.h>

#include <cstdio>
#include <exception>
#include <iterator>
#include <functional>
#include <new>
#include <string>

#include "dendro_gb300.h"
#include "dg_assemble.cuh"
#include "dg_io.cuh"
#include "dg_mg.cuh"

struct dg_ctx_s {
  dg::Context c;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
};
struct dg_octree_s {
  dg::Octree o;
};
struct dg_da_s {
  dg::Mesh m;
};
struct dg_mg_s {
  dg::MG mg;
};
struct dg_csr_s {
  dg::Csr c;
};

namespace {

template <typename F>
int guarded(dg_ctx ctx, F &&f) {
  if (!ctx) return DG_ERR_INVALID_ARG;
  struct CurrentCtx {
    CurrentCtx(dg::Context *c) { dg::current_context() = c; }
    ~CurrentCtx() { dg::current_context() = nullptr; }
  } current(&ctx->c);
  try {
    DG_CUDA(cudaSetDevice(ctx->c.device));
    DG_CUDA(cudaEventRecord(ctx->ev0, ctx->c.stream));
    f();
    DG_CUDA(cudaEventRecord(ctx->ev1, ctx->c.stream));
    DG_CUDA(cudaEventSynchronize(ctx->ev1));
    dg::prof_resolve(ctx->c);
    float ms = 0.f;
    DG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->c.last_error.clear();
    return DG_OK;
  } catch (const dg::Error &e) {
    ctx->c.last_error = e.msg;
    cudaStreamSynchronize(ctx->c.stream);
    return e.code;
  } catch (const std::bad_alloc &) {
    ctx->c.last_error = "host allocation failed";
    return DG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    ctx->c.last_error = e.what();
    return DG_ERR_INTERNAL;
  }
}

template <typename F>
int read_octree_file(dg_ctx ctx, dg_octree *out, F &&reader) {
  if (!out) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() { reader(h->o); });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

// device copy of a host (or device) input array
template <typename T>
const T *device_input(dg::Context &c, const T *p, size_t n, int on_device, dg::DBuf<T> &hold) {
  if (on_device || n == 0) return p;
  hold.alloc(n, c.stream);
  DG_CUDA(cudaMemcpyAsync(hold.get(), p, n * sizeof(T), cudaMemcpyHostToDevice, c.stream));
  return hold.get();
}

template <typename T>
void copy_out(dg::Context &c, T *dst, const T *src, size_t n, int dst_on_device) {
  if (!n) return;
  DG_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          c.stream));
}

int csr_handle(dg_ctx ctx, dg_csr *out, const std::function<void(dg::Csr &)> &make) {
  if (!out) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_csr h = new (std::nothrow) dg_csr_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() { make(h->c); });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}
}  // namespace

extern "C" {

int dg_version(void) { return 1; }

const char *dg_status_string(int s) {
  switch (s) {
    case DG_OK: return "ok";
    case DG_ERR_INVALID_ARG: return "invalid argument";
    case DG_ERR_OUT_OF_MEMORY: return "out of device memory";
    case DG_ERR_CUDA: return "CUDA error";
    case DG_ERR_DOMAIN: return "point outside the domain";
    case DG_ERR_NOT_BALANCED: return "octree is not complete and 2:1 balanced";
    case DG_ERR_TIMEOUT: return "device wait timed out";
    case DG_ERR_INTERNAL: return "internal error";
    case DG_ERR_COMM_SIZE: return "communicator size must be 1";
    case DG_ERR_UNSUPPORTED: return "unsupported option";
    case DG_ERR_CAPACITY: return "input larger than the fixed capacity of a no-allocation entry point";
    default: return "unknown status";
  }
}

int dg_ctx_create(int device, dg_ctx *out) {
  if (!out) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_ctx ctx = new (std::nothrow) dg_ctx_s();
  if (!ctx) return DG_ERR_OUT_OF_MEMORY;
  ctx->c.device = device;
  try {
    DG_CUDA(cudaSetDevice(device));
    DG_CUDA(cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking));
    ctx->c.own_stream = true;
    DG_CUDA(cudaMalloc((void **)&ctx->c.d_flags, sizeof(uint32_t)));
    DG_CUDA(cudaMemset(ctx->c.d_flags, 0, sizeof(uint32_t)));
    DG_CUDA(cudaMalloc((void **)&ctx->c.d_scratch, 64 * sizeof(unsigned long long)));
    DG_CUDA(cudaMallocHost((void **)&ctx->c.h_scratch, 64 * sizeof(unsigned long long)));
    DG_CUDA(cudaDeviceGetAttribute(&ctx->c.num_sms, cudaDevAttrMultiProcessorCount, device));
    DG_CUDA(cudaEventCreate(&ctx->ev0));
    DG_CUDA(cudaEventCreate(&ctx->ev1));
    // keep freed blocks in this process's pool between calls
    cudaMemPool_t pool;
    DG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t thr = ~0ull;
    DG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  } catch (const dg::Error &e) {
    int code = e.code;
    dg_ctx_destroy(ctx);
    return code;
  }
  *out = ctx;
  return DG_OK;
}

int dg_ctx_destroy(dg_ctx ctx) {
  if (!ctx) return DG_ERR_INVALID_ARG;
  cudaSetDevice(ctx->c.device);
  if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
  if (ctx->c.d_flags) cudaFree(ctx->c.d_flags);
  if (ctx->c.d_scratch) cudaFree(ctx->c.d_scratch);
  if (ctx->c.h_scratch) cudaFreeHost(ctx->c.h_scratch);
  if (ctx->c.d_sten64) cudaFree(ctx->c.d_sten64);
  if (ctx->c.d_sten32) cudaFree(ctx->c.d_sten32);
  if (ctx->c.d_comb64) cudaFree(ctx->c.d_comb64);
  if (ctx->c.d_comb32) cudaFree(ctx->c.d_comb32);
  if (ctx->c.d_comb_ds) cudaFree(ctx->c.d_comb_ds);
  if (ctx->c.d_comb_rowabs) cudaFree(ctx->c.d_comb_rowabs);
  if (ctx->c.d_csten64) cudaFree(ctx->c.d_csten64);
  if (ctx->c.d_csten32) cudaFree(ctx->c.d_csten32);
  if (ctx->c.d_cperm) cudaFree(ctx->c.d_cperm);
  if (ctx->c.d_etype_of) cudaFree(ctx->c.d_etype_of);
  if (ctx->c.d_etype_mask) cudaFree(ctx->c.d_etype_mask);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->c.side_ev[0]) cudaEventDestroy(ctx->c.side_ev[0]);
  if (ctx->c.side_ev[1]) cudaEventDestroy(ctx->c.side_ev[1]);
  if (ctx->c.side) cudaStreamDestroy(ctx->c.side);
  if (ctx->c.own_stream && ctx->c.stream) cudaStreamDestroy(ctx->c.stream);
  delete ctx;
  return DG_OK;
}

int dg_ctx_set_stream(dg_ctx ctx, void *stream) {
  if (!ctx) return DG_ERR_INVALID_ARG;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  if (stream) {
    if (ctx->c.own_stream) cudaStreamDestroy(ctx->c.stream);
    ctx->c.own_stream = false;
    ctx->c.stream = (cudaStream_t)stream;
  } else if (!ctx->c.own_stream) {
    if (cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking) != cudaSuccess) return DG_ERR_CUDA;
    ctx->c.own_stream = true;
  }
  return DG_OK;
}

const char *dg_ctx_last_error(dg_ctx ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

int dg_ctx_last_device_ms(dg_ctx ctx, double *ms) {
  if (!ctx || !ms) return DG_ERR_INVALID_ARG;
  *ms = ctx->last_ms;
  return DG_OK;
}

int dg_ctx_profile(dg_ctx ctx, int enable) {
  if (!ctx) return DG_ERR_INVALID_ARG;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  dg::prof_resolve(ctx->c);
  ctx->c.prof_stats.clear();
  ctx->c.prof = enable != 0;
  return DG_OK;
}

int dg_ctx_profile_count(dg_ctx ctx, int *count) {
  if (!ctx || !count) return DG_ERR_INVALID_ARG;
  *count = (int)ctx->c.prof_stats.size();
  return DG_OK;
}

int dg_ctx_profile_entry(dg_ctx ctx, int index, char *name, size_t name_len, double *total_ms,
                         unsigned long long *launches, double *bytes) {
  if (!ctx || index < 0 || index >= (int)ctx->c.prof_stats.size()) return DG_ERR_INVALID_ARG;
  auto it = ctx->c.prof_stats.begin();
  std::advance(it, index);
  if (name && name_len) {
    std::snprintf(name, name_len, "%s", it->first.c_str());
  }
  if (total_ms) *total_ms = it->second.ms;
  if (launches) *launches = it->second.launches;
  if (bytes) *bytes = it->second.bytes;
  return DG_OK;
}

int dg_ctx_set_matvec_form(dg_ctx ctx, int form) {
  if (!ctx || (form != 0 && form != 1)) return DG_ERR_INVALID_ARG;
  ctx->c.matvec_form = form;
  return DG_OK;
}

int dg_dense_spd_inverse(dg_ctx ctx, float *X, size_t n) {
  if (!X && n) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    if (n > 20000) dg::fail(DG_ERR_INVALID_ARG, "dense inverse: at most 20000 rows");
    dg::coarse_inverse(ctx->c, X, n);
    dg::check_device_flags(ctx->c, "dense inverse");
  });
}

int dg_debug_lookback_timeout(dg_ctx ctx, size_t n_keys, unsigned skipped_tiles) {
  return guarded(ctx, [&]() { dg::lookback_timeout_selftest(ctx->c, n_keys, skipped_tiles); });
}

int dg_points_to_octree(dg_ctx ctx, const double *xyz, size_t n, const double gLens[3], unsigned maxDepth,
                        unsigned maxNumPts, int comm_size, int xyz_on_device, dg_octree *out) {
  if (!out || (!xyz && n) || !gLens) return DG_ERR_INVALID_ARG;
  if (comm_size != 1) return DG_ERR_COMM_SIZE;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() {
    if (!(gLens[0] > 0 && gLens[1] > 0 && gLens[2] > 0)) dg::fail(DG_ERR_INVALID_ARG, "gLens must be positive");
    dg::DBuf<double> hold;
    const double *d = device_input(ctx->c, xyz, 3 * n, xyz_on_device, hold);
    dg::points_to_octree(ctx->c, d, n, gLens, maxDepth, maxNumPts, h->o);
  });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_points_to_octree_batch(dg_ctx ctx, const double *xyz, size_t n, const uint64_t *seg_start, size_t nseg,
                              const double gLens[3], unsigned maxDepth, unsigned maxNumPts, int xyz_on_device,
                              dg_octree *out) {
  if (!out || (!xyz && n) || !gLens || !seg_start || nseg == 0) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() {
    if (!(gLens[0] > 0 && gLens[1] > 0 && gLens[2] > 0)) dg::fail(DG_ERR_INVALID_ARG, "gLens must be positive");
    dg::DBuf<double> hold;
    const double *d = device_input(ctx->c, xyz, 3 * n, xyz_on_device, hold);
    dg::points_to_octree(ctx->c, d, n, gLens, maxDepth, maxNumPts, h->o, seg_start, nseg);
  });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_octree_segments(dg_ctx ctx, dg_octree o, size_t *nseg, uint64_t *offsets) {
  if (!o) return DG_ERR_INVALID_ARG;
  if (nseg) *nseg = o->o.nseg;
  if (!offsets) return DG_OK;
  return guarded(ctx, [&]() { dg::octree_segment_offsets(ctx->c, o->o, offsets); });
}

int dg_octree_extract(dg_ctx ctx, dg_octree o, size_t seg, dg_octree *out) {
  if (!o || !out) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() { dg::octree_extract(ctx->c, o->o, seg, h->o); });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_sort_unique_points(dg_ctx ctx, const double *xyz, size_t n, const double gLens[3], unsigned maxDepth,
                          int xyz_on_device, uint32_t *out_xyzl, int out_on_device, size_t *n_unique) {
  if ((!xyz && n) || !gLens || !n_unique || (!out_xyzl && n)) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    if (maxDepth > 30) dg::fail(DG_ERR_INVALID_ARG, "maxDepth must be <= 30");
    dg::DBuf<double> hold;
    const double *d = device_input(ctx->c, xyz, 3 * n, xyz_on_device, hold);
    dg::DBuf<dg::Key128> uk(n ? n : 1, ctx->c.stream);
    bool dups = false;
    size_t nu = dg::sort_points(ctx->c, d, n, gLens, maxDepth, uk.get(), &dups);
    dg::Octree tmp;
    tmp.max_depth = maxDepth;
    tmp.n = nu;
    tmp.keys = uk.get();
    if (out_on_device) {
      dg::octree_to_xyzl(ctx->c, tmp, out_xyzl);
    } else {
      dg::DBuf<uint32_t> dx(4 * (nu ? nu : 1), ctx->c.stream);
      dg::octree_to_xyzl(ctx->c, tmp, dx.get());
      copy_out(ctx->c, out_xyzl, dx.get(), 4 * nu, 0);
      DG_CUDA(cudaStreamSynchronize(ctx->c.stream));
    }
    *n_unique = nu;
  });
}

int dg_balance_octree(dg_ctx ctx, dg_octree in, int incCorner, int comm_size, dg_octree *out) {
  if (!in || !out) return DG_ERR_INVALID_ARG;
  if (comm_size != 1) return DG_ERR_COMM_SIZE;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() { dg::balance_octree(ctx->c, in->o, h->o, incCorner != 0); });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_coarsen_octree(dg_ctx ctx, dg_octree in, dg_octree *out) {
  if (!in || !out) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() { dg::coarsen_octree(ctx->c, in->o, h->o); });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_octree_size(dg_octree o, size_t *n, unsigned *maxDepth) {
  if (!o) return DG_ERR_INVALID_ARG;
  if (n) *n = o->o.n;
  if (maxDepth) *maxDepth = o->o.max_depth;
  return DG_OK;
}

int dg_octree_download(dg_ctx ctx, dg_octree o, uint32_t *xyzl, int dst_on_device) {
  if (!o || (!xyzl && o->o.n)) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    if (dst_on_device) {
      dg::octree_to_xyzl(ctx->c, o->o, xyzl);
    } else {
      dg::DBuf<uint32_t> dx(4 * (o->o.n ? o->o.n : 1), ctx->c.stream);
      dg::octree_to_xyzl(ctx->c, o->o, dx.get());
      copy_out(ctx->c, xyzl, dx.get(), 4 * o->o.n, 0);
    }
  });
}

int dg_octree_upload(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, int src_on_device, dg_octree *out) {
  if (!out || (!xyzl && n) || maxDepth > 30) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() {
    dg::DBuf<uint32_t> hold;
    const uint32_t *d = device_input(ctx->c, xyzl, 4 * n, src_on_device, hold);
    dg::octree_from_xyzl(ctx->c, d, n, maxDepth, h->o);
  });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_sort_octants(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, int removeDuplicates,
                    int src_on_device, uint32_t *out_xyzl, int dst_on_device, size_t *n_out) {
  if ((!xyzl && n) || (!out_xyzl && n) || !n_out || maxDepth > 30) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    dg::DBuf<uint32_t> hold;
    const uint32_t *d = device_input(c, xyzl, 4 * n, src_on_device, hold);
    dg::Octree o;
    dg::sort_octants(c, d, n, maxDepth, removeDuplicates != 0 ? 1 : 0, o);
    dg::DBuf<dg::Key128> own;
    own.adopt(o.keys, o.n, c.stream);  // freed on return
    if (dst_on_device) {
      dg::octree_to_xyzl(c, o, out_xyzl);
    } else if (o.n) {
      dg::DBuf<uint32_t> dx(4 * o.n, c.stream);
      dg::octree_to_xyzl(c, o, dx.get());
      copy_out(c, out_xyzl, dx.get(), 4 * o.n, 0);
    }
    DG_CUDA(cudaStreamSynchronize(c.stream));
    *n_out = o.n;
  });
}

int dg_tree_sort(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, unsigned options, int src_on_device,
                 uint32_t *out_xyzl, int dst_on_device, size_t *n_out) {
  if ((!xyzl && n) || (!out_xyzl && n) || !n_out || maxDepth > 30) return DG_ERR_INVALID_ARG;
  if (options & (DG_TS_CONSTRUCT_OCTREE | DG_TS_BALANCE_OCTREE)) {
    if (ctx) ctx->c.last_error = "SFC_treeSort: construct / balance options: use dg_complete_octree / dg_balance_octree";
    return DG_ERR_UNSUPPORTED;
  }
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    dg::DBuf<uint32_t> hold;
    const uint32_t *d = device_input(c, xyzl, 4 * n, src_on_device, hold);
    dg::Octree o;
    dg::sort_octants(c, d, n, maxDepth, (options & DG_TS_REMOVE_DUPLICATES) ? 2 : 0, o);
    dg::DBuf<dg::Key128> own;
    own.adopt(o.keys, o.n, c.stream);  // freed on return
    if (dst_on_device) {
      dg::octree_to_xyzl(c, o, out_xyzl);
    } else if (o.n) {
      dg::DBuf<uint32_t> dx(4 * o.n, c.stream);
      dg::octree_to_xyzl(c, o, dx.get());
      copy_out(c, out_xyzl, dx.get(), 4 * o.n, 0);
    }
    DG_CUDA(cudaStreamSynchronize(c.stream));
    *n_out = o.n;
  });
}

int dg_complete_octree(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, int isUnique, int isSorted,
                       int src_on_device, dg_octree *out) {
  if (!out || (!xyzl && n) || maxDepth > 30) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_octree h = new (std::nothrow) dg_octree_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() {
    dg::DBuf<uint32_t> hold;
    const uint32_t *d = device_input(ctx->c, xyzl, 4 * n, src_on_device, hold);
    dg::complete_octree(ctx->c, d, n, maxDepth, isUnique != 0, isSorted != 0, h->o);
  });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

const char *dg_ctx_autotune_log(dg_ctx ctx) { return ctx ? ctx->c.tune_log.c_str() : ""; }

int dg_ctx_set_order(dg_ctx ctx, int order) {
  if (!ctx || (order != DG_ORDER_MORTON && order != DG_ORDER_HILBERT)) return DG_ERR_INVALID_ARG;
  ctx->c.order = order;
  return DG_OK;
}

int dg_ctx_get_order(dg_ctx ctx, int *order) {
  if (!ctx || !order) return DG_ERR_INVALID_ARG;
  *order = ctx->c.order;
  return DG_OK;
}

int dg_pts_file_count(const char *path, size_t *n) {
  if (!path || !n) return DG_ERR_INVALID_ARG;
  try {
    *n = dg::pts_file_count(path);
  } catch (const dg::Error &e) {
    return e.code;
  }
  return DG_OK;
}

int dg_pts_file_read(dg_ctx ctx, const char *path, double *xyz, size_t capacity, int dst_on_device, size_t *n) {
  if (!path || !n || (!xyz && capacity)) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() { *n = dg::pts_file_read(ctx->c, path, xyz, capacity, dst_on_device != 0); });
}

int dg_pts_file_write(dg_ctx ctx, const char *path, const double *xyz, size_t n, int src_on_device) {
  if (!path || (!xyz && n)) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() { dg::pts_file_write(ctx->c, path, xyz, n, src_on_device != 0); });
}

int dg_octree_write_text(dg_ctx ctx, dg_octree o, const char *path) {
  if (!o || !path) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() { dg::octree_write_text(ctx->c, o->o, path); });
}

int dg_octree_write_binary(dg_ctx ctx, dg_octree o, const char *path) {
  if (!o || !path) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() { dg::octree_write_binary(ctx->c, o->o, path); });
}

int dg_octree_read_text(dg_ctx ctx, const char *path, dg_octree *out) {
  if (!path) return DG_ERR_INVALID_ARG;
  return read_octree_file(ctx, out, [&](dg::Octree &o) { dg::octree_read_text(ctx->c, path, o); });
}

int dg_octree_read_binary(dg_ctx ctx, const char *path, dg_octree *out) {
  if (!path) return DG_ERR_INVALID_ARG;
  return read_octree_file(ctx, out, [&](dg::Octree &o) { dg::octree_read_binary(ctx->c, path, o); });
}

int dg_octree_free(dg_ctx ctx, dg_octree o) {
  if (!ctx || !o) return DG_ERR_INVALID_ARG;
  cudaSetDevice(ctx->c.device);
  dg::octree_free(ctx->c, o->o);
  cudaStreamSynchronize(ctx->c.stream);
  delete o;
  return DG_OK;
}

int dg_da_build(dg_ctx ctx, dg_octree balanced, dg_da *out) { return dg_da_build_ex(ctx, balanced, 0, out); }

int dg_da_build_ex(dg_ctx ctx, dg_octree balanced, int compressLut, dg_da *out) {
  if (!balanced || !out) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_da h = new (std::nothrow) dg_da_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() {
    if (balanced->o.nseg != 1) dg::fail(DG_ERR_UNSUPPORTED, "DA: one cloud per mesh");
    dg::mesh_build(ctx->c, balanced->o, h->m, compressLut != 0);
  });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_da_memory(dg_da da, size_t *bytes) {
  if (!da || !bytes) return DG_ERR_INVALID_ARG;
  *bytes = dg::mesh_bytes(da->m);
  return DG_OK;
}

int dg_da_sizes(dg_da da, size_t *n_elem, size_t *n_node) {
  if (!da) return DG_ERR_INVALID_ARG;
  if (n_elem) *n_elem = da->m.n_elem;
  if (n_node) *n_node = da->m.n_node;
  return DG_OK;
}

namespace {
__global__ void k_transpose_conn(const uint32_t *__restrict__ conn, size_t E, uint32_t *__restrict__ out) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
#pragma unroll
  for (int k = 0; k < 8; k++) out[8 * e + k] = conn[(size_t)k * E + e];
}
__global__ void k_interleave3(const uint32_t *__restrict__ soa, size_t n, uint32_t *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[3 * i] = soa[i];
  out[3 * i + 1] = soa[n + i];
  out[3 * i + 2] = soa[2 * n + i];
}
}  // namespace

int dg_da_download(dg_ctx ctx, dg_da da, uint32_t *meta, uint32_t *nodes, uint32_t *node_xyz, int dst_on_device) {
  if (!da) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    const size_t E = da->m.n_elem, V = da->m.n_node;
    if (meta) copy_out(c, meta, da->m.meta, E, dst_on_device);
    if (nodes && E) {
      dg::DBuf<uint32_t> t(8 * E, c.stream), dec;
      const uint32_t *conn = dg::mesh_conn(c, da->m, dec);
      {
        dg::ProfScope _prof("da_transpose", (double)E * 64);
        k_transpose_conn<<<dg::grid_for(E, 256), 256, 0, c.stream>>>(conn, E, t.get());
        DG_LAUNCH_CHECK();
      }
      copy_out(c, nodes, t.get(), 8 * E, dst_on_device);
      DG_CUDA(cudaStreamSynchronize(c.stream));
    }
    if (node_xyz && V) {
      dg::DBuf<uint32_t> t(3 * V, c.stream);
      {
        dg::ProfScope _prof("da_interleave", (double)V * 24);
        k_interleave3<<<dg::grid_for(V, 256), 256, 0, c.stream>>>(da->m.node_xyz, V, t.get());
        DG_LAUNCH_CHECK();
      }
      copy_out(c, node_xyz, t.get(), 3 * V, dst_on_device);
      DG_CUDA(cudaStreamSynchronize(c.stream));
    }
  });
}

int dg_da_free(dg_ctx ctx, dg_da da) {
  if (!ctx || !da) return DG_ERR_INVALID_ARG;
  cudaSetDevice(ctx->c.device);
  dg::mesh_free(ctx->c, da->m);
  cudaStreamSynchronize(ctx->c.stream);
  delete da;
  return DG_OK;
}

}  // extern "C"

namespace {
__global__ void k_zero_bdy(const uint8_t *__restrict__ bdy, size_t n, double *__restrict__ b) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && bdy[i]) b[i] = 0.0;
}

template <typename F>
int level_op(dg_ctx ctx, dg_mg mg, size_t n_in, size_t n_out, const void *in, void *out, int precision, int on_device,
             F &&op) {
  if (!mg || !in || !out || (precision != 32 && precision != 64)) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    const size_t es = precision == 64 ? 8 : 4;
    dg::DBuf<unsigned char> hin, hout;
    const void *x = in;
    void *y = out;
    if (!on_device) {
      hin.alloc(n_in * es, c.stream);
      hout.alloc(n_out * es, c.stream);
      DG_CUDA(cudaMemcpyAsync(hin.get(), in, n_in * es, cudaMemcpyHostToDevice, c.stream));
      x = hin.get();
      y = hout.get();
    }
    op(c, x, y);
    if (!on_device) DG_CUDA(cudaMemcpyAsync(out, y, n_out * es, cudaMemcpyDeviceToHost, c.stream));
    DG_CUDA(cudaStreamSynchronize(c.stream));
  });
}
}  // namespace

extern "C" {

int dg_mg_setup(dg_ctx ctx, dg_octree balanced, size_t max_coarse_elems, dg_mg *out) {
  if (!balanced || !out) return DG_ERR_INVALID_ARG;
  *out = nullptr;
  dg_mg h = new (std::nothrow) dg_mg_s();
  if (!h) return DG_ERR_OUT_OF_MEMORY;
  int rc = guarded(ctx, [&]() { dg::mg_setup(ctx->c, balanced->o, max_coarse_elems, h->mg); });
  if (rc != DG_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return DG_OK;
}

int dg_mg_levels(dg_mg mg, size_t *n) {
  if (!mg || !n) return DG_ERR_INVALID_ARG;
  *n = mg->mg.lv.size();
  return DG_OK;
}

int dg_mg_level_sizes(dg_mg mg, size_t level, size_t *n_elem, size_t *n_node) {
  if (!mg || level >= mg->mg.lv.size()) return DG_ERR_INVALID_ARG;
  if (n_elem) *n_elem = mg->mg.lv[level].mesh.n_elem;
  if (n_node) *n_node = mg->mg.lv[level].mesh.n_node;
  return DG_OK;
}

int dg_mg_level_nodes(dg_ctx ctx, dg_mg mg, size_t level, uint32_t *node_xyz, int dst_on_device) {
  if (!mg || level >= mg->mg.lv.size() || !node_xyz) return DG_ERR_INVALID_ARG;
  dg_da_s tmp;
  tmp.m = mg->mg.lv[level].mesh;
  int rc = dg_da_download(ctx, &tmp, nullptr, nullptr, node_xyz, dst_on_device);
  tmp.m = dg::Mesh();
  return rc;
}

int dg_mg_level_octree(dg_ctx ctx, dg_mg mg, size_t level, uint32_t *xyzl, int dst_on_device) {
  if (!mg || level >= mg->mg.lv.size() || !xyzl) return DG_ERR_INVALID_ARG;
  dg_octree_s tmp;
  tmp.o = mg->mg.lv[level].oct;
  int rc = dg_octree_download(ctx, &tmp, xyzl, dst_on_device);
  tmp.o = dg::Octree();
  return rc;
}

int dg_mg_matvec(dg_ctx ctx, dg_mg mg, size_t level, const void *in, void *out, int precision, int on_device) {
  if (!mg || level >= mg->mg.lv.size()) return DG_ERR_INVALID_ARG;
  const dg::MGLevel &L = mg->mg.lv[level];
  const bool ds = precision == 48;  // FP64 vectors, double-single arithmetic
  return level_op(ctx, mg, L.mesh.n_node, L.mesh.n_node, in, out, ds ? 64 : precision, on_device,
                  [&](dg::Context &c, const void *x, void *y) {
                    if (ds) dg::dirichlet_matvec_ds(c, L, (const double *)x, (double *)y);
                    else if (precision == 64) dg::dirichlet_matvec<double>(c, L, (const double *)x, (double *)y);
                    else dg::dirichlet_matvec<float>(c, L, (const float *)x, (float *)y);
                  });
}

int dg_mg_restrict(dg_ctx ctx, dg_mg mg, size_t f, const void *in, void *out, int precision, int on_device) {
  if (!mg || f + 1 >= mg->mg.lv.size()) return DG_ERR_INVALID_ARG;
  return level_op(ctx, mg, mg->mg.lv[f].mesh.n_node, mg->mg.lv[f + 1].mesh.n_node, in, out, precision, on_device,
                  [&](dg::Context &c, const void *x, void *y) {
                    if (precision == 64) dg::mg_restrict<double>(c, mg->mg, (int)f, (const double *)x, (double *)y);
                    else dg::mg_restrict<float>(c, mg->mg, (int)f, (const float *)x, (float *)y);
                  });
}

int dg_mg_prolong(dg_ctx ctx, dg_mg mg, size_t f, const void *in, void *out, int precision, int on_device) {
  if (!mg || f + 1 >= mg->mg.lv.size()) return DG_ERR_INVALID_ARG;
  return level_op(ctx, mg, mg->mg.lv[f + 1].mesh.n_node, mg->mg.lv[f].mesh.n_node, in, out, precision, on_device,
                  [&](dg::Context &c, const void *x, void *y) {
                    if (precision == 64) dg::mg_prolong<double>(c, mg->mg, (int)f, (const double *)x, (double *)y);
                    else dg::mg_prolong<float>(c, mg->mg, (int)f, (const float *)x, (float *)y);
                  });
}

int dg_mg_set_smoother(dg_mg mg, double omega, int nu_pre, int nu_post) {
  if (!mg || !(omega > 0) || nu_pre < 0 || nu_post < 0) return DG_ERR_INVALID_ARG;
  mg->mg.omega = omega;
  mg->mg.nu_pre = nu_pre;
  mg->mg.nu_post = nu_post;
  return DG_OK;
}

int dg_mg_set_cg_operator(dg_mg mg, int precision, double reliable_delta) {
  if (!mg || (precision != 32 && precision != 48 && precision != 64) || !(reliable_delta > 0 && reliable_delta < 1))
    return DG_ERR_INVALID_ARG;
  mg->mg.cg_operator = precision;
  mg->mg.reliable_delta = reliable_delta;
  return DG_OK;
}

int dg_mg_rhs(dg_ctx ctx, dg_mg mg, const double *f, double *b, int on_device) {
  if (!mg) return DG_ERR_INVALID_ARG;
  const dg::MGLevel &L = mg->mg.lv[0];
  return level_op(ctx, mg, L.mesh.n_node, L.mesh.n_node, f, b, 64, on_device,
                  [&](dg::Context &c, const void *x, void *y) {
                    dg::mesh_matvec<double>(c, L.mesh, (const double *)x, (double *)y, 0.0, 1.0);
                    k_zero_bdy<<<dg::grid_for(L.mesh.n_node, 256), 256, 0, c.stream>>>(L.bdy, L.mesh.n_node,
                                                                                     (double *)y);
                    DG_LAUNCH_CHECK();
                  });
}

int dg_mg_solve(dg_ctx ctx, dg_mg mg, const double *b, double *x, int precision, double rtol, int maxit, int on_device,
                int *iterations, double *relres) {
  if (!mg || !b || !x || maxit < 1 || !(rtol > 0)) return DG_ERR_INVALID_ARG;
  const size_t n = mg->mg.lv[0].mesh.n_node;
  dg::MGResult r;
  int rc = level_op(ctx, mg, n, n, b, x, 64, on_device, [&](dg::Context &c, const void *bb, void *xx) {
    dg::mg_solve(c, mg->mg, (const double *)bb, (double *)xx, precision, rtol, maxit, r);
  });
  if (iterations) *iterations = r.iterations;
  if (relres) *relres = r.relres;
  return rc;
}

int dg_mg_free(dg_ctx ctx, dg_mg mg) {
  if (!ctx || !mg) return DG_ERR_INVALID_ARG;
  cudaSetDevice(ctx->c.device);
  dg::mg_free(ctx->c, mg->mg);
  delete mg;
  return DG_OK;
}


int dg_da_assemble(dg_ctx ctx, dg_da da, double lapFac, double massFac, dg_csr *out) {
  if (!da) return DG_ERR_INVALID_ARG;
  return csr_handle(ctx, out, [&](dg::Csr &c) { dg::assemble_csr(ctx->c, da->m, nullptr, lapFac, massFac, c); });
}

int dg_da_assemble_coef(dg_ctx ctx, dg_da da, const double *coef, int coef_on_device, dg_csr *out) {
  if (!da || (!coef && da->m.n_elem)) return DG_ERR_INVALID_ARG;
  return csr_handle(ctx, out, [&](dg::Csr &c) {
    dg::DBuf<double> hold;
    const double *dc = device_input(ctx->c, coef, 2 * da->m.n_elem, coef_on_device, hold);
    dg::assemble_csr(ctx->c, da->m, nullptr, 1.0, 1.0, c, dc);
  });
}

int dg_matvec_coef(dg_ctx ctx, dg_da da, const double *coef, const void *in, void *out, int precision, int on_device) {
  if (!da || !in || !out || (!coef && da->m.n_elem)) return DG_ERR_INVALID_ARG;
  if (precision != 32 && precision != 64) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    const size_t V = da->m.n_node;
    dg::DBuf<double> hc;
    const double *dc = device_input(c, coef, 2 * da->m.n_elem, on_device, hc);
    auto run = [&](auto tag) {
      using T = decltype(tag);
      dg::DBuf<T> hin, hout;
      const T *x = device_input(c, (const T *)in, V, on_device, hin);
      T *y = (T *)out;
      if (!on_device) {
        hout.alloc(V, c.stream);
        y = hout.get();
      }
      dg::mesh_matvec_coef<T>(c, da->m, dc, x, y);
      if (!on_device) copy_out(c, (T *)out, y, V, 0);
      DG_CUDA(cudaStreamSynchronize(c.stream));
    };
    if (precision == 64) run(double());
    else run(float());
  });
}

int dg_da_diagonal(dg_ctx ctx, dg_da da, const double *coef, double lapFac, double massFac, double *diag,
                   int on_device) {
  if (!da || !diag) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    const size_t V = da->m.n_node;
    dg::DBuf<double> hc, hd;
    const double *dc = coef ? device_input(c, coef, 2 * da->m.n_elem, on_device, hc) : nullptr;
    double *d = diag;
    if (!on_device) {
      hd.alloc(V ? V : 1, c.stream);
      d = hd.get();
    }
    dg::mesh_diagonal(c, da->m, dc, lapFac, massFac, d);
    if (!on_device) copy_out(c, diag, d, V, 0);
    DG_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int dg_mg_diagonal(dg_ctx ctx, dg_mg mg, size_t level, double *diag, int on_device) {
  if (!mg || level >= mg->mg.lv.size() || !diag) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    const dg::MGLevel &L = mg->mg.lv[level];
    const size_t V = L.mesh.n_node;
    dg::DBuf<double> hd;
    double *d = diag;
    if (!on_device) {
      hd.alloc(V ? V : 1, c.stream);
      d = hd.get();
    }
    dg::dirichlet_diagonal(c, L, d);
    if (!on_device) copy_out(c, diag, d, V, 0);
    DG_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int dg_mg_assemble(dg_ctx ctx, dg_mg mg, size_t level, dg_csr *out) {
  if (!mg || level >= mg->mg.lv.size()) return DG_ERR_INVALID_ARG;
  const dg::MGLevel &L = mg->mg.lv[level];
  return csr_handle(ctx, out, [&](dg::Csr &c) { dg::assemble_csr(ctx->c, L.mesh, L.bdy, 1.0, 1.0, c); });
}

int dg_csr_sizes(dg_csr a, size_t *n_rows, size_t *nnz, unsigned *max_row_len) {
  if (!a) return DG_ERR_INVALID_ARG;
  if (n_rows) *n_rows = a->c.n_rows;
  if (nnz) *nnz = a->c.nnz;
  if (max_row_len) *max_row_len = a->c.max_row;
  return DG_OK;
}

int dg_csr_download(dg_ctx ctx, dg_csr a, int64_t *row_ptr, uint32_t *col, double *val, int dst_on_device) {
  if (!a) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    const dg::Csr &c = a->c;
    if (row_ptr) copy_out(ctx->c, row_ptr, c.row_ptr, c.n_rows + 1, dst_on_device);
    if (col && c.nnz) copy_out(ctx->c, col, c.col, c.nnz, dst_on_device);
    if (val && c.nnz) copy_out(ctx->c, val, c.val, c.nnz, dst_on_device);
    DG_CUDA(cudaStreamSynchronize(ctx->c.stream));
  });
}

int dg_csr_spmv(dg_ctx ctx, dg_csr a, const double *x, double *y, int on_device) {
  if (!a || (!x && a->c.n_rows) || (!y && a->c.n_rows)) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    const size_t V = a->c.n_rows;
    dg::DBuf<double> hin, hout;
    const double *dx = device_input(c, x, V, on_device, hin);
    double *dy = y;
    if (!on_device) {
      hout.alloc(V ? V : 1, c.stream);
      dy = hout.get();
    }
    dg::csr_spmv(c, a->c, dx, dy);
    if (!on_device) copy_out(c, y, dy, V, 0);
    DG_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int dg_csr_free(dg_ctx ctx, dg_csr a) {
  if (!a) return DG_OK;
  if (ctx) dg::csr_free(ctx->c, a->c);
  else {
    cudaFree(a->c.row_ptr);
    cudaFree(a->c.col);
    cudaFree(a->c.val);
  }
  delete a;
  return DG_OK;
}

int dg_matvec(dg_ctx ctx, dg_da da, const void *in, void *out, int precision, double lapFac, double massFac,
              int on_device) {
  if (!da || !in || !out) return DG_ERR_INVALID_ARG;
  if (precision != 32 && precision != 64) return DG_ERR_INVALID_ARG;
  return guarded(ctx, [&]() {
    dg::Context &c = ctx->c;
    const size_t V = da->m.n_node;
    if (precision == 64) {
      dg::DBuf<double> hin, hout;
      const double *x = device_input(c, (const double *)in, V, on_device, hin);
      double *y = (double *)out;
      if (!on_device) {
        hout.alloc(V, c.stream);
        y = hout.get();
      }
      dg::mesh_matvec<double>(c, da->m, x, y, lapFac, massFac);
      if (!on_device) copy_out(c, (double *)out, y, V, 0);
      DG_CUDA(cudaStreamSynchronize(c.stream));
    } else {
      dg::DBuf<float> hin, hout;
      const float *x = device_input(c, (const float *)in, V, on_device, hin);
      float *y = (float *)out;
      if (!on_device) {
        hout.alloc(V, c.stream);
        y = hout.get();
      }
      dg::mesh_matvec<float>(c, da->m, x, y, lapFac, massFac);
      if (!on_device) copy_out(c, (float *)out, y, V, 0);
      DG_CUDA(cudaStreamSynchronize(c.stream));
    }
  });
}

}  // extern "C"
