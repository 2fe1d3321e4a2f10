// File formats of the reference's point and octree I/O (see dg_io.cuh).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "dg_io.cuh"

namespace dg {
namespace {

constexpr size_t STAGE = size_t(32) << 20;  // bytes per pinned staging buffer

struct File {
  FILE *f = nullptr;
  File(const char *path, const char *mode) : f(std::fopen(path, mode)) {
    if (!f) fail(DG_ERR_INVALID_ARG, std::string("cannot open ") + path);
  }
  ~File() {
    if (f) std::fclose(f);
  }
  size_t size() {
    std::fseek(f, 0, SEEK_END);
    long s = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    return s < 0 ? 0 : (size_t)s;
  }
};

struct Pinned {
  unsigned char *p = nullptr;
  explicit Pinned(size_t bytes) { DG_CUDA(cudaMallocHost((void **)&p, bytes)); }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

// file bytes [off, off + bytes) -> device dst, through two pinned buffers
// (the read of one chunk overlaps the copy of the previous one)
void file_to_device(Context &ctx, File &f, size_t off, size_t bytes, unsigned char *dst) {
  if (!bytes) return;
  std::fseek(f.f, (long)off, SEEK_SET);
  Pinned a(STAGE), b(STAGE);
  unsigned char *buf[2] = {a.p, b.p};
  cudaEvent_t ev[2];
  DG_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  DG_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  size_t done = 0;
  int k = 0;
  bool ok = true;
  while (done < bytes && ok) {
    const size_t m = std::min(STAGE, bytes - done);
    cudaEventSynchronize(ev[k]);  // the copy out of this buffer has finished
    if (std::fread(buf[k], 1, m, f.f) != m) ok = false;
    if (ok) {
      cudaMemcpyAsync(dst + done, buf[k], m, cudaMemcpyHostToDevice, ctx.stream);
      cudaEventRecord(ev[k], ctx.stream);
    }
    done += m;
    k ^= 1;
  }
  cudaStreamSynchronize(ctx.stream);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (!ok) fail(DG_ERR_INVALID_ARG, "file shorter than its header says");
}

// device src -> file, through two pinned buffers
void device_to_file(Context &ctx, const unsigned char *src, size_t bytes, File &f) {
  if (!bytes) return;
  Pinned a(STAGE), b(STAGE);
  unsigned char *buf[2] = {a.p, b.p};
  cudaEvent_t ev[2];
  DG_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  DG_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  size_t issued = 0, written = 0;
  int k = 0;
  auto issue = [&](int slot) {
    const size_t m = std::min(STAGE, bytes - issued);
    cudaMemcpyAsync(buf[slot], src + issued, m, cudaMemcpyDeviceToHost, ctx.stream);
    cudaEventRecord(ev[slot], ctx.stream);
    issued += m;
  };
  issue(0);
  bool ok = true;
  while (written < bytes) {
    if (issued < bytes) issue(k ^ 1);  // next chunk while this one is written
    cudaEventSynchronize(ev[k]);
    const size_t m = std::min(STAGE, bytes - written);
    if (std::fwrite(buf[k], 1, m, f.f) != m) ok = false;
    written += m;
    k ^= 1;
  }
  cudaStreamSynchronize(ctx.stream);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (!ok) fail(DG_ERR_INVALID_ARG, "write to file failed");
}

__device__ __forceinline__ unsigned ndigits(uint32_t v) {
  unsigned d = 1;
  while (v >= 10u) {
    v /= 10u;
    d++;
  }
  return d;
}

__device__ __forceinline__ void put_uint(unsigned char *p, uint32_t v, unsigned d) {
  for (int i = (int)d - 1; i >= 0; i--) {
    p[i] = (unsigned char)('0' + v % 10u);
    v /= 10u;
  }
}

// bytes of each octant's line "x y z level\n"
__global__ void k_line_len(const uint4 *__restrict__ r, size_t n, uint32_t *__restrict__ len) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 v = r[i];
  len[i] = ndigits(v.x) + ndigits(v.y) + ndigits(v.z) + ndigits(v.w) + 4u;
}

__global__ void k_line_emit(const uint4 *__restrict__ r, size_t n, const uint64_t *__restrict__ off,
                            unsigned char *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 v = r[i];
  unsigned char *p = out + off[i];
  const uint32_t f[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const unsigned d = ndigits(f[k]);
    put_uint(p, f[k], d);
    p += d;
    *p++ = (unsigned char)(k == 3 ? '\n' : ' ');
  }
}

// the whitespace fscanf("%u") skips
__device__ __forceinline__ bool is_ws(unsigned char c) { return c == ' ' || (c >= 9 && c <= 13); }
__device__ __forceinline__ bool is_dig(unsigned char c) { return c >= '0' && c <= '9'; }

constexpr int TOK_CHUNK = 64;  // characters per thread

// tokens starting in each thread's chunk; any other character is an error
__global__ void k_tok_count(const unsigned char *__restrict__ s, size_t len, uint32_t *__restrict__ cnt,
                            uint32_t *flags) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t b = t * TOK_CHUNK;
  if (b >= len) return;
  const size_t e = b + TOK_CHUNK < len ? b + TOK_CHUNK : len;
  uint32_t c = 0;
  bool prev_ws = b == 0 || is_ws(s[b - 1]);
  for (size_t i = b; i < e; i++) {
    const unsigned char ch = s[i];
    if (is_dig(ch)) {
      c += prev_ws ? 1u : 0u;
      prev_ws = false;
    } else if (is_ws(ch)) {
      prev_ws = true;
    } else {
      atomicOr(flags, DGF_DOMAIN);  // not a number
      prev_ws = false;
    }
  }
  cnt[t] = c;
}

// parse the tokens that start in each chunk; the first `ntok` are kept
__global__ void k_tok_parse(const unsigned char *__restrict__ s, size_t len, const uint64_t *__restrict__ off,
                            size_t ntok, uint32_t *__restrict__ out, uint32_t *flags) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t b = t * TOK_CHUNK;
  if (b >= len) return;
  const size_t e = b + TOK_CHUNK < len ? b + TOK_CHUNK : len;
  uint64_t k = off[t];
  bool prev_ws = b == 0 || is_ws(s[b - 1]);
  for (size_t i = b; i < e && k < ntok; i++) {
    const unsigned char ch = s[i];
    if (is_dig(ch) && prev_ws) {
      uint64_t v = 0;
      size_t j = i;
      while (j < len && is_dig(s[j]) && v <= 0xffffffffull) v = v * 10 + (s[j++] - '0');
      if (v > 0xffffffffull) atomicOr(flags, DGF_DOMAIN);  // does not fit an unsigned int
      out[k++] = (uint32_t)v;
    }
    prev_ws = is_ws(ch);
  }
}

__global__ void k_to_records(const uint4 *__restrict__ r, size_t n, unsigned D, uint32_t *__restrict__ rec) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 v = r[i];
  uint32_t *o = rec + 7 * i;
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
  o[4] = 1u;  // weight
  o[5] = 3u;  // dim
  o[6] = D;
}

__global__ void k_from_records(const uint32_t *__restrict__ rec, size_t n, unsigned D, uint4 *__restrict__ r,
                               uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t *o = rec + 7 * i;
  if (o[5] != 3u || o[6] != D) atomicOr(flags, DGF_DOMAIN);
  r[i] = make_uint4(o[0], o[1], o[2], o[3] & 31u);  // TreeNode::getLevel() keeps the low 5 bits
}

}  // namespace

// ---- points ---------------------------------------------------------------
size_t pts_file_count(const char *path) {
  File f(path, "rb");
  uint32_t n = 0;
  if (f.size() < 4) return 0;  // an empty point set is written as an empty file
  if (std::fread(&n, 4, 1, f.f) != 1) return 0;
  return n;
}

size_t pts_file_read(Context &ctx, const char *path, double *xyz, size_t capacity, bool dst_on_device) {
  File f(path, "rb");
  const size_t fs = f.size();
  if (fs < 4) return 0;
  uint32_t n32 = 0;
  if (std::fread(&n32, 4, 1, f.f) != 1) fail(DG_ERR_INVALID_ARG, "cannot read the point count");
  const size_t n = n32, bytes = 24 * n;
  if (n > capacity) fail(DG_ERR_INVALID_ARG, "point file holds more points than the output has room for");
  if (fs < 4 + bytes) fail(DG_ERR_INVALID_ARG, "point file shorter than its count says");
  if (dst_on_device) {
    file_to_device(ctx, f, 4, bytes, reinterpret_cast<unsigned char *>(xyz));
  } else if (n && std::fread(xyz, 1, bytes, f.f) != bytes) {
    fail(DG_ERR_INVALID_ARG, "point file shorter than its count says");
  }
  return n;
}

void pts_file_write(Context &ctx, const char *path, const double *xyz, size_t n, bool src_on_device) {
  if (n > 0xffffffffull) fail(DG_ERR_INVALID_ARG, "the point file's count is 32 bits");
  File f(path, "wb");
  if (!n) return;  // as the reference: nothing is written for no points
  const uint32_t n32 = (uint32_t)n;
  if (std::fwrite(&n32, 4, 1, f.f) != 1) fail(DG_ERR_INVALID_ARG, "write to file failed");
  if (src_on_device) {
    device_to_file(ctx, reinterpret_cast<const unsigned char *>(xyz), 24 * n, f);
  } else if (std::fwrite(xyz, 1, 24 * n, f.f) != 24 * n) {
    fail(DG_ERR_INVALID_ARG, "write to file failed");
  }
}

// ---- octrees ----------------------------------------------------------------
static void require_one_cloud(const Octree &o) {
  if (o.nseg != 1) fail(DG_ERR_UNSUPPORTED, "octree files hold one cloud (extract it first)");
}

void octree_write_text(Context &ctx, const Octree &o, const char *path) {
  require_one_cloud(o);
  cudaStream_t s = ctx.stream;
  const size_t n = o.n;
  File f(path, "w");
  if (!n) return;
  std::fprintf(f.f, "%u %u\n%u\n", 3u, o.max_depth, (unsigned)n);
  DBuf<uint32_t> rec(4 * n, s), len(n, s);
  DBuf<uint64_t> off(n + 1, s);
  octree_to_xyzl(ctx, o, rec.get());
  {
    ProfScope _p(ctx, "io_line_len", (double)n * 20);
    k_line_len<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const uint4 *>(rec.get()), n, len.get());
    DG_LAUNCH_CHECK();
  }
  exclusive_scan<uint32_t, uint64_t>(len.get(), off.get(), n, off.get() + n, s);
  const size_t bytes = (size_t)read_scalar(ctx, reinterpret_cast<unsigned long long *>(off.get() + n));
  DBuf<unsigned char> text(bytes, s);
  {
    ProfScope _p(ctx, "io_line_emit", (double)n * 24 + (double)bytes);
    k_line_emit<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const uint4 *>(rec.get()), n, off.get(), text.get());
    DG_LAUNCH_CHECK();
  }
  std::fflush(f.f);
  device_to_file(ctx, text.get(), bytes, f);
}

void octree_read_text(Context &ctx, const char *path, Octree &out) {
  cudaStream_t s = ctx.stream;
  File f(path, "r");
  const size_t fs = f.size();
  // header: dim, maxDepth, count (fscanf("%u") x 3)
  unsigned dim = 0, D = 0;
  unsigned long cnt = 0;
  if (std::fscanf(f.f, "%u %u %lu", &dim, &D, &cnt) != 3) fail(DG_ERR_INVALID_ARG, "octree file: no header");
  if (dim != 3) fail(DG_ERR_UNSUPPORTED, "octree file: only dim 3 is implemented");
  if (D > 30) fail(DG_ERR_INVALID_ARG, "octree file: maxDepth must be <= 30");
  const size_t body = (size_t)std::ftell(f.f), len = fs > body ? fs - body : 0;
  const size_t n = cnt, ntok = 4 * n;
  DBuf<unsigned char> text(len ? len : 1, s);
  file_to_device(ctx, f, body, len, text.get());
  const size_t nthreads = (len + TOK_CHUNK - 1) / TOK_CHUNK;
  DBuf<uint32_t> cnts(nthreads ? nthreads : 1, s), vals(ntok ? ntok : 4, s);
  DBuf<uint64_t> off(nthreads + 1, s);
  DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
  if (nthreads) {
    {
      ProfScope _p(ctx, "io_tok_count", (double)len);
      k_tok_count<<<grid_for(nthreads, 256), 256, 0, s>>>(text.get(), len, cnts.get(), ctx.d_flags);
      DG_LAUNCH_CHECK();
    }
    exclusive_scan<uint32_t, uint64_t>(cnts.get(), off.get(), nthreads, off.get() + nthreads, s);
    const size_t found = (size_t)read_scalar(ctx, reinterpret_cast<unsigned long long *>(off.get() + nthreads));
    if (found < ntok) fail(DG_ERR_INVALID_ARG, "octree file: fewer numbers than its count says");
    {
      ProfScope _p(ctx, "io_tok_parse", (double)len + (double)ntok * 4);
      k_tok_parse<<<grid_for(nthreads, 256), 256, 0, s>>>(text.get(), len, off.get(), ntok, vals.get(), ctx.d_flags);
      DG_LAUNCH_CHECK();
    }
  } else if (ntok) {
    fail(DG_ERR_INVALID_ARG, "octree file: fewer numbers than its count says");
  }
  if (read_scalar(ctx, ctx.d_flags)) {
    DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
    fail(DG_ERR_INVALID_ARG, "octree file: a field is not an unsigned 32-bit number");
  }
  octree_from_xyzl(ctx, vals.get(), n, D, out);
}

void octree_write_binary(Context &ctx, const Octree &o, const char *path) {
  require_one_cloud(o);
  cudaStream_t s = ctx.stream;
  const size_t n = o.n;
  File f(path, "wb");
  DBuf<uint32_t> xyzl(4 * (n ? n : 1), s), rec(7 * (n ? n : 1), s);
  octree_to_xyzl(ctx, o, xyzl.get());
  k_to_records<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const uint4 *>(xyzl.get()), n, o.max_depth, rec.get());
  DG_LAUNCH_CHECK();
  device_to_file(ctx, reinterpret_cast<const unsigned char *>(rec.get()), 28 * n, f);
}

void octree_read_binary(Context &ctx, const char *path, Octree &out) {
  cudaStream_t s = ctx.stream;
  File f(path, "rb");
  const size_t fs = f.size();
  if (fs == 0 || fs % 28) fail(DG_ERR_INVALID_ARG, "binary octree file: size is not a multiple of 28-byte records");
  const size_t n = fs / 28;
  uint32_t first[7];
  if (std::fread(first, 4, 7, f.f) != 7) fail(DG_ERR_INVALID_ARG, "binary octree file: cannot read");
  const unsigned D = first[6];
  if (first[5] != 3u) fail(DG_ERR_UNSUPPORTED, "binary octree file: only dim 3 is implemented");
  if (D > 30) fail(DG_ERR_INVALID_ARG, "binary octree file: maxDepth must be <= 30");
  DBuf<uint32_t> rec(7 * n, s), xyzl(4 * n, s);
  file_to_device(ctx, f, 0, fs, reinterpret_cast<unsigned char *>(rec.get()));
  DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
  k_from_records<<<grid_for(n, 256), 256, 0, s>>>(rec.get(), n, D, reinterpret_cast<uint4 *>(xyzl.get()), ctx.d_flags);
  DG_LAUNCH_CHECK();
  if (read_scalar(ctx, ctx.d_flags)) {
    DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
    fail(DG_ERR_INVALID_ARG, "binary octree file: records disagree on dim or maxDepth");
  }
  octree_from_xyzl(ctx, xyzl.get(), n, D, out);
}

}  // namespace dg
