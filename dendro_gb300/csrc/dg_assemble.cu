// CSR assembly of the element operators (see dg_assemble.cuh).
//
// 1. incidence: one 64-bit key per (element, vertex) pair, node << 32 |
//    element << 3 | vertex, radix-sorted: the pairs of every node, in
//    element order;
// 2. count: one thread per row walks its pairs and merges the 8 nodes of
//    each element into a sorted column list in registers / local memory;
// 3. scan of the row lengths;
// 4. fill: the same walk, now adding
//       lapFac h/2 L[c][t][k][j] + massFac h^3/8 M[c][t][k][j]
//    (odaJac.C:501-516) to the entry of column conn[j][e].
// A row longer than ROW_MAX entries (not met on 2:1 balanced octrees, whose
// rows hold at most a few dozen) is reported as an internal error.
#include "dg_assemble.cuh"
#include "dg_prims.cuh"

namespace dg {
namespace {

constexpr int ROW_MAX = 128;

__global__ void k_incidence(const uint32_t *__restrict__ conn, size_t E, uint64_t *__restrict__ key) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // i = k * E + e
  if (i >= 8 * E) return;
  const size_t k = i / E, e = i - k * E;
  key[i] = ((uint64_t)conn[i] << 32) | (uint64_t)(e * 8 + k);
}

// start[v] = first pair of node v (lower bound of v << 32)
__global__ void k_row_bounds(const uint64_t *__restrict__ key, size_t n, size_t V, uint64_t *__restrict__ start) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v > V) return;
  const uint64_t t = (uint64_t)v << 32;
  size_t lo = 0, hi = n;
  while (lo < hi) {
    const size_t mid = lo + (hi - lo) / 2;
    if (key[mid] < t) lo = mid + 1;
    else hi = mid;
  }
  start[v] = lo;
}

__device__ __forceinline__ int col_lower_bound(const uint32_t *cols, int n, uint32_t c) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cols[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void k_row_count(const uint64_t *__restrict__ key, const uint64_t *__restrict__ start, size_t V,
                            const uint32_t *__restrict__ conn, size_t E, const uint8_t *__restrict__ bdy,
                            uint32_t *__restrict__ len, unsigned *__restrict__ max_row, uint32_t *flags) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  if (bdy && bdy[v]) {
    len[v] = 1;
    atomicMax(max_row, 1u);
    return;
  }
  uint32_t cols[ROW_MAX];
  int n = 0;
  for (uint64_t p = start[v]; p < start[v + 1]; p++) {
    const size_t e = (uint32_t)key[p] >> 3;
    for (int j = 0; j < 8; j++) {
      const uint32_t c = conn[(size_t)j * E + e];
      if (bdy && bdy[c]) continue;
      const int pos = col_lower_bound(cols, n, c);
      if (pos < n && cols[pos] == c) continue;
      if (n == ROW_MAX) {
        atomicOr(flags, DGF_INTERNAL);
        len[v] = 0;
        return;
      }
      for (int q = n; q > pos; q--) cols[q] = cols[q - 1];
      cols[pos] = c;
      n++;
    }
  }
  len[v] = (uint32_t)n;
  atomicMax(max_row, (unsigned)n);
}

// the row's sorted columns are rebuilt as in the count pass and written
// out; each contribution then adds into its entry of the row's slice of val
// (private to the thread, so no atomics), found by a search of the columns
__global__ void k_row_fill(const uint64_t *__restrict__ key, const uint64_t *__restrict__ start, size_t V,
                           const uint32_t *__restrict__ meta, const uint32_t *__restrict__ conn, size_t E,
                           const uint8_t *__restrict__ bdy, const double *__restrict__ sten, double lap_fac,
                           double mass_fac, const double *__restrict__ coef, const uint64_t *__restrict__ row_ptr,
                           uint32_t *__restrict__ col, double *__restrict__ val) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  const uint64_t out = row_ptr[v];
  if (bdy && bdy[v]) {  // omgJac.C:475-486: the boundary row is the identity
    col[out] = (uint32_t)v;
    val[out] = 1.0;
    return;
  }
  const int cap = (int)(row_ptr[v + 1] - out);
  uint32_t cols[ROW_MAX];
  int n = 0;
  for (uint64_t p = start[v]; p < start[v + 1]; p++) {
    const size_t e = (uint32_t)key[p] >> 3;
    for (int j = 0; j < 8; j++) {
      const uint32_t c = conn[(size_t)j * E + e];
      if (bdy && bdy[c]) continue;
      const int pos = col_lower_bound(cols, n, c);
      if (pos < n && cols[pos] == c) continue;
      if (n == cap) return;  // cannot happen after the count pass
      for (int q = n; q > pos; q--) cols[q] = cols[q - 1];
      cols[pos] = c;
      n++;
    }
  }
  for (int q = 0; q < n; q++) {
    col[out + q] = cols[q];
    val[out + q] = 0.0;
  }
  for (uint64_t p = start[v]; p < start[v + 1]; p++) {
    const uint32_t ek = (uint32_t)key[p];
    const size_t e = ek >> 3;
    const unsigned k = ek & 7u;
    const uint32_t me = meta[e];
    const unsigned l = me & 255u, c = (me >> 8) & 7u, t = me >> 24;
    const double h = 1.0 / (double)(1ull << l);
    const double lf = coef ? coef[2 * e] : lap_fac, mf = coef ? coef[2 * e + 1] : mass_fac;
    const double f1 = lf * h * 0.5, f2 = mf * h * h * h * 0.125;
    const double *S = sten + (c * 18 + t) * 128 + 8 * k;
    for (int j = 0; j < 8; j++) {
      const uint32_t cj = conn[(size_t)j * E + e];
      if (bdy && bdy[cj]) continue;
      val[out + col_lower_bound(cols, n, cj)] += f1 * S[j] + f2 * S[64 + j];
    }
  }
}

template <int LANES>
__global__ void k_csr_spmv(const uint64_t *__restrict__ rp, const uint32_t *__restrict__ col,
                           const double *__restrict__ val, size_t n, const double *__restrict__ x,
                           double *__restrict__ y) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t r = t / LANES;
  const unsigned lane = threadIdx.x % LANES;
  double acc = 0.0;
  if (r < n) {
    const uint64_t end = rp[r + 1];
    uint64_t p = rp[r] + lane;
    // two entries per lane per step: both gathers of x in flight together
    for (; p + LANES < end; p += 2 * LANES) {
      const uint32_t c0 = col[p], c1 = col[p + LANES];
      const double v0 = val[p], v1 = val[p + LANES];
      acc = fma(v0, __ldg(x + c0), acc);
      acc = fma(v1, __ldg(x + c1), acc);
    }
    if (p < end) acc = fma(val[p], __ldg(x + col[p]), acc);
  }
  for (int o = LANES / 2; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, LANES);
  if (r < n && lane == 0) y[r] = acc;
}

unsigned bits_of(size_t v) {
  unsigned b = 0;
  while (b < 64 && (v >> b)) b++;
  return b;
}

}  // namespace

void assemble_csr(Context &ctx, const Mesh &m, const uint8_t *bdy, double lap_fac, double mass_fac, Csr &out,
                  const double *coef) {
  cudaStream_t s = ctx.stream;
  ensure_stencils(ctx);
  const size_t E = m.n_elem, V = m.n_node;
  if (E >= ((size_t)1 << 29)) fail(DG_ERR_UNSUPPORTED, "assemble: more than 2^29 elements");
  if (bdy) {
    lap_fac = mass_fac = 1.0;
    coef = nullptr;
  }
  out = Csr();
  out.n_rows = V;
  DBuf<uint64_t> rp(V + 1, s);
  DG_CUDA(cudaMemsetAsync(rp.get(), 0, (V + 1) * sizeof(uint64_t), s));
  if (V == 0 || E == 0) {
    out.row_ptr = reinterpret_cast<int64_t *>(rp.release_ptr());
    return;
  }
  const size_t np = 8 * E;
  DBuf<uint32_t> conn_tmp;
  const uint32_t *conn = mesh_conn(ctx, m, conn_tmp);
  DBuf<uint64_t> ka(np, s), kb(np, s);
  {
    ProfScope _prof(ctx, "csr_incidence", (double)np * 12);
    k_incidence<<<grid_for(np, 256), 256, 0, s>>>(conn, E, ka.get());
    DG_LAUNCH_CHECK();
  }
  uint64_t *key = radix_sort<uint64_t>(ctx, ka.get(), kb.get(), np, 32 + (int)bits_of(V));
  DBuf<uint64_t> start(V + 1, s);
  DBuf<uint32_t> len(V, s);
  DBuf<unsigned> dmax(1, s);
  DG_CUDA(cudaMemsetAsync(dmax.get(), 0, sizeof(unsigned), s));
  {
    ProfScope _prof(ctx, "csr_count", (double)np * 8 * 8);
    k_row_bounds<<<grid_for(V + 1, 256), 256, 0, s>>>(key, np, V, start.get());
    DG_LAUNCH_CHECK();
    k_row_count<<<grid_for(V, 128), 128, 0, s>>>(key, start.get(), V, conn, E, bdy, len.get(), dmax.get(),
                                                  ctx.d_flags);
    DG_LAUNCH_CHECK();
  }
  {
    uint32_t f = read_scalar(ctx, ctx.d_flags);
    if (f & DGF_INTERNAL) {
      DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
      fail(DG_ERR_INTERNAL, "assemble: a matrix row holds more than 128 entries");
    }
  }
  uint64_t *d_total = reinterpret_cast<uint64_t *>(ctx.d_scratch);
  exclusive_scan<uint32_t, uint64_t>(len.get(), rp.get(), V, d_total, s);
  DG_CUDA(cudaMemcpyAsync(rp.get() + V, d_total, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  const size_t nnz = (size_t)read_scalar(ctx, d_total);
  unsigned mr = 0;
  DG_CUDA(cudaMemcpyAsync(&mr, dmax.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  DBuf<uint32_t> col(nnz ? nnz : 1, s);
  DBuf<double> val(nnz ? nnz : 1, s);
  {
    ProfScope _prof(ctx, "csr_fill", (double)np * 8 * 8 + (double)nnz * 12);
    k_row_fill<<<grid_for(V, 128), 128, 0, s>>>(key, start.get(), V, m.meta, conn, E, bdy, ctx.d_sten64, lap_fac,
                                                 mass_fac, coef, rp.get(), col.get(), val.get());
    DG_LAUNCH_CHECK();
  }
  DG_CUDA(cudaStreamSynchronize(s));
  out.nnz = nnz;
  out.max_row = mr;
  out.row_ptr = reinterpret_cast<int64_t *>(rp.release_ptr());
  out.col = col.release_ptr();
  out.val = val.release_ptr();
}

void csr_free(Context &ctx, Csr &c) {
  if (c.row_ptr) cudaFreeAsync(c.row_ptr, ctx.stream);
  if (c.col) cudaFreeAsync(c.col, ctx.stream);
  if (c.val) cudaFreeAsync(c.val, ctx.stream);
  c = Csr();
}

void csr_spmv(Context &ctx, const Csr &c, const double *x, double *y) {
  if (!c.n_rows) return;
  ProfScope _prof(ctx, "csr_spmv", (double)c.nnz * 12 + (double)c.n_rows * 24);
  constexpr int LANES = 4;
  k_csr_spmv<LANES><<<grid_for(LANES * c.n_rows, 256), 256, 0, ctx.stream>>>(
      reinterpret_cast<const uint64_t *>(c.row_ptr), c.col, c.val, c.n_rows, x, y);
  DG_LAUNCH_CHECK();
}

}  // namespace dg
