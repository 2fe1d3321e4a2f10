// Geometric multigrid on the octree meshes (reference: src/omg/blockDiag.cpp
// DAMG set-up, examples/src/backend/omgJac.C Dirichlet operators,
// src/omg/restrictMatVec.cpp and prolongMatVec.cpp transfers; the PETSc
// KSP CG + PCMG V-cycle with Richardson/Jacobi smoothing configured in
// bin/options:48-206 is restated here as plain CUDA + host control).
//
// Transfers.  A coarse element is either a fine element or the parent of 8
// fine elements (coarsen merges one level; balance never refines past the
// fine octree), so every fine node sits at local coordinates in
// {0, 1/2, 1}^3 of the coarse element that contains it.  Its prolongation
// weights are the coarse element's trilinear shape functions there, folded
// through the coarse element's hanging-vertex interpolation; the weights are
// multiples of 1/64 (shape-function values in {1, 1/2, 1/4, 1/8}, shared
// among at most 8 parent corners), exact in FP32 and stored as w * 64 in
// one byte, nonzero ones only (about 3 per fine node).  They reproduce the reference's restriction
// stencils RmatType1 / RmatType2 exactly.  Restriction is the transpose.
// Pairs with a fine or a coarse boundary node carry no weight, as with the
// reference's suppressed Dirichlet DOFs.
#include "dg_mg.cuh"
#include "dg_elem.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>

namespace dg {

void coarsen_octree(Context &ctx, const Octree &in, Octree &out);

namespace {

__global__ void k_node_bdy(const uint32_t *__restrict__ xyz, size_t V, unsigned D, uint8_t *__restrict__ bdy) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V) return;
  const uint32_t dom = 1u << D;
  uint32_t x = xyz[i], y = xyz[V + i], z = xyz[2 * V + i];
  bdy[i] = (x == 0 || y == 0 || z == 0 || x == dom || y == dom || z == dom) ? 1 : 0;
}

// DirichletJacobianMatGetDiagonal: interior diagonal, 1 on the boundary
__global__ void k_dirichlet_diag(const uint32_t *__restrict__ meta, const uint32_t *__restrict__ conn, size_t E,
                                 const double *__restrict__ sten, const uint8_t *__restrict__ bdy,
                                 double *__restrict__ diag) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const uint32_t me = meta[e];
  const unsigned l = me & 255u, c = (me >> 8) & 7u, t = me >> 24;
  const double h = 1.0 / (double)(1ull << l);
  const double f1 = h * 0.5, f2 = h * h * h * 0.125;
  const double *S = sten + (c * 18 + t) * 128;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    uint32_t id = conn[(size_t)k * E + e];
    if (bdy[id]) diag[id] = 1.0;
    else atomicAdd(&diag[id], f1 * S[9 * k] + f2 * S[64 + 9 * k]);
  }
}

__global__ void k_invert(const double *__restrict__ d, size_t n, double *__restrict__ inv64, float *__restrict__ inv32) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = 1.0 / d[i];
  inv64[i] = v;
  inv32[i] = (float)v;
}

// the transfer tables: every fine node's nonzero prolongation weights, in
// the coarse element's vertex order, packed per warp-chunk of 32 nodes: the
// entries of chunk k start at k * TCHUNK, node v's at its chunk's start plus
// tpos[v] & 255, and number tpos[v] >> 8 (at most 8).  Entry e refers to
// coarse node tid[e] with weight tw[e] / 64.
constexpr int TCHUNK = 32 * 8;

// prolongation weights of fine node v (see the file comment): the 8
// vertices of the coarse element that contains it, with weight 0 where the
// fine or the coarse node is on the domain boundary; false if the node does
// not sit at {0, 1/2, 1}^3 of that element
__device__ __forceinline__ bool prolong_weights(size_t v, const uint32_t *__restrict__ fxyz, size_t Vf,
                                                const uint8_t *__restrict__ fbdy, const Key128 *__restrict__ ckeys,
                                                size_t Ec, const uint32_t *__restrict__ cmeta,
                                                const uint32_t *__restrict__ cconn, const uint8_t *__restrict__ cbdy,
                                                unsigned D, uint32_t (&ids)[8], float (&wv)[8]) {
  const uint32_t dom = 1u << D;
  uint32_t p[3] = {fxyz[v], fxyz[Vf + v], fxyz[2 * Vf + v]};
  uint32_t q[3];
#pragma unroll
  for (int a = 0; a < 3; a++) q[a] = p[a] == dom ? dom - 1 : p[a];
  size_t e = find_leaf(ckeys, Ec, morton3(q[0], q[1], q[2]));
  const Key128 ke = ckeys[e];
  const unsigned lc = tag_level(ke);
  uint32_t an[3];
  demorton3(tag_anchor(ke), an[0], an[1], an[2]);
  const uint64_t h = 1ull << (D - lc);
  const uint32_t me = cmeta[e];
  const unsigned c = (me >> 8) & 7u, hm = (me >> 16) & 255u;
  int xi2[3];
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    uint64_t dlt = (uint64_t)p[a] - an[a];
    if (dlt == 0) xi2[a] = 0;
    else if (2 * dlt == h) xi2[a] = 1;
    else if (dlt == h) xi2[a] = 2;
    else {
      ok = false;
      xi2[a] = 0;
    }
  }
  float N[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    float w = 1.f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      float t = 0.5f * (float)xi2[a];
      w *= ((k >> a) & 1) ? t : 1.f - t;
    }
    N[k] = w;
  }
  float wj[8];
#pragma unroll
  for (int j = 0; j < 8; j++) wj[j] = (hm >> j & 1) ? 0.f : N[j];
  // hanging vertex k: the mean of the parent corners c^s, s a subset of k^c
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (!(hm >> k & 1) || N[k] == 0.f) continue;
    const unsigned dd = (unsigned)(k ^ (int)c);
    const float share = N[k] / (float)(1u << __popc(dd));
    for (unsigned s = 0; s < 8; s++)
      if ((s & dd) == s) wj[c ^ s] += share;
  }
  const bool fb = fbdy[v] != 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    ids[j] = cconn[(size_t)j * Ec + e];
    wv[j] = (fb || cbdy[ids[j]]) ? 0.f : wj[j];
  }
  return ok;
}

// the transfer tables of one fine level (one thread per fine node, blocks of
// 256 threads: a warp is a chunk); every weight must be a multiple of 1/64
// in (0, 1] (kept as w * 64 in one byte).  A warp collects its chunk in
// shared memory and writes it out contiguously.  nnz counts the level's
// entries.
__global__ void __launch_bounds__(256, 6)
    k_prolong_map(const uint32_t *__restrict__ fxyz, size_t Vf, const uint8_t *__restrict__ fbdy,
                  const Key128 *__restrict__ ckeys, size_t Ec, const uint32_t *__restrict__ cmeta,
                  const uint32_t *__restrict__ cconn, const uint8_t *__restrict__ cbdy, unsigned D,
                  uint16_t *__restrict__ tpos, uint32_t *__restrict__ tid, uint8_t *__restrict__ tw,
                  unsigned long long *nnz, uint32_t *flags) {
  __shared__ uint32_t s_id[8][TCHUNK];
  __shared__ __align__(16) uint8_t s_w[8][TCHUNK];
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t ids[8];
  float wv[8];
  bool ok = true;
  int cnt = 0;
  if (v < Vf) {
    ok = prolong_weights(v, fxyz, Vf, fbdy, ckeys, Ec, cmeta, cconn, cbdy, D, ids, wv);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (wv[j] != 0.f) {
        cnt++;
        const float k = wv[j] * 64.f;
        ok = ok && k >= 1.f && k <= 64.f && k == truncf(k);
      }
    }
  }
  // the chunk's entries in lane order (every lane of the warp takes part)
  int incl = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (unsigned)d) incl += t;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (v < Vf) {
    const int start = incl - cnt;
    tpos[v] = (uint16_t)(start | cnt << 8);
    int k = start;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (wv[j] != 0.f) {
        s_id[warp][k] = ids[j];
        s_w[warp][k] = (uint8_t)(wv[j] * 64.f);
        k++;
      }
    }
  }
  __syncwarp();
  // chunk v / 32 (the same for every lane; total is 0 for a warp past Vf)
  const size_t cb = (v >> 5) * TCHUNK;
  for (int i = (int)lane; i < total; i += 32) tid[cb + i] = s_id[warp][i];
  const uint32_t *sw4 = reinterpret_cast<const uint32_t *>(s_w[warp]);
  uint32_t *tw4 = reinterpret_cast<uint32_t *>(tw + cb);  // chunks start 256-byte aligned
  for (int i = (int)lane; i < (total + 3) / 4; i += 32) tw4[i] = sw4[i];
  if (lane == 31u) atomicAdd(nnz, (unsigned long long)total);
  if (!ok) atomicOr(flags, DGF_INTERNAL);
}

// weight e of the transfer tables (exact: a multiple of 1/64)
__device__ __forceinline__ float transfer_w(const uint8_t *__restrict__ tw, size_t e) {
  return (float)tw[e] * (1.f / 64.f);
}

// xf = P xc, or xf += P xc with add (at most 8 terms per fine node, in the
// coarse element's vertex order)
template <typename T>
__global__ void k_prolong(const uint16_t *__restrict__ tpos, const uint32_t *__restrict__ tid,
                          const uint8_t *__restrict__ tw, size_t Vf, const T *__restrict__ xc, T *__restrict__ xf,
                          bool add) {
  size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= Vf) return;
  const uint32_t p = tpos[v], ne = p >> 8;
  const size_t e0 = (v >> 5) * TCHUNK + (p & 255u);
  T acc = 0;
#pragma unroll
  for (uint32_t j = 0; j < 8; j++)
    if (j < ne) acc += (T)transfer_w(tw, e0 + j) * xc[tid[e0 + j]];
  xf[v] = add ? xf[v] + acc : acc;
}

// bc += R rf, or with ax given, bc += R (rf - ax) (the V-cycle's residual
// restricted without storing it)
template <typename T>
__global__ void k_restrict(const uint16_t *__restrict__ tpos, const uint32_t *__restrict__ tid,
                           const uint8_t *__restrict__ tw, size_t Vf, const T *__restrict__ rf, T *__restrict__ bc,
                           const T *__restrict__ ax = nullptr) {
  size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= Vf) return;
  const T r = ax ? rf[v] - ax[v] : rf[v];
  if (r == (T)0) return;
  const uint32_t p = tpos[v], ne = p >> 8;
  const size_t e0 = (v >> 5) * TCHUNK + (p & 255u);
#pragma unroll
  for (uint32_t j = 0; j < 8; j++)
    if (j < ne) atomicAdd(&bc[tid[e0 + j]], (T)transfer_w(tw, e0 + j) * r);
}

// damped Jacobi: x = w D^-1 b (first sweep from zero) or x += w D^-1 (b - Ax)
template <typename T>
__global__ void k_jacobi(T *__restrict__ x, const T *__restrict__ b, const T *__restrict__ ax,
                         const T *__restrict__ dinv, T omega, size_t n, bool from_zero) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = from_zero ? omega * dinv[i] * b[i] : x[i] + omega * dinv[i] * (b[i] - ax[i]);
}

template <typename T>
__global__ void k_residual(const T *__restrict__ b, const T *__restrict__ ax, T *__restrict__ r, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = b[i] - ax[i];
}

__global__ void k_assemble_dense(const uint32_t *__restrict__ meta, const uint32_t *__restrict__ conn, size_t E,
                                 const double *__restrict__ sten, const uint8_t *__restrict__ bdy, size_t n,
                                 double *__restrict__ A) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const uint32_t me = meta[e];
  const unsigned l = me & 255u, c = (me >> 8) & 7u, t = me >> 24;
  const double h = 1.0 / (double)(1ull << l);
  const double f1 = h * 0.5, f2 = h * h * h * 0.125;
  const double *S = sten + (c * 18 + t) * 128;
  uint32_t id[8];
#pragma unroll
  for (int k = 0; k < 8; k++) id[k] = conn[(size_t)k * E + e];
  for (int k = 0; k < 8; k++) {
    if (bdy[id[k]]) continue;
    for (int j = 0; j < 8; j++) {
      if (bdy[id[j]]) continue;
      atomicAdd(&A[(size_t)id[k] * n + id[j]], f1 * S[8 * k + j] + f2 * S[64 + 8 * k + j]);
    }
  }
}

__global__ void k_set_bdy_identity(const uint8_t *__restrict__ bdy, size_t n, double *__restrict__ A) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && bdy[i]) A[i * n + i] = 1.0;
}

// coarse solve of the FP64 V-cycle, x = A^-1 b to FP64 accuracy: x = X b,
// then CS_REFINE rounds of r = b - A x (FP64), x += X r, with X the FP32
// inverse and A the assembled FP64 operator; one warp per row
constexpr int CS_REFINE = 3;

template <typename T>
__global__ void k_cs_apply(const float *__restrict__ Xi, size_t n, const T *__restrict__ v, double *__restrict__ x,
                           bool accumulate) {
  const size_t row = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float *a = Xi + row * n;
  double acc = 0.0;
  for (size_t j = lane; j < n; j += 32) acc = fma((double)a[j], (double)v[j], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) x[row] = accumulate ? x[row] + acc : acc;
}

// x = X b in FP32 (one warp per row), the coarse solve of the FP32 V-cycle
__global__ void k_cs_apply_f32(const float *__restrict__ Xi, size_t n, const float *__restrict__ v,
                               float *__restrict__ x) {
  const size_t row = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float *a = Xi + row * n;
  float acc = 0.f;
  for (size_t j = lane; j < n; j += 32) acc = fmaf(a[j], v[j], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) x[row] = acc;
}

template <typename T>
__global__ void k_cs_resid(const double *__restrict__ A, size_t n, const T *__restrict__ b,
                           const double *__restrict__ x, double *__restrict__ r) {
  const size_t row = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const double *a = A + row * n;
  double acc = 0.0;
  for (size_t j = lane; j < n; j += 32) acc = fma(a[j], x[j], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) r[row] = (double)b[row] - acc;
}

template <typename T>
__global__ void k_cs_out(const double *__restrict__ x, size_t n, T *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)x[i];
}

// FP64 <-> FP32 with an exact power-of-two scale (the FP32 parts of the
// solve work on the CG vectors scaled to order one)
__global__ void k_to_float(const double *__restrict__ a, size_t n, float *__restrict__ b, double scale = 1.0) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)(a[i] * scale);
}
__global__ void k_to_double(const float *__restrict__ a, size_t n, double *__restrict__ b, double scale = 1.0) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i] * scale;
}

// block partial sums of a.b (and of a.a when b is null)
__global__ void k_dot_partial(const double *__restrict__ a, const double *__restrict__ b, size_t n,
                              double *__restrict__ part) {
  double acc = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    acc += a[i] * (b ? b[i] : a[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? ws[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}
__global__ void k_sum(const double *__restrict__ part, int np, double *__restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc += part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? ws[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *out = v;
  }
}

__global__ void k_cg_xr(double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                        const double *__restrict__ q, const double *__restrict__ alpha_num,
                        const double *__restrict__ alpha_den, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double alpha = *alpha_num / *alpha_den;
  x[i] += alpha * p[i];
  r[i] -= alpha * q[i];
}
__global__ void k_cg_p(double *__restrict__ p, const double *__restrict__ z, const double *__restrict__ rz_new,
                       const double *__restrict__ rz_old, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = z[i] + (*rz_new / *rz_old) * p[i];
}

}  // namespace

// ------------------------------------------------------------------------
// DirichletJacobianMatMult (omgJac.C:958-1057): boundary rows are the
// identity, boundary columns are skipped (the patch element loop with DIR)
template <typename T>
void dirichlet_matvec(Context &ctx, const MGLevel &L, const T *x, T *y) {
  ensure_stencils(ctx);
  cudaStream_t s = ctx.stream;
  const Mesh &m = L.mesh;
  DG_CUDA(cudaMemsetAsync(y, 0, m.n_node * sizeof(T), s));
  if (m.plid && ctx.matvec_form != 1) {
    launch_matvec_runs<T, true>(ctx, m, x, y, 1.0, 1.0,
                                sizeof(T) == 4 ? "dirichlet_matvec_fp32" : "dirichlet_matvec_fp64",
                                (double)m.n_elem * 36 + (double)m.n_node * (3 * sizeof(T) + 1));
    return;
  }
  const size_t smem = patch_smem<T>();
  ensure_smem_attr(ctx, k_patch_matvec<T, true>, (int)smem);
  int per_sm = 1;
  DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_matvec<T, true>, PATCH, smem));
  const unsigned grid = (unsigned)std::min<size_t>(m.n_patch, (size_t)std::max(per_sm, 1) * ctx.num_sms);
  const T *cs = std::is_same<T, double>::value ? reinterpret_cast<const T *>(ctx.d_csten64)
                                               : reinterpret_cast<const T *>(ctx.d_csten32);
  ProfScope _prof(ctx, sizeof(T) == 4 ? "dirichlet_matvec_fp32" : "dirichlet_matvec_fp64",
                  (double)m.n_elem * 36 + (double)m.n_node * (3 * sizeof(T) + 1));
  const T *ctab = comb_table<T>(ctx, 1.0, 1.0);
  k_patch_matvec<T, true><<<grid, PATCH, smem, s>>>(m.pmeta, m.pinc, m.pexc, m.pnode, m.poff, m.pkeys, m.pkcount,
                                                    m.n_elem, m.n_patch, cs, ctab, ctx.d_cperm, L.bdy, x, y, (T)1,
                                                    (T)1);
  DG_LAUNCH_CHECK();
}

void dirichlet_diagonal(Context &ctx, const MGLevel &L, double *diag) {
  ensure_stencils(ctx);
  const size_t V = L.mesh.n_node, E = L.mesh.n_elem;
  DG_CUDA(cudaMemsetAsync(diag, 0, V * sizeof(double), ctx.stream));
  if (!E) return;
  ProfScope _prof(ctx, "dirichlet_diagonal", (double)E * 36 + (double)V * 9);
  k_dirichlet_diag<<<grid_for(E, 256), 256, 0, ctx.stream>>>(L.mesh.meta, L.mesh.conn, E, ctx.d_sten64, L.bdy, diag);
  DG_LAUNCH_CHECK();
}

// algorithmic bytes of one transfer over fine level F: its tables (2 bytes
// per node, 5 per weight) and vec bytes of vectors per node
static double transfer_bytes(const MGLevel &F, size_t vec) {
  return (double)F.mesh.n_node * (2 + vec) + (double)F.tnnz * 5;
}

template <typename T>
void mg_restrict(Context &ctx, const MG &mg, int f, const T *rf, T *bc) {
  const MGLevel &F = mg.lv[f];
  const MGLevel &C = mg.lv[f + 1];
  cudaStream_t s = ctx.stream;
  DG_CUDA(cudaMemsetAsync(bc, 0, C.mesh.n_node * sizeof(T), s));
  ProfScope _prof(ctx, "mg_restrict", transfer_bytes(F, sizeof(T)));
  k_restrict<T><<<grid_for(F.mesh.n_node, 256), 256, 0, s>>>(F.tpos, F.tid, F.tw, F.mesh.n_node, rf, bc);
  DG_LAUNCH_CHECK();
}

template <typename T>
void mg_prolong(Context &ctx, const MG &mg, int f, const T *xc, T *xf) {
  const MGLevel &F = mg.lv[f];
  ProfScope _prof(ctx, "mg_prolong", transfer_bytes(F, sizeof(T)));
  k_prolong<T><<<grid_for(F.mesh.n_node, 256), 256, 0, ctx.stream>>>(F.tpos, F.tid, F.tw, F.mesh.n_node, xc, xf,
                                                                       false);
  DG_LAUNCH_CHECK();
}

namespace {

template <typename T>
struct VWork {
  std::vector<DBuf<T>> b, x, ax;
  DBuf<double> cx, cr;  // coarse solve iterate and residual (FP64)
};

template <typename T>
const T *dinv_of(const MGLevel &L) {
  return std::is_same<T, double>::value ? reinterpret_cast<const T *>(L.dinv64) : reinterpret_cast<const T *>(L.dinv32);
}

template <typename T>
void vcycle_level(Context &ctx, const MG &mg, VWork<T> &w, int l, const T *b, T *x) {
  cudaStream_t s = ctx.stream;
  const MGLevel &L = mg.lv[l];
  const size_t n = L.mesh.n_node;
  if (l + 1 == (int)mg.lv.size()) {
    const unsigned gw = grid_for(n * 32, 256);
    if constexpr (std::is_same<T, float>::value) {
      // FP32 V-cycle: the result is FP32, so x = X b in FP32 without
      // refinement (the FP64 rounds would be rounded away)
      ProfScope _prof(ctx, "mg_coarse_solve", (double)n * n * 4);
      k_cs_apply_f32<<<gw, 256, 0, s>>>(mg.cinv32, n, b, x);
      DG_LAUNCH_CHECK();
      return;
    }
    ProfScope _prof(ctx, "mg_coarse_solve", (double)n * n * (4 + CS_REFINE * 12));
    k_cs_apply<T><<<gw, 256, 0, s>>>(mg.cinv32, n, b, w.cx.get(), false);
    for (int it = 0; it < CS_REFINE; it++) {
      k_cs_resid<T><<<gw, 256, 0, s>>>(mg.ca64, n, b, w.cx.get(), w.cr.get());
      k_cs_apply<double><<<gw, 256, 0, s>>>(mg.cinv32, n, w.cr.get(), w.cx.get(), true);
    }
    k_cs_out<T><<<grid_for(n, 256), 256, 0, s>>>(w.cx.get(), n, x);
    DG_LAUNCH_CHECK();
    return;
  }
  const T om = (T)mg.omega;
  T *ax = w.ax[l].get();
  const unsigned g = grid_for(n, 256);
  for (int it = 0; it < mg.nu_pre; it++) {
    if (it > 0) dirichlet_matvec<T>(ctx, L, x, ax);
    ProfScope _prof(ctx, "mg_jacobi", (double)n * 4 * sizeof(T));
    k_jacobi<T><<<g, 256, 0, s>>>(x, b, ax, dinv_of<T>(L), om, n, it == 0);
    DG_LAUNCH_CHECK();
  }
  if (mg.nu_pre == 0) DG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(T), s));
  dirichlet_matvec<T>(ctx, L, x, ax);
  T *bc = w.b[l + 1].get(), *xc = w.x[l + 1].get();
  {
    // the residual b - A x restricted to the next level in one pass
    DG_CUDA(cudaMemsetAsync(bc, 0, mg.lv[l + 1].mesh.n_node * sizeof(T), s));
    ProfScope _prof(ctx, "mg_restrict", transfer_bytes(L, 2 * sizeof(T)));
    k_restrict<T><<<g, 256, 0, s>>>(L.tpos, L.tid, L.tw, n, b, bc, ax);
    DG_LAUNCH_CHECK();
  }
  vcycle_level<T>(ctx, mg, w, l + 1, bc, xc);
  {
    ProfScope _prof(ctx, "mg_prolong", transfer_bytes(L, 2 * sizeof(T)));
    k_prolong<T><<<g, 256, 0, s>>>(L.tpos, L.tid, L.tw, n, xc, x, true);
    DG_LAUNCH_CHECK();
  }
  for (int it = 0; it < mg.nu_post; it++) {
    dirichlet_matvec<T>(ctx, L, x, ax);
    ProfScope _prof(ctx, "mg_jacobi", (double)n * 4 * sizeof(T));
    k_jacobi<T><<<g, 256, 0, s>>>(x, b, ax, dinv_of<T>(L), om, n, false);
    DG_LAUNCH_CHECK();
  }
}

template <typename T>
VWork<T> make_work(Context &ctx, const MG &mg) {
  VWork<T> w;
  for (auto &L : mg.lv) {
    size_t n = L.mesh.n_node;
    w.b.emplace_back(n, ctx.stream);
    w.x.emplace_back(n, ctx.stream);
    w.ax.emplace_back(n, ctx.stream);
  }
  w.cx.alloc(mg.nc ? mg.nc : 1, ctx.stream);
  w.cr.alloc(mg.nc ? mg.nc : 1, ctx.stream);
  return w;
}

}  // namespace

template <typename T>
void mg_vcycle(Context &ctx, const MG &mg, const T *b, T *x) {
  VWork<T> w = make_work<T>(ctx, mg);
  vcycle_level<T>(ctx, mg, w, 0, b, x);
}

// ------------------------------------------------------------------------
void mg_free(Context &ctx, MG &mg) {
  for (auto &L : mg.lv) {
    octree_free(ctx, L.oct);
    mesh_free(ctx, L.mesh);
    if (L.bdy) cudaFreeAsync(L.bdy, ctx.stream);
    if (L.dinv64) cudaFreeAsync(L.dinv64, ctx.stream);
    if (L.dinv32) cudaFreeAsync(L.dinv32, ctx.stream);
    if (L.tpos) cudaFreeAsync(L.tpos, ctx.stream);
    if (L.tid) cudaFreeAsync(L.tid, ctx.stream);
    if (L.tw) cudaFreeAsync(L.tw, ctx.stream);
  }
  if (mg.ca64) cudaFreeAsync(mg.ca64, ctx.stream);
  if (mg.cinv32) cudaFreeAsync(mg.cinv32, ctx.stream);
  cudaStreamSynchronize(ctx.stream);
  mg = MG();
}

static void copy_octree(Context &ctx, const Octree &in, Octree &out) {
  out = Octree();
  out.max_depth = in.max_depth;
  out.n = in.n;
  DG_CUDA(cudaMallocAsync((void **)&out.keys, in.n * sizeof(Key128), ctx.stream));
  DG_CUDA(cudaMemcpyAsync(out.keys, in.keys, in.n * sizeof(Key128), cudaMemcpyDeviceToDevice, ctx.stream));
}

void mg_setup(Context &ctx, const Octree &fine, size_t max_coarse_elem, MG &mg) {
  if (fine.nseg != 1) fail(DG_ERR_UNSUPPORTED, "multigrid: one cloud per hierarchy");
  if (max_coarse_elem < 1) fail(DG_ERR_INVALID_ARG, "multigrid: max_coarse_elem must be >= 1");
  ensure_stencils(ctx);
  cudaStream_t s = ctx.stream;
  mg = MG();
  try {
    mg.lv.emplace_back();
    copy_octree(ctx, fine, mg.lv[0].oct);
    mesh_build(ctx, mg.lv[0].oct, mg.lv[0].mesh);
    while (mg.lv.back().mesh.n_elem > max_coarse_elem) {
      Octree c, b;
      coarsen_octree(ctx, mg.lv.back().oct, c);
      if (c.n == mg.lv.back().oct.n) {
        octree_free(ctx, c);
        break;  // nothing left to coarsen
      }
      balance_octree(ctx, c, b);
      octree_free(ctx, c);
      mg.lv.emplace_back();
      mg.lv.back().oct = b;
      mesh_build(ctx, mg.lv.back().oct, mg.lv.back().mesh);
    }
    const unsigned D = fine.max_depth;
    for (auto &L : mg.lv) {
      const size_t V = L.mesh.n_node, E = L.mesh.n_elem;
      DG_CUDA(cudaMallocAsync((void **)&L.bdy, V, s));
      k_node_bdy<<<grid_for(V, 256), 256, 0, s>>>(L.mesh.node_xyz, V, D, L.bdy);
      DG_LAUNCH_CHECK();
      DBuf<double> diag(V, s);
      DG_CUDA(cudaMemsetAsync(diag.get(), 0, V * sizeof(double), s));
      k_dirichlet_diag<<<grid_for(E, 256), 256, 0, s>>>(L.mesh.meta, L.mesh.conn, E, ctx.d_sten64, L.bdy, diag.get());
      DG_LAUNCH_CHECK();
      DG_CUDA(cudaMallocAsync((void **)&L.dinv64, V * sizeof(double), s));
      DG_CUDA(cudaMallocAsync((void **)&L.dinv32, V * sizeof(float), s));
      k_invert<<<grid_for(V, 256), 256, 0, s>>>(diag.get(), V, L.dinv64, L.dinv32);
      DG_LAUNCH_CHECK();
    }
    DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
    DBuf<unsigned long long> nnz(mg.lv.size(), s);  // nonzero weights per fine level
    DG_CUDA(cudaMemsetAsync(nnz.get(), 0, mg.lv.size() * sizeof(unsigned long long), s));
    for (size_t l = 0; l + 1 < mg.lv.size(); l++) {
      MGLevel &F = mg.lv[l];
      const MGLevel &C = mg.lv[l + 1];
      const size_t Vf = F.mesh.n_node;
      const size_t chunks = (Vf + 31) / 32;
      DG_CUDA(cudaMallocAsync((void **)&F.tpos, std::max<size_t>(Vf, 1) * sizeof(uint16_t), s));
      DG_CUDA(cudaMallocAsync((void **)&F.tid, std::max<size_t>(chunks, 1) * TCHUNK * sizeof(uint32_t), s));
      DG_CUDA(cudaMallocAsync((void **)&F.tw, std::max<size_t>(chunks, 1) * TCHUNK, s));
      // per fine node: coordinates, boundary flag, the containing coarse
      // element's key, meta, 8 vertex ids and their boundary flags in; the
      // position word and about 3 entries of 5 bytes out
      ProfScope _prof(ctx, "mg_prolong_map", (double)Vf * (12 + 1 + 16 + 4 + 32 + 8 + 2 + 15));
      k_prolong_map<<<grid_for(Vf, 256), 256, 0, s>>>(F.mesh.node_xyz, Vf, F.bdy, C.oct.keys, C.oct.n, C.mesh.meta,
                                                      C.mesh.conn, C.bdy, D, F.tpos, F.tid, F.tw, nnz.get() + l,
                                                      ctx.d_flags);
      DG_LAUNCH_CHECK();
    }
    if (mg.lv.size() > 1) {
      std::vector<unsigned long long> h(mg.lv.size() - 1);
      DG_CUDA(cudaMemcpyAsync(h.data(), nnz.get(), h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
      DG_CUDA(cudaStreamSynchronize(s));
      for (size_t l = 0; l < h.size(); l++) mg.lv[l].tnnz = (size_t)h[l];
    }
    check_device_flags(ctx, "multigrid transfers");
    // dense inverse of the coarsest operator
    const MGLevel &C = mg.lv.back();
    const size_t n = C.mesh.n_node;
    if (n > 20000) fail(DG_ERR_INVALID_ARG, "multigrid: coarsest level too large for the dense solve");
    mg.nc = n;
    DG_CUDA(cudaMallocAsync((void **)&mg.ca64, n * n * sizeof(double), s));
    DG_CUDA(cudaMallocAsync((void **)&mg.cinv32, n * n * sizeof(float), s));
    DG_CUDA(cudaMemsetAsync(mg.ca64, 0, n * n * sizeof(double), s));
    k_assemble_dense<<<grid_for(C.mesh.n_elem, 128), 128, 0, s>>>(C.mesh.meta, C.mesh.conn, C.mesh.n_elem,
                                                                   ctx.d_sten64, C.bdy, n, mg.ca64);
    DG_LAUNCH_CHECK();
    k_set_bdy_identity<<<grid_for(n, 256), 256, 0, s>>>(C.bdy, n, mg.ca64);
    DG_LAUNCH_CHECK();
    k_to_float<<<grid_for(n * n, 256), 256, 0, s>>>(mg.ca64, n * n, mg.cinv32);
    DG_LAUNCH_CHECK();
    coarse_inverse(ctx, mg.cinv32, n);
    check_device_flags(ctx, "multigrid coarse inverse");
    DG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    mg_free(ctx, mg);
    throw;
  }
}

// ------------------------------------------------------------------------
void mg_solve(Context &ctx, MG &mg, const double *b, double *x, int precision, double rtol, int maxit,
              MGResult &res) {
  if (precision != 32 && precision != 64) fail(DG_ERR_INVALID_ARG, "multigrid: precision must be 32 or 64");
  cudaStream_t s = ctx.stream;
  const MGLevel &L0 = mg.lv[0];
  const size_t n = L0.mesh.n_node;
  const unsigned g = grid_for(n, 256);
  DBuf<double> r(n, s), z(n, s), p(n, s), q(n, s);
  const int nparts = (int)std::min<size_t>(grid_for(n, 256), (size_t)(ctx.num_sms * 4));
  DBuf<double> part(nparts, s), sc(8, s);  // sc: rz, pq, rr, rz_new, bb
  VWork<float> w32;
  VWork<double> w64;
  DBuf<float> r32, z32;
  if (precision == 32) {
    w32 = make_work<float>(ctx, mg);
    r32.alloc(n, s);
    z32.alloc(n, s);
  } else {
    w64 = make_work<double>(ctx, mg);
  }
  auto dot = [&](const double *a, const double *bb, double *out) {
    ProfScope _prof(ctx, "cg_dot", (double)n * (bb ? 16 : 8));
    k_dot_partial<<<nparts, 256, 0, s>>>(a, bb, n, part.get());
    k_sum<<<1, 256, 0, s>>>(part.get(), nparts, out);
    DG_LAUNCH_CHECK();
  };
  // the CG vectors scale with b: the FP32 V-cycle, the FP32 and the
  // double-single operators work on them scaled by 2^ds_exp (exact), of
  // order one, away from FP32's underflow (a fine mesh's load vector is of
  // order h^3, and the residual falls by the tolerance on top)
  int ds_exp = 0;
  auto precond = [&](const double *rin, double *zout) {
    if (precision == 32) {
      k_to_float<<<g, 256, 0, s>>>(rin, n, r32.get(), std::ldexp(1.0, ds_exp));
      vcycle_level<float>(ctx, mg, w32, 0, r32.get(), z32.get());
      k_to_double<<<g, 256, 0, s>>>(z32.get(), n, zout, std::ldexp(1.0, -ds_exp));
      DG_LAUNCH_CHECK();
    } else {
      vcycle_level<double>(ctx, mg, w64, 0, rin, zout);
    }
  };
  double *d_rz = sc.get(), *d_pq = sc.get() + 1, *d_rr = sc.get() + 2, *d_rzn = sc.get() + 3, *d_bb = sc.get() + 4;
  DG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
  DG_CUDA(cudaMemcpyAsync(r.get(), b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  dot(b, nullptr, d_bb);
  double bb = read_scalar(ctx, d_bb);
  res = MGResult();
  if (bb == 0.0) return;
  const double bnorm = std::sqrt(bb);
  ds_exp = std::max(-900, std::min(900, -std::ilogb(bnorm / std::sqrt((double)n))));
  // CG iteration: step A (q = A p, x and r updated, r.r) and step B (the
  // next direction from z = V-cycle(r)); the host reads r.r after each A.
  // With the FP32 operator, q = A p runs through the FP32 element loop and
  // the recurrence residual is replaced by the FP64 one from time to time.
  const bool op32 = precision == 32 && mg.cg_operator == 32;
  DBuf<float> p32, q32;
  if (op32) {
    p32.alloc(n, s);
    q32.alloc(n, s);
  }
  auto step_a = [&]() {
    if (op32) {
      k_to_float<<<g, 256, 0, s>>>(p.get(), n, p32.get(), std::ldexp(1.0, ds_exp));
      dirichlet_matvec<float>(ctx, L0, p32.get(), q32.get());
      k_to_double<<<g, 256, 0, s>>>(q32.get(), n, q.get(), std::ldexp(1.0, -ds_exp));
      DG_LAUNCH_CHECK();
    } else if (precision == 32 && mg.cg_operator == 48) {
      dirichlet_matvec_ds(ctx, L0, p.get(), q.get(), ds_exp);
    } else {
      dirichlet_matvec<double>(ctx, L0, p.get(), q.get());
    }
    dot(p.get(), q.get(), d_pq);
    k_cg_xr<<<g, 256, 0, s>>>(x, r.get(), p.get(), q.get(), d_rz, d_pq, n);
    DG_LAUNCH_CHECK();
    dot(r.get(), nullptr, d_rr);
  };
  auto step_b = [&]() {
    precond(r.get(), z.get());
    dot(r.get(), z.get(), d_rzn);
    k_cg_p<<<g, 256, 0, s>>>(p.get(), z.get(), d_rzn, d_rz, n);
    DG_LAUNCH_CHECK();
    DG_CUDA(cudaMemcpyAsync(d_rz, d_rzn, sizeof(double), cudaMemcpyDeviceToDevice, s));
  };
  precond(r.get(), z.get());
  DG_CUDA(cudaMemcpyAsync(p.get(), z.get(), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  dot(r.get(), z.get(), d_rz);
  // r = b - A x in FP64 (the reliable update of the FP32-operator form)
  auto true_residual = [&]() {
    dirichlet_matvec<double>(ctx, L0, x, q.get());
    k_residual<double><<<g, 256, 0, s>>>(b, q.get(), r.get(), n);
    DG_LAUNCH_CHECK();
    dot(r.get(), nullptr, d_rr);
    return std::sqrt(read_scalar(ctx, d_rr)) / bnorm;
  };
  double anchor = 1.0;  // relative residual at the last replacement
  // the recurrence's relative residual, replaced by the FP64 one when it has
  // fallen far enough (or would stop the iteration)
  auto residual_now = [&]() {
    double rel = std::sqrt(read_scalar(ctx, d_rr)) / bnorm;
    if (op32 && (rel <= rtol || rel <= mg.reliable_delta * anchor)) {
      rel = true_residual();
      anchor = rel;
    }
    return rel;
  };
  step_a();
  int it = 1;
  double relres = residual_now();
  // Iterations after the first: B then A, a few hundred launches (the
  // V-cycle visits every level), captured once into a CUDA graph and
  // replayed, so each iteration costs one launch.  Everything the capture
  // needs (work vectors, stencil tables, kernel attributes) was set up by
  // the first iteration.  With per-kernel profiling on, the launches stay
  // individual so that each can be timed.
  CudaGraph graph;
  const bool use_graph = !ctx.prof && s != nullptr && maxit > 1;
  while (relres > rtol && it < maxit) {
    if (use_graph && !graph.exec) graph.capture(s, [&]() {
      step_b();
      step_a();
    });
    if (graph.exec) {
      DG_CUDA(cudaGraphLaunch(graph.exec, s));
    } else {
      step_b();
      step_a();
    }
    it++;
    relres = residual_now();
  }
  // the true residual, recomputed in FP64
  dirichlet_matvec<double>(ctx, L0, x, q.get());
  k_residual<double><<<g, 256, 0, s>>>(b, q.get(), r.get(), n);
  DG_LAUNCH_CHECK();
  dot(r.get(), nullptr, d_rr);
  res.iterations = it;
  res.relres = std::sqrt(read_scalar(ctx, d_rr)) / bnorm;
}

__global__ void k_absmax_bits(const double *__restrict__ x, size_t n, unsigned long long *__restrict__ out) {
  unsigned long long m = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    m = max(m, (unsigned long long)__double_as_longlong(fabs(x[i])));  // non-negative: bits order as values
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

void dirichlet_matvec_ds(Context &ctx, const MGLevel &L, const double *x, double *y, int scale_exp) {
  const Mesh &m = L.mesh;
  if (!m.plid) {
    dirichlet_matvec<double>(ctx, L, x, y);
    return;
  }
  ensure_stencils(ctx);
  if (scale_exp == DS_SCALE_AUTO) {  // from the largest entry of x
    DG_CUDA(cudaMemsetAsync(ctx.d_scratch, 0, sizeof(unsigned long long), ctx.stream));
    k_absmax_bits<<<grid_for(m.n_node, 256, (unsigned)ctx.num_sms * 4), 256, 0, ctx.stream>>>(x, m.n_node,
                                                                                         ctx.d_scratch);
    DG_LAUNCH_CHECK();
    const double xmax = __builtin_bit_cast(double, (unsigned long long)read_scalar(ctx, ctx.d_scratch));
    scale_exp = xmax > 0 && std::isfinite(xmax) ? std::max(-900, std::min(900, -std::ilogb(xmax))) : 0;
  }
  DG_CUDA(cudaMemsetAsync(y, 0, m.n_node * sizeof(double), ctx.stream));
  launch_matvec_runs_ds<true>(ctx, m, x, y, 1.0, 1.0, scale_exp, "dirichlet_matvec_ds",
                              (double)m.n_elem * 36 + (double)m.n_node * (3 * sizeof(double) + 1));
}

template void dirichlet_matvec<float>(Context &, const MGLevel &, const float *, float *);
template void dirichlet_matvec<double>(Context &, const MGLevel &, const double *, double *);
template void mg_restrict<float>(Context &, const MG &, int, const float *, float *);
template void mg_restrict<double>(Context &, const MG &, int, const double *, double *);
template void mg_prolong<float>(Context &, const MG &, int, const float *, float *);
template void mg_prolong<double>(Context &, const MG &, int, const double *, double *);
template void mg_vcycle<float>(Context &, const MG &, const float *, float *);
template void mg_vcycle<double>(Context &, const MG &, const double *, double *);

}  // namespace dg
