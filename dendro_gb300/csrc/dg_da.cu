// Octree mesh build (ot::DA at one rank: src/oda/oda.cpp:250 ->
// DA_FactoryPart1..3, src/oda/private/odaFactory.cpp, odaBuildNlist.cpp)
// and the Laplacian + mass element loop (examples/src/backend/odaJac.C).
//
// Hanging vertices.  Element e at level l is child c of parent P (level
// l-1).  Only the vertices c^r with r in {1,2,4} (midpoints of P's edges
// through corner c) and r in {3,5,6} (centres of P's faces through corner
// c) can hang.  Such a vertex hangs when one of P's same-size neighbours
// that share that face or edge is an unrefined leaf (2:1 balance bounds the
// neighbour to level l-1).  A hanging vertex k refers to P's vertex k, which
// is always a mesh node; the element type (one of 18 per child number,
// include/oda/cnumEtypes.h) selects the stencil that folds the hanging
// interpolation into the element matrix.
//
// Nodes.  Every node is the anchor of exactly one octant of the reference's
// DA octant set (elements plus the positive-boundary pseudo-octants of
// octFunctions.cpp:681-770).  Here element e owns its anchor (when it does
// not hang) and its vertices on the positive domain boundary, so the node
// set is numbered by one scan over elements; the owner of any vertex is the
// leaf that contains it after clamping boundary coordinates inward.
#include "dg_da.cuh"
#include "dg_elem.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

namespace dg {

// ------------------------------------------------------------------------
// element-type and stencil tables (host)
// ------------------------------------------------------------------------
// The 18 hanging configurations in the reference's type order
// (include/oda/odaUtils.tcc:14-120), as vertex sets relative to the child's
// own corner: relative vertex r = 1, 2, 4 are the edge midpoints, 3, 5, 6 the
// face centres.  Bit r of each entry marks relative vertex r as hanging.
static const uint8_t kCanonRel[18] = {0x00, 0x04, 0x02, 0x06, 0x10, 0x14, 0x12, 0x16, 0x0e,
                                      0x1e, 0x54, 0x56, 0x5e, 0x32, 0x36, 0x3e, 0x76, 0x7e};
// Each child number's table is the canonical one with its axes permuted:
// the relative axis bit that canonical x, y, z map to.
static const uint8_t kAxisPerm[8][3] = {{1, 2, 4}, {2, 1, 4}, {2, 1, 4}, {1, 2, 4},
                                        {1, 4, 2}, {2, 4, 1}, {2, 4, 1}, {1, 4, 2}};

void gen_etype_masks(uint8_t masks[8 * 18]) {
  for (int c = 0; c < 8; c++)
    for (int t = 0; t < 18; t++) {
      uint8_t m = 0;
      for (int r = 0; r < 8; r++) {
        if (!(kCanonRel[t] >> r & 1)) continue;
        int pr = ((r & 1) ? kAxisPerm[c][0] : 0) | ((r & 2) ? kAxisPerm[c][1] : 0) | ((r & 4) ? kAxisPerm[c][2] : 0);
        m |= (uint8_t)(1u << (pr ^ c));
      }
      masks[c * 18 + t] = m;
    }
}

// S[c][t] = P^T K P on the reference element [-1,1]^3 with trilinear shape
// functions; K = stiffness (Laplacian) or mass; P maps the 8 referenced
// values to the child's vertex values (a hanging vertex is the average of
// the parent corners spanning its edge or face).
void gen_stencils(double *lap, double *mass) {
  const double m1[2][2] = {{2.0 / 3.0, 1.0 / 3.0}, {1.0 / 3.0, 2.0 / 3.0}};
  const double a1[2][2] = {{0.5, -0.5}, {-0.5, 0.5}};
  double K[8][8], M[8][8];
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 8; j++) {
      int ix = i & 1, iy = i >> 1 & 1, iz = i >> 2 & 1, jx = j & 1, jy = j >> 1 & 1, jz = j >> 2 & 1;
      K[i][j] = a1[ix][jx] * m1[iy][jy] * m1[iz][jz] + m1[ix][jx] * a1[iy][jy] * m1[iz][jz] +
                m1[ix][jx] * m1[iy][jy] * a1[iz][jz];
      M[i][j] = m1[ix][jx] * m1[iy][jy] * m1[iz][jz];
    }
  uint8_t masks[8 * 18];
  gen_etype_masks(masks);
  for (int c = 0; c < 8; c++)
    for (int t = 0; t < 18; t++) {
      double P[8][8];
      std::memset(P, 0, sizeof(P));
      uint8_t hm = masks[c * 18 + t];
      for (int k = 0; k < 8; k++) {
        if (!(hm >> k & 1)) {
          P[k][k] = 1.0;
          continue;
        }
        int d = k ^ c, cnt = 0;
        for (int s = 0; s < 8; s++) cnt += ((s & d) == s);
        for (int s = 0; s < 8; s++)
          if ((s & d) == s) P[k][c ^ s] += 1.0 / cnt;
      }
      for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
          double sl = 0.0, sm = 0.0;
          for (int a = 0; a < 8; a++)
            for (int b = 0; b < 8; b++) {
              double w = P[a][i] * P[b][j];
              if (w != 0.0) {
                sl += w * K[a][b];
                sm += w * M[a][b];
              }
            }
          size_t o = (((size_t)c * 18 + t) * 8 + i) * 8 + j;
          lap[o] = sl;
          mass[o] = sm;
        }
    }
}


void ensure_stencils(Context &ctx) {
  if (ctx.d_sten64) return;
  std::vector<double> lap(8 * 18 * 64), mass(8 * 18 * 64);
  gen_stencils(lap.data(), mass.data());
  std::vector<double> s64(STEN_ENTRIES);
  std::vector<float> s32(STEN_ENTRIES);
  for (int ct = 0; ct < 8 * 18; ct++)
    for (int q = 0; q < 64; q++) {
      s64[ct * 128 + q] = lap[ct * 64 + q];
      s64[ct * 128 + 64 + q] = mass[ct * 64 + q];
    }
  for (int i = 0; i < STEN_ENTRIES; i++) s32[i] = (float)s64[i];
  uint8_t masks[8 * 18], etype_of[8 * 256];
  gen_etype_masks(masks);
  std::memset(etype_of, 0xff, sizeof(etype_of));
  for (int c = 0; c < 8; c++)
    for (int t = 0; t < 18; t++) etype_of[c * 256 + masks[c * 18 + t]] = (uint8_t)t;
  double *d64 = nullptr;
  float *d32 = nullptr;
  uint8_t *det = nullptr, *dem = nullptr;
  DG_CUDA(cudaMalloc((void **)&d64, STEN_ENTRIES * sizeof(double)));
  DG_CUDA(cudaMalloc((void **)&d32, STEN_ENTRIES * sizeof(float)));
  DG_CUDA(cudaMalloc((void **)&det, sizeof(etype_of)));
  DG_CUDA(cudaMalloc((void **)&dem, sizeof(masks)));
  DG_CUDA(cudaMemcpy(d64, s64.data(), STEN_ENTRIES * sizeof(double), cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(d32, s32.data(), STEN_ENTRIES * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(det, etype_of, sizeof(etype_of), cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(dem, masks, sizeof(masks), cudaMemcpyHostToDevice));
  ctx.d_sten64 = d64;
  ctx.d_sten32 = d32;
  ctx.d_etype_of = det;
  ctx.d_etype_mask = dem;
  // canonical stencils: S(c,t) = S(0,t) relabelled by a cube symmetry
  std::vector<double> c64(fsten_entries<double>(), 0.0);
  std::vector<float> c32(fsten_entries<float>(), 0.0f);
  std::vector<uint32_t> cperm(8 * 18);
  for (int t = 0; t < 18; t++)
    for (int q = 0; q < 64; q++) {
      c64[t * fsten_stride<double>() + q] = lap[t * 64 + q];
      c64[t * fsten_stride<double>() + 64 + q] = mass[t * 64 + q];
      c32[t * fsten_stride<float>() + q] = (float)lap[t * 64 + q];
      c32[t * fsten_stride<float>() + 64 + q] = (float)mass[t * 64 + q];
    }
  static const int axes[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  for (int c = 0; c < 8; c++)
    for (int t = 0; t < 18; t++) {
      double best = 1e300;
      uint32_t best_sig = 0;
      for (int a = 0; a < 6; a++)
        for (int fl = 0; fl < 8; fl++) {
          int pk[8];
          for (int k = 0; k < 8; k++) {
            int nb = 0;
            for (int i = 0; i < 3; i++) nb |= (((k >> axes[a][i]) & 1) ^ ((fl >> i) & 1)) << i;
            pk[k] = nb;
          }
          double err = 0;
          const int ct = c * 18 + t;
          for (int k = 0; k < 8; k++)
            for (int j = 0; j < 8; j++) {
              err = std::max(err, std::fabs(lap[t * 64 + 8 * pk[k] + pk[j]] - lap[ct * 64 + 8 * k + j]));
              err = std::max(err, std::fabs(mass[t * 64 + 8 * pk[k] + pk[j]] - mass[ct * 64 + 8 * k + j]));
            }
          if (err < best) {
            best = err;
            best_sig = 0;
            for (int k = 0; k < 8; k++) best_sig |= (uint32_t)k << (3 * pk[k]);  // slot of relabelled vertex pk[k]
          }
        }
      if (!(best <= 1e-12)) fail(DG_ERR_INTERNAL, "stencil tables: a (child, type) stencil has no canonical form");
      cperm[c * 18 + t] = best_sig;
    }
  double *dc64 = nullptr;
  float *dc32 = nullptr;
  uint32_t *dcp = nullptr;
  DG_CUDA(cudaMalloc((void **)&dc64, c64.size() * sizeof(double)));
  DG_CUDA(cudaMalloc((void **)&dc32, c32.size() * sizeof(float)));
  DG_CUDA(cudaMalloc((void **)&dcp, cperm.size() * sizeof(uint32_t)));
  DG_CUDA(cudaMemcpy(dc64, c64.data(), c64.size() * sizeof(double), cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(dc32, c32.data(), c32.size() * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(dcp, cperm.data(), cperm.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  ctx.d_csten64 = dc64;
  ctx.d_csten32 = dc32;
  ctx.d_cperm = dcp;
}

// ------------------------------------------------------------------------
// mesh build
// ------------------------------------------------------------------------
// Anchor -> element map: no two octants of a linear octree share an anchor,
// so "the element anchored at p" is one look-up.  Open addressing with
// linear probing over a power-of-two table of element indices (at most half
// full); a slot's anchor is read back from the keys.
constexpr uint32_t AH_EMPTY = 0xffffffffu;

__device__ __forceinline__ uint64_t anchor_hash(Key128 a) {
  uint64_t x = a.lo ^ (a.hi * 0x9e3779b97f4a7c15ull);
  x ^= x >> 31;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 29;
  return x;
}

__global__ void k_anchor_insert(const Key128 *__restrict__ keys, size_t n, uint32_t *__restrict__ tab, uint64_t mask) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  uint64_t h = anchor_hash(tag_anchor(keys[e])) & mask;
  for (uint64_t probe = 0; probe <= mask; probe++) {
    if (atomicCAS(&tab[h], AH_EMPTY, (uint32_t)e) == AH_EMPTY) return;
    h = (h + 1) & mask;
  }
}

// element anchored at `pos` (a bare anchor), or AH_EMPTY
__device__ __forceinline__ uint32_t anchor_find(const Key128 *__restrict__ keys, const uint32_t *__restrict__ tab,
                                                uint64_t mask, Key128 pos) {
  uint64_t h = anchor_hash(pos) & mask;
  for (uint64_t probe = 0; probe <= mask; probe++) {
    const uint32_t e = tab[h];
    if (e == AH_EMPTY) return AH_EMPTY;
    if (key_eq(tag_anchor(keys[e]), pos)) return e;
    h = (h + 1) & mask;
  }
  return AH_EMPTY;
}

__device__ __forceinline__ bool is_leaf_at(const Key128 *__restrict__ keys, const uint32_t *__restrict__ tab,
                                           uint64_t mask, int64_t x, int64_t y, int64_t z, unsigned lev, int64_t dom) {
  if (x < 0 || y < 0 || z < 0 || x >= dom || y >= dom || z >= dom) return false;
  const uint32_t j = anchor_find(keys, tab, mask, morton3((uint32_t)x, (uint32_t)y, (uint32_t)z));
  return j != AH_EMPTY && tag_level(keys[j]) == lev;
}

__global__ void k_mesh_elems(const Key128 *__restrict__ keys, size_t n, const uint32_t *__restrict__ tab,
                             uint64_t mask, unsigned D, const uint8_t *__restrict__ etype_of,
                             uint32_t *__restrict__ meta, uint32_t *__restrict__ cnt, uint32_t *flags) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const Key128 ke = keys[e];
  const unsigned l = tag_level(ke);
  uint32_t ux, uy, uz;
  demorton3(tag_anchor(ke), ux, uy, uz);
  const int64_t dom = (int64_t)1 << D, h = (int64_t)1 << (D - l);
  const int64_t x = ux, y = uy, z = uz;
  int c = 0;
  if (l > 0) c = (int)(((x >> (D - l)) & 1) | (((y >> (D - l)) & 1) << 1) | (((z >> (D - l)) & 1) << 2));
  unsigned hm = 0;
  if (l > 1) {
    const int64_t H = 2 * h;
    const int64_t P[3] = {x - ((c & 1) ? h : 0), y - ((c & 2) ? h : 0), z - ((c & 4) ? h : 0)};
    const int64_t d[3] = {(c & 1) ? H : -H, (c & 2) ? H : -H, (c & 4) ? H : -H};
    // neighbours of P towards the child's exterior: leaf[s] for s in 1..7
    bool leaf[8];
    leaf[0] = false;
#pragma unroll
    for (int s = 1; s < 8; s++) {
      if (s == 7) {
        leaf[s] = false;  // the corner neighbour hangs no vertex of e
        continue;
      }
      leaf[s] = is_leaf_at(keys, tab, mask, P[0] + ((s & 1) ? d[0] : 0), P[1] + ((s & 2) ? d[1] : 0),
                           P[2] + ((s & 4) ? d[2] : 0), l - 1, dom);
    }
#pragma unroll
    for (int r = 1; r < 7; r++) {
      const int others = 7 & ~r;
      bool hang = false;
#pragma unroll
      for (int s = 1; s < 7; s++)
        if ((s & others) == s && leaf[s]) hang = true;
      if (hang) hm |= 1u << (c ^ r);
    }
  }
  unsigned et = etype_of[c * 256 + hm];
  if (et == 0xffu) {
    atomicOr(flags, DGF_NOT_BALANCED);
    et = 0;
  }
  meta[e] = l | ((unsigned)c << 8) | (hm << 16) | (et << 24);
  const unsigned bdy = ((x + h == dom) ? 1u : 0u) | ((y + h == dom) ? 2u : 0u) | ((z + h == dom) ? 4u : 0u);
  unsigned owned = 0;
#pragma unroll
  for (int k = 0; k < 8; k++)
    if ((k & bdy) == (unsigned)k && !(hm >> k & 1)) owned++;
  cnt[e] = owned;
}

__global__ void k_mesh_conn(const Key128 *__restrict__ keys, size_t n, const uint32_t *__restrict__ tab,
                            uint64_t mask, unsigned D, const uint32_t *__restrict__ meta,
                            const uint64_t *__restrict__ base, uint32_t *__restrict__ conn, uint32_t *__restrict__ nx,
                            uint32_t *__restrict__ ny, uint32_t *__restrict__ nz, size_t n_node, uint32_t *flags) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const Key128 ke = keys[e];
  const uint32_t me = meta[e];
  const unsigned l = me & 255u, c = (me >> 8) & 7u, hm = (me >> 16) & 255u;
  uint32_t ux, uy, uz;
  demorton3(tag_anchor(ke), ux, uy, uz);
  const int64_t dom = (int64_t)1 << D, h = (int64_t)1 << (D - l);
  const int64_t x = ux, y = uy, z = uz;
  const int64_t px = x - ((c & 1) ? h : 0), py = y - ((c & 2) ? h : 0), pz = z - ((c & 4) ? h : 0);
  // owned nodes: coordinates
  {
    const unsigned bdy = ((x + h == dom) ? 1u : 0u) | ((y + h == dom) ? 2u : 0u) | ((z + h == dom) ? 4u : 0u);
    uint64_t id = base[e];
    for (int k = 0; k < 8; k++) {
      if ((k & bdy) != (unsigned)k || (hm >> k & 1)) continue;
      if (id < n_node) {
        nx[id] = (uint32_t)(x + ((k & 1) ? h : 0));
        ny[id] = (uint32_t)(y + ((k & 2) ? h : 0));
        nz[id] = (uint32_t)(z + ((k & 4) ? h : 0));
      }
      id++;
    }
  }
#pragma unroll 1
  for (int k = 0; k < 8; k++) {
    int64_t v[3];
    if (hm >> k & 1) {
      v[0] = px + ((k & 1) ? 2 * h : 0);
      v[1] = py + ((k & 2) ? 2 * h : 0);
      v[2] = pz + ((k & 4) ? 2 * h : 0);
    } else {
      v[0] = x + ((k & 1) ? h : 0);
      v[1] = y + ((k & 2) ? h : 0);
      v[2] = z + ((k & 4) ? h : 0);
    }
    unsigned kb = 0;
    int64_t cl[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (v[a] == dom) {
        kb |= 1u << a;
        cl[a] = dom - 1;
      } else {
        cl[a] = v[a];
      }
    }
    // the owner is the element anchored at the vertex; on the positive domain
    // boundary, the leaf containing the vertex clamped inward (a search)
    size_t o;
    bool found = true;
    if (k == 0 && !(hm & 1u)) {
      o = e;  // a vertex 0 that does not hang is the element's own anchor
    } else if (kb == 0) {
      const uint32_t f = anchor_find(keys, tab, mask, morton3((uint32_t)cl[0], (uint32_t)cl[1], (uint32_t)cl[2]));
      found = f != AH_EMPTY;
      o = found ? f : 0;
    } else {
      o = find_leaf_from(keys, n, morton3((uint32_t)cl[0], (uint32_t)cl[1], (uint32_t)cl[2]), e);
    }
    const Key128 ko = keys[o];
    const unsigned lo_ = tag_level(ko);
    const int64_t ho = (int64_t)1 << (D - lo_);
    // the owner's anchor: the vertex itself when it was found by its anchor
    // (no decode needed), else decoded from the owner's key
    int64_t oc[3] = {v[0], v[1], v[2]};
    bool ok = found;
    if (kb != 0) {
      uint32_t ox, oy, oz;
      demorton3(tag_anchor(ko), ox, oy, oz);
      oc[0] = ox;
      oc[1] = oy;
      oc[2] = oz;
#pragma unroll
      for (int a = 0; a < 3; a++) ok = ok && ((kb >> a & 1) ? (oc[a] + ho == dom) : (oc[a] == v[a]));
    }
    const unsigned bo = ((oc[0] + ho == dom) ? 1u : 0u) | ((oc[1] + ho == dom) ? 2u : 0u) | ((oc[2] + ho == dom) ? 4u : 0u);
    const unsigned hmo = (meta[o] >> 16) & 255u;
    ok = ok && ((kb & bo) == kb) && !(hmo >> kb & 1);
    unsigned rank = 0;
    for (unsigned q = 0; q < kb; q++)
      if ((q & bo) == q && !(hmo >> q & 1)) rank++;
    uint64_t id = base[o] + rank;
    if (!ok || id >= n_node) {
      atomicOr(flags, DGF_NOT_BALANCED);
      id = 0;
    }
    conn[(size_t)k * n + e] = (uint32_t)id;
  }
}

// ------------------------------------------------------------------------
// element loop tables: per patch, the (element, vertex) pairs grouped by node
// ------------------------------------------------------------------------
__global__ void k_node_incidence(const uint32_t *__restrict__ conn, size_t n8, uint32_t *__restrict__ cnt) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += stride) atomicAdd(&cnt[conn[i]], 1u);
}

// Bitonic sort of BLOCK * I keys held I per thread (key I*t + j in v[j] of
// thread t), ascending.  Compare-exchanges with partners in the same thread
// run in registers, those within a warp by shuffles, and only the strides
// that cross warps go through shared memory (`stage`, BLOCK * I keys).
template <typename K>
__device__ __forceinline__ K keep_of(K mine, K other, bool keep_min) {
  return keep_min ? (other < mine ? other : mine) : (other > mine ? other : mine);
}

template <typename K, int I, int BLOCK>
__device__ void block_sort_regs(K (&v)[I], K *stage) {
  constexpr int N = BLOCK * I;
  const int t = threadIdx.x;
  for (int s = 2; s <= N; s <<= 1) {
    int d = s >> 1;
    for (; d >= 32 * I; d >>= 1) {  // across warps
#pragma unroll
      for (int j = 0; j < I; j++) stage[I * t + j] = v[j];
      __syncthreads();
#pragma unroll
      for (int j = 0; j < I; j++) {
        const int i = I * t + j;
        v[j] = keep_of(v[j], stage[i ^ d], ((i & d) == 0) == ((i & s) == 0));
      }
      __syncthreads();
    }
    for (; d >= I; d >>= 1) {  // within a warp
#pragma unroll
      for (int j = 0; j < I; j++) {
        const int i = I * t + j;
        const K o = __shfl_xor_sync(0xffffffffu, v[j], d / I);
        v[j] = keep_of(v[j], o, ((i & d) == 0) == ((i & s) == 0));
      }
    }
#pragma unroll
    for (int dd = I / 2; dd > 0; dd >>= 1) {  // within the thread
      if (dd < s) {
#pragma unroll
        for (int j = 0; j < I; j++) {
          if (j & dd) continue;
          const bool up = (((I * t + j) & s) == 0);
          const K a = v[j], b = v[j | dd];
          if ((a > b) == up) {
            v[j] = b;
            v[j | dd] = a;
          }
        }
      }
    }
  }
}

// one block per patch: the patch's elements ordered by (type, level, index);
// then its (element, vertex) pairs grouped by node with a shared-memory hash
// table (one run per distinct node; the pairs of a run ordered by slot, so
// sums over a run are reproducible), run starts, and whether each run holds
// every pair of its node in the mesh.  The element loop needs the pairs of a
// node together, not the runs in any order.
constexpr int PS_HT = PATCH_ENT;  // hash slots (>= distinct nodes of a patch)
constexpr uint32_t PS_EMPTY = 0xffffffffu;

struct PatchSortSmem {
  uint32_t hkey[PS_HT];        // node of each hash slot
  uint16_t hrun[PS_HT];        // run of each hash slot
  uint16_t hcnt[PS_HT];        // pairs per hash slot, then placement cursor per run
  uint16_t roff[PATCH_ENT + 1];  // run offsets
  uint32_t rnode[PATCH_ENT];   // node of each run
  uint16_t ent[PATCH_ENT];     // slots grouped by run
  uint8_t rflag[PATCH_ENT];    // bit 0: a run starts here; bit 1 (per run): complete
  uint32_t ek[PATCH];
  uint16_t rank[PATCH];
};

__global__ void __launch_bounds__(PATCH) k_patch_sort(const uint32_t *__restrict__ conn,
                                                      const uint32_t *__restrict__ meta, size_t E,
                                                      const uint32_t *__restrict__ node_pairs,
                                                      uint16_t *__restrict__ pinc, uint16_t *__restrict__ pexc,
                                                      uint32_t *__restrict__ pmeta, uint16_t *__restrict__ pkeys,
                                                      uint16_t *__restrict__ pkcount, uint32_t *__restrict__ run_node,
                                                      uint32_t *__restrict__ n_run, uint16_t *__restrict__ pperm) {
  extern __shared__ __align__(16) unsigned char ps_raw[];
  PatchSortSmem &S = *reinterpret_cast<PatchSortSmem *>(ps_raw);
  const int tid = threadIdx.x;
  const size_t p = blockIdx.x;
  const size_t e0 = p * PATCH;
  const int ne = (int)((E - e0) < (size_t)PATCH ? (E - e0) : (size_t)PATCH);
  for (int i = tid; i < PS_HT; i += PATCH) {
    S.hkey[i] = PS_EMPTY;
    S.hcnt[i] = 0;
  }
  for (int i = tid; i < PATCH_ENT; i += PATCH) S.rflag[i] = 0;
  // element order: (type, level, index); missing elements last
  {
    uint32_t k1[1];
    if (tid < ne) {
      const uint32_t me = meta[e0 + tid];
      k1[0] = ((me >> 24) << 5 | (me & 31u)) << 9 | (uint32_t)tid;
    } else {
      k1[0] = 0xffffffffu;
    }
    block_sort_regs<uint32_t, 1, PATCH>(k1, S.ek);
    __syncthreads();
    S.ek[tid] = k1[0];
    __syncthreads();
  }
  // (type, level) groups of the ordered elements: the patch's stencil keys
  const uint32_t grp = S.ek[tid] >> 9;
  const int gstart = tid < ne && (tid == 0 || (S.ek[tid - 1] >> 9) != grp) ? 1 : 0;
  int nkeys;
  const int kidx = block_excl_scan<int, PATCH>(gstart, nkeys) + gstart - 1;
  if (tid < ne) {
    const uint32_t eo = S.ek[tid] & (PATCH - 1);
    S.rank[eo] = (uint16_t)tid;
    if (pperm) pperm[p * PATCH + tid] = (uint16_t)eo;
    const uint32_t mo = meta[e0 + eo];
    pmeta[p * PATCH + tid] = (mo & 0xff00ffffu) | (uint32_t)(kidx < PKEY_MAX ? kidx : 0) << 16;
    if (gstart && kidx < PKEY_MAX) pkeys[p * PKEY_MAX + kidx] = (uint16_t)grp;
  }
  if (tid == 0) pkcount[p] = (uint16_t)nkeys;
  __syncthreads();
  // 1. one hash slot per distinct node; pairs counted per slot
  uint16_t hpos[8];
  uint16_t slot[8];
  const bool have = tid < ne;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    hpos[k] = 0;
    slot[k] = (uint16_t)(k * PATCH + (have ? S.rank[tid] : 0));
    if (have) {
      const uint32_t g = conn[(size_t)k * E + e0 + tid];
      uint32_t h = (g * 2654435761u) >> (32 - 12);  // PS_HT = 2^12
      for (int probe = 0; probe < PS_HT; probe++) {
        const uint32_t cur = atomicCAS(&S.hkey[h], PS_EMPTY, g);
        if (cur == PS_EMPTY || cur == g) break;
        h = (h + 1) & (PS_HT - 1);
      }
      hpos[k] = (uint16_t)h;
      atomicAdd(reinterpret_cast<unsigned int *>(&S.hcnt[h & ~1u]), (h & 1u) ? 0x10000u : 1u);
    }
  }
  __syncthreads();
  // 2. runs in hash-slot order: run index and offset of each occupied slot
  {
    constexpr int PER = PS_HT / PATCH;  // slots per thread
    int nr = 0, np = 0;
#pragma unroll
    for (int q = 0; q < PER; q++) {
      const int h = tid * PER + q;
      nr += S.hkey[h] != PS_EMPTY ? 1 : 0;
      np += S.hcnt[h];
    }
    int tot_runs, tot_pairs;
    int ur = block_excl_scan<int, PATCH>(nr, tot_runs);
    int up = block_excl_scan<int, PATCH>(np, tot_pairs);
#pragma unroll
    for (int q = 0; q < PER; q++) {
      const int h = tid * PER + q;
      if (S.hkey[h] != PS_EMPTY) {
        S.hrun[h] = (uint16_t)ur;
        S.roff[ur] = (uint16_t)up;
        S.rnode[ur] = S.hkey[h];
        S.rflag[up] = 1;
        up += S.hcnt[h];
        ur++;
      }
    }
    if (tid == 0) {
      S.roff[tot_runs] = (uint16_t)tot_pairs;
      n_run[p] = (uint32_t)tot_runs;
    }
    __syncthreads();
    for (int i = tid; i < PS_HT; i += PATCH) S.hcnt[i] = 0;  // becomes the placement cursor per run
    __syncthreads();
    // 3. place the pairs (any order), then order each run by slot
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (have) {
        const int u = S.hrun[hpos[k]];
        const unsigned old = atomicAdd(reinterpret_cast<unsigned int *>(&S.hcnt[u & ~1]), (u & 1) ? 0x10000u : 1u);
        const int at = (int)S.roff[u] + (int)((old >> ((u & 1) ? 16 : 0)) & 0xffffu);
        S.ent[at] = slot[k];
      }
    __syncthreads();
    for (int u = tid; u < tot_runs; u += PATCH) {
      const int b = S.roff[u], e = S.roff[u + 1];
      for (int i = b + 1; i < e; i++) {  // insertion sort: runs are short
        const uint16_t v = S.ent[i];
        int j = i - 1;
        while (j >= b && S.ent[j] > v) {
          S.ent[j + 1] = S.ent[j];
          j--;
        }
        S.ent[j + 1] = v;
      }
      const uint32_t g = S.rnode[u];
      run_node[p * PATCH_ENT + u] = g;
      if ((uint32_t)(e - b) == node_pairs[g]) S.rflag[b] |= 2;
    }
    __syncthreads();
  }
  // 4. the packed entries, 8 per thread, and runs starting before each thread
  const int nent = 8 * ne;
  int nst = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) nst += (8 * tid + j < nent && (S.rflag[8 * tid + j] & 1)) ? 1 : 0;
  int total;
  const int ex = block_excl_scan<int, PATCH>(nst, total);
  pexc[p * PATCH + tid] = (uint16_t)ex;
  uint32_t e[8];
  uint8_t comp = 0;
  if (ex > 0) {  // the run in progress at this thread's first pair started earlier
    int i = 8 * tid;
    while (i > 0 && !(S.rflag[i] & 1)) i--;
    comp = S.rflag[i] & 2;
  }
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int i = 8 * tid + j;
    e[j] = 0;
    if (i < nent) {
      const uint8_t f = S.rflag[i];
      if (f & 1) comp = f & 2;
      e[j] = (uint32_t)S.ent[i] | ((f & 1) ? ENT_START : 0u) | (comp ? ENT_COMPLETE : 0u);
    }
  }
  reinterpret_cast<uint4 *>(pinc + p * PATCH_ENT)[tid] =
      make_uint4(e[0] | e[1] << 16, e[2] | e[3] << 16, e[4] | e[5] << 16, e[6] | e[7] << 16);
}

__global__ void k_patch_nodes(const uint32_t *__restrict__ run_node, const uint32_t *__restrict__ n_run,
                              const uint64_t *__restrict__ poff, uint32_t *__restrict__ pnode) {
  const size_t p = blockIdx.x;
  const uint32_t nr = n_run[p];
  for (uint32_t i = threadIdx.x; i < nr; i += blockDim.x) pnode[poff[p] + i] = run_node[p * PATCH_ENT + i];
}

// run-form tables from the pair tables: every pair's run index (run starts
// counted from pexc) per slot in shared memory, then per (type, level)
// position the runs of its vertices in the canonical order of its stencil
// (vertex cperm[c][t] digit m at canonical position m), and per run its node
// with the complete flag of its pairs and the domain-boundary flag of the
// node (the Dirichlet rows and columns).
// The runs are numbered in claim order, for the element loop's shared
// memory banks (a run's index mod 32; shared FP32 atomic adds at random
// banks cost about four times those at distinct banks, measured 13.7
// against 3.3 cycles per warp instruction on an SM): in round m = 0..7
// every element claims the run at its canonical position m if no element
// has yet, and the runs a warp claims in one round take consecutive
// indices, so that they fall on distinct banks when that warp touches them
// together.  (A greedy colouring that also avoided the banks of a run's
// other groups gave the same element-loop time at 4 to 7 times the cost.)
__global__ void __launch_bounds__(PATCH) k_patch_runs(const uint16_t *__restrict__ pinc,
                                                      const uint16_t *__restrict__ pexc,
                                                      const uint32_t *__restrict__ pnode,
                                                      const uint64_t *__restrict__ poff,
                                                      const uint32_t *__restrict__ pmeta,
                                                      const uint32_t *__restrict__ cperm, size_t E,
                                                      const uint32_t *__restrict__ node_xyz, size_t V,
                                                      uint32_t dom, uint4 *__restrict__ plid,
                                                      uint32_t *__restrict__ prun) {
  __shared__ uint16_t run_of[PATCH_ENT];
  __shared__ unsigned short newidx[PATCH_ENT];
  __shared__ uint32_t word[PATCH_ENT];
  __shared__ int counter;
  const size_t p = blockIdx.x;
  const int t = threadIdx.x, lane = t & 31;
  const size_t e0 = p * PATCH;
  const int ne = (int)((E - e0) < (size_t)PATCH ? (E - e0) : (size_t)PATCH);
  const uint64_t ub = poff[p];
  const int nr = (int)(poff[p + 1] - ub);
  for (int i = t; i < nr; i += PATCH) newidx[i] = 0xffff;
  if (t == 0) counter = 0;
  if (t < ne) {
    int r = (int)pexc[p * PATCH + t] - 1;
    for (int i = 8 * t; i < 8 * t + 8; i++) {
      const uint32_t ent = pinc[p * PATCH_ENT + i];
      if (ent & ENT_START) {
        r++;
        const uint32_t g = pnode[ub + r];
        const uint32_t cx = node_xyz[g], cy = node_xyz[V + g], cz = node_xyz[2 * V + g];
        const bool on_bdy = cx == 0 || cy == 0 || cz == 0 || cx == dom || cy == dom || cz == dom;
        word[r] = g | ((ent & ENT_COMPLETE) ? PRUN_COMPLETE : 0u) | (on_bdy ? PRUN_BDY : 0u);
      }
      run_of[ent & ENT_SLOT] = (uint16_t)r;
    }
  }
  __syncthreads();
  uint32_t lid[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (t < ne) {
    const uint32_t me = pmeta[p * PATCH + t];
    const uint32_t sig = cperm[((me >> 8) & 7u) * 18 + (me >> 24)];
#pragma unroll
    for (int m = 0; m < 8; m++) lid[m] = run_of[((sig >> (3 * m)) & 7u) * PATCH + t];
  }
#pragma unroll 1
  for (int m = 0; m < 8; m++) {
    uint32_t r = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) r = k == m ? lid[k] : r;
    const bool won = t < ne && atomicCAS(&newidx[r], (unsigned short)0xffff, (unsigned short)0xfffe) == 0xffff;
    const unsigned bal = __ballot_sync(0xffffffffu, won);
    if (bal) {
      const int leader = __ffs(bal) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&counter, __popc(bal));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (won) newidx[r] = (unsigned short)(base + __popc(bal & ((1u << lane) - 1u)));
    }
    __syncthreads();
  }
  if (t < ne) {
    uint32_t w[4];
#pragma unroll
    for (int m = 0; m < 8; m += 2) w[m >> 1] = (uint32_t)newidx[lid[m]] | (uint32_t)newidx[lid[m + 1]] << 16;
    plid[p * PATCH + t] = make_uint4(w[0], w[1], w[2], w[3]);
  }
  for (int u = t; u < nr; u += PATCH) prun[ub + newidx[u]] = word[u];
}

// conn from the patch tables: pair i of patch p belongs to the run counted
// by the run starts up to i (pexc gives the count before pair 8t), its slot
// names the vertex and the element's (type, level) position
__global__ void __launch_bounds__(PATCH) k_conn_from_patches(const uint16_t *__restrict__ pinc,
                                                             const uint16_t *__restrict__ pexc,
                                                             const uint32_t *__restrict__ pnode,
                                                             const uint64_t *__restrict__ poff,
                                                             const uint16_t *__restrict__ pperm, size_t E,
                                                             uint32_t *__restrict__ conn) {
  const size_t p = blockIdx.x;
  const int t = threadIdx.x;
  const size_t e0 = p * PATCH;
  const int ne = (int)((E - e0) < (size_t)PATCH ? (E - e0) : (size_t)PATCH);
  if (t >= ne) return;  // the pairs of a patch's ne elements are its first 8 ne entries
  uint32_t r = pexc[p * PATCH + t];
  const uint64_t ub = poff[p];
  for (int i = 8 * t; i < 8 * t + 8; i++) {
    const uint32_t ent = pinc[p * PATCH_ENT + i];
    if (ent & ENT_START) r++;
    const uint32_t slot = ent & ENT_SLOT;
    const uint32_t v = slot / PATCH, pos = slot % PATCH;
    conn[(size_t)v * E + e0 + pperm[p * PATCH + pos]] = pnode[ub + r - 1];
  }
}

const uint32_t *mesh_conn(Context &ctx, const Mesh &m, DBuf<uint32_t> &tmp) {
  if (!m.compressed) return m.conn;
  tmp.alloc(8 * m.n_elem, ctx.stream);
  ProfScope _prof(ctx, "da_conn_decode", (double)m.n_elem * (16 + 2 + 32) + (double)m.n_elem * 6);
  k_conn_from_patches<<<(unsigned)m.n_patch, PATCH, 0, ctx.stream>>>(m.pinc, m.pexc, m.pnode, m.poff, m.pperm,
                                                                     m.n_elem, tmp.get());
  DG_LAUNCH_CHECK();
  return tmp.get();
}

size_t mesh_bytes(const Mesh &m) {
  const size_t E = m.n_elem, V = m.n_node, np = m.n_patch;
  size_t runs = 0;
  if (np && m.poff) {
    uint64_t r = 0;
    if (cudaMemcpy(&r, m.poff + np, sizeof(uint64_t), cudaMemcpyDeviceToHost) == cudaSuccess) runs = r;
  }
  size_t b = E * 4 + V * 12;                                    // meta, node coordinates
  if (m.conn) b += 8 * E * 4;                                   // conn
  b += np * (PATCH_ENT * 2 + PATCH * 2 + PATCH * 4 + PKEY_MAX * 2 + 2) + (np + 1) * 8 + runs * 4;  // patches
  if (m.pperm) b += np * PATCH * 2;
  if (m.plid) b += np * PATCH * 16 + runs * 4;  // run-form tables
  return b;
}

static void mesh_patches(Context &ctx, Mesh &m) {
  cudaStream_t s = ctx.stream;
  const size_t n = m.n_elem, np = (n + PATCH - 1) / PATCH;
  if (m.n_node >= (size_t)PRUN_BDY) fail(DG_ERR_INVALID_ARG, "DA: too many nodes for the element loop tables");
  DBuf<uint32_t> pairs(m.n_node, s), run_node(np * PATCH_ENT, s), n_run(np, s);
  DBuf<uint16_t> pinc(np * PATCH_ENT, s), pexc(np * PATCH, s);
  DBuf<uint32_t> pmeta(np * PATCH, s);
  DBuf<uint16_t> pkeys(np * PKEY_MAX, s), pkcount(np, s);
  DBuf<uint64_t> poff(np + 1, s);
  DBuf<uint16_t> pperm(np * PATCH, s);
  DG_CUDA(cudaMemsetAsync(pairs.get(), 0, m.n_node * sizeof(uint32_t), s));
  {
    ProfScope _prof(ctx, "da_node_pairs", (double)n * 8 * 8);
    k_node_incidence<<<grid_for(8 * n, 256, (unsigned)ctx.num_sms * 16), 256, 0, s>>>(m.conn, 8 * n, pairs.get());
    DG_LAUNCH_CHECK();
  }
  {
    ProfScope _prof(ctx, "da_patch_sort", (double)n * 8 * 14);
    ensure_smem_attr(ctx, k_patch_sort, (int)sizeof(PatchSortSmem));
    k_patch_sort<<<(unsigned)np, PATCH, sizeof(PatchSortSmem), s>>>(m.conn, m.meta, n, pairs.get(), pinc.get(),
                                                                    pexc.get(), pmeta.get(), pkeys.get(),
                                                                    pkcount.get(), run_node.get(), n_run.get(),
                                                                    pperm.get());
    DG_LAUNCH_CHECK();
  }
  exclusive_scan<uint32_t, uint64_t>(n_run.get(), poff.get(), np, poff.get() + np, s);
  uint64_t nruns = 0;
  DG_CUDA(cudaMemcpyAsync(&nruns, poff.get() + np, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  DBuf<uint32_t> pnode(nruns ? nruns : 1, s);
  {
    ProfScope _prof(ctx, "da_patch_nodes", (double)nruns * 8);
    k_patch_nodes<<<(unsigned)np, 256, 0, s>>>(run_node.get(), n_run.get(), poff.get(), pnode.get());
    DG_LAUNCH_CHECK();
  }
  if (!m.compressed) {  // a compressed DA keeps the pair tables only
    DBuf<uint4> plid(np * PATCH, s);
    DBuf<uint32_t> prun(nruns ? nruns : 1, s);
    {
      ProfScope _prof(ctx, "da_patch_runs", (double)n * (16 + 2 + 4 + 16) + (double)nruns * 8);
      k_patch_runs<<<(unsigned)np, PATCH, 0, s>>>(pinc.get(), pexc.get(), pnode.get(), poff.get(), pmeta.get(),
                                                  ctx.d_cperm, n, m.node_xyz, m.n_node, 1u << m.max_depth,
                                                  plid.get(), prun.get());
      DG_LAUNCH_CHECK();
    }
    m.plid = plid.release_ptr();
    m.prun = prun.release_ptr();
  }
  m.n_patch = np;
  m.pinc = pinc.release_ptr();
  m.pexc = pexc.release_ptr();
  m.pmeta = pmeta.release_ptr();
  m.pkeys = pkeys.release_ptr();
  m.pkcount = pkcount.release_ptr();
  m.pnode = pnode.release_ptr();
  m.poff = poff.release_ptr();
  m.pperm = pperm.release_ptr();
}

void mesh_build(Context &ctx, const Octree &bal, Mesh &m, bool compress) {
  cudaStream_t s = ctx.stream;
  const size_t n = bal.n;
  const unsigned D = bal.max_depth;
  if (n == 0) fail(DG_ERR_INVALID_ARG, "DA: empty octree");
  if (n >= 0xffffffffull / 8) fail(DG_ERR_INVALID_ARG, "DA: too many elements");
  ensure_stencils(ctx);
  m.max_depth = D;
  m.n_elem = n;
  DBuf<uint32_t> meta(n, s), cnt(n, s);
  // anchor -> element map, at most half full
  size_t cap = 1;
  while (cap < 2 * n) cap <<= 1;
  DBuf<uint32_t> atab(cap, s);
  const uint64_t amask = cap - 1;
  DG_CUDA(cudaMemsetAsync(atab.get(), 0xff, cap * sizeof(uint32_t), s));
  {
    ProfScope _prof(ctx, "da_anchor_map", (double)n * 16 + (double)cap * 4);
    k_anchor_insert<<<grid_for(n, 256), 256, 0, s>>>(bal.keys, n, atab.get(), amask);
    DG_LAUNCH_CHECK();
  }
  DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
  {
    ProfScope _prof(ctx, "da_elems", (double)n * 24);
    k_mesh_elems<<<grid_for(n, 256), 256, 0, s>>>(bal.keys, n, atab.get(), amask, D, ctx.d_etype_of, meta.get(),
                                                 cnt.get(), ctx.d_flags);
  DG_LAUNCH_CHECK();
    }
  DBuf<uint64_t> base(n, s);
  uint64_t *d_total = reinterpret_cast<uint64_t *>(ctx.d_scratch);
  exclusive_scan<uint32_t, uint64_t>(cnt.get(), base.get(), n, d_total, s);
  size_t nn = (size_t)read_scalar(ctx, d_total);
  check_device_flags(ctx, "DA");
  if (nn >= 0xffffffffull) fail(DG_ERR_INVALID_ARG, "DA: too many nodes");
  cnt.release();
  DBuf<uint32_t> conn(8 * n, s), nxyz(3 * (nn ? nn : 1), s);
  {
    ProfScope _prof(ctx, "da_conn", (double)n * 56);
    k_mesh_conn<<<grid_for(n, 256), 256, 0, s>>>(bal.keys, n, atab.get(), amask, D, meta.get(), base.get(), conn.get(),
                                                nxyz.get(),
                                               nxyz.get() + nn, nxyz.get() + 2 * nn, nn, ctx.d_flags);
  DG_LAUNCH_CHECK();
    }
  check_device_flags(ctx, "DA");
  m.n_node = nn;
  m.meta = meta.release_ptr();
  m.conn = conn.release_ptr();
  m.node_xyz = nxyz.release_ptr();
  m.compressed = compress;
  mesh_patches(ctx, m);
  if (compress) {  // the element loop needs only the patch tables
    cudaFreeAsync(m.conn, s);
    m.conn = nullptr;
  }
}

void mesh_free(Context &ctx, Mesh &m) {
  if (m.meta) cudaFreeAsync(m.meta, ctx.stream);
  if (m.conn) cudaFreeAsync(m.conn, ctx.stream);
  if (m.node_xyz) cudaFreeAsync(m.node_xyz, ctx.stream);
  if (m.pinc) cudaFreeAsync(m.pinc, ctx.stream);
  if (m.pexc) cudaFreeAsync(m.pexc, ctx.stream);
  if (m.pmeta) cudaFreeAsync(m.pmeta, ctx.stream);
  if (m.pkeys) cudaFreeAsync(m.pkeys, ctx.stream);
  if (m.pkcount) cudaFreeAsync(m.pkcount, ctx.stream);
  if (m.pnode) cudaFreeAsync(m.pnode, ctx.stream);
  if (m.poff) cudaFreeAsync(m.poff, ctx.stream);
  if (m.pperm) cudaFreeAsync(m.pperm, ctx.stream);
  if (m.plid) cudaFreeAsync(m.plid, ctx.stream);
  if (m.prun) cudaFreeAsync(m.prun, ctx.stream);
  m = Mesh();
}

// ------------------------------------------------------------------------
// element loop
// ------------------------------------------------------------------------
template <typename T>
const T *comb_table(Context &ctx, double lap_fac, double mass_fac) {
  ensure_stencils(ctx);
  const bool dbl = std::is_same<T, double>::value;
  T **tab = reinterpret_cast<T **>(dbl ? (void *)&ctx.d_comb64 : (void *)&ctx.d_comb32);
  double *f = dbl ? ctx.comb64_f : ctx.comb32_f;
  bool &ok = dbl ? ctx.comb64_ok : ctx.comb32_ok;
  if (!*tab) DG_CUDA(cudaMalloc((void **)tab, COMB_ENTRIES * sizeof(T)));
  if (!ok || f[0] != lap_fac || f[1] != mass_fac) {
    const T *cs = dbl ? reinterpret_cast<const T *>(ctx.d_csten64) : reinterpret_cast<const T *>(ctx.d_csten32);
    k_comb_table<T><<<(COMB_ENTRIES + 255) / 256, 256, 0, ctx.stream>>>(cs, (T)lap_fac, (T)mass_fac, *tab);
    DG_LAUNCH_CHECK();
    f[0] = lap_fac;
    f[1] = mass_fac;
    ok = true;
  }
  return *tab;
}
template const float *comb_table<float>(Context &, double, double);
template const double *comb_table<double>(Context &, double, double);

// the FP64 combined stencils as (hi, lo) FP32 pairs, per (type, level) laid
// out by (row pair p, column j): (hi[2p][j], hi[2p+1][j], lo[2p][j], lo[2p+1][j])
__global__ void k_split_pairs(const double *__restrict__ in, size_t n_stencils, float4 *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_stencils * 32) return;
  const size_t st = i / 32;
  const int p = (int)(i % 32) / 8, j = (int)(i % 8);
  const double a = in[st * 64 + (2 * p) * 8 + j], b = in[st * 64 + (2 * p + 1) * 8 + j];
  const float ah = __double2float_rn(a), bh = __double2float_rn(b);
  out[i] = make_float4(ah, bh, __double2float_rn(a - (double)ah), __double2float_rn(b - (double)bh));
}

__global__ void k_row_abs_max(const double *__restrict__ comb, float *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // (type, level)
  if (i >= COMB_ENTRIES / 64) return;
  double m = 0.0;
  for (int k = 0; k < 8; k++) {
    double r = 0.0;
    for (int j = 0; j < 8; j++) r += fabs(comb[i * 64 + 8 * k + j]);
    m = fmax(m, r);
  }
  out[i] = __double2float_ru(m * (1.0 + 1e-12));
}

const float4 *comb_table_ds(Context &ctx, double lap_fac, double mass_fac) {
  if (!ctx.d_comb_ds) DG_CUDA(cudaMalloc((void **)&ctx.d_comb_ds, COMB_ENTRIES / 2 * sizeof(float4)));
  if (!ctx.d_comb_rowabs) DG_CUDA(cudaMalloc((void **)&ctx.d_comb_rowabs, COMB_ENTRIES / 64 * sizeof(float)));
  if (!ctx.comb_ds_ok || ctx.comb_ds_f[0] != lap_fac || ctx.comb_ds_f[1] != mass_fac) {
    const double *d = comb_table<double>(ctx, lap_fac, mass_fac);
    k_split_pairs<<<(COMB_ENTRIES / 2 + 255) / 256, 256, 0, ctx.stream>>>(d, COMB_ENTRIES / 64, ctx.d_comb_ds);
    DG_LAUNCH_CHECK();
    k_row_abs_max<<<(COMB_ENTRIES / 64 + 127) / 128, 128, 0, ctx.stream>>>(d, ctx.d_comb_rowabs);
    DG_LAUNCH_CHECK();
    ctx.comb_ds_f[0] = lap_fac;
    ctx.comb_ds_f[1] = mass_fac;
    ctx.comb_ds_ok = true;
  }
  return ctx.d_comb_ds;
}

// the double-single run-form loop (k_patch_matvec_runs_ds): FP64 vectors
template <bool DIR>
void launch_matvec_runs_ds(Context &ctx, const Mesh &m, const double *x, double *y, double lap_fac,
                           double mass_fac, int scale_exp, const char *name, double bytes) {
  const size_t smem = patch_runs_ds_smem();
  ensure_smem_attr(ctx, k_patch_matvec_runs_ds<DIR>, (int)smem);
  int per_sm = 1;
  DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_matvec_runs_ds<DIR>, PATCH, smem));
  if (per_sm < 1) per_sm = 1;
  const unsigned grid = (unsigned)std::min<size_t>(m.n_patch, (size_t)per_sm * ctx.num_sms);
  const float4 *ctab = comb_table_ds(ctx, lap_fac, mass_fac);
  ProfScope _prof(ctx, name, bytes);
  k_patch_matvec_runs_ds<DIR><<<grid, PATCH, smem, ctx.stream>>>(m.pmeta, m.plid, m.prun, m.poff, m.pkeys,
                                                                 m.pkcount, m.n_elem, m.n_patch, ctab,
                                                                 ctx.d_comb_rowabs, x, y,
                                                                 std::ldexp(1.0, scale_exp), -scale_exp);
  DG_LAUNCH_CHECK();
}
template void launch_matvec_runs_ds<true>(Context &, const Mesh &, const double *, double *, double, double, int,
                                          const char *, double);
template void launch_matvec_runs_ds<false>(Context &, const Mesh &, const double *, double *, double, double, int,
                                           const char *, double);

// the run-form element loop (k_patch_matvec_runs); DIR: the Dirichlet
// form (boundary rows and columns from the run words' boundary flag)
template <typename T, bool DIR>
void launch_matvec_runs(Context &ctx, const Mesh &m, const T *x, T *y, double lap_fac,
                        double mass_fac, const char *name, double bytes) {
  const size_t smem = patch_runs_smem<T>();
  ensure_smem_attr(ctx, k_patch_matvec_runs<T, DIR>, (int)smem);
  int per_sm = 1;
  DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_matvec_runs<T, DIR>, PATCH, smem));
  if (per_sm < 1) per_sm = 1;
  const unsigned grid = (unsigned)std::min<size_t>(m.n_patch, (size_t)per_sm * ctx.num_sms);
  const T *cs = std::is_same<T, double>::value ? reinterpret_cast<const T *>(ctx.d_csten64)
                                               : reinterpret_cast<const T *>(ctx.d_csten32);
  const T *ctab = std::is_same<T, double>::value ? comb_table<T>(ctx, lap_fac, mass_fac) : nullptr;
  ProfScope _prof(ctx, name, bytes);
  k_patch_matvec_runs<T, DIR><<<grid, PATCH, smem, ctx.stream>>>(m.pmeta, m.plid, m.prun, m.poff, m.pkeys,
                                                                m.pkcount, m.n_elem, m.n_patch, cs, ctab, x, y,
                                                                (T)lap_fac, (T)mass_fac);
  DG_LAUNCH_CHECK();
}
template void launch_matvec_runs<float, true>(Context &, const Mesh &, const float *, float *,
                                              double, double, const char *, double);
template void launch_matvec_runs<float, false>(Context &, const Mesh &, const float *, float *,
                                               double, double, const char *, double);
template void launch_matvec_runs<double, true>(Context &, const Mesh &, const double *, double *,
                                               double, double, const char *, double);
template void launch_matvec_runs<double, false>(Context &, const Mesh &, const double *,
                                                double *, double, double, const char *, double);

template <typename T>
void mesh_matvec(Context &ctx, const Mesh &m, const T *x, T *y, double lap_fac, double mass_fac) {
  ensure_stencils(ctx);
  cudaStream_t s = ctx.stream;
  DG_CUDA(cudaMemsetAsync(y, 0, m.n_node * sizeof(T), s));
  if (m.plid && ctx.matvec_form != 1) {
    launch_matvec_runs<T, false>(ctx, m, x, y, lap_fac, mass_fac,
                                 sizeof(T) == 4 ? "matvec_fp32" : "matvec_fp64",
                                 (double)m.n_elem * 36 + (double)m.n_node * 3 * sizeof(T));
    return;
  }
  const size_t smem = patch_smem<T>();
  ensure_smem_attr(ctx, k_patch_matvec<T, false>, (int)smem);
  int per_sm = 1;
  DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_matvec<T, false>, PATCH, smem));
  if (per_sm < 1) per_sm = 1;
  const unsigned grid = (unsigned)std::min<size_t>(m.n_patch, (size_t)per_sm * ctx.num_sms);
  const T *cs = std::is_same<T, double>::value ? reinterpret_cast<const T *>(ctx.d_csten64)
                                               : reinterpret_cast<const T *>(ctx.d_csten32);
  const T *ctab = comb_table<T>(ctx, lap_fac, mass_fac);
  {
    ProfScope _prof(ctx, sizeof(T) == 4 ? "matvec_fp32" : "matvec_fp64",
                    (double)m.n_elem * 36 + (double)m.n_node * 3 * sizeof(T));
    k_patch_matvec<T, false><<<grid, PATCH, smem, s>>>(m.pmeta, m.pinc, m.pexc, m.pnode, m.poff, m.pkeys,
                                                       m.pkcount, m.n_elem, m.n_patch, cs, ctab, ctx.d_cperm, nullptr,
                                                       x, y, (T)lap_fac, (T)mass_fac);
    DG_LAUNCH_CHECK();
  }
}

template void mesh_matvec<float>(Context &, const Mesh &, const float *, float *, double, double);
template void mesh_matvec<double>(Context &, const Mesh &, const double *, double *, double, double);

template <typename T>
void mesh_matvec_coef(Context &ctx, const Mesh &m, const double *coef, const T *x, T *y) {
  ensure_stencils(ctx);
  cudaStream_t s = ctx.stream;
  DG_CUDA(cudaMemsetAsync(y, 0, m.n_node * sizeof(T), s));
  const size_t smem = patch_smem<T>();
  ensure_smem_attr(ctx, k_patch_matvec<T, false, true>, (int)smem);
  int per_sm = 1;
  DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_matvec<T, false, true>, PATCH, smem));
  if (per_sm < 1) per_sm = 1;
  const unsigned grid = (unsigned)std::min<size_t>(m.n_patch, (size_t)per_sm * ctx.num_sms);
  const T *cs = std::is_same<T, double>::value ? reinterpret_cast<const T *>(ctx.d_csten64)
                                               : reinterpret_cast<const T *>(ctx.d_csten32);
  ProfScope _prof(ctx, sizeof(T) == 4 ? "matvec_coef_fp32" : "matvec_coef_fp64",
                  (double)m.n_elem * (36 + 16 + 2) + (double)m.n_node * 3 * sizeof(T));
  k_patch_matvec<T, false, true><<<grid, PATCH, smem, s>>>(m.pmeta, m.pinc, m.pexc, m.pnode, m.poff, m.pkeys,
                                                           m.pkcount, m.n_elem, m.n_patch, cs, nullptr, ctx.d_cperm,
                                                           nullptr, x, y, (T)1, (T)1, coef, m.pperm);
  DG_LAUNCH_CHECK();
}
template void mesh_matvec_coef<float>(Context &, const Mesh &, const double *, const float *, float *);
template void mesh_matvec_coef<double>(Context &, const Mesh &, const double *, const double *, double *);

// diagonal entries per element, added atomically (a node's sum is over the
// elements that hold it)
__global__ void k_mesh_diag(const uint32_t *__restrict__ meta, const uint32_t *__restrict__ conn, size_t E,
                            const double *__restrict__ sten, const double *__restrict__ coef, double lap_fac,
                            double mass_fac, double *__restrict__ diag) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const uint32_t me = meta[e];
  const unsigned l = me & 255u, c = (me >> 8) & 7u, t = me >> 24;
  const double h = 1.0 / (double)(1ull << l);
  const double lf = coef ? coef[2 * e] : lap_fac, mf = coef ? coef[2 * e + 1] : mass_fac;
  const double f1 = lf * h / 2.0, f2 = mf * h * h * h / 8.0;
  const double *S = sten + (c * 18 + t) * 128;
#pragma unroll
  for (int k = 0; k < 8; k++) atomicAdd(&diag[conn[(size_t)k * E + e]], f1 * S[9 * k] + f2 * S[64 + 9 * k]);
}

void mesh_diagonal(Context &ctx, const Mesh &m, const double *coef, double lap_fac, double mass_fac, double *diag) {
  ensure_stencils(ctx);
  cudaStream_t s = ctx.stream;
  DG_CUDA(cudaMemsetAsync(diag, 0, m.n_node * sizeof(double), s));
  if (!m.n_elem) return;
  DBuf<uint32_t> tmp;
  const uint32_t *conn = mesh_conn(ctx, m, tmp);
  ProfScope _prof(ctx, "mesh_diagonal", (double)m.n_elem * (4 + 32 + (coef ? 16 : 0)) + (double)m.n_node * 8);
  k_mesh_diag<<<grid_for(m.n_elem, 256), 256, 0, s>>>(m.meta, conn, m.n_elem, ctx.d_sten64, coef, lap_fac, mass_fac,
                                                       diag);
  DG_LAUNCH_CHECK();
}

}  // namespace dg
