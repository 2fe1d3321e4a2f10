/*
 * dg_oracle — CPU restatement of the reference (Dendro4) octree hot path.
 * TEST INFRASTRUCTURE ONLY (see dg_oracle.h): the checker for the CUDA
 * library, never part of it.
 *
 * Reference files cited are paths inside the Dendro4 source tree.
 */
#include "dg_oracle.h"

#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

void dgo_free(void *p) { free(p); }

/* ------------------------------------------------------------------------ */
/* Morton order (include/TreeNode.tcc:211-236): interleave the anchor bits,  */
/* z above y above x within every bit position; equal anchors: lower level   */
/* (the ancestor) first (TreeNode.tcc:131-133).                              */
/* ------------------------------------------------------------------------ */
static u128 spread3(uint32_t v) {
  u128 r = 0;
  for (int b = 0; b < 32; b++)
    if (v >> b & 1u) r |= (u128)1 << (3 * b);
  return r;
}

static u128 morton(uint32_t x, uint32_t y, uint32_t z) {
  return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

/* total order key: anchor Morton (96 bits) then level (5 bits) */
static u128 okey(const dgo_oct *o) { return (morton(o->x, o->y, o->z) << 5) | (u128)(o->lev & 31u); }

static int oct_lt(const dgo_oct *a, const dgo_oct *b) { return okey(a) < okey(b); }
static int oct_eq(const dgo_oct *a, const dgo_oct *b) {
  return a->x == b->x && a->y == b->y && a->z == b->z && a->lev == b->lev;
}
static int oct_le(const dgo_oct *a, const dgo_oct *b) { return okey(a) <= okey(b); }

typedef struct {
  u128 k;
  dgo_oct o;
} keyed_oct;

static int cmp_keyed(const void *pa, const void *pb) {
  const keyed_oct *a = (const keyed_oct *)pa, *b = (const keyed_oct *)pb;
  return (a->k > b->k) - (a->k < b->k);
}

static int cmp_u128(const void *pa, const void *pb) {
  u128 a = *(const u128 *)pa, b = *(const u128 *)pb;
  return (a > b) - (a < b);
}

/* sort octants in Morton order (stable w.r.t. equal records is irrelevant:
 * equal keys mean equal {x,y,z,lev}) */
static int sort_octs(dgo_oct *a, size_t n) {
  if (n < 2) return 0;
  keyed_oct *t = (keyed_oct *)malloc(n * sizeof(keyed_oct));
  if (!t) return DGO_ENOMEM;
  for (size_t i = 0; i < n; i++) {
    t[i].k = okey(&a[i]);
    t[i].o = a[i];
  }
  qsort(t, n, sizeof(keyed_oct), cmp_keyed);
  for (size_t i = 0; i < n; i++) a[i] = t[i].o;
  free(t);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* TreeNode operations used by the walk (Morton build)                       */
/* ------------------------------------------------------------------------ */
static inline uint64_t oct_len(const dgo_oct *o, unsigned D) { return (uint64_t)1 << (D - o->lev); }

/* isAncestor: strictly coarser and containing (TreeNode.tcc:590-609) */
static int is_anc(const dgo_oct *a, const dgo_oct *b, unsigned D) {
  if (!(a->lev < b->lev)) return 0;
  uint64_t la = oct_len(a, D), lb = oct_len(b, D);
  return b->x >= a->x && b->y >= a->y && b->z >= a->z && (uint64_t)b->x + lb <= (uint64_t)a->x + la &&
         (uint64_t)b->y + lb <= (uint64_t)a->y + la && (uint64_t)b->z + lb <= (uint64_t)a->z + la;
}

/* getFirstChild, Morton: same anchor, one level finer (TreeNode.tcc:578-582) */
static dgo_oct first_child(dgo_oct a) {
  a.lev++;
  return a;
}

/* getNext, Morton (TreeNode.tcc:533-549): the octant that follows a in SFC
 * order, climbing while a is a last child. */
static dgo_oct get_next(dgo_oct m, unsigned D) {
  uint32_t mask = 1u << (D - m.lev);
  int i;
  for (i = (int)m.lev; i >= 0; --i) {
    m.x ^= mask;
    if (m.x & mask) break;
    m.y ^= mask;
    if (m.y & mask) break;
    m.z ^= mask;
    if (m.z & mask) break;
    mask <<= 1;
  }
  m.lev = (uint32_t)i;
  return m;
}

/* getDLD, Morton (TreeNode.tcc:453-455): deepest last descendant */
static dgo_oct get_dld(const dgo_oct *a, unsigned D) {
  uint32_t l = (uint32_t)oct_len(a, D);
  dgo_oct r = {a->x + l - 1, a->y + l - 1, a->z + l - 1, D};
  return r;
}

/* ------------------------------------------------------------------------ */
/* points2Octree                                                             */
/* ------------------------------------------------------------------------ */
int dgo_quantize_sort(const double *xyz, size_t n, const double gLens[3], unsigned D, dgo_oct **out) {
  if (D > 30 || (!xyz && n)) return DGO_EINVAL;
  dgo_oct *p = (dgo_oct *)malloc((n ? n : 1) * sizeof(dgo_oct));
  if (!p) return DGO_ENOMEM;
  const double scale = (double)(1u << D);
  for (size_t i = 0; i < n; i++) {
    /* construct.cpp:935-941: (unsigned int)(pts * (double)(1u<<maxDepth) / gLens) */
    p[i].x = (uint32_t)(xyz[3 * i] * scale / gLens[0]);
    p[i].y = (uint32_t)(xyz[3 * i + 1] * scale / gLens[1]);
    p[i].z = (uint32_t)(xyz[3 * i + 2] * scale / gLens[2]);
    p[i].lev = D;
  }
  int rc = sort_octs(p, n);
  if (rc) {
    free(p);
    return rc;
  }
  *out = p;
  return 0;
}

typedef struct {
  dgo_oct *a;
  size_t n, cap;
} oct_vec;

static int ov_push(oct_vec *v, dgo_oct o) {
  if (v->n == v->cap) {
    size_t nc = v->cap ? 2 * v->cap : 1024;
    dgo_oct *na = (dgo_oct *)realloc(v->a, nc * sizeof(dgo_oct));
    if (!na) return DGO_ENOMEM;
    v->a = na;
    v->cap = nc;
  }
  v->a[v->n++] = o;
  return 0;
}

/* std::lower_bound(first, last, value, std::less_equal<TreeNode>()):
 * the first element e in [first,last) with !(e <= value). */
static size_t lower_bound_le(const dgo_oct *a, size_t first, size_t last, const dgo_oct *value) {
  size_t lo = first, hi = last;
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (oct_le(&a[mid], value))
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

/* p2oLocal (src/construct.cpp:976-1076) from leaves = {root}.  The index
 * arithmetic keeps the reference's unsigned 32-bit semantics for the point
 * counters (next_pt, inc). */
int dgo_p2o_local(const dgo_oct *pts, size_t n, unsigned D, unsigned m, dgo_oct **out, size_t *nout) {
  if (m == 0 || D > 30 || n >= 0x7fffffffu) return DGO_EINVAL;
  oct_vec lst = {0, 0, 0};
  const uint32_t num_pts = (uint32_t)n;
  dgo_oct root = {0, 0, 0, 0};
  dgo_oct curr = root;
  dgo_oct last = get_dld(&root, D);
  dgo_oct next = get_next(curr, D);
  uint32_t curr_pt = 0;
  uint32_t next_pt = curr_pt + m;
  int rc = 0;

  /* The walk's getNext climbs above the root after the last octant; at
   * level "-1" it no longer moves and the reference loops forever.  Report
   * that state (and a step bound) instead of looping. */
  const uint64_t max_steps = 64ull * ((uint64_t)n + 1) * (D + 2);
  uint64_t steps = 0;
  while (next_pt < num_pts) { /* :1009 */
    if (curr.lev > D || ++steps > max_steps) {
      rc = DGO_ENOTERM;
      goto fail;
    }
    while (is_anc(&curr, &pts[next_pt - 1], D) & is_anc(&curr, &pts[next_pt], D) & (curr.lev < D)) {
      curr = first_child(curr); /* :1013-1018 */
      next = get_next(curr, D);
    }
    uint32_t inc = m; /* :1021-1031, curr can not be refined past maxDepth */
    while (curr.lev == D - 1) {
      inc = inc << 1;
      next_pt += inc;
      if (next_pt > num_pts) {
        next_pt = num_pts - 1;
        break;
      }
    }
    /* :1037 found_pt = lower_bound(&nodes[curr_pt], &nodes[next_pt], next, less_equal) */
    int found_pt = (int)(lower_bound_le(pts, curr_pt, next_pt, &next) - curr_pt);
    next_pt = curr_pt + (uint32_t)found_pt;
    if ((rc = ov_push(&lst, curr))) goto fail;
    curr = next;
    next = get_next(curr, D);
    if (next_pt > curr_pt) curr_pt = next_pt;
    next_pt = curr_pt + m;
  }

  while (oct_le(&curr, &last)) { /* :1051-1061 */
    if (curr.lev > D || ++steps > max_steps) {
      rc = DGO_ENOTERM;
      goto fail;
    }
    for (;;) {
      dgo_oct dld = get_dld(&curr, D);
      if (!(oct_lt(&last, &dld) && curr.lev < D)) break;
      curr = first_child(curr);
    }
    if ((rc = ov_push(&lst, curr))) goto fail;
    dgo_oct dld = get_dld(&curr, D);
    if (oct_eq(&dld, &last)) break;
    curr = get_next(curr, D);
  }

  /* :1063 std::list::unique (consecutive duplicates) */
  size_t w = 0;
  for (size_t i = 0; i < lst.n; i++)
    if (w == 0 || !oct_eq(&lst.a[w - 1], &lst.a[i])) lst.a[w++] = lst.a[i];
  *out = lst.a ? lst.a : (dgo_oct *)malloc(sizeof(dgo_oct));
  *nout = w;
  return 0;
fail:
  free(lst.a);
  return rc;
}

int dgo_points_to_octree(const double *xyz, size_t n, const double gLens[3], unsigned D, unsigned m, dgo_oct **out,
                         size_t *nout) {
  if (m == 0 || D > 30) return DGO_EINVAL;
  if (D == 0 || n <= m) { /* construct.cpp:916-920, 948-952 */
    dgo_oct *r = (dgo_oct *)malloc(sizeof(dgo_oct));
    if (!r) return DGO_ENOMEM;
    r->x = r->y = r->z = r->lev = 0;
    *out = r;
    *nout = 1;
    return 0;
  }
  dgo_oct *p = NULL;
  int rc = dgo_quantize_sort(xyz, n, gLens, D, &p);
  if (rc) return rc;
  rc = dgo_p2o_local(p, n, D, m, out, nout);
  free(p);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* balance: closure of the internal-node sets, finest level first.           */
/*   I_l   = internal nodes at level l                                       */
/*   I_l-1 = parents of the input leaves at level l, plus, for every q in    */
/*           I_l, the level-(l-1) parents of q's 26 same-level neighbours    */
/*           (these are the 8 parents of q's 3x3x3 block, inside the domain) */
/*   leaves at level l = children(I_l-1) \ I_l                               */
/* ------------------------------------------------------------------------ */
static u128 lvl_index(uint32_t x, uint32_t y, uint32_t z, unsigned lev, unsigned D) {
  unsigned s = D - lev;
  return morton(x >> s, y >> s, z >> s);
}

static int cmp_u128_unique(u128 *a, size_t *n) {
  if (*n > 1) qsort(a, *n, sizeof(u128), cmp_u128);
  size_t w = 0;
  for (size_t i = 0; i < *n; i++)
    if (w == 0 || a[w - 1] != a[i]) a[w++] = a[i];
  *n = w;
  return 0;
}

static void level_index_decode(u128 k, uint32_t *x, uint32_t *y, uint32_t *z) {
  uint32_t a = 0, b = 0, c = 0;
  for (int bit = 0; bit < 32; bit++) {
    a |= (uint32_t)((k >> (3 * bit)) & 1) << bit;
    b |= (uint32_t)((k >> (3 * bit + 1)) & 1) << bit;
    c |= (uint32_t)((k >> (3 * bit + 2)) & 1) << bit;
  }
  *x = a;
  *y = b;
  *z = c;
}

static int u128_contains(const u128 *a, size_t n, u128 v) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < n && a[lo] == v;
}

/* incCorner = 0 (balanceOctree's face + edge form, src/balance.cpp:31 with
 * the 18 neighbour directions of TreeNode::addBalancingDescendants,
 * src/TreeNode.cpp:138-190): a corner neighbour of q imposes nothing, so the
 * one parent that only corner neighbours reach (the outward parent on all
 * three axes) is left out. */
int dgo_balance_ex(const dgo_oct *in, size_t n, unsigned D, int incCorner, dgo_oct **out, size_t *nout) {
  if (D > 30 || n == 0) return DGO_EINVAL;
  if (n == 1) {
    dgo_oct *r = (dgo_oct *)malloc(sizeof(dgo_oct));
    if (!r) return DGO_ENOMEM;
    *r = in[0];
    *out = r;
    *nout = 1;
    return 0;
  }
  unsigned maxL = 0;
  for (size_t i = 0; i < n; i++) {
    /* octants must lie in the domain and be aligned (the reference asserts
     * otherwise, src/octFunctions.cpp:310) */
    if (in[i].lev > D) return DGO_EINVAL;
    uint64_t len = (uint64_t)1 << (D - in[i].lev), dom = (uint64_t)1 << D;
    if (in[i].x >= dom || in[i].y >= dom || in[i].z >= dom || in[i].x % len || in[i].y % len || in[i].z % len)
      return DGO_EINVAL;
    if (in[i].lev > maxL) maxL = in[i].lev;
  }
  /* I[l]: sorted unique level-l Morton indices of internal nodes */
  u128 *I[32] = {0};
  size_t nI[32] = {0};
  int rc = 0;
  const uint64_t dom = (uint64_t)1 << D;
  for (int l = (int)maxL; l >= 1; l--) {
    size_t cnt = 0;
    for (size_t i = 0; i < n; i++) cnt += (in[i].lev == (unsigned)l);
    size_t cap = cnt + 8 * nI[l] + 1;
    u128 *cand = (u128 *)malloc(cap * sizeof(u128));
    if (!cand) {
      rc = DGO_ENOMEM;
      goto done;
    }
    size_t nc = 0;
    for (size_t i = 0; i < n; i++)
      if (in[i].lev == (unsigned)l) cand[nc++] = lvl_index(in[i].x, in[i].y, in[i].z, l - 1, D);
    const uint64_t s = (uint64_t)1 << (D - l); /* side at level l */
    for (size_t i = 0; i < nI[l]; i++) {
      uint32_t qx, qy, qz;
      level_index_decode(I[l][i], &qx, &qy, &qz); /* level-l coordinates */
      uint64_t q[3] = {(uint64_t)qx * s, (uint64_t)qy * s, (uint64_t)qz * s};
      int64_t opt[3][2];
      for (int a = 0; a < 3; a++) {
        uint64_t par = q[a] & ~(2 * s - 1);
        opt[a][0] = (int64_t)par;
        opt[a][1] = (q[a] & s) ? (int64_t)(par + 2 * s) : (int64_t)par - (int64_t)(2 * s);
      }
      for (int c = 0; c < 8; c++) {
        if (c == 7 && !incCorner) continue;
        int64_t p0 = opt[0][c & 1], p1 = opt[1][(c >> 1) & 1], p2 = opt[2][(c >> 2) & 1];
        if (p0 < 0 || p1 < 0 || p2 < 0 || p0 >= (int64_t)dom || p1 >= (int64_t)dom || p2 >= (int64_t)dom) continue;
        cand[nc++] = lvl_index((uint32_t)p0, (uint32_t)p1, (uint32_t)p2, l - 1, D);
      }
    }
    cmp_u128_unique(cand, &nc);
    I[l - 1] = cand;
    nI[l - 1] = nc;
  }
  {
    size_t total = 0;
    for (unsigned l = 0; l < maxL; l++) total += 8 * nI[l];
    dgo_oct *res = (dgo_oct *)malloc((total ? total : 1) * sizeof(dgo_oct));
    if (!res) {
      rc = DGO_ENOMEM;
      goto done;
    }
    size_t w = 0;
    for (unsigned l = 1; l <= maxL; l++) {
      const uint64_t s = (uint64_t)1 << (D - l);
      for (size_t i = 0; i < nI[l - 1]; i++) {
        for (int c = 0; c < 8; c++) {
          u128 ch = (I[l - 1][i] << 3) | (u128)c;
          if (u128_contains(I[l], nI[l], ch)) continue;
          uint32_t cx, cy, cz;
          level_index_decode(ch, &cx, &cy, &cz);
          dgo_oct o = {(uint32_t)(cx * s), (uint32_t)(cy * s), (uint32_t)(cz * s), l};
          res[w++] = o;
        }
      }
    }
    rc = sort_octs(res, w);
    if (rc) {
      free(res);
      goto done;
    }
    *out = res;
    *nout = w;
  }
done:
  for (int l = 0; l < 32; l++) free(I[l]);
  return rc;
}

int dgo_balance(const dgo_oct *in, size_t n, unsigned D, dgo_oct **out, size_t *nout) {
  return dgo_balance_ex(in, n, D, 1, out, nout);
}

/* ------------------------------------------------------------------------ */
/* coarsenOctree (src/coarsen.cpp:53-103): between consecutive first        */
/* children (Morton child number 0), when at least 8 octants separate them,  */
/* the first 8 are replaced by their parent and the rest are kept.           */
/* ------------------------------------------------------------------------ */
static unsigned child_number(const dgo_oct *o, unsigned D) {
  if (o->lev == 0) return 0;
  unsigned sh = D - o->lev;
  return ((o->x >> sh) & 1u) | (((o->y >> sh) & 1u) << 1) | (((o->z >> sh) & 1u) << 2);
}

int dgo_coarsen(const dgo_oct *in, size_t n, unsigned D, dgo_oct **out, size_t *nout) {
  dgo_oct *r = (dgo_oct *)malloc((n ? n : 1) * sizeof(dgo_oct));
  if (!r) return DGO_ENOMEM;
  size_t w = 0;
  if (n < 8) { /* coarsen.cpp:66-70 */
    for (size_t i = 0; i < n; i++) r[w++] = in[i];
  } else {
    size_t prev = 0;
    while (prev < n) {
      size_t curr = prev + 1;
      while (curr < n && child_number(&in[curr], D) != 0) curr++;
      if (curr >= prev + 8) {
        dgo_oct p = in[prev];
        unsigned pl = p.lev ? p.lev - 1 : 0, sh = D - pl;
        p.x = (p.x >> sh) << sh;
        p.y = (p.y >> sh) << sh;
        p.z = (p.z >> sh) << sh;
        p.lev = pl;
        r[w++] = p;
        for (size_t i = prev + 8; i < curr; i++) r[w++] = in[i];
      } else {
        for (size_t i = prev; i < curr; i++) r[w++] = in[i];
      }
      prev = curr;
    }
  }
  *out = r;
  *nout = w;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* completeOctree (src/construct.cpp:518).  At one rank the reference runs   */
/* completeSubtree and then, with its result overwritten, the general path    */
/* (:534-700) with one rank; that path is restated here.                      */
/* ------------------------------------------------------------------------ */
/* getNCA: the deepest octant that contains both */
static dgo_oct nca_of(const dgo_oct *a, const dgo_oct *b, unsigned D) {
  uint32_t d = (a->x ^ b->x) | (a->y ^ b->y) | (a->z ^ b->z);
  unsigned l = D;
  if (d) {
    unsigned h = 31u - (unsigned)__builtin_clz(d); /* highest differing bit */
    l = D - (h + 1);
  }
  if (a->lev < l) l = a->lev;
  if (b->lev < l) l = b->lev;
  uint32_t mask = ~((1u << (D - l)) - 1u);
  dgo_oct r = {a->x & mask, a->y & mask, a->z & mask, l};
  return r;
}

static dgo_oct parent_of(const dgo_oct *a, unsigned D) {
  unsigned l = a->lev ? a->lev - 1 : 0;
  uint32_t mask = ~((1u << (D - l)) - 1u);
  dgo_oct r = {a->x & mask, a->y & mask, a->z & mask, l};
  return r;
}

/* addChildren, Morton order: child c at x + (c&1)h, y + (c>>1&1)h, z + (c>>2)h */
static void children_of(const dgo_oct *p, unsigned D, dgo_oct kids[8]) {
  uint32_t h = (uint32_t)(oct_len(p, D) >> 1);
  for (unsigned c = 0; c < 8; c++) {
    dgo_oct k = {p->x + (c & 1u) * h, p->y + ((c >> 1) & 1u) * h, p->z + ((c >> 2) & 1u) * h, p->lev + 1};
    kids[c] = k;
  }
}

/* the top-down part of appendCompleteRegion (:1113-1142, :1172-1204): the
 * children of t before max, descending into the child that holds max */
static int region_top_down(dgo_oct t, const dgo_oct *max, unsigned D, oct_vec *v) {
  int rc, again;
  do {
    again = 0;
    dgo_oct kids[8];
    children_of(&t, D, kids);
    for (unsigned j = 0; j < 8; j++) {
      if (oct_lt(&kids[j], max) && !is_anc(&kids[j], max, D)) {
        if ((rc = ov_push(v, kids[j]))) return rc;
      } else if (is_anc(&kids[j], max, D)) {
        t = kids[j];
        again = 1;
        break;
      } else {
        break;
      }
    }
  } while (again);
  return 0;
}

/* appendCompleteRegion (:1077-1218) */
static int append_complete_region(dgo_oct first, dgo_oct second, oct_vec *v, int inc_min, int inc_max, unsigned D) {
  int rc;
  dgo_oct min = oct_lt(&first, &second) ? first : second;
  if (inc_min && (rc = ov_push(v, min))) return rc;
  if (oct_eq(&first, &second)) return 0;
  dgo_oct max = oct_lt(&second, &first) ? first : second;
  dgo_oct nca = nca_of(&min, &max, D);
  if (oct_eq(&min, &nca)) {
    if ((rc = region_top_down(min, &max, D, v))) return rc;
  } else {
    dgo_oct cur = min;
    while (oct_lt(&nca, &cur)) {
      dgo_oct par = parent_of(&cur, D), bros[8];
      children_of(&par, D, bros);
      for (unsigned i = 0; i < 8; i++) {
        if (oct_lt(&min, &bros[i]) && oct_lt(&bros[i], &max) && !is_anc(&bros[i], &max, D)) {
          if ((rc = ov_push(v, bros[i]))) return rc;
        } else if (is_anc(&bros[i], &max, D)) {
          if ((rc = region_top_down(bros[i], &max, D, v))) return rc;
          break;
        }
      }
      cur = par;
    }
  }
  if (inc_max && (rc = ov_push(v, max))) return rc;
  return 0;
}

int dgo_complete(const dgo_oct *in, size_t n, unsigned D, int is_unique, int is_sorted, dgo_oct **out, size_t *nout) {
  if (D > 30) return DGO_EINVAL;
  dgo_oct *a = (dgo_oct *)malloc((n ? n : 1) * sizeof(dgo_oct));
  if (!a) return DGO_ENOMEM;
  if (n) memcpy(a, in, n * sizeof(dgo_oct));
  int rc;
  if (!is_unique) {
    /* tree sort with TS_REMOVE_DUPLICATES (include/sfcSort.h:532-575): sort,
     * drop repeats, then replace every octant by its following descendant */
    if ((rc = sort_octs(a, n))) goto fail;
    size_t w = 0;
    for (size_t i = 0; i < n; i++)
      if (w == 0 || !oct_eq(&a[w - 1], &a[i])) a[w++] = a[i];
    size_t m = w;
    w = 0;
    for (size_t i = 0; i < m; i++) {
      if (w > 0 && is_anc(&a[w - 1], &a[i], D))
        a[w - 1] = a[i];
      else
        a[w++] = a[i];
    }
    n = w;
  } else if (!is_sorted) {
    if ((rc = sort_octs(a, n))) goto fail;
  }
  oct_vec v = {0, 0, 0};
  if (n) {
    oct_vec lst = {0, 0, 0};
    dgo_oct min_corner = {0, 0, 0, D}, root = {0, 0, 0, 0};
    dgo_oct max_corner = get_dld(&root, D);
    if (!oct_eq(&a[0], &min_corner) && !is_anc(&a[0], &min_corner, D)) { /* :598-607 */
      dgo_oct nc = nca_of(&a[0], &min_corner, D), kids[8];
      children_of(&nc, D, kids);
      if ((rc = ov_push(&lst, kids[0]))) goto fail_v;
    }
    for (size_t i = 0; i < n; i++)
      if ((rc = ov_push(&lst, a[i]))) goto fail_v;
    if (!oct_eq(&a[n - 1], &max_corner) && !is_anc(&a[n - 1], &max_corner, D)) { /* :610-622 */
      dgo_oct nc = nca_of(&a[n - 1], &max_corner, D), kids[8];
      children_of(&nc, D, kids);
      if ((rc = ov_push(&lst, kids[7]))) goto fail_v;
    }
    for (size_t i = 0; i + 1 < lst.n; i++) { /* :625-640 */
      int anc = is_anc(&lst.a[i], &lst.a[i + 1], D);
      if ((rc = append_complete_region(lst.a[i], lst.a[i + 1], &v, !anc, 0, D))) {
        free(lst.a);
        goto fail_v;
      }
    }
    rc = ov_push(&v, lst.a[lst.n - 1]); /* :645 */
    free(lst.a);
    if (rc) goto fail_v;
  }
  free(a);
  *out = v.a ? v.a : (dgo_oct *)malloc(sizeof(dgo_oct));
  *nout = v.n;
  return 0;
fail_v:
  free(v.a);
fail:
  free(a);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Hilbert order: TreeNode::operator< of the reference's default build       */
/* (-DHILBERT_ORDERING, include/TreeNode.tcc:130-210).  Its rotation tables  */
/* (src/hcurvedata.cpp:329-520) describe a self-similar curve: the base      */
/* cell visits its children in the order below, and each child cell carries */
/* its parent's symmetry composed with a fixed symmetry of its base corner.  */
/* The tables are generated here from those two rows.                        */
/* ------------------------------------------------------------------------ */
static const unsigned char hil_base[8] = {0, 2, 3, 1, 5, 7, 6, 4};
/* per base corner: new bit i of a corner = old bit perm[i] ^ bit i of flip */
static const unsigned char hil_child_perm[8][3] = {{0, 2, 1}, {2, 0, 1}, {2, 1, 0}, {0, 1, 2},
                                                   {0, 2, 1}, {2, 0, 1}, {2, 1, 0}, {0, 1, 2}};
static const unsigned char hil_child_flip[8] = {0, 6, 0, 0, 6, 3, 5, 0};

typedef struct {
  int n;                         /* states */
  unsigned char map[48][8];      /* each state's symmetry, as its corner map */
  unsigned char rank[48][8];     /* [state][corner] -> visit position */
  unsigned char next[48][8];     /* [state][corner] -> child's state */
} hil_tables;

static void hil_build(hil_tables *t) {
  unsigned char rank0[8];
  for (int k = 0; k < 8; k++) rank0[hil_base[k]] = (unsigned char)k;
  t->n = 1;
  for (int c = 0; c < 8; c++) t->map[0][c] = (unsigned char)c;
  for (int s = 0; s < t->n; s++) {
    unsigned char inv[8];
    for (int c = 0; c < 8; c++) inv[t->map[s][c]] = (unsigned char)c;
    for (int c = 0; c < 8; c++) {
      int c0 = inv[c];
      unsigned char child[8];
      for (int q = 0; q < 8; q++) {
        int r = 0;
        for (int i = 0; i < 3; i++) r |= (((q >> hil_child_perm[c0][i]) & 1) ^ ((hil_child_flip[c0] >> i) & 1)) << i;
        child[q] = t->map[s][r];
      }
      int id = 0;
      while (id < t->n && memcmp(t->map[id], child, 8) != 0) id++;
      if (id == t->n) memcpy(t->map[t->n++], child, 8);
      t->rank[s][c] = rank0[c0];
      t->next[s][c] = (unsigned char)id;
    }
  }
}

static unsigned bin_length(unsigned v) { /* binOp::binLength (src/binUtils.cpp:24) */
  unsigned len = 1;
  while (v > 1) {
    v >>= 1;
    len++;
  }
  return len;
}

/* TreeNode::operator< of the Hilbert build, step by step */
static int hil_lt(const dgo_oct *a, const dgo_oct *b, unsigned D, const hil_tables *t) {
  if (a->x == b->x && a->y == b->y && a->z == b->z) return a->lev < b->lev;
  if (a->lev > b->lev) {
    uint64_t len = (uint64_t)1 << (D - b->lev);
    if (!((a->x < b->x || a->x >= b->x + len) || (a->y < b->y || a->y >= b->y + len) ||
          (a->z < b->z || a->z >= b->z + len)))
      return 0;
  } else if (a->lev < b->lev) {
    uint64_t len = (uint64_t)1 << (D - a->lev);
    if (!((b->x < a->x || b->x >= a->x + len) || (b->y < a->y || b->y >= a->y + len) ||
          (b->z < a->z || b->z >= a->z + len)))
      return 1;
  }
  unsigned dx = a->x ^ b->x, dy = a->y ^ b->y, dz = a->z ^ b->z;
  unsigned md = dx > dy ? dx : dy;
  if (dz > md) md = dz;
  unsigned bl = bin_length(md);
  unsigned nx = (a->x >> bl) << bl, ny = (a->y >> bl) << bl, nz = (a->z >> bl) << bl;
  unsigned nca_lev = D - bl;
  int rot = 0;
  for (unsigned i = 0; i < nca_lev; i++) {
    unsigned m = D - i - 1;
    unsigned c = ((nz >> m) & 1u) << 2 | ((ny >> m) & 1u) << 1 | ((nx >> m) & 1u);
    rot = t->next[rot][c];
  }
  unsigned m = D - nca_lev - 1;
  unsigned c1 = ((a->z >> m) & 1u) << 2 | ((a->y >> m) & 1u) << 1 | ((a->x >> m) & 1u);
  unsigned c2 = ((b->z >> m) & 1u) << 2 | ((b->y >> m) & 1u) << 1 | ((b->x >> m) & 1u);
  return t->rank[rot][c1] < t->rank[rot][c2];
}

int dgo_hilbert_sort(dgo_oct *a, size_t n, unsigned D) {
  if (D > 30) return DGO_EINVAL;
  /* the reference's comparison is undefined outside the domain (its NCA
   * level underflows, TreeNode.tcc:176) */
  for (size_t i = 0; i < n; i++)
    if (a[i].lev > D || (a[i].x >> D) || (a[i].y >> D) || (a[i].z >> D)) return DGO_EINVAL;
  if (n < 2) return 0;
  hil_tables t;
  hil_build(&t);
  dgo_oct *tmp = (dgo_oct *)malloc(n * sizeof(dgo_oct));
  if (!tmp) return DGO_ENOMEM;
  /* bottom-up merge sort (stable) with the comparison above */
  dgo_oct *src = a, *dst = tmp;
  for (size_t w = 1; w < n; w *= 2) {
    for (size_t lo = 0; lo < n; lo += 2 * w) {
      size_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      size_t i = lo, j = mid, k = lo;
      while (i < mid && j < hi) dst[k++] = hil_lt(&src[j], &src[i], D, &t) ? src[j++] : src[i++];
      while (i < mid) dst[k++] = src[i++];
      while (j < hi) dst[k++] = src[j++];
    }
    dgo_oct *sw = src;
    src = dst;
    dst = sw;
  }
  if (src != a) memcpy(a, src, n * sizeof(dgo_oct));
  free(tmp);
  return 0;
}

int dgo_hilbert_states(void) {
  hil_tables t;
  hil_build(&t);
  return t.n;
}

/* ------------------------------------------------------------------------ */
/* checkers                                                                  */
/* ------------------------------------------------------------------------ */
int dgo_is_sorted_unique(const dgo_oct *a, size_t n, unsigned D) {
  (void)D;
  for (size_t i = 1; i < n; i++)
    if (!(okey(&a[i - 1]) < okey(&a[i]))) return 0;
  return 1;
}

int dgo_is_linear(const dgo_oct *a, size_t n, unsigned D) {
  for (size_t i = 1; i < n; i++)
    if (is_anc(&a[i - 1], &a[i], D)) return 0;
  return 1;
}

/* complete + linear + sorted: consecutive leaves abut in Morton index space
 * and the leaves tile the root */
int dgo_is_complete(const dgo_oct *a, size_t n, unsigned D) {
  if (n == 0) return 0;
  u128 pos = 0;
  for (size_t i = 0; i < n; i++) {
    if (morton(a[i].x, a[i].y, a[i].z) != pos) return 0;
    pos += (u128)1 << (3 * (D - a[i].lev));
  }
  return pos == ((u128)1 << (3 * D));
}

/* index of the leaf containing the level-D cell at (x,y,z); n if none */
static size_t find_leaf(const u128 *keys, size_t n, uint32_t x, uint32_t y, uint32_t z) {
  u128 k = morton(x, y, z);
  size_t lo = 0, hi = n;
  while (lo < hi) { /* first key > k */
    size_t mid = lo + (hi - lo) / 2;
    if (keys[mid] <= k)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo == 0 ? n : lo - 1;
}

int dgo_is_balanced_ex(const dgo_oct *a, size_t n, unsigned D, int incCorner) {
  u128 *keys = (u128 *)malloc((n ? n : 1) * sizeof(u128));
  if (!keys) return 0;
  for (size_t i = 0; i < n; i++) keys[i] = morton(a[i].x, a[i].y, a[i].z);
  const int64_t dom = (int64_t)1 << D;
  int ok = 1;
  for (size_t i = 0; i < n && ok; i++) {
    int64_t s = (int64_t)1 << (D - a[i].lev);
    for (int dz = -1; dz <= 1 && ok; dz++)
      for (int dy = -1; dy <= 1 && ok; dy++)
        for (int dx = -1; dx <= 1 && ok; dx++) {
          if (!dx && !dy && !dz) continue;
          if (!incCorner && dx && dy && dz) continue;
          int64_t nx = a[i].x + dx * s, ny = a[i].y + dy * s, nz = a[i].z + dz * s;
          if (nx < 0 || ny < 0 || nz < 0 || nx >= dom || ny >= dom || nz >= dom) continue;
          size_t j = find_leaf(keys, n, (uint32_t)nx, (uint32_t)ny, (uint32_t)nz);
          if (j == n || a[j].lev + 1 < a[i].lev) ok = 0;
        }
  }
  free(keys);
  return ok;
}

int dgo_is_balanced(const dgo_oct *a, size_t n, unsigned D) { return dgo_is_balanced_ex(a, n, D, 1); }

uint64_t dgo_fnv1a(const dgo_oct *a, size_t n) {
  uint64_t h = 1469598103934665603ull;
  const unsigned char *p = (const unsigned char *)a;
  for (size_t i = 0; i < n * sizeof(dgo_oct); i++) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

/* ------------------------------------------------------------------------ */
/* element types and stencils                                                */
/* ------------------------------------------------------------------------ */
/* The 18 hanging configurations of a child, as sets of vertices relative to
 * the child's own corner (vertex c XOR r), in the reference's type order
 * (include/oda/odaUtils.tcc:14-120, names of include/oda/cnumEtypes.h):
 * r = 1,2,4 are the three edge midpoints, 3,5,6 the three face centres. */
static const uint8_t k_canon_rel[18] = {
    0x00,                        /* N */
    1u << 2, 1u << 1,            /* Y, X */
    (1u << 1) | (1u << 2),       /* XY */
    1u << 4,                     /* Z */
    (1u << 2) | (1u << 4),       /* ZY */
    (1u << 1) | (1u << 4),       /* ZX */
    (1u << 1) | (1u << 2) | (1u << 4),                       /* ZXY */
    (1u << 1) | (1u << 2) | (1u << 3),                       /* XY_XY */
    (1u << 1) | (1u << 2) | (1u << 3) | (1u << 4),           /* XY_ZXY */
    (1u << 2) | (1u << 4) | (1u << 6),                       /* YZ_ZY */
    (1u << 1) | (1u << 2) | (1u << 4) | (1u << 6),           /* YZ_ZXY */
    (1u << 1) | (1u << 2) | (1u << 3) | (1u << 4) | (1u << 6), /* YZ_XY_ZXY */
    (1u << 1) | (1u << 4) | (1u << 5),                       /* ZX_ZX */
    (1u << 1) | (1u << 2) | (1u << 4) | (1u << 5),           /* ZX_ZXY */
    (1u << 1) | (1u << 2) | (1u << 3) | (1u << 4) | (1u << 5), /* ZX_XY_ZXY */
    (1u << 1) | (1u << 2) | (1u << 4) | (1u << 5) | (1u << 6), /* ZX_YZ_ZXY */
    0x7e                                                     /* ZX_YZ_XY_ZXY */
};
/* Per child number, the axis bit that the canonical X, Y and Z axes of the
 * configuration names map to (each child's table is the canonical one with
 * its axes permuted). */
static const uint8_t k_axis_perm[8][3] = {{1, 2, 4}, {2, 1, 4}, {2, 1, 4}, {1, 2, 4},
                                          {1, 4, 2}, {2, 4, 1}, {2, 4, 1}, {1, 4, 2}};

void dgo_etype_masks(uint8_t masks[8 * 18]) {
  for (int c = 0; c < 8; c++)
    for (int t = 0; t < 18; t++) {
      uint8_t m = 0;
      for (int r = 0; r < 8; r++) {
        if (!(k_canon_rel[t] >> r & 1)) continue;
        int pr = ((r & 1) ? k_axis_perm[c][0] : 0) | ((r & 2) ? k_axis_perm[c][1] : 0) |
                 ((r & 4) ? k_axis_perm[c][2] : 0);
        m |= (uint8_t)(1u << (pr ^ c));
      }
      masks[c * 18 + t] = m;
    }
}

/* trilinear element matrices on [-1,1]^3, vertex k = (k&1, k>>1&1, k>>2&1) */
static void element_matrices(double K[8][8], double Ms[8][8]) {
  const double m1[2][2] = {{2.0 / 3.0, 1.0 / 3.0}, {1.0 / 3.0, 2.0 / 3.0}};
  const double a1[2][2] = {{0.5, -0.5}, {-0.5, 0.5}};
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 8; j++) {
      int ix = i & 1, iy = i >> 1 & 1, iz = i >> 2 & 1;
      int jx = j & 1, jy = j >> 1 & 1, jz = j >> 2 & 1;
      K[i][j] = a1[ix][jx] * m1[iy][jy] * m1[iz][jz] + m1[ix][jx] * a1[iy][jy] * m1[iz][jz] +
                m1[ix][jx] * m1[iy][jy] * a1[iz][jz];
      Ms[i][j] = m1[ix][jx] * m1[iy][jy] * m1[iz][jz];
    }
}

/* interpolation: child vertex values from the 8 referenced values */
static void hanging_interp(int c, uint8_t mask, double P[8][8]) {
  memset(P, 0, 64 * sizeof(double));
  for (int k = 0; k < 8; k++) {
    if (!(mask >> k & 1)) {
      P[k][k] = 1.0;
      continue;
    }
    int d = k ^ c, cnt = 0;
    for (int s = 0; s < 8; s++)
      if ((s & d) == s) cnt++;
    for (int s = 0; s < 8; s++)
      if ((s & d) == s) P[k][c ^ s] += 1.0 / cnt;
  }
}

void dgo_stencils(double *lap, double *mass) {
  double K[8][8], Ms[8][8], P[8][8];
  uint8_t masks[8 * 18];
  element_matrices(K, Ms);
  dgo_etype_masks(masks);
  for (int c = 0; c < 8; c++)
    for (int t = 0; t < 18; t++) {
      hanging_interp(c, masks[c * 18 + t], P);
      for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++) {
          double sl = 0.0, sm = 0.0;
          for (int a = 0; a < 8; a++)
            for (int b = 0; b < 8; b++) {
              double w = P[a][i] * P[b][j];
              if (w != 0.0) {
                sl += w * K[a][b];
                sm += w * Ms[a][b];
              }
            }
          size_t o = (((size_t)c * 18 + t) * 8 + i) * 8 + j;
          if (lap) lap[o] = sl;
          if (mass) mass[o] = sm;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* DA                                                                        */
/* ------------------------------------------------------------------------ */
void dgo_da_free(dgo_da *da) {
  free(da->child);
  free(da->hmask);
  free(da->etype);
  free(da->level);
  free(da->nodes);
  free(da->node_xyz);
  memset(da, 0, sizeof(*da));
}

/* is the octant (x,y,z,lev) a leaf of the sorted linear octree? */
static int is_leaf_at(const dgo_oct *a, const u128 *keys, size_t n, int64_t x, int64_t y, int64_t z, unsigned lev,
                      unsigned D) {
  const int64_t dom = (int64_t)1 << D;
  if (x < 0 || y < 0 || z < 0 || x >= dom || y >= dom || z >= dom) return 0;
  size_t j = find_leaf(keys, n, (uint32_t)x, (uint32_t)y, (uint32_t)z);
  return j < n && a[j].lev == lev && a[j].x == (uint32_t)x && a[j].y == (uint32_t)y && a[j].z == (uint32_t)z;
}

static size_t find_node(const u128 *nk, size_t nn, u128 k) {
  size_t lo = 0, hi = nn;
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (nk[mid] < k)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < nn && nk[lo] == k) ? lo : (size_t)-1;
}

int dgo_da_build(const dgo_oct *a, size_t n, unsigned D, dgo_da *da) {
  memset(da, 0, sizeof(*da));
  if (n == 0 || D > 30) return DGO_EINVAL;
  int rc = 0;
  uint8_t emask[8 * 18], tmap[8][256];
  dgo_etype_masks(emask);
  memset(tmap, 0xff, sizeof(tmap));
  for (int c = 0; c < 8; c++)
    for (int t = 0; t < 18; t++) tmap[c][emask[c * 18 + t]] = (uint8_t)t;

  u128 *keys = (u128 *)malloc(n * sizeof(u128));
  da->child = (uint8_t *)malloc(n);
  da->hmask = (uint8_t *)malloc(n);
  da->etype = (uint8_t *)malloc(n);
  da->level = (uint8_t *)malloc(n);
  da->nodes = (uint32_t *)malloc(8 * n * sizeof(uint32_t));
  u128 *nk = (u128 *)malloc(8 * n * sizeof(u128));
  if (!keys || !da->child || !da->hmask || !da->etype || !da->level || !da->nodes || !nk) {
    rc = DGO_ENOMEM;
    goto fail;
  }
  for (size_t i = 0; i < n; i++) keys[i] = morton(a[i].x, a[i].y, a[i].z);
  const int64_t dom = (int64_t)1 << D;
  size_t nn = 0;
  for (size_t e = 0; e < n; e++) {
    const unsigned l = a[e].lev;
    const int64_t h = (int64_t)1 << (D - l);
    const int64_t x = a[e].x, y = a[e].y, z = a[e].z;
    /* Morton child number (include/oda/oda.tcc:1273-1302) */
    int c = 0;
    if (l > 0) c = (int)(((x / h) & 1) | (((y / h) & 1) << 1) | (((z / h) & 1) << 2));
    uint8_t hm = 0;
    if (l > 1) {
      const int64_t H = 2 * h; /* parent side */
      const int64_t P[3] = {x - ((c & 1) ? h : 0), y - ((c & 2) ? h : 0), z - ((c & 4) ? h : 0)};
      /* shift of the parent towards the child's exterior along each axis */
      const int64_t d[3] = {(c & 1) ? H : -H, (c & 2) ? H : -H, (c & 4) ? H : -H};
      for (int r = 1; r < 7; r++) {
        if (r == 7) continue;
        /* vertex c^r: midpoint along the axes in r; on the parent's boundary
         * (side c) along the others.  It hangs when one of the parent's
         * neighbours sharing that face/edge is an unrefined leaf. */
        int others = 7 & ~r, hang = 0;
        for (int s = 1; s < 8 && !hang; s++) {
          if ((s & others) != s) continue;
          int64_t q[3] = {P[0], P[1], P[2]};
          for (int ax = 0; ax < 3; ax++)
            if (s >> ax & 1) q[ax] += d[ax];
          if (is_leaf_at(a, keys, n, q[0], q[1], q[2], l - 1, D)) hang = 1;
        }
        if (hang) hm |= (uint8_t)(1u << (c ^ r));
      }
    }
    da->child[e] = (uint8_t)c;
    da->hmask[e] = hm;
    da->level[e] = (uint8_t)l;
    if (tmap[c][hm] == 0xff) {
      rc = DGO_EINTERNAL; /* not a 2:1 balanced configuration */
      goto fail;
    }
    da->etype[e] = tmap[c][hm];
    /* nodes owned by this element: anchor, and vertices on the positive
     * domain boundary that no other element anchors */
    int bdy = ((x + h == dom) ? 1 : 0) | ((y + h == dom) ? 2 : 0) | ((z + h == dom) ? 4 : 0);
    for (int k = 0; k < 8; k++) {
      if ((k & bdy) != k || (hm >> k & 1)) continue;
      nk[nn++] = morton((uint32_t)(x + ((k & 1) ? h : 0)), (uint32_t)(y + ((k & 2) ? h : 0)),
                        (uint32_t)(z + ((k & 4) ? h : 0)));
    }
  }
  cmp_u128_unique(nk, &nn);
  da->n_elem = n;
  da->n_node = nn;
  da->node_xyz = (uint32_t *)malloc((nn ? 3 * nn : 3) * sizeof(uint32_t));
  if (!da->node_xyz) {
    rc = DGO_ENOMEM;
    goto fail;
  }
  for (size_t i = 0; i < nn; i++)
    level_index_decode(nk[i], &da->node_xyz[3 * i], &da->node_xyz[3 * i + 1], &da->node_xyz[3 * i + 2]);
  for (size_t e = 0; e < n; e++) {
    const int64_t h = (int64_t)1 << (D - a[e].lev);
    const int c = da->child[e];
    const int64_t x = a[e].x, y = a[e].y, z = a[e].z;
    const int64_t px = x - ((c & 1) ? h : 0), py = y - ((c & 2) ? h : 0), pz = z - ((c & 4) ? h : 0);
    for (int k = 0; k < 8; k++) {
      int64_t vx, vy, vz;
      if (da->hmask[e] >> k & 1) {
        vx = px + ((k & 1) ? 2 * h : 0);
        vy = py + ((k & 2) ? 2 * h : 0);
        vz = pz + ((k & 4) ? 2 * h : 0);
      } else {
        vx = x + ((k & 1) ? h : 0);
        vy = y + ((k & 2) ? h : 0);
        vz = z + ((k & 4) ? h : 0);
      }
      size_t id = find_node(nk, nn, morton((uint32_t)vx, (uint32_t)vy, (uint32_t)vz));
      if (id == (size_t)-1) {
        rc = DGO_EINTERNAL;
        goto fail;
      }
      da->nodes[8 * e + k] = (uint32_t)id;
    }
  }
  free(keys);
  free(nk);
  return 0;
fail:
  free(keys);
  free(nk);
  dgo_da_free(da);
  return rc;
}

int dgo_matvec(const dgo_da *da, unsigned D, const double *in, double *out, double lapFac, double massFac) {
  static double L[8 * 18 * 64], M[8 * 18 * 64];
  static int have = 0;
  if (!have) {
    dgo_stencils(L, M);
    have = 1;
  }
  memset(out, 0, da->n_node * sizeof(double));
  for (size_t e = 0; e < da->n_elem; e++) {
    /* odaJac.C:311-313 + :276-279: h = hFac * 2^(maxD - lev) with the DA's
     * maxD = D + 1 and DA level = level + 1, i.e. h = 2^-level */
    double h = 1.0 / (double)((uint64_t)1 << da->level[e]);
    double f1 = lapFac * h / 2.0, f2 = massFac * h * h * h / 8.0;
    const double *Ls = &L[((size_t)da->child[e] * 18 + da->etype[e]) * 64];
    const double *Ms = &M[((size_t)da->child[e] * 18 + da->etype[e]) * 64];
    const uint32_t *id = &da->nodes[8 * e];
    for (int k = 0; k < 8; k++) {
      double acc = 0.0;
      for (int j = 0; j < 8; j++) acc += (f1 * Ls[8 * k + j] + f2 * Ms[8 * k + j]) * in[id[j]];
      out[id[k]] += acc;
    }
  }
  (void)D;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* multigrid building blocks (examples/src/backend/omgJac.C, src/omg/*)      */
/* ------------------------------------------------------------------------ */
/* boundary flag per node: a node on the boundary of the unit cube
 * (assignBoundaryFlags, src/oda/odaUtils.cpp:2464) */
static int node_on_bdy(const dgo_da *da, size_t i, unsigned D) {
  const uint32_t dom = 1u << D, *p = &da->node_xyz[3 * i];
  return p[0] == 0 || p[1] == 0 || p[2] == 0 || p[0] == dom || p[1] == dom || p[2] == dom;
}

/* DirichletJacobianMatMult (omgJac.C:958-1057): boundary rows identity,
 * boundary columns skipped */
int dgo_dirichlet_matvec(const dgo_da *da, unsigned D, const double *in, double *out) {
  static double L[8 * 18 * 64], M[8 * 18 * 64];
  static int have = 0;
  if (!have) {
    dgo_stencils(L, M);
    have = 1;
  }
  memset(out, 0, da->n_node * sizeof(double));
  for (size_t e = 0; e < da->n_elem; e++) {
    double h = 1.0 / (double)((uint64_t)1 << da->level[e]);
    double f1 = h / 2.0, f2 = h * h * h / 8.0;
    const double *Ls = &L[((size_t)da->child[e] * 18 + da->etype[e]) * 64];
    const double *Ms = &M[((size_t)da->child[e] * 18 + da->etype[e]) * 64];
    const uint32_t *id = &da->nodes[8 * e];
    for (int k = 0; k < 8; k++) {
      if (node_on_bdy(da, id[k], D)) {
        out[id[k]] = in[id[k]];
        continue;
      }
      for (int j = 0; j < 8; j++)
        if (!node_on_bdy(da, id[j], D)) out[id[k]] += (f1 * Ls[8 * k + j] + f2 * Ms[8 * k + j]) * in[id[j]];
    }
  }
  return 0;
}

/* diagonal of the Dirichlet operator (1 on the boundary) */
int dgo_dirichlet_diag(const dgo_da *da, unsigned D, double *diag) {
  double L[8 * 18 * 64], M[8 * 18 * 64];
  dgo_stencils(L, M);
  memset(diag, 0, da->n_node * sizeof(double));
  for (size_t e = 0; e < da->n_elem; e++) {
    double h = 1.0 / (double)((uint64_t)1 << da->level[e]);
    double f1 = h / 2.0, f2 = h * h * h / 8.0;
    const double *Ls = &L[((size_t)da->child[e] * 18 + da->etype[e]) * 64];
    const double *Ms = &M[((size_t)da->child[e] * 18 + da->etype[e]) * 64];
    for (int k = 0; k < 8; k++) {
      uint32_t id = da->nodes[8 * e + k];
      if (node_on_bdy(da, id, D)) diag[id] = 1.0;
      else diag[id] += f1 * Ls[9 * k] + f2 * Ms[9 * k];
    }
  }
  return 0;
}

/* prolongation from a coarse level onto the nodes of a fine level: for every
 * fine node the coarse element holding it (restrictMatVec.cpp:74-146 loops
 * over coarse elements and their fine children with the RmatType1/2
 * stencils; the weights are the coarse shape functions at the fine vertex,
 * folded through the coarse element's hanging interpolation).  Pairs with a
 * boundary node on either level carry no weight.  ids/w: 8 per fine node. */
int dgo_prolong_map(const dgo_da *fine, const dgo_oct *coarse_oct, size_t nc, const dgo_da *coarse, unsigned D,
                    uint32_t *ids, double *w) {
  u128 *keys = (u128 *)malloc((nc ? nc : 1) * sizeof(u128));
  if (!keys) return DGO_ENOMEM;
  for (size_t i = 0; i < nc; i++) keys[i] = morton(coarse_oct[i].x, coarse_oct[i].y, coarse_oct[i].z);
  const uint32_t dom = 1u << D;
  uint8_t masks[8 * 18];
  dgo_etype_masks(masks);
  int rc = 0;
  for (size_t v = 0; v < fine->n_node; v++) {
    const uint32_t *p = &fine->node_xyz[3 * v];
    uint32_t q[3];
    for (int a = 0; a < 3; a++) q[a] = p[a] == dom ? dom - 1 : p[a];
    size_t e = find_leaf(keys, nc, q[0], q[1], q[2]);
    if (e == nc) {
      rc = DGO_EINTERNAL;
      break;
    }
    const dgo_oct *ce = &coarse_oct[e];
    uint64_t h = (uint64_t)1 << (D - ce->lev);
    uint32_t an[3] = {ce->x, ce->y, ce->z};
    int xi2[3];
    for (int a = 0; a < 3; a++) {
      uint64_t d = (uint64_t)p[a] - an[a];
      if (d == 0) xi2[a] = 0;
      else if (2 * d == h) xi2[a] = 1;
      else if (d == h) xi2[a] = 2;
      else {
        rc = DGO_EINTERNAL;
        goto done;
      }
    }
    double P[8][8];
    hanging_interp(coarse->child[e], masks[coarse->child[e] * 18 + coarse->etype[e]], P);
    int fb = node_on_bdy(fine, v, D);
    for (int j = 0; j < 8; j++) {
      double wj = 0.0;
      for (int k = 0; k < 8; k++) {
        double Nk = 1.0;
        for (int a = 0; a < 3; a++) {
          double t = 0.5 * xi2[a];
          Nk *= ((k >> a) & 1) ? t : 1.0 - t;
        }
        wj += Nk * P[k][j];
      }
      uint32_t cid = coarse->nodes[8 * e + j];
      ids[8 * v + j] = cid;
      w[8 * v + j] = (fb || node_on_bdy(coarse, cid, D)) ? 0.0 : wj;
    }
  }
done:
  free(keys);
  return rc;
}

/* The restriction stencils the reference reads from RmatType1Stencils.inp
 * ([cNumCoarse][cNumFine][type][coarse j][fine vertex f]) and
 * RmatType2Stencils.inp ([cNum][type][j][f]) (rmatType1StencilsAux.cpp:14,
 * rmatType2StencilsAux.cpp:15), restated: the coarse element's shape
 * functions at the fine vertex, folded through its hanging interpolation. */
void dgo_rmat_tables(double *r1, double *r2) {
  uint8_t masks[8 * 18];
  dgo_etype_masks(masks);
  for (int cc = 0; cc < 8; cc++)
    for (int t = 0; t < 18; t++) {
      double P[8][8];
      hanging_interp(cc, masks[cc * 18 + t], P);
      for (int j = 0; j < 8; j++)
        for (int f = 0; f < 8; f++) r2[((cc * 18 + t) * 8 + j) * 8 + f] = P[f][j];
      for (int cf = 0; cf < 8; cf++)
        for (int f = 0; f < 8; f++) {
          double N[8];
          for (int k = 0; k < 8; k++) {
            double v = 1.0;
            for (int a = 0; a < 3; a++) {
              double xi = 0.5 * (((cf >> a) & 1) + ((f >> a) & 1));
              v *= ((k >> a) & 1) ? xi : 1.0 - xi;
            }
            N[k] = v;
          }
          for (int j = 0; j < 8; j++) {
            double w = 0.0;
            for (int k = 0; k < 8; k++) w += N[k] * P[k][j];
            r1[((((size_t)cc * 8 + cf) * 18 + t) * 8 + j) * 8 + f] = w;
          }
        }
    }
}
