// GPU quadtree construction for the boundary-node FMM.
//
// The reference bins the nodes into a uniform 2^l x 2^l grid at every level with a
// counting sort (ASSIGN1, cadap2.f:252-409) and loops over all 4^l boxes, empty or
// not (DOINT0DR, cadapdrop2.f:84-197). Here the nodes are sorted once by a Morton key
// at depth 20; the occupied boxes of every level are then the distinct key prefixes,
// each owning a contiguous range of the sorted nodes. Only occupied boxes exist.
// The tree is adaptive: below a uniform floor (the shallowest level of mean occupancy at
// most `leaf_target`), a box with more than `leaf_cap` points is split (DAASSI,
// dapif1.f:1165-1255, with NAPB = leaf_cap); every point's leaf level follows from the
// keys of the points leaf_cap places before and after it in sorted order. V lists follow MKINTL
// (cadap2.f:780-828: children of the parent's neighbours that are not adjacent, at most
// 27); the leaves' U and W lists follow DALI12/DALI34 (dapif2.f:3-356) for leaves of
// different levels.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>

#include <atomic>
#include <mutex>

#include "eb_internal.h"

namespace {

struct __align__(16) Box4 {
  double x, y, z, w;
};
__host__ __device__ __forceinline__ Box4 mk_box4(double a, double b, double c, double d) {
  Box4 r;
  r.x = a; r.y = b; r.z = c; r.w = d;
  return r;
}

__host__ __device__ __forceinline__ unsigned long long spread2(unsigned int v) {
  unsigned long long x = v;
  x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
  x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
  x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}
__host__ __device__ __forceinline__ unsigned int compact2(unsigned long long x) {
  x &= 0x5555555555555555ull;
  x = (x | (x >> 1)) & 0x3333333333333333ull;
  x = (x | (x >> 2)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x >> 4)) & 0x00FF00FF00FF00FFull;
  x = (x | (x >> 8)) & 0x0000FFFF0000FFFFull;
  x = (x | (x >> 16)) & 0x00000000FFFFFFFFull;
  return (unsigned int)x;
}
__host__ __device__ __forceinline__ unsigned long long morton(unsigned int ix, unsigned int iy) {
  return spread2(ix) | (spread2(iy) << 1);
}

__global__ void k_bbox(const double2* __restrict__ z, int n, Box4* __restrict__ part,
                       int* __restrict__ bad) {
  __shared__ double s[4][256];
  double mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
  int nonfinite = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 p = z[i];
    if (!isfinite(p.x) || !isfinite(p.y)) { nonfinite = 1; continue; }
    mnx = fmin(mnx, p.x); mxx = fmax(mxx, p.x);
    mny = fmin(mny, p.y); mxy = fmax(mxy, p.y);
  }
  if (nonfinite) atomicOr(bad, 1);
  s[0][threadIdx.x] = mnx; s[1][threadIdx.x] = mxx; s[2][threadIdx.x] = mny; s[3][threadIdx.x] = mxy;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s[0][threadIdx.x] = fmin(s[0][threadIdx.x], s[0][threadIdx.x + o]);
      s[1][threadIdx.x] = fmax(s[1][threadIdx.x], s[1][threadIdx.x + o]);
      s[2][threadIdx.x] = fmin(s[2][threadIdx.x], s[2][threadIdx.x + o]);
      s[3][threadIdx.x] = fmax(s[3][threadIdx.x], s[3][threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = mk_box4(s[0][0], s[1][0], s[2][0], s[3][0]);
}

// The bounding box and the root square sq = (W, x0, y0, 2^20 / W): the box's larger
// side widened by 1e-9 relative, centred on the box (W = 1 for a single point).
__global__ void k_bbox_final(const Box4* __restrict__ part, int nb, Box4* __restrict__ out,
                             double* __restrict__ sq, int wall, int* __restrict__ bad) {
  __shared__ Box4 sb[256];
  Box4 r = mk_box4(INFINITY, -INFINITY, INFINITY, -INFINITY);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    Box4 p = part[i];
    r.x = fmin(r.x, p.x); r.y = fmax(r.y, p.y); r.z = fmin(r.z, p.z); r.w = fmax(r.w, p.w);
  }
  sb[threadIdx.x] = r;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const Box4 q = sb[threadIdx.x + o];
      Box4& a = sb[threadIdx.x];
      a.x = fmin(a.x, q.x); a.y = fmax(a.y, q.y); a.z = fmin(a.z, q.z); a.w = fmax(a.w, q.w);
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  r = sb[0];
  *out = r;
  if (wall) {
    // the square [xleft, xleft + slength] x [0, slength] of the wall-bounded CADAPDR
    // (cadapdrop.f:142-145), widened by 1e-9 so that no key needs clamping
    if (!(r.z >= 0.0)) atomicOr(bad, 2);
    double w = fmax(__dadd_rn(r.y, -r.x), r.w);
    if (!(w > 0)) w = 1.0;
    w = __dmul_rn(w, 1.0 + 1e-9);
    sq[0] = w;
    sq[1] = r.x;
    sq[2] = 0.0;
    sq[3] = __ddiv_rn((double)(1u << EB_KEY_LEVELS), w);
    return;
  }
  double w = fmax(__dadd_rn(r.y, -r.x), __dadd_rn(r.w, -r.z));
  if (!(w > 0)) w = 1.0;
  w = __dmul_rn(w, 1.0 + 1e-9);
  sq[0] = w;
  sq[1] = __dadd_rn(__dmul_rn(0.5, __dadd_rn(r.x, r.y)), -__dmul_rn(0.5, w));
  sq[2] = __dadd_rn(__dmul_rn(0.5, __dadd_rn(r.z, r.w)), -__dmul_rn(0.5, w));
  sq[3] = __ddiv_rn((double)(1u << EB_KEY_LEVELS), w);
}

// An explicit root square (a forest of independent problems in a grid of cells).
__global__ void k_set_square(double W, double x0, double y0, double* __restrict__ sq) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  sq[0] = W;
  sq[1] = x0;
  sq[2] = y0;
  sq[3] = __ddiv_rn((double)(1u << EB_KEY_LEVELS), W);
}

__global__ void k_keys(const double2* __restrict__ z, int n, const double* __restrict__ sq,
                       unsigned long long* __restrict__ keys, int* __restrict__ idx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x0 = sq[1], y0 = sq[2], inv_cell = sq[3];
  const double maxc = (double)((1u << EB_KEY_LEVELS) - 1);
  double fx = floor((z[i].x - x0) * inv_cell), fy = floor((z[i].y - y0) * inv_cell);
  fx = fmin(fmax(fx, 0.0), maxc);
  fy = fmin(fmax(fy, 0.0), maxc);
  keys[i] = morton((unsigned int)fx, (unsigned int)fy);
  idx[i] = i;
}

// sorted positions, also as float hi + lo pairs packed (hi.x, hi.y, lo.x, lo.y)
__global__ void k_gather_points(const double2* __restrict__ z, const int* __restrict__ perm,
                                int n, double2* __restrict__ zs, float4* __restrict__ zhl) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 p = z[perm[i]];
  zs[i] = p;
  float hx = (float)p.x, hy = (float)p.y;
  zhl[i] = make_float4(hx, hy, (float)(p.x - (double)hx), (float)(p.y - (double)hy));
}

// The points of a direct tree in their given order, with the float hi + lo copies, and a
// flag for a non-finite coordinate.
__global__ void k_direct_points(const double2* __restrict__ z, int n, int* __restrict__ perm,
                                double2* __restrict__ zs, float4* __restrict__ zhl, int* __restrict__ bad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 p = z[i];
  if (!isfinite(p.x) || !isfinite(p.y)) atomicOr(bad, 1);
  perm[i] = i;
  zs[i] = p;
  float hx = (float)p.x, hy = (float)p.y;
  zhl[i] = make_float4(hx, hy, (float)(p.x - (double)hx), (float)(p.y - (double)hy));
}

// Histogram of the first level at which consecutive sorted keys fall in different boxes:
// the occupied boxes of level l in a uniform tree number 1 + sum_{l' <= l} hist[l'].
__global__ void k_level_hist(const unsigned long long* __restrict__ keys, int n, int* __restrict__ hist) {
  __shared__ int sh[EB_KEY_LEVELS + 1];
  for (int i = threadIdx.x; i <= EB_KEY_LEVELS; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long x = keys[i] ^ keys[i - 1];
    if (x == 0) continue;
    const int hb = 63 - __clzll((long long)x);
    atomicAdd(&sh[EB_KEY_LEVELS - hb / 2], 1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= EB_KEY_LEVELS; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// The minimum leaf level: for one problem the shallowest level whose occupied boxes
// hold at most `target` points on average (a uniform floor, which keeps leaves of one
// level, and so no W lists, wherever the points are evenly spread), for a forest the
// level of its cells.
__global__ void k_pick_level(int n, int target, int R, const int* __restrict__ hist, int* __restrict__ lmin) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int L0 = EB_KEY_LEVELS, nb = 1;
  for (int l = 0; l <= EB_KEY_LEVELS; ++l) {
    if (l > 0) nb += hist[l];
    if ((double)n / nb <= (double)target) {
      L0 = l;
      break;
    }
  }
  *lmin = R > 0 ? R : L0;
}

// Levels shared by the keys a and b: the deepest level whose box holds both
// (EB_KEY_LEVELS when the keys are equal, -1 never: the root holds every point).
__device__ __forceinline__ int shared_levels(unsigned long long a, unsigned long long b) {
  const unsigned long long x = a ^ b;
  if (x == 0ull) return EB_KEY_LEVELS;
  const int hb = 63 - __clzll((long long)x);
  return EB_KEY_LEVELS - 1 - hb / 2;
}

// lcpw[w] = levels shared by sorted points w and w + cap (w < n - cap). The box of level
// l around a point holds more than cap points exactly when some window [w, w + cap]
// containing the point has lcpw[w] >= l (a box is a contiguous range of sorted points).
__global__ void k_lcp_window(const unsigned long long* __restrict__ keys, int n, int cap,
                             unsigned char* __restrict__ lcpw) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n - cap) return;
  lcpw[w] = (unsigned char)shared_levels(keys[w], keys[w + cap]);
}

// Leaf level of every sorted point: one more than the deepest level whose box around the
// point holds more than cap points, at most EB_KEY_LEVELS (coincident points), 0 when
// n <= cap, and at least lmin (k_pick_level). Also the deepest leaf level and the number of boxes of every level l >= 1:
// a point starts a box of level l when l <= its leaf level and its key differs from the
// previous point's at level l.
__global__ void k_leaf_level(const unsigned long long* __restrict__ keys, int n, int cap,
                             const int* __restrict__ lmin_d, const unsigned char* __restrict__ lcpw,
                             unsigned char* __restrict__ plev, int* __restrict__ lmax, int* __restrict__ hist) {
  const int lmin = *lmin_d;
  __shared__ int sh[EB_KEY_LEVELS + 1];
  __shared__ int smax;
  for (int i = threadIdx.x; i <= EB_KEY_LEVELS; i += blockDim.x) sh[i] = 0;
  if (threadIdx.x == 0) smax = 0;
  __syncthreads();
  int mymax = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int lam = 0;
    if (n > cap) {
      const int w0 = max(0, i - cap), w1 = min(i, n - 1 - cap);
      int m = 0;
      for (int w = w0; w <= w1; ++w) m = max(m, (int)lcpw[w]);
      lam = min(EB_KEY_LEVELS, m + 1);
    }
    lam = max(lam, lmin);
    plev[i] = (unsigned char)lam;
    mymax = max(mymax, lam);
    const int sl = i > 0 ? shared_levels(keys[i - 1], keys[i]) : -1;
    for (int l = max(1, sl + 1); l <= lam; ++l) atomicAdd(&sh[l], 1);
  }
  atomicMax(&smax, mymax);
  __syncthreads();
  for (int i = threadIdx.x; i <= EB_KEY_LEVELS; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
  if (threadIdx.x == 0) atomicMax(lmax, smax);
}

// Every level at once: flags[l*n + i] = 1 where sorted point i starts an existing box of
// level l (l = 0..L). One exclusive scan over the concatenated rows then gives each head
// its global box id (rows in level order: level l's ids start at lev_off[l]).
__global__ void k_heads_all(const unsigned long long* __restrict__ keys, const unsigned char* __restrict__ plev,
                            int n, int L, int* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int lam = plev[i];
  const int sl = i > 0 ? shared_levels(keys[i - 1], keys[i]) : -1;
  for (int l = 0; l <= L; ++l) flags[(size_t)l * n + i] = (l <= lam) && (l > sl);
}

// Box key, level, first point and parent of every box; a box whose head point also starts
// its parent is the parent's first child (a split box's points all lie in its children).
__global__ void k_boxes_all(const unsigned long long* __restrict__ keys, int n, int L, int nbox,
                            const int* __restrict__ flags, const int* __restrict__ scan,
                            unsigned long long* __restrict__ bkey, unsigned char* __restrict__ blev,
                            int* __restrict__ pt0, int* __restrict__ parent, int* __restrict__ child0) {
  const long long tot = (long long)(L + 1) * n;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < tot;
       idx += (long long)gridDim.x * blockDim.x) {
    if (!flags[idx]) continue;
    const int l = (int)(idx / n), i = (int)(idx - (long long)l * n);
    const int b = scan[idx];
    if (b >= nbox) continue;  // cannot happen: the flags and the level counts agree
    bkey[b] = keys[i] >> (2 * (EB_KEY_LEVELS - l));
    blev[b] = (unsigned char)l;
    pt0[b] = i;
    if (l == 0) {
      parent[b] = -1;
    } else {
      const size_t up = idx - n;
      const int P = scan[up] + flags[up] - 1;
      parent[b] = P;
      if (flags[up]) child0[P] = b;
    }
  }
}

struct LevOffT {
  int v[EB_KEY_LEVELS + 3];
};

// Point range end of every box (binary search for the first key beyond the box's prefix)
// and the children count of its parent.
__global__ void k_boxes_fin(int nbox, const unsigned long long* __restrict__ keys, int n,
                            const unsigned long long* __restrict__ bkey, const unsigned char* __restrict__ blev,
                            const int* __restrict__ pt0, const int* __restrict__ parent,
                            int* __restrict__ pt1, int* __restrict__ nchild) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbox) return;
  const int l = blev[b], sh = 2 * (EB_KEY_LEVELS - l);
  const unsigned long long k = bkey[b];
  int lo = pt0[b] + 1, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((keys[mid] >> sh) > k) hi = mid;
    else lo = mid + 1;
  }
  pt1[b] = lo;
  if (l > 0) atomicAdd(&nchild[parent[b]], 1);
}

__device__ __forceinline__ int find_box(const unsigned long long* __restrict__ bkey, int off,
                                        int nb, unsigned long long key) {
  int lo = 0, hi = nb - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    unsigned long long v = bkey[off + mid];
    if (v == key) return off + mid;
    if (v < key) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

// V lists of every box of levels 2..L in one launch (MKINTL, cadap2.f:780-828: the
// children of the parent's neighbours that are not adjacent to the box; DALI12's list 1,
// dapif2.f:3-171). Only existing boxes are found, so the children of a neighbour that is
// a leaf are absent: its points reach the box's leaves through their U lists.
// One warp per box: the 36 candidates (the children of the 3 x 3 parents around the
// box's parent, in the fixed order qy, qx, cy, cx) are looked up by the lanes, two each,
// and the hits written in candidate order.
__global__ void k_vlist(const unsigned long long* __restrict__ bkey, LevOffT lo, int first, int nbox, int R,
                        int* __restrict__ vlist, unsigned char* __restrict__ vcode,
                        int* __restrict__ vcount) {
  const int gid = first + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (gid >= nbox) return;  // whole warps leave together
  int lev = 0;
  while (gid >= lo.v[lev + 1]) ++lev;
  const int off = lo.v[lev], nb = lo.v[lev + 1] - off;
  const unsigned long long key = bkey[gid];
  if (lev <= R) {  // a forest's boxes of level <= R hold different problems
    if (lane == 0) vcount[gid] = 0;
    return;
  }
  const unsigned long long root = key >> (2 * (lev - R));
  const int ix = (int)compact2(key), iy = (int)compact2(key >> 1);
  const int px = ix >> 1, py = iy >> 1, half = 1 << (lev - 1), side = 1 << lev;
  int cnt = 0;
  for (int base = 0; base < 36; base += 32) {
    const int c = base + lane;
    int s = -1, code = 0;
    if (c < 36) {
      const int qy = py - 1 + c / 12, qx = px - 1 + (c / 4) % 3, cy = (c >> 1) & 1, cx = c & 1;
      const int sx = 2 * qx + cx, sy = 2 * qy + cy, dx = ix - sx, dy = iy - sy;
      const bool inside = qy >= 0 && qy < half && qx >= 0 && qx < half && sx < side && sy < side;
      const bool adjacent = dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1;
      if (inside && !adjacent) {
        s = find_box(bkey, off, nb, morton((unsigned)sx, (unsigned)sy));
        if (s >= 0 && (bkey[s] >> (2 * (lev - R))) != root) s = -1;
        code = (dy + 3) * 7 + (dx + 3);
      }
    }
    const unsigned int m = __ballot_sync(0xffffffffu, s >= 0);
    if (s >= 0) {
      const int pos = cnt + __popc(m & ((1u << lane) - 1u));
      vlist[(size_t)gid * EB_VMAX + pos] = s;
      vcode[(size_t)gid * EB_VMAX + pos] = (unsigned char)code;
    }
    cnt += __popc(m);
  }
  if (lane == 0) vcount[gid] = cnt;
}

// Image lists of the wall y = 0 (the root square's bottom edge) for the boxes of levels
// 2..ld, one thread per box: the source boxes S of the box's level whose mirror image
// across the wall is not adjacent to the box T but lies among the children of the
// mirrored neighbours of T's parent, the reflected interaction list of DOINT0DR (MKINTR,
// cadap2.f:830-877; cadapdrop2.f:159-197). On level 2 every pair is listed whose images
// are not adjacent (it takes the pairs of level 1 as well, whose parents are the root);
// below, only the first two rows have such pairs: T and S in rows 0-1 and S in the
// columns of the children of T's parent's column neighbours. Mirrored, S sits at row
// -1 - iy_S, so the offset T - S' is (ix_T - ix_S, iy_T + iy_S + 1) in box units, dy in
// [1, 7]; the pairs with dy = 1 and |dx| <= 1 (both in row 0, columns adjacent) are left
// to the direct sum of level ld.
__global__ void k_imglist(const unsigned long long* __restrict__ bkey, const unsigned char* __restrict__ blev,
                          LevOffT lo, int first, int nimg, int* __restrict__ ilist,
                          unsigned char* __restrict__ icode, int* __restrict__ icount) {
  const int gid = first + blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nimg) return;
  const int lev = blev[gid];
  const int off = lo.v[lev], nb = lo.v[lev + 1] - off;
  const unsigned long long key = bkey[gid];
  const int ix = (int)compact2(key), iy = (int)compact2(key >> 1), side = 1 << lev;
  int cnt = 0, x0, x1, y1;
  if (lev == 2) {
    x0 = 0; x1 = 3; y1 = 3;
  } else if (iy <= 1) {
    const int px = ix >> 1;
    x0 = max(2 * px - 2, 0); x1 = min(2 * px + 3, side - 1); y1 = 1;
  } else {
    icount[gid] = 0;
    return;
  }
  for (int sy = 0; sy <= y1; ++sy)
    for (int sx = x0; sx <= x1; ++sx) {
      const int dx = ix - sx, dy = iy + sy + 1;
      if (dy == 1 && dx >= -1 && dx <= 1) continue;  // adjacent images: direct sum
      const int s = find_box(bkey, off, nb, morton((unsigned)sx, (unsigned)sy));
      if (s < 0) continue;
      ilist[(size_t)gid * EB_VMAX + cnt] = s;
      icode[(size_t)gid * EB_VMAX + cnt] = (unsigned char)((dy + 3) * 7 + (dx + 3));
      ++cnt;
    }
  icount[gid] = cnt;
}

// Leaves in point order: point i starts its leaf when it heads the box of its leaf level.
__global__ void k_leaf_heads(int n, const unsigned char* __restrict__ plev, const int* __restrict__ flags,
                             int* __restrict__ lflag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  lflag[i] = flags[(size_t)plev[i] * n + i];
}

__global__ void k_leaf_fill(int n, const unsigned char* __restrict__ plev, const int* __restrict__ lflag,
                            const int* __restrict__ lscan, const int* __restrict__ scan,
                            int* __restrict__ leaves) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !lflag[i]) return;
  leaves[lscan[i]] = scan[(size_t)plev[i] * n + i];
}

// The leaf count, from the exclusive scan of the leaf heads.
__global__ void k_leaf_count(int n, const int* __restrict__ lflag, const int* __restrict__ lscan,
                             int* __restrict__ nleaf) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *nleaf = lscan[n - 1] + lflag[n - 1];
}

#define EB_LIST_STACK 72

// U and W lists of every leaf (DALI12 / DALI34, dapif2.f:3-356, for an adaptive tree
// without level restriction). For leaf b of level l:
//  * every existing box C of level l adjacent to b (b itself included): a leaf C goes to
//    U; below a split C, the boxes adjacent to b are followed down to leaves (U), and a
//    box that is not adjacent to b while its parent is goes to W (its multipole is
//    evaluated at b's points: M2P, DABARR's list-3 evaluation);
//  * every leaf of a coarser level m adjacent to b's ancestor of level m goes to U (the
//    dual list 4, evaluated directly: such a leaf holds at most cap points).
// Every pair of points is then covered exactly once by U, W or a V list of a common
// level. FILL = false counts, FILL = true writes at ustart / wstart.
template <bool FILL>
__global__ void k_leaf_lists(int nleaf, const int* __restrict__ nleaf_d, const int* __restrict__ leaves,
                             const unsigned long long* __restrict__ bkey,
                             const unsigned char* __restrict__ blev, LevOffT lo, int R,
                             const int* __restrict__ floor_d,
                             const int* __restrict__ child0, const int* __restrict__ nchild,
                             int* __restrict__ ucnt, int* __restrict__ wcnt,
                             const int* __restrict__ ustart, const int* __restrict__ wstart,
                             int* __restrict__ ulist, int* __restrict__ wlist, int* __restrict__ err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (nleaf_d) nleaf = *nleaf_d;  // counting pass: launched for an upper bound
  if (t >= nleaf) return;
  const int b = leaves[t], l = blev[b];
  const unsigned long long kb = bkey[b];
  const int ix = (int)compact2(kb), iy = (int)compact2(kb >> 1);
  const unsigned long long root = kb >> (2 * (l - R));  // the leaf's problem (R <= l)
  int nu = 0, nw = 0;
  int* uo = FILL ? ulist + ustart[t] : nullptr;
  int* wo = FILL ? wlist + wstart[t] : nullptr;
  int stack[EB_LIST_STACK];
  const int side = 1 << l;
  for (int dy = -1; dy <= 1; ++dy) {
    for (int dx = -1; dx <= 1; ++dx) {
      const int sx = ix + dx, sy = iy + dy;
      if (sx < 0 || sy < 0 || sx >= side || sy >= side) continue;
      const int C = find_box(bkey, lo.v[l], lo.v[l + 1] - lo.v[l], morton((unsigned)sx, (unsigned)sy));
      if (C < 0 || (bkey[C] >> (2 * (l - R))) != root) continue;
      if (nchild[C] == 0) {
        if (FILL) uo[nu] = C;
        ++nu;
        continue;
      }
      int sp = 0;
      for (int c = 0; c < nchild[C]; ++c) stack[sp++] = child0[C] + c;
      while (sp > 0) {
        const int D = stack[--sp];
        const int f = blev[D] - l;
        const unsigned long long kd = bkey[D];
        const int jx = (int)compact2(kd), jy = (int)compact2(kd >> 1);
        const int x0 = ix << f, x1 = ((ix + 1) << f) - 1, y0 = iy << f, y1 = ((iy + 1) << f) - 1;
        const bool adj = jx >= x0 - 1 && jx <= x1 + 1 && jy >= y0 - 1 && jy <= y1 + 1;
        if (!adj) {
          if (FILL) wo[nw] = D;
          ++nw;
        } else if (nchild[D] == 0) {
          if (FILL) uo[nu] = D;
          ++nu;
        } else if (sp + nchild[D] <= EB_LIST_STACK) {
          for (int c = 0; c < nchild[D]; ++c) stack[sp++] = child0[D] + c;
        } else {
          atomicOr(err, 1);
        }
      }
    }
  }
  // no leaf lies above the tree's floor (every box there is split)
  const int mstop = max(R, *floor_d);
  for (int m = l - 1; m >= mstop; --m) {
    const int ax = ix >> (l - m), ay = iy >> (l - m), sm = 1 << m;
    for (int dy = -1; dy <= 1; ++dy) {
      for (int dx = -1; dx <= 1; ++dx) {
        if (dx == 0 && dy == 0) continue;
        const int sx = ax + dx, sy = ay + dy;
        if (sx < 0 || sy < 0 || sx >= sm || sy >= sm) continue;
        const int N = find_box(bkey, lo.v[m], lo.v[m + 1] - lo.v[m], morton((unsigned)sx, (unsigned)sy));
        if (N < 0 || nchild[N] != 0 || (bkey[N] >> (2 * (m - R))) != root) continue;
        if (FILL) uo[nu] = N;
        ++nu;
      }
    }
  }
  if (!FILL) {
    ucnt[t] = nu;
    wcnt[t] = nw;
  }
}

// Algorithmic work of the built tree: near-field pairs (self excluded), M2P evaluations
// (W-list box, target point) and M2L pairs.
__global__ void k_pair_counts(int nleaf, const int* __restrict__ leaves, const int* __restrict__ pt0,
                              const int* __restrict__ pt1, const int* __restrict__ ustart,
                              const int* __restrict__ ulist, const int* __restrict__ wstart,
                              int vfirst, int vlast, const int* __restrict__ vcount,
                              unsigned long long* __restrict__ out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long up = 0, vp = 0, wp = 0;
  if (t < nleaf) {
    const int b = leaves[t];
    const long long nt = pt1[b] - pt0[b];
    long long ns = 0;
    for (int j = ustart[t]; j < ustart[t + 1]; ++j) {
      const int s = ulist[j];
      ns += pt1[s] - pt0[s];
    }
    up = (unsigned long long)(nt * ns - nt);
    wp = (unsigned long long)(nt * (wstart[t + 1] - wstart[t]));
  }
  for (int g = vfirst + blockIdx.x * blockDim.x + threadIdx.x; g < vlast; g += gridDim.x * blockDim.x)
    vp += (unsigned long long)vcount[g];
  up = warp_sum<unsigned long long>(up);
  vp = warp_sum<unsigned long long>(vp);
  wp = warp_sum<unsigned long long>(wp);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out[0], up);
    atomicAdd(&out[1], vp);
    atomicAdd(&out[2], wp);
  }
}

__global__ void k_group_count(int nleaf, const int* __restrict__ nleaf_d, const int* __restrict__ leaves,
                              const int* __restrict__ pt0, const int* __restrict__ pt1, int* __restrict__ cnt) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *nleaf_d) return;
  const int b = leaves[t];
  cnt[t] = (pt1[b] - pt0[b] + EB_GROUP - 1) / EB_GROUP;
}

__global__ void k_group_fill(int nleaf, const int* __restrict__ leaves, const int* __restrict__ pt0,
                             const int* __restrict__ cnt, const int* __restrict__ start,
                             int* __restrict__ gleaf, int* __restrict__ gfirst) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nleaf) return;
  const int b = leaves[t], g0 = start[t];
  for (int g = 0; g < cnt[t]; ++g) {
    gleaf[g0 + g] = t;
    gfirst[g0 + g] = pt0[b] + g * EB_GROUP;
  }
}

__global__ void k_tile_count(int nleaf, const int* __restrict__ nleaf_d, const int* __restrict__ leaves,
                             const int* __restrict__ pt0, const int* __restrict__ pt1, int* __restrict__ cnt) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *nleaf_d) return;
  const int b = leaves[t];
  cnt[t] = (pt1[b] - pt0[b] + EB_NTILE - 1) / EB_NTILE;
}

__global__ void k_tile_fill(int nleaf, const int* __restrict__ leaves, const int* __restrict__ pt0,
                            const int* __restrict__ pt1, const int* __restrict__ cnt,
                            const int* __restrict__ start, int4* __restrict__ tiles) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nleaf) return;
  const int b = leaves[t];
  const int g0 = start[t], c = cnt[t], a = pt0[b], nt = pt1[b] - a;
  for (int g = 0; g < c; ++g)
    tiles[g0 + g] = make_int4(t, a + (int)((long long)g * nt / c), a + (int)((long long)(g + 1) * nt / c), 0);
}

// The FP32 far field's boxes of each leaf: the leaf and its ancestors down to level
// max(2, min(lev, lend)), -1 beyond (levels <= lend hold the L2L-accumulated locals).
__global__ void k_far_boxes(int nleaf, const int* __restrict__ leaves, const unsigned char* __restrict__ blev,
                            const int* __restrict__ parent, int lend, int* __restrict__ anc) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nleaf) return;
  int a = leaves[t];
  const int l = blev[a], lmin = max(2, min(l, lend));
  for (int q = 0; q < EB_FAR_LEVELS; ++q) {
    const int lev = l - q;
    anc[(size_t)t * EB_FAR_LEVELS + q] = lev >= lmin ? a : -1;
    if (lev > lmin) a = parent[a];
  }
}

// Chunks of the boxes whose FP32 multipoles come directly from their points: every box
// of the levels >= lmin and every leaf above them (coarser levels get theirs by M2M).
__global__ void k_chunk_count(int first, int nb, int lmin, const unsigned char* __restrict__ blev,
                              const int* __restrict__ nchild, const int* __restrict__ pt0,
                              const int* __restrict__ pt1, int* __restrict__ cnt) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int g = first + b;
  const bool direct = blev[g] >= lmin || nchild[g] == 0;
  cnt[b] = direct ? (pt1[g] - pt0[g] + EB_CHUNK - 1) / EB_CHUNK : 0;
}

__global__ void k_chunk_fill(int first, int nb, const int* __restrict__ cnt, const int* __restrict__ start,
                             int* __restrict__ chunk_box) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  for (int c = 0; c < cnt[b]; ++c) chunk_box[start[b] + c] = first + b;
}

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

}  // namespace

namespace {
std::atomic<unsigned long long> g_epoch{1};
thread_local bool t_capturing = false;
std::mutex g_deferred_mu;
std::vector<void*> g_deferred;
}  // namespace

unsigned long long eb_devbuf_epoch() { return g_epoch.load(); }
void eb_devbuf_set_capturing(bool on) { t_capturing = on; }
void eb_devbuf_collect() {
  std::vector<void*> v;
  {
    std::lock_guard<std::mutex> lk(g_deferred_mu);
    v.swap(g_deferred);
  }
  for (void* q : v) cudaFree(q);
  if (!v.empty()) g_epoch++;  // no cached graph may keep an address freed here
}

int DevBuf::ensure(size_t nbytes) {
  if (nbytes <= bytes && p) return EB_OK;
  if (p && t_capturing) {
    std::lock_guard<std::mutex> lk(g_deferred_mu);
    g_deferred.push_back(p);
    p = nullptr;
    bytes = 0;
    g_epoch++;
  }
  release();
  size_t want = nbytes < 256 ? 256 : nbytes;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    bytes = 0;
    eb_set_last_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
    return EB_ERR_CUDA;
  }
  bytes = want;
  return EB_OK;
}

void DevBuf::release() {
  if (p) {
    cudaFree(p);
    g_epoch++;
  }
  p = nullptr;
  bytes = 0;
}

// (z - x0 - (i + 1/2) r) / r, the offset of a coordinate from the centre of its leaf in
// leaf units, with both subtractions carried exactly (two-sum, two-product), so that
// for two nodes the offsets differ by exactly (z_j - z_i)/r minus the integer index
// offset of their leaves, up to the final rounding (about 2^-53 of a leaf side).
__device__ __forceinline__ double leaf_offset(double z, double x0, unsigned int i, double r) {
  double s = __dsub_rn(z, x0);
  double bb = __dsub_rn(s, z);
  double e1 = __dadd_rn(__dsub_rn(z, __dsub_rn(s, bb)), __dsub_rn(-x0, bb));
  double ci = (double)i + 0.5;
  double c = __dmul_rn(ci, r);
  double e2 = __fma_rn(ci, r, -c);
  double u = __dsub_rn(s, c);
  double bb2 = __dsub_rn(u, s);
  double e3 = __dadd_rn(__dsub_rn(s, __dsub_rn(u, bb2)), __dsub_rn(-c, bb2));
  return __ddiv_rn(__dadd_rn(u, __dadd_rn(__dsub_rn(e1, e2), e3)), r);
}

// Leaf-relative node coordinates as three floats hi + mid + lo (all 53 bits of the
// double offset), for the double-float near field: wa = (x.hi, y.hi, x.mid, y.mid),
// wb = (x.lo, y.lo). (hi, mid) alone is a double-float. One block per leaf.
__device__ __forceinline__ void split3(double w, float& hi, float& mid, float& lo) {
  hi = __double2float_rn(w);
  double r1 = w - (double)hi;
  mid = __double2float_rn(r1);
  lo = __double2float_rn(r1 - (double)mid);
}

__global__ void k_leaf_coords(const int* __restrict__ leaves, const unsigned long long* __restrict__ bkey,
                              const unsigned char* __restrict__ blev, const int* __restrict__ pt0,
                              const int* __restrict__ pt1, const double2* __restrict__ zs, double x0, double y0,
                              double W, float4* __restrict__ wa, float2* __restrict__ wb) {
  const int b = leaves[blockIdx.x];
  const unsigned long long k = bkey[b];
  const unsigned int ix = compact2(k), iy = compact2(k >> 1);
  const double r = ldexp(W, -(int)blev[b]);  // W / 2^level, exact
  for (int i = pt0[b] + threadIdx.x; i < pt1[b]; i += blockDim.x) {
    double2 z = zs[i];
    float xh, xm, xl, yh, ym, yl;
    split3(leaf_offset(z.x, x0, ix, r), xh, xm, xl);
    split3(leaf_offset(z.y, y0, iy, r), yh, ym, yl);
    wa[i] = make_float4(xh, yh, xm, ym);
    wb[i] = make_float2(xl, yl);
  }
}

// The tree of a problem that takes the direct sums: one kernel and one readback (the
// finiteness check) instead of the build; the FMM's apply then sums all pairs.
static int direct_tree(eb_ctx* ctx, EbTree& t, const double2* z, int n, int leaf_cap) {
  cudaStream_t st = eb_stream(ctx);
  t.direct = true;
  t.n = n;
  t.cap = leaf_cap;
  t.R = 0;
  t.wall = 0;
  t.ld = 0;
  t.L = 0;
  t.nbox = 1;
  t.nleaf = 1;
  t.ngroup = 0;
  t.ntile = 0;
  t.nchunk = 0;
  t.chunk_lmin = 2;
  t.lend = 2;
  t.nu = t.nw = 0;
  t.lev_off[0] = 0;
  for (int l = 1; l < EB_KEY_LEVELS + 2; ++l) t.lev_off[l] = 1;
  t.x0 = t.y0 = 0.0;
  t.W = 1.0;
  if (!t.host) EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&t.host), sizeof(EbTreeHost)));
  EB_TRY(t.perm.ensure(sizeof(int) * (size_t)n));
  EB_TRY(t.zs.ensure(sizeof(double2) * (size_t)n));
  EB_TRY(t.zhl.ensure(sizeof(float4) * (size_t)n));
  EB_TRY(t.bbox.ensure(sizeof(int)));
  // inside an RK call (ctx->defer) the flag accumulates in ctx->d_bad, read after the call
  int* bad = ctx->defer ? ctx->d_bad.as<int>() : t.bbox.as<int>();
  if (!ctx->defer) EB_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), st));
  k_direct_points<<<nblk(n, 256), 256, 0, st>>>(z, n, t.perm.as<int>(), t.zs.as<double2>(), t.zhl.as<float4>(),
                                                bad);
  eb_count_launch(ctx);
  if (!ctx->defer) {
    EB_CUDA_TRY(cudaMemcpyAsync(&t.host->bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    EB_CUDA_TRY(cudaStreamSynchronize(st));
    if (t.host->bad & 1) {
      eb_set_last_error_msg("non-finite node coordinate");
      return EB_ERR_NAN;
    }
  }
  t.u_pairs = (long long)n * (n - 1);
  t.v_pairs = t.w_pairs = 0;
  t.pairs_read = true;
  t.valid = true;
  return eb_check_launch(ctx, "direct tree");
}

int eb_tree_build(eb_ctx* ctx, EbTree& t, const double2* z, int n, int leaf_target, int leaf_cap,
                  const double* root_sq, int root_level, int wall) {
  cudaStream_t st = eb_stream(ctx);
  t.valid = false;
  if (n <= 0) return EB_ERR_ARG;
  if (!root_sq && !wall && ctx->nsim == 0 && ctx->opts.direct_max > 0 && n <= ctx->opts.direct_max)
    return direct_tree(ctx, t, z, n, leaf_cap < 1 ? EB_LEAF_CAP : leaf_cap);
  t.direct = false;
  if (leaf_target < 1) leaf_target = 32;
  if (leaf_cap < 1) leaf_cap = EB_LEAF_CAP;
  t.n = n;
  t.cap = leaf_cap;
  t.R = root_sq ? root_level : 0;
  t.wall = wall && !root_sq;
  t.ld = 0;
  const int BS = 256;
  if (!t.host) EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&t.host), sizeof(EbTreeHost)));
  EbTreeHost* H = t.host;
  t.pairs_read = false;
  // 1. bounding square, on the device
  int nbb = std::min(nblk(n, BS), 1024);
  EB_TRY(t.partial.ensure(sizeof(Box4) * (size_t)nbb));
  EB_TRY(t.bbox.ensure(sizeof(Box4) + sizeof(double) * 4 + sizeof(int) * 8));
  double* sq = reinterpret_cast<double*>(t.bbox.as<char>() + sizeof(Box4));
  int* bad = reinterpret_cast<int*>(sq + 4);
  int* lmax_d = bad + 1;
  int* lerr_d = bad + 2;
  int* nleaf_d = bad + 3;
  int* lmin_d = bad + 4;
  EB_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int) * 3, st));
  k_bbox<<<nbb, BS, 0, st>>>(z, n, t.partial.as<Box4>(), bad);
  eb_count_launch(ctx);
  if (root_sq) k_set_square<<<1, 32, 0, st>>>(root_sq[0], root_sq[1], root_sq[2], sq);
  else k_bbox_final<<<1, 256, 0, st>>>(t.partial.as<Box4>(), nbb, t.bbox.as<Box4>(), sq, t.wall, bad);
  eb_count_launch(ctx);
  // 2. keys and sort (a non-finite coordinate gives clamped keys; reported below)
  EB_TRY(t.keys.ensure(sizeof(unsigned long long) * (size_t)n));
  EB_TRY(t.keys_alt.ensure(sizeof(unsigned long long) * (size_t)n));
  EB_TRY(t.idx_alt.ensure(sizeof(int) * (size_t)n));
  EB_TRY(t.perm.ensure(sizeof(int) * (size_t)n));
  k_keys<<<nblk(n, BS), BS, 0, st>>>(z, n, sq, t.keys_alt.as<unsigned long long>(), t.idx_alt.as<int>());
  eb_count_launch(ctx);
  size_t tmp_sort = 0, tmp_scan = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, t.keys_alt.as<unsigned long long>(),
                                  t.keys.as<unsigned long long>(), t.idx_alt.as<int>(),
                                  t.perm.as<int>(), n, 0, 2 * EB_KEY_LEVELS, st);
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_scan, t.flags.as<int>(), t.scan.as<int>(), n, st);
  EB_TRY(t.cubtmp.ensure(std::max(tmp_sort, tmp_scan)));
  size_t tb = t.cubtmp.bytes;
  EB_CUDA_TRY(cub::DeviceRadixSort::SortPairs(t.cubtmp.p, tb, t.keys_alt.as<unsigned long long>(),
                                              t.keys.as<unsigned long long>(), t.idx_alt.as<int>(),
                                              t.perm.as<int>(), n, 0, 2 * EB_KEY_LEVELS, st));
  eb_count_launch(ctx);
  const unsigned long long* keys = t.keys.as<unsigned long long>();
  // 3. sorted positions
  EB_TRY(t.zs.ensure(sizeof(double2) * (size_t)n));
  EB_TRY(t.zhl.ensure(sizeof(float4) * (size_t)n));
  k_gather_points<<<nblk(n, BS), BS, 0, st>>>(z, t.perm.as<int>(), n, t.zs.as<double2>(), t.zhl.as<float4>());
  eb_count_launch(ctx);
  // 4. leaf level of every point, deepest level, boxes per level
  EB_TRY(t.lcpw.ensure((size_t)n));
  EB_TRY(t.plev.ensure((size_t)n));
  EB_TRY(t.hist.ensure(sizeof(int) * (EB_KEY_LEVELS + 1)));
  EB_CUDA_TRY(cudaMemsetAsync(t.hist.p, 0, sizeof(int) * (EB_KEY_LEVELS + 1), st));
  k_level_hist<<<std::min(nblk(n, BS), ctx->nsm * 4), BS, 0, st>>>(keys, n, t.hist.as<int>());
  k_pick_level<<<1, 32, 0, st>>>(n, leaf_target, t.R, t.hist.as<int>(), lmin_d);
  EB_CUDA_TRY(cudaMemsetAsync(t.hist.p, 0, sizeof(int) * (EB_KEY_LEVELS + 1), st));
  ctx->launches += 2;
  if (n > leaf_cap) {
    k_lcp_window<<<nblk(n - leaf_cap, BS), BS, 0, st>>>(keys, n, leaf_cap, t.lcpw.as<unsigned char>());
    eb_count_launch(ctx);
  }
  k_leaf_level<<<std::min(nblk(n, BS), ctx->nsm * 8), BS, 0, st>>>(keys, n, leaf_cap, lmin_d, t.lcpw.as<unsigned char>(),
                                                                  t.plev.as<unsigned char>(), lmax_d,
                                                                  t.hist.as<int>());
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemcpyAsync(H->sq, sq, sizeof(H->sq), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->bad, bad, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(H->hist, t.hist.p, sizeof(H->hist), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->lmin, lmin_d, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaStreamSynchronize(st));
  if (H->bad & 1) {
    eb_set_last_error_msg("non-finite node coordinate");
    return EB_ERR_NAN;
  }
  if (H->bad & 2) {
    eb_set_last_error_msg("wall-bounded flow: a node lies below the wall y = 0");
    return EB_ERR_ARG;
  }
  t.W = H->sq[0];
  t.x0 = H->sq[1];
  t.y0 = H->sq[2];
  const int L = H->lmax;
  t.L = L;
  t.lev_off[0] = 0;
  for (int l = 0; l <= L; ++l) t.lev_off[l + 1] = t.lev_off[l] + (l == 0 ? 1 : H->hist[l]);
  for (int l = L + 1; l <= EB_KEY_LEVELS; ++l) t.lev_off[l + 1] = t.lev_off[L + 1];
  t.nbox = t.lev_off[L + 1];
  t.lend = std::max(2, L - EB_FAR_LEVELS + 1);
  const size_t NB = (size_t)t.nbox;
  EB_TRY(t.bkey.ensure(sizeof(unsigned long long) * NB));
  EB_TRY(t.blev.ensure(NB));
  EB_TRY(t.pt0.ensure(sizeof(int) * NB));
  EB_TRY(t.pt1.ensure(sizeof(int) * NB));
  EB_TRY(t.parent.ensure(sizeof(int) * NB));
  EB_TRY(t.child0.ensure(sizeof(int) * NB));
  EB_TRY(t.nchild.ensure(sizeof(int) * NB));
  // 5. boxes of every level: heads, one scan, fill, finish
  const size_t nflag = (size_t)(L + 1) * n;
  EB_TRY(t.flags.ensure(sizeof(int) * nflag));
  EB_TRY(t.scan.ensure(sizeof(int) * nflag));
  k_heads_all<<<nblk(n, BS), BS, 0, st>>>(keys, t.plev.as<unsigned char>(), n, L, t.flags.as<int>());
  eb_count_launch(ctx);
  {
    size_t need = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, need, t.flags.as<int>(), t.scan.as<int>(), (int)nflag, st);
    if (need > t.cubtmp.bytes) EB_TRY(t.cubtmp.ensure(need));
  }
  tb = t.cubtmp.bytes;
  EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, t.flags.as<int>(), t.scan.as<int>(), (int)nflag, st));
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemsetAsync(t.child0.p, 0xff, sizeof(int) * NB, st));  // -1: no children
  EB_CUDA_TRY(cudaMemsetAsync(t.nchild.p, 0, sizeof(int) * NB, st));
  k_boxes_all<<<std::min(nblk((long long)nflag, BS), ctx->nsm * 16), BS, 0, st>>>(
      keys, n, L, t.nbox, t.flags.as<int>(), t.scan.as<int>(), t.bkey.as<unsigned long long>(),
      t.blev.as<unsigned char>(), t.pt0.as<int>(), t.parent.as<int>(), t.child0.as<int>());
  eb_count_launch(ctx);
  k_boxes_fin<<<nblk(t.nbox, BS), BS, 0, st>>>(t.nbox, keys, n, t.bkey.as<unsigned long long>(),
                                              t.blev.as<unsigned char>(), t.pt0.as<int>(), t.parent.as<int>(),
                                              t.pt1.as<int>(), t.nchild.as<int>());
  eb_count_launch(ctx);
  LevOffT lo;
  for (int l = 0; l < EB_KEY_LEVELS + 3; ++l) lo.v[l] = t.lev_off[std::min(l, L + 1)];
  // 6. leaves in point order
  EB_TRY(t.lflag.ensure(sizeof(int) * (size_t)n));
  EB_TRY(t.lscan.ensure(sizeof(int) * (size_t)n));
  EB_TRY(t.leaves.ensure(sizeof(int) * NB));
  k_leaf_heads<<<nblk(n, BS), BS, 0, st>>>(n, t.plev.as<unsigned char>(), t.flags.as<int>(), t.lflag.as<int>());
  eb_count_launch(ctx);
  tb = t.cubtmp.bytes;
  EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, t.lflag.as<int>(), t.lscan.as<int>(), n, st));
  eb_count_launch(ctx);
  k_leaf_fill<<<nblk(n, BS), BS, 0, st>>>(n, t.plev.as<unsigned char>(), t.lflag.as<int>(), t.lscan.as<int>(),
                                          t.scan.as<int>(), t.leaves.as<int>());
  eb_count_launch(ctx);
  // 7. V lists of every box of levels >= 2
  EB_TRY(t.vlist.ensure(sizeof(int) * NB * EB_VMAX));
  EB_TRY(t.vcode.ensure(NB * EB_VMAX));
  EB_TRY(t.vcount.ensure(sizeof(int) * NB));
  EB_CUDA_TRY(cudaMemsetAsync(t.vcount.p, 0, sizeof(int) * NB, st));
  if (L >= 2) {
    const int first = t.lev_off[2];
    k_vlist<<<nblk(32LL * (t.nbox - first), 128), 128, 0, st>>>(t.bkey.as<unsigned long long>(), lo, first, t.nbox, t.R,
                                                       t.vlist.as<int>(), t.vcode.as<unsigned char>(),
                                                       t.vcount.as<int>());
    eb_count_launch(ctx);
  }
  // 7b. image lists of the wall (levels 2..ld, ld the uniform floor)
  if (t.wall && L >= 2 && H->lmin >= 2) {
    t.ld = std::min(H->lmin, L);
    const int first = t.lev_off[2], nimg = t.lev_off[t.ld + 1];
    EB_TRY(t.ilist.ensure(sizeof(int) * (size_t)nimg * EB_VMAX));
    EB_TRY(t.icode.ensure((size_t)nimg * EB_VMAX));
    EB_TRY(t.icount.ensure(sizeof(int) * (size_t)nimg));
    EB_CUDA_TRY(cudaMemsetAsync(t.icount.p, 0, sizeof(int) * (size_t)nimg, st));
    k_imglist<<<nblk(nimg - first, 128), 128, 0, st>>>(t.bkey.as<unsigned long long>(), t.blev.as<unsigned char>(),
                                                       lo, first, nimg, t.ilist.as<int>(),
                                                       t.icode.as<unsigned char>(), t.icount.as<int>());
    eb_count_launch(ctx);
  }
  // 8. per-leaf counts, scanned so that one synchronisation sizes them all: U and W list
  // lengths, near-field groups of EB_GROUP targets, shared-memory tiles of at most
  // EB_NTILE targets, and FP32 direct-P2M chunks of at most EB_CHUNK points of every box
  // of the chunked levels (every level up to 256K points, so that no dependent M2M
  // launches remain on the critical path; above that the EB_DIRECT_LEVELS finest).
  // The leaf count is known on the device only: the counting kernels run over nbox
  // threads, stop at that count and leave zeros beyond it, and the scans span nbox + 1
  // entries, so that their last entries are the totals.
  const int NBi = t.nbox;
  EB_TRY(t.ucnt.ensure(sizeof(int) * (NB + 1)));
  EB_TRY(t.wcnt.ensure(sizeof(int) * (NB + 1)));
  EB_TRY(t.ustart.ensure(sizeof(int) * (NB + 1)));
  EB_TRY(t.wstart.ensure(sizeof(int) * (NB + 1)));
  EB_TRY(t.tcount.ensure(sizeof(int) * (NB + 1)));
  EB_TRY(t.tstart.ensure(sizeof(int) * (NB + 1)));
  EB_TRY(t.gcount.ensure(sizeof(int) * (NB + 1)));
  EB_TRY(t.gstart.ensure(sizeof(int) * (NB + 1)));
  k_leaf_count<<<1, 32, 0, st>>>(n, t.lflag.as<int>(), t.lscan.as<int>(), nleaf_d);
  eb_count_launch(ctx);
  for (DevBuf* d : {&t.ucnt, &t.wcnt, &t.tcount, &t.gcount})
    EB_CUDA_TRY(cudaMemsetAsync(d->p, 0, sizeof(int) * (NB + 1), st));
  k_leaf_lists<false><<<nblk(NBi, 128), 128, 0, st>>>(NBi, nleaf_d, t.leaves.as<int>(), t.bkey.as<unsigned long long>(),
                                                       t.blev.as<unsigned char>(), lo, t.R, lmin_d, t.child0.as<int>(),
                                                       t.nchild.as<int>(), t.ucnt.as<int>(), t.wcnt.as<int>(),
                                                       nullptr, nullptr, nullptr, nullptr, lerr_d);
  k_group_count<<<nblk(NBi, BS), BS, 0, st>>>(NBi, nleaf_d, t.leaves.as<int>(), t.pt0.as<int>(), t.pt1.as<int>(),
                                              t.gcount.as<int>());
  k_tile_count<<<nblk(NBi, BS), BS, 0, st>>>(NBi, nleaf_d, t.leaves.as<int>(), t.pt0.as<int>(), t.pt1.as<int>(),
                                             t.tcount.as<int>());
  ctx->launches += 3;
  {
    size_t need = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, need, t.ucnt.as<int>(), t.ustart.as<int>(), NBi + 1, st);
    if (need > t.cubtmp.bytes) EB_TRY(t.cubtmp.ensure(need));
  }
  for (auto pr : {std::make_pair(&t.ucnt, &t.ustart), std::make_pair(&t.wcnt, &t.wstart),
                  std::make_pair(&t.gcount, &t.gstart), std::make_pair(&t.tcount, &t.tstart)}) {
    tb = t.cubtmp.bytes;
    EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, pr.first->as<int>(), pr.second->as<int>(), NBi + 1, st));
    eb_count_launch(ctx);
  }
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[0], nleaf_d, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[1], t.gstart.as<int>() + NBi, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[2], t.tstart.as<int>() + NBi, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[3], t.ustart.as<int>() + NBi, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[4], t.wstart.as<int>() + NBi, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[5], lerr_d, sizeof(int), cudaMemcpyDeviceToHost, st));
  t.nchunk = 0;
  t.chunk_lmin = n <= (1 << 18) ? 2 : std::max(2, L - EB_DIRECT_LEVELS + 1);
  const int cfirst = t.lev_off[std::min(2, L + 1)], nb2 = t.nbox - cfirst;
  if (L >= 2 && nb2 > 0) {
    EB_TRY(t.ccount.ensure(sizeof(int) * (size_t)nb2));
    EB_TRY(t.cstart.ensure(sizeof(int) * (size_t)(nb2 + 1)));
    EB_TRY(t.cdone.ensure(sizeof(int) * (size_t)nb2));
    EB_CUDA_TRY(cudaMemsetAsync(t.cdone.p, 0, sizeof(int) * (size_t)nb2, st));
    k_chunk_count<<<nblk(nb2, BS), BS, 0, st>>>(cfirst, nb2, t.chunk_lmin, t.blev.as<unsigned char>(),
                                                t.nchild.as<int>(), t.pt0.as<int>(), t.pt1.as<int>(),
                                                t.ccount.as<int>());
    eb_count_launch(ctx);
    size_t need = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, need, t.ccount.as<int>(), t.cstart.as<int>(), nb2, st);
    if (need > t.cubtmp.bytes) EB_TRY(t.cubtmp.ensure(need));
    tb = t.cubtmp.bytes;
    EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, t.ccount.as<int>(), t.cstart.as<int>(), nb2, st));
    eb_count_launch(ctx);
    EB_CUDA_TRY(cudaMemcpyAsync(&H->last[6], t.ccount.as<int>() + nb2 - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    EB_CUDA_TRY(cudaMemcpyAsync(&H->last[7], t.cstart.as<int>() + nb2 - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  }
  EB_CUDA_TRY(cudaStreamSynchronize(st));
  if (H->last[5]) {
    eb_set_last_error_msg("tree build: interaction-list traversal deeper than its stack");
    return EB_ERR_WORKSPACE;
  }
  const int nl = H->last[0];
  t.nleaf = nl;
  t.ngroup = H->last[1];
  t.ntile = H->last[2];
  t.nu = H->last[3];
  t.nw = H->last[4];
  // 9. fill the lists and work items
  EB_TRY(t.ulist.ensure(sizeof(int) * (size_t)std::max<long long>(t.nu, 1)));
  EB_TRY(t.wlist.ensure(sizeof(int) * (size_t)std::max<long long>(t.nw, 1)));
  k_leaf_lists<true><<<nblk(nl, 128), 128, 0, st>>>(nl, nullptr, t.leaves.as<int>(), t.bkey.as<unsigned long long>(),
                                                     t.blev.as<unsigned char>(), lo, t.R, lmin_d, t.child0.as<int>(),
                                                     t.nchild.as<int>(), nullptr, nullptr, t.ustart.as<int>(),
                                                     t.wstart.as<int>(), t.ulist.as<int>(), t.wlist.as<int>(),
                                                     lerr_d);
  eb_count_launch(ctx);
  EB_TRY(t.gleaf.ensure(sizeof(int) * (size_t)t.ngroup));
  EB_TRY(t.gfirst.ensure(sizeof(int) * (size_t)t.ngroup));
  k_group_fill<<<nblk(nl, BS), BS, 0, st>>>(nl, t.leaves.as<int>(), t.pt0.as<int>(), t.gcount.as<int>(),
                                            t.gstart.as<int>(), t.gleaf.as<int>(), t.gfirst.as<int>());
  eb_count_launch(ctx);
  EB_TRY(t.tiles.ensure(sizeof(int4) * (size_t)t.ntile));
  k_tile_fill<<<nblk(nl, BS), BS, 0, st>>>(nl, t.leaves.as<int>(), t.pt0.as<int>(), t.pt1.as<int>(),
                                           t.tcount.as<int>(), t.tstart.as<int>(), t.tiles.as<int4>());
  eb_count_launch(ctx);
  EB_TRY(t.anc.ensure(sizeof(int) * (size_t)nl * EB_FAR_LEVELS));
  k_far_boxes<<<nblk(nl, BS), BS, 0, st>>>(nl, t.leaves.as<int>(), t.blev.as<unsigned char>(), t.parent.as<int>(),
                                           t.lend, t.anc.as<int>());
  eb_count_launch(ctx);
  if (L >= 2 && nb2 > 0) {
    t.nchunk = H->last[6] + H->last[7];
    EB_CUDA_TRY(cudaMemcpyAsync(t.cstart.as<int>() + nb2, &t.nchunk, sizeof(int), cudaMemcpyHostToDevice, st));
    EB_TRY(t.chunk_box.ensure(sizeof(int) * (size_t)std::max(t.nchunk, 1)));
    k_chunk_fill<<<nblk(nb2, BS), BS, 0, st>>>(cfirst, nb2, t.ccount.as<int>(), t.cstart.as<int>(),
                                               t.chunk_box.as<int>());
    eb_count_launch(ctx);
  }
  // 10. leaf-relative coordinates for the double-float kernels and the FP32 P2M / far field
  EB_TRY(t.wdf.ensure(sizeof(float4) * (size_t)n));
  EB_TRY(t.wdf_lo.ensure(sizeof(float2) * (size_t)n));
  k_leaf_coords<<<nl, 64, 0, st>>>(t.leaves.as<int>(), t.bkey.as<unsigned long long>(), t.blev.as<unsigned char>(),
                                   t.pt0.as<int>(), t.pt1.as<int>(), t.zs.as<double2>(), t.x0, t.y0, t.W,
                                   t.wdf.as<float4>(), t.wdf_lo.as<float2>());
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "tree build"));
  t.valid = true;
  return EB_OK;
}

// Pair counts (the algorithmic work of the near field, M2P and M2L), counted on the
// device when first asked for after a build (they are statistics, not inputs of any
// apply, so the build does not spend a launch on them).
int eb_tree_pairs(eb_ctx* ctx, EbTree& t) {
  if (!t.pairs_read) {
    if (!t.valid) return EB_ERR_NOGEOM;
    cudaStream_t st = eb_stream(ctx);
    const int BS = 256, nl = t.nleaf, L = t.L;
    EB_TRY(t.pairs.ensure(3 * sizeof(unsigned long long)));
    unsigned long long* cnt = t.pairs.as<unsigned long long>();
    EB_CUDA_TRY(cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned long long), st));
    int vfirst = t.lev_off[std::min(2, L + 1)], vlast = t.nbox;
    k_pair_counts<<<std::max(nblk(nl, BS), 1), BS, 0, st>>>(nl, t.leaves.as<int>(), t.pt0.as<int>(),
                                                           t.pt1.as<int>(), t.ustart.as<int>(), t.ulist.as<int>(),
                                                           t.wstart.as<int>(), vfirst, vlast, t.vcount.as<int>(), cnt);
    eb_count_launch(ctx);
    EB_CUDA_TRY(cudaMemcpyAsync(t.host->pairs, cnt, sizeof(t.host->pairs), cudaMemcpyDeviceToHost, st));
    EB_CUDA_TRY(cudaStreamSynchronize(st));
    t.u_pairs = (long long)t.host->pairs[0];
    t.v_pairs = (long long)t.host->pairs[1];
    t.w_pairs = (long long)t.host->pairs[2];
    t.pairs_read = true;
  }
  return EB_OK;
}

EbTree::~EbTree() {
  if (host) cudaFreeHost(host);
}
