// GPU quadtree construction for the boundary-node FMM.
//
// The reference bins the nodes into a uniform 2^l x 2^l grid at every level with a
// counting sort (ASSIGN1, cadap2.f:252-409) and loops over all 4^l boxes, empty or
// not (DOINT0DR, cadapdrop2.f:84-197). Here the nodes are sorted once by a Morton key
// at depth 20; the occupied boxes of every level are then the distinct key prefixes,
// each owning a contiguous range of the sorted nodes. Only occupied boxes exist.
// The leaf level is the shallowest one whose mean occupancy is at most `leaf_target`.
// Interaction lists follow MKINTL (cadap2.f:780-828: children of the parent's
// neighbours that are not adjacent, at most 27) and MKNBOR (cadap2.f:705-742: the
// 3 x 3 neighbourhood at the leaf level).
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
                             double* __restrict__ sq) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Box4 r = mk_box4(INFINITY, -INFINITY, INFINITY, -INFINITY);
  for (int i = 0; i < nb; ++i) {
    Box4 p = part[i];
    r.x = fmin(r.x, p.x); r.y = fmax(r.y, p.y); r.z = fmin(r.z, p.z); r.w = fmax(r.w, p.w);
  }
  *out = r;
  double w = fmax(__dadd_rn(r.y, -r.x), __dadd_rn(r.w, -r.z));
  if (!(w > 0)) w = 1.0;
  w = __dmul_rn(w, 1.0 + 1e-9);
  sq[0] = w;
  sq[1] = __dadd_rn(__dmul_rn(0.5, __dadd_rn(r.x, r.y)), -__dmul_rn(0.5, w));
  sq[2] = __dadd_rn(__dmul_rn(0.5, __dadd_rn(r.z, r.w)), -__dmul_rn(0.5, w));
  sq[3] = __ddiv_rn((double)(1u << EB_KEY_LEVELS), w);
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

// Histogram of the first level at which consecutive sorted keys fall in different
// boxes: occupied boxes at level l = 1 + sum_{l' <= l} hist[l'].
__global__ void k_level_hist(const unsigned long long* __restrict__ keys, int n,
                             int* __restrict__ hist) {
  __shared__ int sh[EB_KEY_LEVELS + 1];
  for (int i = threadIdx.x; i <= EB_KEY_LEVELS; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += gridDim.x * blockDim.x) {
    unsigned long long x = keys[i] ^ keys[i - 1];
    if (x == 0) continue;
    int hb = 63 - __clzll((long long)x);
    int lfirst = EB_KEY_LEVELS - hb / 2;
    atomicAdd(&sh[lfirst], 1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= EB_KEY_LEVELS; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
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

// Every level at once: flags[l*n + i] = 1 where sorted point i starts a box of level l
// (l = 0..L). One exclusive scan over the concatenated rows then gives each head its
// global box id (rows in level order: level l's ids start at lev_off[l]).
__global__ void k_heads_all(const unsigned long long* __restrict__ keys, int n, int L,
                            int* __restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long k = keys[i], kp = i > 0 ? keys[i - 1] : 0ull;
  for (int l = 0; l <= L; ++l) {
    const int sh = 2 * (EB_KEY_LEVELS - l);
    flags[(size_t)l * n + i] = (i == 0) || ((k >> sh) != (kp >> sh));
  }
}

// Box key, first point and parent of every box; a box whose head point also starts its
// parent is the parent's first child.
__global__ void k_boxes_all(const unsigned long long* __restrict__ keys, int n, int L,
                            const int* __restrict__ flags, const int* __restrict__ scan,
                            unsigned long long* __restrict__ bkey, int* __restrict__ pt0,
                            int* __restrict__ parent, int* __restrict__ child0) {
  const long long tot = (long long)(L + 1) * n;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < tot;
       idx += (long long)gridDim.x * blockDim.x) {
    if (!flags[idx]) continue;
    const int l = (int)(idx / n), i = (int)(idx - (long long)l * n);
    const int b = scan[idx];
    bkey[b] = keys[i] >> (2 * (EB_KEY_LEVELS - l));
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

// Point range end, children count (and no children at the leaf level) of every box.
__global__ void k_boxes_fin(int nbox, LevOffT lo, int L, int n, int* __restrict__ child0,
                            int* __restrict__ nchild, const int* __restrict__ pt0,
                            int* __restrict__ pt1) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbox) return;
  int l = 0;
  while (b >= lo.v[l + 1]) ++l;
  const bool last = b + 1 >= lo.v[l + 1];
  pt1[b] = last ? n : pt0[b + 1];
  if (l == L) {
    child0[b] = -1;
    nchild[b] = 0;
  } else {
    nchild[b] = (last ? lo.v[l + 2] : child0[b + 1]) - child0[b];
  }
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

// V lists of every box of levels 2..L in one launch (the box's level from lev_off).
__global__ void k_vlist(const unsigned long long* __restrict__ bkey, LevOffT lo, int first, int nbox,
                        int* __restrict__ vlist, unsigned char* __restrict__ vcode,
                        int* __restrict__ vcount) {
  const int gid = first + blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nbox) return;
  int lev = 0;
  while (gid >= lo.v[lev + 1]) ++lev;
  const int off = lo.v[lev], nb = lo.v[lev + 1] - off;
  unsigned long long key = bkey[gid];
  int ix = (int)compact2(key), iy = (int)compact2(key >> 1);
  int px = ix >> 1, py = iy >> 1, half = 1 << (lev - 1), side = 1 << lev;
  int cnt = 0;
  for (int qy = py - 1; qy <= py + 1; ++qy) {
    if (qy < 0 || qy >= half) continue;
    for (int qx = px - 1; qx <= px + 1; ++qx) {
      if (qx < 0 || qx >= half) continue;
      for (int cy = 0; cy < 2; ++cy)
        for (int cx = 0; cx < 2; ++cx) {
          int sx = 2 * qx + cx, sy = 2 * qy + cy;
          int dx = ix - sx, dy = iy - sy;
          if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1) continue;
          if (sx >= side || sy >= side) continue;
          int s = find_box(bkey, off, nb, morton((unsigned)sx, (unsigned)sy));
          if (s < 0) continue;
          vlist[(size_t)gid * EB_VMAX + cnt] = s;
          vcode[(size_t)gid * EB_VMAX + cnt] = (unsigned char)((dy + 3) * 7 + (dx + 3));
          ++cnt;
        }
    }
  }
  vcount[gid] = cnt;
}

__global__ void k_ulist(const unsigned long long* __restrict__ bkey, int off, int nb, int lev,
                        int* __restrict__ ulist, int* __restrict__ ucount) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  unsigned long long key = bkey[off + b];
  int ix = (int)compact2(key), iy = (int)compact2(key >> 1);
  int side = 1 << lev, cnt = 0;
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      int sx = ix + dx, sy = iy + dy;
      if (sx < 0 || sy < 0 || sx >= side || sy >= side) continue;
      int s = find_box(bkey, off, nb, morton((unsigned)sx, (unsigned)sy));
      if (s < 0) continue;
      ulist[(size_t)b * EB_UMAX + cnt] = s;
      ++cnt;
    }
  ucount[b] = cnt;
}

__global__ void k_pair_counts(int off, int nleaf, const int* __restrict__ pt0,
                              const int* __restrict__ pt1, const int* __restrict__ ulist,
                              const int* __restrict__ ucount, int vfirst, int vlast,
                              const int* __restrict__ vcount,
                              unsigned long long* __restrict__ out) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long up = 0, vp = 0;
  if (b < nleaf) {
    int nt = pt1[off + b] - pt0[off + b];
    long long ns = 0;
    for (int j = 0; j < ucount[b]; ++j) {
      int s = ulist[(size_t)b * EB_UMAX + j];
      ns += pt1[s] - pt0[s];
    }
    up = (unsigned long long)(nt * ns - nt);
  }
  for (int g = vfirst + blockIdx.x * blockDim.x + threadIdx.x; g < vlast; g += gridDim.x * blockDim.x)
    vp += (unsigned long long)vcount[g];
  up = warp_sum<unsigned long long>(up);
  vp = warp_sum<unsigned long long>(vp);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out[0], up);
    atomicAdd(&out[1], vp);
  }
}

__global__ void k_group_count(int off, int nleaf, const int* __restrict__ pt0,
                              const int* __restrict__ pt1, int* __restrict__ cnt) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaf) return;
  cnt[b] = (pt1[off + b] - pt0[off + b] + EB_GROUP - 1) / EB_GROUP;
}

__global__ void k_group_fill(int off, int nleaf, const int* __restrict__ pt0,
                             const int* __restrict__ cnt, const int* __restrict__ start,
                             int* __restrict__ gleaf, int* __restrict__ gfirst) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaf) return;
  int g0 = start[b];
  for (int g = 0; g < cnt[b]; ++g) {
    gleaf[g0 + g] = b;
    gfirst[g0 + g] = pt0[off + b] + g * EB_GROUP;
  }
}

__global__ void k_tile_count(int off, int nleaf, const int* __restrict__ pt0,
                             const int* __restrict__ pt1, int* __restrict__ cnt) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaf) return;
  cnt[b] = (pt1[off + b] - pt0[off + b] + EB_NTILE - 1) / EB_NTILE;
}

__global__ void k_tile_fill(int off, int nleaf, const int* __restrict__ pt0, const int* __restrict__ pt1,
                            const int* __restrict__ cnt, const int* __restrict__ start,
                            int4* __restrict__ tiles) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaf) return;
  const int g0 = start[b], c = cnt[b], a = pt0[off + b], nt = pt1[off + b] - a;
  for (int g = 0; g < c; ++g)
    tiles[g0 + g] = make_int4(b, a + (int)((long long)g * nt / c), a + (int)((long long)(g + 1) * nt / c), 0);
}

__global__ void k_ancestors(int off, int nleaf, int na, const int* __restrict__ parent, int* __restrict__ anc) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nleaf) return;
  int a = off + b;
  for (int q = 0; q < na; ++q) {
    anc[(size_t)b * na + q] = a;
    if (q + 1 < na) a = parent[a];
  }
}

__global__ void k_chunk_count(int first, int nb, const int* __restrict__ pt0, const int* __restrict__ pt1,
                              int* __restrict__ cnt) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  cnt[b] = (pt1[first + b] - pt0[first + b] + EB_CHUNK - 1) / EB_CHUNK;
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

__global__ void k_leaf_coords(int offL, const unsigned long long* __restrict__ bkey,
                              const int* __restrict__ pt0, const int* __restrict__ pt1,
                              const double2* __restrict__ zs, double x0, double y0, double r,
                              float4* __restrict__ wa, float2* __restrict__ wb) {
  const int b = offL + blockIdx.x;
  const unsigned long long k = bkey[b];
  const unsigned int ix = compact2(k), iy = compact2(k >> 1);
  for (int i = pt0[b] + threadIdx.x; i < pt1[b]; i += blockDim.x) {
    double2 z = zs[i];
    float xh, xm, xl, yh, ym, yl;
    split3(leaf_offset(z.x, x0, ix, r), xh, xm, xl);
    split3(leaf_offset(z.y, y0, iy, r), yh, ym, yl);
    wa[i] = make_float4(xh, yh, xm, ym);
    wb[i] = make_float2(xl, yl);
  }
}

int eb_tree_build(eb_ctx* ctx, EbTree& t, const double2* z, int n, int leaf_target) {
  cudaStream_t st = eb_stream(ctx);
  t.valid = false;
  if (n <= 0) return EB_ERR_ARG;
  if (leaf_target < 1) leaf_target = 32;
  t.n = n;
  const int BS = 256;
  if (!t.host) EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&t.host), sizeof(EbTreeHost)));
  EbTreeHost* H = t.host;
  t.pairs_read = false;
  // 1. bounding square, on the device (read back with the level histogram below)
  int nbb = std::min(nblk(n, BS), 1024);
  EB_TRY(t.partial.ensure(sizeof(Box4) * (size_t)nbb));
  EB_TRY(t.bbox.ensure(sizeof(Box4) + sizeof(double) * 4 + sizeof(int) * 4));
  double* sq = reinterpret_cast<double*>(t.bbox.as<char>() + sizeof(Box4));
  int* bad = reinterpret_cast<int*>(sq + 4);
  EB_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), st));
  k_bbox<<<nbb, BS, 0, st>>>(z, n, t.partial.as<Box4>(), bad);
  eb_count_launch(ctx);
  k_bbox_final<<<1, 32, 0, st>>>(t.partial.as<Box4>(), nbb, t.bbox.as<Box4>(), sq);
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemcpyAsync(H->sq, sq, sizeof(H->sq), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
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
  // 3. sorted positions
  EB_TRY(t.zs.ensure(sizeof(double2) * (size_t)n));
  EB_TRY(t.zhl.ensure(sizeof(float4) * (size_t)n));
  k_gather_points<<<nblk(n, BS), BS, 0, st>>>(z, t.perm.as<int>(), n, t.zs.as<double2>(),
                                              t.zhl.as<float4>());
  eb_count_launch(ctx);
  // 4. occupied boxes per level, leaf level
  EB_TRY(t.hist.ensure(sizeof(int) * (EB_KEY_LEVELS + 1)));
  EB_CUDA_TRY(cudaMemsetAsync(t.hist.p, 0, sizeof(int) * (EB_KEY_LEVELS + 1), st));
  k_level_hist<<<std::min(nblk(n, BS), 1024), BS, 0, st>>>(t.keys.as<unsigned long long>(), n,
                                                          t.hist.as<int>());
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemcpyAsync(H->hist, t.hist.p, sizeof(H->hist), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaStreamSynchronize(st));
  if (H->bad) {
    eb_set_last_error_msg("non-finite node coordinate");
    return EB_ERR_NAN;
  }
  t.W = H->sq[0];
  t.x0 = H->sq[1];
  t.y0 = H->sq[2];
  const int* hist = H->hist;
  int nb[EB_KEY_LEVELS + 1];
  nb[0] = 1;
  for (int l = 1; l <= EB_KEY_LEVELS; ++l) nb[l] = nb[l - 1] + hist[l];
  int L = EB_KEY_LEVELS;
  for (int l = 0; l <= EB_KEY_LEVELS; ++l)
    if ((double)n / nb[l] <= (double)leaf_target) { L = l; break; }
  t.L = L;
  t.lev_off[0] = 0;
  for (int l = 0; l <= L; ++l) t.lev_off[l + 1] = t.lev_off[l] + nb[l];
  t.nbox = t.lev_off[L + 1];
  t.nleaf = nb[L];
  size_t NB = (size_t)t.nbox;
  EB_TRY(t.bkey.ensure(sizeof(unsigned long long) * NB));
  EB_TRY(t.pt0.ensure(sizeof(int) * NB));
  EB_TRY(t.pt1.ensure(sizeof(int) * NB));
  EB_TRY(t.parent.ensure(sizeof(int) * NB));
  EB_TRY(t.child0.ensure(sizeof(int) * NB));
  EB_TRY(t.nchild.ensure(sizeof(int) * NB));
  // 5. boxes of every level in three launches (heads, one scan, fill) and a finish
  const size_t nflag = (size_t)(L + 1) * n;
  EB_TRY(t.flags.ensure(sizeof(int) * nflag));
  EB_TRY(t.scan.ensure(sizeof(int) * nflag));
  k_heads_all<<<nblk(n, BS), BS, 0, st>>>(t.keys.as<unsigned long long>(), n, L, t.flags.as<int>());
  eb_count_launch(ctx);
  {
    size_t need = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, need, t.flags.as<int>(), t.scan.as<int>(), (int)nflag, st);
    if (need > t.cubtmp.bytes) EB_TRY(t.cubtmp.ensure(need));
  }
  tb = t.cubtmp.bytes;
  EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, t.flags.as<int>(), t.scan.as<int>(), (int)nflag, st));
  eb_count_launch(ctx);
  k_boxes_all<<<std::min(nblk((long long)nflag, BS), ctx->nsm * 16), BS, 0, st>>>(
      t.keys.as<unsigned long long>(), n, L, t.flags.as<int>(), t.scan.as<int>(),
      t.bkey.as<unsigned long long>(), t.pt0.as<int>(), t.parent.as<int>(), t.child0.as<int>());
  eb_count_launch(ctx);
  {
    LevOffT lo;
    for (int l = 0; l < EB_KEY_LEVELS + 3; ++l) lo.v[l] = t.lev_off[std::min(l, L + 1)];
    k_boxes_fin<<<nblk(t.nbox, BS), BS, 0, st>>>(t.nbox, lo, L, n, t.child0.as<int>(), t.nchild.as<int>(),
                                                 t.pt0.as<int>(), t.pt1.as<int>());
    eb_count_launch(ctx);
  }
  // 7. interaction lists
  EB_TRY(t.vlist.ensure(sizeof(int) * NB * EB_VMAX));
  EB_TRY(t.vcode.ensure(NB * EB_VMAX));
  EB_TRY(t.vcount.ensure(sizeof(int) * NB));
  EB_CUDA_TRY(cudaMemsetAsync(t.vcount.p, 0, sizeof(int) * NB, st));
  if (L >= 2) {
    LevOffT lo;
    for (int l = 0; l < EB_KEY_LEVELS + 3; ++l) lo.v[l] = t.lev_off[std::min(l, L + 1)];
    const int first = t.lev_off[2];
    k_vlist<<<nblk(t.nbox - first, 128), 128, 0, st>>>(t.bkey.as<unsigned long long>(), lo, first, t.nbox,
                                                       t.vlist.as<int>(), t.vcode.as<unsigned char>(),
                                                       t.vcount.as<int>());
    eb_count_launch(ctx);
  }
  EB_TRY(t.ulist.ensure(sizeof(int) * (size_t)t.nleaf * EB_UMAX));
  EB_TRY(t.ucount.ensure(sizeof(int) * (size_t)t.nleaf));
  k_ulist<<<nblk(t.nleaf, 128), 128, 0, st>>>(t.bkey.as<unsigned long long>(), t.lev_off[L], t.nleaf, L,
                                             t.ulist.as<int>(), t.ucount.as<int>());
  eb_count_launch(ctx);
  // 8. work items, counted and scanned first so that one synchronisation sizes them all:
  // near-field groups of EB_GROUP targets, shared-memory tiles of at most EB_NTILE
  // targets, and FP32 direct-P2M chunks of at most EB_CHUNK points of every box of the
  // chunked levels (every level up to 256K points, so that no dependent M2M launches
  // remain on the critical path; above that the EB_DIRECT_LEVELS finest)
  const int nl = t.nleaf;
  EB_TRY(t.tcount.ensure(sizeof(int) * (size_t)nl));
  EB_TRY(t.tstart.ensure(sizeof(int) * (size_t)nl));
  k_group_count<<<nblk(nl, BS), BS, 0, st>>>(t.lev_off[L], nl, t.pt0.as<int>(), t.pt1.as<int>(),
                                             t.flags.as<int>());
  eb_count_launch(ctx);
  tb = t.cubtmp.bytes;
  EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, t.flags.as<int>(), t.scan.as<int>(), nl, st));
  eb_count_launch(ctx);
  k_tile_count<<<nblk(nl, BS), BS, 0, st>>>(t.lev_off[L], nl, t.pt0.as<int>(), t.pt1.as<int>(),
                                            t.tcount.as<int>());
  eb_count_launch(ctx);
  tb = t.cubtmp.bytes;
  EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, t.tcount.as<int>(), t.tstart.as<int>(), nl, st));
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[0], t.flags.as<int>() + nl - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[1], t.scan.as<int>() + nl - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[2], t.tcount.as<int>() + nl - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaMemcpyAsync(&H->last[3], t.tstart.as<int>() + nl - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  t.nchunk = 0;
  t.chunk_lmin = n <= (1 << 18) ? 2 : std::max(2, L - EB_DIRECT_LEVELS + 1);
  const int cfirst = t.lev_off[t.chunk_lmin], nb2 = t.nbox - cfirst;
  if (L >= 2) {
    EB_TRY(t.ccount.ensure(sizeof(int) * (size_t)nb2));
    EB_TRY(t.cstart.ensure(sizeof(int) * (size_t)(nb2 + 1)));
    EB_TRY(t.cdone.ensure(sizeof(int) * (size_t)nb2));
    EB_CUDA_TRY(cudaMemsetAsync(t.cdone.p, 0, sizeof(int) * (size_t)nb2, st));
    k_chunk_count<<<nblk(nb2, BS), BS, 0, st>>>(cfirst, nb2, t.pt0.as<int>(), t.pt1.as<int>(), t.ccount.as<int>());
    eb_count_launch(ctx);
    size_t need = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, need, t.ccount.as<int>(), t.cstart.as<int>(), nb2, st);
    if (need > t.cubtmp.bytes) EB_TRY(t.cubtmp.ensure(need));
    tb = t.cubtmp.bytes;
    EB_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t.cubtmp.p, tb, t.ccount.as<int>(), t.cstart.as<int>(), nb2, st));
    eb_count_launch(ctx);
    EB_CUDA_TRY(cudaMemcpyAsync(&H->last[4], t.ccount.as<int>() + nb2 - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    EB_CUDA_TRY(cudaMemcpyAsync(&H->last[5], t.cstart.as<int>() + nb2 - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  }
  EB_CUDA_TRY(cudaStreamSynchronize(st));
  t.ngroup = H->last[0] + H->last[1];
  t.ntile = H->last[2] + H->last[3];
  EB_TRY(t.gleaf.ensure(sizeof(int) * (size_t)t.ngroup));
  EB_TRY(t.gfirst.ensure(sizeof(int) * (size_t)t.ngroup));
  k_group_fill<<<nblk(nl, BS), BS, 0, st>>>(t.lev_off[L], nl, t.pt0.as<int>(), t.flags.as<int>(),
                                            t.scan.as<int>(), t.gleaf.as<int>(), t.gfirst.as<int>());
  eb_count_launch(ctx);
  EB_TRY(t.tiles.ensure(sizeof(int4) * (size_t)t.ntile));
  k_tile_fill<<<nblk(nl, BS), BS, 0, st>>>(t.lev_off[L], nl, t.pt0.as<int>(), t.pt1.as<int>(),
                                           t.tcount.as<int>(), t.tstart.as<int>(), t.tiles.as<int4>());
  eb_count_launch(ctx);
  if (L >= 2) {
    EB_TRY(t.anc.ensure(sizeof(int) * (size_t)t.nleaf * (L - 1)));
    k_ancestors<<<nblk(t.nleaf, BS), BS, 0, st>>>(t.lev_off[L], t.nleaf, L - 1, t.parent.as<int>(),
                                                  t.anc.as<int>());
    eb_count_launch(ctx);
    t.nchunk = H->last[4] + H->last[5];
    EB_CUDA_TRY(cudaMemcpyAsync(t.cstart.as<int>() + nb2, &t.nchunk, sizeof(int), cudaMemcpyHostToDevice, st));
    EB_TRY(t.chunk_box.ensure(sizeof(int) * (size_t)t.nchunk));
    k_chunk_fill<<<nblk(nb2, BS), BS, 0, st>>>(cfirst, nb2, t.ccount.as<int>(), t.cstart.as<int>(),
                                               t.chunk_box.as<int>());
    eb_count_launch(ctx);
  }
  // 9. leaf-relative coordinates for the double-float near field
  EB_TRY(t.wdf.ensure(sizeof(float4) * (size_t)n));
  EB_TRY(t.wdf_lo.ensure(sizeof(float2) * (size_t)n));
  k_leaf_coords<<<t.nleaf, 64, 0, st>>>(t.lev_off[L], t.bkey.as<unsigned long long>(), t.pt0.as<int>(),
                                        t.pt1.as<int>(), t.zs.as<double2>(), t.x0, t.y0,
                                        t.W / (double)(1u << L), t.wdf.as<float4>(),
                                        t.wdf_lo.as<float2>());
  eb_count_launch(ctx);
  // 10. pair counts (the algorithmic work of the near field and M2L), copied to the host
  // without waiting; eb_tree_pairs reads them
  EB_TRY(t.pairs.ensure(2 * sizeof(unsigned long long)));
  unsigned long long* cnt = t.pairs.as<unsigned long long>();
  EB_CUDA_TRY(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), st));
  int vfirst = t.lev_off[std::min(2, L + 1)], vlast = t.nbox;
  k_pair_counts<<<std::max(nblk(t.nleaf, BS), 1), BS, 0, st>>>(
      t.lev_off[L], t.nleaf, t.pt0.as<int>(), t.pt1.as<int>(), t.ulist.as<int>(), t.ucount.as<int>(),
      vfirst, vlast, t.vcount.as<int>(), cnt);
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemcpyAsync(H->pairs, cnt, sizeof(H->pairs), cudaMemcpyDeviceToHost, st));
  EB_TRY(eb_check_launch(ctx, "tree build"));
  t.valid = true;
  return EB_OK;
}

int eb_tree_pairs(eb_ctx* ctx, EbTree& t) {
  if (!t.pairs_read) {
    EB_CUDA_TRY(cudaStreamSynchronize(eb_stream(ctx)));
    t.u_pairs = (long long)t.host->pairs[0];
    t.v_pairs = (long long)t.host->pairs[1];
    t.pairs_read = true;
  }
  return EB_OK;
}

EbTree::~EbTree() {
  if (host) cudaFreeHost(host);
}
