// M2L of the FP32 operator as a contraction on the 5th-generation tensor cores.
//
// SLSHIFT (cadap2.f:1149-1215) and DSLNEW (dapif3.f:1200-1289) factor the M2L of an
// interaction-list entry with offset d (in box units) as
//   a_k = M_k d^-k (after moving psi to the target centre),
//   b_m = sum_k C(m+k-1, m) a_k          (a fixed binomial matrix),
//   L_m += (-1)^m d^-m b_m.
// Stacking the entries of a target box's V list turns the middle step into a dense
// product B = A C: A holds one row per entry and real component (Re / Im of a for phi
// and for psi: 4 rows per entry, at most 27 entries = 108 of the 128 rows of a tile) and
// K = 24 columns (k = 1..20, zero beyond the entry's truncation order), C is the 24 x 32
// binomial matrix (m = 0..20). The product runs as tcgen05.mma (kind::tf32, M = 128,
// N = 32, K = 8 per instruction) with the accumulator in tensor memory; FP32 accuracy
// comes from the 3xTF32 split x = x_hi + x_lo (x_hi = tf32(x), x_lo = tf32(x - x_hi)):
// A C ~ A_hi C_hi + A_hi C_lo + A_lo C_hi, nine instructions per tile. The pre- and
// post-scalings, the gathers and the sums over the entries stay on the CUDA cores.
//
// Operands are staged in shared memory in the canonical no-swizzle K-major layout: core
// matrices of 8 rows x 16 bytes (4 tf32), the K-adjacent core matrices 128 bytes apart
// (leading-dimension offset) and the 8-row groups 6 x 128 = 768 bytes apart (stride
// offset). One block of 128 threads takes target boxes in turn; its 32 tensor-memory
// columns are allocated once and freed before it exits, and every wait is bounded (on
// a timeout the block marks its expansions non-finite, which the solver reports).
#include <stdint.h>

#include <algorithm>

#include "eb_internal.h"

namespace {

constexpr int TC_P = 20;        // expansion order of the FP32 operator handled here
constexpr int TC_K = 24;        // K padded to three instructions of 8
constexpr int TC_N = 32;        // output orders m = 0..20, padded
constexpr int TC_ROWS = 128;    // rows of a tile (M)
constexpr int TC_KCH = TC_K / 4;  // 16-byte chunks along K per row group
constexpr uint32_t TC_LBO = 128, TC_SBO = TC_KCH * 128;
constexpr int TC_A_BYTES = TC_ROWS * TC_K * 4;  // 12 KiB
constexpr int TC_B_BYTES = TC_N * TC_K * 4;     // 3 KiB
constexpr int TC_LD = 33;                        // epilogue staging row stride (floats)
constexpr long long TC_WAIT_LIMIT = 1ll << 22;
constexpr int TC_PARTS = 3;                      // epilogue threads per output (3 x 42 <= 128)

// byte offset of element (row, k) in the blocked K-major layout
__device__ __forceinline__ int tc_off(int row, int k) {
  return ((row >> 3) * TC_KCH + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: start address, leading- and stride-dimension byte
// offsets (16-byte units), the fixed version bits 46-48 = 0b001, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(TC_LBO >> 4) << 16) |
         ((uint64_t)(TC_SBO >> 4) << 32) | (1ull << 46);
}

// instruction descriptor: D f32 (bits 4-5 = 1), A and B tf32 (bits 7-9, 10-12 = 2),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                              ((uint32_t)(TC_ROWS >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t taddr, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
      "l"(a), "l"(b), "r"(TC_IDESC), "r"(acc));
}

template <int E>
__global__ void __launch_bounds__(128) k_m2l_tc(int first, int ntarget, const int* __restrict__ vlist,
                                                const unsigned char* __restrict__ vcode,
                                                const int* __restrict__ vcount,
                                                const float* __restrict__ binom, int ldb,
                                                const float2* __restrict__ dinv,
                                                const int* __restrict__ pdv,
                                                const float2* __restrict__ mpole,
                                                float2* __restrict__ local) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sAh = sm;
  unsigned char* sAl = sAh + TC_A_BYTES;
  unsigned char* sBh = sAl + TC_A_BYTES;
  unsigned char* sBl = sBh + TC_B_BYTES;
  float* sD = reinterpret_cast<float*>(sBl + TC_B_BYTES);  // [128][TC_LD]
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t s_taddr;
  __shared__ int s_src[EB_VMAX], s_code[EB_VMAX], s_pd[EB_VMAX];
  __shared__ int s_fail;
  constexpr int ldl = TC_P + 1, ldd = TC_P + 2;
  const int tid = threadIdx.x, warp = tid >> 5;

  // binomial operand (N x K, K-major): row m, column k-1 = C(m+k-1, m), split in two
  for (int idx = tid; idx < TC_N * TC_K; idx += 128) {
    const int m = idx / TC_K, kk = idx - m * TC_K;
    const float c = (m <= TC_P && kk < TC_P) ? binom[(size_t)(m + kk) * ldb + m] : 0.f;
    const float h = tf32_round(c);
    *reinterpret_cast<float*>(sBh + tc_off(m, kk)) = h;
    *reinterpret_cast<float*>(sBl + tc_off(m, kk)) = tf32_round(c - h);
  }
  if (tid == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_taddr)),
                 "r"(TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t taddr = s_taddr;
  uint32_t phase = 0;

  for (int tb = blockIdx.x; tb < ntarget; tb += gridDim.x) {
    const int gid = first + tb;
    const int nv = vcount[gid];
    if (tid < nv) {
      const int code = vcode[(size_t)gid * EB_VMAX + tid];
      s_src[tid] = vlist[(size_t)gid * EB_VMAX + tid];
      s_code[tid] = code;
      s_pd[tid] = pdv[code];
    }
    __syncthreads();
    // A: row 4j + q, q = Re / Im of a_phi, Re / Im of a_psi of entry j; k-1 in columns.
    // One thread per (entry, k) forms both expansions' a_k and writes its four rows.
    for (int idx = tid; idx < (TC_ROWS / 4) * TC_K; idx += 128) {
      const int j = idx / TC_K, kk = idx - j * TC_K;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (j < nv && kk < s_pd[j]) {
        const int code = s_code[j], k = kk + 1;
        const float2* ms = mpole + (size_t)s_src[j] * E * TC_P;
        const float2 sc = dinv[(size_t)code * ldd + k];
        const float2 a = cmul<float>(ms[kk], sc);
        v[0] = a.x;
        v[1] = a.y;
        if (E == 2) {
          float2 mv = ms[TC_P + kk];
          if (k >= 2) {
            const float dxr = (float)(code % 7 - 3), dyr = (float)(code / 7 - 3);
            cfma<float>(mv, make_float2(-dxr * (float)(k - 1), dyr * (float)(k - 1)), ms[kk - 1]);
          }
          const float2 b = cmul<float>(mv, sc);
          v[2] = b.x;
          v[3] = b.y;
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float h = tf32_round(v[q]);
        *reinterpret_cast<float*>(sAh + tc_off(4 * j + q, kk)) = h;
        *reinterpret_cast<float*>(sAl + tc_off(4 * j + q, kk)) = tf32_round(v[q] - h);
      }
    }
    // make the generic-proxy stores visible to the tensor cores' (async) proxy
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ah = smem_u32(sAh), al = smem_u32(sAl), bh = smem_u32(sBh), bl = smem_u32(sBl);
#pragma unroll
      for (int s = 0; s < TC_K / 8; ++s) {
        const uint32_t o = (uint32_t)s * 256u;  // two 16-byte chunks along K per instruction
        tc_mma(taddr, tc_desc(ah + o), tc_desc(bh + o), s > 0 ? 1u : 0u);
        tc_mma(taddr, tc_desc(ah + o), tc_desc(bl + o), 1u);
        tc_mma(taddr, tc_desc(al + o), tc_desc(bh + o), 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar)));
    }
    // every thread waits for the products (bounded)
    {
      uint32_t done = 0;
      long long it = 0;
      while (!done) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(&mbar)), "r"(phase));
        if (++it > TC_WAIT_LIMIT) break;
      }
      if (!done) s_fail = 1;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (s_fail) break;
    // accumulator rows of this warp (lanes 32 warp ..) into shared memory
    {
      uint32_t r[32];
      const uint32_t ta = taddr + ((uint32_t)(warp * 32) << 16);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
            "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
            "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
            "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      float* drow = sD + (size_t)tid * TC_LD;
#pragma unroll
      for (int c = 0; c < 32; ++c) drow[c] = __uint_as_float(r[c]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // L_m = sum_j (-1)^m d_j^-m (b_re + i b_im), m <= pd_j: each output's entries are
    // split over TC_PARTS threads (every TC_PARTS-th entry), their sums added in order
    float2* spart = reinterpret_cast<float2*>(sAh);  // A is consumed: reuse it
    if (tid < TC_PARTS * E * ldl) {
      const int part = tid / (E * ldl), o = tid - part * (E * ldl);
      const int e = o / ldl, m = o - e * ldl;
      float2 acc = make_float2(0.f, 0.f);
      for (int j = part; j < nv; j += TC_PARTS) {
        if (m > s_pd[j]) continue;
        float2 post = dinv[(size_t)s_code[j] * ldd + m];
        if (m & 1) post = make_float2(-post.x, -post.y);
        const float2 b = make_float2(sD[(4 * j + 2 * e) * TC_LD + m], sD[(4 * j + 2 * e + 1) * TC_LD + m]);
        cfma<float>(acc, post, b);
      }
      spart[tid] = acc;
    }
    __syncthreads();
    if (tid < E * ldl) {
      float2 acc = spart[tid];
      for (int part = 1; part < TC_PARTS; ++part) acc = cadd<float>(acc, spart[part * E * ldl + tid]);
      local[(size_t)gid * E * ldl + tid] = acc;
    }
    __syncthreads();
  }
  if (s_fail) {
    // a wait ran out: mark this block's remaining expansions non-finite
    for (int tb = blockIdx.x; tb < ntarget; tb += gridDim.x)
      for (int idx = tid; idx < E * ldl; idx += 128)
        local[(size_t)(first + tb) * E * ldl + idx] = make_float2(__int_as_float(0x7fc00000), 0.f);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(TC_N));
}

}  // namespace

// Launches the tensor-core M2L for the FP32 operator (order 20) over the boxes
// [first, first + ntarget). Returns EB_ERR_ARG for another order.
int eb_m2l_tc(eb_ctx* ctx, int E, int first, int ntarget, const int* vlist, const unsigned char* vcode,
              const int* vcount, const float* binom, int ldb, const float2* dinv, const int* pd,
              const float2* mpole, float2* local, cudaStream_t st) {
  if (ntarget <= 0) return EB_OK;
  const size_t sm = 2 * (size_t)TC_A_BYTES + 2 * (size_t)TC_B_BYTES + sizeof(float) * TC_ROWS * TC_LD + 1024;
  const int grid = std::min(ntarget, ctx->nsm * 4);
  if (E == 2) {
    EB_CUDA_TRY(cudaFuncSetAttribute(k_m2l_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_m2l_tc<2><<<grid, 128, sm, st>>>(first, ntarget, vlist, vcode, vcount, binom, ldb, dinv, pd, mpole, local);
  } else if (E == 1) {
    EB_CUDA_TRY(cudaFuncSetAttribute(k_m2l_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_m2l_tc<1><<<grid, 128, sm, st>>>(first, ntarget, vlist, vcode, vcount, binom, ldb, dinv, pd, mpole, local);
  } else {
    return EB_ERR_ARG;
  }
  eb_count_launch(ctx);
  return EB_OK;
}
