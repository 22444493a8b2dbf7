// Stokes layer sum for callers that cannot allocate GPU memory.
//
// Every other entry point of this library draws its working memory (trees, expansions,
// Krylov vectors) from cudaMalloc through an eb_ctx. Some callers cannot allow that:
// a Fortran or C host that owns all device memory itself and hands the library only
// buffers it allocated at start-up, code running inside a memory-pool or allocator
// callback (where a nested cudaMalloc would deadlock or recurse), and real-time loops
// that forbid any allocation after initialisation. eb_stokes_sum_noalloc serves them:
// it takes device pointers for every input and output, needs no eb_ctx, and keeps its
// only scratch, three complex charges per node, in g_noalloc_charges below, a fixed
// array in the library's own device memory (EB_NOALLOC_MAX_POINTS nodes, 768 KiB),
// which every GPU that loads the library holds until the process exits.
//
// It evaluates the same sum as eb_stokes_sum (what CADAPDR, sign -1, and CADAPMOD,
// sign +1, compute at the nodes, self excluded), by direct summation in FP64.
#include <mutex>

#include "eb_internal.h"

// Per node: P = qa + s qb, Q = qa - s qb, A = -s conj(qa) (the near-field combinations
// of the charges of cadapdrop.f:214-222). Shared by every call on a device; a call
// rewrites the first 3 n entries before reading them, so nothing needs clearing. In host
// code this name stands for the array but is not its device address: kernels receive
// the address cudaGetSymbolAddress returns.
static __device__ __align__(256) double2 g_noalloc_charges[3 * EB_NOALLOC_MAX_POINTS];

namespace {

constexpr int kMaxDevices = 64;
constexpr int kTile = 128;

std::mutex g_mutex;
double2* g_scratch[kMaxDevices] = {nullptr};

__global__ void k_noalloc_charges(int n, const double2* __restrict__ dens,
                                  const double2* __restrict__ dz, const double* __restrict__ h,
                                  double s, double2* __restrict__ ch) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 u = dens[i], d = dz[i];
  double hf = h[i] * (1.0 / (2.0 * EB_PI));
  double2 w = cmul<double>(u, d);
  double2 a = make_double2(w.y * hf, -w.x * hf);  // u dz h / (2 pi i)
  double2 v = csub<double>(cmul<double>(u, cconj<double>(d)), cmul<double>(cconj<double>(u), d));
  double2 b = make_double2(v.y * hf, -v.x * hf);  // (-conj(u) dz + u conj(dz)) h / (2 pi i)
  ch[3 * i] = make_double2(a.x + s * b.x, a.y + s * b.y);
  ch[3 * i + 1] = make_double2(a.x - s * b.x, a.y - s * b.y);
  ch[3 * i + 2] = make_double2(-s * a.x, s * a.y);
}

// gradw_i = sum_{j != i} qa/D + s [conj(qb/D) - D conj(qa) conj(1/D)^2], D = z_j - z_i,
// with source tiles staged in shared memory.
__global__ void __launch_bounds__(kTile) k_noalloc_direct(int n, const double2* __restrict__ z,
                                                         const double2* __restrict__ ch,
                                                         double2* __restrict__ out) {
  __shared__ double2 sz[kTile], sp[kTile], sq[kTile], sa[kTile];
  int i = blockIdx.x * kTile + threadIdx.x;
  double2 zi = (i < n) ? z[i] : make_double2(0.0, 0.0);
  double gx = 0.0, gy = 0.0;
  for (int base = 0; base < n; base += kTile) {
    int j = base + threadIdx.x;
    if (j < n) {
      sz[threadIdx.x] = z[j];
      sp[threadIdx.x] = ch[3 * j];
      sq[threadIdx.x] = ch[3 * j + 1];
      sa[threadIdx.x] = ch[3 * j + 2];
    }
    __syncthreads();
    int m = min(kTile, n - base);
    for (int jj = 0; jj < m; ++jj) {
      if (base + jj == i) continue;
      double dx = sz[jj].x - zi.x, dy = sz[jj].y - zi.y;
      double rr = 1.0 / fma(dx, dx, dy * dy);
      double ix = dx * rr, iy = -dy * rr;
      double2 P = sp[jj], Q = sq[jj], A = sa[jj];
      gx = fma(P.x, ix, fma(-P.y, iy, gx));
      gy = fma(Q.x, iy, fma(Q.y, ix, gy));
      double w2x = fma(ix, ix, -iy * iy), w2y = -2.0 * ix * iy;
      double tx = fma(dx, w2x, -dy * w2y), ty = fma(dx, w2y, dy * w2x);
      gx = fma(A.x, tx, fma(-A.y, ty, gx));
      gy = fma(A.x, ty, fma(A.y, tx, gy));
    }
    __syncthreads();
  }
  if (i < n) out[i] = make_double2(gx, gy);
}

}  // namespace

// Set-up: the first call on each device (with that device current) looks up the device
// address of g_noalloc_charges with cudaGetSymbolAddress and keeps it for later calls.
// Under CUDA's default lazy module loading that lookup is also what loads this
// library's device code onto the device, which reserves device memory for the code and
// for the array: make the first call at start-up, outside allocator callbacks and before
// capturing any stream into a graph. Later calls allocate nothing: there is no
// cudaMalloc, cudaFree or allocating library routine on this path. The address belongs
// to the device's primary context (the one the CUDA runtime uses); callers that run
// their own driver-API contexts or reset the device must not use this entry point.
// Calls that overlap on the GPU (concurrent streams, or several host threads on one
// device) share g_noalloc_charges and race; order them on one stream.
int eb_stokes_sum_noalloc(int n, const double* z, const double* dz, const double* h,
                          const double* dens, int sign, double* gradw, void* stream) {
  if (n <= 0 || !z || !dz || !h || !dens || !gradw || (sign != 1 && sign != -1)) {
    eb_set_last_error_msg("eb_stokes_sum_noalloc: invalid argument");
    return EB_ERR_ARG;
  }
  // complex arrays are read and written as 16-byte double2 values, h as 8-byte doubles
  if ((reinterpret_cast<uintptr_t>(z) | reinterpret_cast<uintptr_t>(dz) | reinterpret_cast<uintptr_t>(dens) |
       reinterpret_cast<uintptr_t>(gradw)) & 15u || (reinterpret_cast<uintptr_t>(h) & 7u)) {
    eb_set_last_error_msg("eb_stokes_sum_noalloc: z, dz, dens, gradw must be 16-byte aligned, h 8-byte aligned");
    return EB_ERR_ARG;
  }
  if (n > EB_NOALLOC_MAX_POINTS) {
    eb_set_last_error_msg("eb_stokes_sum_noalloc: n exceeds EB_NOALLOC_MAX_POINTS (16384 nodes)");
    return EB_ERR_WORKSPACE;
  }
  int dev = 0;
  EB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    eb_set_last_error_msg("eb_stokes_sum_noalloc: device ordinal beyond 63");
    return EB_ERR_ARG;
  }
  double2* ch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_charges);
      if (e != cudaSuccess || !p) {
        eb_set_last_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_charges)", __FILE__, __LINE__);
        return EB_ERR_CUDA;
      }
      g_scratch[dev] = static_cast<double2*>(p);
    }
    ch = g_scratch[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int blocks = (n + kTile - 1) / kTile;
  k_noalloc_charges<<<blocks, kTile, 0, s>>>(n, reinterpret_cast<const double2*>(dens),
                                             reinterpret_cast<const double2*>(dz), h, (double)sign, ch);
  k_noalloc_direct<<<blocks, kTile, 0, s>>>(n, reinterpret_cast<const double2*>(z), ch,
                                            reinterpret_cast<double2*>(gradw));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    eb_set_last_cuda_error(e, "eb_stokes_sum_noalloc launch", __FILE__, __LINE__);
    return EB_ERR_CUDA;
  }
  return EB_OK;
}
