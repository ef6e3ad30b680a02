// Allocation-free BSR3 SpMV with a fused dot product: y = A x and
// dot = (y, w), on device arrays the caller already owns.
//
// Who needs this: code that runs where it must not allocate device memory --
// a solver step inside a host framework that hands out a fixed device arena
// (Flow's linear-solver backends are called between Newton steps and manage
// their own buffers), or a real-time or callback context where cudaMalloc's
// implicit synchronisation is not allowed. The handle API allocates its
// scratch at gbilu_analyze time; this entry point uses no handle and calls
// no cudaMalloc, cudaFree or allocating library routine.
//
// y is written while x and w are read, with no aliasing between them
// assumed by the compiler: y must not alias x or w. (w may alias x.)
//
// Its only scratch is the file-scope device array below: one partial sum per
// CTA plus an arrival counter for the grid-wide reduction. Every GPU that
// loads the library holds this array (about 32 KiB) until the process exits.
// It limits one call to kNoAllocMaxCtas CTAs of 256 block rows each, i.e.
// nb <= 1,048,576 block rows; larger systems are rejected with
// GBILU_BAD_INPUT. Calls share the array: two calls that overlap on the GPU
// (different streams, or different host threads on one device) race on it
// and give wrong sums, so serialise them on one stream.
//
// The device address of the array is looked up once per device, on the
// first call made with that device current (cudaGetSymbolAddress); make that
// first call before any stream capture, since the lookup is not a stream
// operation. Later calls only enqueue work on the given stream. The address
// belongs to the context that was current at the lookup, the device's
// primary context when the caller uses the runtime API: calls made with
// another context current, or after a cudaDeviceReset (which destroys the
// primary context), would use a stale address, so neither is supported.
#include "gbilu.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace {

constexpr int kNoAllocThreads = 256;      // block rows per CTA (one thread each)
constexpr int kNoAllocMaxCtas = 4096;     // scratch holds this many partials
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
  double partial[kNoAllocMaxCtas];
  unsigned int arrived;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_lookup_mutex;
NoAllocScratch *g_scratch_ptr[kMaxDevices] = {};

// y_i = sum_k A_ik x_k over the plain BSR row; (y, w) reduced in a fixed order
// (warp shuffles, then per-CTA partials combined by the last CTA to arrive).
__global__ void __launch_bounds__(kNoAllocThreads)
k_bsr_spmv_dot_noalloc(int nb, const int *__restrict__ rowptr, const int *__restrict__ colind,
                       const double *__restrict__ vals, const double *__restrict__ x,
                       double *__restrict__ y, const double *__restrict__ w, double *dot,
                       NoAllocScratch *scr) {
  __shared__ double red[kNoAllocThreads / 32];
  __shared__ bool last;
  const int i = blockIdx.x * kNoAllocThreads + threadIdx.x;
  double d = 0.0;
  if (i < nb) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const double *b = vals + (size_t)k * 9;
      const int j = colind[k];
      const double x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
      a0 = fma(b[0], x0, a0); a0 = fma(b[1], x1, a0); a0 = fma(b[2], x2, a0);
      a1 = fma(b[3], x0, a1); a1 = fma(b[4], x1, a1); a1 = fma(b[5], x2, a1);
      a2 = fma(b[6], x0, a2); a2 = fma(b[7], x1, a2); a2 = fma(b[8], x2, a2);
    }
    y[3 * i] = a0;
    y[3 * i + 1] = a1;
    y[3 * i + 2] = a2;
    d = a0 * w[3 * i] + a1 * w[3 * i + 1] + a2 * w[3 * i + 2];
  }
  for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kNoAllocThreads / 32; ++k) s += red[k];
    scr->partial[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(&scr->arrived, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double s = 0.0;
    for (unsigned int b = 0; b < gridDim.x; ++b) s += __ldcg(&scr->partial[b]);
    *dot = s;
    scr->arrived = 0u;   // leave the counter at zero for the next call
  }
}

// Device address of the scratch array for the current device (looked up on
// the first call per device, with that device current).
cudaError_t scratch_for_current_device(NoAllocScratch **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_lookup_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<NoAllocScratch *>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int gbilu_bsr_spmv_dot_noalloc(int nb, const int *d_rowptr, const int *d_colind,
                                          const double *d_vals, const double *d_x, double *d_y,
                                          const double *d_w, double *d_dot, void *stream) {
  if (nb <= 0 || !d_rowptr || !d_colind || !d_vals || !d_x || !d_y || !d_w || !d_dot) {
    fprintf(stderr, "ERROR: gbilu_bsr_spmv_dot_noalloc: null pointer or nb <= 0\n");
    return GBILU_BAD_INPUT;
  }
  const long long ctas = (nb + (long long)kNoAllocThreads - 1) / kNoAllocThreads;
  if (ctas > kNoAllocMaxCtas) {
    fprintf(stderr,
            "ERROR: gbilu_bsr_spmv_dot_noalloc: nb = %d exceeds the maximum of %d block rows "
            "of the fixed scratch array\n",
            nb, kNoAllocMaxCtas * kNoAllocThreads);
    return GBILU_BAD_INPUT;
  }
  NoAllocScratch *scr = nullptr;
  cudaError_t e = scratch_for_current_device(&scr);
  if (e != cudaSuccess) {
    fprintf(stderr, "ERROR: gbilu_bsr_spmv_dot_noalloc: cudaGetSymbolAddress: %s\n",
            cudaGetErrorString(e));
    return GBILU_CUDA_ERROR;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the arrival counter must start at zero even if an earlier call failed
  e = cudaMemsetAsync(&scr->arrived, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess) {
    k_bsr_spmv_dot_noalloc<<<(unsigned int)ctas, kNoAllocThreads, 0, s>>>(
        nb, d_rowptr, d_colind, d_vals, d_x, d_y, d_w, d_dot, scr);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "ERROR: gbilu_bsr_spmv_dot_noalloc: %s\n", cudaGetErrorString(e));
    return GBILU_CUDA_ERROR;
  }
  return GBILU_OK;
}
