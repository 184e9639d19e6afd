// probe.cu -- measurement probes (libhbx_probe.so; not part of the C ABI in
// include/hbx.h and not loaded by the engine).
//
// hbx_probe_scan_rate measures the integer peak that the pair-evaluation
// roofline is quoted against: the rate at which one GB300 runs the
// bit-parallel Jaro scan step itself (bitscan.cuh: the same instructions the
// evaluation kernel runs per character -- symbol extraction, Peq row load,
// AND/ANDNOT, carry-chain negation, OR, funnel-shift window move, the grow
// compare), with every Peq row in shared memory and many independent chains
// per thread, so nothing but the SM's issue and integer pipes limits it.
// The rate is counted in the unit of the roofline: 6 operations per 64-bit
// word (3 per 32-bit word) per character.
#include <cuda_runtime.h>

#include <cstdint>

#include "bitscan.cuh"
#include "kernels.cuh"

namespace hbx {
namespace probe {

constexpr int kThreads = 256;
constexpr int kSymbols = 128;  // Peq rows of the table

__device__ __forceinline__ uint32_t mix(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// kChains independent scans per thread, each over W-word masks.
template <int W, int kChains>
__global__ void __launch_bounds__(kThreads) k_scan_rate(uint32_t iters, uint32_t seed,
                                                         uint32_t* sink) {
  constexpr int S = dev::row_words(W);
  __shared__ __align__(16) uint32_t tab[kSymbols * S];
  for (int i = threadIdx.x; i < kSymbols * S; i += blockDim.x) tab[i] = mix((uint32_t)i ^ seed);
  __syncthreads();
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t win[kChains][W], mt[kChains][W];
  uint4 sy[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) {
#pragma unroll
    for (int k = 0; k < W; k++) {
      win[c][k] = mix(tid * 131u + (uint32_t)(c * 17 + k));
      mt[c][k] = 0u;
    }
    sy[c] = make_uint4(mix(tid + 1u + c), mix(tid + 7u + c), mix(tid + 13u + c), mix(tid + 29u + c));
  }
  // the window grows while i < h, as in a scan (h from the seed: a runtime value)
  const uint32_t h = seed & 31u;
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) {
      const uint32_t wds[4] = {sy[c].x, sy[c].y, sy[c].z, sy[c].w};
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          const uint32_t sym = (wds[q] >> (8 * b)) & (uint32_t)(kSymbols - 1);
          uint32_t pe[S];
#pragma unroll
          for (int k = 0; k < S; k++) pe[k] = tab[sym * S + k];
          dev::bp_update<W, S>(pe, win[c], mt[c], (it * 16u + 4u * q + (uint32_t)b) < h ? 1u : 0u);
        }
      // the next 16 characters depend on this chain's state (no hoisting)
      sy[c] = make_uint4(sy[c].y, sy[c].z, sy[c].w, sy[c].x ^ mt[c][0]);
    }
  }
  uint32_t acc = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++)
#pragma unroll
    for (int k = 0; k < W; k++) acc += __popc(mt[c][k]) + win[c][k];
  sink[tid] = acc;
}

}  // namespace probe
}  // namespace hbx

extern "C" {

// Runs the scan-rate probe for W 32-bit words per mask (1, 2, 4 or 8) on
// `device`, grid = SMs x blocks_per_sm blocks of 256 threads, each thread
// running `chains` (4 or 8) independent scans of iters x 16 characters;
// *ops_per_s = operations of the roofline's unit per second (CUDA events
// around the launch, after one untimed launch), *ms = the launch's time.
// Returns 0, or the CUDA error.
int hbx_probe_scan_rate(int device, int words, int chains, int blocks_per_sm, uint32_t iters,
                        double* ops_per_s, double* ms) {
  using namespace hbx::probe;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return (int)e;
  int n_sm = 0;
  e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return (int)e;
  if (blocks_per_sm < 1 || blocks_per_sm > 8 || iters < 1) return (int)cudaErrorInvalidValue;
  void (*kern)(uint32_t, uint32_t, uint32_t*) = nullptr;
  if (chains != 4 && chains != 8) return (int)cudaErrorInvalidValue;
  switch (words * 16 + chains) {
    case 1 * 16 + 4: kern = k_scan_rate<1, 4>; break;
    case 2 * 16 + 4: kern = k_scan_rate<2, 4>; break;
    case 4 * 16 + 4: kern = k_scan_rate<4, 4>; break;
    case 8 * 16 + 4: kern = k_scan_rate<8, 4>; break;
    case 1 * 16 + 8: kern = k_scan_rate<1, 8>; break;
    case 2 * 16 + 8: kern = k_scan_rate<2, 8>; break;
    case 4 * 16 + 8: kern = k_scan_rate<4, 8>; break;
    case 8 * 16 + 8: kern = k_scan_rate<8, 8>; break;
    default: return (int)cudaErrorInvalidValue;
  }
  const int grid = n_sm * blocks_per_sm;
  const size_t n_threads = (size_t)grid * kThreads;
  uint32_t* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float t = 0.0f;
  if ((e = cudaMalloc(&sink, n_threads * sizeof(uint32_t))) != cudaSuccess) return (int)e;
  if ((e = cudaEventCreate(&e0)) == cudaSuccess && (e = cudaEventCreate(&e1)) == cudaSuccess) {
    kern<<<grid, kThreads>>>(iters, 0x2545F491u, sink);  // warm-up
    cudaEventRecord(e0);
    kern<<<grid, kThreads>>>(iters, 0x2545F491u ^ iters, sink);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return (int)e;
  const double chars = (double)n_threads * chains * (double)iters * 16.0;
  if (ms) *ms = t;
  if (ops_per_s) *ops_per_s = chars * 3.0 * words / (t / 1000.0);
  return 0;
}

}  // extern "C"
