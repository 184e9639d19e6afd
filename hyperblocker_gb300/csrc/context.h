// context.h -- the hbx_ctx of the C ABI (device, stream, memory pool).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/hbx.h"

struct hbx_ctx {
  int device = 0;
  int n_sm = 0;
  size_t smem_optin = 0;
  size_t smem_per_sm = 0;  // shared memory of one SM (all resident blocks)
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;  // device memory of this context's sessions and servers
  hbx_opts opts{};
  std::string err;
  std::string device_name;  // keys the autotuner's cache
  void* h_ctr = nullptr;    // page-locked counters of the context's session runs
  // page-locked staging of one-shot results: two chunks of kOutChunkBytes,
  // each with the event of its device-to-host copy (allocated on first use)
  void* h_out = nullptr;
  cudaEvent_t h_out_ev[2] = {nullptr, nullptr};
};
