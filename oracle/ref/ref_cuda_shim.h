// ref_cuda_shim.h -- TEST INFRASTRUCTURE ONLY.
//
// Lets g++ compile the reference's own kernel headers (core/gpu/global_func.cuh,
// core/gpu/device_func.cuh) as ordinary host C++ so that blocking_kernel can
// run on CPU threads as a parity oracle.  Each host thread that runs the
// kernel body sets its own emulated blockIdx/threadIdx first.
#pragma once
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <unordered_map>
#include <vector>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline

struct hbref_dim3 {
  unsigned x, y, z;
};
extern thread_local hbref_dim3 blockIdx;
extern thread_local hbref_dim3 threadIdx;
extern hbref_dim3 blockDim;
extern hbref_dim3 gridDim;

inline int atomicAdd(int* p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicAdd(unsigned* p, unsigned v) {
  return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
}
inline int atomicOr(int* p, int v) { return __atomic_fetch_or(p, v, __ATOMIC_RELAXED); }
inline unsigned atomicOr(unsigned* p, unsigned v) {
  return __atomic_fetch_or(p, v, __ATOMIC_RELAXED);
}
inline unsigned long long atomicOr(unsigned long long* p, unsigned long long v) {
  return __atomic_fetch_or(p, v, __ATOMIC_RELAXED);
}

// Host-side declarations the plan generator header names; the oracle never
// calls them.
typedef int cudaError_t;
#define cudaHostAllocDefault 0
#define cudaHostAllocPortable 1
template <class T>
inline cudaError_t cudaHostAlloc(T** p, size_t n, unsigned) {
  *p = (T*)std::calloc(n ? n : 1, 1);
  return 0;
}
