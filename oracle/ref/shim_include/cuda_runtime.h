// TEST INFRASTRUCTURE ONLY: stands in for <cuda_runtime.h> when the
// reference's kernel headers are compiled by g++ for the CPU oracle.
#pragma once
#include "../ref_cuda_shim.h"
