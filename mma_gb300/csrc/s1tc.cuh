// s1tc.cuh -- launcher of the tensor-core stage 1 of the fast far field (hankel_s1tc.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/mma_hankel.h"

namespace mma {
namespace s1tc {
int stage1_tc_launch(const mma_hankel_problem& P, const void* src, const double2* pre, const float* ptab,
                     const float2* ktab, const float4* rtab, float2 u_ref, float2* Bp, int n_terms, int* status,
                     cudaStream_t st);
}  // namespace s1tc
}  // namespace mma
