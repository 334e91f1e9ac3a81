// Device helpers shared by the belief-propagation kernels.
#pragma once

#include <cuda_runtime.h>

namespace sicc {

// check-node magnitude: alpha*min (beta == 0) or max(alpha*min - beta, 0), one
// rounding per operation
__device__ __forceinline__ float nms_mag(float alpha, float beta, float mn)
{
    const float a = __fmul_rn(alpha, mn);
    if (beta == 0.0f) return a;
    const float d = __fsub_rn(a, beta);
    return d > 0.0f ? d : 0.0f;
}

// previous message of edge j of a row from its compressed state
// (alpha*min1, alpha*min2, argmin in bits 27..31, message signs in bits 0..26)
__device__ __forceinline__ float rebuild(float m1, float m2, unsigned meta, int j)
{
    const float mag = (j == static_cast<int>(meta >> 27)) ? m2 : m1;
    return ((meta >> j) & 1u) ? -mag : mag;
}

}  // namespace sicc
