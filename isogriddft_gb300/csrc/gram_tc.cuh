// Tensor-core (tcgen05) tall-skinny Gram, K6 on the tensor pipe (gram_tc.cu).
#pragma once

#include "common.cuh"

namespace igd {

// Launches the 3xTF32 tcgen05 Gram over FP32 blocks and writes one FP64 a x b
// partial per CTA into part (at most max_blocks CTAs).  Returns the number of
// CTAs launched (> 0), -1 when the shape/alignment is outside this path, or an
// IGD_ERR_* status.  err: the device error word for bounded-wait timeouts.
int gram_tc_launch(long long n, int a, int b, const float* A, long long sa, const float* B, long long sb,
                   const double* w, double* part, int max_blocks, unsigned* err, cudaStream_t st);

}  // namespace igd
