// int_peak.cuh -- measures the GPU's 32-bit integer add/max issue rate, the roofline
// denominator of the DP kernels (their work is integer adds and maxes, not HBM traffic).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace gba {

// Each thread updates 16 independent accumulators with one IADD and one IMNMX per step.
__global__ void __launch_bounds__(256) k_int_peak(int32_t *out, int iters, int seed)
{
    int32_t a[16], b[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        a[k] = seed + threadIdx.x + k;
        b[k] = seed - k;
    }
    const int32_t inc = seed & 7;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a[k] = max(a[k] + inc, b[k]);
            b[k] = max(b[k] - inc, a[k] - 3);
        }
    }
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) s ^= a[k] ^ b[k];
    if (s == 0x7fffffff) out[0] = s;   // keeps the loop live
}

}  // namespace gba
