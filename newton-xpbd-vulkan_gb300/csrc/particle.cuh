// Per-particle prediction shared by the key and gather kernels.
#pragma once
#include "kernels.h"
#include "xmath.cuh"

namespace xpbd {

// integrate_particles.comp:30-59 (the external-force buffer is all zero,
// scene.cpp:82-83, so f0 = 0). Inactive particles keep x and v.
__device__ __forceinline__ void predict(float4 xf, float4 vf, float w, int flags, const PredictParams& p, v3& xp,
                                        v3& vp) {
    v3 x0 = xyz(xf), v0 = xyz(vf);
    if ((flags & 1) == 0) {
        xp = x0;
        vp = v0;
        return;
    }
    const v3 f0 = mk3(0.0f, 0.0f, 0.0f);
    const v3 g = mk3(p.gx, p.gy, p.gz);
    float g_scale = w > 0.0f ? 1.0f : 0.0f;
    v3 v1 = vadd(v0, vmuls(vadd(vmuls(f0, w), vmuls(g, g_scale)), p.dt));
    float v1_mag = vlength(v1);
    if (v1_mag > p.v_max) v1 = vmuls(v1, __fdiv_rn(p.v_max, v1_mag));
    xp = vadd(x0, vmuls(v1, p.dt));
    vp = v1;
}

// Block-wide sum of one value per thread (blockDim.x a multiple of 32, <= 1024).
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) s_warp[warp] = v;
    __syncthreads();
    uint32_t t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_warp[w];
    return t;  // valid in thread 0
}

}  // namespace xpbd
