// Device arithmetic with the evaluation order of the reference's GLSL shaders.
//
// The whole library is compiled with --fmad=false: a multiply followed by an
// add is never fused unless the source calls __fmaf_rn(), which appears
// exactly where the shaders write fma(). Division and square root use the
// IEEE round-to-nearest intrinsics. With these rules every kernel produces the
// same bits as the CPU oracle built with -ffp-contract=off.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.h"

namespace xpbd {

struct v3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ v3 mk3(float x, float y, float z) {
    v3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__device__ __forceinline__ v3 xyz(float4 a) { return mk3(a.x, a.y, a.z); }
__device__ __forceinline__ v3 vadd(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 vmuls(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ v3 vneg(v3 a) { return mk3(-a.x, -a.y, -a.z); }
// GLSL max(x,y) = (x < y) ? y : x ; min(x,y) = (y < x) ? y : x
__device__ __forceinline__ float gmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float gmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
// dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z
__device__ __forceinline__ float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ v3 vcross(v3 a, v3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float vlength(v3 a) { return __fsqrt_rn(vdot(a, a)); }
__device__ __forceinline__ v3 vnormalize(v3 a) {
    float l = vlength(a);
    return mk3(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}
__device__ __forceinline__ v3 vfma_vs(v3 a, float s, v3 c) {  // fma(a, vec3(s), c)
    return mk3(__fmaf_rn(a.x, s, c.x), __fmaf_rn(a.y, s, c.y), __fmaf_rn(a.z, s, c.z));
}

// exact_sqrt / exact_length / exact_dot / exact_div of
// solve_particle_particle_contacts.comp:81-105 (identical copies live in the
// shape-contact and mesh-contact shaders).
// At a == 0 the shader's refinement evaluates fma(0, 0.5 / 0, 0): NaN in IEEE arithmetic
// and undefined under Vulkan's division rules (a particle lying exactly on a mesh surface
// then gets a NaN contact point). The refinement is meant to equal sqrt(a), so 0 is kept.
__device__ __forceinline__ float exact_sqrt(float a) {
    if (a == 0.0f) return a;
    float d = __fsqrt_rn(a);
    float r = __fmaf_rn(-d, d, a);
    return __fmaf_rn(r, __fdiv_rn(0.5f, d), d);
}
__device__ __forceinline__ float exact_length(v3 a) {
    float yy = a.y * a.y;
    float xx_yy = __fmaf_rn(a.x, a.x, yy);
    float sq = __fmaf_rn(a.z, a.z, xx_yy);
    return exact_sqrt(sq);
}
__device__ __forceinline__ float exact_dot(v3 a, v3 b) {
    float y = a.y * b.y;
    float x_y = __fmaf_rn(a.x, b.x, y);
    return __fmaf_rn(a.z, b.z, x_y);
}
__device__ __forceinline__ v3 exact_div(v3 v, float d) {
    float inv_d = __frcp_rn(d);
    v3 q = vmuls(v, inv_d);
    v3 rem = mk3(__fmaf_rn(-d, q.x, v.x), __fmaf_rn(-d, q.y, v.y), __fmaf_rn(-d, q.z, v.z));
    return mk3(__fmaf_rn(rem.x, inv_d, q.x), __fmaf_rn(rem.y, inv_d, q.y), __fmaf_rn(rem.z, inv_d, q.z));
}
// exact_sqrt(a) and its IEEE reciprocal RN(1/exact_sqrt(a)) with one reciprocal where the
// shader's arithmetic has a division and a reciprocal: the refinement's RN(0.5/d0) is
// 0.5 * RN(1/d0) exactly (a power-of-two scaling commutes with rounding, and 1/d0 of a
// float's square root is always a normal number), and the refined root equals d0 in all but
// rare cases, where the reciprocal is taken again. a == 0 gives (0, +inf), as
// exact_sqrt(0) = 0 and RN(1/0).
__device__ __forceinline__ float exact_sqrt_rcp(float a, float& inv) {
    if (a == 0.0f) {
        inv = __frcp_rn(a);
        return a;
    }
    const float d0 = __fsqrt_rn(a);
    const float r0 = __frcp_rn(d0);
    const float r = __fmaf_rn(-d0, d0, a);
    const float d = __fmaf_rn(r, 0.5f * r0, d0);
    inv = d == d0 ? r0 : __frcp_rn(d);
    return d;
}
__device__ __forceinline__ float exact_length_rcp(v3 a, float& inv) {
    float yy = a.y * a.y;
    float xx_yy = __fmaf_rn(a.x, a.x, yy);
    float sq = __fmaf_rn(a.z, a.z, xx_yy);
    return exact_sqrt_rcp(sq, inv);
}
// exact_div with the divisor's IEEE reciprocal inv_d = RN(1/d) supplied
__device__ __forceinline__ v3 exact_div_rcp(v3 v, float d, float inv_d) {
    v3 q = vmuls(v, inv_d);
    v3 rem = mk3(__fmaf_rn(-d, q.x, v.x), __fmaf_rn(-d, q.y, v.y), __fmaf_rn(-d, q.z, v.z));
    return mk3(__fmaf_rn(rem.x, inv_d, q.x), __fmaf_rn(rem.y, inv_d, q.y), __fmaf_rn(rem.z, inv_d, q.z));
}
__device__ __forceinline__ float exact_div1(float v, float d) {  // generate_mesh_contacts.comp:57-62
    float inv_d = __frcp_rn(d);
    float q = v * inv_d;
    float rem = __fmaf_rn(-d, q, v);
    return __fmaf_rn(rem, inv_d, q);
}
// exact_div of apply_particle_deltas.comp:30-36
__device__ __forceinline__ v3 exact_div_apply(v3 a, float b) {
    float y = __frcp_rn(b);
    y = __fmaf_rn(-b, y, 1.0f) * y + y;
    v3 q = vmuls(a, y);
    v3 r = mk3(__fmaf_rn(-q.x, b, a.x), __fmaf_rn(-q.y, b, a.y), __fmaf_rn(-q.z, b, a.z));
    return mk3(__fmaf_rn(r.x, y, q.x), __fmaf_rn(r.y, y, q.y), __fmaf_rn(r.z, y, q.z));
}
__device__ __forceinline__ float diff_product(float a, float b, float c, float d) {
    float cd = c * d;
    float diff = __fmaf_rn(a, b, -cd);
    float err = __fmaf_rn(-c, d, cd);
    return diff + err;
}

// acos(x) for x in [-1,1]: a Taylor series of asin (coefficients
// (2n)!/(4^n (n!)^2 (2n+1)), n=1..11, rounded to float) in Horner form in t^2,
// with acos(x) = 2 asin(sqrt((1-x)/2)) for |x| > 1/2. About 1 ulp; the CPU
// oracle evaluates the identical expression. Only the sign of the angle-weighted
// pseudo-normal depends on it (generate_mesh_contacts.comp:278-282, 390).
__device__ __forceinline__ float asin_series(float t) {
    const float c[11] = {0x1.555556p-3f, 0x1.333334p-4f, 0x1.6db6dcp-5f, 0x1.f1c71cp-6f,
                         0x1.6e8ba2p-6f, 0x1.1c4ec4p-6f, 0x1.c9999ap-7f, 0x1.7a8788p-7f,
                         0x1.3fde50p-7f, 0x1.12ef3cp-7f, 0x1.df3bd4p-8f};
    float t2 = t * t;
    float acc = c[10];
#pragma unroll
    for (int k = 9; k >= 0; k--) acc = acc * t2 + c[k];
    acc = acc * t2;
    return t + t * acc;
}
__device__ __forceinline__ float series_acos(float x) {
    const float half_pi = 0x1.921fb6p+0f;
    const float pi = 0x1.921fb6p+1f;
    float ax = fabsf(x);
    if (ax <= 0.5f) return half_pi - asin_series(x);
    float s = __fsqrt_rn((1.0f - ax) * 0.5f);
    float a = 2.0f * asin_series(s);
    return x > 0.0f ? a : pi - a;
}

// float -> int of an integral float; saturates at +-2^30, NaN -> 0 (GLSL leaves
// out-of-range conversions undefined; the oracle uses the same rule).
__device__ __forceinline__ int32_t f2i(float f) {
    if (!(f == f)) return 0;
    if (f >= 1073741824.0f) return 1073741824;
    if (f <= -1073741824.0f) return -1073741824;
    return (int32_t)f;
}
__device__ __forceinline__ int32_t imax0(int32_t a) { return a < 0 ? 0 : a; }

// Hash-grid keys. The reference's key (grid_cell_indices.comp:17-25,
// solve_particle_particle_contacts.comp:67-79) is the cell index on a 128^3 grid that wraps
// every 128 cells per axis, so cells 128 apart share a key ("aliens"): the neighbour loop
// visits their particles and rejects them by distance. With `split` the key also carries
// bit 7 of each axis' unwrapped cell coordinate in bits 21..23 (the grid wraps every 256
// cells). The sort is stable from particle order, so a cell's particles are in particle
// order either way and the particles of one true cell appear in a split key's range in the
// same relative order as in the reference's range; only aliens 128 cells away are gone,
// and those are never accepted. Bits 0..20 are the reference's key.
__device__ __forceinline__ uint32_t grid_key(int32_t gx, int32_t gy, int32_t gz, bool split) {
    // g* = imax0(cell + kGridOrigin) >= 0
    const uint32_t k = (uint32_t)((gz % kGridDim) * (kGridDim * kGridDim) + (gy % kGridDim) * kGridDim +
                                  (gx % kGridDim));
    if (!split) return k;
    return k | ((((uint32_t)gx >> 7) & 1u) << 21) | ((((uint32_t)gy >> 7) & 1u) << 22) |
           ((((uint32_t)gz >> 7) & 1u) << 23);
}
__device__ __forceinline__ uint32_t hash_grid_index(v3 p, float inv, bool split) {
    const int32_t gx = imax0(f2i(floorf(p.x * inv)) + kGridOrigin);
    const int32_t gy = imax0(f2i(floorf(p.y * inv)) + kGridOrigin);
    const int32_t gz = imax0(f2i(floorf(p.z * inv)) + kGridOrigin);
    return grid_key(gx, gy, gz, split);
}
__device__ __forceinline__ int32_t cell_index(int32_t x, int32_t y, int32_t z, bool split) {
    return (int32_t)grid_key(imax0(x + kGridOrigin), imax0(y + kGridOrigin), imax0(z + kGridOrigin), split);
}

struct q4 {
    float x, y, z, w;
};
// quat_rotate / quat_rotate_inv of solve_particle_shape_contacts.comp:50-68
__device__ __forceinline__ v3 quat_rotate(q4 q, v3 x) {
    float c = 2.0f * q.w * q.w - 1.0f;
    float d = 2.0f * ((q.x * x.x + q.y * x.y) + q.z * x.z);
    return mk3((x.x * c + q.x * d) + (q.y * x.z - q.z * x.y) * q.w * 2.0f,
               (x.y * c + q.y * d) + (q.z * x.x - q.x * x.z) * q.w * 2.0f,
               (x.z * c + q.z * d) + (q.x * x.y - q.y * x.x) * q.w * 2.0f);
}
__device__ __forceinline__ v3 quat_rotate_inv(q4 q, v3 x) {
    float c = 2.0f * q.w * q.w - 1.0f;
    float d = 2.0f * ((q.x * x.x + q.y * x.y) + q.z * x.z);
    return mk3((x.x * c + q.x * d) - (q.y * x.z - q.z * x.y) * q.w * 2.0f,
               (x.y * c + q.y * d) - (q.z * x.x - q.x * x.z) * q.w * 2.0f,
               (x.z * c + q.z * d) - (q.x * x.y - q.y * x.x) * q.w * 2.0f);
}

// ---- memory-order helpers for decoupled look-back (PTX ISA: ld.acquire / st.release) ----
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// a relaxed load: no ordering of later accesses, so several can be in flight at once
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace xpbd
