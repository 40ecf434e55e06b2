// Contact ranking / compaction, reference-layout debug tables, state packing.
#include "contact.cuh"
#include "kernels.h"
#include "particle.cuh"
#include "xmath.cuh"

namespace xpbd {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

size_t contact_scan_words(int64_t n) {
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    return (size_t)(tiles > 0 ? tiles : 1) * 2 + 2;
}

// (plane contacts, generic slots) of a particle; with ds.cslot set instead
// (slots whose shape belongs to a dynamic body, 0)
__device__ __forceinline__ uint2 particle_counts(const uint32_t* __restrict__ cinfo, int64_t i, const DynSlots& ds) {
    const uint32_t info = cinfo[i];
    if (!ds.cslot) return make_uint2(info & kPlaneBit, (uint32_t)info_slots(info));
    return make_uint2((uint32_t)info_dyn(info), 0u);
}

// phase 1: per-tile sums
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(int64_t n, const uint32_t* __restrict__ cinfo,
                                                             DynSlots ds, uint32_t* __restrict__ tile_sums,
                                                             const uint32_t* skip, int64_t cap) {
    if (skip && (int64_t)*skip <= cap) return;
    __shared__ uint32_t s_a[kScanThreads / 32], s_b[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    uint32_t a = 0, b = 0;
    for (int j = 0; j < kScanItems; j++) {
        const int64_t i = base + j * kScanThreads + threadIdx.x;
        if (i < n) {
            const uint2 c = particle_counts(cinfo, i, ds);
            a += c.x;
            b += c.y;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        s_a[warp] = a;
        s_b[warp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t ta = 0, tb = 0;
        for (int w = 0; w < kScanThreads / 32; w++) {
            ta += s_a[w];
            tb += s_b[w];
        }
        tile_sums[blockIdx.x * 2] = ta;
        tile_sums[blockIdx.x * 2 + 1] = tb;
    }
}

// phase 2: one block scans the tile sums in place (exclusive) and writes the totals
__global__ void __launch_bounds__(1024) k_scan_tiles(int tiles, uint32_t* __restrict__ tile_sums,
                                                    uint32_t* __restrict__ totals, const uint32_t* skip, int64_t cap) {
    if (skip && (int64_t)*skip <= cap) return;
    __shared__ uint32_t s_a[32], s_b[32];
    __shared__ uint32_t carry_a, carry_b;
    if (threadIdx.x == 0) carry_a = carry_b = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < tiles; base += blockDim.x) {
        const int t = base + threadIdx.x;
        uint32_t a = t < tiles ? tile_sums[t * 2] : 0u, b = t < tiles ? tile_sums[t * 2 + 1] : 0u;
        uint32_t ia = a, ib = b;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t ya = __shfl_up_sync(0xffffffffu, ia, o), yb = __shfl_up_sync(0xffffffffu, ib, o);
            if (lane >= o) {
                ia += ya;
                ib += yb;
            }
        }
        if (lane == 31) {
            s_a[warp] = ia;
            s_b[warp] = ib;
        }
        __syncthreads();
        uint32_t oa = carry_a, ob = carry_b, ta = 0, tb = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            if (w < warp) {
                oa += s_a[w];
                ob += s_b[w];
            }
            ta += s_a[w];
            tb += s_b[w];
        }
        if (t < tiles) {
            tile_sums[t * 2] = oa + ia - a;
            tile_sums[t * 2 + 1] = ob + ib - b;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            carry_a += ta;
            carry_b += tb;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        totals[0] = carry_a;
        totals[1] = carry_b;
    }
}

// phase 3: per-particle exclusive ranks
__global__ void __launch_bounds__(kScanThreads) k_scan_down(int64_t n, const uint32_t* __restrict__ cinfo,
                                                           DynSlots ds, const uint32_t* __restrict__ tile_sums,
                                                           uint2* __restrict__ rank, const uint32_t* skip, int64_t cap) {
    if (skip && (int64_t)*skip <= cap) return;
    __shared__ uint32_t s_a[kScanThreads / 32], s_b[kScanThreads / 32];
    // thread t owns kScanItems consecutive particles of the tile
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    uint32_t a = 0, b = 0;
    uint2 c[kScanItems];
    for (int j = 0; j < kScanItems; j++) {
        const int64_t i = base + j;
        c[j] = i < n ? particle_counts(cinfo, i, ds) : make_uint2(0, 0);
        a += c[j].x;
        b += c[j].y;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t ia = a, ib = b;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t ya = __shfl_up_sync(0xffffffffu, ia, o), yb = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) {
            ia += ya;
            ib += yb;
        }
    }
    if (lane == 31) {
        s_a[warp] = ia;
        s_b[warp] = ib;
    }
    __syncthreads();
    uint32_t oa = tile_sums[blockIdx.x * 2], ob = tile_sums[blockIdx.x * 2 + 1];
    for (int w = 0; w < warp; w++) {
        oa += s_a[w];
        ob += s_b[w];
    }
    oa += ia - a;
    ob += ib - b;
    for (int j = 0; j < kScanItems; j++) {
        const int64_t i = base + j;
        if (i < n) rank[i] = make_uint2(oa, ob);
        oa += c[j].x;
        ob += c[j].y;
    }
}

void launch_contact_scan(cudaStream_t s, int64_t n, const uint32_t* cinfo, uint2* rank, uint32_t* totals,
                         uint32_t* workspace, const uint32_t* skip_count, int64_t cap) {
    if (n <= 0) {
        cudaMemsetAsync(totals, 0, 2 * sizeof(uint32_t), s);
        return;
    }
    const int tiles = (int)((n + kScanTile - 1) / kScanTile);
    const DynSlots none{nullptr, 0, nullptr, nullptr};
    k_scan_reduce<<<tiles, kScanThreads, 0, s>>>(n, cinfo, none, workspace, skip_count, cap);
    k_scan_tiles<<<1, 1024, 0, s>>>(tiles, workspace, totals, skip_count, cap);
    k_scan_down<<<tiles, kScanThreads, 0, s>>>(n, cinfo, none, workspace, rank, skip_count, cap);
}

void launch_dyn_scan(cudaStream_t s, int64_t n, const uint32_t* cinfo, DynSlots ds, uint2* rank, uint32_t* totals,
                     uint32_t* workspace) {
    if (n <= 0) {
        cudaMemsetAsync(totals, 0, 2 * sizeof(uint32_t), s);
        return;
    }
    const int tiles = (int)((n + kScanTile - 1) / kScanTile);
    k_scan_reduce<<<tiles, kScanThreads, 0, s>>>(n, cinfo, ds, workspace, nullptr, 0);
    k_scan_tiles<<<1, 1024, 0, s>>>(tiles, workspace, totals, nullptr, 0);
    k_scan_down<<<tiles, kScanThreads, 0, s>>>(n, cinfo, ds, workspace, rank, nullptr, 0);
}

__global__ void k_contact_compact(int64_t n, const uint32_t* __restrict__ cinfo, const float4* __restrict__ cslot,
                                  int slot_cap, const uint2* __restrict__ rank, const uint32_t* __restrict__ totals,
                                  int64_t contact_max, const float4* __restrict__ x_prev, float altitude,
                                  int32_t* part, int32_t* shape, float* bpos, float* bvel, float* nrm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t info = cinfo[i];
    if (!info) return;
    const uint2 rk = rank[i];
    const int ncon = (int)(info & kPlaneBit) + info_slots(info);
    const v3 xp = xyz(x_prev[i]);
    for (int c = 0; c < ncon; c++) {
        int64_t pos;
        if ((info & kPlaneBit) && c == 0)
            pos = rk.x;
        else
            pos = (int64_t)totals[0] + rk.y + (c - (int)(info & kPlaneBit));
        if (pos >= contact_max) continue;
        const Contact ct = load_contact(info, c, cslot + (size_t)i * slot_cap * 3, xp, altitude);
        part[pos] = (int32_t)i;
        shape[pos] = ct.shape;
        bpos[pos * 3] = ct.bpos.x;
        bpos[pos * 3 + 1] = ct.bpos.y;
        bpos[pos * 3 + 2] = ct.bpos.z;
        bvel[pos * 3] = ct.bvel.x;
        bvel[pos * 3 + 1] = ct.bvel.y;
        bvel[pos * 3 + 2] = ct.bvel.z;
        nrm[pos * 3] = ct.nrm.x;
        nrm[pos * 3 + 1] = ct.nrm.y;
        nrm[pos * 3 + 2] = ct.nrm.z;
    }
}

void launch_contact_compact(cudaStream_t s, int64_t n, const uint32_t* cinfo, const float4* cslot, int slot_cap,
                            const uint2* rank, const uint32_t* totals, int64_t contact_max, const float4* x_prev,
                            float altitude, int32_t* part, int32_t* shape, float* bpos, float* bvel, float* nrm) {
    if (n <= 0) return;
    k_contact_compact<<<(int)((n + 255) / 256), 256, 0, s>>>(n, cinfo, cslot, slot_cap, rank, totals, contact_max,
                                                             x_prev, altitude, part, shape, bpos, bvel, nrm);
}

__global__ void k_cell_tables(const int4* __restrict__ table, const uint32_t* __restrict__ stamp_p,
                              int32_t* __restrict__ starts, int32_t* __restrict__ ends) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kNumCells) return;
    const uint32_t stamp = *stamp_p;
    const int4 e = table[c];
    const bool live = (uint32_t)e.z == stamp;
    starts[c] = live ? e.x : 0;
    ends[c] = live ? e.y : 0;
}

void launch_cell_tables(cudaStream_t s, const int4* table, const uint32_t* stamp, int32_t* starts, int32_t* ends) {
    k_cell_tables<<<(kNumCells + 255) / 256, 256, 0, s>>>(table, stamp, starts, ends);
}

__global__ void k_unpack_xyz(int64_t n, const float4* __restrict__ a, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = a[i];
    out[i * 3] = v.x;
    out[i * 3 + 1] = v.y;
    out[i * 3 + 2] = v.z;
}
__global__ void k_pack_xyz(int64_t n, const float* __restrict__ in, float4* __restrict__ a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = make_float4(in[i * 3], in[i * 3 + 1], in[i * 3 + 2], 0.0f);
}
void launch_unpack_xyz(cudaStream_t s, int64_t n, const float4* a, float* out) {
    if (n > 0) k_unpack_xyz<<<(int)((n + 255) / 256), 256, 0, s>>>(n, a, out);
}
void launch_pack_xyz(cudaStream_t s, int64_t n, const float* in, float4* a) {
    if (n > 0) k_pack_xyz<<<(int)((n + 255) / 256), 256, 0, s>>>(n, in, a);
}

}  // namespace xpbd
