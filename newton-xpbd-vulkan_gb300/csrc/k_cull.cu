// Reach grids: a conservative cell mask per mesh of the points from which the BVH
// traversal of generate_mesh_contacts.comp:201-331 can reach a leaf. Before its
// first triangle test the traversal prunes every node whose squared box distance
// exceeds the fixed bound (max_dist + eps)^2, and a node's box contains its
// descendants' boxes, so a point farther than that bound from every leaf box pops
// no leaf. The mask marks the cells of each leaf box (one cell of slack for
// rounding) and dilates them by the reach in cells along x, y and z, which covers
// the box inflated by the reach in every direction.
#include <algorithm>

#include "kernels.h"

namespace xpbd {

namespace {

constexpr int kCullThreads = 256;

// index of the mesh whose range [off[m], off[m+1]) holds v (off has nm + 1 entries)
__device__ __forceinline__ int owner(const uint32_t* __restrict__ off, int nm, uint64_t v) {
    int lo = 0, hi = nm - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((uint64_t)__ldg(&off[mid]) <= v)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int cell_of(float v, float o, float inv, int n) {
    const float f = (v - o) * inv;
    if (!(f >= 0.0f)) return 0;
    if (!(f < (float)n)) return n - 1;
    return min((int)f, n - 1);
}

// sets cells [x0, x1] of one row of 32-cell words
__device__ __forceinline__ void set_row(uint32_t* row, int x0, int x1) {
    for (int wx = x0 >> 5; wx <= (x1 >> 5); wx++) {
        const int b0 = max(x0 - wx * 32, 0), b1 = min(x1 - wx * 32, 31);
        const uint32_t hi = b1 == 31 ? 0xffffffffu : ((1u << (b1 + 1)) - 1u);
        const uint32_t m = hi & ~((1u << b0) - 1u);
        atomicOr(row + wx, m);
    }
}

__global__ void k_cull_mark(int nm, const uint32_t* __restrict__ node_off, int64_t total_nodes,
                            const uint8_t* __restrict__ reachable, const float4* __restrict__ nl,
                            const float4* __restrict__ nu, const float4* __restrict__ org,
                            const int4* __restrict__ dim, const uint32_t* __restrict__ off, uint32_t* bits) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total_nodes || !reachable[g]) return;
    const float4 l = nl[g], h = nu[g];
    if (((__float_as_uint(l.w) >> 30) & 3u) == 0u) return;  // inner node
    const int m = owner(node_off, nm, (uint64_t)g);
    const int4 d = dim[m];
    if (d.x == 0) return;
    const float4 o = org[m];
    const int x0 = max(cell_of(l.x, o.x, o.w, d.x) - 1, 0), x1 = min(cell_of(h.x, o.x, o.w, d.x) + 1, d.x - 1);
    const int y0 = max(cell_of(l.y, o.y, o.w, d.y) - 1, 0), y1 = min(cell_of(h.y, o.y, o.w, d.y) + 1, d.y - 1);
    const int z0 = max(cell_of(l.z, o.z, o.w, d.z) - 1, 0), z1 = min(cell_of(h.z, o.z, o.w, d.z) + 1, d.z - 1);
    const int nwx = (d.x + 31) >> 5;
    uint32_t* base = bits + off[m];
    for (int z = z0; z <= z1; z++)
        for (int y = y0; y <= y1; y++) set_row(base + ((size_t)z * d.y + y) * nwx, x0, x1);
}

// out = in dilated by k cells along x (k < 32)
__global__ void k_cull_dilate_x(int nm, int64_t total_words, const int4* __restrict__ dim,
                                const uint32_t* __restrict__ off, const uint32_t* __restrict__ in, uint32_t* out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_words) return;
    const int m = owner(off, nm, (uint64_t)t);
    const int4 d = dim[m];
    const int64_t local = t - off[m];
    const int nwx = (d.x + 31) >> 5;
    if (d.x == 0 || local >= (int64_t)nwx * d.y * d.z) return;
    const int wx = (int)(local % nwx);
    const uint32_t cur = in[t];
    const uint32_t prev = wx > 0 ? in[t - 1] : 0u, next = wx + 1 < nwx ? in[t + 1] : 0u;
    uint32_t r = cur;
    for (int s = 1; s <= d.w; s++) {
        r |= (cur << s) | (prev >> (32 - s));  // cell x - s set
        r |= (cur >> s) | (next << (32 - s));  // cell x + s set
    }
    if (wx == nwx - 1 && (d.x & 31)) r &= (1u << (d.x & 31)) - 1u;  // no cells past nx
    out[t] = r;
}

// out = in dilated by k rows along y (axis 1) or layers along z (axis 2)
__global__ void k_cull_dilate_yz(int nm, int64_t total_words, const int4* __restrict__ dim,
                                 const uint32_t* __restrict__ off, int axis, const uint32_t* __restrict__ in,
                                 uint32_t* out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_words) return;
    const int m = owner(off, nm, (uint64_t)t);
    const int4 d = dim[m];
    const int64_t local = t - off[m];
    const int nwx = (d.x + 31) >> 5;
    if (d.x == 0 || local >= (int64_t)nwx * d.y * d.z) return;
    const int64_t row = local / nwx;
    const int y = (int)(row % d.y), z = (int)(row / d.y);
    const int c = axis == 1 ? y : z, n = axis == 1 ? d.y : d.z;
    const int64_t stride = axis == 1 ? (int64_t)nwx : (int64_t)nwx * d.y;
    const int lo = max(c - d.w, 0), hi = min(c + d.w, n - 1);
    uint32_t r = 0;
    for (int q = lo; q <= hi; q++) r |= in[t + (int64_t)(q - c) * stride];
    out[t] = r;
}

}  // namespace

void launch_cull_build(cudaStream_t s, int nm, const uint32_t* node_off, int64_t total_nodes,
                       const uint8_t* reachable, const float4* nl, const float4* nu, const float4* org,
                       const int4* dim, const uint32_t* off, int64_t total_words, uint32_t* bits, uint32_t* tmp) {
    if (nm <= 0 || total_words <= 0) return;
    const int wb = (int)((total_words + kCullThreads - 1) / kCullThreads);
    cudaMemsetAsync(tmp, 0, (size_t)total_words * sizeof(uint32_t), s);
    if (total_nodes > 0)
        k_cull_mark<<<(int)((total_nodes + kCullThreads - 1) / kCullThreads), kCullThreads, 0, s>>>(
            nm, node_off, total_nodes, reachable, nl, nu, org, dim, off, tmp);
    k_cull_dilate_x<<<wb, kCullThreads, 0, s>>>(nm, total_words, dim, off, tmp, bits);
    k_cull_dilate_yz<<<wb, kCullThreads, 0, s>>>(nm, total_words, dim, off, 1, bits, tmp);
    k_cull_dilate_yz<<<wb, kCullThreads, 0, s>>>(nm, total_words, dim, off, 2, tmp, bits);
}

}  // namespace xpbd
