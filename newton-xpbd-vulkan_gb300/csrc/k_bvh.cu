// GPU LBVH build and refit with the reference builder's topology
// (MeshLbvhBuilder::build, src/mesh_lbvh.h:49-223; refit of
// src/mesh_bvh.h:142-181).
//
// Build: triangle bounds and the total box (std::min / std::max semantics, so
// the values equal the host builder's bit for bit), 30-bit Morton codes of the
// centroids (mesh_lbvh.h:85-103), a stable onesweep sort by code, clz64 deltas,
// then the bottom-up construction: one thread per leaf climbs, choosing the
// parent with the builder's rule (larger shared prefix, ties by the parity of
// the two neighbouring primitives); the second child to reach a node writes its
// box and climbs on (the first stops), so the tree is the sequential builder's
// in any arrival order. Leaves are then collapsed where a node covers <= 4
// primitives or sits at depth >= 32 (mark_packed_leaf_nodes), and the packed
// node words are rebased into the solver's global node / primitive arrays.
//
// Refit: the same bottom-up unions over the original binary tree with the new
// vertex positions; a collapsed leaf's box is the union of its range, which is
// its subtree's union, so writing the reachable nodes gives the reference's
// recursive refit.
#include "kernels.h"
#include "xmath.cuh"

namespace xpbd {

namespace {

__device__ __forceinline__ float smin(float a, float b) { return b < a ? b : a; }  // std::min(a, b)
__device__ __forceinline__ float smax(float a, float b) { return a < b ? b : a; }  // std::max(a, b)

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // mesh_lbvh.h:12-19
    v &= 0x3ffu;
    v = (v ^ (v << 16)) & 0xff0000ffu;
    v = (v ^ (v << 8)) & 0x0300f00fu;
    v = (v ^ (v << 4)) & 0x030c30c3u;
    v = (v ^ (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ uint32_t quantize1024(float f) {  // mesh_lbvh.h:21-26
    const int i = __float2int_rz(f * 1024.0f);
    return (uint32_t)max(0, min(1023, i));
}

// bounds of triangle t (vertex 0, then min/max with vertices 1 and 2)
__device__ __forceinline__ void tri_bounds(const float* __restrict__ verts, const uint32_t* __restrict__ tris,
                                           uint32_t t, v3& lo, v3& hi) {
    const uint32_t i0 = tris[t * 3];
    lo = hi = mk3(verts[i0 * 3], verts[i0 * 3 + 1], verts[i0 * 3 + 2]);
    for (int k = 1; k < 3; k++) {
        const uint32_t i = tris[t * 3 + k];
        const v3 p = mk3(verts[i * 3], verts[i * 3 + 1], verts[i * 3 + 2]);
        lo = mk3(smin(lo.x, p.x), smin(lo.y, p.y), smin(lo.z, p.z));
        hi = mk3(smax(hi.x, p.x), smax(hi.y, p.y), smax(hi.z, p.z));
    }
}

constexpr int kBvhThreads = 256;

}  // namespace

// triangle boxes + per-block partial total box
__global__ void __launch_bounds__(kBvhThreads) k_lbvh_bounds(int n, const float* __restrict__ verts,
                                                            const uint32_t* __restrict__ tris, float4* tb,
                                                            float4* partial) {
    __shared__ float s[6][kBvhThreads];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    v3 lo = mk3(1e30f, 1e30f, 1e30f), hi = mk3(-1e30f, -1e30f, -1e30f);
    if (t < n) {
        v3 l, h;
        tri_bounds(verts, tris, (uint32_t)t, l, h);
        tb[t * 2] = make_float4(l.x, l.y, l.z, 0.0f);
        tb[t * 2 + 1] = make_float4(h.x, h.y, h.z, 0.0f);
        lo = l;
        hi = h;
    }
    s[0][threadIdx.x] = lo.x;
    s[1][threadIdx.x] = lo.y;
    s[2][threadIdx.x] = lo.z;
    s[3][threadIdx.x] = hi.x;
    s[4][threadIdx.x] = hi.y;
    s[5][threadIdx.x] = hi.z;
    __syncthreads();
    if (threadIdx.x == 0) {  // in index order: the same min/max chain as the host loop over triangles
        float r[6] = {1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f};
        for (int k = 0; k < kBvhThreads; k++) {
            if (blockIdx.x * blockDim.x + k >= n) break;
            for (int a = 0; a < 3; a++) r[a] = smin(r[a], s[a][k]);
            for (int a = 3; a < 6; a++) r[a] = smax(r[a], s[a][k]);
        }
        partial[blockIdx.x * 2] = make_float4(r[0], r[1], r[2], 0.0f);
        partial[blockIdx.x * 2 + 1] = make_float4(r[3], r[4], r[5], 0.0f);
    }
}

// total box (block partials in order), Morton codes, digit histograms of the 4 sort passes
__global__ void __launch_bounds__(kBvhThreads) k_lbvh_morton(int n, int blocks, const float4* __restrict__ tb,
                                                            const float4* __restrict__ partial,
                                                            uint32_t* __restrict__ keys, uint32_t* hist) {
    __shared__ float s_inv[3], s_lo[3];
    __shared__ uint32_t s_hist[4 * 256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) s_hist[i] = 0;
    if (threadIdx.x == 0) {
        float r[6] = {1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f};
        for (int b = 0; b < blocks; b++) {
            const float4 l = partial[b * 2], h = partial[b * 2 + 1];
            r[0] = smin(r[0], l.x);
            r[1] = smin(r[1], l.y);
            r[2] = smin(r[2], l.z);
            r[3] = smax(r[3], h.x);
            r[4] = smax(r[4], h.y);
            r[5] = smax(r[5], h.z);
        }
        for (int a = 0; a < 3; a++) {
            s_lo[a] = r[a];
            s_inv[a] = __fdiv_rn(1.0f, (r[a + 3] - r[a]) + 0.0001f);  // mesh_lbvh.h:85-88
        }
    }
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const float4 l = tb[t * 2], h = tb[t * 2 + 1];
        const uint32_t qx = quantize1024((0.5f * (l.x + h.x) - s_lo[0]) * s_inv[0]);
        const uint32_t qy = quantize1024((0.5f * (l.y + h.y) - s_lo[1]) * s_inv[1]);
        const uint32_t qz = quantize1024((0.5f * (l.z + h.z) - s_lo[2]) * s_inv[2]);
        const uint32_t key = (spread10(qz) << 2) | (spread10(qy) << 1) | spread10(qx);
        keys[t] = key;
        for (int p = 0; p < 4; p++) atomicAdd(&s_hist[p * 256 + ((key >> (p * 8)) & 255u)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

// leaves (sorted order), ranges and clz64 deltas (mesh_lbvh.h:110-145)
__global__ void k_lbvh_leaves(int n, const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ sprims,
                              const float4* __restrict__ tb, float4* nlo, float4* nhi, int* range_l, int* range_r,
                              int* deltas) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = sprims[i];
    nlo[i] = tb[p * 2];
    nhi[i] = tb[p * 2 + 1];
    range_l[i] = i;
    range_r[i] = i;
    if (i + 1 < n) {
        const uint32_t x = skeys[i] ^ skeys[i + 1];  // 64-bit keys with the 30-bit code in the low word
        deltas[i] = x ? 32 + __clz(x) : 64;
    }
}

// bottom-up construction (mesh_lbvh.h:147-203); counter[] zeroed beforehand
__global__ void k_lbvh_climb(int n, const int* __restrict__ deltas, const uint32_t* __restrict__ sprims,
                             float4* nlo, float4* nhi, int* range_l, int* range_r, int* parent, int* child_l,
                             int* child_r, int* counter, int* root_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int curr = i;
    while (true) {
        const int left = ((volatile int*)range_l)[curr];
        const int right = ((volatile int*)range_r)[curr];
        if (left == 0 && right == n - 1) {
            *root_out = curr;
            parent[curr] = -1;
            break;
        }
        bool parent_right;
        if (left == 0) {
            parent_right = true;
        } else if (right != n - 1 && deltas[right] >= deltas[left - 1]) {
            parent_right = deltas[right] == deltas[left - 1] ? (((sprims[left - 1] % 2u) ^ (sprims[right] % 2u)) != 0)
                                                             : true;
        } else {
            parent_right = false;
        }
        int par;
        if (parent_right) {
            par = right + n;
            parent[curr] = par;
            child_l[par] = curr;
            range_l[par] = left;
        } else {
            par = left + n - 1;
            parent[curr] = par;
            child_r[par] = curr;
            range_r[par] = right;
        }
        __threadfence();
        if (atomicAdd(&counter[par], 1) == 0) break;  // the sibling's thread finishes this node
        __threadfence();
        const int lc = ((volatile int*)child_l)[par], rc = ((volatile int*)child_r)[par];
        const float4 ll = __ldcg(&nlo[lc]), rl = __ldcg(&nlo[rc]), lh = __ldcg(&nhi[lc]), rh = __ldcg(&nhi[rc]);
        nlo[par] = make_float4(smin(ll.x, rl.x), smin(ll.y, rl.y), smin(ll.z, rl.z), 0.0f);
        nhi[par] = make_float4(smax(lh.x, rh.x), smax(lh.y, rh.y), smax(lh.z, rh.z), 0.0f);
        curr = par;
    }
}

// leaf collapse (mark_packed_leaf_nodes, mesh_lbvh.h:205-222) and rebased packed nodes
__global__ void k_lbvh_pack(int n, const float4* __restrict__ nlo, const float4* __restrict__ nhi,
                            const int* __restrict__ range_l, const int* __restrict__ range_r,
                            const int* __restrict__ parent, const int* __restrict__ child_l,
                            const int* __restrict__ child_r, const int* __restrict__ counter,
                            const uint32_t* __restrict__ sprims, const int* __restrict__ root, uint32_t node_base,
                            uint32_t prim_base, uint32_t tri_base, float4* nl, float4* nu, uint32_t* prim,
                            uint32_t* root_global, uint8_t* marked) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 2 * n) return;
    const bool is_node = j < n || counter[j] > 0;
    uint32_t lw = 0, uw = 0;
    float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f), h = l;
    bool leaf = false;
    if (is_node) {
        l = nlo[j];
        h = nhi[j];
        if (j < n) {
            lw = (uint32_t)j;
            uw = (uint32_t)j + 1;
            leaf = true;
        } else {
            lw = (uint32_t)child_l[j];
            uw = (uint32_t)child_r[j];
        }
        int depth = 1;
        for (int p = parent[j]; p != -1; p = parent[p]) depth++;
        const int left = range_l[j], right = range_r[j] + 1;
        if (right - left <= 4 || depth >= 32) {
            lw = (uint32_t)left;
            uw = (uint32_t)right;
            leaf = true;
        }
    }
    marked[j] = leaf ? 1 : 0;
    const uint32_t plw = leaf ? ((lw & 0x3FFFFFFFu) + prim_base) | (1u << 30) : (lw & 0x3FFFFFFFu) + node_base;
    const uint32_t puw = leaf ? (uw & 0x3FFFFFFFu) + prim_base : (uw & 0x3FFFFFFFu) + node_base;
    nl[node_base + j] = make_float4(l.x, l.y, l.z, __uint_as_float(plw));
    nu[node_base + j] = make_float4(h.x, h.y, h.z, __uint_as_float(puw));
    if (j < n) prim[prim_base + j] = sprims[j] + tri_base;
    if (j == *root) *root_global = node_base + (uint32_t)j;
}

// a node is reachable from the root when no proper ancestor is a (collapsed) leaf
__global__ void k_lbvh_reachable(int n, const int* __restrict__ parent, const int* __restrict__ counter,
                                 const uint8_t* __restrict__ marked, uint8_t* reachable) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 2 * n) return;
    bool r = j < n || counter[j] > 0;
    for (int p = r ? parent[j] : -1; p != -1 && r; p = parent[p])
        if (marked[p]) r = false;
    reachable[j] = r ? 1 : 0;
}

// refit: leaf boxes from the new vertices, then the bottom-up unions (counter zeroed)
__global__ void k_lbvh_refit_climb(int n, const float* __restrict__ verts, const uint32_t* __restrict__ tris,
                                   const uint32_t* __restrict__ prim_local, const int* __restrict__ parent,
                                   const int* __restrict__ child_l, const int* __restrict__ child_r, float4* nlo,
                                   float4* nhi, int* counter) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // mesh_bvh.h:149-163 over the leaf's one triangle: 1e30 then each vertex
    const uint32_t t = prim_local[i];
    v3 lo = mk3(1e30f, 1e30f, 1e30f), hi = mk3(-1e30f, -1e30f, -1e30f);
    for (int k = 0; k < 3; k++) {
        const uint32_t v = tris[t * 3 + k];
        lo = mk3(smin(lo.x, verts[v * 3]), smin(lo.y, verts[v * 3 + 1]), smin(lo.z, verts[v * 3 + 2]));
        hi = mk3(smax(hi.x, verts[v * 3]), smax(hi.y, verts[v * 3 + 1]), smax(hi.z, verts[v * 3 + 2]));
    }
    nlo[i] = make_float4(lo.x, lo.y, lo.z, 0.0f);
    nhi[i] = make_float4(hi.x, hi.y, hi.z, 0.0f);
    int curr = i;
    while (true) {
        const int par = parent[curr];
        if (par < 0) break;
        __threadfence();
        if (atomicAdd(&counter[par], 1) == 0) break;
        __threadfence();
        const int lc = child_l[par], rc = child_r[par];
        const float4 ll = __ldcg(&nlo[lc]), rl = __ldcg(&nlo[rc]), lh = __ldcg(&nhi[lc]), rh = __ldcg(&nhi[rc]);
        nlo[par] = make_float4(smin(ll.x, rl.x), smin(ll.y, rl.y), smin(ll.z, rl.z), 0.0f);
        nhi[par] = make_float4(smax(lh.x, rh.x), smax(lh.y, rh.y), smax(lh.z, rh.z), 0.0f);
        curr = par;
    }
}

__global__ void k_lbvh_refit_write(int n, const uint8_t* __restrict__ reachable, const float4* __restrict__ nlo,
                                   const float4* __restrict__ nhi, float4* nl, float4* nu) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 2 * n || !reachable[j]) return;
    const float4 l = nlo[j], h = nhi[j];
    nl[j] = make_float4(l.x, l.y, l.z, nl[j].w);
    nu[j] = make_float4(h.x, h.y, h.z, nu[j].w);
}

// One thread per node slot of the mesh: a reachable inner node X with children (a, b)
// writes the record of a. Leaves and unreachable slots write nothing.
__global__ void k_node_pairs(int n, uint32_t node_base, const uint8_t* __restrict__ reachable,
                             const float4* __restrict__ nl, const float4* __restrict__ nu, float4* pair) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 2 * n || !reachable[j]) return;
    const uint32_t x = node_base + (uint32_t)j;
    const uint32_t lw = __float_as_uint(nl[x].w), uw = __float_as_uint(nu[x].w);
    if ((lw >> 30) & 3u) return;
    const uint32_t a = lw & 0x3FFFFFFFu, b = uw & 0x3FFFFFFFu;
    float4* rec = pair + (size_t)a * 4;
    rec[0] = nl[a];
    rec[1] = nu[a];
    rec[2] = nl[b];
    rec[3] = nu[b];
}

void launch_node_pairs(cudaStream_t st, int n, uint32_t node_base, const uint8_t* reachable, const float4* nl,
                       const float4* nu, float4* pair) {
    if (n <= 0) return;
    k_node_pairs<<<(2 * n + kBvhThreads - 1) / kBvhThreads, kBvhThreads, 0, st>>>(n, node_base, reachable, nl, nu,
                                                                                  pair);
}

size_t lbvh_scratch_words(int n) {
    const size_t nn = (size_t)(n > 0 ? n : 1);
    const size_t blocks = (nn + kBvhThreads - 1) / kBvhThreads;
    const SortPlan sp = make_sort_plan((int64_t)nn, 30, 8, 8);
    return nn * 8                    // triangle boxes (2 float4)
           + blocks * 8              // block partial boxes
           + nn * 5                  // keys, 2 x (key, id) sort buffers
           + 4 * 256 + 4 * sort_lookback_words(sp) + 4  // histograms, look-back, tile counters
           + nn * 2 * 8              // node boxes (2 float4 per node slot)
           + nn * 2 * 3              // range_l, range_r, counter
           + nn + 8;                 // deltas, root
}

namespace {
struct LbvhScratch {
    float4 *tb, *partial, *nlo, *nhi;
    uint32_t *keys, *pk0, *pv0, *pk1, *pv1, *hist, *lookback, *tiles;
    int *range_l, *range_r, *counter, *deltas, *root;
    size_t lb_words;
};
LbvhScratch carve(uint32_t* w, int n) {
    const size_t nn = (size_t)(n > 0 ? n : 1);
    const size_t blocks = (nn + kBvhThreads - 1) / kBvhThreads;
    const SortPlan sp = make_sort_plan((int64_t)nn, 30, 8, 8);
    LbvhScratch s;
    size_t o = 0;
    auto f4 = [&](size_t count) {
        float4* p = reinterpret_cast<float4*>(w + o);
        o += count * 4;
        return p;
    };
    auto u32 = [&](size_t count) {
        uint32_t* p = w + o;
        o += count;
        return p;
    };
    s.tb = f4(nn * 2);
    s.partial = f4(blocks * 2);
    s.nlo = f4(nn * 2);
    s.nhi = f4(nn * 2);
    s.keys = u32(nn);
    s.pk0 = u32(nn);
    s.pv0 = u32(nn);
    s.pk1 = u32(nn);
    s.pv1 = u32(nn);
    s.hist = u32(4 * 256);
    s.lb_words = sort_lookback_words(sp);
    s.lookback = u32(4 * s.lb_words);
    s.tiles = u32(4);
    s.range_l = reinterpret_cast<int*>(u32(nn * 2));
    s.range_r = reinterpret_cast<int*>(u32(nn * 2));
    s.counter = reinterpret_cast<int*>(u32(nn * 2));
    s.deltas = reinterpret_cast<int*>(u32(nn));
    s.root = reinterpret_cast<int*>(u32(8));
    return s;
}
}  // namespace

void launch_lbvh_build(cudaStream_t st, int n, const float* verts, const uint32_t* tris, uint32_t node_base,
                       uint32_t prim_base, uint32_t tri_base, float4* nl, float4* nu, uint32_t* prim,
                       uint32_t* root_global, LbvhTopology topo, uint32_t* scratch, DeviceStatus* status) {
    if (n <= 0) return;
    LbvhScratch s = carve(scratch, n);
    const int blocks = (n + kBvhThreads - 1) / kBvhThreads;
    const int nodes_blocks = (2 * n + kBvhThreads - 1) / kBvhThreads;
    cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * (4 * 256 + 4 * s.lb_words + 4), st);
    cudaMemsetAsync(s.counter, 0, sizeof(int) * 2 * (size_t)n, st);
    cudaMemsetAsync(s.nlo, 0, sizeof(float4) * 4 * (size_t)n, st);  // nlo and nhi (adjacent)
    cudaMemsetAsync(topo.parent, 0xff, sizeof(int) * 2 * (size_t)n, st);
    k_lbvh_bounds<<<blocks, kBvhThreads, 0, st>>>(n, verts, tris, s.tb, s.partial);
    k_lbvh_morton<<<blocks, kBvhThreads, 0, st>>>(n, blocks, s.tb, s.partial, s.keys, s.hist);
    const SortPlan sp = make_sort_plan((int64_t)n, 30, 8, 8);
    const uint32_t* ki = s.keys;
    const uint32_t* vi = nullptr;
    uint32_t* ko[2] = {s.pk0, s.pk1};
    uint32_t* vo[2] = {s.pv0, s.pv1};
    for (int p = 0; p < sp.passes; p++) {
        launch_onesweep_pass(st, n, sp, p, ki, vi, ko[p & 1], vo[p & 1], s.hist + p * 256,
                             s.lookback + (size_t)p * s.lb_words, s.tiles + p, status);
        ki = ko[p & 1];
        vi = vo[p & 1];
    }
    cudaMemcpyAsync(topo.prim_local, vi, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, st);
    k_lbvh_leaves<<<blocks, kBvhThreads, 0, st>>>(n, ki, vi, s.tb, s.nlo, s.nhi, s.range_l, s.range_r, s.deltas);
    k_lbvh_climb<<<blocks, kBvhThreads, 0, st>>>(n, s.deltas, vi, s.nlo, s.nhi, s.range_l, s.range_r, topo.parent,
                                                 topo.child_l, topo.child_r, s.counter, s.root);
    k_lbvh_pack<<<nodes_blocks, kBvhThreads, 0, st>>>(n, s.nlo, s.nhi, s.range_l, s.range_r, topo.parent,
                                                      topo.child_l, topo.child_r, s.counter, vi, s.root, node_base,
                                                      prim_base, tri_base, nl, nu, prim, root_global, topo.marked);
    k_lbvh_reachable<<<nodes_blocks, kBvhThreads, 0, st>>>(n, topo.parent, s.counter, topo.marked, topo.reachable);
}

void launch_lbvh_refit(cudaStream_t st, int n, const float* verts, const uint32_t* tris, LbvhTopology topo,
                       float4* nl, float4* nu, uint32_t* scratch) {
    if (n <= 0) return;
    LbvhScratch s = carve(scratch, n);
    const int blocks = (n + kBvhThreads - 1) / kBvhThreads;
    const int nodes_blocks = (2 * n + kBvhThreads - 1) / kBvhThreads;
    cudaMemsetAsync(s.counter, 0, sizeof(int) * 2 * (size_t)n, st);
    k_lbvh_refit_climb<<<blocks, kBvhThreads, 0, st>>>(n, verts, tris, topo.prim_local, topo.parent, topo.child_l,
                                                       topo.child_r, s.nlo, s.nhi, s.counter);
    k_lbvh_refit_write<<<nodes_blocks, kBvhThreads, 0, st>>>(n, topo.reachable, s.nlo, s.nhi, nl, nu);
}

}  // namespace xpbd
