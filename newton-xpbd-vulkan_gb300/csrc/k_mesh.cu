// Particle contact generation against the ground plane and triangle meshes
// (generate_plane_contacts.comp, generate_mesh_contacts.comp). One thread per
// particle writes its own contacts into per-particle slots, so the contact
// order is fixed (plane, then meshes in index order) without a global atomic
// slot counter.
#include <algorithm>

#include "kernels.h"
#include "mesh.cuh"
#include "particle.cuh"
#include "xmath.cuh"

namespace xpbd {

// first walk index >= wi whose mesh p may reach (mesh_far), nwalk if none: the
// meshes skipped would end their queries without a contact
__device__ __forceinline__ int first_near(const MeshTables& mt, int wi, int nwalk, v3 p) {
    for (; wi < nwalk; wi++)
        if (!mesh_far(mt, mt.walk_list ? __ldg(&mt.walk_list[wi]) : wi, p)) break;
    return wi;
}

// Triage before the traversal (one thread per particle, in queue order): the plane
// test (generate_plane_contacts.comp:37-38) for every particle; particles that may
// reach a mesh (mesh_far) are appended to the near list, in queue order within a
// warp, and every other particle's contact info is final here.
__global__ void __launch_bounds__(256) k_collide_triage(int64_t n, const uint32_t* __restrict__ order,
                                                        const float4* __restrict__ x, const float* __restrict__ r,
                                                        const int* __restrict__ flags, PlaneParams pl,
                                                        MeshTables mt, uint32_t* __restrict__ cinfo,
                                                        uint32_t* ccount, uint32_t* queue, uint32_t* near) {
    __shared__ uint32_t s_warp[8];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int nwalk = mt.walk_list ? mt.walk_count : mt.n_meshes;
    bool is_near = false;
    uint32_t count = 0;
    int64_t i = -1;
    if (t < n) {
        i = order ? (int64_t)__ldg(&order[t]) : t;
        uint32_t info = 0;
        if (flags[i] & 1) {
            const v3 p = xyz(x[i]);
            if (pl.enabled) {
                const float dist = p.z - pl.altitude;
                if (dist < pl.margin + r[i]) info |= kPlaneBit;
            }
            is_near = first_near(mt, 0, nwalk, p) < nwalk;
        }
        if (!is_near) {
            cinfo[i] = info;
            count = info & kPlaneBit;
        }
    }
    const uint32_t m = __ballot_sync(0xffffffffu, is_near);
    if (m) {
        const int leader = __ffs(m) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(queue + 1, (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (is_near) near[base + __popc(m & lanemask_lt())] = (uint32_t)i;
    }
    const uint32_t tot = block_sum(count, s_warp);
    if (threadIdx.x == 0 && tot) atomicAdd(ccount, tot);
}

// Contact generation with persistent warps over the near list (k_collide_triage).
// kCollideLanes lanes of each warp take particles; a warp refills them from the list
// once none of them is busy. Every iteration each busy lane advances its own
// traversal by one step: it pops stack entries until one needs a load (pruned
// entries cost no load), then either orders the children of an inner node (one
// 64-byte sibling record) or tests one triangle of the leaf it holds (one 64-byte
// triangle cache entry). A warp is never held back by a lane with a long run of
// inner nodes before its next leaf: its time is set by its longest particle, not by
// the sum of its per-leaf maxima. The time of the kernel is that of its longest
// chains of dependent steps, so fewer particles per warp (more warps sharing the
// near list, fewer divergent paths per iteration) is faster as long as the list
// fits the resident warps in one round: a warp uses ceil(near / warps) lanes.
// Each particle's own sequence of node visits and triangle tests is that of the
// shader, so its contacts are unchanged.
constexpr int kCollideThreads = 32;  // one warp per block (see launch_collide_walk)

__global__ void __launch_bounds__(kCollideThreads, 32) k_collide(int64_t n, const float4* __restrict__ x,
                                                 const float* __restrict__ r, PlaneParams pl, MeshTables mt,
                                                 int slot_cap, uint32_t* __restrict__ cinfo,
                                                 float4* __restrict__ cslot, uint32_t* ccount, uint32_t* queue,
                                                 const uint32_t* __restrict__ near, DeviceStatus* st) {
    __shared__ uint32_t s_warp[kCollideThreads / 32];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const float eps_md = mt.avg_edge * 1e-3f;
    const float eps2 = eps_md * eps_md;
    int64_t i = -1;
    bool stack_ovf = false, slot_ovf = false;
    v3 p = mk3(0.0f, 0.0f, 0.0f);
    float radius = 0.0f;
    uint32_t info = 0, count = 0;
    uint32_t pc = 0, phi = 0;  // triangles [pc, phi) of the leaf being tested
    int used = 0, ci = 0, wi = 0;
    // meshes walked here: all of them, or the static ones when some belong to dynamic bodies
    const int nwalk = mt.walk_list ? mt.walk_count : mt.n_meshes;
    const uint64_t n_near = queue[1];  // written by k_collide_triage
    const uint64_t warps = (uint64_t)gridDim.x * (kCollideThreads / 32);
    const uint64_t per_warp = (n_near + warps - 1) / warps;
    const int lanes = per_warp < 1 ? 1 : (per_warp > 32 ? 32 : (int)per_warp);
    bool done = lane >= lanes;
    MeshWalk<LocalStack> w;
    w.sp = 0;
    w.overflow = false;
    while (true) {
        // refill once no lane is busy
        if (__ballot_sync(FULL, i >= 0) == 0) {
            const bool need = !done && i < 0;
            const uint32_t m = __ballot_sync(FULL, need);
            if (m) {
                const int leader = __ffs(m) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(queue, (uint32_t)__popc(m));
                base = __shfl_sync(FULL, base, leader);
                if (need) {
                    const uint64_t t = (uint64_t)base + (uint64_t)__popc(m & lt);
                    if (t >= n_near) {
                        done = true;
                    } else {
                        i = (int64_t)__ldg(&near[t]);
                        p = xyz(x[i]);
                        radius = r[i];
                        info = 0;
                        used = 0;
                        if (pl.enabled) {  // generate_plane_contacts.comp:37-38
                            const float dist = p.z - pl.altitude;
                            if (dist < pl.margin + radius) info |= kPlaneBit;
                        }
                        wi = first_near(mt, 0, nwalk, p);  // < nwalk: the triage listed it
                        if (wi < nwalk) {
                            ci = mt.walk_list ? __ldg(&mt.walk_list[wi]) : wi;
                            walk_begin(w, mt, ci, radius, p);
                            pc = phi = 0;
                        } else {
                            cinfo[i] = info;
                            count += info & kPlaneBit;
                            i = -1;
                        }
                    }
                }
            }
        }
        if (__all_sync(FULL, done)) break;
        if (i < 0) continue;
        // one step: pop until an entry needs a load, then an inner node or one triangle
        uint32_t ca = 0, cb = 0;
        bool inner = false;
        while (pc >= phi && w.sp > 0) {
            const int e = walk_pop_entry(w, eps_md, ca, cb);
            if (e == 1) {
                pc = ca;
                phi = cb;
            } else if (e == 2) {
                inner = true;
                break;
            }
        }
        if (inner || pc < phi) {
            const float4* rec = inner ? mt.pair + (size_t)ca * 4 : mt.tri_cache + (size_t)pc * 4;
            const float4 f0 = __ldg(rec), f1 = __ldg(rec + 1), f2 = __ldg(rec + 2), f3 = __ldg(rec + 3);
            if (inner) {
                walk_children(w, p, eps_md, f0, f1, f2, f3);
            } else {
                // degenerate: |cross|/(|e0|^2+|e1|^2+|e2|^2) < 1e-6 (generate_mesh_contacts.comp:250-251)
                if (f3.w >= 0.0f) walk_tri(w, p, eps_md, eps2, f0, f1, f2, f3);
                pc++;
            }
        }
        while (pc >= phi && w.sp == 0) {  // mesh ci done: emit its contact, move to the next mesh
            v3 bp, bv, nn;
            if (walk_finish(w, mt, ci, p, bp, bv, nn)) {
                if (used < slot_cap) {
                    float4* s = cslot + ((size_t)i * slot_cap + used) * 3;
                    s[0] = make_float4(bp.x, bp.y, bp.z, __int_as_float(ci + 1));
                    s[1] = make_float4(nn.x, nn.y, nn.z, 0.0f);
                    s[2] = make_float4(bv.x, bv.y, bv.z, 0.0f);
                    used++;
                } else {
                    slot_ovf = true;
                }
            }
            stack_ovf |= w.overflow;
            w.overflow = false;
            wi = first_near(mt, wi + 1, nwalk, p);
            if (wi < nwalk) {
                ci = mt.walk_list ? __ldg(&mt.walk_list[wi]) : wi;
                walk_begin(w, mt, ci, radius, p);
                pc = phi = 0;
                break;
            }
            info |= (uint32_t)used << 1;
            cinfo[i] = info;
            count += (info & kPlaneBit) + (uint32_t)used;
            i = -1;
            break;
        }
    }
    if (stack_ovf) {
        atomicOr(&st->error_bits, kErrStackOverflow);
        atomicAdd(&st->stack_overflows, 1u);
    }
    if (slot_ovf) {
        atomicOr(&st->error_bits, kErrSlotOverflow);
        atomicAdd(&st->slot_overflows, 1u);
    }
    const uint32_t tot = block_sum(count, s_warp);
    if (threadIdx.x == 0 && tot) atomicAdd(ccount, tot);
}

void launch_collide_triage(cudaStream_t s, int64_t n, const uint32_t* order, const float4* x, const float* r,
                           const int* flags, PlaneParams pl, MeshTables mt, uint32_t* cinfo, uint32_t* ccount,
                           uint32_t* queue, uint32_t* near) {
    if (n <= 0) return;
    k_collide_triage<<<(int)((n + 255) / 256), 256, 0, s>>>(n, order, x, r, flags, pl, mt, cinfo, ccount, queue,
                                                             near);
}

// One warp per block, 32 blocks per SM (the same resident warps as four-warp blocks):
// a block's registers are released as soon as its own warp is done, so the sort chain
// running beside the traversal takes over the SMs of the warps that finish first
// (bench frame 2.89 -> 2.80 ms; the traversal itself is as fast either way).
void launch_collide_walk(cudaStream_t s, int64_t n, const float4* x, const float* r, PlaneParams pl, MeshTables mt,
                         int slot_cap, uint32_t* cinfo, float4* cslot, uint32_t* ccount, uint32_t* queue,
                         const uint32_t* near, DeviceStatus* st, int blocks_per_sm) {
    if (n <= 0) return;
    const int threads = kCollideThreads;
    const int blocks = (int)std::min<int64_t>((n * 32 + threads - 1) / threads,
                                              (int64_t)device_sm_count() * std::max(1, std::min(blocks_per_sm, 32)));
    k_collide<<<blocks, threads, 0, s>>>(n, x, r, pl, mt, slot_cap, cinfo, cslot, ccount, queue, near, st);
}

void launch_collide(cudaStream_t s, int64_t n, const uint32_t* order, const float4* x, const float* r,
                    const int* flags, PlaneParams pl, MeshTables mt, int slot_cap, uint32_t* cinfo, float4* cslot,
                    uint32_t* ccount, uint32_t* queue, uint32_t* near, DeviceStatus* st) {
    launch_collide_triage(s, n, order, x, r, flags, pl, mt, cinfo, ccount, queue, near);
    launch_collide_walk(s, n, x, r, pl, mt, slot_cap, cinfo, cslot, ccount, queue, near, st);
}

// Triangle data that generate_mesh_contacts.comp:239-251 and :117 recompute on
// every visit, evaluated once per leaf slot with the same operations.
__global__ void k_tri_cache(int64_t first, int64_t count, const uint32_t* __restrict__ prim,
                            const uint32_t* __restrict__ tris, const float* __restrict__ verts,
                            float4* __restrict__ cache) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int64_t pc = first + k;
    const uint32_t t = prim[pc];
    const v3 a = ldv(verts, tris[t * 3]), b = ldv(verts, tris[t * 3 + 1]), c = ldv(verts, tris[t * 3 + 2]);
    const v3 e0 = vsub(b, a), e1 = vsub(c, a), e2 = vsub(c, b);
    const v3 normal = vcross(e0, e1);
    const float e0n = vdot(e0, e0), e1n = vdot(e1, e1), e2n = vdot(e2, e2);
    const bool skip = __fdiv_rn(vlength(normal), (e0n + e1n + e2n)) < 1.0e-6f;
    const v3 tn = vnormalize(normal);  // normalize(cross(ab, ac)), ab = e0, ac = e1
    cache[pc * 4 + 0] = make_float4(a.x, a.y, a.z, __uint_as_float(t));
    cache[pc * 4 + 1] = make_float4(b.x, b.y, b.z, e0n);
    cache[pc * 4 + 2] = make_float4(c.x, c.y, c.z, e1n);
    cache[pc * 4 + 3] = make_float4(tn.x, tn.y, tn.z, skip ? -1.0f : e2n);
}

void launch_tri_cache(cudaStream_t s, int64_t first, int64_t count, const uint32_t* prim, const uint32_t* tris,
                      const float* verts, float4* cache) {
    if (count <= 0) return;
    k_tri_cache<<<(int)((count + 255) / 256), 256, 0, s>>>(first, count, prim, tris, verts, cache);
}

__global__ void k_iota(int64_t n, uint32_t* out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint32_t)i;
}
void launch_iota(cudaStream_t s, int64_t n, uint32_t* out) {
    if (n > 0) k_iota<<<(int)((n + 255) / 256), 256, 0, s>>>(n, out);
}

}  // namespace xpbd
