// Rigid bodies: body integration (integrate_bodies.comp), body delta
// application (apply_body_deltas.comp), rigid contact solve
// (solve_body_contact_positions.comp), the rigid contact generator those
// shaders lack, and particle contacts against the meshes of moving bodies.
//
// Body b belongs to mesh b (shape b + 1, scene.cpp:213). A body with inverse
// mass > 0 is dynamic: its mesh vertices are in the body frame and its state
// changes every substep. The reference dispatches none of these shaders (its
// body table is static, scene.cpp:220-238), so their host order is the one of
// an XPBD iteration: particle deltas, body deltas from particle contacts
// (applied without constraint weights), then rigid contacts solved on that
// state and applied with weights.
//
// Every per-body sum runs in a fixed order (entry order of the particle
// contacts, then own vertices before partners' vertices for the rigid
// contacts), replacing the shaders' float atomics.
#include <algorithm>

#include "contact.cuh"
#include "kernels.h"
#include "mesh.cuh"
#include "particle.cuh"
#include "xmath.cuh"

namespace xpbd {

// ---- Warp-convention quaternion helpers as written in integrate_bodies.comp:44-73,
// apply_body_deltas.comp:43-58 and solve_body_contact_positions.comp:44-61 ----
__device__ __forceinline__ v3 wq_rot(q4 q, v3 v) {  // v + 2*cross(q.xyz, cross(q.xyz, v) + v*q.w)
    const v3 qv = mk3(q.x, q.y, q.z);
    const v3 t = vadd(vcross(qv, v), vmuls(v, q.w));
    return vadd(v, vmuls(vcross(qv, t), 2.0f));
}
__device__ __forceinline__ v3 wq_rot_inv(q4 q, v3 v) {
    q4 c = q;
    c.x = -q.x;
    c.y = -q.y;
    c.z = -q.z;
    return wq_rot(c, v);
}
__device__ __forceinline__ q4 wq_mul(q4 p, q4 q) {
    const v3 c = vcross(mk3(p.x, p.y, p.z), mk3(q.x, q.y, q.z));
    q4 r;
    r.w = p.w * q.w - vdot(mk3(p.x, p.y, p.z), mk3(q.x, q.y, q.z));
    r.x = (p.w * q.x + q.w * p.x) + c.x;
    r.y = (p.w * q.y + q.w * p.y) + c.y;
    r.z = (p.w * q.z + q.w * p.z) + c.z;
    return r;
}
__device__ __forceinline__ q4 q_axpy(q4 a, q4 b, float s) {
    q4 r;
    r.x = a.x + b.x * s;
    r.y = a.y + b.y * s;
    r.z = a.z + b.z * s;
    r.w = a.w + b.w * s;
    return r;
}
__device__ __forceinline__ q4 q_normalize(q4 a) {  // v / length(v), IEEE sqrt and division
    const float l = __fsqrt_rn(((a.x * a.x + a.y * a.y) + a.z * a.z) + a.w * a.w);
    q4 r;
    r.x = __fdiv_rn(a.x, l);
    r.y = __fdiv_rn(a.y, l);
    r.z = __fdiv_rn(a.z, l);
    r.w = __fdiv_rn(a.w, l);
    return r;
}
// 3x3 (9 floats, column-major) times vector: col0*v.x + col1*v.y + col2*v.z
__device__ __forceinline__ v3 colmul(const float* m, v3 v) {
    return mk3((m[0] * v.x + m[3] * v.y) + m[6] * v.z, (m[1] * v.x + m[4] * v.y) + m[7] * v.z,
               (m[2] * v.x + m[5] * v.y) + m[8] * v.z);
}
__device__ __forceinline__ q4 f4q(float4 a) {
    q4 r;
    r.x = a.x;
    r.y = a.y;
    r.z = a.z;
    r.w = a.w;
    return r;
}
__device__ __forceinline__ void st_state(float4* q, float4* qd, int b, v3 p, q4 r, v3 v, v3 w) {
    q[b * 2] = make_float4(p.x, p.y, p.z, 0.0f);
    q[b * 2 + 1] = make_float4(r.x, r.y, r.z, r.w);
    qd[b * 2] = make_float4(v.x, v.y, v.z, 0.0f);
    qd[b * 2 + 1] = make_float4(w.x, w.y, w.z, 0.0f);
}

// apply_body_deltas.comp:58-119 for body b with delta (dp, dq)
__device__ void apply_body_delta(const BodyArrays& ba, int b, float dt, const float4* q, const float4* qd, v3 dp,
                                 v3 dq, float inv_weight, int use_weights, float4* qo, float4* qdo) {
    const float inv_m = ba.invm[b];
    if (inv_m == 0.0f) {
        qo[b * 2] = q[b * 2];
        qo[b * 2 + 1] = q[b * 2 + 1];
        qdo[b * 2] = qd[b * 2];
        qdo[b * 2 + 1] = qd[b * 2 + 1];
        return;
    }
    const v3 pos0 = xyz(q[b * 2]);
    const q4 quat0 = f4q(q[b * 2 + 1]);
    const v3 v0 = xyz(qd[b * 2]), w0 = xyz(qd[b * 2 + 1]);
    const float* I9 = ba.I + b * 9;
    const float* Iinv9 = ba.invI + b * 9;
    const v3 com = mk3(ba.com[b * 3], ba.com[b * 3 + 1], ba.com[b * 3 + 2]);
    float weight = 1.0f;
    if (use_weights) {
        if (inv_weight > 0.0f) weight = __fdiv_rn(1.0f, inv_weight);
    }
    dp = vmuls(dp, inv_m * weight);
    const v3 dq_w = vmuls(dq, weight);
    const v3 wb = wq_rot_inv(quat0, w0);
    const v3 dwb = colmul(Iinv9, wq_rot_inv(quat0, dq_w));
    const v3 tb = vadd(vcross(dwb, colmul(I9, vadd(wb, dwb))), vcross(wb, colmul(I9, dwb)));
    const v3 dw1 = wq_rot(quat0, vsub(dwb, vmuls(colmul(Iinv9, tb), dt)));
    q4 dq4;
    dq4.x = dw1.x * dt;
    dq4.y = dw1.y * dt;
    dq4.z = dw1.z * dt;
    dq4.w = 0.0f;
    const q4 quat1 = q_normalize(q_axpy(quat0, wq_mul(dq4, quat0), 0.5f));
    const v3 x_com = vadd(pos0, wq_rot(quat0, com));
    v3 p1 = vadd(x_com, vmuls(dp, dt));
    p1 = vsub(p1, wq_rot(quat1, com));
    v3 v1 = vadd(v0, dp), w1 = vadd(w0, dw1);
    if (vlength(v1) < 1e-4f) v1 = mk3(0.0f, 0.0f, 0.0f);
    if (vlength(w1) < 1e-4f) w1 = mk3(0.0f, 0.0f, 0.0f);
    st_state(qo, qdo, b, p1, quat1, v1, w1);
}

// integrate_bodies.comp:75-130 (body forces are zero); the pre-integration state
// is kept as the substep's previous state
__global__ void k_body_integrate(BodyArrays ba, float4* __restrict__ q_prev, float4* __restrict__ qd_prev,
                                 RigidParams rp) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= ba.nb) return;
    const float4 q0 = ba.q[b * 2], q1 = ba.q[b * 2 + 1], d0 = ba.qd[b * 2], d1 = ba.qd[b * 2 + 1];
    q_prev[b * 2] = q0;
    q_prev[b * 2 + 1] = q1;
    qd_prev[b * 2] = d0;
    qd_prev[b * 2 + 1] = d1;
    if (ba.flags[b] & 2) return;  // KINEMATIC: unchanged
    const float dt = rp.dt;
    const v3 x0 = xyz(q0), v0 = xyz(d0), w0 = xyz(d1);
    const q4 r0 = f4q(q1);
    const v3 f0 = mk3(0.0f, 0.0f, 0.0f), t0 = f0;
    const v3 com = mk3(ba.com[b * 3], ba.com[b * 3 + 1], ba.com[b * 3 + 2]);
    const float inv_mass = ba.invm[b];
    const v3 g = mk3(rp.gx, rp.gy, rp.gz);
    const v3 x_com = vadd(x0, wq_rot(r0, com));
    const float m_scale = inv_mass != 0.0f ? 1.0f : 0.0f;
    const v3 v1 = vadd(v0, vmuls(vadd(vmuls(f0, inv_mass), vmuls(g, m_scale)), dt));
    const v3 x1 = vadd(x_com, vmuls(v1, dt));
    const v3 wb = wq_rot_inv(r0, w0);
    const v3 Iwb = colmul(ba.I + b * 9, wb);
    const v3 tb = vsub(wq_rot_inv(r0, t0), vcross(wb, Iwb));
    const v3 dwb = vmuls(colmul(ba.invI + b * 9, tb), dt);
    v3 w1 = wq_rot(r0, vadd(wb, dwb));
    q4 wq;
    wq.x = w1.x;
    wq.y = w1.y;
    wq.z = w1.z;
    wq.w = 0.0f;
    const q4 r1 = q_normalize(q_axpy(r0, wq_mul(wq, r0), 0.5f * dt));
    w1 = vmuls(w1, 1.0f - rp.damping * dt);
    st_state(ba.q, ba.qd, b, vsub(x1, wq_rot(r1, com)), r1, v1, w1);
}

void launch_body_integrate(cudaStream_t s, BodyArrays ba, float4* q_prev, float4* qd_prev, RigidParams rp) {
    if (ba.nb <= 0) return;
    k_body_integrate<<<(ba.nb + 127) / 128, 128, 0, s>>>(ba, q_prev, qd_prev, rp);
}

// ---------------------------------------------------------------- broad phase ----
// World box of each dynamic body's mesh: the body-frame root box of its BVH,
// rotated and translated (quat_rotate of solve_particle_shape_contacts.comp:50-58).
__global__ void k_body_bounds(BodyArrays ba, RigidTables rt, MeshTables mt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rt.n_dyn) return;
    const int b = rt.dyn[i];
    const uint32_t root = mt.roots[b];
    const v3 lo = xyz(mt.nl[root]), hi = xyz(mt.nu[root]);
    const v3 pos = xyz(ba.q[b * 2]);
    const q4 rot = f4q(ba.q[b * 2 + 1]);
    v3 wl = mk3(3.0e38f, 3.0e38f, 3.0e38f), wh = mk3(-3.0e38f, -3.0e38f, -3.0e38f);
    for (int c = 0; c < 8; c++) {
        const v3 corner = mk3((c & 1) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 4) ? hi.z : lo.z);
        const v3 p = vadd(pos, quat_rotate(rot, corner));
        wl = mk3(fminf(wl.x, p.x), fminf(wl.y, p.y), fminf(wl.z, p.z));
        wh = mk3(fmaxf(wh.x, p.x), fmaxf(wh.y, p.y), fmaxf(wh.z, p.z));
    }
    rt.wbox[i * 2] = make_float4(wl.x, wl.y, wl.z, mt.margins[b]);
    rt.wbox[i * 2 + 1] = make_float4(wh.x, wh.y, wh.z, 0.0f);
}

// Pairs of dynamic bodies whose boxes, widened by the rigid contact margin, their
// shape margins and a rounding pad, overlap. One warp per body; partners ascending.
__global__ void k_body_pairs(RigidTables rt, RigidParams rp, DeviceStatus* st) {
    const int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= rt.n_dyn) return;
    const float4 il = rt.wbox[i * 2], ih = rt.wbox[i * 2 + 1];
    const float ei = rp.margin + il.w + rt.pad;
    int count = 0;
    for (int j0 = 0; j0 < rt.n_dyn; j0 += 32) {
        const int j = j0 + lane;
        bool ov = false;
        if (j < rt.n_dyn && j != i && rt.dyn_scene[j] == rt.dyn_scene[i]) {
            const float4 jl = rt.wbox[j * 2], jh = rt.wbox[j * 2 + 1];
            const float ej = rp.margin + jl.w + rt.pad;
            ov = (il.x - ei <= jh.x + ej) && (jl.x - ej <= ih.x + ei) && (il.y - ei <= jh.y + ej) &&
                 (jl.y - ej <= ih.y + ei) && (il.z - ei <= jh.z + ej) && (jl.z - ej <= ih.z + ei);
        }
        const uint32_t m = __ballot_sync(0xffffffffu, ov);
        if (ov) {
            const int pos = count + __popc(m & lanemask_lt());
            if (pos < kPartnerCap) rt.partners[i * kPartnerCap + pos] = rt.dyn[j];
        }
        count += __popc(m);
    }
    if (lane == 0) {
        rt.partner_count[i] = count < kPartnerCap ? count : kPartnerCap;
        if (count > kPartnerCap) atomicOr(&st->error_bits, kErrBodyOverflow);
    }
}

// ------------------------------------------------------------- box grid ----
__device__ __forceinline__ uint32_t box_cell_hash(int ix, int iy, int iz, int scene, int size) {
    return (((uint32_t)ix * 73856093u) ^ ((uint32_t)iy * 19349663u) ^ ((uint32_t)iz * 83492791u) ^
            ((uint32_t)scene * 2654435761u)) &
           (uint32_t)(size - 1);
}
__device__ __forceinline__ int cell_of(float v, float cs) { return f2i(floorf(v / cs)); }

// cell (x, y, z) of the widened world box of dynamic body i that thread slot c (0 ..
// kBoxCells - 1, kBoxAxis cells per axis from the box's lowest cell) stands for; false
// past the box's own cell range
__device__ __forceinline__ bool box_cell(const RigidTables& rt, int i, int c, int& x, int& y, int& z) {
    const float4 l = rt.wbox[i * 2], h = rt.wbox[i * 2 + 1];
    const float e = rt.grid_reach + l.w;
    x = cell_of(l.x - e, rt.grid_cs) + c % kBoxAxis;
    y = cell_of(l.y - e, rt.grid_cs) + (c / kBoxAxis) % kBoxAxis;
    z = cell_of(l.z - e, rt.grid_cs) + c / (kBoxAxis * kBoxAxis);
    return x <= cell_of(h.x + e, rt.grid_cs) && y <= cell_of(h.y + e, rt.grid_cs) && z <= cell_of(h.z + e, rt.grid_cs);
}

// each dynamic body's widened world box counts itself into the buckets of the cells it
// covers, one thread per (body, cell)
__global__ void k_boxgrid_count(RigidTables rt, DeviceStatus* st) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= rt.n_dyn * kBoxCells) return;
    const int i = g / kBoxCells, c = g % kBoxCells;
    int x, y, z;
    if (box_cell(rt, i, c, x, y, z))
        atomicAdd(&rt.grid_count[box_cell_hash(x, y, z, rt.dyn_scene[i], rt.grid_size)], 1u);
    if (c == kBoxCells - 1) {  // a box wider than kBoxAxis cells per axis would lose cells: report it
        const float4 l = rt.wbox[i * 2], h = rt.wbox[i * 2 + 1];
        const float e = rt.grid_reach + l.w;
        if (cell_of(h.x + e, rt.grid_cs) - cell_of(l.x - e, rt.grid_cs) > kBoxAxis - 1 ||
            cell_of(h.y + e, rt.grid_cs) - cell_of(l.y - e, rt.grid_cs) > kBoxAxis - 1 ||
            cell_of(h.z + e, rt.grid_cs) - cell_of(l.z - e, rt.grid_cs) > kBoxAxis - 1)
            atomicOr(&st->error_bits, kErrBodyOverflow);
    }
}

// Exclusive scan of the bucket counts in three launches (the bucket count grows with the
// number of dynamic bodies): the sum of every tile of kBoxScanTile counts, one block's scan
// of the tile sums, then every tile's own scan from its offset. Each thread reads its 4
// counts as one uint4; the counts become fill cursors (zeroed).
constexpr int kBoxScanThreads = 256;
constexpr int kBoxScanTile = 4 * kBoxScanThreads;

__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t own, uint32_t* s_warp, uint32_t& total) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t incl = own;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t before = 0;
    total = 0;
    for (int w = 0; w < kBoxScanThreads / 32; w++) {
        const uint32_t v = s_warp[w];
        if (w < warp) before += v;
        total += v;
    }
    return before + incl - own;
}

__global__ void __launch_bounds__(kBoxScanThreads) k_boxgrid_tile_sums(RigidTables rt, uint32_t* tile_sum) {
    __shared__ uint32_t s_warp[kBoxScanThreads / 32];
    const int b = blockIdx.x * kBoxScanTile + threadIdx.x * 4;
    uint4 c = make_uint4(0u, 0u, 0u, 0u);
    if (b < rt.grid_size) c = *reinterpret_cast<const uint4*>(rt.grid_count + b);
    uint32_t total;
    block_excl_scan256(c.x + c.y + c.z + c.w, s_warp, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place (tiles <= 4 x 1024), the grand total
// into grid_start[grid_size]
__global__ void __launch_bounds__(1024) k_boxgrid_scan(RigidTables rt, uint32_t* tile_sum, int tiles) {
    __shared__ uint32_t s_warp[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t v[4] = {0u, 0u, 0u, 0u};
    for (int j = 0; j < 4; j++)
        if (tid * 4 + j < tiles) v[j] = tile_sum[tid * 4 + j];
    const uint32_t own = v[0] + v[1] + v[2] + v[3];
    uint32_t incl = own;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    uint32_t run = (warp ? s_warp[warp - 1] : 0u) + incl - own;
    for (int j = 0; j < 4; j++) {
        if (tid * 4 + j < tiles) tile_sum[tid * 4 + j] = run;
        run += v[j];
    }
    if (tid == 0) rt.grid_start[rt.grid_size] = s_warp[31];
}

__global__ void __launch_bounds__(kBoxScanThreads) k_boxgrid_tile_scan(RigidTables rt, const uint32_t* tile_sum) {
    __shared__ uint32_t s_warp[kBoxScanThreads / 32];
    const int b = blockIdx.x * kBoxScanTile + threadIdx.x * 4;
    uint4 c = make_uint4(0u, 0u, 0u, 0u);
    if (b < rt.grid_size) c = *reinterpret_cast<const uint4*>(rt.grid_count + b);
    uint32_t total;
    const uint32_t start = tile_sum[blockIdx.x] + block_excl_scan256(c.x + c.y + c.z + c.w, s_warp, total);
    if (b < rt.grid_size) {
        *reinterpret_cast<uint4*>(rt.grid_start + b) =
            make_uint4(start, start + c.x, start + c.x + c.y, start + c.x + c.y + c.z);
        *reinterpret_cast<uint4*>(rt.grid_count + b) = make_uint4(0u, 0u, 0u, 0u);
    }
}

__global__ void k_boxgrid_fill(RigidTables rt) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= rt.n_dyn * kBoxCells) return;
    const int i = g / kBoxCells, c = g % kBoxCells;
    int x, y, z;
    if (!box_cell(rt, i, c, x, y, z)) return;
    const uint32_t b = box_cell_hash(x, y, z, rt.dyn_scene[i], rt.grid_size);
    rt.grid_list[rt.grid_start[b] + atomicAdd(&rt.grid_count[b], 1u)] = make_int4(i, x, y, z);
}

void launch_body_pairs(cudaStream_t s, BodyArrays ba, RigidTables rt, MeshTables mt, RigidParams rp,
                       DeviceStatus* st) {
    if (rt.n_dyn <= 0) return;
    k_body_bounds<<<(rt.n_dyn + 127) / 128, 128, 0, s>>>(ba, rt, mt);
    k_body_pairs<<<(rt.n_dyn * 32 + 127) / 128, 128, 0, s>>>(rt, rp, st);
    cudaMemsetAsync(rt.grid_count, 0, sizeof(uint32_t) * (size_t)rt.grid_size, s);
    const int cells = (rt.n_dyn * kBoxCells + 127) / 128;
    k_boxgrid_count<<<cells, 128, 0, s>>>(rt, st);
    const int tiles = (rt.grid_size + kBoxScanTile - 1) / kBoxScanTile;
    k_boxgrid_tile_sums<<<tiles, kBoxScanThreads, 0, s>>>(rt, rt.grid_tiles);
    k_boxgrid_scan<<<1, 1024, 0, s>>>(rt, rt.grid_tiles, tiles);
    k_boxgrid_tile_scan<<<tiles, kBoxScanThreads, 0, s>>>(rt, rt.grid_tiles);
    k_boxgrid_fill<<<cells, 128, 0, s>>>(rt);
}

// ---------------------------------------------------------------- rigid contacts ----
// One warp per vertex of a dynamic body's mesh: the vertex against the ground plane,
// then the closest-point query of generate_mesh_contacts.comp (radius 0, the rigid
// margin in place of the soft contact margin) against the static meshes and the
// overlapping dynamic bodies' meshes, in mesh index order (lane 0 merges the two
// ascending lists 32 candidates at a time, each lane queries one). The first
// kRigidSlots contacts are kept. Slot record (5 float4): (p0, shape1 bits),
// (p1, thickness0), (normal, thickness1), (offset0, 0), (offset1, 0).
__global__ void __launch_bounds__(128) k_rigid_contacts(BodyArrays ba, RigidTables rt, MeshTables mt, RigidParams rp,
                                                       DeviceStatus* st) {
    __shared__ int s_cand[4][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int d = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (d >= rt.n_vert) return;  // uniform per warp
    const float4 lv = rt.dv_local[d];
    const int a = __float_as_int(lv.w);
    const v3 V = xyz(lv);
    const v3 pos_a = xyz(ba.q[a * 2]);
    const q4 rot_a = f4q(ba.q[a * 2 + 1]);
    const v3 P = vadd(pos_a, quat_rotate(rot_a, V));
    const float th0 = mt.margins[a];
    float4* out = rt.rc + (size_t)d * kRigidSlots * 5;
    int cnt = 0;
    bool ovf = false, stack_ovf = false;
    if (rp.plane) {
        const float dist = P.z - rp.altitude;
        if (dist < rp.margin) {
            if (lane == 0) {
                const v3 n = mk3(0.0f, 0.0f, -1.0f);
                const float th1 = 0.0f;
                const v3 o0 = quat_rotate_inv(rot_a, vmuls(n, th0)), o1 = vmuls(n, -th1);
                out[0] = make_float4(V.x, V.y, V.z, __int_as_float(0));
                out[1] = make_float4(P.x, P.y, rp.altitude, th0);
                out[2] = make_float4(n.x, n.y, n.z, th1);
                out[3] = make_float4(o0.x, o0.y, o0.z, 0.0f);
                out[4] = make_float4(o1.x, o1.y, o1.z, 0.0f);
            }
            cnt = 1;
        }
    }
    MeshTables rmt = mt;
    rmt.soft_margin = rp.margin;
    const int ia = rt.dyn_index[a];
    const int pc = rt.partner_count[ia];
    const int* partners = rt.partners + ia * kPartnerCap;
    const int total = mt.walk_count + pc;
    int si = 0, pi = 0;  // merge cursors (lane 0)
    for (int c0 = 0; c0 < total; c0 += 32) {
        if (lane == 0) {
            for (int k = 0; k < 32; k++) {
                int m = -1;
                if (si < mt.walk_count || pi < pc) {
                    const int ms = si < mt.walk_count ? mt.walk_list[si] : 0x7fffffff;
                    const int mp = pi < pc ? partners[pi] : 0x7fffffff;
                    if (ms < mp) {
                        m = ms;
                        si++;
                    } else {
                        m = mp;
                        pi++;
                    }
                }
                s_cand[warp][k] = m;
            }
        }
        __syncwarp();
        const int m = s_cand[warp][lane];
        __syncwarp();
        bool found = false;
        v3 bpos, nrm, pos_m = mk3(0.0f, 0.0f, 0.0f);
        q4 rot_m;
        rot_m.x = rot_m.y = rot_m.z = 0.0f;
        rot_m.w = 1.0f;
        bool pz = false;
        if (m >= 0 && m != a) {
            pz = rt.dyn_index[m] >= 0;
            bool near = true;
            if (pz) {  // the vertex is far outside the partner's world box: no contact within the margin
                const int im = rt.dyn_index[m];
                const float4 l = rt.wbox[im * 2], h = rt.wbox[im * 2 + 1];
                const float e = rp.margin + l.w + rt.pad;
                near = P.x >= l.x - e && P.x <= h.x + e && P.y >= l.y - e && P.y <= h.y + e && P.z >= l.z - e &&
                       P.z <= h.z + e;
            }
            if (near) {
                v3 Q = P;
                if (pz) {
                    pos_m = xyz(ba.q[m * 2]);
                    rot_m = f4q(ba.q[m * 2 + 1]);
                    Q = quat_rotate_inv(rot_m, vsub(P, pos_m));
                }
                v3 bvel;
                found = mesh_query(rmt, m, 0.0f, Q, bpos, bvel, nrm, stack_ovf);
            }
        }
        const uint32_t fm = __ballot_sync(0xffffffffu, found);
        if (found) {
            const int slot = cnt + __popc(fm & lanemask_lt());
            if (slot < kRigidSlots) {
                const float th1 = mt.margins[m];
                const v3 n = vneg(pz ? quat_rotate(rot_m, nrm) : nrm);
                const v3 o0 = quat_rotate_inv(rot_a, vmuls(n, th0));
                const v3 o1 = pz ? quat_rotate_inv(rot_m, vmuls(n, -th1)) : vmuls(n, -th1);
                float4* o = out + slot * 5;
                o[0] = make_float4(V.x, V.y, V.z, __int_as_float(m + 1));
                o[1] = make_float4(bpos.x, bpos.y, bpos.z, th0);
                o[2] = make_float4(n.x, n.y, n.z, th1);
                o[3] = make_float4(o0.x, o0.y, o0.z, 0.0f);
                o[4] = make_float4(o1.x, o1.y, o1.z, 0.0f);
            }
        }
        cnt += __popc(fm);
    }
    if (cnt > kRigidSlots) {
        ovf = true;
        cnt = kRigidSlots;
    }
    const bool any_stack = __any_sync(0xffffffffu, stack_ovf);
    if (lane == 0) {
        rt.rc_count[d] = cnt;
        if (ovf) atomicAdd(&st->rigid_slot_overflows, 1u);  // extra contacts dropped, in order
        if (any_stack) {
            atomicOr(&st->error_bits, kErrStackOverflow);
            atomicAdd(&st->stack_overflows, 1u);
        }
    }
}

void launch_rigid_contacts(cudaStream_t s, BodyArrays ba, RigidTables rt, MeshTables mt, RigidParams rp,
                           DeviceStatus* st) {
    if (rt.n_vert <= 0) return;
    k_rigid_contacts<<<(rt.n_vert * 32 + 127) / 128, 128, 0, s>>>(ba, rt, mt, rp, st);
}

// ---------------------------------------------------------------- particle contacts on moving meshes ----
// One thread per particle (hash-grid order): the bodies listed in the particle's cell
// of the box grid whose widened world box holds the particle are queried in their body
// frame (generate_mesh_contacts.comp with the pose inverted); each contact is inserted
// into the particle's slots at its mesh's place, so the list order does not matter.
// Boxes of the box grid that a particle at p (radius r, scene `scene`) may touch, in
// bucket order: f(mesh, q, rot) for each dynamic body of the particle's scene whose
// widened world box holds p and whose root box (body frame, q = p in that frame) is
// within the traversal's first bound.
template <class F>
__device__ __forceinline__ void posed_candidates(const MeshTables& mt, const RigidTables& rt, v3 p, float radius,
                                                 int scene, F&& f) {
    const int cx = cell_of(p.x, rt.grid_cs), cy = cell_of(p.y, rt.grid_cs), cz = cell_of(p.z, rt.grid_cs);
    const uint32_t b = box_cell_hash(cx, cy, cz, scene, rt.grid_size);
    const uint32_t k0 = rt.grid_start[b], k1 = rt.grid_start[b + 1];
    for (uint32_t k = k0; k < k1; k++) {
        const int4 en = __ldg(&rt.grid_list[k]);
        if (en.y != cx || en.z != cy || en.w != cz) continue;  // another cell of this bucket
        const int ci = en.x;
        if (rt.dyn_scene[ci] != scene) continue;  // another scene's body in this cell
        const float4 l = rt.wbox[ci * 2], h = rt.wbox[ci * 2 + 1];
        const float e = (mt.soft_margin + l.w) + radius + rt.pad;
        if (!(p.x >= l.x - e && p.x <= h.x + e && p.y >= l.y - e && p.y <= h.y + e && p.z >= l.z - e &&
              p.z <= h.z + e))
            continue;
        const int mesh = rt.dyn[ci];
        const v3 pos_m = xyz(mt.pose[mesh * 2]);
        const q4 rot_m = f4q(mt.pose[mesh * 2 + 1]);
        const v3 q = quat_rotate_inv(rot_m, vsub(p, pos_m));
        {  // the traversal's first test (root box in the body frame) without starting a traversal
            const uint32_t root = __ldg(&mt.roots[mesh]);
            const float md = mt.soft_margin + l.w + radius;  // walk_begin's max_dist
            if (dist_sq_aabb(q, xyz(__ldg(&mt.nl[root])), xyz(__ldg(&mt.nu[root]))) > md * md) continue;
        }
        if (!f(mesh, q, rot_m)) return;
    }
}

constexpr int kPosedCand = kPosedListWords - 1;  // candidates a list entry carries
constexpr int kPosedWarps = 4;
// list entry: word 0 = particle | (listed candidates << 28) | kPosedMore, words 1.. = the
// candidate meshes in candidate order (-1 past the count)
constexpr uint32_t kPosedMore = 0x80000000u;  // the particle has more than kPosedCand candidates
constexpr uint32_t kPosedIndex = 0x0fffffffu;
struct PosedEntry {
    uint32_t w[kPosedListWords];
};
__device__ __forceinline__ PosedEntry load_entry(const uint32_t* list, int64_t t) {
    PosedEntry e;
    const uint4* src = reinterpret_cast<const uint4*>(list + (size_t)t * kPosedListWords);
#pragma unroll
    for (int j = 0; j < kPosedListWords / 4; j++) {
        const uint4 q = src[j];
        e.w[4 * j] = q.x;
        e.w[4 * j + 1] = q.y;
        e.w[4 * j + 2] = q.z;
        e.w[4 * j + 3] = q.w;
    }
    return e;
}
// the number of candidates a list entry holds (kPosedCand + 1: more follow)
__device__ __forceinline__ int posed_listed(const PosedEntry& e) {
    return (e.w[0] & kPosedMore) ? kPosedCand + 1 : (int)((e.w[0] >> 28) & 7u);
}

// Triage (one thread per particle, in the previous substep's grid order): particles with
// at least one candidate moving mesh go to the posed list, in grid order within a warp,
// each with its first kPosedCand candidate meshes.
__global__ void __launch_bounds__(128) k_posed_triage(int64_t n, const uint32_t* __restrict__ order,
                                                      const float4* __restrict__ x, const float* __restrict__ r,
                                                      const int* __restrict__ flags, MeshTables mt, RigidTables rt,
                                                      uint32_t* counter, uint32_t* list) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int c[kPosedCand];
#pragma unroll
    for (int j = 0; j < kPosedCand; j++) c[j] = -1;
    int nc = 0;
    int64_t i = -1;
    if (t < n) {
        i = order ? (int64_t)order[t] : t;
        if (flags[i] & 1)
            posed_candidates(mt, rt, xyz(x[i]), r[i], rt.pscene ? (int)rt.pscene[i] : 0, [&](int mesh, v3, q4) {
                if (nc < kPosedCand) c[nc] = mesh;
                return ++nc <= kPosedCand;
            });
    }
    const bool any = nc > 0;
    const uint32_t m = __ballot_sync(0xffffffffu, any);
    if (m) {
        const int leader = __ffs(m) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (any) {
            uint32_t w[kPosedListWords];
            w[0] = (uint32_t)i | ((uint32_t)min(nc, kPosedCand) << 28) | (nc > kPosedCand ? kPosedMore : 0u);
#pragma unroll
            for (int j = 0; j < kPosedCand; j++) w[j + 1] = (uint32_t)c[j];
            uint4* dst = reinterpret_cast<uint4*>(list + (size_t)(base + __popc(m & lanemask_lt())) * kPosedListWords);
#pragma unroll
            for (int j = 0; j < kPosedListWords / 4; j++) dst[j] = make_uint4(w[4 * j], w[4 * j + 1], w[4 * j + 2], w[4 * j + 3]);
        }
    }
}

// Particles against the moving meshes (generate_mesh_contacts.comp:197-411 in each body's
// frame) for the posed list, one warp per 32 listed particles. Each lane copies its
// particle's first kPosedCand candidate meshes, listed by the triage, to shared memory; the
// warp then runs all (particle, mesh) queries of those lists one per lane, so lanes with one
// candidate do not wait for lanes with three. Each result goes to the hit buffer at (list
// entry, candidate): the slots are not touched here, so this kernel can run beside the
// static-mesh traversal, and k_posed_merge inserts the hits afterwards.
struct PosedHit {
    float4 a, b, c;  // (body_pos, found), (normal, 0), (body_vel, 0)
};
static_assert(kPosedHitWords == kPosedCand * 3, "hit buffer layout: kPosedCand hits of 3 float4 per list entry");

__device__ __forceinline__ void posed_insert(float4* base, int& used, int slot_cap, bool& slot_ovf, int mesh,
                                             v3 bp, v3 nw, v3 bv) {
    if (used >= slot_cap) {
        slot_ovf = true;
        return;
    }
    int pos = used;
    while (pos > 0 && __float_as_int(base[(pos - 1) * 3].w) > mesh + 1) pos--;
    for (int k2 = used; k2 > pos; k2--) {
        base[k2 * 3] = base[(k2 - 1) * 3];
        base[k2 * 3 + 1] = base[(k2 - 1) * 3 + 1];
        base[k2 * 3 + 2] = base[(k2 - 1) * 3 + 2];
    }
    base[pos * 3] = make_float4(bp.x, bp.y, bp.z, __int_as_float(mesh + 1));
    base[pos * 3 + 1] = make_float4(nw.x, nw.y, nw.z, 0.0f);
    base[pos * 3 + 2] = make_float4(bv.x, bv.y, bv.z, 0.0f);
    used++;
}


__global__ void __launch_bounds__(32 * kPosedWarps, 6) k_collide_posed(
    const uint32_t* __restrict__ list, const uint32_t* __restrict__ counter, const float4* __restrict__ x,
    const float* __restrict__ r, MeshTables mt, PosedHit* __restrict__ hits, DeviceStatus* st) {
    __shared__ int s_cand[kPosedWarps][32][kPosedCand];
    __shared__ float4 s_pos[kPosedWarps][32];
    __shared__ uint32_t s_off[kPosedWarps][33];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t listed = (int64_t)*counter;
    const int64_t stride = (int64_t)gridDim.x * kPosedWarps * 32;
    bool stack_ovf = false;
    // chunks of 32 list entries per warp, grid-stride over the list
    for (int64_t t0 = ((int64_t)blockIdx.x * kPosedWarps + warp) * 32; t0 < listed; t0 += stride) {
        const int64_t t = t0 + lane;
        uint32_t own = 0;
        float4 po = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (t < listed) {
            const PosedEntry e = load_entry(list, t);
            const int64_t i = (int64_t)(e.w[0] & kPosedIndex);
            const float4 xi = x[i];
            po = make_float4(xi.x, xi.y, xi.z, r[i]);
            own = (uint32_t)min(posed_listed(e), kPosedCand);
            for (uint32_t j = 0; j < own; j++) s_cand[warp][lane][j] = (int)e.w[j + 1];
        }
        s_pos[warp][lane] = po;
        uint32_t incl = own;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        s_off[warp][lane] = incl - own;
        if (lane == 31) s_off[warp][32] = incl;
        __syncwarp();
        const uint32_t total = s_off[warp][32];
        // the warp's (particle, mesh) queries, one per lane
        for (uint32_t pr = (uint32_t)lane; pr < total; pr += 32) {
            int o = 0;
            while (o < 31 && s_off[warp][o + 1] <= pr) o++;
            const uint32_t kc = pr - s_off[warp][o];
            const int mesh = s_cand[warp][o][kc];
            const float4 pq = s_pos[warp][o];
            const v3 pos_m = xyz(mt.pose[mesh * 2]);
            const q4 rot_m = f4q(mt.pose[mesh * 2 + 1]);
            const v3 q = quat_rotate_inv(rot_m, vsub(xyz(pq), pos_m));  // as posed_candidates computes it
            v3 bp, bv, nn;
            PosedHit h;
            if (mesh_query(mt, mesh, pq.w, q, bp, bv, nn, stack_ovf)) {
                const v3 nw = quat_rotate(rot_m, nn);
                h.a = make_float4(bp.x, bp.y, bp.z, 1.0f);
                h.b = make_float4(nw.x, nw.y, nw.z, 0.0f);
                h.c = make_float4(bv.x, bv.y, bv.z, 0.0f);
            } else {
                h.a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                h.b = h.a;
                h.c = h.a;
            }
            hits[(size_t)(t0 + o) * kPosedCand + kc] = h;
        }
        __syncwarp();  // the chunk's shared lists are read before the next chunk writes them
    }
    if (stack_ovf) {
        atomicOr(&st->error_bits, kErrStackOverflow);
        atomicAdd(&st->stack_overflows, 1u);
    }
}

// The hits of every list entry inserted into its particle's slots after the static-mesh
// contacts, in the shader's mesh loop order (posed_insert places each by its mesh index);
// candidates past kPosedCand are listed again and queried here, in candidate order. One
// thread per list entry, grid-stride over the list (its length is on the device).
__global__ void __launch_bounds__(128) k_posed_merge(const uint32_t* __restrict__ list,
                                                     const uint32_t* __restrict__ counter,
                                                     const float4* __restrict__ x, const float* __restrict__ r,
                                                     MeshTables mt, RigidTables rt, const PosedHit* __restrict__ hits,
                                                     int slot_cap, uint32_t* __restrict__ cinfo,
                                                     float4* __restrict__ cslot, uint32_t* ccount, DeviceStatus* st) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t listed = (int64_t)*counter;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    if ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31) >= listed) return;  // the whole warp is idle
    bool stack_ovf = false, slot_ovf = false;
    uint32_t added = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < listed; t += stride) {
        int used0 = 0, used = 0;
        const PosedEntry e = load_entry(list, t);
        const int64_t i = (int64_t)(e.w[0] & kPosedIndex);
        const int ncand = posed_listed(e);
        const uint32_t info = cinfo[i];
        used0 = used = info_slots(info);
        float4* base = cslot + (size_t)i * slot_cap * 3;
        for (int k = 0; k < min(ncand, kPosedCand); k++) {
            const PosedHit h = hits[(size_t)t * kPosedCand + k];
            if (h.a.w != 0.0f)
                posed_insert(base, used, slot_cap, slot_ovf, (int)e.w[k + 1], xyz(h.a), xyz(h.b), xyz(h.c));
        }
        if (ncand > kPosedCand) {  // the rest, in candidate order
            const v3 p = xyz(x[i]);
            const float radius = r[i];
            int k = 0;
            posed_candidates(mt, rt, p, radius, rt.pscene ? (int)rt.pscene[i] : 0, [&](int mesh, v3 q, q4 rot_m) {
                if (k++ < kPosedCand) return true;
                v3 bp, bv, nn;
                if (mesh_query(mt, mesh, radius, q, bp, bv, nn, stack_ovf))
                    posed_insert(base, used, slot_cap, slot_ovf, mesh, bp, quat_rotate(rot_m, nn), bv);
                return true;
            });
        }
        // every slot added here belongs to a dynamic body
        if (used != used0)
            cinfo[i] = (info & kPlaneBit) | ((uint32_t)used << 1) | ((uint32_t)(used - used0) << 16);
        added += (uint32_t)(used - used0);
    }
    if (slot_ovf) {
        atomicOr(&st->error_bits, kErrSlotOverflow);
        atomicAdd(&st->slot_overflows, 1u);
    }
    if (stack_ovf) {
        atomicOr(&st->error_bits, kErrStackOverflow);
        atomicAdd(&st->stack_overflows, 1u);
    }
    uint32_t tot = added;
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
    if (lane == 0 && tot) atomicAdd(ccount, tot);
}

void launch_posed_triage(cudaStream_t s, int64_t n, const uint32_t* order, const float4* x, const float* r,
                         const int* flags, MeshTables mt, RigidTables rt, uint32_t* counter, uint32_t* list) {
    if (n <= 0 || rt.n_dyn <= 0) return;
    k_posed_triage<<<(int)((n + 127) / 128), 128, 0, s>>>(n, order, x, r, flags, mt, rt, counter, list);
}

void launch_posed_queries(cudaStream_t s, int64_t n, const float4* x, const float* r, MeshTables mt, RigidTables rt,
                          const uint32_t* counter, const uint32_t* list, float4* hits, DeviceStatus* st) {
    if (n <= 0 || rt.n_dyn <= 0) return;
    // grid-stride over the listed entries (their count is on the device): about four rounds
    // of resident blocks, so a slow chunk does not hold up the end of the launch
    const int blocks = (int)std::min<int64_t>((n + 32 * kPosedWarps - 1) / (32 * kPosedWarps),
                                              (int64_t)device_sm_count() * 6 * 4);
    k_collide_posed<<<blocks, 32 * kPosedWarps, 0, s>>>(list, counter, x, r, mt, reinterpret_cast<PosedHit*>(hits),
                                                       st);
}

void launch_posed_merge(cudaStream_t s, int64_t n, const float4* x, const float* r, MeshTables mt, RigidTables rt,
                        int slot_cap, uint32_t* cinfo, float4* cslot, uint32_t* ccount, const uint32_t* counter,
                        const uint32_t* list, const float4* hits, DeviceStatus* st) {
    if (n <= 0 || rt.n_dyn <= 0) return;
    const int blocks = (int)std::min<int64_t>((n + 127) / 128, (int64_t)device_sm_count() * 16);
    k_posed_merge<<<blocks, 128, 0, s>>>(list, counter, x, r, mt, rt,
                                                          reinterpret_cast<const PosedHit*>(hits), slot_cap, cinfo,
                                                          cslot, ccount, st);
}

// ---------------------------------------------------------------- body-delta entries ----
// Body-delta entry keys (the body of each dynamic slot, at entry rank[i].x + j) and the
// digit histograms of the sort passes, counted per block in shared memory first: the
// keys are few bodies, so direct global atomics would pile onto a handful of bins.
__global__ void __launch_bounds__(256) k_dyn_emit(int64_t n, const uint32_t* __restrict__ cinfo, DynSlots ds,
                                                  const uint2* __restrict__ rank, uint32_t cap, int bits, int passes,
                                                  uint32_t* __restrict__ keys, uint32_t* hist, DeviceStatus* st) {
    __shared__ uint32_t s_hist[4 * 256];
    const int nb = passes << bits;  // passes <= 4, bits <= 8
    for (int k = threadIdx.x; k < nb; k += blockDim.x) s_hist[k] = 0;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool ovf = false;
    const uint32_t info = i < n ? cinfo[i] : 0u;
    if (info_dyn(info) != 0) {
        const int used = info_slots(info);
        uint32_t e = rank[i].x;
        for (int j = 0; j < used; j++) {
            const int shape = __float_as_int(ds.cslot[((size_t)i * ds.slot_cap + j) * 3].w);
            const int body = ds.shape_body[shape];
            if (body >= 0 && ds.body_invm[body] > 0.0f) {
                if (e < cap) {
                    keys[e] = (uint32_t)body;
                    for (int p = 0; p < passes; p++)
                        atomicAdd(&s_hist[(p << bits) + (((uint32_t)body >> (p * bits)) & ((1u << bits) - 1u))], 1u);
                } else {
                    ovf = true;
                }
                e++;
            }
        }
    }
    if (ovf) atomicOr(&st->error_bits, kErrBodyOverflow);
    __syncthreads();
    for (int k = threadIdx.x; k < nb; k += blockDim.x)
        if (s_hist[k]) atomicAdd(&hist[k], s_hist[k]);
}

void launch_dyn_emit(cudaStream_t s, int64_t n, const uint32_t* cinfo, DynSlots ds, const uint2* rank, uint32_t cap,
                     const SortPlan& sp, uint32_t* keys, uint32_t* hist, DeviceStatus* st) {
    if (n <= 0) return;
    k_dyn_emit<<<(int)((n + 255) / 256), 256, 0, s>>>(n, cinfo, ds, rank, cap, sp.bits, sp.passes, keys, hist, st);
}

__global__ void k_body_segments(uint32_t cap, const uint32_t* __restrict__ count, const uint32_t* __restrict__ skeys,
                                uint2* __restrict__ seg) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t e = *count < cap ? *count : cap;
    if (t >= e) return;
    const uint32_t key = skeys[t];
    if (t == 0 || skeys[t - 1] != key) seg[key].x = t;
    if (t == e - 1 || skeys[t + 1] != key) seg[key].y = t + 1;
}

void launch_body_segments(cudaStream_t s, uint32_t cap, const uint32_t* count, const uint32_t* skeys, uint2* seg) {
    if (cap == 0) return;
    k_body_segments<<<(cap + 255) / 256, 256, 0, s>>>(cap, count, skeys, seg);
}

// One warp per body: the body's particle-contact deltas summed in entry order (the
// canonical contact order), then apply_body_deltas.comp with their count as the
// constraint weight (or none when particle_weighting is off).
// 16-byte global -> shared copies that complete asynchronously (PTX cp.async, L2 only)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Per body: the sum of its particle-contact deltas in entry order, then apply_body_deltas.comp.
// One warp per body. The sum is one dependent chain of float additions (the fixed order makes it
// deterministic and equal to the oracle's), so its time is set by the body with the most
// entries; what bounds it is how fast the entries arrive: they are gathered 128 at a time into
// shared memory by asynchronous copies issued a chunk ahead, with the chunk after that's entry
// indices already loading, while lane 0 sums the current chunk.
constexpr int kBodyChunk = 128;
__global__ void __launch_bounds__(128) k_body_particles(BodyArrays ba, const uint2* __restrict__ seg,
                                                       const uint32_t* __restrict__ sorted,
                                                       const float4* __restrict__ bdel,
                                                       const float4* __restrict__ q_in,
                                                       const float4* __restrict__ qd_in, float4* __restrict__ q_out,
                                                       float4* __restrict__ qd_out, RigidParams rp) {
    constexpr int PER_LANE = kBodyChunk / 32;
    __shared__ __align__(16) float4 s_a[4][2][kBodyChunk];
    __shared__ __align__(16) float4 s_c[4][2][kBodyChunk];
    const int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (b >= ba.nb) return;
    // lanes 0-6 each sum one component of the entries in entry order: linear x, y, z, the
    // count (w: 1 for a contact with a delta, 0 without), angular x, y, z
    float part = 0.0f;
    if (ba.invm[b] > 0.0f) {
        const uint2 sg = seg[b];
        uint32_t idx[PER_LANE];  // entry ids of the next chunk to copy
        const auto load_ids = [&](uint32_t base) {
#pragma unroll
            for (int j = 0; j < PER_LANE; j++) {
                const uint32_t k = base + (uint32_t)(j * 32 + lane);
                idx[j] = k < sg.y ? __ldg(&sorted[k]) : 0xffffffffu;
            }
        };
        const auto copy_chunk = [&](int buf) {
#pragma unroll
            for (int j = 0; j < PER_LANE; j++)
                if (idx[j] != 0xffffffffu) {
                    cp_async16(&s_a[w][buf][j * 32 + lane], &bdel[(size_t)idx[j] * 2]);
                    cp_async16(&s_c[w][buf][j * 32 + lane], &bdel[(size_t)idx[j] * 2 + 1]);
                }
            cp_async_commit();
        };
        load_ids(sg.x);
        copy_chunk(0);
        load_ids(sg.x + kBodyChunk);
        int buf = 0;
        for (uint32_t base = sg.x; base < sg.y; base += kBodyChunk) {
            copy_chunk(buf ^ 1);                 // the next chunk (an empty group past the end)
            load_ids(base + 2 * kBodyChunk);      // the chunk after it
            cp_async_wait_prev();                 // this chunk has arrived
            __syncwarp();
            if (lane < 7) {
                // an entry of a contact that produced no delta is all zeros (k_solve writes it
                // so): a sum that starts at +0 is never -0, so adding +0 leaves it unchanged
                // and the loop needs no test
                const float* src = lane < 4 ? reinterpret_cast<const float*>(&s_a[w][buf][0]) + lane
                                            : reinterpret_cast<const float*>(&s_c[w][buf][0]) + (lane - 4);
                const int m = (int)min((uint32_t)kBodyChunk, sg.y - base);
#pragma unroll 8
                for (int l = 0; l < m; l++) part += src[l * 4];
            }
            __syncwarp();  // the buffer is refilled by the next round's copies
            buf ^= 1;
        }
        cp_async_wait_all();
    }
    float c[7];
#pragma unroll
    for (int j = 0; j < 7; j++) c[j] = __shfl_sync(0xffffffffu, part, j);
    if (lane == 0)
        apply_body_delta(ba, b, rp.dt, q_in, qd_in, mk3(c[0], c[1], c[2]), mk3(c[4], c[5], c[6]), c[3],
                         rp.particle_weighting, q_out, qd_out);
}

void launch_body_particles(cudaStream_t s, BodyArrays ba, const uint2* seg, const uint32_t* sorted_entries,
                           const float4* bdel, const float4* q_in, const float4* qd_in, float4* q_out,
                           float4* qd_out, RigidParams rp) {
    if (ba.nb <= 0) return;
    k_body_particles<<<(ba.nb * 32 + 127) / 128, 128, 0, s>>>(ba, seg, sorted_entries, bdel, q_in, qd_in, q_out,
                                                             qd_out, rp);
}

// ---------------------------------------------------------------- rigid contact solve ----
struct RigidContact {
    int shape1;
    v3 p0, p1, n, off0, off1;
    float th0, th1;
};
__device__ __forceinline__ RigidContact load_rc(const float4* s) {
    RigidContact c;
    const float4 a = s[0], b = s[1], d = s[2], e = s[3], f = s[4];
    c.p0 = xyz(a);
    c.shape1 = __float_as_int(a.w);
    c.p1 = xyz(b);
    c.th0 = b.w;
    c.n = xyz(d);
    c.th1 = d.w;
    c.off0 = xyz(e);
    c.off1 = xyz(f);
    return c;
}

// compute_contact_constraint_delta, solve_body_contact_positions.comp:63-83
__device__ __forceinline__ float constraint_delta(float err, q4 qa, q4 qb, float m_inv_a, float m_inv_b,
                                                  const float* ia, const float* ib, v3 lin_a, v3 lin_b, v3 ang_a,
                                                  v3 ang_b, float relax, float dt) {
    float denom = 0.0f;
    denom += vdot(lin_a, lin_a) * m_inv_a;
    denom += vdot(lin_b, lin_b) * m_inv_b;
    const v3 ra = wq_rot_inv(qa, ang_a), rb = wq_rot_inv(qb, ang_b);
    denom += vdot(ra, colmul(ia, ra));
    denom += vdot(rb, colmul(ib, rb));
    float dl = -err;
    if (denom > 0.0f) dl = __fdiv_rn(dl, dt * denom);
    return dl * relax;
}

// solve_body_contact_positions.comp:97-265 for one contact of shape_a (no impulse output)
__device__ bool body_contact(const BodyArrays& ba, const float4* q, const float4* qd, int shape_a,
                             const RigidContact& c, const RigidParams& rp, v3& lin_da, v3& ang_da, v3& lin_db,
                             v3& ang_db) {
    const float zero9[9] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const int shape_b = c.shape1;
    if (shape_a == shape_b) return false;
    const int body_a = shape_a >= 0 ? ba.shape_body[shape_a] : -1;
    const int body_b = shape_b >= 0 ? ba.shape_body[shape_b] : -1;
    if (body_a == body_b) return false;
    v3 pos_a = mk3(0.0f, 0.0f, 0.0f), pos_b = pos_a;
    q4 quat_a;
    quat_a.x = quat_a.y = quat_a.z = 0.0f;
    quat_a.w = 1.0f;
    q4 quat_b = quat_a;
    if (body_a >= 0) {
        pos_a = xyz(q[body_a * 2]);
        quat_a = f4q(q[body_a * 2 + 1]);
    }
    if (body_b >= 0) {
        pos_b = xyz(q[body_b * 2]);
        quat_b = f4q(q[body_b * 2 + 1]);
    }
    const v3 bx_a = vadd(wq_rot(quat_a, c.p0), pos_a);
    const v3 bx_b = vadd(wq_rot(quat_b, c.p1), pos_b);
    const v3 n = c.n;
    const float d = vdot(n, vsub(bx_b, bx_a)) - (c.th0 + c.th1);
    if (d >= 0.0f) return false;
    float m_inv_a = 0.0f, m_inv_b = 0.0f;
    const float* ia = zero9;
    const float* ib = zero9;
    v3 com_a = mk3(0.0f, 0.0f, 0.0f), com_b = com_a, omega_a = com_a, omega_b = com_a;
    if (body_a >= 0) {
        m_inv_a = ba.invm[body_a];
        ia = ba.invI + body_a * 9;
        com_a = mk3(ba.com[body_a * 3], ba.com[body_a * 3 + 1], ba.com[body_a * 3 + 2]);
        omega_a = xyz(qd[body_a * 2 + 1]);
    }
    if (body_b >= 0) {
        m_inv_b = ba.invm[body_b];
        ib = ba.invI + body_b * 9;
        com_b = mk3(ba.com[body_b * 3], ba.com[body_b * 3 + 1], ba.com[body_b * 3 + 2]);
        omega_b = xyz(qd[body_b * 2 + 1]);
    }
    int nz = 0;
    float mu = 0.0f, mu_t = 0.0f, mu_r = 0.0f;
    if (shape_a >= 0) {
        nz += 1;
        mu += ba.shape_mu[shape_a];
        mu_t += rp.mu_t;
        mu_r += rp.mu_r;
    }
    if (shape_b >= 0) {
        nz += 1;
        mu += ba.shape_mu[shape_b];
        mu_t += rp.mu_t;
        mu_r += rp.mu_r;
    }
    if (nz > 0) {
        mu = __fdiv_rn(mu, (float)nz);
        mu_t = __fdiv_rn(mu_t, (float)nz);
        mu_r = __fdiv_rn(mu_r, (float)nz);
    }
    const v3 r_a = vsub(bx_a, vadd(wq_rot(quat_a, com_a), pos_a));
    const v3 r_b = vsub(bx_b, vadd(wq_rot(quat_b, com_b), pos_b));
    const v3 angular_a = vneg(vcross(r_a, n));
    const v3 angular_b = vcross(r_b, n);
    const float lambda_n = constraint_delta(d, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, vneg(n), n, angular_a,
                                            angular_b, rp.relax, rp.dt);
    lin_da = vmuls(vneg(n), lambda_n);
    lin_db = vmuls(n, lambda_n);
    ang_da = vmuls(angular_a, lambda_n);
    ang_db = vmuls(angular_b, lambda_n);
    if (mu > 0.0f) {
        const v3 sbx_a = vadd(wq_rot(quat_a, vadd(c.p0, c.off0)), pos_a);
        const v3 sbx_b = vadd(wq_rot(quat_b, vadd(c.p1, c.off1)), pos_b);
        const v3 delta = vsub(sbx_b, sbx_a);
        v3 fdel = vsub(delta, vmuls(n, vdot(n, delta)));
        const v3 fr_a = vsub(sbx_a, vadd(wq_rot(quat_a, com_a), pos_a));
        const v3 fr_b = vsub(sbx_b, vadd(wq_rot(quat_b, com_b), pos_b));
        v3 rel = mk3(0.0f, 0.0f, 0.0f);
        if (body_a >= 0 && (ba.flags[body_a] & 2)) {
            const v3 va = vadd(xyz(qd[body_a * 2]), vcross(omega_a, fr_a));
            rel = vsub(rel, vsub(va, vmuls(n, vdot(n, va))));
        }
        if (body_b >= 0 && (ba.flags[body_b] & 2)) {
            const v3 vb = vadd(xyz(qd[body_b * 2]), vcross(omega_b, fr_b));
            rel = vadd(rel, vsub(vb, vmuls(n, vdot(n, vb))));
        }
        fdel = vadd(fdel, vmuls(rel, rp.dt));
        const float err = vlength(fdel);
        if (err > 0.0f) {
            const v3 perp = vnormalize(fdel);
            const v3 angular_a_fr = vneg(vcross(fr_a, perp));
            const v3 angular_b_fr = vcross(fr_b, perp);
            float lambda_fr = constraint_delta(err, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, vneg(perp), perp,
                                               angular_a_fr, angular_b_fr, rp.relax, rp.dt);
            lambda_fr = gmax(lambda_fr, -lambda_n * mu);
            lin_da = vsub(lin_da, vmuls(perp, lambda_fr));
            lin_db = vadd(lin_db, vmuls(perp, lambda_fr));
            ang_da = vadd(ang_da, vmuls(angular_a_fr, lambda_fr));
            ang_db = vadd(ang_db, vmuls(angular_b_fr, lambda_fr));
        }
    }
    v3 delta_omega = vsub(omega_b, omega_a);
    const v3 zero = mk3(0.0f, 0.0f, 0.0f);
    if (mu_t > 0.0f) {
        const float err = vdot(delta_omega, n) * rp.dt;
        if (fabsf(err) > 0.0f) {
            float lt = constraint_delta(err, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, zero, zero, vneg(n), n,
                                        rp.relax, rp.dt);
            lt = gclamp(lt, -lambda_n * mu_t, lambda_n * mu_t);
            ang_da = vsub(ang_da, vmuls(n, lt));
            ang_db = vadd(ang_db, vmuls(n, lt));
        }
    }
    if (mu_r > 0.0f) {
        delta_omega = vsub(delta_omega, vmuls(n, vdot(n, delta_omega)));
        const float err = vlength(delta_omega) * rp.dt;
        if (err > 0.0f) {
            const v3 roll_n = vnormalize(delta_omega);
            float lr = constraint_delta(err, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, zero, zero, vneg(roll_n),
                                        roll_n, rp.relax, rp.dt);
            lr = gmax(lr, -lambda_n * mu_r);
            ang_da = vsub(ang_da, vmuls(roll_n, lr));
            ang_db = vadd(ang_db, vmuls(roll_n, lr));
        }
    }
    return true;
}

// Adds the lanes' contributions to (lin, ang, cnt) in lane order (every lane ends
// with the same sums).
__device__ __forceinline__ void warp_ordered_add(bool ok, v3 l, v3 g, v3& lin, v3& ang, float& cnt) {
    const uint32_t m = __ballot_sync(0xffffffffu, ok);
    for (uint32_t r = m; r; r &= r - 1) {
        const int src = __ffs(r) - 1;
        const v3 ls = mk3(__shfl_sync(0xffffffffu, l.x, src), __shfl_sync(0xffffffffu, l.y, src),
                          __shfl_sync(0xffffffffu, l.z, src));
        const v3 gs = mk3(__shfl_sync(0xffffffffu, g.x, src), __shfl_sync(0xffffffffu, g.y, src),
                          __shfl_sync(0xffffffffu, g.z, src));
        lin = vadd(lin, ls);
        ang = vadd(ang, gs);
        cnt += 1.0f;
    }
}

// One warp per body: its rigid contacts as shape0 (own vertices), then as shape1 (the
// overlapping bodies' vertices on its mesh, partners ascending), one slot per lane in
// (vertex, slot) order and summed in that order; then apply_body_deltas.comp with the
// contact count as constraint weight.
__global__ void __launch_bounds__(128) k_body_rigid(BodyArrays ba, RigidTables rt, const float4* __restrict__ q_in,
                                                   const float4* __restrict__ qd_in, float4* __restrict__ q_out,
                                                   float4* __restrict__ qd_out, RigidParams rp) {
    const int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (b >= ba.nb) return;  // uniform per warp
    v3 lin = mk3(0.0f, 0.0f, 0.0f), ang = lin;
    float cnt = 0.0f;
    const int ib = rt.dyn_index[b];
    if (ib >= 0) {
        const uint32_t v0 = rt.dv_start[b], v1 = rt.dv_start[b + 1];
        const uint32_t ns = (v1 - v0) * kRigidSlots;
        for (uint32_t c0 = 0; c0 < ns; c0 += 32) {
            const uint32_t idx = c0 + lane;
            bool ok = false;
            v3 la = mk3(0.0f, 0.0f, 0.0f), aa = la, lb, ab;
            if (idx < ns) {
                const uint32_t d = v0 + idx / kRigidSlots;
                const int j = (int)(idx % kRigidSlots);
                if (j < rt.rc_count[d]) {
                    const RigidContact c = load_rc(rt.rc + ((size_t)d * kRigidSlots + j) * 5);
                    ok = body_contact(ba, q_in, qd_in, b + 1, c, rp, la, aa, lb, ab);
                }
            }
            warp_ordered_add(ok, la, aa, lin, ang, cnt);
        }
        const int pc = rt.partner_count[ib];
        for (int pi = 0; pi < pc; pi++) {
            const int a = rt.partners[ib * kPartnerCap + pi];
            const uint32_t w0 = rt.dv_start[a], w1 = rt.dv_start[a + 1];
            const uint32_t na = (w1 - w0) * kRigidSlots;
            for (uint32_t c0 = 0; c0 < na; c0 += 32) {
                const uint32_t idx = c0 + lane;
                bool ok = false;
                v3 la, aa, lb = mk3(0.0f, 0.0f, 0.0f), ab = lb;
                if (idx < na) {
                    const uint32_t d = w0 + idx / kRigidSlots;
                    const int j = (int)(idx % kRigidSlots);
                    if (j < rt.rc_count[d]) {
                        const float4* sp = rt.rc + ((size_t)d * kRigidSlots + j) * 5;
                        if (__float_as_int(sp[0].w) == b + 1) {
                            const RigidContact c = load_rc(sp);
                            ok = body_contact(ba, q_in, qd_in, a + 1, c, rp, la, aa, lb, ab);
                        }
                    }
                }
                warp_ordered_add(ok, lb, ab, lin, ang, cnt);
            }
        }
    }
    if (lane == 0) apply_body_delta(ba, b, rp.dt, q_in, qd_in, lin, ang, cnt, rp.con_weighting, q_out, qd_out);
}

void launch_body_rigid(cudaStream_t s, BodyArrays ba, RigidTables rt, const float4* q_in, const float4* qd_in,
                       float4* q_out, float4* qd_out, RigidParams rp) {
    if (ba.nb <= 0) return;
    k_body_rigid<<<(ba.nb * 32 + 127) / 128, 128, 0, s>>>(ba, rt, q_in, qd_in, q_out, qd_out, rp);
}

}  // namespace xpbd
