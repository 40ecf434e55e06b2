// Hand-written adjoint of one substep (plane + particle-particle contacts, one
// solver iteration, restitution), for gradients of a loss on the final state
// with respect to initial positions / velocities, inverse masses and the
// contact parameters (soft_contact_mu, particle_mu, soft_contact_restitution).
//
// The forward substep is x_p = x0 + v_p dt, v_p = v0 + g dt; delta = plane
// terms + w relax sum_j pair_d(i, j); x1 = x_p + delta; v1 = (x1 - x0) / dt;
// restitution sets v1.z = max(-e v0.z, 0) for plane contacts moving in.
// Contact sets and the branch of every friction max() are those of the forward
// pass (recomputed from the substep's start state), so the adjoint is the exact
// derivative of the piecewise-smooth map the forward evaluates.
//
// Two kernels per substep, both in hash-grid order: adj_local (restitution,
// apply and plane terms of each particle, and dL/d(sum_j pair_d) of each
// particle) and adj_pairs (one pass over the neighbours that gathers every
// pair's derivative without atomics, then the adjoint of the integration).
#include "kernels.h"
#include "particle.cuh"
#include "xmath.cuh"

namespace xpbd {

namespace {

// Exact reverse-mode derivative of one pair term of
// solve_particle_particle_contacts.comp:159-177 (pair_d = diff / (w_i + w_j)) for
// the upstream gradient G; forward values are evaluated as the forward does so
// that the friction branch agrees.
__device__ __forceinline__ v3 pair_backward(v3 raw, v3 vrel, float ri, float rj, float wi, float wj, float k_mu,
                                            float dt, v3 G, v3& g_u, v3& g_vrel, float& g_w, float& g_kmu) {
    const float d = exact_length(raw);
    const float err = d - ri - rj;
    const float denom = wi + wj;
    const v3 nn = exact_div(raw, d);
    const float vn = exact_dot(nn, vrel);
    const v3 vt = mk3(__fmaf_rn(vn, -nn.x, vrel.x), __fmaf_rn(vn, -nn.y, vrel.y), __fmaf_rn(vn, -nn.z, vrel.z));
    const float vt_len = exact_length(vt);
    const float a = k_mu * err, b = -vt_len * dt;
    const bool branch_a = !(a < b);
    const float lf = branch_a ? a : b;
    const v3 vt_dir = vt_len > 0.0f ? exact_div(vt, vt_len) : mk3(0.0f, 0.0f, 0.0f);
    const v3 p2 = vmuls(nn, err);
    const v3 diff = mk3(__fmaf_rn(vt_dir.x, lf, -p2.x), __fmaf_rn(vt_dir.y, lf, -p2.y), __fmaf_rn(vt_dir.z, lf, -p2.z));
    const v3 pair_d = exact_div(diff, denom);
    const float inv_den = 1.0f / denom;
    const v3 g_diff = vmuls(G, inv_den);
    g_w = -vdot(G, diff) * inv_den * inv_den;
    const v3 g_vt_dir = vmuls(g_diff, lf);
    const float g_lf = vdot(g_diff, vt_dir);
    v3 g_nn = vmuls(g_diff, -err);
    float g_err = -vdot(g_diff, nn);
    float g_vt_len = 0.0f;
    if (branch_a) {
        g_err += k_mu * g_lf;
        g_kmu += err * g_lf;
    } else {
        g_vt_len = -dt * g_lf;
    }
    v3 g_vt = mk3(0.0f, 0.0f, 0.0f);
    if (vt_len > 0.0f)
        g_vt = vadd(vmuls(vsub(g_vt_dir, vmuls(vt_dir, vdot(vt_dir, g_vt_dir))), 1.0f / vt_len),
                    vmuls(vt_dir, g_vt_len));
    v3 gv = g_vt;
    const float g_vn = -vdot(g_vt, nn);
    g_nn = vadd(g_nn, vmuls(g_vt, -vn));
    g_nn = vadd(g_nn, vmuls(vrel, g_vn));
    gv = vadd(gv, vmuls(nn, g_vn));
    g_vrel = gv;
    g_u = vadd(vmuls(vsub(g_nn, vmuls(nn, vdot(nn, g_nn))), 1.0f / d), vmuls(nn, g_err));
    return pair_d;
}

// Visits the particles of the cells covering [x - R, x + R] (the forward's cell walk,
// solve_particle_particle_contacts.comp:126-141) and calls f(sorted index).
template <class F>
__device__ __forceinline__ void for_cells(v3 x, float R, float inv, bool split, const int4* __restrict__ table,
                                          uint32_t stamp, F&& f) {
    const int32_t xs = f2i(floorf((x.x - R) * inv)), ys = f2i(floorf((x.y - R) * inv)),
                  zs = f2i(floorf((x.z - R) * inv));
    const int32_t xe = min(f2i(floorf((x.x + R) * inv)), xs + kGridDim - 1);
    const int32_t ye = min(f2i(floorf((x.y + R) * inv)), ys + kGridDim - 1);
    const int32_t ze = min(f2i(floorf((x.z + R) * inv)), zs + kGridDim - 1);
    for (int32_t cz = zs; cz <= ze; cz++)
        for (int32_t cy = ys; cy <= ye; cy++)
            for (int32_t cx = xs; cx <= xe; cx++) {
                const int4 e = __ldg(&table[cell_index(cx, cy, cz, split)]);
                if ((uint32_t)e.z != stamp) continue;
                for (int kk = e.x; kk < e.y; kk++) f(kk);
            }
}

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace

constexpr int kAdjThreads = 128;

// Per-particle part: restitution, apply and plane terms (no neighbour access).
// Writes dL/d(sum_j pair_d) of the particle (gacc) for the pair kernel.
__global__ void __launch_bounds__(kAdjThreads) k_adj_local(AdjointArgs a) {
    __shared__ float s_red[3][kAdjThreads / 32];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float g_mu = 0.0f, g_e = 0.0f;
    if (k < a.n) {
        const uint32_t id = a.sids[k];
        const float4 ox = a.rx[k], ov = a.rv[k];
        const v3 xp = xyz(ox), vp = xyz(ov);
        const float r = ox.w, w = ov.w;
        const v3 x0 = xyz(a.x0[id]), v0 = xyz(a.v0[id]);
        // plane contact of the substep (generate_plane_contacts.comp:32-38 on the start position)
        const bool plane = a.plane_on && (a.flags[id] & 1) && (x0.z - a.altitude < a.margin + r);
        const v3 gx1 = xyz(a.gx_in[id]);
        v3 gv1 = xyz(a.gv_in[id]);
        v3 gx0a = mk3(0.0f, 0.0f, 0.0f), gv0a = gx0a;
        // restitution (apply_particle_shape_restitution.comp:283-315): v.z <- max(-e v0.z, 0)
        if (a.restitution_on && plane) {
            const float c_old = (x0.z - a.altitude) - r;
            if (!(c_old > a.ka) && v0.z < 0.0f) {
                const float g_rt = gv1.z;
                gv1.z = 0.0f;
                if ((-a.restitution) * v0.z > 0.0f) {
                    gv0a.z += g_rt * (-a.restitution);
                    g_e += g_rt * (-v0.z);
                }
            }
        }
        // apply (apply_particle_deltas.comp:43-54): x1 = x_p + delta, v1 = (x1 - x0) / dt
        const float inv_dt = 1.0f / a.dt;
        const v3 gdelta = vadd(gx1, vmuls(gv1, inv_dt));
        gx0a = vsub(gx0a, vmuls(gv1, inv_dt));
        v3 gxp = gdelta, gvp = mk3(0.0f, 0.0f, 0.0f);
        // plane (solve_particle_shape_contacts.comp with a static body: w2 = 0, fd = diff relax)
        if (plane) {
            const float c = (xp.z - a.altitude) - r;
            if (!(c > a.ka)) {
                const v3 vt = mk3(vp.x, vp.y, 0.0f);
                const float vt_len = exact_length(vt);
                const float av = a.mu_plane * c, bv = -vt_len * a.dt;
                const bool branch_a = !(av < bv);
                const float lf = branch_a ? av : bv;
                const v3 vt_dir = vt_len > 0.0f ? exact_div(vt, vt_len) : mk3(0.0f, 0.0f, 0.0f);
                const v3 g_diff = vmuls(gdelta, a.relax);
                const v3 g_vt_dir = vmuls(g_diff, lf);
                const float g_lf = vdot(g_diff, vt_dir);
                float g_c = -g_diff.z, g_vt_len = 0.0f;
                if (branch_a) {
                    g_c += a.mu_plane * g_lf;
                    g_mu += c * g_lf;
                } else {
                    g_vt_len = -a.dt * g_lf;
                }
                if (vt_len > 0.0f) {
                    const v3 g_vt =
                        vadd(vmuls(vsub(g_vt_dir, vmuls(vt_dir, vdot(vt_dir, g_vt_dir))), 1.0f / vt_len),
                             vmuls(vt_dir, g_vt_len));
                    gvp.x += g_vt.x;
                    gvp.y += g_vt.y;
                }
                gxp.z += g_c;
            }
        }
        const v3 gacc = vmuls(gdelta, w * a.relax);  // total = sum_j pair_d * w * relax
        a.gacc[k] = make_float4(gacc.x, gacc.y, gacc.z, 0.0f);
        a.part_xp[k] = make_float4(gxp.x, gxp.y, gxp.z, 0.0f);
        a.part_vp[k] = make_float4(gvp.x, gvp.y, gvp.z, 0.0f);
        a.part_x0[k] = make_float4(gx0a.x, gx0a.y, gx0a.z, 0.0f);
        a.part_v0[k] = make_float4(gv0a.x, gv0a.y, gv0a.z, 0.0f);
        a.part_gd[k] = make_float4(gdelta.x, gdelta.y, gdelta.z, 0.0f);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    g_mu = warp_sum(g_mu);
    g_e = warp_sum(g_e);
    if (lane == 0) {
        s_red[0][warp] = g_mu;
        s_red[1][warp] = 0.0f;
        s_red[2][warp] = g_e;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        float t = 0.0f;
        for (int wv = 0; wv < kAdjThreads / 32; wv++) t += s_red[threadIdx.x][wv];
        a.block_params[(size_t)blockIdx.x * 3 + threadIdx.x] = t;
    }
}

// Pair part, one neighbour pass. The pair term is odd in (x_i - x_j, v_i - v_j), so its
// Jacobian J is the same for the ordered pairs (i, j) and (j, i), and i's state receives
// J^T (G_i - G_j) from the two sums that hold the pair (G = dL/d sum, the neighbour
// relation being symmetric); likewise both inverse masses of a pair appear in both
// terms through 1 / (w_i + w_j). Then the adjoint of the integration.
__global__ void __launch_bounds__(kAdjThreads) k_adj_pairs(AdjointArgs a) {
    __shared__ float s_red[kAdjThreads / 32];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float g_kmu = 0.0f;
    if (k < a.n) {
        const uint32_t id = a.sids[k];
        const float4 ox = a.rx[k], ov = a.rv[k];
        const v3 xp = xyz(ox), vp = xyz(ov);
        const float r = ox.w, w = ov.w;
        v3 gxp = xyz(a.part_xp[k]), gvp = xyz(a.part_vp[k]);
        const v3 Gi = xyz(a.gacc[k]);
        float gw = 0.0f;
        v3 acc = mk3(0.0f, 0.0f, 0.0f);
        const float R = r + a.max_radius + a.k_coh;
        for_cells(xp, R, a.inv, a.split_keys != 0, a.table, *a.stamp, [&](int kk) {
            if (kk == (int)k) return;
            const float4 nx = __ldg(&a.rx[kk]);
            const v3 raw = vsub(xp, xyz(nx));
            if (fabsf(raw.x) > R || fabsf(raw.y) > R || fabsf(raw.z) > R) return;
            const float d = exact_length(raw);
            const float err = d - r - nx.w;
            if (err > a.k_coh || d <= 0.0f) return;
            const float4 nv = __ldg(&a.rv[kk]);
            if (w + nv.w <= 0.0f) return;
            const v3 Gj = xyz(__ldg(&a.gacc[kk]));
            v3 g_u, g_vrel;
            float g_den, unused = 0.0f;
            const v3 vrel = vsub(vp, xyz(nv));
            const v3 pd = pair_backward(raw, vrel, r, nx.w, w, nv.w, a.k_mu, a.dt, vsub(Gi, Gj), g_u, g_vrel, g_den,
                                        unused);
            acc = vadd(acc, pd);
            gxp = vadd(gxp, g_u);
            gvp = vadd(gvp, g_vrel);
            gw += g_den;
            // particle_mu: the ordered term (i, j) of i's own sum (branch of the friction max)
            const float vn = exact_dot(exact_div(raw, d), vrel);
            const v3 nn = exact_div(raw, d);
            const v3 vt = mk3(__fmaf_rn(vn, -nn.x, vrel.x), __fmaf_rn(vn, -nn.y, vrel.y), __fmaf_rn(vn, -nn.z, vrel.z));
            const float vt_len = exact_length(vt);
            if (!(a.k_mu * err < -vt_len * a.dt) && vt_len > 0.0f)
                g_kmu += err * vdot(Gi, exact_div(vt, vt_len)) / (w + nv.w);
        });
        gw += vdot(xyz(a.part_gd[k]), acc) * a.relax;
        // integrate (integrate_particles.comp:45-52): x_p = x0 + v_p dt, v_p = v0 + g dt
        gvp = vadd(gvp, vmuls(gxp, a.dt));
        const v3 gx0 = vadd(xyz(a.part_x0[k]), gxp), gv0 = vadd(xyz(a.part_v0[k]), gvp);
        a.gx_out[id] = make_float4(gx0.x, gx0.y, gx0.z, 0.0f);
        a.gv_out[id] = make_float4(gv0.x, gv0.y, gv0.z, 0.0f);
        a.gw[id] += gw;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    g_kmu = warp_sum(g_kmu);
    if (lane == 0) s_red[warp] = g_kmu;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int wv = 0; wv < kAdjThreads / 32; wv++) t += s_red[wv];
        a.block_params[(size_t)blockIdx.x * 3 + 1] = t;
    }
}

// Adds the per-block parameter gradients to the double accumulators in a fixed order:
// one warp per parameter, lane l summing blocks l, l + 32, ... and the lanes combined by
// a fixed shuffle tree (deterministic run to run).
__global__ void k_adj_params(int blocks, const float* __restrict__ block_params, double* acc) {
    const int p = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (p >= 3) return;
    double t = 0.0;
    for (int b = lane; b < blocks; b += 32) t += (double)block_params[(size_t)b * 3 + p];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) acc[p] += t;
}

__global__ void k_bump_stamp(uint32_t* stamp) { *stamp += 1u; }

void launch_bump_stamp(cudaStream_t s, uint32_t* stamp) { k_bump_stamp<<<1, 1, 0, s>>>(stamp); }

void launch_adjoint_substep(cudaStream_t s, const AdjointArgs& a) {
    if (a.n <= 0) return;
    const int blocks = (int)((a.n + kAdjThreads - 1) / kAdjThreads);
    k_adj_local<<<blocks, kAdjThreads, 0, s>>>(a);
    k_adj_pairs<<<blocks, kAdjThreads, 0, s>>>(a);
    k_adj_params<<<1, 96, 0, s>>>(blocks, a.block_params, a.param_acc);
}

size_t adjoint_block_count(int64_t n) { return (size_t)((n + kAdjThreads - 1) / kAdjThreads); }

}  // namespace xpbd
