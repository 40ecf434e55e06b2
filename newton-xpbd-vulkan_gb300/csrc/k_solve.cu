// Fused XPBD iteration: one thread per particle in hash-grid order computes
// its shape-contact deltas (solve_particle_shape_contacts.comp), its
// particle-particle delta (solve_particle_particle_contacts.comp), applies
// them (apply_particle_deltas.comp) and, on the last iteration, the
// restitution increments (apply_particle_shape_restitution.comp).
//
// The reference accumulates deltas and restitution with float atomicAdd from
// one thread per contact, so its summation order varies run to run. Here each
// particle owns its contacts and sums them in the canonical order (plane, then
// mesh slots, then the particle-particle total), which makes the step
// deterministic and needs no delta buffer, no fill and no atomics.
#include "contact.cuh"
#include "kernels.h"
#include "xmath.cuh"

namespace xpbd {

constexpr int kSolveThreads = 64;
constexpr int kPairCap = 12;  // accepted neighbours buffered per thread before the pair math runs

// Pair math of solve_particle_particle_contacts.comp:159-207 for the neighbours
// buffered in shared memory (slot kk, distance d), accumulated in buffer order.
template <bool DIAG>
__device__ __forceinline__ void pair_block(int np, const int (*s_kk)[kSolveThreads], const float (*s_d)[kSolveThreads],
                                           const float4* __restrict__ rx, const float4* __restrict__ rv,
                                           const uint32_t* __restrict__ sids, v3 xp, v3 vp, float radius, float w1,
                                           uint32_t id, const SolveParams& sp, const SolveDiag& dg, v3& acc) {
    for (int q = 0; q < np; q++) {
        const int kk = s_kk[q][threadIdx.x];
        const float d = s_d[q][threadIdx.x];
        const float4 nx = __ldg(&rx[kk]);
        const float4 nv = __ldg(&rv[kk]);
        const v3 raw = vsub(xp, xyz(nx));
        const float err = d - radius - nx.w;
        const float denom = w1 + nv.w;
        if (denom <= 0.0f) continue;
        const v3 nn = exact_div(raw, d);
        const v3 vrel = vsub(vp, xyz(nv));
        const float vn = exact_dot(nn, vrel);
        const v3 vt = mk3(__fmaf_rn(vn, -nn.x, vrel.x), __fmaf_rn(vn, -nn.y, vrel.y), __fmaf_rn(vn, -nn.z, vrel.z));
        const float vt_len = exact_length(vt);
        const float lambda_f = gmax(sp.k_mu * err, -vt_len * sp.dt);
        const v3 vt_dir = vt_len > 0.0f ? exact_div(vt, vt_len) : mk3(0.0f, 0.0f, 0.0f);
        const v3 p2 = vmuls(nn, err);
        const v3 diff = mk3(__fmaf_rn(vt_dir.x, lambda_f, -p2.x), __fmaf_rn(vt_dir.y, lambda_f, -p2.y),
                            __fmaf_rn(vt_dir.z, lambda_f, -p2.z));
        const v3 pair_d = exact_div(diff, denom);
        acc = vadd(acc, pair_d);
        if (DIAG && dg.pair_header) {  // solve_particle_particle_contacts.comp:180-207
            const uint32_t slot = atomicAdd(&dg.pair_header[0], 1u);
            if (slot < dg.max_pairs) {
                float* rec = dg.pairs + (size_t)slot * 20;
                const v3 t = mk3(__fmaf_rn(pair_d.x, w1, 0.0f), __fmaf_rn(pair_d.y, w1, 0.0f),
                                 __fmaf_rn(pair_d.z, w1, 0.0f));
                rec[0] = __uint_as_float(id);
                rec[1] = __uint_as_float(__ldg(&sids[kk]));
                rec[2] = d;
                rec[3] = err;
                rec[4] = nn.x;
                rec[5] = nn.y;
                rec[6] = nn.z;
                rec[7] = vrel.x;
                rec[8] = vrel.y;
                rec[9] = vrel.z;
                rec[10] = vn;
                rec[11] = vt_len;
                rec[12] = denom;
                rec[13] = err;
                rec[14] = lambda_f;
                rec[15] = __fmaf_rn(t.x, sp.relax, 0.0f);
                rec[16] = __fmaf_rn(t.y, sp.relax, 0.0f);
                rec[17] = __fmaf_rn(t.z, sp.relax, 0.0f);
                rec[18] = __uint_as_float((uint32_t)sp.iter_index);
                rec[19] = 0.0f;
            } else {
                atomicAdd(&dg.pair_header[1], 1u);
            }
        }
    }
}

// The particle-particle part of one particle's iteration (solve_particle_particle_contacts.comp:
// 116-217 and the relaxation of apply_particle_deltas.comp): the candidate filter (:145-157)
// runs first and buffers accepted neighbours; the pair math then runs over the buffer in
// candidate order, so lanes stay in step. Returns the relaxed total delta.
template <bool ALL_ACTIVE, bool DIAG>
__device__ __forceinline__ v3 pp_total(int64_t k, int pflag, v3 xp, v3 vp, float radius, float w1, uint32_t id,
                                       const float4* __restrict__ rx, const float4* __restrict__ rv,
                                       const int* __restrict__ rf, const int4* __restrict__ table, bool split,
                                       uint32_t stamp,
                                       const uint32_t* __restrict__ sids, const SolveParams& sp, const SolveDiag& dg,
                                       int (*s_kk)[kSolveThreads], float (*s_d)[kSolveThreads]) {
    const int is_proxy = pflag & 2;
    const float R = radius + sp.max_radius + sp.k_coh;
    const float inv = sp.inv;
    const int32_t xs = f2i(floorf((xp.x - R) * inv)), ys = f2i(floorf((xp.y - R) * inv)),
                  zs = f2i(floorf((xp.z - R) * inv));
    const int32_t xe = min(f2i(floorf((xp.x + R) * inv)), xs + kGridDim - 1);
    const int32_t ye = min(f2i(floorf((xp.y + R) * inv)), ys + kGridDim - 1);
    const int32_t ze = min(f2i(floorf((xp.z + R) * inv)), zs + kGridDim - 1);
    v3 acc = mk3(0.0f, 0.0f, 0.0f);
    int np = 0;
    // cells xs..xe of one (cy, cz) row have consecutive keys unless the row wraps at 128
    // or is clamped at 0 (then the alias bit of x is the same for the whole row); their
    // particles then form one run of the sorted order, in the reference's visit order (x
    // ascending, then sorted order within a cell)
    const int32_t xo = xs + kGridOrigin;
    const bool row_run = xo >= 0 && (xo % kGridDim) + (xe - xs) < kGridDim;
    for (int32_t cz = zs; cz <= ze; cz++) {
        for (int32_t cy = ys; cy <= ye; cy++) {
            for (int32_t cx = xs; cx <= xe; cx++) {
                int lo, hi;
                if (row_run) {
                    const int c0 = cell_index(xs, cy, cz, split);
                    lo = 0x7fffffff;
                    hi = -1;
                    for (int j = 0; j <= xe - xs; j++) {
                        const int4 e = __ldg(&table[c0 + j]);
                        if ((uint32_t)e.z == stamp) {
                            lo = min(lo, e.x);
                            hi = max(hi, e.y);
                        }
                    }
                    cx = xe;  // the run covers the whole row
                } else {
                    const int4 e = __ldg(&table[cell_index(cx, cy, cz, split)]);
                    if ((uint32_t)e.z != stamp) continue;
                    lo = e.x;
                    hi = e.y;
                }
                // candidates in groups of 4: the group's records are loaded together,
                // then tested one by one in order
                for (int kk0 = lo; kk0 < hi; kk0 += 4) {
                    float4 nxs[4];
#pragma unroll
                    for (int u = 0; u < 4; u++)
                        nxs[u] = kk0 + u < hi ? __ldg(&rx[kk0 + u]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int kk = kk0 + u;
                        if (kk >= hi) break;
                        if (kk == k) continue;
                        const int nflag = ALL_ACTIVE ? 1 : __ldg(&rf[kk]);
                        if ((nflag & 1) == 0) continue;
                        if (!ALL_ACTIVE && is_proxy != 0 && (((nflag & 2) != 0) || (__ldg(&rv[kk].w) <= 0.0f)))
                            continue;
                        const float4 nx = nxs[u];
                        const v3 raw = vsub(xp, xyz(nx));
                        if (fabsf(raw.x) > R || fabsf(raw.y) > R || fabsf(raw.z) > R) continue;
                        // exact_length's squared sum; a candidate whose distance provably exceeds
                        // r_i + r_j + cohesion (1.5e-5 relative margin, far above the rounding of
                        // the filter) is rejected before the refined square root
                        const float sq = __fmaf_rn(raw.z, raw.z, __fmaf_rn(raw.x, raw.x, raw.y * raw.y));
                        const float reach = ((radius + nx.w) + sp.k_coh) * 1.0000153f;
                        if (sq > reach * reach) continue;
                        const float d = exact_sqrt(sq);
                        const float err = d - radius - nx.w;
                        if (err > sp.k_coh || d <= 0.0f) continue;
                        s_kk[np][threadIdx.x] = kk;
                        s_d[np][threadIdx.x] = d;
                        if (++np == kPairCap) {
                            pair_block<DIAG>(np, s_kk, s_d, rx, rv, sids, xp, vp, radius, w1, id, sp, dg, acc);
                            np = 0;
                        }
                    }
                }
            }
        }
    }
    pair_block<DIAG>(np, s_kk, s_d, rx, rv, sids, xp, vp, radius, w1, id, sp, dg, acc);
    const v3 dw = mk3(__fmaf_rn(acc.x, w1, 0.0f), __fmaf_rn(acc.y, w1, 0.0f), __fmaf_rn(acc.z, w1, 0.0f));
    return mk3(__fmaf_rn(dw.x, sp.relax, 0.0f), __fmaf_rn(dw.y, sp.relax, 0.0f), __fmaf_rn(dw.z, sp.relax, 0.0f));
}

// Fused XPBD iteration of one particle in sorted order. PP selects how the
// particle-particle total is obtained: kPPFused computes it here; kPPOnly computes only it
// and writes it to pp[k] (no other output; run beside the contact generation, which it
// does not read); kPPApply reads it from pp[k] and does the rest. Both ways add the same
// total to the shape deltas in the same order.
enum { kPPFused = 0, kPPOnly = 1, kPPApply = 2 };

template <bool LAST, bool ALL_ACTIVE, bool DIAG, int PP>
__global__ void __launch_bounds__(kSolveThreads, 16) k_solve(
    int64_t n, const uint32_t* __restrict__ sids, const uint32_t* __restrict__ skeys, const float4* __restrict__ rx,
    const float4* __restrict__ rv, const int* __restrict__ rf, const int4* __restrict__ table_all,
    const uint32_t* __restrict__ stamp_p,
    const float4* __restrict__ x0a, const float4* __restrict__ v0a, const uint32_t* __restrict__ cinfo,
    const float4* __restrict__ cslot, ContactRanks cr, BodyTables bt, SolveParams sp, float4* __restrict__ rx_out,
    float4* __restrict__ rv_out, float4* __restrict__ x_out, float4* __restrict__ v_out, SolveDiag dg,
    BodyDeltaOut bo, float4* __restrict__ pp) {
    __shared__ int s_kk[PP == kPPApply ? 1 : kPairCap][kSolveThreads];
    __shared__ float s_d[PP == kPPApply ? 1 : kPairCap][kSolveThreads];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t id = sids[k];
    const float4 ox = rx[k], ov = rv[k];
    const int pflag = ALL_ACTIVE ? 1 : rf[k];
    const v3 xp = xyz(ox), vp = xyz(ov);
    const float radius = ox.w, w1 = ov.w;
    if constexpr (PP == kPPOnly) {
        v3 total = mk3(0.0f, 0.0f, 0.0f);
        if (pflag & 1) {
            const int4* __restrict__ table = skeys ? table_all + ((size_t)(skeys[k] >> 21) << 21) : table_all;
            total = pp_total<ALL_ACTIVE, DIAG>(k, pflag, xp, vp, radius, w1, id, rx, rv, rf, table, sp.split_keys != 0,
                                               *stamp_p, sids, sp, dg, s_kk, s_d);
        }
        pp[k] = make_float4(total.x, total.y, total.z, 0.0f);
        return;
    }
    v3 x_new = xp, v_new = vp;
    v3 delta = mk3(0.0f, 0.0f, 0.0f);

    if (pflag & 1) {
        const uint32_t info = cinfo ? cinfo[id] : 0u;
        const v3 x0 = xyz(x0a[id]);
        const int ncon = (int)(info & kPlaneBit) + info_slots(info);
        const float4* slots = cslot + (size_t)id * sp.slot_cap * 3;
        // shape contacts, canonical order (scene.cpp:946-947)
        uint32_t dyn_e = bo.bdel ? bo.dyn_rank[id].x : 0u;
        for (int c = 0; c < ncon; c++) {
            const Contact ct = load_contact(info, c, slots, x0, sp.altitude);
            bool ok = false;
            v3 fd, dtot, rr;
            if (contact_kept(info, c, cr, id, sp.contact_max)) {
                ok = shape_delta(ct, pflag, xp, vp, radius, w1, bt, sp, fd, dtot, rr);
                if (ok) delta = vadd(delta, fd);
            }
            if (bo.bdel) {  // body delta of a dynamic-body contact (:193-199), summed per body later
                const int body = bt.shape_body[ct.shape];
                if (body >= 0 && bt.body_invm[body] > 0.0f) {
                    float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a;
                    if (ok) {
                        const v3 dv = mk3(__fdiv_rn(dtot.x, sp.dt), __fdiv_rn(dtot.y, sp.dt), __fdiv_rn(dtot.z, sp.dt));
                        const v3 dw = vcross(rr, dv);
                        a = make_float4(-dv.x, -dv.y, -dv.z, 1.0f);
                        b = make_float4(-dw.x, -dw.y, -dw.z, 0.0f);
                    }
                    bo.bdel[(size_t)dyn_e * 2] = a;
                    bo.bdel[(size_t)dyn_e * 2 + 1] = b;
                    dyn_e++;
                }
            }
        }
        v3 total;
        if constexpr (PP == kPPApply) {
            total = xyz(pp[k]);
        } else {
            // this particle's scene table (scene-major keys); one scene: the whole table
            const int4* __restrict__ table = skeys ? table_all + ((size_t)(skeys[k] >> 21) << 21) : table_all;
            total = pp_total<ALL_ACTIVE, DIAG>(k, pflag, xp, vp, radius, w1, id, rx, rv, rf, table, sp.split_keys != 0,
                                               *stamp_p, sids, sp, dg, s_kk, s_d);
        }
        delta = vadd(delta, total);
        // apply_particle_deltas.comp:43-54
        x_new = vadd(xp, delta);
        v_new = exact_div_apply(vsub(x_new, x0), sp.dt);
        const float v_mag = vlength(v_new);
        if (v_mag > sp.v_max) {
            v_new = vmuls(v_new, __fdiv_rn(sp.v_max, v_mag));
            x_new = vadd(x0, vmuls(v_new, sp.dt));
        }
        if (LAST && sp.enable_restitution && ncon) {
            const v3 v_old = xyz(v0a[id]);
            const v3 v_snap = v_new;
            for (int c = 0; c < ncon; c++) {
                if (!contact_kept(info, c, cr, id, sp.contact_max)) continue;
                const Contact ct = load_contact(info, c, slots, x0, sp.altitude);
                v3 dv;
                if (restitution_dv(ct, v_snap, x0, v_old, radius, bt, sp, dv)) v_new = vadd(v_new, dv);
            }
        }
    }
    if (dg.delta_out) {
        dg.delta_out[(size_t)id * 3 + 0] = delta.x;
        dg.delta_out[(size_t)id * 3 + 1] = delta.y;
        dg.delta_out[(size_t)id * 3 + 2] = delta.z;
    }
    if (LAST) {
        x_out[id] = make_float4(x_new.x, x_new.y, x_new.z, 0.0f);
        v_out[id] = make_float4(v_new.x, v_new.y, v_new.z, 0.0f);
    } else {
        rx_out[k] = make_float4(x_new.x, x_new.y, x_new.z, radius);
        rv_out[k] = make_float4(v_new.x, v_new.y, v_new.z, w1);
    }
}

// apply_particle_shape_restitution.comp:48-116 after the body passes: the last iteration
// has written the final state in particle order; one thread per particle (particle order,
// so the contact headers are read coalesced) adds the restitution increments of its
// contacts (canonical order, on the pre-restitution velocity) to its velocity. Particles
// without a contact, and inactive ones (:256), keep their state.
__global__ void __launch_bounds__(kSolveThreads) k_restitute(
    int64_t n, const int* __restrict__ flags, const float* __restrict__ radii, const float4* __restrict__ x0a,
    const float4* __restrict__ v0a, const uint32_t* __restrict__ cinfo, const float4* __restrict__ cslot,
    ContactRanks cr, BodyTables bt, SolveParams sp, float4* __restrict__ v_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t info = cinfo[i];
    const int ncon = (int)(info & kPlaneBit) + info_slots(info);
    if (ncon == 0 || !(flags[i] & 1)) return;
    const uint32_t id = (uint32_t)i;
    const v3 x0 = xyz(x0a[i]), v_old = xyz(v0a[i]);
    const float4* slots = cslot + (size_t)i * sp.slot_cap * 3;
    const v3 v_snap = xyz(v_out[i]);
    v3 v_new = v_snap;
    for (int c = 0; c < ncon; c++) {
        if (!contact_kept(info, c, cr, id, sp.contact_max)) continue;
        const Contact ct = load_contact(info, c, slots, x0, sp.altitude);
        v3 dv;
        if (restitution_dv(ct, v_snap, x0, v_old, radii[i], bt, sp, dv)) v_new = vadd(v_new, dv);
    }
    v_out[i] = make_float4(v_new.x, v_new.y, v_new.z, 0.0f);
}

void launch_restitute(cudaStream_t s, int64_t n, const int* flags, const float* radii, const float4* x0,
                      const float4* v0, const uint32_t* cinfo, const float4* cslot, ContactRanks cr, BodyTables bt,
                      SolveParams sp, float4* v_out) {
    if (n <= 0) return;
    const int blocks = (int)((n + kSolveThreads - 1) / kSolveThreads);
    k_restitute<<<blocks, kSolveThreads, 0, s>>>(n, flags, radii, x0, v0, cinfo, cslot, cr, bt, sp, v_out);
}

void launch_solve(cudaStream_t s, int64_t n, bool last, bool all_active, const uint32_t* sids, const uint32_t* skeys,
                  const float4* rx, const float4* rv, const int* rf, const int4* table, const uint32_t* stamp,
                  const float4* x0, const float4* v0, const uint32_t* cinfo, const float4* cslot, ContactRanks cr,
                  BodyTables bt, SolveParams sp, float4* rx_out, float4* rv_out, float4* x_out, float4* v_out,
                  SolveDiag dg, BodyDeltaOut bo, int pp_mode, float4* pp) {
    if (n <= 0) return;
    const int threads = kSolveThreads;
    const int blocks = (int)((n + threads - 1) / threads);
    const bool diag = dg.pair_header != nullptr;
#define XPBD_SOLVE(L, A, D, P)                                                                                     \
    if (last == L && all_active == A && diag == D && pp_mode == P) {                                              \
        k_solve<L, A, D, P><<<blocks, threads, 0, s>>>(n, sids, skeys, rx, rv, rf, table, stamp, x0, v0, cinfo,   \
                                                       cslot, cr, bt, sp, rx_out, rv_out, x_out, v_out, dg, bo, pp); \
        return;                                                                                                     \
    }
    XPBD_SOLVE(true, true, false, kPPFused)
    XPBD_SOLVE(true, false, false, kPPFused)
    XPBD_SOLVE(false, true, false, kPPFused)
    XPBD_SOLVE(false, false, false, kPPFused)
    XPBD_SOLVE(true, true, true, kPPFused)
    XPBD_SOLVE(true, false, true, kPPFused)
    XPBD_SOLVE(false, true, true, kPPFused)
    XPBD_SOLVE(false, false, true, kPPFused)
    // the split (no diagnostics): the particle-particle part alone, then the rest
    if (pp_mode == kPPOnly) last = false;  // writes pp only
    XPBD_SOLVE(false, true, false, kPPOnly)
    XPBD_SOLVE(false, false, false, kPPOnly)
    XPBD_SOLVE(true, true, false, kPPApply)
    XPBD_SOLVE(true, false, false, kPPApply)
    XPBD_SOLVE(false, true, false, kPPApply)
    XPBD_SOLVE(false, false, false, kPPApply)
#undef XPBD_SOLVE
}

}  // namespace xpbd
