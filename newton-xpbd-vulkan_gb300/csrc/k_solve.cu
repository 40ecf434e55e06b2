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
#include <stdexcept>
#include <type_traits>

#include "contact.cuh"
#include "kernels.h"
#include "xmath.cuh"

namespace xpbd {

constexpr int kSolveThreads = 64;
constexpr int kPairCap = 12;  // accepted neighbours buffered per thread before the pair math runs
constexpr int kCoopCap = 12;  // accepted neighbours buffered per lane for the warp's pair pass
// How a solve kernel computes the particle-particle totals (the solver times both on its scene
// and keeps the faster; the results are the same bits): each thread its own neighbours' pair
// terms, or the warp's pair pass
enum { kFormThread = 0, kFormWarp = 1, kFormStaged = 2, kFormParticleWarp = 3 };

// Shared staging of a block's neighbourhood (the staged form): the sorted records of every
// (y, z) row of cells the block's particles reach, copied once; the per-cell bounds of those
// rows; and each row's first sorted slot and offset in the staged copy. A block stages when
// its particles reach at most 3 x 3 rows, kStageX cells along x without a wrap of the
// 128-cell grid (so each row's cells hold one run of the sorted order), and kStageCap
// records in all; otherwise its threads read the records from global memory as in form 0.
constexpr int kStageX = 40;
constexpr int kStageRows = 9;
constexpr int kStageCap = 512;
struct SolveStage {
    float4 rx[kStageCap];
    int cs[kStageRows][kStageX];  // cell start in the sorted order, -1: no particle this substep
    int ce[kStageRows][kStageX];  // cell end
    int lo[kStageRows];           // the row's first sorted slot
    int off[kStageRows];          // its first record in rx
    int len[kStageRows];
    int box[6];                   // block's cell range: x min, x max, y min, y max, z min, z max
    int ok;
};
// the cells a particle at xp (radius) reaches (solve_particle_particle_contacts.comp:119-131)
struct CellRange {
    int32_t xs, xe, ys, ye, zs, ze;
};
__device__ __forceinline__ CellRange cell_range(v3 xp, float radius, const SolveParams& sp) {
    const float R = radius + sp.max_radius + sp.k_coh;
    const float inv = sp.inv;
    CellRange c;
    c.xs = f2i(floorf((xp.x - R) * inv));
    c.ys = f2i(floorf((xp.y - R) * inv));
    c.zs = f2i(floorf((xp.z - R) * inv));
    c.xe = min(f2i(floorf((xp.x + R) * inv)), c.xs + kGridDim - 1);
    c.ye = min(f2i(floorf((xp.y + R) * inv)), c.ys + kGridDim - 1);
    c.ze = min(f2i(floorf((xp.z + R) * inv)), c.zs + kGridDim - 1);
    return c;
}

// Pair term of solve_particle_particle_contacts.comp:153-177 for a candidate the filter kept
// at squared distance sq (exact_length's sum): the refined distance, the neighbour test
// (:157) and the delta of a particle at (xp, vp), radius, inverse mass w1 from neighbour
// record (nx, nv); .w = 0 when the pair adds nothing (not a neighbour, or zero combined
// inverse mass, :166).
__device__ __forceinline__ float4 pair_term_body(float4 nx, float4 nv, float sq, v3 xp, v3 vp, float radius,
                                                 float w1, float k_mu, float k_coh, float dt) {
    float inv_d, inv_vt;
    const float d = exact_sqrt_rcp(sq, inv_d);
    const float err = d - radius - nx.w;
    if (err > k_coh || d <= 0.0f) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const v3 raw = vsub(xp, xyz(nx));
    const float denom = w1 + nv.w;
    if (denom <= 0.0f) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const v3 nn = exact_div_rcp(raw, d, inv_d);
    const v3 vrel = vsub(vp, xyz(nv));
    const float vn = exact_dot(nn, vrel);
    const v3 vt = mk3(__fmaf_rn(vn, -nn.x, vrel.x), __fmaf_rn(vn, -nn.y, vrel.y), __fmaf_rn(vn, -nn.z, vrel.z));
    const float vt_len = exact_length_rcp(vt, inv_vt);
    const float lambda_f = gmax(k_mu * err, -vt_len * dt);
    const v3 vt_dir = vt_len > 0.0f ? exact_div_rcp(vt, vt_len, inv_vt) : mk3(0.0f, 0.0f, 0.0f);
    const v3 p2 = vmuls(nn, err);
    const v3 diff = mk3(__fmaf_rn(vt_dir.x, lambda_f, -p2.x), __fmaf_rn(vt_dir.y, lambda_f, -p2.y),
                        __fmaf_rn(vt_dir.z, lambda_f, -p2.z));
    const v3 pair_d = exact_div(diff, denom);
    return make_float4(pair_d.x, pair_d.y, pair_d.z, 1.0f);
}
// the same, out of line (the rare path of a lane whose buffer fills)
__device__ __noinline__ float4 pair_term(float4 nx, float4 nv, float sq, v3 xp, v3 vp, float radius, float w1,
                                         float k_mu, float k_coh, float dt) {
    return pair_term_body(nx, nv, sq, xp, vp, radius, w1, k_mu, k_coh, dt);
}

// Pair math of solve_particle_particle_contacts.comp:159-207 for the neighbours
// buffered in shared memory (slot kk, distance d), accumulated in buffer order.
template <bool DIAG>
__device__ __forceinline__ void pair_block(int np, const int (*s_kk)[kSolveThreads], const float (*s_d)[kSolveThreads],
                                           const float4* __restrict__ rx, const float4* __restrict__ rv,
                                           const uint32_t* __restrict__ sids, v3 xp, v3 vp, float radius, float w1,
                                           uint32_t id, const SolveParams& sp, const SolveDiag& dg, v3& acc) {
    for (int q = 0; q < np; q++) {
        const int kk = s_kk[q][threadIdx.x];
        const float4 nx = __ldg(&rx[kk]);
        const float4 nv = __ldg(&rv[kk]);
        float inv_d, inv_vt;
        const float d = exact_sqrt_rcp(s_d[q][threadIdx.x], inv_d);  // the buffer holds squared distances
        const float err = d - radius - nx.w;
        if (err > sp.k_coh || d <= 0.0f) continue;  // :157
        const v3 raw = vsub(xp, xyz(nx));
        const float denom = w1 + nv.w;
        if (denom <= 0.0f) continue;
        const v3 nn = exact_div_rcp(raw, d, inv_d);
        const v3 vrel = vsub(vp, xyz(nv));
        const float vn = exact_dot(nn, vrel);
        const v3 vt = mk3(__fmaf_rn(vn, -nn.x, vrel.x), __fmaf_rn(vn, -nn.y, vrel.y), __fmaf_rn(vn, -nn.z, vrel.z));
        const float vt_len = exact_length_rcp(vt, inv_vt);
        const float lambda_f = gmax(sp.k_mu * err, -vt_len * sp.dt);
        const v3 vt_dir = vt_len > 0.0f ? exact_div_rcp(vt, vt_len, inv_vt) : mk3(0.0f, 0.0f, 0.0f);
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

// The candidate filter of solve_particle_particle_contacts.comp:116-157 for the particle in
// sorted slot k: accept(kk, sq) for every candidate slot kk within reach (squared distance sq,
// the refined distance and the neighbour test of :153-157 follow in the pair term), in the
// shader's visit order (cells x fastest, then y, then z; sorted order within a cell).
template <bool ALL_ACTIVE, class F>
__device__ __forceinline__ void pp_filter(int64_t k, int pflag, v3 xp, float radius, const float4* __restrict__ rx,
                                          const float4* __restrict__ rv, const int* __restrict__ rf,
                                          const int4* __restrict__ table, bool split, uint32_t stamp,
                                          const SolveParams& sp, F&& accept, const SolveStage* st = nullptr) {
    const int is_proxy = pflag & 2;
    const float R = radius + sp.max_radius + sp.k_coh;
    const CellRange cr = cell_range(xp, radius, sp);
    const int32_t xs = cr.xs, ys = cr.ys, zs = cr.zs, xe = cr.xe, ye = cr.ye, ze = cr.ze;
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
                const float4* src = rx;  // where candidate kk's record is read: rx[kk], or the stage
                if (st) {
                    // the block staged this row (its range covers every thread's rows and cells)
                    const int ny = st->box[3] - st->box[2] + 1;
                    const int r = (cz - st->box[4]) * ny + (cy - st->box[2]);
                    lo = 0x7fffffff;
                    hi = -1;
                    for (int32_t x = xs; x <= xe; x++) {
                        const int c0 = st->cs[r][x - st->box[0]];
                        if (c0 >= 0) {
                            lo = min(lo, c0);
                            hi = max(hi, st->ce[r][x - st->box[0]]);
                        }
                    }
                    src = st->rx + (st->off[r] - st->lo[r]);
                    cx = xe;  // the run covers the whole row
                } else if (row_run) {
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
                // candidates in pairs: the pair's records are loaded together, then tested
                // in order (pairs measured faster than fours and than single loads: fewer live
                // registers, fewer spills, and rows are short)
                for (int kk0 = lo; kk0 < hi; kk0 += 2) {
                    float4 nxs[2];
#pragma unroll
                    for (int u = 0; u < 2; u++)
                        nxs[u] = kk0 + u < hi ? (st ? src[kk0 + u] : __ldg(&rx[kk0 + u]))
                                              : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
                    for (int u = 0; u < 2; u++) {
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
                        accept(kk, sq);
                    }
                }
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
                                       int (*s_kk)[kSolveThreads], float (*s_d)[kSolveThreads],
                                       const SolveStage* st = nullptr) {
    v3 acc = mk3(0.0f, 0.0f, 0.0f);
    int np = 0;
    pp_filter<ALL_ACTIVE>(
        k, pflag, xp, radius, rx, rv, rf, table, split, stamp, sp,
        [&](int kk, float sq) {
            s_kk[np][threadIdx.x] = kk;
            s_d[np][threadIdx.x] = sq;
            if (++np == kPairCap) {
                pair_block<DIAG>(np, s_kk, s_d, rx, rv, sids, xp, vp, radius, w1, id, sp, dg, acc);
                np = 0;
            }
        },
        st);
    pair_block<DIAG>(np, s_kk, s_d, rx, rv, sids, xp, vp, radius, w1, id, sp, dg, acc);
    const v3 dw = mk3(__fmaf_rn(acc.x, w1, 0.0f), __fmaf_rn(acc.y, w1, 0.0f), __fmaf_rn(acc.z, w1, 0.0f));
    return mk3(__fmaf_rn(dw.x, sp.relax, 0.0f), __fmaf_rn(dw.y, sp.relax, 0.0f), __fmaf_rn(dw.z, sp.relax, 0.0f));
}

// Shared memory of one warp's pair pass (pp_total_warp).
struct WarpPairs {
    int kk[kCoopCap][32];  // accepted neighbour slots of each lane, candidate order
    float sq[kCoopCap][32];  // their squared distances
    float4 own_x[32];      // (xp, radius) of each lane's particle
    float4 own_v[32];      // (vp, inverse mass)
    uint32_t off[33];      // exclusive prefix of the lanes' buffered counts
    float4 res[32];        // pair terms of the current 32 buffered neighbours
};

// pp_total for a whole warp (all 32 lanes call it; active = false for a lane with nothing to
// add). Each lane filters its candidates in the shader's order and buffers the accepted ones;
// the warp then computes the pair terms of all buffered neighbours 32 at a time, so a lane
// with few neighbours does not idle while another works through many, and each lane adds its
// own terms in its candidate order. A lane whose buffer fills before its filter is done adds
// that buffer's terms itself first. Each particle's sum runs over the same terms in the same
// order as pp_total, so both give the same bits.
template <bool ALL_ACTIVE>
__device__ __forceinline__ v3 pp_total_warp(bool active, int64_t k, int pflag, v3 xp, v3 vp, float radius, float w1,
                                            const float4* __restrict__ rx, const float4* __restrict__ rv,
                                            const int* __restrict__ rf, const int4* __restrict__ table, bool split,
                                            uint32_t stamp, const SolveParams& sp, WarpPairs& wp) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    v3 acc = mk3(0.0f, 0.0f, 0.0f);
    int np = 0;
    if (active) {
        pp_filter<ALL_ACTIVE>(k, pflag, xp, radius, rx, rv, rf, table, split, stamp, sp, [&](int kk, float sq) {
            wp.kk[np][lane] = kk;
            wp.sq[np][lane] = sq;
            if (++np == kCoopCap) {
                for (int q = 0; q < np; q++) {
                    const int j = wp.kk[q][lane];
                    const float4 t = pair_term(__ldg(&rx[j]), __ldg(&rv[j]), wp.sq[q][lane], xp, vp, radius, w1,
                                               sp.k_mu, sp.k_coh, sp.dt);
                    if (t.w != 0.0f) acc = vadd(acc, xyz(t));
                }
                np = 0;
            }
        });
    }
    uint32_t incl = (uint32_t)np;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t my_off = incl - (uint32_t)np;
    wp.off[lane] = my_off;
    if (lane == 31) wp.off[32] = incl;
    wp.own_x[lane] = make_float4(xp.x, xp.y, xp.z, radius);
    wp.own_v[lane] = make_float4(vp.x, vp.y, vp.z, w1);
    __syncwarp();
    const uint32_t total = wp.off[32];
    for (uint32_t c = 0; c < total; c += 32) {
        const uint32_t t = c + (uint32_t)lane;
        if (t < total) {
            int o = 0;  // the lane whose buffer holds term t: the last o with off[o] <= t
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (o + step < 32 && wp.off[o + step] <= t) o += step;
            const uint32_t q = t - wp.off[o];
            const int j = wp.kk[q][o];
            const float4 ox = wp.own_x[o], ov = wp.own_v[o];
            wp.res[lane] = pair_term_body(__ldg(&rx[j]), __ldg(&rv[j]), wp.sq[q][o], xyz(ox), xyz(ov), ox.w, ov.w,
                                          sp.k_mu, sp.k_coh, sp.dt);
        }
        __syncwarp();
        const uint32_t lo = max(my_off, c), hi = min(my_off + (uint32_t)np, c + 32u);
        for (uint32_t u = lo; u < hi; u++) {
            const float4 r = wp.res[u - c];
            if (r.w != 0.0f) acc = vadd(acc, xyz(r));
        }
        __syncwarp();
    }
    const v3 dw = mk3(__fmaf_rn(acc.x, w1, 0.0f), __fmaf_rn(acc.y, w1, 0.0f), __fmaf_rn(acc.z, w1, 0.0f));
    return mk3(__fmaf_rn(dw.x, sp.relax, 0.0f), __fmaf_rn(dw.y, sp.relax, 0.0f), __fmaf_rn(dw.z, sp.relax, 0.0f));
}

// Fused XPBD iteration of one particle in sorted order. PP selects how the
// particle-particle total is obtained: kPPFused computes it here; kPPOnly computes only it
// and writes it to pp[k] (no other output; run beside the contact generation, which it
// does not read); kPPApply reads it from pp[k] and does the rest. Both ways add the same
// total to the shape deltas in the same order.
enum { kPPFused = 0, kPPOnly = 1, kPPApply = 2 };

// The particle-particle total of one particle computed by a whole warp (the per-particle-warp
// form; every lane calls it for the same particle and gets the same total). The lanes take
// the particle's candidates 32 at a time in the filter's order (rows of cells z outer, y
// inner, x ascending within a row), each testing one candidate as pp_filter does and
// computing its pair term; the accepted terms of a round are then added in lane order, which
// is candidate order. A row's cells have consecutive keys up to the grid's wrap (every 128
// cells, where the reference's key wraps and a split key's alias bit changes) and again
// after it, so a row is one run of the sorted order, or two when it crosses the wrap: the
// cells before it, then the cells after it, which is the row's x order. A particle with more
// than 32 such runs, or with cells clamped at grid coordinate 0, is done by lane 0 alone in
// the filter's order.
template <bool ALL_ACTIVE>
__device__ __forceinline__ v3 pp_total_pwarp(int64_t k, int pflag, v3 xp, v3 vp, float radius, float w1,
                                             const float4* __restrict__ rx, const float4* __restrict__ rv,
                                             const int* __restrict__ rf, const int4* __restrict__ table, bool split,
                                             uint32_t stamp, const SolveParams& sp) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int is_proxy = pflag & 2;
    const float R = radius + sp.max_radius + sp.k_coh;
    const CellRange cr = cell_range(xp, radius, sp);
    const int nyr = cr.ye - cr.ys + 1, rows = nyr * (cr.ze - cr.zs + 1);
    const int32_t xo = cr.xs + kGridOrigin;
    const int ncx = cr.xe - cr.xs + 1;  // at most kGridDim (cell_range)
    // cells of a row before the wrap; the rest (if any) follow it
    const int first = xo >= 0 ? min(ncx, kGridDim - (xo % kGridDim)) : ncx;
    const int nseg = first < ncx ? 2 : 1;
    const int segs = rows * nseg;  // runs of the sorted order, in visit order
    v3 acc = mk3(0.0f, 0.0f, 0.0f);
    if (xo < 0 || segs > 32) {
        if (lane == 0)
            pp_filter<ALL_ACTIVE>(k, pflag, xp, radius, rx, rv, rf, table, split, stamp, sp, [&](int kk, float sq) {
                const float4 t = pair_term(__ldg(&rx[kk]), __ldg(&rv[kk]), sq, xp, vp, radius, w1, sp.k_mu,
                                           sp.k_coh, sp.dt);
                if (t.w != 0.0f) acc = vadd(acc, xyz(t));
            });
        acc = mk3(__shfl_sync(FULL, acc.x, 0), __shfl_sync(FULL, acc.y, 0), __shfl_sync(FULL, acc.z, 0));
    } else {
        int lo = 0x7fffffff, hi = -1;  // lane s: the sorted range of run s
        if (lane < segs) {
            const int row = lane / nseg, after = lane - row * nseg;  // after: the run past the wrap
            const int c0 = cell_index(cr.xs + (after ? first : 0), cr.ys + row % nyr, cr.zs + row / nyr, split);
            const int ncell = after ? ncx - first : first;
            // the first three cells' entries are loaded together (a run rarely has more)
            int4 e3[3];
#pragma unroll
            for (int j = 0; j < 3; j++) e3[j] = j < ncell ? __ldg(&table[c0 + j]) : make_int4(0, -1, 0, 0);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                if (j < ncell && (uint32_t)e3[j].z == stamp) {
                    lo = min(lo, e3[j].x);
                    hi = max(hi, e3[j].y);
                }
            }
            for (int j = 3; j < ncell; j++) {
                const int4 e = __ldg(&table[c0 + j]);
                if ((uint32_t)e.z == stamp) {
                    lo = min(lo, e.x);
                    hi = max(hi, e.y);
                }
            }
        }
        const int len = hi > lo ? hi - lo : 0;
        int incl = len;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const int excl = incl - len;
        const int total_c = __shfl_sync(FULL, incl, 31);
        for (int base = 0; base < total_c; base += 32) {
            const int c = base + lane;
            int r = 0;  // the run of candidate c: the last run starting at or before it
            for (int q = 1; q < segs; q++)
                if (__shfl_sync(FULL, excl, q) <= c) r = q;
            const int kk = __shfl_sync(FULL, lo, r) + (c - __shfl_sync(FULL, excl, r));
            float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (c < total_c && kk != k) {
                const int nflag = ALL_ACTIVE ? 1 : __ldg(&rf[kk]);
                bool ok = (nflag & 1) != 0;
                if (!ALL_ACTIVE && ok && is_proxy != 0 && (((nflag & 2) != 0) || (__ldg(&rv[kk].w) <= 0.0f)))
                    ok = false;
                if (ok) {
                    // both records at once: the velocity is needed by every accepted candidate
                    const float4 nx = __ldg(&rx[kk]);
                    const float4 nv = __ldg(&rv[kk]);
                    const v3 raw = vsub(xp, xyz(nx));
                    if (!(fabsf(raw.x) > R || fabsf(raw.y) > R || fabsf(raw.z) > R)) {
                        const float sq = __fmaf_rn(raw.z, raw.z, __fmaf_rn(raw.x, raw.x, raw.y * raw.y));
                        const float reach = ((radius + nx.w) + sp.k_coh) * 1.0000153f;
                        if (!(sq > reach * reach))
                            t = pair_term_body(nx, nv, sq, xp, vp, radius, w1, sp.k_mu, sp.k_coh, sp.dt);
                    }
                }
            }
            for (uint32_t m = __ballot_sync(FULL, t.w != 0.0f); m; m &= m - 1) {
                const int src = __ffs(m) - 1;
                acc = vadd(acc, mk3(__shfl_sync(FULL, t.x, src), __shfl_sync(FULL, t.y, src),
                                    __shfl_sync(FULL, t.z, src)));
            }
        }
    }
    const v3 dw = mk3(__fmaf_rn(acc.x, w1, 0.0f), __fmaf_rn(acc.y, w1, 0.0f), __fmaf_rn(acc.z, w1, 0.0f));
    return mk3(__fmaf_rn(dw.x, sp.relax, 0.0f), __fmaf_rn(dw.y, sp.relax, 0.0f), __fmaf_rn(dw.z, sp.relax, 0.0f));
}

// The staged form's block setup (every thread of the block calls it; `active` = this thread
// filters neighbours): the block's cell range, then, when it qualifies, the cell bounds of its
// rows and their sorted records in shared memory. Returns whether the block staged (the same
// for all its threads).
__device__ __forceinline__ bool stage_block(SolveStage& st, bool active, v3 xp, float radius, const SolveParams& sp,
                                            const float4* __restrict__ rx, const int4* __restrict__ table, bool split,
                                            uint32_t stamp) {
    const int tid = threadIdx.x;
    if (tid < 6) st.box[tid] = (tid & 1) ? (int)0x80000000 : 0x7fffffff;
    __syncthreads();
    if (active) {
        const CellRange c = cell_range(xp, radius, sp);
        atomicMin(&st.box[0], c.xs);
        atomicMax(&st.box[1], c.xe);
        atomicMin(&st.box[2], c.ys);
        atomicMax(&st.box[3], c.ye);
        atomicMin(&st.box[4], c.zs);
        atomicMax(&st.box[5], c.ze);
    }
    __syncthreads();
    const int x0 = st.box[0], x1 = st.box[1], y0 = st.box[2], y1 = st.box[3], z0 = st.box[4], z1 = st.box[5];
    const int xo = x0 + kGridOrigin;
    // no thread filters, more than 3 x 3 rows, rows too long or wrapping: no staging
    if (x0 > x1 || y1 - y0 > 2 || z1 - z0 > 2 || x1 - x0 >= kStageX || xo < 0 || (xo % kGridDim) + (x1 - x0) >= kGridDim)
        return false;
    const int nx = x1 - x0 + 1, ny = y1 - y0 + 1, rows = ny * (z1 - z0 + 1);
    for (int c = tid; c < rows * nx; c += kSolveThreads) {
        const int r = c / nx, x = c - r * nx;
        const int4 e = __ldg(&table[cell_index(x0 + x, y0 + r % ny, z0 + r / ny, split)]);
        const bool live = (uint32_t)e.z == stamp;
        st.cs[r][x] = live ? e.x : -1;
        st.ce[r][x] = live ? e.y : -1;
    }
    __syncthreads();
    if (tid < rows) {
        int lo = 0x7fffffff, hi = -1;
        for (int x = 0; x < nx; x++) {
            if (st.cs[tid][x] >= 0) {
                lo = min(lo, st.cs[tid][x]);
                hi = max(hi, st.ce[tid][x]);
            }
        }
        st.lo[tid] = hi > lo ? lo : 0;
        st.len[tid] = hi > lo ? hi - lo : 0;
    }
    __syncthreads();
    if (tid == 0) {
        int off = 0;
        for (int r = 0; r < rows; r++) {
            st.off[r] = off;
            off += st.len[r];
        }
        st.ok = off <= kStageCap;
    }
    __syncthreads();
    if (!st.ok) return false;
    for (int r = 0; r < rows; r++)
        for (int i = tid; i < st.len[r]; i += kSolveThreads) st.rx[st.off[r] + i] = __ldg(&rx[st.lo[r] + i]);
    __syncthreads();
    return true;
}

template <bool LAST, bool ALL_ACTIVE, bool DIAG, int PP, int FORM>
__global__ void __launch_bounds__(kSolveThreads, 16) k_solve(
    int64_t n, const uint32_t* __restrict__ sids, const uint32_t* __restrict__ skeys, const float4* __restrict__ rx,
    const float4* __restrict__ rv, const int* __restrict__ rf, const int4* __restrict__ table_all,
    const uint32_t* __restrict__ stamp_p,
    const float4* __restrict__ x0a, const float4* __restrict__ v0a, const uint32_t* __restrict__ cinfo,
    const float4* __restrict__ cslot, ContactRanks cr, BodyTables bt, SolveParams sp, float4* __restrict__ rx_out,
    float4* __restrict__ rv_out, float4* __restrict__ x_out, float4* __restrict__ v_out, SolveDiag dg,
    BodyDeltaOut bo, float4* __restrict__ pp) {
    // the warp's pair pass (pp_total_warp) computes the particle-particle totals; the
    // diagnostic kernels keep the per-thread form, which records every pair as it is summed
    constexpr bool WARP = FORM == kFormWarp && !DIAG && PP != kPPApply;
    // the staged form: the block's neighbourhood records in shared memory (SolveStage)
    constexpr bool STAGED = FORM == kFormStaged && !DIAG && PP != kPPApply;
    // the per-particle-warp form: one particle per warp (pp_total_pwarp), lane 0 then goes on
    constexpr bool PWARP = FORM == kFormParticleWarp && !DIAG && PP != kPPApply;
    __shared__ int s_kk[(PP == kPPApply || WARP) ? 1 : kPairCap][kSolveThreads];
    __shared__ float s_d[(PP == kPPApply || WARP) ? 1 : kPairCap][kSolveThreads];
    __shared__ WarpPairs s_wp[WARP ? kSolveThreads / 32 : 1];
    __shared__ typename std::conditional<STAGED, SolveStage, char>::type s_stage;
    const int64_t k0 = PWARP ? (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5)
                             : (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (!WARP && !STAGED && k0 >= n) return;  // (whole warps in the per-particle-warp form)
    const bool valid = k0 < n;  // every lane of a warp reaches the warp's pair pass (every thread the staging)
    const int64_t k = valid ? k0 : n - 1;
    const uint32_t id = sids[k];
    const float4 ox = rx[k], ov = rv[k];
    const int pflag = valid ? (ALL_ACTIVE ? 1 : rf[k]) : 0;
    const v3 xp = xyz(ox), vp = xyz(ov);
    const float radius = ox.w, w1 = ov.w;
    v3 total = mk3(0.0f, 0.0f, 0.0f);
    const SolveStage* stage = nullptr;
    if constexpr (STAGED) {
        // one scene only (scene-major keys index per-scene tables)
        if (!skeys && stage_block(s_stage, valid && (pflag & 1) != 0, xp, radius, sp, rx, table_all,
                                  sp.split_keys != 0, *stamp_p))
            stage = &s_stage;
        if (!valid) return;
    }
    // the per-particle-warp form loads lane 0's shape-contact inputs before the pair pass, so
    // their latency overlaps it instead of following it
    uint32_t pre_info = 0u;
    float4 pre_x0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), pre_v0 = pre_x0;
    if constexpr (PWARP && PP != kPPOnly) {
        if (pflag & 1) {
            pre_info = cinfo ? cinfo[id] : 0u;
            pre_x0 = x0a[id];
            if (LAST && sp.enable_restitution) pre_v0 = v0a[id];
        }
    }
    if constexpr (PWARP) {
        if (pflag & 1) {  // the same particle in every lane
            const int4* __restrict__ table = skeys ? table_all + ((size_t)(skeys[k] >> 21) << 21) : table_all;
            total = pp_total_pwarp<ALL_ACTIVE>(k, pflag, xp, vp, radius, w1, rx, rv, rf, table, sp.split_keys != 0,
                                               *stamp_p, sp);
        }
        if ((threadIdx.x & 31) != 0) return;
    }
    if constexpr (WARP) {
        // this particle's scene table (scene-major keys); one scene: the whole table
        const int4* __restrict__ table = skeys ? table_all + ((size_t)(skeys[k] >> 21) << 21) : table_all;
        total = pp_total_warp<ALL_ACTIVE>((pflag & 1) != 0, k, pflag, xp, vp, radius, w1, rx, rv, rf, table,
                                          sp.split_keys != 0, *stamp_p, sp, s_wp[threadIdx.x >> 5]);
        if (!valid) return;
    }
    if constexpr (PP == kPPOnly) {
        if constexpr (!WARP && !PWARP) {
            if (pflag & 1) {
                const int4* __restrict__ table = skeys ? table_all + ((size_t)(skeys[k] >> 21) << 21) : table_all;
                total = pp_total<ALL_ACTIVE, DIAG>(k, pflag, xp, vp, radius, w1, id, rx, rv, rf, table,
                                                   sp.split_keys != 0, *stamp_p, sids, sp, dg, s_kk, s_d, stage);
            }
        }
        pp[k] = make_float4(total.x, total.y, total.z, 0.0f);
        return;
    }
    v3 x_new = xp, v_new = vp;
    v3 delta = mk3(0.0f, 0.0f, 0.0f);

    if (pflag & 1) {
        const uint32_t info = PWARP ? pre_info : (cinfo ? cinfo[id] : 0u);
        const v3 x0 = xyz(PWARP ? pre_x0 : x0a[id]);
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
        if constexpr (PP == kPPApply) {
            total = xyz(pp[k]);
        } else if constexpr (!WARP && !PWARP) {
            // this particle's scene table (scene-major keys); one scene: the whole table
            const int4* __restrict__ table = skeys ? table_all + ((size_t)(skeys[k] >> 21) << 21) : table_all;
            total = pp_total<ALL_ACTIVE, DIAG>(k, pflag, xp, vp, radius, w1, id, rx, rv, rf, table, sp.split_keys != 0,
                                               *stamp_p, sids, sp, dg, s_kk, s_d, stage);
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
            const v3 v_old = xyz(PWARP ? pre_v0 : v0a[id]);
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
                  SolveDiag dg, BodyDeltaOut bo, int pp_mode, float4* pp, int form) {
    if (n <= 0) return;
    const int threads = kSolveThreads;
    const bool diag = dg.pair_header != nullptr;
    // the warp forms apply where the particle-particle totals are computed without diagnostics
    if (diag || pp_mode == kPPApply) form = kFormThread;
    const int64_t per_block = form == kFormParticleWarp ? threads / 32 : threads;
    const int blocks = (int)((n + per_block - 1) / per_block);
#define XPBD_SOLVE(L, A, D, P, F)                                                                                  \
    if (last == L && all_active == A && diag == D && pp_mode == P && form == F) {                                 \
        k_solve<L, A, D, P, F><<<blocks, threads, 0, s>>>(n, sids, skeys, rx, rv, rf, table, stamp, x0, v0, cinfo, \
                                                          cslot, cr, bt, sp, rx_out, rv_out, x_out, v_out, dg, bo,  \
                                                          pp);                                                      \
        return;                                                                                                     \
    }
    XPBD_SOLVE(true, true, false, kPPFused, kFormThread)
    XPBD_SOLVE(true, false, false, kPPFused, kFormThread)
    XPBD_SOLVE(false, true, false, kPPFused, kFormThread)
    XPBD_SOLVE(false, false, false, kPPFused, kFormThread)
    XPBD_SOLVE(true, true, false, kPPFused, kFormWarp)
    XPBD_SOLVE(true, false, false, kPPFused, kFormWarp)
    XPBD_SOLVE(false, true, false, kPPFused, kFormWarp)
    XPBD_SOLVE(false, false, false, kPPFused, kFormWarp)
    XPBD_SOLVE(true, true, false, kPPFused, kFormStaged)
    XPBD_SOLVE(true, false, false, kPPFused, kFormStaged)
    XPBD_SOLVE(false, true, false, kPPFused, kFormStaged)
    XPBD_SOLVE(false, false, false, kPPFused, kFormStaged)
    XPBD_SOLVE(true, true, false, kPPFused, kFormParticleWarp)
    XPBD_SOLVE(true, false, false, kPPFused, kFormParticleWarp)
    XPBD_SOLVE(false, true, false, kPPFused, kFormParticleWarp)
    XPBD_SOLVE(false, false, false, kPPFused, kFormParticleWarp)
    XPBD_SOLVE(true, true, true, kPPFused, kFormThread)
    XPBD_SOLVE(true, false, true, kPPFused, kFormThread)
    XPBD_SOLVE(false, true, true, kPPFused, kFormThread)
    XPBD_SOLVE(false, false, true, kPPFused, kFormThread)
    // the split (no diagnostics): the particle-particle part alone, then the rest
    if (pp_mode == kPPOnly) last = false;  // writes pp only
    XPBD_SOLVE(false, true, false, kPPOnly, kFormThread)
    XPBD_SOLVE(false, false, false, kPPOnly, kFormThread)
    XPBD_SOLVE(false, true, false, kPPOnly, kFormWarp)
    XPBD_SOLVE(false, false, false, kPPOnly, kFormWarp)
    XPBD_SOLVE(false, true, false, kPPOnly, kFormStaged)
    XPBD_SOLVE(false, false, false, kPPOnly, kFormStaged)
    XPBD_SOLVE(false, true, false, kPPOnly, kFormParticleWarp)
    XPBD_SOLVE(false, false, false, kPPOnly, kFormParticleWarp)
    XPBD_SOLVE(true, true, false, kPPApply, kFormThread)
    XPBD_SOLVE(true, false, false, kPPApply, kFormThread)
    XPBD_SOLVE(false, true, false, kPPApply, kFormThread)
    XPBD_SOLVE(false, false, false, kPPApply, kFormThread)
#undef XPBD_SOLVE
    throw std::runtime_error("no solve kernel for these options");
}

}  // namespace xpbd
