// Closest-point query of one point against one triangle mesh's BVH
// (generate_mesh_contacts.comp:197-411), shared by the particle contact
// kernels and the rigid contact kernel.
#pragma once
#include "kernels.h"
#include "xmath.cuh"

namespace xpbd {

__device__ __forceinline__ float dist_sq_aabb(v3 p, v3 lo, v3 hi) {  // generate_mesh_contacts.comp:32-35
    const v3 d = mk3(gmax(gmax(lo.x - p.x, 0.0f), p.x - hi.x), gmax(gmax(lo.y - p.y, 0.0f), p.y - hi.y),
                     gmax(gmax(lo.z - p.z, 0.0f), p.z - hi.z));
    return vdot(d, d);
}

__device__ __forceinline__ float comp(v3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// True when p (in mesh ci's frame) lies in a clear cell of the mesh's reach grid or
// outside it, or is not finite: then no leaf box is within the traversal's initial
// bound (margin + shape margin + radius + eps) and the query ends without testing
// a triangle, i.e. without a contact (the bound only shrinks once a triangle is
// tested, and a node's box distance never exceeds its descendants').
__device__ __forceinline__ bool mesh_far(const MeshTables& mt, int ci, v3 p) {
    if (!mt.cull_bits) return false;
    const int4 d = __ldg(&mt.cull_dim[ci]);
    if (d.x == 0) return false;
    const float4 o = __ldg(&mt.cull_org[ci]);
    const float fx = (p.x - o.x) * o.w, fy = (p.y - o.y) * o.w, fz = (p.z - o.z) * o.w;
    if (!(fx >= 0.0f && fx < (float)d.x && fy >= 0.0f && fy < (float)d.y && fz >= 0.0f && fz < (float)d.z))
        return true;
    const int ix = min((int)fx, d.x - 1), iy = min((int)fy, d.y - 1), iz = min((int)fz, d.z - 1);
    const uint32_t nwx = ((uint32_t)d.x + 31u) >> 5;
    const uint32_t word = __ldg(&mt.cull_off[ci]) + ((uint32_t)iz * (uint32_t)d.y + (uint32_t)iy) * nwx + ((uint32_t)ix >> 5);
    return ((__ldg(&mt.cull_bits[word]) >> (ix & 31)) & 1u) == 0u;
}

// generate_mesh_contacts.comp:77-113, split into the part that depends on the ray
// only (axis order and shear constants, computed once per ray) and the per-triangle
// test; the operations and their order are the shader's.
struct WoopRay {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__device__ __forceinline__ WoopRay woop_setup(v3 dir) {
    const v3 adir = mk3(fabsf(dir.x), fabsf(dir.y), fabsf(dir.z));
    WoopRay r;
    int kz = 0;
    if (adir.y > adir.x) kz = 1;
    if (adir.z > (kz == 1 ? adir.y : adir.x)) kz = 2;
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    if (comp(dir, kz) < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = __fdiv_rn(comp(dir, kx), comp(dir, kz));
    r.Sy = __fdiv_rn(comp(dir, ky), comp(dir, kz));
    r.Sz = __fdiv_rn(1.0f, comp(dir, kz));
    return r;
}

__device__ __forceinline__ bool woop_hit(const WoopRay& r, v3 p, v3 a, v3 b, v3 c) {
    const v3 A = vsub(a, p), B = vsub(b, p), C = vsub(c, p);
    const float Ax = comp(A, r.kx) - r.Sx * comp(A, r.kz), Ay = comp(A, r.ky) - r.Sy * comp(A, r.kz);
    const float Bx = comp(B, r.kx) - r.Sx * comp(B, r.kz), By = comp(B, r.ky) - r.Sy * comp(B, r.kz);
    const float Cx = comp(C, r.kx) - r.Sx * comp(C, r.kz), Cy = comp(C, r.ky) - r.Sy * comp(C, r.kz);
    const float U = diff_product(Cx, By, Cy, Bx);
    const float V = diff_product(Ax, Cy, Ay, Cx);
    const float W = diff_product(Bx, Ay, By, Ax);
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * comp(A, r.kz), Bz = r.Sz * comp(B, r.kz), Cz = r.Sz * comp(C, r.kz);
    const float T = U * Az + V * Bz + W * Cz;
    if ((T < 0.0f && det > 0.0f) || (T > 0.0f && det < 0.0f)) return false;
    return true;
}

// generate_mesh_contacts.comp:115-179; the triangle normal normalize(cross(b-a, c-a)) depends on
// the triangle only and is read from the triangle cache instead of being recomputed per visit
static __device__ void closest_point_triangle(v3 p, v3 a, v3 b, v3 c, v3& cp, v3& bary) {
    const v3 ab = vsub(b, a), ac = vsub(c, a), ap = vsub(p, a);
    float u, v;
    const float d1 = exact_dot(ab, ap), d2 = exact_dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) {
        v = 0.0f;
        u = 1.0f;
    } else {
        const v3 bp = vsub(p, b);
        const float d3 = exact_dot(ab, bp), d4 = exact_dot(ac, bp);
        if (d3 >= 0.0f && d4 <= d3) {
            v = 1.0f;
            u = 0.0f;
        } else {
            const float vc = __fmaf_rn(d1, d4, -(d2 * d3));
            if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
                v = exact_div1(d1, d1 - d3);
                u = 1.0f - v;
            } else {
                const v3 cp_p = vsub(p, c);
                const float d5 = exact_dot(ab, cp_p), d6 = exact_dot(ac, cp_p);
                if (d6 >= 0.0f && d5 <= d6) {
                    v = 0.0f;
                    u = 0.0f;
                } else {
                    const float vb = __fmaf_rn(d5, d2, -(d1 * d6));
                    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
                        const float w_val = exact_div1(d2, d2 - d6);
                        v = 0.0f;
                        u = 1.0f - w_val;
                    } else {
                        const float va = __fmaf_rn(d3, d6, -(d5 * d4));
                        if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
                            const float w_val = exact_div1(d4 - d3, (d4 - d3) + (d5 - d6));
                            v = 1.0f - w_val;
                            u = (1.0f - v) - w_val;
                        } else {
                            const float sum_vavb = va + vb;
                            const float sum_all = vc + sum_vavb;
                            const float r0 = __frcp_rn(sum_all);
                            const float rem = __fmaf_rn(-sum_all, r0, 1.0f);
                            const float denom = __fmaf_rn(rem, r0, r0);
                            v = vb * denom;
                            u = __fmaf_rn(-vc, denom, 1.0f - v);
                        }
                    }
                }
            }
        }
    }
    const float w_out = (1.0f - u) - v;
    bary = mk3(u, v, w_out);
    cp = vadd(vadd(vmuls(a, u), vmuls(b, v)), vmuls(c, w_out));
}

__device__ __forceinline__ v3 ldv(const float* __restrict__ p, uint32_t i) {
    return mk3(__ldg(p + i * 3), __ldg(p + i * 3 + 1), __ldg(p + i * 3 + 2));
}

// Traversal stack of one thread (32 entries, local memory). An entry keeps, besides
// the node, the squared box distance and the packed child words read when its parent
// ordered its children, so a pop needs no load.
struct LocalStack {
    float nds[32];
    uint32_t lw[32], uw[32];
    __device__ __forceinline__ void put(uint32_t k, float d, uint32_t l, uint32_t u) {
        nds[k] = d;
        lw[k] = l;
        uw[k] = u;
    }
    __device__ __forceinline__ float dist(uint32_t k) const { return nds[k]; }
    __device__ __forceinline__ void words(uint32_t k, uint32_t& l, uint32_t& u) const {
        l = lw[k];
        u = uw[k];
    }
};

// Traversal state of one particle against one mesh (generate_mesh_contacts.comp:201-331).
template <class Stack>
struct MeshWalk {
    Stack stk;
    uint32_t sp;
    float min_dist, min_dist_sq, max_dist;
    v3 acc;
    uint32_t min_face;
    float sv_v, sv_w;
    bool found, wt, overflow;
};

template <class W>
__device__ __forceinline__ void walk_push(W& w, float nds, float4 lo4, float4 hi4) {
    if (w.sp < 32) {
        w.stk.put(w.sp, nds, __float_as_uint(lo4.w), __float_as_uint(hi4.w));
        w.sp++;
    } else {
        w.overflow = true;
    }
}

template <class W>
__device__ __forceinline__ void walk_begin(W& w, const MeshTables& mt, int ci, float radius, v3 p) {
    w.max_dist = mt.soft_margin + __ldg(&mt.margins[ci]) + radius;
    w.sp = 0;
    const uint32_t root = __ldg(&mt.roots[ci]);
    const float4 lo4 = __ldg(&mt.nl[root]), hi4 = __ldg(&mt.nu[root]);
    walk_push(w, dist_sq_aabb(p, xyz(lo4), xyz(hi4)), lo4, hi4);
    w.min_dist = w.max_dist;
    w.acc = mk3(0.0f, 0.0f, 0.0f);
    w.min_face = 0;
    w.sv_v = 0.0f;
    w.sv_w = 0.0f;
    w.found = false;
    w.wt = __ldg(&mt.watertight[ci]) != 0;
    w.min_dist_sq = w.max_dist * w.max_dist;
}

// Pops one stack entry (:221-235, :315-330). Returns 0 when the entry is pruned by
// the current distance bound, 1 for a leaf (its primitive range in a, b) and 2 for
// an inner node (its children in a, b, whose boxes walk_children then takes).
template <class W>
__device__ __forceinline__ int walk_pop_entry(W& w, float eps_md, uint32_t& a, uint32_t& b) {
    --w.sp;
    const float nds = w.stk.dist(w.sp);
    if (w.wt) {
        if (nds > w.min_dist_sq) return 0;
    } else {
        if (nds > (w.min_dist + eps_md) * (w.min_dist + eps_md)) return 0;
    }
    uint32_t lpk, upk;
    w.stk.words(w.sp, lpk, upk);
    a = lpk & 0x3FFFFFFFu;
    b = upk & 0x3FFFFFFFu;
    return ((lpk >> 30) & 3u) ? 1 : 2;
}

// Orders and pushes the children of the inner node just popped (:316-330).
template <class W>
__device__ __forceinline__ void walk_children(W& w, v3 p, float eps_md, float4 llo, float4 lhi, float4 rlo,
                                              float4 rhi) {
    const float lds = dist_sq_aabb(p, xyz(llo), xyz(lhi)), rds = dist_sq_aabb(p, xyz(rlo), xyz(rhi));
    const float thresh = w.wt ? w.min_dist_sq : ((w.min_dist + eps_md) * (w.min_dist + eps_md));
    // the shader's 32-entry stack has no bound check; a push past it is dropped here
    // and reported through the status word
    if (lds < rds) {
        if (rds < thresh) walk_push(w, rds, rlo, rhi);
        if (lds < thresh) walk_push(w, lds, llo, lhi);
    } else {
        if (lds < thresh) walk_push(w, lds, llo, lhi);
        if (rds < thresh) walk_push(w, rds, rlo, rhi);
    }
}

// Pops one node. Returns true when it is a leaf that passed the distance test; its
// primitive range is returned for evaluation before the next pop.
template <class W>
__device__ __forceinline__ bool walk_pop(W& w, const MeshTables& mt, v3 p, float eps_md, uint32_t& lo,
                                         uint32_t& hi) {
    uint32_t a, b;
    const int r = walk_pop_entry(w, eps_md, a, b);
    if (r == 1) {
        lo = a;
        hi = b;
        return true;
    }
    if (r == 2) {
        const float4* rec = mt.pair + (size_t)a * 4;  // nl[a], nu[a], nl[b], nu[b]
        walk_children(w, p, eps_md, __ldg(rec), __ldg(rec + 1), __ldg(rec + 2), __ldg(rec + 3));
    }
    return false;
}

// Test of one triangle against p (:239-313), the part that does not depend on the
// traversal state: closest point, its distance (squared for watertight meshes) and,
// for open meshes when the distance is below `below`, the angle weight of the
// triangle normal at the closest point.
struct TriHit {
    float d;       // squared distance (watertight) or exact_length distance (open)
    float v, w;    // barycentric v, w of the closest point
    float weight;  // normal weight (open meshes, when d < below)
    v3 tn;         // unit normal
    uint32_t t;    // triangle
};

// From the triangle's four cache words (a, tri id), (b, |e0|^2), (c, |e1|^2),
// (unit normal, |e2|^2); degenerate triangles (:250-251) are skipped by the caller
// (normal word w < 0).
__device__ __forceinline__ TriHit tri_hit(bool wt, v3 p, float eps2, float below, float4 qa, float4 qb, float4 qc,
                                          float4 qn) {
    const float PI_ = 3.14159265359f;
    TriHit h;
    h.t = __float_as_uint(qa.w);
    const v3 a = xyz(qa), b = xyz(qb), c = xyz(qc);
    h.tn = xyz(qn);
    v3 cp, tb;
    closest_point_triangle(p, a, b, c, cp, tb);
    h.v = tb.y;
    h.w = tb.z;
    h.weight = 0.0f;
    if (wt) {
        const v3 diff = vsub(cp, p);
        h.d = vdot(diff, diff);
    } else {
        // exact_length's squared sum; a triangle whose distance provably reaches `below`
        // (1.5e-5 relative margin, far above the rounding of the test) cannot change the
        // traversal state, which acts only on d < below, and skips the refined root
        const v3 dd = vsub(cp, p);
        const float sq = __fmaf_rn(dd.z, dd.z, __fmaf_rn(dd.x, dd.x, dd.y * dd.y));
        const float lim = below * 1.0000153f;
        if (sq > lim * lim) {
            h.d = __int_as_float(0x7f800000);  // +inf
            return h;
        }
        h.d = exact_sqrt(sq);
        if (h.d < below) {
            const v3 e0 = vsub(b, a), e1 = vsub(c, a), e2 = vsub(c, b);
            const float e0n = qb.w, e1n = qc.w, e2n = qn.w;
            const v3 cp_p = vsub(cp, a), cq_p = vsub(cp, b), cr_p = vsub(cp, c);
            const float lcp = vdot(cp_p, cp_p), lcq = vdot(cq_p, cq_p), lcr = vdot(cr_p, cr_p);
            if (lcp < eps2) {
                h.weight = series_acos(gclamp(vdot(vnormalize(e0), vnormalize(e1)), -1.0f, 1.0f));
            } else if (lcq < eps2) {
                h.weight = series_acos(gclamp(vdot(vnormalize(e2), vnormalize(vneg(e0))), -1.0f, 1.0f));
            } else if (lcr < eps2) {
                h.weight = series_acos(gclamp(vdot(vnormalize(vneg(e1)), vnormalize(vneg(e2))), -1.0f, 1.0f));
            } else {
                const float e0cp = vdot(e0, cp_p), e2cq = vdot(e2, cq_p), e1cp = vdot(e1, cp_p);
                if ((lcp * e0n - e0cp * e0cp < eps2 * e0n) || (lcq * e2n - e2cq * e2cq < eps2 * e2n) ||
                    (lcp * e1n - e1cp * e1cp < eps2 * e1n))
                    h.weight = PI_;
                else
                    h.weight = 2.0f * PI_;
            }
        }
    }
    return h;
}

// The traversal state update of one tested triangle (:257-313), in test order.
template <class W>
__device__ __forceinline__ void walk_apply(W& w, const TriHit& h, float eps_md) {
    if (w.wt) {
        if (h.d < w.min_dist_sq) {
            w.min_dist_sq = h.d;
            w.min_face = h.t;
            w.sv_v = h.v;
            w.sv_w = h.w;
            w.found = true;
        }
    } else if (h.d < w.min_dist + eps_md) {
        if (h.d > w.min_dist - eps_md) {
            w.acc = vadd(w.acc, vmuls(h.tn, h.weight));
            if (h.d < w.min_dist) {
                w.min_dist = h.d;
                w.min_face = h.t;
                w.sv_v = h.v;
                w.sv_w = h.w;
            }
        } else {
            w.min_dist = h.d;
            w.min_face = h.t;
            w.sv_v = h.v;
            w.sv_w = h.w;
            w.acc = vmuls(h.tn, h.weight);
        }
        w.found = true;
    }
}

// One triangle of a leaf tested and applied by one thread.
template <class W>
__device__ __forceinline__ void walk_tri(W& w, v3 p, float eps_md, float eps2, float4 qa, float4 qb, float4 qc,
                                         float4 qn) {
    walk_apply(w, tri_hit(w.wt, p, eps2, w.min_dist + eps_md, qa, qb, qc, qn), eps_md);
}

// Evaluates the triangles of one leaf (:237-314).
template <class W>
__device__ __forceinline__ void walk_leaf(W& w, const MeshTables& mt, v3 p, float eps_md, float eps2,
                                          uint32_t lo, uint32_t hi) {
    for (uint32_t pc = lo; pc < hi; pc++) {
        const float4 qn = __ldg(&mt.tri_cache[pc * 4 + 3]);
        if (qn.w < 0.0f) continue;  // degenerate: |cross|/(|e0|^2+|e1|^2+|e2|^2) < 1e-6 (:250-251)
        walk_tri(w, p, eps_md, eps2, __ldg(&mt.tri_cache[pc * 4]), __ldg(&mt.tri_cache[pc * 4 + 1]),
                 __ldg(&mt.tri_cache[pc * 4 + 2]), qn);
    }
}

// Contact emission after the traversal of mesh ci (:333-411).
template <class W>
__device__ __forceinline__ bool walk_finish(W& w, const MeshTables& mt, int ci, v3 p, v3& body_pos,
                                            v3& shape_v, v3& nrm) {
    if (w.wt) w.min_dist = exact_sqrt(w.min_dist_sq);
    if (!(w.found && w.min_dist < w.max_dist)) return false;
    const float u_mesh = (1.0f - w.sv_v) - w.sv_w;
    const float v_mesh = w.sv_v;
    const uint32_t i0 = __ldg(&mt.tris[w.min_face * 3]), i1 = __ldg(&mt.tris[w.min_face * 3 + 1]),
                   i2 = __ldg(&mt.tris[w.min_face * 3 + 2]);
    const v3 v0 = ldv(mt.verts, i0), v1 = ldv(mt.verts, i1), v2 = ldv(mt.verts, i2);
    const float w_eval = (1.0f - u_mesh) - v_mesh;
    const v3 shape_p = vfma_vs(v2, w_eval, vfma_vs(v0, u_mesh, vmuls(v1, v_mesh)));
    const v3 vel0 = ldv(mt.vels, i0), vel1 = ldv(mt.vels, i1), vel2 = ldv(mt.vels, i2);
    shape_v = vfma_vs(vel2, w_eval, vfma_vs(vel0, u_mesh, vmuls(vel1, v_mesh)));
    float sign;
    if (w.wt) {
        const WoopRay ray = woop_setup(mk3(1.029700994f, 1.086472273f, 1.034694910f));
        uint32_t hits = 0;
        const uint32_t po = __ldg(&mt.prim_off[ci]), pn = __ldg(&mt.prim_cnt[ci]);
        for (uint32_t ti = 0; ti < pn; ti++) {
            const float4* q = mt.tri_cache + (size_t)(po + ti) * 4;
            if (woop_hit(ray, p, xyz(__ldg(q)), xyz(__ldg(q + 1)), xyz(__ldg(q + 2)))) hits++;
        }
        sign = (hits & 1u) ? -1.0f : 1.0f;
    } else {
        sign = vdot(w.acc, vsub(p, shape_p)) > 0.0f ? 1.0f : -1.0f;
    }
    const v3 delta = vsub(p, shape_p);
    float inv_len;
    const float delta_len = exact_length_rcp(delta, inv_len);
    nrm = delta_len > 0.0f ? vmuls(exact_div_rcp(delta, delta_len, inv_len), sign) : mk3(0.0f, 0.0f, 1.0f);
    const float d = delta_len * sign;
    body_pos = vfma_vs(vneg(nrm), d, p);
    return true;
}

// Whole query of point p (in the mesh's own frame) against mesh ci by one thread.
__device__ __forceinline__ bool mesh_query(const MeshTables& mt, int ci, float radius, v3 p, v3& body_pos,
                                           v3& shape_v, v3& nrm, bool& overflow) {
    const float eps_md = mt.avg_edge * 1e-3f;
    const float eps2 = eps_md * eps_md;
    MeshWalk<LocalStack> w;
    w.overflow = false;
    walk_begin(w, mt, ci, radius, p);
    while (w.sp > 0) {
        uint32_t lo, hi;
        if (walk_pop(w, mt, p, eps_md, lo, hi)) walk_leaf(w, mt, p, eps_md, eps2, lo, hi);
    }
    overflow |= w.overflow;
    return walk_finish(w, mt, ci, p, body_pos, shape_v, nrm);
}

}  // namespace xpbd
