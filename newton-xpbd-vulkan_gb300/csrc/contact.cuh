// Particle-vs-shape contact math shared by the solve kernel and the
// contact-list kernels.
#pragma once
#include "kernels.h"
#include "xmath.cuh"

namespace xpbd {

struct Contact {
    v3 bpos, nrm, bvel;
    int shape;
};

// Contact k of a particle (plane contact first, then the generic slots), in
// the canonical slot order; `keep` is false when the contact_max cap drops it.
__device__ __forceinline__ Contact load_contact(uint32_t info, int k, const float4* __restrict__ slots, v3 x_prev,
                                                float altitude) {
    Contact c;
    if ((info & kPlaneBit) && k == 0) {  // generate_plane_contacts.comp:43-53
        c.bpos = mk3(x_prev.x, x_prev.y, altitude);
        c.nrm = mk3(0.0f, 0.0f, 1.0f);
        c.bvel = mk3(0.0f, 0.0f, 0.0f);
        c.shape = 0;
        return c;
    }
    const int j = k - (int)(info & kPlaneBit);
    const float4 a = slots[j * 3 + 0], b = slots[j * 3 + 1], d = slots[j * 3 + 2];
    c.bpos = xyz(a);
    c.shape = __float_as_int(a.w);
    c.nrm = xyz(b);
    c.bvel = xyz(d);
    return c;
}

__device__ __forceinline__ void body_pose(const BodyTables& bt, int body, v3& pos, q4& rot, v3& com) {
    if (body >= 0) {
        const float4 p = bt.body_q[body * 2], q = bt.body_q[body * 2 + 1];
        pos = xyz(p);
        rot.x = q.x;
        rot.y = q.y;
        rot.z = q.z;
        rot.w = q.w;
        com = mk3(bt.body_com[body * 3], bt.body_com[body * 3 + 1], bt.body_com[body * 3 + 2]);
    } else {
        pos = mk3(0.0f, 0.0f, 0.0f);
        rot.x = rot.y = rot.z = 0.0f;
        rot.w = 1.0f;
        com = mk3(0.0f, 0.0f, 0.0f);
    }
}

// solve_particle_shape_contacts.comp:109-191 for one contact of an active
// particle. Returns false when the contact is skipped; fd is the particle delta.
__device__ __forceinline__ bool shape_delta(const Contact& ct, int pflag, v3 px, v3 pv, float radius, float w1,
                                            const BodyTables& bt, const SolveParams& sp, v3& fd, v3& delta_total_out,
                                            v3& r_out) {
    const int body = bt.shape_body[ct.shape];
    if (pflag & 2) {
        if (body < 0) return false;
        if (bt.body_flags[body] & 4) return false;
        if (bt.body_invm[body] == 0.0f) return false;
    }
    v3 X_pos, X_com;
    q4 X_rot;
    body_pose(bt, body, X_pos, X_rot, X_com);
    const v3 bx = vadd(X_pos, quat_rotate(X_rot, ct.bpos));
    const v3 r = vsub(bx, vadd(X_pos, quat_rotate(X_rot, X_com)));
    const v3 n = ct.nrm;
    const v3 d_px = vsub(px, bx);
    const float c = __fmaf_rn(n.z, d_px.z, __fmaf_rn(n.x, d_px.x, n.y * d_px.y)) - radius;
    if (c > sp.ka) return false;
    const float mu = 0.5f * (sp.soft_mu + bt.shape_mu[ct.shape]);
    v3 body_v = mk3(0.0f, 0.0f, 0.0f), body_w = body_v;
    if (body >= 0) {
        body_v = xyz(bt.body_qd[body * 2]);
        body_w = xyz(bt.body_qd[body * 2 + 1]);
    }
    const v3 bv = vadd(vadd(body_v, vcross(body_w, r)), quat_rotate(X_rot, ct.bvel));
    const v3 v = vsub(pv, bv);
    const float lambda_n = c;
    const v3 delta_n = vmuls(n, lambda_n);
    float vn = n.y * v.y;
    vn = __fmaf_rn(n.x, v.x, vn);
    vn = __fmaf_rn(n.z, v.z, vn);
    const v3 vt = mk3(__fmaf_rn(-n.x, vn, v.x), __fmaf_rn(-n.y, vn, v.y), __fmaf_rn(-n.z, vn, v.z));
    float w2 = 0.0f;
    if (body >= 0) {
        const v3 ra = quat_rotate_inv(X_rot, vcross(r, n));
        const float* M = bt.body_invI + body * 9;
        const v3 Mra = mk3((M[0] * ra.x + M[1] * ra.y) + M[2] * ra.z, (M[3] * ra.x + M[4] * ra.y) + M[5] * ra.z,
                           (M[6] * ra.x + M[7] * ra.y) + M[8] * ra.z);
        w2 = bt.body_invm[body] + vdot(ra, Mra);
    }
    const float denom = w1 + w2;
    if (denom == 0.0f) return false;
    float inv_vt;
    const float vt_len = exact_length_rcp(vt, inv_vt);
    const float lambda_f = gmax(mu * lambda_n, -vt_len * sp.dt);
    const v3 vt_dir = vt_len > 0.0f ? exact_div_rcp(vt, vt_len, inv_vt) : mk3(0.0f, 0.0f, 0.0f);
    const v3 diff = mk3(__fmaf_rn(vt_dir.x, lambda_f, -delta_n.x), __fmaf_rn(vt_dir.y, lambda_f, -delta_n.y),
                        __fmaf_rn(vt_dir.z, lambda_f, -delta_n.z));
    const v3 delta_total = vmuls(exact_div(diff, denom), sp.relax);
    fd = mk3(w1 * delta_total.x, w1 * delta_total.y, w1 * delta_total.z);
    delta_total_out = delta_total;
    r_out = r;
    return true;
}

// apply_particle_shape_restitution.comp:253-315 for one contact of an active
// particle; v_new is the velocity before any restitution increment.
__device__ __forceinline__ bool restitution_dv(const Contact& ct, v3 v_new, v3 px_old, v3 v_old, float radius,
                                               const BodyTables& bt, const SolveParams& sp, v3& dv) {
    const int body = bt.shape_body[ct.shape];
    v3 X_pos, X_com;
    q4 X_rot;
    body_pose(bt, body, X_pos, X_rot, X_com);
    const v3 bx = vadd(X_pos, quat_rotate(X_rot, ct.bpos));
    const v3 n = ct.nrm;
    const v3 d_px = vsub(px_old, bx);
    const float c = __fmaf_rn(n.z, d_px.z, __fmaf_rn(n.x, d_px.x, n.y * d_px.y)) - radius;
    if (c > sp.ka) return false;
    v3 X_pos_prev = X_pos;
    q4 X_rot_prev = X_rot;
    if (body >= 0) {
        const float4 pp = bt.body_q_prev[body * 2], pq = bt.body_q_prev[body * 2 + 1];
        X_pos_prev = xyz(pp);
        X_rot_prev.x = pq.x;
        X_rot_prev.y = pq.y;
        X_rot_prev.z = pq.z;
        X_rot_prev.w = pq.w;
    }
    const v3 bx_prev = vadd(X_pos_prev, quat_rotate(X_rot_prev, ct.bpos));
    const v3 r = vsub(bx_prev, vadd(X_pos_prev, quat_rotate(X_rot_prev, X_com)));
    const v3 bv_contact = quat_rotate(X_rot_prev, ct.bvel);
    v3 bv_old = bv_contact, bv_new = bv_contact;
    if (body >= 0) {
        const v3 bvo = xyz(bt.body_qd_prev[body * 2]), bwo = xyz(bt.body_qd_prev[body * 2 + 1]);
        const v3 bvn = xyz(bt.body_qd[body * 2]), bwn = xyz(bt.body_qd[body * 2 + 1]);
        bv_old = vadd(vadd(bvo, vcross(bwo, r)), bv_contact);
        bv_new = vadd(vadd(bvn, vcross(bwn, r)), bv_contact);
    }
    const v3 vdo = vsub(v_old, bv_old);
    const float rel_old = __fmaf_rn(n.z, vdo.z, __fmaf_rn(n.y, vdo.y, n.x * vdo.x));
    const v3 vdn = vsub(v_new, bv_new);
    const float rel_new = __fmaf_rn(n.z, vdn.z, __fmaf_rn(n.x, vdn.x, n.y * vdn.y));
    if (!(rel_old < 0.0f)) return false;
    const float rt = gmax((-sp.restitution) * rel_old, 0.0f);
    const float scalar = (-rel_new) + rt;
    dv = mk3(n.x * scalar, n.y * scalar, n.z * scalar);
    return true;
}

__device__ __forceinline__ bool contact_kept(uint32_t info, int k, const ContactRanks& cr, uint32_t id,
                                             int64_t contact_max) {
    if (!cr.rank) return true;
    if (cr.count && (int64_t)*cr.count <= contact_max) return true;  // nothing over the cap
    const uint2 rk = cr.rank[id];
    if ((info & kPlaneBit) && k == 0) return (int64_t)rk.x < contact_max;
    const int j = k - (int)(info & kPlaneBit);
    return (int64_t)cr.totals[0] + (int64_t)rk.y + j < contact_max;
}

}  // namespace xpbd
