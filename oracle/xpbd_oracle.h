/*
 * CPU oracle for the XPBD particle substep — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's compute shaders, executed in the
 * dispatch order of XpbdSolver::step (src/scene.cpp:805-992). Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product (libxpbd_gb300.so) never links or calls it.
 *
 * Parity status: the shader math is restated from source because the
 * reference's shaders cannot run here (no Vulkan). The BVH builder is pinned
 * against the reference's own mesh_lbvh.h/mesh_bvh.h compiled in place
 * (oracle/_ref); the shader arithmetic is "parity unpinned" against a live
 * reference run (none exists) and is pinned only by this restatement.
 *
 * Canonical orders (the reference's float atomics make these nondeterministic):
 *   - contact slots: plane block (ascending particle) then mesh block
 *     (ascending particle, then mesh index) — the order a serialised
 *     atomicAdd counter would give (generate_plane_contacts.comp:40,
 *     generate_mesh_contacts.comp:398);
 *   - particle deltas: 0 + shape deltas in ascending slot order, then the
 *     particle-particle total (solve_particle_shape_contacts.comp:189-191,
 *     solve_particle_particle_contacts.comp:213-217, scene.cpp:946-952);
 *   - restitution: every contact reads the pre-restitution velocity and the
 *     velocity increments are added in ascending slot order
 *     (apply_particle_shape_restitution.comp:259,312-314).
 *
 * Build: see oracle/Makefile. Compiled with -ffp-contract=off so that every
 * fused multiply-add is the explicit fmaf() of the shader source.
 * With -DOR_F64 the same source builds the FP64 twin used for drift checks.
 */
#pragma once
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors vkx::SolverConfig (src/scene.h:14-41), numeric fields only. */
typedef struct or_config {
    float dt;
    int32_t substeps;
    int32_t iterations;
    float particle_v_max;
    float soft_contact_mu;
    float shape_material_mu;
    float soft_contact_relaxation;
    float particle_adhesion;
    float particle_mu;
    float particle_cohesion;
    float particle_max_radius;
    float search_radius;
    float soft_contact_margin;
    int32_t enable_restitution;
    float soft_contact_restitution;
    int32_t has_ground_plane;
    float ground_plane_altitude;
    float gravity[3];
} or_config;

typedef struct or_solver or_solver;

/* 1 for the FP32 build, 2 for the FP64 twin. */
int or_precision(void);
/* OpenMP thread count used by the per-particle loops (<=0: library default). */
void or_set_threads(int n);
int or_get_threads(void);

or_solver* or_create(const or_config* cfg, int64_t num_particles, int64_t max_contacts);
void or_destroy(or_solver* s);

int or_add_mesh(or_solver* s, const float* verts, int64_t num_verts, const uint32_t* tris,
                int64_t num_tris, float shape_margin, const float* rot_xyzw, int watertight_override);
int or_finalize_meshes(or_solver* s);
int or_update_mesh(or_solver* s, int64_t mesh_index, const float* verts, int64_t num_verts,
                   const float* vels);
int or_set_particles(or_solver* s, const float* q, const float* qd, const float* inv_mass,
                     const float* radii, const int32_t* flags, int64_t n);
/* Rigid bodies (an extension: the reference's body table is static,
 * scene.cpp:220-238). Body b belongs to mesh b (shape b + 1). q: 8 floats/body
 * (pos xyz, pad, quat xyzw); qd: 8 floats/body (lin xyz, pad, ang xyz, pad);
 * com: 3/body; inertia and inv_inertia: 9/body (symmetric, so the row-major read
 * of solve_particle_shape_contacts.comp:46-48 and the column-major reads of
 * integrate_bodies.comp:51-54, apply_body_deltas.comp:53-55 agree); inv_m and
 * flags: 1/body. Any pointer may be NULL to keep the current values. A body with
 * inv_m > 0 is dynamic: its mesh's vertices are in the body frame, and every
 * substep integrates it and applies particle and rigid contact deltas to it. */
int or_set_bodies(or_solver* s, const float* q, const float* qd, const float* com, const float* inertia,
                  const float* inv_inertia, const float* inv_m, const int32_t* flags, int64_t n_bodies);
void or_get_bodies(const or_solver* s, float* q, float* qd);
typedef struct or_body_params {
    float angular_damping;            /* integrate_bodies.comp push constant */
    float rigid_contact_margin;       /* vertex-vs-shape contact generation distance */
    float rigid_contact_relaxation;   /* solve_body_contact_positions.comp push constant */
    int32_t rigid_contact_con_weighting; /* apply_body_deltas.comp use_constraint_weights */
    float rigid_mu_torsional;
    float rigid_mu_rolling;
    int32_t particle_contact_con_weighting; /* average the particle-contact body deltas per body */
} or_body_params;
void or_set_body_params(or_solver* s, const or_body_params* p);
int64_t or_rigid_contact_overflows(const or_solver* s);

int or_step(or_solver* s, float dt, int substeps, int iterations);
int or_collide_only(or_solver* s);
int or_step_solve_only(or_solver* s, float dt, int substeps, int iterations);
int or_set_contact_data(or_solver* s, const int32_t* particles, const int32_t* shapes,
                        const float* body_positions, const float* normals, int64_t count);

void or_get_positions(const or_solver* s, float* out_xyz);
void or_get_velocities(const or_solver* s, float* out_xyz);
void or_get_state64(const or_solver* s, double* x_out, double* v_out);

/* Differentiable rollout (extension; no reference counterpart). or_rollout steps
 * `frames` frames like or_step and keeps the state at the start of every substep;
 * or_rollout_backward runs the adjoint of those substeps for the gradient of a loss
 * with respect to the final positions / velocities (gx_final, gv_final; 3n each,
 * gv_final may be NULL) and returns, in double precision, the gradients with respect
 * to the initial positions and velocities (3n each), the inverse masses (n) and
 * params[4] = {soft_contact_mu, shape_material_mu, particle_mu,
 * soft_contact_restitution}. Supported: ground plane and particle-particle contacts,
 * no meshes, every particle active, equal radii, one solver iteration, the v_max
 * clamp inactive (returns -2 when a clamp fired). Contact sets and the branches of the
 * friction max() are taken as fixed at their forward values. */
int or_rollout(or_solver* s, float dt, int substeps, int iterations, int frames);
int or_rollout_backward(or_solver* s, const float* gx_final, const float* gv_final, double* gx0, double* gv0,
                        double* gw, double* params);
int64_t or_contact_count(const or_solver* s);      /* clamped to contact_max */
int64_t or_contact_count_raw(const or_solver* s);  /* unclamped counter value */
void or_get_contacts(const or_solver* s, int32_t* particles, int32_t* shapes, float* body_pos,
                     float* body_vel, float* normals);
void or_get_sorted(const or_solver* s, uint32_t* cells, uint32_t* ids);
void or_get_cell_starts(const or_solver* s, int32_t* out); /* 128^3 entries */
void or_get_cell_ends(const or_solver* s, int32_t* out);
void or_get_deltas(const or_solver* s, float* out_xyz);
/* Packed node arrays of mesh `mesh_index` as built (before global rebasing):
 * n_nodes*4 floats each, .w carries the packed uint32 (src/scene.cpp:1416-1436). */
int64_t or_mesh_bvh_node_count(const or_solver* s, int64_t mesh_index);
void or_get_mesh_bvh(const or_solver* s, int64_t mesh_index, float* lowers, float* uppers);
int or_mesh_is_watertight_flag(const or_solver* s, int64_t mesh_index);
float or_mesh_avg_edge(const or_solver* s, int64_t mesh_index);

/* Stand-alone building blocks (for unit tests against the compiled reference). */
int or_bvh_build(const float* pts, int64_t num_pts, const uint32_t* tris, int64_t num_tris,
                 float* lowers, float* uppers, uint32_t* prims, uint32_t* root);
void or_bvh_refit(const float* pts, const uint32_t* tris, float* lowers, float* uppers,
                  const uint32_t* prims, uint32_t root);
int or_tris_watertight(const uint32_t* tris, int64_t num_tris, int64_t num_verts);
void or_closest_point_triangle(const float* p, const float* a, const float* b, const float* c,
                               float* cp, float* tri_normal, float* bary);
float or_acos(float x);

#ifdef __cplusplus
}
#endif
