/*
 * C ABI of libxpbd_gb300.so — a GB300 (sm_103a) XPBD particle substep that is
 * a drop-in for the reference's `vkxpbd` module (src/bindings.cpp:8-300 over
 * vkx::XpbdSolver, src/scene.h:74-135).
 *
 * Plain C types only: host pointers and sizes in, host buffers out. Every
 * function returns 0 on success and a negative value on failure; the message
 * of the last failure on the calling thread is returned by xpbd_last_error().
 * The error strings of the reference are kept ("XpbdSolver not initialized",
 * "Particle count mismatch", ...). A solver is not thread-safe (neither is the
 * reference's, src/context.h:31); calls block until the GPU work they start
 * has finished, like the reference's fence waits (src/scene.cpp:1003).
 */
#ifndef XPBD_GB300_H
#define XPBD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XPBD_ABI_VERSION 1
#define XPBD_NUM_CELLS (128 * 128 * 128) /* hash grid size, src/scene.cpp:17-18 */

typedef struct xpbd_solver xpbd_solver;

/* vkx::SolverConfig (src/scene.h:14-41), field for field; defaults from
 * xpbd_config_default(). shader_dir, compat_mode and enable_validation are
 * accepted and ignored (there are no shaders and no Vulkan layers). */
typedef struct xpbd_config {
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
    char shader_dir[256];
    int32_t device_index;
    int32_t compat_mode;
    int32_t enable_validation;
    int32_t enable_diagnostics;
    int32_t enable_profile;
    uint32_t max_diag_pairs;
    int32_t substep_batch_size;
} xpbd_config;

/* vkx::GPUPairRecord (src/scene.h:43-64). */
typedef struct xpbd_pair_record {
    uint32_t i, j;
    float dist, err;
    float normal[3];
    float vrel[3];
    float vn, vt_len, denom, lambda_n, lambda_f;
    float delta_i[3];
    uint32_t iter_index, pad0;
} xpbd_pair_record;

/* ---- library ------------------------------------------------------------ */
const char* xpbd_last_error(void);
int xpbd_abi_version(void);
void xpbd_config_default(xpbd_config* cfg);                  /* SolverConfig() */
int xpbd_device_count(int* count);                           /* enumerate_devices, bindings.cpp:48 */
int xpbd_device_name(int index, char* buf, size_t cap);

/* ---- scene build (src/scene.h:79-92) -------------------------------------- */
int xpbd_create(xpbd_solver** out);                          /* XpbdSolver() */
int xpbd_destroy(xpbd_solver* s);
int xpbd_init(xpbd_solver* s, const xpbd_config* cfg, size_t num_particles,
              size_t max_contacts);                          /* init, scene.cpp:65-152 */
/* shape_rot_xyzw may be NULL (identity); watertight_override -1 = auto-detect,
 * 0/1 = forced (scene.cpp:154-202). */
int xpbd_add_mesh(xpbd_solver* s, const float* verts, size_t num_verts, const uint32_t* tris,
                  size_t num_tris, float shape_margin, const float* shape_rot_xyzw,
                  int watertight_override);
int xpbd_finalize_meshes(xpbd_solver* s);                    /* scene.cpp:204-390 */
/* q: n*3 floats; qd, inv_mass, radii, flags may be NULL (scene.cpp:592-615). */
int xpbd_set_particles(xpbd_solver* s, const float* q, const float* qd, const float* inv_mass,
                       const float* radii, const int32_t* flags, size_t n);
/* vels may be NULL (zero velocity), scene.cpp:617-696. */
int xpbd_update_mesh(xpbd_solver* s, size_t mesh_index, const float* verts, size_t num_verts,
                     const float* vels);

/* ---- stepping ------------------------------------------------------------- */
int xpbd_step(xpbd_solver* s, float dt, int substeps, int iterations); /* scene.cpp:698-1092 */
int xpbd_collide_only(xpbd_solver* s);                                  /* scene.cpp:1229-1245 */
int xpbd_step_solve_only(xpbd_solver* s, float dt, int substeps, int iterations); /* :1094-1227 */

/* ---- readback (scene.cpp:1247-1436) ---------------------------------------- */
int xpbd_get_positions(xpbd_solver* s, float* out_xyz, size_t n);
int xpbd_get_velocities(xpbd_solver* s, float* out_xyz, size_t n);
size_t xpbd_particle_count(const xpbd_solver* s);
size_t xpbd_mesh_count(const xpbd_solver* s);
int xpbd_last_contact_count(const xpbd_solver* s);
/* Contacts of the last collision pass in canonical order (plane contacts by
 * particle, then mesh contacts by particle and mesh); each array holds at least
 * xpbd_last_contact_count() entries (x3 floats for the vector arrays); any
 * pointer may be NULL. */
int xpbd_get_contacts(xpbd_solver* s, int32_t* particles, int32_t* shapes, float* normals,
                      float* body_positions, float* body_velocities);
int xpbd_set_contact_data(xpbd_solver* s, const int32_t* particles, const int32_t* shapes,
                          const float* body_positions, const float* normals, int contact_count);
int xpbd_get_sorted_cells(xpbd_solver* s, uint32_t* out, size_t n);
int xpbd_get_sorted_point_ids(xpbd_solver* s, uint32_t* out, size_t n);
int xpbd_get_cell_starts(xpbd_solver* s, int32_t* out, size_t n); /* n = XPBD_NUM_CELLS */
int xpbd_get_cell_ends(xpbd_solver* s, int32_t* out, size_t n);
/* Deltas of the last solver iteration (recorded while enable_diagnostics is set). */
int xpbd_get_deltas(xpbd_solver* s, float* out_xyz, size_t n);
/* Node halves of mesh `mesh_index` as built: 4 floats per node, .w = packed
 * uint32 bits. Call with NULL buffers to get the node count. */
int xpbd_get_mesh_bvh(xpbd_solver* s, size_t mesh_index, float* lowers, float* uppers,
                      size_t cap_nodes, size_t* num_nodes);

/* ---- diagnostics (bindings.cpp:239-287) ------------------------------------ */
int xpbd_get_diag_pair_count(xpbd_solver* s, uint32_t* out);
int xpbd_get_diag_overflow_count(xpbd_solver* s, uint32_t* out);
int xpbd_reset_diag_buffers(xpbd_solver* s);
int xpbd_get_diag_pairs(xpbd_solver* s, xpbd_pair_record* out, size_t cap, size_t* count);
/* which: 0 = p11_diag (u32), 1 = p11_apply_diag (u32), 2 = shape_contact_diag (f32),
 * 3 = mesh_candidate_diag (u32); 4-byte words. NULL out returns the length. */
int xpbd_get_aux_diag(xpbd_solver* s, int which, void* out, size_t cap, size_t* count);
int xpbd_print_profiler_summary(xpbd_solver* s);

/* ---- extensions (no counterpart in the reference) -------------------------- */
/* Device status bits of the last step (1 = look-back timeout, 2 = BVH stack
 * overflow, 4 = mesh contact slots full) and their counters. */
int xpbd_get_status(xpbd_solver* s, uint32_t out[4]);
/* Test hook of the sort's bounded wait (the reference's fence wait has none,
 * src/scene.cpp:1003): process-wide, in every later step's particle sort and in
 * xpbd_sort_keys_noalloc, tile `hold_tile` of the first radix pass never publishes
 * its prefix, so the look-back wait of the tile after it gives up after wait_ns
 * (0 < wait_ns <= 1e9) and the step fails with "device wait timed out" (its result
 * is discarded; every index stays in range). hold_tile < 0 restores normal
 * operation (waits bounded by 1 s). Solvers re-record their frame graphs. */
int xpbd_debug_lookback_hold(int64_t hold_tile, uint64_t wait_ns);
/* xpbd_step without the wait: the frame's graph is queued on the solver's
 * stream and the call returns. xpbd_sync (or any state call) waits, reads the
 * contact count and checks the status word. */
int xpbd_step_async(xpbd_solver* s, float dt, int substeps, int iterations);
int xpbd_sync(xpbd_solver* s);
/* The solver's cudaStream_t (as an opaque pointer) for event timing and for
 * ordering work of other libraries against the solver. */
void* xpbd_stream(xpbd_solver* s);
/* Per-kernel timing: with profiling on, frame graphs carry event-record nodes
 * around every kernel; synchronous steps accumulate device milliseconds per
 * stage. Stage names come from xpbd_stage_name. */
int xpbd_set_profiling(xpbd_solver* s, int on);
int xpbd_get_stage_times(xpbd_solver* s, double* ms, size_t cap, size_t* num_stages, uint64_t* substeps);
int xpbd_reset_stage_times(xpbd_solver* s);
const char* xpbd_stage_name(int index);
/* out = {kernel launches per frame, memset nodes per frame, frames run, cached graphs} */
int xpbd_get_frame_stats(xpbd_solver* s, uint64_t out[4]);
/* Kernels launched by all frames run so far (the frame graphs' kernel nodes, frame by
 * frame: exact also when consecutive frames replay different graphs). */
int xpbd_get_kernels_launched(xpbd_solver* s, uint64_t* total);

/* Rigid bodies — an extension: the reference's body table is static
 * (src/scene.cpp:220-238) and its body shaders (integrate_bodies.comp,
 * apply_body_deltas.comp, solve_body_contact_positions.comp) are never
 * dispatched. Body b belongs to mesh b (shape b + 1, src/scene.cpp:213). A body
 * with inv_mass > 0 is dynamic: its mesh's vertices are in the body frame, and
 * every substep integrates it, applies the body deltas of its particle contacts
 * and solves its rigid contacts (its mesh's vertices against the ground plane
 * and the other meshes). Bodies with inv_mass == 0 keep the reference's static
 * behaviour (world-space mesh, identity pose). Arrays hold one row per mesh:
 * q (pos xyz, quat xyzw) x7, qd (linear, angular) x6, com x3, inertia and
 * inv_inertia x9 (symmetric), inv_mass, flags (2 = kinematic). NULL keeps the
 * current values. Call after xpbd_finalize_meshes. */
typedef struct xpbd_body_params {
    float angular_damping;             /* integrate_bodies.comp push constant */
    float rigid_contact_margin;        /* vertex-to-shape distance that makes a rigid contact */
    float rigid_contact_relaxation;    /* solve_body_contact_positions.comp push constant */
    int32_t rigid_contact_con_weighting; /* apply_body_deltas.comp use_constraint_weights */
    float rigid_mu_torsional;
    float rigid_mu_rolling;
    int32_t particle_contact_con_weighting; /* particle-contact body deltas averaged per body */
} xpbd_body_params;
void xpbd_body_params_default(xpbd_body_params* p);
int xpbd_set_body_params(xpbd_solver* s, const xpbd_body_params* p);
int xpbd_set_bodies(xpbd_solver* s, const float* q, const float* qd, const float* com, const float* inertia,
                    const float* inv_inertia, const float* inv_mass, const int32_t* flags, size_t num_bodies);
int xpbd_get_bodies(xpbd_solver* s, float* q, float* qd, size_t num_bodies);
/* Batched solvers (xpbd_batch_init): the scene of each body, -1 for a static body shared
 * by every scene. A dynamic body then meets only the particles and dynamic bodies of its
 * own scene, so each scene steps as it would alone (with the batch's mesh 0 supplying
 * the average edge length, as mesh 0 does in a single scene). Default: scene 0. */
int xpbd_set_body_scenes(xpbd_solver* s, const int32_t* scene_of_body, size_t num_bodies);

/* Differentiable rollout — an extension with no reference counterpart: the
 * hand-written adjoint of the substep (integration, ground-plane and
 * particle-particle contact projection, delta apply, restitution).
 * xpbd_rollout steps `frames` frames exactly like xpbd_step and stores the state
 * every checkpoint_frames frames; xpbd_rollout_backward replays each checkpointed
 * segment and runs the adjoint of its substeps in reverse, returning the gradient
 * of a loss on the final state (grad_x_final, grad_v_final: n*3 floats;
 * grad_v_final may be NULL) with respect to the initial positions and velocities
 * (n*3 each), the inverse masses (n) and params[4] = {soft_contact_mu,
 * shape_material_mu, particle_mu, soft_contact_restitution}. Output pointers may be
 * NULL. Contact sets and friction branches are those of the forward pass. Covered:
 * one scene, ground plane and particle contacts (no meshes or bodies), every
 * particle active, particles of equal radius, one solver iteration. The solver is
 * left at the rollout's final state. */
/* Frame cache — the add-on's per-frame np.save of get_positions()
 * (newton_vulkan_plugin.py:626-631) without the wait: after every later step the
 * positions are copied to pinned host memory on the solver's stream and written
 * as <directory>/frame_%04d.npy (float32, shape (n, 3); numbering from
 * first_frame) by a writer thread while the GPU runs the next frame.
 * xpbd_record_stop waits for the pending files and reports how many were written
 * (an I/O error is reported by the next step or by xpbd_record_stop). */
int xpbd_record_start(xpbd_solver* s, const char* directory, int first_frame);
int xpbd_record_stop(xpbd_solver* s, int* frames_written);

/* Sort autotuner (autotuned sort parameters for batched scenes): times every
 * onesweep variant (digit width 8 or 7 bits, 2 to 32 keys per thread) on the
 * scene's current keys and keeps the fastest. Runs by itself on the first step of a
 * solver with XPBD_AUTOTUNE_MIN particles or more; results never depend on the
 * choice (the sort is stable). best = {bits, keys per thread};
 * times_us[XPBD_SORT_VARIANTS] = the variants in the order
 * (8,2) (8,4) (8,8) (8,16) (7,4) (7,8) (7,16) (7,32). */
#define XPBD_SORT_VARIANTS 8
#define XPBD_AUTOTUNE_MIN 65536
int xpbd_autotune(xpbd_solver* s, int best[2], double* times_us);
/* Fixes the sort variant instead: (bits, keys per thread) among the variants above. */
int xpbd_set_sort_variant(xpbd_solver* s, int bits, int keys_per_thread);

/* How the first solver iteration of a substep with meshes is ordered against contact
 * generation (no counterpart in the reference; results are identical either way):
 * 0 = fused after the contacts, 1 = its particle-particle part computed beside contact
 * generation and the rest after it, -1 (default) = each solver times both over its first
 * frames, keeps the faster (the split within 1%), and times both again every 16 frames. xpbd_get_solve_split
 * reports the form in use (-1 while timing). */
int xpbd_set_solve_split(xpbd_solver* s, int mode);
int xpbd_get_solve_split(const xpbd_solver* s, int* mode);
/* Form of the solve kernel (no counterpart in the reference; results are identical in every
 * form): 0 = each thread computes the pair terms of its own particle's neighbours, 1 = the
 * lanes of a warp compute their neighbours' pair terms together (balanced when neighbour
 * counts differ), 2 = as 0 with each block's neighbourhood records staged in shared memory
 * (one scene only; slower on the benchmark scenes, so never chosen by the timing), 3 = one
 * warp per particle (the lanes test its candidates and compute its pair terms together), -1
 * (default) = form 3 for scenes of at most 8,192 particles, form 0 up to 16,383, and from
 * 16,384 particles forms 0 and 1 timed on the solver's own last substep after its first
 * frame and again every 64 frames, switching only to a form faster by more than 2%.
 * xpbd_get_solve_form reports the form in use. */
int xpbd_set_solve_form(xpbd_solver* s, int form);
int xpbd_get_solve_form(const xpbd_solver* s, int* form);

/* New contact / material parameters after init (e.g. between rollouts of an
 * optimisation): every numeric field of cfg except device_index and the
 * diagnostics / profiling switches, which stay as at init. */
int xpbd_update_config(xpbd_solver* s, const xpbd_config* cfg);
int xpbd_rollout(xpbd_solver* s, float dt, int substeps, int iterations, int frames, int checkpoint_frames);
int xpbd_rollout_backward(xpbd_solver* s, const float* grad_x_final, const float* grad_v_final, float* grad_x0,
                          float* grad_v0, float* grad_inv_mass, double* grad_params);

/* Batched scenes (the xpbd_batch_* family). One solver steps n_scenes
 * independent scenes in one graph per frame, one launch per kernel for all of
 * them. Each scene has its own 128^3 hash grid (the scene id is the high part of
 * the sort key), so scene s steps exactly as a solver initialised with
 * scene_counts[s] particles would. Particles are the concatenation of the
 * scenes' particles in scene order: xpbd_set_particles, xpbd_get_positions and
 * the other particle calls take all of them, scene s at offset
 * offsets[s] = scene_counts[0] + ... + scene_counts[s-1]. Meshes, the plane and
 * the configuration are shared by all scenes; max_contacts (0 = 2 x total
 * particles) caps the whole batch. 1 <= n_scenes <= 2048. The cell-table getter
 * reports scene 0. */
int xpbd_batch_init(xpbd_solver* s, const xpbd_config* cfg, const size_t* scene_counts, size_t n_scenes,
                    size_t max_contacts);
size_t xpbd_batch_scene_count(xpbd_solver* s);
/* offsets: n_scenes + 1 entries (the last is the total particle count) */
int xpbd_batch_scene_offsets(xpbd_solver* s, size_t* offsets, size_t cap);

/* Allocation-free sort — no counterpart in the reference. For callers that
 * cannot allocate device memory while they run (work captured into a CUDA
 * graph owned by another framework, plugins inside an application with its own
 * device memory pool, real-time loops that forbid allocator calls): the stable
 * hash-grid radix sort of n keys of key_bits bits, values = input index, from
 * device buffer d_keys into device buffers d_sorted_keys / d_sorted_ids, queued
 * on `stream` (a cudaStream_t; NULL = legacy default stream). It calls no
 * cudaMalloc/cudaFree: its scratch is a static device array of about 10.5 MiB
 * that every GPU loading the library holds until exit, so n is limited to
 * XPBD_NOALLOC_MAX_KEYS. The first call on a device resolves that array's
 * device address (make it before any stream capture). All calls share the
 * array: calls that overlap on the GPU race and give wrong results. d_keys must
 * not overlap d_sorted_keys or d_sorted_ids (rejected). The call returns once
 * the sort has finished on `stream`: it reads back an 8-byte status word and
 * fails ("device wait timed out") when a bounded wait inside the sort ran out,
 * in which case the output is invalid. Called while `stream` is being captured
 * into a CUDA graph (where no synchronisation is allowed) it only records the
 * sort and returns 0; after a replay of that graph has finished,
 * xpbd_sort_keys_noalloc_status reads the replay's status word. The array's
 * device address is resolved once per device ordinal for the life of the
 * process, so a cudaDeviceReset in between is not supported. */
#define XPBD_NOALLOC_MAX_KEYS (1 << 20)
int xpbd_sort_keys_noalloc(const uint32_t* d_keys, uint32_t* d_sorted_keys, uint32_t* d_sorted_ids, size_t n,
                           int key_bits, void* stream);
/* The status of the last allocation-free sort on the current device (or of the
 * last replay of a graph that recorded one), read after its stream finished:
 * 0, or -1 with "device wait timed out" (output invalid). */
int xpbd_sort_keys_noalloc_status(void);

#ifdef __cplusplus
}
#endif

#endif /* XPBD_GB300_H */
