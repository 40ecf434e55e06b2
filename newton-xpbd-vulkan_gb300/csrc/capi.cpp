// extern "C" boundary of libxpbd_gb300.so (declared in include/xpbd.h).
// Each entry point catches C++ exceptions, stores the message in a
// thread-local string and returns -1, so no exception crosses the ABI.
#include <algorithm>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>

#include "../../include/xpbd.h"
#include "solver.h"

struct xpbd_solver {
    xpbd::Solver impl;
};

namespace {
thread_local std::string g_last_error;

template <class F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
    } catch (...) {
        g_last_error = "unknown error";
    }
    return -1;
}

xpbd::Solver& S(xpbd_solver* s) {
    if (!s) throw std::runtime_error("null solver handle");
    return s->impl;
}
const xpbd::Solver& CS(const xpbd_solver* s) {
    if (!s) throw std::runtime_error("null solver handle");
    return s->impl;
}
}  // namespace

extern "C" {

const char* xpbd_last_error(void) { return g_last_error.c_str(); }
int xpbd_abi_version(void) { return XPBD_ABI_VERSION; }

void xpbd_config_default(xpbd_config* c) {  // src/scene.h:15-40
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->dt = 1.0f / 60.0f;
    c->substeps = 1;
    c->iterations = 2;
    c->particle_v_max = 1e5f;
    c->soft_contact_mu = 0.5f;
    c->shape_material_mu = 1.0f;
    c->soft_contact_relaxation = 0.9f;
    c->particle_adhesion = 0.0f;
    c->particle_mu = 0.5f;
    c->particle_cohesion = 0.0f;
    c->particle_max_radius = 0.02f;
    c->search_radius = 0.04f;
    c->soft_contact_margin = 0.01f;
    c->enable_restitution = 0;
    c->soft_contact_restitution = 0.0f;
    c->has_ground_plane = 1;
    c->ground_plane_altitude = 0.0f;
    c->gravity[0] = 0.0f;
    c->gravity[1] = 0.0f;
    c->gravity[2] = -9.81f;
    std::strncpy(c->shader_dir, "shaders", sizeof(c->shader_dir) - 1);
    c->device_index = -1;
    c->max_diag_pairs = 100000;
    c->substep_batch_size = 15;
}

int xpbd_device_count(int* count) {
    return guarded([&] {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
        if (count) *count = n;
    });
}

int xpbd_device_name(int index, char* buf, size_t cap) {
    return guarded([&] {
        cudaDeviceProp p;
        XPBD_CUDA(cudaGetDeviceProperties(&p, index));
        if (buf && cap) {
            std::strncpy(buf, p.name, cap - 1);
            buf[cap - 1] = 0;
        }
    });
}

int xpbd_create(xpbd_solver** out) {
    return guarded([&] {
        if (!out) throw std::runtime_error("null output pointer");
        *out = new xpbd_solver();
    });
}

int xpbd_destroy(xpbd_solver* s) {
    return guarded([&] { delete s; });
}

int xpbd_init(xpbd_solver* s, const xpbd_config* cfg, size_t num_particles, size_t max_contacts) {
    return guarded([&] {
        xpbd_config c;
        if (cfg)
            c = *cfg;
        else
            xpbd_config_default(&c);
        S(s).init(c, num_particles, max_contacts);
    });
}

int xpbd_add_mesh(xpbd_solver* s, const float* verts, size_t num_verts, const uint32_t* tris, size_t num_tris,
                  float shape_margin, const float* rot, int wt) {
    return guarded([&] { S(s).add_mesh(verts, num_verts, tris, num_tris, shape_margin, rot, wt); });
}

int xpbd_finalize_meshes(xpbd_solver* s) {
    return guarded([&] { S(s).finalize_meshes(); });
}

int xpbd_set_particles(xpbd_solver* s, const float* q, const float* qd, const float* inv_mass, const float* radii,
                       const int32_t* flags, size_t n) {
    return guarded([&] { S(s).set_particles(q, qd, inv_mass, radii, flags, n); });
}

int xpbd_update_mesh(xpbd_solver* s, size_t mesh_index, const float* verts, size_t num_verts, const float* vels) {
    return guarded([&] { S(s).update_mesh(mesh_index, verts, num_verts, vels); });
}

int xpbd_step(xpbd_solver* s, float dt, int substeps, int iterations) {
    return guarded([&] { S(s).step(dt, substeps, iterations); });
}

int xpbd_collide_only(xpbd_solver* s) {
    return guarded([&] { S(s).collide_only(); });
}

int xpbd_step_solve_only(xpbd_solver* s, float dt, int substeps, int iterations) {
    return guarded([&] { S(s).step_solve_only(dt, substeps, iterations); });
}

int xpbd_get_positions(xpbd_solver* s, float* out, size_t n) {
    return guarded([&] { S(s).get_positions(out, n); });
}

int xpbd_get_velocities(xpbd_solver* s, float* out, size_t n) {
    return guarded([&] { S(s).get_velocities(out, n); });
}

size_t xpbd_particle_count(const xpbd_solver* s) { return s ? s->impl.particle_count() : 0; }
size_t xpbd_mesh_count(const xpbd_solver* s) { return s ? s->impl.mesh_count() : 0; }
int xpbd_last_contact_count(const xpbd_solver* s) { return s ? s->impl.last_contact_count() : 0; }

int xpbd_get_contacts(xpbd_solver* s, int32_t* particles, int32_t* shapes, float* normals, float* body_positions,
                      float* body_velocities) {
    return guarded([&] { S(s).get_contacts(particles, shapes, normals, body_positions, body_velocities); });
}

int xpbd_set_contact_data(xpbd_solver* s, const int32_t* particles, const int32_t* shapes,
                          const float* body_positions, const float* normals, int contact_count) {
    return guarded([&] { S(s).set_contact_data(particles, shapes, body_positions, normals, contact_count); });
}

int xpbd_get_sorted_cells(xpbd_solver* s, uint32_t* out, size_t n) {
    return guarded([&] { S(s).get_sorted(out, nullptr, n); });
}

int xpbd_get_sorted_point_ids(xpbd_solver* s, uint32_t* out, size_t n) {
    return guarded([&] { S(s).get_sorted(nullptr, out, n); });
}

int xpbd_get_cell_starts(xpbd_solver* s, int32_t* out, size_t n) {
    return guarded([&] {
        if (n < (size_t)XPBD_NUM_CELLS) throw std::runtime_error("cell table buffer too small");
        S(s).get_cell_tables(out, nullptr);
    });
}

int xpbd_get_cell_ends(xpbd_solver* s, int32_t* out, size_t n) {
    return guarded([&] {
        if (n < (size_t)XPBD_NUM_CELLS) throw std::runtime_error("cell table buffer too small");
        S(s).get_cell_tables(nullptr, out);
    });
}

int xpbd_get_deltas(xpbd_solver* s, float* out, size_t n) {
    return guarded([&] { S(s).get_deltas(out, n); });
}

int xpbd_get_mesh_bvh(xpbd_solver* s, size_t mesh_index, float* lowers, float* uppers, size_t cap_nodes,
                      size_t* num_nodes) {
    return guarded([&] {
        size_t k = S(s).mesh_bvh(mesh_index, lowers, uppers, cap_nodes);
        if (num_nodes) *num_nodes = k;
    });
}

int xpbd_get_diag_pair_count(xpbd_solver* s, uint32_t* out) {
    return guarded([&] { *out = S(s).diag_pair_count(); });
}

int xpbd_get_diag_overflow_count(xpbd_solver* s, uint32_t* out) {
    return guarded([&] { *out = S(s).diag_overflow_count(); });
}

int xpbd_reset_diag_buffers(xpbd_solver* s) {
    return guarded([&] { S(s).reset_diag_buffers(); });
}

int xpbd_get_diag_pairs(xpbd_solver* s, xpbd_pair_record* out, size_t cap, size_t* count) {
    return guarded([&] {
        size_t k = S(s).diag_pairs(out, cap);
        if (count) *count = k;
    });
}

int xpbd_get_aux_diag(xpbd_solver* s, int which, void* out, size_t cap, size_t* count) {
    return guarded([&] {
        size_t k = S(s).aux_diag(which, out, cap);
        if (count) *count = k;
    });
}

int xpbd_print_profiler_summary(xpbd_solver* s) {
    return guarded([&] { S(s).print_profiler_summary(); });
}

int xpbd_get_status(xpbd_solver* s, uint32_t out[4]) {
    return guarded([&] { S(s).status(out); });
}

int xpbd_set_solve_form(xpbd_solver* s, int form) {
    return guarded([&] { S(s).set_solve_form(form); });
}

int xpbd_get_solve_form(const xpbd_solver* s, int* form) {
    return guarded([&] {
        if (!s) throw std::runtime_error("null solver");
        if (form) *form = s->impl.solve_form();
    });
}

int xpbd_debug_lookback_hold(int64_t hold_tile, uint64_t wait_ns) {
    return guarded([&] { xpbd::set_lookback_debug(hold_tile, wait_ns); });
}

int xpbd_step_async(xpbd_solver* s, float dt, int substeps, int iterations) {
    return guarded([&] { S(s).step_async(dt, substeps, iterations); });
}

int xpbd_sync(xpbd_solver* s) {
    return guarded([&] { S(s).sync(); });
}

void* xpbd_stream(xpbd_solver* s) { return s ? (void*)s->impl.stream() : nullptr; }

int xpbd_set_profiling(xpbd_solver* s, int on) {
    return guarded([&] { S(s).set_profiling(on != 0); });
}

int xpbd_get_stage_times(xpbd_solver* s, double* ms, size_t cap, size_t* num_stages, uint64_t* substeps) {
    return guarded([&] {
        double tmp[32];
        size_t k = S(s).stage_times(tmp, 32, substeps);
        if (ms)
            for (size_t i = 0; i < std::min(k, cap); i++) ms[i] = tmp[i];
        if (num_stages) *num_stages = k;
    });
}

int xpbd_reset_stage_times(xpbd_solver* s) {
    return guarded([&] { S(s).reset_stage_times(); });
}

const char* xpbd_stage_name(int index) { return xpbd::Solver::stage_name(index); }

int xpbd_get_frame_stats(xpbd_solver* s, uint64_t out[4]) {
    return guarded([&] { S(s).frame_stats(out); });
}

int xpbd_get_kernels_launched(xpbd_solver* s, uint64_t* total) {
    return guarded([&] {
        if (!total) throw std::runtime_error("xpbd_get_kernels_launched: total is NULL");
        *total = S(s).kernels_launched();
    });
}

void xpbd_body_params_default(xpbd_body_params* p) {
    if (!p) return;
    p->angular_damping = 0.0f;
    p->rigid_contact_margin = 0.01f;
    p->rigid_contact_relaxation = 0.8f;
    p->rigid_contact_con_weighting = 1;
    p->rigid_mu_torsional = 0.0f;
    p->rigid_mu_rolling = 0.0f;
    p->particle_contact_con_weighting = 1;
}

int xpbd_set_body_params(xpbd_solver* s, const xpbd_body_params* p) {
    return guarded([&] {
        xpbd_body_params d;
        xpbd_body_params_default(&d);
        S(s).set_body_params(p ? *p : d);
    });
}

int xpbd_set_bodies(xpbd_solver* s, const float* q, const float* qd, const float* com, const float* inertia,
                    const float* inv_inertia, const float* inv_mass, const int32_t* flags, size_t nb) {
    return guarded([&] { S(s).set_bodies(q, qd, com, inertia, inv_inertia, inv_mass, flags, nb); });
}

int xpbd_get_bodies(xpbd_solver* s, float* q, float* qd, size_t nb) {
    return guarded([&] { S(s).get_bodies(q, qd, nb); });
}

int xpbd_set_body_scenes(xpbd_solver* s, const int32_t* scene_of_body, size_t nb) {
    return guarded([&] { S(s).set_body_scenes(scene_of_body, nb); });
}

int xpbd_record_start(xpbd_solver* s, const char* directory, int first_frame) {
    return guarded([&] {
        if (!directory) throw std::runtime_error("xpbd_record_start: directory is NULL");
        S(s).record_start(directory, first_frame);
    });
}

int xpbd_record_stop(xpbd_solver* s, int* frames_written) {
    return guarded([&] {
        const int k = S(s).record_stop();
        if (frames_written) *frames_written = k;
    });
}

int xpbd_autotune(xpbd_solver* s, int best[2], double* times_us) {
    return guarded([&] {
        int b = 0, i = 0;
        const std::vector<double> t = S(s).autotune_sort(&b, &i);
        if (best) {
            best[0] = b;
            best[1] = i;
        }
        if (times_us)
            for (size_t k = 0; k < t.size(); k++) times_us[k] = t[k];
    });
}

int xpbd_set_sort_variant(xpbd_solver* s, int bits, int keys_per_thread) {
    return guarded([&] { S(s).set_sort_variant(bits, keys_per_thread); });
}

int xpbd_set_solve_split(xpbd_solver* s, int mode) {
    return guarded([&] { S(s).set_solve_split(mode); });
}

int xpbd_get_solve_split(const xpbd_solver* s, int* mode) {
    return guarded([&] {
        if (!mode) throw std::runtime_error("xpbd_get_solve_split: mode is NULL");
        *mode = CS(s).solve_split();
    });
}

int xpbd_update_config(xpbd_solver* s, const xpbd_config* cfg) {
    return guarded([&] {
        if (!cfg) throw std::runtime_error("xpbd_update_config: cfg is NULL");
        S(s).update_config(*cfg);
    });
}

int xpbd_rollout(xpbd_solver* s, float dt, int substeps, int iterations, int frames, int checkpoint_frames) {
    return guarded([&] { S(s).rollout(dt, substeps, iterations, frames, checkpoint_frames); });
}

int xpbd_rollout_backward(xpbd_solver* s, const float* grad_x_final, const float* grad_v_final, float* grad_x0,
                          float* grad_v0, float* grad_inv_mass, double* grad_params) {
    return guarded([&] {
        if (!grad_x_final) throw std::runtime_error("xpbd_rollout_backward: grad_x_final is NULL");
        S(s).rollout_backward(grad_x_final, grad_v_final, grad_x0, grad_v0, grad_inv_mass, grad_params);
    });
}

int xpbd_batch_init(xpbd_solver* s, const xpbd_config* cfg, const size_t* scene_counts, size_t n_scenes,
                    size_t max_contacts) {
    return guarded([&] {
        if (!scene_counts) throw std::runtime_error("xpbd_batch_init: scene_counts is NULL");
        xpbd_config c;
        if (cfg)
            c = *cfg;
        else
            xpbd_config_default(&c);
        S(s).init_batched(c, scene_counts, n_scenes, max_contacts);
    });
}

size_t xpbd_batch_scene_count(xpbd_solver* s) { return s ? s->impl.scene_count() : 0; }

int xpbd_batch_scene_offsets(xpbd_solver* s, size_t* offsets, size_t cap) {
    return guarded([&] {
        if (S(s).scene_count() + 1 > cap) throw std::runtime_error("xpbd_batch_scene_offsets: buffer too small");
        S(s).scene_offsets(offsets);
    });
}

int xpbd_sort_keys_noalloc(const uint32_t* d_keys, uint32_t* d_sorted_keys, uint32_t* d_sorted_ids, size_t n,
                           int key_bits, void* stream) {
    return guarded([&] {
        xpbd::sort_keys_noalloc(d_keys, d_sorted_keys, d_sorted_ids, (int64_t)n, key_bits,
                                static_cast<cudaStream_t>(stream));
    });
}

int xpbd_sort_keys_noalloc_status(void) {
    return guarded([&] { xpbd::sort_keys_noalloc_status(); });
}

}  // extern "C"
