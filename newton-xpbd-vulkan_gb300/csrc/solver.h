// Host scene driver: the GB300 counterpart of vkx::XpbdSolver
// (src/scene.h:74-227, src/scene.cpp). Owns all device memory of one scene,
// records one CUDA graph per (dt, substeps, iterations, state parity) and
// replays it per frame.
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/xpbd.h"
#include "kernels.h"

namespace xpbd {

void cuda_check(cudaError_t e, const char* what, const char* file, int line);
#define XPBD_CUDA(x) ::xpbd::cuda_check((x), #x, __FILE__, __LINE__)

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void alloc(size_t count, bool zero = true) {
        release();
        n = count;
        if (count) {
            XPBD_CUDA(cudaMalloc(&p, count * sizeof(T)));
            if (zero) XPBD_CUDA(cudaMemset(p, 0, count * sizeof(T)));
        }
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

struct MeshData {  // src/scene.h:66-72
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    float shape_margin = 0.0f;
    float shape_rot[4] = {0.f, 0.f, 0.f, 1.f};
    bool is_watertight = false;
    float avg_edge = 0.0f;
};

bool tris_watertight(const uint32_t* tris, size_t num_tris, size_t num_verts);

// Writes frame_%04d.npy files of the positions after every step from a worker thread,
// overlapping the next frame (recorder.cpp).
class FrameRecorder {
   public:
    ~FrameRecorder();
    void start(int device, size_t n, const std::string& dir, int first_frame);
    int stop();  // waits for pending writes; returns the number of files written
    void enqueue(cudaStream_t stream, const float* d_xyz);
    bool active() const { return active_; }

   private:
    static constexpr int kSlots = 3;
    struct Slot {
        float* host = nullptr;
        cudaEvent_t done = nullptr;
        bool busy = false;
        int frame = 0;
    };
    void run();
    Slot slots_[kSlots];
    std::thread worker_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<int> queue_;
    std::string dir_, header_, error_;
    size_t n_ = 0;
    int device_ = 0, next_frame_ = 1, written_ = 0;
    bool active_ = false, stop_flag_ = false;
};

class Solver {
   public:
    static constexpr int kMaxStages = 32;  // >= the number of profiler stages (solver.cpp)
    Solver();
    ~Solver();

    void init(const xpbd_config& cfg, size_t num_particles, size_t max_contacts);
    // Independent scenes stepped together: particles are the concatenation of the
    // scenes' particles; each scene has its own 128^3 hash grid, so each steps exactly
    // as it would alone. At most 2048 scenes (the scene id rides in the sort key).
    void init_batched(const xpbd_config& cfg, const size_t* scene_counts, size_t n_scenes, size_t max_contacts);
    size_t scene_count() const { return scene_off_.empty() ? 0 : scene_off_.size() - 1; }
    void scene_offsets(size_t* out) const {
        for (size_t i = 0; i < scene_off_.size(); i++) out[i] = scene_off_[i];
    }
    void add_mesh(const float* verts, size_t num_verts, const uint32_t* tris, size_t num_tris, float shape_margin,
                  const float* rot_xyzw, int watertight_override);
    void finalize_meshes();
    void set_particles(const float* q, const float* qd, const float* inv_mass, const float* radii,
                       const int32_t* flags, size_t n);
    void update_mesh(size_t mesh_index, const float* verts, size_t num_verts, const float* vels);
    // rigid bodies (one per mesh): q (pos xyz, quat xyzw) x7, qd (lin, ang) x6, com x3,
    // inertia and inv_inertia x9, inv_mass, flags; null pointers keep the current values
    void set_bodies(const float* q, const float* qd, const float* com, const float* inertia,
                    const float* inv_inertia, const float* inv_mass, const int32_t* flags, size_t nb);
    void get_bodies(float* q, float* qd, size_t nb);
    // batched: scene of each body (-1: static, shared by every scene)
    void set_body_scenes(const int32_t* scenes, size_t nb);
    // frame cache: positions of every later step written to dir/frame_%04d.npy
    void record_start(const std::string& dir, int first_frame);
    int record_stop();
    void set_body_params(const xpbd_body_params& p);
    // differentiable rollout: `frames` frames like step(), checkpointing the state every
    // checkpoint_frames frames; rollout_backward runs the adjoint of the whole rollout
    void rollout(float dt, int substeps, int iterations, int frames, int checkpoint_frames);
    // new material / contact parameters (every field but the sizes, device and diagnostics)
    void update_config(const xpbd_config& cfg);
    // sort autotuner: times the onesweep variants on the current keys, keeps the fastest;
    // returns the times (us) of {8b x 8, 8b x 16, 7b x 16, 7b x 32}
    std::vector<double> autotune_sort(int* best_bits, int* best_items);
    void set_sort_variant(int bits, int items);
    void set_solve_split(int mode);               // -1 timed choice, 0 fused, 1 split
    int solve_split() const { return split_choice_; }
    // form of the solve kernel (kernels.h kSolveForms): -1 timed choice (default), or a form
    void set_solve_form(int form);
    int solve_form() const { return solve_form_; }
    uint64_t kernels_launched() const { return kernels_total_; }
    void rollout_backward(const float* gx_final, const float* gv_final, float* gx0, float* gv0, float* gw,
                          double* params);
    void step(float dt, int substeps, int iterations);
    void collide_only();
    void step_solve_only(float dt, int substeps, int iterations);

    void get_positions(float* out, size_t n);
    void get_velocities(float* out, size_t n);
    size_t particle_count() const { return n_; }
    size_t mesh_count() const { return meshes_.size(); }
    int last_contact_count() const { return contact_count_; }
    void get_contacts(int32_t* part, int32_t* shape, float* nrm, float* bpos, float* bvel);
    void set_contact_data(const int32_t* part, const int32_t* shape, const float* bpos, const float* nrm,
                          int count);
    void get_sorted(uint32_t* cells, uint32_t* ids, size_t n);
    void get_cell_tables(int32_t* starts, int32_t* ends);
    void get_deltas(float* out, size_t n);
    size_t mesh_bvh(size_t mesh_index, float* lowers, float* uppers, size_t cap);
    uint32_t diag_pair_count();
    uint32_t diag_overflow_count();
    void reset_diag_buffers();
    size_t diag_pairs(xpbd_pair_record* out, size_t cap);
    size_t aux_diag(int which, void* out, size_t cap);
    void print_profiler_summary();
    void status(uint32_t out[4]) const;
    // extensions used by the benchmark harness
    void step_async(float dt, int substeps, int iterations);
    void sync();
    cudaStream_t stream() const { return stream_; }
    void set_profiling(bool on);
    size_t stage_times(double* ms, size_t cap, uint64_t* substeps) const;
    void reset_stage_times();
    void frame_stats(uint64_t out[4]) const;
    static const char* stage_name(int i);
    static int stage_count();

   private:
    enum class Mode { Step, SolveOnly };
    struct GraphKey {
        uint32_t dt_bits;
        int substeps, iterations, parity, mode, timed, split, form;
        bool operator<(const GraphKey& o) const {
            return std::tie(dt_bits, substeps, iterations, parity, mode, timed, split, form) <
                   std::tie(o.dt_bits, o.substeps, o.iterations, o.parity, o.mode, o.timed, o.split, o.form);
        }
    };
    struct FrameGraph {
        cudaGraphExec_t exec = nullptr;
        std::vector<std::pair<cudaEvent_t, int>> marks;  // stage events captured as graph nodes
        uint64_t kernels = 0, memsets = 0;
    };
    void require_init() const;
    void clear_graphs();
    void clear_backward_graphs();
    void ensure_cull();
    void upload_dyn_scenes();
    void upload_xyz(const float* h, float4* d, size_t n);
    void download_xyz(const float4* d, float* h, size_t n);
    void ensure_substep_capacity(int substeps);
    void record_frame(Mode mode, float dt, int substeps, int iterations, int parity);
    void record_substep(Mode mode, int sub, int iterations, float sdt, int src);
    void run_frame(Mode mode, float dt, int substeps, int iterations, bool sync);
    void finish_frame(int substeps);
    void accumulate_stage_times(const FrameGraph& fg);
    void compact_contacts();
    void check_sort_order();
    PredictParams predict_params(float sdt) const;
    SolveParams solve_params(float sdt, int it) const;
    BodyTables body_tables() const;
    MeshTables mesh_tables() const;
    LbvhTopology topology(size_t mesh) const;
    BodyArrays body_arrays() const;
    RigidTables rigid_tables() const;
    RigidParams rigid_params(float sdt) const;
    void prof_mark(int slot);
    void apply_sort_plan(int bits, int items);
    bool sort_tuned_ = false;
    // one-warp blocks per SM of the static-mesh traversal while the moving-mesh queries run
    // beside it on the second stream (32, the SM's block limit, when it runs alone)
    static constexpr int kWalkBlocksBeside = 16;
    // Solve-kernel form: timed on the scene's own last substep (its last iteration launched
    // again with its outputs in scratch buffers) after the first frame and again every
    // kSolveRetime frames, as the scene evolves; every form gives the same bits. A retime
    // launches the scene's last iteration eight more times, so it is rare, and the form in
    // use is kept unless the other is faster by more than 2%.
    static constexpr uint64_t kSolveRetime = 64;
    static constexpr size_t kSolveTuneMinParticles = 16384;  // smaller scenes keep the default
    // the default form: one warp per particle for small scenes, whose solve time is one
    // particle's latency (4,096 particles: 28.8 -> 20.8 us per substep; slower from 16,384)
    static constexpr size_t kParticleWarpMaxParticles = 8192;
    int default_solve_form() const { return n_ <= kParticleWarpMaxParticles ? 3 : 0; }
    int solve_form_ = 0, solve_form_forced_ = -1;
    uint64_t solve_form_frame_ = 0;
    bool solve_form_timed_ = false;
    float last_sdt_ = 0.0f;
    int last_substeps_ = 0, last_iterations_ = 0;
    bool last_was_step_ = false;
    void autotune_solve();
    uint32_t lb_debug_seen_ = 0;  // lookback_debug_generation() the frame graphs were recorded under
    void count_kernel(int k = 1);
    void count_memset();

    xpbd_config cfg_{};
    bool initialized_ = false, finalized_ = false;
    int device_ = 0;
    size_t n_ = 0;
    int64_t contact_max_ = 0;
    int contact_count_ = 0;
    cudaStream_t stream_ = nullptr;
    // second stream of the frame graph: the mesh traversal runs on it beside the
    // integrate / sort / gather chain, which does not read contacts
    cudaStream_t aux_ = nullptr;
    cudaStream_t walk_stream_ = nullptr;  // the static-mesh traversal beside the moving-mesh chain
    cudaEvent_t fork_ = nullptr, join_ = nullptr, triaged_ = nullptr, walked_ = nullptr;
    // Whether the first iteration's particle-particle part runs before the join, beside the
    // contact generation (split) or after it, fused with the rest (the faster depends on how
    // long the contact chain is next to the sort and the solve): -1 undecided, in which case
    // the next kSplitTrials frames run both ways under events and the faster is kept.
    // Results are the same either way.
    // The choice is timed again every kSplitRetime frames (both graphs exist by then, so
    // two frames each way): a scene's balance moves as it evolves (bodies settling into a
    // pile multiply the moving-mesh queries). Within 1% the split is kept.
    static constexpr int kSplitTrials = 6;
    static constexpr int kSplitRetime = 16;
    int split_choice_ = -1;
    int split_frames_ = 0;  // frames since the last choice
    int split_forced_ = -1;  // set_solve_split: kept across graph rebuilds
    int split_trials_ = 0;
    bool split_now_ = false;
    cudaEvent_t split_ev_[kSplitTrials][2] = {};

    std::vector<MeshData> meshes_;
    std::vector<size_t> vert_offsets_, node_offsets_, prim_offsets_;
    std::vector<float> all_verts_, all_vels_;

    // particle state, original order: [parity]
    DevBuf<float4> x_[2], v_[2];
    DevBuf<float> w_, r_;
    DevBuf<int> flags_;
    int cur_ = 0;
    bool all_active_ = false;
    // batched scenes
    std::vector<size_t> scene_off_;  // n_scenes + 1 prefix offsets
    DevBuf<uint32_t> pscene_;        // scene of each particle (batched only)
    int key_bits_ = 21;
    // hash grid and sort
    SortPlan plan_{};
    DevBuf<uint32_t> keys_, pair_k_[2], pair_v_[2];
    // one scene sorts split keys (the reference's cell key + 3 alias bits); the sorted-order
    // getters re-sort the reference's 21-bit keys on demand into ref_k_ / ref_v_
    bool split_keys_ = false;
    DevBuf<uint32_t> ref_k_[2], ref_v_[2];
    const uint32_t* sort_reference_layout(const uint32_t** ids);
    DevBuf<uint32_t> sort_scratch_;  // hist | lookback | tile counters (cleared per substep)
    size_t hist_off_ = 0, lb_off_ = 0, tc_off_ = 0, cq_off_ = 0;
    DevBuf<int4> table_;
    DevBuf<uint32_t> stamp_;
    DevBuf<float4> rx_[2], rv_[2];
    DevBuf<float4> pp_;  // first iteration's particle-particle totals (sorted order) when split
    DevBuf<int> rf_;
    // contacts
    int slot_cap_ = 1;
    DevBuf<uint32_t> cinfo_;
    DevBuf<float4> cslot_;
    DevBuf<uint32_t> ccount_;  // one counter per substep of the frame
    int ccount_cap_ = 0;
    bool need_ranks_ = false;
    DevBuf<uint2> rank_;
    DevBuf<uint32_t> totals_, scan_ws_;
    int last_collide_src_ = 0;  // parity of the positions the last collision pass read
    // injected contacts (set_contact_data / step_solve_only)
    bool injected_ = false;
    int inj_cap_ = 1;
    DevBuf<uint32_t> inj_info_;
    DevBuf<float4> inj_slot_;
    std::vector<int32_t> inj_part_, inj_shape_;
    std::vector<float> inj_bpos_, inj_nrm_;
    // shapes / bodies / meshes on device
    DevBuf<int> shape_body_;
    DevBuf<float> shape_mu_;
    DevBuf<float4> body_q_, body_qd_;
    DevBuf<float> body_com_, body_invI_, body_invm_;
    DevBuf<int> body_flags_;
    // dynamic bodies
    DevBuf<float> body_I_;
    bool dyn_any_ = false;
    bool dyn_tables_ready_ = false;  // the dynamic-body tables match dyn_list_ and the meshes
    std::vector<int> dyn_list_;
    xpbd_body_params body_params_{0.0f, 0.01f, 0.8f, 1, 0.0f, 0.0f, 1};
    DevBuf<float4> body_q_mid_, body_qd_mid_, body_q_prev_, body_qd_prev_;
    DevBuf<int> dyn_, dyn_index_, posed_, walk_list_, partners_, partner_count_, rc_count_;
    int walk_count_ = 0, n_dyn_verts_ = 0, grid_size_ = 0;
    float dyn_half_diag_ = 0.0f, dyn_max_margin_ = 0.0f;
    DevBuf<uint32_t> grid_count_, grid_start_, grid_tiles_;
    DevBuf<int4> grid_list_;
    DevBuf<uint32_t> posed_list_;  // per substep: (particle, its first candidate moving meshes) entries
    DevBuf<float4> posed_hits_;    // per list entry: the query results of its listed candidates
    std::vector<int32_t> body_scene_;  // batched: scene of each body (-1: every scene)
    DevBuf<int> dyn_scene_;            // scene of each dynamic body (dyn index)
    DevBuf<uint32_t> dv_start_;
    DevBuf<float4> dv_local_, wbox_, rc_;
    uint32_t entry_cap_ = 0;
    SortPlan eplan_{};
    size_t ehist_off_ = 0, elb_off_ = 0, etc_off_ = 0;
    DevBuf<uint32_t> esort_scratch_, ekeys_, epk_[2], epv_[2];
    const uint32_t* sorted_entries_ = nullptr;
    DevBuf<uint2> seg_, dyn_rank_;
    DevBuf<uint32_t> dyn_totals_, dyn_ws_;
    DevBuf<float4> bdel_;
    DevBuf<float4> nl_, nu_;
    DevBuf<float> verts_, vels_;
    DevBuf<uint32_t> tris_, prim_, roots_, prim_off_, prim_cnt_;
    DevBuf<float4> tri_cache_;
    DevBuf<float4> node_pair_;  // MeshTables::pair, 4 per node slot
    // reach grids (MeshTables::cull_*), rebuilt by ensure_cull when meshes, radii or
    // the contact margin change
    DevBuf<float4> cull_org_;
    DevBuf<int4> cull_dim_;
    DevBuf<uint32_t> cull_off_, cull_bits_, cull_tmp_, node_off_dev_;
    DevBuf<uint32_t> near_;  // particles the collision kernel traverses, per substep
    bool cull_dirty_ = true;
    float r_min_ = 0.0f, r_max_ = 0.0f;
    bool r_finite_ = true;
    DevBuf<int> topo_parent_, topo_child_l_, topo_child_r_;
    DevBuf<uint8_t> topo_marked_, topo_reachable_;
    DevBuf<uint32_t> topo_prim_, bvh_scratch_;
    DevBuf<float> margins_;
    DevBuf<int> watertight_;
    float avg_edge0_ = 0.0f;
    // frame recorder
    FrameRecorder recorder_;
    DevBuf<float> rec_stage_;
    // differentiable rollout
    bool rollout_valid_ = false;
    float ro_dt_ = 0.0f;
    int ro_substeps_ = 0, ro_frames_ = 0, ro_ckpt_ = 0;
    DevBuf<float4> ckpt_, traj_, gx_, gv_, gacc_, part_xp_, part_vp_, part_x0_, part_v0_, part_gd_;
    DevBuf<uint32_t> traj_keys_;
    DevBuf<float> gw_, block_params_;
    DevBuf<double> param_acc_;
    void prepare_grid(float sdt, int src);
    // diagnostics
    DevBuf<float> delta_;
    DevBuf<uint32_t> diag_header_;
    DevBuf<float> diag_pairs_;
    DevBuf<DeviceStatus> status_;
    DeviceStatus host_status_{};
    // staging
    DevBuf<float> xyz_stage_;
    float* pinned_ = nullptr;  // 64 words: the per-frame readback
    size_t pinned_words_ = 0;
    DevBuf<int32_t> c_part_, c_shape_;
    DevBuf<float> c_bpos_, c_bvel_, c_nrm_;
    DevBuf<int32_t> cell_starts_, cell_ends_;
    // graphs
    std::map<GraphKey, FrameGraph> graphs_;
    std::map<std::pair<int, uint32_t>, cudaGraphExec_t> bwd_graphs_;  // rollout_backward segments by (substeps, dt)
    FrameGraph* recording_ = nullptr;  // graph being captured (marks and node counts go here)
    int pending_substeps_ = 0;         // frame launched by step_async and not yet synced
    uint64_t frames_run_ = 0;
    uint64_t last_kernels_ = 0, last_memsets_ = 0;
    uint64_t kernels_total_ = 0;  // kernels launched by all frames run
    // profiler (stage names follow scene.cpp:1481-1505 where the stages correspond)
    bool profiling_ = false;
    double prof_ms_[kMaxStages] = {0};
    uint64_t prof_substeps_ = 0;
    double prof_wall_ms_ = 0.0;
};

}  // namespace xpbd
