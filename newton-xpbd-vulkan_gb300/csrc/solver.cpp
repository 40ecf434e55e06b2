// Host scene driver (see solver.h). Mirrors src/scene.cpp's public behaviour;
// the Vulkan command-buffer recording, descriptor sets, staging buffers and
// fences are replaced by device allocations, one stream and one CUDA graph per
// frame.
#include "solver.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

namespace xpbd {

void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
    if (e == cudaSuccess) return;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "CUDA error %d (%s) at %s:%d: %s", (int)e, cudaGetErrorString(e), file, line,
                  what);
    throw std::runtime_error(buf);
}

namespace {
// profiler stage slots, one per kernel (names follow scene.cpp:1481-1505 where they correspond)
enum ProfSlot {
    P_CLEAR = 0, P_CONTACT, P_INTEGRATE_KEYS, P_SORT0, P_SORT1, P_SORT2, P_SORT3, P_RANKS, P_CELLS, P_SOLVE,
    P_BODY_CONTACT, P_BODY_ENTRIES, P_BODY_INTEGRATE, P_BODY_ITER, P_RESTITUTION, P_POSED, P_RIGID,
    P_BODY_RIGID_ITER, P_COUNT
};
static_assert(P_COUNT <= Solver::kMaxStages, "profiler stage table too small");
const char* kProfNames[P_COUNT] = {
    "0. Sort scratch clear (memset)", "1. Contact Gen (plane + mesh)", "2b. Integrate + Cell Keys",
    "2e. Onesweep Pass 0", "2e. Onesweep Pass 1", "2e. Onesweep Pass 2", "2e. Onesweep Pass 3",
    "1b. Contact Ranks (cap)", "2g. Cell Table + Gather", "3. Solve+Apply(+Restitution)",
    "1c. Body Pairs (world boxes)", "1f. Body Delta Entries (scan, sort)", "2c. Integrate Bodies",
    "3b. Body Deltas (particle contacts)", "3c. Restitution (bodies)", "1d. Contacts on Moving Meshes",
    "1e. Rigid Contacts", "3d. Body Deltas (rigid contacts)"};
uint32_t f2u(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
float u2f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
bool env_on(const char* name) {
    const char* e = std::getenv(name);
    return e && (std::strcmp(e, "1") == 0 || std::strcmp(e, "true") == 0);
}
}  // namespace

Solver::Solver() = default;

Solver::~Solver() {
    if (!initialized_) return;
    cudaSetDevice(device_);
    try {
        recorder_.stop();
    } catch (...) {
    }
    if (stream_) cudaStreamSynchronize(stream_);
    if (profiling_) print_profiler_summary();
    clear_graphs();
    if (pinned_) cudaFreeHost(pinned_);
    if (stream_) cudaStreamDestroy(stream_);
    if (aux_) cudaStreamDestroy(aux_);
    if (walk_stream_) cudaStreamDestroy(walk_stream_);
    if (fork_) cudaEventDestroy(fork_);
    if (join_) cudaEventDestroy(join_);
    if (triaged_) cudaEventDestroy(triaged_);
    if (walked_) cudaEventDestroy(walked_);
    for (auto& e : split_ev_)
        for (auto& x : e)
            if (x) cudaEventDestroy(x);
}

void Solver::require_init() const {
    if (!initialized_) throw std::runtime_error("XpbdSolver not initialized");
}

void Solver::clear_graphs() {
    if (pending_substeps_ && stream_) cudaStreamSynchronize(stream_);
    for (auto& kv : graphs_) {
        cudaGraphExecDestroy(kv.second.exec);
        for (auto& m : kv.second.marks) cudaEventDestroy(m.first);
    }
    graphs_.clear();
    clear_backward_graphs();
    split_choice_ = split_forced_;
    split_trials_ = 0;
}

void Solver::clear_backward_graphs() {
    for (auto& kv : bwd_graphs_) cudaGraphExecDestroy(kv.second);
    bwd_graphs_.clear();
}

void Solver::init(const xpbd_config& cfg, size_t num_particles, size_t max_contacts) {
    init_batched(cfg, &num_particles, 1, max_contacts);
}

void Solver::init_batched(const xpbd_config& cfg, const size_t* scene_counts, size_t n_scenes, size_t max_contacts) {
    if (initialized_) throw std::runtime_error("XpbdSolver::init called twice");
    if (n_scenes < 1 || n_scenes > 2048) throw std::runtime_error("init: between 1 and 2048 scenes");
    cfg_ = cfg;
    scene_off_.assign(n_scenes + 1, 0);
    for (size_t s = 0; s < n_scenes; s++) scene_off_[s + 1] = scene_off_[s] + scene_counts[s];
    const size_t num_particles = scene_off_[n_scenes];
    n_ = num_particles;
    solve_form_ = default_solve_form();
    contact_max_ = (int64_t)(max_contacts ? max_contacts : num_particles * 2);  // scene.cpp:68
    key_bits_ = 21;
    while (n_scenes > 1 && (size_t(1) << (key_bits_ - 21)) < n_scenes) key_bits_++;
    split_keys_ = n_scenes == 1 && (num_particles >= kSplitKeysMinParticles || env_on("VKXPBD_SPLIT_KEYS"));
    if (split_keys_) key_bits_ = kSplitKeyBits;
    int ndev = 0;
    XPBD_CUDA(cudaGetDeviceCount(&ndev));
    if (ndev == 0) throw std::runtime_error("no CUDA device");
    device_ = cfg.device_index >= 0 ? cfg.device_index : 0;
    if (device_ >= ndev) throw std::runtime_error("device_index out of range");
    XPBD_CUDA(cudaSetDevice(device_));
    XPBD_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    XPBD_CUDA(cudaStreamCreateWithFlags(&aux_, cudaStreamNonBlocking));
    XPBD_CUDA(cudaStreamCreateWithFlags(&walk_stream_, cudaStreamNonBlocking));
    XPBD_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
    XPBD_CUDA(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
    XPBD_CUDA(cudaEventCreateWithFlags(&triaged_, cudaEventDisableTiming));
    XPBD_CUDA(cudaEventCreateWithFlags(&walked_, cudaEventDisableTiming));

    for (int p = 0; p < 2; p++) {
        x_[p].alloc(n_);
        v_[p].alloc(n_);
        rx_[p].alloc(n_);
        rv_[p].alloc(n_);
    }
    pp_.alloc(n_);
    w_.alloc(n_);
    r_.alloc(n_);
    flags_.alloc(n_);
    rf_.alloc(n_);
    keys_.alloc(n_);
    for (int p = 0; p < 2; p++) {
        pair_k_[p].alloc(n_);
        pair_v_[p].alloc(n_);
    }
    if (n_scenes > 1) {
        std::vector<uint32_t> ps(n_);
        for (size_t s = 0; s < n_scenes; s++)
            for (size_t i = scene_off_[s]; i < scene_off_[s + 1]; i++) ps[i] = (uint32_t)s;
        pscene_.alloc(n_, false);
        if (n_) XPBD_CUDA(cudaMemcpy(pscene_.p, ps.data(), n_ * 4, cudaMemcpyHostToDevice));
    }
    // digit width 8, 16 keys per thread above 1M particles, 8 below (more tiles per SM);
    // scenes of 1M particles and more are re-tuned on their first step (autotune_sort)
    apply_sort_plan(8, n_ >= (1u << 20) ? 16 : 8);
    table_.alloc(split_keys_ ? (size_t(1) << kSplitKeyBits) : (size_t)n_scenes * kNumCells);
    stamp_.alloc(1);
    cinfo_.alloc(n_);
    near_.alloc(n_, false);
    slot_cap_ = 1;
    cslot_.alloc(std::max<size_t>(n_, 1) * 3);
    ensure_substep_capacity(16);
    rank_.alloc(n_);
    totals_.alloc(2);
    scan_ws_.alloc(contact_scan_words((int64_t)n_));
    status_.alloc(1);
    diag_header_.alloc(2);
    xyz_stage_.alloc(std::max<size_t>(n_, 1) * 3);
    pinned_words_ = 64;  // the per-frame readback (contact count, status)
    XPBD_CUDA(cudaMallocHost(&pinned_, pinned_words_ * sizeof(float)));
    if (cfg_.enable_diagnostics) {
        delta_.alloc(std::max<size_t>(n_, 1) * 3);
        uint32_t mp = cfg_.max_diag_pairs ? cfg_.max_diag_pairs : 100000u;
        diag_pairs_.alloc((size_t)mp * 20);
    }
    profiling_ = cfg_.enable_profile || env_on("VKXPBD_PROFILE");
    if (profiling_) std::printf("[Newton GB300] GPU profiler ENABLED (CUDA events)\n");
    initialized_ = true;
}

void Solver::apply_sort_plan(int bits, int items) {
    plan_ = make_sort_plan((int64_t)n_, key_bits_, bits, items);
    hist_off_ = 0;
    lb_off_ = (size_t)plan_.passes << plan_.bits;
    tc_off_ = lb_off_ + (size_t)plan_.passes * sort_lookback_words(plan_);
    cq_off_ = tc_off_ + (size_t)plan_.passes;  // collision work counter, near-list and posed-list lengths
    sort_scratch_.alloc(cq_off_ + 3);
    // the final sort buffer doubles as the collision pass's thread -> particle order (any
    // permutation gives the same contacts)
    launch_iota(stream_, (int64_t)n_, pair_v_[(plan_.passes - 1) & 1].p);
    XPBD_CUDA(cudaStreamSynchronize(stream_));
    clear_graphs();
}

// Times every onesweep variant (digit width, keys per thread) on this scene's own keys
// and keeps the fastest; the sort is stable, so the choice never changes a result.
std::vector<double> Solver::autotune_sort(int* best_bits, int* best_items) {
    require_init();
    sync();
    static const int kCand[][2] = {{8, 2}, {8, 4}, {8, 8}, {8, 16}, {7, 4}, {7, 8}, {7, 16}, {7, 32}};
    std::vector<double> us;
    double best = 1e30;
    int bb = plan_.bits, bi = plan_.items;
    cudaEvent_t e0, e1;
    XPBD_CUDA(cudaEventCreate(&e0));
    XPBD_CUDA(cudaEventCreate(&e1));
    const PredictParams pp = predict_params(cfg_.dt / (float)std::max(1, cfg_.substeps));
    PlaneParams pl{0, 0.0f, 0.0f};
    for (const auto& c : kCand) {
        apply_sort_plan(c[0], c[1]);
        double t_best = 1e30;
        for (int rep = 0; rep < 3; rep++) {
            XPBD_CUDA(cudaMemsetAsync(sort_scratch_.p, 0, sort_scratch_.bytes(), stream_));
            launch_predict_keys(stream_, (int64_t)n_, x_[cur_].p, v_[cur_].p, w_.p, r_.p, flags_.p, pscene_.p, pp,
                                pl, keys_.p, plan_, sort_scratch_.p + hist_off_, nullptr, nullptr, stamp_.p);
            XPBD_CUDA(cudaEventRecord(e0, stream_));
            const uint32_t* kin = keys_.p;
            const uint32_t* vin = nullptr;
            const size_t lbw = sort_lookback_words(plan_);
            for (int p = 0; p < plan_.passes; p++) {
                launch_onesweep_pass(stream_, (int64_t)n_, plan_, p, kin, vin, pair_k_[p & 1].p, pair_v_[p & 1].p,
                                     sort_scratch_.p + hist_off_ + ((size_t)p << plan_.bits),
                                     sort_scratch_.p + lb_off_ + (size_t)p * lbw, sort_scratch_.p + tc_off_ + p,
                                     status_.p);
                kin = pair_k_[p & 1].p;
                vin = pair_v_[p & 1].p;
            }
            XPBD_CUDA(cudaEventRecord(e1, stream_));
            XPBD_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            XPBD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            t_best = std::min(t_best, (double)ms * 1e3);
        }
        us.push_back(t_best);
        if (t_best < best) {
            best = t_best;
            bb = c[0];
            bi = c[1];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply_sort_plan(bb, bi);
    finish_frame(1);  // a device error of the trial sorts is raised here
    sort_tuned_ = true;
    if (best_bits) *best_bits = bb;
    if (best_items) *best_items = bi;
    return us;
}

void Solver::set_solve_split(int mode) {
    require_init();
    if (mode < -1 || mode > 1) throw std::runtime_error("set_solve_split: -1 (timed choice), 0 (fused) or 1 (split)");
    sync();
    split_forced_ = mode;
    split_choice_ = mode;
    split_trials_ = 0;
}

void Solver::set_solve_form(int form) {
    require_init();
    if (form < -1 || form >= kSolveForms) throw std::runtime_error("set_solve_form: -1 (timed choice), 0, 1, 2 or 3");
    sync();
    solve_form_forced_ = form;
    solve_form_ = form >= 0 ? form : default_solve_form();
    solve_form_timed_ = false;
}

// Times every form of the solve kernel on the last substep of the last frame: its last
// iteration is launched again on the records, cell table and contacts still in memory, with
// its outputs in scratch buffers (the records of the other iteration parity, which that
// iteration does not read, and the body-delta entries, which the next frame rebuilds), so the
// state is untouched. The fastest form is kept; every form gives the same bits.
void Solver::autotune_solve() {
    sync();
    const int it = last_iterations_ - 1;
    SolveParams sp = solve_params(last_sdt_, it);
    if (dyn_any_) sp.enable_restitution = 0;
    ContactRanks cr{nullptr, nullptr};
    if (need_ranks_) {
        cr.rank = rank_.p;
        cr.totals = totals_.p;
        cr.count = ccount_.p + (last_substeps_ - 1);
    }
    const uint32_t* sids = pair_v_[(plan_.passes - 1) & 1].p;
    const uint32_t* skeys = pscene_.p ? pair_k_[(plan_.passes - 1) & 1].p : nullptr;
    const int src = last_collide_src_;
    const BodyDeltaOut bo{dyn_any_ ? bdel_.p : nullptr, dyn_any_ ? dyn_rank_.p : nullptr};
    const SolveDiag dg{nullptr, nullptr, nullptr, 0};
    float4* sx = rx_[(it + 1) & 1].p;  // scratch outputs
    float4* sv = rv_[(it + 1) & 1].p;
    // two timed rounds, forms in opposite orders (a drift cancels); the first timing of a
    // solver has a warm-up round before them (first launches load the kernels)
    constexpr int kReps = 2;
    cudaEvent_t ev[2 * kSolveTimedForms * kReps];
    for (auto& e : ev) XPBD_CUDA(cudaEventCreate(&e));
    for (int rep = solve_form_timed_ ? 1 : 0; rep <= kReps; rep++) {
        for (int k = 0; k < kSolveTimedForms; k++) {
            const int f = (rep & 1) ? k : kSolveTimedForms - 1 - k;
            cudaEvent_t* e = ev + 2 * (f * kReps + std::max(rep - 1, 0));
            if (rep) XPBD_CUDA(cudaEventRecord(e[0], stream_));
            launch_solve(stream_, (int64_t)n_, true, all_active_, sids, skeys, rx_[it & 1].p, rv_[it & 1].p, rf_.p,
                         table_.p, stamp_.p, x_[src].p, v_[src].p, cinfo_.p, cslot_.p, cr, body_tables(), sp,
                         nullptr, nullptr, sx, sv, dg, bo, 0, nullptr, f);
            if (rep) XPBD_CUDA(cudaEventRecord(e[1], stream_));
        }
    }
    XPBD_CUDA(cudaGetLastError());
    XPBD_CUDA(cudaStreamSynchronize(stream_));
    double ms[kSolveTimedForms] = {0.0};
    for (int f = 0; f < kSolveTimedForms; f++)
        for (int r = 0; r < kReps; r++) {
            float t = 0.0f;
            XPBD_CUDA(cudaEventElapsedTime(&t, ev[2 * (f * kReps + r)], ev[2 * (f * kReps + r) + 1]));
            ms[f] += t;
        }
    for (auto& e : ev) cudaEventDestroy(e);
    int best = solve_form_timed_ && solve_form_ < kSolveTimedForms ? solve_form_ : 0;  // the form in use
    for (int f = 0; f < kSolveTimedForms; f++)
        if (f != best && ms[f] < ms[best] * 0.98) best = f;
    solve_form_ = best;
    solve_form_timed_ = true;
    solve_form_frame_ = frames_run_;
}

void Solver::set_sort_variant(int bits, int items) {
    require_init();
    sync();
    if (!((bits == 8 && (items == 2 || items == 4 || items == 8 || items == 16)) ||
          (bits == 7 && (items == 4 || items == 8 || items == 16 || items == 32))))
        throw std::runtime_error("set_sort_variant: bits 8 with 2, 4, 8 or 16 keys per thread, or bits 7 with 4, 8, "
                                 "16 or 32");
    apply_sort_plan(bits, items);
    sort_tuned_ = true;  // an explicit choice is kept
}

void Solver::ensure_substep_capacity(int substeps) {
    if (substeps <= ccount_cap_) return;
    int cap = std::max(substeps, 16);
    ccount_.alloc((size_t)cap);
    ccount_cap_ = cap;
    clear_graphs();
}

void Solver::add_mesh(const float* verts, size_t num_verts, const uint32_t* tris, size_t num_tris,
                      float shape_margin, const float* rot, int wt_override) {
    MeshData md;
    md.vertices.assign(verts, verts + num_verts * 3);
    md.indices.assign(tris, tris + num_tris * 3);
    md.shape_margin = shape_margin;
    if (rot) std::memcpy(md.shape_rot, rot, sizeof(float) * 4);
    md.is_watertight = wt_override >= 0 ? (wt_override != 0) : tris_watertight(tris, num_tris, num_verts);
    for (size_t i = 0; i < num_tris * 3; i++)
        if (tris[i] >= num_verts) throw std::runtime_error("add_mesh: triangle index out of range");
    meshes_.push_back(std::move(md));
    finalized_ = false;
}

void Solver::finalize_meshes() {
    if (!initialized_) throw std::runtime_error("XpbdSolver::init must be called before finalize_meshes");
    XPBD_CUDA(cudaSetDevice(device_));
    dyn_tables_ready_ = false;
    const size_t nm = meshes_.size(), nshapes = 1 + nm;
    // shapes: 0 = plane (body -1), c+1 = mesh c (body c); all bodies static (scene.cpp:206-247)
    std::vector<int> sb(nshapes);
    std::vector<float> smu(nshapes, cfg_.shape_material_mu);
    sb[0] = -1;
    for (size_t c = 0; c < nm; c++) sb[1 + c] = (int)c;
    shape_body_.alloc(nshapes);
    shape_mu_.alloc(nshapes);
    XPBD_CUDA(cudaMemcpy(shape_body_.p, sb.data(), nshapes * sizeof(int), cudaMemcpyHostToDevice));
    XPBD_CUDA(cudaMemcpy(shape_mu_.p, smu.data(), nshapes * sizeof(float), cudaMemcpyHostToDevice));
    const size_t nb = std::max<size_t>(nm, 1);
    std::vector<float4> bq(nb * 2, make_float4(0, 0, 0, 0));
    for (size_t b = 0; b < nb; b++) bq[b * 2 + 1] = make_float4(0, 0, 0, 1);
    body_q_.alloc(nb * 2);
    XPBD_CUDA(cudaMemcpy(body_q_.p, bq.data(), bq.size() * sizeof(float4), cudaMemcpyHostToDevice));
    body_qd_.alloc(nb * 2);
    body_com_.alloc(nb * 3);
    body_invI_.alloc(nb * 9);
    body_invm_.alloc(nb);
    body_flags_.alloc(nb);
    body_I_.alloc(nb * 9);
    dyn_any_ = false;
    dyn_list_.clear();

    // concatenated vertex / triangle arrays, then one LBVH per mesh built on the GPU
    // straight into the packed global node arrays (scene.cpp:249-386)
    all_verts_.clear();
    std::vector<uint32_t> all_tris;
    vert_offsets_.assign(nm, 0);
    node_offsets_.assign(nm, 0);
    prim_offsets_.assign(nm, 0);
    size_t total_nodes = 0, total_prims = 0;
    for (size_t c = 0; c < nm; c++) {
        MeshData& m = meshes_[c];
        const uint32_t vo = (uint32_t)(all_verts_.size() / 3);
        vert_offsets_[c] = vo;
        all_verts_.insert(all_verts_.end(), m.vertices.begin(), m.vertices.end());
        const size_t to = all_tris.size() / 3;
        for (uint32_t t : m.indices) all_tris.push_back(t + vo);
        const size_t nt = m.indices.size() / 3;
        if (nt == 0) throw std::runtime_error("add_mesh: mesh has no triangles");
        double sum_len = 0.0;  // scene.cpp:274-281
        for (size_t t = 0; t < nt; t++)
            for (int e = 0; e < 3; e++) {
                const uint32_t i0 = all_tris[(to + t) * 3 + e], i1 = all_tris[(to + t) * 3 + (e + 1) % 3];
                const float dx = all_verts_[i1 * 3] - all_verts_[i0 * 3];
                const float dy = all_verts_[i1 * 3 + 1] - all_verts_[i0 * 3 + 1];
                const float dz = all_verts_[i1 * 3 + 2] - all_verts_[i0 * 3 + 2];
                sum_len += std::sqrt(dx * dx + dy * dy + dz * dz);
            }
        m.avg_edge = (float)(sum_len / (double)(nt * 3));
        node_offsets_[c] = total_nodes;
        prim_offsets_[c] = total_prims;
        total_nodes += 2 * nt;
        total_prims += nt;
    }
    all_vels_.assign(all_verts_.size(), 0.0f);
    // contact slots per particle: one per mesh up to 8; 16 when there are more meshes (bodies)
    slot_cap_ = (int)std::max<size_t>(1, nm <= 8 ? nm : 16);
    cslot_.alloc(std::max<size_t>(n_, 1) * (size_t)slot_cap_ * 3, false);
    if (nm > 0) {
        std::vector<uint32_t> poff(nm), pcnt(nm);
        std::vector<float> margins(nm);
        std::vector<int> wt(nm);
        size_t max_nt = 0;
        for (size_t c = 0; c < nm; c++) {
            const size_t nt = meshes_[c].indices.size() / 3;
            poff[c] = (uint32_t)prim_offsets_[c];
            pcnt[c] = (uint32_t)nt;
            margins[c] = meshes_[c].shape_margin;
            wt[c] = meshes_[c].is_watertight ? 1 : 0;
            max_nt = std::max(max_nt, nt);
        }
        auto up = [&](auto& dev, const auto& host) {
            dev.alloc(host.size(), false);
            XPBD_CUDA(cudaMemcpy(dev.p, host.data(), host.size() * sizeof(host[0]), cudaMemcpyHostToDevice));
        };
        up(prim_off_, poff);
        up(prim_cnt_, pcnt);
        up(margins_, margins);
        up(watertight_, wt);
        up(verts_, all_verts_);
        up(vels_, all_vels_);
        up(tris_, all_tris);
        nl_.alloc(total_nodes, false);
        nu_.alloc(total_nodes, false);
        prim_.alloc(total_prims, false);
        roots_.alloc(nm, false);
        topo_parent_.alloc(total_nodes, false);
        topo_child_l_.alloc(total_nodes, true);
        topo_child_r_.alloc(total_nodes, true);
        topo_marked_.alloc(total_nodes, false);
        topo_reachable_.alloc(total_nodes, false);
        topo_prim_.alloc(total_prims, false);
        bvh_scratch_.alloc(lbvh_scratch_words((int)max_nt), false);
        for (size_t c = 0; c < nm; c++)
            launch_lbvh_build(stream_, (int)pcnt[c], verts_.p, tris_.p + (size_t)prim_offsets_[c] * 3,
                              (uint32_t)node_offsets_[c], (uint32_t)prim_offsets_[c], (uint32_t)prim_offsets_[c],
                              nl_.p, nu_.p, prim_.p, roots_.p + c, topology(c), bvh_scratch_.p, status_.p);
        std::vector<uint32_t> noff(nm + 1);
        for (size_t c = 0; c < nm; c++) noff[c] = (uint32_t)node_offsets_[c];
        noff[nm] = (uint32_t)total_nodes;
        up(node_off_dev_, noff);
        cull_dirty_ = true;
        node_pair_.alloc(total_nodes * 4, false);
        for (size_t c = 0; c < nm; c++)
            launch_node_pairs(stream_, (int)pcnt[c], (uint32_t)node_offsets_[c], topo_reachable_.p + node_offsets_[c],
                              nl_.p, nu_.p, node_pair_.p);
        avg_edge0_ = meshes_[0].avg_edge;  // mesh 0's average edge for every mesh (scene.cpp:325)
        tri_cache_.alloc(total_prims * 4, false);
        launch_tri_cache(stream_, 0, (int64_t)total_prims, prim_.p, tris_.p, verts_.p, tri_cache_.p);
        XPBD_CUDA(cudaStreamSynchronize(stream_));
    }
    const int64_t possible = (int64_t)n_ * ((cfg_.has_ground_plane ? 1 : 0) + (int64_t)nm);
    need_ranks_ = possible > contact_max_;
    clear_graphs();
    finalized_ = true;
}

void Solver::set_particles(const float* q, const float* qd, const float* inv_mass, const float* radii,
                           const int32_t* flags, size_t n) {
    if (!initialized_) throw std::runtime_error("XpbdSolver not initialized");
    if (n != n_) throw std::runtime_error("Particle count mismatch");
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    rollout_valid_ = false;
    if (n == 0) return;
    upload_xyz(q, x_[cur_].p, n);
    if (qd)
        upload_xyz(qd, v_[cur_].p, n);
    else
        XPBD_CUDA(cudaMemsetAsync(v_[cur_].p, 0, n * sizeof(float4), stream_));
    XPBD_CUDA(cudaStreamSynchronize(stream_));
    auto up = [&](void* dst, const void* src) {
        XPBD_CUDA(cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyHostToDevice, stream_));
        XPBD_CUDA(cudaStreamSynchronize(stream_));
    };
    if (inv_mass) up(w_.p, inv_mass);
    if (radii) {
        up(r_.p, radii);
        float lo = 0.0f, hi = 0.0f;
        bool fin = true, first = true;
        for (size_t i = 0; i < n; i++) {
            if (!std::isfinite(radii[i])) {
                fin = false;
                continue;
            }
            lo = first ? radii[i] : std::min(lo, radii[i]);
            hi = first ? radii[i] : std::max(hi, radii[i]);
            first = false;
        }
        if (lo != r_min_ || hi != r_max_ || fin != r_finite_) {
            cull_dirty_ = true;
            if (hi != r_max_) clear_graphs();  // the frame graphs carry the box grid's reach
        }
        r_min_ = lo;
        r_max_ = hi;
        r_finite_ = fin;
    }
    if (flags) {
        up(flags_.p, flags);
        bool all = true;
        for (size_t i = 0; i < n && all; i++) all = (flags[i] & 3) == 1;
        if (all != all_active_) clear_graphs();  // the graphs bake in the all-active kernel variant
        all_active_ = all;
    }
}

void Solver::update_mesh(size_t mi, const float* verts, size_t num_verts, const float* vels) {
    if (!finalized_) throw std::runtime_error("update_mesh: call finalize_meshes() first");
    if (mi >= meshes_.size()) throw std::runtime_error("update_mesh: mesh_index out of range");
    MeshData& m = meshes_[mi];
    if (num_verts != m.vertices.size() / 3) throw std::runtime_error("update_mesh: vertex count mismatch");
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    const size_t vs = vert_offsets_[mi];
    std::memcpy(all_verts_.data() + vs * 3, verts, num_verts * 3 * sizeof(float));
    if (vels)
        std::memcpy(all_vels_.data() + vs * 3, vels, num_verts * 3 * sizeof(float));
    else
        std::fill(all_vels_.begin() + vs * 3, all_vels_.begin() + (vs + num_verts) * 3, 0.0f);
    std::copy(verts, verts + num_verts * 3, m.vertices.begin());
    dyn_tables_ready_ = false;  // a dynamic mesh's extent sizes the box grid: the next set_bodies rebuilds
    // upload this mesh's vertices, then refit its BVH on the GPU (topology unchanged,
    // scene.cpp:657-695 refits on the host and re-uploads every node)
    const size_t nb = node_offsets_[mi], pb = prim_offsets_[mi], nt = m.indices.size() / 3;
    XPBD_CUDA(cudaMemcpyAsync(verts_.p + vs * 3, verts, num_verts * 3 * sizeof(float), cudaMemcpyHostToDevice,
                              stream_));
    XPBD_CUDA(cudaMemcpyAsync(vels_.p + vs * 3, all_vels_.data() + vs * 3, num_verts * 3 * sizeof(float),
                              cudaMemcpyHostToDevice, stream_));
    launch_lbvh_refit(stream_, (int)nt, verts_.p, tris_.p + pb * 3, topology(mi), nl_.p + nb, nu_.p + nb,
                      bvh_scratch_.p);
    launch_node_pairs(stream_, (int)nt, (uint32_t)nb, topo_reachable_.p + nb, nl_.p, nu_.p, node_pair_.p);
    launch_tri_cache(stream_, (int64_t)pb, (int64_t)nt, prim_.p, tris_.p, verts_.p, tri_cache_.p);
    cull_dirty_ = true;
    XPBD_CUDA(cudaStreamSynchronize(stream_));
}

PredictParams Solver::predict_params(float sdt) const {
    PredictParams p;
    p.dt = sdt;
    p.v_max = cfg_.particle_v_max;
    p.gx = cfg_.gravity[0];
    p.gy = cfg_.gravity[1];
    p.gz = cfg_.gravity[2];
    p.inv = 1.0f / cfg_.search_radius;
    p.split_keys = split_keys_ ? 1 : 0;
    return p;
}

SolveParams Solver::solve_params(float sdt, int it) const {
    SolveParams s;
    s.dt = sdt;
    s.relax = cfg_.soft_contact_relaxation;
    s.v_max = cfg_.particle_v_max;
    s.inv = 1.0f / cfg_.search_radius;
    s.max_radius = cfg_.particle_max_radius;
    s.k_mu = cfg_.particle_mu;
    s.k_coh = cfg_.particle_cohesion;
    s.soft_mu = cfg_.soft_contact_mu;
    s.ka = cfg_.particle_adhesion;
    s.restitution = cfg_.soft_contact_restitution;
    s.enable_restitution = cfg_.enable_restitution ? 1 : 0;
    s.altitude = cfg_.ground_plane_altitude;
    s.slot_cap = injected_ ? inj_cap_ : slot_cap_;
    s.iter_index = it;
    s.contact_max = contact_max_;
    s.split_keys = split_keys_ ? 1 : 0;
    return s;
}

BodyTables Solver::body_tables() const {
    BodyTables b;
    b.shape_body = shape_body_.p;
    b.shape_mu = shape_mu_.p;
    b.body_q = body_q_.p;
    b.body_qd = body_qd_.p;
    b.body_com = body_com_.p;
    b.body_invI = body_invI_.p;
    b.body_invm = body_invm_.p;
    b.body_flags = body_flags_.p;
    b.body_q_prev = dyn_any_ ? body_q_prev_.p : body_q_.p;
    b.body_qd_prev = dyn_any_ ? body_qd_prev_.p : body_qd_.p;
    return b;
}

BodyArrays Solver::body_arrays() const {
    BodyArrays a;
    a.q = body_q_.p;
    a.qd = body_qd_.p;
    a.com = body_com_.p;
    a.I = body_I_.p;
    a.invI = body_invI_.p;
    a.invm = body_invm_.p;
    a.flags = body_flags_.p;
    a.shape_body = shape_body_.p;
    a.shape_mu = shape_mu_.p;
    a.nb = (int)meshes_.size();
    return a;
}

RigidTables Solver::rigid_tables() const {
    RigidTables t;
    t.n_dyn = (int)dyn_list_.size();
    t.dyn = dyn_.p;
    t.dyn_index = dyn_index_.p;
    t.dv_start = dv_start_.p;
    t.dv_local = dv_local_.p;
    t.wbox = wbox_.p;
    t.partners = partners_.p;
    t.partner_count = partner_count_.p;
    t.rc = rc_.p;
    t.rc_count = rc_count_.p;
    t.pad = 1e-3f;
    t.n_vert = n_dyn_verts_;
    t.dyn_scene = dyn_scene_.p;
    t.pscene = pscene_.p;
    // box grid: a particle's side of the widening (soft margin + radius + pad, radii bounded
    // by the larger of particle_max_radius and the largest finite radius set); cells
    // 1 / (kBoxAxis - 1) of the largest widened box, so a box covers at most kBoxAxis cells
    // per axis
    t.grid_size = grid_size_;
    t.grid_reach = cfg_.soft_contact_margin + std::max(cfg_.particle_max_radius, r_max_) + 2.0f * t.pad;
    t.grid_cs =
        (2.0f * dyn_half_diag_ + 2.0f * (t.grid_reach + dyn_max_margin_)) * 1.01f / (float)(kBoxAxis - 1) + 1e-4f;
    t.grid_count = grid_count_.p;
    t.grid_start = grid_start_.p;
    t.grid_tiles = grid_tiles_.p;
    t.grid_list = grid_list_.p;
    return t;
}

RigidParams Solver::rigid_params(float sdt) const {
    RigidParams r;
    r.dt = sdt;
    r.damping = body_params_.angular_damping;
    r.margin = body_params_.rigid_contact_margin;
    r.relax = body_params_.rigid_contact_relaxation;
    r.con_weighting = body_params_.rigid_contact_con_weighting;
    r.mu_t = body_params_.rigid_mu_torsional;
    r.mu_r = body_params_.rigid_mu_rolling;
    r.particle_weighting = body_params_.particle_contact_con_weighting;
    r.gx = cfg_.gravity[0];
    r.gy = cfg_.gravity[1];
    r.gz = cfg_.gravity[2];
    r.plane = cfg_.has_ground_plane ? 1 : 0;
    r.altitude = cfg_.ground_plane_altitude;
    return r;
}

void Solver::set_body_params(const xpbd_body_params& p) {
    body_params_ = p;
    clear_graphs();
}

// Scene of each body in a batched solver (-1: shared by every scene, for static
// bodies). A dynamic body meets only the particles and dynamic bodies of its scene.
void Solver::set_body_scenes(const int32_t* scenes, size_t nb) {
    if (!finalized_) throw std::runtime_error("set_body_scenes: call finalize_meshes() first");
    if (nb != meshes_.size()) throw std::runtime_error("set_body_scenes: one scene per mesh");
    const int ns = (int)scene_off_.size() - 1;
    for (size_t b = 0; b < nb; b++)
        if (scenes[b] < -1 || scenes[b] >= ns) throw std::runtime_error("set_body_scenes: scene out of range");
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    body_scene_.assign(scenes, scenes + nb);
    if (dyn_any_) upload_dyn_scenes();
    clear_graphs();
}

void Solver::upload_dyn_scenes() {
    std::vector<int> ds(std::max<size_t>(dyn_list_.size(), 1), 0);
    for (size_t k = 0; k < dyn_list_.size(); k++) {
        const int b = dyn_list_[k];
        ds[k] = (size_t)b < body_scene_.size() ? body_scene_[b] : 0;
        if (ds[k] < 0)
            throw std::runtime_error("set_body_scenes: a dynamic body needs a scene (-1 is for static bodies)");
    }
    dyn_scene_.alloc(ds.size(), false);
    XPBD_CUDA(cudaMemcpy(dyn_scene_.p, ds.data(), ds.size() * sizeof(int), cudaMemcpyHostToDevice));
}

void Solver::set_bodies(const float* q, const float* qd, const float* com, const float* inertia,
                        const float* inv_inertia, const float* inv_mass, const int32_t* flags, size_t nb) {
    if (!finalized_) throw std::runtime_error("set_bodies: call finalize_meshes() first");
    if (nb != meshes_.size()) throw std::runtime_error("set_bodies: one body per mesh");
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    if (nb == 0) return;
    std::vector<float4> hq(nb * 2), hqd(nb * 2);
    std::vector<float> hcom(nb * 3), hI(nb * 9), hinvI(nb * 9), hinvm(nb);
    std::vector<int> hfl(nb);
    XPBD_CUDA(cudaMemcpy(hq.data(), body_q_.p, nb * 2 * sizeof(float4), cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(hqd.data(), body_qd_.p, nb * 2 * sizeof(float4), cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(hcom.data(), body_com_.p, nb * 3 * 4, cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(hI.data(), body_I_.p, nb * 9 * 4, cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(hinvI.data(), body_invI_.p, nb * 9 * 4, cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(hinvm.data(), body_invm_.p, nb * 4, cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(hfl.data(), body_flags_.p, nb * 4, cudaMemcpyDeviceToHost));
    for (size_t b = 0; b < nb; b++) {
        if (q) {  // (pos xyz, quat xyzw)
            hq[b * 2] = make_float4(q[b * 7], q[b * 7 + 1], q[b * 7 + 2], 0.0f);
            hq[b * 2 + 1] = make_float4(q[b * 7 + 3], q[b * 7 + 4], q[b * 7 + 5], q[b * 7 + 6]);
        }
        if (qd) {  // (linear, angular)
            hqd[b * 2] = make_float4(qd[b * 6], qd[b * 6 + 1], qd[b * 6 + 2], 0.0f);
            hqd[b * 2 + 1] = make_float4(qd[b * 6 + 3], qd[b * 6 + 4], qd[b * 6 + 5], 0.0f);
        }
        if (com) std::memcpy(&hcom[b * 3], com + b * 3, 12);
        if (inertia) std::memcpy(&hI[b * 9], inertia + b * 9, 36);
        if (inv_inertia) std::memcpy(&hinvI[b * 9], inv_inertia + b * 9, 36);
        if (inv_mass) hinvm[b] = inv_mass[b];
        if (flags) hfl[b] = flags[b];
    }
    XPBD_CUDA(cudaMemcpy(body_q_.p, hq.data(), nb * 2 * sizeof(float4), cudaMemcpyHostToDevice));
    XPBD_CUDA(cudaMemcpy(body_qd_.p, hqd.data(), nb * 2 * sizeof(float4), cudaMemcpyHostToDevice));
    XPBD_CUDA(cudaMemcpy(body_com_.p, hcom.data(), nb * 3 * 4, cudaMemcpyHostToDevice));
    XPBD_CUDA(cudaMemcpy(body_I_.p, hI.data(), nb * 9 * 4, cudaMemcpyHostToDevice));
    XPBD_CUDA(cudaMemcpy(body_invI_.p, hinvI.data(), nb * 9 * 4, cudaMemcpyHostToDevice));
    XPBD_CUDA(cudaMemcpy(body_invm_.p, hinvm.data(), nb * 4, cudaMemcpyHostToDevice));
    XPBD_CUDA(cudaMemcpy(body_flags_.p, hfl.data(), nb * 4, cudaMemcpyHostToDevice));

    // dynamic bodies: inverse mass > 0; their meshes are in the body frame
    std::vector<int> dyn_list, dyn_index(nb, -1), posed(nb, 0), walk;
    for (size_t b = 0; b < nb; b++) {
        if (hinvm[b] > 0.0f) {
            dyn_index[b] = (int)dyn_list.size();
            dyn_list.push_back((int)b);
            posed[b] = 1;
        } else {
            walk.push_back((int)b);
        }
    }
    // the same dynamic bodies as before over unchanged meshes (a new state of the same
    // scene): the tables, their buffers and the captured graphs stay; only the body arrays
    // above change, and the graphs read them from device memory
    if (dyn_tables_ready_ && dyn_list == dyn_list_) return;
    dyn_list_ = dyn_list;
    dyn_tables_ready_ = false;
    dyn_any_ = !dyn_list_.empty();
    clear_graphs();
    if (!dyn_any_) return;
    auto up = [&](auto& dev, const auto& host) {
        dev.alloc(std::max<size_t>(host.size(), 1), false);
        if (!host.empty())
            XPBD_CUDA(cudaMemcpy(dev.p, host.data(), host.size() * sizeof(host[0]), cudaMemcpyHostToDevice));
    };
    std::vector<uint32_t> dv_start(nb + 1, 0);
    std::vector<float4> dv_local;
    for (size_t b = 0; b < nb; b++) {
        dv_start[b] = (uint32_t)dv_local.size();
        if (!posed[b]) continue;
        const std::vector<float>& v = meshes_[b].vertices;
        for (size_t k = 0; k + 2 < v.size(); k += 3) {
            int bi = (int)b;
            float bw;
            std::memcpy(&bw, &bi, 4);
            dv_local.push_back(make_float4(v[k], v[k + 1], v[k + 2], bw));
        }
    }
    dv_start[nb] = (uint32_t)dv_local.size();
    n_dyn_verts_ = (int)dv_local.size();
    // largest half-diagonal of a dynamic mesh's body-frame box and largest shape margin
    dyn_half_diag_ = 0.0f;
    dyn_max_margin_ = 0.0f;
    for (int b : dyn_list_) {
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        const std::vector<float>& v = meshes_[b].vertices;
        for (size_t k = 0; k + 2 < v.size(); k += 3)
            for (int a = 0; a < 3; a++) {
                lo[a] = std::min(lo[a], v[k + a]);
                hi[a] = std::max(hi[a], v[k + a]);
            }
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        dyn_half_diag_ = std::max(dyn_half_diag_, 0.5f * std::sqrt(dx * dx + dy * dy + dz * dz));
        dyn_max_margin_ = std::max(dyn_max_margin_, meshes_[b].shape_margin);
    }
    grid_size_ = 64;
    while ((size_t)grid_size_ < (size_t)kBoxBuckets * dyn_list_.size()) grid_size_ *= 2;
    grid_count_.alloc((size_t)grid_size_, true);
    grid_start_.alloc((size_t)grid_size_ + 1, true);
    grid_tiles_.alloc((size_t)grid_size_ / 1024 + 1, true);
    if (grid_size_ > 4096 * 1024) throw std::runtime_error("too many dynamic bodies for the box grid");
    grid_list_.alloc(std::max<size_t>(dyn_list_.size() * kBoxCells, 1), true);
    if (n_ >= ((size_t)1 << 28)) throw std::runtime_error("dynamic bodies need fewer than 2^28 particles");
    posed_list_.alloc(std::max<size_t>(n_, 1) * kPosedListWords, false);
    posed_hits_.alloc(std::max<size_t>(n_, 1) * kPosedHitWords, false);
    up(dyn_, dyn_list_);
    up(dyn_index_, dyn_index);
    upload_dyn_scenes();
    up(posed_, posed);
    up(walk_list_, walk);
    walk_count_ = (int)walk.size();
    up(dv_start_, dv_start);
    up(dv_local_, dv_local);
    const size_t nd = dyn_list_.size();
    wbox_.alloc(nd * 2, true);
    partners_.alloc(nd * kPartnerCap, true);
    partner_count_.alloc(nd, true);
    rc_.alloc(std::max<size_t>((size_t)n_dyn_verts_, 1) * kRigidSlots * 5, true);
    rc_count_.alloc(std::max<size_t>((size_t)n_dyn_verts_, 1), true);
    body_q_mid_.alloc(nb * 2, true);
    body_qd_mid_.alloc(nb * 2, true);
    body_q_prev_.alloc(nb * 2, true);
    body_qd_prev_.alloc(nb * 2, true);
    // body-delta entries of the particle contacts: one per slot with a dynamic body
    entry_cap_ = (uint32_t)std::min<size_t>(2 * n_ + 4096, (size_t)0x7fffffff);
    int kb = 1;
    while ((size_t(1) << kb) < nb) kb++;
    eplan_ = make_sort_plan((int64_t)entry_cap_, kb, 8, 8);
    ehist_off_ = 0;
    elb_off_ = (size_t)eplan_.passes << eplan_.bits;
    etc_off_ = elb_off_ + (size_t)eplan_.passes * sort_lookback_words(eplan_);
    esort_scratch_.alloc(etc_off_ + (size_t)eplan_.passes, true);
    ekeys_.alloc(entry_cap_, false);
    for (int p = 0; p < 2; p++) {
        epk_[p].alloc(entry_cap_, false);
        epv_[p].alloc(entry_cap_, false);
    }
    seg_.alloc(nb, true);
    bdel_.alloc((size_t)entry_cap_ * 2, false);
    dyn_rank_.alloc(std::max<size_t>(n_, 1), false);
    dyn_totals_.alloc(2, true);
    dyn_ws_.alloc(contact_scan_words((int64_t)n_), true);
    dyn_tables_ready_ = true;
}

void Solver::get_bodies(float* q, float* qd, size_t nb) {
    require_init();
    if (nb != meshes_.size()) throw std::runtime_error("get_bodies: one body per mesh");
    sync();
    if (nb == 0) return;
    std::vector<float4> hq(nb * 2), hqd(nb * 2);
    XPBD_CUDA(cudaMemcpy(hq.data(), body_q_.p, nb * 2 * sizeof(float4), cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(hqd.data(), body_qd_.p, nb * 2 * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t b = 0; b < nb; b++) {
        if (q) {
            const float4 a = hq[b * 2], c = hq[b * 2 + 1];
            const float v[7] = {a.x, a.y, a.z, c.x, c.y, c.z, c.w};
            std::memcpy(q + b * 7, v, sizeof(v));
        }
        if (qd) {
            const float4 a = hqd[b * 2], c = hqd[b * 2 + 1];
            const float v[6] = {a.x, a.y, a.z, c.x, c.y, c.z};
            std::memcpy(qd + b * 6, v, sizeof(v));
        }
    }
}

// Reach grid of each mesh, in the mesh's own frame: cells of about a quarter of the
// reach, covering the mesh's vertex box padded by the reach plus slack. The reach
// bounds |margin + shape margin + r + eps| + |eps| over the particles' radii (both
// extremes, since the traversal squares the bound) with a relative and an absolute
// slack for rounding. A mesh gets no grid (is never culled) when a radius, the
// margin or a vertex is not finite, or once 2^23 words are spent.
void Solver::ensure_cull() {
    if (!cull_dirty_ || !finalized_) return;
    cull_dirty_ = false;
    const size_t nm = meshes_.size();
    if (nm == 0) return;
    const double eps = (double)(avg_edge0_ * 1e-3f);
    const bool ok = r_finite_ && std::isfinite(cfg_.soft_contact_margin) && std::isfinite(eps);
    std::vector<float4> org(nm, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    std::vector<int4> dim(nm, make_int4(0, 0, 0, 0));
    std::vector<uint32_t> off(nm + 1, 0);
    const uint64_t kMeshCells = 1ull << 24, kTotalWords = 1ull << 23;
    uint64_t words = 0;
    for (size_t c = 0; c < nm; c++) {
        off[c] = (uint32_t)words;
        off[c + 1] = (uint32_t)words;
        const MeshData& m = meshes_[c];
        const size_t v0 = vert_offsets_[c], nv = m.vertices.size() / 3;
        if (!ok || nv == 0 || !std::isfinite(m.shape_margin)) continue;
        double lo[3], hi[3], amax = 0.0;
        bool fin = true;
        for (int k = 0; k < 3; k++) lo[k] = hi[k] = all_verts_[v0 * 3 + k];
        for (size_t v = 0; v < nv; v++)
            for (int k = 0; k < 3; k++) {
                const double q = all_verts_[(v0 + v) * 3 + k];
                fin = fin && std::isfinite(q);
                lo[k] = std::min(lo[k], q);
                hi[k] = std::max(hi[k], q);
                amax = std::max(amax, std::fabs(q));
            }
        if (!fin) continue;
        const double base = (double)cfg_.soft_contact_margin + (double)m.shape_margin;
        const double reach =
            std::max(std::fabs(base + r_max_ + eps), std::fabs(base + r_min_ + eps)) + std::fabs(eps);
        const double R = reach * 1.001 + 1e-6 * (1.0 + amax);
        double ext = 0.0;
        for (int k = 0; k < 3; k++) ext = std::max(ext, hi[k] - lo[k]);
        double cell = std::max(R * 0.25, (ext + 2.0 * R) * 1e-4);
        int dims[3] = {0, 0, 0}, kd = 0;
        uint64_t cells = 0;
        for (int attempt = 0; attempt < 8; attempt++) {
            kd = (int)std::ceil(R / cell) + 1;
            const double pad = (kd + 2) * cell;
            cells = 1;
            for (int k = 0; k < 3; k++) {
                dims[k] = (int)std::ceil((hi[k] - lo[k] + 2.0 * pad) / cell) + 1;
                cells *= (uint64_t)dims[k];
            }
            if (cells <= kMeshCells) break;
            cell *= std::cbrt((double)cells / (double)kMeshCells) * 1.01;
        }
        const uint64_t w = (uint64_t)((dims[0] + 31) / 32) * (uint64_t)dims[1] * (uint64_t)dims[2];
        if (kd >= 32 || cells > kMeshCells || words + w > kTotalWords) continue;
        const double pad = (kd + 2) * cell;
        org[c] = make_float4((float)(lo[0] - pad), (float)(lo[1] - pad), (float)(lo[2] - pad), (float)(1.0 / cell));
        dim[c] = make_int4(dims[0], dims[1], dims[2], kd);
        words += w;
        off[c + 1] = (uint32_t)words;
    }
    if (words == 0) {
        if (cull_bits_.n) clear_graphs();  // the frame graphs hold the grid pointers
        cull_bits_.release();
        cull_tmp_.release();
        return;
    }
    bool moved = false;
    auto put = [&](auto& dev, const auto& host) {
        if (dev.n < host.size()) {
            dev.alloc(host.size(), false);
            moved = true;
        }
        XPBD_CUDA(cudaMemcpy(dev.p, host.data(), host.size() * sizeof(host[0]), cudaMemcpyHostToDevice));
    };
    put(cull_org_, org);
    put(cull_dim_, dim);
    put(cull_off_, off);
    if (cull_bits_.n < words) {
        cull_bits_.alloc(words, false);
        cull_tmp_.alloc(words, false);
        moved = true;
    }
    if (moved) clear_graphs();
    launch_cull_build(stream_, (int)nm, node_off_dev_.p, (int64_t)nl_.n, topo_reachable_.p, nl_.p, nu_.p,
                      cull_org_.p, cull_dim_.p, cull_off_.p, (int64_t)words, cull_bits_.p, cull_tmp_.p);
    XPBD_CUDA(cudaGetLastError());
    XPBD_CUDA(cudaStreamSynchronize(stream_));
}

MeshTables Solver::mesh_tables() const {
    MeshTables m{};
    m.nl = nl_.p;
    m.nu = nu_.p;
    m.verts = verts_.p;
    m.vels = vels_.p;
    m.tris = tris_.p;
    m.prim = prim_.p;
    m.roots = roots_.p;
    m.margins = margins_.p;
    m.watertight = watertight_.p;
    m.prim_off = prim_off_.p;
    m.prim_cnt = prim_cnt_.p;
    m.tri_cache = tri_cache_.p;
    m.pair = node_pair_.p;
    m.cull_org = cull_org_.p;
    m.cull_dim = cull_dim_.p;
    m.cull_off = cull_off_.p;
    m.cull_bits = cull_bits_.n ? cull_bits_.p : nullptr;
    m.pose = body_q_.p;
    m.posed = dyn_any_ ? posed_.p : nullptr;
    m.walk_list = dyn_any_ ? walk_list_.p : nullptr;
    m.walk_count = dyn_any_ ? walk_count_ : (int)meshes_.size();
    m.n_meshes = (int)meshes_.size();
    m.avg_edge = avg_edge0_;
    m.soft_margin = cfg_.soft_contact_margin;
    return m;
}

void Solver::prof_mark(int slot) {
    if (!recording_ || !profiling_) return;
    cudaEvent_t e;
    XPBD_CUDA(cudaEventCreate(&e));
    // "external" so that capture turns it into an event-record node of the frame graph
    XPBD_CUDA(cudaEventRecordWithFlags(e, stream_, cudaEventRecordExternal));
    recording_->marks.emplace_back(e, slot);
}
void Solver::count_kernel(int k) {
    if (recording_) recording_->kernels += (uint64_t)k;
}
void Solver::count_memset() {
    if (recording_) recording_->memsets += 1;
}

// One substep reading state parity `src` and writing parity 1-src.
void Solver::record_substep(Mode mode, int sub, int iterations, float sdt, int src) {
    const int64_t n = (int64_t)n_;
    const int dst = 1 - src;
    const PredictParams pp = predict_params(sdt);
    PlaneParams pl;
    pl.enabled = cfg_.has_ground_plane ? 1 : 0;
    pl.margin = cfg_.soft_contact_margin;
    pl.altitude = cfg_.ground_plane_altitude;
    uint32_t* ccount = ccount_.p + sub;
    const bool gen = mode == Mode::Step;
    const bool mesh_pass = gen && !meshes_.empty();
    DeviceStatus* st = status_.p;

    const bool bodies = gen && dyn_any_;  // dynamic bodies step with the particles
    const RigidParams rp = rigid_params(sdt);
    const BodyArrays ba = body_arrays();
    const RigidTables rt = rigid_tables();
    const DynSlots ds{cslot_.p, slot_cap_, shape_body_.p, body_invm_.p};

    // a scene of one sort tile sorts in one block (launch_sort_small) and reads no digit
    // histogram; without a mesh pass and bodies nothing else uses the sort scratch either
    const bool small_sort = n <= kSmallSortMaxKeys;
    prof_mark(-1);
    if (!small_sort || mesh_pass || bodies) {
        XPBD_CUDA(cudaMemsetAsync(sort_scratch_.p, 0, sort_scratch_.bytes(), stream_));
        count_memset();
    }
    if (bodies) {
        XPBD_CUDA(cudaMemsetAsync(esort_scratch_.p, 0, esort_scratch_.bytes(), stream_));
        XPBD_CUDA(cudaMemsetAsync(seg_.p, 0, seg_.bytes(), stream_));
        count_memset();
        count_memset();
    }
    prof_mark(P_CLEAR);
    if (bodies) {
        launch_body_pairs(stream_, ba, rt, mesh_tables(), rp, st);
        count_kernel(7);  // bounds, pairs, box grid count, three scan kernels, fill
        count_memset();
        prof_mark(P_BODY_CONTACT);
    }
    // Contact generation forks after the static-mesh triage (which reads the previous order
    // that the sort below overwrites). With dynamic bodies the second stream runs the
    // moving-mesh triage, its queries (results to the hit buffer) and the rigid contacts, a
    // third stream the static-mesh traversal, and the main stream the integrate / sort /
    // gather chain (the sort waits for the moving-mesh triage) and the first iteration's
    // particle-particle part when split, none of which reads their outputs; once the
    // traversal is done the second stream merges the hits into the slots behind the static
    // contacts and builds the body-delta entries. The join comes before the bodies integrate
    // and before the first reader of contacts. Without bodies the static-mesh traversal runs
    // on the second stream beside the sort chain. Profiling keeps one stream in stage order
    // so that each stage's events bracket its own kernels.
    const bool fork = mesh_pass && !profiling_;
    const MeshTables mt = mesh_tables();
    const uint32_t* prev_order = pair_v_[(plan_.passes - 1) & 1].p;
    uint32_t* posed_counter = sort_scratch_.p + cq_off_ + 2;
    const auto posed_queries = [&](cudaStream_t s) {
        launch_posed_triage(s, n, prev_order, x_[src].p, r_.p, flags_.p, mt, rt, posed_counter, posed_list_.p);
        if (fork) XPBD_CUDA(cudaEventRecord(triaged_, s));
        launch_posed_queries(s, n, x_[src].p, r_.p, mt, rt, posed_counter, posed_list_.p, posed_hits_.p, st);
        count_kernel(2);  // triage + queries
    };
    const auto posed_merge = [&](cudaStream_t s) {
        launch_posed_merge(s, n, x_[src].p, r_.p, mt, rt, slot_cap_, cinfo_.p, cslot_.p, ccount, posed_counter,
                           posed_list_.p, posed_hits_.p, st);
        count_kernel();
    };
    const auto body_entries = [&](cudaStream_t s) {
        // body-delta entries: dynamic slots in contact order, grouped by body (stable sort)
        launch_dyn_scan(s, n, cinfo_.p, ds, dyn_rank_.p, dyn_totals_.p, dyn_ws_.p);
        launch_dyn_emit(s, n, cinfo_.p, ds, dyn_rank_.p, entry_cap_, eplan_, ekeys_.p,
                        esort_scratch_.p + ehist_off_, st);
        count_kernel(4);
        const uint32_t* ek = ekeys_.p;
        const uint32_t* ev = nullptr;
        const size_t elbw = sort_lookback_words(eplan_);
        for (int p = 0; p < eplan_.passes; p++) {
            launch_onesweep_pass(s, (int64_t)entry_cap_, eplan_, p, ek, ev, epk_[p & 1].p, epv_[p & 1].p,
                                 esort_scratch_.p + ehist_off_ + ((size_t)p << eplan_.bits),
                                 esort_scratch_.p + elb_off_ + (size_t)p * elbw, esort_scratch_.p + etc_off_ + p, st,
                                 dyn_totals_.p);
            count_kernel();
            ek = epk_[p & 1].p;
            ev = epv_[p & 1].p;
        }
        launch_body_segments(s, entry_cap_, dyn_totals_.p, ek, seg_.p);
        count_kernel();
        sorted_entries_ = ev;
    };
    if (mesh_pass)
        launch_collide_triage(stream_, n, prev_order, x_[src].p, r_.p, flags_.p, pl, mt, cinfo_.p, ccount,
                              sort_scratch_.p + cq_off_, near_.p);
    cudaStream_t walk_s = stream_;  // the static-mesh traversal's stream
    if (fork) {
        XPBD_CUDA(cudaEventRecord(fork_, stream_));
        XPBD_CUDA(cudaStreamWaitEvent(aux_, fork_, 0));
        if (bodies) {
            // a third stream for the static traversal: beside the moving-mesh chain and the
            // main stream's sort chain and first particle-particle pass
            XPBD_CUDA(cudaStreamWaitEvent(walk_stream_, fork_, 0));
            walk_s = walk_stream_;
            posed_queries(aux_);
            launch_rigid_contacts(aux_, ba, rt, mt, rp, st);  // reads only the substep-start poses
            count_kernel();
        } else {
            walk_s = aux_;
        }
    }
    if (mesh_pass) {
        launch_collide_walk(walk_s, n, x_[src].p, r_.p, pl, mt, slot_cap_, cinfo_.p, cslot_.p, ccount,
                            sort_scratch_.p + cq_off_, near_.p, st, fork && bodies ? kWalkBlocksBeside : 32);
        count_kernel(2);  // triage + traversal
        prof_mark(P_CONTACT);
    }
    if (fork && bodies) {  // the hits join the slots once the static contacts are in place
        XPBD_CUDA(cudaEventRecord(walked_, walk_s));
        XPBD_CUDA(cudaStreamWaitEvent(aux_, walked_, 0));
        posed_merge(aux_);
        body_entries(aux_);
    }
    if (fork) XPBD_CUDA(cudaEventRecord(join_, aux_));
    if (bodies && !fork) {
        posed_queries(stream_);
        posed_merge(stream_);
        prof_mark(P_POSED);
        launch_rigid_contacts(stream_, ba, rt, mt, rp, st);
        count_kernel();
        prof_mark(P_RIGID);
        body_entries(stream_);
        prof_mark(P_BODY_ENTRIES);
    }
    // plane contacts are fused into the key kernel when there is no mesh pass
    uint32_t* key_cinfo = (gen && !mesh_pass) ? cinfo_.p : nullptr;
    launch_predict_keys(stream_, n, x_[src].p, v_[src].p, w_.p, r_.p, flags_.p, pscene_.p, pp, pl, keys_.p, plan_,
                        small_sort ? nullptr : sort_scratch_.p + hist_off_, key_cinfo, ccount, stamp_.p);
    count_kernel();
    prof_mark(P_INTEGRATE_KEYS);
    const uint32_t* kin = keys_.p;
    const uint32_t* vin = nullptr;
    const size_t lbw = sort_lookback_words(plan_);
    if (fork && bodies) XPBD_CUDA(cudaStreamWaitEvent(stream_, triaged_, 0));  // it has read the previous order
    const int last = (plan_.passes - 1) & 1;  // the buffers the last pass writes (read by the rest)
    if (launch_sort_small(stream_, n, key_bits_, keys_.p, pair_k_[last].p, pair_v_[last].p)) {
        // a scene of one tile: every pass in one launch (the same stable order)
        count_kernel();
        prof_mark(P_SORT0);
        kin = pair_k_[last].p;
        vin = pair_v_[last].p;
    } else {
        for (int p = 0; p < plan_.passes; p++) {
            uint32_t* ko = pair_k_[p & 1].p;
            uint32_t* vo = pair_v_[p & 1].p;
            launch_onesweep_pass(stream_, n, plan_, p, kin, vin, ko, vo,
                                 sort_scratch_.p + hist_off_ + ((size_t)p << plan_.bits),
                                 sort_scratch_.p + lb_off_ + (size_t)p * lbw, sort_scratch_.p + tc_off_ + p, st,
                                 nullptr, true);
            count_kernel();
            prof_mark(P_SORT0 + std::min(p, 3));
            kin = ko;
            vin = vo;
        }
    }
    const uint32_t* skeys = kin;
    const uint32_t* sids = vin;
    const uint32_t* info = injected_ && !gen ? inj_info_.p : cinfo_.p;
    const float4* slots = injected_ && !gen ? inj_slot_.p : cslot_.p;
    launch_cells_gather(stream_, n, skeys, sids, x_[src].p, v_[src].p, w_.p, r_.p, flags_.p, pp, table_.p,
                        stamp_.p, rx_[0].p, rv_[0].p, rf_.p);
    count_kernel();
    prof_mark(P_CELLS);
    SolveDiag dg{nullptr, nullptr, nullptr, 0};
    if (cfg_.enable_diagnostics) {
        dg.delta_out = delta_.p;
        dg.pair_header = diag_header_.p;
        dg.pairs = diag_pairs_.p;
        dg.max_pairs = cfg_.max_diag_pairs ? cfg_.max_diag_pairs : 100000u;
    }
    const BodyTables bt = body_tables();
    const BodyDeltaOut bo{bodies ? bdel_.p : nullptr, bodies ? dyn_rank_.p : nullptr};
    // the first iteration's particle-particle part reads no contact: it runs before the join
    const bool split = fork && split_now_ && iterations > 0 && !cfg_.enable_diagnostics;
    if (split) {
        launch_solve(stream_, n, false, all_active_, sids, pscene_.p ? skeys : nullptr, rx_[0].p, rv_[0].p, rf_.p,
                     table_.p, stamp_.p, x_[src].p, v_[src].p, info, slots, ContactRanks{nullptr, nullptr}, bt,
                     solve_params(sdt, 0), nullptr, nullptr, nullptr, nullptr, dg, BodyDeltaOut{nullptr, nullptr}, 1,
                     pp_.p, solve_form_);
        count_kernel();
    }
    if (fork) XPBD_CUDA(cudaStreamWaitEvent(stream_, join_, 0));  // contacts complete
    if (bodies) {  // after every reader of the substep-start poses
        launch_body_integrate(stream_, ba, body_q_prev_.p, body_qd_prev_.p, rp);
        count_kernel();
        prof_mark(P_BODY_INTEGRATE);
    }
    ContactRanks cr{nullptr, nullptr};
    if (gen && need_ranks_) {
        // contacts past contact_max are dropped in the canonical order; a substep with at
        // most contact_max contacts keeps them all and skips the scan on the device
        launch_contact_scan(stream_, n, info, rank_.p, totals_.p, scan_ws_.p, ccount, contact_max_);
        count_kernel(3);
        prof_mark(P_RANKS);
        cr.rank = rank_.p;
        cr.totals = totals_.p;
        cr.count = ccount;
    }
    for (int it = 0; it < iterations; it++) {
        // the last iteration writes the final state in particle order; with dynamic bodies
        // its restitution waits for the last body pass (below)
        const bool last = it == iterations - 1;
        SolveParams sp = solve_params(sdt, it);
        if (bodies) sp.enable_restitution = 0;
        launch_solve(stream_, n, last, all_active_, sids, pscene_.p ? skeys : nullptr, rx_[it & 1].p,
                     rv_[it & 1].p, rf_.p, table_.p, stamp_.p, x_[src].p, v_[src].p, info, slots, cr, bt, sp,
                     rx_[(it + 1) & 1].p, rv_[(it + 1) & 1].p, x_[dst].p, v_[dst].p, dg, bo,
                     split && it == 0 ? 2 : 0, pp_.p, solve_form_);
        count_kernel();
        prof_mark(P_SOLVE);
        if (bodies) {
            launch_body_particles(stream_, ba, seg_.p, sorted_entries_, bdel_.p, body_q_.p, body_qd_.p,
                                  body_q_mid_.p, body_qd_mid_.p, rp);
            count_kernel();
            prof_mark(P_BODY_ITER);
            launch_body_rigid(stream_, ba, rt, body_q_mid_.p, body_qd_mid_.p, body_q_.p, body_qd_.p, rp);
            count_kernel();
            prof_mark(P_BODY_RIGID_ITER);
        }
    }
    if (bodies && iterations > 0 && cfg_.enable_restitution) {
        launch_restitute(stream_, n, flags_.p, r_.p, x_[src].p, v_[src].p, info, slots, cr, bt,
                         solve_params(sdt, iterations - 1), v_[dst].p);
        count_kernel();
        prof_mark(P_RESTITUTION);
    }
    if (iterations <= 0) {  // no solver iteration: the predicted state is the result
        XPBD_CUDA(cudaMemcpyAsync(x_[dst].p, x_[src].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
        XPBD_CUDA(cudaMemcpyAsync(v_[dst].p, v_[src].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
    }
}

void Solver::record_frame(Mode mode, float dt, int substeps, int iterations, int parity) {
    const float sdt = dt / (float)substeps;  // scene.cpp:701
    XPBD_CUDA(cudaMemsetAsync(ccount_.p, 0, (size_t)substeps * sizeof(uint32_t), stream_));
    count_memset();
    int src = parity;
    for (int sub = 0; sub < substeps; sub++) {
        record_substep(mode, sub, iterations, sdt, src);
        src = 1 - src;
    }
}

void Solver::run_frame(Mode mode, float dt, int substeps, int iterations, bool sync_now) {
    if (substeps <= 0) throw std::runtime_error("step: substeps must be positive");
    if (pending_substeps_) sync();
    rollout_valid_ = false;  // the stored rollout no longer ends at the current state
    ensure_substep_capacity(substeps);
    if (n_ == 0) return;
    if (lb_debug_seen_ != lookback_debug_generation()) {  // the sort's test hook changed: re-record
        clear_graphs();
        lb_debug_seen_ = lookback_debug_generation();
    }
    ensure_cull();
    if (!sort_tuned_ && n_ >= (1u << 20)) {  // large scenes: pick the sort variant on the real keys
        const int cc = contact_count_;
        autotune_sort(nullptr, nullptr);
        contact_count_ = cc;
    }
    if (solve_form_forced_ < 0 && last_was_step_ && n_ >= kSolveTuneMinParticles && !profiling_ &&
        !cfg_.enable_diagnostics && (!solve_form_timed_ || frames_run_ - solve_form_frame_ >= kSolveRetime))
        autotune_solve();
    auto t0 = std::chrono::high_resolution_clock::now();
    const bool split_ok = mode == Mode::Step && !meshes_.empty() && !profiling_ && iterations > 0 &&
                          !cfg_.enable_diagnostics;
    int trial = -1;
    if (split_ok && split_forced_ < 0 && split_choice_ >= 0 && ++split_frames_ >= kSplitRetime) {
        split_choice_ = -1;  // time both ways again, without the first-use frames
        split_trials_ = 2;
    }
    if (split_ok && split_choice_ < 0) {
        // frames 0 and 1 build each graph (not compared); then fused, split, split, fused,
        // so that a steady change of the frame time between frames cancels in the sums
        trial = split_trials_++;
        split_now_ = trial == 1 || trial == 3 || trial == 4;
    } else {
        split_now_ = split_ok && split_choice_ == 1;
    }
    GraphKey key{f2u(dt), substeps, iterations, cur_, (int)mode, profiling_ ? 1 : 0, split_now_ ? 1 : 0,
                 solve_form_};
    auto it = graphs_.find(key);
    if (it == graphs_.end()) {
        FrameGraph fg;
        cudaGraph_t g;
        recording_ = &fg;
        XPBD_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        try {
            record_frame(mode, dt, substeps, iterations, cur_);
        } catch (...) {
            recording_ = nullptr;
            cudaStreamEndCapture(stream_, &g);
            for (auto& m : fg.marks) cudaEventDestroy(m.first);
            throw;
        }
        recording_ = nullptr;
        XPBD_CUDA(cudaStreamEndCapture(stream_, &g));
        XPBD_CUDA(cudaGraphInstantiate(&fg.exec, g, 0));
        cudaGraphDestroy(g);
        it = graphs_.emplace(key, std::move(fg)).first;
    }
    if (trial >= 0) {
        for (auto& x : split_ev_[trial])
            if (!x) XPBD_CUDA(cudaEventCreate(&x));
        XPBD_CUDA(cudaEventRecord(split_ev_[trial][0], stream_));
    }
    XPBD_CUDA(cudaGraphLaunch(it->second.exec, stream_));
    if (trial >= 0) {
        XPBD_CUDA(cudaEventRecord(split_ev_[trial][1], stream_));
        if (trial == kSplitTrials - 1) {  // both ways timed: keep the faster
            XPBD_CUDA(cudaEventSynchronize(split_ev_[trial][1]));
            float sum[2] = {0.0f, 0.0f};
            for (int t = 2; t < kSplitTrials; t++) {
                float ms = 0.0f;
                XPBD_CUDA(cudaEventElapsedTime(&ms, split_ev_[t][0], split_ev_[t][1]));
                sum[(t == 3 || t == 4) ? 1 : 0] += ms;
            }
            // within 1% the split is kept: it is never slower by more on the benchmark scenes,
            // and a scene whose contact chain grows (bodies pressing into a pile) turns it faster
            split_choice_ = sum[1] < sum[0] * 1.01f ? 1 : 0;
            split_frames_ = 0;
        }
    }
    if (recorder_.active()) {  // this frame's positions to the writer thread (after the graph)
        launch_unpack_xyz(stream_, (int64_t)n_, x_[cur_ ^ (substeps & 1)].p, rec_stage_.p);
        recorder_.enqueue(stream_, rec_stage_.p);
    }
    last_kernels_ = it->second.kernels;
    kernels_total_ += it->second.kernels + (recorder_.active() ? 1 : 0);
    last_memsets_ = it->second.memsets;
    frames_run_++;
    last_collide_src_ = cur_ ^ ((substeps - 1) & 1);
    last_sdt_ = dt / (float)substeps;
    last_substeps_ = substeps;
    last_iterations_ = iterations;
    last_was_step_ = mode == Mode::Step && iterations > 0;
    cur_ ^= (substeps & 1);
    pending_substeps_ = substeps;
    if (!sync_now) return;
    sync();
    if (profiling_) {
        accumulate_stage_times(it->second);
        prof_wall_ms_ += std::chrono::duration<double, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
        prof_substeps_ += (uint64_t)substeps;
    }
}

void Solver::accumulate_stage_times(const FrameGraph& fg) {
    for (size_t k = 1; k < fg.marks.size(); k++) {
        const int slot = fg.marks[k].second;
        if (slot < 0) continue;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, fg.marks[k - 1].first, fg.marks[k].first) == cudaSuccess) prof_ms_[slot] += ms;
    }
}

void Solver::sync() {
    if (!pending_substeps_) return;
    const int s = pending_substeps_;
    pending_substeps_ = 0;
    finish_frame(s);
}

void Solver::finish_frame(int substeps) {
    // one small readback per frame: the last substep's contact count + status (scene.cpp:1086-1091)
    XPBD_CUDA(cudaMemcpyAsync(pinned_, ccount_.p + (substeps - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost,
                              stream_));
    XPBD_CUDA(cudaMemcpyAsync(pinned_ + 1, status_.p, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, stream_));
    XPBD_CUDA(cudaMemsetAsync(status_.p, 0, sizeof(DeviceStatus), stream_));
    XPBD_CUDA(cudaStreamSynchronize(stream_));
    uint32_t raw;
    std::memcpy(&raw, pinned_, 4);
    std::memcpy(&host_status_, pinned_ + 1, sizeof(DeviceStatus));
    contact_count_ = (int)std::min<int64_t>((int64_t)raw, contact_max_);
    if (host_status_.error_bits & kErrLookbackTimeout) {
        // the failed sort's ids (with duplicates and holes) would be the next collision
        // pass's particle order: start it from the identity again
        launch_iota(stream_, (int64_t)n_, pair_v_[(plan_.passes - 1) & 1].p);
        XPBD_CUDA(cudaStreamSynchronize(stream_));
        throw std::runtime_error("device wait timed out in the onesweep look-back (result discarded)");
    }
    if (host_status_.error_bits & kErrStackOverflow)
        throw std::runtime_error("BVH traversal stack overflow (more than 32 pending nodes)");
    if (host_status_.error_bits & kErrSlotOverflow)
        throw std::runtime_error("more mesh contacts for one particle than contact slots");
    if (host_status_.error_bits & kErrBodyOverflow)
        throw std::runtime_error("body tables full (more than 256 overlapping bodies, or more body-delta entries "
                                 "than 2 x particles + 4096)");
    if (env_on("VKXPBD_CHECK_SORT_ORDER")) check_sort_order();
}

void Solver::step(float dt, int substeps, int iterations) {
    if (!finalized_) finalize_meshes();  // scene.cpp:699
    XPBD_CUDA(cudaSetDevice(device_));
    if (injected_) clear_graphs();
    injected_ = false;
    run_frame(Mode::Step, dt, substeps, iterations, true);
}

void Solver::step_async(float dt, int substeps, int iterations) {
    if (!finalized_) finalize_meshes();
    XPBD_CUDA(cudaSetDevice(device_));
    if (injected_) clear_graphs();
    injected_ = false;
    run_frame(Mode::Step, dt, substeps, iterations, false);
}

void Solver::set_profiling(bool on) {
    require_init();
    if (on == profiling_) return;
    sync();
    profiling_ = on;
}

size_t Solver::stage_times(double* ms, size_t cap, uint64_t* substeps) const {
    for (size_t i = 0; i < std::min<size_t>(cap, P_COUNT); i++) ms[i] = prof_ms_[i];
    if (substeps) *substeps = prof_substeps_;
    return P_COUNT;
}

void Solver::reset_stage_times() {
    for (double& v : prof_ms_) v = 0.0;
    prof_substeps_ = 0;
    prof_wall_ms_ = 0.0;
}

void Solver::frame_stats(uint64_t out[4]) const {
    out[0] = last_kernels_;
    out[1] = last_memsets_;
    out[2] = frames_run_;
    out[3] = graphs_.size();
}

const char* Solver::stage_name(int i) { return (i >= 0 && i < P_COUNT) ? kProfNames[i] : ""; }
int Solver::stage_count() { return P_COUNT; }

void Solver::step_solve_only(float dt, int substeps, int iterations) {
    if (!finalized_) finalize_meshes();
    XPBD_CUDA(cudaSetDevice(device_));
    if (!injected_) {  // no injected contacts: solve with none
        inj_info_.alloc(n_);
        inj_slot_.alloc(std::max<size_t>(n_, 1) * 3);
        inj_cap_ = 1;
        injected_ = true;
        clear_graphs();
    }
    const int keep = contact_count_;
    run_frame(Mode::SolveOnly, dt, substeps, iterations, true);
    contact_count_ = keep;
}

void Solver::collide_only() {
    require_init();
    if (!finalized_) finalize_meshes();
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    if (injected_) clear_graphs();
    injected_ = false;
    PlaneParams pl;
    pl.enabled = cfg_.has_ground_plane ? 1 : 0;
    pl.margin = cfg_.soft_contact_margin;
    pl.altitude = cfg_.ground_plane_altitude;
    ensure_substep_capacity(1);
    ensure_cull();
    XPBD_CUDA(cudaMemsetAsync(ccount_.p, 0, sizeof(uint32_t), stream_));
    XPBD_CUDA(cudaMemsetAsync(sort_scratch_.p + cq_off_, 0, 2 * sizeof(uint32_t), stream_));
    launch_collide(stream_, (int64_t)n_, pair_v_[(plan_.passes - 1) & 1].p, x_[cur_].p, r_.p, flags_.p, pl,
                   mesh_tables(), slot_cap_, cinfo_.p, cslot_.p, ccount_.p, sort_scratch_.p + cq_off_, near_.p,
                   status_.p);
    last_collide_src_ = cur_;
    finish_frame(1);
}

void Solver::set_contact_data(const int32_t* part, const int32_t* shape, const float* bpos, const float* nrm,
                              int count) {
    require_init();
    if (!finalized_) finalize_meshes();
    XPBD_CUDA(cudaSetDevice(device_));
    contact_count_ = count;  // scene.cpp:1309
    const size_t m = count > 0 ? std::min<size_t>((size_t)count, (size_t)contact_max_) : 0;
    inj_part_.assign(part, part + m);
    inj_shape_.assign(shape, shape + m);
    inj_bpos_.assign(bpos, bpos + m * 3);
    inj_nrm_.assign(nrm, nrm + m * 3);
    // bucket by particle, keeping the given order inside a particle
    std::vector<uint32_t> cnt(n_, 0);
    for (size_t t = 0; t < m; t++) {
        if (part[t] < 0 || (size_t)part[t] >= n_) throw std::runtime_error("set_contact_data: particle index out of range");
        if (shape[t] < 0 || (size_t)shape[t] > meshes_.size())
            throw std::runtime_error("set_contact_data: shape index out of range");
        cnt[part[t]]++;
    }
    uint32_t cap = 1;
    for (uint32_t c : cnt) cap = std::max(cap, c);
    std::vector<float4> slots(n_ * cap * 3, make_float4(0, 0, 0, 0));
    std::vector<uint32_t> info(n_, 0);
    for (size_t t = 0; t < m; t++) {
        const size_t i = (size_t)part[t];
        const uint32_t k = info[i] >> 1;
        float4* s = &slots[(i * cap + k) * 3];
        s[0] = make_float4(bpos[t * 3], bpos[t * 3 + 1], bpos[t * 3 + 2], u2f((uint32_t)shape[t]));
        s[1] = make_float4(nrm[t * 3], nrm[t * 3 + 1], nrm[t * 3 + 2], 0.0f);
        s[2] = make_float4(0, 0, 0, 0);  // the reference uploads no body velocity here
        info[i] = (k + 1) << 1;
    }
    if (!injected_ || (int)cap != inj_cap_) clear_graphs();
    inj_cap_ = (int)cap;
    inj_info_.alloc(n_, false);
    inj_slot_.alloc(std::max<size_t>(n_ * cap * 3, 1), false);
    if (n_) {
        XPBD_CUDA(cudaMemcpy(inj_info_.p, info.data(), n_ * 4, cudaMemcpyHostToDevice));
        XPBD_CUDA(cudaMemcpy(inj_slot_.p, slots.data(), slots.size() * sizeof(float4), cudaMemcpyHostToDevice));
    }
    injected_ = true;
}

// Host xyz arrays <-> device float4 state: one copy straight from or to the caller's
// (pageable) memory plus a pack / unpack kernel; on Grace the CUDA driver moves pageable
// memory over NVLink-C2C directly, several times faster than staging it through a
// pinned buffer with a host memcpy.
void Solver::upload_xyz(const float* h, float4* d, size_t n) {
    XPBD_CUDA(cudaMemcpyAsync(xyz_stage_.p, h, n * 3 * sizeof(float), cudaMemcpyHostToDevice, stream_));
    launch_pack_xyz(stream_, (int64_t)n, xyz_stage_.p, d);
}

void Solver::download_xyz(const float4* d, float* h, size_t n) {
    launch_unpack_xyz(stream_, (int64_t)n, d, xyz_stage_.p);
    XPBD_CUDA(cudaMemcpyAsync(h, xyz_stage_.p, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    XPBD_CUDA(cudaStreamSynchronize(stream_));
}

void Solver::get_positions(float* out, size_t n) {
    if (!initialized_) return;
    n = std::min(n, n_);
    if (n == 0) return;
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    download_xyz(x_[cur_].p, out, n);
}

void Solver::get_velocities(float* out, size_t n) {
    if (!initialized_) return;
    n = std::min(n, n_);
    if (n == 0) return;
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    download_xyz(v_[cur_].p, out, n);
}

void Solver::compact_contacts() {
    const size_t cm = (size_t)std::max<int64_t>(contact_max_, 1);
    if (c_part_.n < cm) {
        c_part_.alloc(cm, false);
        c_shape_.alloc(cm, false);
        c_bpos_.alloc(cm * 3, false);
        c_bvel_.alloc(cm * 3, false);
        c_nrm_.alloc(cm * 3, false);
    }
    launch_contact_scan(stream_, (int64_t)n_, cinfo_.p, rank_.p, totals_.p, scan_ws_.p);
    launch_contact_compact(stream_, (int64_t)n_, cinfo_.p, cslot_.p, slot_cap_, rank_.p, totals_.p, contact_max_,
                           x_[last_collide_src_].p, cfg_.ground_plane_altitude, c_part_.p, c_shape_.p, c_bpos_.p,
                           c_bvel_.p, c_nrm_.p);
}

void Solver::get_contacts(int32_t* part, int32_t* shape, float* nrm, float* bpos, float* bvel) {
    if (!initialized_ || contact_count_ <= 0) return;
    const size_t m = (size_t)contact_count_;
    if (injected_) {  // the buffers hold the injected contacts (scene.cpp:1304-1315)
        const size_t k = std::min(m, inj_part_.size());
        if (part) std::memcpy(part, inj_part_.data(), k * 4);
        if (shape) std::memcpy(shape, inj_shape_.data(), k * 4);
        if (nrm) std::memcpy(nrm, inj_nrm_.data(), k * 12);
        if (bpos) std::memcpy(bpos, inj_bpos_.data(), k * 12);
        if (bvel) std::memset(bvel, 0, k * 12);
        return;
    }
    XPBD_CUDA(cudaSetDevice(device_));
    compact_contacts();
    auto dl = [&](void* dst, const void* src, size_t bytes) {
        if (dst) XPBD_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream_));
    };
    dl(part, c_part_.p, m * 4);
    dl(shape, c_shape_.p, m * 4);
    dl(nrm, c_nrm_.p, m * 12);
    dl(bpos, c_bpos_.p, m * 12);
    dl(bvel, c_bvel_.p, m * 12);
    XPBD_CUDA(cudaStreamSynchronize(stream_));
}

// The last sort in the reference's layout: the stable sort of the 21-bit cell keys (the
// split keys of the last substep, still in keys_ in particle order, with the alias bits
// cleared) from particle order, as gpu_sort.h sorts them. Its scratch is the substep's,
// which every substep clears first.
const uint32_t* Solver::sort_reference_layout(const uint32_t** ids) {
    if (!ref_k_[0].p)
        for (int p = 0; p < 2; p++) {
            ref_k_[p].alloc(n_, false);
            ref_v_[p].alloc(n_, false);
        }
    XPBD_CUDA(cudaMemsetAsync(sort_scratch_.p, 0, sort_scratch_.bytes(), stream_));
    launch_mask_keys(stream_, (int64_t)n_, keys_.p, (1u << 21) - 1u, ref_k_[1].p, plan_, sort_scratch_.p + hist_off_);
    const uint32_t* kin = ref_k_[1].p;
    const uint32_t* vin = nullptr;
    const size_t lbw = sort_lookback_words(plan_);
    for (int p = 0; p < plan_.passes; p++) {
        launch_onesweep_pass(stream_, (int64_t)n_, plan_, p, kin, vin, ref_k_[p & 1].p, ref_v_[p & 1].p,
                             sort_scratch_.p + hist_off_ + ((size_t)p << plan_.bits),
                             sort_scratch_.p + lb_off_ + (size_t)p * lbw, sort_scratch_.p + tc_off_ + p, status_.p);
        kin = ref_k_[p & 1].p;
        vin = ref_v_[p & 1].p;
    }
    *ids = vin;
    return kin;
}

void Solver::get_sorted(uint32_t* cells, uint32_t* ids, size_t n) {
    if (!initialized_) return;
    n = std::min(n, n_);
    XPBD_CUDA(cudaSetDevice(device_));
    const int fin = (plan_.passes - 1) & 1;
    const uint32_t* sk = pair_k_[fin].p;
    const uint32_t* sv = pair_v_[fin].p;
    if (split_keys_ && n_ > 0) sk = sort_reference_layout(&sv);
    if (cells) XPBD_CUDA(cudaMemcpyAsync(cells, sk, n * 4, cudaMemcpyDeviceToHost, stream_));
    if (ids) XPBD_CUDA(cudaMemcpyAsync(ids, sv, n * 4, cudaMemcpyDeviceToHost, stream_));
    XPBD_CUDA(cudaStreamSynchronize(stream_));
}

void Solver::get_cell_tables(int32_t* starts, int32_t* ends) {
    require_init();
    XPBD_CUDA(cudaSetDevice(device_));
    if (!cell_starts_.p) {
        cell_starts_.alloc(kNumCells, false);
        cell_ends_.alloc(kNumCells, false);
    }
    if (split_keys_) {
        const uint32_t* sv = nullptr;
        const uint32_t* sk = sort_reference_layout(&sv);
        launch_cell_bounds(stream_, (int64_t)n_, sk, cell_starts_.p, cell_ends_.p);
    } else {
        launch_cell_tables(stream_, table_.p, stamp_.p, cell_starts_.p, cell_ends_.p);
    }
    if (starts) XPBD_CUDA(cudaMemcpyAsync(starts, cell_starts_.p, kNumCells * 4, cudaMemcpyDeviceToHost, stream_));
    if (ends) XPBD_CUDA(cudaMemcpyAsync(ends, cell_ends_.p, kNumCells * 4, cudaMemcpyDeviceToHost, stream_));
    XPBD_CUDA(cudaStreamSynchronize(stream_));
}

void Solver::get_deltas(float* out, size_t n) {
    if (!initialized_) return;
    n = std::min(n, n_);
    if (!delta_.p) {
        std::memset(out, 0, n * 12);
        return;
    }
    XPBD_CUDA(cudaSetDevice(device_));
    XPBD_CUDA(cudaMemcpy(out, delta_.p, n * 12, cudaMemcpyDeviceToHost));
}

LbvhTopology Solver::topology(size_t c) const {
    LbvhTopology t;
    const size_t nb = node_offsets_[c], pb = prim_offsets_[c];
    t.parent = topo_parent_.p + nb;
    t.child_l = topo_child_l_.p + nb;
    t.child_r = topo_child_r_.p + nb;
    t.marked = topo_marked_.p + nb;
    t.reachable = topo_reachable_.p + nb;
    t.prim_local = topo_prim_.p + pb;
    return t;
}

// The mesh's node halves as the builder made them (mesh-local packed words), read back
// from the global arrays (the packing of scene.cpp:287-321 undone).
size_t Solver::mesh_bvh(size_t mi, float* lowers, float* uppers, size_t cap) {
    if (mi >= meshes_.size() || !finalized_) return 0;
    const size_t nn = 2 * (meshes_[mi].indices.size() / 3), nb = node_offsets_[mi], pb = prim_offsets_[mi];
    if (!lowers && !uppers) return nn;
    sync();
    std::vector<float4> l(nn), u(nn);
    XPBD_CUDA(cudaMemcpy(l.data(), nl_.p + nb, nn * sizeof(float4), cudaMemcpyDeviceToHost));
    XPBD_CUDA(cudaMemcpy(u.data(), nu_.p + nb, nn * sizeof(float4), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nn && i < cap; i++) {
        const uint32_t lw = f2u(l[i].w), uw = f2u(u[i].w);
        const bool leaf = (lw >> 30) & 3u;
        const uint32_t base = (uint32_t)(leaf ? pb : nb);
        const float lo[4] = {l[i].x, l[i].y, l[i].z, u2f(((lw & 0x3FFFFFFFu) - base) | (leaf ? (1u << 30) : 0u))};
        const float hi[4] = {u[i].x, u[i].y, u[i].z, u2f((uw & 0x3FFFFFFFu) - base)};
        if (lowers) std::memcpy(lowers + i * 4, lo, 16);
        if (uppers) std::memcpy(uppers + i * 4, hi, 16);
    }
    return nn;
}

uint32_t Solver::diag_pair_count() {
    if (!initialized_) return 0;
    uint32_t h[2];
    XPBD_CUDA(cudaSetDevice(device_));
    XPBD_CUDA(cudaMemcpy(h, diag_header_.p, 8, cudaMemcpyDeviceToHost));
    return h[0];
}
uint32_t Solver::diag_overflow_count() {
    if (!initialized_) return 0;
    uint32_t h[2];
    XPBD_CUDA(cudaSetDevice(device_));
    XPBD_CUDA(cudaMemcpy(h, diag_header_.p, 8, cudaMemcpyDeviceToHost));
    return h[1];
}
void Solver::reset_diag_buffers() {
    if (!initialized_) return;
    XPBD_CUDA(cudaSetDevice(device_));
    XPBD_CUDA(cudaMemset(diag_header_.p, 0, 8));
}
size_t Solver::diag_pairs(xpbd_pair_record* out, size_t cap) {
    if (!diag_pairs_.p) return 0;
    const uint32_t mp = cfg_.max_diag_pairs ? cfg_.max_diag_pairs : 100000u;
    const size_t avail = std::min<uint32_t>(diag_pair_count(), mp);  // bindings.cpp:364-372
    const size_t k = std::min(avail, cap);
    if (out && k) XPBD_CUDA(cudaMemcpy(out, diag_pairs_.p, k * sizeof(xpbd_pair_record), cudaMemcpyDeviceToHost));
    return avail;
}
// The reference binds these buffers but no shader writes them (the shape,
// apply and mesh shaders declare no binding for them), so they read back as
// zeros of the sizes scene.cpp:117-128 allocates.
size_t Solver::aux_diag(int which, void* out, size_t cap) {
    size_t len = 32;
    if (which == 2)
        len = cfg_.enable_diagnostics ? (size_t)4 * (size_t)(contact_max_ > 0 ? contact_max_ : 100000) * 32 : 32;
    if (!initialized_) len = 0;
    if (out) std::memset(out, 0, std::min(cap, len) * 4);
    return len;
}

void Solver::status(uint32_t out[4]) const {
    out[0] = host_status_.error_bits;
    out[1] = host_status_.lookback_timeouts;
    out[2] = host_status_.stack_overflows;
    out[3] = host_status_.slot_overflows;
}

void Solver::check_sort_order() {  // scene.cpp:1064-1084
    std::vector<uint32_t> keys(n_);
    get_sorted(keys.data(), nullptr, n_);
    for (size_t i = 1; i < keys.size(); i++)
        if (keys[i] < keys[i - 1]) {
            std::fprintf(stderr, "[VKXPBD SORT CHECK ERROR] keys[%zu] = %u < keys[%zu] = %u!\n", i, keys[i], i - 1,
                         keys[i - 1]);
            return;
        }
    std::printf("[VKXPBD DEBUG] Sort check passed: %zu keys strictly non-decreasing.\n", keys.size());
}

void Solver::print_profiler_summary() {
    if (!profiling_ || prof_substeps_ == 0) return;
    double total = 0;
    for (int i = 0; i < P_COUNT; i++) total += prof_ms_[i];
    const double ns = (double)prof_substeps_;
    const double gap = prof_wall_ms_ > total ? prof_wall_ms_ - total : 0.0;
    std::printf("\n========================================================================================================\n");
    std::printf("                               VKXPBD GPU TIMESTAMP PROFILER SUMMARY (CUDA events)                      \n");
    std::printf("========================================================================================================\n");
    std::printf("Total Substeps Recorded: %llu\n", (unsigned long long)prof_substeps_);
    std::printf("Wall-Clock Step Time:    %10.2f ms (%8.4f ms/substep)\n", prof_wall_ms_, prof_wall_ms_ / ns);
    std::printf("Summed GPU Active Time:  %10.2f ms (%8.4f ms/substep)\n", total, total / ns);
    std::printf("Host / Sync Idle Gap:    %10.2f ms (%8.4f ms/substep, %5.1f%% of wall)\n", gap, gap / ns,
                gap / (prof_wall_ms_ > 0 ? prof_wall_ms_ : 1.0) * 100.0);
    std::printf("%-35s | %10s | %14s | %10s\n", "Kernel / Stage Group", "Total (ms)", "Per-Substep (ms)", "% GPU Time");
    for (int i = 0; i < P_COUNT; i++)
        std::printf("%-35s | %10.2f | %14.4f | %9.2f%%\n", kProfNames[i], prof_ms_[i], prof_ms_[i] / ns,
                    prof_ms_[i] / (total > 0 ? total : 1.0) * 100.0);
    std::printf("========================================================================================================\n\n");
    std::fflush(stdout);
}

void Solver::record_start(const std::string& dir, int first_frame) {
    require_init();
    sync();
    rec_stage_.alloc(std::max<size_t>(n_, 1) * 3, false);
    recorder_.start(device_, n_, dir, first_frame);
}

int Solver::record_stop() {
    sync();
    return recorder_.stop();
}

void Solver::update_config(const xpbd_config& c) {
    require_init();
    sync();
    const xpbd_config old = cfg_;
    cfg_ = c;
    // fixed after init: the device, diagnostics buffers and profiling
    cfg_.device_index = old.device_index;
    cfg_.enable_diagnostics = old.enable_diagnostics;
    cfg_.max_diag_pairs = old.max_diag_pairs;
    cfg_.enable_profile = old.enable_profile;
    if (finalized_ && shape_mu_.p) {
        std::vector<float> smu(shape_mu_.n, cfg_.shape_material_mu);
        XPBD_CUDA(cudaMemcpy(shape_mu_.p, smu.data(), smu.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    clear_graphs();  // the frame graphs carry the parameters
    cull_dirty_ = true;
    rollout_valid_ = false;
}

// ---------------------------------------------------------------- differentiable rollout ----
void Solver::rollout(float dt, int substeps, int iterations, int frames, int checkpoint_frames) {
    require_init();
    if (!finalized_) finalize_meshes();
    if (!meshes_.empty() || dyn_any_ || pscene_.p || injected_)
        throw std::runtime_error("rollout: the adjoint covers the ground plane and particle contacts of one scene");
    if (iterations != 1) throw std::runtime_error("rollout: the adjoint covers one solver iteration");
    if (!all_active_) throw std::runtime_error("rollout: every particle must be active");
    if (substeps <= 0 || frames <= 0 || checkpoint_frames <= 0) throw std::runtime_error("rollout: bad counts");
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    const size_t n = n_;
    const int n_ckpt = (frames + checkpoint_frames - 1) / checkpoint_frames + 1;
    ckpt_.alloc((size_t)n_ckpt * 2 * std::max<size_t>(n, 1), false);
    auto save = [&](int slot) {
        float4* dst = ckpt_.p + (size_t)slot * 2 * n;
        XPBD_CUDA(cudaMemcpyAsync(dst, x_[cur_].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
        XPBD_CUDA(cudaMemcpyAsync(dst + n, v_[cur_].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
    };
    for (int f = 0; f < frames; f++) {
        if (f % checkpoint_frames == 0) save(f / checkpoint_frames);
        run_frame(Mode::Step, dt, substeps, 1, false);
    }
    sync();
    save(n_ckpt - 1);
    XPBD_CUDA(cudaStreamSynchronize(stream_));
    ro_dt_ = dt;
    ro_substeps_ = substeps;
    ro_frames_ = frames;
    ro_ckpt_ = checkpoint_frames;
    rollout_valid_ = true;
}

// Sorted records, cell table and plane contacts of the substep starting at x_[src], v_[src]
// (the first kernels of record_substep).
void Solver::prepare_grid(float sdt, int src) {
    const int64_t n = (int64_t)n_;
    const PredictParams pp = predict_params(sdt);
    PlaneParams pl;
    pl.enabled = cfg_.has_ground_plane ? 1 : 0;
    pl.margin = cfg_.soft_contact_margin;
    pl.altitude = cfg_.ground_plane_altitude;
    DeviceStatus* st = status_.p;
    XPBD_CUDA(cudaMemsetAsync(sort_scratch_.p, 0, sort_scratch_.bytes(), stream_));
    launch_predict_keys(stream_, n, x_[src].p, v_[src].p, w_.p, r_.p, flags_.p, nullptr, pp, pl, keys_.p, plan_,
                        sort_scratch_.p + hist_off_, cinfo_.p, ccount_.p, stamp_.p);
    const uint32_t* kin = keys_.p;
    const uint32_t* vin = nullptr;
    const size_t lbw = sort_lookback_words(plan_);
    for (int p = 0; p < plan_.passes; p++) {
        launch_onesweep_pass(stream_, n, plan_, p, kin, vin, pair_k_[p & 1].p, pair_v_[p & 1].p,
                             sort_scratch_.p + hist_off_ + ((size_t)p << plan_.bits),
                             sort_scratch_.p + lb_off_ + (size_t)p * lbw, sort_scratch_.p + tc_off_ + p, st);
        kin = pair_k_[p & 1].p;
        vin = pair_v_[p & 1].p;
    }
    launch_cells_gather(stream_, n, kin, vin, x_[src].p, v_[src].p, w_.p, r_.p, flags_.p, pp, table_.p, stamp_.p,
                        rx_[0].p, rv_[0].p, rf_.p);
}

void Solver::rollout_backward(const float* gx_final, const float* gv_final, float* gx0, float* gv0, float* gw,
                              double* params) {
    if (!rollout_valid_) throw std::runtime_error("rollout_backward: no rollout to differentiate");
    XPBD_CUDA(cudaSetDevice(device_));
    sync();
    const size_t n = n_;
    const float sdt = ro_dt_ / (float)ro_substeps_;  // as record_frame computes it
    const int n_seg = (ro_frames_ + ro_ckpt_ - 1) / ro_ckpt_;
    const size_t nn = std::max<size_t>(n, 1);
    // buffers keep their addresses between calls (the segment graphs hold them)
    bool moved = false;
    auto ensure = [&](auto& buf, size_t count) {
        if (buf.n != count) {
            buf.alloc(count, false);
            moved = true;
        }
    };
    ensure(gx_, nn);
    ensure(gv_, nn);
    ensure(gw_, nn);
    ensure(gacc_, nn);
    ensure(part_xp_, nn);
    ensure(part_vp_, nn);
    ensure(part_x0_, nn);
    ensure(part_v0_, nn);
    ensure(part_gd_, nn);
    const size_t blocks = adjoint_block_count((int64_t)n);
    ensure(block_params_, std::max<size_t>(blocks, 1) * 3);
    ensure(param_acc_, 3);
    // per replayed substep: start state (x, v) and the sorted (key, id) pairs
    ensure(traj_, (size_t)ro_ckpt_ * ro_substeps_ * 2 * nn);
    ensure(traj_keys_, (size_t)ro_ckpt_ * ro_substeps_ * 2 * nn);
    if (moved) clear_backward_graphs();
    XPBD_CUDA(cudaMemsetAsync(gw_.p, 0, gw_.bytes(), stream_));
    XPBD_CUDA(cudaMemsetAsync(param_acc_.p, 0, param_acc_.bytes(), stream_));
    // upstream gradients (host xyz -> device float4)
    auto upload = [&](const float* h, float4* d) {
        if (h) {
            upload_xyz(h, d, n);
            XPBD_CUDA(cudaStreamSynchronize(stream_));
        } else {
            XPBD_CUDA(cudaMemsetAsync(d, 0, n * sizeof(float4), stream_));
        }
    };
    upload(gx_final, gx_.p);
    upload(gv_final, gv_.p);
    AdjointArgs a{};
    a.n = (int64_t)n;
    a.table = table_.p;
    a.stamp = stamp_.p;
    a.flags = flags_.p;
    a.gx_in = gx_.p;
    a.gv_in = gv_.p;
    a.gx_out = gx_.p;
    a.gv_out = gv_.p;
    a.gw = gw_.p;
    a.gacc = gacc_.p;
    a.part_xp = part_xp_.p;
    a.part_vp = part_vp_.p;
    a.part_x0 = part_x0_.p;
    a.part_v0 = part_v0_.p;
    a.part_gd = part_gd_.p;
    a.block_params = block_params_.p;
    a.param_acc = param_acc_.p;
    a.dt = sdt;
    a.inv = 1.0f / cfg_.search_radius;
    a.relax = cfg_.soft_contact_relaxation;
    a.ka = cfg_.particle_adhesion;
    a.altitude = cfg_.ground_plane_altitude;
    a.margin = cfg_.soft_contact_margin;
    a.plane_on = cfg_.has_ground_plane ? 1 : 0;
    a.mu_plane = 0.5f * (cfg_.soft_contact_mu + cfg_.shape_material_mu);
    a.k_mu = cfg_.particle_mu;
    a.k_coh = cfg_.particle_cohesion;
    a.max_radius = cfg_.particle_max_radius;
    a.restitution = cfg_.soft_contact_restitution;
    a.restitution_on = cfg_.enable_restitution ? 1 : 0;
    a.split_keys = split_keys_ ? 1 : 0;
    a.rx = rx_[0].p;
    a.rv = rv_[0].p;
    a.x0 = x_[0].p;
    a.v0 = v_[0].p;
    // one segment: replay from the checkpoint already in x_[0], v_[0] keeping every
    // substep's start state and sort, then the adjoint of its substeps, last first (cell
    // table and sorted records rebuilt from the stored sort); captured once per segment
    // length and step, replayed for every segment
    const PredictParams pp = predict_params(sdt);
    split_now_ = false;  // the replayed substeps keep the fused solve
    auto segment = [&](int S) {
        int src = 0;
        const int fin = (plan_.passes - 1) & 1;
        for (int t = 0; t < S; t++) {
            float4* tr = traj_.p + (size_t)t * 2 * n;
            uint32_t* tk = traj_keys_.p + (size_t)t * 2 * n;
            XPBD_CUDA(cudaMemcpyAsync(tr, x_[src].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
            XPBD_CUDA(cudaMemcpyAsync(tr + n, v_[src].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
            if (t + 1 < S) {
                record_substep(Mode::Step, 0, 1, sdt, src);
                src = 1 - src;
            } else {
                prepare_grid(sdt, src);  // the segment's last substep: its sort only
            }
            XPBD_CUDA(cudaMemcpyAsync(tk, pair_k_[fin].p, n * 4, cudaMemcpyDeviceToDevice, stream_));
            XPBD_CUDA(cudaMemcpyAsync(tk + n, pair_v_[fin].p, n * 4, cudaMemcpyDeviceToDevice, stream_));
        }
        for (int t = S - 1; t >= 0; t--) {
            const float4* tr = traj_.p + (size_t)t * 2 * n;
            const uint32_t* tk = traj_keys_.p + (size_t)t * 2 * n;
            launch_bump_stamp(stream_, stamp_.p);
            launch_cells_gather(stream_, (int64_t)n, tk, tk + n, tr, tr + n, w_.p, r_.p, flags_.p, pp, table_.p,
                                stamp_.p, rx_[0].p, rv_[0].p, rf_.p);
            AdjointArgs at = a;
            at.sids = tk + n;
            at.x0 = tr;
            at.v0 = tr + n;
            launch_adjoint_substep(stream_, at);
        }
    };
    for (int c = n_seg - 1; c >= 0; c--) {
        const int nf = std::min(ro_ckpt_, ro_frames_ - c * ro_ckpt_);
        const int S = nf * ro_substeps_;
        const float4* ck = ckpt_.p + (size_t)c * 2 * n;
        XPBD_CUDA(cudaMemcpyAsync(x_[0].p, ck, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
        XPBD_CUDA(cudaMemcpyAsync(v_[0].p, ck + n, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
        const std::pair<int, uint32_t> key(S, f2u(sdt));
        auto it = bwd_graphs_.find(key);
        if (it == bwd_graphs_.end()) {
            cudaGraph_t g;
            XPBD_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
            try {
                segment(S);
            } catch (...) {
                cudaStreamEndCapture(stream_, &g);
                throw;
            }
            XPBD_CUDA(cudaStreamEndCapture(stream_, &g));
            cudaGraphExec_t exec;
            XPBD_CUDA(cudaGraphInstantiate(&exec, g, 0));
            cudaGraphDestroy(g);
            it = bwd_graphs_.emplace(key, exec).first;
        }
        XPBD_CUDA(cudaGraphLaunch(it->second, stream_));
    }
    XPBD_CUDA(cudaStreamSynchronize(stream_));
    auto download = [&](const float4* d, float* h) {
        if (!h) return;
        download_xyz(d, h, n);
    };
    download(gx_.p, gx0);
    download(gv_.p, gv0);
    if (gw) XPBD_CUDA(cudaMemcpy(gw, gw_.p, n * sizeof(float), cudaMemcpyDeviceToHost));
    double acc[3];
    XPBD_CUDA(cudaMemcpy(acc, param_acc_.p, sizeof(acc), cudaMemcpyDeviceToHost));
    if (params) {  // soft_contact_mu, shape_material_mu (plane mu = their mean), particle_mu, restitution
        params[0] = 0.5 * acc[0];
        params[1] = 0.5 * acc[0];
        params[2] = acc[1];
        params[3] = acc[2];
    }
    // leave the solver at the rollout's final state
    const float4* fin = ckpt_.p + (size_t)((ro_frames_ + ro_ckpt_ - 1) / ro_ckpt_) * 2 * n;
    XPBD_CUDA(cudaMemcpyAsync(x_[cur_].p, fin, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
    XPBD_CUDA(cudaMemcpyAsync(v_[cur_].p, fin + n, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_));
    const int cc = contact_count_;
    finish_frame(1);  // raises on a device-side error of the replay
    contact_count_ = cc;
}

}  // namespace xpbd
