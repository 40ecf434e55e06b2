// Launch interface between the host scene driver (solver.cpp) and the sm_103a
// kernels (k_*.cu). Plain structs of device pointers and scalars; every launch
// takes the solver's stream so that a frame can be captured into one graph.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/xpbd.h"

namespace xpbd {

constexpr int kGridDim = 128;                                   // hash grid, src/scene.cpp:17-18
constexpr int kNumCells = kGridDim * kGridDim * kGridDim;
constexpr int kSplitKeyBits = 24;  // one scene: the reference's 21-bit key + 3 alias bits
// one-scene solvers from this many particles sort split keys (their cell table has 2^24
// entries, 256 MiB); smaller ones sort the reference's keys (128^3 entries, 32 MiB)
constexpr size_t kSplitKeysMinParticles = 32768;
constexpr int kGridOrigin = 1 << 20;                            // grid_cell_indices.comp:20

// Device-side status word read back after every frame. A kernel that gives
// up (bounded wait expired, fixed-size buffer full) sets a bit and continues;
// the host turns a set bit into an error instead of hanging or faulting.
struct DeviceStatus {
    uint32_t error_bits;
    uint32_t lookback_timeouts;
    uint32_t stack_overflows;
    uint32_t slot_overflows;
    uint32_t rigid_slot_overflows;  // rigid contacts dropped past kRigidSlots per vertex (as the oracle)
    uint32_t pad[3];
};
enum : uint32_t {
    kErrLookbackTimeout = 1u,  // a decoupled look-back wait expired
    kErrStackOverflow = 2u,    // BVH traversal stack (32 entries) full
    kErrSlotOverflow = 4u,     // more mesh contacts for one particle than slots
    kErrBodyOverflow = 8u,     // body partner list or body-delta entries full
};

// Per-particle contact header (cinfo[i]): bit 0 = plane contact (shape 0),
// bits 1..15 = number of generic contact slots used in cslot, bits 16..31 = how many
// of them belong to dynamic bodies.
// A generic slot is 3 float4: (body_pos.xyz, shape as int bits),
// (normal.xyz, 0), (body_vel.xyz, 0).
constexpr uint32_t kPlaneBit = 1u;
__host__ __device__ __forceinline__ int info_slots(uint32_t info) { return (int)((info >> 1) & 0x7fffu); }
__host__ __device__ __forceinline__ int info_dyn(uint32_t info) { return (int)(info >> 16); }

struct PredictParams {
    float dt, v_max, gx, gy, gz, inv;
    int split_keys;  // one scene with split cell keys (the reference's key + alias bits)
};
struct PlaneParams {
    int enabled;
    float margin, altitude;
};

struct BodyTables {
    const int* shape_body;   // [n_shapes]
    const float* shape_mu;   // [n_shapes]
    const float4* body_q;    // 2 per body: (pos, pad), (quat xyzw)
    const float4* body_qd;   // 2 per body: (lin, pad), (ang, pad)
    const float* body_com;   // 3 per body
    const float* body_invI;  // 9 per body, row-major (solve_particle_shape_contacts.comp:46-48)
    const float* body_invm;  // [n_bodies]
    const int* body_flags;   // [n_bodies]
    // body state at the start of the substep (restitution); equal to body_q / body_qd
    // while every body is static (scene.cpp:577-580)
    const float4* body_q_prev;
    const float4* body_qd_prev;
};

struct MeshTables {
    const float4* nl;         // packed node lowers (xyz, packed word)
    const float4* nu;         // packed node uppers
    const float* verts;       // 3 per vertex
    const float* vels;        // 3 per vertex
    const uint32_t* tris;     // 3 per triangle, global vertex indices
    const uint32_t* prim;     // global triangle index per leaf slot
    const uint32_t* roots;    // [n_meshes]
    const float* margins;     // [n_meshes]
    const int* watertight;    // [n_meshes]
    const uint32_t* prim_off; // [n_meshes]
    const uint32_t* prim_cnt; // [n_meshes]
    // per leaf slot: (a.xyz, triangle id bits), (b.xyz, |e0|^2), (c.xyz, |e1|^2),
    // (unit normal.xyz, |e2|^2 or -1 when the triangle is skipped as degenerate)
    const float4* tri_cache;
    // sibling records keyed by left child: pair[a*4 .. a*4+3] = nl[a], nu[a], nl[b], nu[b]
    // for every inner node with children (a, b), so one pop reads one 64-byte record
    const float4* pair;
    // reach grids (one per mesh, null: none): bit set for every cell within reach of a
    // leaf box. cull_org[m] = (origin.xyz, 1/cell), cull_dim[m] = (nx, ny, nz, dilation
    // in cells; nx = 0: no grid), words of mesh m from cull_off[m], x fastest, 32 cells
    // per word. A particle in a clear cell (or outside the grid) cannot reach any leaf.
    const float4* cull_org;
    const int4* cull_dim;
    const uint32_t* cull_off;
    const uint32_t* cull_bits;
    // meshes whose body is dynamic hold body-frame vertices: pose = the bodies' state
    // (2 float4 per mesh), posed[m] != 0 for those meshes, walk_list = the other meshes
    // (null: every mesh is static)
    const float4* pose;
    const int* posed;
    const int* walk_list;
    int walk_count;
    int n_meshes;
    float avg_edge;           // mesh 0's average edge length (scene.cpp:325)
    float soft_margin;
};

struct SolveParams {
    float dt, relax, v_max, inv, max_radius;
    float k_mu, k_coh;        // particle_mu, particle_cohesion
    float soft_mu, ka;        // soft_contact_mu, particle_adhesion
    float restitution;
    int enable_restitution;
    float altitude;
    int slot_cap;             // generic contact slots per particle
    int iter_index;
    int split_keys;           // cell keys of the sort: split (one scene) or the reference's
    int64_t contact_max;
};

// Per-slot body deltas written by the solve kernel for contacts with dynamic bodies
// (solve_particle_shape_contacts.comp:193-199): entry dyn_rank[particle].x + j for the
// particle's j-th dynamic slot, 2 float4 (-delta_v, valid), (-delta_w, 0).
struct BodyDeltaOut {
    float4* bdel;
    const uint2* dyn_rank;  // .x
};

// Optional debugging outputs of the solve kernel.
struct SolveDiag {
    float* delta_out;         // [3n] last iteration's deltas in particle order, or null
    uint32_t* pair_header;    // [2]: pair count, overflow count
    float* pairs;             // 20 words per record (vkx::GPUPairRecord layout)
    uint32_t max_pairs;
};

// Contact ranks for the contact_max cap and for compaction (canonical order:
// plane block by particle, then generic block by particle and slot).
struct ContactRanks {
    const uint2* rank;        // per particle (exclusive plane count, exclusive slot count), or null
    const uint32_t* totals;   // [2] total plane contacts, total slot contacts
    // the substep's contact count, or null: when it is at most contact_max every contact
    // is kept and the ranks (not computed then) are not read
    const uint32_t* count = nullptr;
};

// ---------------------------------------------------------------- sort ----
struct SortPlan {
    int bits;      // digit width
    int passes;    // ceil(key_bits / bits)
    int threads;   // CTA size (== 2^bits for the shipped variants)
    int items;     // keys per thread
    int tile;      // threads * items
    int tiles;     // ceil(n / tile)
};
SortPlan make_sort_plan(int64_t n, int key_bits, int bits, int items);
size_t sort_lookback_words(const SortPlan& p);  // per pass

// keys[i] (+ optional plane contacts, + all-pass digit histograms into hist unless it is null)
// Batched scenes: pscene[i] is particle i's scene and the key becomes (scene << 21) | cell,
// which is also the entry of a scene-major table of 128^3 cells per scene (pscene == null:
// one scene).
void launch_predict_keys(cudaStream_t s, int64_t n, const float4* x, const float4* v, const float* w,
                         const float* r, const int* flags, const uint32_t* pscene, PredictParams pp, PlaneParams pl,
                         uint32_t* keys, const SortPlan& sp, uint32_t* hist, uint32_t* cinfo,
                         uint32_t* ccount, uint32_t* stamp);
// every pass of a stable LSD sort of at most kSmallSortMaxKeys keys (key_bits wide, 8-bit
// digits) in one launch of one block; values = input index. Returns false (nothing launched)
// for more keys.
constexpr int64_t kSmallSortMaxKeys = 4096;
bool launch_sort_small(cudaStream_t s, int64_t n, int key_bits, const uint32_t* keys_in, uint32_t* keys_out,
                       uint32_t* vals_out);
// one onesweep pass; vals_in == nullptr means vals are the element index; n_dev (optional)
// holds the element count on the device (at most n, the capacity the grid is sized for).
// debug_hold: the pass honours the look-back test hook (set_lookback_debug)
void launch_onesweep_pass(cudaStream_t s, int64_t n, const SortPlan& sp, int pass, const uint32_t* keys_in,
                          const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                          const uint32_t* hist_pass, uint32_t* lookback, uint32_t* tile_counter,
                          DeviceStatus* st, const uint32_t* n_dev = nullptr, bool debug_hold = false);
// Test hook of the bounded look-back wait: in every later sort pass launched with
// debug_hold (the particle sort of a step and the allocation-free sort), tile hold_tile of
// the first pass never publishes its prefix, so its successors' waits run out after
// wait_ns (0 < wait_ns <= 1 s) and set kErrLookbackTimeout. The output of such a sort is
// wrong (duplicates and holes holding earlier contents of the buffers) but every slot it
// writes stays below n (the scatter is bounded). hold_tile < 0 restores normal operation.
// lookback_debug_generation() changes on every call (solvers then re-record their graphs).
void set_lookback_debug(int64_t hold_tile, uint64_t wait_ns);
uint32_t lookback_debug_generation();
// SM count of the current device (cudaDevAttrMultiProcessorCount), cached per device
int device_sm_count();
// cell table + sorted-order particle records
void launch_cells_gather(cudaStream_t s, int64_t n, const uint32_t* skeys, const uint32_t* sids, const float4* x,
                         const float4* v, const float* w, const float* r, const int* flags, PredictParams pp,
                         int4* table, const uint32_t* stamp, float4* rx, float4* rv, int* rf);
// plane + mesh contact generation over the particles order[0..n) (any permutation);
// *queue is the work-queue counter and must be zero at launch
// queue: 2 zeroed words (work counter, near-list length); near: n words of scratch
void launch_collide(cudaStream_t s, int64_t n, const uint32_t* order, const float4* x, const float* r,
                    const int* flags, PlaneParams pl, MeshTables mt, int slot_cap, uint32_t* cinfo, float4* cslot,
                    uint32_t* ccount, uint32_t* queue, uint32_t* near, DeviceStatus* st);
// the two halves of launch_collide: the triage (reads `order`, writes the near list and the
// contact words of the particles it settles) and the traversal of the near list
void launch_collide_triage(cudaStream_t s, int64_t n, const uint32_t* order, const float4* x, const float* r,
                           const int* flags, PlaneParams pl, MeshTables mt, uint32_t* cinfo, uint32_t* ccount,
                           uint32_t* queue, uint32_t* near);
// (at most blocks_per_sm one-warp blocks per SM: fewer leave room for a kernel beside it)
void launch_collide_walk(cudaStream_t s, int64_t n, const float4* x, const float* r, PlaneParams pl, MeshTables mt,
                         int slot_cap, uint32_t* cinfo, float4* cslot, uint32_t* ccount, uint32_t* queue,
                         const uint32_t* near, DeviceStatus* st, int blocks_per_sm = 32);
// per-leaf-slot triangle cache for the slots [first, first + count)
void launch_tri_cache(cudaStream_t s, int64_t first, int64_t count, const uint32_t* prim, const uint32_t* tris,
                      const float* verts, float4* cache);
void launch_iota(cudaStream_t s, int64_t n, uint32_t* out);
// fused shape solve + particle-particle solve + apply (+ restitution on the last iteration)
// skeys (sorted keys) is passed for batched scenes so that each particle looks up its own
// scene's table; null for one scene. pp_mode 1 computes only the particle-particle totals
// (pp[k], sorted order; reads no contact), pp_mode 2 is the rest of the iteration taking
// its totals from pp; 0 does both (required with diagnostics)
void launch_solve(cudaStream_t s, int64_t n, bool last, bool all_active, const uint32_t* sids, const uint32_t* skeys,
                  const float4* rx, const float4* rv, const int* rf, const int4* table, const uint32_t* stamp,
                  const float4* x0,
                  const float4* v0, const uint32_t* cinfo, const float4* cslot, ContactRanks cr, BodyTables bt,
                  SolveParams sp, float4* rx_out, float4* rv_out, float4* x_out, float4* v_out, SolveDiag dg,
                  BodyDeltaOut bo = BodyDeltaOut{nullptr, nullptr}, int pp_mode = 0, float4* pp = nullptr,
                  int form = 0);
// forms of the solve kernel (launch_solve's `form`): 0 = each thread sums its own neighbours'
// pair terms, 1 = the lanes of a warp compute their neighbours' pair terms together, 2 = as 0
// with the block's neighbourhood records staged in shared memory, 3 = one warp per particle
// (its lanes test the candidates and compute the pair terms 32 at a time: small scenes,
// whose time is one particle's latency); same bits
constexpr int kSolveForms = 4;
// the forms the solver times on its scene and chooses from (the staged form measured slower
// on every benchmark scene: it stays selectable, and tested, but is not timed)
constexpr int kSolveTimedForms = 2;
// restitution (apply_particle_shape_restitution.comp) after the body passes of the last
// iteration, in particle order on the final state the last iteration wrote (v_out)
void launch_restitute(cudaStream_t s, int64_t n, const int* flags, const float* radii, const float4* x0,
                      const float4* v0, const uint32_t* cinfo, const float4* cslot, ContactRanks cr, BodyTables bt,
                      SolveParams sp, float4* v_out);
// exclusive scan of per-particle (plane bit, slot count) for the contact_max cap / compaction
size_t contact_scan_words(int64_t n);
// (skip_count, cap): the scan does nothing when *skip_count <= cap (no contact over the cap)
void launch_contact_scan(cudaStream_t s, int64_t n, const uint32_t* cinfo, uint2* rank, uint32_t* totals,
                         uint32_t* workspace, const uint32_t* skip_count = nullptr, int64_t cap = 0);
// exclusive scan of each particle's number of contact slots with a dynamic body
// (rank[i].x; totals[0] = all of them)
struct DynSlots {
    const float4* cslot;
    int slot_cap;
    const int* shape_body;
    const float* body_invm;
};
void launch_dyn_scan(cudaStream_t s, int64_t n, const uint32_t* cinfo, DynSlots ds, uint2* rank, uint32_t* totals,
                     uint32_t* lookback);
// canonical SoA contact list (for the getters)
void launch_contact_compact(cudaStream_t s, int64_t n, const uint32_t* cinfo, const float4* cslot, int slot_cap,
                            const uint2* rank, const uint32_t* totals, int64_t contact_max, const float4* x_prev,
                            float altitude, int32_t* part, int32_t* shape, float* bpos, float* bvel, float* nrm);
// reference-layout cell tables from the stamped table (table of one scene)
void launch_cell_tables(cudaStream_t s, const int4* table, const uint32_t* stamp, int32_t* starts, int32_t* ends);
// out = keys & mask with the digit histograms of every pass of sp added to hist
void launch_mask_keys(cudaStream_t s, int64_t n, const uint32_t* keys, uint32_t mask, uint32_t* out,
                      const SortPlan& sp, uint32_t* hist);
// per-cell [start, end) of sorted 21-bit keys over the 128^3 cells (0 for empty cells)
void launch_cell_bounds(cudaStream_t s, int64_t n, const uint32_t* skeys, int32_t* starts, int32_t* ends);
// stable sort of n keys (values = input index) using only the static scratch array of noalloc.cu
void sort_keys_noalloc(const uint32_t* keys, uint32_t* sorted_keys, uint32_t* sorted_ids, int64_t n, int key_bits,
                       cudaStream_t s);
// the status of the last sort (or graph replay of one) on the current device: throws when a
// bounded wait inside it ran out; call after the stream has finished
void sort_keys_noalloc_status();
// ---------------------------------------------------------------- bodies ----
// Body b belongs to mesh b. Dynamic bodies (inv_m > 0) are listed in `dyn` (ascending);
// their mesh vertices are dv_local[dv_start[b] .. dv_start[b + 1]) (body frame).
struct BodyArrays {
    float4* q;            // current state (2 float4 per body)
    float4* qd;
    const float* com;     // 3 per body
    const float* I;       // 9 per body
    const float* invI;    // 9 per body
    const float* invm;
    const int* flags;
    const int* shape_body;
    const float* shape_mu;
    int nb;
};
struct RigidParams {
    float dt, damping, margin, relax;
    int con_weighting;
    float mu_t, mu_r;
    int particle_weighting;
    float gx, gy, gz;
    int plane;
    float altitude;
};
constexpr int kPartnerCap = 256;  // dynamic bodies whose boxes overlap one dynamic body
constexpr int kRigidSlots = 4;    // rigid contacts per body vertex
struct RigidTables {
    int n_dyn;
    const int* dyn;               // dynamic body ids, ascending
    const int* dyn_index;         // body -> index in dyn, or -1
    const uint32_t* dv_start;     // [nb + 1] vertex ranges per body (empty for static bodies)
    const float4* dv_local;       // body-frame vertex, w = body id bits
    float4* wbox;                 // 2 per dynamic body: world box lower, upper (w = shape margin)
    int* partners;                // kPartnerCap per dynamic body
    int* partner_count;
    float4* rc;                   // kRigidSlots * 5 float4 per vertex
    int* rc_count;
    float pad;                    // conservative widening of the world boxes
    int n_vert;                   // dv_start[nb]
    // batched scenes: the scene of each dynamic body and of each particle (null: all in
    // scene 0); bodies meet only bodies and particles of their own scene
    const int* dyn_scene;
    const uint32_t* pscene;
    // hashed grid of the dynamic bodies' world boxes (widened by grid_reach) for the particle
    // queries: cell size grid_cs >= 1 / (kBoxAxis - 1) of any widened box, so a box covers
    // at most kBoxAxis cells per axis, kBoxCells in all; bucket h lists (dyn index, cell x, y, z) entries, any order, in
    // grid_list[grid_start[h] ..); a particle takes only the entries of its own cell
    // (hash collisions never list a body twice for one cell)
    int grid_size;                // buckets (power of two)
    float grid_cs, grid_reach;
    uint32_t* grid_count;         // [grid_size]
    uint32_t* grid_start;         // [grid_size + 1]
    uint32_t* grid_tiles;         // scan scratch: [grid_size / 1024], at most 4,096 tiles
    int4* grid_list;              // [kBoxCells * n_dyn]
};
constexpr int kBoxAxis = 6;
constexpr int kBoxCells = kBoxAxis * kBoxAxis * kBoxAxis;
constexpr int kBoxBuckets = 64;  // buckets per dynamic body (rounded up to a power of two in all)
// integrate_bodies.comp for every body; saves the pre-integration state to q_prev
void launch_body_integrate(cudaStream_t s, BodyArrays ba, float4* q_prev, float4* qd_prev, RigidParams rp);
// world boxes of the dynamic bodies and their overlapping pairs
void launch_body_pairs(cudaStream_t s, BodyArrays ba, RigidTables rt, MeshTables mt, RigidParams rp, DeviceStatus* st);
// rigid contacts of every dynamic-body vertex against the plane and the other meshes
void launch_rigid_contacts(cudaStream_t s, BodyArrays ba, RigidTables rt, MeshTables mt, RigidParams rp,
                           DeviceStatus* st);
// particle contacts against the meshes of dynamic bodies in three launches: the triage
// (reads `order`; lists the particles near a moving mesh with their first candidates:
// counter = one zeroed word, list = kPosedListWords words per particle), the queries of the
// listed candidates (results to `hits`, kPosedHitWords float4 per particle; no slot is
// touched, so they may run beside the static-mesh traversal), and the merge of the hits
// into the slots in mesh order after that traversal. Particle indices below 2^28.
constexpr int kPosedListWords = 8;                        // the particle and 7 candidates
constexpr int kPosedHitWords = 3 * (kPosedListWords - 1);  // float4 per list entry in `hits`
void launch_posed_triage(cudaStream_t s, int64_t n, const uint32_t* order, const float4* x, const float* r,
                         const int* flags, MeshTables mt, RigidTables rt, uint32_t* counter, uint32_t* list);
void launch_posed_queries(cudaStream_t s, int64_t n, const float4* x, const float* r, MeshTables mt, RigidTables rt,
                          const uint32_t* counter, const uint32_t* list, float4* hits, DeviceStatus* st);
void launch_posed_merge(cudaStream_t s, int64_t n, const float4* x, const float* r, MeshTables mt, RigidTables rt,
                        int slot_cap, uint32_t* cinfo, float4* cslot, uint32_t* ccount, const uint32_t* counter,
                        const uint32_t* list, const float4* hits, DeviceStatus* st);
// body-delta entries: key = body of each dynamic slot at position rank[i].x + j, digit histograms
void launch_dyn_emit(cudaStream_t s, int64_t n, const uint32_t* cinfo, DynSlots ds, const uint2* rank,
                     uint32_t cap, const SortPlan& sp, uint32_t* keys, uint32_t* hist, DeviceStatus* st);
// [start, end) of every body in the sorted entry keys (seg zeroed beforehand)
void launch_body_segments(cudaStream_t s, uint32_t cap, const uint32_t* count, const uint32_t* skeys, uint2* seg);
// per body: sum of its particle-contact deltas in entry order, then apply_body_deltas.comp
// without constraint weights (q_in -> q_out)
void launch_body_particles(cudaStream_t s, BodyArrays ba, const uint2* seg, const uint32_t* sorted_entries,
                           const float4* bdel, const float4* q_in, const float4* qd_in, float4* q_out,
                           float4* qd_out, RigidParams rp);
// per body: solve_body_contact_positions.comp over its rigid contacts, then apply_body_deltas.comp
// with constraint weights (q_in -> q_out)
void launch_body_rigid(cudaStream_t s, BodyArrays ba, RigidTables rt, const float4* q_in, const float4* qd_in,
                       float4* q_out, float4* qd_out, RigidParams rp);

// ----------------------------------------------------------------- LBVH ----
// Per-mesh topology of the original binary tree (node slots 0 .. 2T-1, local
// indices), kept for the GPU refit.
struct LbvhTopology {
    int* parent;
    int* child_l;
    int* child_r;
    uint8_t* marked;       // node is a (collapsed) leaf
    uint8_t* reachable;    // node is reachable from the root of the collapsed tree
    uint32_t* prim_local;  // triangle of each leaf slot, mesh-local
};
size_t lbvh_scratch_words(int num_tris);
// Reach grids of all meshes (MeshTables::cull_*): mark the cells of every reachable
// leaf box of node slots [0, total_nodes) (node_off: first slot of each mesh, nm + 1
// entries), then dilate by each grid's reach along x, y and z. tmp has total_words.
void launch_cull_build(cudaStream_t s, int nm, const uint32_t* node_off, int64_t total_nodes,
                       const uint8_t* reachable, const float4* nl, const float4* nu, const float4* org,
                       const int4* dim, const uint32_t* off, int64_t total_words, uint32_t* bits, uint32_t* tmp);
// Sibling records of one mesh's reachable inner nodes (MeshTables::pair), after a
// build or refit of its node slots [node_base, node_base + 2 num_tris).
void launch_node_pairs(cudaStream_t s, int num_tris, uint32_t node_base, const uint8_t* reachable, const float4* nl,
                       const float4* nu, float4* pair);
// build of one mesh of num_tris triangles (tris: that mesh's triangles, global vertex
// indices) into the global node arrays at node_base, the primitive array at prim_base
// (triangle ids + tri_base) and *root_global
void launch_lbvh_build(cudaStream_t s, int num_tris, const float* verts, const uint32_t* tris, uint32_t node_base,
                       uint32_t prim_base, uint32_t tri_base, float4* nl, float4* nu, uint32_t* prim,
                       uint32_t* root_global, LbvhTopology topo, uint32_t* scratch, DeviceStatus* st);
// refit after the vertices moved; nl / nu point at the mesh's first node
void launch_lbvh_refit(cudaStream_t s, int num_tris, const float* verts, const uint32_t* tris, LbvhTopology topo,
                       float4* nl, float4* nu, uint32_t* scratch);

// -------------------------------------------------------------- adjoint ----
// One substep's adjoint (k_adjoint.cu). Arrays rx/rv/sids/table are the forward's
// sorted records of that substep; x0/v0/cinfo its start state and plane contacts;
// gx/gv the gradient of the loss with respect to the substep's end state (in) and
// start state (out; may alias the input); gw accumulates dL/d(inverse mass).
struct AdjointArgs {
    int64_t n;
    const uint32_t* sids;
    const float4* rx;
    const float4* rv;
    const int4* table;
    const uint32_t* stamp;
    const float4* x0;
    const float4* v0;
    const int* flags;
    const float4* gx_in;
    const float4* gv_in;
    float4* gx_out;
    float4* gv_out;
    float* gw;
    float4* gacc;      // scratch, sorted order: dL/d(sum_j pair_d) of each particle
    float4* part_xp;   // scratch, sorted order: own-state partials (w = dL/dw part)
    float4* part_vp;
    float4* part_x0;
    float4* part_v0;
    float4* part_gd;      // scratch, sorted order: dL/d delta
    float* block_params;  // 3 per block
    double* param_acc;    // [3]: plane mu (effective), particle mu, restitution
    float dt, inv, relax, ka, altitude, margin, mu_plane, k_mu, k_coh, max_radius, restitution;
    int restitution_on, plane_on, split_keys;
};
void launch_adjoint_substep(cudaStream_t s, const AdjointArgs& a);
// new generation for the stamped cell table (before a cell table is rebuilt without the key kernel)
void launch_bump_stamp(cudaStream_t s, uint32_t* stamp);
size_t adjoint_block_count(int64_t n);

// float4 state <-> packed xyz
void launch_unpack_xyz(cudaStream_t s, int64_t n, const float4* a, float* out);
void launch_pack_xyz(cudaStream_t s, int64_t n, const float* in, float4* a);

}  // namespace xpbd
