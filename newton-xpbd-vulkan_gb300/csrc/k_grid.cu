// Hash-grid construction: cell keys, onesweep radix sort, cell table + sorted
// particle records. Replaces grid_cell_indices.comp, gpu_sort.h's
// histogram/scan/scatter passes (sort_histogram.comp, sort_scan_{a,b,c}.comp,
// sort_scatter.comp) and grid_offsets.comp with its 16 MiB of fills.
#include <algorithm>
#include <atomic>
#include <stdexcept>
#include <string>

#include "kernels.h"
#include "particle.cuh"
#include "xmath.cuh"

namespace xpbd {

namespace {
std::atomic<int> g_sm_count[64];
}  // namespace

int device_sm_count() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaGetDevice failed: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) throw std::runtime_error("device ordinal out of range (at most 64 devices)");
    int c = g_sm_count[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
    e = cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || c <= 0)
        throw std::runtime_error(std::string("cudaDeviceGetAttribute(MultiProcessorCount) failed: ") +
                                 cudaGetErrorString(e));
    g_sm_count[dev].store(c, std::memory_order_relaxed);
    return c;
}

// ---------------------------------------------------------------------------
// Keys + digit histograms of every sort pass (+ plane contacts when no mesh)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_predict_keys(int64_t n, const float4* __restrict__ x,
                                                      const float4* __restrict__ v, const float* __restrict__ w,
                                                      const float* __restrict__ r, const int* __restrict__ flags,
                                                      const uint32_t* __restrict__ pscene, PredictParams pp,
                                                      PlaneParams pl, uint32_t* __restrict__ keys,
                                                      int bits, int passes, uint32_t* __restrict__ hist,
                                                      uint32_t* __restrict__ cinfo, uint32_t* ccount, uint32_t* stamp) {
    extern __shared__ uint32_t s_hist[];  // passes << bits
    __shared__ uint32_t s_warp[8];
    const int bins = 1 << bits;
    for (int i = threadIdx.x; i < passes * bins; i += blockDim.x) s_hist[i] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0 && stamp) *stamp += 1u;  // new grid generation for this substep
    __syncthreads();
    uint32_t contacts = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // the trip count is uniform across the block so every lane takes part in match_any
    const int64_t trips = (n + stride - 1) / stride;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t i = t * stride + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0;
        if (valid) {
            const float4 xf = x[i];
            const int fl = flags[i];
            v3 xp, vp;
            predict(xf, v[i], w[i], fl, pp, xp, vp);
            // one scene: split key; batched: scene-major key = entry of the scene's table
            key = pscene ? (hash_grid_index(xp, pp.inv, false) | (pscene[i] << 21))
                         : hash_grid_index(xp, pp.inv, pp.split_keys != 0);
            keys[i] = key;
            if (cinfo) {  // generate_plane_contacts.comp:32-38 on the pre-integration position
                uint32_t info = 0;
                if (pl.enabled && (fl & 1)) {
                    float dist = xf.z - pl.altitude;
                    if (dist < pl.margin + r[i]) info = kPlaneBit;
                }
                cinfo[i] = info;
                contacts += info;
            }
        }
        for (int p = 0; p < passes; p++) {
            const uint32_t d = valid ? ((key >> (p * bits)) & (uint32_t)(bins - 1)) : 0xffffffffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&s_hist[p * bins + d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * bins; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
    if (cinfo) {
        uint32_t tot = block_sum(contacts, s_warp);
        if (threadIdx.x == 0 && tot) atomicAdd(ccount, tot);
    }
}

void launch_predict_keys(cudaStream_t s, int64_t n, const float4* x, const float4* v, const float* w,
                         const float* r, const int* flags, const uint32_t* pscene, PredictParams pp, PlaneParams pl,
                         uint32_t* keys, const SortPlan& sp, uint32_t* hist, uint32_t* cinfo, uint32_t* ccount,
                         uint32_t* stamp) {
    if (n <= 0) return;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sm_count() * 8);
    const int passes = hist ? sp.passes : 0;  // no histogram wanted: none built
    size_t smem = sizeof(uint32_t) * (size_t)passes << sp.bits;
    k_predict_keys<<<blocks, 256, smem, s>>>(n, x, v, w, r, flags, pscene, pp, pl, keys, sp.bits, passes, hist,
                                            cinfo, ccount, stamp);
}

// out[i] = keys[i] & mask and the digit histograms of every pass (the reference-layout view
// of split keys, sorted on demand for the sorted-order getters)
__global__ void __launch_bounds__(256) k_mask_keys(int64_t n, const uint32_t* __restrict__ keys, uint32_t mask,
                                                   uint32_t* __restrict__ out, int bits, int passes,
                                                   uint32_t* __restrict__ hist) {
    extern __shared__ uint32_t s_hist[];  // passes << bits
    const int bins = 1 << bits;
    for (int i = threadIdx.x; i < passes * bins; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t key = keys[i] & mask;
        out[i] = key;
        for (int p = 0; p < passes; p++) atomicAdd(&s_hist[p * bins + ((key >> (p * bits)) & (uint32_t)(bins - 1))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * bins; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

void launch_mask_keys(cudaStream_t s, int64_t n, const uint32_t* keys, uint32_t mask, uint32_t* out,
                      const SortPlan& sp, uint32_t* hist) {
    if (n <= 0) return;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sm_count() * 8);
    k_mask_keys<<<blocks, 256, sizeof(uint32_t) * ((size_t)sp.passes << sp.bits), s>>>(n, keys, mask, out, sp.bits,
                                                                                      sp.passes, hist);
}

// grid_offsets.comp:16-34 over sorted keys of the reference layout (starts and ends zeroed
// first, as the zero fills of scene.cpp:918-922)
__global__ void k_cell_bounds(int64_t n, const uint32_t* __restrict__ skeys, int32_t* __restrict__ starts,
                              int32_t* __restrict__ ends) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t c = skeys[t];
    if (t == 0 || skeys[t - 1] != c) starts[c] = (int32_t)t;
    if (t == n - 1 || skeys[t + 1] != c) ends[c] = (int32_t)(t + 1);
}

void launch_cell_bounds(cudaStream_t s, int64_t n, const uint32_t* skeys, int32_t* starts, int32_t* ends) {
    cudaMemsetAsync(starts, 0, sizeof(int32_t) * kNumCells, s);
    cudaMemsetAsync(ends, 0, sizeof(int32_t) * kNumCells, s);
    if (n > 0) k_cell_bounds<<<(int)((n + 255) / 256), 256, 0, s>>>(n, skeys, starts, ends);
}

// ---------------------------------------------------------------------------
// Onesweep pass (stable LSD radix sort with decoupled look-back)
//
// Tiles take a ticket from an atomic counter so that a tile only waits on
// tiles that started earlier. Inside a tile every warp ranks its keys in index
// order with __match_any_sync (stable), warp-local digit counts are turned
// into tile offsets with warp-shuffle scans, the tile publishes its per-digit
// aggregate, looks back over its predecessors, and finally scatters through
// shared memory so that global writes run in digit order (coalesced).
// Every look-back wait is bounded by a 1 s timer; on expiry the kernel sets
// kErrLookbackTimeout and continues (the host raises an error).
// ---------------------------------------------------------------------------
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr uint64_t kWaitLimitNs = 1000000000ull;
constexpr int kLookWindow = 8;
constexpr uint32_t kNoHold = 0xffffffffu;

namespace {
// test hook of the bounded wait (set_lookback_debug): tile g_hold_tile of the first pass
// of every sort never publishes, and waits give up after g_wait_ns
std::atomic<uint32_t> g_hold_tile{kNoHold};
std::atomic<uint64_t> g_wait_ns{kWaitLimitNs};
std::atomic<uint32_t> g_debug_generation{0};
}  // namespace

void set_lookback_debug(int64_t hold_tile, uint64_t wait_ns) {
    if (hold_tile < 0) {
        g_hold_tile.store(kNoHold);
        g_wait_ns.store(kWaitLimitNs);
    } else {
        if (hold_tile >= (int64_t)kNoHold) throw std::runtime_error("set_lookback_debug: tile index too large");
        if (wait_ns == 0 || wait_ns > kWaitLimitNs)
            throw std::runtime_error("set_lookback_debug: wait limit must be in (0, 1 s]");
        g_hold_tile.store((uint32_t)hold_tile);
        g_wait_ns.store(wait_ns);
    }
    g_debug_generation.fetch_add(1u);
}
uint32_t lookback_debug_generation() { return g_debug_generation.load(); }

template <int THREADS>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_scan, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_scan[warp] = incl;
    __syncthreads();
    uint32_t off = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < THREADS / 32; i++) {
        uint32_t t = s_scan[i];
        if (i < warp) off += t;
        tot += t;
    }
    __syncthreads();
    total = tot;
    return off + incl - v;
}

template <int BITS, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS) k_onesweep(int64_t n, int shift, const uint32_t* __restrict__ keys_in,
                                                      const uint32_t* __restrict__ vals_in,
                                                      uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                      const uint32_t* __restrict__ hist, uint32_t* lookback,
                                                      uint32_t* tile_counter, DeviceStatus* st,
                                                      const uint32_t* __restrict__ n_dev, uint32_t hold_tile,
                                                      uint64_t wait_ns) {
    constexpr int BINS = 1 << BITS;
    constexpr int WARPS = THREADS / 32;
    constexpr int TILE = THREADS * ITEMS;
    static_assert(BINS == THREADS, "one digit per thread");
    extern __shared__ uint32_t smem[];
    uint32_t* s_whist = smem;                 // WARPS * BINS
    uint32_t* s_keys = s_whist + WARPS * BINS;  // TILE
    uint32_t* s_vals = s_keys + TILE;          // TILE
    uint32_t* s_gbase = s_vals + TILE;         // BINS
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_scan[WARPS];
    __shared__ uint32_t s_texcl[BINS];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = tid; i < WARPS * BINS; i += THREADS) s_whist[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const int64_t base = (int64_t)tile * TILE;
    if (n_dev) {  // device-side count: the tiles past it have nothing to sort and nobody waits on them
        const int64_t nd = (int64_t)*n_dev;
        if (nd < n) n = nd;
        if (base >= n) return;
    }
    const int valid_n = (n - base) < (int64_t)TILE ? (int)(n - base) : TILE;
    const uint32_t lt = lanemask_lt();

    uint32_t kreg[ITEMS], vreg[ITEMS], rreg[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
        const int local = warp * 32 * ITEMS + j * 32 + lane;
        const bool valid = local < valid_n;
        const int64_t gi = base + local;
        uint32_t key = 0, val = 0;
        if (valid) {
            key = keys_in[gi];
            val = vals_in ? vals_in[gi] : (uint32_t)gi;
        }
        const uint32_t d = valid ? ((key >> shift) & (BINS - 1)) : (uint32_t)BINS;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t old = 0;
        if (valid) old = s_whist[warp * BINS + d];
        __syncwarp();
        if (valid && (peers & lt) == 0) s_whist[warp * BINS + d] = old + __popc(peers);
        __syncwarp();
        kreg[j] = key;
        vreg[j] = val;
        rreg[j] = old + __popc(peers & lt);
    }
    __syncthreads();

    // thread `tid` owns digit `tid`: warp prefix (in place) and tile total
    uint32_t tot = 0;
#pragma unroll
    for (int wv = 0; wv < WARPS; wv++) {
        uint32_t c = s_whist[wv * BINS + tid];
        s_whist[wv * BINS + tid] = tot;
        tot += c;
    }
    uint32_t dummy;
    const uint32_t tile_excl = block_excl_scan<THREADS>(tot, s_scan, dummy);
    const uint32_t glob_excl = block_excl_scan<THREADS>(hist[tid], s_scan, dummy);

    // decoupled look-back for digit `tid`, kLookWindow predecessors per round trip: when
    // all tiles start together every predecessor holds only its aggregate at first, and
    // a one-tile-at-a-time walk costs one dependent load per tile. A status word holds
    // its flag and count together and nothing else a predecessor wrote is read here, so
    // relaxed loads (all of a window in flight at once) suffice.
    uint32_t* my = lookback + (size_t)tile * BINS + tid;
    uint32_t prev = 0;
    // a held tile (test hook) publishes nothing: its successor's wait runs out
    const bool publish = tile != hold_tile;
    if (tile == 0) {
        if (publish) st_release(my, kFlagInc | tot);
    } else {
        if (publish) st_release(my, kFlagAgg | tot);
        int64_t p = (int64_t)tile - 1;
        uint64_t t0 = 0;
        bool found = false;
        while (!found) {
            uint32_t sv[kLookWindow];
#pragma unroll
            for (int j = 0; j < kLookWindow; j++)
                sv[j] = p - j >= 0 ? ld_relaxed(lookback + (size_t)(p - j) * BINS + tid) : kFlagInc;
            int used = 0;  // leading published entries consumed, nearest first
#pragma unroll
            for (int j = 0; j < kLookWindow; j++) {
                if (used != j || found) continue;
                const uint32_t flag = sv[j] & ~kCountMask;
                if (flag == 0) continue;  // not published yet: resume from here
                prev += sv[j] & kCountMask;
                used = j + 1;
                if (flag == kFlagInc) found = true;
            }
            if (found) break;
            if (used == 0) {
                const uint64_t now = globaltimer_ns();
                if (t0 == 0) {
                    t0 = now;
                } else if (now - t0 > wait_ns) {
                    atomicOr(&st->error_bits, kErrLookbackTimeout);
                    atomicAdd(&st->lookback_timeouts, 1u);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            p -= used;
            t0 = 0;
        }
        if (publish) st_release(my, kFlagInc | ((prev + tot) & kCountMask));
    }
    // output slot = s_gbase[d] + position in the tile's digit-sorted order (modular arithmetic)
    s_gbase[tid] = glob_excl + prev - tile_excl;
    s_texcl[tid] = tile_excl;
    __syncthreads();
    // tile-sorted position = tile digit start + warp prefix + rank within the warp
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
        const int local = warp * 32 * ITEMS + j * 32 + lane;
        if (local < valid_n) {
            const uint32_t d = (kreg[j] >> shift) & (BINS - 1);
            const uint32_t pos = s_texcl[d] + s_whist[warp * BINS + d] + rreg[j];
            s_keys[pos] = kreg[j];
            s_vals[pos] = vreg[j];
        }
    }
    __syncthreads();
    // A slot is below n whenever the histograms match the input and every look-back
    // completed. After a wait that ran out, this pass's slots are still below n, but the
    // next pass's input then holds duplicates and holes that its (up-front) histograms do
    // not count, so its slots could run past n: the bound keeps a failed sort in range.
    const uint32_t n_out = (uint32_t)n;
    for (int i = tid; i < valid_n; i += THREADS) {
        const uint32_t key = s_keys[i];
        const uint32_t g = s_gbase[(key >> shift) & (BINS - 1)] + (uint32_t)i;
        if (g < n_out) {
            keys_out[g] = key;
            vals_out[g] = s_vals[i];
        }
    }
}

SortPlan make_sort_plan(int64_t n, int key_bits, int bits, int items) {
    if (bits != 8 && bits != 7) throw std::runtime_error("unsupported radix digit width");
    SortPlan p;
    p.bits = bits;
    p.passes = (key_bits + bits - 1) / bits;
    p.threads = 1 << bits;
    p.items = items;
    p.tile = p.threads * items;
    p.tiles = (int)((n + p.tile - 1) / p.tile);
    if (p.tiles < 1) p.tiles = 1;
    return p;
}
size_t sort_lookback_words(const SortPlan& p) { return (size_t)p.tiles << p.bits; }

template <int BITS, int ITEMS>
static void onesweep_variant(cudaStream_t s, int64_t n, const SortPlan& sp, int pass, const uint32_t* ki,
                             const uint32_t* vi, uint32_t* ko, uint32_t* vo, const uint32_t* hist, uint32_t* lb,
                             uint32_t* tc, DeviceStatus* st, const uint32_t* n_dev, bool debug_hold) {
    constexpr int THREADS = 1 << BITS;
    constexpr int TILE = THREADS * ITEMS;
    size_t smem = sizeof(uint32_t) * ((size_t)(THREADS / 32) * (1 << BITS) + 2 * TILE + (1 << BITS));
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_onesweep<BITS, THREADS, ITEMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        attr_set = true;
    }
    const uint32_t hold = (debug_hold && pass == 0) ? g_hold_tile.load() : kNoHold;
    k_onesweep<BITS, THREADS, ITEMS><<<sp.tiles, THREADS, smem, s>>>(n, pass * BITS, ki, vi, ko, vo, hist, lb, tc,
                                                                     st, n_dev, hold, g_wait_ns.load());
}

void launch_onesweep_pass(cudaStream_t s, int64_t n, const SortPlan& sp, int pass, const uint32_t* keys_in,
                          const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                          const uint32_t* hist_pass, uint32_t* lookback, uint32_t* tile_counter,
                          DeviceStatus* st, const uint32_t* n_dev, bool debug_hold) {
    if (n <= 0) return;
#define XPBD_OS(B, I)                                                                                      \
    if (sp.bits == B && sp.items == I)                                                                     \
        return onesweep_variant<B, I>(s, n, sp, pass, keys_in, vals_in, keys_out, vals_out, hist_pass, \
                                      lookback, tile_counter, st, n_dev, debug_hold);
    XPBD_OS(8, 2)
    XPBD_OS(8, 4)
    XPBD_OS(8, 8)
    XPBD_OS(8, 16)
    XPBD_OS(7, 4)
    XPBD_OS(7, 8)
    XPBD_OS(7, 16)
    XPBD_OS(7, 32)
#undef XPBD_OS
    throw std::runtime_error("no onesweep variant for this sort plan");
}

// ---------------------------------------------------------------------------
// Small sorts: every pass of the stable LSD radix sort of at most kSmallSortKeys keys in one
// block and one launch, the keys held in shared memory between passes (a small scene's sort
// is three dependent launches of one tile otherwise). Each pass ranks the keys as a onesweep
// tile does (warps in index order, __match_any_sync within a warp), so the permutation is
// the same stable order.
// ---------------------------------------------------------------------------
constexpr int kSmallSortThreads = 256, kSmallSortItems = 16;
constexpr int kSmallSortKeys = kSmallSortThreads * kSmallSortItems;
static_assert(kSmallSortKeys == kSmallSortMaxKeys, "the one-block sort's capacity");

__global__ void __launch_bounds__(kSmallSortThreads) k_sort_small(int n, int passes, const uint32_t* __restrict__ keys_in,
                                                                  uint32_t* __restrict__ keys_out,
                                                                  uint32_t* __restrict__ vals_out) {
    constexpr int BITS = 8, BINS = 1 << BITS, THREADS = kSmallSortThreads, ITEMS = kSmallSortItems;
    constexpr int WARPS = THREADS / 32, TILE = kSmallSortKeys;
    static_assert(BINS == THREADS, "one digit per thread");
    extern __shared__ uint32_t smem[];
    uint32_t* s_k[2] = {smem, smem + TILE};
    uint32_t* s_v[2] = {smem + 2 * TILE, smem + 3 * TILE};
    uint32_t* s_whist = smem + 4 * TILE;  // WARPS * BINS
    __shared__ uint32_t s_scan[WARPS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < n; i += THREADS) {
        s_k[0][i] = keys_in[i];
        s_v[0][i] = (uint32_t)i;
    }
    const uint32_t lt = lanemask_lt();
    int cur = 0;
    for (int p = 0; p < passes; p++) {
        for (int i = tid; i < WARPS * BINS; i += THREADS) s_whist[i] = 0;
        __syncthreads();
        uint32_t kreg[ITEMS], vreg[ITEMS], rreg[ITEMS], dreg[ITEMS];
#pragma unroll
        for (int j = 0; j < ITEMS; j++) {
            const int local = warp * 32 * ITEMS + j * 32 + lane;
            const bool valid = local < n;
            const uint32_t key = valid ? s_k[cur][local] : 0u;
            const uint32_t d = valid ? ((key >> (p * BITS)) & (BINS - 1)) : (uint32_t)BINS;
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            uint32_t old = 0;
            if (valid) old = s_whist[warp * BINS + d];
            __syncwarp();
            if (valid && (peers & lt) == 0) s_whist[warp * BINS + d] = old + __popc(peers);
            __syncwarp();
            kreg[j] = key;
            vreg[j] = valid ? s_v[cur][local] : 0u;
            rreg[j] = old + __popc(peers & lt);
            dreg[j] = d;
        }
        __syncthreads();
        // thread `tid` owns digit `tid`: the warps' exclusive prefix in place, the digit's total
        uint32_t tot = 0;
        for (int wv = 0; wv < WARPS; wv++) {
            const uint32_t c = s_whist[wv * BINS + tid];
            s_whist[wv * BINS + tid] = tot;
            tot += c;
        }
        uint32_t dummy;
        const uint32_t digit_base = block_excl_scan<THREADS>(tot, s_scan, dummy);
        // each (warp, digit) start = digit start + the warps before it
        for (int wv = 0; wv < WARPS; wv++) s_whist[wv * BINS + tid] += digit_base;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < ITEMS; j++) {
            if (dreg[j] < (uint32_t)BINS) {
                const uint32_t dst = s_whist[warp * BINS + dreg[j]] + rreg[j];
                s_k[cur ^ 1][dst] = kreg[j];
                s_v[cur ^ 1][dst] = vreg[j];
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    for (int i = tid; i < n; i += THREADS) {
        keys_out[i] = s_k[cur][i];
        vals_out[i] = s_v[cur][i];
    }
}

bool launch_sort_small(cudaStream_t s, int64_t n, int key_bits, const uint32_t* keys_in, uint32_t* keys_out,
                       uint32_t* vals_out) {
    if (n <= 0 || n > kSmallSortKeys) return false;
    const size_t smem = sizeof(uint32_t) * ((size_t)4 * kSmallSortKeys + (size_t)(kSmallSortThreads / 32) * 256);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_sort_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr_set = true;
    }
    k_sort_small<<<1, kSmallSortThreads, smem, s>>>((int)n, (key_bits + 7) / 8, keys_in, keys_out, vals_out);
    return true;
}

// ---------------------------------------------------------------------------
// Cell table (start, end, generation stamp) + sorted-order particle records
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_cells_gather(int64_t n, const uint32_t* __restrict__ skeys,
                                                      const uint32_t* __restrict__ sids, const float4* __restrict__ x,
                                                      const float4* __restrict__ v, const float* __restrict__ w,
                                                      const float* __restrict__ r, const int* __restrict__ flags,
                                                      PredictParams pp, int* __restrict__ table,
                                                      const uint32_t* __restrict__ stamp, float4* __restrict__ rx,
                                                      float4* __restrict__ rv, int* __restrict__ rf) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = skeys[k];
    // grid_offsets.comp:20-34 without the table fills: a stale entry is
    // recognised by its generation stamp instead of being zeroed
    if (k == 0 || skeys[k - 1] != key) {
        table[(size_t)key * 4 + 0] = (int)k;
        table[(size_t)key * 4 + 2] = (int)*stamp;
    }
    if (k == n - 1 || skeys[k + 1] != key) table[(size_t)key * 4 + 1] = (int)(k + 1);
    const uint32_t id = sids[k];
    const int fl = flags[id];
    const float wi = w[id];
    v3 xp, vp;
    predict(x[id], v[id], wi, fl, pp, xp, vp);
    rx[k] = make_float4(xp.x, xp.y, xp.z, r[id]);
    rv[k] = make_float4(vp.x, vp.y, vp.z, wi);
    rf[k] = fl;
}

void launch_cells_gather(cudaStream_t s, int64_t n, const uint32_t* skeys, const uint32_t* sids, const float4* x,
                         const float4* v, const float* w, const float* r, const int* flags, PredictParams pp,
                         int4* table, const uint32_t* stamp, float4* rx, float4* rv, int* rf) {
    if (n <= 0) return;
    int blocks = (int)((n + 255) / 256);
    k_cells_gather<<<blocks, 256, 0, s>>>(n, skeys, sids, x, v, w, r, flags, pp, reinterpret_cast<int*>(table),
                                          stamp, rx, rv, rf);
}

}  // namespace xpbd
