// Allocation-free stable key sort: the hash-grid onesweep sort with its scratch
// memory in a file-scope device array instead of cudaMalloc'd buffers.
//
// Who needs it: code that must not allocate device memory while it runs — work
// recorded into a CUDA graph owned by another framework (an allocation would
// have to be captured too), callbacks and plugins that run inside a host
// application whose device memory is handed out by its own pool allocator, and
// real-time loops that forbid allocator calls (and their implicit device
// synchronisation) after start-up. They pass input and output buffers; every
// other byte the sort touches lives in g_noalloc_scratch below.
//
// Limits: at most kNoAllocMaxKeys keys per call. The array (about 10.5 MiB) is
// held by every GPU that loads this module until the process exits. All calls
// share it: calls that overlap on the GPU (different streams, or different host
// threads without ordering) race on it and give wrong results. The histograms,
// look-back words, tile counters and status block are cleared at the start of
// every call. The input must not overlap either output (a pass may write the
// output while an earlier one still reads the input). A call returns once the
// sort has finished on its stream: it reads back the status block, and a
// look-back wait that ran out (the output is then wrong) makes the call fail. A call
// recorded into a stream capture only records the sort; the status block then holds
// each replay's outcome (sort_keys_noalloc_status reads it).
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "kernels.h"
#include "solver.h"
#include "xmath.cuh"

#define XPBD_CUDA_NOALLOC(x) XPBD_CUDA(x)

namespace xpbd {

constexpr int64_t kNoAllocMaxKeys = int64_t(1) << 20;
constexpr int kNoAllocBits = 8;     // digit width
constexpr int kNoAllocItems = 8;    // keys per thread -> 2048-key tiles
constexpr int kNoAllocMaxPasses = 4;
constexpr int64_t kNoAllocTiles = kNoAllocMaxKeys / ((int64_t(1) << kNoAllocBits) * kNoAllocItems);
// layout (32-bit words): pair keys | pair ids | histograms | look-back | tile counters
constexpr int64_t kNaPairK = 0;
constexpr int64_t kNaPairV = kNaPairK + kNoAllocMaxKeys;
constexpr int64_t kNaHist = kNaPairV + kNoAllocMaxKeys;
constexpr int64_t kNaLook = kNaHist + (int64_t)kNoAllocMaxPasses * (1 << kNoAllocBits);
constexpr int64_t kNaTiles = kNaLook + (int64_t)kNoAllocMaxPasses * kNoAllocTiles * (1 << kNoAllocBits);
constexpr int64_t kNaStatus = kNaTiles + kNoAllocMaxPasses;  // DeviceStatus (8 words)
constexpr int64_t kNaWords = kNaStatus + 8;
static_assert(sizeof(DeviceStatus) == 8 * sizeof(uint32_t), "status block size");

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNaWords];

// per-pass digit histograms of the input keys
__global__ void __launch_bounds__(256) k_key_hist(int64_t n, const uint32_t* __restrict__ keys, int bits, int passes,
                                                  uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_hist[kNoAllocMaxPasses << kNoAllocBits];
    const int bins = 1 << bits;
    for (int i = threadIdx.x; i < passes * bins; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t trips = (n + stride - 1) / stride;
    for (int64_t t = 0; t < trips; t++) {
        const int64_t i = t * stride + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? keys[i] : 0u;
        for (int p = 0; p < passes; p++) {
            const uint32_t d = valid ? ((key >> (p * bits)) & (uint32_t)(bins - 1)) : 0xffffffffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&s_hist[p * bins + d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * bins; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

namespace {
std::mutex g_setup_mutex;
uint32_t* g_scratch_ptr[64] = {nullptr};  // device address of g_noalloc_scratch per device ordinal

// Resolves the device address of the scratch array for the current device. The
// name g_noalloc_scratch in host code is only a host-side stand-in, so kernels
// get this address instead. Done once per device, on that device's first call.
uint32_t* scratch_for_current_device() {
    int dev = 0;
    XPBD_CUDA_NOALLOC(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw std::runtime_error("xpbd_sort_keys_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw std::runtime_error(std::string("xpbd_sort_keys_noalloc: cudaGetSymbolAddress failed: ") +
                                     cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<uint32_t*>(p);
    }
    return g_scratch_ptr[dev];
}
}  // namespace

void sort_keys_noalloc(const uint32_t* keys, uint32_t* sorted_keys, uint32_t* sorted_ids, int64_t n, int key_bits,
                       cudaStream_t s) {
    if (n < 0 || n > kNoAllocMaxKeys)
        throw std::runtime_error("xpbd_sort_keys_noalloc: n must be at most 1048576 keys");
    if (key_bits < 1 || key_bits > 32) throw std::runtime_error("xpbd_sort_keys_noalloc: key_bits must be in 1..32");
    if (n == 0) return;
    if (!keys || !sorted_keys || !sorted_ids) throw std::runtime_error("xpbd_sort_keys_noalloc: null buffer");
    const auto overlap = [n](const uint32_t* a, const uint32_t* b) { return a < b + n && b < a + n; };
    if (overlap(keys, sorted_keys) || overlap(keys, sorted_ids) || overlap(sorted_keys, sorted_ids))
        throw std::runtime_error("xpbd_sort_keys_noalloc: the input and output buffers must not overlap");
    uint32_t* base = scratch_for_current_device();
    const SortPlan plan = make_sort_plan(n, key_bits, kNoAllocBits, kNoAllocItems);
    // zero histograms, look-back words and tile counters (the key/id pair needs no clearing)
    XPBD_CUDA_NOALLOC(cudaMemsetAsync(base + kNaHist, 0, (size_t)(kNaWords - kNaHist) * sizeof(uint32_t), s));
    const int64_t max_blocks = (int64_t)device_sm_count() * 8;
    const int blocks = (int)((n + 255) / 256 < max_blocks ? (n + 255) / 256 : max_blocks);
    k_key_hist<<<blocks, 256, 0, s>>>(n, keys, plan.bits, plan.passes, base + kNaHist);
    XPBD_CUDA_NOALLOC(cudaGetLastError());
    // ping-pong so that the last pass lands in the caller's output buffers
    const uint32_t* kin = keys;
    const uint32_t* vin = nullptr;
    for (int p = 0; p < plan.passes; p++) {
        const bool to_out = ((plan.passes - 1 - p) & 1) == 0;
        uint32_t* ko = to_out ? sorted_keys : base + kNaPairK;
        uint32_t* vo = to_out ? sorted_ids : base + kNaPairV;
        launch_onesweep_pass(s, n, plan, p, kin, vin, ko, vo, base + kNaHist + ((int64_t)p << plan.bits),
                             base + kNaLook + (int64_t)p * kNoAllocTiles * (1 << kNoAllocBits),
                             base + kNaTiles + p, reinterpret_cast<DeviceStatus*>(base + kNaStatus), nullptr,
                             true);
        XPBD_CUDA(cudaGetLastError());
        kin = ko;
        vin = vo;
    }
    // recorded into a graph (a stream capture allows no synchronisation): the status block
    // holds each replay's outcome, read with sort_keys_noalloc_status after the replay
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    XPBD_CUDA_NOALLOC(cudaStreamIsCapturing(s, &capturing));
    if (capturing != cudaStreamCaptureStatusNone) return;
    // the status block of this call (a bounded look-back wait sets a bit instead of hanging)
    DeviceStatus host{};
    XPBD_CUDA_NOALLOC(
        cudaMemcpyAsync(&host, base + kNaStatus, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
    XPBD_CUDA_NOALLOC(cudaStreamSynchronize(s));
    if (host.error_bits & kErrLookbackTimeout)
        throw std::runtime_error("xpbd_sort_keys_noalloc: device wait timed out in the onesweep look-back "
                                 "(output invalid)");
}

void sort_keys_noalloc_status() {
    uint32_t* base = scratch_for_current_device();
    DeviceStatus host{};
    XPBD_CUDA_NOALLOC(cudaMemcpy(&host, base + kNaStatus, sizeof(DeviceStatus), cudaMemcpyDeviceToHost));
    if (host.error_bits & kErrLookbackTimeout)
        throw std::runtime_error("xpbd_sort_keys_noalloc: device wait timed out in the onesweep look-back "
                                 "(output invalid)");
}

}  // namespace xpbd
