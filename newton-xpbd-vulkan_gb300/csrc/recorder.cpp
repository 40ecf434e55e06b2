// Frame recorder: the add-on's per-frame cache (newton_vulkan_plugin.py:626-631
// saves get_positions() as frame_%04d.npy after every step) without the wait.
// After each frame's graph the positions are unpacked on the solver's stream
// and copied into one of a few pinned host slots; a writer thread waits for that
// copy's event and writes the .npy file while the GPU runs the next frame.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "solver.h"

namespace xpbd {

namespace {
// NPY format 1.0: magic, version, little-endian header length, a Python dict literal
// padded with spaces to a multiple of 64 bytes including the trailing newline.
std::string npy_header(size_t n) {
    std::string dict = "{'descr': '<f4', 'fortran_order': False, 'shape': (" + std::to_string(n) + ", 3), }";
    const size_t base = 10;
    size_t total = base + dict.size() + 1;
    const size_t pad = (64 - total % 64) % 64;
    dict.append(pad, ' ');
    dict.push_back('\n');
    std::string h("\x93NUMPY\x01\x00", 8);
    const uint16_t len = (uint16_t)dict.size();
    h.push_back((char)(len & 0xff));
    h.push_back((char)(len >> 8));
    return h + dict;
}
}  // namespace

FrameRecorder::~FrameRecorder() {
    try {
        stop();
    } catch (...) {
    }
}

void FrameRecorder::start(int device, size_t n, const std::string& dir, int first_frame) {
    stop();
    device_ = device;
    n_ = n;
    dir_ = dir;
    next_frame_ = first_frame;
    written_ = 0;
    error_.clear();
    header_ = npy_header(n);
    for (Slot& s : slots_) {
        XPBD_CUDA(cudaMallocHost(&s.host, std::max<size_t>(n, 1) * 3 * sizeof(float)));
        XPBD_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
        s.busy = false;
    }
    stop_flag_ = false;
    active_ = true;
    worker_ = std::thread([this] { run(); });
}

int FrameRecorder::stop() {
    if (!active_) return written_;
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_flag_ = true;
    }
    cv_.notify_all();
    worker_.join();
    for (Slot& s : slots_) {
        cudaFreeHost(s.host);
        cudaEventDestroy(s.done);
        s.host = nullptr;
        s.done = nullptr;
    }
    active_ = false;
    if (!error_.empty()) throw std::runtime_error(error_);
    return written_;
}

// Queues this frame's positions (device xyz staging already filled on `stream`).
void FrameRecorder::enqueue(cudaStream_t stream, const float* d_xyz) {
    if (!active_) return;
    std::unique_lock<std::mutex> lk(mu_);
    if (!error_.empty()) throw std::runtime_error(error_);
    int slot = -1;
    cv_.wait(lk, [&] {
        for (int k = 0; k < kSlots; k++)
            if (!slots_[k].busy) {
                slot = k;
                return true;
            }
        return false;
    });
    Slot& s = slots_[slot];
    s.busy = true;
    s.frame = next_frame_++;
    lk.unlock();
    XPBD_CUDA(cudaMemcpyAsync(s.host, d_xyz, n_ * 3 * sizeof(float), cudaMemcpyDeviceToHost, stream));
    XPBD_CUDA(cudaEventRecord(s.done, stream));
    lk.lock();
    queue_.push_back(slot);
    lk.unlock();
    cv_.notify_all();
}

void FrameRecorder::run() {
    cudaSetDevice(device_);
    while (true) {
        int slot;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return stop_flag_ || !queue_.empty(); });
            if (queue_.empty()) return;  // stopping and nothing left
            slot = queue_.front();
            queue_.pop_front();
        }
        Slot& s = slots_[slot];
        std::string err;
        if (cudaEventSynchronize(s.done) != cudaSuccess) err = "frame recorder: copy failed";
        if (err.empty()) {
            char name[32];
            std::snprintf(name, sizeof(name), "frame_%04d.npy", s.frame);
            const std::string path = dir_ + "/" + name;
            FILE* f = std::fopen(path.c_str(), "wb");
            if (!f) {
                err = "frame recorder: cannot open " + path + ": " + std::strerror(errno);
            } else {
                const size_t bytes = n_ * 3 * sizeof(float);
                bool ok = std::fwrite(header_.data(), 1, header_.size(), f) == header_.size();
                ok = ok && std::fwrite(s.host, 1, bytes, f) == bytes;
                ok = (std::fclose(f) == 0) && ok;
                if (!ok) err = "frame recorder: write failed for " + path;
            }
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (!err.empty() && error_.empty()) error_ = err;
            if (err.empty()) written_++;
            s.busy = false;
        }
        cv_.notify_all();
    }
}

}  // namespace xpbd
