// Error type used inside the library; the C ABI converts it into a status code and a message.
#pragma once

#include <stdint.h>

#include <stdexcept>
#include <string>

#include <cuda_runtime_api.h>

#include "../../include/reina/reina_c.h"

namespace rt {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] inline void fail(int code, const std::string& msg) { throw Error(code, msg); }

// The meaning of the bits of a device error word, for messages: bit 1 traversal stack overflow, bit 2
// traversal step limit, bit 4 queue or path index out of range (checked build).
inline std::string device_error_text(uint32_t e) {
    std::string t;
    if (e & 1u) t += " (traversal stack overflow)";
    if (e & 2u) t += " (traversal step limit)";
    if (e & 4u) t += " (queue or path index out of range, checked build)";
    return t;
}

inline void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation) fail(REINA_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
        fail(REINA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// Owning device allocation (cudaMalloc / cudaFree).
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) { alloc(bytes); }
    ~DeviceBuffer() { release(); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_), stream_(o.stream_), async_(o.async_) {
        o.ptr_ = nullptr; o.bytes_ = 0; o.async_ = false;
    }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
        if (this != &o) {
            release();
            ptr_ = o.ptr_; bytes_ = o.bytes_; stream_ = o.stream_; async_ = o.async_;
            o.ptr_ = nullptr; o.bytes_ = 0; o.async_ = false;
        }
        return *this;
    }
    void alloc(size_t bytes) {
        release();
        if (bytes == 0) return;
        check_cuda(cudaMalloc(&ptr_, bytes), "cudaMalloc");
        bytes_ = bytes;
    }
    // Stream-ordered allocation from `pool` on `st`; release() then frees it on the same stream, without
    // the device-wide synchronization a plain free can cause.  Usable on other streams once they are
    // ordered after `st`.
    void alloc_async(size_t bytes, cudaMemPool_t pool, cudaStream_t st) {
        release();
        if (bytes == 0) return;
        check_cuda(cudaMallocFromPoolAsync(&ptr_, bytes, pool, st), "cudaMallocFromPoolAsync");
        bytes_ = bytes;
        stream_ = st;
        async_ = true;
    }
    // Grows (never shrinks) the allocation to at least `bytes`; contents are not preserved.
    void reserve(size_t bytes) { if (bytes > bytes_) alloc(bytes); }
    void release() {
        if (ptr_) {
            if (async_) cudaFreeAsync(ptr_, stream_);
            else cudaFree(ptr_);
        }
        ptr_ = nullptr;
        bytes_ = 0;
        async_ = false;
    }
    template <class T> T* as() const { return static_cast<T*>(ptr_); }
    void* get() const { return ptr_; }
    size_t bytes() const { return bytes_; }
    void upload(const void* src, size_t bytes) {
        reserve(bytes);
        if (bytes) check_cuda(cudaMemcpy(ptr_, src, bytes, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    }

private:
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
    cudaStream_t stream_ = nullptr;
    bool async_ = false;
};

}  // namespace rt
