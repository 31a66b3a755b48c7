// kf_util.h — error type, CUDA checks and device-memory ownership helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/kf.h"

namespace kf {

// Internal exception; converted to a status code + kf_last_error() at the C-ABI.
struct KfError : std::runtime_error {
    int code;
    KfError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define KF_CUDA_CHECK(x)                                                                                   \
    do {                                                                                                   \
        cudaError_t e_ = (x);                                                                              \
        if (e_ != cudaSuccess) {                                                                           \
            throw ::kf::KfError(e_ == cudaErrorMemoryAllocation ? KF_ERR_OUT_OF_MEMORY : KF_ERR_CUDA,      \
                                std::string(#x) + ": " + cudaGetErrorString(e_));                          \
        }                                                                                                  \
    } while (0)

#define KF_REQUIRE(cond, code, msg)                                                                        \
    do {                                                                                                   \
        if (!(cond)) throw ::kf::KfError((code), (msg));                                                   \
    } while (0)

// Owning device array (cudaMalloc). Grows on demand, never shrinks.
template <class T> struct DeviceBuffer {
    T* ptr = nullptr;
    size_t count = 0;
    size_t cap = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr(o.ptr), count(o.count), cap(o.cap) {
        o.ptr = nullptr;
        o.count = o.cap = 0;
    }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
        if (this != &o) {
            release();
            ptr = o.ptr;
            count = o.count;
            cap = o.cap;
            o.ptr = nullptr;
            o.count = o.cap = 0;
        }
        return *this;
    }
    ~DeviceBuffer() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = cap = 0;
    }
    void resize(size_t n, cudaStream_t st) {
        if (n > cap) {
            if (ptr) {
                cudaStreamSynchronize(st);
                cudaFree(ptr);
                ptr = nullptr;
            }
            void* p = nullptr;
            KF_CUDA_CHECK(cudaMalloc(&p, sizeof(T) * (n ? n : 1)));
            ptr = static_cast<T*>(p);
            cap = n;
        }
        count = n;
    }
    void upload(const T* host, size_t n, cudaStream_t st) {
        resize(n, st);
        if (n) KF_CUDA_CHECK(cudaMemcpyAsync(ptr, host, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    }
    size_t bytes() const { return sizeof(T) * count; }
};

// Stream-ordered temporaries (cudaMallocAsync), freed on the same stream at scope exit.
struct TempAlloc {
    cudaStream_t st;
    std::vector<void*> ptrs;
    explicit TempAlloc(cudaStream_t s) : st(s) {}
    TempAlloc(const TempAlloc&) = delete;
    TempAlloc& operator=(const TempAlloc&) = delete;
    template <class T> T* alloc(size_t n) {
        void* p = nullptr;
        KF_CUDA_CHECK(cudaMallocAsync(&p, sizeof(T) * (n ? n : 1), st));
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~TempAlloc() {
        for (void* p : ptrs) cudaFreeAsync(p, st);
    }
};

} // namespace kf
