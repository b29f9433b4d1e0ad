// util.cuh -- error reporting and small RAII helpers for the host side.
#pragma once
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "../../include/ocl_gb300.h"

namespace oclg {

void set_error(const std::string& msg);

// Key of the calling thread's current CUDA context: the driver's context id
// (unique for the life of the process, so a context created after a device
// reset gets a new key), or device ordinal + 1 where the driver does not
// report ids.  Caches of device state (workspaces, function attributes,
// symbol addresses) are keyed by it.  Returns 0 and sets the error on failure.
uint64_t context_key();

// Evaluate a CUDA call; on failure record the message and return DEVICE_ERROR
// (or OOM for allocation failures) from the enclosing function.
#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t err__ = (call);                                                      \
        if (err__ != cudaSuccess) {                                                      \
            ::oclg::set_error(std::string(#call) + ": " + cudaGetErrorString(err__));    \
            return err__ == cudaErrorMemoryAllocation ? OCL_GB300_OOM : OCL_GB300_DEVICE_ERROR; \
        }                                                                                \
    } while (0)

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    bool alloc(size_t count) {
        release();
        n = count;
        if (count == 0) return true;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
            p = nullptr;
            set_error("cudaMalloc failed");
            return false;
        }
        return true;
    }
    // Grow-only: keeps the buffer (and its contents) when it already holds
    // `count` elements; reallocating frees, and a free synchronises the device.
    bool reserve(size_t count) {
        if (count <= n && (p || count == 0)) return true;
        return alloc(count);
    }
    bool ok() const { return n == 0 || p != nullptr; }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
};

}  // namespace oclg
