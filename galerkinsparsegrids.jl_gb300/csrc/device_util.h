// device_util.h -- device buffers with an HBM budget, error checks.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/sgdg.h"
#include "sgdg_core.h"

namespace sgdg {

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            throw ::sgdg::Error(e_ == cudaErrorMemoryAllocation ? SGDG_ENOMEM_BUDGET : SGDG_ECUDA,     \
                                std::string(#call) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

inline std::atomic<int64_t> g_budget{0};
inline std::atomic<int64_t> g_in_use{0};

inline void require_gpu() {
    static int state = -1;  // -1 unknown, 0 none, 1 ok
    if (state == 1) return;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        state = 0;
        throw Error(SGDG_ENOGPU,
                    std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
    }
    state = 1;
}

// Device allocation counted against the HBM budget (sgdg_set_hbm_budget).
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    explicit DevBuf(size_t n) { alloc(n); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
        o.p = nullptr;
        o.bytes = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        release();
        p = o.p;
        bytes = o.bytes;
        o.p = nullptr;
        o.bytes = 0;
        return *this;
    }
    void alloc(size_t n) {
        release();
        if (n == 0) n = 16;
        const int64_t b = g_budget.load();
        if (b > 0 && g_in_use.load() + (int64_t)n > b)
            throw Error(SGDG_ENOMEM_BUDGET, "HBM budget exceeded: requested " + std::to_string(n) + " bytes, " +
                                                std::to_string(g_in_use.load()) + " of " + std::to_string(b) +
                                                " in use");
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            throw Error(SGDG_ENOMEM_BUDGET, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        bytes = n;
        g_in_use += (int64_t)n;
    }
    void release() {
        if (p) {
            cudaFree(p);
            g_in_use -= (int64_t)bytes;
        }
        p = nullptr;
        bytes = 0;
    }
    ~DevBuf() { release(); }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

template <class T>
DevBuf upload(const std::vector<T>& v, cudaStream_t st) {
    DevBuf b(v.size() * sizeof(T));
    if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return b;
}

}  // namespace sgdg
