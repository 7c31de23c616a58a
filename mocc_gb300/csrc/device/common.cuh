// Shared device helpers.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../host/geom.hpp"

namespace mocgpu {

#define MOCGPU_CUDA(call)                                                                                        \
    do {                                                                                                         \
        cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess)                                                                                   \
            throw ::mocgpu::Error(20, std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " + __FILE__ + \
                                          ":" + std::to_string(__LINE__));                                       \
    } while (0)

// Status flags a kernel may raise (OR-ed into a device word, read by the host).
enum DeviceStatus : unsigned {
    DEV_OK = 0,
    DEV_NONPOSITIVE_PIN_FLUX = 1u << 0,
    DEV_NAN = 1u << 1,
    DEV_BAD_INDEX = 1u << 2,
    DEV_CMFD_NOT_CONVERGED = 1u << 3,
    DEV_NEGATIVE_SPLIT_FLUX = 1u << 4, // transverse-leakage splitting met a negative scalar flux
};

// Host<->device bytes moved by the library (reported by the C ABI).
void note_copy_bytes(cudaMemcpyKind kind, size_t bytes);
inline cudaError_t copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s)
{
    note_copy_bytes(kind, bytes);
    return cudaMemcpyAsync(dst, src, bytes, kind, s);
}

// Test hook: after `after` more device allocations through DevBuf, the next
// one fails as if the device were out of memory (negative: never). Lets the
// host's failure paths be tested without exhausting a GPU.
void set_alloc_fault(int64_t after);
bool alloc_fault_due();

template <typename T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count)
    {
        release();
        if (count && alloc_fault_due())
            throw ::mocgpu::Error(20, "CUDA error: out of memory (injected allocation failure)");
        n = count;
        if (count) MOCGPU_CUDA(cudaMalloc(&p, count * sizeof(T)));
    }
    void upload(const T *h, size_t count)
    {
        alloc(count);
        if (count) {
            note_copy_bytes(cudaMemcpyHostToDevice, count * sizeof(T));
            MOCGPU_CUDA(cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice));
        }
    }
    template <typename V> void upload(const V &v) { upload(v.data(), v.size()); }
    // Copies into the existing allocation when the size matches (no allocation).
    template <typename V> void assign(const V &v)
    {
        if (v.size() != n) {
            upload(v);
            return;
        }
        if (n) {
            note_copy_bytes(cudaMemcpyHostToDevice, n * sizeof(T));
            MOCGPU_CUDA(cudaMemcpy(p, v.data(), n * sizeof(T), cudaMemcpyHostToDevice));
        }
    }
    void zero(cudaStream_t s = 0)
    {
        if (n) MOCGPU_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
    size_t bytes() const { return n * sizeof(T); }
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum; every thread gets the result. scratch needs 32 doubles.
__device__ __forceinline__ double block_sum(double v, double *scratch)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    double t = (threadIdx.x < (unsigned)nw) ? scratch[threadIdx.x] : 0.0;
    if (wid == 0) {
        t = warp_sum(t);
        if (lane == 0) scratch[0] = t;
    }
    __syncthreads();
    double r = scratch[0];
    __syncthreads();
    return r;
}

// Two block-wide sums at once; scratch needs 64 doubles.
__device__ __forceinline__ void block_sum2(double &a, double &b, double *scratch)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    __syncthreads();
    if (lane == 0) {
        scratch[wid] = a;
        scratch[32 + wid] = b;
    }
    __syncthreads();
    if (wid == 0) {
        double ta = (lane < nw) ? scratch[lane] : 0.0;
        double tb = (lane < nw) ? scratch[32 + lane] : 0.0;
        ta = warp_sum(ta);
        tb = warp_sum(tb);
        if (lane == 0) {
            scratch[0] = ta;
            scratch[32] = tb;
        }
    }
    __syncthreads();
    a = scratch[0];
    b = scratch[32];
    __syncthreads();
}

} // namespace mocgpu
