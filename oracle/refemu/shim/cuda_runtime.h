// cuda_runtime.h stand-in for the host emulation of the reference (see
// ../cj_cuda_emu.h): device memory is host memory, streams and events are
// no-ops.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../cj_cuda_emu.h"

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2 };
typedef void* cudaStream_t;
typedef void* cudaEvent_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                      cudaMemcpyDeviceToDevice, cudaMemcpyDefault };
#define cudaHostAllocDefault 0

namespace cj_emu {
inline std::set<void*>& device_allocs() { static std::set<void*> s; return s; }
inline std::set<void*>& host_allocs() { static std::set<void*> s; return s; }
inline cudaError_t dev_alloc(void** p, size_t n)
{
    *p = calloc(n ? n : 1, 1);
    if (!*p) return cudaErrorMemoryAllocation;
    device_allocs().insert(*p);
    return cudaSuccess;
}
inline cudaError_t dev_free(void* p)
{
    if (!p) return cudaSuccess;
    auto it = device_allocs().find(p);
    if (it == device_allocs().end()) return cudaErrorInvalidValue;   // not device memory: left alone
    device_allocs().erase(it);
    free(p);
    return cudaSuccess;
}
inline cudaError_t host_alloc(void** p, size_t n)
{
    *p = calloc(n ? n : 1, 1);
    if (!*p) return cudaErrorMemoryAllocation;
    host_allocs().insert(*p);
    return cudaSuccess;
}
inline cudaError_t host_free(void* p)
{
    if (!p) return cudaSuccess;
    auto it = host_allocs().find(p);
    if (it == host_allocs().end()) return cudaErrorInvalidValue;
    host_allocs().erase(it);
    free(p);
    return cudaSuccess;
}
}  // namespace cj_emu

template <typename T> inline cudaError_t cudaMalloc(T** p, size_t n) { return cj_emu::dev_alloc((void**)p, n); }
template <typename T> inline cudaError_t cudaMallocAsync(T** p, size_t n, cudaStream_t = 0) { return cj_emu::dev_alloc((void**)p, n); }
inline cudaError_t cudaFree(void* p) { return cj_emu::dev_free(p); }
inline cudaError_t cudaFreeAsync(void* p, cudaStream_t = 0) { return cj_emu::dev_free(p); }
template <typename T> inline cudaError_t cudaMallocHost(T** p, size_t n) { return cj_emu::host_alloc((void**)p, n); }
template <typename T> inline cudaError_t cudaHostAlloc(T** p, size_t n, unsigned = 0) { return cj_emu::host_alloc((void**)p, n); }
inline cudaError_t cudaFreeHost(void* p) { return cj_emu::host_free(p); }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { if (n) memmove(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t = 0) { if (n) memmove(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemset(void* d, int v, size_t n) { memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t = 0) { memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t) { return "emulated"; }
inline cudaError_t cudaEventCreate(cudaEvent_t* e) { *e = nullptr; return cudaSuccess; }
inline cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t = 0) { return cudaSuccess; }
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) { *ms = 0.f; return cudaSuccess; }
inline cudaError_t cudaMemGetInfo(size_t* f, size_t* t) { *f = (size_t)64 << 30; *t = (size_t)64 << 30; return cudaSuccess; }
inline cudaError_t cudaDeviceReset() { return cudaSuccess; }
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
