// cj_cuda_emu.h -- host emulation of the CUDA features the reference's parse
// path uses, so that its own sources (cujson/parse_standard_json.cu,
// cujson/parse_json_lines.cu, cujson/utils.cu) compile with g++ and run on the
// CPU.  TEST INFRASTRUCTURE ONLY: it produces golden outputs of the reference
// itself for the parity tests; nothing in the product uses it.
//
//   - kernels are plain functions; a launch runs every thread of a block as a
//     fiber (ucontext) on the calling thread, one block after another, and
//     __syncthreads switches to the next fiber until all of the block's
//     fibers reached it;  __shared__ variables are function statics (one block
//     runs at a time, and the kernels initialise them before use);
//   - atomics are plain read-modify-writes (fibers never interleave inside one);
//   - the SIMD video intrinsics follow their documented per-byte / per-halfword
//     definitions; shifts by >= 32 never reach them;
//   - device memory is host memory: cudaMalloc returns zeroed memory, copies
//     are memcpy, streams and events are no-ops;
//   - exit() inside the parse (invalid input) throws cj_ref_exit instead.
#pragma once

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ucontext.h>

#include <functional>
#include <set>
#include <stdexcept>
#include <vector>

// ---- qualifiers -----------------------------------------------------------------
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static
#define __launch_bounds__(...)

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

struct cj_ref_exit {
    int code;
};

namespace cj_emu {

inline dim3 g_threadIdx, g_blockIdx, g_blockDim, g_gridDim;

struct Fiber {
    ucontext_t ctx;
    bool done = false;
    bool at_barrier = false;
};

inline ucontext_t g_sched;
inline Fiber* g_cur = nullptr;
inline std::function<void()>* g_body = nullptr;
constexpr size_t kStack = 256 * 1024;

inline void fiber_entry()
{
    (*g_body)();
    g_cur->done = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

inline void syncthreads()
{
    g_cur->at_barrier = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

inline void launch(dim3 grid, dim3 block, const std::function<void()>& f)
{
    static std::vector<Fiber> fibers;
    static std::vector<std::vector<char>> stacks;
    std::function<void()> body = f;
    g_body = &body;
    g_gridDim = grid;
    g_blockDim = block;
    const unsigned nt = block.x * block.y * block.z;
    if (fibers.size() < nt) {
        fibers.resize(nt);
        stacks.resize(nt);
        for (auto& s : stacks)
            if (s.size() != kStack) s.resize(kStack);
    }
    for (unsigned bz = 0; bz < grid.z; bz++)
        for (unsigned by = 0; by < grid.y; by++)
            for (unsigned bx = 0; bx < grid.x; bx++) {
                g_blockIdx = dim3(bx, by, bz);
                for (unsigned t = 0; t < nt; t++) {
                    Fiber& fb = fibers[t];
                    fb.done = false;
                    fb.at_barrier = false;
                    getcontext(&fb.ctx);
                    fb.ctx.uc_stack.ss_sp = stacks[t].data();
                    fb.ctx.uc_stack.ss_size = kStack;
                    fb.ctx.uc_link = nullptr;
                    makecontext(&fb.ctx, (void (*)())fiber_entry, 0);
                }
                while (true) {
                    bool running = false;
                    for (unsigned t = 0; t < nt; t++) {
                        Fiber& fb = fibers[t];
                        if (fb.done || fb.at_barrier) continue;
                        g_threadIdx = dim3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
                        g_cur = &fb;
                        swapcontext(&g_sched, &fb.ctx);
                        running = true;
                    }
                    bool all_done = true;
                    for (unsigned t = 0; t < nt; t++) all_done &= fibers[t].done;
                    if (all_done) break;
                    if (!running || true) {
                        // every live fiber waits at the barrier: release it
                        for (unsigned t = 0; t < nt; t++) fibers[t].at_barrier = false;
                    }
                }
            }
}

inline uint32_t bytewise(uint32_t a, uint32_t b, int (*f)(uint32_t, uint32_t))
{
    uint32_t r = 0;
    for (int i = 0; i < 4; i++) {
        const uint32_t x = (a >> (8 * i)) & 0xFF, y = (b >> (8 * i)) & 0xFF;
        r |= ((uint32_t)f(x, y) & 0xFFu) << (8 * i);
    }
    return r;
}

}  // namespace cj_emu

#define threadIdx (cj_emu::g_threadIdx)
#define blockIdx (cj_emu::g_blockIdx)
#define blockDim (cj_emu::g_blockDim)
#define gridDim (cj_emu::g_gridDim)
#define __syncthreads() cj_emu::syncthreads()

// ---- integer intrinsics (documented semantics) -----------------------------------
inline int __popc(uint32_t x) { return __builtin_popcount(x); }
inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((uint32_t)x); }
inline int __ffs(int x) { return x == 0 ? 0 : __builtin_ctz((uint32_t)x) + 1; }

// per byte: 0xFF where the relation holds, else 0x00
inline unsigned int __vcmpeq4(unsigned int a, unsigned int b)
{
    return cj_emu::bytewise(a, b, [](uint32_t x, uint32_t y) { return x == y ? 0xFF : 0; });
}
inline unsigned int __vcmpgtu4(unsigned int a, unsigned int b)
{
    return cj_emu::bytewise(a, b, [](uint32_t x, uint32_t y) { return x > y ? 0xFF : 0; });
}
inline unsigned int __vcmpltu4(unsigned int a, unsigned int b)
{
    return cj_emu::bytewise(a, b, [](uint32_t x, uint32_t y) { return x < y ? 0xFF : 0; });
}
inline unsigned int __vcmpgeu4(unsigned int a, unsigned int b)
{
    return cj_emu::bytewise(a, b, [](uint32_t x, uint32_t y) { return x >= y ? 0xFF : 0; });
}
// per byte, unsigned saturated a - b
inline unsigned int __vsubus4(unsigned int a, unsigned int b)
{
    return cj_emu::bytewise(a, b, [](uint32_t x, uint32_t y) { return x > y ? (int)(x - y) : 0; });
}
// per byte, signed saturated a - b
inline unsigned int __vsubss4(unsigned int a, unsigned int b)
{
    return cj_emu::bytewise(a, b, [](uint32_t x, uint32_t y) {
        int d = (int)(int8_t)x - (int)(int8_t)y;
        d = d < -128 ? -128 : (d > 127 ? 127 : d);
        return d & 0xFF;
    });
}
// per halfword: 0xFFFF where equal
inline unsigned int __vcmpeq2(unsigned int a, unsigned int b)
{
    unsigned int r = 0;
    if ((a & 0xFFFFu) == (b & 0xFFFFu)) r |= 0xFFFFu;
    if ((a >> 16) == (b >> 16)) r |= 0xFFFF0000u;
    return r;
}

namespace cj_emu {
template <typename T> struct same { using type = T; };
}
// the value converts to the pointee type, as with CUDA's typed overloads
template <typename T>
inline T atomicOr(T* p, typename cj_emu::same<T>::type v) { T o = *p; *p = o | v; return o; }
template <typename T>
inline T atomicAnd(T* p, typename cj_emu::same<T>::type v) { T o = *p; *p = o & v; return o; }
template <typename T>
inline T atomicAdd(T* p, typename cj_emu::same<T>::type v) { T o = *p; *p = o + v; return o; }
template <typename T>
inline T atomicExch(T* p, typename cj_emu::same<T>::type v) { T o = *p; *p = v; return o; }
template <typename T>
inline T atomicMax(T* p, typename cj_emu::same<T>::type v) { T o = *p; if (v > o) *p = v; return o; }
template <typename T>
inline T atomicMin(T* p, typename cj_emu::same<T>::type v) { T o = *p; if (v < o) *p = v; return o; }
