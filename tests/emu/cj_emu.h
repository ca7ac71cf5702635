// cj_emu.h -- a CPU emulation of the CUDA features the parse kernels use, so
// that cujson_gb300/csrc/cj_scan.cu and cj_pair.cu can be compiled with g++
// and run on a machine without a GPU.  TEST INFRASTRUCTURE ONLY.
//
// Every thread of a block is a fiber (ucontext); blocks run one after another.
// __syncthreads is a block barrier; warp collectives (__shfl*_sync,
// __ballot_sync, __any_sync, __all_sync, __reduce_*_sync, __match_any_sync,
// __syncwarp) are warp barriers at which every one of the 32 lanes must
// arrive with the same operation -- a collective reached by only some lanes,
// or by lanes doing different operations, stops the program with a message
// (the kernels use full-warp masks only).  __shared__ variables are statics
// (one block at a time), dynamic shared memory is a per-launch buffer.
// Atomics are plain read-modify-writes: fibers switch only at barriers.
#pragma once

#include <ucontext.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <type_traits>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__
#define __shared__ static
#define __launch_bounds__(...)
#define __align__(n) __attribute__((aligned(n)))

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct uint2 { uint32_t x, y; };
struct uint4 { uint32_t x, y, z, w; };
struct int4 { int32_t x, y, z, w; };
inline uint2 make_uint2(uint32_t x, uint32_t y) { return {x, y}; }
inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return {x, y, z, w}; }
inline int4 make_int4(int32_t x, int32_t y, int32_t z, int32_t w) { return {x, y, z, w}; }

typedef int cudaError_t;
typedef void* cudaStream_t;
typedef void* cudaEvent_t;
inline int cudaEventRecord(cudaEvent_t, cudaStream_t = nullptr) { return 0; }
enum { cudaSuccess = 0 };

namespace cj_emu {

enum Op { kNone, kShfl, kShflUp, kShflDown, kShflXor, kBallot, kAny, kAll, kRedAdd, kRedOr, kMatch, kSyncWarp,
          kRedMinS, kRedMaxS, kRedMinU, kRedMaxU };

struct Fiber {
    ucontext_t ctx;
    bool done = false;
    int wait = 0;            // 1: block barrier, 2: warp collective
};

struct Warp {
    int arrived = 0;
    int op = kNone;
    uint64_t in[32], aux[32], out[32];
};

inline ucontext_t g_sched;
inline std::vector<Fiber> g_fibers;
inline std::vector<Warp> g_warps;
inline std::vector<std::vector<char>> g_stacks;
inline int g_cur = 0;
inline unsigned g_nt = 0;
inline dim3 g_tid, g_bid, g_bdim, g_gdim;
inline std::function<void()>* g_body = nullptr;
inline std::vector<uint8_t> g_dyn_smem;
constexpr size_t kStack = 128 * 1024;

[[noreturn]] inline void fail(const char* what)
{
    fprintf(stderr, "cj_emu: %s (block %u, thread %d)\n", what, g_bid.x, g_cur);
    abort();
}

inline void fiber_entry()
{
    (*g_body)();
    g_fibers[g_cur].done = true;
    swapcontext(&g_fibers[g_cur].ctx, &g_sched);
}

inline void yield() { swapcontext(&g_fibers[g_cur].ctx, &g_sched); }

inline void syncthreads()
{
    g_fibers[g_cur].wait = 1;
    yield();
}

inline uint64_t collective(int op, uint64_t v, uint64_t aux)
{
    const int lane = g_cur & 31;
    Warp& w = g_warps[g_cur >> 5];
    if (w.arrived == 0) w.op = op;
    else if (w.op != op) fail("lanes of a warp in different collectives");
    w.in[lane] = v;
    w.aux[lane] = aux;
    if (++w.arrived < 32) {
        g_fibers[g_cur].wait = 2;
        yield();
        return w.out[lane];
    }
    // the last lane to arrive computes every lane's result and releases the others
    for (int l = 0; l < 32; l++) {
        uint64_t r = 0;
        switch (op) {
        case kShfl: r = w.in[w.aux[l] & 31]; break;
        case kShflUp: r = (uint64_t)l >= w.aux[l] ? w.in[l - w.aux[l]] : w.in[l]; break;
        case kShflDown: r = l + w.aux[l] < 32 ? w.in[l + w.aux[l]] : w.in[l]; break;
        case kShflXor: r = w.in[(l ^ w.aux[l]) & 31]; break;
        case kBallot: case kAny: case kAll:
            for (int k = 0; k < 32; k++) r |= (uint64_t)(w.in[k] != 0) << k;
            if (op == kAny) r = r != 0;
            if (op == kAll) r = r == 0xFFFFFFFFull;
            break;
        case kRedAdd: for (int k = 0; k < 32; k++) r = (uint32_t)(r + w.in[k]); break;
        case kRedOr: for (int k = 0; k < 32; k++) r |= w.in[k]; break;
        case kMatch: for (int k = 0; k < 32; k++) r |= (uint64_t)(w.in[k] == w.in[l]) << k; break;
        case kRedMinS: case kRedMaxS: {
            int32_t m = (int32_t)w.in[0];
            for (int k = 1; k < 32; k++) {
                const int32_t x = (int32_t)w.in[k];
                m = (op == kRedMinS) ? (x < m ? x : m) : (x > m ? x : m);
            }
            r = (uint32_t)m;
            break;
        }
        case kRedMinU: case kRedMaxU: {
            uint32_t m = (uint32_t)w.in[0];
            for (int k = 1; k < 32; k++) {
                const uint32_t x = (uint32_t)w.in[k];
                m = (op == kRedMinU) ? (x < m ? x : m) : (x > m ? x : m);
            }
            r = m;
            break;
        }
        default: break;
        }
        w.out[l] = r;
    }
    w.arrived = 0;
    const int base = g_cur & ~31;
    for (int l = 0; l < 32; l++)
        if (base + l != g_cur) g_fibers[base + l].wait = 0;
    return w.out[lane];
}

// Runs `body` for every thread of every block of `grid`.
inline void launch(dim3 grid, dim3 block, size_t dyn_smem, const std::function<void()>& body)
{
    std::function<void()> b = body;
    g_body = &b;
    g_gdim = grid;
    g_bdim = block;
    g_nt = block.x * block.y * block.z;
    if (g_nt % 32) fail("block size not a multiple of 32");
    g_fibers.assign(g_nt, Fiber());
    g_warps.assign(g_nt / 32, Warp());
    if (g_stacks.size() < g_nt) g_stacks.resize(g_nt);
    for (auto& s : g_stacks) if (s.size() != kStack) s.resize(kStack);
    g_dyn_smem.assign(dyn_smem + 16, 0);
    for (unsigned bx = 0; bx < grid.x; bx++) {
        g_bid = dim3(bx, 0, 0);
        for (unsigned t = 0; t < g_nt; t++) {
            Fiber& f = g_fibers[t];
            f.done = false;
            f.wait = 0;
            getcontext(&f.ctx);
            f.ctx.uc_stack.ss_sp = g_stacks[t].data();
            f.ctx.uc_stack.ss_size = kStack;
            f.ctx.uc_link = nullptr;
            makecontext(&f.ctx, (void (*)())fiber_entry, 0);
        }
        for (auto& w : g_warps) w.arrived = 0;
        while (true) {
            bool ran = false;
            for (unsigned t = 0; t < g_nt; t++) {
                Fiber& f = g_fibers[t];
                if (f.done || f.wait) continue;
                g_cur = (int)t;
                g_tid = dim3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
                swapcontext(&g_sched, &f.ctx);
                ran = true;
            }
            if (ran) continue;
            bool all_done = true, any_coll = false, any_bar = false;
            for (unsigned t = 0; t < g_nt; t++) {
                all_done &= g_fibers[t].done;
                any_coll |= g_fibers[t].wait == 2;
                any_bar |= g_fibers[t].wait == 1;
            }
            if (all_done) break;
            if (any_coll) { g_cur = -1; fail("a warp collective that not every lane reached"); }
            if (any_bar) {
                for (unsigned t = 0; t < g_nt; t++) if (g_fibers[t].wait == 1) g_fibers[t].wait = 0;
            }
        }
    }
}

template <class T> inline uint64_t to_u64(T v) { uint64_t r = 0; memcpy(&r, &v, sizeof(T)); return r; }
template <class T> inline T from_u64(uint64_t v) { T r; memcpy(&r, &v, sizeof(T)); return r; }

}  // namespace cj_emu

#define threadIdx (cj_emu::g_tid)
#define blockIdx (cj_emu::g_bid)
#define blockDim (cj_emu::g_bdim)
#define gridDim (cj_emu::g_gdim)
inline void __syncthreads() { cj_emu::syncthreads(); }
inline void __syncwarp(unsigned = 0xFFFFFFFFu) { cj_emu::collective(cj_emu::kSyncWarp, 0, 0); }

template <class T> inline T __shfl_sync(unsigned, T v, int src, int = 32)
{ return cj_emu::from_u64<T>(cj_emu::collective(cj_emu::kShfl, cj_emu::to_u64(v), (uint64_t)src)); }
template <class T> inline T __shfl_up_sync(unsigned, T v, unsigned d, int = 32)
{ return cj_emu::from_u64<T>(cj_emu::collective(cj_emu::kShflUp, cj_emu::to_u64(v), d)); }
template <class T> inline T __shfl_down_sync(unsigned, T v, unsigned d, int = 32)
{ return cj_emu::from_u64<T>(cj_emu::collective(cj_emu::kShflDown, cj_emu::to_u64(v), d)); }
template <class T> inline T __shfl_xor_sync(unsigned, T v, int m, int = 32)
{ return cj_emu::from_u64<T>(cj_emu::collective(cj_emu::kShflXor, cj_emu::to_u64(v), (uint64_t)m)); }
inline unsigned __ballot_sync(unsigned, int p) { return (unsigned)cj_emu::collective(cj_emu::kBallot, p != 0, 0); }
inline int __any_sync(unsigned, int p) { return (int)cj_emu::collective(cj_emu::kAny, p != 0, 0); }
inline int __all_sync(unsigned, int p) { return (int)cj_emu::collective(cj_emu::kAll, p != 0, 0); }
inline unsigned __vcmpltu4(unsigned a, unsigned b)
{
    unsigned r = 0;
    for (int i = 0; i < 4; i++)
        if (((a >> (8 * i)) & 0xFFu) < ((b >> (8 * i)) & 0xFFu)) r |= 0xFFu << (8 * i);
    return r;
}
inline unsigned __vcmpeq4(unsigned a, unsigned b)
{
    unsigned r = 0;
    for (int i = 0; i < 4; i++)
        if (((a >> (8 * i)) & 0xFFu) == ((b >> (8 * i)) & 0xFFu)) r |= 0xFFu << (8 * i);
    return r;
}
inline unsigned __reduce_add_sync(unsigned, unsigned v) { return (unsigned)cj_emu::collective(cj_emu::kRedAdd, v, 0); }
inline unsigned __reduce_or_sync(unsigned, unsigned v) { return (unsigned)cj_emu::collective(cj_emu::kRedOr, v, 0); }
inline unsigned __match_any_sync(unsigned, unsigned v) { return (unsigned)cj_emu::collective(cj_emu::kMatch, v, 0); }
inline int __reduce_min_sync(unsigned, int v) { return (int)(uint32_t)cj_emu::collective(cj_emu::kRedMinS, (uint32_t)v, 0); }
inline int __reduce_max_sync(unsigned, int v) { return (int)(uint32_t)cj_emu::collective(cj_emu::kRedMaxS, (uint32_t)v, 0); }
inline unsigned __reduce_min_sync(unsigned, unsigned v) { return (unsigned)cj_emu::collective(cj_emu::kRedMinU, v, 0); }
inline unsigned __reduce_max_sync(unsigned, unsigned v) { return (unsigned)cj_emu::collective(cj_emu::kRedMaxU, v, 0); }

inline int __popc(uint32_t x) { return __builtin_popcount(x); }
inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((uint32_t)x); }
inline int __ffs(int x) { return x == 0 ? 0 : __builtin_ctz((uint32_t)x) + 1; }
inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned sh)
{
    return (unsigned)((((unsigned long long)hi << 32) | lo) >> (sh & 31u));
}
inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
inline int __ffsll(long long x) { return x == 0 ? 0 : __builtin_ctzll((unsigned long long)x) + 1; }
inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll((unsigned long long)x); }
inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) {
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
inline long long __double_as_longlong(double d) { long long r; std::memcpy(&r, &d, sizeof r); return r; }
inline void __nanosleep(unsigned) {}
inline void __threadfence() {}
inline void __threadfence_system() {}
template <class T> inline T __ldg(const T* p) { return *p; }
template <class T> inline T __ldcg(const T* p) { return *p; }
template <class T> inline T __ldcs(const T* p) { return *p; }
template <class T> inline void __stcg(T* p, T v) { *p = v; }

template <class T> inline T atomicAdd(T* p, T v) { T o = *p; *p = o + v; return o; }
template <class T> inline T atomicOr(T* p, T v) { T o = *p; *p = o | v; return o; }
template <class T> inline T atomicAnd(T* p, T v) { T o = *p; *p = o & v; return o; }
template <class T> inline T atomicMax(T* p, T v) { T o = *p; if (v > o) *p = v; return o; }
template <class T> inline T atomicMin(T* p, T v) { T o = *p; if (v < o) *p = v; return o; }
template <class T> inline T atomicCAS(T* p, T c, T v) { T o = *p; if (o == c) *p = v; return o; }

template <class A, class B> inline typename std::common_type<A, B>::type min(A a, B b) { return a < b ? a : b; }
template <class A, class B> inline typename std::common_type<A, B>::type max(A a, B b) { return a > b ? a : b; }
