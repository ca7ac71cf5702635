// cj_noalloc.cu -- cj_parse_standard_noalloc: the standard-document parse for
// callers that must not allocate memory.
//
// Every other entry point takes its device memory from a context arena that
// grows with cudaMalloc.  Some callers cannot allow that: a service that owns
// the device's memory and hands out fixed budgets, or a latency-critical
// loop where the device-wide synchronisation of cudaMalloc/cudaFree would
// stall unrelated streams.  This entry point allocates nothing, on the device
// or the host.  Its scratch is one file-scope __device__ array sized for
// documents of up to CJ_NOALLOC_MAX_BYTES; the input and the output are the
// caller's own device buffers.  It runs the same kernels as the arena path
// (the scan's tables, prefix and emit kernels, then pair and spine) plus one
// that writes the reference layout.
//
// The scratch is shared by every call on a device, so calls on one device
// must not overlap: two calls in flight at once (from two host threads, or on
// two streams without ordering between them) race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

using namespace cj;

namespace {

constexpr size_t up(size_t x, size_t m) { return (x + m - 1) / m * m; }

constexpr size_t kMax = CJ_NOALLOC_MAX_BYTES;
constexpr size_t kInBytes = up(kMax, kPadBytes) + kPadBytes;
constexpr int kRegionSteps = kRegionStepsDefault;
constexpr size_t kRegions = kMax / ((size_t)kRegionSteps * kStepBytes) + 2;
constexpr size_t kPrefixBlocks = (kRegions + kPrefixPerBlock - 1) / kPrefixPerBlock;
constexpr size_t kScap = kMax + 1;                        // S <= bytes
constexpr size_t kChunks = (kMax + kChunk - 1) / kChunk + 1;

constexpr size_t tree_level(size_t n, int l) { return l == 0 ? n : tree_level((n + 31) / 32, l - 1); }
constexpr size_t tree_total(size_t n, int l) { return l > kTreeLevels ? 0 : tree_level(n, l) + tree_total(n, l + 1); }
constexpr size_t kTree = tree_total(kChunks, 1);

// Scratch layout; every member starts on a 256-byte boundary.
struct alignas(256) Scratch {
    alignas(256) uint8_t in[kInBytes];
    alignas(256) int32_t pos[kScap];
    alignas(256) int32_t pair[kScap];
    alignas(256) uint2 brk[kScap];
    alignas(256) uint4 rtab[kRegions * 4];
    alignas(256) uint4 bagg[kPrefixBlocks * 4];
    alignas(256) uint4 work[kRegions * 2];
    alignas(256) uint4 masks[kRegions * kRegionSteps * 32];
    alignas(256) uint32_t spine[kChunks * kChunk];
    alignas(256) int4 cinfo[kChunks];
    alignas(256) unsigned long long tree[kTree];
    alignas(256) Segment seg;
    alignas(256) SegmentOut seg_out;
    alignas(256) Ctrl ctrl;
};

// The scratch itself (about 22 MiB for the 1 MiB limit).  Zero at load; the
// pairing min-tree is epoch-tagged, and is cleared again when the epoch wraps
// and on the first call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(Scratch)];

struct DeviceState {
    bool ready = false;
    Scratch* scratch = nullptr;
    int sm_count = 0;
    uint32_t epoch = 0;
};

constexpr int kMaxDevices = 64;
std::mutex g_mu;
DeviceState g_dev[kMaxDevices];

// Writes the one segment of the document and clears the run counters.
__global__ void noalloc_setup(Scratch* s, uint64_t n)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Segment seg;
    seg.dev_off = 0;
    seg.len = n;
    seg.logical_off = 0;
    seg.out_base = 0;
    seg.brk_base = 0;
    seg.first_region = 0;
    seg.n_regions = (uint32_t)((n + (uint64_t)kRegionSteps * kStepBytes - 1) / ((uint64_t)kRegionSteps * kStepBytes));
    seg.flags = 0;
    seg.pad = 0;
    s->seg = seg;
    s->seg_out = SegmentOut{};
    s->ctrl = Ctrl{};
}

// Reference layout into the caller's buffer: [0]=0, [1..S] positions,
// [S+1]=S+1, [S+2..2S+1] pair row, [2S+2], [2S+3] = 0.  Writes nothing when
// 2S+4 entries do not fit, or when the document is invalid (any error flag,
// or a close below depth 0; the pairing kernels before it have set them all).
__global__ void noalloc_layout(const Scratch* s, int32_t* out, uint64_t cap)
{
    const uint64_t S = s->ctrl.s_total;
    if (S > kScap - 1 || 2 * S + 4 > cap) return;
    if (s->ctrl.error_flags != 0u || s->ctrl.neg_min_level > 0) return;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < S + 2; i += stride) {
        int32_t p, q;
        if (i == 0) {
            p = 0;
            q = (int32_t)(S + 1);      // out[S+1]
        } else if (i <= S) {
            p = s->pos[i - 1];
            q = s->pair[i - 1];        // out[S+1+i]
        } else {
            p = 0;                     // out[2S+2] and out[2S+3]
            q = 0;
        }
        if (i <= S) {
            out[i] = p;
            out[S + 1 + i] = q;
        } else {
            out[2 * S + 2] = p;
            out[2 * S + 3] = q;
        }
    }
}

cj_status cuda_status(cudaError_t e)
{
    return e == cudaSuccess ? CJ_OK : CJ_ERR_CUDA;
}

// One-time setup for the current device: resolve the scratch address and
// clear the epoch-tagged min-tree.
cj_status device_setup(int dev, cudaStream_t stream, DeviceState& d)
{
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) return CJ_ERR_CUDA;
    if (cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return CJ_ERR_CUDA;
    Scratch* s = static_cast<Scratch*>(ptr);
    // cleared and finished before the call goes on, so no later call, on any
    // stream, can run beside this clear
    if (cudaMemsetAsync(s->tree, 0, sizeof(s->tree), stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
        return CJ_ERR_CUDA;
    d.scratch = s;
    d.epoch = 0;
    d.ready = true;
    return CJ_OK;
}

cj_status parse_noalloc(const uint8_t* d_data, size_t size, int32_t* d_out, size_t out_cap,
                        cj_parse_info* info, void* stream_handle)
{
    if (info) *info = cj_parse_info{};
    if (!d_data || !d_out || size == 0) return CJ_ERR_INVALID_ARGUMENT;
    if (size > CJ_NOALLOC_MAX_BYTES) return CJ_ERR_TOO_LARGE;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_handle);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CJ_ERR_NO_DEVICE;
    if (dev < 0 || dev >= kMaxDevices) return CJ_ERR_INVALID_ARGUMENT;

    DeviceState* d;
    uint32_t epoch;
    {
        std::lock_guard<std::mutex> g(g_mu);
        d = &g_dev[dev];
        if (!d->ready) {
            cj_status st = device_setup(dev, stream, *d);
            if (st) return st;
        }
        d->epoch = (d->epoch + 1) & 0x3FFFFFFFu;
        if (d->epoch == 0) {
            Scratch* s = d->scratch;
            if (cudaMemsetAsync(s->tree, 0, sizeof(s->tree), stream) != cudaSuccess ||
                cudaStreamSynchronize(stream) != cudaSuccess)
                return CJ_ERR_CUDA;
            d->epoch = 1;
        }
        epoch = d->epoch;
    }
    Scratch* s = d->scratch;
    const uint32_t n_regions = (uint32_t)((size + (uint64_t)kRegionSteps * kStepBytes - 1) /
                                          ((uint64_t)kRegionSteps * kStepBytes));

    cj_status st;
    if ((st = cuda_status(cudaMemcpyAsync(s->in, d_data, size, cudaMemcpyDeviceToDevice, stream)))) return st;
    noalloc_setup<<<1, 32, 0, stream>>>(s, size);

    ScanParams sp{};
    sp.dependent_launch = 1;
    sp.in = s->in;
    sp.segs = &s->seg;
    sp.region_seg = nullptr;
    sp.n_segs = 1;
    sp.n_regions = n_regions;
    sp.pos = s->pos;
    sp.pair = s->pair;
    sp.brk = s->brk;
    sp.out_cap = kScap;
    sp.brk_cap = kScap;
    sp.rtab = s->rtab;
    sp.bagg = s->bagg;
    sp.masks = s->masks;
    sp.work = s->work;
    sp.ctrl = &s->ctrl;
    sp.seg_out = &s->seg_out;
    sp.region_steps = kRegionSteps;
    sp.sm_count = d->sm_count;
    launch_scan(sp, false, ScanShape{0, 0}, stream);

    PairParams pp{};
    pp.dependent_launch = 1;
    pp.brk = s->brk;
    pp.pair = s->pair;
    pp.spine = s->spine;
    pp.cinfo = s->cinfo;
    pp.tree = s->tree;
    {
        size_t off = 0, n = kChunks;
        pp.tree_off[0] = 0;
        for (int l = 1; l <= kTreeLevels; l++) {
            n = (n + 31) / 32;
            pp.tree_off[l] = off;
            off += n;
        }
    }
    pp.ctrl = &s->ctrl;
    pp.epoch = epoch;
    pp.chunk_cap = (uint32_t)kChunks;
    const size_t max_chunks = (size + kChunk - 1) / kChunk;
    const int grid = (int)std::min<size_t>((max_chunks + 7) / 8 + 1, (size_t)d->sm_count * 8);
    launch_pair(pp, grid, stream);
    launch_spine(pp, grid, stream);

    const int lgrid = (int)std::min<size_t>((size + 2 + 255) / 256, (size_t)d->sm_count * 4);
    noalloc_layout<<<lgrid, 256, 0, stream>>>(s, d_out, out_cap);
    if ((st = cuda_status(cudaGetLastError()))) return st;

    Ctrl c;
    if ((st = cuda_status(cudaMemcpyAsync(&c, &s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream)))) return st;
    if ((st = cuda_status(cudaStreamSynchronize(stream)))) return st;

    uint32_t flags = c.error_flags;
    if (c.neg_min_level > 0) flags |= CJ_FLAG_BRACKETS;
    cj_status verdict = CJ_OK;
    if (flags & CJ_FLAG_TIMEOUT) verdict = CJ_ERR_TIMEOUT;
    else if (flags & CJ_FLAG_OVERFLOW) verdict = CJ_ERR_CUDA;     // inconsistent scan counts (a defect)
    else if (flags & CJ_FLAG_UTF8) verdict = CJ_ERR_INVALID_UTF8;
    else if (flags & CJ_FLAG_BRACKETS) verdict = CJ_ERR_INVALID_BRACKETS;
    if (info) {
        info->n_structural = c.s_total;
        info->n_brackets = c.k_total;
        info->max_depth = c.max_depth;
        info->status = verdict;
        info->error_flags = flags;
        info->n_segments = 1;
    }
    if (verdict != CJ_OK) return verdict;
    if ((uint64_t)(2 * c.s_total + 4) > out_cap) return CJ_ERR_CAPACITY;
    return CJ_OK;
}

}  // namespace

extern "C" cj_status cj_parse_standard_noalloc(const uint8_t* d_data, size_t size, int32_t* d_out,
                                               size_t out_cap, cj_parse_info* info, void* stream)
{
    const cj_status st = parse_noalloc(d_data, size, d_out, out_cap, info, stream);
    cj_set_last_status(st);
    return st;
}
