// cj_api.cu -- host orchestration and the C ABI (include/cujson_gb300.h).
//
// Replaces the reference's drivers parse_standard_json
// (cujson/parse_standard_json.cu:1584-1687) and parse_json_lines
// (cujson/parse_json_lines.cu:1092-1264).  Differences in shape, not in output:
//   - one device arena per context, grown to the largest input and reused, in
//     place of ~8 cudaMalloc/cudaFree per call;
//   - three kernel launches (scan, pair, spine) on a non-blocking stream, with
//     no host synchronisation until the verdict and counts are read;
//   - JSON-Lines chunks are parsed in the same launch (each chunk is a segment
//     whose string/escape state and depth restart), not one after another;
//   - errors are returned as a status; the process never exits.
#include <cuda.h>            // driver API types of the stream memory write entry point
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

using namespace cj;

bool cj::dependent_launch_enabled()
{
    static const bool on = [] {
        const char* e = getenv("CJ_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

namespace {

thread_local int g_last_status = CJ_OK;

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;   // elements
};

size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

// Pinned host blocks handed out by the library (result buffers, cj_host_alloc)
// are kept when freed and handed out again: pinning a large buffer costs far
// more than copying into it, and a caller that parses file after file frees
// and asks for buffers of about the same size each time.  A block is reused
// for a request of at least half its size; kept blocks beyond kPinnedKeep
// bytes are released, largest first.  Blocks the library did not hand out are
// released with cudaFreeHost.
constexpr size_t kPinnedKeep = 8ull << 30;
struct PinnedPool {
    std::mutex mu;
    std::unordered_map<void*, size_t> live;       // handed out: size
    std::multimap<size_t, void*> kept;            // freed, kept: size -> block
    size_t kept_bytes = 0;
};
PinnedPool& pinned_pool()
{
    static PinnedPool* p = new PinnedPool();      // never destroyed: blocks may be freed at exit
    return *p;
}
void* pinned_alloc(size_t bytes)
{
    PinnedPool& pp = pinned_pool();
    bytes = std::max<size_t>(bytes, 1);
    {
        std::lock_guard<std::mutex> g(pp.mu);
        auto it = pp.kept.lower_bound(bytes);
        if (it != pp.kept.end() && it->first / 2 <= bytes) {
            void* p = it->second;
            pp.live[p] = it->first;
            pp.kept_bytes -= it->first;
            pp.kept.erase(it);
            return p;
        }
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> g(pp.mu);
    pp.live[p] = bytes;
    return p;
}
void pinned_free(void* p)
{
    if (!p) return;
    PinnedPool& pp = pinned_pool();
    std::vector<void*> drop;
    {
        std::lock_guard<std::mutex> g(pp.mu);
        auto it = pp.live.find(p);
        if (it == pp.live.end()) {
            drop.push_back(p);
        } else {
            pp.kept.emplace(it->second, p);
            pp.kept_bytes += it->second;
            pp.live.erase(it);
            while (pp.kept_bytes > kPinnedKeep && !pp.kept.empty()) {
                auto last = std::prev(pp.kept.end());
                pp.kept_bytes -= last->first;
                drop.push_back(last->second);
                pp.kept.erase(last);
            }
        }
    }
    for (void* q : drop) cudaFreeHost(q);
}
size_t pinned_trim()
{
    PinnedPool& pp = pinned_pool();
    std::vector<void*> drop;
    size_t bytes = 0;
    {
        std::lock_guard<std::mutex> g(pp.mu);
        for (auto& kv : pp.kept) drop.push_back(kv.second);
        bytes = pp.kept_bytes;
        pp.kept.clear();
        pp.kept_bytes = 0;
    }
    for (void* q : drop) cudaFreeHost(q);
    return bytes;
}

// recorded run: start, after the scan's tables, prefix and emit kernels, after
// pair, after spine
constexpr size_t kEventsPerRun = 6;

}  // namespace

struct cj_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;

    DevBuf<uint8_t> in;
    DevBuf<int32_t> pos, pair;
    DevBuf<uint2> brk;
    DevBuf<uint4> rtab, bagg;           // region and prefix-block transfer tables
    DevBuf<uint4> work;                 // the emit kernel's work items (2 per region)
    DevBuf<uint4> masks;                // per region step: mask words for the emit kernel
    DevBuf<Segment> segs;
    DevBuf<SegmentOut> seg_out;
    DevBuf<uint32_t> region_seg;
    DevBuf<uint32_t> spine;
    DevBuf<int4> cinfo;
    DevBuf<unsigned long long> tree;
    Ctrl* d_ctrl = nullptr;
    uint64_t tree_off[kTreeLevels + 1] = {};
    size_t chunk_cap = 0;

    Ctrl* h_ctrl = nullptr;             // pinned mirrors
    std::vector<Segment> h_segs;
    std::vector<uint32_t> h_region_seg;
    SegmentOut* h_seg_out = nullptr;
    size_t h_seg_out_cap = 0;

    uint32_t epoch = 0;
    bool staged = false;
    bool lines = false;
    size_t n_bytes = 0;
    uint32_t n_segs = 0;
    uint32_t n_regions = 0;
    int run_region_steps = kRegionStepsDefault;   // region size of the staged layout
    int64_t launches = 0;
    size_t dev_bytes = 0;

    bool dependent_launch = true;       // the kernels after the first of a run are dependent launches
    int timing = 0;                     // 0 off, 1 an event at every kernel boundary, 2 scan and run ends,
                                        // 3 run ends only
    std::vector<cudaEvent_t> events;   // kEventsPerRun per recorded run
    size_t events_used = 0;

    // batches of independent documents
    bool batch = false;
    uint64_t batch_chunks = 0;          // pairing chunks of the batch layout
    DevBuf<uint32_t> seg_err;
    DevBuf<int32_t> seg_depth;
    DevBuf<uint64_t> rchunk_off;
    DevBuf<uint64_t> layout_off;
    DevBuf<int32_t> layout;
    DevBuf<uint8_t> pack;               // packed staging copy of a batch
    DevBuf<uint64_t> pack_off;          // per document: packed byte offset, then word offsets
    std::vector<uint64_t> h_pack_off;
    bool batch_read = false;            // host mirrors below are current
    std::vector<SegmentOut> h_bseg_out;
    std::vector<uint32_t> h_seg_err;
    std::vector<int32_t> h_seg_depth;
    std::vector<uint64_t> h_layout_off;

    // CUDA graph of the staged run, replayed by cj_run_staged_graph
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_valid = false;
    int64_t graph_launches = 0;         // kernels one replay launches
    uint64_t arena_gen = 0;             // bumped whenever a device buffer is (re)allocated

    // one-shot parses of large inputs: copies on copy_stream overlap the scan,
    // which scans a region only once d_ready covers its bytes
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_reset = nullptr, ev_copied = nullptr;
    cudaEvent_t ev_plan = nullptr;      // orders the device planner after the caller's stream
    unsigned long long* d_ready = nullptr;
    bool overlap_run = false;
    uint32_t input_wait_limit = 0;      // 0: the kernel's default
    // cuStreamWriteValue64 when the driver offers it (no kernel needs to run
    // beside the scan to raise d_ready); else a one-thread kernel does it
    CUresult (*write64)(CUstream, CUdeviceptr, cuuint64_t, unsigned int) = nullptr;

    // streamed one-shot parses into pinned host memory: the scan runs in waves
    // of wave_regions regions (0: one scan over all), each wave leaving its end
    // value in wave_carry[w] and, written by the kernel, in pinned h_wave[w],
    // and recording wave_ev[w], so that the positions of a finished wave go to
    // the host on d2h_stream while later input bytes are still arriving
    cudaStream_t d2h_stream = nullptr;
    uint32_t wave_regions = 0;
    uint32_t n_waves = 0;
    DevBuf<uint4> wave_carry;
    DevBuf<uint32_t> wave_nwork;        // per wave: work items, table and emit tickets
    uint4* h_wave = nullptr;
    uint4* d_h_wave = nullptr;          // h_wave as the device addresses it
    size_t h_wave_cap = 0;
    std::vector<cudaEvent_t> wave_ev;
    cudaEvent_t ev_d2h = nullptr;

    // value decoding over the staged result (cj_decode_values)
    DevBuf<uint8_t> val_type, val_str;
    DevBuf<uint64_t> val_num;
    DevBuf<uint32_t> val_len, val_long;
    DevBuf<unsigned long long> val_counts;
    DevBuf<uint64_t> pow5;
    uint64_t val_slots = 0;             // slots of the last decode (0: none)

    // queries over a staged JSON-Lines result
    DevBuf<unsigned long long> q_count;
    DevBuf<long long> q_out;

    // JSON-Lines chunk planning of device buffers (cj_plan_lines_count_device)
    DevBuf<uint32_t> plan_counts;
    DevBuf<uint2> plan_req;
    DevBuf<unsigned long long> plan_pos;
    DevBuf<unsigned long long> plan_bounds;   // cj_plan_lines_bytes_device: boundaries, counters

    // launch shapes (0 = default), set by cj_context_set_tuning / cj_autotune_staged
    int tune_region_steps = 0;
    int tune_tables_per_sm = 0;
    int tune_emit_per_sm = 0;
    uint32_t tune_pair_blocks = 0;
    uint32_t tune_pair_threads = 0;
    uint32_t tune_prefetch_steps = 0;
    int tune_stream_wave_mib = 0;
    bool wave_stream = false;           // the waves of this run report to the host (streamed parse)
};

namespace {

#define CJ_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            return (e_ == cudaErrorMemoryAllocation) ? CJ_ERR_OUT_OF_MEMORY  \
                                                     : CJ_ERR_CUDA;          \
        }                                                                    \
    } while (0)

template <typename T>
cj_status ensure(cj_context* ctx, DevBuf<T>& b, size_t n)
{
    if (n <= b.cap && b.p) return CJ_OK;
    if (b.p) { cudaFree(b.p); ctx->dev_bytes -= b.cap * sizeof(T); b.p = nullptr; b.cap = 0; }
    size_t want = std::max<size_t>(n + n / 8, 64);
    CJ_CUDA(cudaMalloc((void**)&b.p, want * sizeof(T)));
    b.cap = want;
    ctx->arena_gen++;
    ctx->dev_bytes += want * sizeof(T);
    return CJ_OK;
}

template <typename T>
void release(DevBuf<T>& b) { if (b.p) cudaFree(b.p); b.p = nullptr; b.cap = 0; }

int region_steps(const cj_context* ctx)
{
    return ctx->tune_region_steps ? ctx->tune_region_steps : kRegionStepsDefault;
}

// regions of an input of `bytes` in `segs` segments, for any region size
size_t max_regions(size_t bytes, size_t segs)
{
    return bytes / ((size_t)kRegionStepsAllowed[0] * kStepBytes) + segs + 1;
}

cj_status reserve_regions(cj_context* ctx, size_t regions)
{
    cj_status st;
    if ((st = ensure(ctx, ctx->rtab, regions * 4))) return st;
    if ((st = ensure(ctx, ctx->work, regions * 2))) return st;
    if ((st = ensure(ctx, ctx->region_seg, regions))) return st;
    if ((st = ensure(ctx, ctx->bagg, prefix_blocks(regions) * 4))) return st;
    return CJ_OK;
}

// Size every buffer for an input of `bytes` in `segs` segments.  S, the
// structural count, is at most the byte count, and so is the bracket count.
cj_status reserve(cj_context* ctx, size_t bytes, size_t segs)
{
    size_t padded = round_up(bytes, kPadBytes) + segs * (size_t)kPadBytes;
    size_t s_cap = bytes + 1;
    size_t chunks = (bytes + kChunk - 1) / kChunk + 1;
    cj_status st;
    if ((st = ensure(ctx, ctx->in, padded + 64))) return st;
    if ((st = ensure(ctx, ctx->pos, s_cap))) return st;
    if ((st = ensure(ctx, ctx->pair, s_cap))) return st;
    if ((st = ensure(ctx, ctx->brk, s_cap))) return st;
    if ((st = reserve_regions(ctx, max_regions(bytes, segs)))) return st;
    if ((st = ensure(ctx, ctx->masks, masks_cap(bytes, segs)))) return st;
    if ((st = ensure(ctx, ctx->segs, segs))) return st;
    if ((st = ensure(ctx, ctx->seg_out, segs))) return st;
    if ((st = ensure(ctx, ctx->spine, chunks * (size_t)kChunk))) return st;
    if ((st = ensure(ctx, ctx->cinfo, chunks))) return st;
    if (chunks > ctx->chunk_cap) {
        size_t off = 0, n = chunks;
        ctx->tree_off[0] = 0;
        for (int l = 1; l <= kTreeLevels; l++) {
            n = (n + 31) / 32;
            ctx->tree_off[l] = off;
            off += n;
        }
        bool fresh = ctx->tree.cap < off;
        if ((st = ensure(ctx, ctx->tree, off))) return st;
        if (fresh)
            CJ_CUDA(cudaMemsetAsync(ctx->tree.p, 0, ctx->tree.cap * sizeof(unsigned long long), ctx->stream));
        ctx->chunk_cap = chunks;
    }
    if (!ctx->h_ctrl) CJ_CUDA(cudaMallocHost((void**)&ctx->h_ctrl, sizeof(Ctrl)));
    if (ctx->h_seg_out_cap < segs) {
        if (ctx->h_seg_out) cudaFreeHost(ctx->h_seg_out);
        size_t want = std::max<size_t>(segs, 16);
        CJ_CUDA(cudaMallocHost((void**)&ctx->h_seg_out, want * sizeof(SegmentOut)));
        ctx->h_seg_out_cap = want;
    }
    return CJ_OK;
}

// Cut every segment of ctx->h_segs (dev_off, len set) into regions of the
// tuned size and queue the copies of the segment table and the region ->
// segment map (the host vectors must live until the stream passes them).
cj_status place_regions(cj_context* ctx)
{
    const int R = region_steps(ctx);
    const uint64_t rb = (uint64_t)R * kStepBytes;
    const size_t n = ctx->h_segs.size();
    uint64_t regions = 0;
    for (size_t i = 0; i < n; i++) {
        Segment& g = ctx->h_segs[i];
        g.first_region = (uint32_t)regions;
        g.n_regions = (uint32_t)((g.len + rb - 1) / rb);
        regions += g.n_regions;
    }
    if (regions >= 0xFFFFFFFFull) return CJ_ERR_TOO_LARGE;
    ctx->run_region_steps = R;
    ctx->n_regions = (uint32_t)regions;
    CJ_CUDA(cudaMemcpyAsync(ctx->segs.p, ctx->h_segs.data(), n * sizeof(Segment), cudaMemcpyHostToDevice,
                            ctx->stream));
    if (n > 1) {
        ctx->h_region_seg.resize(regions);
        for (size_t i = 0; i < n; i++)
            for (uint32_t t = 0; t < ctx->h_segs[i].n_regions; t++)
                ctx->h_region_seg[ctx->h_segs[i].first_region + t] = (uint32_t)i;
        CJ_CUDA(cudaMemcpyAsync(ctx->region_seg.p, ctx->h_region_seg.data(), regions * sizeof(uint32_t),
                                cudaMemcpyHostToDevice, ctx->stream));
    }
    return CJ_OK;
}

// Lay the chunks out on 1 KiB boundaries, cut them into regions and copy them
// to the device.
cj_status stage(cj_context* ctx, const uint8_t* const* chunks, const size_t* sizes, size_t n,
                bool lines)
{
    ctx->staged = false;
    ctx->graph_valid = false;
    if (!chunks || !sizes || n == 0) return CJ_ERR_INVALID_ARGUMENT;
    size_t total = 0;
    for (size_t i = 0; i < n; i++) {
        if (!chunks[i] || sizes[i] == 0) return CJ_ERR_INVALID_ARGUMENT;
        total += sizes[i];
    }
    if (total > CJ_MAX_INPUT_BYTES) return CJ_ERR_TOO_LARGE;
    CJ_CUDA(cudaSetDevice(ctx->device));
    cj_status st = reserve(ctx, total, n);
    if (st) return st;

    ctx->h_segs.resize(n);
    uint64_t dev_off = 0, logical = 0;
    for (size_t i = 0; i < n; i++) {
        Segment& s = ctx->h_segs[i];
        s.dev_off = dev_off;
        s.len = sizes[i];
        s.logical_off = logical;
        s.out_base = 0;
        s.brk_base = 0;
        s.flags = (i > 0) ? kSegContinue : 0u;
        s.pad = 0;
        dev_off += round_up(sizes[i], kPadBytes);
        logical += sizes[i];
    }
    for (size_t i = 0; i < n; i++)
        CJ_CUDA(cudaMemcpyAsync(ctx->in.p + ctx->h_segs[i].dev_off, chunks[i], sizes[i],
                                cudaMemcpyHostToDevice, ctx->stream));
    if ((st = place_regions(ctx))) return st;
    // host vectors must outlive the copies
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->n_bytes = total;
    ctx->n_segs = (uint32_t)n;
    ctx->lines = lines;
    ctx->batch = false;
    ctx->graph_valid = false;
    ctx->staged = true;
    return CJ_OK;
}

uint32_t pair_threads(const cj_context* ctx)
{
    return ctx->tune_pair_threads ? ctx->tune_pair_threads : 256u;
}

// Every kernel of one staged run, on the context stream, without host
// synchronisation.  `graph` selects the form that a CUDA graph replays: the
// epoch stays fixed and the pairing min-tree is cleared by the run itself
// instead of being told apart by epoch.
cj_status enqueue(cj_context* ctx, bool graph)
{
    if (!graph) {
        ctx->epoch = (ctx->epoch + 1) & 0x3FFFFFFFu;
        if (ctx->epoch == 0) {
            // epoch wrapped: stale min-tree tags could alias, so clear them
            CJ_CUDA(cudaMemsetAsync(ctx->tree.p, 0, ctx->tree.cap * sizeof(unsigned long long), ctx->stream));
            ctx->epoch = 1;
        }
    } else {
        CJ_CUDA(cudaMemsetAsync(ctx->tree.p, 0, ctx->tree.cap * sizeof(unsigned long long), ctx->stream));
    }
    CJ_CUDA(cudaMemsetAsync(ctx->d_ctrl, 0, sizeof(Ctrl), ctx->stream));
    if (ctx->batch) {
        CJ_CUDA(cudaMemsetAsync(ctx->seg_err.p, 0, ctx->n_segs * sizeof(uint32_t), ctx->stream));
        CJ_CUDA(cudaMemsetAsync(ctx->seg_depth.p, 0, ctx->n_segs * sizeof(int32_t), ctx->stream));
        // chunks without records read as kNoLevel (bytes 0x7F) in the next-lower search
        CJ_CUDA(cudaMemsetAsync(ctx->cinfo.p, 0x7F, (ctx->batch_chunks + 1) * sizeof(int4), ctx->stream));
    }

    cudaEvent_t* ev = nullptr;
    if (ctx->timing && !graph) {
        if (ctx->events_used + kEventsPerRun > ctx->events.size()) {
            for (size_t i = 0; i < kEventsPerRun; i++) {
                cudaEvent_t e;
                CJ_CUDA(cudaEventCreate(&e));
                ctx->events.push_back(e);
            }
        }
        ev = ctx->events.data() + ctx->events_used;
        ctx->events_used += kEventsPerRun;
        CJ_CUDA(cudaEventRecord(ev[0], ctx->stream));
    }
    const bool fine = ev && ctx->timing == 1;

    ScanParams sp{};
    sp.in = ctx->in.p;
    sp.segs = ctx->segs.p;
    sp.region_seg = (ctx->n_segs > 1) ? ctx->region_seg.p : nullptr;
    sp.n_segs = ctx->n_segs;
    sp.n_regions = ctx->n_regions;
    sp.pos = ctx->pos.p;
    sp.pair = ctx->pair.p;
    sp.brk = ctx->brk.p;
    sp.out_cap = ctx->pos.cap;
    sp.brk_cap = ctx->brk.cap;
    sp.rtab = ctx->rtab.p;
    sp.bagg = ctx->bagg.p;
    sp.masks = ctx->masks.p;
    sp.work = ctx->work.p;
    sp.ctrl = ctx->d_ctrl;
    sp.seg_out = ctx->seg_out.p;
    sp.seg_err = ctx->batch ? ctx->seg_err.p : nullptr;
    sp.ready = ctx->overlap_run ? ctx->d_ready : nullptr;
    sp.input_wait_limit = ctx->input_wait_limit;
    sp.region_steps = ctx->run_region_steps;
    sp.sm_count = ctx->sm_count;
    sp.prefetch_steps = ctx->tune_prefetch_steps;
    sp.dependent_launch = ctx->dependent_launch ? 1u : 0u;
    ScanShape shape{ctx->tune_tables_per_sm, ctx->tune_emit_per_sm};
    if (ctx->n_waves > 1) {
        // waves: each scans its regions from the previous wave's end value,
        // with its own work list (work items of wave w start at 2 * r_begin)
        CJ_CUDA(cudaMemsetAsync(ctx->wave_nwork.p, 0, 3 * ctx->n_waves * sizeof(uint32_t), ctx->stream));
        for (uint32_t w = 0; w < ctx->n_waves; w++) {
            ScanParams wp = sp;
            wp.r_begin = w * ctx->wave_regions;
            wp.r_end = std::min<uint32_t>(ctx->n_regions, wp.r_begin + ctx->wave_regions);
            wp.carry_in = w ? ctx->wave_carry.p + (w - 1) : nullptr;
            wp.carry_out = ctx->wave_carry.p + w;
            wp.carry_host = ctx->wave_stream ? ctx->d_h_wave + w : nullptr;
            wp.n_work = ctx->wave_nwork.p + 3 * w;
            wp.tickets = ctx->wave_nwork.p + 3 * w + 1;
            wp.work = ctx->work.p + 2 * (size_t)wp.r_begin;
            launch_scan(wp, ctx->lines, shape, ctx->stream, fine ? ev + 1 : nullptr);
            ctx->launches += scan_launches(wp.r_end - wp.r_begin);
            // no copy on the stream between waves: a copy queued behind a
            // scan that waits for input bytes could hold up the input's copies
            if (ctx->wave_stream) CJ_CUDA(cudaEventRecord(ctx->wave_ev[w], ctx->stream));
        }
    } else {
        launch_scan(sp, ctx->lines, shape, ctx->stream, fine ? ev + 1 : nullptr);
        ctx->launches += scan_launches(ctx->n_regions);
    }
    if (ev && ctx->timing == 2) {
        // coarse timing: no events between the scan's kernels, which would
        // keep each from being scheduled while the one before it finishes
        for (int k = 1; k <= 3; k++) CJ_CUDA(cudaEventRecord(ev[k], ctx->stream));
    }
    if (ctx->batch) {
        launch_batch_prefix(ctx->segs.p, ctx->seg_out.p, ctx->n_segs, ctx->layout_off.p, ctx->rchunk_off.p,
                            ctx->stream, ctx->dependent_launch);
        ctx->launches += 1;
    }

    PairParams pp{};
    pp.dependent_launch = ctx->dependent_launch ? 1u : 0u;
    pp.brk = ctx->brk.p;
    pp.pair = ctx->pair.p;
    pp.spine = ctx->spine.p;
    pp.cinfo = ctx->cinfo.p;
    pp.tree = ctx->tree.p;
    for (int l = 0; l <= kTreeLevels; l++) pp.tree_off[l] = ctx->tree_off[l];
    pp.ctrl = ctx->d_ctrl;
    pp.epoch = ctx->epoch;
    pp.chunk_cap = (uint32_t)ctx->chunk_cap;
    pp.rchunk_off = ctx->batch ? ctx->rchunk_off.p : nullptr;
    pp.n_bsegs = ctx->batch ? ctx->n_segs : 0u;
    pp.segs = ctx->segs.p;
    pp.seg_out = ctx->seg_out.p;
    pp.seg_err = ctx->batch ? ctx->seg_err.p : nullptr;
    pp.seg_depth = ctx->batch ? ctx->seg_depth.p : nullptr;
    pp.n_chunks = ctx->batch ? ctx->batch_chunks : 0;
    const uint32_t pthreads = pair_threads(ctx);
    // batch: the chunks holding records are at most bytes / 8 / kChunk + one per document
    const size_t max_chunks = ctx->batch ? ctx->n_bytes / 8 / kChunk + ctx->n_segs
                                         : (ctx->n_bytes + kChunk - 1) / kChunk;
    const size_t warps_per_block = pthreads / 32;
    int grid = (int)std::min<size_t>((max_chunks + warps_per_block - 1) / warps_per_block + 1,
                                     (size_t)ctx->sm_count * 8 * 256 / pthreads);
    if (ctx->tune_pair_blocks) grid = (int)std::min<size_t>((size_t)grid, ctx->tune_pair_blocks);
    launch_pair(pp, grid, ctx->stream, (int)pthreads);
    if (fine) CJ_CUDA(cudaEventRecord(ev[4], ctx->stream));
    launch_spine(pp, grid, ctx->stream, (int)pthreads);
    // timing 3 (the run's ends only): the scan's events at the run's end
    if (ev && ctx->timing == 3)
        for (int k = 1; k <= 3; k++) CJ_CUDA(cudaEventRecord(ev[k], ctx->stream));
    if (ev && !fine) CJ_CUDA(cudaEventRecord(ev[4], ctx->stream));
    if (ev) CJ_CUDA(cudaEventRecord(ev[5], ctx->stream));
    ctx->launches += 2;
    if (ctx->batch) {
        launch_batch_layout(ctx->segs.p, ctx->seg_out.p, ctx->n_segs, ctx->pos.p, ctx->pair.p,
                            ctx->layout_off.p, ctx->layout.p, ctx->sm_count, ctx->stream, ctx->dependent_launch);
        ctx->launches += 1;
        ctx->batch_read = false;
    }
    CJ_CUDA(cudaGetLastError());
    return CJ_OK;
}

cj_status run(cj_context* ctx)
{
    if (!ctx->staged) return CJ_ERR_NOT_STAGED;
    CJ_CUDA(cudaSetDevice(ctx->device));
    return enqueue(ctx, false);
}

// Capture the staged run once into a CUDA graph, then replay it.
cj_status run_graph(cj_context* ctx)
{
    if (!ctx->staged) return CJ_ERR_NOT_STAGED;
    CJ_CUDA(cudaSetDevice(ctx->device));
    if (!ctx->graph_valid) {
        if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
        ctx->epoch = (ctx->epoch + 1) & 0x3FFFFFFFu;
        if (ctx->epoch == 0) ctx->epoch = 1;
        CJ_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int64_t launches0 = ctx->launches;
        cj_status st = enqueue(ctx, true);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        ctx->graph_launches = ctx->launches - launches0;
        ctx->launches = launches0;
        if (st) { if (g) cudaGraphDestroy(g); return st; }
        if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return CJ_ERR_CUDA; }
        e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { ctx->graph_exec = nullptr; return CJ_ERR_CUDA; }
        ctx->graph_valid = true;
    }
    CJ_CUDA(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += ctx->graph_launches;
    ctx->batch_read = false;
    return CJ_OK;
}

// Raises the count of input bytes present; runs after each chunk's copy on
// the copy stream.
__global__ void mark_ready(unsigned long long* ready, unsigned long long bytes)
{
    if (threadIdx.x == 0) {
        __threadfence_system();
        asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(ready), "l"(bytes) : "memory");
    }
}

constexpr size_t kOverlapMin = 64ull << 20;     // smaller inputs: one copy, then the run
// copy granularity of an overlapped run: each piece is followed by a write of
// the bytes present, which orders the copy before it and leaves the copy
// engine a short gap (streamed 1 GiB parse: 5.76 / 5.56 / 5.47 / 5.43 ms with
// 16 / 32 / 64 / 128 MiB pieces)
#ifndef CJ_OVERLAP_CHUNK_MIB
#define CJ_OVERLAP_CHUNK_MIB 128
#endif
constexpr size_t kOverlapChunk = (size_t)CJ_OVERLAP_CHUNK_MIB << 20;
constexpr size_t kWaveBytes = 128ull << 20;     // default input bytes per scan wave of a streamed parse

// input bytes per wave of a streamed parse (0: not streamed)
uint64_t stream_wave_bytes(const cj_context* ctx)
{
    if (ctx->tune_stream_wave_mib < 0) return 0;
    return ctx->tune_stream_wave_mib ? (uint64_t)ctx->tune_stream_wave_mib << 20 : kWaveBytes;
}

// Wave layout of a streamed parse over the placed regions: waves of
// `wave_bytes` of regions, their end values on the device and in pinned host
// memory, and one event per wave.
cj_status prepare_waves(cj_context* ctx, uint64_t wave_bytes)
{
    const uint64_t rb = (uint64_t)ctx->run_region_steps * kStepBytes;
    ctx->wave_regions = (uint32_t)std::max<uint64_t>(1, wave_bytes / rb);
    const uint32_t nw = (uint32_t)((ctx->n_regions + (uint64_t)ctx->wave_regions - 1) / ctx->wave_regions);
    cj_status st;
    if ((st = ensure(ctx, ctx->wave_carry, nw))) return st;
    if ((st = ensure(ctx, ctx->wave_nwork, 3 * (size_t)nw))) return st;
    ctx->n_waves = nw;
    ctx->wave_stream = true;
    if (ctx->h_wave_cap < nw) {
        if (ctx->h_wave) cudaFreeHost(ctx->h_wave);
        ctx->h_wave = nullptr;
        ctx->h_wave_cap = 0;
        const size_t want = std::max<size_t>(nw, 32);
        CJ_CUDA(cudaMallocHost((void**)&ctx->h_wave, want * sizeof(uint4)));
        ctx->h_wave_cap = want;
        if (cudaHostGetDevicePointer((void**)&ctx->d_h_wave, ctx->h_wave, 0) != cudaSuccess) {
            cudaGetLastError();
            cudaFreeHost(ctx->h_wave);
            ctx->h_wave = nullptr;
            ctx->d_h_wave = nullptr;
            ctx->h_wave_cap = 0;
            return CJ_ERR_CUDA;
        }
    }
    while (ctx->wave_ev.size() < nw) {
        cudaEvent_t e;
        CJ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->wave_ev.push_back(e);
    }
    // an aborted wave leaves its end value zero (below the previous one)
    memset(ctx->h_wave, 0, nw * sizeof(uint4));
    return CJ_OK;
}

// Stage and run in one go, the input's copy overlapping the scan: the small
// tables go first, then the scan is launched and the input follows in chunks
// on the copy stream, each chunk raising d_ready.
cj_status stage_overlapped(cj_context* ctx, const uint8_t* const* chunks, const size_t* sizes, size_t n,
                           bool lines, bool waves = false)
{
    ctx->staged = false;
    ctx->graph_valid = false;
    if (!chunks || !sizes || n == 0) return CJ_ERR_INVALID_ARGUMENT;
    size_t total = 0;
    for (size_t i = 0; i < n; i++) {
        if (!chunks[i] || sizes[i] == 0) return CJ_ERR_INVALID_ARGUMENT;
        total += sizes[i];
    }
    if (total > CJ_MAX_INPUT_BYTES) return CJ_ERR_TOO_LARGE;
    CJ_CUDA(cudaSetDevice(ctx->device));
    cj_status st = reserve(ctx, total, n);
    if (st) return st;
    ctx->h_segs.resize(n);
    uint64_t dev_off = 0, logical = 0;
    for (size_t i = 0; i < n; i++) {
        Segment& g = ctx->h_segs[i];
        g.dev_off = dev_off;
        g.len = sizes[i];
        g.logical_off = logical;
        g.out_base = 0;
        g.brk_base = 0;
        g.flags = (i > 0) ? kSegContinue : 0u;
        g.pad = 0;
        dev_off += round_up(sizes[i], kPadBytes);
        logical += sizes[i];
    }
    if ((st = place_regions(ctx))) return st;
    ctx->n_waves = 0;
    ctx->wave_stream = false;
    if (waves && (st = prepare_waves(ctx, stream_wave_bytes(ctx)))) return st;
    CJ_CUDA(cudaMemsetAsync(ctx->d_ready, 0, sizeof(unsigned long long), ctx->stream));
    CJ_CUDA(cudaEventRecord(ctx->ev_reset, ctx->stream));
    ctx->n_bytes = total;
    ctx->n_segs = (uint32_t)n;
    ctx->lines = lines;
    ctx->batch = false;
    ctx->staged = true;
    ctx->overlap_run = true;
    st = enqueue(ctx, false);
    ctx->overlap_run = false;
    if (st) { ctx->n_waves = 0; return st; }
    CJ_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_reset, 0));
    for (size_t i = 0; i < n; i++) {
        const Segment& g = ctx->h_segs[i];
        for (uint64_t o = 0; o < g.len; o += kOverlapChunk) {
            const uint64_t c = std::min<uint64_t>(kOverlapChunk, g.len - o);
            CJ_CUDA(cudaMemcpyAsync(ctx->in.p + g.dev_off + o, chunks[i] + o, c, cudaMemcpyHostToDevice,
                                    ctx->copy_stream));
            const uint64_t upto = (o + c == g.len) ? round_up(g.len, kPadBytes) : o + c;
            if (ctx->write64) {
                // default flags: the write follows a barrier that orders the copy before it
                if (ctx->write64((CUstream)ctx->copy_stream, (CUdeviceptr)ctx->d_ready, g.dev_off + upto,
                                 CU_STREAM_WRITE_VALUE_DEFAULT) != CUDA_SUCCESS)
                    return CJ_ERR_CUDA;
            } else {
                mark_ready<<<1, 32, 0, ctx->copy_stream>>>(ctx->d_ready, g.dev_off + upto);
                ctx->launches += 1;
            }
        }
    }
    CJ_CUDA(cudaGetLastError());
    CJ_CUDA(cudaEventRecord(ctx->ev_copied, ctx->copy_stream));
    CJ_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied, 0));
    // the scan spins on these copies: make sure they are submitted now, not
    // when the host next waits on a stream that depends on them (the streamed
    // parse waits on each wave's event, which does not)
    const cudaError_t q = cudaStreamQuery(ctx->copy_stream);
    if (q != cudaSuccess && q != cudaErrorNotReady) return CJ_ERR_CUDA;
    return CJ_OK;
}

bool is_pinned(const void* p);
cj_status read_info(cj_context* ctx, cj_parse_info* info);

// One-shot parse of a large pinned input into pinned host memory, streamed:
// the input's copy, the scan (in waves) and the positions' copy back overlap.
// Each wave's positions go to host_out as soon as the wave is scanned (while
// the copy engine still brings in later bytes); the pair row follows the
// pairing, which needs every bracket.  On a non-OK status host_out may hold
// part of a result.
cj_status parse_streamed(cj_context* ctx, const uint8_t* const* chunks, const size_t* sizes, size_t n,
                         bool lines, int32_t* out, size_t cap, cj_parse_info* info)
{
    cj_status st = stage_overlapped(ctx, chunks, sizes, n, lines, true);
    if (st) return st;
    const uint32_t nw = ctx->n_waves;
    ctx->n_waves = 0;                     // later runs of the staged input scan in one go
    ctx->wave_stream = false;
    uint64_t s_prev = 0, s_pair = UINT64_MAX;
    for (uint32_t w = 0; w < nw; w++) {
        CJ_CUDA(cudaEventSynchronize(ctx->wave_ev[w]));
        const uint64_t s_w = ctx->h_wave[w].y;
        // an aborted or failed wave (end value below the last one, or past the
        // input) ends the streaming; the verdict below reports it
        if (s_w < s_prev || s_w > ctx->n_bytes || 2 * s_w + 4 > cap) break;
        if (s_w > s_prev)
            CJ_CUDA(cudaMemcpyAsync(out + 1 + s_prev, ctx->pos.p + s_prev, (s_w - s_prev) * sizeof(int32_t),
                                    cudaMemcpyDeviceToHost, ctx->d2h_stream));
        s_prev = s_w;
        if (w + 1 == nw && s_w > 0) {
            // the last wave gives S, so the pair row's place in host_out: its
            // copy follows the pairing kernels on the stream, with no round
            // trip through the host (the input's copies are all done by now)
            CJ_CUDA(cudaMemcpyAsync(out + s_w + 2, ctx->pair.p, s_w * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                    ctx->stream));
            s_pair = s_w;
        }
    }
    cj_parse_info local;
    if (!info) info = &local;
    st = read_info(ctx, info);
    if (!st && info->status != CJ_OK) st = (cj_status)info->status;
    const uint64_t S = (uint64_t)info->n_structural;
    if (!st && 2 * S + 4 > cap) st = CJ_ERR_CAPACITY;
    if (!st) {
        if (S > s_prev)
            CJ_CUDA(cudaMemcpyAsync(out + 1 + s_prev, ctx->pos.p + s_prev, (S - s_prev) * sizeof(int32_t),
                                    cudaMemcpyDeviceToHost, ctx->d2h_stream));
        if (S > 0 && S != s_pair)
            CJ_CUDA(cudaMemcpyAsync(out + S + 2, ctx->pair.p, S * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                    ctx->d2h_stream));
        out[0] = 0;
        out[S + 1] = (int32_t)(S + 1);
        out[2 * S + 2] = 0;
        out[2 * S + 3] = 0;
    }
    CJ_CUDA(cudaStreamSynchronize(ctx->d2h_stream));
    return st;
}

bool is_pinned(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// One-shot staging and run: overlapped for large pinned inputs (a copy from
// pageable memory goes through the driver's staging and may synchronise with
// other work), else copy then run.
cj_status stage_run(cj_context* ctx, const uint8_t* const* chunks, const size_t* sizes, size_t n, bool lines)
{
    size_t total = 0;
    bool pinned = chunks != nullptr;
    for (size_t i = 0; sizes && i < n; i++) {
        total += sizes[i];
        if (pinned && (!chunks[i] || !is_pinned(chunks[i]))) pinned = false;
    }
    if (total >= kOverlapMin && pinned) return stage_overlapped(ctx, chunks, sizes, n, lines);
    cj_status st = stage(ctx, chunks, sizes, n, lines);
    if (!st) st = run(ctx);
    return st;
}

// One-shot JSON-Lines parse of a host buffer whose chunks are planned on the
// device: the buffer goes to the staging area (`pack`) in kOverlapChunk
// pieces on the copy stream, each piece's newlines counted per 64 KiB block as
// soon as it lands (chunk-count plans); the plan is finished on the device,
// every chunk moved to its 1 KiB-aligned place in `in` (batch_scatter) and the
// chunks run as cj_parse_lines runs them.
cj_status stage_lines_planned(cj_context* ctx, const uint8_t* data, size_t size, size_t chunk_count,
                              size_t chunk_bytes, std::vector<size_t>& sizes)
{
    ctx->staged = false;
    ctx->graph_valid = false;
    if (!data || size == 0) return CJ_ERR_INVALID_ARGUMENT;
    if (size > CJ_MAX_INPUT_BYTES) return CJ_ERR_TOO_LARGE;
    CJ_CUDA(cudaSetDevice(ctx->device));
    cj_status st;
    const size_t nb = (size + kPlanBlockBytes - 1) / kPlanBlockBytes;
    if ((st = ensure(ctx, ctx->pack, size + 16))) return st;
    if (chunk_count) {
        if ((st = ensure(ctx, ctx->plan_counts, nb))) return st;
        if ((st = ensure(ctx, ctx->plan_req, chunk_count + 1))) return st;
        if ((st = ensure(ctx, ctx->plan_pos, chunk_count + 1))) return st;
    }
    // the copy, and the newline counts of each piece behind it
    CJ_CUDA(cudaEventRecord(ctx->ev_reset, ctx->stream));
    CJ_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_reset, 0));
    for (uint64_t o = 0; o < size; o += kOverlapChunk) {
        const uint64_t c = std::min<uint64_t>(kOverlapChunk, size - o);
        CJ_CUDA(cudaMemcpyAsync(ctx->pack.p + o, data + o, c, cudaMemcpyHostToDevice, ctx->copy_stream));
        if (chunk_count) {
            launch_plan_count(ctx->pack.p + o, c, ctx->plan_counts.p + o / kPlanBlockBytes, ctx->copy_stream);
            ctx->launches += 1;
        }
    }
    CJ_CUDA(cudaGetLastError());
    CJ_CUDA(cudaEventRecord(ctx->ev_copied, ctx->copy_stream));
    CJ_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied, 0));
    if (chunk_count) {
        std::vector<uint32_t> counts(nb);
        CJ_CUDA(cudaMemcpyAsync(counts.data(), ctx->plan_counts.p, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
        CJ_CUDA(cudaStreamSynchronize(ctx->stream));
        sizes.assign(chunk_count, 0);
        if (plan_lines_count_finish(ctx->pack.p, size, chunk_count, sizes.data(), counts.data(), data[size - 1],
                                    ctx->plan_req.p, ctx->plan_pos.p, ctx->stream) != cudaSuccess)
            return CJ_ERR_CUDA;
        ctx->launches += 1;
    } else {
        size_t n = 0;
        if ((st = cj_plan_lines_bytes_device(ctx, ctx->pack.p, size, chunk_bytes, nullptr, 0, &n, ctx->stream)))
            return st;
        sizes.assign(n, 0);
        if ((st = cj_plan_lines_bytes_device(ctx, ctx->pack.p, size, chunk_bytes, sizes.data(), n, &n,
                                             ctx->stream)))
            return st;
        ctx->launches += 2;
    }
    // chunks as cj_parse_lines takes them: an empty chunk is refused
    const size_t n = sizes.size();
    if (n == 0) return CJ_ERR_INVALID_ARGUMENT;
    for (size_t k = 0; k < n; k++)
        if (sizes[k] == 0) return CJ_ERR_INVALID_ARGUMENT;
    if ((st = reserve(ctx, size, n))) return st;
    if ((st = ensure(ctx, ctx->pack_off, 2 * (n + 1)))) return st;
    ctx->h_segs.resize(n);
    ctx->h_pack_off.assign(2 * (n + 1), 0);
    uint64_t dev_off = 0, logical = 0, wo = 0;
    for (size_t k = 0; k < n; k++) {
        Segment& g = ctx->h_segs[k];
        g.dev_off = dev_off;
        g.len = sizes[k];
        g.logical_off = logical;
        g.out_base = 0;
        g.brk_base = 0;
        g.flags = (k > 0) ? kSegContinue : 0u;
        g.pad = 0;
        ctx->h_pack_off[k] = logical;
        ctx->h_pack_off[n + 1 + k] = wo;
        dev_off += round_up(sizes[k], kPadBytes);
        logical += sizes[k];
        wo += (sizes[k] + 3) / 4;
    }
    ctx->h_pack_off[n] = logical;
    ctx->h_pack_off[2 * n + 1] = wo;
    CJ_CUDA(cudaMemcpyAsync(ctx->pack_off.p, ctx->h_pack_off.data(), ctx->h_pack_off.size() * sizeof(uint64_t),
                            cudaMemcpyHostToDevice, ctx->stream));
    if ((st = place_regions(ctx))) return st;
    launch_batch_scatter(ctx->pack.p, ctx->pack_off.p, ctx->pack_off.p + n + 1, ctx->segs.p, (uint32_t)n, wo,
                         ctx->in.p, ctx->sm_count, ctx->stream);
    ctx->launches += 1;
    CJ_CUDA(cudaGetLastError());
    // host vectors must outlive the copies
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->n_bytes = size;
    ctx->n_segs = (uint32_t)n;
    ctx->lines = true;
    ctx->batch = false;
    ctx->staged = true;
    return CJ_OK;
}

cj_status read_info(cj_context* ctx, cj_parse_info* info)
{
    if (!ctx->staged) return CJ_ERR_NOT_STAGED;
    CJ_CUDA(cudaMemcpyAsync(ctx->h_ctrl, ctx->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaMemcpyAsync(ctx->h_seg_out, ctx->seg_out.p, ctx->n_segs * sizeof(SegmentOut),
                            cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    const Ctrl& c = *ctx->h_ctrl;
    uint32_t flags = c.error_flags;
    if (c.neg_min_level > 0) flags |= CJ_FLAG_BRACKETS;
    if (flags & CJ_FLAG_TIMEOUT) flags |= (c.gave_up & 0xFFu) << 16;
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
        info->n_segments = (int32_t)ctx->n_segs;
    }
    return CJ_OK;
}

// Reference layout into host_out (2*(S+2) entries).
cj_status copy_result(cj_context* ctx, int64_t S, int32_t* out, size_t cap)
{
    if ((size_t)(2 * S + 4) > cap) return CJ_ERR_CAPACITY;
    out[0] = 0;
    out[S + 1] = (int32_t)(S + 1);
    out[2 * S + 2] = 0;
    out[2 * S + 3] = 0;
    if (S > 0) {
        CJ_CUDA(cudaMemcpyAsync(out + 1, ctx->pos.p, (size_t)S * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, ctx->stream));
        CJ_CUDA(cudaMemcpyAsync(out + S + 2, ctx->pair.p, (size_t)S * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, ctx->stream));
    }
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    return CJ_OK;
}

cj_status to_result(cj_context* ctx, const cj_parse_info& info, cj_result* out)
{
    int64_t S = info.n_structural;
    int32_t* buf = static_cast<int32_t*>(pinned_alloc((size_t)(2 * S + 4) * sizeof(int32_t)));
    if (!buf) return CJ_ERR_OUT_OF_MEMORY;
    cj_status st = copy_result(ctx, S, buf, (size_t)(2 * S + 4));
    if (st) { pinned_free(buf); return st; }
    int64_t* seg_sizes = (int64_t*)malloc(sizeof(int64_t) * (ctx->n_segs ? ctx->n_segs : 1));
    if (!seg_sizes) {
        pinned_free(buf);
        return CJ_ERR_OUT_OF_MEMORY;
    }
    out->structural = buf;
    out->pair_pos = buf + S + 1;
    out->n_structural = S;
    out->total = S + 2;
    out->max_depth = info.max_depth;
    out->status = CJ_OK;
    out->n_segments = ctx->n_segs;
    out->segment_sizes = seg_sizes;
    uint32_t prev = 0;
    for (uint32_t i = 0; i < ctx->n_segs; i++) {
        out->segment_sizes[i] = (int64_t)(ctx->h_seg_out[i].s_end - prev);
        prev = ctx->h_seg_out[i].s_end;
    }
    return CJ_OK;
}

// ---- batches of independent documents ---------------------------------------
//
// Device layout of a batch of n documents with sizes b_i:
//   in:    document i at dev_off_i = sum_{j<i} round_up(b_j, 1 KiB)
//   pos, pair: out_base_i = sum_{j<i} (b_j + 1)            (S_i <= b_i)
//   brk:   brk_base_i = sum_{j<i} round_up(b_j, kChunk)   (K_i <= b_i; chunk-aligned,
//          so a pairing chunk never holds two documents)
//   layout: every document's 2*(S_i+2) result back to back (offsets on the device)
cj_status reserve_batch(cj_context* ctx, uint64_t in_bytes, uint64_t out_cap, uint64_t brk_cap,
                        uint64_t regions, size_t n, uint64_t layout_cap, uint64_t pack_bytes)
{
    const uint64_t chunks = brk_cap / kChunk + 1;
    cj_status st;
    if ((st = ensure(ctx, ctx->in, in_bytes + 64))) return st;
    if ((st = ensure(ctx, ctx->pos, out_cap))) return st;
    if ((st = ensure(ctx, ctx->pair, out_cap))) return st;
    if ((st = ensure(ctx, ctx->brk, brk_cap + 1))) return st;
    if ((st = reserve_regions(ctx, regions))) return st;
    if ((st = ensure(ctx, ctx->masks, masks_cap(in_bytes, n)))) return st;
    if ((st = ensure(ctx, ctx->segs, n))) return st;
    if ((st = ensure(ctx, ctx->seg_out, n))) return st;
    if ((st = ensure(ctx, ctx->spine, chunks * (size_t)kChunk))) return st;
    if ((st = ensure(ctx, ctx->cinfo, chunks))) return st;
    if ((st = ensure(ctx, ctx->seg_err, n))) return st;
    if ((st = ensure(ctx, ctx->seg_depth, n))) return st;
    if ((st = ensure(ctx, ctx->rchunk_off, n + 1))) return st;
    if ((st = ensure(ctx, ctx->layout_off, n + 1))) return st;
    if ((st = ensure(ctx, ctx->layout, layout_cap))) return st;
    if (pack_bytes) {
        if ((st = ensure(ctx, ctx->pack, pack_bytes + 16))) return st;
        if ((st = ensure(ctx, ctx->pack_off, 2 * (n + 1)))) return st;
    }
    if (chunks > ctx->chunk_cap) {
        size_t off = 0, m = chunks;
        ctx->tree_off[0] = 0;
        for (int l = 1; l <= kTreeLevels; l++) {
            m = (m + 31) / 32;
            ctx->tree_off[l] = off;
            off += m;
        }
        if ((st = ensure(ctx, ctx->tree, off))) return st;
        ctx->chunk_cap = chunks;
    }
    // a fresh or regrown tree array must not hold stale tags
    CJ_CUDA(cudaMemsetAsync(ctx->tree.p, 0, ctx->tree.cap * sizeof(unsigned long long), ctx->stream));
    if (!ctx->h_ctrl) CJ_CUDA(cudaMallocHost((void**)&ctx->h_ctrl, sizeof(Ctrl)));
    return CJ_OK;
}

// `docs` (one host pointer per document) or `packed` (documents back to back)
cj_status stage_batch(cj_context* ctx, const uint8_t* const* docs, const uint8_t* packed,
                      const size_t* sizes, size_t n, bool lines, bool tables_only = false)
{
    // a captured graph stays valid for a new batch of the same document sizes
    // in the same buffers
    bool same = ctx->graph_valid && ctx->batch && ctx->staged && ctx->lines == lines && sizes &&
                ctx->h_segs.size() == n;
    for (size_t i = 0; same && i < n; i++) same = ctx->h_segs[i].len == sizes[i];
    const uint64_t gen0 = ctx->arena_gen;
    ctx->staged = false;
    ctx->graph_valid = false;
    if (!sizes || n == 0 || n > 0xFFFFFFFEu || (!docs && !packed && !tables_only)) return CJ_ERR_INVALID_ARGUMENT;
    // region capacity for the smallest region size, so a tuning change needs no regrowth
    uint64_t in_bytes = 0, out_cap = 0, brk_cap = 0, regions = 0, layout_cap = 0, total = 0;
    const uint64_t rb = (uint64_t)kRegionStepsAllowed[0] * kStepBytes;
    for (size_t i = 0; i < n; i++) {
        if (sizes[i] == 0 || (docs && !docs[i])) return CJ_ERR_INVALID_ARGUMENT;
        if (sizes[i] > CJ_MAX_INPUT_BYTES) return CJ_ERR_TOO_LARGE;
        in_bytes += round_up(sizes[i], kPadBytes);
        out_cap += sizes[i] + 1;
        brk_cap += round_up(sizes[i], kChunk);
        regions += (sizes[i] + rb - 1) / rb;
        layout_cap += 2 * (uint64_t)sizes[i] + 4;
        total += sizes[i];
    }
    if (regions >= 0xFFFFFFFFull) return CJ_ERR_TOO_LARGE;
    CJ_CUDA(cudaSetDevice(ctx->device));
    cj_status st = reserve_batch(ctx, in_bytes, out_cap, brk_cap, regions + 1, n, layout_cap,
                                 (packed && !tables_only) ? total : 0);
    if (st) return st;

    ctx->h_segs.resize(n);
    uint64_t dev_off = 0, out_base = 0, brk_base = 0;
    for (size_t i = 0; i < n; i++) {
        Segment& g = ctx->h_segs[i];
        g.dev_off = dev_off;
        g.len = sizes[i];
        g.logical_off = 0;
        g.out_base = out_base;
        g.brk_base = brk_base;
        g.flags = 0;
        g.pad = 0;
        dev_off += round_up(sizes[i], kPadBytes);
        out_base += sizes[i] + 1;
        brk_base += round_up(sizes[i], kChunk);
    }
    if (tables_only) {
        // the caller copies the data (cj_parse_batch_padded)
    } else if (packed) {
        // one copy of the packed documents, then a kernel moves each one to
        // its aligned place
        ctx->h_pack_off.assign(2 * (n + 1), 0);
        uint64_t so = 0, wo = 0;
        for (size_t i = 0; i < n; i++) {
            ctx->h_pack_off[i] = so;
            ctx->h_pack_off[n + 1 + i] = wo;
            so += sizes[i];
            wo += (sizes[i] + 3) / 4;
        }
        ctx->h_pack_off[n] = so;
        ctx->h_pack_off[2 * n + 1] = wo;
        CJ_CUDA(cudaMemcpyAsync(ctx->pack.p, packed, total, cudaMemcpyHostToDevice, ctx->stream));
        CJ_CUDA(cudaMemcpyAsync(ctx->pack_off.p, ctx->h_pack_off.data(), ctx->h_pack_off.size() * sizeof(uint64_t),
                                cudaMemcpyHostToDevice, ctx->stream));
    } else {
        for (size_t i = 0; i < n; i++)
            CJ_CUDA(cudaMemcpyAsync(ctx->in.p + ctx->h_segs[i].dev_off, docs[i], sizes[i],
                                    cudaMemcpyHostToDevice, ctx->stream));
    }
    if ((st = place_regions(ctx))) return st;
    if (packed && !tables_only) {
        launch_batch_scatter(ctx->pack.p, ctx->pack_off.p, ctx->pack_off.p + n + 1, ctx->segs.p, (uint32_t)n,
                             ctx->h_pack_off[2 * n + 1], ctx->in.p, ctx->sm_count, ctx->stream);
        ctx->launches += 1;
    }
    ctx->batch_chunks = brk_cap / kChunk;
    CJ_CUDA(cudaGetLastError());
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));   // host vectors must outlive the copies
    ctx->n_bytes = total;
    ctx->n_segs = (uint32_t)n;
    ctx->lines = lines;
    ctx->batch = true;
    ctx->batch_read = false;
    ctx->graph_valid = same && ctx->arena_gen == gen0 && !tables_only;
    ctx->staged = true;
    return CJ_OK;
}

// A batch whose host buffer already has the device layout (every document at
// its 1 KiB-aligned offset, cj_batch_padded_offsets): the run starts at once
// and the copy follows on the copy stream in chunks; the scan takes a region
// once the bytes counter covers it (as in stage_overlapped).  Without the
// driver's stream write the copy simply precedes the run.
cj_status parse_batch_padded(cj_context* ctx, const uint8_t* padded, const size_t* sizes, size_t n, bool lines)
{
    if (!padded) return CJ_ERR_INVALID_ARGUMENT;
    cj_status st = stage_batch(ctx, nullptr, nullptr, sizes, n, lines, true);
    if (st) return st;
    const Segment& last = ctx->h_segs[n - 1];
    const uint64_t bytes = last.dev_off + round_up(last.len, kPadBytes);
    if (!ctx->write64) {
        CJ_CUDA(cudaMemcpyAsync(ctx->in.p, padded, bytes, cudaMemcpyHostToDevice, ctx->stream));
        return run(ctx);
    }
    CJ_CUDA(cudaMemsetAsync(ctx->d_ready, 0, sizeof(unsigned long long), ctx->stream));
    CJ_CUDA(cudaEventRecord(ctx->ev_reset, ctx->stream));
    ctx->overlap_run = true;
    st = enqueue(ctx, false);
    ctx->overlap_run = false;
    if (st) return st;
    CJ_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_reset, 0));
    for (uint64_t o = 0; o < bytes; o += kOverlapChunk) {
        const uint64_t c = std::min<uint64_t>(kOverlapChunk, bytes - o);
        CJ_CUDA(cudaMemcpyAsync(ctx->in.p + o, padded + o, c, cudaMemcpyHostToDevice, ctx->copy_stream));
        if (ctx->write64((CUstream)ctx->copy_stream, (CUdeviceptr)ctx->d_ready, o + c,
                         CU_STREAM_WRITE_VALUE_DEFAULT) != CUDA_SUCCESS)
            return CJ_ERR_CUDA;
    }
    CJ_CUDA(cudaEventRecord(ctx->ev_copied, ctx->copy_stream));
    CJ_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied, 0));
    return CJ_OK;
}

// per-document counts, verdicts, depths and layout offsets into host mirrors
cj_status read_batch(cj_context* ctx)
{
    if (!ctx->staged || !ctx->batch) return CJ_ERR_NOT_STAGED;
    if (ctx->batch_read) return CJ_OK;
    const size_t n = ctx->n_segs;
    ctx->h_bseg_out.resize(n);
    ctx->h_seg_err.resize(n);
    ctx->h_seg_depth.resize(n);
    ctx->h_layout_off.resize(n + 1);
    CJ_CUDA(cudaMemcpyAsync(ctx->h_ctrl, ctx->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaMemcpyAsync(ctx->h_bseg_out.data(), ctx->seg_out.p, n * sizeof(SegmentOut),
                            cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaMemcpyAsync(ctx->h_seg_err.data(), ctx->seg_err.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            ctx->stream));
    CJ_CUDA(cudaMemcpyAsync(ctx->h_seg_depth.data(), ctx->seg_depth.p, n * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaMemcpyAsync(ctx->h_layout_off.data(), ctx->layout_off.p, (n + 1) * sizeof(uint64_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->batch_read = true;
    return CJ_OK;
}

cj_status doc_verdict(const cj_context* ctx, size_t i)
{
    if (ctx->h_ctrl->error_flags & CJ_FLAG_TIMEOUT) return CJ_ERR_TIMEOUT;
    if (ctx->h_ctrl->error_flags & CJ_FLAG_OVERFLOW) return CJ_ERR_CUDA;   // inconsistent scan counts
    const uint32_t e = ctx->h_seg_err[i];
    if (e & CJ_FLAG_UTF8) return CJ_ERR_INVALID_UTF8;
    if (e & CJ_FLAG_BRACKETS) return CJ_ERR_INVALID_BRACKETS;
    return CJ_OK;
}

cj_status finish(cj_status st) { g_last_status = st; return st; }

}  // namespace

extern "C" {

cj_status cj_context_create(int device, cj_context** out)
{
    if (!out) return CJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return CJ_ERR_NO_DEVICE;
    if (device < 0) CJ_CUDA(cudaGetDevice(&device));
    if (device >= n) return CJ_ERR_INVALID_ARGUMENT;
    CJ_CUDA(cudaSetDevice(device));
    cj_context* ctx = new cj_context();
    ctx->device = device;
    if (cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        ctx->sm_count < 1) {
        delete ctx;
        return CJ_ERR_CUDA;
    }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_reset, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_copied, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_plan, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_d2h, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void**)&ctx->d_ready, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc((void**)&ctx->d_ctrl, sizeof(Ctrl)) != cudaSuccess) {
        cj_context_destroy(ctx);
        return CJ_ERR_CUDA;
    }
    {
        // every kernel an overlapped run launches behind a waiting scan
        cudaFuncAttributes a;
        if (preload_scan_kernels() != cudaSuccess || preload_pair_kernels() != cudaSuccess ||
            preload_batch_kernels() != cudaSuccess || preload_value_kernels() != cudaSuccess ||
            cudaFuncGetAttributes(&a, (const void*)mark_ready) != cudaSuccess) {
            cj_context_destroy(ctx);
            return CJ_ERR_CUDA;
        }
    }
    {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue64", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess && fn) {
            auto w = reinterpret_cast<CUresult (*)(CUstream, CUdeviceptr, cuuint64_t, unsigned int)>(fn);
            if (w((CUstream)ctx->copy_stream, (CUdeviceptr)ctx->d_ready, 0, CU_STREAM_WRITE_VALUE_DEFAULT) ==
                    CUDA_SUCCESS &&
                cudaStreamSynchronize(ctx->copy_stream) == cudaSuccess)
                ctx->write64 = w;
        }
        cudaGetLastError();
    }
    *out = ctx;
    return CJ_OK;
}

void cj_context_destroy(cj_context* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    release(ctx->in); release(ctx->pos); release(ctx->pair); release(ctx->brk);
    release(ctx->rtab); release(ctx->bagg); release(ctx->work); release(ctx->masks);
    release(ctx->segs); release(ctx->seg_out); release(ctx->region_seg);
    release(ctx->spine); release(ctx->cinfo); release(ctx->tree);
    release(ctx->seg_err); release(ctx->seg_depth); release(ctx->rchunk_off);
    release(ctx->layout_off); release(ctx->layout); release(ctx->pack); release(ctx->pack_off);
    release(ctx->q_count); release(ctx->q_out);
    release(ctx->val_type); release(ctx->val_str); release(ctx->val_num); release(ctx->val_len);
    release(ctx->val_long); release(ctx->val_counts); release(ctx->pow5);
    release(ctx->plan_counts); release(ctx->plan_req); release(ctx->plan_pos); release(ctx->plan_bounds);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->d_ready) cudaFree(ctx->d_ready);
    if (ctx->ev_reset) cudaEventDestroy(ctx->ev_reset);
    if (ctx->ev_copied) cudaEventDestroy(ctx->ev_copied);
    if (ctx->ev_plan) cudaEventDestroy(ctx->ev_plan);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->d2h_stream) {
        cudaStreamSynchronize(ctx->d2h_stream);
        cudaStreamDestroy(ctx->d2h_stream);
    }
    if (ctx->ev_d2h) cudaEventDestroy(ctx->ev_d2h);
    for (cudaEvent_t e : ctx->wave_ev) cudaEventDestroy(e);
    release(ctx->wave_carry); release(ctx->wave_nwork);
    if (ctx->h_wave) cudaFreeHost(ctx->h_wave);
    if (ctx->d_ctrl) cudaFree(ctx->d_ctrl);
    if (ctx->h_ctrl) cudaFreeHost(ctx->h_ctrl);
    if (ctx->h_seg_out) cudaFreeHost(ctx->h_seg_out);
    for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

cj_status cj_context_set_dependent_launch(cj_context* ctx, int enable)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    ctx->dependent_launch = enable != 0;
    ctx->graph_valid = false;           // a captured graph holds the old launches
    return CJ_OK;
}

cj_status cj_context_timing(cj_context* ctx, int enable)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    ctx->timing = enable < 0 ? 0 : (enable > 3 ? 1 : enable);
    ctx->events_used = 0;
    return CJ_OK;
}

cj_status cj_context_phase_ms(cj_context* ctx, double* scan_ms, double* pair_ms, double* spine_ms,
                              int64_t* runs)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    double a = 0, b = 0, c = 0;
    for (size_t i = 0; i + kEventsPerRun <= ctx->events_used; i += kEventsPerRun) {
        float x = 0, y = 0, z = 0;
        CJ_CUDA(cudaEventElapsedTime(&x, ctx->events[i], ctx->events[i + 3]));
        CJ_CUDA(cudaEventElapsedTime(&y, ctx->events[i + 3], ctx->events[i + 4]));
        CJ_CUDA(cudaEventElapsedTime(&z, ctx->events[i + 4], ctx->events[i + 5]));
        a += x; b += y; c += z;
    }
    if (scan_ms) *scan_ms = a;
    if (pair_ms) *pair_ms = b;
    if (spine_ms) *spine_ms = c;
    if (runs) *runs = (int64_t)(ctx->events_used / kEventsPerRun);
    return CJ_OK;
}

cj_status cj_context_scan_phase_ms(cj_context* ctx, double* tables_ms, double* prefix_ms, double* emit_ms,
                                   int64_t* runs)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    double a = 0, b = 0, c = 0;
    for (size_t i = 0; i + kEventsPerRun <= ctx->events_used; i += kEventsPerRun) {
        float x = 0, y = 0, z = 0;
        CJ_CUDA(cudaEventElapsedTime(&x, ctx->events[i], ctx->events[i + 1]));
        CJ_CUDA(cudaEventElapsedTime(&y, ctx->events[i + 1], ctx->events[i + 2]));
        CJ_CUDA(cudaEventElapsedTime(&z, ctx->events[i + 2], ctx->events[i + 3]));
        a += x; b += y; c += z;
    }
    if (tables_ms) *tables_ms = a;
    if (prefix_ms) *prefix_ms = b;
    if (emit_ms) *emit_ms = c;
    if (runs) *runs = (int64_t)(ctx->events_used / kEventsPerRun);
    return CJ_OK;
}

cj_status cj_context_span_ms(cj_context* ctx, double* ms)
{
    if (!ctx || !ms) return CJ_ERR_INVALID_ARGUMENT;
    *ms = 0;
    if (ctx->events_used < kEventsPerRun) return CJ_OK;
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    float x = 0;
    CJ_CUDA(cudaEventElapsedTime(&x, ctx->events[0], ctx->events[ctx->events_used - 1]));
    *ms = x;
    return CJ_OK;
}

void* cj_host_alloc(size_t bytes) { return pinned_alloc(bytes); }
void cj_host_free(void* p) { pinned_free(p); }
size_t cj_host_pool_trim(void) { return pinned_trim(); }

cj_status cj_context_reserve(cj_context* ctx, size_t max_bytes, size_t max_segments)
{
    if (!ctx || max_segments == 0) return CJ_ERR_INVALID_ARGUMENT;
    if (max_bytes > CJ_MAX_INPUT_BYTES) return CJ_ERR_TOO_LARGE;
    CJ_CUDA(cudaSetDevice(ctx->device));
    return reserve(ctx, max_bytes, max_segments);
}

void* cj_context_stream(cj_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
int64_t cj_context_launch_count(cj_context* ctx) { return ctx ? ctx->launches : 0; }
size_t cj_context_device_bytes(cj_context* ctx) { return ctx ? ctx->dev_bytes : 0; }
size_t cj_context_staged_bytes(cj_context* ctx) { return (ctx && ctx->staged) ? ctx->n_bytes : 0; }

cj_context* cj_default_context(void)
{
    static std::mutex mu;
    static cj_context* ctx = nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!ctx) {
        if (cj_context_create(-1, &ctx) != CJ_OK) ctx = nullptr;
    }
    return ctx;
}

cj_status cj_parse_standard(cj_context* ctx, const uint8_t* data, size_t size, cj_result* out)
{
    if (out) memset(out, 0, sizeof(*out));
    if (!ctx || !out || !data || size == 0) return finish(CJ_ERR_INVALID_ARGUMENT);
    const uint8_t* chunks[1] = {data};
    size_t sizes[1] = {size};
    cj_status st = stage_run(ctx, chunks, sizes, 1, false);
    cj_parse_info info;
    if (!st) st = read_info(ctx, &info);
    if (!st && info.status != CJ_OK) st = (cj_status)info.status;
    if (!st) st = to_result(ctx, info, out);
    out->status = st;
    return finish(st);
}

cj_status cj_parse_lines(cj_context* ctx, const uint8_t* const* chunks, const size_t* chunk_sizes,
                         size_t n_chunks, cj_result* out)
{
    if (out) memset(out, 0, sizeof(*out));
    if (!ctx || !out) return finish(CJ_ERR_INVALID_ARGUMENT);
    cj_status st = stage_run(ctx, chunks, chunk_sizes, n_chunks, true);
    cj_parse_info info;
    if (!st) st = read_info(ctx, &info);
    if (!st && info.status != CJ_OK) st = (cj_status)info.status;
    if (!st) st = to_result(ctx, info, out);
    out->status = st;
    return finish(st);
}

cj_status cj_parse_lines_planned(cj_context* ctx, const uint8_t* host_data, size_t size, size_t chunk_count,
                                 size_t chunk_bytes, cj_result* out)
{
    if (out) memset(out, 0, sizeof(*out));
    if (!ctx || !out) return finish(CJ_ERR_INVALID_ARGUMENT);
    std::vector<size_t> sizes;
    cj_status st = stage_lines_planned(ctx, host_data, size, chunk_count, chunk_bytes, sizes);
    if (!st) st = run(ctx);
    cj_parse_info info;
    if (!st) st = read_info(ctx, &info);
    if (!st && info.status != CJ_OK) st = (cj_status)info.status;
    if (!st) st = to_result(ctx, info, out);
    out->status = st;
    return finish(st);
}

void cj_result_free(cj_result* res)
{
    if (!res) return;
    if (res->structural) pinned_free(res->structural);
    free(res->segment_sizes);
    memset(res, 0, sizeof(*res));
}

cj_status cj_parse_into(cj_context* ctx, const uint8_t* data, size_t size, int lines_mode,
                        int32_t* host_out, size_t out_cap, cj_parse_info* info)
{
    if (!ctx || !data || size == 0 || !host_out) return finish(CJ_ERR_INVALID_ARGUMENT);
    const uint8_t* chunks[1] = {data};
    size_t sizes[1] = {size};
    // streamed when the input makes at least two waves
    const uint64_t wb = stream_wave_bytes(ctx);
    if (wb && size >= 2 * wb && size >= kOverlapMin && size <= CJ_MAX_INPUT_BYTES && is_pinned(data) &&
        is_pinned(host_out))
        return finish(parse_streamed(ctx, chunks, sizes, 1, lines_mode != 0, host_out, out_cap, info));
    cj_status st = stage_run(ctx, chunks, sizes, 1, lines_mode != 0);
    cj_parse_info local;
    if (!info) info = &local;
    if (!st) st = read_info(ctx, info);
    if (!st && info->status != CJ_OK) st = (cj_status)info->status;
    if (!st) st = copy_result(ctx, info->n_structural, host_out, out_cap);
    return finish(st);
}

cj_status cj_stage_standard(cj_context* ctx, const uint8_t* data, size_t size)
{
    if (!ctx || !data || size == 0) return CJ_ERR_INVALID_ARGUMENT;
    const uint8_t* chunks[1] = {data};
    size_t sizes[1] = {size};
    return stage(ctx, chunks, sizes, 1, false);
}

cj_status cj_stage_lines(cj_context* ctx, const uint8_t* const* chunks, const size_t* chunk_sizes,
                         size_t n_chunks)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    return stage(ctx, chunks, chunk_sizes, n_chunks, true);
}

cj_status cj_run_staged(cj_context* ctx)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    return run(ctx);
}

cj_status cj_staged_info(cj_context* ctx, cj_parse_info* info)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    return read_info(ctx, info);
}

cj_status cj_copy_staged_result(cj_context* ctx, int32_t* host_out, size_t out_cap)
{
    if (!ctx || !host_out) return CJ_ERR_INVALID_ARGUMENT;
    cj_parse_info info;
    cj_status st = read_info(ctx, &info);
    if (st) return st;
    return copy_result(ctx, info.n_structural, host_out, out_cap);
}

cj_status cj_staged_device_outputs(cj_context* ctx, const int32_t** d_positions,
                                   const int32_t** d_pair_row)
{
    if (!ctx || !ctx->staged) return CJ_ERR_NOT_STAGED;
    if (d_positions) *d_positions = ctx->pos.p;
    if (d_pair_row) *d_pair_row = ctx->pair.p;
    return CJ_OK;
}

cj_status cj_stage_batch(cj_context* ctx, const uint8_t* const* docs, const size_t* sizes, size_t n_docs,
                         int lines_mode)
{
    if (!ctx || !docs) return finish(CJ_ERR_INVALID_ARGUMENT);
    return finish(stage_batch(ctx, docs, nullptr, sizes, n_docs, lines_mode != 0));
}

cj_status cj_stage_batch_packed(cj_context* ctx, const uint8_t* packed, const size_t* sizes, size_t n_docs,
                                int lines_mode)
{
    if (!ctx || !packed) return finish(CJ_ERR_INVALID_ARGUMENT);
    return finish(stage_batch(ctx, nullptr, packed, sizes, n_docs, lines_mode != 0));
}

cj_status cj_batch_padded_offsets(const size_t* sizes, size_t n_docs, size_t* offsets, size_t* total)
{
    if (!sizes || !total || (n_docs && !offsets)) return CJ_ERR_INVALID_ARGUMENT;
    size_t o = 0;
    for (size_t i = 0; i < n_docs; i++) {
        offsets[i] = o;
        o += round_up(sizes[i], kPadBytes);
    }
    *total = o;
    return CJ_OK;
}

cj_status cj_parse_batch_padded(cj_context* ctx, const uint8_t* padded, const size_t* sizes, size_t n_docs,
                                int lines_mode)
{
    if (!ctx) return finish(CJ_ERR_INVALID_ARGUMENT);
    return finish(parse_batch_padded(ctx, padded, sizes, n_docs, lines_mode != 0));
}

cj_status cj_batch_info(cj_context* ctx, int32_t* status, int64_t* n_structural, int32_t* max_depth,
                        int64_t* layout_offsets, size_t n_docs)
{
    if (!ctx) return finish(CJ_ERR_INVALID_ARGUMENT);
    cj_status st = read_batch(ctx);
    if (st) return finish(st);
    if (n_docs != ctx->n_segs) return finish(CJ_ERR_INVALID_ARGUMENT);
    for (size_t i = 0; i < n_docs; i++) {
        if (status) status[i] = doc_verdict(ctx, i);
        if (n_structural) n_structural[i] = std::min<int64_t>(ctx->h_bseg_out[i].s_end, ctx->h_segs[i].len);
        if (max_depth) max_depth[i] = ctx->h_seg_depth[i];
    }
    if (layout_offsets)
        for (size_t i = 0; i <= n_docs; i++) layout_offsets[i] = (int64_t)ctx->h_layout_off[i];
    return finish(CJ_OK);
}

cj_status cj_copy_batch_result(cj_context* ctx, int32_t* host_out, size_t out_cap)
{
    if (!ctx || !host_out) return finish(CJ_ERR_INVALID_ARGUMENT);
    cj_status st = read_batch(ctx);
    if (st) return finish(st);
    const uint64_t total = ctx->h_layout_off[ctx->n_segs];
    if (total > out_cap) return finish(CJ_ERR_CAPACITY);
    if (cudaMemcpyAsync(host_out, ctx->layout.p, total * sizeof(int32_t), cudaMemcpyDeviceToHost,
                        ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return finish(CJ_ERR_CUDA);
    return finish(CJ_OK);
}

cj_status cj_run_staged_graph(cj_context* ctx)
{
    if (!ctx) return finish(CJ_ERR_INVALID_ARGUMENT);
    return finish(run_graph(ctx));
}

cj_status cj_context_set_tuning(cj_context* ctx, const cj_tuning* t)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    const int rk = t ? std::max(0, t->region_kib) : 0;
    const int sw = t ? std::max(-1, t->stream_wave_mib) : 0;
    const int tb = t ? std::max(0, t->scan_blocks_per_sm) : 0;
    const int eb = t ? std::max(0, t->emit_blocks_per_sm) : 0;
    const uint32_t pb = t ? (uint32_t)std::max(0, t->pair_blocks) : 0u;
    const uint32_t pt = t ? (uint32_t)std::max(0, t->pair_threads) : 0u;
    const uint32_t pf = t ? (uint32_t)std::max(0, t->prefetch_steps) : 0u;
    if (pt && pt != 64 && pt != 128 && pt != 256) return CJ_ERR_INVALID_ARGUMENT;
    if (pf && (pf < 2 || pf > 8)) return CJ_ERR_INVALID_ARGUMENT;
    if (rk && !region_steps_valid(rk)) return CJ_ERR_INVALID_ARGUMENT;
    ctx->tune_region_steps = rk;
    ctx->tune_tables_per_sm = tb;
    ctx->tune_emit_per_sm = eb;
    ctx->tune_pair_blocks = pb;
    ctx->tune_pair_threads = pt;
    ctx->tune_prefetch_steps = pf;
    ctx->tune_stream_wave_mib = sw;
    ctx->graph_valid = false;
    if (ctx->staged && ctx->run_region_steps != region_steps(ctx)) {
        // the staged input is cut into regions of the new size
        CJ_CUDA(cudaSetDevice(ctx->device));
        cj_status st = place_regions(ctx);
        if (st) { ctx->staged = false; return st; }
        CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return CJ_OK;
}

cj_status cj_context_get_tuning(cj_context* ctx, cj_tuning* t)
{
    if (!ctx || !t) return CJ_ERR_INVALID_ARGUMENT;
    t->region_kib = region_steps(ctx) * kStepBytes / 1024;
    t->scan_blocks_per_sm = ctx->tune_tables_per_sm;
    t->emit_blocks_per_sm = ctx->tune_emit_per_sm;
    t->pair_blocks = (int32_t)ctx->tune_pair_blocks;
    t->pair_threads = (int32_t)pair_threads(ctx);
    t->prefetch_steps = ctx->tune_prefetch_steps ? (int32_t)ctx->tune_prefetch_steps : 4;
    t->stream_wave_mib = ctx->tune_stream_wave_mib;
    t->ms = 0.f;
    return CJ_OK;
}

cj_status cj_autotune_staged(cj_context* ctx, int32_t reps, cj_tuning* best, cj_tuning* tried,
                             size_t tried_cap, size_t* n_tried)
{
    if (!ctx || reps < 1) return finish(CJ_ERR_INVALID_ARGUMENT);
    if (!ctx->staged) return finish(CJ_ERR_NOT_STAGED);
    CJ_CUDA(cudaSetDevice(ctx->device));
    const uint32_t sm = (uint32_t)ctx->sm_count;
    // region size (4, 8, 16 KiB) x L2 prefetch distance (2, 4, 8 steps) x
    // resident scan blocks per SM (as many as fit, or 2) x pairing threads
    // per block x pairing blocks
    std::vector<cj_tuning> cand;
    for (int rk : {4, 8, 16})
        for (int pf : {2, 4, 8})
            for (int tb : {0, 2})
                for (int pt : {128, 256})
                    for (uint32_t pb : {0u, sm * 4}) {
                        cj_tuning t;
                        t.region_kib = rk;
                        t.prefetch_steps = pf;
                        t.scan_blocks_per_sm = tb;
                        t.emit_blocks_per_sm = tb;
                        t.pair_threads = pt;
                        t.pair_blocks = (int32_t)pb;
                        t.stream_wave_mib = ctx->tune_stream_wave_mib;
                        t.ms = 0.f;
                        cand.push_back(t);
                    }
    cudaEvent_t e0, e1;
    CJ_CUDA(cudaEventCreate(&e0));
    CJ_CUDA(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    cj_tuning win = cand[0];
    size_t k = 0;
    for (cj_tuning& t : cand) {
        cj_status st = cj_context_set_tuning(ctx, &t);
        if (!st) st = run_graph(ctx);   // capture + one untimed replay
        if (st) { cudaEventDestroy(e0); cudaEventDestroy(e1); return finish(st); }
        if (cudaEventRecord(e0, ctx->stream) != cudaSuccess) return finish(CJ_ERR_CUDA);
        for (int r = 0; r < reps; r++)
            if ((st = run_graph(ctx))) { cudaEventDestroy(e0); cudaEventDestroy(e1); return finish(st); }
        if (cudaEventRecord(e1, ctx->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
            return finish(CJ_ERR_CUDA);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        t.ms = ms / (float)reps;
        if (tried && k < tried_cap) tried[k] = t;
        k++;
        if (t.ms < best_ms) { best_ms = t.ms; win = t; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (n_tried) *n_tried = k;
    cj_status st = cj_context_set_tuning(ctx, &win);
    if (st) return finish(st);
    if (best) *best = win;
    return finish(CJ_OK);
}

namespace {

const char* kTuningKeys[] = {"region_kib", "scan_blocks_per_sm", "emit_blocks_per_sm", "pair_blocks",
                             "pair_threads", "prefetch_steps", "stream_wave_mib"};

int32_t* tuning_field(cj_tuning& t, int i)
{
    int32_t* f[] = {&t.region_kib, &t.scan_blocks_per_sm, &t.emit_blocks_per_sm, &t.pair_blocks,
                    &t.pair_threads, &t.prefetch_steps, &t.stream_wave_mib};
    return f[i];
}

std::string gpu_name(int device)
{
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        cudaGetLastError();
        return "unknown";
    }
    std::string n = prop.name;
    for (char& c : n)
        if (c == '"' || c == '\\' || c == '\n') c = ' ';
    return n;
}

// the lines of a tuning file, without the one for `gpu`
std::vector<std::string> tuning_lines_except(const char* path, const std::string& gpu, std::string* mine)
{
    std::vector<std::string> keep;
    FILE* f = fopen(path, "r");
    if (!f) return keep;
    const std::string key = "{\"gpu\": \"" + gpu + "\"";
    char buf[1024];
    while (fgets(buf, sizeof buf, f)) {
        std::string line(buf);
        while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
        if (line.empty()) continue;
        if (line.compare(0, key.size(), key) == 0) {
            if (mine) *mine = line;
        } else {
            keep.push_back(line);
        }
    }
    fclose(f);
    return keep;
}

}  // namespace

cj_status cj_tuning_save(cj_context* ctx, const char* path)
{
    if (!ctx || !path) return CJ_ERR_INVALID_ARGUMENT;
    cj_tuning t;
    cj_context_get_tuning(ctx, &t);
    const std::string gpu = gpu_name(ctx->device);
    std::vector<std::string> lines = tuning_lines_except(path, gpu, nullptr);
    std::string mine = "{\"gpu\": \"" + gpu + "\"";
    for (int i = 0; i < 7; i++) mine += std::string(", \"") + kTuningKeys[i] + "\": " + std::to_string(*tuning_field(t, i));
    mine += "}";
    lines.push_back(mine);
    FILE* f = fopen(path, "w");
    if (!f) return CJ_ERR_INVALID_ARGUMENT;
    for (const std::string& l : lines) fprintf(f, "%s\n", l.c_str());
    return fclose(f) == 0 ? CJ_OK : CJ_ERR_INVALID_ARGUMENT;
}

cj_status cj_tuning_load(cj_context* ctx, const char* path)
{
    if (!ctx || !path) return CJ_ERR_INVALID_ARGUMENT;
    std::string mine;
    tuning_lines_except(path, gpu_name(ctx->device), &mine);
    if (mine.empty()) return CJ_ERR_INVALID_ARGUMENT;      // no entry for this GPU
    cj_tuning t;
    memset(&t, 0, sizeof t);
    for (int i = 0; i < 7; i++) {
        const std::string k = std::string("\"") + kTuningKeys[i] + "\": ";
        const size_t at = mine.find(k);
        if (at == std::string::npos) return CJ_ERR_INVALID_ARGUMENT;
        *tuning_field(t, i) = (int32_t)strtol(mine.c_str() + at + k.size(), nullptr, 10);
    }
    return cj_context_set_tuning(ctx, &t);
}

static_assert(CJ_VAL_NONE == kValNone && CJ_VAL_STRING == kValString && CJ_VAL_INT == kValInt &&
                  CJ_VAL_DOUBLE == kValDouble && CJ_VAL_TRUE == kValTrue && CJ_VAL_FALSE == kValFalse &&
                  CJ_VAL_NULL == kValNull && CJ_VAL_INVALID == kValInvalid &&
                  CJ_VAL_TYPES == kValTypes,
              "value types of the C ABI and the kernels");

cj_status cj_decode_values(cj_context* ctx, cj_value_counts* counts)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    if (!ctx->staged || ctx->batch) return CJ_ERR_NOT_STAGED;
    cj_parse_info info;
    cj_status st = read_info(ctx, &info);
    if (st) return st;
    if (info.status != CJ_OK) return (cj_status)info.status;
    CJ_CUDA(cudaSetDevice(ctx->device));
    const uint64_t S = (uint64_t)info.n_structural, slots = S + 1;
    if ((st = ensure(ctx, ctx->val_type, slots + 4))) return st;     // read a word at a time
    if ((st = ensure(ctx, ctx->val_num, slots))) return st;
    if ((st = ensure(ctx, ctx->val_len, slots))) return st;
    if ((st = ensure(ctx, ctx->val_str, ctx->n_bytes + 1))) return st;
    // the lists of the second kernel, then their counters: slots longer than
    // 256 bytes (at most n / 257 of them), and escaped strings and numbers
    // for the exact conversion (those past n / 64 are decoded in place)
    const uint64_t long_cap = std::min<uint64_t>(ctx->n_bytes / 256 + 1, 0xFFFFFFFFull);
    const uint64_t short_cap = std::min<uint64_t>(ctx->n_bytes / 64 + 1, 0xFFFFFFFFull);
    if ((st = ensure(ctx, ctx->val_long, long_cap + short_cap + 3))) return st;
    if ((st = ensure(ctx, ctx->val_counts, kValTypes))) return st;
    if (!ctx->pow5.p) {
        if ((st = ensure(ctx, ctx->pow5, 2 * 651))) return st;
        CJ_CUDA(cudaMemcpy(ctx->pow5.p, kPow5Table, sizeof(kPow5Table), cudaMemcpyHostToDevice));
    }
    ValueParams vp{};
    vp.dependent_launch = ctx->dependent_launch ? 1u : 0u;
    vp.in = ctx->in.p;
    vp.segs = ctx->segs.p;
    vp.n_segs = ctx->n_segs;
    vp.pos = ctx->pos.p;
    vp.S = (uint32_t)S;
    vp.n_bytes = ctx->n_bytes;
    vp.type = ctx->val_type.p;
    vp.num = ctx->val_num.p;
    vp.len = ctx->val_len.p;
    vp.str_out = ctx->val_str.p;
    vp.long_list = ctx->val_long.p;
    vp.long_cap = (uint32_t)long_cap;
    vp.short_list = ctx->val_long.p + long_cap;
    vp.short_cap = (uint32_t)short_cap;
    vp.counters = ctx->val_long.p + long_cap + short_cap;
    vp.counts = ctx->val_counts.p;
    vp.pow5 = ctx->pow5.p;
    CJ_CUDA(cudaMemsetAsync(vp.counters, 0, 3 * sizeof(uint32_t), ctx->stream));
    CJ_CUDA(cudaMemsetAsync(ctx->val_counts.p, 0, kValTypes * sizeof(unsigned long long), ctx->stream));
    if (launch_decode_values(vp, ctx->sm_count, ctx->stream) != cudaSuccess) return CJ_ERR_CUDA;
    ctx->launches += 4;
    ctx->val_slots = slots;
    if (counts) {
        unsigned long long c[kValTypes];
        CJ_CUDA(cudaMemcpyAsync(c, ctx->val_counts.p, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
        CJ_CUDA(cudaStreamSynchronize(ctx->stream));
        counts->n_slots = (int64_t)slots;
        for (int k = 0; k < kValTypes; k++) counts->by_type[k] = (int64_t)c[k];
    }
    return CJ_OK;
}

cj_status cj_values_device(cj_context* ctx, const uint8_t** type, const uint64_t** num, const uint32_t** len,
                           const uint8_t** strings)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    if (!ctx->val_slots) return CJ_ERR_NOT_STAGED;
    if (type) *type = ctx->val_type.p;
    if (num) *num = ctx->val_num.p;
    if (len) *len = ctx->val_len.p;
    if (strings) *strings = ctx->val_str.p;
    return CJ_OK;
}

cj_status cj_copy_values(cj_context* ctx, uint8_t* type, uint64_t* num, uint32_t* len, size_t slot_cap,
                         uint8_t* strings, size_t string_cap)
{
    if (!ctx) return CJ_ERR_INVALID_ARGUMENT;
    if (!ctx->val_slots) return CJ_ERR_NOT_STAGED;
    if ((type || num || len) && slot_cap < ctx->val_slots) return CJ_ERR_CAPACITY;
    if (strings && string_cap < ctx->n_bytes) return CJ_ERR_CAPACITY;
    CJ_CUDA(cudaSetDevice(ctx->device));
    const size_t n = ctx->val_slots;
    if (type) CJ_CUDA(cudaMemcpyAsync(type, ctx->val_type.p, n, cudaMemcpyDeviceToHost, ctx->stream));
    if (num) CJ_CUDA(cudaMemcpyAsync(num, ctx->val_num.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (len) CJ_CUDA(cudaMemcpyAsync(len, ctx->val_len.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (strings && ctx->n_bytes)
        CJ_CUDA(cudaMemcpyAsync(strings, ctx->val_str.p, ctx->n_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    return CJ_OK;
}

cj_status cj_run_staged_starved(cj_context* ctx, uint32_t polls, cj_parse_info* info)
{
    if (!ctx || polls == 0) return finish(CJ_ERR_INVALID_ARGUMENT);
    if (!ctx->staged || ctx->batch) return finish(CJ_ERR_NOT_STAGED);
    if (cudaSetDevice(ctx->device) != cudaSuccess ||
        cudaMemsetAsync(ctx->d_ready, 0, sizeof(unsigned long long), ctx->stream) != cudaSuccess)
        return finish(CJ_ERR_CUDA);
    ctx->overlap_run = true;
    ctx->input_wait_limit = polls;
    cj_status st = enqueue(ctx, false);
    ctx->overlap_run = false;
    ctx->input_wait_limit = 0;
    cj_parse_info local;
    if (!info) info = &local;
    if (!st) st = read_info(ctx, info);
    if (!st) st = (cj_status)info->status;
    return finish(st);
}

namespace {

cj_status run_query(cj_context* ctx, const char* key, size_t key_len, const char* value, long value_len,
                    int64_t* out, size_t cap, int64_t* n)
{
    if (!ctx || !key || !n || (value_len > 0 && !value)) return CJ_ERR_INVALID_ARGUMENT;
    if (key_len > 256 || value_len > 256) return CJ_ERR_INVALID_ARGUMENT;
    if (!ctx->staged || ctx->batch || !ctx->lines) return CJ_ERR_NOT_STAGED;
    cj_parse_info info;
    cj_status st = read_info(ctx, &info);       // the staged run has finished
    if (st) return st;
    if (info.status != CJ_OK) return (cj_status)info.status;
    if ((st = ensure(ctx, ctx->q_count, 3))) return st;
    if (out && cap && (st = ensure(ctx, ctx->q_out, 3 * cap))) return st;
    CJ_CUDA(cudaMemsetAsync(ctx->q_count.p, 0, 3 * sizeof(unsigned long long), ctx->stream));
    if (info.n_structural > 0) {
        CJ_CUDA(launch_query(ctx->in.p, ctx->segs.p, ctx->n_segs, ctx->pos.p, ctx->pair.p, ctx->brk.p,
                             (uint32_t)info.n_structural, (uint32_t)info.n_brackets, key, (int)key_len, value,
                             (int)value_len, (int64_t)ctx->n_bytes, ctx->q_count.p,
                             (out && cap) ? ctx->q_out.p : nullptr, (out && cap) ? cap : 0, ctx->sm_count,
                             ctx->stream));
        ctx->launches += 1;
    }
    unsigned long long cnt[2] = {0, 0};
    CJ_CUDA(cudaMemcpyAsync(cnt, ctx->q_count.p, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    CJ_CUDA(cudaStreamSynchronize(ctx->stream));
    if (cnt[1]) return CJ_ERR_INVALID_BRACKETS;       // a malformed result (not reached for a valid one)
    *n = (int64_t)cnt[0];
    const unsigned long long m_all = cnt[0];
    if (out && cap) {
        const size_t m = std::min<size_t>(cap, (size_t)m_all);
        CJ_CUDA(cudaMemcpyAsync(out, ctx->q_out.p, 3 * m * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
        CJ_CUDA(cudaStreamSynchronize(ctx->stream));
        // records in document order
        std::vector<size_t> idx(m);
        for (size_t i = 0; i < m; i++) idx[i] = i;
        std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return out[3 * a] < out[3 * b]; });
        std::vector<int64_t> tmp(3 * m);
        for (size_t i = 0; i < m; i++)
            for (int k = 0; k < 3; k++) tmp[3 * i + k] = out[3 * idx[i] + k];
        std::copy(tmp.begin(), tmp.end(), out);
        if (m_all > cap) return CJ_ERR_CAPACITY;
    }
    return CJ_OK;
}

}  // namespace

cj_status cj_query_count(cj_context* ctx, const char* key, size_t key_len, const char* value,
                         size_t value_len, int64_t* count)
{
    return finish(run_query(ctx, key, key_len, value ? value : "", (long)value_len, nullptr, 0, count));
}

cj_status cj_query_values(cj_context* ctx, const char* key, size_t key_len, int64_t* out, size_t cap,
                          int64_t* n_records)
{
    return finish(run_query(ctx, key, key_len, nullptr, -1, out, cap, n_records));
}

const char* cj_status_string(int status)
{
    switch (status) {
    case CJ_OK: return "ok";
    case CJ_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CJ_ERR_INVALID_UTF8: return "invalid UTF-8";
    case CJ_ERR_INVALID_BRACKETS: return "unbalanced or mismatched brackets";
    case CJ_ERR_TOO_LARGE: return "input larger than int32 positions allow";
    case CJ_ERR_OUT_OF_MEMORY: return "out of device memory";
    case CJ_ERR_CUDA: return "CUDA runtime error";
    case CJ_ERR_TIMEOUT: return "bounded device wait expired";
    case CJ_ERR_NO_DEVICE: return "no CUDA device";
    case CJ_ERR_CAPACITY: return "output buffer too small";
    case CJ_ERR_NOT_STAGED: return "no staged input";
    default: return "unknown status";
    }
}

int cj_last_status(void) { return g_last_status; }
void cj_set_last_status(int status) { g_last_status = status; }
const char* cj_last_error(void) { return cj_status_string(g_last_status); }

cj_status cj_plan_lines_bytes_device(cj_context* ctx, const uint8_t* d_data, size_t size, size_t chunk_bytes,
                                     size_t* chunk_sizes, size_t cap, size_t* n_chunks, void* stream)
{
    if (!ctx || !n_chunks || (!d_data && size)) return CJ_ERR_INVALID_ARGUMENT;
    CJ_CUDA(cudaSetDevice(ctx->device));
    *n_chunks = 0;
    if (size == 0) return CJ_OK;
    CJ_CUDA(cudaEventRecord(ctx->ev_plan, (cudaStream_t)stream));
    CJ_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_plan, 0));
    const size_t keep = chunk_sizes ? cap : 0;            // boundaries kept on the device
    cj_status st;
    if ((st = ensure(ctx, ctx->plan_bounds, keep + 2))) return st;
    if (plan_lines_bytes_device(d_data, size, chunk_bytes, chunk_sizes, keep, n_chunks, ctx->plan_bounds.p + 2,
                                ctx->plan_bounds.p, ctx->stream) != cudaSuccess)
        return CJ_ERR_CUDA;
    if (chunk_sizes && *n_chunks > cap) return CJ_ERR_CAPACITY;
    return CJ_OK;
}

cj_status cj_plan_lines_count_device(cj_context* ctx, const uint8_t* d_data, size_t size, size_t chunk_count,
                                     size_t* chunk_sizes, void* stream)
{
    if (!ctx || chunk_count == 0 || !chunk_sizes || (!d_data && size)) return CJ_ERR_INVALID_ARGUMENT;
    CJ_CUDA(cudaSetDevice(ctx->device));
    if (size == 0) {
        for (size_t i = 0; i < chunk_count; i++) chunk_sizes[i] = 0;
        return CJ_OK;
    }
    // the planner runs on the context stream, after the work queued so far on
    // `stream` (the one that fills d_data; NULL: the legacy default stream)
    CJ_CUDA(cudaEventRecord(ctx->ev_plan, (cudaStream_t)stream));
    CJ_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_plan, 0));
    const size_t nb = (size + 65535) / 65536;
    cj_status st;
    if ((st = ensure(ctx, ctx->plan_counts, nb))) return st;
    if ((st = ensure(ctx, ctx->plan_req, chunk_count + 1))) return st;
    if ((st = ensure(ctx, ctx->plan_pos, chunk_count + 1))) return st;
    return plan_lines_count_device(d_data, size, chunk_count, chunk_sizes, ctx->plan_counts.p, ctx->plan_req.p,
                                   ctx->plan_pos.p, ctx->stream) == cudaSuccess ? CJ_OK : CJ_ERR_CUDA;
}

}  // extern "C"
