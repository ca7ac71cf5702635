// cj_emu_driver.cpp -- runs the parse kernels (cujson_gb300/csrc/cj_scan.cu,
// cj_pair.cu, compiled for the CPU with cj_emu.h) the way the library's host
// code does, on one document, one JSON-Lines input in chunks, or a batch of
// independent documents.  TEST INFRASTRUCTURE ONLY: tests/test_emu.py checks
// its results against the oracle.
//
// Every device buffer is allocated so that it ends right before a page that
// may not be touched (mmap + PROT_NONE), so a write or read past the end of any
// buffer the kernels are given stops the process.
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

using namespace cj;

namespace {

struct Guarded {
    void* base = nullptr;
    size_t total = 0;
    ~Guarded() { if (base) munmap(base, total); }
};

std::vector<Guarded*> g_allocs;

// `bytes` of zeroed memory ending at a guard page
template <typename T>
T* galloc(size_t n)
{
    const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    size_t bytes = std::max<size_t>(n * sizeof(T), 1);
    bytes = (bytes + alignof(T) - 1) / alignof(T) * alignof(T);
    const size_t span = (bytes + page - 1) / page * page;
    Guarded* g = new Guarded();
    g->total = span + page;
    g->base = mmap(nullptr, g->total, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (g->base == MAP_FAILED) abort();
    mprotect((char*)g->base + span, page, PROT_NONE);
    g_allocs.push_back(g);
    // 16-byte aligned end: the kernels' vector loads need that alignment
    char* p = (char*)g->base + span - bytes;
    p = (char*)((uintptr_t)p & ~(uintptr_t)15);
    return reinterpret_cast<T*>(p);
}

void free_all()
{
    for (Guarded* g : g_allocs) delete g;
    g_allocs.clear();
}

constexpr size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

// The whole run: segments laid out as the library lays them, scan, pairing.
// `batch`: independent documents (own output and bracket bases, per-document
// verdicts); otherwise one document or JSON-Lines chunks continuing counts.
// `wave_regions` > 0: the scan runs in waves of that many regions, each from
// the previous wave's end value, as a streamed parse runs it.
// `vals` (optional): after a valid parse, the value decoder's outputs too
struct ValOut {
    uint8_t* type;
    uint64_t* num;
    uint32_t* len;
    uint8_t* strings;
    int64_t* counts;
};

int run(const uint8_t* data, const size_t* sizes, size_t n, bool lines, bool batch, int region_steps,
        int32_t* out_pos, int32_t* out_pair, size_t cap, int64_t* out_S, uint32_t* out_flags,
        uint32_t* doc_flags, int64_t* doc_S, uint32_t wave_regions = 0, const ValOut* vals = nullptr)
{
    size_t total = 0, padded = 0;
    for (size_t i = 0; i < n; i++) { total += sizes[i]; padded += round_up(sizes[i], kPadBytes); }
    const uint64_t rb = (uint64_t)region_steps * kStepBytes;
    // device input: each segment at a 1 KiB boundary, exactly as large as the
    // library allocates (padded + 64)
    uint8_t* in = galloc<uint8_t>(padded + 64);
    std::vector<Segment> segs(n);
    std::vector<uint32_t> region_seg;
    uint64_t dev_off = 0, logical = 0, out_base = 0, brk_base = 0;
    uint32_t regions = 0;
    for (size_t i = 0; i < n; i++) {
        Segment& g = segs[i];
        g.dev_off = dev_off;
        g.len = sizes[i];
        g.logical_off = batch ? 0 : logical;
        g.out_base = batch ? out_base : 0;
        g.brk_base = batch ? brk_base : 0;
        g.flags = (!batch && i > 0) ? kSegContinue : 0u;
        g.pad = 0;
        g.first_region = regions;
        g.n_regions = (uint32_t)((sizes[i] + rb - 1) / rb);
        for (uint32_t t = 0; t < g.n_regions; t++) region_seg.push_back((uint32_t)i);
        regions += g.n_regions;
        memcpy(in + dev_off, data + logical, sizes[i]);
        dev_off += round_up(sizes[i], kPadBytes);
        logical += sizes[i];
        out_base += sizes[i] + 1;
        brk_base += round_up(sizes[i], kChunk);
    }
    const size_t s_cap = batch ? out_base : total + 1;
    const size_t b_cap = batch ? brk_base + 1 : total + 1;
    int32_t* pos = galloc<int32_t>(s_cap);
    int32_t* pair = galloc<int32_t>(s_cap);
    uint2* brk = galloc<uint2>(b_cap);
    Segment* d_segs = galloc<Segment>(n);
    std::copy(segs.begin(), segs.end(), d_segs);
    uint32_t* d_region_seg = galloc<uint32_t>(std::max<size_t>(regions, 1));
    std::copy(region_seg.begin(), region_seg.end(), d_region_seg);
    uint4* rtab = galloc<uint4>((size_t)regions * 4);
    uint4* bagg = galloc<uint4>(prefix_blocks(regions) * 4);
    uint4* work = galloc<uint4>((size_t)regions * 2);
    uint4* masks = galloc<uint4>((size_t)regions * region_steps * 32);
    Ctrl* ctrl = galloc<Ctrl>(1);
    SegmentOut* seg_out = galloc<SegmentOut>(n);
    uint32_t* seg_err = batch ? galloc<uint32_t>(n) : nullptr;
    int32_t* seg_depth = batch ? galloc<int32_t>(n) : nullptr;
    const uint64_t chunks = (batch ? brk_base : total) / kChunk + 1;
    uint32_t* spine = galloc<uint32_t>(chunks * kChunk);
    int4* cinfo = galloc<int4>(chunks);
    if (batch) memset(cinfo, 0x7F, chunks * sizeof(int4));
    PairParams pp{};
    {
        size_t off = 0, m = chunks;
        pp.tree_off[0] = 0;
        for (int l = 1; l <= kTreeLevels; l++) { m = (m + 31) / 32; pp.tree_off[l] = off; off += m; }
        pp.tree = galloc<unsigned long long>(off);
    }

    ScanParams sp{};
    sp.in = in;
    sp.segs = d_segs;
    sp.region_seg = n > 1 ? d_region_seg : nullptr;
    sp.n_segs = (uint32_t)n;
    sp.n_regions = regions;
    sp.pos = pos;
    sp.pair = pair;
    sp.brk = brk;
    sp.out_cap = s_cap;
    sp.brk_cap = b_cap;
    sp.rtab = rtab;
    sp.bagg = bagg;
    sp.masks = masks;
    sp.work = work;
    sp.ctrl = ctrl;
    sp.seg_out = seg_out;
    sp.seg_err = seg_err;
    sp.region_steps = region_steps;
    sp.sm_count = 3;
    if (wave_regions) {
        const uint32_t nw = (regions + wave_regions - 1) / wave_regions;
        uint4* carry = galloc<uint4>(nw);
        uint32_t* nwork = galloc<uint32_t>(3 * (size_t)nw);
        for (uint32_t w = 0; w < nw; w++) {
            ScanParams wp = sp;
            wp.r_begin = w * wave_regions;
            wp.r_end = std::min(regions, wp.r_begin + wave_regions);
            wp.carry_in = w ? carry + (w - 1) : nullptr;
            wp.carry_out = carry + w;
            wp.n_work = nwork + 3 * w;
            wp.tickets = nwork + 3 * w + 1;
            wp.work = work + 2 * (size_t)wp.r_begin;
            launch_scan(wp, lines, ScanShape{0, 0}, nullptr);
            // the wave's end value holds the counts through its last region
            if (wp.r_end == regions && !batch && (carry[w].y != ctrl->s_total || carry[w].z != ctrl->k_total))
                ctrl->error_flags |= CJ_FLAG_OVERFLOW;
        }
    } else {
        launch_scan(sp, lines, ScanShape{0, 0}, nullptr);
    }

    uint64_t* rchunk_off = nullptr;
    if (batch) {
        // what batch_prefix computes: record-holding chunks before each document
        rchunk_off = galloc<uint64_t>(n + 1);
        uint64_t acc = 0;
        for (size_t i = 0; i < n; i++) {
            rchunk_off[i] = acc;
            const uint64_t K = std::min<uint64_t>(seg_out[i].k_end, sizes[i]);
            acc += (K + kChunk - 1) / kChunk;
        }
        rchunk_off[n] = acc;
    }
    pp.brk = brk;
    pp.pair = pair;
    pp.spine = spine;
    pp.cinfo = cinfo;
    pp.ctrl = ctrl;
    pp.epoch = 1;
    pp.chunk_cap = (uint32_t)chunks;
    pp.rchunk_off = rchunk_off;
    pp.n_bsegs = batch ? (uint32_t)n : 0u;
    pp.segs = d_segs;
    pp.seg_out = seg_out;
    pp.seg_err = seg_err;
    pp.seg_depth = seg_depth;
    pp.n_chunks = batch ? brk_base / kChunk : 0;
    const int grid = 3;
    launch_pair(pp, grid, nullptr, 128);
    launch_spine(pp, grid, nullptr, 128);

    uint32_t flags = ctrl->error_flags;
    if (ctrl->neg_min_level > 0) flags |= CJ_FLAG_BRACKETS;
    *out_flags = flags;
    if (vals && !batch && flags == 0) {
        const uint64_t S = ctrl->s_total, slots = S + 1;
        ValueParams vp{};
        vp.in = in;
        vp.segs = d_segs;
        vp.n_segs = (uint32_t)n;
        vp.pos = pos;
        vp.S = (uint32_t)S;
        vp.n_bytes = total;
        vp.type = galloc<uint8_t>(slots + 4);
        vp.num = galloc<uint64_t>(slots);
        vp.len = galloc<uint32_t>(slots);
        vp.str_out = galloc<uint8_t>(total + 1);
        const uint64_t long_cap = total / 256 + 1, short_cap = total / 64 + 1;
        vp.long_list = galloc<uint32_t>(long_cap + short_cap + 3);
        vp.long_cap = (uint32_t)long_cap;
        vp.short_list = vp.long_list + long_cap;
        vp.short_cap = (uint32_t)short_cap;
        vp.counters = vp.long_list + long_cap + short_cap;
        vp.counts = galloc<unsigned long long>(kValTypes);
        uint64_t* pow5 = galloc<uint64_t>(2 * 651);
        std::copy(kPow5Table, kPow5Table + 2 * 651, pow5);
        vp.pow5 = pow5;
        launch_decode_values(vp, 3, nullptr);
        std::copy(vp.type, vp.type + slots, vals->type);
        std::copy(vp.num, vp.num + slots, vals->num);
        std::copy(vp.len, vp.len + slots, vals->len);
        std::copy(vp.str_out, vp.str_out + total, vals->strings);
        for (int k = 0; k < kValTypes; k++) vals->counts[k] = (int64_t)vp.counts[k];
    }
    if (batch) {
        // documents back to back in the output arrays
        size_t o = 0;
        for (size_t i = 0; i < n; i++) {
            const uint64_t S = std::min<uint64_t>(seg_out[i].s_end, sizes[i]);
            doc_flags[i] = seg_err[i];
            doc_S[i] = (int64_t)S;
            for (uint64_t k = 0; k < S && o < cap; k++, o++) {
                out_pos[o] = pos[segs[i].out_base + k];
                out_pair[o] = pair[segs[i].out_base + k];
            }
        }
        *out_S = (int64_t)o;
    } else {
        const uint64_t S = ctrl->s_total;
        *out_S = (int64_t)S;
        for (uint64_t k = 0; k < S && k < cap; k++) { out_pos[k] = pos[k]; out_pair[k] = pair[k]; }
        if (doc_S) {
            for (size_t i = 0; i < n; i++) doc_S[i] = seg_out[i].s_end;
        }
    }
    free_all();
    return 0;
}

}  // namespace

extern "C" int cje_parse(const uint8_t* data, const size_t* sizes, size_t n, int lines, int region_steps,
                         int32_t* out_pos, int32_t* out_pair, size_t cap, int64_t* out_S, uint32_t* out_flags,
                         int64_t* seg_S)
{
    return run(data, sizes, n, lines != 0, false, region_steps, out_pos, out_pair, cap, out_S, out_flags,
               nullptr, seg_S);
}

extern "C" int cje_parse_values(const uint8_t* data, const size_t* sizes, size_t n, int lines, int64_t* out_S,
                                uint32_t* out_flags, uint8_t* type, uint64_t* num, uint32_t* len, uint8_t* strings,
                                int64_t* counts, int32_t* scratch_pos, int32_t* scratch_pair, size_t cap)
{
    ValOut v{type, num, len, strings, counts};
    return run(data, sizes, n, lines != 0, false, 4, scratch_pos, scratch_pair, cap, out_S, out_flags, nullptr,
               nullptr, 0, &v);
}

extern "C" int cje_parse_waves(const uint8_t* data, const size_t* sizes, size_t n, int lines, int region_steps,
                               uint32_t wave_regions, int32_t* out_pos, int32_t* out_pair, size_t cap,
                               int64_t* out_S, uint32_t* out_flags)
{
    return run(data, sizes, n, lines != 0, false, region_steps, out_pos, out_pair, cap, out_S, out_flags,
               nullptr, nullptr, wave_regions);
}

extern "C" int cje_parse_batch(const uint8_t* data, const size_t* sizes, size_t n, int region_steps,
                               int32_t* out_pos, int32_t* out_pair, size_t cap, int64_t* out_S,
                               uint32_t* out_flags, uint32_t* doc_flags, int64_t* doc_S)
{
    return run(data, sizes, n, false, true, region_steps, out_pos, out_pair, cap, out_S, out_flags, doc_flags,
               doc_S);
}
