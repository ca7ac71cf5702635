// cj_scan.cu -- the structural scan: UTF-8 validation, tokenization (quote,
// backslash and structural classes, escape carry, in-string mask), structural
// compaction and bracket levels, in three or four launches with no waits between
// thread blocks:
//
//   scan_tables  (one warp per region, regions of 4/8/16 KiB in grid-stride
//                 order) reads the input once: bit-sliced classification,
//                 UTF-8 validation on the same bit planes, escapes and the
//                 in-string mask, and the region's transfer table -- for each
//                 of the 4 entry states (escape pending, inside a string): the
//                 exit state, structural count, bracket count and depth delta.
//   prefix_reduce (256 regions per block, one per thread) composes each
//                 block's tables (only when there is more than one block).
//   prefix_apply  (the same blocks) composes the blocks before its own, the
//                 warps (chunks of 32 regions) before each warp and the regions
//                 before each region, and writes the segment ends, the totals,
//                 and the work list: every region that holds structurals
//                 outside strings, with its entry and end values.
//   scan_emit    (one warp per listed region) reads the mask words the table
//                 kernel stored for the region's steps that hold structural
//                 characters (opens, closes, braces and other structurals, and
//                 the structurals inside strings for an entry outside one),
//                 flips the in-string part by the region's now known entry
//                 state, and writes the 1-based positions, zeroed pair entries
//                 and bracket records (structural index, level, open flag,
//                 brace or bracket) through a per-warp staging buffer in shared
//                 memory, so that every global store is coalesced.
//
// A launch may cover a wave of regions [r_begin, r_end) only, starting from
// the previous wave's end value (a streamed parse scans in waves so that each
// wave's positions can leave for the host while later input still arrives).
//
// The input crosses HBM once; the masks (512 bytes per KiB, only for steps
// with structural characters) are written once and read back only for the
// regions that hold structurals outside strings.  Nothing spins on another
// block: the only wait is for input bytes still being copied (an overlapped
// one-shot parse), bounded, with a timeout flag.
//
// This replaces the reference's stage 1 (checkAscii + checkUTF8,
// cujson/parse_standard_json.cu:186-327) and stage 2 (bitMapCreatorSimd :446,
// findEscapedQuoteMerge_NEW :767, thrust::exclusive_scan :1163,
// inStringFinderBaseline :851, findOutUsefulStringMerge :916, two
// thrust::inclusive_scan + host syncs :1245-1255, removeCopy :954), and the
// depth computation of stage 3 (depth_init_MathAPI :1346 + u8 inclusive_scan
// :1537 + transform_if :1540).
#include <cuda_runtime.h>

#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

namespace cj {

namespace {

constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr int kThreads = 256;                  // 8 warps per block (tables, emit, prefix)
constexpr int kWarpsPerBlock = kThreads / 32;
constexpr uint32_t kInputWaitLimit = 1u << 22; // polls (>= 256 ns each) for input bytes
// how many steps ahead of the current one the table kernel asks for a step to
// be brought into L2 when ScanParams::prefetch_steps is 0 (the register load
// is one step ahead)
#ifndef CJ_L2_AHEAD
#define CJ_L2_AHEAD 4
#endif
constexpr int kL2Ahead = CJ_L2_AHEAD;
__device__ __forceinline__ int l2_ahead(const ScanParams& P) {
    return P.prefetch_steps ? (int)P.prefetch_steps : kL2Ahead;
}

// resident blocks per SM the table and emit kernels are compiled for (their
// register budgets: 65536 / (256 x blocks))
#ifndef CJ_TABLES_MIN_BLOCKS
#define CJ_TABLES_MIN_BLOCKS 4
#endif
#ifndef CJ_EMIT_MIN_BLOCKS
#define CJ_EMIT_MIN_BLOCKS 4
#endif
constexpr int kTablesMinBlocks = CJ_TABLES_MIN_BLOCKS;

constexpr int kEmitMinBlocks = CJ_EMIT_MIN_BLOCKS;
// emit staging, per warp: positions and bracket records of the steps since the
// last flush (a step whose counts exceed them is written directly)
constexpr int kPosStage = 512;
constexpr int kBrkStage = 256;

// Bits of a region table's `st` that the table algebra ignores (it reads bits
// 0-3 only): the region's wflip, and which of its steps have stored masks.
constexpr int kTabFlipBit = 4;
constexpr int kTabStepsShift = 16;

// (CJ_EMU: the CPU emulation of the kernels in tests/emu, test infrastructure)
__device__ __forceinline__ uint32_t lanemask_lt() {
#ifdef CJ_EMU
    return (1u << (threadIdx.x & 31)) - 1u;
#else
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
#endif
}

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
#ifdef CJ_EMU
    return *reinterpret_cast<const volatile unsigned long long*>(p);
#else
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
#endif
}

__device__ __forceinline__ bool aborted(const Ctrl* ctrl) {
    return (*reinterpret_cast<const volatile uint32_t*>(&ctrl->error_flags) & CJ_FLAG_TIMEOUT) != 0u;
}

__device__ __noinline__ void give_up(Ctrl* ctrl, uint32_t where) {
    atomicCAS(&ctrl->gave_up, 0u, where);
    atomicOr(&ctrl->error_flags, CJ_FLAG_TIMEOUT);
}

// A region as the kernels see it: its segment and its place there.
struct Region {
    const uint8_t* base;   // the segment's first byte in the device input
    uint64_t off;          // region start within the segment
    uint64_t seg_len;
    uint64_t seg_log;      // added to byte positions
    uint64_t out_base;     // output index base of the segment
    uint64_t brk_base;     // bracket-record base of the segment
    uint32_t segi;
    uint32_t local;        // region number within the segment
    uint32_t n_local;      // regions of the segment
    uint32_t seg_flags;
    int len;               // bytes of the region
};

__device__ __forceinline__ void region_of(const ScanParams& P, uint32_t r, int region_bytes, Region& g) {
    const uint32_t segi = P.region_seg ? __ldg(P.region_seg + r) : 0u;
    const Segment* sp = P.segs + segi;
    g.segi = segi;
    g.local = r - __ldg(&sp->first_region);
    g.n_local = __ldg(&sp->n_regions);
    g.seg_len = __ldg(&sp->len);
    g.off = (uint64_t)g.local * (uint64_t)region_bytes;
    const uint64_t rem = g.seg_len - g.off;
    g.len = rem < (uint64_t)region_bytes ? (int)rem : region_bytes;
    g.base = P.in + __ldg(&sp->dev_off);
    g.seg_log = __ldg(&sp->logical_off);
    g.out_base = __ldg(&sp->out_base);
    g.brk_base = __ldg(&sp->brk_base);
    g.seg_flags = __ldg(&sp->flags);
}

// zero the bytes of a 16-byte chunk at or beyond `valid` (chunk-relative)
__device__ __forceinline__ void mask_chunk(uint4& v, int valid) {
    uint32_t* w = &v.x;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int vb = valid - 4 * k;
        if (vb <= 0) w[k] = 0;
        else if (vb < 4) w[k] &= (1u << (8 * vb)) - 1u;
    }
}

// Bounded wait until the region's bytes are in device memory (overlapped
// one-shot parses: the host's copies raise P.ready); false if given up.
__device__ __forceinline__ bool wait_input(const ScanParams& P, const Region& g) {
    if (!P.ready) return true;
    const uint64_t padded = (g.seg_len + kPadBytes - 1) / kPadBytes * kPadBytes;
    const uint64_t end = g.off + (uint64_t)((g.len + kStepBytes - 1) / kStepBytes) * kStepBytes;
    const uint64_t need = (uint64_t)(g.base - P.in) + (end < padded ? end : padded);
    const uint32_t limit = P.input_wait_limit ? P.input_wait_limit : kInputWaitLimit;
    uint32_t spins = 0;
    while (ld_acquire64(P.ready) < need) {
        if (++spins > limit || ((spins & 255u) == 0u && aborted(P.ctrl))) {
            give_up(P.ctrl, kGaveInput);
            return false;
        }
        __nanosleep(256);
    }
    return true;
}

// ---- per-warp step stream ---------------------------------------------------------
// A warp's regions (every nw-th region from its first) are read as one stream of 1 KiB steps: each lane holds its own 32 bytes
// of the next step in registers, loaded while the current step is processed,
// so the reads of the next region start during the last step of the current
// one.  (Plain loads streamed at ~97 % of the measured HBM bandwidth in a
// probe on this GPU; 16-byte cp.async copies into shared memory reached ~57 %.)
constexpr uint32_t kNoRegion = 0xFFFFFFFFu;

struct Stream {
    uint4 a, b;            // the lane's 32 bytes of the next step
    uint32_t c;            // the region of the next step (kNoRegion: none)
    uint32_t ahead;        // lane 0: the ticket drawn for the region after it
    int j, n;              // that step's number in its region, the region's step count
    const uint8_t* src;    // the lane's bytes of step 0 of that region
};

// Regions after each warp's first come from a ticket counter, so a warp that
// drew quiet regions (backslash runs) takes more of them while another works
// through dense ones.  Each warp draws its next ticket as it enters a region
// and reads it only when the region is done, so the atomic's latency is hidden
// behind a whole region.
struct TicketWalk {
    uint32_t* ticket;      // tickets drawn so far
    uint32_t base, n;      // ticket t is region base + t, below n
    // lane 0's ticket (the other lanes get 0)
    __device__ __forceinline__ uint32_t draw(int lane) const { return lane == 0 ? atomicAdd(ticket, 1u) : 0u; }
    // the region of lane 0's ticket, in every lane
    __device__ __forceinline__ uint32_t region(uint32_t drawn) const {
        const uint32_t t = __shfl_sync(FULL, drawn, 0);
        return (t < n - min(n, base)) ? base + t : kNoRegion;
    }
};

__device__ __forceinline__ void prefetch_l2(const void* p) {
#ifndef CJ_EMU
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
#else
    (void)p;
#endif
}

__device__ __forceinline__ void stream_load(Stream& st) {
    const uint4* p = reinterpret_cast<const uint4*>(st.src + (size_t)st.j * kStepBytes);
    st.a = __ldcg(p);
    st.b = __ldcg(p + 1);
}


// point the stream at step 0 of cursor c's region and load it (after the wait
// for its input bytes of an overlapped parse; a wait that gives up ends the
// stream)
template <int R, typename Walk>
__device__ __forceinline__ void stream_enter(const ScanParams& P, Stream& st, uint32_t c, int lane,
                                             const Walk& walk) {
    st.c = c;
    st.j = 0;
    st.n = 0;
    if (c == kNoRegion) return;
    st.ahead = walk.draw(lane);
    Region g;
    region_of(P, c, R * kStepBytes, g);
    if (P.ready && !__shfl_sync(FULL, lane == 0 ? wait_input(P, g) : true, 0)) { st.c = kNoRegion; return; }
    st.n = (g.len + kStepBytes - 1) / kStepBytes;
    st.src = g.base + g.off + lane * kBytesPerThread;
    stream_load(st);
    const int ahead = l2_ahead(P);
    for (int k = 1; k < ahead; k++)
        if (k < st.n) prefetch_l2(st.src + (size_t)k * kStepBytes);
}

// take the next step (lo, hi), load the one after it, and ask for the one
// after that to be brought into L2 (within the region), so that the load
// issued one step ahead mostly waits for L2, not HBM
template <int R, typename Walk>
__device__ __forceinline__ void stream_take(const ScanParams& P, Stream& st, uint4& lo, uint4& hi, int lane,
                                            const Walk& walk) {
    lo = st.a;
    hi = st.b;
    if (st.c == kNoRegion) return;
    if (++st.j < st.n) {
        stream_load(st);
        const int ahead = l2_ahead(P);
        if (st.j + ahead - 1 < st.n) prefetch_l2(st.src + (size_t)(st.j + ahead - 1) * kStepBytes);
    } else {
        stream_enter<R>(P, st, walk.region(st.ahead), lane, walk);
    }
}

// ---- transfer-table helpers ---------------------------------------------------------

__device__ __forceinline__ void load_tab(const uint4* p, Ent t[4]) {
#pragma unroll
    for (int s = 0; s < 4; s++) {
        const uint4 v = __ldcg(p + s);
        t[s].st = v.x; t[s].s = v.y; t[s].k = v.z; t[s].d = (int32_t)v.w;
    }
}

__device__ __forceinline__ void store_tab(uint4* p, const Ent t[4]) {
#pragma unroll
    for (int s = 0; s < 4; s++) p[s] = make_uint4(t[s].st, t[s].s, t[s].k, (uint32_t)t[s].d);
}

__device__ __forceinline__ void shfl_tab(const Ent t[4], Ent u[4], int src_delta, bool up) {
#pragma unroll
    for (int s = 0; s < 4; s++) {
        if (up) {
            u[s].st = __shfl_up_sync(FULL, t[s].st, src_delta);
            u[s].s = __shfl_up_sync(FULL, t[s].s, src_delta);
            u[s].k = __shfl_up_sync(FULL, t[s].k, src_delta);
            u[s].d = __shfl_up_sync(FULL, t[s].d, src_delta);
        } else {
            u[s].st = __shfl_down_sync(FULL, t[s].st, src_delta);
            u[s].s = __shfl_down_sync(FULL, t[s].s, src_delta);
            u[s].k = __shfl_down_sync(FULL, t[s].k, src_delta);
            u[s].d = __shfl_down_sync(FULL, t[s].d, src_delta);
        }
    }
}

// composition of the 32 lanes' tables in lane order, in lane 0
__device__ __forceinline__ void warp_reduce_tab(Ent t[4], int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        Ent u[4];
        shfl_tab(t, u, o, false);
        if ((lane & (2 * o - 1)) == 0 && lane + o < 32) tab_compose(t, u, t);
    }
}

// ---- scan_tables --------------------------------------------------------------

// Transfer table of one region (the whole warp; lanes 0-3 write entries 0-3).
// The region is classified assuming it is entered outside any string and
// escape; the table then follows for all 4 entry states: an escape pending at
// entry only matters when the first byte after the region's leading backslash
// run is a quote (`wflip`), and entering inside a string flips the in-string
// mask of the whole region, which swaps the counts of structurals outside and
// inside strings.  The steps come from the warp's stream `st`.
template <bool LINES, int R, typename Walk>
__device__ __forceinline__ void region_table(const ScanParams& P, const Region& g, uint4* out, uint4* mout,
                                             int lane, uint32_t lt, Stream& st, const Walk& walk)
{
    const int nsteps = (g.len + kStepBytes - 1) / kStepBytes;
    // the 4 bytes before the region (their UTF-8 leads carry in): loaded now,
    // used only once the first step is classified
    const uint32_t pw = g.off > 0 ? __ldcg(reinterpret_cast<const uint32_t*>(g.base + g.off) - 1) : 0u;
    uint32_t ucarry = 0;                   // UTF-8 carry into the step (warp uniform)
    uint32_t carry = 0, par = 0;           // escape carry / quote parity (warp uniform)
    uint32_t started = 0, wflip = 0;       // first non-all-backslash lane seen / its flip
    uint32_t in_run = 0;                   // the previous step ended in a backslash
    uint32_t steps = 0;                    // steps whose mask words were stored
    // per lane, two counts per register (low half: outside strings for an entry
    // outside one; high half: all): structurals, brackets, opens (<= 512 each)
    uint32_t n_c = 0, n_k = 0, n_o = 0;
    for (int j = 0; j < nsteps; j++) {
        uint4 lo, hi;
        stream_take<R>(P, st, lo, hi, lane, walk);
        const int step_len = min(kStepBytes, g.len - j * kStepBytes);
        const int valid = min(kBytesPerThread, step_len - lane * kBytesPerThread);
        if (valid < kBytesPerThread) {
            if (16 > valid) mask_chunk(lo, valid);
            mask_chunk(hi, valid - 16);
        }
        const uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        if (in_run) {
            // after a step that ended in a backslash: a step of 1 KiB of
            // backslashes (inside a long run) is an even run (the escape carry
            // passes through), opens no UTF-8 sequence, and has no quote or
            // structural byte -- nothing changes
            uint32_t d = 0;
#pragma unroll
            for (int k = 0; k < 8; k++) d |= w[k] ^ 0x5C5C5C5Cu;
            if (__all_sync(FULL, d == 0u)) { ucarry = 0u; continue; }
        }
        uint32_t planes[8];
        bit_planes32(w, planes);
        const Classes c = classify_planes<LINES>(planes);

        // UTF-8 on the bit planes, on steps that hold a non-ASCII byte or
        // continue a sequence from the bytes before them
        if (j == 0 && (pw & 0x80808000u)) ucarry = utf8_carry_word(pw);
        if (__any_sync(FULL, c.hi != 0u) || ucarry != 0u) {
            const uint32_t cout = utf8_carry_planes(planes);
            uint32_t cin = __shfl_up_sync(FULL, cout, 1);
            if (lane == 0) cin = ucarry;
            ucarry = __shfl_sync(FULL, cout, 31);
            if (valid > 0) {
                const bool seg_end = g.off + (uint64_t)(j * kStepBytes + lane * kBytesPerThread + kBytesPerThread) >= g.seg_len;
                if (utf8_errors_planes(planes, cin, seg_end)) {
                    if (P.seg_err) atomicOr(P.seg_err + g.segi, CJ_FLAG_UTF8);
                    else atomicOr(&P.ctrl->error_flags, CJ_FLAG_UTF8);
                }
            }
        } else {
            ucarry = 0u;
        }

        // escapes: carry from the nearest earlier lane that is not all backslashes
        uint32_t lane_carry;
        const uint32_t ends_bs = __ballot_sync(FULL, (int32_t)c.bs < 0);   // lanes ending in a backslash
        in_run = ends_bs >> 31;
        if (!ends_bs) {
            lane_carry = (lane == 0) ? carry : 0u;
            if (!started) {
                wflip = __shfl_sync(FULL, (c.q >> (__ffs(~c.bs) - 1)) & 1u, 0);
                started = 1;
            }
            carry = 0;
        } else {
            const bool all_bs = (c.bs == FULL);
            const uint32_t nonall = __ballot_sync(FULL, !all_bs);
            const uint32_t couts = __ballot_sync(FULL, escape_cout(c.bs) != 0u);
            const uint32_t prior = nonall & lt;
            lane_carry = prior ? (couts >> (31 - __clz(prior))) & 1u : carry;
            if (nonall) {
                if (!started) {
                    const uint32_t flipc = all_bs ? 0u : ((c.q >> (__ffs(~c.bs) - 1)) & 1u);
                    wflip = __shfl_sync(FULL, flipc, __ffs(nonall) - 1);
                    started = 1;
                }
                carry = (couts >> (31 - __clz(nonall))) & 1u;
            } else {
                continue;
            }
        }
        uint32_t dummy;
        const uint32_t esc = escaped32(c.bs, lane_carry, &dummy);
        const uint32_t rq = c.q & ~esc;
        const uint32_t qb = __ballot_sync(FULL, __popc(rq) & 1u);
        const uint32_t lpar = par ^ (__popc(qb & lt) & 1u);
        par ^= __popc(qb) & 1u;
        const uint32_t M = prefix_xor(rq) ^ (lpar ? FULL : 0u);
        n_c += (uint32_t)__popc(c.st & ~M) | ((uint32_t)__popc(c.st) << 16);
        n_k += (uint32_t)__popc(c.br & ~M) | ((uint32_t)__popc(c.br) << 16);
        n_o += (uint32_t)__popc(c.op & ~M) | ((uint32_t)__popc(c.op) << 16);
        // the step's four mask words for the emit kernel, when it holds any
        // structural character: opens, closes, `x` (braces among brackets and
        // every other structural) and the structurals inside strings for an
        // entry outside one
        if (__any_sync(FULL, c.st != 0u)) {
            __stcg(mout + (size_t)j * 32, make_uint4(c.op, c.br & ~c.op, c.cur | (c.st & ~c.br), c.st & M));
            steps |= 1u << j;
        }
    }
    const int32_t C0 = (int32_t)__reduce_add_sync(FULL, n_c & 0xFFFFu), Ct = (int32_t)__reduce_add_sync(FULL, n_c >> 16);
    const int32_t K0 = (int32_t)__reduce_add_sync(FULL, n_k & 0xFFFFu), Kt = (int32_t)__reduce_add_sync(FULL, n_k >> 16);
    const int32_t O0 = (int32_t)__reduce_add_sync(FULL, n_o & 0xFFFFu), Ot = (int32_t)__reduce_add_sync(FULL, n_o >> 16);
    const int32_t D0 = 2 * O0 - K0, Dt = 2 * Ot - Kt;
    if (lane < 4) {
        // a segment's first region is entered outside strings at depth 0 whatever
        // came before: every entry state reads as state 0, with the reset bits
        const bool first = g.local == 0;
        const uint32_t s = first ? 0u : (uint32_t)lane;
        const uint32_t escin = s >> 1, instr = s & 1u;
        const uint32_t e = instr ^ (escin & wflip);
        uint32_t st = ((started ? carry : escin) << 1) | (e ^ par) | (wflip << kTabFlipBit) |
                      (steps << kTabStepsShift);
        if (first) st |= kResetState | ((g.seg_flags & kSegContinue) ? 0u : kResetCounts);
        out[lane] = make_uint4(st, (uint32_t)(e ? Ct - C0 : C0), (uint32_t)(e ? Kt - K0 : K0),
                               (uint32_t)(e ? Dt - D0 : D0));
    }
}

template <bool LINES, int R>
__global__ void __launch_bounds__(kThreads, kTablesMinBlocks) scan_tables(ScanParams P)
{
    allow_next_grid();
    const int lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const uint32_t nw = gridDim.x * kWarpsPerBlock;
    const uint32_t n = P.r_end;
    const uint32_t first = P.r_begin + blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (first >= n) return;
    const TicketWalk walk{P.tickets ? P.tickets : &P.ctrl->tables_ticket, P.r_begin + nw, n};
    Stream st;
    stream_enter<R>(P, st, first, lane, walk);
    // the stream holds the next region's first step when a region's table is done
    for (uint32_t r = first; r != kNoRegion; r = st.c) {
        if (P.ready && aborted(P.ctrl)) break;     // the wait for input bytes gave up
        Region g;
        region_of(P, r, R * kStepBytes, g);
        region_table<LINES, R>(P, g, P.rtab + (size_t)r * 4, P.masks + (size_t)r * R * 32 + lane, lane, lt, st,
                               walk);
    }
}

// ---- prefix over the region tables --------------------------------------------------
// Blocks of kPrefixPerBlock regions, one per thread; a warp's 32 regions are a
// chunk.  Both kernels are shallow -- a warp scan or reduction of tables per
// level -- and use small blocks, so that the table compositions spread over
// every SM.

constexpr int kPrefixWarps = kPrefixPerBlock / 32;


// ---- state-first prefix ------------------------------------------------------------
// Applying tables one after another, the string/escape state follows from the
// tables' state maps alone (4 entries of 2 bits: one byte), and once each
// table's entry state is known its counts are a plain prefix sum (restarted
// by the reset bits).  So the prefix is two cheap scans -- of state maps, then
// of the counts each table gives for its entry state -- instead of a scan of
// whole 4-entry tables.

constexpr uint32_t kMapIdentity = 0xE4u;     // state s -> s

__device__ __forceinline__ uint32_t map_of(const Ent t[4]) {
    return (t[0].st & 3u) | ((t[1].st & 3u) << 2) | ((t[2].st & 3u) << 4) | ((t[3].st & 3u) << 6);
}
__device__ __forceinline__ uint32_t map_at(uint32_t m, uint32_t s) { return (m >> (2u * s)) & 3u; }
// map a, then map b
__device__ __forceinline__ uint32_t map_then(uint32_t a, uint32_t b) {
    return map_at(b, a & 3u) | (map_at(b, (a >> 2) & 3u) << 2) | (map_at(b, (a >> 4) & 3u) << 4) |
           (map_at(b, (a >> 6) & 3u) << 6);
}

// counts added by a run of tables, and whether the run restarts them
struct Sums {
    uint32_t s, k;
    int32_t d;
    uint32_t f;            // kResetState | kResetCounts seen in the run
};
__device__ __forceinline__ Sums sums_zero() { Sums z; z.s = 0; z.k = 0; z.d = 0; z.f = 0; return z; }
__device__ __forceinline__ Sums sums_of(const Ent& x) {
    Sums r; r.s = x.s; r.k = x.k; r.d = x.d; r.f = x.st & (kResetState | kResetCounts); return r;
}
// run a, then run b
__device__ __forceinline__ Sums sums_then(const Sums& a, const Sums& b) {
    Sums r;
    r.s = (b.f & kResetCounts) ? b.s : a.s + b.s;
    r.k = (b.f & kResetCounts) ? b.k : a.k + b.k;
    r.d = (b.f & kResetState) ? b.d : a.d + b.d;
    r.f = a.f | b.f;
    return r;
}
__device__ __forceinline__ Sums shfl_up_sums(const Sums& a, int o) {
    Sums r;
    r.s = __shfl_up_sync(FULL, a.s, o);
    r.k = __shfl_up_sync(FULL, a.k, o);
    r.d = __shfl_up_sync(FULL, a.d, o);
    r.f = __shfl_up_sync(FULL, a.f, o);
    return r;
}
// value v, then a run with sums p ending in state st
__device__ __forceinline__ Ent apply_sums(const Ent& v, const Sums& p, uint32_t st) {
    Ent r;
    r.st = st;
    r.s = (p.f & kResetCounts) ? p.s : v.s + p.s;
    r.k = (p.f & kResetCounts) ? p.k : v.k + p.k;
    r.d = (p.f & kResetState) ? p.d : v.d + p.d;
    return r;
}

// Exclusive scans over the block's threads, in thread order: state maps
// (identity before the first) and sums (zero before the first).  `m_ex` and
// `p_ex` are the thread's prefixes; the block's totals go to *m_tot / *p_tot
// when given.  Three __syncthreads; every thread of the block calls it.
__device__ __forceinline__ void block_scan_maps(uint32_t m, uint32_t* sm, int lane, int warp, uint32_t& m_ex,
                                                uint32_t* m_tot) {
    uint32_t mi = m;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, mi, o);
        if (lane >= o) mi = map_then(y, mi);
    }
    uint32_t mx = __shfl_up_sync(FULL, mi, 1);
    if (lane == 0) mx = kMapIdentity;
    if (lane == 31) sm[warp] = mi;
    __syncthreads();
    if (warp == 0) {
        uint32_t c = lane < kPrefixWarps ? sm[lane] : kMapIdentity;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, c, o);
            if (lane >= o) c = map_then(y, c);
        }
        uint32_t cx = __shfl_up_sync(FULL, c, 1);
        if (lane == 0) cx = kMapIdentity;
        const uint32_t tot = __shfl_sync(FULL, c, 31);
        __syncwarp();
        if (lane < kPrefixWarps) sm[lane] = cx;
        if (lane == 0) sm[kPrefixWarps] = tot;
    }
    __syncthreads();
    m_ex = map_then(sm[warp], mx);
    if (m_tot) *m_tot = sm[kPrefixWarps];
    __syncthreads();
}

__device__ __forceinline__ void block_scan_sums(const Sums& v, Sums* sm, int lane, int warp, Sums& p_ex,
                                                Sums* p_tot) {
    Sums si = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Sums y = shfl_up_sums(si, o);
        if (lane >= o) si = sums_then(y, si);
    }
    Sums sx = shfl_up_sums(si, 1);
    if (lane == 0) sx = sums_zero();
    if (lane == 31) sm[warp] = si;
    __syncthreads();
    if (warp == 0) {
        Sums c = lane < kPrefixWarps ? sm[lane] : sums_zero();
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const Sums y = shfl_up_sums(c, o);
            if (lane >= o) c = sums_then(y, c);
        }
        Sums cx = shfl_up_sums(c, 1);
        if (lane == 0) cx = sums_zero();
        Sums tot;
        tot.s = __shfl_sync(FULL, c.s, 31);
        tot.k = __shfl_sync(FULL, c.k, 31);
        tot.d = __shfl_sync(FULL, c.d, 31);
        tot.f = __shfl_sync(FULL, c.f, 31);
        __syncwarp();
        if (lane < kPrefixWarps) sm[lane] = cx;
        if (lane == 0) sm[kPrefixWarps] = tot;
    }
    __syncthreads();
    p_ex = sums_then(sm[warp], sx);
    if (p_tot) *p_tot = sm[kPrefixWarps];
    __syncthreads();
}

// Block b: the composition of its regions' tables.
__global__ void __launch_bounds__(kPrefixPerBlock) prefix_reduce(ScanParams P)
{
    __shared__ Ent s_w[kPrefixWarps][4];
    allow_next_grid();
    wait_previous_grid();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t r = P.r_begin + blockIdx.x * (uint32_t)kPrefixPerBlock + threadIdx.x;
    Ent t[4];
    if (r < P.r_end) load_tab(P.rtab + (size_t)r * 4, t);
    else tab_identity(t);
    warp_reduce_tab(t, lane);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 4; k++) s_w[warp][k] = t[k];
    }
    __syncthreads();
    if (warp == 0) {
        if (lane < kPrefixWarps) {
#pragma unroll
            for (int k = 0; k < 4; k++) t[k] = s_w[lane][k];
        } else {
            tab_identity(t);
        }
        warp_reduce_tab(t, lane);
        if (lane == 0) store_tab(P.bagg + (size_t)blockIdx.x * 4, t);
    }
}

// Block b: entry values, segment ends, totals and the emit work list.
__global__ void __launch_bounds__(kPrefixPerBlock) prefix_apply(ScanParams P)
{
    __shared__ uint32_t s_map[kPrefixWarps + 1];
    __shared__ Sums s_sum[kPrefixWarps + 1];
    __shared__ uint32_t s_cnt[kPrefixWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    allow_next_grid();
    wait_previous_grid();
    if (aborted(P.ctrl)) return;          // a timed-out run writes no outputs
    const uint32_t n = P.n_regions;
    const uint32_t b = blockIdx.x;

    // the value before the scan
    Ent v0 = ent_identity(0);
    if (P.carry_in) {
        const uint4 c = __ldcg(P.carry_in);
        v0.st = c.x; v0.s = c.y; v0.k = c.z; v0.d = (int32_t)c.w;
    }
    // the value before this block: every thread takes a run of the blocks'
    // aggregate tables before it (from prefix_reduce), first for its state
    // map, then, once the state at the run's start is known, for its sums
    Ent vb = v0;
    if (b > 0) {
        const uint32_t units = b;
        const uint4* src = P.bagg;
        const uint32_t q = (units + kPrefixPerBlock - 1) / kPrefixPerBlock;
        const uint32_t lo = min(units, threadIdx.x * q), hi = min(units, lo + q);
        uint32_t m = kMapIdentity;
        for (uint32_t i = lo; i < hi; i++) {
            const uint4* u = src + (size_t)i * 4;
            const uint32_t um = (__ldcg(&u[0].x) & 3u) | ((__ldcg(&u[1].x) & 3u) << 2) |
                                ((__ldcg(&u[2].x) & 3u) << 4) | ((__ldcg(&u[3].x) & 3u) << 6);
            m = map_then(m, um);
        }
        uint32_t m_ex, m_tot;
        block_scan_maps(m, s_map, lane, warp, m_ex, &m_tot);
        uint32_t e = map_at(m_ex, v0.st & 3u);
        Sums run = sums_zero();
        for (uint32_t i = lo; i < hi; i++) {
            // the whole table, so that no load waits for the previous state
            Ent u[4];
            load_tab(src + (size_t)i * 4, u);
            const Ent xe = ent_select(u, e);
            run = sums_then(run, sums_of(xe));
            e = xe.st & 3u;
        }
        Sums p_ex, p_tot;
        block_scan_sums(run, s_sum, lane, warp, p_ex, &p_tot);
        vb = apply_sums(v0, p_tot, map_at(m_tot, v0.st & 3u));
    }

    // this block's regions: the state each is entered in, then the counts
    // before each
    const uint32_t r = P.r_begin + b * (uint32_t)kPrefixPerBlock + threadIdx.x;
    const bool in_range = r < P.r_end;
    Ent t[4];
    if (in_range) load_tab(P.rtab + (size_t)r * 4, t);
    else tab_identity(t);
    uint32_t m_ex;
    block_scan_maps(map_of(t), s_map, lane, warp, m_ex, nullptr);
    const uint32_t e_state = map_at(m_ex, vb.st & 3u);
    const Ent x = ent_select(t, e_state);
    Sums p_ex;
    block_scan_sums(in_range ? sums_of(x) : sums_zero(), s_sum, lane, warp, p_ex, nullptr);
    const Ent v = apply_sums(vb, p_ex, e_state);

    bool work = false;
    Ent e = v, nv = v;
    uint32_t steps_flip = 0;
    if (in_range) {
        const uint32_t raw = t[0].st;           // the region's own table: wflip, stored steps
        nv = ent_apply(v, t);
        // the entry value as the region starts: a segment's first region starts
        // in state 0 at depth 0 (and at count 0 for an independent document)
        if (x.st & kResetState) { e.st = 0; e.d = 0; }
        if (x.st & kResetCounts) { e.s = 0; e.k = 0; }
        work = x.s != 0u;
        // whether the region's in-string mask (computed for an entry outside
        // strings and escapes) is flipped: entering inside a string, or with an
        // escape pending before a leading quote; a segment's first region is
        // entered in state 0
        const uint32_t instr = e.st & 1u, escin = (e.st >> 1) & 1u;
        const uint32_t flip = instr ^ (escin & ((raw >> kTabFlipBit) & 1u));
        steps_flip = (raw >> kTabStepsShift) | (flip << 31);
        const uint32_t segi = P.region_seg ? __ldg(P.region_seg + r) : 0u;
        const Segment* sp = P.segs + segi;
        if (r + 1 == __ldg(&sp->first_region) + __ldg(&sp->n_regions)) {
            SegmentOut so;
            so.s_end = nv.s;
            so.k_end = nv.k;
            so.depth_end = nv.d;
            so.instr_end = nv.st & 1u;
            P.seg_out[segi] = so;
            if (nv.d != 0) {
                if (P.seg_err) atomicOr(P.seg_err + segi, CJ_FLAG_BRACKETS);
                else atomicOr(&P.ctrl->error_flags, CJ_FLAG_BRACKETS);
            }
        }
        if (r + 1 == n) {
            P.ctrl->s_total = nv.s;
            P.ctrl->k_total = nv.k;
        }
        if (r + 1 == P.r_end) {
            const uint4 c = make_uint4(nv.st, nv.s, nv.k, (uint32_t)nv.d);
            if (P.carry_out) *P.carry_out = c;
            if (P.carry_host) {
                __stcg(P.carry_host, c);
                __threadfence_system();
            }
        }
    }

    // the block's regions with structurals go to the work list (one atomic per block)
    const uint32_t bal = __ballot_sync(FULL, work);
    if (lane == 0) s_cnt[warp] = __popc(bal);
    __syncthreads();
    if (warp == 0) {
        const uint32_t cnt = lane < kPrefixWarps ? s_cnt[lane] : 0u;
        uint32_t x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        const uint32_t tot = __shfl_sync(FULL, x, 31);
        uint32_t base = 0;
        if (lane == 0 && tot) base = atomicAdd(P.n_work ? P.n_work : &P.ctrl->n_work, tot);
        base = __shfl_sync(FULL, base, 0);
        if (lane < kPrefixWarps) s_cnt[lane] = base + x - cnt;
    }
    __syncthreads();
    if (work) {
        const uint32_t o = s_cnt[warp] + __popc(bal & lanemask_lt());
        P.work[2 * (size_t)o] = make_uint4(r, steps_flip, e.s, e.k);
        P.work[2 * (size_t)o + 1] = make_uint4((uint32_t)e.d, nv.s, nv.k, (uint32_t)nv.d);
    }
}

// ---- scan_emit --------------------------------------------------------------------

struct EmitStage {
    int32_t pos[kPosStage];
    uint2 brk[kBrkStage];
};

// Write the staged entries: positions (and zeroed pair entries) at output
// indices s0.., bracket records at k0...  Out-of-capacity writes are dropped
// and flagged (they cannot happen with consistent counts).
__device__ __forceinline__ void emit_flush(const ScanParams& P, const Region& g, const EmitStage& st,
                                           uint32_t s0, uint32_t ns, uint32_t k0, uint32_t nk, int lane)
{
    __syncwarp();
    int32_t* pos = P.pos + g.out_base;
    int32_t* pair = P.pair + g.out_base;
    uint2* brk = P.brk + g.brk_base;
    const uint64_t pcap = P.out_cap - min(P.out_cap, g.out_base);
    const uint64_t bcap = P.brk_cap - min(P.brk_cap, g.brk_base);
    bool bad = false;
    for (uint32_t i = lane; i < ns; i += 32) {
        const uint64_t o = (uint64_t)s0 + i;
        if (o < pcap) { pos[o] = st.pos[i]; pair[o] = 0; } else bad = true;
    }
    for (uint32_t i = lane; i < nk; i += 32) {
        const uint64_t o = (uint64_t)k0 + i;
        if (o < bcap) brk[o] = st.brk[i]; else bad = true;
    }
    if (__any_sync(FULL, bad) && lane == 0) atomicOr(&P.ctrl->error_flags, CJ_FLAG_OVERFLOW);
    __syncwarp();
}

// One listed region: the steps whose mask words were stored, with the
// region's in-string mask flipped (`flip` all ones) or not by its entry state.
__device__ __forceinline__ void emit_region(const ScanParams& P, const Region& g, const uint4* mk,
                                            uint32_t steps, uint32_t flip, uint32_t s_base, uint32_t k_base,
                                            int32_t d_base, EmitStage& st, uint32_t expect_s, uint32_t expect_k,
                                            int32_t expect_d, int lane)
{
    uint32_t s_flush = s_base, k_flush = k_base;   // output indices of stage[0]
    const uint64_t pos_lane = g.seg_log + g.off + (uint64_t)lane * kBytesPerThread + 1u;
    // every stored step into L2 now, so that the one-ahead loads below wait
    // for L2, not HBM
    for (uint32_t m = steps; m; m &= m - 1u) prefetch_l2(mk + (size_t)(__ffs(m) - 1) * 32);
    uint32_t rem = steps;
    uint4 nm = make_uint4(0, 0, 0, 0);
    if (rem) nm = __ldcg(mk + (size_t)(__ffs(rem) - 1) * 32);
    while (rem) {
        const int j = __ffs(rem) - 1;
        rem &= rem - 1u;
        const uint4 m = nm;
        if (rem) nm = __ldcg(mk + (size_t)(__ffs(rem) - 1) * 32);   // the next stored step
        const uint32_t opw = m.x, brw = m.x | m.y, xw = m.z;
        const uint32_t stm = (brw | xw) & ~(m.w ^ flip);
        if (!__any_sync(FULL, stm)) continue;           // nothing outside strings in this step
        const uint32_t brm = brw & stm;
        const uint32_t opm = opw & stm;
        const uint32_t curm = xw & brw;
        // the three counts (each <= 32 per lane) packed in 10-bit fields: one
        // scan.  The exclusive prefixes stay <= 31 * 32 < 1024 per field; a
        // step's totals (up to 1024) are taken field by field from lane 31's
        // prefix and own count, never from the packed inclusive sum.
        const uint32_t own = (uint32_t)__popc(stm) | ((uint32_t)__popc(brm) << 10) |
                             ((uint32_t)__popc(opm) << 20);
        uint32_t incl = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        const uint32_t ex = incl - own;
        const uint32_t ex31 = __shfl_sync(FULL, ex, 31), own31 = __shfl_sync(FULL, own, 31);
        const uint32_t n1 = (ex31 & 0x3FFu) + (own31 & 0x3FFu);
        const uint32_t n2 = ((ex31 >> 10) & 0x3FFu) + ((own31 >> 10) & 0x3FFu);
        const uint32_t n3 = ((ex31 >> 20) & 0x3FFu) + ((own31 >> 20) & 0x3FFu);
        const uint32_t e1 = ex & 0x3FFu, e2 = (ex >> 10) & 0x3FFu, e3 = (ex >> 20) & 0x3FFu;
        int32_t depth = d_base + 2 * (int32_t)e3 - (int32_t)e2;
        const uint32_t pos0 = (uint32_t)(pos_lane + (uint64_t)j * kStepBytes);
        uint32_t staged_s = s_base - s_flush, staged_k = k_base - k_flush;
        if (staged_s + n1 > (uint32_t)kPosStage || staged_k + n2 > (uint32_t)kBrkStage) {
            emit_flush(P, g, st, s_flush, staged_s, k_flush, staged_k, lane);
            s_flush = s_base; k_flush = k_base;
            staged_s = 0; staged_k = 0;
        }
        if (n1 > (uint32_t)kPosStage || n2 > (uint32_t)kBrkStage) {
            // a step denser than the stage: scattered stores, one structural
            // per lane per round (only in pathological inputs)
            int32_t* pos = P.pos + g.out_base;
            int32_t* pair = P.pair + g.out_base;
            uint2* brk = P.brk + g.brk_base;
            const uint64_t pcap = P.out_cap - min(P.out_cap, g.out_base);
            const uint64_t bcap = P.brk_cap - min(P.brk_cap, g.brk_base);
            uint32_t r = s_base + e1, kr = k_base + e2;
            uint32_t mm = stm;
            bool bad = false;
            while (mm) {
                const int b = __ffs(mm) - 1;
                mm &= mm - 1u;
                if (r < pcap) { pos[r] = (int32_t)(pos0 + (uint32_t)b); pair[r] = 0; } else bad = true;
                if ((brm >> b) & 1u) {
                    const uint32_t is_open = (opm >> b) & 1u;
                    const int32_t lvl = is_open ? depth : depth - 1;
                    depth += is_open ? 1 : -1;
                    const uint32_t cur = ((curm >> b) & 1u) ? kCurly : 0u;
                    if (kr < bcap) brk[kr] = make_uint2(r | cur, ((uint32_t)lvl << 1) | is_open); else bad = true;
                    kr++;
                }
                r++;
            }
            if (__any_sync(FULL, bad) && lane == 0) atomicOr(&P.ctrl->error_flags, CJ_FLAG_OVERFLOW);
            s_flush = s_base + n1;
            k_flush = k_base + n2;
        } else {
            // positions into the stage
            uint32_t i = staged_s + e1;
            uint32_t mm = stm;
            while (mm) {
                const int b = __ffs(mm) - 1;
                mm &= mm - 1u;
                st.pos[i++] = (int32_t)(pos0 + (uint32_t)b);
            }
            // bracket records into the stage
            uint32_t kk = staged_k + e2;
            const uint32_t sl = s_base + e1;   // structural index of the lane's first structural
            mm = brm;
            while (mm) {
                const int b = __ffs(mm) - 1;
                mm &= mm - 1u;
                const uint32_t is_open = (opm >> b) & 1u;
                const int32_t lvl = is_open ? depth : depth - 1;
                depth += is_open ? 1 : -1;
                const uint32_t sidx = sl + (uint32_t)__popc(stm & ((1u << b) - 1u));
                const uint32_t cur = ((curm >> b) & 1u) ? kCurly : 0u;
                st.brk[kk++] = make_uint2(sidx | cur, ((uint32_t)lvl << 1) | is_open);
            }
        }
        s_base += n1;
        k_base += n2;
        d_base += 2 * (int32_t)n3 - (int32_t)n2;
    }
    emit_flush(P, g, st, s_flush, s_base - s_flush, k_flush, k_base - k_flush, lane);
    // the region's end must be the value its table gives (the table kernel's
    // counts); a mismatch marks the run, and the pairing kernels then skip it
    if (lane == 0 && (s_base != expect_s || k_base != expect_k || d_base != expect_d))
        atomicOr(&P.ctrl->error_flags, CJ_FLAG_OVERFLOW);
}

template <int R>
__global__ void __launch_bounds__(kThreads, kEmitMinBlocks) scan_emit(ScanParams P)
{
    __shared__ EmitStage s_stage[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    allow_next_grid();
    wait_previous_grid();
    if (aborted(P.ctrl)) return;
    const uint32_t n = *reinterpret_cast<const volatile uint32_t*>(P.n_work ? P.n_work : &P.ctrl->n_work);
    const uint32_t nw = gridDim.x * kWarpsPerBlock;
    uint32_t* ticket = P.tickets ? P.tickets + 1 : &P.ctrl->emit_ticket;
    // the first item by warp number, the later ones (when there are more
    // items than warps) from a ticket counter, drawn one item ahead, so that
    // warps with sparse regions take more
    const bool more = n > nw;
    uint32_t i = blockIdx.x * kWarpsPerBlock + warp;
    while (i < n) {
        uint32_t t = n;
        if (more && lane == 0) t = atomicAdd(ticket, 1u);
        const uint4 a = __ldcg(P.work + 2 * (size_t)i), b = __ldcg(P.work + 2 * (size_t)i + 1);
        Region g;
        region_of(P, a.x, R * kStepBytes, g);
        emit_region(P, g, P.masks + (size_t)a.x * R * 32 + lane, a.y & 0xFFFFu, (a.y >> 31) ? FULL : 0u, a.z, a.w,
                    (int32_t)b.x, s_stage[warp], b.y, b.z, (int32_t)b.w, lane);
        t = __shfl_sync(FULL, t, 0);
        i = (t < n) ? nw + t : n;
    }
}

template <int R>
void launch_r(const ScanParams& p, bool lines, int tables_grid, int emit_grid, cudaStream_t stream,
              cudaEvent_t* ev)
{
    const uint32_t nb = (p.r_end - p.r_begin + kPrefixPerBlock - 1) / kPrefixPerBlock;
#ifdef CJ_EMU
    (void)stream; (void)ev;
    cj_emu::launch(tables_grid, kThreads, 0, [&] { if (lines) scan_tables<true, R>(p); else scan_tables<false, R>(p); });
    if (nb > 1) cj_emu::launch(nb, kPrefixPerBlock, 0, [&] { prefix_reduce(p); });
    cj_emu::launch(nb, kPrefixPerBlock, 0, [&] { prefix_apply(p); });
    cj_emu::launch(emit_grid, kThreads, 0, [&] { scan_emit<R>(p); });
#else
    if (lines) scan_tables<true, R><<<tables_grid, kThreads, 0, stream>>>(p);
    else scan_tables<false, R><<<tables_grid, kThreads, 0, stream>>>(p);
    if (ev) cudaEventRecord(ev[0], stream);
    const bool dep = p.dependent_launch != 0;
    if (nb > 1) launch_dependent(prefix_reduce, (int)nb, kPrefixPerBlock, 0, stream, dep, p);
    launch_dependent(prefix_apply, (int)nb, kPrefixPerBlock, 0, stream, dep, p);
    if (ev) cudaEventRecord(ev[1], stream);
    launch_dependent(scan_emit<R>, emit_grid, kThreads, 0, stream, dep, p);
    if (ev) cudaEventRecord(ev[2], stream);
#endif
}

template <int R>
int blocks_per_sm(bool lines, bool emit)
{
#ifdef CJ_EMU
    (void)lines; (void)emit;
    return 2;
#else
    int n = 0;
    cudaError_t e;
    if (emit) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, scan_emit<R>, kThreads, 0);
    else e = lines ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, scan_tables<true, R>, kThreads, 0)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, scan_tables<false, R>, kThreads, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
#endif
}

}  // namespace

bool region_steps_valid(int r) { return r == 4 || r == 8 || r == 16; }

cudaError_t preload_scan_kernels()
{
#ifdef CJ_EMU
    return cudaSuccess;
#else
    cudaFuncAttributes a;
    const void* fns[] = {
        (const void*)scan_tables<false, 4>, (const void*)scan_tables<false, 8>, (const void*)scan_tables<false, 16>,
        (const void*)scan_tables<true, 4>,  (const void*)scan_tables<true, 8>,  (const void*)scan_tables<true, 16>,
        (const void*)scan_emit<4>,          (const void*)scan_emit<8>,          (const void*)scan_emit<16>,
        (const void*)prefix_reduce,         (const void*)prefix_apply,
    };
    for (const void* f : fns) {
        const cudaError_t e = cudaFuncGetAttributes(&a, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
#endif
}

int scan_launches(uint32_t n_regions)
{
    if (n_regions == 0) return 0;
    return n_regions > (uint32_t)kPrefixPerBlock ? 4 : 3;
}

void launch_scan(const ScanParams& p0, bool lines, const ScanShape& shape, cudaStream_t stream, cudaEvent_t* ev)
{
    ScanParams p = p0;
    if (p.r_end == 0 || p.r_end > p.n_regions) p.r_end = p.n_regions;
    if (p.r_begin >= p.r_end) {
        for (int i = 0; ev && i < 3; i++) cudaEventRecord(ev[i], stream);
        return;
    }
    const int R = region_steps_valid(p.region_steps) ? p.region_steps : kRegionStepsDefault;
    const int sm = p.sm_count > 0 ? p.sm_count : 1;
    auto grid = [&](int per_sm_occ, int want_per_sm) {
        const int per_sm = want_per_sm > 0 ? (want_per_sm < per_sm_occ ? want_per_sm : per_sm_occ) : per_sm_occ;
        const uint32_t need = (p.r_end - p.r_begin + kWarpsPerBlock - 1) / kWarpsPerBlock;
        const uint32_t cap = (uint32_t)(per_sm * sm);
        return (int)(need < cap ? need : cap);
    };
    // occupancy per (R, lines, kernel): asked once
    static int occ[3][2][2] = {};
    const int ri = R == 4 ? 0 : (R == 8 ? 1 : 2);
    int* o = occ[ri][lines ? 1 : 0];
    if (!o[0]) {
        o[0] = R == 4 ? blocks_per_sm<4>(lines, false) : R == 8 ? blocks_per_sm<8>(lines, false) : blocks_per_sm<16>(lines, false);
        o[1] = R == 4 ? blocks_per_sm<4>(lines, true) : R == 8 ? blocks_per_sm<8>(lines, true) : blocks_per_sm<16>(lines, true);
    }
    const int tg = grid(o[0], shape.tables_blocks_per_sm), eg = grid(o[1], shape.emit_blocks_per_sm);
    if (R == 4) launch_r<4>(p, lines, tg, eg, stream, ev);
    else if (R == 8) launch_r<8>(p, lines, tg, eg, stream, ev);
    else launch_r<16>(p, lines, tg, eg, stream, ev);
}

}  // namespace cj
