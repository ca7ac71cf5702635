// cj_scan.cu -- the single-pass structural scan (persistent, TMA-staged,
// warp-independent, software-pipelined across tiles).
//
// A persistent grid of CTAs (one per SM: 16 classifying warps and
// kCoords = 2 coordinator warps) takes 112 KiB tiles in document order from an
// atomic ticket; the coordinator of ticket i draws ticket i + 1 once every
// warp has finished phase A of ticket i, and keeps the tile's segment geometry
// in shared memory.  Each classifying warp owns a contiguous 7 KiB region of a
// tile and works through it in 1 KiB steps (32 lanes x 32 bytes) staged in its
// own 3-deep shared-memory ring by bulk TMA copies (cp.async.bulk completing
// on per-warp mbarriers).
//
//   A. (ticket i) every classifying warp, on its own: builds the quote,
//      backslash, structural and bracket bitmaps of each lane's 32 bytes
//      (bit-sliced: 8 bit planes, one logic operation per class and 32 bytes),
//      validates UTF-8 on the same planes (only on steps holding non-ASCII
//      bytes or continuing a sequence; a packed carry word moves lane to lane),
//      resolves escapes and the in-string mask assuming its region is entered
//      outside any string and escape (carries move lane to lane with ballots,
//      step to step in registers), keeps four mask words per lane and step in
//      shared memory and sums the counts into a transfer table: for each of the
//      4 entry states (escape, in-string), the exit state, structural count,
//      bracket count and depth delta.  Steps of 1 KiB of backslashes (inside
//      long backslash runs) change nothing but the escape carry and are
//      skipped early.
//   B. (ticket i, coordinator i % kCoords, while the classifying warps run the
//      next tickets) composes the 16 warp tables into the tile's table,
//      publishes it (decoupled look-back descriptor), finds the tile's
//      exclusive prefix by look-back (64 predecessors per round, loaded in
//      parallel and composed with an ordered shuffle reduction), publishes the
//      inclusive value and derives each warp's entry value.
//   C. (ticket i, after phase A of ticket i + 2) every classifying warp replays
//      its masks with its entry value and writes 1-based structural
//      positions, a zeroed pair row and one bracket record (structural index,
//      level, open flag, brace or bracket) per bracket.
// Hand-offs between the roles are mbarriers (tile_ready, a_done,
// prefix_ready; see Smem) with bounded waits; with three mask slots a
// look-back has two phase A's of slack before the classifying warps wait.
//
// This replaces the reference's stage 1 (checkAscii + checkUTF8,
// cujson/parse_standard_json.cu:186-327) and stage 2 (bitMapCreatorSimd :446,
// findEscapedQuoteMerge_NEW :767, thrust::exclusive_scan :1163,
// inStringFinderBaseline :851, findOutUsefulStringMerge :916, two
// thrust::inclusive_scan + host syncs :1245-1255, removeCopy :954), and the
// depth computation of stage 3 (depth_init_MathAPI :1346 + u8 inclusive_scan
// :1537 + transform_if :1540), in one kernel and one read of the input.
#include <cuda_runtime.h>

#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

namespace cj {

namespace {

constexpr int kStages = 3;                // TMA ring depth per warp
// Per lane and step, four mask words: open brackets, close brackets, `x`
// (curly among brackets, and every other structural: , : and '\n') and the
// structurals that are inside a string when the region is entered outside
// one.  Structurals = open | close | x; brackets = open | close.
constexpr int kMaskFields = 4;
constexpr int kSlots = 3;                 // mask slots: phase C runs two tiles behind phase A
constexpr uint32_t kSpinLimit = 1u << 16; // look-back polls before giving up
constexpr uint32_t kLookSleepMin = 64;    // ns between look-back polls, doubling per poll ...
constexpr uint32_t kLookSleepMax = 1024;  // ... up to this: a waiting look-back costs few issue slots
constexpr int kLookPerLane = 2;           // predecessors per lane and look-back round
constexpr uint32_t kWaitLimit = 1u << 20; // mbarrier polls (each suspends <= kPollNs) before giving up
constexpr uint32_t kPollNs = 1000;
constexpr uint32_t kInputWaitLimit = 1u << 22;   // polls (>= 256 ns each) for input bytes
constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr uint32_t kNoTile = 0xFFFFFFFFu;

// 128-byte aligned: bulk TMA destinations and 16-byte shared loads of every
// warp's ring need (at least) 16-byte aligned stage addresses
struct __align__(128) WarpSmem {
    uint8_t ring[kStages][kStepBytes];
    unsigned long long mbar[kStages];
};
static_assert(sizeof(WarpSmem) % 128 == 0, "warp rings must stay 128-byte aligned");
static_assert(kStepBytes % 16 == 0, "TMA copies need 16-byte multiples");

// everything phase C needs about one tile
struct __align__(16) Slot {
    uint32_t masks[kWarps][kStepsPerWarp][kMaskFields][32];
    Ent wtab[kWarps][4];       // per-warp transfer tables
    Ent wentry[kWarps];        // per-warp entry values (after the look-back)
    uint32_t we[kWarps];       // per-warp flip, then per-warp in-string inversion
};

// A tile as the coordinator hands it out: its ticket and the geometry of its
// segment, so the classifying warps never wait on global loads for them.
struct __align__(16) TileInfo {
    const uint8_t* seg_base;   // the segment's first byte in the device input
    uint64_t tile_off;         // tile start within the segment
    uint64_t seg_len;
    uint64_t seg_log;          // added to byte positions
    uint64_t out_base;         // output index base of the segment
    uint64_t brk_base;         // bracket-record base of the segment
    uint32_t tile;             // kNoTile: no tiles left
    uint32_t segi;
    int32_t tile_len;
    uint32_t flags;            // kTileFirst | kTileLast | kTileImmediate
};
constexpr uint32_t kTileFirst = 1u, kTileLast = 2u, kTileImmediate = 4u;
constexpr int kTickets = 8;    // ticket ring: ticket i lives in info[i % kTickets]
// a coordinator reads tickets i - kCoords + 1 .. i before any warp can have
// finished phase A of ticket i + 3 (see the coordinator loop)
static_assert(kTickets >= kCoords + 3, "ticket ring too short for the coordinators");

struct __align__(128) Smem {
    WarpSmem w[kWarps];
    Slot slot[kSlots];
    TileInfo info[kTickets];
    // hand-offs, all mbarriers (bounded waits; no warp waits on another
    // classifying warp).  The i-th tile a CTA takes is ticket i: its info in
    // info[i % kTickets], its masks in slot[i % kSlots].
    //   tile_ready[i % kTickets]  coordinator -> classifying warps: info is set
    //   a_done[i % kSlots]        classifying warps (one arrival each) -> coordinator
    //   prefix_ready[i % kSlots]  coordinator -> classifying warps: entry values are set
    unsigned long long tile_ready[kTickets], a_done[kSlots], prefix_ready[kSlots];
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one bulk copy of kStepBytes global -> shared, completing on `bar`
__device__ __forceinline__ void tma_load(void* dst, const void* src, unsigned long long* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_u32(bar)), "r"((uint32_t)kStepBytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"((uint32_t)kStepBytes), "r"(smem_u32(bar)) : "memory");
}

// the run has been given up (some bounded wait expired): every other wait
// then ends at once, so that a stall costs one wait's limit, not one per tile
__device__ __noinline__ bool aborted(const Ctrl* ctrl) {
    return (*reinterpret_cast<const volatile uint32_t*>(&ctrl->error_flags) & CJ_FLAG_TIMEOUT) != 0u;
}

// where a bounded wait gave up (Ctrl::gave_up; the first one is kept)
enum : uint32_t { kGaveTileReady = 1, kGaveADone, kGavePrefixReady, kGaveLookBack, kGaveCopy, kGaveInput };

__device__ __noinline__ void give_up(Ctrl* ctrl, uint32_t where) {
    atomicCAS(&ctrl->gave_up, 0u, where);
    atomicOr(&ctrl->error_flags, CJ_FLAG_TIMEOUT);
}

// bounded wait for phase `parity` of `bar`; false if the limit was hit or (with
// `ctrl`) the run was given up.  Waits for a warp's own bulk copies pass no
// `ctrl`: a copy in flight is always waited for, so no CTA exits with one
// still writing into its shared memory.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, const Ctrl* ctrl) {
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(smem_u32(bar)), "r"(parity), "n"(kPollNs) : "memory");
        if (done) return true;
        if (ctrl && (i & 255u) == 255u && aborted(ctrl)) return false;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void load_table(const uint4* agg, uint32_t tile, Ent t[4]) {
#pragma unroll
    for (int s = 0; s < 4; s++) {
        uint4 v = __ldcg(agg + (size_t)tile * 4 + s);
        t[s].st = v.x; t[s].s = v.y; t[s].k = v.z; t[s].d = (int32_t)v.w;
    }
}

// zero the bytes of a 16-byte chunk at or beyond `valid` (chunk-relative)
__device__ __forceinline__ void mask_chunk(uint4& v, int valid) {
    uint32_t* w = &v.x;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int vb = valid - 4 * k;
        if (vb <= 0) w[k] = 0;
        else if (vb < 4) w[k] &= (1u << (8 * vb)) - 1u;
    }
}

// the info of ticket `tile` (kNoTile past the last tile)
__device__ __forceinline__ void tile_info(const ScanParams& P, uint32_t tile, TileInfo& g) {
    g.tile = tile;
    if (tile == kNoTile) return;
    const uint32_t segi = P.tile_seg ? __ldg(P.tile_seg + tile) : 0u;
    const Segment* sp = P.segs + segi;
    const uint32_t first = __ldg(&sp->first_tile);
    const uint32_t ntiles = __ldg(&sp->n_tiles);
    const uint32_t flags = __ldg(&sp->flags);
    const uint32_t tin = tile - first;
    const uint64_t seg_len = __ldg(&sp->len);
    const uint64_t tile_off = (uint64_t)tin * kTileBytes;
    const uint64_t rem = seg_len - tile_off;
    g.segi = segi;
    g.seg_len = seg_len;
    g.tile_off = tile_off;
    g.tile_len = rem < (uint64_t)kTileBytes ? (int)rem : kTileBytes;
    g.seg_base = P.in + __ldg(&sp->dev_off);
    g.seg_log = __ldg(&sp->logical_off);
    g.out_base = __ldg(&sp->out_base);
    g.brk_base = __ldg(&sp->brk_base);
    g.flags = (tin == 0 ? kTileFirst : 0u) | (tin + 1 == ntiles ? kTileLast : 0u) |
              ((tin == 0 && !(flags & kSegContinue)) ? kTileImmediate : 0u);
}

// bytes of warp `warp`'s region of a tile, and its 1 KiB steps
__device__ __forceinline__ int region_len(const TileInfo& g, int warp) {
    return max(0, min(kWarpBytes, g.tile_len - warp * kWarpBytes));
}

// Lane 0 of a classifying warp: start the bulk copies of the first steps of
// its region into the ring (every stage must be free).
__device__ __forceinline__ void start_region(const TileInfo& g, WarpSmem& W, int warp) {
    const int nsteps = (region_len(g, warp) + kStepBytes - 1) / kStepBytes;
    const uint8_t* reg_src = g.seg_base + g.tile_off + (uint64_t)warp * kWarpBytes;
    fence_proxy_async();
    for (int j = 0; j < kStages && j < nsteps; j++)
        tma_load(W.ring[j], reg_src + (size_t)j * kStepBytes, &W.mbar[j]);
}

// the 4 input bytes before warp `warp`'s region of a tile (0 at a segment start)
__device__ __forceinline__ uint32_t region_prev_word(const TileInfo& g, int warp) {
    const uint64_t off = g.tile_off + (uint64_t)warp * kWarpBytes;
    return (off > 0 && region_len(g, warp) > 0)
               ? __ldg(reinterpret_cast<const uint32_t*>(g.seg_base + off) - 1) : 0u;
}

// Phase A of one warp's region: classify, validate, resolve strings, keep masks.
// `prev_word` holds region_prev_word (the 4 input bytes before the region).
template <bool LINES>
__device__ __forceinline__ void phase_a(const ScanParams& P, const TileInfo& g, WarpSmem& W, Slot& sl,
                                        uint32_t& parity, int warp, int lane, uint32_t lt, uint32_t prev_word)
{
    const int reg_off = warp * kWarpBytes;
    const int reg_len = region_len(g, warp);
    const int nsteps = (reg_len + kStepBytes - 1) / kStepBytes;
    const uint8_t* reg_src = g.seg_base + g.tile_off + reg_off;
    if (lane == 0) start_region(g, W, warp);
    uint32_t ucarry = 0;                   // UTF-8 carry into the step (warp uniform)
    uint32_t carry = 0, par = 0;           // escape carry / quote parity (warp uniform)
    uint32_t started = 0, wflip = 0;       // first non-all-backslash lane seen / its flip
    uint32_t in_run = 0;                   // the previous step ended in 32 backslashes
    uint32_t n_c0 = 0, n_ct = 0, n_k0 = 0, n_kt = 0, n_o0 = 0, n_ot = 0;   // per lane
    for (int j = 0; j < nsteps; j++) {
        const int st_i = j % kStages;
        if (!mbar_wait(&W.mbar[st_i], (parity >> st_i) & 1u, nullptr)) {
            if (lane == 0) give_up(P.ctrl, kGaveCopy);
        }
        parity ^= 1u << st_i;
        const int step_len = min(kStepBytes, reg_len - j * kStepBytes);
        const int my0 = lane * kBytesPerThread;
        const int valid = min(kBytesPerThread, step_len - my0);
        // two 16-byte reads (a two-way bank conflict between lanes l and
        // l + 4; rotating the halves to avoid it costs eight selects per step
        // and was measured 1 % slower)
        uint4 lo = *reinterpret_cast<const uint4*>(&W.ring[st_i][my0]);
        uint4 hi = *reinterpret_cast<const uint4*>(&W.ring[st_i][my0 + 16]);
        __syncwarp();
        if (lane == 0 && j + kStages < nsteps) {
            fence_proxy_async();
            tma_load(W.ring[st_i], reg_src + (size_t)(j + kStages) * kStepBytes, &W.mbar[st_i]);
        }
        if (16 > valid) mask_chunk(lo, valid);
        if (32 > valid) mask_chunk(hi, valid - 16);
        const uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        uint32_t (&m)[kMaskFields][32] = sl.masks[warp][j];
        if (in_run) {
            // inside a long backslash run: a step of 1 KiB of backslashes is an
            // even run (the escape carry passes through), opens no UTF-8
            // sequence, and has no quote or structural byte, so the string
            // state and the counts stay and phase C has nothing to write --
            // checked without classifying
            uint32_t d = 0;
#pragma unroll
            for (int k = 0; k < 8; k++) d |= w[k] ^ 0x5C5C5C5Cu;
            if (__all_sync(FULL, d == 0u)) {
                m[0][lane] = 0u; m[1][lane] = 0u; m[2][lane] = 0u; m[3][lane] = 0u;
                ucarry = 0u;
                continue;
            }
        }
        uint32_t planes[8];
        bit_planes32(w, planes);
        const Classes c = classify_planes<LINES>(planes);

        // UTF-8 on the bit planes, on steps that hold a non-ASCII byte or
        // continue a sequence from the bytes before them.  A lane's carry-out
        // depends on its own bytes only, so one shuffle hands it on.
        if (j == 0 && (prev_word & 0x80808000u)) ucarry = utf8_carry_word(prev_word);
        if (__any_sync(FULL, c.hi != 0u) || ucarry != 0u) {
            const uint32_t cout = utf8_carry_planes(planes);
            uint32_t cin = __shfl_up_sync(FULL, cout, 1);
            if (lane == 0) cin = ucarry;
            ucarry = __shfl_sync(FULL, cout, 31);
            if (valid > 0) {
                const bool seg_end = g.tile_off + (uint64_t)(reg_off + j * kStepBytes + my0 + kBytesPerThread) >= g.seg_len;
                if (utf8_errors_planes(planes, cin, seg_end)) {
                    if (P.seg_err) atomicOr(P.seg_err + g.segi, CJ_FLAG_UTF8);
                    else atomicOr(&P.ctrl->error_flags, CJ_FLAG_UTF8);
                }
            }
        } else {
            ucarry = 0u;           // an all-ASCII step opens no sequence
        }

        // escapes: carry from the nearest earlier lane that is not all backslashes
        uint32_t lane_carry;
        if (!__any_sync(FULL, (int32_t)c.bs < 0)) {
            // no lane ends in a backslash: only lane 0 can receive a carry
            lane_carry = (lane == 0) ? carry : 0u;
            in_run = 0;
            if (!started) {
                wflip = __shfl_sync(FULL, (c.q >> (__ffs(~c.bs) - 1)) & 1u, 0);
                started = 1;
            }
            carry = 0;
        } else {
            // an all-backslash lane is an even run and passes its carry
            // through; the carry-outs of all lanes come in one ballot
            const bool all_bs = (c.bs == FULL);
            const uint32_t nonall = __ballot_sync(FULL, !all_bs);
            const uint32_t couts = __ballot_sync(FULL, escape_cout(c.bs) != 0u);
            const uint32_t prior = nonall & lt;
            lane_carry = prior ? (couts >> (31 - __clz(prior))) & 1u : carry;
            if (nonall) {
                if (!started) {
                    // whether the region's first byte after its leading
                    // backslash run is a quote (needed once per region)
                    const uint32_t flipc = all_bs ? 0u : ((c.q >> (__ffs(~c.bs) - 1)) & 1u);
                    wflip = __shfl_sync(FULL, flipc, __ffs(nonall) - 1);
                    started = 1;
                }
                carry = (couts >> (31 - __clz(nonall))) & 1u;
                in_run = (nonall >> 31) ^ 1u;    // lane 31: 32 backslashes
            } else {
                // every byte of the step is a backslash (inside a long run):
                // an even run, so the escape carry passes through, and with
                // no quote or structural byte the string state and counts
                // stay and phase C has nothing to write
                m[0][lane] = 0u; m[1][lane] = 0u; m[2][lane] = 0u; m[3][lane] = 0u;
                in_run = 1;
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
        const uint32_t br = c.br;
        n_c0 += __popc(c.st & ~M); n_ct += __popc(c.st);
        n_k0 += __popc(br & ~M);   n_kt += __popc(br);
        n_o0 += __popc(c.op & ~M); n_ot += __popc(c.op);
        m[0][lane] = c.op;
        m[1][lane] = br & ~c.op;
        m[2][lane] = c.cur | (c.st & ~br);
        m[3][lane] = c.st & M;
    }
    // the warp's transfer table, relative to the state it is entered in
    const int32_t C0 = (int32_t)__reduce_add_sync(FULL, n_c0), Ct = (int32_t)__reduce_add_sync(FULL, n_ct);
    const int32_t K0 = (int32_t)__reduce_add_sync(FULL, n_k0), Kt = (int32_t)__reduce_add_sync(FULL, n_kt);
    const int32_t O0 = (int32_t)__reduce_add_sync(FULL, n_o0), Ot = (int32_t)__reduce_add_sync(FULL, n_ot);
    const int32_t D0 = 2 * O0 - K0, Dt = 2 * Ot - Kt;
    if (lane < 4) {
        const uint32_t escin = (uint32_t)lane >> 1, instr = (uint32_t)lane & 1u;
        const uint32_t e = instr ^ (escin & wflip);
        Ent t;
        t.st = ((started ? carry : escin) << 1) | (e ^ par);
        t.s = (uint32_t)(e ? Ct - C0 : C0);
        t.k = (uint32_t)(e ? Kt - K0 : K0);
        t.d = e ? Dt - D0 : D0;
        sl.wtab[warp][lane] = t;
        if (lane == 0) {
            sl.we[warp] = wflip;
        }
    }
}

__device__ __forceinline__ Ent shfl_ent(Ent e, int src) {
    Ent r;
    r.st = __shfl_sync(FULL, e.st, src);
    r.s = __shfl_sync(FULL, e.s, src);
    r.k = __shfl_sync(FULL, e.k, src);
    r.d = __shfl_sync(FULL, e.d, src);
    return r;
}

__device__ __forceinline__ Ent shfl_up_ent(Ent e, int o) {
    Ent r;
    r.st = __shfl_up_sync(FULL, e.st, o);
    r.s = __shfl_up_sync(FULL, e.s, o);
    r.k = __shfl_up_sync(FULL, e.k, o);
    r.d = __shfl_up_sync(FULL, e.d, o);
    return r;
}

// Coordinator, whole warp: given the slot's exclusive prefix `excl` and its
// table T, publish the inclusive value (lane 0) and set every classifying
// warp's entry value, lane w for warp w from its exclusive prefix table pre.
__device__ __forceinline__ void finish_prefix(const ScanParams& P, const TileInfo& g, Slot& sl, Ent excl,
                                              const Ent T[4], const Ent pre[4], uint32_t ep, int lane)
{
    const Ent incl = ent_apply(excl, T);
    if (lane == 0) {
        // the release store orders the descriptor before the flag
        __stcg(P.desc_incl + g.tile, make_uint4(incl.st, incl.s, incl.k, (uint32_t)incl.d));
        st_release(P.desc_flag + g.tile, (ep << 2) | kFlagIncl);
        if (g.flags & kTileLast) {
            SegmentOut so;
            so.s_end = incl.s;
            so.k_end = incl.k;
            so.depth_end = incl.d;
            so.instr_end = incl.st & 1u;
            P.seg_out[g.segi] = so;
            if (incl.d != 0) {
                if (P.seg_err) atomicOr(P.seg_err + g.segi, CJ_FLAG_BRACKETS);
                else atomicOr(&P.ctrl->error_flags, CJ_FLAG_BRACKETS);
            }
        }
        if (g.tile + 1 == P.n_tiles) {
            P.ctrl->s_total = incl.s;
            P.ctrl->k_total = incl.k;
        }
    }
    Ent v = excl;
    if (g.flags & kTileFirst) { v.st = 0; v.d = 0; }
    if (lane < kWarps) {
        const Ent e = ent_apply(v, pre);
        const uint32_t es = e.st & 3u;
        sl.wentry[lane] = e;
        sl.we[lane] = (es & 1u) ^ ((es >> 1) & sl.we[lane]);   // e = instr ^ (esc & flip)
    }
}

// Warp 0: decoupled look-back for the slot's tile; returns the exclusive
// prefix (valid in lane 0).
__device__ __forceinline__ Ent look_back(const ScanParams& P, uint32_t tile, uint32_t ep, int lane)
{
    // Each round inspects kLookBack = 32 * kLookPerLane predecessors; lane l
    // covers indices l*kLookPerLane .. +kLookPerLane-1 (index i is tile
    // pred_hi - i).  Flags first, then -- once no predecessor before the
    // nearest inclusive one is still unpublished -- the aggregate tables below
    // it and that inclusive value, all loaded in parallel.
    constexpr int R = kLookPerLane;
    Ent acc[4];
    tab_identity(acc);
    int64_t pred_hi = (int64_t)tile - 1;
    uint32_t spins = 0, sleep_ns = kLookSleepMin;
    while (true) {
        uint32_t st_bits = 0;           // 2 bits per index: status
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int64_t p = pred_hi - (lane * R + r);
            uint32_t status = kFlagIncl;
            if (p >= 0) {
                const uint32_t f = ld_acquire(P.desc_flag + p);
                status = ((f >> 2) == ep) ? (f & 3u) : 0u;
            }
            st_bits |= status << (2 * r);
        }
        int r_incl = R, r_notr = R;
#pragma unroll
        for (int r = R - 1; r >= 0; r--) {
            const uint32_t stt = (st_bits >> (2 * r)) & 3u;
            if (stt == kFlagIncl) r_incl = r;
            if (stt == 0u) r_notr = r;
        }
        const uint32_t incl = __ballot_sync(FULL, r_incl < R);
        const int nl = incl ? __ffs(incl) - 1 : 32;                  // lane holding the nearest inclusive
        const int n_incl = __shfl_sync(FULL, r_incl, nl & 31);
        const int lim = (nl == 32) ? R * 32 : nl * R + n_incl;       // indices below use aggregates
        const bool blocked = (lane * R + r_notr) < lim && r_notr < R;
        if (__any_sync(FULL, blocked)) {
            if (++spins > kSpinLimit || ((spins & 255u) == 0u && aborted(P.ctrl))) {
                if (lane == 0) give_up(P.ctrl, kGaveLookBack);
                return ent_identity(0);
            }
            // the look-back has a whole phase A of slack before its entry
            // values are needed, so it backs off rather than polling hard
            __nanosleep(sleep_ns);
            sleep_ns = min(2u * sleep_ns, kLookSleepMax);
            continue;
        }
        // this lane's tables, farthest first, and the inclusive value
        uint4 iv = make_uint4(0, 0, 0, 0);
        if (lane == nl) {
            const int64_t pi = pred_hi - (lane * R + n_incl);
            if (pi >= 0) iv = __ldcg(P.desc_incl + pi);     // before tile 0: the zero value
        }
        Ent t[4];
        tab_identity(t);
#pragma unroll
        for (int r = R - 1; r >= 0; r--) {
            const int i = lane * R + r;
            if (i < lim) {
                Ent u[4];
                load_table(P.desc_agg, (uint32_t)(pred_hi - i), u);
                tab_compose(t, u, t);
            }
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            Ent u[4];
#pragma unroll
            for (int s = 0; s < 4; s++) {
                u[s].st = __shfl_down_sync(FULL, t[s].st, o);
                u[s].s = __shfl_down_sync(FULL, t[s].s, o);
                u[s].k = __shfl_down_sync(FULL, t[s].k, o);
                u[s].d = __shfl_down_sync(FULL, t[s].d, o);
            }
            if (lane + o < 32) tab_compose(u, t, t);
        }
        if (incl) {
            iv.x = __shfl_sync(FULL, iv.x, nl);
            iv.y = __shfl_sync(FULL, iv.y, nl);
            iv.z = __shfl_sync(FULL, iv.z, nl);
            iv.w = __shfl_sync(FULL, iv.w, nl);
            Ent v;
            v.st = iv.x; v.s = iv.y; v.k = iv.z; v.d = (int32_t)iv.w;
            return ent_apply(ent_apply(v, t), acc);
        }
        tab_compose(t, acc, acc);
        pred_hi -= 32 * R;
    }
}

// Phase C of one warp's region.
__device__ __forceinline__ void phase_c(const ScanParams& P, const TileInfo& g, const Slot& sl,
                                        int warp, int lane)
{
    const int reg_off = warp * kWarpBytes;
    const int reg_len = region_len(g, warp);
    const int nsteps = (reg_len + kStepBytes - 1) / kStepBytes;
    const uint64_t seg_log = g.seg_log;
    const uint64_t seg_outb = g.out_base;
    const uint64_t seg_brkb = g.brk_base;
    const Ent entry = sl.wentry[warp];
    const uint32_t flip = sl.we[warp] ? FULL : 0u;
    uint32_t s_base = entry.s, k_base = entry.k;
    int32_t d_base = entry.d;
    int32_t* __restrict__ pos = P.pos + seg_outb;
    int32_t* __restrict__ pair = P.pair + seg_outb;
    uint2* __restrict__ brk = P.brk + seg_brkb;
    const uint64_t pos_base = seg_log + g.tile_off + (uint64_t)reg_off + (uint64_t)lane * kBytesPerThread + 1u;
    for (int j = 0; j < nsteps; j++) {
        const uint32_t (&m)[kMaskFields][32] = sl.masks[warp][j];
        const uint32_t opw = m[0][lane], brw = opw | m[1][lane], xw = m[2][lane];
        uint32_t stm = (brw | xw) & ~(m[3][lane] ^ flip);
        if (!__any_sync(FULL, stm)) continue;      // nothing outside strings in this step
        const uint32_t brm = brw & stm;
        const uint32_t opm = opw & stm;
        const uint32_t curm = xw & brw;
        // the three counts (each <= 32 per lane) packed in 10-bit fields: one
        // scan; exclusive prefixes stay <= 31 * 32 < 1024 per field
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
        uint32_t r = s_base + e1, kr = k_base + e2;
        int32_t depth = d_base + 2 * (int32_t)e3 - (int32_t)e2;
        const uint64_t pos0 = pos_base + (uint64_t)j * kStepBytes;
        while (stm) {
            const int b = __ffs(stm) - 1;
            stm &= stm - 1u;
            pos[r] = (int32_t)(pos0 + (uint64_t)b);
            pair[r] = 0;
            if ((brm >> b) & 1u) {
                const uint32_t is_open = (opm >> b) & 1u;
                const int32_t lvl = is_open ? depth : depth - 1;
                depth += is_open ? 1 : -1;
                const uint32_t cur = ((curm >> b) & 1u) ? kCurly : 0u;
                brk[kr] = make_uint2(r | cur, ((uint32_t)lvl << 1) | is_open);
                kr++;
            }
            r++;
        }
        s_base += n1;
        k_base += n2;
        d_base += 2 * (int32_t)n3 - (int32_t)n2;
    }
}

}  // namespace

size_t scan_smem_bytes() { return sizeof(Smem); }

// Coordinator lane 0: the next tile from the ticket counter and its info,
// once its input bytes are in device memory (bounded wait; the timeout flag
// on expiry).
__device__ __forceinline__ void draw_tile(const ScanParams& P, TileInfo& g)
{
    const uint32_t t = atomicAdd(&P.ctrl->tile_ticket, 1u);
    tile_info(P, t < P.n_tiles ? t : kNoTile, g);
    if (g.tile == kNoTile || !P.ready) return;
    const uint64_t padded = (g.seg_len + kPadBytes - 1) / kPadBytes * kPadBytes;
    const uint64_t end = g.tile_off + (uint64_t)kTileBytes;
    const uint64_t need = (uint64_t)(g.seg_base - P.in) + (end < padded ? end : padded);
    const uint32_t limit = P.input_wait_limit ? P.input_wait_limit : kInputWaitLimit;
    uint32_t spins = 0;
    while (ld_acquire64(P.ready) < need) {
        if (++spins > limit || ((spins & 255u) == 0u && aborted(P.ctrl))) {
            give_up(P.ctrl, kGaveInput);
            break;
        }
        __nanosleep(256);
    }
}

template <bool LINES>
__global__ void __launch_bounds__(kThreads, 1) scan_kernel(ScanParams P)
{
    extern __shared__ __align__(128) uint8_t smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t ep = P.epoch & 0x3FFFFFFFu;

    if (warp < kWarps && lane == 0) {
        for (int s = 0; s < kStages; s++) mbar_init(&S.w[warp].mbar[s], 1);
        fence_mbar_init();
    }
    if (warp == kWarps && lane == 0) {
        for (int k = 0; k < kTickets; k++) mbar_init(&S.tile_ready[k], 1);
        for (int s = 0; s < kSlots; s++) {
            mbar_init(&S.a_done[s], kWarps);
            mbar_init(&S.prefix_ready[s], 1);
        }
        fence_mbar_init();
    }
    __syncthreads();

    if (warp >= kWarps) {
        // ---- coordinators: hand out tiles, publish, look back, derive entries --------
        // Coordinator c resolves tickets c, c + kCoords, ...: a tile's
        // look-back and composition may take kCoords phase A's without
        // holding up the tiles after it.  Ticket i + 1 is drawn by ticket i's
        // coordinator as soon as every warp has finished phase A of ticket i,
        // so tiles are taken in the order their phase A begins and a
        // look-back rarely waits on a predecessor that has not started.
        const uint32_t c = (uint32_t)(warp - kWarps);
        if (c == 0 && lane == 0) {
            draw_tile(P, S.info[0]);
            mbar_arrive(&S.tile_ready[0]);
        }
        __syncwarp();
        for (uint32_t i = c;; i += kCoords) {
            // ticket t + 1 is drawn after phase A of ticket t, and only if
            // ticket t is a tile: walk the tickets since this coordinator's
            // previous one (always drawn) up to i, and stop at the first one
            // past the last tile.  A ticket t read here is overwritten at the
            // earliest by ticket t + kTickets, drawn after phase A of ticket
            // t + kTickets - 1 >= i + 3, which every warp runs after phase C
            // of ticket i, i.e. after this coordinator has resolved ticket i.
            bool more = true;
            for (uint32_t t = (i >= kCoords - 1 ? i - (kCoords - 1) : 0u); more && t <= i; t++) {
                if (!__shfl_sync(FULL, mbar_wait(&S.tile_ready[t % kTickets], (t / kTickets) & 1u, P.ctrl), 0)) {
                    if (lane == 0) give_up(P.ctrl, kGaveTileReady);
                    more = false;
                } else if (S.info[t % kTickets].tile == kNoTile) {
                    more = false;
                }
            }
            if (!more) break;
            const TileInfo& g = S.info[i % kTickets];
            const uint32_t tile = g.tile;
            if (tile == kNoTile) break;
            const uint32_t s = i % kSlots;
            Slot& sl = S.slot[s];
            if (!mbar_wait(&S.a_done[s], (i / kSlots) & 1u, P.ctrl) && lane == 0) give_up(P.ctrl, kGaveADone);
            if (lane == 0) {
                // info[(i + 1) % kTickets] last held ticket i + 1 - kTickets,
                // whose phase C ended before any warp's phase A of ticket i
                // began, and which every coordinator has read
                draw_tile(P, S.info[(i + 1) % kTickets]);
                mbar_arrive(&S.tile_ready[(i + 1) % kTickets]);
            }
            // inclusive scan of the 16 warp tables over lanes 0..15, then the
            // tile's table (lane 15) and each warp's exclusive prefix table
            Ent t[4];
            if (lane < kWarps) {
#pragma unroll
                for (int k = 0; k < 4; k++) t[k] = sl.wtab[lane][k];
            } else {
                tab_identity(t);
            }
#pragma unroll
            for (int o = 1; o < kWarps; o <<= 1) {
                Ent u[4];
#pragma unroll
                for (int k = 0; k < 4; k++) u[k] = shfl_up_ent(t[k], o);
                if (lane >= o) tab_compose(u, t, t);
            }
            Ent T[4], pre[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                T[k] = shfl_ent(t[k], kWarps - 1);
                pre[k] = shfl_up_ent(t[k], 1);
            }
            if (lane == 0) tab_identity(pre);
            if (g.flags & kTileFirst) {
                // a segment starts outside strings and escapes, at depth 0
                const Ent t0 = T[0];
#pragma unroll
                for (int k = 0; k < 4; k++) { T[k] = t0; T[k].st |= 4u; }
            }
            Ent excl = ent_identity(0);
            if (!(g.flags & kTileImmediate)) {
                if (lane == 0) {
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        __stcg(P.desc_agg + (size_t)tile * 4 + k,
                               make_uint4(T[k].st, T[k].s, T[k].k, (uint32_t)T[k].d));
                    st_release(P.desc_flag + tile, (ep << 2) | kFlagAgg);
                }
                excl = shfl_ent(look_back(P, tile, ep, lane), 0);
            }
            finish_prefix(P, g, sl, excl, T, pre, ep, lane);
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.prefix_ready[s]);
            __syncwarp();
        }
        return;
    }

    // ---- classifying warps -----------------------------------------------------------
    // Ticket i: phase A into slot i % kSlots, then phase C of ticket i - 2, so
    // a tile's look-back has two phase A's of slack before its entry values
    // are needed.
    WarpSmem& W = S.w[warp];
    const uint32_t lt = lanemask_lt();
    uint32_t parity = 0;          // bit j: phase parity of ring stage j
    for (uint32_t i = 0;; i++) {
        // a wait that expired (lane 0 decides for the warp) ends the warp's
        // work: the ticket is then not trusted
        const bool got_tile =
            __shfl_sync(FULL, mbar_wait(&S.tile_ready[i % kTickets], (i / kTickets) & 1u, P.ctrl), 0);
        if (!got_tile && lane == 0) give_up(P.ctrl, kGaveTileReady);
        const uint32_t tile = got_tile ? S.info[i % kTickets].tile : kNoTile;
        if (tile != kNoTile) {
            const TileInfo& g = S.info[i % kTickets];
            phase_a<LINES>(P, g, W, S.slot[i % kSlots], parity, warp, lane, lt, region_prev_word(g, warp));
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.a_done[i % kSlots]);
        }
        // phase C of ticket i - 2, and after the last ticket also of i - 1
        const uint32_t c_lo = i >= 2 ? i - 2 : 0u;
        const uint32_t c_hi = (tile == kNoTile) ? i : (i >= 2 ? i - 1 : 0u);
        for (uint32_t k = c_lo; k < c_hi; k++) {
            const uint32_t q = k % kSlots;
            const bool got_prefix =
                __shfl_sync(FULL, mbar_wait(&S.prefix_ready[q], (k / kSlots) & 1u, P.ctrl), 0);
            if (got_prefix) {
                phase_c(P, S.info[k % kTickets], S.slot[q], warp, lane);
            } else if (lane == 0) {
                give_up(P.ctrl, kGavePrefixReady);   // no entry value: no writes
            }
        }
        if (tile == kNoTile) break;
    }
}

template __global__ void scan_kernel<false>(ScanParams);
template __global__ void scan_kernel<true>(ScanParams);

void launch_scan(const ScanParams& p, bool lines, int grid, cudaStream_t stream)
{
    if (p.n_tiles == 0) return;
    const size_t smem = sizeof(Smem);
    if (lines) scan_kernel<true><<<grid, kThreads, smem, stream>>>(p);
    else scan_kernel<false><<<grid, kThreads, smem, stream>>>(p);
}

const void* scan_kernel_ptr() { return (const void*)scan_kernel<false>; }

cudaError_t scan_configure()
{
    const int smem = (int)sizeof(Smem);
    cudaError_t e = cudaFuncSetAttribute(scan_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(scan_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

}  // namespace cj
