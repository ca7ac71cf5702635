// cj_scan.cu -- the single-pass structural scan (persistent, TMA-staged,
// warp-independent).
//
// A persistent grid of CTAs takes 128 KiB tiles in document order from an
// atomic ticket.  Each of the 8 warps of a CTA owns a contiguous 16 KiB region
// of the tile and works through it in 1 KiB steps (32 lanes x 32 bytes),
// staged in its own 3-deep shared-memory ring by bulk TMA copies
// (cp.async.bulk completing on per-warp mbarriers).  Per tile:
//   A. every warp, on its own: builds the quote, backslash, structural and
//      bracket bitmaps of each lane's 32 bytes, validates UTF-8 where
//      non-ASCII bytes occur, resolves escapes and the in-string mask assuming
//      its region is entered outside any string and escape (the carries move
//      lane to lane with ballots and shuffles, step to step in registers), keeps
//      the masks in shared memory and sums the counts.  Its result is a
//      transfer table: for each of the 4 entry states (escape, in-string), the
//      exit state, structural count, bracket count and depth delta.
//   B. warp 0 composes the 8 warp tables into the tile's table, publishes it,
//      and finds the tile's exclusive prefix by decoupled look-back
//      (32 predecessors per step, loaded in parallel, composed with an ordered
//      shuffle reduction); then derives each warp's entry value.
//   C. every warp replays its masks with its now known entry value and writes
//      1-based structural positions, a zeroed pair row, and one bracket record
//      (structural index, level, open flag, brace or bracket) per bracket.
// Only three CTA-wide barriers per tile.
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
constexpr int kMaskFields = 5;            // st, br, op, cur, M per lane per step
constexpr uint32_t kSpinLimit = 1u << 22; // look-back polls before giving up
constexpr uint32_t kWaitLimit = 1u << 20; // mbarrier polls before giving up
constexpr uint32_t FULL = 0xFFFFFFFFu;

// 128-byte aligned: bulk TMA destinations and 16-byte shared loads of every
// warp's ring need (at least) 16-byte aligned stage addresses
struct __align__(128) WarpSmem {
    uint8_t ring[kStages][kStepBytes];
    uint32_t masks[kStepsPerWarp][kMaskFields][32];
    unsigned long long mbar[kStages];
};
static_assert(sizeof(WarpSmem) % 128 == 0, "warp rings must stay 128-byte aligned");
static_assert(kStepBytes % 16 == 0, "TMA copies need 16-byte multiples");

struct __align__(128) Smem {
    WarpSmem w[kWarps];
    Ent wtab[kWarps][4];       // per-warp transfer tables
    Ent wentry[kWarps];        // per-warp entry values (after the look-back)
    uint32_t we[kWarps];       // per-warp flip, then per-warp in-string inversion
    uint32_t tile;
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

// bounded wait for phase `parity` of `bar`; false if the limit was hit
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void load_table(const uint4* agg, uint32_t tile, Ent t[4]) {
#pragma unroll
    for (int s = 0; s < 4; s++) {
        uint4 v = __ldcg(agg + (size_t)tile * 4 + s);
        t[s].st = v.x; t[s].s = v.y; t[s].k = v.z; t[s].d = (int32_t)v.w;
    }
}

// length of the sequence a lead byte starts (1 for ASCII, 0 for
// continuations and the bytes that never start a sequence: C0, C1, F5-FF)
__device__ __forceinline__ int lead_len(uint32_t b) {
    if (b < 0x80) return 1;
    if (b >= 0xC2 && b <= 0xDF) return 2;
    if (b >= 0xE0 && b <= 0xEF) return 3;
    if (b >= 0xF0 && b <= 0xF4) return 4;
    return 0;
}

// continuation bytes still owed at the start of a lane's 32 bytes, given the
// four bytes before them (`pw`, little endian: byte 3 is the one just before)
__device__ __forceinline__ int utf8_owed(uint32_t pw) {
    if ((pw & 0x80808000u) == 0) return 0;
#pragma unroll
    for (int k = 1; k <= 3; k++) {
        const uint32_t b = (pw >> (8 * (4 - k))) & 0xFFu;
        if ((b & 0xC0u) == 0x80u) continue;
        const int L = lead_len(b);
        return L > k ? L - k : 0;
    }
    return 0;
}

// RFC 3629 check of one lane's bytes tb[0..valid) (valid <= 32), the four
// bytes before them in `pw`.  Only the non-ASCII bytes (`na`, bit j = byte j)
// and the bytes owed to a lead in `pw` are visited: a continuation byte must lie
// inside the span of the lead 1-3 bytes before it (and, as the second byte of
// an E0 / ED / F0 / F4 sequence, inside the restricted range); a lead must be
// followed by continuation bytes inside this lane's range, and a sequence
// running past the range is checked by the next lane through its `pw` -- or
// fails here when the segment ends first (`seg_end`).
__device__ __noinline__ bool utf8_ok(const uint8_t* tb, int valid, uint32_t pw, uint32_t na,
                                     bool seg_end) {
    const int owed = utf8_owed(pw);
    for (int p = 0; p < owed; p++)
        if (p >= valid || (tb[p] & 0xC0u) != 0x80u) return false;
    while (na) {
        const int p = __ffs(na) - 1;
        na &= na - 1u;
        const uint32_t b = tb[p];
        if ((b & 0xC0u) == 0x80u) {
            int k = 1;
            uint32_t lb = 0;
            for (; k <= 3; k++) {
                lb = (p - k >= 0) ? tb[p - k] : ((pw >> (8 * (4 + p - k))) & 0xFFu);
                if ((lb & 0xC0u) != 0x80u) break;
            }
            if (k > 3 || lead_len(lb) <= k) return false;
            if (k == 1) {
                if (lb == 0xE0u && b < 0xA0u) return false;
                if (lb == 0xEDu && b > 0x9Fu) return false;
                if (lb == 0xF0u && b < 0x90u) return false;
                if (lb == 0xF4u && b > 0x8Fu) return false;
            }
            continue;
        }
        const int L = lead_len(b);
        if (L == 0) return false;
        for (int i = 1; i < L; i++) {
            const int q = p + i;
            if (q >= 32) { if (seg_end) return false; break; }
            if (q >= valid) return false;
            if ((tb[q] & 0xC0u) != 0x80u) return false;
        }
    }
    return true;
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

// inclusive warp scan of three counters
__device__ __forceinline__ void warp_scan3(uint32_t& a, uint32_t& b, uint32_t& c, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t ta = __shfl_up_sync(FULL, a, o);
        uint32_t tb = __shfl_up_sync(FULL, b, o);
        uint32_t tc = __shfl_up_sync(FULL, c, o);
        if (lane >= o) { a += ta; b += tb; c += tc; }
    }
}

}  // namespace

size_t scan_smem_bytes() { return sizeof(Smem); }

template <bool LINES>
__global__ void __launch_bounds__(kThreads, 2) scan_kernel(ScanParams P)
{
    extern __shared__ __align__(128) uint8_t smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    WarpSmem& W = S.w[warp];
    const uint32_t lt = lanemask_lt();
    const uint32_t ep = P.epoch & 0x3FFFFFFFu;

    if (lane == 0) {
        for (int s = 0; s < kStages; s++) mbar_init(&W.mbar[s], 1);
        fence_mbar_init();
    }
    __syncwarp();
    uint32_t parity = 0;   // bit s: phase parity to wait for on stage s

    while (true) {
        if (tid == 0) S.tile = atomicAdd(&P.ctrl->tile_ticket, 1u);
        __syncthreads();
        const uint32_t tile = S.tile;
        if (tile >= P.n_tiles) break;

        const uint32_t segi = P.tile_seg ? __ldg(P.tile_seg + tile) : 0u;
        const Segment* sp = P.segs + segi;
        const uint64_t seg_dev = __ldg(&sp->dev_off);
        const uint64_t seg_len = __ldg(&sp->len);
        const uint32_t seg_first_tile = __ldg(&sp->first_tile);
        const uint32_t seg_ntiles = __ldg(&sp->n_tiles);
        const uint32_t seg_flags = __ldg(&sp->flags);
        const uint32_t tin = tile - seg_first_tile;
        const uint64_t tile_off = (uint64_t)tin * kTileBytes;
        const uint64_t rem = seg_len - tile_off;
        const int tile_len = rem < (uint64_t)kTileBytes ? (int)rem : kTileBytes;
        const bool seg_first = (tin == 0);
        const bool seg_last = (tin + 1 == seg_ntiles);
        const bool immediate = seg_first && !(seg_flags & kSegContinue);
        const uint8_t* seg_base = P.in + seg_dev;
        const int reg_off = warp * kWarpBytes;                       // within the tile
        const int reg_len = max(0, min(kWarpBytes, tile_len - reg_off));
        const int nsteps = (reg_len + kStepBytes - 1) / kStepBytes;
        const uint8_t* reg_src = seg_base + tile_off + reg_off;

        if (lane == 0) {
            fence_proxy_async();
            for (int j = 0; j < kStages && j < nsteps; j++)
                tma_load(W.ring[j], reg_src + (size_t)j * kStepBytes, &W.mbar[j]);
        }

        // ---- A. this warp's region ---------------------------------------------
        uint32_t carry = 0, par = 0;           // escape carry / quote parity (warp uniform)
        uint32_t started = 0, wflip = 0;       // first non-all-backslash lane seen / its flip
        uint32_t prev_last = (tile_off + (uint64_t)reg_off > 0 && nsteps > 0)
                                 ? __ldg(reinterpret_cast<const uint32_t*>(reg_src) - 1) : 0u;
        uint32_t n_c0 = 0, n_ct = 0, n_k0 = 0, n_kt = 0, n_o0 = 0, n_ot = 0;   // per lane
        for (int j = 0; j < nsteps; j++) {
            const int st_i = j % kStages;
            if (!mbar_wait(&W.mbar[st_i], (parity >> st_i) & 1u)) {
                if (lane == 0) atomicOr(&P.ctrl->error_flags, CJ_FLAG_TIMEOUT);
            }
            parity ^= 1u << st_i;
            const int step_len = min(kStepBytes, reg_len - j * kStepBytes);
            const int my0 = lane * kBytesPerThread;
            const int valid = min(kBytesPerThread, step_len - my0);
            // two 16-byte reads, chunk order rotated per lane group so the eight
            // lanes of each shared-memory wavefront touch distinct banks
            Classes c;
            c.q = c.bs = c.st = c.op = c.cl = c.cur = c.hi = 0;
            uint32_t last_word = 0, na = 0;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const int r = k ^ ((lane >> 2) & 1);
                uint4 v = *reinterpret_cast<const uint4*>(&W.ring[st_i][my0 + 16 * r]);
                if (16 * r + 16 > valid) mask_chunk(v, valid - 16 * r);
                if (r == 1) last_word = v.w;
                const uint32_t w[4] = {v.x, v.y, v.z, v.w};
                const Classes h = classify16<LINES>(w);
                const int sh = 16 * r;
                c.q |= h.q << sh; c.bs |= h.bs << sh; c.st |= h.st << sh;
                c.op |= h.op << sh; c.cl |= h.cl << sh; c.cur |= h.cur << sh;
                if (h.hi) {
#pragma unroll
                    for (int q = 0; q < 4; q++) na |= gather4(w[q] & 0x80808080u) << (sh + 4 * q);
                }
            }
            // UTF-8 (before the stage is handed back to the TMA engine)
            {
                uint32_t pw = __shfl_up_sync(FULL, last_word, 1);
                if (lane == 0) pw = prev_last;
                if (valid > 0 && (na || (pw & 0x80808000u))) {
                    const bool seg_end = tile_off + (uint64_t)(reg_off + j * kStepBytes + my0 + kBytesPerThread) >= seg_len;
                    if (!utf8_ok(&W.ring[st_i][my0], valid, pw, na, seg_end))
                        atomicOr(&P.ctrl->error_flags, CJ_FLAG_UTF8);
                }
                prev_last = __shfl_sync(FULL, last_word, 31);
            }
            __syncwarp();
            if (lane == 0 && j + kStages < nsteps) {
                fence_proxy_async();
                tma_load(W.ring[st_i], reg_src + (size_t)(j + kStages) * kStepBytes, &W.mbar[st_i]);
            }

            // escapes: carry from the nearest earlier lane that is not all backslashes
            uint32_t cout0;
            (void)escaped32(c.bs, 0u, &cout0);
            const bool all_bs = (c.bs == FULL);
            const uint32_t nonall = __ballot_sync(FULL, !all_bs);
            const uint32_t prior = nonall & lt;
            const uint32_t cin_lane = __shfl_sync(FULL, cout0, prior ? 31 - __clz(prior) : 0);
            const uint32_t lane_carry = prior ? cin_lane : carry;
            const uint32_t flipc = all_bs ? 0u : ((c.q >> (__ffs(~c.bs) - 1)) & 1u);
            const uint32_t first_flip = __shfl_sync(FULL, flipc, nonall ? __ffs(nonall) - 1 : 0);
            const uint32_t last_cout = __shfl_sync(FULL, cout0, nonall ? 31 - __clz(nonall) : 0);
            if (nonall) {
                if (!started) wflip = first_flip;
                started = 1;
                carry = last_cout;
            }
            uint32_t dummy;
            const uint32_t esc = escaped32(c.bs, lane_carry, &dummy);
            const uint32_t rq = c.q & ~esc;
            const uint32_t qb = __ballot_sync(FULL, __popc(rq) & 1u);
            const uint32_t lpar = par ^ (__popc(qb & lt) & 1u);
            par ^= __popc(qb) & 1u;
            const uint32_t M = prefix_xor(rq) ^ (lpar ? FULL : 0u);
            const uint32_t br = c.op | c.cl;
            n_c0 += __popc(c.st & ~M); n_ct += __popc(c.st);
            n_k0 += __popc(br & ~M);   n_kt += __popc(br);
            n_o0 += __popc(c.op & ~M); n_ot += __popc(c.op);
            W.masks[j][0][lane] = c.st;
            W.masks[j][1][lane] = br;
            W.masks[j][2][lane] = c.op;
            W.masks[j][3][lane] = c.cur;
            W.masks[j][4][lane] = M;
        }
        {
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
                S.wtab[warp][lane] = t;
                if (lane == 0) S.we[warp] = wflip;
            }
        }
        __syncthreads();

        // ---- B. tile table and decoupled look-back (warp 0) ------------------------
        if (warp == 0) {
            Ent T[4];
            tab_identity(T);
#pragma unroll
            for (int v = 0; v < kWarps; v++) tab_compose(T, S.wtab[v], T);
            if (seg_first) {
                // a segment starts outside strings and escapes, at depth 0
                const Ent t0 = T[0];
#pragma unroll
                for (int s = 0; s < 4; s++) { T[s] = t0; T[s].st |= 4u; }
            }
            Ent excl = ent_identity(0);
            if (!immediate) {
                if (lane == 0) {
#pragma unroll
                    for (int s = 0; s < 4; s++)
                        __stcg(P.desc_agg + (size_t)tile * 4 + s,
                               make_uint4(T[s].st, T[s].s, T[s].k, (uint32_t)T[s].d));
                    __threadfence();
                    st_release(P.desc_flag + tile, (ep << 2) | kFlagAgg);
                }
                Ent acc[4];
                tab_identity(acc);
                int64_t pred_hi = (int64_t)tile - 1;
                uint32_t spins = 0;
                while (true) {
                    const int64_t p = pred_hi - lane;
                    uint32_t status = kFlagIncl;
                    if (p >= 0) {
                        uint32_t f = ld_acquire(P.desc_flag + p);
                        status = ((f >> 2) == ep) ? (f & 3u) : 0u;
                    }
                    const uint32_t incl = __ballot_sync(FULL, status == kFlagIncl);
                    const uint32_t notr = __ballot_sync(FULL, status == 0u);
                    const int n = incl ? __ffs(incl) - 1 : 32;
                    const uint32_t below = (n == 32) ? FULL : ((1u << n) - 1u);
                    if (notr & below) {
                        if (++spins > kSpinLimit) {
                            if (lane == 0) atomicOr(&P.ctrl->error_flags, CJ_FLAG_TIMEOUT);
                            excl = ent_identity(0);
                            break;
                        }
                        __nanosleep(32);
                        continue;
                    }
                    Ent t[4];
                    if (lane < n) load_table(P.desc_agg, (uint32_t)p, t);
                    else tab_identity(t);
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
                        uint4 iv = make_uint4(0, 0, 0, 0);
                        if (lane == n) iv = __ldcg(P.desc_incl + p);
                        iv.x = __shfl_sync(FULL, iv.x, n);
                        iv.y = __shfl_sync(FULL, iv.y, n);
                        iv.z = __shfl_sync(FULL, iv.z, n);
                        iv.w = __shfl_sync(FULL, iv.w, n);
                        Ent v;
                        v.st = iv.x; v.s = iv.y; v.k = iv.z; v.d = (int32_t)iv.w;
                        excl = ent_apply(ent_apply(v, t), acc);   // valid in lane 0
                        break;
                    }
                    tab_compose(t, acc, acc);
                    pred_hi -= 32;
                }
            }
            if (lane == 0) {
                const Ent incl = ent_apply(excl, T);
                __stcg(P.desc_incl + tile, make_uint4(incl.st, incl.s, incl.k, (uint32_t)incl.d));
                __threadfence();
                st_release(P.desc_flag + tile, (ep << 2) | kFlagIncl);
                Ent v = excl;
                if (seg_first) { v.st = 0; v.d = 0; }
                for (int w = 0; w < kWarps; w++) {
                    const uint32_t es = v.st & 3u;
                    S.wentry[w] = v;
                    S.we[w] = (es & 1u) ^ ((es >> 1) & S.we[w]);   // e = instr ^ (esc & flip)
                    v = ent_apply(v, S.wtab[w]);
                }
                if (seg_last) {
                    SegmentOut so;
                    so.s_end = incl.s;
                    so.k_end = incl.k;
                    so.depth_end = incl.d;
                    so.instr_end = incl.st & 1u;
                    P.seg_out[segi] = so;
                    if (incl.d != 0) atomicOr(&P.ctrl->error_flags, CJ_FLAG_BRACKETS);
                }
                if (tile + 1 == P.n_tiles) {
                    P.ctrl->s_total = incl.s;
                    P.ctrl->k_total = incl.k;
                }
            }
        }
        __syncthreads();

        // ---- C. this warp's outputs --------------------------------------------------
        {
            const uint64_t seg_log = __ldg(&sp->logical_off);
            const uint64_t seg_outb = __ldg(&sp->out_base);
            const uint64_t seg_brkb = __ldg(&sp->brk_base);
            const Ent entry = S.wentry[warp];
            const uint32_t flip = S.we[warp] ? FULL : 0u;
            uint32_t s_base = entry.s, k_base = entry.k;
            int32_t d_base = entry.d;
            int32_t* __restrict__ pos = P.pos + seg_outb;
            int32_t* __restrict__ pair = P.pair + seg_outb;
            uint2* __restrict__ brk = P.brk + seg_brkb;
            const uint64_t pos_base = seg_log + tile_off + (uint64_t)reg_off + (uint64_t)lane * kBytesPerThread + 1u;
            for (int j = 0; j < nsteps; j++) {
                const uint32_t Mf = W.masks[j][4][lane] ^ flip;
                uint32_t stm = W.masks[j][0][lane] & ~Mf;
                const uint32_t brm = W.masks[j][1][lane] & ~Mf;
                const uint32_t opm = W.masks[j][2][lane] & ~Mf;
                const uint32_t curm = W.masks[j][3][lane];
                const uint32_t own1 = (uint32_t)__popc(stm);
                const uint32_t own2 = (uint32_t)__popc(brm);
                const uint32_t own3 = (uint32_t)__popc(opm);
                uint32_t i1 = own1, i2 = own2, i3 = own3;
                warp_scan3(i1, i2, i3, lane);
                const uint32_t n1 = __shfl_sync(FULL, i1, 31), n2 = __shfl_sync(FULL, i2, 31),
                               n3 = __shfl_sync(FULL, i3, 31);
                uint32_t r = s_base + i1 - own1, kr = k_base + i2 - own2;
                int32_t depth = d_base + 2 * (int32_t)(i3 - own3) - (int32_t)(i2 - own2);
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
        // the next ticket's barrier separates these reads from the next tile's writes
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
