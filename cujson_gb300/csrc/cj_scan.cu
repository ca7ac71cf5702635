// cj_scan.cu -- the single-pass structural scan.
//
// One CTA per 8 KiB tile (256 threads x 32 bytes), tiles taken in launch order
// from an atomic ticket.  Per tile:
//   1. load 32 bytes per thread and build the quote, backslash, structural and
//      open/close bitmaps (one 32-bit word per class per thread);
//   2. validate UTF-8 (RFC 3629) where non-ASCII bytes occur;
//   3. resolve escapes and the in-string mask inside the tile, assuming the
//      tile is entered outside any string and escape;
//   4. publish the tile's transfer table (4 entry states -> exit state,
//      structural count, bracket count, depth delta) and find its exclusive
//      prefix by decoupled look-back over the predecessors' tables;
//   5. write 1-based structural positions, a zeroed pair row, and one bracket
//      record (structural index, level, open flag, brace/bracket) per bracket.
//
// This replaces the reference's stage 1 (checkAscii + checkUTF8,
// cujson/parse_standard_json.cu:186-327) and stage 2 (bitMapCreatorSimd :446,
// findEscapedQuoteMerge_NEW :767, thrust::exclusive_scan :1163,
// inStringFinderBaseline :851, findOutUsefulStringMerge :916, two
// thrust::inclusive_scan + host syncs :1245-1255, removeCopy :954), and the
// depth computation of stage 3 (depth_init_MathAPI :1346 + u8 inclusive_scan
// :1537 + transform_if :1540), in one kernel and one read of the input.
#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

namespace cj {

namespace {

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

__device__ __forceinline__ uint4 ld_stream(const uint4* p) {
    uint4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ void load_table(const uint4* agg, uint32_t tile, Ent t[4]) {
#pragma unroll
    for (int s = 0; s < 4; s++) {
        uint4 v = __ldcg(agg + (size_t)tile * 4 + s);
        t[s].st = v.x; t[s].s = v.y; t[s].k = v.z; t[s].d = (int32_t)v.w;
    }
}

__device__ __forceinline__ int lead_len(uint32_t b) {
    if (b >= 0xC2 && b <= 0xDF) return 2;
    if (b >= 0xE0 && b <= 0xEF) return 3;
    if (b >= 0xF0 && b <= 0xF4) return 4;
    return 1;
}

// RFC 3629 check of the sequences touching bytes [o0, o0+32) of a segment:
// every lead must be followed by the right continuation bytes (with the
// restricted second-byte ranges of E0, ED, F0 and F4), and every continuation
// byte must lie inside the span of a lead 1-3 bytes before it.
__device__ __noinline__ bool utf8_ok32(const uint8_t* sb, uint64_t slen, uint64_t o0) {
    for (int j = 0; j < 32; j++) {
        uint64_t o = o0 + (uint64_t)j;
        if (o >= slen) break;
        uint32_t b = sb[o];
        if (b < 0x80) continue;
        if (b < 0xC0) {
            bool ok = false;
            for (uint64_t k = 1; k <= 3 && k <= o; k++) {
                uint32_t pb = sb[o - k];
                if ((pb & 0xC0) == 0x80) continue;
                ok = lead_len(pb) > (int)k;
                break;
            }
            if (!ok) return false;
            continue;
        }
        int L;
        uint32_t lo = 0x80, hi = 0xBF;
        if (b <= 0xC1) return false;
        else if (b <= 0xDF) L = 2;
        else if (b == 0xE0) { L = 3; lo = 0xA0; }
        else if (b == 0xED) { L = 3; hi = 0x9F; }
        else if (b <= 0xEF) L = 3;
        else if (b == 0xF0) { L = 4; lo = 0x90; }
        else if (b <= 0xF3) L = 4;
        else if (b == 0xF4) { L = 4; hi = 0x8F; }
        else return false;
        if (o + (uint64_t)L > slen) return false;
        uint32_t b1 = sb[o + 1];
        if (b1 < lo || b1 > hi) return false;
        for (int k = 2; k < L; k++)
            if ((sb[o + k] & 0xC0) != 0x80) return false;
    }
    return true;
}

constexpr uint32_t kSpinLimit = 1u << 22;

}  // namespace

template <bool LINES>
__global__ void __launch_bounds__(kThreads) scan_kernel(ScanParams P)
{
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_w_nonall[kWarps], s_w_cout[kWarps], s_w_flip[kWarps], s_w_qpar[kWarps];
    __shared__ uint32_t s_w_v1[kWarps], s_w_v2[kWarps], s_w_v3[kWarps];
    __shared__ Ent s_excl;
    __shared__ uint32_t s_e;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t FULL = 0xFFFFFFFFu;

    if (tid == 0) s_tile = atomicAdd(&P.ctrl->tile_ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= P.n_tiles) return;

    const uint32_t segi = P.tile_seg ? __ldg(P.tile_seg + tile) : 0u;
    const Segment* sp = P.segs + segi;
    const uint64_t seg_dev = __ldg(&sp->dev_off);
    const uint64_t seg_len = __ldg(&sp->len);
    const uint64_t seg_log = __ldg(&sp->logical_off);
    const uint64_t seg_outb = __ldg(&sp->out_base);
    const uint64_t seg_brkb = __ldg(&sp->brk_base);
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

    // ---- 1. load and classify -------------------------------------------------
    const int my0 = tid * kBytesPerThread;
    const uint4* tp4 = reinterpret_cast<const uint4*>(seg_base + tile_off) + tid * 2;
    uint4 va = ld_stream(tp4), vb = ld_stream(tp4 + 1);
    uint32_t w[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
    if (my0 + kBytesPerThread > tile_len) {
        int valid = tile_len - my0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            int vbytes = valid - 4 * k;
            if (vbytes <= 0) w[k] = 0;
            else if (vbytes < 4) w[k] &= (1u << (8 * vbytes)) - 1u;
        }
    }
    const Classes c = classify32<LINES>(w);

    // ---- 2. UTF-8 ---------------------------------------------------------------
    if (c.hi) {
        if (!utf8_ok32(seg_base, seg_len, tile_off + (uint64_t)my0))
            atomicOr(&P.ctrl->error_flags, CJ_FLAG_UTF8);
    }

    // ---- 3. escapes and strings inside the tile ------------------------------------
    uint32_t cout0;
    (void)escaped32(c.bs, 0u, &cout0);
    const bool all_bs = (c.bs == FULL);
    const uint32_t first_nb = all_bs ? 0u : (uint32_t)(__ffs(~c.bs) - 1);
    const uint32_t flipc = all_bs ? 0u : ((c.q >> first_nb) & 1u);
    const uint32_t lt = lanemask_lt();
    const uint32_t nonall = __ballot_sync(FULL, !all_bs);
    const uint32_t prior = nonall & lt;
    const uint32_t cin_lane = __shfl_sync(FULL, cout0, prior ? 31 - __clz(prior) : 0);
    const uint32_t wcout = __shfl_sync(FULL, cout0, nonall ? 31 - __clz(nonall) : 0);
    const uint32_t wflip = __shfl_sync(FULL, flipc, nonall ? __ffs(nonall) - 1 : 0);
    if (lane == 0) {
        s_w_nonall[warp] = nonall != 0u;
        s_w_cout[warp] = wcout;
        s_w_flip[warp] = wflip;
    }
    __syncthreads();

    uint32_t wcarry = 0;   // carry into this warp, tile entered without escape
    for (int v = warp - 1; v >= 0; v--)
        if (s_w_nonall[v]) { wcarry = s_w_cout[v]; break; }
    const uint32_t carry = prior ? cin_lane : wcarry;
    uint32_t dummy;
    const uint32_t esc = escaped32(c.bs, carry, &dummy);
    const uint32_t rq = c.q & ~esc;
    const uint32_t qp = __popc(rq) & 1u;
    const uint32_t qb = __ballot_sync(FULL, qp);
    if (lane == 0) s_w_qpar[warp] = __popc(qb) & 1u;
    __syncthreads();

    uint32_t par = __popc(qb & lt) & 1u;
    for (int v = 0; v < warp; v++) par ^= s_w_qpar[v];
    // in-string mask assuming the tile is entered outside a string
    const uint32_t M = prefix_xor(rq) ^ (par ? FULL : 0u);
    const uint32_t br = c.op | c.cl;
    const uint32_t own1 = (uint32_t)__popc(c.st & ~M) | ((uint32_t)__popc(c.st) << 16);
    const uint32_t own2 = (uint32_t)__popc(br & ~M) | ((uint32_t)__popc(br) << 16);
    const uint32_t own3 = (uint32_t)__popc(c.op & ~M) | ((uint32_t)__popc(c.op) << 16);
    uint32_t i1 = own1, i2 = own2, i3 = own3;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t1 = __shfl_up_sync(FULL, i1, o);
        uint32_t t2 = __shfl_up_sync(FULL, i2, o);
        uint32_t t3 = __shfl_up_sync(FULL, i3, o);
        if (lane >= o) { i1 += t1; i2 += t2; i3 += t3; }
    }
    if (lane == 31) { s_w_v1[warp] = i1; s_w_v2[warp] = i2; s_w_v3[warp] = i3; }
    __syncthreads();

    uint32_t pre1 = i1 - own1, pre2 = i2 - own2, pre3 = i3 - own3;
    uint32_t tot1 = 0, tot2 = 0, tot3 = 0;
#pragma unroll
    for (int v = 0; v < kWarps; v++) {
        if (v < warp) { pre1 += s_w_v1[v]; pre2 += s_w_v2[v]; pre3 += s_w_v3[v]; }
        tot1 += s_w_v1[v]; tot2 += s_w_v2[v]; tot3 += s_w_v3[v];
    }

    // ---- 4. transfer table and decoupled look-back (warp 0) ---------------------
    if (warp == 0) {
        uint32_t tall = 1, tcout = 0, tflip = 0, tqpar = 0;
        for (int v = 0; v < kWarps; v++) {
            tqpar ^= s_w_qpar[v];
            if (s_w_nonall[v]) { if (tall) tflip = s_w_flip[v]; tall = 0; tcout = s_w_cout[v]; }
        }
        const int32_t C0 = (int32_t)(tot1 & 0xFFFFu), Ct = (int32_t)(tot1 >> 16);
        const int32_t K0 = (int32_t)(tot2 & 0xFFFFu), Kt = (int32_t)(tot2 >> 16);
        const int32_t O0 = (int32_t)(tot3 & 0xFFFFu), Ot = (int32_t)(tot3 >> 16);
        const int32_t D0 = 2 * O0 - K0, Dt = 2 * Ot - Kt;
        Ent T[4];
        uint32_t Tev[4];
#pragma unroll
        for (uint32_t s = 0; s < 4; s++) {
            uint32_t escin = seg_first ? 0u : (s >> 1);
            uint32_t instr = seg_first ? 0u : (s & 1u);
            uint32_t e = instr ^ (escin & tflip);
            uint32_t oesc = tall ? escin : tcout;
            uint32_t oin = e ^ tqpar;
            T[s].st = (oesc << 1) | oin | (seg_first ? 4u : 0u);
            T[s].s = (uint32_t)(e ? Ct - C0 : C0);
            T[s].k = (uint32_t)(e ? Kt - K0 : K0);
            T[s].d = e ? Dt - D0 : D0;
            Tev[s] = e;
        }

        const uint32_t ep = P.epoch & 0x3FFFFFFFu;
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
            bool done = false;
            while (!done) {
                int64_t p = pred_hi - lane;
                uint32_t status = kFlagIncl;
                if (p >= 0) {
                    uint32_t f = ld_acquire(P.desc_flag + p);
                    status = ((f >> 2) == ep) ? (f & 3u) : 0u;
                }
                uint32_t incl = __ballot_sync(FULL, status == kFlagIncl);
                uint32_t notr = __ballot_sync(FULL, status == 0u);
                if (incl) {
                    int n = __ffs(incl) - 1;
                    if ((notr & ((1u << n) - 1u)) == 0u) {
                        if (lane == 0) {
                            uint4 iv = __ldcg(P.desc_incl + (pred_hi - n));
                            Ent v;
                            v.st = iv.x; v.s = iv.y; v.k = iv.z; v.d = (int32_t)iv.w;
                            for (int i = n - 1; i >= 0; i--) {
                                Ent t[4];
                                load_table(P.desc_agg, (uint32_t)(pred_hi - i), t);
                                v = ent_apply(v, t);
                            }
                            excl = ent_apply(v, acc);
                        }
                        done = true;
                        continue;
                    }
                } else if (notr == 0u) {
                    // 32 aggregates and no inclusive value: fold them and step back
                    if (lane == 0) {
                        Ent wt[4];
                        tab_identity(wt);
                        for (int i = 31; i >= 0; i--) {
                            Ent t[4];
                            load_table(P.desc_agg, (uint32_t)(pred_hi - i), t);
                            tab_compose(wt, t, wt);
                        }
                        tab_compose(wt, acc, acc);
                    }
                    pred_hi -= 32;
                    continue;
                }
                // a nearer predecessor has not published yet
                if (++spins > kSpinLimit) {
                    if (lane == 0) atomicOr(&P.ctrl->error_flags, CJ_FLAG_TIMEOUT);
                    excl = ent_identity(0);
                    done = true;
                } else {
                    __nanosleep(64);
                }
            }
        }
        if (lane == 0) {
            Ent incl = ent_apply(excl, T);
            __stcg(P.desc_incl + tile, make_uint4(incl.st, incl.s, incl.k, (uint32_t)incl.d));
            __threadfence();
            st_release(P.desc_flag + tile, (ep << 2) | kFlagIncl);

            Ent entry = excl;
            if (seg_first) { entry.st = 0; entry.d = 0; }
            s_excl = entry;
            s_e = Tev[entry.st & 3u];
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

    // ---- 5. outputs --------------------------------------------------------------
    const Ent entry = s_excl;
    const uint32_t e = s_e;
    const uint32_t Mf = M ^ (e ? FULL : 0u);
    uint32_t stm = c.st & ~Mf;
    if (!stm) return;
    const uint32_t brm = br & ~Mf;
    const uint32_t opm = c.op & ~Mf;
    const uint32_t p1lo = pre1 & 0xFFFFu, p1hi = pre1 >> 16;
    const uint32_t p2lo = pre2 & 0xFFFFu, p2hi = pre2 >> 16;
    const uint32_t p3lo = pre3 & 0xFFFFu, p3hi = pre3 >> 16;
    const uint32_t s_idx0 = entry.s + (e ? p1hi - p1lo : p1lo);
    uint32_t k_idx = entry.k + (e ? p2hi - p2lo : p2lo);
    const int32_t d0 = 2 * (int32_t)p3lo - (int32_t)p2lo;
    const int32_t dt = 2 * (int32_t)p3hi - (int32_t)p2hi;
    int32_t depth = entry.d + (e ? dt - d0 : d0);
    const uint64_t pos0 = seg_log + tile_off + (uint64_t)my0 + 1u;

    int32_t* __restrict__ pos = P.pos + seg_outb;
    int32_t* __restrict__ pair = P.pair + seg_outb;
    uint2* __restrict__ brk = P.brk + seg_brkb;
    uint32_t s_idx = s_idx0;
    while (stm) {
        const int j = __ffs(stm) - 1;
        stm &= stm - 1u;
        pos[s_idx] = (int32_t)(pos0 + (uint64_t)j);
        pair[s_idx] = 0;
        if ((brm >> j) & 1u) {
            const uint32_t is_open = (opm >> j) & 1u;
            const int32_t lvl = is_open ? depth : depth - 1;
            depth += is_open ? 1 : -1;
            const uint32_t cur = ((c.cur >> j) & 1u) ? kCurly : 0u;
            brk[k_idx] = make_uint2(s_idx | cur, ((uint32_t)lvl << 1) | is_open);
            k_idx++;
        }
        s_idx++;
    }
}

template __global__ void scan_kernel<false>(ScanParams);
template __global__ void scan_kernel<true>(ScanParams);

void launch_scan(const ScanParams& p, bool lines, cudaStream_t stream)
{
    if (p.n_tiles == 0) return;
    if (lines) scan_kernel<true><<<p.n_tiles, kThreads, 0, stream>>>(p);
    else scan_kernel<false><<<p.n_tiles, kThreads, 0, stream>>>(p);
}

}  // namespace cj
