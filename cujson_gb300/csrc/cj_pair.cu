// cj_pair.cu -- nesting recognition: open/close pairing by depth buckets.
//
// The reference keys every bracket by its depth (uint8), stable-sorts the
// brackets by that key with thrust::stable_sort_by_key and pairs neighbours
// (cujson/parse_standard_json.cu:1519-1582, validate_expand_MathAPI_new2
// :1432-1514).  Here no sort is needed: every bracket record already carries
// its level (depth before an open, depth after a close), so a matching pair
// shares a level and, inside one level's bucket, opens and closes alternate
// in document order.  The pass keeps one slot per level ("bucket head") that
// holds the currently open bracket of that level:
//
//   kernel pair_chunks: one warp walks a chunk of 512 records, 32 at a time.
//     __match_any_sync groups the lanes of a round by level; a close pairs
//     with the previous same-level lane of its round, else with its level's
//     bucket head.  The last lane of each level group then updates the head
//     (an open becomes the head, a close empties it).  What stays unmatched
//     in a chunk is its "spine": closes at levels entry-1 .. min (one per
//     level) and opens at levels min .. exit-1 (one per level).
//   kernel pair_spine: an unmatched open at level d in chunk c pairs with the
//     unmatched close at level d of the first later chunk whose minimum depth
//     is <= d, found through a 32-ary min-tree over the chunk minima.
//
// Levels are int32, so nesting is unbounded (the reference's uint8 key aliases
// past depth 256).  Validation: every level >= 0, every pair of the same kind,
// and depth 0 at the end of each segment (checked by the scan).
#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

#include <climits>

namespace cj {

namespace {

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
__device__ __forceinline__ uint32_t lanemask_gt() {
#ifdef CJ_EMU
    return ~((2u << (threadIdx.x & 31)) - 1u);
#else
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_gt;" : "=r"(m));
    return m;
#endif
}

// pair_spine: chunks after an open's own that are checked directly, and the
// count of far matches in a round above which each lane walks its own
constexpr int kSpineWindow = 4;
constexpr int kSpineWarpMax = 8;

__device__ __forceinline__ unsigned long long tree_pack(uint32_t epoch, int32_t level) {
    return ((unsigned long long)epoch << 32) | (uint32_t)(0x7FFFFFFF - level);
}

__device__ __forceinline__ int32_t tree_value(const PairParams& P, int lvl, uint64_t i) {
    if (lvl == 0) return __ldcg(&P.cinfo[i].y);
    unsigned long long v = __ldcg(P.tree + P.tree_off[lvl] + i);
    if ((uint32_t)(v >> 32) != P.epoch) return INT_MAX;
    return 0x7FFFFFFF - (int32_t)(uint32_t)v;
}

// entries of min-tree level lvl over nch chunks: ceil(nch / 32^lvl)
__device__ __forceinline__ uint64_t level_size(uint64_t nch, int lvl) {
    const int sh = 5 * lvl;
    return (nch + (1ull << sh) - 1) >> sh;
}

// first chunk index > c whose minimum depth is <= d, or -1
__device__ int64_t next_le(const PairParams& P, uint64_t nch, uint64_t c, int32_t d) {
    uint64_t i = c + 1;
    int lvl = 0;
    while (true) {
        if (i >= level_size(nch, lvl)) return -1;
        uint64_t gend = (i | 31) + 1;
        if (gend > level_size(nch, lvl)) gend = level_size(nch, lvl);
        bool found = false;
        for (; i < gend; i++)
            if (tree_value(P, lvl, i) <= d) { found = true; break; }
        if (found) break;
        if (lvl == kTreeLevels) return -1;
        i = gend >> 5;
        lvl++;
    }
    while (lvl > 0) {
        lvl--;
        i *= 32;
        uint64_t gend = i + 32;
        if (gend > level_size(nch, lvl)) gend = level_size(nch, lvl);
        for (; i < gend; i++)
            if (tree_value(P, lvl, i) <= d) break;
        if (i >= gend) return -1;   // inconsistent tree (only on a timeout path)
    }
    return (int64_t)i;
}

// The same search by the whole warp (every lane gets the result): each level's
// group of 32 entries is read at once, one lane per entry, and a ballot finds
// the first that qualifies -- one dependent load per level instead of up to 32.
__device__ int64_t next_le_warp(const PairParams& P, uint64_t nch, uint64_t c, int32_t d, int lane) {
    uint64_t i = c + 1;
    int lvl = 0;
    while (true) {
        if (i >= level_size(nch, lvl)) return -1;
        const uint64_t g0 = i & ~31ull, j = g0 + (uint64_t)lane;
        const bool ok = j >= i && j < level_size(nch, lvl) && tree_value(P, lvl, j) <= d;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        if (m) { i = g0 + (uint64_t)(__ffs(m) - 1); break; }
        if (lvl == kTreeLevels) return -1;
        i = (g0 >> 5) + 1;
        lvl++;
    }
    while (lvl > 0) {
        lvl--;
        const uint64_t g0 = i * 32, j = g0 + (uint64_t)lane;
        const bool ok = j < level_size(nch, lvl) && tree_value(P, lvl, j) <= d;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        if (!m) return -1;          // inconsistent tree (only on a timeout path)
        i = g0 + (uint64_t)(__ffs(m) - 1);
    }
    return (int64_t)i;
}

// batch: the document of work item w, largest d with rchunk_off[d] <= w
__device__ __forceinline__ uint32_t doc_of_item(const PairParams& P, uint64_t w)
{
    uint32_t lo = 0, hi = P.n_bsegs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldcg(P.rchunk_off + mid) <= w) lo = mid;
        else hi = mid;
    }
    return lo;
}

}  // namespace

__global__ void __launch_bounds__(256) pair_chunks(PairParams P)
{
    allow_next_grid();
    wait_previous_grid();
#ifdef CJ_EMU
    uint32_t* s_heads_all = reinterpret_cast<uint32_t*>(cj_emu::g_dyn_smem.data());
#else
    extern __shared__ uint32_t s_heads_all[];
#endif
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    uint32_t* heads = s_heads_all + wib * kHeads;
    const uint32_t FULL = 0xFFFFFFFFu;
    const bool batch = P.rchunk_off != nullptr;
    // a scan whose emitted records disagree with its counts is not paired
    if (__ldcg(&P.ctrl->error_flags) & CJ_FLAG_OVERFLOW) return;
    const uint32_t K = batch ? 0u : P.ctrl->k_total;
    const uint64_t items = batch ? __ldcg(P.rchunk_off + P.n_bsegs) : ((uint64_t)K + kChunk - 1) / kChunk;
    const uint64_t gwarp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint32_t lt = lanemask_lt(), gt = lanemask_gt();

    for (uint64_t w = gwarp; w < items; w += nwarps) {
        uint64_t c = w;
        int cnt;
        uint32_t segi = 0, S;
        int32_t* __restrict__ pair = P.pair;
        if (batch) {
            segi = doc_of_item(P, w);
            const uint64_t local = w - __ldcg(P.rchunk_off + segi);
            c = __ldg(&P.segs[segi].brk_base) / kChunk + local;
            const uint64_t left = (uint64_t)__ldcg(&P.seg_out[segi].k_end) - local * kChunk;
            cnt = (int)min((uint64_t)kChunk, left);
            pair += __ldg(&P.segs[segi].out_base);
            S = __ldcg(&P.seg_out[segi].s_end);
        } else {
            cnt = (int)min((uint64_t)kChunk, (uint64_t)K - c * kChunk);
            S = P.ctrl->s_total;
        }
        const uint64_t base = c * kChunk;
        uint32_t err = 0;
        // the chunk's records, all loaded at once (one per lane per round)
        uint2 recs[kChunk / 32];
#pragma unroll
        for (int j = 0; j < kChunk / 32; j++) {
            const int i = j * 32 + lane;
            recs[j] = i < cnt ? __ldcg(P.brk + base + i) : make_uint2(0u, 0u);
        }
        const uint32_t r0y = __shfl_sync(FULL, recs[0].y, 0);
        const uint2 r0 = make_uint2(0u, r0y);
        const int32_t L0 = (int32_t)r0.y >> 1;
        // the head slots this chunk's records use (levels L0 - kChunk ..
        // L0 + kChunk map to slots 0 .. kHeads - 1): only those are cleared
        // here and read back at the end
        int32_t smin = kHeads - 1, smax = 0;
#pragma unroll
        for (int j = 0; j < kChunk / 32; j++) {
            if (j * 32 + lane < cnt) {
                const int32_t sl = ((int32_t)recs[j].y >> 1) - L0 + kChunk;
                smin = min(smin, max(sl, 0));
                smax = max(smax, min(sl, kHeads - 1));
            }
        }
        smin = __reduce_min_sync(FULL, smin);
        smax = __reduce_max_sync(FULL, smax);
        for (int i = smin + lane; i <= smax; i += 32) heads[i] = kEmpty;
        const int32_t d_entry = (r0.y & 1u) ? L0 : L0 + 1;
        int32_t dmin = d_entry, maxd = INT_MIN;
        int32_t last_lvl = 0;
        uint32_t last_open = 0;
        __syncwarp();

#pragma unroll
        for (int j = 0; j < kChunk / 32; j++) {
            const int r = j * 32;
            if (r >= cnt) break;
            const bool valid = (r + lane) < cnt;
            const uint2 rec = recs[j];
            const int32_t lvl = (int32_t)rec.y >> 1;
            const uint32_t is_open = rec.y & 1u;
            const uint32_t key = valid ? (uint32_t)lvl : (0xC0000000u | (uint32_t)lane);
            const uint32_t peers = __match_any_sync(FULL, key);
            const uint32_t prevp = peers & lt;
            const int plane = prevp ? 31 - __clz(prevp) : lane;
            const uint32_t p_x = __shfl_sync(FULL, rec.x, plane);
            const uint32_t p_open = __shfl_sync(FULL, is_open, plane);
            const int slot = lvl - L0 + kChunk;
            if (valid && !is_open) {
                uint32_t partner = kEmpty;
                if (prevp) {
                    if (p_open) partner = p_x;
                    else err |= CJ_FLAG_BRACKETS;     // two closes in a row at one level
                } else if (slot >= 0 && slot < kHeads) {
                    partner = heads[slot];
                    if (partner == kEmpty) {
                        // unmatched inside the chunk: part of the spine
                        const int32_t idx = d_entry - 1 - lvl;
                        if (idx >= 0 && idx < kChunk) P.spine[base + idx] = rec.x;
                        else err |= CJ_FLAG_BRACKETS;
                    }
                }
                if (partner != kEmpty) {
                    if ((partner ^ rec.x) & kCurly) err |= CJ_FLAG_BRACKETS;
                    if ((partner & ~kCurly) < S) pair[partner & ~kCurly] = (int32_t)((rec.x & ~kCurly) + 1u);
                    else err |= CJ_FLAG_BRACKETS;
                }
            }
            __syncwarp();
            if (valid && (peers & gt) == 0u && slot >= 0 && slot < kHeads)
                heads[slot] = is_open ? rec.x : kEmpty;
            __syncwarp();
            if (valid) {
                if (!is_open) dmin = min(dmin, lvl);
                else maxd = max(maxd, lvl + 1);
            }
            const int lastlane = min(31, cnt - r - 1);
            last_lvl = __shfl_sync(FULL, lvl, lastlane);
            last_open = __shfl_sync(FULL, is_open, lastlane);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dmin = min(dmin, __shfl_xor_sync(FULL, dmin, o));
            maxd = max(maxd, __shfl_xor_sync(FULL, maxd, o));
        }
        const int32_t d_exit = last_open ? last_lvl + 1 : last_lvl;
        for (int i = smin + lane; i <= smax; i += 32) {
            const uint32_t h = heads[i];
            if (h != kEmpty) {
                const int32_t lvl = i - kChunk + L0;
                const int32_t idx = lvl - dmin;
                if (idx >= 0 && idx < kChunk) P.spine[base + (kChunk - 1 - idx)] = h;
                else err |= CJ_FLAG_BRACKETS;
            }
        }
        err = __reduce_or_sync(FULL, err);
        if (lane == 0) {
            P.cinfo[c] = make_int4(d_entry, dmin, d_exit, 0);
            if (batch) {
                if (dmin < 0) err |= CJ_FLAG_BRACKETS;
                if (err) atomicOr(P.seg_err + segi, err);
                if (maxd > 0) atomicMax(P.seg_depth + segi, maxd);
            } else {
                if (dmin < 0) atomicMax(&P.ctrl->neg_min_level, -dmin);
                if (err) atomicOr(&P.ctrl->error_flags, err);
            }
            if (maxd > 0) atomicMax(&P.ctrl->max_depth, maxd);
            const unsigned long long pk = tree_pack(P.epoch, dmin);
            for (int l = 1; l <= kTreeLevels; l++)
                atomicMax(P.tree + P.tree_off[l] + (c >> (5 * l)), pk);
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(256) pair_spine(PairParams P)
{
    const int lane = threadIdx.x & 31;
    const bool batch = P.rchunk_off != nullptr;
    wait_previous_grid();
    if (__ldcg(&P.ctrl->error_flags) & CJ_FLAG_OVERFLOW) return;
    const uint32_t K = batch ? 0u : P.ctrl->k_total;
    const uint64_t nch = batch ? P.n_chunks : ((uint64_t)K + kChunk - 1) / kChunk;
    const uint64_t items = batch ? __ldcg(P.rchunk_off + P.n_bsegs) : nch;
    const uint64_t gwarp = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t w = gwarp; w < items; w += nwarps) {
        uint32_t err = 0;
        uint32_t segi = 0, S;
        uint64_t c = w, c_end = nch;               // chunks of this record sequence: [.., c_end)
        int32_t* __restrict__ pair = P.pair;
        if (batch) {
            segi = doc_of_item(P, w);
            const uint64_t first = __ldg(&P.segs[segi].brk_base) / kChunk;
            c = first + (w - __ldcg(P.rchunk_off + segi));
            c_end = first + (__ldcg(P.rchunk_off + segi + 1) - __ldcg(P.rchunk_off + segi));
            S = __ldcg(&P.seg_out[segi].s_end);
            pair += __ldg(&P.segs[segi].out_base);
        } else {
            S = P.ctrl->s_total;
        }
        const int4 ci = __ldcg(&P.cinfo[c]);
        const int32_t n_uo = ci.z - ci.y;          // opens still open at chunk end
        const int32_t n_uc = ci.x - ci.y;          // closes unmatched inside the chunk
        // the matching close of the open at level d (structural ox) is the
        // unmatched close at level d of chunk c2
        auto resolve = [&](int64_t c2, int32_t d, uint32_t ox) {
            if (c2 < 0 || (uint64_t)c2 >= c_end) { err |= CJ_FLAG_BRACKETS; return; }   // none, or past the document
            const int4 cj2 = __ldcg(&P.cinfo[c2]);
            const int32_t idx = cj2.x - 1 - d;
            if (idx < 0 || idx >= kChunk || idx >= cj2.x - cj2.y) { err |= CJ_FLAG_BRACKETS; return; }
            const uint32_t cx = __ldcg(P.spine + (uint64_t)c2 * kChunk + idx);
            if ((ox ^ cx) & kCurly) err |= CJ_FLAG_BRACKETS;
            if ((ox & ~kCurly) >= S || (cx & ~kCurly) >= S) { err |= CJ_FLAG_BRACKETS; return; }
            pair[ox & ~kCurly] = (int32_t)((cx & ~kCurly) + 1u);
        };
        if (n_uo < 0 || n_uc < 0 || n_uo + n_uc > kChunk) {
            err = CJ_FLAG_BRACKETS;
        } else {
            for (int32_t base = 0; base < n_uo; base += 32) {
                // one open per lane: most match in one of the next few chunks,
                // read together
                const int32_t i = base + lane;
                const bool valid = i < n_uo;
                const int32_t d = ci.y + i;
                const uint32_t ox = valid ? __ldcg(P.spine + c * kChunk + (kChunk - 1 - i)) : 0u;
                int64_t c2 = -1;
                if (valid) {
                    int32_t v[kSpineWindow];
#pragma unroll
                    for (int k = 0; k < kSpineWindow; k++)
                        v[k] = (c + 1 + k < nch) ? __ldcg(&P.cinfo[c + 1 + k].y) : INT_MAX;
#pragma unroll
                    for (int k = kSpineWindow - 1; k >= 0; k--)
                        if (v[k] <= d) c2 = (int64_t)(c + 1 + k);
                }
                const bool far = valid && c2 < 0 && c + 1 + kSpineWindow < nch;
                if (valid && !far) resolve(c2, d, ox);
                uint32_t pend = __ballot_sync(0xFFFFFFFFu, far);
                if (__popc(pend) >= kSpineWarpMax) {
                    // many far matches (deep nesting): a walk per lane
                    if (far) resolve(next_le(P, nch, c, d), d, ox);
                } else {
                    // a few: the warp walks the min-tree for each in turn
                    while (pend) {
                        const int src = __ffs(pend) - 1;
                        pend &= pend - 1u;
                        const int32_t ds = __shfl_sync(0xFFFFFFFFu, d, src);
                        const int64_t c2w = next_le_warp(P, nch, c, ds, lane);
                        if (lane == src) resolve(c2w, d, ox);
                    }
                }
            }
        }
        err = __reduce_or_sync(0xFFFFFFFFu, err);
        if (lane == 0 && err) atomicOr(batch ? P.seg_err + segi : &P.ctrl->error_flags, err);
    }
}

cudaError_t preload_pair_kernels()
{
#ifdef CJ_EMU
    return cudaSuccess;
#else
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, (const void*)pair_chunks);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)pair_spine);
    return e;
#endif
}

void launch_pair(const PairParams& p, int grid, cudaStream_t stream, int threads)
{
    // one bucket-head table per warp: 4.1 KB each, 32.8 KB at 256 threads
    // (threads <= 256 stays under the 48 KB default)
    const size_t smem = sizeof(uint32_t) * kHeads * (size_t)(threads / 32);
#ifdef CJ_EMU
    (void)stream;
    cj_emu::launch(grid, threads, smem, [&] { pair_chunks(p); });
#else
    launch_dependent(pair_chunks, grid, threads, smem, stream, p.dependent_launch != 0, p);
#endif
}

void launch_spine(const PairParams& p, int grid, cudaStream_t stream, int threads)
{
#ifdef CJ_EMU
    (void)stream;
    cj_emu::launch(grid, threads, 0, [&] { pair_spine(p); });
#else
    launch_dependent(pair_spine, grid, threads, 0, stream, p.dependent_launch != 0, p);
#endif
}

}  // namespace cj
