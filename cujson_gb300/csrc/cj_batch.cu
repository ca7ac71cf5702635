// cj_batch.cu -- device helpers for batches of independent documents.
//
// A batch is many standard documents parsed by one launch of the scan and
// pairing kernels: every document is a segment of its own (string state,
// escapes, depth and counts restart at its first byte), with its own region
// of the position, pair and bracket-record arrays and its own verdict.  The
// reference parses one document per call; this mode has no counterpart there.
//
//   batch_scatter       packed host layout (documents back to back, one H2D
//                       copy) -> the scan's layout (every document on a 1 KiB
//                       boundary, as the bulk copies need 16-byte alignment)
//   batch_prefix        per-document prefixes (after the scan) of the result
//                       layout sizes and of the pairing chunks holding records
//   batch_layout        each document's result in the reference layout
//                       (2*(S+2) int32), back to back, for one D2H copy
#include <cuda_runtime.h>

#include <algorithm>

#include "cj_device.cuh"
#include "cj_kernels.h"

namespace cj {

namespace {

constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr int kPieceWords = 16;   // words of 4 bytes per scatter work item

// the document holding global word w: largest d with word_off[d] <= w
__device__ __forceinline__ uint32_t doc_of_word(const uint64_t* word_off, uint32_t n, uint64_t w)
{
    uint32_t lo = 0, hi = n;   // word_off[lo] <= w < word_off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(word_off + mid) <= w) lo = mid;
        else hi = mid;
    }
    return lo;
}

}  // namespace

// Every thread copies pieces of kPieceWords destination words.  Destination
// words are aligned; each is assembled from the two source words that cover
// it (funnel shift by the source's byte misalignment).  The packed buffer
// carries 8 bytes of slack past its end for the second word.  Bytes past a
// document's end that land in its last word are padding the scan never reads
// as input.
__global__ void __launch_bounds__(256) batch_scatter(const uint8_t* __restrict__ packed,
                                                     const uint64_t* __restrict__ src_off,
                                                     const uint64_t* __restrict__ word_off,
                                                     const Segment* __restrict__ segs, uint32_t n,
                                                     uint8_t* __restrict__ in)
{
    const uint64_t total = __ldg(word_off + n);
    const uint64_t pieces = (total + kPieceWords - 1) / kPieceWords;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < pieces; p += stride) {
        uint64_t w = p * kPieceWords;
        const uint64_t wend = min(total, w + kPieceWords);
        uint32_t d = doc_of_word(word_off, n, w);
        while (w < wend) {
            while (d + 1 < n && __ldg(word_off + d + 1) <= w) d++;
            const uint64_t dw = w - __ldg(word_off + d);           // word within the document
            const uint64_t src = __ldg(src_off + d) + 4 * dw;
            const uint32_t sh = (uint32_t)(src & 3u) * 8u;
            const uint32_t* s32 = reinterpret_cast<const uint32_t*>(packed + (src & ~3ull));
            const uint32_t a = __ldg(s32), b = __ldg(s32 + 1);
            uint32_t* d32 = reinterpret_cast<uint32_t*>(in + __ldg(&segs[d].dev_off)) + dw;
            *d32 = sh ? __funnelshift_r(a, b, sh) : a;
            w++;
        }
    }
}

// One block, after the scan: per document, exclusive prefixes of
//   layout_off:  its result layout size 2*(S+2) (off[n] = total), with S
//                clamped to the document's byte count (an upper bound that
//                holds for every verdict, so the layout writes stay in bounds);
//   rchunk_off:  its pairing chunks that hold records, ceil(K/kChunk), K
//                clamped to the byte count as well.
__global__ void __launch_bounds__(1024) batch_prefix(const Segment* __restrict__ segs,
                                                     const SegmentOut* __restrict__ seg_out, uint32_t n,
                                                     uint64_t* __restrict__ layout_off,
                                                     uint64_t* __restrict__ rchunk_off)
{
    __shared__ uint64_t warp_tot[2][32];
    __shared__ uint64_t carry_s[2];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    allow_next_grid();
    wait_previous_grid();
    if (tid == 0) carry_s[0] = carry_s[1] = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t i = base + tid;
        uint64_t v[2] = {0, 0};
        if (i < n) {
            const uint64_t len = __ldg(&segs[i].len);
            const uint64_t S = min((uint64_t)__ldcg(&seg_out[i].s_end), len);
            const uint64_t K = min((uint64_t)__ldcg(&seg_out[i].k_end), len);
            v[0] = 2 * S + 4;
            v[1] = (K + kChunk - 1) / kChunk;
        }
        uint64_t x[2] = {v[0], v[1]};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
            for (int a = 0; a < 2; a++) {
                const uint64_t y = __shfl_up_sync(FULL, x[a], o);
                if (lane >= o) x[a] += y;
            }
        }
        if (lane == 31) { warp_tot[0][wid] = x[0]; warp_tot[1][wid] = x[1]; }
        __syncthreads();
        if (wid < 2) {
            uint64_t t = lane < nw ? warp_tot[wid][lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(FULL, t, o);
                if (lane >= o) t += y;
            }
            if (lane < nw) warp_tot[wid][lane] = t;   // inclusive over warps
        }
        __syncthreads();
        if (i < n) {
            layout_off[i] = carry_s[0] + (wid ? warp_tot[0][wid - 1] : 0) + x[0] - v[0];
            rchunk_off[i] = carry_s[1] + (wid ? warp_tot[1][wid - 1] : 0) + x[1] - v[1];
        }
        __syncthreads();
        if (tid == 0) {
            carry_s[0] += warp_tot[0][nw - 1];
            carry_s[1] += warp_tot[1][nw - 1];
        }
        __syncthreads();
    }
    if (tid == 0) {
        layout_off[n] = carry_s[0];
        rchunk_off[n] = carry_s[1];
    }
}

// Every document's reference layout, flat over the whole batch: element g of
// the layout buffer belongs to document d with off[d] <= g < off[d+1] and is,
// with i = g - off[d] and S = S_d, [0]=0, [1..S] positions, [S+1]=S+1,
// [S+2..2S+1] pair row, [2S+2], [2S+3] = 0.  A warp writes a run of
// 32 * kLayoutRun consecutive elements, lane l the elements base + 32k + l
// (coalesced); lane 0 finds the run's first document by binary search and
// every lane then walks forward through the documents its elements reach.
constexpr int kLayoutRun = 16;

__global__ void __launch_bounds__(256) batch_layout(const Segment* __restrict__ segs,
                                                    const SegmentOut* __restrict__ seg_out, uint32_t n,
                                                    const int32_t* __restrict__ pos,
                                                    const int32_t* __restrict__ pair,
                                                    const uint64_t* __restrict__ off,
                                                    int32_t* __restrict__ layout)
{
    const int lane = threadIdx.x & 31;
    wait_previous_grid();
    const uint64_t total = __ldcg(off + n);
    const uint64_t per_run = 32ull * kLayoutRun;
    const uint64_t runs = (total + per_run - 1) / per_run;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t r = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < runs; r += nwarps) {
        const uint64_t g0 = r * per_run;
        uint32_t d = 0;
        if (lane == 0) {
            uint32_t lo = 0, hi = n;        // off[lo] <= g0 < off[hi]
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (__ldcg(off + mid) <= g0) lo = mid;
                else hi = mid;
            }
            d = lo;
        }
        d = __shfl_sync(FULL, d, 0);
        uint64_t dbeg = __ldcg(off + d), dend = __ldcg(off + d + 1);
        uint64_t S = min((uint64_t)__ldcg(&seg_out[d].s_end), (uint64_t)__ldg(&segs[d].len));
        uint64_t b = __ldg(&segs[d].out_base);
        for (int k = 0; k < kLayoutRun; k++) {
            const uint64_t g = g0 + 32ull * k + lane;
            if (g >= total) break;
            while (g >= dend) {
                d++;
                dbeg = dend;
                dend = __ldcg(off + d + 1);
                S = min((uint64_t)__ldcg(&seg_out[d].s_end), (uint64_t)__ldg(&segs[d].len));
                b = __ldg(&segs[d].out_base);
            }
            const uint64_t i = g - dbeg;
            int32_t v;
            if (i == 0) v = 0;
            else if (i <= S) v = __ldcg(pos + b + i - 1);
            else if (i == S + 1) v = (int32_t)(S + 1);
            else if (i <= 2 * S + 1) v = __ldcg(pair + b + (i - S - 2));
            else v = 0;
            layout[g] = v;
        }
    }
}

cudaError_t preload_batch_kernels()
{
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, (const void*)batch_scatter);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)batch_prefix);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)batch_layout);
    return e;
}

void launch_batch_scatter(const uint8_t* packed, const uint64_t* src_off, const uint64_t* word_off,
                          const Segment* segs, uint32_t n, uint64_t total_words, uint8_t* in, int sm_count,
                          cudaStream_t stream)
{
    const uint64_t pieces = (total_words + kPieceWords - 1) / kPieceWords;
    const uint64_t want = (pieces + 255) / 256;
    const int grid = (int)std::min<uint64_t>(want ? want : 1, (uint64_t)sm_count * 16);
    batch_scatter<<<grid, 256, 0, stream>>>(packed, src_off, word_off, segs, n, in);
}

void launch_batch_prefix(const Segment* segs, const SegmentOut* seg_out, uint32_t n, uint64_t* layout_off,
                         uint64_t* rchunk_off, cudaStream_t stream, bool dep)
{
    launch_dependent(batch_prefix, 1, 1024, 0, stream, dep, segs, seg_out, n, layout_off, rchunk_off);
}

void launch_batch_layout(const Segment* segs, const SegmentOut* seg_out, uint32_t n, const int32_t* pos,
                         const int32_t* pair, const uint64_t* off, int32_t* layout, int sm_count,
                         cudaStream_t stream, bool dep)
{
    launch_dependent(batch_layout, sm_count * 8, 256, 0, stream, dep, segs, seg_out, n, pos, pair, off, layout);
}

}  // namespace cj
