// cj_plan.cu -- JSON-Lines chunk planning on the device
// (cj_plan_lines_count_device).
//
// The reference's loadJSONLines_chunkCount (cujson/load_file.cu:38-103) reads
// the file, finds every line start with a serial host scan for '\n'
// (:71-78), and gives chunk i lines/chunkCount lines, one more for the first
// lines % chunkCount chunks; a last line without '\n' ends at the end of the
// file.  Here the same plan is computed for a buffer already in device memory:
//   plan_count   newlines per 64 KiB block (one CTA per block);
//   (host)       exclusive prefix of the block counts, the boundary line of
//                every chunk and, for each, the block and rank of the newline
//                that ends the line before it;
//   plan_locate  one CTA per boundary finds that newline inside its block.
// Only the block counts (4 bytes per 64 KiB) and one position per chunk
// cross to the host.
//
// loadJSONLines_chunkSizeBytes / _chunkSizeMegaBytes (load_file.cu:109-254)
// close a chunk before the line that would make it longer than the byte
// limit (a line longer than the limit gets a chunk of its own, after an empty
// one when it is the first line).  plan_bytes walks the chunk boundaries on
// the device with one warp: from a chunk start B the next boundary is the end
// of the last line that ends within B + limit, found by reading backwards
// from B + limit in 1 KiB windows (or, when no line ends there, the end of the
// line that starts at B); only the boundaries cross to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

namespace cj {

namespace {

constexpr uint64_t kPlanBlock = kPlanBlockBytes;   // bytes per counting block
constexpr int kPlanThreads = 256;
constexpr uint64_t kPerThread = kPlanBlock / kPlanThreads;

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = __reduce_add_sync(0xFFFFFFFFu, v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    uint32_t t = 0;
    if (threadIdx.x < kPlanThreads / 32) t = red[threadIdx.x];
    if (warp == 0) t = __reduce_add_sync(0xFFFFFFFFu, t);
    return t;   // valid in thread 0
}

// newlines of block blockIdx.x (bytes [b * kPlanBlock, min(n, (b + 1) * kPlanBlock)))
__global__ void __launch_bounds__(kPlanThreads) plan_count(const uint8_t* __restrict__ d, uint64_t n,
                                                           uint32_t* __restrict__ counts)
{
    __shared__ uint32_t red[kPlanThreads / 32];
    const uint64_t lo = (uint64_t)blockIdx.x * kPlanBlock;
    const uint64_t hi = min(n, lo + kPlanBlock);
    uint32_t c = 0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += kPlanThreads) c += (__ldg(d + i) == '\n') ? 1u : 0u;
    c = block_sum(c, red);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

// request q: the newline of rank req[q].y (0-based) inside block req[q].x;
// its byte position goes to pos[q]
__global__ void __launch_bounds__(kPlanThreads) plan_locate(const uint8_t* __restrict__ d, uint64_t n,
                                                            const uint2* __restrict__ req,
                                                            uint64_t* __restrict__ pos)
{
    __shared__ uint32_t cnt[kPlanThreads];
    const uint2 rq = req[blockIdx.x];
    const uint64_t lo = (uint64_t)rq.x * kPlanBlock;
    const uint64_t t_lo = min(n, lo + threadIdx.x * kPerThread);
    const uint64_t t_hi = min(n, t_lo + kPerThread);
    uint32_t c = 0;
    for (uint64_t i = t_lo; i < t_hi; i++) c += (__ldg(d + i) == '\n') ? 1u : 0u;
    cnt[threadIdx.x] = c;
    __syncthreads();
    // exclusive prefix of the threads' counts (ranges are in thread order)
    uint32_t before = 0;
    for (int t = 0; t < (int)threadIdx.x; t++) before += cnt[t];
    if (rq.y >= before && rq.y < before + c) {
        uint32_t k = rq.y - before;
        for (uint64_t i = t_lo; i < t_hi; i++) {
            if (__ldg(d + i) == '\n') {
                if (k == 0) { pos[blockIdx.x] = i; break; }
                k--;
            }
        }
    }
}

// the last newline in [lo, hi] (hi >= lo), or -1; every lane gets it
__device__ int64_t last_newline(const uint8_t* __restrict__ d, uint64_t lo, uint64_t hi, int lane) {
    uint64_t top = hi;                       // window [max(lo, top - 1023), top]
    while (true) {
        const uint64_t w0 = top >= lo + 1023 ? top - 1023 : lo;
        const uint64_t a = w0 + (uint64_t)lane * 32;
        int64_t mine = -1;
        for (int k = 31; k >= 0 && mine < 0; k--) {
            const uint64_t i = a + (uint64_t)k;
            if (i <= top && __ldg(d + i) == '\n') mine = (int64_t)i;
        }
        const uint32_t hit = __ballot_sync(0xFFFFFFFFu, mine >= 0);
        if (hit) return __shfl_sync(0xFFFFFFFFu, mine, 31 - __clz(hit));
        if (w0 == lo) return -1;
        top = w0 - 1;
    }
}

// the first newline in [lo, n), or -1; every lane gets it
__device__ int64_t first_newline(const uint8_t* __restrict__ d, uint64_t lo, uint64_t n, int lane) {
    for (uint64_t w0 = lo; w0 < n; w0 += 1024) {
        const uint64_t a = w0 + (uint64_t)lane * 32;
        int64_t mine = -1;
        for (int k = 0; k < 32 && mine < 0; k++) {
            const uint64_t i = a + (uint64_t)k;
            if (i < n && __ldg(d + i) == '\n') mine = (int64_t)i;
        }
        const uint32_t hit = __ballot_sync(0xFFFFFFFFu, mine >= 0);
        if (hit) return __shfl_sync(0xFFFFFFFFu, mine, __ffs(hit) - 1);
    }
    return -1;
}

// One warp: the chunk boundaries (starts after 0) of the byte-limit plan;
// the first `cap` go to bounds[], their number to count[0] and the last one
// (0 when there is none) to count[1].
__global__ void __launch_bounds__(32) plan_bytes(const uint8_t* __restrict__ d, uint64_t n, uint64_t limit,
                                                 uint64_t* __restrict__ bounds, uint64_t cap,
                                                 unsigned long long* __restrict__ count)
{
    const int lane = threadIdx.x;
    uint64_t B = 0, k = 0;
    bool first = true;
    while (n > B + limit) {
        // the end of the last line that ends within B + limit (B itself, a
        // line start, when none does)
        const int64_t p = limit ? last_newline(d, B, B + limit - 1, lane) : -1;
        uint64_t next;
        if (p >= 0) {
            next = (uint64_t)p + 1;
        } else if (first) {
            next = 0;                        // the first line is longer than the limit: an empty chunk
        } else {
            // the line that starts at B is longer than the limit: it is the chunk
            const int64_t q = first_newline(d, B + limit, n, lane);
            if (q < 0 || (uint64_t)q + 1 >= n) break;    // the last line: no boundary after it
            next = (uint64_t)q + 1;
        }
        if (lane == 0 && k < cap) bounds[k] = next;
        k++;
        first = false;
        B = next;
    }
    if (lane == 0) {
        count[0] = k;
        count[1] = B;
    }
}

}  // namespace

cudaError_t plan_lines_bytes_device(const uint8_t* d_data, size_t size, size_t chunk_bytes, size_t* chunk_sizes,
                                    size_t cap, size_t* n_chunks, unsigned long long* d_bounds,
                                    unsigned long long* d_count, cudaStream_t stream)
{
    plan_bytes<<<1, 32, 0, stream>>>(d_data, size, chunk_bytes, reinterpret_cast<uint64_t*>(d_bounds), cap, d_count);
    cudaError_t e = cudaGetLastError();
    unsigned long long cnt[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, d_count, sizeof(cnt), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return e;
    // chunks: one before each boundary, and the rest of the buffer after the last
    const uint64_t nb = cnt[0], last = cnt[1];
    const size_t total = (size_t)nb + (last < size ? 1 : 0);
    *n_chunks = total;
    if (!chunk_sizes || total > cap) return cudaSuccess;
    std::vector<unsigned long long> b(nb);
    if (!b.empty()) {
        e = cudaMemcpyAsync(b.data(), d_bounds, b.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return e;
    }
    uint64_t prev = 0;
    for (size_t i = 0; i < nb; i++) { chunk_sizes[i] = (size_t)(b[i] - prev); prev = b[i]; }
    if (prev < size) chunk_sizes[nb] = size - (size_t)prev;
    return cudaSuccess;
}

void launch_plan_count(const uint8_t* d_data, size_t size, uint32_t* d_counts, cudaStream_t stream)
{
    const uint64_t nb = (size + kPlanBlock - 1) / kPlanBlock;
    if (nb) plan_count<<<(unsigned)nb, kPlanThreads, 0, stream>>>(d_data, size, d_counts);
}

cudaError_t plan_lines_count_device(const uint8_t* d_data, size_t size, size_t chunk_count,
                                    size_t* chunk_sizes, uint32_t* d_counts, uint2* d_req,
                                    unsigned long long* d_pos, cudaStream_t stream)
{
    const uint64_t nb = (size + kPlanBlock - 1) / kPlanBlock;
    std::vector<uint32_t> counts(nb);
    launch_plan_count(d_data, size, d_counts, stream);
    cudaError_t e = cudaMemcpyAsync(counts.data(), d_counts, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                    stream);
    uint8_t last = '\n';
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last, d_data + size - 1, 1, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return e;
    return plan_lines_count_finish(d_data, size, chunk_count, chunk_sizes, counts.data(), last, d_req, d_pos,
                                   stream);
}

cudaError_t plan_lines_count_finish(const uint8_t* d_data, size_t size, size_t chunk_count, size_t* chunk_sizes,
                                    const uint32_t* counts, uint8_t last, uint2* d_req, unsigned long long* d_pos,
                                    cudaStream_t stream)
{
    const uint64_t nb = (size + kPlanBlock - 1) / kPlanBlock;
    cudaError_t e = cudaSuccess;

    // newlines before each block, and in all
    std::vector<uint64_t> before(nb + 1, 0);
    for (uint64_t b = 0; b < nb; b++) before[b + 1] = before[b] + counts[b];
    const uint64_t nl = before[nb];
    const uint64_t lines = nl + (last != '\n' ? 1u : 0u);     // a last line without '\n'
    const uint64_t per = lines / chunk_count, extra = lines % chunk_count;

    // the line that starts chunk i (i = 0..chunk_count) and where it starts:
    // line j > 0 starts after the j-th newline, or at the end for the open
    // last line
    std::vector<uint64_t> first_line(chunk_count + 1), start(chunk_count + 1, 0);
    std::vector<uint2> req;
    std::vector<size_t> req_of(chunk_count + 1, (size_t)-1);
    for (size_t i = 0; i <= chunk_count; i++) {
        const uint64_t j = (uint64_t)i * per + std::min<uint64_t>(i, extra);
        first_line[i] = j;
        if (j == 0) {
            start[i] = 0;
        } else if (j > nl) {
            start[i] = size;
        } else {
            const uint64_t r = j - 1;                                      // 0-based newline rank
            const uint64_t b = (uint64_t)(std::upper_bound(before.begin(), before.end(), r) - before.begin()) - 1;
            req_of[i] = req.size();
            req.push_back(make_uint2((uint32_t)b, (uint32_t)(r - before[b])));
        }
    }
    if (!req.empty()) {
        std::vector<unsigned long long> pos(req.size());
        e = cudaMemcpyAsync(d_req, req.data(), req.size() * sizeof(uint2), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) {
            plan_locate<<<(unsigned)req.size(), kPlanThreads, 0, stream>>>(d_data, size, d_req,
                                                                          reinterpret_cast<uint64_t*>(d_pos));
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(pos.data(), d_pos, pos.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return e;
        for (size_t i = 0; i <= chunk_count; i++)
            if (req_of[i] != (size_t)-1) start[i] = (size_t)pos[req_of[i]] + 1;
    }
    for (size_t i = 0; i < chunk_count; i++) chunk_sizes[i] = start[i + 1] - start[i];
    return cudaSuccess;
}

}  // namespace cj
