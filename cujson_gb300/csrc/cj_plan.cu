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
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "cj_device.cuh"
#include "cj_kernels.h"
#include "cujson_gb300.h"

namespace cj {

namespace {

constexpr uint64_t kPlanBlock = 65536;      // bytes per counting block
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

}  // namespace

cudaError_t plan_lines_count_device(const uint8_t* d_data, size_t size, size_t chunk_count,
                                    size_t* chunk_sizes, uint32_t* d_counts, uint2* d_req,
                                    unsigned long long* d_pos, cudaStream_t stream)
{
    const uint64_t nb = (size + kPlanBlock - 1) / kPlanBlock;
    std::vector<uint32_t> counts(nb);
    plan_count<<<(unsigned)nb, kPlanThreads, 0, stream>>>(d_data, size, d_counts);
    cudaError_t e = cudaMemcpyAsync(counts.data(), d_counts, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                    stream);
    uint8_t last = '\n';
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last, d_data + size - 1, 1, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return e;

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
