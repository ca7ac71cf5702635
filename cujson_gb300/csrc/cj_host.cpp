// cj_host.cpp -- host-side loaders and JSON-Lines chunk planning (C ABI).
//
// Restates the reference's loaders (cujson/load_file.cu): a file is read into
// one pinned host buffer (loadJSON :7); for JSON Lines the line starts are
// collected (one after every '\n', plus the end of the file when the last
// line has no newline, :71-78) and grouped into chunks either by a chunk count
// (lines spread evenly, the first `lines % count` chunks one line longer,
// :83-101) or by a byte limit (a chunk is closed before the line that would
// make it exceed the limit, :151-173; a first line longer than the limit yields
// an empty first chunk, which parse_json_lines rejects).  The newline scan runs
// on several host threads; the chunk boundaries are identical to a serial scan.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "cujson_gb300.h"

namespace {

// offsets of every line start after the first (byte after each '\n')
std::vector<size_t> line_starts(const uint8_t* data, size_t n)
{
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < (1u << 20)) nt = 1;
    std::vector<std::vector<size_t>> parts(nt);
    std::vector<std::thread> pool;
    const size_t per = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
        pool.emplace_back([&, t] {
            const size_t lo = std::min(n, (size_t)t * per), hi = std::min(n, lo + per);
            const uint8_t* p = data + lo;
            const uint8_t* end = data + hi;
            while (p < end) {
                const void* q = memchr(p, '\n', (size_t)(end - p));
                if (!q) break;
                const uint8_t* nl = static_cast<const uint8_t*>(q);
                parts[t].push_back((size_t)(nl - data) + 1);
                p = nl + 1;
            }
        });
    }
    for (auto& th : pool) th.join();
    std::vector<size_t> out;
    for (auto& v : parts) out.insert(out.end(), v.begin(), v.end());
    return out;
}

// 0, every line start, and the end of the file if it is not already a start
std::vector<size_t> line_offsets(const uint8_t* data, size_t n)
{
    std::vector<size_t> off;
    off.push_back(0);
    std::vector<size_t> s = line_starts(data, n);
    off.insert(off.end(), s.begin(), s.end());
    if (off.back() < n) off.push_back(n);
    return off;
}

}  // namespace

extern "C" {

cj_status cj_load_file(const char* path, uint8_t** data, size_t* size)
{
    if (!path || !data || !size) return CJ_ERR_INVALID_ARGUMENT;
    *data = nullptr;
    *size = 0;
    FILE* f = fopen(path, "rb");
    if (!f) return CJ_ERR_INVALID_ARGUMENT;
    if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return CJ_ERR_INVALID_ARGUMENT; }
    long len = ftell(f);
    if (len < 0) { fclose(f); return CJ_ERR_INVALID_ARGUMENT; }
    fseek(f, 0, SEEK_SET);
    uint8_t* buf = nullptr;
    if (cudaHostAlloc((void**)&buf, len > 0 ? (size_t)len : 1, cudaHostAllocDefault) != cudaSuccess) {
        fclose(f);
        return CJ_ERR_OUT_OF_MEMORY;
    }
    size_t got = len > 0 ? fread(buf, 1, (size_t)len, f) : 0;
    fclose(f);
    if (got != (size_t)len) { cudaFreeHost(buf); return CJ_ERR_INVALID_ARGUMENT; }
    *data = buf;
    *size = (size_t)len;
    return CJ_OK;
}

cj_status cj_plan_lines_count(const uint8_t* data, size_t size, size_t chunk_count,
                              size_t* chunk_sizes)
{
    if ((!data && size) || chunk_count == 0 || !chunk_sizes) return CJ_ERR_INVALID_ARGUMENT;
    std::vector<size_t> off = line_offsets(data, size);
    const size_t lines = off.size() - 1;
    const size_t per = lines / chunk_count, extra = lines % chunk_count;
    size_t li = 0;
    for (size_t i = 0; i < chunk_count; i++) {
        const size_t n = per + (i < extra ? 1 : 0);
        chunk_sizes[i] = off[li + n] - off[li];
        li += n;
    }
    return CJ_OK;
}

cj_status cj_plan_lines_bytes(const uint8_t* data, size_t size, size_t chunk_bytes,
                              size_t* chunk_sizes, size_t cap, size_t* n_chunks)
{
    if ((!data && size) || !n_chunks) return CJ_ERR_INVALID_ARGUMENT;
    std::vector<size_t> off = line_offsets(data, size);
    std::vector<size_t> sizes;
    size_t chunk_start = 0, cur = 0;
    for (size_t i = 1; i < off.size(); i++) {
        const size_t line_start = off[i - 1], line_end = off[i];
        if (line_end - chunk_start > chunk_bytes) {
            sizes.push_back(cur - chunk_start);
            chunk_start = line_start;
        }
        cur = line_end;
    }
    if (chunk_start < size) sizes.push_back(size - chunk_start);
    *n_chunks = sizes.size();
    if (chunk_sizes) {
        if (cap < sizes.size()) return CJ_ERR_CAPACITY;
        std::copy(sizes.begin(), sizes.end(), chunk_sizes);
    }
    return CJ_OK;
}

}  // extern "C"
