// cujson_api.h -- the reference's parse and load functions, as inline
// wrappers over the C ABI of libcujson_gb300 (include/cujson_gb300.h).
//
//   loadJSON                          <- cujson/load_file.cu:7
//   loadJSONLines_chunkCount          <- cujson/load_file.cu:38
//   loadJSONLines_chunkSizeBytes      <- cujson/load_file.cu:109
//   loadJSONLines_chunkSizeMegaBytes  <- cujson/load_file.cu:182
//   parse_standard_json               <- cujson/parse_standard_json.cu:1584
//   parse_json_lines                  <- cujson/parse_json_lines.cu:1092
//
// Differences a caller can observe, all deliberate: invalid input returns an
// empty cuJSONResult (structural == nullptr) and the status is available from
// cj_last_status() instead of the process exiting; parse_standard_json leaves
// the input buffer alone (the reference's cudaFree on a pinned pointer fails
// and leaves it alone too); the JSON-Lines virtual root slots are written;
// pair_pos is 0 at non-open entries; `depth` holds the deepest nesting.
#ifndef CUJSON_API_H
#define CUJSON_API_H

#include <cuda_runtime.h>

#include <chrono>
#include <iostream>
#include <string>
#include <vector>

#include "../cujson_gb300.h"
#include "cujson_types.h"

using namespace std;

namespace cujson_detail {

inline cuJSONResult to_result(cj_result& r, int chunk_count)
{
    cuJSONResult out{};
    out.inputJSON = nullptr;
    out.chunkCount = chunk_count;
    out.bufferSize = 0;
    int prefix = 0;
    for (int64_t i = 0; i < r.n_segments; i++) {
        out.resultSizes.push_back((int)r.segment_sizes[i]);
        prefix += (int)r.segment_sizes[i];
        out.resultSizesPrefix.push_back(prefix);
    }
    out.structural = r.structural;
    out.pair_pos = r.pair_pos;
    out.depth = r.max_depth;
    out.totalResultSize = (int)r.total;
    out.fileSize = (int)r.total;
    free(r.segment_sizes);       // the result buffer itself now belongs to the caller
    r.segment_sizes = nullptr;
    return out;
}

inline cuJSONLinesInput lines_input(uint8_t* data, size_t size, const std::vector<size_t>& sizes)
{
    cuJSONLinesInput in;
    in.data = data;
    in.size = size;
    in.chunkCount = sizes.size();
    size_t off = 0;
    for (size_t s : sizes) {
        in.chunks.push_back(data + off);
        in.chunksSize.push_back(s);
        off += s;
    }
    return in;
}

}  // namespace cujson_detail

inline cuJSONInput loadJSON(const std::string& filePath)
{
    uint8_t* data = nullptr;
    size_t size = 0;
    if (cj_load_file(filePath.c_str(), &data, &size) != CJ_OK) return cuJSONInput{nullptr, 0};
    return cuJSONInput{data, size};
}

inline cuJSONLinesInput loadJSONLines_chunkCount(const std::string& filePath, size_t chunkCount = 1)
{
    cuJSONLinesInput in;
    in.data = nullptr;
    in.size = 0;
    in.chunkCount = chunkCount;
    uint8_t* data = nullptr;
    size_t size = 0;
    if (chunkCount == 0 || cj_load_file(filePath.c_str(), &data, &size) != CJ_OK) return in;
    std::vector<size_t> sizes(chunkCount);
    cj_plan_lines_count(data, size, chunkCount, sizes.data());
    return cujson_detail::lines_input(data, size, sizes);
}

inline cuJSONLinesInput loadJSONLines_chunkSizeBytes(const std::string& filePath, size_t chunkSizeBytes)
{
    cuJSONLinesInput in;
    in.data = nullptr;
    in.size = 0;
    in.chunkCount = 0;
    uint8_t* data = nullptr;
    size_t size = 0;
    if (cj_load_file(filePath.c_str(), &data, &size) != CJ_OK) return in;
    size_t n = 0;
    cj_plan_lines_bytes(data, size, chunkSizeBytes, nullptr, 0, &n);
    std::vector<size_t> sizes(n);
    cj_plan_lines_bytes(data, size, chunkSizeBytes, sizes.data(), n, &n);
    return cujson_detail::lines_input(data, size, sizes);
}

inline cuJSONLinesInput loadJSONLines_chunkSizeMegaBytes(const std::string& filePath,
                                                         size_t chunkSizeMegaBytes)
{
    return loadJSONLines_chunkSizeBytes(filePath, chunkSizeMegaBytes * 1024 * 1024);
}

inline cuJSONResult parse_standard_json(cuJSONInput input)
{
    if (input.data == nullptr || input.size == 0) {
        cj_set_last_status(CJ_ERR_INVALID_ARGUMENT);
        return cuJSONResult{};
    }
    cj_context* ctx = cj_default_context();
    if (!ctx) {
        cj_set_last_status(CJ_ERR_NO_DEVICE);
        return cuJSONResult{};
    }
    cj_result r;
    if (cj_parse_standard(ctx, input.data, input.size, &r) != CJ_OK) return cuJSONResult{};
    return cujson_detail::to_result(r, 1);
}

inline cuJSONResult parse_json_lines(cuJSONLinesInput input)
{
    // the reference's argument checks, cujson/parse_json_lines.cu:1103-1150
    if (input.size == 0 || input.data == nullptr || input.chunkCount == 0 ||
        input.chunks.size() < input.chunkCount || input.chunksSize.size() < input.chunkCount) {
        cj_set_last_status(CJ_ERR_INVALID_ARGUMENT);
        return cuJSONResult{};
    }
    for (size_t i = 0; i < input.chunkCount; i++) {
        if (input.chunksSize[i] == 0 || input.chunksSize[i] > input.size || input.chunks[i] == nullptr) {
            cj_set_last_status(CJ_ERR_INVALID_ARGUMENT);
            return cuJSONResult{};
        }
    }
    cj_context* ctx = cj_default_context();
    if (!ctx) {
        cj_set_last_status(CJ_ERR_NO_DEVICE);
        return cuJSONResult{};
    }
    std::vector<const uint8_t*> ptrs(input.chunks.begin(), input.chunks.begin() + input.chunkCount);
    cj_result r;
    cj_status st = cj_parse_lines(ctx, ptrs.data(), input.chunksSize.data(), input.chunkCount, &r);
    if (st != CJ_OK) return cuJSONResult{};
    cuJSONResult out = cujson_detail::to_result(r, (int)input.chunkCount);
    cudaFreeHost(input.data);   // as the reference does, cujson/parse_json_lines.cu:1261
    return out;
}

#endif  // CUJSON_API_H
