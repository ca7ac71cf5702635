// cujson_types.h -- the reference's public types, same layout and names
// (cujson/cujson_types.h:9-39), so code written against the reference compiles
// and links unchanged against this library.
#ifndef CUJSON_TYPES_H
#define CUJSON_TYPES_H

#include <cstddef>
#include <cstdint>
#include <vector>

struct cuJSONInput {
    uint8_t* data;                     // pinned host buffer with the document
    size_t size;                       // bytes
};

struct cuJSONLinesInput {
    uint8_t* data;                     // pinned host buffer with all lines
    size_t chunkCount;                 // number of chunks
    size_t size;                       // bytes
    std::vector<uint8_t*> chunks;      // start of every chunk (whole lines)
    std::vector<size_t> chunksSize;    // bytes of every chunk
};

struct cuJSONResult {
    uint8_t* inputJSON;                // not set (kept for layout)
    int chunkCount;                    // 1, or the number of JSON-Lines chunks
    int bufferSize;                    // not set (kept for layout)
    std::vector<int> resultSizes;      // structurals per chunk
    std::vector<int> resultSizesPrefix;// running sums of resultSizes
    int32_t* structural;               // [0]=0, [1..S] 1-based positions, [S+1]=S+1
    int32_t* pair_pos;                 // structural + S + 1; close index at opens
    int depth;                         // deepest nesting
    int totalResultSize;               // S + 2
    int fileSize;                      // S + 2
};

enum tokens_type_enum { OBJECT, ARRAY, KEYVALUE, VALUE, CLOSING };
typedef tokens_type_enum token_type;

enum primitive_type_enum { NUMBER, TRUE, FALSE, NULL_TYPE, STRING };
typedef primitive_type_enum primitive_type;

#endif  // CUJSON_TYPES_H
