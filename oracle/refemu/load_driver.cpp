// load_driver.cpp -- runs the reference's own JSON-Lines loaders
// (cujson/load_file.cu: loadJSONLines_chunkCount :38, loadJSONLines_chunkSizeBytes
// :109, loadJSONLines_chunkSizeMegaBytes :182), compiled for the CPU with the
// cuda_runtime.h stand-in of this directory (cudaHostAlloc is a host
// allocation), on one file and prints the chunk plan they return.
// TEST INFRASTRUCTURE ONLY: its output is the golden chunk plans under
// tests/golden/ (make_plan_golden.py) and the chunk sizes of the JSON-Lines
// golden cases.
//
// usage: ref_loader <file> count|bytes|megabytes <n>
// output (text): chunkCount, then "offset size" per chunk, offsets relative to
// the start of the loaded buffer.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "cuda_runtime.h"
#include "load_file.cu"

int main(int argc, char** argv)
{
    if (argc != 4) return 2;
    const std::string path = argv[1], mode = argv[2];
    const size_t n = (size_t)strtoull(argv[3], nullptr, 10);
    cuJSONLinesInput in;
    if (mode == "count") in = loadJSONLines_chunkCount(path, n);
    else if (mode == "bytes") in = loadJSONLines_chunkSizeBytes(path, n);
    else if (mode == "megabytes") in = loadJSONLines_chunkSizeMegaBytes(path, n);
    else return 2;
    if (in.data == nullptr) return 3;
    if (in.chunks.size() != in.chunksSize.size()) return 4;
    printf("%zu\n", in.chunkCount);
    for (size_t i = 0; i < in.chunks.size(); i++)
        printf("%zu %zu\n", (size_t)(in.chunks[i] - in.data), in.chunksSize[i]);
    cudaFreeHost(in.data);
    return 0;
}
