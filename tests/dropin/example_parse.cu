// example_parse.cu -- a program written against the drop-in headers the way a
// user of the reference writes one (load, parse, iterate, free), that also
// dumps the result buffer so a test can compare it with the oracle.
//
// usage: example_parse std <file> <layout out>
//        example_parse lines <file> <chunk count> <layout out>
//        example_parse lines_mb <file> <chunk MiB> <layout out>
// layout out: int32 [S, depth, n_chunks, chunk structural counts, buffer[2*(S+2)]]
// Prints "first: <getValue at $[0]>" and exits 0 on success, 3 on a parse
// that returns an empty result.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cujson/cujson.h"

static bool dump(const cuJSONResult& r, const char* path)
{
    FILE* f = fopen(path, "wb");
    if (!f) return false;
    const int S = r.totalResultSize - 2;
    std::vector<int32_t> head = {S, r.depth, (int32_t)r.resultSizes.size()};
    for (int s : r.resultSizes) head.push_back(s);
    bool ok = fwrite(head.data(), 4, head.size(), f) == head.size() &&
              fwrite(r.structural, 4, (size_t)(2 * S + 4), f) == (size_t)(2 * S + 4);
    fclose(f);
    return ok;
}

int main(int argc, char** argv)
{
    if (argc < 4) return 2;
    const std::string mode = argv[1], path = argv[2];
    cuJSONResult tree;
    const char* out;
    if (mode == "std") {
        cuJSONInput input = loadJSON(path);
        if (!input.data) return 2;
        tree = parse_standard_json(input);
        cudaFreeHost(input.data);
        out = argv[3];
    } else {
        if (argc < 5) return 2;
        const size_t arg = (size_t)atoll(argv[3]);
        cuJSONLinesInput input = mode == "lines" ? loadJSONLines_chunkCount(path, arg)
                                                 : loadJSONLines_chunkSizeMegaBytes(path, arg);
        if (!input.data) return 2;
        tree = parse_json_lines(input);
        if (tree.structural == nullptr) cudaFreeHost(input.data);   // consumed only on success
        out = argv[4];
    }
    if (tree.structural == nullptr) {
        printf("empty result, status %d\n", cj_last_status());
        return 3;
    }
    if (!dump(tree, out)) return 2;
    if (mode == "std") {
        cuJSONIterator itr(&tree, path.c_str());
        itr.gotoArrayIndex(0);
        printf("first: %s\n", itr.getValue().substr(0, 40).c_str());
        itr.freeJson();
    } else {
        cuJSONLinesIterator itr(&tree, path.c_str());
        itr.gotoArrayIndex(0);
        printf("first: %s\n", itr.getValue().substr(0, 40).c_str());
        itr.freeJson();
    }
    cudaDeviceReset();
    return 0;
}
