// driver.cpp -- runs the reference's own parse code (compiled for the CPU
// through cj_cuda_emu.h, see oracle/build_ref.py) on one input and writes
// what it returned.  TEST INFRASTRUCTURE ONLY: its outputs are golden vectors
// for the parity tests.
//
// usage: refemu_std   <input> <output>
//        refemu_lines <input> <output> <chunk size>...
// output (int32 little-endian): status (0 ok, 1 the reference called exit()
// -- its invalid-input path --, 2 empty result), S, then structural[1..S],
// then pair_pos[1..S] with the entries at non-opens set to 0 (the reference
// leaves them uninitialised).
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <inttypes.h>
#include <sys/resource.h>
#include <time.h>

#include <algorithm>
#include <bitset>
#include <chrono>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <queue>
#include <sstream>
#include <string>
#include <thread>
#include <vector>
#include <x86intrin.h>

#include "cuda_runtime.h"

// the reference ends the process on invalid input; here that becomes an exception
#define exit(c) throw cj_ref_exit{(c)}

#include "utils.cu"
#if CJ_REF_LINES
#include "parse_json_lines.cu"
#else
#include "parse_standard_json.cu"
#endif

#undef exit

static void write_out(const char* path, int32_t status, const std::vector<int32_t>& st,
                      const std::vector<int32_t>& pr)
{
    FILE* f = fopen(path, "wb");
    if (!f) std::exit(3);
    const int32_t S = (int32_t)st.size();
    fwrite(&status, 4, 1, f);
    fwrite(&S, 4, 1, f);
    if (S) {
        fwrite(st.data(), 4, S, f);
        fwrite(pr.data(), 4, S, f);
    }
    fclose(f);
}

int main(int argc, char** argv)
{
#if CJ_REF_LINES
    if (argc < 4) return 2;
#else
    if (argc != 3) return 2;
#endif
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    fseek(f, 0, SEEK_END);
    const size_t n = (size_t)ftell(f);
    fseek(f, 0, SEEK_SET);
    uint8_t* data = nullptr;
    cudaHostAlloc(&data, n + 64, cudaHostAllocDefault);
    if (fread(data, 1, n, f) != n) return 2;
    fclose(f);
    std::vector<uint8_t> copy(data, data + n);   // the lines parse frees its input

    cuJSONResult r;
    int32_t status = 0;
    try {
#if CJ_REF_LINES
        cuJSONLinesInput in;
        in.data = data;
        in.size = n;
        size_t off = 0;
        for (int i = 3; i < argc; i++) {
            const size_t cs = (size_t)strtoull(argv[i], nullptr, 10);
            in.chunks.push_back(data + off);
            in.chunksSize.push_back(cs);
            off += cs;
        }
        in.chunkCount = in.chunks.size();
        r = parse_json_lines(in);
#else
        cuJSONInput in{data, n};
        r = parse_standard_json(in);
#endif
    } catch (const cj_ref_exit&) {
        status = 1;
    }
    std::vector<int32_t> st, pr;
    if (status == 0 && r.structural == nullptr) status = 2;
    if (status == 0) {
        const int32_t S = r.totalResultSize - 2;
        for (int32_t i = 1; i <= S; i++) {
            const int32_t p = r.structural[i];
            st.push_back(p);
            const uint8_t c = (p >= 1 && (size_t)p <= n) ? copy[p - 1] : 0;
            pr.push_back((c == '{' || c == '[') ? r.pair_pos[i] : 0);
        }
    }
    write_out(argv[2], status, st, pr);
    return 0;
}
