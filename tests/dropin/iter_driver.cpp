// iter_driver.cpp -- runs a query script through a query iterator and writes
// one answer line per step.  Built twice from this one source: against
// include/cujson/cujson_iter.h (the product), and, by the recipe in
// oracle/build_ref.py, against the reference's own iterator sources
// (cujson/query/query_iterator*.cpp, prepended with -include), so that both
// answer the same scripts on the same parse result.
//
// CJ_ITER_LINES=1 selects cuJSONLinesIterator, 0 cuJSONIterator.
//
// usage: iter_driver <json file> <layout file> <script file> <answers file>
//   layout: int32 little-endian [S, depth, n_chunks, chunk_sizes[n_chunks],
//           buffer[2*(S+2)]] -- the reference result buffer (structural
//           slots 0..S+1, pair_pos = structural + S + 1).
//   script: one step per line, strings hex-encoded:
//     R            reset()
//     A <n>        gotoArrayIndex(n)
//     K <hex>      gotoKey(key)
//     F <hex>      findKey(key)             (node unchanged)
//     I <n>        increamentIndex(n)
//     V            getValue()
//     G            getKey()                 (only at a ':'; otherwise "skip")
//     D            getChar(i) for every i   (the whole node sequence)
//     S <n>        gotoNextSibling(n)       (JSON Lines only)
//     C <hex> <hex> checkKeyValue(key, value) (JSON Lines only)
//   answers: "<step> <return> <node> <nodeType> <hex string or ->"
#ifndef CJ_ITER_LINES
#define CJ_ITER_LINES 0
#endif

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#ifndef CJ_ITER_REF
#include "cujson/cujson_iter.h"
#endif

#if CJ_ITER_LINES
typedef cuJSONLinesIterator Iter;
#else
typedef cuJSONIterator Iter;
#endif

static std::string hex(const std::string& s)
{
    static const char* d = "0123456789abcdef";
    std::string o;
    for (unsigned char c : s) {
        o.push_back(d[c >> 4]);
        o.push_back(d[c & 15]);
    }
    return o.empty() ? std::string("-") : o;
}

static std::string unhex(const std::string& h)
{
    std::string o;
    if (h == "-") return o;
    for (size_t i = 0; i + 1 < h.size(); i += 2) o.push_back((char)std::stoi(h.substr(i, 2), nullptr, 16));
    return o;
}

int main(int argc, char** argv)
{
    if (argc != 5) {
        fprintf(stderr, "usage: %s json layout script answers\n", argv[0]);
        return 2;
    }
    std::ifstream lf(argv[2], std::ios::binary);
    std::vector<char> raw((std::istreambuf_iterator<char>(lf)), std::istreambuf_iterator<char>());
    std::vector<int32_t> words(raw.size() / 4);
    for (size_t i = 0; i < words.size(); i++) {
        const unsigned char* b = reinterpret_cast<const unsigned char*>(raw.data()) + 4 * i;
        words[i] = (int32_t)((uint32_t)b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24);
    }
    if (words.size() < 3) return 2;
    const int S = words[0], depth = words[1], n_chunks = words[2];
    if (n_chunks < 0 || words.size() != (size_t)(3 + n_chunks + 2 * (S + 2))) {
        fprintf(stderr, "bad layout file\n");
        return 2;
    }
    // result buffer with room past the end, as the reference's is read by the
    // iterators only inside [0, 2S+4)
    std::vector<int32_t> buffer(words.begin() + 3 + n_chunks, words.end());

    cuJSONResult res;
    res.inputJSON = nullptr;
    res.chunkCount = n_chunks;
    res.bufferSize = 0;
    int prefix = 0;
    for (int i = 0; i < n_chunks; i++) {
        res.resultSizes.push_back(words[3 + i]);
        prefix += words[3 + i];
        res.resultSizesPrefix.push_back(prefix);
    }
    res.structural = buffer.data();
    res.pair_pos = buffer.data() + S + 1;
    res.depth = depth;
    res.totalResultSize = S + 2;
    res.fileSize = S + 2;

    Iter itr(&res, argv[1]);
    std::ifstream sf(argv[3]);
    std::ofstream out(argv[4]);
    std::string line;
    while (std::getline(sf, line)) {
        if (line.empty()) continue;
        std::istringstream ls(line);
        std::string op, a, b;
        ls >> op >> a >> b;
        long ret = 0;
        std::string text = "-";
        try {
            if (op == "R") {
                itr.reset();
            } else if (op == "A") {
                ret = itr.gotoArrayIndex(std::stoi(a));
            } else if (op == "K") {
                ret = itr.gotoKey(unhex(a));
            } else if (op == "F") {
                ret = itr.findKey(unhex(a));
            } else if (op == "I") {
                ret = itr.increamentIndex(std::stoi(a));
            } else if (op == "V") {
                text = hex(itr.getValue());
            } else if (op == "G") {
                if (itr.getChar(itr.node) == ':') text = hex(itr.getKey());
                else text = "skip";
            } else if (op == "D") {
                std::string seq;
                for (int i = 0; i < S + 2; i++) seq.push_back(itr.getChar(i));
                text = hex(seq);
#if CJ_ITER_LINES
            } else if (op == "S") {
                ret = itr.gotoNextSibling(std::stoi(a));
            } else if (op == "C") {
                ret = itr.checkKeyValue(unhex(a), unhex(b)) ? 1 : 0;
#endif
            } else {
                text = "unknown";
            }
        } catch (const std::exception&) {
            text = "exception";
        }
        out << op << " " << ret << " " << itr.node << " " << (int)itr.nodeType << " " << text << "\n";
    }
    return 0;
}
