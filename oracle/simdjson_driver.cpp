// simdjson_driver.cpp -- times simdjson (the copy the reference ships under
// paper_reproduced/related_works/simdjson/, compiled from there by
// oracle/build_ref.py) on one input file.  TEST / MEASUREMENT INFRASTRUCTURE:
// a CPU data point beside the GPU parse, never part of the product.
//
// usage: simdjson_bench <file> <mode> <threads> <reps>
//   mode dom       dom::parser::parse -- UTF-8 validation, structural index
//                  and the full tape (all of cuJSON's stages)
//   mode index     ondemand::parser::iterate -- UTF-8 validation and the
//                  structural index (cuJSON's stages 1-2)
//   mode lines     dom::parser::parse_many over a JSON-Lines file
// Each thread runs its own parser over the same bytes (independent
// instances); prints one line: mode threads bytes seconds GB/s.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

#include "simdjson.h"

int main(int argc, char** argv)
{
    if (argc < 5) {
        fprintf(stderr, "usage: %s file dom|index|lines threads reps\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[2];
    const int threads = atoi(argv[3]), reps = atoi(argv[4]);
    simdjson::padded_string doc;
    if (simdjson::padded_string::load(argv[1]).get(doc)) {
        fprintf(stderr, "cannot load %s\n", argv[1]);
        return 1;
    }
    std::atomic<int> bad{0};
    auto work = [&]() {
        if (mode == "dom") {
            simdjson::dom::parser p;
            p.allocate(doc.size(), 1024);
            for (int r = 0; r < reps; r++) {
                simdjson::dom::element e;
                if (p.parse(doc).get(e)) bad++;
            }
        } else if (mode == "index") {
            simdjson::ondemand::parser p(doc.size());
            for (int r = 0; r < reps; r++) {
                simdjson::ondemand::document d;
                if (p.iterate(doc).get(d)) bad++;
            }
        } else {
            simdjson::dom::parser p;
            for (int r = 0; r < reps; r++) {
                simdjson::dom::document_stream s;
                if (p.parse_many(doc, 1 << 24).get(s)) { bad++; continue; }
                size_t n = 0;
                for (auto d : s) {
                    if (d.error()) { bad++; break; }
                    n++;
                }
                if (!n) bad++;
            }
        }
    };
    std::vector<std::thread> pool;
    const auto t0 = std::chrono::steady_clock::now();
    for (int t = 0; t < threads; t++) pool.emplace_back(work);
    for (auto& th : pool) th.join();
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const double bytes = (double)doc.size() * reps * threads;
    printf("%s %d %zu %.4f %.3f%s\n", mode.c_str(), threads, doc.size(), s, bytes / s / 1e9,
           bad ? " ERRORS" : "");
    return bad ? 1 : 0;
}
