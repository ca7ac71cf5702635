// cj_synth.cpp -- seeded synthetic JSON / JSON-Lines generator.
//
// The reference is evaluated on six ~1 GB real-world datasets that are not
// available offline.  These generators stand in for them: standard documents
// (a top-level array of objects), JSON-Lines files of object records with
// lognormal sizes, and the invalid / adversarial variants the batch and serving
// workloads need.  Everything is derived from one 64-bit seed through
// std::mt19937_64, block by block, so output is identical on every machine and
// for any thread count.
#include "cj_synth.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

struct Gen {
    std::mt19937_64 rng;
    const cj_synth_params& p;
    std::string out;

    Gen(uint64_t seed, const cj_synth_params& prm) : rng(seed), p(prm) {}

    uint64_t u64() { return rng(); }
    // uniform integer in [lo, hi]
    int64_t uni(int64_t lo, int64_t hi) {
        return lo + (int64_t)(rng() % (uint64_t)(hi - lo + 1));
    }
    double unit() { return (rng() >> 11) * (1.0 / 9007199254740992.0); }

    void key() {
        static const char alpha[] = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ0123456789_";
        int len = (int)uni(3, 20);
        out.push_back('"');
        for (int i = 0; i < len; i++) out.push_back(alpha[rng() % 63]);
        out.push_back('"');
    }

    // one UTF-8 character of 2, 3 or 4 bytes, always well formed
    void utf8_char() {
        int kind = (int)uni(2, 4);
        uint32_t cp;
        if (kind == 2) cp = (uint32_t)uni(0x80, 0x7FF);
        else if (kind == 3) {
            do { cp = (uint32_t)uni(0x800, 0xFFFF); } while (cp >= 0xD800 && cp <= 0xDFFF);
        } else cp = (uint32_t)uni(0x10000, 0x10FFFF);
        if (cp < 0x800) {
            out.push_back((char)(0xC0 | (cp >> 6)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        } else if (cp < 0x10000) {
            out.push_back((char)(0xE0 | (cp >> 12)));
            out.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        } else {
            out.push_back((char)(0xF0 | (cp >> 18)));
            out.push_back((char)(0x80 | ((cp >> 12) & 0x3F)));
            out.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        }
    }

    // printable ASCII body character: letters, digits, spaces and the JSON
    // structural characters (so the in-string mask is exercised), never a quote
    // or a backslash
    char plain_char() {
        static const char pool[] =
            "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ0123456789     .-_/{}[]:,";
        return pool[rng() % (sizeof(pool) - 1)];
    }

    void string_value(int64_t max_len) {
        int64_t len = uni(p.str_min, p.str_max);
        if (max_len > 0 && len > max_len) len = std::max<int64_t>(1, max_len);
        double kind = unit();
        out.push_back('"');
        if (p.huge_string_frac > 0 && unit() < p.huge_string_frac) {
            huge_string_body();
        } else if (kind < 0.70) {
            for (int64_t i = 0; i < len; i++) out.push_back(plain_char());
        } else if (kind < 0.95) {
            // 5% of positions are an escaped quote or an escaped backslash
            for (int64_t i = 0; i < len; i++) {
                if (unit() < 0.05) {
                    out.push_back('\\');
                    out.push_back((rng() & 1) ? '"' : '\\');
                } else out.push_back(plain_char());
            }
        } else {
            for (int64_t i = 0; i < len; i++) {
                if (unit() < 0.3) utf8_char(); else out.push_back(plain_char());
            }
        }
        out.push_back('"');
    }

    // >64 KB string made of long backslash runs (even lengths, so each run is
    // a sequence of escaped backslashes), escaped quotes after even runs, and
    // plain text -- the runs cross every tile and word boundary
    void huge_string_body() {
        int64_t len = uni(p.huge_string_min, p.huge_string_max);
        int64_t written = 0;
        while (written < len) {
            double r = unit();
            if (r < 0.4) {
                int64_t run = 2 * uni(1, 6000);
                out.append((size_t)run, '\\');
                written += run;
                if (rng() & 1) { out.append("\\\""); written += 2; }
            } else {
                int64_t k = uni(1, 400);
                for (int64_t i = 0; i < k; i++) out.push_back(plain_char());
                written += k;
            }
        }
    }

    void number() {
        if (rng() & 1) {
            int64_t v = (int64_t)u64();
            out += std::to_string(v);
        } else {
            char buf[64];
            double mant = (unit() * 2.0 - 1.0) * 9.999;
            int ex = (int)uni(-300, 300);
            snprintf(buf, sizeof buf, "%.*fe%+d", (int)uni(1, 9), mant, ex);
            out += buf;
        }
    }

    void ws() { if ((rng() & 7) == 0) out.push_back(' '); }

    void value(int depth) {
        double r = unit();
        if (r < 0.40) string_value(0);
        else if (r < 0.65) number();
        else if (r < 0.75) {
            int k = (int)(rng() % 3);
            out += (k == 0) ? "true" : (k == 1) ? "false" : "null";
        } else if (depth < p.max_depth) {
            int n = (int)uni(0, p.nested_max_items);
            if (rng() & 1) {
                out.push_back('{');
                for (int i = 0; i < n; i++) {
                    if (i) { out.push_back(','); ws(); }
                    key(); out.push_back(':'); ws(); value(depth + 1);
                }
                out.push_back('}');
            } else {
                out.push_back('[');
                for (int i = 0; i < n; i++) {
                    if (i) { out.push_back(','); ws(); }
                    value(depth + 1);
                }
                out.push_back(']');
            }
        } else {
            string_value(0);
        }
    }

    // a top-level record object with keys_min..keys_max members
    void record_object(int depth) {
        int n = (int)uni(p.keys_min, p.keys_max);
        out.push_back('{');
        for (int i = 0; i < n; i++) {
            if (i) { out.push_back(','); ws(); }
            key(); out.push_back(':'); ws(); value(depth + 1);
        }
        out.push_back('}');
    }

    // a JSON-Lines record of roughly `target` bytes
    void sized_record(size_t target) {
        size_t start = out.size();
        out.push_back('{');
        bool first = true;
        while (out.size() - start + 2 < target || first) {
            if (!first) out.push_back(',');
            first = false;
            key(); out.push_back(':');
            int64_t room = (int64_t)target - (int64_t)(out.size() - start) - 3;
            double r = unit();
            if (r < 0.40 || room < 24) string_value(std::max<int64_t>(1, room));
            else if (r < 0.65) number();
            else if (r < 0.75) out += (rng() & 1) ? "true" : "null";
            else value(1);
        }
        out.push_back('}');
    }
};

// Fill `budget` bytes with comma-separated top-level objects (no leading or
// trailing comma), padding with spaces.  Each block has its own RNG stream.
void fill_block(uint64_t seed, const cj_synth_params& p, size_t budget, uint8_t* dst)
{
    Gen g(seed, p);
    g.out.reserve(budget + 4096);
    std::string one;
    size_t used = 0;
    bool first = true;
    while (true) {
        size_t mark = g.out.size();
        if (!first) g.out.push_back(',');
        g.record_object(1);
        if (g.out.size() > budget) {          // does not fit: drop it
            g.out.resize(mark);
            break;
        }
        first = false;
        used = g.out.size();
        if (budget - used < 16) break;
    }
    memcpy(dst, g.out.data(), used);
    memset(dst + used, ' ', budget - used);
}

// Event-log records: one object per line shaped like a public activity feed
// (an id, an event "type", actor / repo / payload objects, a timestamp) -- the
// record shape the reference's real-world query runs over (counting the
// records whose "type" is "PushEvent").  Values are random; what the shape
// exercises is the query: nested objects that hold a "type" member of their
// own, "type" placed after them in some records, absent in some, near-miss
// values, spacing after ',' and ':' in some records, and blank lines.
struct EventGen {
    std::mt19937_64 rng;
    std::string out;
    explicit EventGen(uint64_t seed) : rng(seed) {}

    double unit() { return (rng() >> 11) * (1.0 / 9007199254740992.0); }
    int64_t uni(int64_t lo, int64_t hi) { return lo + (int64_t)(rng() % (uint64_t)(hi - lo + 1)); }

    void word(int lo, int hi) {
        static const char a[] = "abcdefghijklmnopqrstuvwxyz0123456789-";
        int n = (int)uni(lo, hi);
        for (int i = 0; i < n; i++) out.push_back(a[rng() % 37]);
    }
    void hex(int n) {
        static const char h[] = "0123456789abcdef";
        for (int i = 0; i < n; i++) out.push_back(h[rng() & 15]);
    }
    void num(int64_t lo, int64_t hi) { out += std::to_string(uni(lo, hi)); }
    void text(int lo, int hi) {        // free text with escapes and a few UTF-8 characters
        static const char a[] = "abcdefghijklmnopqrstuvwxyz ABCDEFGHIJ .,:;{}[]-_/#0123456789";
        int n = (int)uni(lo, hi);
        for (int i = 0; i < n; i++) {
            double r = unit();
            if (r < 0.02) out += "\\n";
            else if (r < 0.03) out += "\\\"";
            else if (r < 0.035) out += "\xc3\xa9";
            else out.push_back(a[rng() % (sizeof(a) - 1)]);
        }
    }

    const char* sep;   // "," or ", "
    const char* col;   // ":" or ": "
    void key(const char* k) {
        out.push_back('"');
        out += k;
        out.push_back('"');
        out += col;
    }
    void str_member(const char* k, bool first = false) {
        if (!first) out += sep;
        key(k);
    }

    void user(const char* k) {         // {"id":..,"login":"..","type":"User",..}
        out += sep;
        key(k);
        out += "{";
        key("id"); num(1, 99999999);
        out += sep; key("login"); out += '"'; word(3, 16); out += '"';
        out += sep; key("gravatar_id"); out += "\"\"";
        if (unit() < 0.5) { out += sep; key("type"); out += unit() < 0.9 ? "\"User\"" : "\"Organization\""; }
        out += sep; key("url"); out += "\"https://api.example.invalid/users/"; word(3, 16); out += '"';
        out += "}";
    }
    void repo() {
        out += sep; key("repo"); out += "{";
        key("id"); num(1, 99999999);
        out += sep; key("name"); out += '"'; word(3, 12); out += '/'; word(2, 20); out += '"';
        out += sep; key("url"); out += "\"https://api.example.invalid/repos/"; word(3, 12); out += '"';
        out += "}";
    }
    void payload(int kind) {
        out += sep; key("payload"); out += "{";
        if (kind == 0) {               // pushes: commits with messages
            int n = (int)uni(1, 6);
            key("push_id"); num(1, 999999999);
            out += sep; key("size"); out += std::to_string(n);
            out += sep; key("distinct_size"); out += std::to_string(n);
            out += sep; key("ref"); out += "\"refs/heads/"; word(3, 12); out += '"';
            out += sep; key("head"); out += '"'; hex(40); out += '"';
            out += sep; key("before"); out += '"'; hex(40); out += '"';
            out += sep; key("commits"); out += "[";
            for (int i = 0; i < n; i++) {
                if (i) out += sep;
                out += "{"; key("sha"); out += '"'; hex(40); out += '"';
                out += sep; key("author"); out += "{"; key("email"); out += '"'; word(3, 10); out += "@example.invalid\"";
                out += sep; key("name"); out += '"'; word(3, 14); out += "\"}";
                out += sep; key("message"); out += '"'; text(8, 160); out += '"';
                out += sep; key("distinct"); out += (rng() & 1) ? "true" : "false";
                out += "}";
            }
            out += "]";
        } else if (kind == 1) {        // branch / tag creation
            key("ref"); out += '"'; word(3, 12); out += '"';
            out += sep; key("ref_type"); out += (rng() & 1) ? "\"branch\"" : "\"tag\"";
            out += sep; key("master_branch"); out += "\"main\"";
            out += sep; key("description"); out += unit() < 0.3 ? std::string("null") : std::string("\"x\"");
        } else if (kind == 2) {        // issues and comments, with nested users that have a "type"
            key("action"); out += "\"created\"";
            out += sep; key("issue"); out += "{";
            key("number"); num(1, 99999);
            out += sep; key("title"); out += '"'; text(4, 60); out += '"';
            user("user");
            out += sep; key("labels"); out += "[";
            int n = (int)uni(0, 3);
            for (int i = 0; i < n; i++) {
                if (i) out += sep;
                out += "{"; key("name"); out += '"'; word(3, 10); out += "\"}";
            }
            out += "]";
            out += sep; key("body"); out += '"'; text(0, 300); out += '"';
            out += "}";
        } else {                       // one-word actions
            key("action"); out += "\"started\"";
        }
        out += "}";
    }

    // One record; returns 1 if its top-level "type" is exactly PushEvent.
    int record() {
        static const char* types[] = {"PushEvent", "CreateEvent", "WatchEvent", "IssueCommentEvent",
                                      "PullRequestEvent", "IssuesEvent", "ForkEvent", "DeleteEvent",
                                      "GollumEvent", "ReleaseEvent", "MemberEvent", "PublicEvent"};
        static const double cum[] = {0.50, 0.62, 0.72, 0.80, 0.85, 0.89, 0.92, 0.95, 0.96, 0.97, 0.98, 1.0};
        const bool spaced = unit() < 0.2;
        sep = spaced ? ", " : ",";
        col = spaced ? ": " : ":";
        double r = unit();
        int t = 0;
        while (cum[t] < r) t++;
        const int pk = t == 0 ? 0 : t == 1 || t == 7 ? 1 : t == 3 || t == 5 ? 2 : 3;
        // where "type" goes: 0 second (usual), 1 after the nested objects, 2 absent
        double w = unit();
        const int place = w < 0.94 ? 0 : w < 0.99 ? 1 : 2;
        // the value written: the type name, or (1%) a near miss
        std::string tv = std::string("\"") + types[t] + "\"";
        double m = unit();
        if (m < 0.0025) tv = "\"PushEventX\"";
        else if (m < 0.005) tv = "\"pushEvent\"";
        else if (m < 0.0075) tv = "null";
        else if (m < 0.01) tv = "{\"type\":\"PushEvent\"}";
        const int hit = place != 2 && tv == "\"PushEvent\"";
        out += "{";
        key("id"); out += '"'; num(1000000000, 9999999999); out += '"';
        if (place == 0) { out += sep; key("type"); out += tv; }
        user("actor");
        repo();
        payload(pk);
        if (place == 1) { out += sep; key("type"); out += tv; }
        out += sep; key("public"); out += (unit() < 0.98) ? "true" : "false";
        out += sep; key("created_at"); out += "\"2015-01-";
        out += std::to_string(10 + uni(0, 18)); out += "T"; out += std::to_string(10 + uni(0, 13));
        out += ":00:00Z\"";
        if (unit() < 0.2) user("org");
        out += "}";
        return hit;
    }
};

void run_parallel(size_t nblocks, unsigned threads, const std::function<void(size_t)>& fn)
{
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    threads = (unsigned)std::min<size_t>(threads, std::max<size_t>(1, nblocks));
    std::vector<std::thread> pool;
    std::atomic<size_t> next{0};
    for (unsigned t = 0; t < threads; t++)
        pool.emplace_back([&] {
            for (size_t b; (b = next.fetch_add(1)) < nblocks;) fn(b);
        });
    for (auto& th : pool) th.join();
}
}  // namespace

extern "C" {

void cj_synth_default_params(cj_synth_params* p)
{
    memset(p, 0, sizeof(*p));
    p->max_depth = 6;
    p->keys_min = 10;
    p->keys_max = 30;
    p->nested_max_items = 4;
    p->str_min = 8;
    p->str_max = 200;
    p->huge_string_frac = 0.0;
    p->huge_string_min = 64 * 1024;
    p->huge_string_max = 256 * 1024;
    p->block_bytes = 4u << 20;
    p->record_median = 200.0;
    p->record_sigma = 0.7;
    p->record_min = 50;
    p->record_max = 2048;
    p->threads = 0;
}

// Standard JSON: '[' + blocks of objects joined by ',' + ']' and spaces, exactly
// `size` bytes.  Needs size >= 2.
size_t cj_synth_document(uint64_t seed, size_t size, const cj_synth_params* pp, uint8_t* out)
{
    cj_synth_params p;
    if (pp) p = *pp; else cj_synth_default_params(&p);
    if (size < 2 || !out) return 0;
    size_t bb = p.block_bytes ? p.block_bytes : (4u << 20);
    // blocks of objects fill [1, size-1); each block after the first is
    // preceded by one separator byte
    memset(out, ' ', size);
    std::vector<size_t> off, len;
    size_t pos = 1, end = size - 1;
    while (pos < end) {
        if (!off.empty()) { pos++; if (pos >= end) break; }
        size_t want = std::min(bb, end - pos);
        if (end - pos - want < bb / 4) want = end - pos;   // no tiny tail block
        off.push_back(pos); len.push_back(want); pos += want;
    }
    size_t nblocks = off.size();
    out[0] = '[';
    run_parallel(nblocks, p.threads, [&](size_t b) {
        fill_block(seed * 0x9E3779B97F4A7C15ull + b + 1, p, len[b], out + off[b]);
    });
    // a ',' between two blocks is only valid when both hold an object; put it
    // in the separator slot when the previous block's text ends in '}' and the
    // next one starts with '{'
    for (size_t b = 1; b < nblocks; b++) {
        size_t s = off[b] - 1;
        if (len[b] == 0 || out[off[b]] != '{') continue;
        // find the last non-space byte before the separator
        size_t q = s;
        bool prev_obj = false;
        while (q > 0) { q--; if (out[q] != ' ') { prev_obj = (out[q] == '}'); break; } }
        if (prev_obj) out[s] = ',';
    }
    out[0] = '[';
    out[size - 1] = ']';
    return size;
}

// JSON Lines: records of lognormal size (clamped), one per line, exactly `size`
// bytes; the last line is padded with spaces and ends in '\n'.  Returns bytes
// written and the record count through *n_records.
size_t cj_synth_lines(uint64_t seed, size_t size, const cj_synth_params* pp, uint8_t* out,
                      uint64_t* n_records)
{
    cj_synth_params p;
    if (pp) p = *pp; else cj_synth_default_params(&p);
    if (!out || size < 4) return 0;
    size_t bb = p.block_bytes ? p.block_bytes : (4u << 20);
    size_t nblocks = std::max<size_t>(1, size / bb);     // the last block takes the tail
    std::vector<uint64_t> counts(nblocks, 0);
    run_parallel(nblocks, p.threads, [&](size_t b) {
        size_t start = b * bb, budget = (b + 1 == nblocks) ? size - start : bb;
        Gen g(seed * 0xD1B54A32D192ED03ull + b + 7, p);
        g.out.reserve(budget + 4096);
        std::lognormal_distribution<double> ln(std::log(p.record_median), p.record_sigma);
        size_t used = 0;
        uint64_t cnt = 0;
        while (true) {
            size_t mark = g.out.size();
            double t = ln(g.rng);
            size_t target = (size_t)std::clamp(t, (double)p.record_min, (double)p.record_max);
            g.sized_record(target);
            g.out.push_back('\n');
            if (g.out.size() > budget) { g.out.resize(mark); break; }
            used = g.out.size();
            cnt++;
        }
        memcpy(out + start, g.out.data(), used);
        // pad: spaces then a newline, so the block is a whole number of lines
        if (budget > used) {
            memset(out + start + used, ' ', budget - used);
            out[start + budget - 1] = '\n';
            if (budget - used == 1 && used == 0) out[start] = '\n';
        }
        counts[b] = cnt;
    });
    if (n_records) {
        uint64_t t = 0;
        for (auto c : counts) t += c;
        *n_records = t;
    }
    return size;
}

// Event-log JSON Lines (EventGen above), exactly `size` bytes, blocks of 4 MiB
// generated in parallel; blank lines between some records; the tail of every
// block is spaces and a newline.  Returns bytes written; the record count and
// the count of records whose top-level "type" is "PushEvent" through the
// pointers.
size_t cj_synth_events(uint64_t seed, size_t size, uint8_t* out, uint64_t* n_records, uint64_t* n_push)
{
    if (!out || size < 4) return 0;
    const size_t bb = 4u << 20;
    const size_t nblocks = std::max<size_t>(1, size / bb);
    std::vector<uint64_t> counts(nblocks, 0), hits(nblocks, 0);
    run_parallel(nblocks, 0, [&](size_t b) {
        const size_t start = b * bb, budget = (b + 1 == nblocks) ? size - start : bb;
        EventGen g(seed * 0xA0761D6478BD642Full + b + 11);
        g.out.reserve(budget + 8192);
        size_t used = 0;
        uint64_t cnt = 0, hit = 0;
        while (true) {
            const size_t mark = g.out.size();
            const int h = g.record();
            g.out.push_back('\n');
            if (g.unit() < 0.002) g.out.push_back('\n');
            if (g.out.size() > budget) { g.out.resize(mark); break; }
            used = g.out.size();
            cnt++;
            hit += h;
        }
        memcpy(out + start, g.out.data(), used);
        if (budget > used) {
            memset(out + start + used, ' ', budget - used);
            out[start + budget - 1] = '\n';
        }
        counts[b] = cnt;
        hits[b] = hit;
    });
    uint64_t c = 0, h = 0;
    for (size_t b = 0; b < nblocks; b++) { c += counts[b]; h += hits[b]; }
    if (n_records) *n_records = c;
    if (n_push) *n_push = h;
    return size;
}

// Nesting `depth` deep: '[' * depth + ']' * depth (2*depth bytes).
size_t cj_synth_deep(size_t depth, uint8_t* out)
{
    memset(out, '[', depth);
    memset(out + depth, ']', depth);
    return 2 * depth;
}

// One string of `body` bytes of backslash runs: ["\\\\...\"..."] with even runs
// and escaped quotes, exactly body + 4 bytes.
size_t cj_synth_backslash_string(uint64_t seed, size_t body, uint8_t* out)
{
    std::mt19937_64 rng(seed);
    out[0] = '[';
    out[1] = '"';
    size_t i = 2, end = 2 + body;
    while (i < end) {
        size_t run = 2 * (1 + rng() % 4000);
        if (i + run > end) run = (end - i) & ~(size_t)1;
        if (run == 0) break;
        memset(out + i, '\\', run);
        i += run;
        if (i + 2 <= end && (rng() & 1)) { out[i++] = '\\'; out[i++] = '"'; }
        else if (i < end) { out[i++] = 'x'; }
    }
    while (i < end) out[i++] = 'y';
    out[end] = '"';
    out[end + 1] = ']';
    return body + 4;
}

// Make a generated document invalid in place.  kind 1: overlong C0 80,
// 2: overlong E0 80 80, 3: surrogate ED A0 80 -- written over the body of the
// first string long enough; kind 4: remove the final ']' (unbalanced);
// kind 5: turn the final ']' into '}' (mismatched).  Returns 1 on success.
int cj_synth_corrupt(uint8_t* doc, size_t n, int kind, uint64_t seed)
{
    if (kind >= 4) {
        for (size_t i = n; i-- > 0;) {
            if (doc[i] == ']') { doc[i] = (kind == 4) ? ' ' : '}'; return 1; }
        }
        return 0;
    }
    static const uint8_t seqs[3][3] = {{0xC0, 0x80, 0}, {0xE0, 0x80, 0x80}, {0xED, 0xA0, 0x80}};
    size_t len = (kind == 1) ? 2 : 3;
    // start looking at a seeded offset and find a plain run inside a string
    size_t start = n ? (size_t)(seed % n) : 0;
    for (size_t pass = 0; pass < 2; pass++) {
        size_t lo = pass ? 0 : start, hi = pass ? start : n;
        int in_str = 0;
        // recompute string state from the beginning: cheap enough for tests
        size_t bs = 0;
        for (size_t i = 0; i < n; i++) {
            uint8_t c = doc[i];
            if (c == '"' && (bs & 1) == 0) in_str ^= 1;
            bs = (c == '\\') ? bs + 1 : 0;
            if (i < lo || i >= hi || !in_str || c == '"') continue;
            bool ok = (i + len + 1 < n);
            for (size_t k = 0; ok && k < len + 1; k++) {
                uint8_t d = doc[i + k];
                if (d == '"' || d == '\\' || d >= 0x80) ok = false;
            }
            if (ok) { memcpy(doc + i, seqs[kind - 1], len); return 1; }
        }
    }
    return 0;
}

}  // extern "C"
