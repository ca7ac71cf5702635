// cj_model.cpp -- sequential CPU model of the parse kernels (test helper).
//
// Runs the scan kernels' algorithm region by region, with the same bit
// functions (cujson_gb300/csrc/cj_device.cuh): the per-region transfer tables
// (computed as if each region were entered outside strings and escapes), their
// composition in randomly sized blocks (checked against the running value),
// and the emit pass from each region's exact entry state; then the pairing
// kernels' chunk and spine logic with __match_any_sync emulated per 32-record
// round.  Tests compare it with the oracle to check the algorithm itself
// without a GPU.
#include <algorithm>
#include <array>
#include <climits>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "cj_device.cuh"

struct uint2 { uint32_t x, y; };
struct int4 { int32_t x, y, z, w; };

using namespace cj;

namespace {

struct Seg { uint64_t off, len, logical; bool cont; };

bool utf8_ok32(const uint8_t* sb, uint64_t slen, uint64_t o0) {
    auto lead_len = [](uint32_t b) {
        if (b >= 0xC2 && b <= 0xDF) return 2;
        if (b >= 0xE0 && b <= 0xEF) return 3;
        if (b >= 0xF0 && b <= 0xF4) return 4;
        return 1;
    };
    for (int j = 0; j < 32; j++) {
        uint64_t o = o0 + j;
        if (o >= slen) break;
        uint32_t b = sb[o];
        if (b < 0x80) continue;
        if (b < 0xC0) {
            bool ok = false;
            for (uint64_t k = 1; k <= 3 && k <= o; k++) {
                uint32_t pb = sb[o - k];
                if ((pb & 0xC0) == 0x80) continue;
                ok = lead_len(pb) > (int)k;
                break;
            }
            if (!ok) return false;
            continue;
        }
        int L; uint32_t lo = 0x80, hi = 0xBF;
        if (b <= 0xC1) return false;
        else if (b <= 0xDF) L = 2;
        else if (b == 0xE0) { L = 3; lo = 0xA0; }
        else if (b == 0xED) { L = 3; hi = 0x9F; }
        else if (b <= 0xEF) L = 3;
        else if (b == 0xF0) { L = 4; lo = 0x90; }
        else if (b <= 0xF3) L = 4;
        else if (b == 0xF4) { L = 4; hi = 0x8F; }
        else return false;
        if (o + L > slen) return false;
        if (sb[o + 1] < lo || sb[o + 1] > hi) return false;
        for (int k = 2; k < L; k++) if ((sb[o + k] & 0xC0) != 0x80) return false;
    }
    return true;
}

}  // namespace

extern "C" int cjm_parse(const uint8_t* data, size_t n, int lines, const size_t* chunk_sizes,
                         size_t n_chunks, int32_t* out_pos, int32_t* out_pair, size_t cap,
                         int64_t* out_S, uint32_t* out_flags, uint64_t seed)
{
    size_t one = n;
    if (!chunk_sizes) { chunk_sizes = &one; n_chunks = 1; }
    std::vector<Seg> segs;
    uint64_t logical = 0;
    for (size_t i = 0; i < n_chunks; i++) {
        segs.push_back({logical, chunk_sizes[i], logical, i > 0});
        logical += chunk_sizes[i];
    }
    std::mt19937_64 rng(seed);
    uint32_t flags = 0;
    std::vector<int32_t> pos, pair;
    std::vector<uint2> brk;
    // region size as the tuned kernels choose it (4, 8 or 16 KiB), drawn per call
    const int R = kRegionStepsAllowed[rng() % 3];
    const uint64_t RB = (uint64_t)R * kStepBytes;
    constexpr int W = 16 * kStepBytes / 32;    // 32-byte words of the largest region

    // ---- scan_tables: one transfer table per region ------------------------------
    struct RegionRef { size_t seg; uint64_t off; int len; bool first; };
    std::vector<RegionRef> regions;
    std::vector<std::array<Ent, 4>> tabs;
    for (size_t si = 0; si < segs.size(); si++) {
        const Seg& sg = segs[si];
        const uint8_t* sb = data + sg.off;
        const uint64_t nreg = (sg.len + RB - 1) / RB;
        for (uint64_t ri = 0; ri < nreg; ri++) {
            const uint64_t off = ri * RB;
            const int len = (int)std::min<uint64_t>(RB, sg.len - off);
            const bool first = ri == 0;
            regions.push_back({si, off, len, first});
            static Classes c[W];
            static uint32_t cout0[W];
            static bool all_bs[W];
            const int nw = (len + 31) / 32;
            // UTF-8 as the kernel checks it: on the bit planes, the carry handed
            // lane to lane and step to step, and taken afresh from the 4 bytes
            // before each region
            uint32_t pw = 0;
            for (int b = 0; b < 4; b++) {
                const int64_t o = (int64_t)off - 4 + b;
                if (o >= 0) pw |= (uint32_t)sb[o] << (8 * b);
            }
            uint32_t ucarry = utf8_carry_word(pw);
            for (int t = 0; t < nw; t++) {
                uint32_t w[8];
                for (int k = 0; k < 8; k++) {
                    uint32_t v = 0;
                    for (int b = 0; b < 4; b++) {
                        const int o = t * 32 + k * 4 + b;
                        if (o < len) v |= (uint32_t)sb[off + o] << (8 * b);
                    }
                    w[k] = v;
                }
                uint32_t P[8];
                bit_planes32(w, P);
                c[t] = lines ? classify_planes<true>(P) : classify_planes<false>(P);
                const bool seg_end = off + (uint64_t)t * 32 + 32 >= sg.len;
                const uint32_t next = utf8_carry_planes(P);
                if (utf8_errors_planes(P, ucarry, seg_end)) flags |= 1;
                ucarry = next;
                escaped32(c[t].bs, 0, &cout0[t]);
                all_bs[t] = c[t].bs == 0xFFFFFFFFu;
            }
            // the region entered without escape and outside strings
            uint32_t carry = 0, par = 0;
            bool tall = true;
            uint32_t tflip = 0, tcout = 0;
            int32_t C0 = 0, Ct = 0, K0 = 0, Kt = 0, O0 = 0, Ot = 0;
            for (int t = 0; t < nw; t++) {
                uint32_t dummy;
                const uint32_t esc = escaped32(c[t].bs, carry, &dummy);
                const uint32_t rq = c[t].q & ~esc;
                const uint32_t M = prefix_xor(rq) ^ (par ? 0xFFFFFFFFu : 0u);
                par ^= __builtin_popcount(rq) & 1;
                if (!all_bs[t]) {
                    if (tall) tflip = (c[t].q >> __builtin_ctz(~c[t].bs)) & 1;
                    tall = false;
                    carry = cout0[t];
                    tcout = cout0[t];
                }
                C0 += __builtin_popcount(c[t].st & ~M); Ct += __builtin_popcount(c[t].st);
                K0 += __builtin_popcount(c[t].br & ~M); Kt += __builtin_popcount(c[t].br);
                O0 += __builtin_popcount(c[t].op & ~M); Ot += __builtin_popcount(c[t].op);
            }
            const int32_t D0 = 2 * O0 - K0, Dt = 2 * Ot - Kt;
            std::array<Ent, 4> T;
            for (uint32_t st = 0; st < 4; st++) {
                const uint32_t s0 = first ? 0 : st;
                const uint32_t escin = s0 >> 1, instr = s0 & 1;
                const uint32_t e = instr ^ (escin & tflip);
                T[st].st = ((tall ? escin : tcout) << 1) | (e ^ par);
                if (first) T[st].st |= kResetState | (sg.cont ? 0u : kResetCounts);
                T[st].s = e ? Ct - C0 : C0;
                T[st].k = e ? Kt - K0 : K0;
                T[st].d = e ? Dt - D0 : D0;
            }
            tabs.push_back(T);
        }
    }

    // ---- prefix: entry values by composing tables in random blocks -------------
    // (the prefix kernels compose per-thread runs, warp scans and block
    // aggregates; any grouping must give the running value)
    const size_t NR = regions.size();
    std::vector<Ent> entry(NR);
    {
        Ent run = ent_identity(0);
        size_t r = 0;
        Ent base = ent_identity(0);
        while (r < NR) {
            const size_t blk = 1 + rng() % 37;
            const size_t hi = std::min(NR, r + blk);
            Ent acc[4];
            tab_identity(acc);
            for (size_t u = r; u < hi; u++) {
                // the value before region u from the block start: base, then acc
                const Ent v = ent_apply(base, acc);
                if (v.st != run.st || v.s != run.s || v.k != run.k || v.d != run.d) flags |= 0x100;
                entry[u] = v;
                run = ent_apply(run, tabs[u].data());
                tab_compose(acc, tabs[u].data(), acc);
            }
            base = ent_apply(base, acc);
            r = hi;
        }
    }

    // ---- scan_emit: every region again, from its exact entry state --------------
    for (size_t ri = 0; ri < NR; ri++) {
        const RegionRef& rr = regions[ri];
        const Seg& sg = segs[rr.seg];
        const uint8_t* sb = data + sg.off;
        const Ent& T0 = tabs[ri][0];
        Ent e = entry[ri];
        if (T0.st & kResetState) { e.st = 0; e.d = 0; }
        if (T0.st & kResetCounts) { e.s = 0; e.k = 0; }
        uint32_t carry = (e.st >> 1) & 1, par = e.st & 1;
        uint32_t sidx = e.s, kidx = e.k;
        int32_t depth = e.d;
        if (sidx != pos.size()) flags |= 0x200;
        if (kidx != brk.size()) flags |= 0x400;
        const int nw = (rr.len + 31) / 32;
        for (int t = 0; t < nw; t++) {
            uint32_t w[8];
            for (int k = 0; k < 8; k++) {
                uint32_t v = 0;
                for (int b = 0; b < 4; b++) {
                    const int o = t * 32 + k * 4 + b;
                    if (o < rr.len) v |= (uint32_t)sb[rr.off + o] << (8 * b);
                }
                w[k] = v;
            }
            const Classes c = lines ? classify32<true>(w) : classify32<false>(w);
            const uint32_t esc = escaped32(c.bs, carry, &carry);
            const uint32_t rq = c.q & ~esc;
            const uint32_t M = prefix_xor(rq) ^ (par ? 0xFFFFFFFFu : 0u);
            par ^= __builtin_popcount(rq) & 1;
            uint32_t stm = c.st & ~M;
            const uint32_t brm = c.br & stm, opm = c.op & stm;
            const uint64_t pos0 = sg.logical + rr.off + (uint64_t)t * 32 + 1;
            while (stm) {
                const int j = __builtin_ctz(stm);
                stm &= stm - 1;
                pos.push_back((int32_t)(pos0 + j));
                pair.push_back(0);
                if ((brm >> j) & 1) {
                    const uint32_t op = (opm >> j) & 1;
                    const int32_t lvl = op ? depth : depth - 1;
                    depth += op ? 1 : -1;
                    const uint32_t cur = ((c.cur >> j) & 1) ? kCurly : 0;
                    brk.push_back({sidx | cur, ((uint32_t)lvl << 1) | op});
                }
                sidx++;
            }
        }
        // the region's end agrees with the next region's entry value
        const Ent nv = ent_apply(entry[ri], tabs[ri].data());
        if (nv.s != sidx || nv.d != depth) flags |= 0x800;
        const bool seg_last = ri + 1 == NR || regions[ri + 1].seg != rr.seg;
        if (seg_last && nv.d != 0) flags |= 2;
    }

    // ---- pairing: chunks of kChunk records, rounds of 32 --------------------------
    const uint64_t K = brk.size();
    const uint64_t nch = (K + kChunk - 1) / kChunk;
    std::vector<uint32_t> spine(nch * kChunk, 0);
    std::vector<int4> cinfo(nch);
    int32_t neg_min = 0;
    for (uint64_t ch = 0; ch < nch; ch++) {
        uint64_t base = ch * kChunk;
        int cnt = (int)std::min<uint64_t>(kChunk, K - base);
        std::vector<uint32_t> heads(kHeads, kEmpty);
        int32_t L0 = (int32_t)brk[base].y >> 1;
        int32_t d_entry = (brk[base].y & 1) ? L0 : L0 + 1;
        int32_t dmin = d_entry, last_lvl = 0;
        uint32_t last_open = 0;
        for (int r = 0; r < cnt; r += 32) {
            int m = std::min(32, cnt - r);
            struct L { uint32_t x; int32_t lvl; uint32_t op; int slot; };
            L ln[32];
            for (int l = 0; l < m; l++) {
                uint2 rec = brk[base + r + l];
                ln[l] = {rec.x, (int32_t)rec.y >> 1, rec.y & 1u, 0};
                ln[l].slot = ln[l].lvl - L0 + kChunk;
            }
            for (int l = 0; l < m; l++) {
                if (ln[l].op) continue;
                int plane = -1;
                for (int q = l - 1; q >= 0; q--) if (ln[q].lvl == ln[l].lvl) { plane = q; break; }
                uint32_t partner = kEmpty;
                if (plane >= 0) {
                    if (ln[plane].op) partner = ln[plane].x; else flags |= 2;
                } else if (ln[l].slot >= 0 && ln[l].slot < kHeads) {
                    partner = heads[ln[l].slot];
                    if (partner == kEmpty) {
                        int32_t idx = d_entry - 1 - ln[l].lvl;
                        if (idx >= 0 && idx < kChunk) spine[base + idx] = ln[l].x; else flags |= 2;
                    }
                }
                if (partner != kEmpty) {
                    if ((partner ^ ln[l].x) & kCurly) flags |= 2;
                    pair[partner & ~kCurly] = (int32_t)((ln[l].x & ~kCurly) + 1);
                }
            }
            for (int l = 0; l < m; l++) {
                bool last = true;
                for (int q = l + 1; q < m; q++) if (ln[q].lvl == ln[l].lvl) last = false;
                if (last && ln[l].slot >= 0 && ln[l].slot < kHeads)
                    heads[ln[l].slot] = ln[l].op ? ln[l].x : kEmpty;
                if (!ln[l].op) dmin = std::min(dmin, ln[l].lvl);
            }
            last_lvl = ln[m - 1].lvl;
            last_open = ln[m - 1].op;
        }
        int32_t d_exit = last_open ? last_lvl + 1 : last_lvl;
        for (int i = 0; i < kHeads; i++) {
            if (heads[i] == kEmpty) continue;
            int32_t lvl = i - kChunk + L0, idx = lvl - dmin;
            if (idx >= 0 && idx < kChunk) spine[base + (kChunk - 1 - idx)] = heads[i]; else flags |= 2;
        }
        cinfo[ch] = {d_entry, dmin, d_exit, 0};
        if (dmin < 0) neg_min = std::max(neg_min, -dmin);
    }
    for (uint64_t ch = 0; ch < nch; ch++) {
        int4 ci = cinfo[ch];
        int32_t n_uo = ci.z - ci.y, n_uc = ci.x - ci.y;
        if (n_uo < 0 || n_uc < 0 || n_uo + n_uc > kChunk) { flags |= 2; continue; }
        for (int32_t i = 0; i < n_uo; i++) {
            int32_t d = ci.y + i;
            uint32_t ox = spine[ch * kChunk + (kChunk - 1 - i)];
            int64_t c2 = -1;
            for (uint64_t q = ch + 1; q < nch; q++) if (cinfo[q].y <= d) { c2 = (int64_t)q; break; }
            if (c2 < 0) { flags |= 2; continue; }
            int32_t idx = cinfo[c2].x - 1 - d;
            if (idx < 0 || idx >= kChunk || idx >= cinfo[c2].x - cinfo[c2].y) { flags |= 2; continue; }
            uint32_t cx = spine[c2 * kChunk + idx];
            if ((ox ^ cx) & kCurly) flags |= 2;
            pair[ox & ~kCurly] = (int32_t)((cx & ~kCurly) + 1);
        }
    }
    if (neg_min > 0) flags |= 2;
    *out_S = (int64_t)pos.size();
    *out_flags = flags;
    for (size_t i = 0; i < pos.size() && i < cap; i++) { out_pos[i] = pos[i]; out_pair[i] = pair[i]; }
    return 0;
}

// Character classes of the kernels' bit-sliced classifier (classify32) against
// their byte-by-byte definition: every byte value at every one of the 32
// positions (the other bytes random), then `n_random` random 32-byte blocks.
// Returns the number of mismatching blocks.
extern "C" int cjm_classify_check(uint64_t seed, int n_random)
{
    std::mt19937_64 rng(seed);
    int bad = 0;
    auto one = [&](const uint8_t* b, bool lines) {
        uint32_t w[8];
        for (int k = 0; k < 8; k++)
            w[k] = (uint32_t)b[4 * k] | ((uint32_t)b[4 * k + 1] << 8) | ((uint32_t)b[4 * k + 2] << 16) |
                   ((uint32_t)b[4 * k + 3] << 24);
        const Classes c = lines ? classify32<true>(w) : classify32<false>(w);
        uint32_t q = 0, bs = 0, st = 0, op = 0, br = 0, cur = 0, hi = 0;
        for (int j = 0; j < 32; j++) {
            const uint8_t x = b[j];
            const uint32_t bit = 1u << j;
            if (x == '"') q |= bit;
            if (x == '\\') bs |= bit;
            if (x == '{' || x == '}' || x == '[' || x == ']' || x == ':' || x == ',' || (lines && x == '\n'))
                st |= bit;
            if (x == '{' || x == '[') op |= bit;
            if (x == '{' || x == '}' || x == '[' || x == ']') br |= bit;
            if (x == '{' || x == '}') cur |= bit;
            if (x >= 0x80) hi |= bit;
        }
        if (c.q != q || c.bs != bs || c.st != st || c.op != op || c.br != br || c.cur != cur || c.hi != hi) bad++;
    };
    uint8_t b[32];
    for (int lines = 0; lines < 2; lines++) {
        for (int j = 0; j < 32; j++)
            for (int v = 0; v < 256; v++) {
                for (int k = 0; k < 32; k++) b[k] = (uint8_t)rng();
                b[j] = (uint8_t)v;
                one(b, lines != 0);
            }
        const char alphabet[] = "\"\\{}[]:,\n \t0aZ";
        for (int i = 0; i < n_random; i++) {
            for (int k = 0; k < 32; k++)
                b[k] = (i & 1) ? (uint8_t)rng() : (uint8_t)alphabet[rng() % (sizeof(alphabet) - 1)];
            one(b, lines != 0);
        }
    }
    return bad;
}
