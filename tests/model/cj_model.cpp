// cj_model.cpp -- sequential CPU model of the parse kernels (test helper).
//
// Runs the scan kernel's algorithm tile by tile and thread by thread, with the
// same bit functions (cujson_gb300/csrc/cj_device.cuh), the same transfer
// tables and the same look-back composition, then the pairing kernels' chunk
// and spine logic with __match_any_sync emulated per 32-record round.  Tests
// compare it with the oracle to check the algorithm itself without a GPU.
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
    std::vector<Ent> incl_hist;                    // inclusive value per tile
    std::vector<std::array<Ent, 4>> agg_hist;      // aggregate table per tile
    std::vector<bool> immediate_hist;

    for (const Seg& sg : segs) {
        const uint8_t* sb = data + sg.off;
        uint64_t ntiles = (sg.len + kTileBytes - 1) / kTileBytes;
        for (uint64_t tin = 0; tin < ntiles; tin++) {
            const uint64_t tile_off = tin * kTileBytes;
            const int tile_len = (int)std::min<uint64_t>(kTileBytes, sg.len - tile_off);
            const bool seg_first = tin == 0, seg_last = tin + 1 == ntiles;
            const bool immediate = seg_first && !sg.cont;
            constexpr int W = kTileBytes / 32;    // 32-byte words per tile
            static Classes c[W];
            static uint32_t cout0[W];
            static bool all_bs[W];
            uint32_t ucarry = 0;
            for (int t = 0; t < W; t++) {
                uint32_t w[8];
                for (int k = 0; k < 8; k++) {
                    uint32_t v = 0;
                    for (int b = 0; b < 4; b++) {
                        int off = t * 32 + k * 4 + b;
                        if (off < tile_len) v |= (uint32_t)sb[tile_off + off] << (8 * b);
                    }
                    w[k] = v;
                }
                uint32_t P[8];
                bit_planes32(w, P);
                c[t] = lines ? classify_planes<true>(P) : classify_planes<false>(P);
                {
                    // UTF-8 as the kernel checks it: on the bit planes, the
                    // carry handed lane to lane and step to step, and taken
                    // afresh from the 4 bytes before each warp region
                    const int64_t o0 = (int64_t)tile_off + t * 32;
                    if ((t * 32) % kWarpBytes == 0) {
                        uint32_t pw = 0;   // previous 4 bytes of the segment (zero before its start)
                        for (int b = 0; b < 4; b++) {
                            const int64_t o = o0 - 4 + b;
                            if (o >= 0 && (uint64_t)o < sg.len) pw |= (uint32_t)sb[o] << (8 * b);
                        }
                        ucarry = utf8_carry_word(pw);
                    }
                    const bool seg_end = (uint64_t)(o0 + 32) >= sg.len;
                    const uint32_t next = utf8_carry_planes(P);
                    if (utf8_errors_planes(P, ucarry, seg_end)) flags |= 1;
                    ucarry = next;
                }
                escaped32(c[t].bs, 0, &cout0[t]);
                all_bs[t] = c[t].bs == 0xFFFFFFFFu;
            }
            // carries (tile entered without escape), parities, masks, counts
            static uint32_t M[W], own1[W], own2[W], own3[W];
            uint32_t carry = 0, par = 0;
            bool tall = true;
            uint32_t tflip = 0, tcout = 0;
            for (int t = 0; t < W; t++) {
                uint32_t dummy;
                uint32_t esc = escaped32(c[t].bs, carry, &dummy);
                uint32_t rq = c[t].q & ~esc;
                M[t] = prefix_xor(rq) ^ (par ? 0xFFFFFFFFu : 0u);
                par ^= __builtin_popcount(rq) & 1;
                if (!all_bs[t]) {
                    if (tall) {
                        int fnb = __builtin_ctz(~c[t].bs);
                        tflip = (c[t].q >> fnb) & 1;
                    }
                    tall = false;
                    carry = cout0[t];
                    tcout = cout0[t];
                }
                uint32_t br = c[t].br;
                own1[t] = __builtin_popcount(c[t].st & ~M[t]) | (__builtin_popcount(c[t].st) << 16);
                own2[t] = __builtin_popcount(br & ~M[t]) | (__builtin_popcount(br) << 16);
                own3[t] = __builtin_popcount(c[t].op & ~M[t]) | (__builtin_popcount(c[t].op) << 16);
            }
            uint32_t tqpar = par;
            int32_t C0 = 0, Ct = 0, K0 = 0, Kt = 0, O0 = 0, Ot = 0;
            for (int t = 0; t < W; t++) {
                C0 += own1[t] & 0xFFFF; Ct += own1[t] >> 16;
                K0 += own2[t] & 0xFFFF; Kt += own2[t] >> 16;
                O0 += own3[t] & 0xFFFF; Ot += own3[t] >> 16;
            }
            int32_t D0 = 2 * O0 - K0, Dt = 2 * Ot - Kt;
            std::array<Ent, 4> T;
            uint32_t Tev[4];
            for (uint32_t s = 0; s < 4; s++) {
                uint32_t escin = seg_first ? 0 : (s >> 1), instr = seg_first ? 0 : (s & 1);
                uint32_t e = instr ^ (escin & tflip);
                uint32_t oesc = tall ? escin : tcout;
                T[s].st = (oesc << 1) | (e ^ tqpar) | (seg_first ? 4u : 0u);
                T[s].s = e ? Ct - C0 : C0;
                T[s].k = e ? Kt - K0 : K0;
                T[s].d = e ? Dt - D0 : D0;
                Tev[s] = e;
            }
            size_t tile = agg_hist.size();
            Ent excl = ent_identity(0);
            if (!immediate) {
                // look back through a random number of aggregate-only tiles
                size_t back = 1 + rng() % 40;
                size_t lo = tile;
                while (lo > 0 && tile - lo < back && !immediate_hist[lo - 1]) lo--;
                // tiles [lo, tile) contribute aggregates; tile lo-1 its inclusive value
                Ent acc[4];
                tab_identity(acc);
                for (size_t u = lo; u < tile; u++) tab_compose(acc, agg_hist[u].data(), acc);
                Ent base = (lo > 0) ? incl_hist[lo - 1] : ent_identity(0);
                excl = ent_apply(base, acc);
                Ent direct = incl_hist[tile - 1];
                if (excl.st != direct.st || excl.s != direct.s || excl.k != direct.k || excl.d != direct.d)
                    flags |= 0x100;   // composition disagrees with the running value
            }
            Ent incl = ent_apply(excl, T.data());
            agg_hist.push_back(T);
            incl_hist.push_back(incl);
            immediate_hist.push_back(immediate);
            Ent entry = excl;
            if (seg_first) { entry.st = 0; entry.d = 0; }
            uint32_t e = Tev[entry.st & 3];
            if (seg_last && incl.d != 0) flags |= 2;
            // outputs
            uint32_t pre1lo = 0, pre1hi = 0, pre2lo = 0, pre2hi = 0, pre3lo = 0, pre3hi = 0;
            for (int t = 0; t < W; t++) {
                uint32_t Mf = M[t] ^ (e ? 0xFFFFFFFFu : 0u);
                uint32_t stm = c[t].st & ~Mf, brm = c[t].br & ~Mf, opm = c[t].op & ~Mf;
                uint32_t p1lo = pre1lo, p1hi = pre1hi, p2lo = pre2lo, p2hi = pre2hi;
                uint32_t p3lo = pre3lo, p3hi = pre3hi;
                uint32_t sidx = entry.s + (e ? p1hi - p1lo : p1lo);
                uint32_t kidx = entry.k + (e ? p2hi - p2lo : p2lo);
                int32_t d0 = 2 * (int32_t)p3lo - (int32_t)p2lo, dt = 2 * (int32_t)p3hi - (int32_t)p2hi;
                int32_t depth = entry.d + (e ? dt - d0 : d0);
                uint64_t pos0 = sg.logical + tile_off + t * 32 + 1;
                while (stm) {
                    int j = __builtin_ctz(stm);
                    stm &= stm - 1;
                    if (pos.size() != sidx) flags |= 0x200;
                    pos.push_back((int32_t)(pos0 + j));
                    pair.push_back(0);
                    if ((brm >> j) & 1) {
                        uint32_t op = (opm >> j) & 1;
                        int32_t lvl = op ? depth : depth - 1;
                        depth += op ? 1 : -1;
                        uint32_t cur = ((c[t].cur >> j) & 1) ? kCurly : 0;
                        if (brk.size() != kidx) flags |= 0x400;
                        brk.push_back({sidx | cur, ((uint32_t)lvl << 1) | op});
                        kidx++;
                    }
                    sidx++;
                }
                pre1lo += own1[t] & 0xFFFF; pre1hi += own1[t] >> 16;
                pre2lo += own2[t] & 0xFFFF; pre2hi += own2[t] >> 16;
                pre3lo += own3[t] & 0xFFFF; pre3hi += own3[t] >> 16;
            }
        }
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
