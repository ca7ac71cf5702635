// cj_device.cuh -- data layout shared by the parse kernels and the host
// orchestration, plus the word-level bit algorithms (host+device so the CPU
// model in cj_model.cpp can exercise exactly the code the kernels run).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define CJ_HD __host__ __device__ __forceinline__
#else
#define CJ_HD inline
#endif

namespace cj {

// ---- tiling ---------------------------------------------------------------
// A warp step is what one warp classifies at once: 32 lanes x 32 bytes, so a
// lane owns one 32-bit word of every character-class bitmap (bit j = byte j
// of its 32 bytes).  A region is what one warp scans as a unit: kRegionSteps
// consecutive steps of one segment (the last region of a segment may be
// shorter).  The scan computes one transfer table per region, composes them
// in document order, and then emits each region's outputs from its entry
// value.  The region size is chosen per run from kRegionStepsAllowed.
constexpr int kBytesPerThread = 32;
constexpr int kStepBytes = 32 * kBytesPerThread;          // 1 KiB
constexpr int kPadBytes = kStepBytes;                     // segment padding granule
constexpr int kRegionStepsAllowed[3] = {4, 8, 16};        // 4, 8 or 16 KiB regions
constexpr int kRegionStepsDefault = 16;
constexpr int kPrefixPerBlock = 256;                      // regions per block of the prefix kernels

// Pairing: one warp matches a chunk of this many bracket records.
constexpr int kChunk = 512;
constexpr int kHeads = 2 * kChunk + 1;   // level slots per chunk (levels L0-C .. L0+C)
constexpr int kTreeLevels = 6;           // min-tree levels above the chunk array

// ---- segments ---------------------------------------------------------------
// A segment is one standard document or one JSON-Lines chunk.  Segments start
// on kPadBytes boundaries of the device input and are padded to a whole number
// of warp steps; regions are counted per segment.  Escape/string state and depth start
// afresh in every segment; structural and bracket counts continue from the
// previous segment when kSegContinue is set (JSON-Lines: one merged result),
// and restart at 0 otherwise (independent documents).
constexpr uint32_t kSegContinue = 1u;

struct Segment {
    uint64_t dev_off;      // byte offset of the segment in the device input
    uint64_t len;          // bytes
    uint64_t logical_off;  // added to byte positions (reference lastChunkIndex)
    uint64_t out_base;     // output index base (independent documents)
    uint64_t brk_base;     // bracket-record base (independent documents)
    uint32_t first_region;
    uint32_t n_regions;
    uint32_t flags;
    uint32_t pad;
};

struct SegmentOut {        // written by the prefix kernel for each segment's last region
    uint32_t s_end;        // structural count at segment end (global if continuing)
    uint32_t k_end;        // bracket count at segment end
    int32_t  depth_end;    // nesting depth at segment end (0 when balanced)
    uint32_t instr_end;    // 1 if the segment ends inside a string
};

// Control block, zeroed before every run.
struct Ctrl {
    uint32_t n_work;          // regions with structurals to emit (the emit kernel's work list)
    uint32_t error_flags;     // CJ_FLAG_* bits
    uint32_t s_total;
    uint32_t k_total;
    int32_t  neg_min_level;   // max(-level) over brackets; > 0 means a close below depth 0
    int32_t  max_depth;
    uint32_t gave_up;         // the first bounded wait that expired (kGave* codes), 0 if none
    uint32_t tables_ticket;   // regions drawn by the table kernel's warps after their first
    uint32_t emit_ticket;     // work items drawn by the emit kernel's warps after their first
};

// where a bounded wait gave up (Ctrl::gave_up)
enum : uint32_t { kGaveInput = 6 };

// ---- region transfer tables ---------------------------------------------------
// Entry state of a region: bit1 = previous byte is an unescaped backslash (the
// first byte is escaped), bit0 = inside a string.  A region's table maps each
// of the 4 entry states to (exit state, structural count, bracket count, depth
// delta).  Bit 2 of `st` marks a state and depth reset (a segment's first
// region: it starts outside strings at depth 0), bit 3 a count reset (an
// independent document's first region: its counts start at 0).
struct Ent {
    uint32_t st;   // bits 0-1 exit state, bit 2 state/depth reset, bit 3 count reset
    uint32_t s;
    uint32_t k;
    int32_t  d;
};

constexpr uint32_t kResetState = 4u, kResetCounts = 8u;

CJ_HD Ent ent_identity(uint32_t state) { Ent e; e.st = state; e.s = 0; e.k = 0; e.d = 0; return e; }

// t[i] through selects, so tables stay in registers (no local-memory indexing)
CJ_HD Ent ent_select(const Ent t[4], uint32_t i) {
    Ent lo = (i & 1u) ? t[1] : t[0];
    Ent hi = (i & 1u) ? t[3] : t[2];
    return (i & 2u) ? hi : lo;
}

// value v (state, counts, absolute depth) followed by table t
CJ_HD Ent ent_apply(Ent v, const Ent t[4]) {
    const Ent x = ent_select(t, v.st & 3u);
    Ent r;
    r.st = x.st & 3u;
    r.s = (x.st & kResetCounts) ? x.s : v.s + x.s;
    r.k = (x.st & kResetCounts) ? x.k : v.k + x.k;
    r.d = (x.st & kResetState) ? x.d : v.d + x.d;
    return r;
}

// table a followed by table b
CJ_HD void tab_compose(const Ent a[4], const Ent b[4], Ent out[4]) {
    Ent tmp[4];
    for (int s = 0; s < 4; s++) {
        const Ent x = a[s];
        const Ent y = ent_select(b, x.st & 3u);
        tmp[s].st = (y.st & 3u) | ((x.st | y.st) & (kResetState | kResetCounts));
        tmp[s].s = (y.st & kResetCounts) ? y.s : x.s + y.s;
        tmp[s].k = (y.st & kResetCounts) ? y.k : x.k + y.k;
        tmp[s].d = (y.st & kResetState) ? y.d : x.d + y.d;
    }
    for (int s = 0; s < 4; s++) out[s] = tmp[s];
}

CJ_HD void tab_identity(Ent t[4]) { for (uint32_t s = 0; s < 4; s++) t[s] = ent_identity(s); }

// ---- bracket records ---------------------------------------------------------
// x = structural index | (1 << 31 if '{' / '}'), y = (level << 1) | is_open.
// level of an open = depth before it, level of a close = depth after it, so a
// matching pair shares its level.
constexpr uint32_t kCurly = 0x80000000u;
constexpr uint32_t kEmpty = 0xFFFFFFFFu;

// ---- word-level bit algorithms ----------------------------------------------

// byte selection of the 8 bytes {x, y} (x = bytes 0-3): result byte i is the
// byte numbered by nibble i of s (0-7)
CJ_HD uint32_t byte_perm(uint32_t x, uint32_t y, uint32_t s) {
#ifdef __CUDA_ARCH__
    return __byte_perm(x, y, s);
#else
    const uint64_t v = ((uint64_t)y << 32) | x;
    uint32_t r = 0;
    for (int i = 0; i < 4; i++) r |= (uint32_t)((v >> (8 * ((s >> (4 * i)) & 7u))) & 0xFFu) << (8 * i);
    return r;
#endif
}

// 4x4 byte transpose: afterwards byte i of a, b, c, d is byte 0, 1, 2, 3 of
// the old i-th word (columns of the rows a, b, c, d)
CJ_HD void transpose_bytes4(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
    const uint32_t ab_lo = byte_perm(a, b, 0x5140u), ab_hi = byte_perm(a, b, 0x7362u);   // a0 b0 a1 b1 / a2 b2 a3 b3
    const uint32_t cd_lo = byte_perm(c, d, 0x5140u), cd_hi = byte_perm(c, d, 0x7362u);
    a = byte_perm(ab_lo, cd_lo, 0x5410u);
    b = byte_perm(ab_lo, cd_lo, 0x7632u);
    c = byte_perm(ab_hi, cd_hi, 0x5410u);
    d = byte_perm(ab_hi, cd_hi, 0x7632u);
}

// exchange the bits of a at positions p + s with the bits of b at positions p,
// for every p set in m (a delta swap between two registers)
CJ_HD void swap_bits(uint32_t& a, uint32_t& b, int s, uint32_t m) {
    const uint32_t t = ((a >> s) ^ b) & m;
    b ^= t;
    a ^= t << s;
}

// Bit planes of 32 bytes held as 8 little-endian words: afterwards bit j of
// p[k] is bit k of byte j.  First a byte transpose leaves byte b of word r
// holding byte 8b + r (r = 0..7), so the bit at position 8b + k of word r is
// bit k of byte 8b + r; three delta-swap rounds then exchange the three bits
// of the word number r with the three low bits of the position (k), giving
// word k, position 8b + r.
CJ_HD void bit_planes32(const uint32_t w[8], uint32_t p[8]) {
    uint32_t v0 = w[0], v1 = w[2], v2 = w[4], v3 = w[6];   // bytes 8b + 0..3
    uint32_t v4 = w[1], v5 = w[3], v6 = w[5], v7 = w[7];   // bytes 8b + 4..7
    transpose_bytes4(v0, v1, v2, v3);
    transpose_bytes4(v4, v5, v6, v7);
    swap_bits(v0, v1, 1, 0x55555555u); swap_bits(v2, v3, 1, 0x55555555u);
    swap_bits(v4, v5, 1, 0x55555555u); swap_bits(v6, v7, 1, 0x55555555u);
    swap_bits(v0, v2, 2, 0x33333333u); swap_bits(v1, v3, 2, 0x33333333u);
    swap_bits(v4, v6, 2, 0x33333333u); swap_bits(v5, v7, 2, 0x33333333u);
    swap_bits(v0, v4, 4, 0x0F0F0F0Fu); swap_bits(v1, v5, 4, 0x0F0F0F0Fu);
    swap_bits(v2, v6, 4, 0x0F0F0F0Fu); swap_bits(v3, v7, 4, 0x0F0F0F0Fu);
    p[0] = v0; p[1] = v1; p[2] = v2; p[3] = v3; p[4] = v4; p[5] = v5; p[6] = v6; p[7] = v7;
}

struct Classes {
    uint32_t q, bs, st, op, br, cur, hi;
};

// Character classes of 32 bytes held as 8 little-endian words; bit j of each
// mask is byte j: quote, backslash, structural ({ } [ ] : , and '\n' in
// JSON-Lines mode), open ({ [), bracket (any of { } [ ]), curly ({ }) and
// `hi` (bytes >= 0x80, the non-ASCII test).
//
// Bit-sliced: the bytes are turned into 8 bit planes (bit_planes32) and each
// class is a boolean function of the planes, 32 bytes per logic operation.
//   " 0x22 = 0010 0010      \ 0x5C = 0101 1100
//   , 0x2C = 0010 1100      : 0x3A = 0011 1010      \n 0x0A = 0000 1010
//   [ 0x5B = 0101 1011      ] 0x5D = 0101 1101      { 0x7B, } 0x7D (bit 5 set)
// The four brackets are exactly 01x11yz1 with y != z (open: y = 0, z = 1), the
// comma and the colon exactly 001a1bc0 with b != a and c == a.
template <bool LINES>
CJ_HD Classes classify_planes(const uint32_t P[8]) {
    const uint32_t n7 = ~P[7];
    Classes c;
    c.br = n7 & P[6] & P[4] & P[3] & P[0] & (P[1] ^ P[2]);
    c.op = c.br & P[1];
    c.cur = c.br & P[5];
    const uint32_t u = n7 & ~P[6] & P[5];                                        // 0x20 .. 0x3F
    c.q = u & P[1] & ~(P[4] | P[3] | P[2] | P[0]);
    c.bs = n7 & P[6] & ~P[5] & P[4] & P[3] & P[2] & ~(P[1] | P[0]);
    const uint32_t cc = u & P[3] & ~P[0] & (P[4] ^ P[2]) & ~(P[4] ^ P[1]);     // , :
    c.st = c.br | cc;
    if (LINES) c.st |= n7 & P[3] & P[1] & ~(P[6] | P[5] | P[4] | P[2] | P[0]);   // '\n'
    c.hi = P[7];
    return c;
}

template <bool LINES>
CJ_HD Classes classify32(const uint32_t w[8]) {
    uint32_t P[8];
    bit_planes32(w, P);
    return classify_planes<LINES>(P);
}

// carry out of a 32-byte word entered without escape: whether its trailing
// backslash run has odd length (not meaningful for an all-backslash word)
CJ_HD uint32_t escape_cout(uint32_t bs) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__clz(~bs) & 1u;
#else
    return (uint32_t)(bs == 0xFFFFFFFFu ? 0 : __builtin_clz(~bs)) & 1u;
#endif
}

// Escaped-character mask of one 32-byte word.  `carry` = 1 when byte 0 is
// escaped by an odd backslash run ending in the previous word.  Within a run of
// backslashes that starts fresh at position s, the bytes s+1, s+3, ... are
// escaped (each backslash at s, s+2, ... escapes its successor).  Runs starting
// at odd positions are found with one addition: adding their start bit clears
// the run and sets the bit after it, and the XOR with the run marks its span.
// *cout receives the carry for the next word.
CJ_HD uint32_t escaped32(uint32_t bs, uint32_t carry, uint32_t* cout) {
    const uint32_t ODD = 0xAAAAAAAAu;
    uint32_t b = bs & ~carry;              // an escaped first byte starts no run
    uint32_t starts = b & ~(b << 1);
    uint32_t os = starts & ODD;
    uint64_t t = (uint64_t)b + os;
    uint32_t tl = (uint32_t)t;
    *cout = (uint32_t)(t >> 32);
    uint32_t odd_span = (tl ^ b) ^ os;     // s+1 .. s+L of odd-start runs
    uint32_t span = b << 1;                // s+1 .. s+L of every run
    return (span & (ODD ^ odd_span)) | carry;
}

// ---- UTF-8 on bit planes ------------------------------------------------------
// RFC 3629 validity of one lane's 32 bytes from their bit planes (bit j of
// P[k] = bit k of byte j; bytes past the end of the segment are zero).  Leads
// 110xxxxx, 1110xxxx and 11110xxx expect continuation bytes (10xxxxxx) at
// their next 1, 2 or 3 positions; the expected positions must be exactly the
// continuation bytes.  11111xxx, C0 and C1 (overlong 2-byte forms) and F5-F7
// (beyond U+10FFFF) are rejected, and the byte after E0 / ED / F0 / F4 must be
// >= A0 / <= 9F / >= 90 / <= 8F (overlong 3- and 4-byte forms, surrogates,
// beyond U+10FFFF).  `cin` is the carry word of the 32 bytes before (the
// previous lane's utf8_carry_planes).  A sequence still open at the
// end of the lane is the next lane's to check unless the segment ends there
// (`seg_end`).  Returns nonzero on an error.
//
// Carry word: bit 0 lead needing >= 1 byte at position 31, bits 1-2 leads
// needing >= 2 at 30-31, bits 3-5 leads needing 3 at 29-31, bits 6-9 an E0,
// ED, F0 or F4 at position 31.
CJ_HD uint32_t utf8_carry_out(uint32_t L1, uint32_t L2, uint32_t L3, uint32_t e0, uint32_t ed,
                              uint32_t f0, uint32_t f4) {
    return (L1 >> 31) | ((L2 >> 30) << 1) | ((L3 >> 29) << 3) | ((e0 >> 31) << 6) | ((ed >> 31) << 7) |
           ((f0 >> 31) << 8) | ((f4 >> 31) << 9);
}

// leads and special bytes of one lane's 32 bytes, from its bit planes
struct Utf8Lane {
    uint32_t cont, L1, L2, L3, bad, c0c1, f5f7, e0, ed, f0, f4;
};

CJ_HD Utf8Lane utf8_lane(const uint32_t P[8]) {
    Utf8Lane u;
    const uint32_t t76 = P[7] & P[6];
    u.cont = P[7] & ~P[6];
    const uint32_t l2 = t76 & ~P[5];
    const uint32_t t765 = t76 & P[5];
    const uint32_t l3 = t765 & ~P[4];
    const uint32_t t7654 = t765 & P[4];
    u.L3 = t7654 & ~P[3];                                             // 11110xxx
    u.bad = t7654 & P[3];                                             // F8..FF
    u.L2 = l3 | u.L3;
    u.L1 = l2 | u.L2;
    const uint32_t lo3 = P[2] | P[1] | P[0];
    u.c0c1 = l2 & ~(P[4] | P[3] | P[2] | P[1]);                      // C0, C1
    u.f5f7 = u.L3 & P[2] & (P[1] | P[0]);                             // F5, F6, F7
    u.e0 = l3 & ~(P[3] | lo3);                                        // E0
    u.ed = l3 & P[3] & P[2] & ~P[1] & P[0];                           // ED
    u.f0 = u.L3 & ~lo3;                                               // F0
    u.f4 = u.L3 & P[2] & ~(P[1] | P[0]);                              // F4
    return u;
}

// the carry word this lane hands to the next (it depends on its bytes only)
CJ_HD uint32_t utf8_carry_planes(const uint32_t P[8]) {
    const Utf8Lane u = utf8_lane(P);
    return utf8_carry_out(u.L1, u.L2, u.L3, u.e0, u.ed, u.f0, u.f4);
}

CJ_HD uint32_t utf8_errors_planes(const uint32_t P[8], uint32_t cin, bool seg_end) {
    const Utf8Lane u = utf8_lane(P);
    const uint32_t E = (u.L1 << 1) | (u.L2 << 2) | (u.L3 << 3) | (cin & 1u) | ((cin >> 1) & 3u) |
                       ((cin >> 3) & 7u);
    const uint32_t b54 = P[5] | P[4];
    uint32_t err = (E ^ u.cont) | u.bad | u.c0c1 | u.f5f7;
    err |= ((u.e0 << 1) | ((cin >> 6) & 1u)) & ~P[5];                // E0 then < A0
    err |= ((u.ed << 1) | ((cin >> 7) & 1u)) & P[5];                 // ED then >= A0
    err |= ((u.f0 << 1) | ((cin >> 8) & 1u)) & ~b54;                 // F0 then < 90
    err |= ((u.f4 << 1) | ((cin >> 9) & 1u)) & b54;                  // F4 then >= 90
    if (seg_end) err |= (u.L1 >> 31) | (u.L2 >> 30) | (u.L3 >> 29);
    return err;
}

// carry word of the 4 bytes of `w` as the last bytes before a lane (byte 3 at
// position 31); the same bits utf8_errors_planes hands on
CJ_HD uint32_t utf8_carry_word(uint32_t w) {
    uint32_t L1 = 0, L2 = 0, L3 = 0, e0 = 0, ed = 0, f0 = 0, f4 = 0;
    for (int k = 1; k < 4; k++) {
        const uint32_t b = (w >> (8 * k)) & 0xFFu;
        const uint32_t bit = 1u << (28 + k);                            // positions 29, 30, 31
        const bool is2 = (b & 0xE0u) == 0xC0u, is3 = (b & 0xF0u) == 0xE0u, is4 = (b & 0xF8u) == 0xF0u;
        if (is2 || is3 || is4) L1 |= bit;
        if (is3 || is4) L2 |= bit;
        if (is4) L3 |= bit;
        if (b == 0xE0u) e0 |= bit;
        if (b == 0xEDu) ed |= bit;
        if (b == 0xF0u) f0 |= bit;
        if (b == 0xF4u) f4 |= bit;
    }
    return utf8_carry_out(L1, L2, L3, e0, ed, f0, f4);
}

// inclusive prefix XOR over the bits of x
CJ_HD uint32_t prefix_xor(uint32_t x) {
    x ^= x << 1;
    x ^= x << 2;
    x ^= x << 4;
    x ^= x << 8;
    x ^= x << 16;
    return x;
}

}  // namespace cj
