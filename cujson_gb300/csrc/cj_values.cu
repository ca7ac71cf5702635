// cj_values.cu -- value decoding over a parsed result: the scalar between
// every two structurals decoded -- strings unescaped to UTF-8, numbers to
// int64 or double, true / false / null.  The reference stops at the index:
// its iterator hands out the raw bytes of a value (getValue,
// cujson/query/query_iterator.cpp:512); this is the "value decoding" step that
// would follow it.
//
// Slots: slot 0 is the text before the first structural, slot i (1 <= i <= S)
// the text after structural i up to the next one (or the end of the input).
// Each slot's text, less JSON whitespace at both ends, is one of: nothing,
// a string, a number, a literal -- anything else is marked invalid.
//
//   decode_slots   one thread per slot; a string without escapes copied four
//                  bytes a store; a slot longer than kShortBytes, or a string
//                  that holds an escape, goes to a list instead, so that one
//                  long or escaped string does not hold up a warp of short
//                  plain ones;
//   decode_deferred, decode_swept: below.
//
// A string's decoded bytes are written at its own content offset in the
// output buffer (decoding never lengthens a string), so no prefix sum is
// needed; its decoded length goes to len[].  Numbers: an integer without a
// fraction or exponent that fits int64 is exact; otherwise the correctly
// rounded double, by Clinger's fast path (exact powers of ten, at most 2^53
// and 10^22) or the Eisel-Lemire algorithm (a 128-bit product with a
// truncated power of five, D. Lemire 2021); inputs of more than 19
// significant digits are tried at both neighbours of their truncation.  The
// rare inputs that neither decides (a product too close to a halfway point,
// subnormal results) join the second kernel's list and are converted exactly
// there: the decimal-shift method (the "simple decimal conversion" of
// Go's strconv and of Nigel Tao's Wuffs) -- the digits held as a big decimal,
// shifted by powers of two into [1/2, 1), then 53 bits more, then rounded half
// to even; 800 digits are held, more only set a sticky flag, and the
// exact halfway points of doubles need at most 767.
//
//   decode_deferred  a warp per listed slot: the long list (slots longer than
//                    kShortBytes) a warp each in turn, then the short list
//                    (escaped strings, numbers for the exact conversion) from
//                    a ticket; whitespace trimmed and strings decoded by the
//                    whole warp, numbers by one lane with a digit buffer per
//                    warp in shared memory;
//   decode_swept     only when the short list overflowed: the deferred
//                    numbers it did not hold, found by a pass over the types;
//   count_types      the totals per type.
#include <cuda_runtime.h>

#include <algorithm>

#include "cj_device.cuh"
#include "cj_kernels.h"

namespace cj {

namespace {

constexpr uint32_t kShortBytes = 256;     // longer slots go to the second kernel
constexpr uint32_t FULL_MASK = 0xFFFFFFFFu;
constexpr int kValThreads = 256;

__device__ __forceinline__ bool is_ws(uint8_t c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

// the byte at logical offset x: segments are searched once per slot and then
// followed forward
struct Reader {
    const ValueParams* P;
    uint32_t seg;
    uint64_t lo, hi;          // logical range of the current segment
    const uint8_t* base;      // its first byte on the device
    __device__ void seek(uint64_t x) {
        uint32_t a = 0, b = P->n_segs;
        while (b - a > 1) {
            const uint32_t m = (a + b) >> 1;
            if (__ldg(&P->segs[m].logical_off) <= x) a = m;
            else b = m;
        }
        set(a);
    }
    __device__ void set(uint32_t s) {
        seg = s;
        lo = __ldg(&P->segs[s].logical_off);
        hi = lo + __ldg(&P->segs[s].len);
        base = P->in + __ldg(&P->segs[s].dev_off);
    }
    __device__ uint8_t at(uint64_t x) {
        if (x < lo) seek(x);                                   // back into an earlier segment
        while (x >= hi && seg + 1 < P->n_segs) set(seg + 1);
        return x < hi ? __ldg(base + (x - lo)) : (uint8_t)' ';
    }
};

__device__ __forceinline__ int hexval(uint8_t c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'f') return c - 'a' + 10;
    if (c >= 'A' && c <= 'F') return c - 'A' + 10;
    return -1;
}

// the string whose quotes are at logical offsets a and b (b > a): its
// decoded bytes from out[a + 1] on; returns the decoded length, or -1 when
// the content is not a valid JSON string
__device__ int64_t decode_string(Reader& rd, uint64_t a, uint64_t b, uint8_t* out)
{
    uint64_t o = a + 1;
    for (uint64_t x = a + 1; x < b;) {
        const uint8_t c = rd.at(x);
        if (c < 0x20u) return -1;                         // control characters must be escaped
        if (c == '"') return -1;                          // an inner quote ends the string early
        if (c != '\\') { out[o++] = c; x++; continue; }
        if (x + 1 >= b) return -1;
        const uint8_t e = rd.at(x + 1);
        uint8_t r;
        switch (e) {
            case '"': r = '"'; break;
            case '\\': r = '\\'; break;
            case '/': r = '/'; break;
            case 'b': r = '\b'; break;
            case 'f': r = '\f'; break;
            case 'n': r = '\n'; break;
            case 'r': r = '\r'; break;
            case 't': r = '\t'; break;
            case 'u': {
                if (x + 6 > b) return -1;
                uint32_t cp = 0;
                for (int k = 0; k < 4; k++) {
                    const int h = hexval(rd.at(x + 2 + k));
                    if (h < 0) return -1;
                    cp = (cp << 4) | (uint32_t)h;
                }
                x += 6;
                if (cp >= 0xD800u && cp <= 0xDBFFu) {
                    // a high surrogate must be followed by an escaped low one
                    if (x + 6 > b || rd.at(x) != '\\' || rd.at(x + 1) != 'u') return -1;
                    uint32_t lo = 0;
                    for (int k = 0; k < 4; k++) {
                        const int h = hexval(rd.at(x + 2 + k));
                        if (h < 0) return -1;
                        lo = (lo << 4) | (uint32_t)h;
                    }
                    if (lo < 0xDC00u || lo > 0xDFFFu) return -1;
                    x += 6;
                    cp = 0x10000u + ((cp - 0xD800u) << 10) + (lo - 0xDC00u);
                } else if (cp >= 0xDC00u && cp <= 0xDFFFu) {
                    return -1;                            // a lone low surrogate
                }
                if (cp < 0x80u) {
                    out[o++] = (uint8_t)cp;
                } else if (cp < 0x800u) {
                    out[o++] = (uint8_t)(0xC0u | (cp >> 6));
                    out[o++] = (uint8_t)(0x80u | (cp & 0x3Fu));
                } else if (cp < 0x10000u) {
                    out[o++] = (uint8_t)(0xE0u | (cp >> 12));
                    out[o++] = (uint8_t)(0x80u | ((cp >> 6) & 0x3Fu));
                    out[o++] = (uint8_t)(0x80u | (cp & 0x3Fu));
                } else {
                    out[o++] = (uint8_t)(0xF0u | (cp >> 18));
                    out[o++] = (uint8_t)(0x80u | ((cp >> 12) & 0x3Fu));
                    out[o++] = (uint8_t)(0x80u | ((cp >> 6) & 0x3Fu));
                    out[o++] = (uint8_t)(0x80u | (cp & 0x3Fu));
                }
                continue;
            }
            default: return -1;
        }
        out[o++] = r;
        x += 2;
    }
    return (int64_t)(o - (a + 1));
}

// the 4 bytes at p, whatever its alignment (two aligned loads; the input
// buffer has slack after every segment)
__device__ __forceinline__ uint32_t load4(const uint8_t* p)
{
    const uintptr_t u = reinterpret_cast<uintptr_t>(p);
    const uint32_t* q = reinterpret_cast<const uint32_t*>(u & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(u & 3u) * 8u;
    const uint32_t lo = __ldg(q);
    return sh ? __funnelshift_r(lo, __ldg(q + 1), sh) : lo;
}

// a string without escapes, quotes or control bytes (most strings), copied
// to out at its own offsets, four bytes a store in the middle: content
// [s0, e), all in the reader's current segment (the closing quote's).
// Returns its length, or -1 when it holds a byte that needs decode_string.
__device__ int64_t copy_plain(Reader& rd, uint64_t s0, uint64_t e, uint8_t* out)
{
    const uint8_t* src = rd.base + (s0 - rd.lo);                // logical offset x at src + (x - s0)
    uint64_t x = s0;
    for (; x < e && (x & 3u); x++) {
        const uint8_t c = __ldg(src + (x - s0));
        if (c == '\\' || c == '"' || c < 0x20u) return -1;
        out[x] = c;
    }
    for (; x + 4 <= e; x += 4) {
        const uint32_t v = load4(src + (x - s0));
        if (__vcmpeq4(v, 0x5C5C5C5Cu) | __vcmpeq4(v, 0x22222222u) | __vcmpltu4(v, 0x20202020u)) return -1;
        *reinterpret_cast<uint32_t*>(out + x) = v;
    }
    for (; x < e; x++) {
        const uint8_t c = __ldg(src + (x - s0));
        if (c == '\\' || c == '"' || c < 0x20u) return -1;
        out[x] = c;
    }
    return (int64_t)(e - s0);
}

// ---- long strings: a warp per string ------------------------------------------------
//
// The string's content is taken 512 bytes a step, 16 bytes a lane, staged in
// shared memory with 8 bytes before and 12 after.  Whether a byte is escaped
// (its predecessor a backslash that is not itself escaped) is a two-state
// recurrence: each lane's 16 bytes map the state at their start to the state
// at their end, and a warp scan of those maps gives every lane its starting
// state.  A lane then classifies its bytes within a window of 8 bytes before
// and 12 after its own (an escape reaches 11 bytes ahead, the low half of a
// surrogate pair looks 6 back), counts what each emits, and writes at its
// offset from a warp prefix sum.

constexpr int kLaneBytes = 16;
constexpr int kWinBefore = 8, kWinAfter = 12;
constexpr int kWarpStep = 32 * kLaneBytes;
constexpr int kWin = kWinBefore + kLaneBytes + kWinAfter;
constexpr int kStage = kWinBefore + kWarpStep + kWinAfter;

__device__ __forceinline__ int hex4(const uint8_t* p)
{
    const int x = hexval(p[0]), y = hexval(p[1]), z = hexval(p[2]), w = hexval(p[3]);
    return (x | y | z | w) < 0 ? -1 : (x << 12) | (y << 8) | (z << 4) | w;
}

__device__ __forceinline__ int utf8_put(uint32_t cp, uint8_t* o)
{
    const int n = cp < 0x80u ? 1 : cp < 0x800u ? 2 : cp < 0x10000u ? 3 : 4;
    if (o) {
        if (n == 1) {
            o[0] = (uint8_t)cp;
        } else {
            o[0] = (uint8_t)((0xFF00u >> n) | (cp >> (6 * (n - 1))));     // 110x, 1110, 11110 leads
            for (int k = 1; k < n; k++) o[k] = (uint8_t)(0x80u | ((cp >> (6 * (n - 1 - k))) & 0x3Fu));
        }
    }
    return n;
}

// what window byte j (kWinBefore <= j < kWinBefore + kLaneBytes, at content
// offset q < len) emits: its byte count (written to o when o is set), or -1
// when the string is invalid there.  st: bit k set when window byte k is a
// backslash that starts an escape.
__device__ int emit_byte(const uint8_t* w, uint64_t st, int j, uint64_t q, uint64_t len, uint8_t* o)
{
    const uint8_t c = w[j];
    if ((st >> j) & 1) {
        if (q + 1 >= len) return -1;                 // the backslash would escape the closing quote
        uint8_t r;
        switch (w[j + 1]) {
            case '"': r = '"'; break;
            case '\\': r = '\\'; break;
            case '/': r = '/'; break;
            case 'b': r = '\b'; break;
            case 'f': r = '\f'; break;
            case 'n': r = '\n'; break;
            case 'r': r = '\r'; break;
            case 't': r = '\t'; break;
            case 'u': {
                if (q + 5 >= len) return -1;
                const int cu = hex4(w + j + 2);
                if (cu < 0) return -1;
                if (cu >= 0xD800 && cu <= 0xDBFF) {
                    if (q + 11 >= len || w[j + 6] != '\\' || w[j + 7] != 'u') return -1;
                    const int lo = hex4(w + j + 8);
                    if (lo < 0xDC00 || lo > 0xDFFF) return -1;
                    return utf8_put(0x10000u + ((uint32_t)(cu - 0xD800) << 10) + (uint32_t)(lo - 0xDC00), o);
                }
                if (cu >= 0xDC00 && cu <= 0xDFFF) {
                    // only as the second half of a pair, which the first half emitted
                    const int hi = hex4(w + j - 4);
                    return (((st >> (j - 6)) & 1) && w[j - 5] == 'u' && hi >= 0xD800 && hi <= 0xDBFF) ? 0 : -1;
                }
                return utf8_put((uint32_t)cu, o);
            }
            default: return -1;
        }
        if (o) o[0] = r;
        return 1;
    }
    if ((st >> (j - 1)) & 1) return 0;                          // the escaped character
    for (int t = 2; t <= 5; t++)                                // a hex digit of an escaped u
        if (((st >> (j - t)) & 1) && w[j - t + 1] == 'u') return 0;
    if (c < 0x20u || c == '"') return -1;
    if (o) o[0] = c;
    return 1;
}

// the four-bit mask of the bytes of w equal to the byte of c4 (repeated), and
// of those below it: bit i for byte i
__device__ __forceinline__ uint32_t nib_eq(uint32_t w, uint32_t c4)
{
    return ((__vcmpeq4(w, c4) & 0x80808080u) * 0x00204081u) >> 28;
}
__device__ __forceinline__ uint32_t nib_lt(uint32_t w, uint32_t c4)
{
    return ((__vcmpltu4(w, c4) & 0x80808080u) * 0x00204081u) >> 28;
}

// escape starts (backslashes that are not themselves escaped) of the bytes
// whose backslashes are `bs` (bit i = byte i), byte 0 escaped when e0: each
// run of backslashes starts an escape at every other byte from its first --
// from its second when the run starts at an escaped byte 0.  The runs that
// start at odd bits are found by the carry of one addition per run.
__device__ __forceinline__ uint64_t escape_starts(uint64_t bs, uint32_t e0)
{
    constexpr uint64_t kEven = 0x5555555555555555ull;
    const uint64_t starts = bs & ~(bs << 1);
    const uint64_t os = (starts & ~kEven) | (e0 ? (bs & 1ull) : 0ull);     // runs whose first escape is at an odd bit
    const uint64_t odd_runs = ((bs + os) ^ bs) & bs;
    return ((bs & ~odd_runs) & kEven) | (odd_runs & ~kEven);
}

__device__ __forceinline__ uint8_t unescape(uint8_t c)
{
    return c == 'b' ? '\b' : c == 'f' ? '\f' : c == 'n' ? '\n' : c == 'r' ? '\r' : c == 't' ? '\t' : c;
}

// a warp decodes the content src[0, len) of one string into out, staging its
// input through `stage` (kStage bytes) and its output through `ostage`
// (kWarpStep + 8 bytes) of shared memory, this warp's; every lane returns the
// decoded length, or -1 when it is not a valid JSON string.  A lane whose
// window holds no escaped u takes its bytes by masks: an escape start emits
// its unescaped character, the escaped character nothing, any other byte
// itself; a lane with an escaped u goes byte by byte.
__device__ int64_t decode_string_warp(const uint8_t* __restrict__ src, uint64_t len, uint8_t* __restrict__ out,
                                      uint8_t* stage, uint8_t* ostage)
{
    const int lane = (int)(threadIdx.x & 31);
    const uint8_t* w = stage + kLaneBytes * lane;               // this lane's window
    const uint32_t* ww = reinterpret_cast<const uint32_t*>(w);
    uint32_t carry = 0;           // escaped-state at the step's first byte
    uint32_t prev8 = 0;           // that state 8 bytes before lane 0's first byte
    uint64_t done = 0;            // bytes written
    // the staged bytes of a step, loaded one step ahead
    constexpr int kPer = (kStage + 31) / 32;
    uint32_t nx[kPer];
    auto load_step = [&](uint64_t c) {
#pragma unroll
        for (int r = 0; r < kPer; r++) {
            const int64_t q = (int64_t)c - kWinBefore + lane + 32 * r;
            nx[r] = (q >= 0 && (uint64_t)q < len && lane + 32 * r < kStage) ? __ldg(src + q) : 0u;
        }
    };
    load_step(0);
    for (uint64_t c0 = 0; c0 < len; c0 += kWarpStep) {
        __syncwarp();
#pragma unroll
        for (int r = 0; r < kPer; r++)
            if (lane + 32 * r < kStage) stage[lane + 32 * r] = (uint8_t)nx[r];
        __syncwarp();
        if (c0 + kWarpStep < len) load_step(c0 + kWarpStep);
        // masks of the window's 36 bytes: backslashes, u, quotes, control bytes
        uint64_t B = 0, U = 0, Q = 0, C = 0;
#pragma unroll
        for (int k = 0; k < kWin / 4; k++) {
            const uint32_t x = ww[k];
            B |= (uint64_t)nib_eq(x, 0x5C5C5C5Cu) << (4 * k);
            U |= (uint64_t)nib_eq(x, 0x75757575u) << (4 * k);
            Q |= (uint64_t)nib_eq(x, 0x22222222u) << (4 * k);
            C |= (uint64_t)nib_lt(x, 0x20202020u) << (4 * k);
        }
        // this lane's state map over its own 16 bytes, then the warp's scan of maps
        const uint64_t bown = (B >> kWinBefore) & 0xFFFFull;
        const uint64_t st0 = escape_starts(bown, 0), st1 = escape_starts(bown, 1);
        uint32_t m = (uint32_t)((st0 >> 15) & 1u) | (uint32_t)(((st1 >> 15) & 1u) << 1);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t up = __shfl_up_sync(~0u, m, d);
            if (lane >= d) m = ((m >> (up & 1u)) & 1u) | (((m >> ((up >> 1) & 1u)) & 1u) << 1);
        }
        const uint32_t excl = __shfl_up_sync(~0u, m, 1);
        const uint32_t cin = lane ? (excl >> carry) & 1u : carry;
        carry = (__shfl_sync(~0u, m, 31) >> carry) & 1u;
        // the state 8 bytes in, handed to the next lane as its window's start
        const uint32_t e8 = (uint32_t)(((cin ? st1 : st0) >> 7) & 1u);
        uint32_t start = __shfl_up_sync(~0u, e8, 1);
        if (lane == 0) start = prev8;
        prev8 = __shfl_sync(~0u, e8, 31);
        const uint64_t st = escape_starts(B & ((1ull << kWin) - 1), start);
        const uint64_t esc = (st << 1) | start;                 // escaped bytes
        // count and check this lane's bytes
        const uint64_t q0 = c0 + (uint64_t)kLaneBytes * lane;
        const int own = q0 >= len ? 0 : len - q0 < (uint64_t)kLaneBytes ? (int)(len - q0) : kLaneBytes;
        const uint64_t ownm = (((1ull << own) - 1) << kWinBefore);
        const bool slow = (U & esc & (0x1FFFFFull << 4)) != 0;  // an escaped u whose escape reaches this lane
        int n = 0;
        bool bad = false;
        if (slow) {
            for (int j = 0; j < own; j++) {
                const int k = emit_byte(w, st, kWinBefore + j, q0 + j, len, nullptr);
                bad |= k < 0;
                n += k;
            }
        } else {
            n = __popcll(ownm & ~esc);
            bad = (ownm & ~esc & ~st & (Q | C)) != 0;            // a bare quote or control byte
            // escapes: of what follows each start, a backslash or quote is
            // always valid; the rest are checked one by one
            const uint64_t est = st & ownm;
            if (est >> (kWinBefore + own - 1) & 1ull && q0 + own == len) bad = true;   // the last byte
            for (uint64_t r = (est << 1) & ~(B | Q); r; r &= r - 1) {
                const uint8_t c = w[__ffsll((long long)r) - 1];
                bad |= !(c == '/' || c == 'b' || c == 'f' || c == 'n' || c == 'r' || c == 't');
            }
        }
        if (__any_sync(~0u, bad)) return -1;
        int pre = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int up = __shfl_up_sync(~0u, pre, d);
            if (lane >= d) pre += up;
        }
        uint8_t* o = ostage + (pre - n);
        if (slow) {
            for (int j = 0; j < own; j++) o += emit_byte(w, st, kWinBefore + j, q0 + j, len, o);
        } else {
            for (uint64_t r = ownm & ~esc; r; r &= r - 1) {
                const int j = __ffsll((long long)r) - 1;
                *o++ = (st >> j) & 1ull ? unescape(w[j + 1]) : w[j];
            }
        }
        __syncwarp();
        const int total = __shfl_sync(~0u, pre, 31);
        for (int k = lane; k < total; k += 32) out[done + k] = ostage[k];
        done += (uint64_t)total;
    }
    return (int64_t)done;
}

// ---- numbers -------------------------------------------------------------------

constexpr int kQMin = -342, kQMax = 308;
constexpr uint64_t kInfBits = 0x7FF0000000000000ull;

// Eisel-Lemire: the correctly rounded double of w * 10^q (w != 0, at most 19
// digits), as bits, or -1 when the 128-bit product cannot decide it
__device__ int64_t eisel_lemire(uint64_t w, int32_t q, const uint64_t* __restrict__ pow5)
{
    if (q < kQMin) return 0;                                   // rounds to +0
    if (q > kQMax) return (int64_t)kInfBits;
    const int lz = __clzll((long long)w);
    w <<= lz;
    const int idx = 2 * (q - kQMin);
    uint64_t hi = __umul64hi(w, __ldg(pow5 + idx)), lo = w * __ldg(pow5 + idx);
    if ((hi & 0x1FFull) == 0x1FFull) {
        // the truncated table entry may matter: add the next 64 bits
        const uint64_t hi2 = __umul64hi(w, __ldg(pow5 + idx + 1));
        lo += hi2;
        if (hi2 > lo) hi++;
    }
    if (lo == ~0ull && (q < -27 || q > 55)) return -1;
    const int upperbit = (int)(hi >> 63);
    uint64_t m = hi >> (upperbit + 9);
    int32_t p2 = (int32_t)((((152170 + 65536) * q) >> 16) + 63) + upperbit - lz + 1023;
    if (p2 <= 0) return -1;                                    // subnormal or zero: not decided here
    // exactly halfway between two doubles (only possible for small |q|):
    // round to even
    if (lo <= 1 && q >= -4 && q <= 23 && (m & 3u) == 1u && (m << (upperbit + 9)) == hi) m &= ~1ull;
    m += m & 1u;
    m >>= 1;
    if (m >= (2ull << 52)) {
        m = 1ull << 52;
        p2++;
    }
    m &= ~(1ull << 52);
    if (p2 >= 0x7FF) return (int64_t)kInfBits;
    return (int64_t)(((uint64_t)p2 << 52) | m);
}

__device__ const double kExact10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                        1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// a number token [a, b): type and value bits
__device__ uint8_t decode_number(Reader& rd, uint64_t a, uint64_t b, const uint64_t* pow5, uint64_t& bits)
{
    uint64_t x = a;
    bool neg = false;
    if (rd.at(x) == '-') { neg = true; x++; }
    if (x >= b) return kValInvalid;
    uint64_t w = 0;
    int digits = 0;               // significant digits kept in w (at most 19)
    int32_t drop = 0;             // integer-part digits beyond the 19 kept
    bool truncated = false;       // a nonzero digit was dropped
    bool nonzero = false;
    const uint64_t int_start = x;
    uint8_t c = rd.at(x);
    if (c == '0') {
        x++;
    } else if (c >= '1' && c <= '9') {
        while (x < b && (c = rd.at(x)) >= '0' && c <= '9') {
            if (digits < 19) { w = w * 10 + (c - '0'); digits++; nonzero = true; }
            else { drop++; if (c != '0') truncated = true; }
            x++;
        }
    } else {
        return kValInvalid;
    }
    const uint64_t int_digits = x - int_start;
    bool frac = false, expo = false;
    int32_t frac_kept = 0;
    if (x < b && rd.at(x) == '.') {
        frac = true;
        x++;
        const uint64_t f0 = x;
        while (x < b && (c = rd.at(x)) >= '0' && c <= '9') {
            if (!nonzero && c == '0') {
                frac_kept++;      // leading zeros of a value below 1: not significant
            } else if (digits < 19) {
                w = w * 10 + (c - '0');
                digits++;
                frac_kept++;
                nonzero = true;
            } else if (c != '0') {
                truncated = true;
            }
            x++;
        }
        if (x == f0) return kValInvalid;
    }
    int64_t e10 = 0;
    if (x < b && ((c = rd.at(x)) == 'e' || c == 'E')) {
        expo = true;
        x++;
        bool eneg = false;
        if (x < b && ((c = rd.at(x)) == '+' || c == '-')) { eneg = c == '-'; x++; }
        const uint64_t e0 = x;
        while (x < b && (c = rd.at(x)) >= '0' && c <= '9') {
            if (e10 < 100000) e10 = e10 * 10 + (c - '0');
            x++;
        }
        if (x == e0) return kValInvalid;
        if (eneg) e10 = -e10;
    }
    if (x != b) return kValInvalid;
    if (!frac && !expo) {
        // an integer: exact in int64 when it fits
        if (int_digits <= 19 && drop == 0) {
            if (!neg && w <= 0x7FFFFFFFFFFFFFFFull) { bits = w; return kValInt; }
            if (neg && w <= 0x8000000000000000ull) { bits = (uint64_t)(-(int64_t)(w - 1) - 1); return kValInt; }
        }
    }
    const int64_t q64 = e10 + drop - frac_kept;
    if (w == 0) {
        bits = neg ? 0x8000000000000000ull : 0ull;
        return kValDouble;
    }
    if (q64 < -100000 || q64 > 100000) {
        bits = (q64 > 0 ? kInfBits : 0ull) | (neg ? 0x8000000000000000ull : 0ull);
        return kValDouble;
    }
    const int32_t q = (int32_t)q64;
    int64_t r;
    if (!truncated && w <= (1ull << 53) && q >= -22 && q <= 22) {
        // Clinger's fast path: both operands exact, one correctly rounded operation
        double d = (double)w;
        d = q < 0 ? d / kExact10[-q] : d * kExact10[q];
        r = (int64_t)__double_as_longlong(d);
    } else {
        r = eisel_lemire(w, q, pow5);
        // more than 19 significant digits: the value lies between w and w + 1
        // at this exponent; decided only when both round alike
        if (r >= 0 && truncated && eisel_lemire(w + 1, q, pow5) != r) r = -1;
    }
    if (r < 0) return kValDeferred;
    bits = (uint64_t)r | (neg ? 0x8000000000000000ull : 0ull);
    return kValDouble;
}

// ---- the exact conversion ----------------------------------------------------------

constexpr int kDecHold = 800;                 // digits held between shifts
constexpr int kDecBuf = kDecHold + 20;        // room for the digits one left shift adds
constexpr int kDeferredThreads = 128;       // four warps, a digit buffer each
constexpr int kSweptThreads = 32;           // a digit buffer per thread

// value = 0.d[0] d[1] ... d[nd-1] * 10^dp; `trunc`: nonzero digits beyond
// d[nd-1] were dropped (the value is a little above what is held)
struct Decimal {
    uint8_t* d;
    int nd;
    int dp;
    bool trunc;
};

__device__ void dec_trim(Decimal& x)
{
    while (x.nd > 0 && x.d[x.nd - 1] == 0) x.nd--;
    if (x.nd == 0) x.dp = 0;
}

// x /= 2^k, 1 <= k <= 60
__device__ void dec_shr(Decimal& x, int k)
{
    const uint64_t mask = (1ull << k) - 1;
    uint64_t n = 0;
    int r = 0, w = 0;
    while ((n >> k) == 0) {               // digits until the quotient's first one is nonzero
        if (r < x.nd) {
            n = n * 10 + x.d[r];
        } else {
            if (n == 0) { x.nd = 0; x.dp = 0; return; }
            n *= 10;
        }
        r++;
    }
    x.dp -= r - 1;
    while (r < x.nd) {                    // one digit out per digit in: w < r throughout
        const uint8_t c = (uint8_t)(n >> k);
        n = (n & mask) * 10 + x.d[r++];
        x.d[w++] = c;
    }
    while (n > 0) {                       // the remainder's digits
        const uint8_t c = (uint8_t)(n >> k);
        n = (n & mask) * 10;
        if (w < kDecHold) x.d[w++] = c;
        else if (c) x.trunc = true;
    }
    x.nd = w;
    dec_trim(x);
}

// x *= 2^k, 1 <= k <= 60: digits from the last, each written 19 places
// further on (2^60 * 9 carries into at most 19 new digits), then moved down
__device__ void dec_shl(Decimal& x, int k)
{
    if (x.nd == 0) return;
    constexpr int kOff = 19;
    const int end = x.nd + kOff;
    int w = end;
    uint64_t n = 0;
    for (int r = x.nd - 1; r >= 0; r--) {
        n += (uint64_t)x.d[r] << k;
        const uint64_t q = n / 10;
        x.d[--w] = (uint8_t)(n - 10 * q);
        n = q;
    }
    while (n > 0) {
        const uint64_t q = n / 10;
        x.d[--w] = (uint8_t)(n - 10 * q);
        n = q;
    }
    int len = end - w;
    x.dp += len - x.nd;
    if (len > kDecHold) {
        for (int j = w + kDecHold; j < end; j++)
            if (x.d[j]) x.trunc = true;
        len = kDecHold;
    }
    for (int j = 0; j < len; j++) x.d[j] = x.d[w + j];
    x.nd = len;
    dec_trim(x);
}

// floor(k * log2(10)) for 1 <= k <= 18: the shift that keeps a value below
// 10^-k below 1
__device__ __forceinline__ int dec_shift_for(int k) { return k >= 18 ? 59 : (k * 217706) >> 16; }

// the integer nearest x (x < 2^53 + 1), ties to even
__device__ uint64_t dec_round(const Decimal& x)
{
    if (x.nd == 0 || x.dp < 0) return 0;
    uint64_t n = 0;
    int i = 0;
    for (; i < x.dp && i < x.nd; i++) n = n * 10 + x.d[i];
    for (; i < x.dp; i++) n *= 10;
    bool up = false;
    if (x.dp < x.nd) {
        const uint8_t c = x.d[x.dp];
        // trailing zeros are trimmed: a digit after the 5 means above half
        up = c > 5 || (c == 5 && (x.trunc || x.dp + 1 < x.nd || (n & 1)));
    }
    return n + up;
}

// the number token [a, b) (its syntax already checked) as the correctly
// rounded double's bits, sign included
__device__ uint64_t decode_number_exact(Reader& rd, uint64_t a, uint64_t b, uint8_t* digits)
{
    Decimal x{digits, 0, 0, false};
    uint64_t p = a;
    const bool neg = rd.at(p) == '-';
    if (neg) p++;
    uint8_t c;
    for (; p < b && (c = rd.at(p)) >= '0' && c <= '9'; p++) {
        if (x.nd == 0 && c == '0') continue;                     // a leading zero
        if (x.nd < kDecHold) x.d[x.nd++] = (uint8_t)(c - '0');
        else if (c != '0') x.trunc = true;
        x.dp++;
    }
    if (p < b && rd.at(p) == '.') {
        for (p++; p < b && (c = rd.at(p)) >= '0' && c <= '9'; p++) {
            if (x.nd == 0 && c == '0') { x.dp--; continue; }     // zeros before the first digit
            if (x.nd < kDecHold) x.d[x.nd++] = (uint8_t)(c - '0');
            else if (c != '0') x.trunc = true;
        }
    }
    if (p < b) {                                                 // the exponent
        p++;
        bool eneg = false;
        if ((c = rd.at(p)) == '+' || c == '-') { eneg = c == '-'; p++; }
        int e = 0;
        for (; p < b; p++)
            if (e < 100000) e = e * 10 + (rd.at(p) - '0');
        x.dp += eneg ? -e : e;
    }
    dec_trim(x);
    const uint64_t sign = neg ? 0x8000000000000000ull : 0ull;
    if (x.nd == 0 || x.dp < -330) return sign;                   // below half the least subnormal
    if (x.dp > 310) return sign | kInfBits;
    int e2 = 0;
    while (x.dp > 0) {
        const int k = x.dp >= 18 ? 60 : dec_shift_for(x.dp);
        dec_shr(x, k);
        e2 += k;
    }
    while (x.dp < 0 || (x.dp == 0 && x.d[0] < 5)) {
        const int k = x.dp == 0 ? 1 : dec_shift_for(-x.dp);
        dec_shl(x, k);
        e2 -= k;
    }
    // the value is v * 2^e2 with v in [1/2, 1): 1.f * 2^(e2 - 1)
    int e = e2 - 1;
    if (e > 1023) return sign | kInfBits;
    if (e < -1022) {                                             // subnormal: down to 2^-1022
        for (int s = -1022 - e; s > 0; s -= 60) dec_shr(x, s < 60 ? s : 60);
        e = -1022;
    }
    dec_shl(x, 53);
    uint64_t m = dec_round(x);
    if (m == (1ull << 53)) {
        m >>= 1;
        if (++e > 1023) return sign | kInfBits;
    }
    if (m < (1ull << 52)) return sign | m;                      // subnormal (or zero)
    return sign | ((uint64_t)(e + 1023) << 52) | (m & ((1ull << 52) - 1));
}

// the trimmed text of slot i: [a, b) (a == b: nothing)
// the text of slot i, untrimmed: [a, b)
__device__ __forceinline__ void slot_bounds(const ValueParams& P, uint64_t i, uint64_t& a, uint64_t& b)
{
    a = i == 0 ? 0 : (uint64_t)(uint32_t)__ldg(P.pos + i - 1);          // positions are 1-based
    b = i == P.S ? P.n_bytes : (uint64_t)(uint32_t)__ldg(P.pos + i) - 1;
    if (b < a) b = a;
}

// [a, b) less JSON whitespace at both ends, by one thread
__device__ void trim(Reader& rd, uint64_t& a, uint64_t& b)
{
    rd.seek(a);
    while (a < b && is_ws(rd.at(a))) a++;
    while (b > a && is_ws(rd.at(b - 1))) b--;
}

// the same by a warp, 512 bytes a step from each end; every lane gets the
// result (a slot may hold a long run of whitespace)
__device__ void trim_warp(Reader& rd, uint64_t& a, uint64_t& b)
{
    const int lane = (int)(threadIdx.x & 31);
    rd.seek(a);
    uint64_t base = a;
    for (; base < b; base += 32 * kLaneBytes) {
        uint32_t m = 0;                                   // this lane's non-whitespace bytes
        for (int k = 0; k < kLaneBytes; k++) {
            const uint64_t x = base + (uint64_t)(kLaneBytes * lane + k);
            m |= (uint32_t)(x < b && !is_ws(rd.at(x))) << k;
        }
        const uint32_t any = __ballot_sync(~0u, m != 0);
        if (any) {
            const int src = __ffs(any) - 1;
            base += (uint64_t)(kLaneBytes * src + __ffs(__shfl_sync(~0u, m, src)) - 1);
            break;
        }
    }
    a = base < b ? base : b;
    uint64_t top = b;                                     // one past the last byte looked at
    for (; top > a; top -= top - a < 32 * kLaneBytes ? top - a : 32 * kLaneBytes) {
        uint32_t m = 0;
        for (int k = 0; k < kLaneBytes; k++) {
            const uint64_t d = (uint64_t)(kLaneBytes * lane + k) + 1;
            m |= (uint32_t)(d <= top - a && !is_ws(rd.at(top - d))) << k;
        }
        const uint32_t any = __ballot_sync(~0u, m != 0);
        if (any) {
            const int src = __ffs(any) - 1;
            top -= (uint64_t)(kLaneBytes * src + __ffs(__shfl_sync(~0u, m, src)) - 1);
            break;
        }
    }
    b = top;
}

// slot i's trimmed text [a, b) decoded.  With defer_escapes, a string that
// holds an escape is left to the warp kernel (kValDeferred): one long escaped
// string would otherwise hold up the 31 other slots of its warp.
__device__ uint8_t decode_slot(const ValueParams& P, Reader& rd, uint64_t i, uint64_t a, uint64_t b,
                               bool defer_escapes)
{
    if (a == b) return kValNone;
    const uint8_t c = rd.at(a);
    if (c == '"') {
        if (b - a < 2 || rd.at(b - 1) != '"') return kValInvalid;
        int64_t n = a >= rd.lo ? copy_plain(rd, a + 1, b - 1, P.str_out) : -1;
        if (n < 0 && defer_escapes) return kValDeferred;
        if (n < 0) n = decode_string(rd, a, b - 1, P.str_out);
        if (n < 0) return kValInvalid;
        P.num[i] = a + 1;                 // where the decoded bytes start
        P.len[i] = (uint32_t)n;
        return kValString;
    }
    if (c == 't' || c == 'f' || c == 'n') {
        const char* lit = c == 't' ? "true" : c == 'f' ? "false" : "null";
        const uint64_t n = c == 'f' ? 5 : 4;
        if (b - a != n) return kValInvalid;
        for (uint64_t k = 0; k < n; k++)
            if (rd.at(a + k) != (uint8_t)lit[k]) return kValInvalid;
        return c == 't' ? kValTrue : c == 'f' ? kValFalse : kValNull;
    }
    if (c == '-' || (c >= '0' && c <= '9')) {
        uint64_t bits = 0;
        const uint8_t t = decode_number(rd, a, b, P.pow5, bits);
        if (t == kValInt || t == kValDouble) P.num[i] = bits;
        return t;
    }
    return kValInvalid;
}

__global__ void __launch_bounds__(kValThreads) decode_slots(ValueParams P)
{
    allow_next_grid();
    const uint64_t n = (uint64_t)P.S + 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        Reader rd{&P, 0, 0, 0, nullptr};
        uint64_t a, b;
        slot_bounds(P, i, a, b);
        P.num[i] = 0;
        P.len[i] = 0;
        const bool long_slot = b - a > kShortBytes;
        uint8_t t = kValNone;
        if (!long_slot) {
            trim(rd, a, b);
            t = decode_slot(P, rd, i, a, b, true);
        }
        if (long_slot) {
            const uint32_t k = atomicAdd(P.counters, 1u);
            if (k < P.long_cap) {
                P.long_list[k] = (uint32_t)i;                        // decided by decode_deferred
            } else {                                                 // (cannot fill: kept for safety)
                trim(rd, a, b);
                t = decode_slot(P, rd, i, a, b, false);
            }
        } else if (t == kValDeferred) {
            const uint32_t k = atomicAdd(P.counters + 1, 1u);
            if (k < P.short_cap) P.short_list[k] = (uint32_t)i;       // decided by decode_deferred
            else t = decode_slot(P, rd, i, a, b, false);             // strings here; numbers left for decode_swept
        }
        P.type[i] = t;
    }
}

__device__ void decode_deferred_number(const ValueParams& P, Reader& rd, uint64_t i, uint64_t a, uint64_t b,
                                       uint8_t* digits)
{
    P.num[i] = decode_number_exact(rd, a, b, digits);
    P.type[i] = kValDouble;
}

// a warp per listed slot: trimmed by the warp, then a string decoded by the
// whole warp, anything else by its first lane
__device__ void decode_listed(const ValueParams& P, uint64_t i, uint8_t* stage, uint8_t* ostage, uint8_t* digits)
{
    const uint32_t lane = threadIdx.x & 31;
    Reader rd{&P, 0, 0, 0, nullptr};
    uint64_t a, b;
    slot_bounds(P, i, a, b);
    trim_warp(rd, a, b);
    if (a < b && rd.at(a) == '"' && b - a >= 2 && rd.at(b - 1) == '"' && a >= rd.lo) {
        // the whole string lies in the segment of its closing quote
        const int64_t m = decode_string_warp(rd.base + (a + 1 - rd.lo), b - a - 2, P.str_out + a + 1, stage, ostage);
        if (lane == 0) {
            P.num[i] = m < 0 ? 0 : a + 1;
            P.len[i] = m < 0 ? 0u : (uint32_t)m;
            P.type[i] = m < 0 ? kValInvalid : kValString;
        }
    } else if (lane == 0) {
        const uint8_t t = decode_slot(P, rd, i, a, b, false);
        if (t == kValDeferred) decode_deferred_number(P, rd, i, a, b, digits);
        else P.type[i] = t;
    }
}

// the long slots first, a warp each in turn; then the short list, taken four
// entries at a time from a ticket, so that warps done early take more
__global__ void __launch_bounds__(kDeferredThreads) decode_deferred(ValueParams P)
{
    constexpr int kWarps = kDeferredThreads / 32;
    constexpr uint32_t kTake = 4;
    __shared__ uint8_t digits[kWarps][kDecBuf];
    __shared__ __align__(16) uint8_t stage[kWarps][kStage];
    __shared__ uint8_t ostage[kWarps][kWarpStep + 8];    // a step's escape may emit 3 bytes past its input
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    allow_next_grid();
    wait_previous_grid();
    const uint32_t nl = min(__ldcg(P.counters), P.long_cap), ns = min(__ldcg(P.counters + 1), P.short_cap);
    for (uint32_t k = blockIdx.x * kWarps + warp; k < nl; k += gridDim.x * kWarps)
        decode_listed(P, P.long_list[k], stage[warp], ostage[warp], digits[warp]);
    for (;;) {
        uint32_t k = 0;
        if (lane == 0) k = atomicAdd(P.counters + 2, kTake);
        k = __shfl_sync(FULL_MASK, k, 0);
        if (k >= ns) break;
        for (uint32_t e = k; e < k + kTake && e < ns; e++)
            decode_listed(P, P.short_list[e], stage[warp], ostage[warp], digits[warp]);
    }
}

// only when the list overflowed: a thread per slot, the deferred numbers the
// list did not hold
__global__ void __launch_bounds__(kSweptThreads) decode_swept(ValueParams P)
{
    __shared__ uint8_t digits[kSweptThreads][kDecBuf];
    allow_next_grid();
    wait_previous_grid();
    if (P.counters[0] <= P.long_cap && P.counters[1] <= P.short_cap) return;   // the lists held every entry
    const uint64_t n = (uint64_t)P.S + 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (P.type[i] != kValDeferred) continue;
        Reader rd{&P, 0, 0, 0, nullptr};
        uint64_t a, b;
        slot_bounds(P, i, a, b);
        trim(rd, a, b);
        decode_deferred_number(P, rd, i, a, b, digits[threadIdx.x]);
    }
}

// type counts: four slots a word, a count per type in registers, summed by
// warp, block and grid
__global__ void __launch_bounds__(kValThreads) count_types(ValueParams P)
{
    __shared__ unsigned long long c[kValTypes];
    if (threadIdx.x < kValTypes) c[threadIdx.x] = 0;
    wait_previous_grid();
    __syncthreads();
    const uint64_t n = (uint64_t)P.S + 1, words = (n + 3) / 4;
    uint32_t k[kValTypes] = {};
    const uint32_t* tw = reinterpret_cast<const uint32_t*>(P.type);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t w = __ldg(tw + i);
        const uint64_t left = n - 4 * i;
        const uint32_t live = left >= 4 ? 0x01010101u : (0x01010101u >> (8 * (4 - (uint32_t)left)));
#pragma unroll
        for (int t = 0; t < kValTypes; t++) k[t] += __popc(__vcmpeq4(w, 0x01010101u * (uint32_t)t) & live);
    }
#pragma unroll
    for (int t = 0; t < kValTypes; t++) {
        const uint32_t v = __reduce_add_sync(FULL_MASK, k[t]);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&c[t], (unsigned long long)v);
    }
    __syncthreads();
    if (threadIdx.x < kValTypes && c[threadIdx.x]) atomicAdd(P.counts + threadIdx.x, c[threadIdx.x]);
}

}  // namespace

cudaError_t launch_decode_values(const ValueParams& p, int sm_count, cudaStream_t stream)
{
    const uint64_t n = (uint64_t)p.S + 1;
    const int grid = (int)std::min<uint64_t>((n + kValThreads - 1) / kValThreads, (uint64_t)sm_count * 8);
#ifdef CJ_EMU
    (void)stream;
    cj_emu::launch(grid, kValThreads, 0, [&] { decode_slots(p); });
    cj_emu::launch(sm_count * 2, kDeferredThreads, 0, [&] { decode_deferred(p); });
    cj_emu::launch(sm_count * 2, kSweptThreads, 0, [&] { decode_swept(p); });
    cj_emu::launch(grid, kValThreads, 0, [&] { count_types(p); });
    return cudaSuccess;
#else
    decode_slots<<<grid, kValThreads, 0, stream>>>(p);
    const bool dep = p.dependent_launch != 0;
    launch_dependent(decode_deferred, sm_count * 16, kDeferredThreads, 0, stream, dep, p);
    launch_dependent(decode_swept, sm_count * 8, kSweptThreads, 0, stream, dep, p);
    launch_dependent(count_types, grid, kValThreads, 0, stream, dep, p);
    return cudaGetLastError();
#endif
}

cudaError_t preload_value_kernels()
{
#ifdef CJ_EMU
    return cudaSuccess;
#else
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, (const void*)decode_slots);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)decode_deferred);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)decode_swept);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)count_types);
    return e;
#endif
}

// the 128-bit powers of five (pow5_table.py), copied to the device once
extern const uint64_t kPow5Table[2 * 651];
const uint64_t kPow5Table[2 * 651] = {
#include "cj_pow5.inc"
};

}  // namespace cj
