/*
 * cj_oracle.c -- CPU oracle for the cuJSON parse path (TEST INFRASTRUCTURE).
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg, as the checker.  The product never calls it.  See cj_oracle.h for the
 * output contract.  Each function names the reference code it restates.
 */
#include "cj_oracle.h"

#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------------------
 * Strict UTF-8 (RFC 3629, table 3-7 of the Unicode standard).  The reference's
 * stage 1 (cujson/parse_standard_json.cu:264-327) is meant to implement this
 * check; its predicate is defective (see cjo_utf8_refcompat below), so the
 * strict verdict is the specification itself.
 * ------------------------------------------------------------------------- */
int cjo_utf8_valid(const uint8_t* s, size_t n)
{
    size_t i = 0;
    while (i < n) {
        uint8_t c = s[i];
        if (c < 0x80) { i++; continue; }
        size_t len;
        uint8_t lo = 0x80, hi = 0xBF;          /* range of the 2nd byte */
        if (c >= 0xC2 && c <= 0xDF)      { len = 2; }
        else if (c == 0xE0)              { len = 3; lo = 0xA0; }
        else if (c >= 0xE1 && c <= 0xEC) { len = 3; }
        else if (c == 0xED)              { len = 3; hi = 0x9F; }
        else if (c >= 0xEE && c <= 0xEF) { len = 3; }
        else if (c == 0xF0)              { len = 4; lo = 0x90; }
        else if (c >= 0xF1 && c <= 0xF3) { len = 4; }
        else if (c == 0xF4)              { len = 4; hi = 0x8F; }
        else return 0;                       /* 80..C1, F5..FF */
        if (i + len > n) return 0;
        if (s[i + 1] < lo || s[i + 1] > hi) return 0;
        for (size_t k = 2; k < len; k++)
            if ((s[i + k] & 0xC0) != 0x80) return 0;
        i += len;
    }
    return 1;
}

/* ---------------------------------------------------------------------------
 * The reference's per-word UTF-8 predicate, restated from the documented
 * semantics of the SIMD-in-word intrinsics it uses.  Follows
 * checkUTF8 (cujson/parse_standard_json.cu:210-262), vectorizedClassification
 * (:9-150) and continuationBytes (:152-183).  The reference records each
 * word's result with atomicExch into one shared word, so the verdict depends on
 * thread order; this restatement ORs every word's result instead, which is the
 * most-rejecting outcome of that race.
 * ------------------------------------------------------------------------- */
static uint32_t bytewise(uint32_t a, uint32_t b, int op)
{
    uint32_t r = 0;
    for (int k = 0; k < 4; k++) {
        uint32_t x = (a >> (8 * k)) & 0xFF, y = (b >> (8 * k)) & 0xFF, v = 0;
        switch (op) {
        case 0: v = (x == y) ? 0xFF : 0; break;          /* vcmpeq4  */
        case 1: v = (x < y) ? 0xFF : 0; break;           /* vcmpltu4 */
        case 2: v = (x >= y) ? 0xFF : 0; break;          /* vcmpgeu4 */
        case 3: v = (x > y) ? 0xFF : 0; break;           /* vcmpgtu4 */
        case 4: v = (x > y) ? (x - y) : 0; break;        /* vsubus4  */
        }
        r |= v << (8 * k);
    }
    return r;
}
#define EQ4(a, b)  bytewise((a), (b), 0)
#define LT4(a, b)  bytewise((a), (b), 1)
#define GE4(a, b)  bytewise((a), (b), 2)
#define GT4(a, b)  bytewise((a), (b), 3)
#define SUBUS4(a, b) bytewise((a), (b), 4)

static uint32_t ref_word_error(uint32_t current, uint32_t previous)
{
    const uint32_t max_val = 0xBFDFEFFFu;   /* per-byte "incomplete lead" limits */
    uint32_t prev_incomplete = SUBUS4(previous, max_val);
    if ((current & 0x80808080u) == 0) return prev_incomplete;

    uint64_t dist = ((uint64_t)current << 32) | previous;
    uint32_t prev1 = (uint32_t)(dist >> 24);
    uint32_t prev2 = (uint32_t)(dist >> 16);
    uint32_t prev3 = (uint32_t)(dist >> 8);

    /* vectorizedClassification: the first-byte classes are computed and then
     * overwritten by "class == 0" -> TWO_CONTS (parse_standard_json.cu:122-123),
     * which leaves 0x80 exactly where prev1 is a continuation byte. */
    uint32_t byte1_classes =
        (LT4(prev1, 0x80808080u) & 0x02020202u) | (GE4(prev1, 0xC0C0C0C0u) & 0x01010101u);
    uint32_t byte_1 = EQ4(byte1_classes, 0) & 0x80808080u;

    uint32_t hi = (current >> 4) & 0x0F0F0F0Fu;
    uint32_t lt12 = LT4(hi, 0x0C0C0C0Cu);
    uint32_t byte_2_high =
        ((LT4(hi, 0x08080808u) | GT4(hi, 0x0B0B0B0Bu)) & 0x01010101u) |
        (lt12 & GE4(hi, 0x08080808u) & (0x02020202u | 0x20202020u | 0x80808080u)) |
        (lt12 & GT4(hi, 0x08080808u) & 0x08080808u) |
        (EQ4(hi, 0x08080808u) & 0x40404040u) |
        (GT4(hi, 0x09090909u) & lt12 & 0x10101010u);
    uint32_t sc = byte_1 & byte_2_high;

    /* continuationBytes: a byte two after a 3/4-byte lead or three after a
     * 4-byte lead must be a continuation ("must32"); compared with sc. */
    uint32_t third = SUBUS4(prev2, 0xDFDFDFDFu);
    uint32_t fourth = SUBUS4(prev3, 0xEFEFEFEFu);
    uint32_t must32 = GT4(third | fourth, 0);
    return (must32 & 0x80808080u) ^ sc;
}

int cjo_utf8_refcompat(const uint8_t* s, size_t n)
{
    size_t words = (n + 3) / 4;
    int has_high = 0;
    for (size_t i = 0; i < n; i++) if (s[i] & 0x80) { has_high = 1; break; }
    if (!has_high) return 1;   /* checkAscii short-cut, :290-295 */
    uint32_t prev = 0, acc = 0;
    for (size_t j = 0; j < words; j++) {
        uint32_t cur = 0;
        for (int k = 0; k < 4; k++) {
            size_t p = 4 * j + (size_t)k;
            if (p < n) cur |= (uint32_t)s[p] << (8 * k);   /* zero padded, :1616-1619 */
        }
        acc |= ref_word_error(cur, j ? prev : 0);
        prev = cur;
    }
    return acc == 0;
}

/* ---------------------------------------------------------------------------
 * Structural scan, serial form.
 *
 * The reference builds bitmaps of backslashes, quotes and { } [ ] : ,
 * (bitMapCreatorSimd, parse_standard_json.cu:446-571; JSON Lines adds '\n',
 * parse_json_lines.cu:453-458), removes quotes preceded by an odd run of
 * backslashes (findEscapedQuoteMerge_NEW, :767-834), turns the real quotes into
 * an in-string mask by prefix XOR plus the parity of earlier words
 * (inStringFinderBaseline, :851-862 and utils.cu:141), keeps the structural
 * characters outside that mask (findOutUsefulStringMerge, :916-937) and
 * compacts them into 1-based byte positions (removeCopy, :1007).  Escapes are
 * decided by backslash runs alone, inside or outside strings.  The serial loop
 * below computes the same sets one byte at a time.
 *
 * Pairing: the reference keys each bracket by its depth, stable-sorts by that
 * key and pairs neighbours (Parser, :1519-1582); for balanced input that is
 * the stack matching done here.
 * ------------------------------------------------------------------------- */
typedef struct { int32_t sidx; int32_t curly; } open_ent;

uint32_t cjo_parse(const uint8_t* buf, size_t n, int lines_mode,
                   const size_t* chunk_sizes, size_t n_chunks,
                   int32_t* structural, int32_t* pair_row, size_t cap,
                   cjo_stats* st)
{
    cjo_stats local;
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    uint32_t flags = 0;

    size_t one = n;
    if (!chunk_sizes) { chunk_sizes = &one; n_chunks = 1; }

    size_t stack_cap = 1024;
    open_ent* stack = (open_ent*)malloc(stack_cap * sizeof(open_ent));
    int64_t S = 0;
    size_t base = 0;

    for (size_t ch = 0; ch < n_chunks; ch++) {
        size_t len = chunk_sizes[ch];
        if (base + len > n) len = (base < n) ? n - base : 0;
        const uint8_t* p = buf + base;

        if (!cjo_utf8_valid(p, len)) flags |= CJO_ERR_UTF8;

        int in_str = 0;
        uint64_t bs_run = 0;
        size_t depth = 0;
        for (size_t i = 0; i < len; i++) {
            uint8_t c = p[i];
            if (c == '"') {
                if ((bs_run & 1) == 0) in_str ^= 1;
            } else if (!in_str) {
                int is_open = (c == '{' || c == '[');
                int is_close = (c == '}' || c == ']');
                int is_st = is_open || is_close || c == ':' || c == ',' ||
                            (lines_mode && c == '\n');
                if (is_st) {
                    int64_t sidx = S++;
                    if ((size_t)sidx < cap) {
                        if (structural) structural[sidx] = (int32_t)(base + i + 1);
                        if (pair_row) pair_row[sidx] = 0;
                    } else {
                        flags |= CJO_ERR_CAPACITY;
                    }
                    if (is_open) {
                        if (depth == stack_cap) {
                            stack_cap *= 2;
                            stack = (open_ent*)realloc(stack, stack_cap * sizeof(open_ent));
                        }
                        stack[depth].sidx = (int32_t)sidx;
                        stack[depth].curly = (c == '{');
                        depth++;
                        st->n_opens++;
                        if ((int64_t)depth > st->max_depth) st->max_depth = (int32_t)depth;
                        st->n_brackets++;
                    } else if (is_close) {
                        st->n_brackets++;
                        if (depth == 0) {
                            flags |= CJO_ERR_BRACKETS;
                        } else {
                            depth--;
                            if (stack[depth].curly != (c == '}')) flags |= CJO_ERR_BRACKETS;
                            if (pair_row && (size_t)stack[depth].sidx < cap)
                                pair_row[stack[depth].sidx] = (int32_t)(sidx + 1);
                        }
                    }
                }
            }
            bs_run = (c == '\\') ? bs_run + 1 : 0;
        }
        if (depth != 0) flags |= CJO_ERR_BRACKETS;
        base += len;
    }
    free(stack);
    st->n_structural = S;
    st->flags = flags;
    return flags;
}
