/*
 * cj_oracle_query.c -- CPU oracle for key/value queries over a JSON-Lines
 * parse result.
 *
 * TEST INFRASTRUCTURE ONLY (see cj_oracle.h): the checker of the device query
 * engine, never linked into the product.
 *
 * It restates, step for step and serially, the reference's real-world query
 * loop (real_world_use_case/main.cu:70-86):
 *
 *     itr.gotoArrayIndex(0);
 *     for each record:  if (itr.checkKeyValue(key, value)) count++;
 *                       itr.gotoNextSibling(1);
 *
 * with cuJSONLinesIterator's rules (cujson/query/query_iterator.cpp):
 *   - the constructor's layout fix-ups: structural[0] = 0,
 *     structural[S+1] = fileSize - 1, pair_pos[0] = S + 1 (:86-114);
 *   - getChar (:128), jumpSpacesForward / Backward (:139, :147),
 *     jumpValueBackward / Forward (:155, :166);
 *   - gotoArrayIndex (:233) and gotoArrayIndexSiblingHelper (:301) through
 *     gotoNextSibling (:370): step over containers with pair_pos, count ','
 *     (a newline entry reads as ',') and ' ' as separators, stop at ']' or at
 *     the virtual close;
 *   - getString (:435), findKey (:447), getValue (:512), checkKeyValue (:614).
 * The loop runs until gotoNextSibling fails, i.e. once per top-level
 * separator plus one, which is what the reference's fixed iteration count
 * does on a file of that many records.
 *
 * Two reads the reference makes outside the file (getChar of the virtual root
 * reads byte -1; slices past the end) read as 0 / are clamped here, as in the
 * drop-in iterator; slices with negative length are "" (the reference throws
 * std::length_error there).
 *
 * Parity of this restatement with the reference's own iterator is pinned by
 * tests/golden/query_golden.json, made by running the reference's iterator
 * sources on the same inputs (tests/golden/make_query_golden.py).
 */
#include "cj_oracle.h"

#include <stdlib.h>
#include <string.h>

typedef struct {
    const uint8_t* buf;
    int64_t n;
    const int32_t* pos;   /* 1-based byte positions, S entries */
    const int32_t* pair;  /* 1-based close index at opens, S entries */
    int64_t S;
} view_t;

static uint8_t at(const view_t* v, int64_t b) { return (b >= 0 && b < v->n) ? v->buf[b] : 0; }

/* structural[idx] of the reference layout after the iterator's constructor */
static int64_t structural(const view_t* v, int64_t idx)
{
    if (idx <= 0) return 0;
    if (idx == v->S + 1) return v->n - 1;
    if (idx > v->S + 1) return 0;
    return v->pos[idx - 1];
}

static int64_t pair_pos(const view_t* v, int64_t idx)
{
    if (idx == 0) return v->S + 1;
    if (idx < 1 || idx > v->S) return idx;
    return v->pair[idx - 1];
}

static char get_char(const view_t* v, int64_t idx)
{
    if (idx < 0 || idx > v->S + 1) return '\0';
    const uint8_t c = at(v, structural(v, idx) - 1);
    if (c == '\n') return ',';
    if (idx == v->S + 1) return ']';
    if (idx == 0) return '[';
    return (char)c;
}

static void clamp_slice(const view_t* v, int64_t* start, int64_t* len)
{
    if (*len <= 0 || *start < 0 || *start >= v->n) {
        *len = 0;
        return;
    }
    if (*start + *len > v->n) *len = v->n - *start;
}

/* gotoArrayIndexSiblingHelper(1) from `node`: the next separator, or 0 */
static int64_t next_sibling(const view_t* v, int64_t node)
{
    int total = 2;
    int64_t nx = node + 1;
    char c = get_char(v, nx);
    while (total != 1 && c != ']' && nx != v->S + 1) {
        if (c == '[' || c == '{') {
            const int64_t j = pair_pos(v, nx);
            if (j <= nx) return 0;            /* not a valid result */
            nx = j;
        }
        if (c == ',' || c == '\n' || c == ' ') total--;
        nx++;
        c = get_char(v, nx);
    }
    return total == 1 ? nx - 1 : 0;
}

/* findKey from `node`: the ':' node of the key, 0 if absent; *rec = the '{' */
static int64_t find_key(const view_t* v, int64_t node, const uint8_t* key, int64_t key_len, int64_t* rec)
{
    const char cur = get_char(v, node);
    int64_t nx = node;
    if (cur == ':' || cur == ',' || cur == '\n') nx = node + 1;
    if (cur == '[' && get_char(v, node + 1) == '{') nx = node + 1;
    if (get_char(v, nx) != '{') return 0;
    *rec = nx;
    const int64_t end = pair_pos(v, nx);
    nx++;
    char c = get_char(v, nx);
    while (nx < end && c != '}') {
        if (c == '[' || c == '{') {
            const int64_t j = pair_pos(v, nx);
            if (j <= nx) return 0;
            nx = j;
        }
        if (c == ':') {
            /* getString(structural[nx-1]-1, structural[nx]-1) */
            int64_t s = structural(v, nx - 1);          /* (startPos) + 1 */
            while (at(v, s) == ' ') s++;
            int64_t e = structural(v, nx) - 2;          /* (endPos) - 1 */
            while (e >= 0 && at(v, e) == ' ') e--;
            int64_t ks = s + 1, kl = llabs(e - s - 1);
            clamp_slice(v, &ks, &kl);
            if (kl == key_len && (key_len == 0 || memcmp(v->buf + ks, key, (size_t)key_len) == 0)) return nx;
        }
        nx++;
        c = get_char(v, nx);
    }
    return 0;
}

/* getValue at the ':' node `colon`: the slice (start, length) */
static void get_value(const view_t* v, int64_t colon, int64_t* start, int64_t* len)
{
    const int64_t si = colon + 1;
    const char c = get_char(v, si);
    int64_t a, b;
    if (c == '[' || c == '{') {
        a = structural(v, si) - 1;
        b = structural(v, pair_pos(v, si)) - 1;
    } else {
        a = structural(v, colon);                      /* jumpValueForward(structural-1) */
        for (;;) {
            const uint8_t ch = at(v, a);
            if (ch == '"') { a++; break; }
            if (ch != ' ') break;
            a++;
        }
        b = structural(v, si) - 2;                     /* jumpValueBackward(structural-1) */
        while (b >= 0) {
            const uint8_t ch = at(v, b);
            if (ch == '"') { b--; break; }
            if (ch != ' ') break;
            b--;
        }
    }
    *start = a;
    *len = b - a + 1;
    clamp_slice(v, start, len);
}

int64_t cjo_query_lines(const uint8_t* buf, size_t n, const int32_t* positions, const int32_t* pair_row,
                        size_t S, const uint8_t* key, size_t key_len, const uint8_t* value, size_t value_len,
                        int check_value, int64_t* out, size_t cap)
{
    view_t v = {buf, (int64_t)n, positions, pair_row, (int64_t)S};
    int64_t count = 0;
    int64_t node = 0;              /* gotoArrayIndex(0) stays on the virtual root */
    int64_t arr = 0;               /* currArrayNode */
    for (;;) {
        int64_t rec = 0;
        const int64_t colon = find_key(&v, node, key, (int64_t)key_len, &rec);
        if (colon) {
            int64_t vs, vl;
            get_value(&v, colon, &vs, &vl);
            const int ok = !check_value ||
                           (vl == (int64_t)value_len && (vl == 0 || memcmp(buf + vs, value, (size_t)vl) == 0));
            if (ok) {
                if (out && (size_t)count < cap) {
                    out[3 * count] = structural(&v, rec) - 1;
                    out[3 * count + 1] = vs;
                    out[3 * count + 2] = vl;
                }
                count++;
            }
        }
        node = arr;                /* gotoNextSibling(1) */
        const int64_t nx = next_sibling(&v, node);
        if (!nx) break;
        node = arr = nx;
    }
    return count;
}
