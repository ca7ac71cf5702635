/*
 * cj_oracle.h -- CPU oracle for the cuJSON parse path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the cujson_gb300 library,
 * its C-ABI or its drop-in headers) links, loads or calls this code.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and
 * only as the checker or the timed CPU baseline.
 *
 * It is a byte-serial restatement of what the reference computes for one
 * document (parse_standard_json) or one JSON-Lines buffer split into chunks
 * (parse_json_lines):
 *   - structural positions: 1-based byte offsets of { } [ ] : , (and '\n' in
 *     JSON-Lines mode) that lie outside strings
 *       (cujson/parse_standard_json.cu:446-571 bitmaps, :767-834 escapes,
 *        :851-862 in-string mask, :916-937 masking, :953-1021 compaction;
 *        cujson/parse_json_lines.cu:453-458 for the newline class);
 *   - the pair row: for the structural at 0-based index i that opens a
 *     container, pair_row[i] = 1-based structural index of its matching close;
 *     0 for every other entry (the reference leaves those uninitialised;
 *     cujson/parse_standard_json.cu:1497-1512 writes only opens);
 *   - the verdict: strict RFC 3629 UTF-8 plus balanced, type-matched brackets.
 *
 * Parity status: pinned.  tests/golden/parse_golden.json holds the outputs of
 * the reference's own parse code (its CUDA sources run on the CPU through the
 * emulation that oracle/build_ref.py builds) on 32 inputs -- hand-written,
 * seeded documents up to 1 MiB, backslash runs, nesting to depth 300, JSON
 * Lines in up to 4 chunks, planted errors -- and tests/test_parse_golden.py
 * checks this restatement against them bit for bit, apart from the documented
 * divergences (strict UTF-8, int32 depth).
 */
#ifndef CJ_ORACLE_H
#define CJ_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* verdict bits */
#define CJO_ERR_UTF8      1u   /* ill-formed UTF-8 (RFC 3629) */
#define CJO_ERR_BRACKETS  2u   /* unbalanced or mismatched { } [ ] */
#define CJO_ERR_CAPACITY  4u   /* output arrays too small */

typedef struct cjo_stats {
    int64_t  n_structural;  /* S */
    int64_t  n_brackets;    /* opens + closes outside strings */
    int64_t  n_opens;
    int32_t  max_depth;     /* deepest nesting seen (0 for no containers) */
    uint32_t flags;         /* CJO_ERR_* bits */
} cjo_stats;

/*
 * Parse `n` bytes.  In JSON-Lines mode (`lines_mode` != 0) the buffer is the
 * concatenation of `n_chunks` chunks of `chunk_sizes[i]` bytes; each chunk is
 * parsed on its own (string/escape state and depth start afresh, brackets must
 * balance inside the chunk), with byte positions and structural indices global
 * across chunks (cujson/parse_json_lines.cu:1133-1224).  chunk_sizes == NULL
 * means one chunk of `n` bytes.
 *
 * `structural` and `pair_row` must hold `cap` int32 entries each (either may
 * be NULL to only count).  Returns the CJO_ERR_* bits (also in st->flags).
 */
uint32_t cjo_parse(const uint8_t* buf, size_t n, int lines_mode,
                   const size_t* chunk_sizes, size_t n_chunks,
                   int32_t* structural, int32_t* pair_row, size_t cap,
                   cjo_stats* st);

/* Strict RFC 3629 validation of one byte range: 1 = well formed. */
int cjo_utf8_valid(const uint8_t* buf, size_t n);

/*
 * The reference's own UTF-8 predicate, OR-reduced over all 32-bit words
 * instead of raced through atomicExch (cujson/parse_standard_json.cu:9-184,
 * :210-262).  Audit only: it accepts many ill-formed inputs.  1 = accepted.
 */
int cjo_utf8_refcompat(const uint8_t* buf, size_t n);

/*
 * The reference's real-world query loop over a JSON-Lines result
 * (cj_oracle_query.c): visit every record the way gotoArrayIndex(0) +
 * gotoNextSibling(1) do, apply findKey(key) and getValue, and count the records
 * that have `key` (check_value == 0) or whose value for it equals `value`
 * (checkKeyValue).  `positions` / `pair_row` as cjo_parse writes them for the
 * whole file.  Writes up to `cap` triples (record byte offset, value byte
 * offset, value length) to `out` in visiting order; returns the count.
 */
int64_t cjo_query_lines(const uint8_t* buf, size_t n, const int32_t* positions, const int32_t* pair_row,
                        size_t S, const uint8_t* key, size_t key_len, const uint8_t* value, size_t value_len,
                        int check_value, int64_t* out, size_t cap);

#ifdef __cplusplus
}
#endif
#endif
