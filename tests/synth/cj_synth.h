/* cj_synth.h -- seeded synthetic JSON / JSON-Lines generators (test and
 * benchmark data, not part of the parser library).
 *
 * The reference is evaluated on ~1 GB real-world datasets that are not
 * available offline; these generators stand in for them.  Deterministic for a
 * given seed on every machine and for any thread count.  Built into
 * tests/synth/_build/libcj_synth.so by tests/synth/build.py. */
#ifndef CJ_SYNTH_H
#define CJ_SYNTH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cj_synth_params {
    int32_t  max_depth;          /* nesting limit of values */
    int32_t  keys_min, keys_max; /* members per top-level object */
    int32_t  nested_max_items;   /* members / elements per nested container */
    int32_t  str_min, str_max;   /* string lengths */
    double   huge_string_frac;   /* fraction of strings that are huge */
    int64_t  huge_string_min, huge_string_max;
    uint64_t block_bytes;        /* independent generation block */
    double   record_median, record_sigma;   /* JSON-Lines lognormal sizes */
    int64_t  record_min, record_max;
    uint32_t threads;            /* 0 = all host threads */
} cj_synth_params;

void   cj_synth_default_params(cj_synth_params* p);
size_t cj_synth_document(uint64_t seed, size_t size, const cj_synth_params* p, uint8_t* out);
size_t cj_synth_lines(uint64_t seed, size_t size, const cj_synth_params* p, uint8_t* out,
                      uint64_t* n_records);
size_t cj_synth_events(uint64_t seed, size_t size, uint8_t* out, uint64_t* n_records, uint64_t* n_push);
size_t cj_synth_deep(size_t depth, uint8_t* out);
size_t cj_synth_backslash_string(uint64_t seed, size_t body, uint8_t* out);
int    cj_synth_corrupt(uint8_t* doc, size_t n, int kind, uint64_t seed);

#ifdef __cplusplus
}
#endif
#endif
