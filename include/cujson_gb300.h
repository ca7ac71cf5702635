/*
 * cujson_gb300.h -- C ABI of the GB300-native cuJSON parse path.
 *
 * Plain C: pointers, sizes and status codes, no C++ or torch types.  The
 * drop-in C++ headers include/cujson/cujson.h and include/cujson/cujsonlines.h
 * (which keep the reference's type layouts and function names) are thin
 * inline wrappers over these entry points; other languages bind them directly
 * (ctypes, cgo, JNI).
 *
 * Reference interfaces replaced (file:line within AutomataLab/cuJSON):
 *   cj_parse_standard  <- cuJSONResult parse_standard_json(cuJSONInput)
 *                         cujson/parse_standard_json.h:9, parse_standard_json.cu:1584
 *   cj_parse_lines     <- cuJSONResult parse_json_lines(cuJSONLinesInput)
 *                         cujson/parse_json_lines.h:9, parse_json_lines.cu:1092
 *   cj_result_free     <- cuJSONIterator::freeJson (cudaFreeHost of the result)
 *                         cujson/query/query_iterator_standard_json.cpp:143-146
 * Everything else here (contexts, staged device-resident runs, the generator)
 * has no counterpart in the reference, which has no library boundary at all.
 *
 * Result layout (identical to the reference's pinned result buffer,
 * cujson/parse_standard_json.cu:1659-1680): one pinned int32 buffer of
 * 2*(S+2) entries.  structural = buf; structural[0] = 0 (virtual root '['),
 * structural[1..S] = 1-based byte offsets of { } [ ] : , (and '\n' for JSON
 * Lines) outside strings, structural[S+1] = S+1 (virtual ']').
 * pair_pos = buf + S + 1; pair_pos[0] = S+1; for each open at structural index
 * i (1-based), pair_pos[i] = the structural index of its matching close.
 * Deliberate differences: pair_pos at non-open entries is 0 (the reference
 * leaves it uninitialised), the JSON-Lines virtual-root slots are written, and
 * errors return a status instead of calling exit(0).
 */
#ifndef CUJSON_GB300_H
#define CUJSON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CJ_ABI_VERSION 1

typedef enum cj_status {
    CJ_OK = 0,
    CJ_ERR_INVALID_ARGUMENT = 1,  /* null data, zero size, bad chunk table */
    CJ_ERR_INVALID_UTF8 = 2,      /* ill-formed UTF-8 (RFC 3629) */
    CJ_ERR_INVALID_BRACKETS = 3,  /* unbalanced or mismatched { } [ ] */
    CJ_ERR_TOO_LARGE = 4,         /* input does not fit int32 positions */
    CJ_ERR_OUT_OF_MEMORY = 5,
    CJ_ERR_CUDA = 6,              /* a CUDA runtime call failed */
    CJ_ERR_TIMEOUT = 7,           /* a bounded device-side wait expired */
    CJ_ERR_NO_DEVICE = 8,
    CJ_ERR_CAPACITY = 9,          /* caller-provided output buffer too small */
    CJ_ERR_NOT_STAGED = 10        /* cj_run_staged without a staged input */
} cj_status;

/* detail bits in cj_parse_info.error_flags */
#define CJ_FLAG_UTF8        0x01u
#define CJ_FLAG_BRACKETS    0x02u
#define CJ_FLAG_TIMEOUT     0x04u
#define CJ_FLAG_OVERFLOW    0x08u   /* an output index past its buffer (never with
                                       consistent counts; the write is dropped) */
/* with CJ_FLAG_TIMEOUT: bits 16-23 say which bounded wait of the scan expired
 * first (6: input bytes from the host, the only wait of the scan kernels) */
#define CJ_TIMEOUT_WAIT(flags) (((flags) >> 16) & 0xFFu)

/* Largest input in bytes: positions are int32 (reference, cujson_types.h:26). */
#define CJ_MAX_INPUT_BYTES 2147483646ull

typedef struct cj_parse_info {
    int64_t  n_structural;   /* S */
    int64_t  n_brackets;     /* opens + closes outside strings */
    int32_t  max_depth;      /* deepest nesting (the reference never sets it) */
    int32_t  status;         /* cj_status verdict */
    uint32_t error_flags;    /* CJ_FLAG_* */
    int32_t  n_segments;     /* 1, or the number of JSON-Lines chunks */
} cj_parse_info;

/* Result of cj_parse_standard / cj_parse_lines.  `structural` is a pinned
 * host allocation (cudaMallocHost) released by cj_result_free. */
typedef struct cj_result {
    int32_t* structural;
    int32_t* pair_pos;
    int64_t  n_structural;         /* S */
    int64_t  total;                /* S + 2 (cuJSONResult::totalResultSize) */
    int32_t  max_depth;
    int32_t  status;
    int64_t  n_segments;
    int64_t* segment_sizes;        /* malloc'd: S per JSON-Lines chunk */
} cj_result;

typedef struct cj_context cj_context;

/* ---- contexts -------------------------------------------------------------
 * A context owns one device, one non-blocking stream and a device arena that
 * grows to the largest input seen.  A context is not thread safe; use one per
 * host thread.  `device` < 0 means the current device. */
cj_status cj_context_create(int device, cj_context** out);
void      cj_context_destroy(cj_context* ctx);
/* Pre-size the arena for inputs up to `max_bytes` in up to `max_segments`
 * JSON-Lines chunks (avoids growth inside timed regions). */
cj_status cj_context_reserve(cj_context* ctx, size_t max_bytes, size_t max_segments);
void*     cj_context_stream(cj_context* ctx);           /* cudaStream_t */
int64_t   cj_context_launch_count(cj_context* ctx);     /* kernels launched so far */
size_t    cj_context_device_bytes(cj_context* ctx);     /* arena size */
size_t    cj_context_staged_bytes(cj_context* ctx);     /* input bytes of the staged input (0: none) */

/* Process-wide default context on the current device (used by the drop-in
 * C++ headers); created on first use. */
cj_context* cj_default_context(void);

/* ---- one-shot parses (drop-in semantics) ------------------------------------ */
cj_status cj_parse_standard(cj_context* ctx, const uint8_t* host_data, size_t size,
                            cj_result* out);
cj_status cj_parse_lines(cj_context* ctx, const uint8_t* const* chunks,
                         const size_t* chunk_sizes, size_t n_chunks, cj_result* out);
/* One-shot JSON-Lines parse of one host buffer, its chunks planned on the
 * device (no counterpart call in the reference: it replaces the host '\n'
 * scan of loadJSONLines_chunkCount / _chunkSizeBytes, cujson/load_file.cu:
 * 71-78 and :141-173, followed by parse_json_lines).  chunk_count != 0: the
 * plan of cj_plan_lines_count (newlines counted per 64 KiB block on the device
 * as each 128 MiB piece of the copy lands); else the plan of
 * cj_plan_lines_bytes with `chunk_bytes`.  The result, segment sizes
 * included, is that of planning the buffer on the host and calling
 * cj_parse_lines; a plan with an empty chunk is refused with
 * CJ_ERR_INVALID_ARGUMENT, as parse_json_lines refuses one. */
cj_status cj_parse_lines_planned(cj_context* ctx, const uint8_t* host_data, size_t size, size_t chunk_count,
                                 size_t chunk_bytes, cj_result* out);
void      cj_result_free(cj_result* res);

/* One-shot parse into a caller-provided host buffer (pinned for full speed)
 * of `out_cap` int32 entries, in the layout above; needs 2*(S+2) entries.
 * `lines_mode` != 0 treats the input as one JSON-Lines chunk.  (Replaces
 * parse_standard_json's H2D, stages and D2H, cujson/parse_standard_json.cu:
 * 1584-1687, into memory the caller owns.)  With pinned input and output and
 * an input of at least two streaming waves (cj_tuning.stream_wave_mib, 128 MiB
 * by default) the parse is streamed: the input's copy, the scan in waves and
 * the copy of each wave's positions back overlap, and the pair row follows
 * the pairing.  On a non-OK status host_out may hold part of a result. */
cj_status cj_parse_into(cj_context* ctx, const uint8_t* host_data, size_t size, int lines_mode,
                        int32_t* host_out, size_t out_cap, cj_parse_info* info);

/* ---- parse without allocating -----------------------------------------------
 * This entry point has no counterpart in the reference, which allocates
 * device memory on every call.  It exists for callers that may not allocate:
 * a host program that owns the device's memory and gives each library a fixed
 * budget, or a latency-critical loop in which the device-wide synchronisation
 * that cudaMalloc and cudaFree bring would stall its other streams.
 *
 * Parses one standard JSON document of `size` bytes that is already in device
 * memory (`d_data`) and writes the reference layout (2*(S+2) int32, as above)
 * into the caller's device buffer `d_out` of `out_cap` entries, on `stream`
 * (a cudaStream_t; NULL is the default stream) of the current device.  It
 * allocates nothing, on the device or the host: its scratch is a fixed
 * __device__ array of the library, sized for documents of at most
 * CJ_NOALLOC_MAX_BYTES (about 22 MiB of device memory).  Larger documents are
 * refused with CJ_ERR_TOO_LARGE; an `out_cap` under 2*(S+2) with
 * CJ_ERR_CAPACITY.  Returns once the parse has finished, with `info` filled
 * and the verdict as the status.  `d_out` is written only when the status is
 * CJ_OK: after an invalid document (CJ_ERR_INVALID_UTF8,
 * CJ_ERR_INVALID_BRACKETS, CJ_ERR_TIMEOUT) or a refusal it holds what it held
 * before the call.
 *
 * The first call on each device resolves the scratch address, sets up the
 * kernels and clears the scratch (waiting for the clear to finish); make that
 * first call before any stream capture.  All calls on one device share the
 * scratch: calls must not overlap -- two in flight at once, from two host
 * threads or on two streams without ordering between them, race on it. */
#define CJ_NOALLOC_MAX_BYTES 1048576ull
cj_status cj_parse_standard_noalloc(const uint8_t* d_data, size_t size, int32_t* d_out,
                                    size_t out_cap, cj_parse_info* info, void* stream);

/* ---- staged, device-resident runs -------------------------------------------
 * Stage copies the input into the context arena (synchronously); run launches
 * the parse kernels on the context stream without any host synchronisation;
 * info synchronises and reads the verdict and counts; copy_result writes the
 * reference layout into a host buffer.  Used for device-resident throughput. */
cj_status cj_stage_standard(cj_context* ctx, const uint8_t* host_data, size_t size);
cj_status cj_stage_lines(cj_context* ctx, const uint8_t* const* chunks,
                         const size_t* chunk_sizes, size_t n_chunks);
cj_status cj_run_staged(cj_context* ctx);
cj_status cj_staged_info(cj_context* ctx, cj_parse_info* info);
cj_status cj_copy_staged_result(cj_context* ctx, int32_t* host_out, size_t out_cap);
/* Device pointers of the staged run's outputs (valid until the next run):
 * positions[S] (1-based byte offsets) and pair_row[S] (pair_row[i] = 1-based
 * close index for opens, else 0). */
cj_status cj_staged_device_outputs(cj_context* ctx, const int32_t** d_positions,
                                   const int32_t** d_pair_row);

/* Replays the staged run as a CUDA graph: the first call after staging (or
 * after a tuning change) captures every memset and kernel of the run into a
 * graph; later calls launch that graph.  Results as cj_run_staged. */
cj_status cj_run_staged_graph(cj_context* ctx);

/* Failure-detection check (no reference counterpart): runs the staged input
 * while the device count of input bytes present stays at zero, so the scan's
 * bounded wait for input gives up after `polls` polls; the kernel
 * sets its timeout flag, finishes, and the context stays usable.  Returns the
 * run's verdict: CJ_ERR_TIMEOUT. */
cj_status cj_run_staged_starved(cj_context* ctx, uint32_t polls, cj_parse_info* info);

/* ---- queries on the device over a staged JSON-Lines result -------------------
 * The reference answers such queries on the host with its iterator, one record
 * at a time (cuJSONLinesIterator::checkKeyValue / findKey / getValue,
 * cujson/query/query_iterator.cpp:614, :447, :512; the loop of
 * real_world_use_case/main.cu:70-86, whose gotoNextSibling visits every '{'
 * that opens the result or follows a top-level ',' or newline).  Here the
 * device finds those records among the parse's bracket records (the level-0
 * brace opens) of the input last staged with cj_stage_lines (or parsed with
 * cj_parse_lines) and run, and applies the iterator's rules to each: the first
 * top-level member whose key equals `key` decides.
 * cj_query_count counts the records whose value for `key` is `value`
 * (checkKeyValue); cj_query_values returns, for every record that has `key`,
 * 3 int64 -- the record's byte offset, the value's byte offset and length as
 * getValue slices it -- in document order; with `out` NULL or `cap` 0 it only
 * counts them.  CJ_ERR_CAPACITY when more than `cap` records have the key:
 * `*n_records` is the full count and `out` holds `cap` of the triples (in
 * document order, not necessarily the first ones).  Keys and values are at
 * most 256 bytes; a result that is not valid returns its verdict. */
cj_status cj_query_count(cj_context* ctx, const char* key, size_t key_len, const char* value,
                         size_t value_len, int64_t* count);
cj_status cj_query_values(cj_context* ctx, const char* key, size_t key_len, int64_t* out, size_t cap,
                          int64_t* n_records);

/* ---- batches of independent documents ---------------------------------------
 * No counterpart in the reference, which parses one document per call
 * (parse_standard_json, cujson/parse_standard_json.cu:1584).  n_docs standard
 * documents are parsed by one run (one scan launch over all of them, then
 * the pairing and a layout kernel); each keeps its own string state, depth,
 * positions and verdict, exactly as if it had been parsed alone.
 *
 * cj_stage_batch copies each document (host pointers, pinned for speed);
 * cj_stage_batch_packed takes the documents back to back in one host buffer
 * and copies them with one transfer.  lines_mode != 0: every document is a
 * JSON-Lines buffer parsed as one chunk (as cj_parse_lines with one chunk).  Then cj_run_staged or
 * cj_run_staged_graph; then cj_batch_info (per document: status, S, depth,
 * and the offsets of each document's result in the batch layout, n_docs+1
 * entries in int32 units) and cj_copy_batch_result (every document's
 * 2*(S+2) reference layout, back to back, at those offsets).  A document
 * whose status is not CJ_OK has a layout of unspecified content. */
cj_status cj_stage_batch(cj_context* ctx, const uint8_t* const* docs, const size_t* sizes,
                         size_t n_docs, int lines_mode);
cj_status cj_stage_batch_packed(cj_context* ctx, const uint8_t* packed, const size_t* sizes,
                                size_t n_docs, int lines_mode);
/* A batch whose host buffer already has the device layout: document i at
 * offsets[i] from cj_batch_padded_offsets (1 KiB-aligned, back to back),
 * `*total` bytes in all.  cj_parse_batch_padded launches the run at once and
 * copies the buffer (pinned for the overlap) in chunks behind it: the scan
 * takes a region as soon as its bytes have arrived, so copy and parse overlap.
 * Results as after cj_run_staged (cj_batch_info, cj_copy_batch_result). */
cj_status cj_batch_padded_offsets(const size_t* sizes, size_t n_docs, size_t* offsets, size_t* total);
cj_status cj_parse_batch_padded(cj_context* ctx, const uint8_t* padded, const size_t* sizes, size_t n_docs,
                                int lines_mode);
cj_status cj_batch_info(cj_context* ctx, int32_t* status, int64_t* n_structural, int32_t* max_depth,
                        int64_t* layout_offsets, size_t n_docs);
cj_status cj_copy_batch_result(cj_context* ctx, int32_t* host_out, size_t out_cap);

/* ---- launch shapes and the autotuner ----------------------------------------
 * No counterpart in the reference (its launch shapes are constants).  The
 * scan cuts each document into regions of region_kib; the scan kernels run
 * scan_blocks_per_sm / emit_blocks_per_sm blocks per SM; the pairing kernels
 * pair_blocks blocks of pair_threads.  0 = default.  Setting a tuning on a
 * context with a staged input re-cuts that input into regions of the new
 * size.  cj_autotune_staged times `reps` graph replays of the staged input
 * for each candidate shape, keeps the fastest in the context and reports it
 * (and, optionally, every candidate tried with its mean milliseconds). */
typedef struct cj_tuning {
    int32_t region_kib;          /* bytes one warp scans as a unit: 4, 8 or 16 KiB (0: 16) */
    int32_t scan_blocks_per_sm;  /* resident 256-thread blocks per SM of the scan's table and */
    int32_t emit_blocks_per_sm;  /* emit kernels (0: as many as fit) */
    int32_t pair_blocks;         /* pairing grid (0: sized to the bracket count) */
    int32_t pair_threads;        /* pairing threads per block: 64, 128 or 256 (0: 256) */
    int32_t prefetch_steps;      /* how many 1 KiB steps ahead the scan asks for input to be
                                    brought into L2: 2..8 (0: 4); the staging depth */
    int32_t stream_wave_mib;     /* cj_parse_into of >= 2 waves of pinned input into pinned
                                    output: waves of this many MiB whose positions are copied
                                    back while later input arrives (0: 128; -1: not streamed) */
    float   ms;                  /* mean replay time when measured */
} cj_tuning;
cj_status cj_context_set_tuning(cj_context* ctx, const cj_tuning* tuning);   /* NULL: defaults */
cj_status cj_context_get_tuning(cj_context* ctx, cj_tuning* tuning);
cj_status cj_autotune_staged(cj_context* ctx, int32_t reps, cj_tuning* best, cj_tuning* tried,
                             size_t tried_cap, size_t* n_tried);
/* The context's tuning kept in a file of one JSON line per GPU name
 * ({"gpu": "<name>", "region_kib": .., ...}): cj_tuning_save writes (or
 * replaces) this GPU's line, cj_tuning_load applies it (CJ_ERR_INVALID_ARGUMENT
 * when the file has no line for this GPU; the tuning is then unchanged). */
cj_status cj_tuning_save(cj_context* ctx, const char* path);
cj_status cj_tuning_load(cj_context* ctx, const char* path);

/* ---- serving: a request loop with continuous batching -------------------------
 * No counterpart in the reference.  A server owns `slots` contexts on one
 * device and a scheduler thread.  Any host thread submits documents (standard
 * or JSON Lines, one chunk); the scheduler batches waiting requests of one
 * kind, oldest first, admitting them while a batch stays within
 * max_batch_docs and the slot's share of `memory_budget` (device bytes), and
 * keeps up to `slots` batches in flight so that the copies of one overlap
 * the kernels of another.  Requests that arrive meanwhile join the next batch
 * as soon as a slot frees up.  Each request is parsed as an independent
 * document: its result is the same alone and in any mix.  `data` must stay
 * valid (and unchanged) until the request has completed; pinned memory makes
 * its copy asynchronous.  A document too large for a slot's share of the
 * budget is refused at submission (CJ_ERR_TOO_LARGE). */
typedef struct cj_server cj_server;
typedef struct cj_server_config {
    int32_t  device;             /* -1: current device */
    uint32_t slots;              /* batches in flight, 1..8 (0: 2) */
    uint32_t max_batch_docs;     /* 0: 1024 */
    uint64_t memory_budget;      /* device bytes for requests in flight (0: 16 GiB) */
} cj_server_config;
typedef struct cj_server_stats {
    uint64_t batches, docs, bytes, max_batch_docs;
    uint64_t peak_admitted_bytes;   /* largest device-byte estimate admitted to one batch */
    uint64_t device_bytes;          /* arena bytes the slots hold now */
    int32_t  fault;                 /* first failure of a batch, or CJ_OK */
} cj_server_stats;
cj_status cj_server_create(const cj_server_config* cfg, cj_server** out);
void      cj_server_destroy(cj_server* s);   /* finishes the requests in flight first */
cj_status cj_server_submit(cj_server* s, const uint8_t* data, size_t size, int lines_mode,
                           uint64_t* ticket);
/* Waits for a request (timeout_ms < 0: no limit; CJ_ERR_TIMEOUT when it
 * expires); info->status is the request's verdict; latency_s the time from
 * submission to completion. */
cj_status cj_server_wait(cj_server* s, uint64_t ticket, int64_t timeout_ms, cj_parse_info* info,
                         double* latency_s);
/* Copies a completed request's reference layout (2*(S+2) int32; nothing for
 * an invalid document) and releases the request; returns its verdict. */
cj_status cj_server_take(cj_server* s, uint64_t ticket, int32_t* host_out, size_t out_cap);
cj_status cj_server_get_stats(cj_server* s, cj_server_stats* out);
/* Load generator: submits docs[i] at arrival_s[i] seconds after the call
 * (lines[i] != 0: JSON Lines; lines may be NULL), waits for all, and reports
 * each request's verdict and latency and the time until the last completion. */
cj_status cj_server_replay(cj_server* s, const uint8_t* const* docs, const size_t* sizes,
                           const int32_t* lines, const double* arrival_s, size_t n, int32_t* status,
                           double* latency_s, double* makespan_s);

/* ---- measurement and host memory --------------------------------------------
 * With timing enabled, every run records CUDA events on the context stream;
 * cj_context_phase_ms synchronises and returns the summed milliseconds of the
 * scan, pair and spine kernels over the runs recorded since timing was
 * (re-)enabled.  enable = 1: an event at every kernel boundary (each phase
 * timed, but a kernel then cannot be scheduled while the one before it
 * finishes); enable = 2: events only at the run's start, the scan's end and
 * the run's end -- the scan timed as it runs untimed; pair_ms is then pair +
 * spine and the scan's split reads as all tables; enable = 3: events only at
 * the run's start and end -- the whole run timed as it runs untimed (scan_ms
 * then covers the whole run). */
cj_status cj_context_timing(cj_context* ctx, int enable);
/* Dependent launches (default on): each kernel of a run after the first may
 * be scheduled while the one before it finishes, and waits on the device for
 * its results.  Its blocks then hold SM resources while they wait, which a
 * kernel of another stream sharing the GPU could have used; a context whose
 * stream shares the GPU with others' (the server's slots) may turn them off. */
cj_status cj_context_set_dependent_launch(cj_context* ctx, int enable);
cj_status cj_context_phase_ms(cj_context* ctx, double* scan_ms, double* pair_ms,
                              double* spine_ms, int64_t* runs);
/* The scan's own split over the same runs: its table kernel (one read of the
 * input), its prefix kernels and its emit kernel (positions and bracket
 * records); their sum is the scan time of cj_context_phase_ms. */
cj_status cj_context_scan_phase_ms(cj_context* ctx, double* tables_ms, double* prefix_ms,
                                   double* emit_ms, int64_t* runs);
/* Milliseconds from the first recorded run's start to the last one's end. */
cj_status cj_context_span_ms(cj_context* ctx, double* ms);
/* Pinned host memory for callers without the CUDA runtime headers.  Blocks
 * the library hands out (these, and the result buffers of cj_parse_standard /
 * cj_parse_lines) are kept when freed with cj_host_free / cj_result_free and
 * handed out again for a request of at least half their size, since pinning a
 * large buffer costs far more than filling it; up to 8 GiB is kept.
 * cj_host_pool_trim releases every kept block and returns their bytes.  A
 * block may also be released with cudaFreeHost. */
void* cj_host_alloc(size_t bytes);
void  cj_host_free(void* p);
size_t cj_host_pool_trim(void);

/* ---- value decoding ------------------------------------------------------------
 * No counterpart call in the reference, whose iterator hands out a value's raw
 * bytes (getValue, cujson/query/query_iterator.cpp:512).  cj_decode_values
 * decodes every scalar of the staged (not batch) result on the device: slot 0
 * is the text before the first structural, slot i (1..S) the text after
 * structural i up to the next one; each, less JSON whitespace at both ends, is
 * nothing, a string (unescaped to UTF-8), an integer that fits int64 (exact),
 * another number (the correctly rounded double, round-half-even, subnormals
 * and overflow to infinity included), true, false, null, or invalid.  Per slot:
 * type[i]; num[i] = the int64, the double's bits, or for a string the offset
 * of its decoded bytes in `strings`; len[i] = a string's decoded length.
 * `strings` has one byte per input byte (a string's decoded bytes start at its
 * content's logical offset).  The arrays stay on the device
 * (cj_values_device) until the next decode; cj_copy_values copies them out
 * (S + 1 slots; n_bytes string bytes). */
enum {
    CJ_VAL_NONE = 0, CJ_VAL_STRING = 1, CJ_VAL_INT = 2, CJ_VAL_DOUBLE = 3, CJ_VAL_TRUE = 4, CJ_VAL_FALSE = 5,
    CJ_VAL_NULL = 6, CJ_VAL_INVALID = 7, CJ_VAL_TYPES = 8
};
typedef struct cj_value_counts {
    int64_t n_slots;
    int64_t by_type[8];          /* slots of each CJ_VAL_* type */
} cj_value_counts;
cj_status cj_decode_values(cj_context* ctx, cj_value_counts* counts);
cj_status cj_values_device(cj_context* ctx, const uint8_t** type, const uint64_t** num, const uint32_t** len,
                           const uint8_t** strings);
cj_status cj_copy_values(cj_context* ctx, uint8_t* type, uint64_t* num, uint32_t* len, size_t slot_cap,
                         uint8_t* strings, size_t string_cap);

/* ---- loaders and JSON-Lines chunk planning ----------------------------------
 * cj_load_file reads a whole file into pinned host memory (free it with
 * cj_host_free or cudaFreeHost); replaces loadJSON, cujson/load_file.cu:7.
 * cj_plan_lines_count splits a buffer into `chunk_count` chunks of whole lines
 * (replaces loadJSONLines_chunkCount, cujson/load_file.cu:38);
 * cj_plan_lines_bytes closes a chunk before the line that would make it
 * exceed `chunk_bytes` (replaces loadJSONLines_chunkSizeBytes /
 * _chunkSizeMegaBytes, cujson/load_file.cu:109, :182).  With chunk_sizes ==
 * NULL it only counts the chunks. */
cj_status cj_load_file(const char* path, uint8_t** data, size_t* size);
cj_status cj_plan_lines_count(const uint8_t* data, size_t size, size_t chunk_count,
                              size_t* chunk_sizes);
cj_status cj_plan_lines_bytes(const uint8_t* data, size_t size, size_t chunk_bytes,
                              size_t* chunk_sizes, size_t cap, size_t* n_chunks);
/* cj_plan_lines_count_device: the plan of cj_plan_lines_count for a buffer
 * already in device memory (d_data, `size` bytes), computed on the device on
 * the context's stream -- newlines counted per 64 KiB block, then the one
 * newline that ends each chunk's last line located in its block; only the
 * block counts and one position per chunk cross to the host (chunk_sizes is
 * host memory of chunk_count entries).  `stream` (a cudaStream_t; NULL = the
 * legacy default stream) is the stream whose work fills d_data: the planner
 * reads d_data only after everything queued on it before this call, so a
 * buffer still being written by an asynchronous copy or kernel there is
 * planned correctly.  Returns after the plan is on the host.  Replaces the
 * host '\n' scan of loadJSONLines_chunkCount (cujson/load_file.cu:71-78) for
 * device-resident input; the chunk boundaries are the reference's
 * (tests/test_plan_golden.py). */
cj_status cj_plan_lines_count_device(cj_context* ctx, const uint8_t* d_data, size_t size,
                                     size_t chunk_count, size_t* chunk_sizes, void* stream);
/* cj_plan_lines_bytes_device: the plan of cj_plan_lines_bytes for a buffer
 * already in device memory, computed on the device (one warp walks the chunk
 * boundaries, reading backwards from each chunk start + chunk_bytes to the
 * newline that ends the chunk); arguments and results as cj_plan_lines_bytes,
 * `stream` as for cj_plan_lines_count_device.  Replaces the host '\n' scan of
 * loadJSONLines_chunkSizeBytes (cujson/load_file.cu:109-180) for
 * device-resident input. */
cj_status cj_plan_lines_bytes_device(cj_context* ctx, const uint8_t* d_data, size_t size, size_t chunk_bytes,
                                     size_t* chunk_sizes, size_t cap, size_t* n_chunks, void* stream);

const char* cj_status_string(int status);
/* Status of the calling thread's last drop-in parse (parse_standard_json /
 * parse_json_lines return an empty result on failure, as the reference's
 * callers expect). */
int cj_last_status(void);
void cj_set_last_status(int status);
/* The same as a message (cj_status_string(cj_last_status())): where the
 * reference printed a reason and called exit(0) (parse_standard_json.cu,
 * parse_json_lines.cu on invalid input), a caller reads it here. */
const char* cj_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
