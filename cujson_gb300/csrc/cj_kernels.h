// cj_kernels.h -- kernel parameter blocks and launchers (host and device).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cj_device.cuh"

namespace cj {

// Programmatic dependent launch.  A kernel launched by launch_dependent may
// be scheduled while the kernel before it on the stream is still running; it
// calls wait_previous_grid() before touching anything that kernel wrote (the
// wait returns once that grid has completed and its writes are visible; for
// a plain launch it returns at once).  allow_next_grid() lets the next
// kernel's blocks be scheduled as soon as every block of this grid has
// started; without it they are scheduled as this grid's blocks exit.
__device__ __forceinline__ void wait_previous_grid()
{
#ifdef __CUDA_ARCH__
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
__device__ __forceinline__ void allow_next_grid()
{
#ifdef __CUDA_ARCH__
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}
// whether launch_dependent sets the attribute (CJ_PDL=0 in the environment
// turns it off, for comparison)
bool dependent_launch_enabled();
#ifndef CJ_EMU
// (dep false: a plain launch -- for a context whose stream shares the GPU with
// others, where a dependent kernel waiting on its SMs would hold resources
// another stream's kernels could use)
template <typename... Params, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(Params...), int grid, int block, size_t smem,
                                    cudaStream_t stream, bool dep, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (dep && dependent_launch_enabled()) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}
#endif

struct ScanParams {
    const uint8_t* in;
    const Segment* segs;
    const uint32_t* region_seg; // region -> segment (nullptr: one segment)
    uint32_t n_segs;
    uint32_t n_regions;
    int32_t* pos;
    int32_t* pair;
    uint2* brk;
    uint64_t out_cap;           // entries of pos and pair
    uint64_t brk_cap;           // entries of brk
    uint4* rtab;                // 4 entries per region: transfer tables
    uint4* bagg;                // 4 per block of kPrefixPerBlock regions: block tables
    uint4* masks;               // per region and step, 32 lanes: the 4 mask words of the steps
                                // that hold structural characters (masks_cap(...) entries)
    uint4* work;                // 2 per region with structurals to emit (ctrl->n_work of them):
                                // {region, stored steps | flip << 31, s, k}, {depth, end s, end k, end depth}
    Ctrl* ctrl;
    SegmentOut* seg_out;
    uint32_t* seg_err;          // per-segment verdict bits (independent documents),
                                // nullptr: verdicts go to ctrl->error_flags
    // Bytes of the input layout (`in`, from its start) already in device
    // memory, raised by the host's copies while the scan runs; a region is
    // scanned once its bytes are there.  nullptr: all input is present.
    const unsigned long long* ready;
    uint32_t input_wait_limit;  // polls before a wait for input gives up (0: default)
    int region_steps;           // 1 KiB steps per region: 4, 8 or 16
    int sm_count;
    uint32_t prefetch_steps;    // the table kernel's L2 prefetch distance in steps (0: 4)
    uint32_t dependent_launch;  // nonzero: the kernels after the first are dependent launches
    // A wave: the launch scans regions [r_begin, r_end) only (r_end 0: all),
    // starting from the value in carry_in (nullptr: the document start) and
    // leaving the value after r_end - 1 in carry_out (nullptr: not kept);
    // its work items are counted in n_work (nullptr: ctrl->n_work).  The end
    // value also goes to carry_host (nullptr: not), a device-visible pointer
    // into pinned host memory, so that the host reads it once the wave's
    // kernels are done without a copy between them on the stream.
    uint32_t r_begin, r_end;
    const uint4* carry_in;
    uint4* carry_out;
    uint4* carry_host;
    uint32_t* n_work;
    // the table and emit kernels' ticket counters, zero at launch (nullptr:
    // ctrl->tables_ticket and ctrl->emit_ticket); a wave has its own pair
    uint32_t* tickets;
};

// Launch shape of the scan kernels (0 = as many blocks as fit).
struct ScanShape {
    int tables_blocks_per_sm;
    int emit_blocks_per_sm;
};

// scratch sizes of one scan over `n_regions` regions
inline uint64_t prefix_blocks(uint64_t n_regions) { return (n_regions + kPrefixPerBlock - 1) / kPrefixPerBlock; }
// mask entries (uint4) for `bytes` of input in `segs` segments, any region size
inline uint64_t masks_cap(uint64_t bytes, uint64_t segs) { return (bytes / 1024 + (segs + 1) * 16) * 32; }

struct PairParams {
    const uint2* brk;
    int32_t* pair;
    uint32_t* spine;                      // per chunk, kChunk slots: unmatched closes
                                          // from the front, unmatched opens from the back
    int4* cinfo;                          // per chunk: entry depth, min depth, exit depth
    unsigned long long* tree;             // min-tree levels 1..kTreeLevels
    uint64_t tree_off[kTreeLevels + 1];   // start of each level in `tree`
    Ctrl* ctrl;
    uint32_t epoch;
    uint32_t chunk_cap;
    // Independent documents (batch): each document's bracket records start on
    // a chunk boundary at its segment's brk_base, so a chunk never holds two
    // documents; the record count of a segment is its seg_out[].k_end.  Only
    // chunks that hold records are work items: rchunk_off[d] is the number of
    // such chunks before document d (n_bsegs + 1 entries).  Chunks without
    // records keep the cinfo fill kNoLevel.  Verdicts and depths go per segment.
    // rchunk_off == nullptr: one record sequence of ctrl->k_total records.
    const uint64_t* rchunk_off;
    uint32_t n_bsegs;
    const Segment* segs;
    const SegmentOut* seg_out;
    uint32_t* seg_err;
    int32_t* seg_depth;
    uint64_t n_chunks;                    // size of the batch's chunk index space
    uint32_t dependent_launch;            // nonzero: both kernels are dependent launches
};

// cinfo fill of a batch chunk without records (bytes 0x7F): above every level
constexpr int32_t kNoLevel = 0x7F7F7F7F;

// tables, (block reduce,) apply, emit: scan_launches(n) kernels on `stream`
// `ev` (optional): 3 events recorded after the table, prefix and emit kernels
void launch_scan(const ScanParams& p, bool lines, const ScanShape& shape, cudaStream_t stream,
                 cudaEvent_t* ev = nullptr);
int scan_launches(uint32_t n_regions);
bool region_steps_valid(int r);
void launch_pair(const PairParams& p, int grid, cudaStream_t stream, int threads = 256);
void launch_spine(const PairParams& p, int grid, cudaStream_t stream, int threads = 256);

// Load the kernels of a file now (cudaFuncGetAttributes on each).  With lazy
// module loading a kernel is loaded at its first launch, and that load can
// wait for the kernels already running; an overlapped run queues kernels
// behind a scan that waits for input bytes the host has not yet queued, so
// every kernel such a run launches must be loaded before its first one.
cudaError_t preload_scan_kernels();
cudaError_t preload_pair_kernels();
cudaError_t preload_batch_kernels();

// value decoding over a staged result (cj_values.cu): per slot (the text
// before the first structural, and after each), a type, an int64 / double /
// decoded-string offset, and a decoded string length
enum : uint8_t {
    kValNone = 0, kValString = 1, kValInt = 2, kValDouble = 3, kValTrue = 4, kValFalse = 5, kValNull = 6,
    kValInvalid = 7,
    kValDeferred = 8               // internal: a number for the exact decimal conversion
};
constexpr int kValTypes = 8;
struct ValueParams {
    const uint8_t* in;
    const Segment* segs;
    uint32_t n_segs;
    const int32_t* pos;            // the staged result's positions (1-based, logical)
    uint32_t S;
    uint64_t n_bytes;              // logical input bytes
    uint8_t* type;                 // S + 1 slots
    uint64_t* num;                 // int64 / double bits / decoded string's offset in str_out
    uint32_t* len;                 // decoded string length
    uint8_t* str_out;              // n_bytes: decoded strings at their content offsets
    uint32_t* long_list;           // slots longer than the first kernel takes, for the second
    uint32_t long_cap;
    uint32_t* short_list;          // escaped strings and numbers for the exact conversion, likewise
    uint32_t short_cap;
    uint32_t* counters;            // entries wanted in each list, then the short list's ticket
    unsigned long long* counts;    // kValTypes
    const uint64_t* pow5;          // kPow5Table on the device
    uint32_t dependent_launch;     // nonzero: the kernels after the first are dependent launches
};
cudaError_t launch_decode_values(const ValueParams& p, int sm_count, cudaStream_t stream);
cudaError_t preload_value_kernels();
extern const uint64_t kPow5Table[2 * 651];

// key/value queries over a staged JSON-Lines result (cj_query.cu)
// JSON-Lines chunk plan of a device buffer (cj_plan.cu); scratch: nb =
// ceil(size / 64 KiB) counts, chunk_count + 1 requests and positions
cudaError_t plan_lines_count_device(const uint8_t* d_data, size_t size, size_t chunk_count,
                                    size_t* chunk_sizes, uint32_t* d_counts, uint2* d_req,
                                    unsigned long long* d_pos, cudaStream_t stream);
// the same in two parts: newlines per 64 KiB block of d_data (the counts of a
// sub-range starting on a block boundary go to its blocks' slots), then, with
// the counts and the buffer's last byte on the host, the chunk sizes
void launch_plan_count(const uint8_t* d_data, size_t size, uint32_t* d_counts, cudaStream_t stream);
cudaError_t plan_lines_count_finish(const uint8_t* d_data, size_t size, size_t chunk_count, size_t* chunk_sizes,
                                    const uint32_t* counts, uint8_t last, uint2* d_req, unsigned long long* d_pos,
                                    cudaStream_t stream);
constexpr uint64_t kPlanBlockBytes = 65536;
// JSON-Lines byte-limit plan of a device buffer (cj_plan.cu); scratch: cap
// boundaries and 2 counters.  Sizes are written only when they fit in cap.
cudaError_t plan_lines_bytes_device(const uint8_t* d_data, size_t size, size_t chunk_bytes, size_t* chunk_sizes,
                                    size_t cap, size_t* n_chunks, unsigned long long* d_bounds,
                                    unsigned long long* d_count, cudaStream_t stream);

cudaError_t launch_query(const uint8_t* in, const Segment* segs, uint32_t n_segs, const int32_t* pos,
                         const int32_t* pair, const uint2* brk, uint32_t S, uint32_t K, const char* key,
                         int key_len, const char* value, int value_len, int64_t n_bytes, unsigned long long* count,
                         long long* out, unsigned long long cap, int sm_count, cudaStream_t stream);

// batches of independent documents (cj_batch.cu)
void launch_batch_scatter(const uint8_t* packed, const uint64_t* src_off, const uint64_t* word_off,
                          const Segment* segs, uint32_t n, uint64_t total_words, uint8_t* in, int sm_count,
                          cudaStream_t stream);
void launch_batch_prefix(const Segment* segs, const SegmentOut* seg_out, uint32_t n, uint64_t* layout_off,
                         uint64_t* rchunk_off, cudaStream_t stream, bool dep);
void launch_batch_layout(const Segment* segs, const SegmentOut* seg_out, uint32_t n, const int32_t* pos,
                         const int32_t* pair, const uint64_t* off, int32_t* layout, int sm_count,
                         cudaStream_t stream, bool dep);

}  // namespace cj
