// cj_kernels.h -- kernel parameter blocks and launchers (host and device).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cj_device.cuh"

namespace cj {

struct ScanParams {
    const uint8_t* in;
    const Segment* segs;
    const uint32_t* tile_seg;   // tile -> segment (nullptr: one segment)
    uint32_t n_segs;
    uint32_t n_tiles;
    int32_t* pos;
    int32_t* pair;
    uint2* brk;
    uint32_t* desc_flag;
    uint4* desc_agg;            // 4 entries per tile (tiles of kTileBytes)
    uint4* desc_incl;           // 1 entry per tile
    Ctrl* ctrl;
    SegmentOut* seg_out;
    uint32_t epoch;
};

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
};

void launch_scan(const ScanParams& p, bool lines, int grid, cudaStream_t stream);
cudaError_t scan_configure();      // opt in to the scan kernel's dynamic shared memory
size_t scan_smem_bytes();
const void* scan_kernel_ptr();     // for occupancy queries
void launch_pair(const PairParams& p, int grid, cudaStream_t stream);
void launch_spine(const PairParams& p, int grid, cudaStream_t stream);

}  // namespace cj
