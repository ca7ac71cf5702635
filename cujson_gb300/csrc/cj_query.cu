// cj_query.cu -- key/value queries over a staged JSON-Lines result, on the
// device.
//
// The reference answers queries on the host, one iterator step at a time
// (cujson/query/query_iterator.cpp: gotoArrayIndex :233, gotoNextSibling :370,
// findKey :447, getValue :512, checkKeyValue :614), e.g. counting the records
// whose "type" is "PushEvent" (real_world_use_case/main.cu:70-86).  The records
// that loop visits are the '{' entries that open the result (structural 0) or
// follow a top-level separator (a ',' entry, or a newline entry, which the
// iterator's getChar reports as ','); every other top-level item is skipped.
//
// Here one persistent kernel does it; each warp takes tiles of 1024 entries on
// its own (no block-wide barrier, so a slow record holds up only its warp).
// First the warp reads the tile's structural positions coalesced, eight
// independent loads per lane at a time, and compacts in shared memory every
// entry that starts a line (index 0, or the entry after a newline entry).
// Then each lane takes a line, walks its top-level items up to the next
// newline entry, jumping containers with the pair row, and queries each record
// it meets with the iterator's rules, on 0-based byte offsets where a byte
// outside the file reads as 0:
//   key of the ':' at s:  from the first non-space after the previous
//       structural (a) to the last non-space before the ':' (b), the slice
//       [a+1, a+1+|b-a-1|) (getString, which drops one byte at each end);
//   value: for '{' / '[' after the ':' the container from its open to its
//       close; else from jumpValueForward(':') to jumpValueBackward(next
//       structural): spaces skipped, one quote dropped at each end;
//   slices clamp to the file, an empty or negative length is "".
// The first member whose key equals the query key decides (findKey).
//
// A line whose walk meets a close bracket it did not open started inside a
// container: a record spans lines (not JSON Lines).  The iterator's walk jumps
// such records whole, which a line-parallel walk cannot follow, so the kernel
// raises a flag and the query is refused rather than answered differently.
#include <cuda_runtime.h>

#include <algorithm>

#include "cj_device.cuh"
#include "cj_kernels.h"

namespace cj {

namespace {

constexpr int kMaxQuery = 256;   // key and value bytes

struct QueryParams {
    const uint8_t* in;
    const Segment* segs;
    uint32_t n_segs;
    const int32_t* pos;
    const int32_t* pair;
    uint32_t S;
    int64_t n_bytes;              // file length (all chunks)
    uint8_t key[kMaxQuery];
    uint8_t value[kMaxQuery];
    int key_len, value_len;       // value_len < 0: no value comparison (extract only)
    unsigned long long* count;    // [0] matches, [1] set when a record spans lines, [2] tile ticket
    long long* out;               // 3 per match: record byte offset, value offset, value length
    unsigned long long cap;       // matches that fit `out`
};

// The segment that holds the last byte read: logical bytes [lo, hi) start at
// device address `base`.  Records and lines rarely cross a segment, so the
// table is searched only when a read leaves the current one.
struct SegCursor {
    int64_t lo = 0, hi = 0;
    const uint8_t* base = nullptr;
};

__device__ __forceinline__ void seek(const QueryParams& Q, SegCursor& c, int64_t b)
{
    uint32_t lo = 0, hi = Q.n_segs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((int64_t)__ldg(&Q.segs[mid].logical_off) <= b) lo = mid;
        else hi = mid;
    }
    const Segment* g = Q.segs + lo;
    c.lo = (int64_t)__ldg(&g->logical_off);
    c.hi = c.lo + (int64_t)__ldg(&g->len);
    c.base = Q.in + __ldg(&g->dev_off);
}

// byte at 0-based file offset b (0 outside the file)
__device__ __forceinline__ uint8_t at(const QueryParams& Q, SegCursor& c, int64_t b)
{
    if (b < 0 || b >= Q.n_bytes) return 0;
    if (b < c.lo || b >= c.hi) {
        seek(Q, c, b);
        if (b < c.lo || b >= c.hi) return 0;     // segments tile the file; never taken
    }
    return __ldg(c.base + (b - c.lo));
}

// the byte of structural entry i (0-based index into pos)
__device__ __forceinline__ uint8_t entry(const QueryParams& Q, SegCursor& c, int64_t i)
{
    return at(Q, c, (int64_t)__ldg(Q.pos + i) - 1);
}

// slice [start, start+len) clamped to the file, as the iterator's slice()
__device__ __forceinline__ void clamp_slice(const QueryParams& Q, int64_t& start, int64_t& len)
{
    if (len <= 0 || start < 0 || start >= Q.n_bytes) {
        len = 0;
        return;
    }
    if (start + len > Q.n_bytes) len = Q.n_bytes - start;
}

__device__ __forceinline__ bool equals(const QueryParams& Q, SegCursor& c, int64_t start, int64_t len,
                                       const uint8_t* want, int want_len)
{
    if (len != want_len) return false;
    for (int k = 0; k < want_len; k++)
        if (at(Q, c, start + k) != want[k]) return false;
    return true;
}

// Query the record whose '{' is entry r (its close at entry `close`): true
// when it matches, with the value's slice.
__device__ bool query_record(const QueryParams& Q, SegCursor& cur, int64_t r, int64_t close, long long& out_vs,
                             long long& out_vl)
{
    for (int64_t i = r + 1; i < close; i++) {
        const uint8_t b = entry(Q, cur, i);
        if (b == '}') break;
        if (b == '{' || b == '[') {
            const int64_t c = (int64_t)__ldg(Q.pair + i) - 1;
            if (c <= i) return false;
            i = c;                                  // the close; the loop steps past it
            continue;
        }
        if (b != ':') continue;
        // the key (getString)
        int64_t a = (int64_t)__ldg(Q.pos + i - 1);               // previous structural + 1
        while (at(Q, cur, a) == ' ') a++;
        int64_t e = (int64_t)__ldg(Q.pos + i) - 2;               // byte before the ':'
        while (e >= 0 && at(Q, cur, e) == ' ') e--;
        int64_t ks = a + 1, kl = e - a - 1;
        if (kl < 0) kl = -kl;
        clamp_slice(Q, ks, kl);
        if (!equals(Q, cur, ks, kl, Q.key, Q.key_len)) continue;
        // the value (getValue at the ':')
        const int64_t j = i + 1;
        const uint8_t bj = entry(Q, cur, j);
        int64_t vs, ve;
        if (bj == '{' || bj == '[') {
            vs = (int64_t)__ldg(Q.pos + j) - 1;
            ve = (int64_t)__ldg(Q.pos + (int64_t)__ldg(Q.pair + j) - 1) - 1;
        } else {
            vs = (int64_t)__ldg(Q.pos + i);                      // jumpValueForward
            for (;;) {
                const uint8_t ch = at(Q, cur, vs);
                if (ch == '"') { vs++; break; }
                if (ch != ' ') break;
                vs++;
            }
            ve = (int64_t)__ldg(Q.pos + j) - 2;                  // jumpValueBackward
            while (ve >= 0) {
                const uint8_t ch = at(Q, cur, ve);
                if (ch == '"') { ve--; break; }
                if (ch != ' ') break;
                ve--;
            }
        }
        int64_t vl = ve - vs + 1;
        clamp_slice(Q, vs, vl);
        if (Q.value_len >= 0 && !equals(Q, cur, vs, vl, Q.value, Q.value_len)) return false;
        out_vs = vs;
        out_vl = vl;
        return true;
    }
    return false;
}

}  // namespace

constexpr int kQThreads = 256;
constexpr int kQWarps = kQThreads / 32;
constexpr int kQPerLane = 32;
constexpr int kQTile = 32 * kQPerLane;            // structural entries per warp tile
constexpr int kQStage = 32;                       // matches staged per warp tile (extract mode)

struct QueryShared {
    uint16_t lines[kQWarps][kQTile];              // line starts, offsets in the warp's tile
    long long staged[kQWarps][3 * kQStage];       // extract mode: matches of the warp's tile
    uint32_t n_lines[kQWarps];
    uint32_t n_staged[kQWarps];
    uint32_t warp_sum[kQWarps];
};

// device address of the byte at 0-based file offset b (inside the file)
__device__ __forceinline__ const uint8_t* byte_ptr(const QueryParams& Q, SegCursor& c, int64_t b)
{
    if (b < c.lo || b >= c.hi) seek(Q, c, b);
    return c.base + (b - c.lo);
}

// A match: counted per lane (count mode), or staged in shared memory and
// written out once per warp tile (extract mode; a full stage falls back to a
// global slot per match).
__device__ __forceinline__ void record_match(const QueryParams& Q, QueryShared& sh, uint32_t w, uint32_t& mine,
                                             long long rec, long long vs, long long vl)
{
    if (!Q.out) {
        mine++;
        return;
    }
    const uint32_t k = atomicAdd(&sh.n_staged[w], 1u);
    if (k < (uint32_t)kQStage) {
        sh.staged[w][3 * k] = rec;
        sh.staged[w][3 * k + 1] = vs;
        sh.staged[w][3 * k + 2] = vl;
        return;
    }
    const unsigned long long m = atomicAdd(Q.count, 1ull);
    if (m < Q.cap) {
        Q.out[3 * m] = rec;
        Q.out[3 * m + 1] = vs;
        Q.out[3 * m + 2] = vl;
    }
}

// Walk the line that starts at entry t: query every record that opens it or
// follows a top-level ','.
__device__ void walk_line(const QueryParams& Q, QueryShared& sh, uint32_t w, uint32_t& mine, int64_t t)
{
    SegCursor cur;
    bool item_start = true;
    for (int64_t u = t; u < (int64_t)Q.S; u++) {
        const uint8_t b = entry(Q, cur, u);
        if (b == '\n') break;
        if (b == '}' || b == ']') {                // closes what this line did not open
            atomicOr(Q.count + 1, 1ull);
            break;
        }
        if (b == '{' || b == '[') {
            const int64_t c = (int64_t)__ldg(Q.pair + u) - 1;
            if (c <= u || c >= (int64_t)Q.S) {       // not a valid result
                atomicOr(Q.count + 1, 2ull);
                break;
            }
            if (b == '{' && item_start) {
                long long vs, vl;
                if (query_record(Q, cur, u, c, vs, vl))
                    record_match(Q, sh, w, mine, (long long)__ldg(Q.pos + u) - 1, vs, vl);
            }
            u = c;
            item_start = false;
            continue;
        }
        item_start = b == ',';
    }
}

__global__ void __launch_bounds__(kQThreads, 6) query_tiles(QueryParams Q)
{
    __shared__ QueryShared sh;
    const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint64_t gwarp = (uint64_t)blockIdx.x * kQWarps + w;
    const uint64_t n_warps = (uint64_t)gridDim.x * kQWarps;
    uint32_t mine = 0;
    SegCursor cur;
    const uint64_t n_tiles = ((uint64_t)Q.S + kQTile - 1) / kQTile;
    // the first tile of each warp by its index, the rest from a ticket counter,
    // so that warps with slow records take fewer tiles
    for (uint64_t tile = gwarp; tile < n_tiles;) {
        const int64_t base = (int64_t)tile * kQTile;
        if (lane == 0) {
            sh.n_lines[w] = base == 0 ? 1u : 0u;   // entry 0 starts the first line
            sh.lines[w][0] = 0;
            sh.n_staged[w] = 0;
        }
        __syncwarp();
        // entries t in [base-1, base+kQTile-1): a newline at t starts a line at t+1
#pragma unroll 1
        for (int j0 = 0; j0 < kQPerLane; j0 += 8) {
            int32_t p[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int64_t t = base - 1 + (int64_t)(j0 + j) * 32 + lane;
                p[j] = (t >= 0 && t + 1 < (int64_t)Q.S) ? __ldg(Q.pos + t) : 0;
            }
            const uint8_t* a[8];
#pragma unroll
            for (int j = 0; j < 8; j++) a[j] = p[j] > 0 ? byte_ptr(Q, cur, (int64_t)p[j] - 1) : nullptr;
            uint8_t b[8];
#pragma unroll
            for (int j = 0; j < 8; j++) b[j] = a[j] ? __ldg(a[j]) : 0;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const bool nl = b[j] == '\n';
                const uint32_t m = __ballot_sync(0xffffffffu, nl);
                if (!m) continue;
                uint32_t b0 = 0;
                if (lane == 0) {
                    b0 = sh.n_lines[w];
                    sh.n_lines[w] = b0 + __popc(m);
                }
                b0 = __shfl_sync(0xffffffffu, b0, 0);
                if (nl) sh.lines[w][b0 + __popc(m & ((1u << lane) - 1))] = (uint16_t)((j0 + j) * 32 + lane);
            }
        }
        __syncwarp();
        const uint32_t n_lines = sh.n_lines[w];
        for (uint32_t k = lane; k < n_lines; k += 32) walk_line(Q, sh, w, mine, base + sh.lines[w][k]);
        if (Q.out) {
            __syncwarp();
            const uint32_t n = min(sh.n_staged[w], (uint32_t)kQStage);
            unsigned long long slot = 0;
            if (lane == 0 && n) slot = atomicAdd(Q.count, (unsigned long long)n);
            slot = __shfl_sync(0xffffffffu, slot, 0);
            for (uint32_t k = lane; k < n; k += 32) {
                const unsigned long long m = slot + k;
                if (m < Q.cap) {
                    Q.out[3 * m] = sh.staged[w][3 * k];
                    Q.out[3 * m + 1] = sh.staged[w][3 * k + 1];
                    Q.out[3 * m + 2] = sh.staged[w][3 * k + 2];
                }
            }
        }
        __syncwarp();
        unsigned long long next = 0;
        if (lane == 0) next = n_warps + atomicAdd(Q.count + 2, 1ull);
        tile = __shfl_sync(0xffffffffu, next, 0);
    }
    if (!Q.out) {
        // one count per block
        uint32_t v = mine;
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh.warp_sum[w] = v;
        __syncthreads();
        if (tid == 0) {
            unsigned long long total = 0;
            for (int i = 0; i < kQWarps; i++) total += sh.warp_sum[i];
            if (total) atomicAdd(Q.count, total);
        }
    }
}

cudaError_t launch_query(const uint8_t* in, const Segment* segs, uint32_t n_segs, const int32_t* pos,
                         const int32_t* pair, uint32_t S, const char* key, int key_len, const char* value,
                         int value_len, int64_t n_bytes, unsigned long long* count, long long* out,
                         unsigned long long cap, int sm_count, cudaStream_t stream)
{
    if (key_len < 0 || key_len > kMaxQuery || value_len > kMaxQuery) return cudaErrorInvalidValue;
    QueryParams Q{};
    Q.in = in;
    Q.segs = segs;
    Q.n_segs = n_segs;
    Q.pos = pos;
    Q.pair = pair;
    Q.S = S;
    Q.n_bytes = n_bytes;
    for (int k = 0; k < key_len; k++) Q.key[k] = (uint8_t)key[k];
    for (int k = 0; k < value_len; k++) Q.value[k] = (uint8_t)value[k];
    Q.key_len = key_len;
    Q.value_len = value_len;
    Q.count = count;
    Q.out = out;
    Q.cap = cap;
    const uint64_t tiles = ((uint64_t)S + kQTile - 1) / kQTile;
    const uint64_t blocks = (tiles + kQWarps - 1) / kQWarps;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)sm_count * 8));
    query_tiles<<<grid, kQThreads, 0, stream>>>(Q);
    return cudaGetLastError();
}

}  // namespace cj
