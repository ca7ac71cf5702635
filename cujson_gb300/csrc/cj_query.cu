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
// Here the records come from the parse itself: the scan kernel leaves one
// bracket record per bracket (structural index, nesting level, open flag,
// brace or square) on the device, and the iterator's records are exactly the
// '{' opens at level 0 whose previous entry is a ',' or a newline entry (or
// that are entry 0) -- a separator just before a level-0 open is itself at
// level 0.  One persistent kernel, warp by warp: a warp reads a tile of 512
// bracket records coalesced, compacts the level-0 brace opens in shared
// memory, and each lane then checks a candidate's previous entry and queries
// the record with the iterator's rules, on 0-based byte offsets where a byte
// outside the file reads as 0:
//   key of the ':' at s:  from the first non-space after the previous
//       structural (a) to the last non-space before the ':' (b), the slice
//       [a+1, a+1+|b-a-1|) (getString, which drops one byte at each end);
//   value: for '{' / '[' after the ':' the container from its open to its
//       close; else from jumpValueForward(':') to jumpValueBackward(next
//       structural): spaces skipped, one quote dropped at each end;
//   slices clamp to the file, an empty or negative length is "".
// The first member whose key equals the query key decides (findKey).  The
// depth comes from the parse, so records that span lines are found exactly as
// the iterator's walk finds them.
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
    const uint2* brk;             // bracket records: x = structural index | kCurly, y = level << 1 | open
    uint32_t S;
    uint32_t K;                   // bracket records
    int64_t n_bytes;              // file length (all chunks)
    uint8_t key[kMaxQuery];
    uint8_t value[kMaxQuery];
    int key_len, value_len;       // value_len < 0: no value comparison (extract only)
    unsigned long long* count;    // [0] matches, [1] set on a malformed result, [2] tile ticket
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
constexpr int kQPerLane = 16;
constexpr int kQTile = 32 * kQPerLane;            // bracket records per warp tile
constexpr int kQStage = 32;                       // matches staged per warp tile (extract mode)

struct QueryShared {
    uint32_t recs[kQWarps][kQTile];               // candidate records: structural index of the '{'
    long long staged[kQWarps][3 * kQStage];       // extract mode: matches of the warp's tile
    uint32_t n_recs[kQWarps];
    uint32_t n_staged[kQWarps];
    uint32_t warp_sum[kQWarps];
};

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

// The level-0 '{' at entry u: a record if it is entry 0 or follows a ',' or a
// newline entry; query it.
__device__ __forceinline__ void query_candidate(const QueryParams& Q, QueryShared& sh, uint32_t w, uint32_t& mine,
                                                int64_t u)
{
    SegCursor cur;
    if (u > 0) {
        const uint8_t prev = entry(Q, cur, u - 1);
        if (prev != ',' && prev != '\n') return;
    }
    const int64_t c = (int64_t)__ldg(Q.pair + u) - 1;
    if (c <= u || c >= (int64_t)Q.S) {           // not a valid result
        atomicOr(Q.count + 1, 1ull);
        return;
    }
    long long vs, vl;
    if (query_record(Q, cur, u, c, vs, vl)) record_match(Q, sh, w, mine, (long long)__ldg(Q.pos + u) - 1, vs, vl);
}

__global__ void __launch_bounds__(kQThreads, 6) query_tiles(QueryParams Q)
{
    __shared__ QueryShared sh;
    const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint64_t gwarp = (uint64_t)blockIdx.x * kQWarps + w;
    const uint64_t n_warps = (uint64_t)gridDim.x * kQWarps;
    uint32_t mine = 0;
    const uint64_t n_tiles = ((uint64_t)Q.K + kQTile - 1) / kQTile;
    // the first tile of each warp by its index, the rest from a ticket counter,
    // so that warps with slow records take fewer tiles
    for (uint64_t tile = gwarp; tile < n_tiles;) {
        const uint64_t base = tile * kQTile;
        if (lane == 0) {
            sh.n_recs[w] = 0;
            sh.n_staged[w] = 0;
        }
        __syncwarp();
        // level-0 brace opens among the tile's bracket records
#pragma unroll 1
        for (int j0 = 0; j0 < kQPerLane; j0 += 8) {
            uint2 r[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const uint64_t t = base + (uint64_t)(j0 + j) * 32 + lane;
                r[j] = t < Q.K ? __ldg(Q.brk + t) : make_uint2(0u, 0u);
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const bool rec = (r[j].y == 1u) && (r[j].x & kCurly);       // open, level 0, brace
                const uint32_t m = __ballot_sync(0xffffffffu, rec);
                if (!m) continue;
                uint32_t b0 = 0;
                if (lane == 0) {
                    b0 = sh.n_recs[w];
                    sh.n_recs[w] = b0 + __popc(m);
                }
                b0 = __shfl_sync(0xffffffffu, b0, 0);
                if (rec) sh.recs[w][b0 + __popc(m & ((1u << lane) - 1))] = r[j].x & ~kCurly;
            }
        }
        __syncwarp();
        const uint32_t n = sh.n_recs[w];
        for (uint32_t k = lane; k < n; k += 32) query_candidate(Q, sh, w, mine, (int64_t)sh.recs[w][k]);
        if (Q.out) {
            __syncwarp();
            const uint32_t ns = min(sh.n_staged[w], (uint32_t)kQStage);
            unsigned long long slot = 0;
            if (lane == 0 && ns) slot = atomicAdd(Q.count, (unsigned long long)ns);
            slot = __shfl_sync(0xffffffffu, slot, 0);
            for (uint32_t k = lane; k < ns; k += 32) {
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
                         const int32_t* pair, const uint2* brk, uint32_t S, uint32_t K, const char* key,
                         int key_len, const char* value,
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
    Q.brk = brk;
    Q.S = S;
    Q.K = K;
    Q.n_bytes = n_bytes;
    for (int k = 0; k < key_len; k++) Q.key[k] = (uint8_t)key[k];
    for (int k = 0; k < value_len; k++) Q.value[k] = (uint8_t)value[k];
    Q.key_len = key_len;
    Q.value_len = value_len;
    Q.count = count;
    Q.out = out;
    Q.cap = cap;
    const uint64_t tiles = ((uint64_t)K + kQTile - 1) / kQTile;
    const uint64_t blocks = (tiles + kQWarps - 1) / kQWarps;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)sm_count * 6));
    query_tiles<<<grid, kQThreads, 0, stream>>>(Q);
    return cudaGetLastError();
}

}  // namespace cj
