// ORDER BY on the device: a stable least-significant-digit radix sort of row
// ids by a list of keys (int32 or uint64 columns, ascending or descending).
//
// The reference executor treats SORT as a pass-through (executor/
// ddor_executor.cpp:209-211); its unused host routine sort_table
// (kernels/sort.hpp:7-103) orders rows by the collation keys with std::sort,
// int32 keys compared as signed, aggregate (uint64) keys as unsigned.  This
// sort orders by the same comparisons; ties keep row order (stable), which
// std::sort does not promise.
//
// Each key becomes one or two 32-bit words whose unsigned order is the key's
// order: an int32 with its sign bit flipped, a uint64 as its low then its high
// word, and every bit inverted for a descending key.  Words are sorted from
// the last key's low word to the first key's high word.  Each word is
// gathered once through the current order into a word array, then sorted 8
// bits per pass with (word, row id) pairs carried along, each pass a stable
// counting sort of 4096-row tiles (256 threads x 16 rows, row j * 256 + t of
// a tile in thread t): per tile digit counts (digit-major, so that one
// exclusive scan gives every tile's first slot per digit), the scan, then a
// scatter that walks the tile's 16 rows of 256 in order -- a row's place among
// equal digits comes from the rows of earlier steps (a running count per
// digit), of earlier warps in this step (per-warp counts) and of lower lanes
// of its own warp (a warp match).
#include <algorithm>
#include <cstdint>
#include <utility>

#include "common.cuh"

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;                          // rows per thread
constexpr int kSortTile = kSortThreads * kSortItems;    // rows per block
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kScanThreads = 1024;

struct SortPass {
    const void *col;  // key column
    int wide;         // 1: uint64 column
    int hi;           // uint64: high word
    int desc;
};

__device__ __forceinline__ uint32_t key_word(const SortPass &p, uint32_t row)
{
    uint32_t w;
    if (p.wide) {
        const uint64_t v = static_cast<const uint64_t *>(p.col)[row];
        w = p.hi ? (uint32_t)(v >> 32) : (uint32_t)v;
    } else {
        w = (uint32_t)static_cast<const int32_t *>(p.col)[row] ^ 0x80000000u;
    }
    return p.desc ? ~w : w;
}

// word[i] = the pass's key word of row perm[i] (one gather per word).
__global__ void k_gather_word(const SortPass p, const uint32_t *__restrict__ perm, uint32_t n,
                              uint32_t *__restrict__ word)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        word[i] = key_word(p, perm[i]);
}

__global__ void __launch_bounds__(kSortThreads) k_radix_count(const uint32_t *__restrict__ word, int shift,
                                                                 uint32_t n, uint32_t *__restrict__ hist, uint32_t nb)
{
    __shared__ uint32_t cnt[kSortWarps][256];
    const uint32_t warp = threadIdx.x >> 5;
    for (uint32_t k = threadIdx.x; k < kSortWarps * 256; k += kSortThreads) (&cnt[0][0])[k] = 0;
    __syncthreads();
    const uint32_t tile = blockIdx.x * (uint32_t)kSortTile;
#pragma unroll 4
    for (int j = 0; j < kSortItems; j++) {
        const uint32_t i = tile + (uint32_t)j * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[warp][(word[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) t += cnt[w][threadIdx.x];
    hist[threadIdx.x * nb + blockIdx.x] = t;
}

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp, uint32_t &total);

// Moves the (word, row id) pairs of one tile to their slots of this digit
// pass, stably.  Warp w owns the tile's rows [512 w, 512 w + 512) and ranks
// them on its own in 16 steps of 32 (a warp match gives the lanes of one
// digit; a per-warp count per digit carries the earlier steps), with no block
// barrier.  Then per digit the counts of earlier warps and of smaller digits
// give each row its place in the tile order; the tile is ordered in shared
// memory and goes out in runs of equal digits, so consecutive threads write
// consecutive slots.
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint32_t *__restrict__ word,
                                                                   const uint32_t *__restrict__ perm, int shift,
                                                                   uint32_t n, const uint32_t *__restrict__ offs,
                                                                   uint32_t nb, uint32_t *__restrict__ word_out,
                                                                   uint32_t *__restrict__ perm_out)
{
    constexpr uint32_t kWarpRows = 32 * kSortItems;
    __shared__ uint32_t s_w[kSortTile], s_r[kSortTile];
    __shared__ uint32_t wc[kSortWarps][256];  // per warp and digit: count, then the earlier warps' count
    __shared__ uint32_t first[256], tpre[256], s_warp[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t tile = blockIdx.x * (uint32_t)kSortTile;
    const uint32_t rows = min((uint32_t)kSortTile, n - tile);
    for (uint32_t k = threadIdx.x; k < kSortWarps * 256; k += kSortThreads) (&wc[0][0])[k] = 0;
    first[threadIdx.x] = offs[threadIdx.x * nb + blockIdx.x];
    __syncthreads();
    uint32_t w[kSortItems], r[kSortItems], rank[kSortItems];
    const uint32_t base = warp * kWarpRows;
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        const uint32_t k = base + (uint32_t)j * 32 + lane;
        const bool valid = k < rows;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        rank[j] = 0xFFFFFFFFu;
        if (vmask == 0) continue;  // warp-uniform
        if (valid) {
            w[j] = word[tile + k];
            r[j] = perm[tile + k];
            const uint32_t d = (w[j] >> shift) & 255u;
            const unsigned peers = __match_any_sync(vmask, d);
            const uint32_t below = __popc(peers & ((1u << lane) - 1u));
            rank[j] = wc[warp][d] + below;
            __syncwarp(vmask);
            if (below == 0) wc[warp][d] += __popc(peers);  // the group's lowest lane
        }
        __syncwarp();
    }
    __syncthreads();
    // per digit: earlier warps' counts (in place) and the tile's count
    uint32_t cnt = 0;
#pragma unroll
    for (int q = 0; q < kSortWarps; q++) {
        const uint32_t c = wc[q][threadIdx.x];
        wc[q][threadIdx.x] = cnt;
        cnt += c;
    }
    uint32_t total;
    tpre[threadIdx.x] = block_exclusive_scan(cnt, s_warp, total);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        if (rank[j] == 0xFFFFFFFFu) continue;
        const uint32_t d = (w[j] >> shift) & 255u;
        const uint32_t at = tpre[d] + wc[warp][d] + rank[j];
        s_w[at] = w[j];
        s_r[at] = r[j];
    }
    __syncthreads();
    // out in tile order: slot p of digit d goes to first[d] + (p - tpre[d])
    for (uint32_t p = threadIdx.x; p < rows; p += kSortThreads) {
        const uint32_t x = s_w[p];
        const uint32_t d = (x >> shift) & 255u;
        const uint32_t at = first[d] + (p - tpre[d]);
        word_out[at] = x;
        perm_out[at] = s_r[p];
    }
}

__global__ void k_iota(uint32_t *perm, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) perm[i] = i;
}

// Exclusive scan of m counts in three steps: blocks of 1024 in place (block
// sums aside), the block sums, then the sums added back.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp, uint32_t &total)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < blockDim.x / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[blockDim.x / 32 - 1];
    const uint32_t r = x - v + (warp ? s_warp[warp - 1] : 0);
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_local(uint32_t *a, uint32_t m, uint32_t *sums)
{
    __shared__ uint32_t s_warp[32];
    const uint32_t i = blockIdx.x * kScanThreads + threadIdx.x;
    const uint32_t v = i < m ? a[i] : 0;
    uint32_t total;
    const uint32_t r = block_exclusive_scan(v, s_warp, total);
    if (i < m) a[i] = r;
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t *sums, uint32_t k)
{
    __shared__ uint32_t s_warp[32];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < k; base += kScanThreads) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < k ? sums[i] : 0;
        uint32_t total;
        const uint32_t r = block_exclusive_scan(v, s_warp, total);
        if (i < k) sums[i] = r + carry;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(uint32_t *a, uint32_t m, const uint32_t *sums)
{
    const uint32_t i = blockIdx.x * kScanThreads + threadIdx.x;
    if (i < m) a[i] += sums[blockIdx.x];
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Scratch {
    uint32_t *perm_b, *word_a, *word_b, *hist, *sums;
};

size_t scratch_layout(uint64_t n, char *base, Scratch *s)
{
    const uint64_t nb = (n + kSortTile - 1) / kSortTile;
    const uint64_t m = nb * 256;
    const uint64_t nsum = (m + kScanThreads - 1) / kScanThreads;
    size_t off = 0;
    auto take = [&](uint64_t bytes) {
        char *p = base ? base + off : nullptr;
        off += align256(bytes);
        return reinterpret_cast<uint32_t *>(p);
    };
    Scratch t;
    t.perm_b = take(std::max<uint64_t>(n, 1) * 4);
    t.word_a = take(std::max<uint64_t>(n, 1) * 4);
    t.word_b = take(std::max<uint64_t>(n, 1) * 4);
    t.hist = take(std::max<uint64_t>(m, 1) * 4);
    t.sums = take(std::max<uint64_t>(nsum, 1) * 4);
    if (s) *s = t;
    return off;
}

}  // namespace

extern "C" {

size_t sdb_sort_scratch_bytes(uint64_t n) { return scratch_layout(n, nullptr, nullptr); }

int sdb_sort_rows(const void *const *keys, const int *key_types, const int *descending, int nkeys, uint64_t n,
                  uint32_t *perm, void *scratch, size_t scratch_bytes, sdb_stream_t stream)
{
    if (nkeys < 1 || nkeys > 16 || !keys || !key_types || !descending)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_sort_rows: 1..16 keys with types and directions");
    if (n > (1ull << 31)) return sdb_set_error(SDB_ERR_INVALID, "sdb_sort_rows: at most 2^31 rows");
    if (n == 0) return SDB_OK;
    if (!perm || !sdb::aligned(perm, 4)) return sdb_set_error(SDB_ERR_INVALID, "sdb_sort_rows: perm NULL or misaligned");
    const size_t need = scratch_layout(n, nullptr, nullptr);
    if (!scratch || scratch_bytes < need || !sdb::aligned(scratch, 256))
        return sdb_set_error(SDB_ERR_INVALID, "sdb_sort_rows: scratch of %zu bytes (256-byte aligned) needed", need);
    for (int k = 0; k < nkeys; k++) {
        if (key_types[k] != 0 && key_types[k] != 1)
            return sdb_set_error(SDB_ERR_INVALID, "sdb_sort_rows: key type %d (0 int32, 1 uint64)", key_types[k]);
        if (!keys[k] || !sdb::aligned(keys[k], key_types[k] ? 8 : 4))
            return sdb_set_error(SDB_ERR_INVALID, "sdb_sort_rows: key %d NULL or misaligned", k);
    }
    cudaStream_t s = (cudaStream_t)stream;
    Scratch sc;
    scratch_layout(n, static_cast<char *>(scratch), &sc);
    const uint32_t n32 = (uint32_t)n;
    const uint32_t nb = (n32 + kSortTile - 1) / kSortTile;
    const uint32_t m = nb * 256;
    const uint32_t nsum = (m + kScanThreads - 1) / kScanThreads;
    k_iota<<<std::min<uint32_t>((n32 + 255) / 256, 4096), 256, 0, s>>>(perm, n32);
    int st = sdb_check_launch("sdb_sort_rows");
    if (st != SDB_OK) return st;
    uint32_t *cur = perm, *nxt = sc.perm_b;
    for (int k = nkeys - 1; k >= 0; k--) {
        const int words = key_types[k] ? 2 : 1;
        for (int w = 0; w < words; w++) {
            const SortPass p{keys[k], key_types[k], w, descending[k] ? 1 : 0};
            uint32_t *wc = sc.word_a, *wn = sc.word_b;
            k_gather_word<<<std::min<uint32_t>((n32 + 255) / 256, 4096), 256, 0, s>>>(p, cur, n32, wc);
            sdb_count_launches(1);
            for (int shift = 0; shift < 32; shift += 8) {
                k_radix_count<<<nb, kSortThreads, 0, s>>>(wc, shift, n32, sc.hist, nb);
                k_scan_local<<<nsum, kScanThreads, 0, s>>>(sc.hist, m, sc.sums);
                k_scan_sums<<<1, kScanThreads, 0, s>>>(sc.sums, nsum);
                k_scan_add<<<nsum, kScanThreads, 0, s>>>(sc.hist, m, sc.sums);
                k_radix_scatter<<<nb, kSortThreads, 0, s>>>(wc, cur, shift, n32, sc.hist, nb, wn, nxt);
                sdb_count_launches(4);  // the four launches before the checked one
                st = sdb_check_launch("sdb_sort_rows");
                if (st != SDB_OK) return st;
                std::swap(cur, nxt);
                std::swap(wc, wn);
            }
        }
    }
    // four passes per word leave the result in perm
    return SDB_OK;
}

}  // extern "C"
