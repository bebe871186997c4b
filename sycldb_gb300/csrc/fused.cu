// Fused operator chain (sdb_fused_chain) for sm_103a.
//
// One pass over a segment applies a KernelBundle's kernels in order with each
// row's flag held in a register (4 rows per thread as a 4-bit mask), instead
// of one HBM round trip per kernel.  The values computed are those of the
// composed K2-K13 kernels followed by K7 (scalar SUM) or K8 (group-by SUM):
//   - a row's flag evolves op by op exactly as the flag buffers would;
//   - column loads happen only for rows (4-row groups) whose result can still
//     change: after the last op that can turn a false flag true (a NONE/OR
//     selection), a group with no live row stops and loads nothing more, so
//     at low selectivity later columns cost only the sectors that hold a
//     surviving row;
//   - intermediate columns (join values, projections) live in registers and
//     are stored only when the caller asks for them (out_col);
//   - group-by partial sums are privatised in shared memory per block
//     (64-bit shared atomics) and flushed once per touched slot; the first
//     block to touch a slot runs the reference's first-writer exchange
//     (kernels/aggregation.hpp:329-333) on the global occupancy word.
// Grids are persistent: (#SMs x resident blocks), grid-stride over 4-row
// groups; fact columns are read with streaming (evict-first) 128-bit loads,
// hash tables through the read-only path so they stay in L2.
#include <algorithm>
#include <cstdio>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <cstring>
#include <utility>
#include <vector>

#include "common.cuh"

namespace {

__device__ unsigned long long g_errors;

unsigned long long read_errors(cudaStream_t s)
{
    unsigned long long v = 0, zero = 0;
    cudaMemcpyFromSymbolAsync(&v, g_errors, sizeof v, 0, cudaMemcpyDeviceToHost, s);
    cudaMemcpyToSymbolAsync(g_errors, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    return v;
}
const int g_reader_registered = (sdb_errors_add_reader(&read_errors), 0);

constexpr int kThreads = 256;

// T_BUILD covers SDB_TERM_BUILD_KEYS and SDB_TERM_BUILD_KV (told apart at run time)
enum Term { T_FLAGS = 0, T_SUM = 1, T_GROUP = 2, T_BUILD = 3 };

// A selection of a column against literals as an interval test:
// in = (a - lo <= span) | (a - lo2 <= span2) in unsigned 32-bit arithmetic,
// negated when neg; combined into the flag with `logic` (SDB_NONE / AND / OR).
struct RangeTest {
    const int32_t *col;
    int32_t lo, lo2;
    uint32_t span, span2;
    int32_t logic, neg;
};
constexpr int kRangeTests = 3;

struct ChainLaunch {
    sdb_chain_desc d;
    int32_t dead_from;   // ops at index >= dead_from cannot revive a dead row
    int32_t vec;         // all column pointers 16-byte aligned, flags 4-byte aligned
    uint32_t mults[SDB_CHAIN_MAX_KEYS];
    // builds whose ops are all selections of columns against literals: the
    // ops as interval tests (n_tests >= 0), evaluated with every column of a
    // tile loaded at once; -1: the general op-by-op pass
    int32_t n_tests;
    RangeTest tests[kRangeTests];
};

// Block tile: kThreads x ITEMS consecutive rows.  Thread t owns rows
// tile + t + k * kThreads (k < ITEMS), so each per-item load of a warp is one
// coalesced 128-byte request, and every op issues the loads of all its items
// before it consumes any (ITEMS independent loads in flight per thread).  A
// thread's flags are an ITEMS-bit mask; values the ops produce (join values,
// projections) stay in registers, NREGS per row.
template <int NREGS, int ITEMS>
struct Tile {
    uint64_t base;       // row of item 0
    uint32_t valid;      // bit k: row base + k * kThreads exists
    uint32_t live;       // bit k: that row's flag
    int32_t reg[NREGS][ITEMS];
};

template <int NREGS, int ITEMS>
__device__ __forceinline__ void reg_get(const Tile<NREGS, ITEMS> &T, int idx, int32_t (&out)[ITEMS])
{
#pragma unroll
    for (int k = 0; k < ITEMS; k++) out[k] = T.reg[0][k];
#pragma unroll
    for (int r = 1; r < NREGS; r++)
        if (idx == r) {
#pragma unroll
            for (int k = 0; k < ITEMS; k++) out[k] = T.reg[r][k];
        }
}

template <int NREGS, int ITEMS>
__device__ __forceinline__ void reg_set(Tile<NREGS, ITEMS> &T, int idx, const int32_t (&in)[ITEMS], uint32_t mask)
{
#pragma unroll
    for (int r = 0; r < NREGS; r++)
        if (idx == r) {
#pragma unroll
            for (int k = 0; k < ITEMS; k++)
                if ((mask >> k) & 1u) T.reg[r][k] = in[k];
        }
}

__device__ __forceinline__ uint64_t row_of(uint64_t base, int k) { return base + (uint64_t)k * kThreads; }

// Operand values for the items of `need` (other items unspecified).  Column
// loads are evict-first (STREAM) for fact columns read once, plain for
// dimension columns that several chains of a batch read.
template <bool STREAM = true, int NREGS, int ITEMS>
__device__ __forceinline__ void fetch(const sdb_operand &o, const Tile<NREGS, ITEMS> &T, uint32_t need,
                                      int32_t (&v)[ITEMS])
{
    if (o.kind == SDB_SRC_COL) {
#pragma unroll
        for (int k = 0; k < ITEMS; k++)
            if ((need >> k) & 1u) v[k] = STREAM ? __ldcs(o.col + row_of(T.base, k)) : __ldg(o.col + row_of(T.base, k));
    } else if (o.kind == SDB_SRC_REG) {
        reg_get(T, o.reg, v);
    } else {
#pragma unroll
        for (int k = 0; k < ITEMS; k++) v[k] = o.lit;
    }
}

// One item's operand value (the rare first-writer path).
template <int NREGS, int ITEMS>
__device__ __forceinline__ int32_t operand_item(const sdb_operand &o, const Tile<NREGS, ITEMS> &T, int k)
{
    if (o.kind == SDB_SRC_COL) return __ldg(o.col + row_of(T.base, k));
    if (o.kind == SDB_SRC_LIT) return o.lit;
    int32_t v = T.reg[0][k];
#pragma unroll
    for (int r = 1; r < NREGS; r++)
        if (o.reg == r) v = T.reg[r][k];
    return v;
}

template <int ITEMS>
__device__ __forceinline__ void store_masked(int32_t *col, uint64_t base, const int32_t (&v)[ITEMS], uint32_t mask)
{
#pragma unroll
    for (int k = 0; k < ITEMS; k++)
        if ((mask >> k) & 1u) col[row_of(base, k)] = v[k];
}

// Evaluates the op list on a thread's items; on return T.live holds the flags.
template <bool STREAM = true, int NREGS, int ITEMS, class LC>
__device__ __forceinline__ void run_ops(const LC &Lc, Tile<NREGS, ITEMS> &T)
{
    const sdb_chain_desc &d = Lc.d;
    if (d.flags_in) {
        uint8_t f[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; k++)
            if ((T.valid >> k) & 1u) f[k] = STREAM ? __ldcs(d.flags_in + row_of(T.base, k)) : __ldg(d.flags_in + row_of(T.base, k));
        T.live = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; k++)
            if ((T.valid >> k) & 1u) T.live |= (uint32_t)(f[k] != 0) << k;
    } else {
        T.live = T.valid;
    }

#pragma unroll 1
    for (int i = 0; i < d.n_ops; i++) {
        if (T.live == 0 && i >= Lc.dead_from) break;
        const sdb_chain_op &op = d.ops[i];
        int32_t a[ITEMS], c[ITEMS];
        switch (op.kind) {
        case SDB_OP_SELECT: {
            const uint32_t need = op.logic_op == SDB_AND ? T.live : T.valid;
            fetch<STREAM>(op.a, T, need, a);
            fetch<STREAM>(op.b, T, need, c);
            uint32_t m = 0;
#pragma unroll
            for (int k = 0; k < ITEMS; k++) m |= (uint32_t)sdb::compare(op.cmp_op, a[k], c[k]) << k;
            T.live = sdb::logical4(op.logic_op, T.live, m & need) & T.valid;
            break;
        }
        case SDB_OP_SEARCH_RANGE:
        case SDB_OP_SEARCH_POINTS: {
            const uint32_t need = op.logic_op == SDB_AND ? T.live : T.valid;
            fetch<STREAM>(op.a, T, need, a);
            uint32_t m = 0;
            if (op.kind == SDB_OP_SEARCH_RANGE) {
#pragma unroll
                for (int k = 0; k < ITEMS; k++) m |= (uint32_t)(a[k] >= op.lo && a[k] <= op.hi) << k;
            } else {
#pragma unroll
                for (int k = 0; k < ITEMS; k++) m |= (uint32_t)(a[k] == op.lo || a[k] == op.hi) << k;
            }
            T.live = sdb::logical4(op.logic_op, T.live, m & need) & T.valid;
            break;
        }
        case SDB_OP_SEMI_PROBE: {
            const uint32_t need = T.live;
            fetch<STREAM>(op.a, T, need, a);
            const uint8_t *ht = static_cast<const uint8_t *>(op.ht);
            uint8_t h[ITEMS];
            if (op.ht_log2) {  // open-addressing table
                const uint32_t *w = static_cast<const uint32_t *>(op.ht);
#pragma unroll
                for (int k = 0; k < ITEMS; k++) {
                    h[k] = 0;
                    if (((need >> k) & 1u) && a[k] >= op.lo && a[k] <= op.hi) {
                        const int64_t s = sdb::oa_find<1>(w, op.ht_log2, sdb::oa_tag(a[k], op.lo));
                        h[k] = s >= 0 ? (uint8_t)(__ldg(w + s) & 1u) : 0;
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < ITEMS; k++) {
                    h[k] = 0;
                    if (((need >> k) & 1u) && a[k] >= op.lo && a[k] <= op.hi)
                        h[k] = __ldg(ht + ((uint32_t)a[k] - (uint32_t)op.lo));
                }
            }
            uint32_t m = 0;
#pragma unroll
            for (int k = 0; k < ITEMS; k++) m |= (uint32_t)(h[k] != 0) << k;
            T.live = m & need;
            break;
        }
        case SDB_OP_FULL_PROBE: {
            const uint32_t need = T.live;
            fetch<STREAM>(op.a, T, need, a);
            const int2 *ht = static_cast<const int2 *>(op.ht);
            int2 e[ITEMS];
            if (op.ht_log2) {  // open-addressing table: hit = the word's flag bit
#pragma unroll
                for (int k = 0; k < ITEMS; k++) {
                    e[k] = make_int2(0, 0);
                    if (((need >> k) & 1u) && a[k] >= op.lo && a[k] <= op.hi) {
                        const int64_t s = sdb::oa_find<2>(static_cast<const uint32_t *>(op.ht), op.ht_log2,
                                                          sdb::oa_tag(a[k], op.lo));
                        if (s >= 0) {
                            e[k] = __ldg(ht + s);
                            e[k].x &= 1;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < ITEMS; k++) {
                    e[k] = make_int2(0, 0);
                    if (((need >> k) & 1u) && a[k] >= op.lo && a[k] <= op.hi)
                        e[k] = __ldg(ht + ((uint32_t)a[k] - (uint32_t)op.lo));
                }
            }
            uint32_t m = 0;
#pragma unroll
            for (int k = 0; k < ITEMS; k++) {
                m |= (uint32_t)(e[k].x == 1) << k;
                c[k] = e[k].y;
            }
            m &= need;
            T.live = m;
            reg_set(T, op.out_reg, c, m);
            if (op.out_col && m) store_masked(op.out_col, T.base, c, m);
            break;
        }
        case SDB_OP_BINOP: {
            const uint32_t need = T.live;
            fetch<STREAM>(op.a, T, need, a);
            fetch<STREAM>(op.b, T, need, c);
#pragma unroll
            for (int k = 0; k < ITEMS; k++) a[k] = sdb::binop(a[k], c[k], op.bin_op);
            reg_set(T, op.out_reg, a, need);
            if (op.out_col && need) store_masked(op.out_col, T.base, a, need);
            break;
        }
        case SDB_OP_FILL: {
#pragma unroll
            for (int k = 0; k < ITEMS; k++) a[k] = op.a.lit;
            reg_set(T, op.out_reg, a, T.valid);
            if (op.out_col && T.valid) store_masked(op.out_col, T.base, a, T.valid);
            break;
        }
        default:
            break;
        }
    }
}

// Block-private group-by partials: a shared-memory table of kCap entries
// (slot id + 64-bit sum, 24 KB).  Slots index it directly when P <= kCap;
// otherwise it is an open-addressing table (bounded linear probing) and a
// row that finds no entry goes straight to the global arrays.
constexpr uint32_t kCap = 2048;
constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr int kMaxProbe = 16;

template <uint32_t CAP = kCap>
__device__ __forceinline__ bool smem_group_add(uint32_t *s_key, unsigned long long *s_sum, uint32_t slot,
                                               unsigned long long v, bool direct, bool &first)
{
    static_assert((CAP & (CAP - 1)) == 0, "table size must be a power of two");
    uint32_t h = direct ? slot : ((slot * 2654435761u) >> (32 - __builtin_ctz(CAP)));
#pragma unroll 1
    for (int p = 0; p < (direct ? 1 : kMaxProbe); p++) {
        uint32_t k = s_key[h];
        if (k == kEmpty) {
            k = atomicCAS(&s_key[h], kEmpty, slot);
            if (k == kEmpty) {
                first = true;
                atomicAdd(&s_sum[h], v);
                return true;
            }
        }
        if (k == slot) {
            first = false;
            atomicAdd(&s_sum[h], v);
            return true;
        }
        h = (h + 1) & (CAP - 1);
    }
    return false;
}

// Resident blocks per SM a tile size targets (register cap 64 / 85 / 128
// per thread at 256 threads per block).
__host__ __device__ constexpr int min_blocks_of(int ITEMS) { return ITEMS <= 4 ? 4 : (ITEMS <= 8 ? 3 : 2); }

// Hash-table build over a thread's items with the chain's final flags (K10 /
// K12): each row of `rows` writes its slot, a live row a hit (and its value),
// a dead row a miss.  `rows` is every valid row, or only the live ones when
// the table is known to be zero (ht_zeroed: a miss would write a zero over a
// zero).  A key outside the table is counted as an error and skipped, as in
// the standalone builds.
template <int ITEMS>
__device__ __forceinline__ void build_store(const sdb_chain_desc &d, uint32_t rows, uint32_t live,
                                            const int32_t (&key)[ITEMS], const int32_t (&val)[ITEMS])
{
    const bool kv = d.terminal == SDB_TERM_BUILD_KV;
    const uint32_t len = (uint32_t)d.ht_len;  // > 0
    if (d.ht_log2) {  // open-addressing table over keys ht_min .. ht_min + len - 1
        uint32_t *w = static_cast<uint32_t *>(d.ht_out);
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            if (!((rows >> k) & 1u)) continue;
            const bool hit = (live >> k) & 1u;
            if ((uint32_t)key[k] - (uint32_t)d.ht_min >= len) {
                atomicAdd(&g_errors, 1ull);
                continue;
            }
            const uint32_t tag = sdb::oa_tag(key[k], d.ht_min);
            const int64_t h = kv ? sdb::oa_put<2>(w, d.ht_log2, tag, hit) : sdb::oa_put<1>(w, d.ht_log2, tag, hit);
            if (h == -2) atomicAdd(&g_errors, 1ull);
            else if (kv && h >= 0 && hit) static_cast<int32_t *>(d.ht_out)[2 * h + 1] = val[k];
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
        if (!((rows >> k) & 1u)) continue;
        // (key - min) % len: a key inside the table is its own slot; the
        // remainder only for the others
        uint32_t h = (uint32_t)key[k] - (uint32_t)d.ht_min;
        if (__builtin_expect(h >= len, 0)) {
            const int64_t w = sdb::ht_slot(key[k], d.ht_len, d.ht_min);
            if (w < 0 || w >= d.ht_len) {
                atomicAdd(&g_errors, 1ull);
                continue;
            }
            h = (uint32_t)w;
        }
        const bool hit = (live >> k) & 1u;
        if (kv) {
            int32_t *ht2 = static_cast<int32_t *>(d.ht_out) + 2 * (uint64_t)h;
            if (hit)
                *reinterpret_cast<int2 *>(ht2) = make_int2(1, val[k]);
            else
                ht2[0] = 0;
        } else {
            static_cast<uint8_t *>(d.ht_out)[h] = hit ? 1 : 0;
        }
    }
}

template <bool STREAM, int NREGS, int ITEMS>
__device__ __forceinline__ void build_rows(const sdb_chain_desc &d, const Tile<NREGS, ITEMS> &T)
{
    int32_t key[ITEMS], val[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; k++) val[k] = 0;
    const uint32_t rows = d.ht_zeroed ? T.live : T.valid;
    if (rows == 0) return;
    fetch<STREAM>(d.build_key, T, rows, key);
    if (d.terminal == SDB_TERM_BUILD_KV) fetch<STREAM>(d.build_val, T, T.live, val);
    build_store(d, rows, T.live, key, val);
}

// A build chain in interval-test form (NT tests) over tiles t, t + stride,
// ... < t_end (kThreads x ITEMS rows each).  Per tile and thread: the input
// flags and every test's column are loaded before any is used (one memory
// round trip instead of one per op), the key and the value with them (every
// valid row writes), or after the tests for the live rows only (ht_zeroed),
// so that a warp without a live row stops there.  The chain's parameters are
// read once, before the tiles.
template <bool STREAM, int ITEMS, int NT>
__device__ __forceinline__ void build_tiles(const ChainLaunch &L, uint32_t t, uint32_t t_end, uint32_t stride)
{
    const sdb_chain_desc &d = L.d;
    auto ld = [](const int32_t *p) { return STREAM ? __ldcs(p) : __ldg(p); };
    const uint32_t n = (uint32_t)d.n;  // interval-test chains have fewer than 2^32 rows
    const bool kv = d.terminal == SDB_TERM_BUILD_KV;
    const bool zeroed = d.ht_zeroed != 0;
    const uint8_t *fin = d.flags_in;
    const int32_t *kcol = d.build_key.kind == SDB_SRC_COL ? d.build_key.col : nullptr;
    const int32_t *vcol = d.build_val.kind == SDB_SRC_COL ? d.build_val.col : nullptr;
    const int32_t klit = d.build_key.lit, vlit = d.build_val.lit;
    const int32_t *tcol[NT > 0 ? NT : 1];
    uint32_t tlo[NT > 0 ? NT : 1], tlo2[NT > 0 ? NT : 1], tspan[NT > 0 ? NT : 1], tspan2[NT > 0 ? NT : 1];
    uint32_t tneg[NT > 0 ? NT : 1];
    int32_t tlogic[NT > 0 ? NT : 1];
#pragma unroll
    for (int j = 0; j < NT; j++) {
        tcol[j] = L.tests[j].col;
        tlo[j] = (uint32_t)L.tests[j].lo;
        tlo2[j] = (uint32_t)L.tests[j].lo2;
        tspan[j] = L.tests[j].span;
        tspan2[j] = L.tests[j].span2;
        tneg[j] = (uint32_t)L.tests[j].neg;
        tlogic[j] = L.tests[j].logic;
    }
    for (; t < t_end; t += stride) {
        const uint32_t base = t * (uint32_t)(kThreads * ITEMS) + threadIdx.x;
        uint32_t valid = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; k++) valid |= (uint32_t)(base + (uint32_t)(k * kThreads) < n) << k;
        int32_t x[NT > 0 ? NT : 1][ITEMS], key[ITEMS], val[ITEMS];
        uint8_t f[ITEMS];
        auto load_kv = [&](uint32_t rows) {
#pragma unroll
            for (int k = 0; k < ITEMS; k++) {
                if (!((rows >> k) & 1u)) continue;
                const uint32_t r = base + (uint32_t)(k * kThreads);
                key[k] = kcol ? ld(kcol + r) : klit;
                if (kv) val[k] = vcol ? ld(vcol + r) : vlit;
            }
        };
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            f[k] = 1;
            key[k] = val[k] = 0;
#pragma unroll
            for (int j = 0; j < NT; j++) x[j][k] = 0;
        }
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            if (!((valid >> k) & 1u)) continue;
            const uint32_t r = base + (uint32_t)(k * kThreads);
            if (fin) f[k] = STREAM ? __ldcs(fin + r) : __ldg(fin + r);
#pragma unroll
            for (int j = 0; j < NT; j++) x[j][k] = ld(tcol[j] + r);
        }
        if (!zeroed) load_kv(valid);
        uint32_t live = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; k++) live |= (uint32_t)(f[k] != 0) << k;
        live &= valid;
#pragma unroll
        for (int j = 0; j < NT; j++) {
            uint32_t m = 0;
#pragma unroll
            for (int k = 0; k < ITEMS; k++) {
                const uint32_t a = (uint32_t)x[j][k];
                m |= ((((a - tlo[j]) <= tspan[j]) | ((a - tlo2[j]) <= tspan2[j])) ^ tneg[j]) << k;
            }
            live = tlogic[j] == SDB_NONE ? (m & valid) : (tlogic[j] == SDB_AND ? (live & m) : ((live | m) & valid));
        }
        if (zeroed) {
            if (live == 0) continue;
            load_kv(live);
        }
        build_store(d, zeroed ? live : valid, live, key, val);
    }
}

template <bool STREAM, int ITEMS>
__device__ __forceinline__ void build_tiles_any(const ChainLaunch &L, uint32_t t, uint32_t t_end, uint32_t stride)
{
    switch (L.n_tests) {
    case 0: build_tiles<STREAM, ITEMS, 0>(L, t, t_end, stride); break;
    case 1: build_tiles<STREAM, ITEMS, 1>(L, t, t_end, stride); break;
    case 2: build_tiles<STREAM, ITEMS, 2>(L, t, t_end, stride); break;
    case 3: build_tiles<STREAM, ITEMS, 3>(L, t, t_end, stride); break;
    default: build_tiles<STREAM, ITEMS, kRangeTests>(L, t, t_end, stride); break;
    }
}

template <int TERM, int NREGS, int ITEMS>
__global__ void __launch_bounds__(kThreads, min_blocks_of(ITEMS)) k_chain(const __grid_constant__ ChainLaunch L)
{
    const sdb_chain_desc &d = L.d;
    __shared__ uint32_t s_key[TERM == T_GROUP ? kCap : 1];
    __shared__ unsigned long long s_sum[TERM == T_GROUP ? kCap : 1];
    const bool direct = d.P <= kCap;
    if (TERM == T_GROUP) {
        for (uint32_t i = threadIdx.x; i < kCap; i += blockDim.x) {
            s_key[i] = kEmpty;
            s_sum[i] = 0;
        }
        __syncthreads();
    }

    constexpr uint64_t kTile = (uint64_t)kThreads * ITEMS;
    if (TERM == T_BUILD && L.n_tests >= 0) {
        build_tiles_any<true, ITEMS>(L, blockIdx.x, (uint32_t)((d.n + kTile - 1) / kTile), gridDim.x);
        return;
    }
    uint64_t acc = 0;
    Tile<NREGS, ITEMS> T;
#pragma unroll
    for (int r = 0; r < NREGS; r++)
#pragma unroll
        for (int k = 0; k < ITEMS; k++) T.reg[r][k] = 0;

    for (uint64_t tile = (uint64_t)blockIdx.x * kTile; tile < d.n; tile += (uint64_t)gridDim.x * kTile) {
        T.base = tile + threadIdx.x;
        T.valid = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; k++) T.valid |= (uint32_t)(row_of(T.base, k) < d.n) << k;
        run_ops(L, T);

        if (TERM == T_FLAGS || d.flags_out) {
#pragma unroll
            for (int k = 0; k < ITEMS; k++)
                if ((T.valid >> k) & 1u) d.flags_out[row_of(T.base, k)] = (uint8_t)((T.live >> k) & 1u);
        }
        if (TERM == T_BUILD) {
            build_rows<true>(d, T);
            continue;
        }
        if (T.live == 0) continue;
        if (TERM == T_SUM) {
            int32_t v[ITEMS];
            fetch(d.value, T, T.live, v);
#pragma unroll
            for (int k = 0; k < ITEMS; k++)
                if ((T.live >> k) & 1u) acc += sdb::widen(v[k]);
        } else if (TERM == T_GROUP) {
            int32_t v[ITEMS], kv[ITEMS];
            uint32_t h[ITEMS];
            fetch(d.value, T, T.live, v);
#pragma unroll
            for (int k = 0; k < ITEMS; k++) h[k] = 0;
#pragma unroll
            for (int kk = 0; kk < SDB_CHAIN_MAX_KEYS; kk++) {
                if (kk < d.n_keys) {
                    fetch(d.keys[kk], T, T.live, kv);
#pragma unroll
                    for (int k = 0; k < ITEMS; k++) h[k] += ((uint32_t)kv[k] - (uint32_t)d.key_min[kk]) * L.mults[kk];
                }
            }
#pragma unroll
            for (int k = 0; k < ITEMS; k++) {
                if (!((T.live >> k) & 1u)) continue;
                const int64_t s = sdb::group_slot(h[k], d.P);
                if (s < 0 || (uint64_t)s >= d.P) {
                    atomicAdd(&g_errors, 1ull);
                    continue;
                }
                const unsigned long long val = (unsigned long long)sdb::widen(v[k]);
                bool first = false;
                if (smem_group_add(s_key, s_sum, (uint32_t)s, val, direct, first)) {
                    if (first) first = atomicExch(&d.occ[s], 1u) == 0u;
                } else {
                    first = d.occ[s] == 0u && atomicExch(&d.occ[s], 1u) == 0u;
                    atomicAdd(reinterpret_cast<unsigned long long *>(&d.out_sum[s]), val);
                }
                if (first) {
#pragma unroll
                    for (int kk = 0; kk < SDB_CHAIN_MAX_KEYS; kk++)
                        if (kk < d.n_keys) d.out_keys[kk][s] = operand_item(d.keys[kk], T, k);
                }
            }
        }
    }

    if (TERM == T_SUM) {
        __shared__ uint64_t part[kThreads / 32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t t = 0;
            for (int w = 0; w < kThreads / 32; w++) t += part[w];
            if (t) atomicAdd(reinterpret_cast<unsigned long long *>(d.sum_out), (unsigned long long)t);
        }
    } else if (TERM == T_GROUP) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < kCap; i += blockDim.x) {
            const uint32_t k = s_key[i];
            if (k != kEmpty) atomicAdd(reinterpret_cast<unsigned long long *>(&d.out_sum[k]), s_sum[i]);
        }
    }
}

int num_sms() { return sdb::device_sms(); }

template <int TERM, int NREGS, int ITEMS>
int launch_term(const ChainLaunch &L, cudaStream_t s)
{
    auto kern = k_chain<TERM, NREGS, ITEMS>;
    static const int per_sm = [&] {  // initialised once, thread-safe
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, kThreads, 0) != cudaSuccess || v < 1) v = 1;
        return v;
    }();
    const uint64_t tile = (uint64_t)kThreads * ITEMS;
    uint64_t blocks = (L.d.n + tile - 1) / tile;
    const uint64_t cap = (uint64_t)num_sms() * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    kern<<<(unsigned)blocks, kThreads, 0, s>>>(L);
    return sdb_check_launch("sdb_fused_chain");
}

// Hash-table builds: dimension tables are small, one tile shape serves.
int launch_build(const ChainLaunch &L, int nregs, cudaStream_t s)
{
    if (nregs <= 2) return launch_term<T_BUILD, 2, 4>(L, s);
    if (nregs <= 4) return launch_term<T_BUILD, 4, 4>(L, s);
    return launch_term<T_BUILD, 8, 4>(L, s);
}

// The build chains of a batch in one persistent launch.  Tile t of the batch
// (kThreads x kBuildItems rows) belongs to chain c with tile_start[c] <= t <
// tile_start[c + 1] (no empty chains); block b takes the contiguous tiles
// [b T / G, (b + 1) T / G), so it meets few chains, and copies a chain's
// launch record into shared memory when it moves on to that chain.  Column
// loads keep lines in L2: the chains of a batch often read the same
// dimension columns.
constexpr int kBuildItems = 8;

template <int NREGS, bool GENERAL>  // GENERAL: some chain is not in interval-test form
__global__ void __launch_bounds__(kThreads, GENERAL ? 2 : min_blocks_of(kBuildItems))
    k_build_batch(const ChainLaunch *__restrict__ Ls, const uint32_t *__restrict__ tile_start, int n_chains)
{
    constexpr int ITEMS = kBuildItems;
    constexpr uint64_t kTile = (uint64_t)kThreads * ITEMS;
    __shared__ ChainLaunch sL;
    const uint64_t total = tile_start[n_chains];
    const uint32_t t0 = (uint32_t)(total * blockIdx.x / gridDim.x);
    const uint32_t t1 = (uint32_t)(total * (blockIdx.x + 1) / gridDim.x);
    int cur = -1;
    Tile<NREGS, ITEMS> T;
#pragma unroll
    for (int r = 0; r < NREGS; r++)
#pragma unroll
        for (int k = 0; k < ITEMS; k++) T.reg[r][k] = 0;
    // the block's tiles, one chain's run of them at a time
    for (uint32_t t = t0; t < t1;) {
        int lo = 0, hi = n_chains - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tile_start[mid] <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        if (lo != cur) {
            __syncthreads();  // every thread is done with the previous record
            const uint32_t *src = reinterpret_cast<const uint32_t *>(Ls + lo);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&sL);
            for (uint32_t i = threadIdx.x; i < (uint32_t)(sizeof(ChainLaunch) / 4); i += kThreads) dst[i] = src[i];
            __syncthreads();
            cur = lo;
        }
        const uint32_t first = tile_start[lo];
        const uint32_t end = min(t1, tile_start[lo + 1]);
        if (!GENERAL || sL.n_tests >= 0) {
            build_tiles_any<false, ITEMS>(sL, t - first, end - first, 1);
            t = end;
            continue;
        }
        const sdb_chain_desc &d = sL.d;
        for (; t < end; t++) {
            T.base = (uint64_t)(t - first) * kTile + threadIdx.x;
            T.valid = 0;
#pragma unroll
            for (int k = 0; k < ITEMS; k++) T.valid |= (uint32_t)(row_of(T.base, k) < d.n) << k;
            run_ops<false>(sL, T);
            if (d.flags_out) {
#pragma unroll
                for (int k = 0; k < ITEMS; k++)
                    if ((T.valid >> k) & 1u) d.flags_out[row_of(T.base, k)] = (uint8_t)((T.live >> k) & 1u);
            }
            build_rows<false>(d, T);
        }
    }
}

template <int NREGS, bool GENERAL>
int launch_build_batch_t(const ChainLaunch *Ls, const uint32_t *tile_start, int n, uint32_t tiles, cudaStream_t s)
{
    auto kern = k_build_batch<NREGS, GENERAL>;
    static const int per_sm = [&] {  // initialised once, thread-safe
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, kThreads, 0) != cudaSuccess || v < 1) v = 1;
        return v;
    }();
    const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)num_sms() * per_sm));
    kern<<<(unsigned)blocks, kThreads, 0, s>>>(Ls, tile_start, n);
    return sdb_check_launch("sdb_chain_batch_launch");
}

// nregs = 0: every chain is in interval-test form
int launch_build_batch(const ChainLaunch *Ls, const uint32_t *tile_start, int n, uint32_t tiles, int nregs,
                       cudaStream_t s)
{
    if (nregs == 0) return launch_build_batch_t<1, false>(Ls, tile_start, n, tiles, s);
    if (nregs <= 2) return launch_build_batch_t<2, true>(Ls, tile_start, n, tiles, s);
    if (nregs <= 4) return launch_build_batch_t<4, true>(Ls, tile_start, n, tiles, s);
    return launch_build_batch_t<8, true>(Ls, tile_start, n, tiles, s);
}

// Variants: 0, 1, 2 = 4, 8, 16 rows per thread.  Chains needing up to 2
// registers take all three; up to 4 registers, 4 or 8 rows; up to 8, 4 rows.
template <int TERM>
int launch_regs(const ChainLaunch &L, int nregs, int variant, cudaStream_t s)
{
    if (nregs <= 2) {
        if (variant <= 0) return launch_term<TERM, 2, 4>(L, s);
        if (variant == 1) return launch_term<TERM, 2, 8>(L, s);
        return launch_term<TERM, 2, 16>(L, s);
    }
    if (nregs <= 4) {
        if (variant <= 0) return launch_term<TERM, 4, 4>(L, s);
        return launch_term<TERM, 4, 8>(L, s);
    }
    return launch_term<TERM, 8, 4>(L, s);
}

// ------------------------------------------------------------------ dense
// Shape-specialised pass for the common chains.  The op sequence is a
// compile-time pack, so each op is straight-line code (no dispatch), and the
// columns the chain reads (up to kSlots distinct ones) are loaded for the
// NEXT tile while the current tile is probed: DRAM latency overlaps the
// hash-table probes instead of sitting in each row's dependency chain.  Every
// chain column is read in full (dense), so the pass is bound by HBM
// bandwidth at 4 B per column per row.
namespace dense {

// lo <= a <= hi (empty when lo > hi).
__device__ __forceinline__ bool in_range(int32_t a, int32_t lo, int32_t hi) { return a >= lo && a <= hi; }

constexpr int kItems = 4;  // rows per thread per tile of the passes without late slots
// Rows per thread per tile: CARRY 3 (late slots, two staged columns) takes 8
// -- the same shared memory per stage as four columns of 4 rows -- the others
// 4.  A thread copies items / 4 16-byte pieces per staged column and tile.
template <int CARRY>
__host__ __device__ constexpr int items_of() { return CARRY == 3 ? 8 : kItems; }
constexpr int kSlots = 4;
// Slots per ring stage: CARRY 3 stages only its first two slots (the late
// ones, renumbered last, are not staged) and spends the space on more stages.
template <int CARRY>
__host__ __device__ constexpr int stage_slots() { return CARRY == 3 ? 2 : kSlots; }
constexpr int kMaxOps = 8;

struct Src {
    int32_t src;  // 0 prefetched column slot, 1 register, 2 literal
    int32_t idx;
    int32_t lit;
    int32_t pad;
};

struct Op {
    int32_t kind, cmp, logic, bin;
    Src a, b;
    int32_t lo, hi, out_reg;
    int32_t smem_bits;  // SEMI: probe the shared-memory bitmap copy of ht
    const void *ht;
    int32_t *out_col;
};

struct Launch {
    uint64_t n;
    const uint8_t *flags_in;
    uint8_t *flags_out;
    const int32_t *slot[kSlots];
    int32_t nslot, n_ops;
    Op ops[kMaxOps];
    Src value;
    uint64_t *sum_out;
    int32_t n_keys;
    uint32_t tail_slots;  // slots read after the first op (bit s = slot s): what a carried row keeps
    uint32_t late_slots;  // CARRY 3: tail slots read only after the second compaction level -- not
                          // staged; a row carries its row number there and the second level loads them
    int32_t nstaged;      // slots staged by the copy ring: 0 .. nstaged-1 (all nslot but for CARRY 3)
    Src keys[SDB_CHAIN_MAX_KEYS];
    int32_t key_min[SDB_CHAIN_MAX_KEYS];
    uint32_t mults[SDB_CHAIN_MAX_KEYS];
    uint64_t P;
    int32_t *out_keys[SDB_CHAIN_MAX_KEYS];
    uint64_t *out_sum;
    uint32_t *occ;
    const uint8_t *bitmap_ht;  // semi-join table staged as a bitmap (NULL: none)
    uint32_t bitmap_len;       // its entries
    int32_t bitmap_kv;         // 1: bitmap_ht is a key/value table (int2 entries, bit = x == 1)
    int32_t nregs;             // registers the chain uses (an instantiation needs NREGS >= nregs)
};

// Largest semi-join table staged as a shared-memory bitmap (32 KB of bits).
constexpr uint32_t kBitmapMax = 1u << 18;
// Block-private group-by table of the specialised pass (6 KB): small enough
// for five resident blocks per SM; a group-by has few live slots per block.
constexpr uint32_t kDenseCap = 512;

// ---- operand bindings -------------------------------------------------------
// A binding fixes at compile time where each operand of a chain shape comes
// from: column slot i (code i), register r (code 8 + r) or a literal (code 16,
// its value still read at run time); kAny reads the operand's Src at run time.
// Dyn binds nothing.  The bound passes of the hot shapes (the shapes'
// canonical bindings, checked on the host before a launch) read every operand
// straight from its register or staged row, and values that no later op
// reads are never moved.
constexpr int kAny = -1;
constexpr int kLitCode = 16;
__host__ __device__ constexpr int bslot(int i) { return i; }
__host__ __device__ constexpr int breg(int r) { return 8 + r; }
__host__ __device__ constexpr uint32_t code_bit(int c) { return c >= 0 && c < 8 ? 1u << c : 0u; }

struct Dyn {
    static constexpr bool bound = false;
    __host__ __device__ static constexpr int a(int) { return kAny; }
    __host__ __device__ static constexpr int b(int) { return kAny; }
    __host__ __device__ static constexpr int out(int) { return kAny; }
    __host__ __device__ static constexpr int value() { return kAny; }
    __host__ __device__ static constexpr int n_keys() { return kAny; }
    __host__ __device__ static constexpr int key(int) { return kAny; }
};

// Star join (semi, full, full -> group-by): semi(slot 0); full(slot 1) -> r0;
// full(slot 2) -> r1; group by (r1, r0), sum slot 3.
struct StarBind : Dyn {
    static constexpr bool bound = true;
    __host__ __device__ static constexpr int a(int i) { return bslot(i); }
    __host__ __device__ static constexpr int out(int i) { return i == 1 ? 0 : (i == 2 ? 1 : kAny); }
    __host__ __device__ static constexpr int value() { return bslot(3); }
    __host__ __device__ static constexpr int n_keys() { return 2; }
    __host__ __device__ static constexpr int key(int q) { return q == 0 ? breg(1) : (q == 1 ? breg(0) : kAny); }
};

// Range filter + join + projection -> group-by (date join): search(slot 0);
// full(slot 1) -> r0; r1 = slot 2 op slot 0; group by r0, sum r1.
struct DateJoinBind : Dyn {
    static constexpr bool bound = true;
    __host__ __device__ static constexpr int a(int i) { return bslot(i); }
    __host__ __device__ static constexpr int b(int i) { return i == 2 ? bslot(0) : kAny; }
    __host__ __device__ static constexpr int out(int i) { return i == 1 ? 0 : (i == 2 ? 1 : kAny); }
    __host__ __device__ static constexpr int value() { return breg(1); }
    __host__ __device__ static constexpr int n_keys() { return 1; }
    __host__ __device__ static constexpr int key(int q) { return q == 0 ? breg(0) : kAny; }
};

// Filter-project-sum: search(slot 0), search(slot 1), select(slot 2 cmp
// literal); r0 = slot 3 op slot 1; sum r0.
struct FilterSumBind : Dyn {
    static constexpr bool bound = true;
    __host__ __device__ static constexpr int a(int i) { return bslot(i); }
    __host__ __device__ static constexpr int b(int i) { return i == 2 ? kLitCode : (i == 3 ? bslot(1) : kAny); }
    __host__ __device__ static constexpr int out(int i) { return i == 3 ? 0 : kAny; }
    __host__ __device__ static constexpr int value() { return breg(0); }
    __host__ __device__ static constexpr int n_keys() { return 0; }
};

// Three full probes with the smallest table pre-tested (SSB flight 3 after
// prefilter_by_bitmap): bitmap test of slot 1; full(slot 0) -> r0;
// full(slot 1) -> r1 again for its value; full(slot 2) -> r2; group by
// (r0, r1, r2), sum slot 3.
struct Flight3Bind : Dyn {
    static constexpr bool bound = true;
    __host__ __device__ static constexpr int a(int i) { return i == 1 ? bslot(0) : (i == 3 ? bslot(2) : bslot(1)); }
    __host__ __device__ static constexpr int out(int i) { return i == 0 ? kAny : i - 1; }
    __host__ __device__ static constexpr int value() { return bslot(3); }
    __host__ __device__ static constexpr int n_keys() { return 3; }
    __host__ __device__ static constexpr int key(int q) { return q < 3 ? breg(q) : kAny; }
};

// Flight 4's second pass (its semi joins run first into the incoming flags):
// full(slot 0) -> r0; full(slot 1) -> r1; r2 = slot 2 op slot 3; group by
// (r1, r0), sum r2.
struct Flight4Bind : Dyn {
    static constexpr bool bound = true;
    __host__ __device__ static constexpr int a(int i) { return bslot(i); }
    __host__ __device__ static constexpr int b(int i) { return i == 2 ? bslot(3) : kAny; }
    __host__ __device__ static constexpr int out(int i) { return i; }
    __host__ __device__ static constexpr int value() { return breg(2); }
    __host__ __device__ static constexpr int n_keys() { return 2; }
    __host__ __device__ static constexpr int key(int q) { return q == 0 ? breg(1) : (q == 1 ? breg(0) : kAny); }
};

// Slots op i of a bound shape reads.
template <class B, int... KS>
__host__ __device__ constexpr uint32_t bound_op_bits(int i)
{
    constexpr int kinds[] = {KS...};
    const int k = kinds[i];
    if (k == SDB_OP_FILL) return 0u;
    const bool uses_b = k == SDB_OP_SELECT || k == SDB_OP_BINOP;
    return code_bit(B::a(i)) | (uses_b ? code_bit(B::b(i)) : 0u);
}

// The tail and late slot masks of a bound shape (what convert and
// late_slots_of compute from the launch): the tail is what a compacted row
// keeps -- the slots the ops after the first read (from the first on when
// the rows are compacted on their incoming flags, SPLIT 0).
template <class B, int TERM, int SPLIT, int... KS>
__host__ __device__ constexpr uint32_t bound_tail()
{
    uint32_t m = 0;
    for (int i = SPLIT == 0 ? 0 : 1; i < (int)sizeof...(KS); i++) m |= bound_op_bits<B, KS...>(i);
    if (TERM != T_FLAGS) m |= code_bit(B::value());
    for (int q = 0; q < B::n_keys(); q++) m |= code_bit(B::key(q));
    return m;
}
template <class B, int TERM, int SPLIT, int... KS>
__host__ __device__ constexpr uint32_t bound_late()
{
    uint32_t e = 0;
    for (int i = 0; i <= SPLIT && i < (int)sizeof...(KS); i++) e |= bound_op_bits<B, KS...>(i);
    return bound_tail<B, TERM, SPLIT, KS...>() & ~e;
}

// Tile rows are staged in shared memory by cp.async: thread t's kItems rows
// (tile + kItems t ..) of every chain column arrive as kItems / 4 16-byte
// copies per column into a ring of STAGES stages, issued STAGES - 1 tiles
// ahead.  Each thread reads back only what it copied, so no block barrier is
// needed.

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, uint32_t src_bytes)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int NREGS, int IT = kItems>
struct State {
    static constexpr int kIt = IT;
    int32_t reg[NREGS][IT];
    const uint32_t *bits;  // shared-memory bitmap of the staged semi-join table
    const int4 *stage;  // this thread's copies of the current tile: stage[slot * kThreads * IT / 4 + q]
    uint64_t base;      // row of item 0 (items are base .. base + IT - 1)
    uint32_t valid, live;
};

template <int NREGS, int IT>
__device__ __forceinline__ void fetch4(const Src &s, const State<NREGS, IT> &S, int32_t (&v)[IT])
{
    constexpr int kItems = IT, kQ = IT / 4;
    if (s.src == 0) {
#pragma unroll
        for (int q = 0; q < kQ; q++) {
            const int4 x = S.stage[s.idx * kThreads * kQ + q];
            v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
        }
    } else if (s.src == 1) {
#pragma unroll
        for (int k = 0; k < kItems; k++) v[k] = S.reg[0][k];
#pragma unroll
        for (int i = 1; i < NREGS; i++)
            if (s.idx == i) {
#pragma unroll
                for (int k = 0; k < kItems; k++) v[k] = S.reg[i][k];
            }
    } else {
#pragma unroll
        for (int k = 0; k < kItems; k++) v[k] = s.lit;
    }
}

template <int NREGS, int IT>
__device__ __forceinline__ void set_regs(State<NREGS, IT> &S, int r, const int32_t (&v)[IT], uint32_t mask)
{
    constexpr int kItems = IT;
#pragma unroll
    for (int i = 0; i < NREGS; i++)
        if (r == i) {
#pragma unroll
            for (int k = 0; k < kItems; k++)
                if ((mask >> k) & 1u) S.reg[i][k] = v[k];
        }
}

// fetch4 / set_regs with the operand's binding code C (kAny: at run time).
template <int C, int NREGS, int IT>
__device__ __forceinline__ void fetch4c(const Src &s, const State<NREGS, IT> &S, int32_t (&v)[IT])
{
    constexpr int kItems = IT, kQ = IT / 4;
    if constexpr (C == kAny) {
        fetch4(s, S, v);
    } else if constexpr (C < 8) {
#pragma unroll
        for (int q = 0; q < kQ; q++) {
            const int4 x = S.stage[C * kThreads * kQ + q];
            v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
        }
    } else if constexpr (C < kLitCode) {
        static_assert(C - 8 < NREGS, "bound register outside the instantiation");
#pragma unroll
        for (int k = 0; k < kItems; k++) v[k] = S.reg[C - 8][k];
    } else {
#pragma unroll
        for (int k = 0; k < kItems; k++) v[k] = s.lit;
    }
}

template <int OUT, int NREGS, int IT>
__device__ __forceinline__ void set_regs_c(State<NREGS, IT> &S, int r, const int32_t (&v)[IT], uint32_t mask)
{
    constexpr int kItems = IT;
    if constexpr (OUT == kAny) {
        set_regs(S, r, v, mask);
    } else {
        static_assert(OUT < NREGS, "bound register outside the instantiation");
#pragma unroll
        for (int k = 0; k < kItems; k++)
            if ((mask >> k) & 1u) S.reg[OUT][k] = v[k];
    }
}

template <int IT>
__device__ __forceinline__ void store4(int32_t *col, uint64_t base, const int32_t (&v)[IT], uint32_t mask)
{
    constexpr int kItems = IT;
#pragma unroll
    for (int k = 0; k < kItems; k++)
        if ((mask >> k) & 1u) col[base + k] = v[k];
}

template <int K, int A, int BB, int OUT, int NREGS, int IT>
__device__ __forceinline__ void step(const Op &op, State<NREGS, IT> &S)
{
    constexpr int kItems = IT;
    int32_t a[kItems], b[kItems];
    if (K == SDB_OP_SELECT || K == SDB_OP_SEARCH_RANGE || K == SDB_OP_SEARCH_POINTS) {
        const bool and_op = op.logic == SDB_AND;
        if (and_op && S.live == 0) return;
        const uint32_t need = and_op ? S.live : S.valid;
        fetch4c<A>(op.a, S, a);
        if (K == SDB_OP_SELECT) fetch4c<BB>(op.b, S, b);
        uint32_t m = 0;
#pragma unroll
        for (int k = 0; k < kItems; k++) {
            bool c;
            if (K == SDB_OP_SELECT) c = sdb::compare(op.cmp, a[k], b[k]);
            else if (K == SDB_OP_SEARCH_RANGE) c = in_range(a[k], op.lo, op.hi);
            else c = a[k] == op.lo || a[k] == op.hi;
            m |= (uint32_t)c << k;
        }
        S.live = sdb::logical4(op.logic, S.live, m & need) & S.valid;
    } else if (K == SDB_OP_SEMI_PROBE) {
        if (S.live == 0) return;
        fetch4c<A>(op.a, S, a);
        const uint8_t *ht = static_cast<const uint8_t *>(op.ht);
        uint32_t m = 0;
        if (op.smem_bits) {
            // branch-free: out-of-range keys read word 0 and are masked off
#pragma unroll
            for (int k = 0; k < kItems; k++) {
                const uint32_t ok = in_range(a[k], op.lo, op.hi);
                const uint32_t h = ok ? (uint32_t)a[k] - (uint32_t)op.lo : 0u;
                m |= ((S.bits[h >> 5] >> (h & 31u)) & ok) << k;
            }
        } else {
            uint8_t h[kItems];
#pragma unroll
            for (int k = 0; k < kItems; k++) {
                h[k] = 0;
                if (((S.live >> k) & 1u) && in_range(a[k], op.lo, op.hi))
                    h[k] = __ldg(ht + ((uint32_t)a[k] - (uint32_t)op.lo));
            }
#pragma unroll
            for (int k = 0; k < kItems; k++) m |= (uint32_t)(h[k] != 0) << k;
        }
        S.live &= m;
    } else if (K == SDB_OP_FULL_PROBE) {
        if (S.live == 0) return;
        fetch4c<A>(op.a, S, a);
        const int2 *ht = static_cast<const int2 *>(op.ht);
        int2 e[kItems];
#pragma unroll
        for (int k = 0; k < kItems; k++) {
            e[k] = make_int2(0, 0);
            if (((S.live >> k) & 1u) && in_range(a[k], op.lo, op.hi))
                e[k] = __ldg(ht + ((uint32_t)a[k] - (uint32_t)op.lo));
        }
        uint32_t m = 0;
#pragma unroll
        for (int k = 0; k < kItems; k++) {
            m |= (uint32_t)(e[k].x == 1) << k;
            b[k] = e[k].y;
        }
        m &= S.live;
        S.live = m;
        set_regs_c<OUT>(S, op.out_reg, b, m);
        if (op.out_col && m) store4(op.out_col, S.base, b, m);
    } else if (K == SDB_OP_BINOP) {
        if (S.live == 0) return;
        fetch4c<A>(op.a, S, a);
        fetch4c<BB>(op.b, S, b);
#pragma unroll
        for (int k = 0; k < kItems; k++) a[k] = sdb::binop(a[k], b[k], op.bin);
        set_regs_c<OUT>(S, op.out_reg, a, S.live);
        if (op.out_col) store4(op.out_col, S.base, a, S.live);
    } else if (K == SDB_OP_FILL) {
#pragma unroll
        for (int k = 0; k < kItems; k++) a[k] = op.a.lit;
        set_regs_c<OUT>(S, op.out_reg, a, S.valid);
        if (op.out_col) store4(op.out_col, S.base, a, S.valid);
    }
}

template <class B, int NREGS, int BEGIN, int... KS, int IT, int... IS>
__device__ __forceinline__ void run_steps(const Launch &L, State<NREGS, IT> &S, std::integer_sequence<int, IS...>)
{
    constexpr int kinds[] = {KS...};
    (step<kinds[BEGIN + IS], B::a(BEGIN + IS), B::b(BEGIN + IS), B::out(BEGIN + IS)>(L.ops[BEGIN + IS], S), ...);
}

// Sparse phase: after op SPLIT - 1 each warp compacts its surviving rows
// (ballot-free: a warp prefix sum of the lanes' live-bit counts) into a
// shared-memory list, and the remaining ops run one row per lane over that
// dense list instead of over mostly-dead 4-row groups.
template <int NREGS, int IT = kItems>
struct Row {
    static constexpr int kRegs = NREGS;
    int32_t reg[NREGS];
    const int32_t *wstage;  // the warp's 32 x kItems staged rows of slot 0 (slot s at + s * kItems * kThreads)
    uint32_t r;             // row within the warp's 32 x kItems
    uint64_t grow;          // global row
    bool live;
};

// A row whose slot values sit in registers (rows carried from one tile to the
// next; the chain writes no column after its first op, so no global row).
template <int NREGS>
struct VRow {
    static constexpr int kRegs = NREGS;
    static constexpr uint64_t grow = 0;
    int32_t reg[NREGS];
    int32_t v0, v1, v2, v3;  // slot values (scalars: selected, never indexed)
    bool live;
};

template <int NREGS>
__device__ __forceinline__ int32_t fetch1(const Src &s, const VRow<NREGS> &R)
{
    if (s.src == 0) return s.idx == 0 ? R.v0 : (s.idx == 1 ? R.v1 : (s.idx == 2 ? R.v2 : R.v3));
    if (s.src == 1) {
        int32_t v = R.reg[0];
#pragma unroll
        for (int i = 1; i < NREGS; i++) v = s.idx == i ? R.reg[i] : v;
        return v;
    }
    return s.lit;
}

template <int NREGS, int IT>
__device__ __forceinline__ int32_t fetch1(const Src &s, const Row<NREGS, IT> &R)
{
    if (s.src == 0) return R.wstage[s.idx * IT * kThreads + R.r];
    if (s.src == 1) {
        int32_t v = R.reg[0];
#pragma unroll
        for (int i = 1; i < NREGS; i++) v = s.idx == i ? R.reg[i] : v;
        return v;
    }
    return s.lit;
}

// fetch1 with the operand's binding code C (kAny: at run time).
template <int C, int NREGS>
__device__ __forceinline__ int32_t fetch1c(const Src &s, const VRow<NREGS> &R)
{
    if constexpr (C == kAny) {
        return fetch1(s, R);
    } else if constexpr (C < 8) {
        static_assert(C < kSlots, "bound slot outside the launch");
        return C == 0 ? R.v0 : (C == 1 ? R.v1 : (C == 2 ? R.v2 : R.v3));
    } else if constexpr (C < kLitCode) {
        static_assert(C - 8 < NREGS, "bound register outside the instantiation");
        return R.reg[C - 8];
    } else {
        return s.lit;
    }
}

template <int C, int NREGS, int IT>
__device__ __forceinline__ int32_t fetch1c(const Src &s, const Row<NREGS, IT> &R)
{
    if constexpr (C == kAny) {
        return fetch1(s, R);
    } else if constexpr (C < 8) {
        return R.wstage[C * IT * kThreads + R.r];
    } else if constexpr (C < kLitCode) {
        static_assert(C - 8 < NREGS, "bound register outside the instantiation");
        return R.reg[C - 8];
    } else {
        return s.lit;
    }
}

// One op on one row per lane.
template <int K, int A, int BB, int OUT, class RowT>
__device__ __forceinline__ void step1(const Op &op, RowT &R, const uint32_t *bits)
{
    constexpr int NREGS = RowT::kRegs;
    if (!R.live) return;
    if (K == SDB_OP_SELECT) {
        R.live = sdb::compare(op.cmp, fetch1c<A>(op.a, R), fetch1c<BB>(op.b, R));
    } else if (K == SDB_OP_SEARCH_RANGE) {
        R.live = in_range(fetch1c<A>(op.a, R), op.lo, op.hi);
    } else if (K == SDB_OP_SEARCH_POINTS) {
        const int32_t a = fetch1c<A>(op.a, R);
        R.live = a == op.lo || a == op.hi;
    } else if (K == SDB_OP_SEMI_PROBE) {
        const int32_t a = fetch1c<A>(op.a, R);
        const bool ok = in_range(a, op.lo, op.hi);
        const uint32_t i = ok ? (uint32_t)a - (uint32_t)op.lo : 0u;
        const bool hit = op.smem_bits ? ((bits[i >> 5] >> (i & 31u)) & 1u) != 0
                                      : __ldg(static_cast<const uint8_t *>(op.ht) + i) != 0;
        R.live = ok && hit;
    } else if (K == SDB_OP_FULL_PROBE) {
        const int32_t a = fetch1c<A>(op.a, R);
        const bool ok = in_range(a, op.lo, op.hi);
        const int2 e = __ldg(static_cast<const int2 *>(op.ht) + (ok ? (uint32_t)a - (uint32_t)op.lo : 0u));
        R.live = ok && e.x == 1;
        if constexpr (OUT == kAny) {
#pragma unroll
            for (int i = 0; i < NREGS; i++) R.reg[i] = (R.live && op.out_reg == i) ? e.y : R.reg[i];
        } else {
            R.reg[OUT] = R.live ? e.y : R.reg[OUT];
        }
        if (R.live && op.out_col) op.out_col[R.grow] = e.y;
    } else if (K == SDB_OP_BINOP) {
        const int32_t v = sdb::binop(fetch1c<A>(op.a, R), fetch1c<BB>(op.b, R), op.bin);
        if constexpr (OUT == kAny) {
#pragma unroll
            for (int i = 0; i < NREGS; i++) R.reg[i] = op.out_reg == i ? v : R.reg[i];
        } else {
            R.reg[OUT] = v;
        }
        if (op.out_col) op.out_col[R.grow] = v;
    }
}

template <class B, int NREGS, int BEGIN, int... KS, class RowT, int... IS>
__device__ __forceinline__ void run_steps1(const Launch &L, RowT &R, const uint32_t *bits,
                                           std::integer_sequence<int, IS...>)
{
    constexpr int kinds[] = {KS...};
    (step1<kinds[BEGIN + IS], B::a(BEGIN + IS), B::b(BEGIN + IS), B::out(BEGIN + IS)>(L.ops[BEGIN + IS], R, bits),
     ...);
}

// Adds the lane's row (when `row`) to the group-by (block table first, global
// on overflow) and runs the first-writer exchange; key(std::integral_constant
// <int, q>) gives the row's key q, nk the number of keys.  All 32 lanes of the warp call it (with row false where the
// lane holds none): the lanes that take part in the warp aggregation are
// named by a ballot over the full warp, never by the lanes that happen to
// be converged.
// Writes the first-writer's key values of slot sl: key(std::integral_constant
// <int, q>) gives key q.
template <class KeyFn, int... KK>
__device__ __forceinline__ void write_keys(const Launch &L, int nk, int64_t sl, KeyFn &key,
                                           std::integer_sequence<int, KK...>)
{
    ((KK < nk ? (void)(L.out_keys[KK][sl] = key(std::integral_constant<int, KK>{})) : (void)0), ...);
}

template <class KeyFn>
__device__ __forceinline__ void group_row(const Launch &L, uint32_t *s_key, unsigned long long *s_sum, bool direct,
                                          bool row, uint32_t h, int32_t value, int nk, KeyFn key)
{
    const int64_t sl = row ? sdb::group_slot(h, L.P) : 0;
    const bool bad = row && (sl < 0 || (uint64_t)sl >= L.P);
    if (bad) atomicAdd(&g_errors, 1ull);
    const bool go = row && !bad;
    const unsigned mask = __ballot_sync(0xffffffffu, go);
    if (!go) return;
    unsigned long long val = (unsigned long long)sdb::widen(value);
    // warp aggregation: lanes here with the same slot sum their values (exactly:
    // 16-bit halves reduced in 32 bits, then recombined in 64) and only the
    // lowest of them updates the table
    const unsigned peers = __match_any_sync(mask, (unsigned)sl);
    if (__popc(peers) > 1) {
        const uint32_t lo = __reduce_add_sync(peers, (uint32_t)value & 0xffffu);
        const int32_t hi = (int32_t)__reduce_add_sync(peers, (uint32_t)(value >> 16));
        if ((threadIdx.x & 31u) != (unsigned)(__ffs(peers) - 1)) return;
        val = (unsigned long long)((int64_t)hi * 65536 + (int64_t)lo);
    }
    bool first = false;
    if (smem_group_add<kDenseCap>(s_key, s_sum, (uint32_t)sl, val, direct, first)) {
        if (first) first = atomicExch(&L.occ[sl], 1u) == 0u;
    } else {
        first = L.occ[sl] == 0u && atomicExch(&L.occ[sl], 1u) == 0u;
        atomicAdd(reinterpret_cast<unsigned long long *>(&L.out_sum[sl]), val);
    }
    if (first) write_keys(L, nk, sl, key, std::make_integer_sequence<int, SDB_CHAIN_MAX_KEYS>{});
}

// SPLIT = number of ops run on 4-row groups; the rest run on the compacted
// rows.  SPLIT == sizeof...(KS) + 1 means no compaction (all ops dense, which
// also serves SDB_TERM_FLAGS).
template <int STAGES, int CARRY>
__host__ __device__ constexpr int dense_min_blocks() { return CARRY == 3 ? 5 : (STAGES >= 3 ? 3 : 5); }

// ---- pieces shared by the single-chain pass and the batched pass ----------

template <int TERM>
__device__ __forceinline__ void group_table_reset(uint32_t *s_key, unsigned long long *s_sum)
{
    if (TERM == T_GROUP)
        for (uint32_t i = threadIdx.x; i < kDenseCap; i += blockDim.x) {
            s_key[i] = kEmpty;
            s_sum[i] = 0;
        }
}

// Packs the chain's semi-join table into the shared-memory bitmap: word w
// holds entries 32w .. 32w + 31.
__device__ __forceinline__ void stage_bitmap(const Launch &L, uint32_t *s_bits)
{
    if (!L.bitmap_ht) return;
    const uint32_t words = (L.bitmap_len + 31) / 32;
    if (L.bitmap_kv) {  // a key/value table: entry j's occupancy word x == 1
        const int4 *q = reinterpret_cast<const int4 *>(L.bitmap_ht);  // two entries per int4
        for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) {
            uint32_t bits = 0;
            const uint32_t e0 = w * 32;
            if (e0 + 32 <= L.bitmap_len) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int4 v = __ldg(q + e0 / 2 + j);
                    bits |= ((uint32_t)(v.x == 1) | ((uint32_t)(v.z == 1) << 1)) << (2 * j);
                }
            } else {
                const int2 *e = reinterpret_cast<const int2 *>(L.bitmap_ht);
                for (uint32_t j = 0; j < 32 && e0 + j < L.bitmap_len; j++) bits |= (uint32_t)(e[e0 + j].x == 1) << j;
            }
            s_bits[w] = bits;
        }
        return;
    }
    for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) {
        uint32_t bits = 0;
        const uint32_t e0 = w * 32;
        if (e0 + 32 <= L.bitmap_len && sdb::aligned(L.bitmap_ht, 4)) {
            const uint32_t *q = reinterpret_cast<const uint32_t *>(L.bitmap_ht + e0);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const uint32_t x = __vcmpne4(__ldg(q + j), 0u);
                bits |= (((x >> 7) & 1u) | ((x >> 14) & 2u) | ((x >> 21) & 4u) | ((x >> 28) & 8u)) << (4 * j);
            }
        } else {
            for (uint32_t j = 0; j < 32 && e0 + j < L.bitmap_len; j++) bits |= (uint32_t)(L.bitmap_ht[e0 + j] != 0) << j;
        }
        s_bits[w] = bits;
    }
}

// Copies this thread's 4 rows of slot columns 0 .. nstaged-1 of `tile` (rows
// tile + 4t .. +3) into ring stage `st` (SS slots per stage); rows past the
// end are zero-filled or skipped.  Always commits one group (possibly empty) so every thread
// counts groups the same way.
template <int STAGES, int SS, int IT>
__device__ __forceinline__ void issue_tile(const int32_t *const *slot, int nstaged, uint64_t n, int4 *s_buf, int st,
                                           uint64_t tile)
{
    constexpr int kItems = IT, kQ = IT / 4;
    const uint64_t r0 = tile + (uint64_t)kItems * threadIdx.x;
#pragma unroll
    for (int q = 0; q < kQ; q++) {
        const uint64_t r = r0 + 4 * q;
        if (r < n) {
            const uint64_t left = n - r;
            const uint32_t bytes = left >= 4 ? 16u : (uint32_t)(left * 4);
#pragma unroll
            for (int sl = 0; sl < SS; sl++)
                if (sl < nstaged)
                    cp_async16(&s_buf[((st * SS + sl) * kThreads + threadIdx.x) * kQ + q], slot[sl] + r, bytes);
        }
    }
    cp_async_commit();
}

// One tile of one chain: the ops before SPLIT on 4-row groups, then (if
// SPLIT <= N) warp compaction and the remaining ops one row per lane, then
// the terminal into the block's partials.
// The terminal for one row held by one lane.
// The group slot hash of a row: sum over its keys of (key - min) * mult.
template <class B, class RowT, int... KK>
__device__ __forceinline__ uint32_t key_hash(const Launch &L, const RowT &R, int nk, std::integer_sequence<int, KK...>)
{
    uint32_t h = 0;
    ((h += KK < nk ? ((uint32_t)fetch1c<B::key(KK)>(L.keys[KK], R) - (uint32_t)L.key_min[KK]) * L.mults[KK] : 0u),
     ...);
    return h;
}

template <int TERM, class B, class RowT>
__device__ __forceinline__ void finish_row(const Launch &L, RowT &R, uint32_t *s_key, unsigned long long *s_sum,
                                           bool direct, uint64_t &acc)
{
    if (TERM == T_SUM) {
        if (R.live) acc += sdb::widen(fetch1c<B::value()>(L.value, R));
    } else if (TERM == T_GROUP) {
        // every lane of the warp reaches group_row (its warp aggregation
        // needs the whole warp); values of a lane without a live row are
        // read from its registers or staged rows and not used
        const int nk = B::n_keys() == kAny ? L.n_keys : B::n_keys();
        const uint32_t h = key_hash<B>(L, R, nk, std::make_integer_sequence<int, SDB_CHAIN_MAX_KEYS>{});
        auto key = [&R, &L](auto q) { return fetch1c<B::key(decltype(q)::value)>(L.keys[decltype(q)::value], R); };
        group_row(L, s_key, s_sum, direct, R.live, h, fetch1c<B::value()>(L.value, R), nk, key);
    }
}

// The ops from SPLIT on and the terminal, for one row held by one lane.
template <int TERM, class B, int NREGS, int SPLIT, int... KS, class RowT>
__device__ __forceinline__ void sparse_row(const Launch &L, RowT &R, const uint32_t *s_bits, uint32_t *s_key,
                                           unsigned long long *s_sum, bool direct, uint64_t &acc)
{
    constexpr int N = sizeof...(KS);
#pragma unroll
    for (int i = 0; i < NREGS; i++) R.reg[i] = 0;
    run_steps1<B, NREGS, SPLIT, KS...>(L, R, s_bits, std::make_integer_sequence<int, N - SPLIT>{});
    finish_row<TERM, B>(L, R, s_key, s_sum, direct, acc);
}


// Carried rows: a warp keeps the up to 31 surviving rows of a tile that do
// not fill a last group of 32 -- row j's tail-slot values in lane j's
// registers (`ce`) -- and runs them with the next tile's survivors, so the
// row-per-lane phase runs full warps.  drain runs what is left (at the end of
// a block's rows of a chain).
// Second compaction level (CARRY 2): the rows that survive the first
// row-per-lane op are moved, by warp shuffles, into a warp-wide group held in
// registers (lane j: pending row j) and the remaining ops run only on full
// groups of 32 -- for a star join, where ~4 % of the rows survive the part
// probe, the date probe and the group-by then run on full warps.
template <int NREGS>
struct Level2 {
    VRow<NREGS> r;   // lane j: pending row j
    uint32_t n = 0;  // pending rows (warp-uniform)
    uint8_t *src = nullptr;  // the warp's 32-entry list: entry k = lane of the k-th live row of a group
};

// Row k (0-based, k < cnt) among the warp's live rows, whose lanes the
// caller listed in src (entry k = lane of the k-th live row); every lane
// calls it with its own k (k >= cnt: no row).
template <int NREGS>
__device__ __forceinline__ VRow<NREGS> take_row(const VRow<NREGS> &R, const uint8_t *src_list, uint32_t k, uint32_t cnt)
{
    const int src = k < cnt ? (int)src_list[k] : 0;
    VRow<NREGS> o;
    o.v0 = __shfl_sync(0xffffffffu, R.v0, src);
    o.v1 = __shfl_sync(0xffffffffu, R.v1, src);
    o.v2 = __shfl_sync(0xffffffffu, R.v2, src);
    o.v3 = __shfl_sync(0xffffffffu, R.v3, src);
#pragma unroll
    for (int i = 0; i < NREGS; i++) o.reg[i] = __shfl_sync(0xffffffffu, R.reg[i], src);
    o.live = k < cnt;
    return o;
}

// The ops after the first row-per-lane op and the terminal, for the rows of
// a level-2 group (lane j: row j while F.live).  CARRY 3 first loads the late
// slots of each live row from its row number.
template <int TERM, class B, int NREGS, int SPLIT, int CARRY, int... KS>
__device__ __forceinline__ void level2_run(const Launch &L, VRow<NREGS> &F, const uint32_t *s_bits, uint32_t *s_key,
                                           unsigned long long *s_sum, bool direct, uint64_t &acc)
{
    constexpr int N = sizeof...(KS);
    if constexpr (CARRY == 3) {
        const uint32_t late = B::bound ? bound_late<B, TERM, SPLIT, KS...>() : L.late_slots;
        if (F.live) {
            if (late & 1u) F.v0 = __ldg(L.slot[0] + (uint32_t)F.v0);
            if (late & 2u) F.v1 = __ldg(L.slot[1] + (uint32_t)F.v1);
            if (late & 4u) F.v2 = __ldg(L.slot[2] + (uint32_t)F.v2);
            if (late & 8u) F.v3 = __ldg(L.slot[3] + (uint32_t)F.v3);
        }
    }
    run_steps1<B, NREGS, SPLIT + 1, KS...>(L, F, s_bits, std::make_integer_sequence<int, N - SPLIT - 1>{});
    finish_row<TERM, B>(L, F, s_key, s_sum, direct, acc);
}

// After the first row-per-lane op of a group: appends its live rows to the
// level-2 rows and runs the remaining ops whenever 32 are pending.
template <int TERM, class B, int NREGS, int SPLIT, int CARRY, int... KS>
__device__ __forceinline__ void level2_push(const Launch &L, const VRow<NREGS> &R, Level2<NREGS> &Q,
                                            const uint32_t *s_bits, uint32_t *s_key, unsigned long long *s_sum,
                                            bool direct, uint64_t &acc)
{
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned live = __ballot_sync(0xffffffffu, R.live);
    const uint32_t cnt = __popc(live);
    if (cnt == 0) return;
    // list the live lanes in order (each writes its own entry), so that every
    // lane finds the source of its row with one load
    if (R.live) Q.src[__popc(live & ((1u << lane) - 1u))] = (uint8_t)lane;
    __syncwarp();
    const uint32_t n2 = Q.n;
    {
        const uint32_t k = lane >= n2 ? lane - n2 : 32u;
        const VRow<NREGS> got = take_row(R, Q.src, k, cnt);
        if (lane >= n2 && k < cnt) Q.r = got;
    }
    if (n2 + cnt >= 32) {
        VRow<NREGS> F = Q.r;
        F.live = true;
        level2_run<TERM, B, NREGS, SPLIT, CARRY, KS...>(L, F, s_bits, s_key, s_sum, direct, acc);
        const uint32_t used = 32 - n2;
        const VRow<NREGS> got = take_row(R, Q.src, lane + used, cnt);
        if (lane < cnt - used) Q.r = got;
        Q.n = cnt - used;
    } else {
        Q.n = n2 + cnt;
    }
    __syncwarp();  // every lane has read the list before it is written again
}

// Whether CARRY 2 or 3 uses the second level: there are ops after the first
// row-per-lane op.
template <int SPLIT, int... KS>
__host__ __device__ constexpr bool use_level2(int carry)
{
    return carry >= 2 && SPLIT + 1 < (int)sizeof...(KS);
}

// The first row-per-lane op and then the second level, for one group.
template <int TERM, class B, int NREGS, int SPLIT, int CARRY, int... KS>
__device__ __forceinline__ void level2_group(const Launch &L, VRow<NREGS> &R, Level2<NREGS> &Q, const uint32_t *s_bits,
                                             uint32_t *s_key, unsigned long long *s_sum, bool direct, uint64_t &acc)
{
    constexpr int kinds[] = {KS...};
#pragma unroll
    for (int i = 0; i < NREGS; i++) R.reg[i] = 0;
    step1<kinds[SPLIT], B::a(SPLIT), B::b(SPLIT), B::out(SPLIT)>(L.ops[SPLIT], R, s_bits);
    level2_push<TERM, B, NREGS, SPLIT, CARRY, KS...>(L, R, Q, s_bits, s_key, s_sum, direct, acc);
}

// Runs whatever the warp still holds (at the end of a block's rows of a chain).
template <int TERM, class B, int NREGS, int SPLIT, int CARRY, int... KS>
__device__ __forceinline__ void drain_carry(const Launch &L, uint32_t &carry, const int4 &ce, Level2<NREGS> &Q,
                                            const uint32_t *s_bits, uint32_t *s_key, unsigned long long *s_sum,
                                            bool direct, uint64_t &acc)
{
    const uint32_t lane = threadIdx.x & 31u;
    if (carry) {
        const int4 e = ce;
        VRow<NREGS> R;
        R.v0 = e.x;
        R.v1 = e.y;
        R.v2 = e.z;
        R.v3 = e.w;
        R.live = lane < carry;
        if constexpr (use_level2<SPLIT, KS...>(CARRY))
            level2_group<TERM, B, NREGS, SPLIT, CARRY, KS...>(L, R, Q, s_bits, s_key, s_sum, direct, acc);
        else
            sparse_row<TERM, B, NREGS, SPLIT, KS...>(L, R, s_bits, s_key, s_sum, direct, acc);
    }
    carry = 0;
    if constexpr (use_level2<SPLIT, KS...>(CARRY)) {
        if (Q.n) {
            VRow<NREGS> F = Q.r;
            F.live = lane < Q.n;
            level2_run<TERM, B, NREGS, SPLIT, CARRY, KS...>(L, F, s_bits, s_key, s_sum, direct, acc);
        }
        Q.n = 0;
    }
    __syncwarp();
}

// What a compacted row keeps of slot s: its staged value when a later op
// reads the slot, or (CARRY 3, late slot) its row number, row0 + r.
template <int CARRY, class B, int TERM, int SPLIT, int SL, int... KS>
__device__ __forceinline__ int32_t tail_value(const Launch &L, const int32_t *ws, uint32_t r, uint64_t row0)
{
    if constexpr (B::bound) {
        constexpr uint32_t tail = bound_tail<B, TERM, SPLIT, KS...>();
        constexpr uint32_t late = CARRY == 3 ? bound_late<B, TERM, SPLIT, KS...>() : 0u;
        if constexpr (!((tail >> SL) & 1u)) return 0;
        else if constexpr ((late >> SL) & 1u) return (int32_t)(uint32_t)(row0 + r);
        else return ws[SL * items_of<CARRY>() * kThreads + r];
    } else {
        if (!((L.tail_slots >> SL) & 1u)) return 0;
        if (CARRY == 3 && ((L.late_slots >> SL) & 1u)) return (int32_t)(uint32_t)(row0 + r);
        return ws[SL * items_of<CARRY>() * kThreads + r];
    }
}

template <int TERM, class B, int NREGS, int SPLIT, int CARRY, int... KS>
__device__ __forceinline__ void tile_body(const Launch &L, State<NREGS, items_of<CARRY>()> &S, const int4 *s_buf, int st,
                                          uint64_t tile,
                                          uint8_t *s_list, uint32_t *s_key, unsigned long long *s_sum,
                                          const uint32_t *s_bits, bool direct, uint64_t &acc, uint32_t &carry,
                                          int4 &ce, Level2<NREGS> &Q)
{
    constexpr int N = sizeof...(KS);
    constexpr bool kCompact = SPLIT <= N;
    constexpr int kDenseOps = kCompact ? SPLIT : N;
    constexpr int kItems = items_of<CARRY>(), kQ = kItems / 4;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    constexpr int SS = stage_slots<CARRY>();
    S.stage = &s_buf[(st * SS * kThreads + threadIdx.x) * kQ];
    S.base = tile + (uint64_t)kItems * threadIdx.x;
    if (S.base + kItems <= L.n) {
        S.valid = (1u << kItems) - 1u;
    } else {
        S.valid = 0;
#pragma unroll
        for (int k = 0; k < kItems; k++) S.valid |= (uint32_t)(S.base + k < L.n) << k;
    }
    if (L.flags_in && S.valid) {
        uint32_t m = 0;
        if (kItems == 8 && S.valid == 0xffu && sdb::aligned(L.flags_in, 8)) {  // 8 flags in one load
            const uint64_t f = *reinterpret_cast<const uint64_t *>(L.flags_in + S.base);
#pragma unroll
            for (int k = 0; k < 8; k++) m |= (uint32_t)(((f >> (8 * k)) & 0xffu) != 0) << k;
        } else {
#pragma unroll
            for (int k = 0; k < kItems; k++)
                if ((S.valid >> k) & 1u) m |= (uint32_t)(L.flags_in[S.base + k] != 0) << k;
        }
        S.live = m;
    } else {
        S.live = S.valid;
    }
    run_steps<B, NREGS, 0, KS...>(L, S, std::make_integer_sequence<int, kDenseOps>{});

    if constexpr (kCompact) {
        // warp prefix sum of the live-row counts
        const uint32_t cnt = __popc(S.live);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint8_t *list = s_list + warp * 32 * kItems;
        uint32_t pos = incl - cnt;
#pragma unroll
        for (int k = 0; k < kItems; k++)
            if ((S.live >> k) & 1u) list[pos++] = (uint8_t)(lane * kItems + k);
        __syncwarp();
        const int32_t *ws = reinterpret_cast<const int32_t *>(&s_buf[(st * SS * kThreads + warp * 32) * kQ]);
        if constexpr (CARRY > 0) {
            // entries 0 .. carry-1 are the carried rows (entry j in lane j),
            // then this tile's survivors
            const uint32_t avail = carry + total;
            const uint64_t row0 = tile + (uint64_t)warp * 32 * kItems;  // row of the warp's staged row 0
            auto entry = [&](uint32_t idx) {
                VRow<NREGS> R;
                if (idx < carry) {  // only in the first group: idx == lane
                    R.v0 = ce.x;
                    R.v1 = ce.y;
                    R.v2 = ce.z;
                    R.v3 = ce.w;
                } else {
                    const uint32_t r = list[idx - carry];
                    R.v0 = tail_value<CARRY, B, TERM, SPLIT, 0, KS...>(L, ws, r, row0);
                    R.v1 = tail_value<CARRY, B, TERM, SPLIT, 1, KS...>(L, ws, r, row0);
                    R.v2 = tail_value<CARRY, B, TERM, SPLIT, 2, KS...>(L, ws, r, row0);
                    R.v3 = tail_value<CARRY, B, TERM, SPLIT, 3, KS...>(L, ws, r, row0);
                }
                R.live = true;
                return R;
            };
            uint32_t b = 0;
            for (; b + 32 <= avail; b += 32) {
                VRow<NREGS> R = entry(b + lane);
                if constexpr (use_level2<SPLIT, KS...>(CARRY))
                    level2_group<TERM, B, NREGS, SPLIT, CARRY, KS...>(L, R, Q, s_bits, s_key, s_sum, direct, acc);
                else
                    sparse_row<TERM, B, NREGS, SPLIT, KS...>(L, R, s_bits, s_key, s_sum, direct, acc);
            }
            const uint32_t rem = avail - b;
            if (lane < rem && b + lane >= carry) {  // carry a survivor of this tile
                const uint32_t r = list[b + lane - carry];
                ce.x = tail_value<CARRY, B, TERM, SPLIT, 0, KS...>(L, ws, r, row0);
                ce.y = tail_value<CARRY, B, TERM, SPLIT, 1, KS...>(L, ws, r, row0);
                ce.z = tail_value<CARRY, B, TERM, SPLIT, 2, KS...>(L, ws, r, row0);
                ce.w = tail_value<CARRY, B, TERM, SPLIT, 3, KS...>(L, ws, r, row0);
            }
            carry = rem;
            __syncwarp();
        } else {
            Row<NREGS, kItems> R;
            R.wstage = ws;
            for (uint32_t b = 0; b < total; b += 32) {
                const uint32_t idx = b + lane;
                R.live = idx < total;
                R.r = R.live ? list[idx] : 0;
                R.grow = tile + (uint64_t)warp * 32 * kItems + R.r;
                sparse_row<TERM, B, NREGS, SPLIT, KS...>(L, R, s_bits, s_key, s_sum, direct, acc);
            }
            __syncwarp();
        }
    } else {
        if (TERM == T_FLAGS || L.flags_out) {
#pragma unroll
            for (int k = 0; k < kItems; k++)
                if ((S.valid >> k) & 1u) L.flags_out[S.base + k] = (uint8_t)((S.live >> k) & 1u);
        }
        if (TERM == T_SUM && S.live) {
            int32_t v[kItems];
            fetch4(L.value, S, v);
#pragma unroll
            for (int k = 0; k < kItems; k++)
                if ((S.live >> k) & 1u) acc += sdb::widen(v[k]);
        } else if (TERM == T_GROUP && __any_sync(0xffffffffu, S.live != 0)) {
            // the whole warp runs the group-by of its items (group_row's
            // warp aggregation needs every lane); staged values of dead or
            // missing rows are read and not used
            int32_t v[kItems];
            fetch4(L.value, S, v);
            uint32_t h[kItems] = {};
#pragma unroll
            for (int kk = 0; kk < SDB_CHAIN_MAX_KEYS; kk++)
                if (kk < L.n_keys) {
                    int32_t kv[kItems];
                    fetch4(L.keys[kk], S, kv);
#pragma unroll
                    for (int k = 0; k < kItems; k++) h[k] += ((uint32_t)kv[k] - (uint32_t)L.key_min[kk]) * L.mults[kk];
                }
#pragma unroll
            for (int k = 0; k < kItems; k++)
                group_row(L, s_key, s_sum, direct, ((S.live >> k) & 1u) != 0, h[k], v[k], L.n_keys, [&](auto q) {
                    int32_t kv[kItems];
                    fetch4(L.keys[decltype(q)::value], S, kv);
                    return kv[k];
                });
        }
    }
}

// Flushes a block's partials of one chain into its global outputs: one
// 64-bit atomic per block for SUM, one per touched slot for group-by.  The
// caller synchronises the block before and (to reuse the table) after.
template <int TERM>
__device__ __forceinline__ void block_flush(const Launch &L, uint32_t *s_key, unsigned long long *s_sum,
                                            uint64_t *s_part, uint64_t &acc)
{
    if (TERM == T_SUM) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
        acc = 0;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t t = 0;
            for (int w = 0; w < kThreads / 32; w++) t += s_part[w];
            if (t) atomicAdd(reinterpret_cast<unsigned long long *>(L.sum_out), (unsigned long long)t);
        }
    } else if (TERM == T_GROUP) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < kDenseCap; i += blockDim.x) {
            const uint32_t k = s_key[i];
            if (k != kEmpty) atomicAdd(reinterpret_cast<unsigned long long *>(&L.out_sum[k]), s_sum[i]);
        }
    }
}

template <class B, int TERM, int NREGS, int STAGES, int SPLIT, int CARRY, int... KS>
__global__ void __launch_bounds__(kThreads, dense_min_blocks<STAGES, CARRY>()) k_dense(const __grid_constant__ Launch L)
{
    constexpr int kStages = STAGES;
    constexpr bool kCompact = SPLIT <= (int)sizeof...(KS);
    constexpr int kItems = items_of<CARRY>(), kQ = kItems / 4;
    constexpr int SS = stage_slots<CARRY>();
    extern __shared__ int4 s_buf[];  // [kStages][SS][kThreads][kQ], then the semi-join bitmap
    __shared__ uint32_t s_key[TERM == T_GROUP ? kDenseCap : 1];
    __shared__ unsigned long long s_sum[TERM == T_GROUP ? kDenseCap : 1];
    __shared__ uint8_t s_list[kCompact ? kThreads * kItems : 1];  // per warp: 32 x kItems row offsets
    __shared__ uint64_t s_part[kThreads / 32];
    __shared__ uint8_t s_l2src[CARRY >= 2 ? kThreads : 1];
    uint32_t carry = 0;  // rows the warp carries (warp-uniform)
    int4 ce = make_int4(0, 0, 0, 0);
    Level2<NREGS> Q;
    Q.src = s_l2src + (CARRY >= 2 ? (threadIdx.x & ~31u) : 0u);
    const bool direct = L.P <= kDenseCap;
    uint32_t *s_bits = reinterpret_cast<uint32_t *>(s_buf + kStages * SS * kThreads * kQ);
    constexpr uint64_t kTile = (uint64_t)kThreads * kItems;
    const uint64_t stride = (uint64_t)gridDim.x * kTile;
    uint64_t tile = (uint64_t)blockIdx.x * kTile;
    // the first tiles' copies go out before the group table and the bitmap
    // are set up (the ring lies before the bitmap in shared memory), so
    // their DRAM latency overlaps the bitmap's L2 reads
#pragma unroll
    for (int p = 0; p < kStages - 1; p++) issue_tile<kStages, SS, kItems>(L.slot, L.nstaged, L.n, s_buf, p, tile + p * stride);
    group_table_reset<TERM>(s_key, s_sum);
    stage_bitmap(L, s_bits);
    if (TERM == T_GROUP || L.bitmap_ht) __syncthreads();

    State<NREGS, kItems> S;
    S.bits = s_bits;
#pragma unroll
    for (int r = 0; r < NREGS; r++)
#pragma unroll
        for (int k = 0; k < kItems; k++) S.reg[r][k] = 0;
    uint64_t acc = 0;

    int st = 0;
    for (; tile < L.n; tile += stride) {
        issue_tile<kStages, SS, kItems>(L.slot, L.nstaged, L.n, s_buf, (st + kStages - 1) % kStages,
                                tile + (kStages - 1) * stride);
        cp_async_wait<kStages - 1>();
        tile_body<TERM, B, NREGS, SPLIT, CARRY, KS...>(L, S, s_buf, st, tile, s_list, s_key, s_sum, s_bits, direct, acc,
                                                   carry, ce, Q);
        st = (st + 1) % kStages;
    }
    cp_async_wait<0>();
    if constexpr (CARRY > 0)
        drain_carry<TERM, B, NREGS, SPLIT, CARRY, KS...>(L, carry, ce, Q, s_bits, s_key, s_sum, direct, acc);
    block_flush<TERM>(L, s_key, s_sum, s_part, acc);
}

// Paired pass: two chains of one bound shape whose staged slots are the same
// columns over the same rows (two plans of a batch that scan the same fact
// rows with their own literals and tables).  Each tile is copied into the
// ring once and both chains run on it, each with its own group table,
// bitmap, carried rows and second-level rows; late columns are each chain's
// own.  The host checks that the staged slots, row count and incoming flags
// (none) agree.
constexpr int kPair = 2;
struct LaunchPair {
    Launch L[kPair];
    uint32_t bits_off[kPair];  // each chain's bitmap: its first word after the ring
};

template <class B, int TERM, int NREGS, int STAGES, int SPLIT, int CARRY, int... KS>
__global__ void __launch_bounds__(kThreads, 4) k_dense_pair(const __grid_constant__ LaunchPair P)
{
    static_assert(B::bound && CARRY == 3, "the paired pass runs the bound carry-3 shapes");
    constexpr int kStages = STAGES;
    constexpr bool kCompact = SPLIT <= (int)sizeof...(KS);
    constexpr int kItems = items_of<CARRY>(), kQ = kItems / 4;
    constexpr int SS = stage_slots<CARRY>();
    extern __shared__ int4 s_buf[];  // [kStages][SS][kThreads][kQ], then the chains' bitmaps
    __shared__ uint32_t s_key[kPair][TERM == T_GROUP ? kDenseCap : 1];
    __shared__ unsigned long long s_sum[kPair][TERM == T_GROUP ? kDenseCap : 1];
    __shared__ uint8_t s_list[kCompact ? kThreads * kItems : 1];  // reused by the chains in turn
    __shared__ uint64_t s_part[kThreads / 32];
    __shared__ uint8_t s_l2src[kPair][kThreads];
    const Launch &L0 = P.L[0];  // the staged slots, row count and tiles are L0's (and L1's)
    uint32_t carry[kPair];
    int4 ce[kPair];
    Level2<NREGS> Q[kPair];
    bool direct[kPair];
    uint64_t acc[kPair];
    uint32_t *s_bits[kPair];
    uint32_t *ring_end = reinterpret_cast<uint32_t *>(s_buf + kStages * SS * kThreads * kQ);
#pragma unroll
    for (int c = 0; c < kPair; c++) {
        carry[c] = 0;
        ce[c] = make_int4(0, 0, 0, 0);
        Q[c].src = s_l2src[c] + (threadIdx.x & ~31u);
        direct[c] = P.L[c].P <= kDenseCap;
        acc[c] = 0;
        s_bits[c] = ring_end + P.bits_off[c];
    }
    constexpr uint64_t kTile = (uint64_t)kThreads * kItems;
    const uint64_t stride = (uint64_t)gridDim.x * kTile;
    uint64_t tile = (uint64_t)blockIdx.x * kTile;
#pragma unroll
    for (int p = 0; p < kStages - 1; p++)
        issue_tile<kStages, SS, kItems>(L0.slot, L0.nstaged, L0.n, s_buf, p, tile + p * stride);
#pragma unroll
    for (int c = 0; c < kPair; c++) {
        group_table_reset<TERM>(s_key[c], s_sum[c]);
        stage_bitmap(P.L[c], s_bits[c]);
    }
    __syncthreads();

    State<NREGS, kItems> S;
#pragma unroll
    for (int r = 0; r < NREGS; r++)
#pragma unroll
        for (int k = 0; k < kItems; k++) S.reg[r][k] = 0;

    int st = 0;
    for (; tile < L0.n; tile += stride) {
        issue_tile<kStages, SS, kItems>(L0.slot, L0.nstaged, L0.n, s_buf, (st + kStages - 1) % kStages,
                                        tile + (kStages - 1) * stride);
        cp_async_wait<kStages - 1>();
#pragma unroll
        for (int c = 0; c < kPair; c++) {
            S.bits = s_bits[c];
            tile_body<TERM, B, NREGS, SPLIT, CARRY, KS...>(P.L[c], S, s_buf, st, tile, s_list, s_key[c], s_sum[c],
                                                           s_bits[c], direct[c], acc[c], carry[c], ce[c], Q[c]);
        }
        st = (st + 1) % kStages;
    }
    cp_async_wait<0>();
#pragma unroll
    for (int c = 0; c < kPair; c++)
        drain_carry<TERM, B, NREGS, SPLIT, CARRY, KS...>(P.L[c], carry[c], ce[c], Q[c], s_bits[c], s_key[c], s_sum[c],
                                                         direct[c], acc[c]);
#pragma unroll
    for (int c = 0; c < kPair; c++) {
        if (c) __syncthreads();  // the first flush has read s_part
        block_flush<TERM>(P.L[c], s_key[c], s_sum[c], s_part, acc[c]);
    }
}

// A run of consecutive tiles of one chain: the unit the batched pass pulls
// from its work queue.
struct Span {
    uint32_t chain, t0, t1, pad;
};

// Batched pass: one persistent launch over many chains of one shape.  Blocks
// pull spans from a device work queue (one 32-bit head counter, zero before
// the launch) until it runs dry; nothing waits on anything.  The current
// chain's descriptor lives in shared memory; when a block's next span belongs
// to another chain it flushes the previous chain's partials, then loads the
// new descriptor, resets its group table and re-stages the semi-join bitmap.
// Within a span the tiles go through the same cp.async ring as the
// single-chain pass.
template <class B, int TERM, int NREGS, int STAGES, int SPLIT, int CARRY, int... KS>
__global__ void __launch_bounds__(kThreads, dense_min_blocks<STAGES, CARRY>())
    k_batch(const Launch *__restrict__ launches, const Span *__restrict__ spans, uint32_t n_spans,
            uint32_t *__restrict__ head)
{
    __shared__ uint8_t s_l2src[CARRY >= 2 ? kThreads : 1];
    uint32_t carry = 0;
    int4 ce = make_int4(0, 0, 0, 0);
    Level2<NREGS> Q;
    Q.src = s_l2src + (CARRY >= 2 ? (threadIdx.x & ~31u) : 0u);
    constexpr int kStages = STAGES;
    constexpr bool kCompact = SPLIT <= (int)sizeof...(KS);
    constexpr int kItems = items_of<CARRY>(), kQ = kItems / 4;
    constexpr uint64_t kTile = (uint64_t)kThreads * kItems;
    extern __shared__ int4 s_buf[];
    __shared__ uint32_t s_key[TERM == T_GROUP ? kDenseCap : 1];
    __shared__ unsigned long long s_sum[TERM == T_GROUP ? kDenseCap : 1];
    __shared__ uint8_t s_list[kCompact ? kThreads * kItems : 1];
    __shared__ uint64_t s_part[kThreads / 32];
    __shared__ Launch s_L;
    __shared__ uint32_t s_next;
    constexpr int SS = stage_slots<CARRY>();
    uint32_t *s_bits = reinterpret_cast<uint32_t *>(s_buf + kStages * SS * kThreads * kQ);

    State<NREGS, kItems> S;
    S.bits = s_bits;
#pragma unroll
    for (int r = 0; r < NREGS; r++)
#pragma unroll
        for (int k = 0; k < kItems; k++) S.reg[r][k] = 0;
    uint64_t acc = 0;
    uint32_t cur = ~0u;

    for (;;) {
        if (threadIdx.x == 0) s_next = atomicAdd(head, 1u);
        __syncthreads();
        const uint32_t sp = s_next;
        __syncthreads();  // every thread has read s_next before thread 0 writes it again
        if (sp >= n_spans) break;
        const Span span = spans[sp];
        if (span.chain != cur) {
            if (cur != ~0u) block_flush<TERM>(s_L, s_key, s_sum, s_part, acc);
            __syncthreads();
            const uint32_t *src = reinterpret_cast<const uint32_t *>(&launches[span.chain]);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&s_L);
            for (uint32_t w = threadIdx.x; w < sizeof(Launch) / 4; w += blockDim.x) dst[w] = src[w];
            group_table_reset<TERM>(s_key, s_sum);
            __syncthreads();
            stage_bitmap(s_L, s_bits);
            __syncthreads();
            cur = span.chain;
        }
        const bool direct = s_L.P <= kDenseCap;
        const uint64_t n = s_L.n;
#pragma unroll
        for (int p = 0; p < kStages - 1; p++) {
            const uint32_t t = span.t0 + p;
            if (t < span.t1) issue_tile<kStages, SS, kItems>(s_L.slot, s_L.nstaged, n, s_buf, p, (uint64_t)t * kTile);
            else cp_async_commit();
        }
        int st = 0;
        for (uint32_t t = span.t0; t < span.t1; t++) {
            const uint32_t tn = t + kStages - 1;
            if (tn < span.t1)
                issue_tile<kStages, SS, kItems>(s_L.slot, s_L.nstaged, n, s_buf, (st + kStages - 1) % kStages,
                                        (uint64_t)tn * kTile);
            else cp_async_commit();
            cp_async_wait<kStages - 1>();
            tile_body<TERM, B, NREGS, SPLIT, CARRY, KS...>(s_L, S, s_buf, st, (uint64_t)t * kTile, s_list, s_key, s_sum,
                                                       s_bits, direct, acc, carry, ce, Q);
            st = (st + 1) % kStages;
        }
        cp_async_wait<0>();
        // parked rows belong to this span's chain: run them before the next pull
        if constexpr (CARRY > 0)
            drain_carry<TERM, B, NREGS, SPLIT, CARRY, KS...>(s_L, carry, ce, Q, s_bits, s_key, s_sum, direct, acc);
    }
    if (cur != ~0u) block_flush<TERM>(s_L, s_key, s_sum, s_part, acc);
}

// Launches of the specialised passes, and of those the bound ones (host
// counters, read by sdb_fused_launch_counts).
std::atomic<uint64_t> g_dense_launches{0}, g_bound_launches{0};

template <class B, int TERM, int NREGS, int STAGES, int SPLIT, int CARRY, int... KS>
int launch_stages(const Launch &L, cudaStream_t s)
{
    auto kern = k_dense<B, TERM, NREGS, STAGES, SPLIT, CARRY, KS...>;
    const int ring = STAGES * stage_slots<CARRY>() * kThreads * (items_of<CARRY>() / 4) * (int)sizeof(int4);
    const int smem = ring + (L.bitmap_ht ? (int)(((L.bitmap_len + 31) / 32) * 4) : 0);
    static const bool attr = [&] {  // once per instantiation, thread-safe
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ring + (int)(kBitmapMax / 8));
        return true;
    }();
    (void)attr;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const uint64_t tile = (uint64_t)kThreads * items_of<CARRY>();
    uint64_t blocks = (L.n + tile - 1) / tile;
    const uint64_t cap = (uint64_t)num_sms() * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(L);
    g_dense_launches.fetch_add(1, std::memory_order_relaxed);
    if (B::bound) g_bound_launches.fetch_add(1, std::memory_order_relaxed);
    return sdb_check_launch("sdb_fused_chain (dense)");
}

// Ring stages 3 or 2; rows carried between tiles (carry 1; 2: and the second
// compaction level) only with compaction and a 2-stage ring; carry 3 (as 2,
// and late slots) with a 2-stage ring of two slots and 8-row tiles per thread,
// for a launch that prepare_late accepted.
template <class B, int TERM, int NREGS, int SPLIT, int... KS>
int launch(const Launch &L, int stages, int carry, cudaStream_t s)
{
    constexpr bool kCompact = SPLIT <= (int)sizeof...(KS);
    constexpr bool kLate = kCompact && use_level2<SPLIT, KS...>(3);
    if constexpr (B::bound || SPLIT == 0) {  // bound and SPLIT-0 passes are carry-3 passes
        static_assert(kLate, "a bound shape needs the second level");
        return launch_stages<B, TERM, NREGS, 2, SPLIT, 3, KS...>(L, s);
    } else {
        if (kLate && carry == 3) return launch_stages<Dyn, TERM, NREGS, 2, SPLIT, kLate ? 3 : 0, KS...>(L, s);
        if (stages >= 3) return launch_stages<Dyn, TERM, NREGS, 3, SPLIT, 0, KS...>(L, s);
        if (kCompact && carry >= 2) return launch_stages<Dyn, TERM, NREGS, 2, SPLIT, kCompact ? 2 : 0, KS...>(L, s);
        if (kCompact && carry == 1) return launch_stages<Dyn, TERM, NREGS, 2, SPLIT, kCompact ? 1 : 0, KS...>(L, s);
        return launch_stages<Dyn, TERM, NREGS, 2, SPLIT, 0, KS...>(L, s);
    }
}

// Slot bit of an operand (bit s: column slot s), and the slots an op reads.
inline uint32_t slot_bit(const Src &x) { return x.src == 0 ? (1u << x.idx) : 0u; }
inline uint32_t op_slots(const Op &o)
{
    if (o.kind == SDB_OP_FILL) return 0;
    const bool uses_b = o.kind == SDB_OP_SELECT || o.kind == SDB_OP_BINOP;
    return slot_bit(o.a) | (uses_b ? slot_bit(o.b) : 0u);
}

// Chains of two or three full probes (a star join whose dimensions all give
// values, e.g. SSB flight 3): the probe whose table is the smallest (at most
// kBitmapMax entries, 16-byte aligned) is first tested against a
// shared-memory bitmap of its table's occupancy, the other probes run on the
// rows that pass, and the tested probe runs again right after the first of
// them, for its value (a hit, by the test).  The same rows survive and every
// register gets the same value, so results do not change; the probes of the
// rows the bitmap rejects are skipped, and the first op becomes a bitmap test
// the passes can compact after.
void prefilter_by_bitmap(Launch &D, int terminal)
{
    if (terminal == SDB_TERM_FLAGS || D.flags_out || D.bitmap_ht || D.n_ops < 2 || D.n_ops > 3) return;
    int j = -1;
    uint64_t best = ~0ull;
    for (int i = 0; i < D.n_ops; i++) {
        const Op &o = D.ops[i];
        if (o.kind != SDB_OP_FULL_PROBE || o.out_col || o.a.src != 0) return;
        const uint64_t len = (uint64_t)((int64_t)o.hi - (int64_t)o.lo + 1);
        if (len >= 1 && len <= kBitmapMax && sdb::aligned(o.ht, 16) && len < best) {
            best = len;
            j = i;
        }
    }
    if (j < 0) return;
    Op ops[kMaxOps];
    int n = 0;
    ops[n] = D.ops[j];
    ops[n].kind = SDB_OP_SEMI_PROBE;
    ops[n].smem_bits = 1;
    n++;
    bool again = false;
    for (int i = 0; i < D.n_ops; i++) {
        if (i == j) continue;
        ops[n++] = D.ops[i];
        if (!again) {
            ops[n++] = D.ops[j];
            again = true;
        }
    }
    for (int i = 0; i < n; i++) D.ops[i] = ops[i];
    D.n_ops = n;
    D.bitmap_ht = static_cast<const uint8_t *>(D.ops[0].ht);
    D.bitmap_len = (uint32_t)best;
    D.bitmap_kv = 1;
}

// Converts a checked chain into a dense launch.  Returns false when the chain
// reads more than kSlots distinct columns, has too many ops or registers.
bool convert(const ChainLaunch &C, int nregs, Launch &D)
{
    const sdb_chain_desc &c = C.d;
    if (c.n_ops > kMaxOps || nregs > 4) return false;
    std::memset(&D, 0, sizeof D);
    D.nregs = nregs;
    D.n = c.n;
    D.flags_in = c.flags_in;
    D.flags_out = c.flags_out;
    D.n_ops = c.n_ops;
    auto map = [&](const sdb_operand &o, Src &out) -> bool {
        out.src = o.kind == SDB_SRC_COL ? 0 : (o.kind == SDB_SRC_REG ? 1 : 2);
        out.lit = o.lit;
        out.idx = o.reg;
        if (o.kind == SDB_SRC_COL) {
            int i = 0;
            while (i < D.nslot && D.slot[i] != o.col) i++;
            if (i == D.nslot) {
                if (D.nslot == kSlots || !sdb::aligned(o.col, 16)) return false;
                D.slot[D.nslot++] = o.col;
            }
            out.idx = i;
        }
        return true;
    };
    for (int k = 0; k < c.n_ops; k++) {
        const sdb_chain_op &o = c.ops[k];
        Op &d = D.ops[k];
        d.kind = o.kind;
        d.cmp = o.cmp_op;
        d.logic = o.logic_op;
        d.bin = o.bin_op;
        d.lo = o.lo;
        d.hi = o.hi;
        d.out_reg = o.out_reg;
        d.ht = o.ht;
        d.out_col = o.out_col;
        // open-addressing tables go through the general pass
        if ((o.kind == SDB_OP_SEMI_PROBE || o.kind == SDB_OP_FULL_PROBE) && o.ht_log2) return false;
        if (o.kind == SDB_OP_SEMI_PROBE && !D.bitmap_ht) {
            const uint64_t len = (uint64_t)((int64_t)o.hi - (int64_t)o.lo + 1);
            if (len >= 1 && len <= kBitmapMax) {
                D.bitmap_ht = static_cast<const uint8_t *>(o.ht);
                D.bitmap_len = (uint32_t)len;
                d.smem_bits = 1;
            }
        }
        const bool uses_b = o.kind == SDB_OP_SELECT || o.kind == SDB_OP_BINOP;
        if (o.kind != SDB_OP_FILL && !map(o.a, d.a)) return false;
        if (o.kind == SDB_OP_FILL) { d.a.src = 2; d.a.lit = o.a.lit; }
        if (uses_b && !map(o.b, d.b)) return false;
    }
    if (c.terminal != SDB_TERM_FLAGS && !map(c.value, D.value)) return false;
    D.sum_out = c.sum_out;
    if (c.terminal == SDB_TERM_GROUPBY) {
        D.n_keys = c.n_keys;
        for (int j = 0; j < c.n_keys; j++) {
            if (!map(c.keys[j], D.keys[j])) return false;
            D.key_min[j] = c.key_min[j];
            D.mults[j] = C.mults[j];
            D.out_keys[j] = c.out_keys[j];
        }
    }
    D.P = c.P;
    D.out_sum = c.out_sum;
    D.occ = c.occ;
    prefilter_by_bitmap(D, c.terminal);
    // slots a row still needs after the first op
    D.tail_slots = 0;
    for (int k = 1; k < D.n_ops; k++) D.tail_slots |= op_slots(D.ops[k]);
    if (c.terminal != SDB_TERM_FLAGS) D.tail_slots |= slot_bit(D.value);
    for (int j = 0; j < D.n_keys; j++) D.tail_slots |= slot_bit(D.keys[j]);
    D.late_slots = 0;
    D.nstaged = D.nslot;
    return true;
}

// Late slots of a chain whose ops from SPLIT on run on compacted rows with
// the second level: the tail slots that neither the ops on 4-row groups nor
// the first row-per-lane op read.  None when a row number does not fit 31
// bits.
template <int SPLIT>
uint32_t late_slots_of(const Launch &D)
{
    if (D.n >= (1ull << 31)) return 0;
    uint32_t early = 0;
    for (int k = 0; k <= SPLIT && k < D.n_ops; k++) early |= op_slots(D.ops[k]);
    return D.tail_slots & ~early;
}

// Whether the ops from index `split` on can run on compacted rows: no flags
// output, and every later op only keeps or clears a row's flag (no NONE/OR
// selection, no literal fill); ops before the split produce no register.
bool can_compact(const Launch &D, int term, int split)
{
    if (term == T_FLAGS || D.flags_out || split < 0 || split > D.n_ops) return false;
    for (int i = 0; i < D.n_ops; i++) {
        const Op &o = D.ops[i];
        const bool makes_reg = o.kind == SDB_OP_FULL_PROBE || o.kind == SDB_OP_BINOP || o.kind == SDB_OP_FILL;
        if (i < split && makes_reg) return false;
        if (i >= split) {
            if (o.kind == SDB_OP_FILL) return false;
            if ((o.kind == SDB_OP_SELECT || o.kind == SDB_OP_SEARCH_RANGE || o.kind == SDB_OP_SEARCH_POINTS) &&
                o.logic != SDB_AND)
                return false;
        }
    }
    return true;
}

// Whether compacted rows can be carried from one tile to the next: besides
// compaction after the first op (or, with incoming flags, before it), no op
// after it writes a column (a carried row keeps its slot values, not its row
// number).
bool can_carry(const Launch &D, int term)
{
    for (int i = 1; i < D.n_ops; i++)
        if (D.ops[i].out_col) return false;
    if (can_compact(D, term, 1)) return true;
    // or compaction on the incoming flags, before the first op (which then
    // writes no column either)
    return D.flags_in && !D.ops[0].out_col && can_compact(D, term, 0);
}

// Whether D's operands are exactly binding B's (and the slot masks the bound
// pass derives from it match the launch's), so the bound pass reads what the
// launch means.
template <class B, int TERM, int SPLIT, int... KS>
bool bound_ok(const Launch &D)
{
    constexpr int kinds[] = {KS...};
    constexpr int N = sizeof...(KS);
    auto code = [](const Src &x) { return x.src == 0 ? bslot(x.idx) : (x.src == 1 ? breg(x.idx) : kLitCode); };
    if (D.n_ops != N) return false;
    for (int i = 0; i < N; i++) {
        const Op &o = D.ops[i];
        const int k = kinds[i];
        if (o.kind != k) return false;
        if (k != SDB_OP_FILL && code(o.a) != B::a(i)) return false;
        if ((k == SDB_OP_SELECT || k == SDB_OP_BINOP) && code(o.b) != B::b(i)) return false;
        if ((k == SDB_OP_FULL_PROBE || k == SDB_OP_BINOP || k == SDB_OP_FILL) && o.out_reg != B::out(i)) return false;
    }
    if (TERM != T_FLAGS && code(D.value) != B::value()) return false;
    if (TERM == T_GROUP) {
        if (D.n_keys != B::n_keys()) return false;
        for (int q = 0; q < D.n_keys; q++)
            if (code(D.keys[q]) != B::key(q)) return false;
    }
    constexpr uint32_t late = bound_late<B, TERM, SPLIT, KS...>();
    const uint32_t all = (1u << D.nslot) - 1u, staged = (1u << D.nstaged) - 1u;
    return D.tail_slots == bound_tail<B, TERM, SPLIT, KS...>() && D.late_slots == late && late == (all & ~staged);
}

// Calls f.run<B, TERM, NREGS, SPLIT, KS...>() for the instantiation that
// matches D, or returns SDB_ERR_UNSUPPORTED (without calling f).  `compact`:
// 1 = compact after the first op when allowed; `bind`: a hot shape whose
// operands match its canonical binding takes the bound pass (B), else B is
// Dyn (only carry-3 launches, readied by prepare_late, bind).
template <class F>
int with_shape(const Launch &D, int term, int compact, F &f, bool bind = false)
{
    int k[kMaxOps];
    for (int i = 0; i < D.n_ops; i++) k[i] = D.ops[i].kind;
    const int n = D.n_ops;
    const bool c1 = compact && can_compact(D, term, 1);
    // r2: the chain fits the 2-register instantiations (the flight-3 and
    // flight-4 ones have 4)
    const bool r2 = D.nregs <= 2;
    // star join: semi + full + full -> group-by (SSB flight 2)
    if (r2 && term == T_GROUP && n == 3 && k[0] == SDB_OP_SEMI_PROBE && k[1] == SDB_OP_FULL_PROBE &&
        k[2] == SDB_OP_FULL_PROBE) {
        if (c1 && bind && bound_ok<StarBind, T_GROUP, 1, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE>(D))
            return f.template run<StarBind, T_GROUP, 2, 1, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE>();
        return c1 ? f.template run<Dyn, T_GROUP, 2, 1, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE>()
                  : f.template run<Dyn, T_GROUP, 2, 4, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE>();
    }
    // two semi probes -> flags (the flag-only front of a chain split in two)
    if (r2 && term == T_FLAGS && n == 2 && k[0] == SDB_OP_SEMI_PROBE && k[1] == SDB_OP_SEMI_PROBE)
        return f.template run<Dyn, T_FLAGS, 2, 3, SDB_OP_SEMI_PROBE, SDB_OP_SEMI_PROBE>();
    // full + full + projection -> group-by (SSB flight 4 after its semi joins);
    // under carry 3 (bind), with incoming flags, the rows are compacted on
    // those flags before the first probe (SPLIT 0)
    if (D.nregs <= 4 && term == T_GROUP && n == 3 && k[0] == SDB_OP_FULL_PROBE && k[1] == SDB_OP_FULL_PROBE &&
        k[2] == SDB_OP_BINOP) {
        if (bind && compact && D.flags_in && can_compact(D, term, 0)) {
            if (bound_ok<Flight4Bind, T_GROUP, 0, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>(D))
                return f.template run<Flight4Bind, T_GROUP, 4, 0, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>();
            return f.template run<Dyn, T_GROUP, 4, 0, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>();
        }
        return f.template run<Dyn, T_GROUP, 4, 4, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>();
    }
    // full + full -> group-by
    if (r2 && term == T_GROUP && n == 2 && k[0] == SDB_OP_FULL_PROBE && k[1] == SDB_OP_FULL_PROBE)
        return f.template run<Dyn, T_GROUP, 2, 3, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE>();
    // three full probes, the smallest table pre-tested by its bitmap
    // (prefilter_by_bitmap) -> three-key group-by (SSB flight 3)
    if (D.nregs <= 4 && term == T_GROUP && n == 4 && k[0] == SDB_OP_SEMI_PROBE && k[1] == SDB_OP_FULL_PROBE &&
        k[2] == SDB_OP_FULL_PROBE && k[3] == SDB_OP_FULL_PROBE) {
        if (c1 && bind &&
            bound_ok<Flight3Bind, T_GROUP, 1, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE>(D))
            return f.template run<Flight3Bind, T_GROUP, 4, 1, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE,
                                  SDB_OP_FULL_PROBE>();
        return c1 ? f.template run<Dyn, T_GROUP, 4, 1, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE,
                                   SDB_OP_FULL_PROBE>()
                  : f.template run<Dyn, T_GROUP, 4, 5, SDB_OP_SEMI_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE,
                                   SDB_OP_FULL_PROBE>();
    }
    // three full probes -> three-key group-by (none of the tables small enough for a bitmap)
    if (D.nregs <= 4 && term == T_GROUP && n == 3 && k[0] == SDB_OP_FULL_PROBE && k[1] == SDB_OP_FULL_PROBE &&
        k[2] == SDB_OP_FULL_PROBE)
        return f.template run<Dyn, T_GROUP, 4, 4, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE, SDB_OP_FULL_PROBE>();
    // range filter + one join + projection -> group-by
    if (r2 && term == T_GROUP && n == 3 && k[0] == SDB_OP_SEARCH_RANGE && k[1] == SDB_OP_FULL_PROBE &&
        k[2] == SDB_OP_BINOP) {
        if (c1 && bind && bound_ok<DateJoinBind, T_GROUP, 1, SDB_OP_SEARCH_RANGE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>(D))
            return f.template run<DateJoinBind, T_GROUP, 2, 1, SDB_OP_SEARCH_RANGE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>();
        return c1 ? f.template run<Dyn, T_GROUP, 2, 1, SDB_OP_SEARCH_RANGE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>()
                  : f.template run<Dyn, T_GROUP, 2, 4, SDB_OP_SEARCH_RANGE, SDB_OP_FULL_PROBE, SDB_OP_BINOP>();
    }
    // filter-project-sum (SSB flight 1)
    if (r2 && term == T_SUM && n == 4 && k[0] == SDB_OP_SEARCH_RANGE && k[1] == SDB_OP_SEARCH_RANGE &&
        k[2] == SDB_OP_SELECT && k[3] == SDB_OP_BINOP) {
        if (c1 && bind &&
            bound_ok<FilterSumBind, T_SUM, 1, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE, SDB_OP_SELECT, SDB_OP_BINOP>(D))
            return f.template run<FilterSumBind, T_SUM, 2, 1, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE, SDB_OP_SELECT,
                                  SDB_OP_BINOP>();
        return c1 ? f.template run<Dyn, T_SUM, 2, 1, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE, SDB_OP_SELECT, SDB_OP_BINOP>()
                  : f.template run<Dyn, T_SUM, 2, 5, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE, SDB_OP_SELECT, SDB_OP_BINOP>();
    }
    if (r2 && term == T_SUM && n == 4 && k[0] == SDB_OP_SEARCH_RANGE && k[1] == SDB_OP_SEARCH_RANGE &&
        k[2] == SDB_OP_SEARCH_RANGE && k[3] == SDB_OP_BINOP)
        return c1 ? f.template run<Dyn, T_SUM, 2, 1, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE,
                                   SDB_OP_BINOP>()
                  : f.template run<Dyn, T_SUM, 2, 5, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE, SDB_OP_SEARCH_RANGE,
                                   SDB_OP_BINOP>();
    return SDB_ERR_UNSUPPORTED;
}

struct LateProbe {
    Launch &D;
    template <class B, int TERM, int NREGS, int SPLIT, int... KS>
    int run()
    {
        constexpr bool kLate = SPLIT <= (int)sizeof...(KS) && use_level2<SPLIT, KS...>(3);
        if (SPLIT == 0 && kLate) D.tail_slots |= op_slots(D.ops[0]);  // rows compacted before the first op
        D.late_slots = kLate ? late_slots_of<SPLIT>(D) : 0u;
        return SDB_OK;
    }
};

// Fills D.late_slots for the instantiation with_shape picks with compaction.
void set_late_slots(Launch &D, int term)
{
    LateProbe p{D};
    if (with_shape(D, term, 1, p, true) != SDB_OK) D.late_slots = 0;
}

// Readies D for carry 3: finds its late slots and renumbers the slots so the
// staged ones come first (every operand, mask and pointer renamed alike).
// False when the chain has no late slot or more than two staged ones; D then
// stages every slot again (run_all_staged) and runs as it did under carry 2.
void run_all_staged(Launch &D)
{
    D.late_slots = 0;
    D.nstaged = D.nslot;
}

bool prepare_late(Launch &D, int term)
{
    set_late_slots(D, term);
    if (!D.late_slots) {
        run_all_staged(D);
        return false;
    }
    int perm[kSlots];
    int k = 0;
    for (int s = 0; s < D.nslot; s++)
        if (!((D.late_slots >> s) & 1u)) perm[s] = k++;
    const int staged = k;
    for (int s = 0; s < D.nslot; s++)
        if ((D.late_slots >> s) & 1u) perm[s] = k++;
    auto rename = [&](Src &x) {
        if (x.src == 0) x.idx = perm[x.idx];
    };
    for (int i = 0; i < D.n_ops; i++) {
        rename(D.ops[i].a);
        rename(D.ops[i].b);
    }
    rename(D.value);
    for (int j = 0; j < D.n_keys; j++) rename(D.keys[j]);
    auto remask = [&](uint32_t m) {
        uint32_t r = 0;
        for (int s = 0; s < D.nslot; s++)
            if ((m >> s) & 1u) r |= 1u << perm[s];
        return r;
    };
    D.tail_slots = remask(D.tail_slots);
    D.late_slots = remask(D.late_slots);
    const int32_t *old[kSlots];
    for (int s = 0; s < kSlots; s++) old[s] = D.slot[s];
    for (int s = 0; s < D.nslot; s++) D.slot[perm[s]] = old[s];
    D.nstaged = staged;
    if (staged > stage_slots<3>()) {
        run_all_staged(D);
        return false;
    }
    return true;
}

// Shape identity of a launch: which kernel instantiation with_shape picks.
struct ShapeProbe {
    int id = -1;
    template <class B, int TERM, int NREGS, int SPLIT, int... KS>
    int run()
    {
        static const int kId = next_shape_id();
        id = kId;
        return SDB_OK;
    }
    static int next_shape_id()
    {
        static std::atomic<int> n{0};
        return n++;
    }
};

struct SingleLauncher {
    const Launch &D;
    int stages;
    int carry;
    cudaStream_t s;
    template <class B, int TERM, int NREGS, int SPLIT, int... KS>
    int run()
    {
        return launch<B, TERM, NREGS, SPLIT, KS...>(D, stages, carry, s);
    }
};

int dispatch(const ChainLaunch &C, int nregs, int term, int compact, int stages, int carry, cudaStream_t s)
{
    Launch D;
    if (!convert(C, nregs, D)) return SDB_ERR_UNSUPPORTED;
    if (carry == 3 && !(compact && can_carry(D, term) && prepare_late(D, term))) {
        carry = 2;  // as variant 7
        stages = 2;
    }
    if (!can_carry(D, term)) carry = 0;
    SingleLauncher f{D, stages, carry, s};
    return with_shape(D, term, compact, f, carry == 3);
}

// One launch of k_batch over the chains of one shape group.
template <class B, int TERM, int NREGS, int STAGES, int SPLIT, int CARRY, int... KS>
int batch_stages(const Launch *launches, const Span *spans, uint32_t n_spans, uint32_t *head, uint32_t bitmap_words,
                 cudaStream_t s)
{
    auto kern = k_batch<B, TERM, NREGS, STAGES, SPLIT, CARRY, KS...>;
    const int ring = STAGES * stage_slots<CARRY>() * kThreads * (items_of<CARRY>() / 4) * (int)sizeof(int4);
    const int smem = ring + (int)(bitmap_words * 4);
    static const bool attr = [&] {  // once per instantiation, thread-safe
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ring + (int)(kBitmapMax / 8));
        return true;
    }();
    (void)attr;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    uint64_t blocks = (uint64_t)num_sms() * per_sm;
    if (blocks > n_spans) blocks = n_spans;
    if (blocks == 0) return SDB_OK;
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(launches, spans, n_spans, head);
    g_dense_launches.fetch_add(1, std::memory_order_relaxed);
    if (B::bound) g_bound_launches.fetch_add(1, std::memory_order_relaxed);
    return sdb_check_launch("sdb_chain_batch_launch");
}

struct BatchLauncher {
    const Launch *launches;
    const Span *spans;
    uint32_t n_spans;
    uint32_t *head;
    uint32_t bitmap_words;
    int stages;
    int carry;
    cudaStream_t s;
    template <class B, int TERM, int NREGS, int SPLIT, int... KS>
    int run()
    {
        constexpr bool kCompact = SPLIT <= (int)sizeof...(KS);
        constexpr bool kLate = kCompact && use_level2<SPLIT, KS...>(3);
        if constexpr (B::bound || SPLIT == 0) {  // bound and SPLIT-0 passes are carry-3 passes
            static_assert(kLate, "a bound shape needs the second level");
            return batch_stages<B, TERM, NREGS, 2, SPLIT, 3, KS...>(launches, spans, n_spans, head, bitmap_words, s);
        } else {
            if (kLate && carry == 3)
                return batch_stages<Dyn, TERM, NREGS, 2, SPLIT, kLate ? 3 : 0, KS...>(launches, spans, n_spans, head,
                                                                                    bitmap_words, s);
            if (stages >= 3)
                return batch_stages<Dyn, TERM, NREGS, 3, SPLIT, 0, KS...>(launches, spans, n_spans, head,
                                                                        bitmap_words, s);
            if (kCompact && carry >= 2)
                return batch_stages<Dyn, TERM, NREGS, 2, SPLIT, kCompact ? 2 : 0, KS...>(launches, spans, n_spans,
                                                                                       head, bitmap_words, s);
            if (kCompact && carry == 1)
                return batch_stages<Dyn, TERM, NREGS, 2, SPLIT, kCompact ? 1 : 0, KS...>(launches, spans, n_spans,
                                                                                       head, bitmap_words, s);
            return batch_stages<Dyn, TERM, NREGS, 2, SPLIT, 0, KS...>(launches, spans, n_spans, head, bitmap_words,
                                                                    s);
        }
    }
};

// Whether with_shape binds D (its shape's bound pass runs it).
struct BoundProbe {
    bool bound = false;
    template <class B, int TERM, int NREGS, int SPLIT, int... KS>
    int run()
    {
        bound = B::bound;
        return SDB_OK;
    }
};

// The bound shapes with a paired pass: those of the served mix (star join,
// date join, filter-project-sum).
template <class B>
constexpr bool has_pair_pass()
{
    return std::is_same<B, StarBind>::value || std::is_same<B, DateJoinBind>::value ||
           std::is_same<B, FilterSumBind>::value;
}

template <class B, int TERM, int NREGS, int STAGES, int SPLIT, int CARRY, int... KS>
int launch_pair_stages(LaunchPair &P, cudaStream_t s)
{
    auto kern = k_dense_pair<B, TERM, NREGS, STAGES, SPLIT, CARRY, KS...>;
    const int ring = STAGES * stage_slots<CARRY>() * kThreads * (items_of<CARRY>() / 4) * (int)sizeof(int4);
    uint32_t words = 0;
    for (int c = 0; c < kPair; c++) {
        P.bits_off[c] = words;
        if (P.L[c].bitmap_ht) words += (P.L[c].bitmap_len + 31) / 32;
    }
    const int smem = ring + (int)(words * 4);
    static const bool attr = [&] {  // once per instantiation, thread-safe
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ring + kPair * (int)(kBitmapMax / 8));
        return true;
    }();
    (void)attr;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const uint64_t tile = (uint64_t)kThreads * items_of<CARRY>();
    uint64_t blocks = (P.L[0].n + tile - 1) / tile;
    const uint64_t cap = (uint64_t)num_sms() * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(P);
    g_dense_launches.fetch_add(1, std::memory_order_relaxed);
    g_bound_launches.fetch_add(1, std::memory_order_relaxed);
    return sdb_check_launch("sdb_chain_launch_pair");
}

// Whether the shape with_shape picks has a paired pass.
struct PairProbe {
    bool ok = false;
    template <class B, int TERM, int NREGS, int SPLIT, int... KS>
    int run()
    {
        ok = B::bound && has_pair_pass<B>();
        return SDB_OK;
    }
};

// Launches the paired pass for the shape with_shape picks (bound, with a
// paired pass), else returns SDB_ERR_UNSUPPORTED without launching.
struct PairLauncher {
    LaunchPair &P;
    cudaStream_t s;
    template <class B, int TERM, int NREGS, int SPLIT, int... KS>
    int run()
    {
        if constexpr (B::bound && has_pair_pass<B>())
            return launch_pair_stages<B, TERM, NREGS, 2, SPLIT, 3, KS...>(P, s);
        else
            return SDB_ERR_UNSUPPORTED;
    }
};

// Whether two launches readied for carry 3 (prepare_late) can share one
// paired pass: the same bound shape, the same staged columns over the same
// rows, no incoming or outgoing flags.
bool pairable(const Launch &A, const Launch &B, int term_a, int term_b)
{
    if (term_a != term_b || (term_a != T_SUM && term_a != T_GROUP)) return false;
    if (A.n != B.n || A.n == 0 || A.flags_in || B.flags_in || A.flags_out || B.flags_out) return false;
    if (A.nstaged != B.nstaged || A.nslot != B.nslot || A.late_slots != B.late_slots) return false;
    for (int i = 0; i < A.nstaged; i++)
        if (A.slot[i] != B.slot[i]) return false;
    ShapeProbe pa, pb;
    if (with_shape(A, term_a, 1, pa, true) != SDB_OK || with_shape(B, term_b, 1, pb, true) != SDB_OK || pa.id != pb.id)
        return false;
    PairProbe pp;
    return with_shape(A, term_a, 1, pp, true) == SDB_OK && pp.ok;
}

}  // namespace dense

// Tuning table: variant per (terminal, register class, kind of the first op,
// log2 rows bucket); -1 = default.  Set by sdb_chain_tune_set(_op) (the
// autotuner persists its choices and loads them at start-up).  The first op
// tells the shapes of one terminal apart (a star join starts with a semi
// join, a date join with a range filter).
constexpr int kOpClasses = 8;  // SDB_OP_* kinds 0..6, 7 = no op
// entries are read and written from any thread (the request server launches
// from its own): relaxed atomics, all -1 until set
std::atomic<int> g_tune[3][3][kOpClasses][40];
std::atomic<bool> g_tune_init{false};

int op_class(const sdb_chain_desc &d) { return d.n_ops > 0 && d.ops[0].kind >= 0 && d.ops[0].kind < 7 ? d.ops[0].kind : 7; }

std::atomic<int> &tune_entry(int term, int nregs, int opc, uint64_t rows);

int reg_class(int nregs) { return nregs <= 2 ? 0 : (nregs <= 4 ? 1 : 2); }
int rows_bucket(uint64_t n)
{
    int b = 0;
    while (b < 39 && (1ull << (b + 1)) <= n) b++;
    return b;
}

std::atomic<int> &tune_entry(int term, int nregs, int opc, uint64_t rows)
{
    static std::once_flag once;
    std::call_once(once, [] {
        for (auto &a : g_tune)
            for (auto &b : a)
                for (auto &c : b)
                    for (auto &e : c) e.store(-1, std::memory_order_relaxed);
        g_tune_init.store(true);
    });
    return g_tune[term][reg_class(nregs)][opc][rows_bucket(rows)];
}

int default_variant(int nregs) { return nregs <= 4 ? 1 : 0; }

constexpr int kDenseVariant = 3;
[[maybe_unused]] constexpr int kCompactVariant = 4;  // compacted, 3-stage ring
constexpr int kCompact2Variant = 5;  // as 4 with a 2-stage copy ring
constexpr int kCarryVariant = 6;     // as 5, compacted rows carried across tiles
constexpr int kLevel2Variant = 7;    // as 6, plus a second compaction after the first row-per-lane op
constexpr int kLateVariant = 8;      // as 7, the columns read only after the second compaction loaded per row
constexpr int kMaxVariant = 8;

int variant_stages(int v) { return (v == kCompact2Variant || v >= kCarryVariant) ? 2 : 3; }
int variant_carry(int v)
{
    return v == kLateVariant ? 3 : (v == kLevel2Variant ? 2 : (v == kCarryVariant ? 1 : 0));
}

bool operand_ok(const sdb_operand &o, int &nregs, bool &vec, const char **why)
{
    if (o.kind == SDB_SRC_COL) {
        if (!o.col) { *why = "column operand is NULL"; return false; }
        if (!sdb::aligned(o.col, 4)) { *why = "column operand not 4-byte aligned"; return false; }
        if (!sdb::aligned(o.col, 16)) vec = false;
    } else if (o.kind == SDB_SRC_REG) {
        if (o.reg < 0 || o.reg >= SDB_CHAIN_MAX_REGS) { *why = "register index out of range"; return false; }
        nregs = std::max(nregs, o.reg + 1);
    } else if (o.kind != SDB_SRC_LIT) {
        *why = "unknown operand kind";
        return false;
    }
    return true;
}

// A build chain's ops as interval tests (RangeTest), or -1 when some op is
// not a selection of a column against literals (or uses a code the general
// pass treats specially) or there are more than kRangeTests.  Each test holds
// for exactly the values the op's comparison holds for.
int range_tests(const sdb_chain_desc &c, RangeTest *out)
{
    constexpr int32_t kMin = INT32_MIN, kMax = INT32_MAX;
    if (c.n_ops > kRangeTests || c.n >= (1ull << 32) - 4096) return -1;
    if ((c.build_key.kind != SDB_SRC_COL && c.build_key.kind != SDB_SRC_LIT) ||
        (c.terminal == SDB_TERM_BUILD_KV && c.build_val.kind != SDB_SRC_COL && c.build_val.kind != SDB_SRC_LIT))
        return -1;
    for (int i = 0; i < c.n_ops; i++) {
        const sdb_chain_op &o = c.ops[i];
        RangeTest t{};
        if (o.a.kind != SDB_SRC_COL || o.logic_op < SDB_NONE || o.logic_op > SDB_OR) return -1;
        t.col = o.a.col;
        t.logic = o.logic_op;
        bool never = false;
        if (o.kind == SDB_OP_SELECT) {
            if (o.b.kind != SDB_SRC_LIT) return -1;
            const int32_t v = o.b.lit;
            switch (o.cmp_op) {
            case SDB_EQ: t.lo = v; t.span = 0; break;
            case SDB_NE: t.lo = v; t.span = 0; t.neg = 1; break;
            case SDB_LT:
                if (v == kMin) never = true;
                else { t.lo = kMin; t.span = (uint32_t)(v - 1) - (uint32_t)kMin; }
                break;
            case SDB_LE: t.lo = kMin; t.span = (uint32_t)v - (uint32_t)kMin; break;
            case SDB_GT:
                if (v == kMax) never = true;
                else { t.lo = v + 1; t.span = (uint32_t)kMax - (uint32_t)(v + 1); }
                break;
            case SDB_GE: t.lo = v; t.span = (uint32_t)kMax - (uint32_t)v; break;
            default: return -1;
            }
            t.lo2 = t.lo;
            t.span2 = t.span;
        } else if (o.kind == SDB_OP_SEARCH_RANGE) {
            if (o.lo > o.hi) never = true;
            else { t.lo = t.lo2 = o.lo; t.span = t.span2 = (uint32_t)o.hi - (uint32_t)o.lo; }
        } else if (o.kind == SDB_OP_SEARCH_POINTS) {
            t.lo = o.lo;
            t.lo2 = o.hi;
            t.span = t.span2 = 0;
        } else {
            return -1;
        }
        if (never) {  // no value: the complement of every value
            t.lo = t.lo2 = kMin;
            t.span = t.span2 = 0xffffffffu;
            t.neg = 1;
        }
        out[i] = t;
    }
    return c.n_ops;
}

}  // namespace

// Checks a descriptor and fills the launch record; shared with the batched
// form (batch.cu).
int sdb_chain_prepare(const sdb_chain_desc *c, void *launch_out, size_t launch_bytes, int *nregs_out, int *term_out)
{
    if (!c) return sdb_set_error(SDB_ERR_INVALID, "sdb_fused_chain: NULL descriptor");
    if (launch_bytes < sizeof(ChainLaunch)) return sdb_set_error(SDB_ERR_INVALID, "launch record too small");
    if (c->n_ops < 0 || c->n_ops > SDB_CHAIN_MAX_OPS)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_fused_chain: n_ops=%d outside [0,%d]", c->n_ops, SDB_CHAIN_MAX_OPS);
    ChainLaunch L;
    std::memset(&L, 0, sizeof L);
    L.d = *c;
    bool vec = sdb::aligned(c->flags_in, 4) && sdb::aligned(c->flags_out, 4);
    int nregs = 1;
    const char *why = "";
    int dead_from = 0;
    for (int k = 0; k < c->n_ops; k++) {
        const sdb_chain_op &op = c->ops[k];
        switch (op.kind) {
        case SDB_OP_SELECT:
            if (!operand_ok(op.a, nregs, vec, &why) || !operand_ok(op.b, nregs, vec, &why)) goto bad;
            if (op.logic_op != SDB_AND) dead_from = k + 1;
            break;
        case SDB_OP_SEARCH_RANGE:
        case SDB_OP_SEARCH_POINTS:
            if (!operand_ok(op.a, nregs, vec, &why)) goto bad;
            if (op.logic_op != SDB_AND) dead_from = k + 1;
            break;
        case SDB_OP_SEMI_PROBE:
        case SDB_OP_FULL_PROBE:
            if (!operand_ok(op.a, nregs, vec, &why)) goto bad;
            if (!op.ht) { why = "probe without a hash table"; goto bad; }
            if (op.kind == SDB_OP_FULL_PROBE && !sdb::aligned(op.ht, 8)) { why = "key/value table must be 8-byte aligned"; goto bad; }
            if (op.ht_log2 < 0 || op.ht_log2 > 31) { why = "ht_log2 outside [0,31]"; goto bad; }
            if (op.ht_log2 && (!sdb::aligned(op.ht, 4) || op.lo > op.hi || (uint32_t)op.hi - (uint32_t)op.lo >= 0x7fffffffu)) {
                why = "open-addressing probe: table not aligned, or key range empty or of 2^31 keys or more";
                goto bad;
            }
            if (op.kind == SDB_OP_FULL_PROBE) {
                if (op.out_reg < 0 || op.out_reg >= SDB_CHAIN_MAX_REGS) { why = "out_reg out of range"; goto bad; }
                nregs = std::max(nregs, op.out_reg + 1);
            }
            break;
        case SDB_OP_BINOP:
            if (!operand_ok(op.a, nregs, vec, &why) || !operand_ok(op.b, nregs, vec, &why)) goto bad;
            if (op.bin_op < SDB_MUL || op.bin_op > SDB_SUB) { why = "unknown binary operation"; goto bad; }
            if (op.out_reg < 0 || op.out_reg >= SDB_CHAIN_MAX_REGS) { why = "out_reg out of range"; goto bad; }
            nregs = std::max(nregs, op.out_reg + 1);
            break;
        case SDB_OP_FILL:
            if (op.a.kind != SDB_SRC_LIT) { why = "FILL takes a literal"; goto bad; }
            if (op.out_reg < 0 || op.out_reg >= SDB_CHAIN_MAX_REGS) { why = "out_reg out of range"; goto bad; }
            nregs = std::max(nregs, op.out_reg + 1);
            if (op.out_col) dead_from = k + 1;  // FillKernel writes every row
            break;
        default:
            why = "unknown op kind";
            goto bad;
        }
        if ((op.kind == SDB_OP_FULL_PROBE || op.kind == SDB_OP_BINOP || op.kind == SDB_OP_FILL) && op.out_col &&
            !sdb::aligned(op.out_col, 4)) {
            why = "out_col misaligned";
            goto bad;
        }
    }
    L.dead_from = dead_from;
    switch (c->terminal) {
    case SDB_TERM_FLAGS:
        if (!c->flags_out) { why = "SDB_TERM_FLAGS needs flags_out"; goto bad; }
        *term_out = T_FLAGS;
        break;
    case SDB_TERM_SUM:
        if (!c->sum_out) { why = "SDB_TERM_SUM needs sum_out"; goto bad; }
        if (!sdb::aligned(c->sum_out, 8)) { why = "sum_out not 8-byte aligned"; goto bad; }
        if (!operand_ok(c->value, nregs, vec, &why)) goto bad;
        *term_out = T_SUM;
        break;
    case SDB_TERM_GROUPBY: {
        if (c->n_keys < 1 || c->n_keys > SDB_CHAIN_MAX_KEYS) { why = "n_keys outside [1,4]"; goto bad; }
        if (c->P == 0 || !c->out_sum || !c->occ) { why = "group-by needs P > 0, out_sum and occ"; goto bad; }
        if (!sdb::aligned(c->out_sum, 8) || !sdb::aligned(c->occ, 4)) { why = "out_sum/occ misaligned"; goto bad; }
        if (!operand_ok(c->value, nregs, vec, &why)) goto bad;
        uint32_t mult = 1;
        for (int j = 0; j < c->n_keys; j++) {
            if (!operand_ok(c->keys[j], nregs, vec, &why)) goto bad;
            if (!c->out_keys[j] || !sdb::aligned(c->out_keys[j], 4)) { why = "group-by needs 4-byte aligned out_keys"; goto bad; }
            L.mults[j] = mult;
            mult *= (uint32_t)c->key_max[j] - (uint32_t)c->key_min[j] + 1u;
        }
        *term_out = T_GROUP;
        break;
    }
    case SDB_TERM_BUILD_KEYS:
    case SDB_TERM_BUILD_KV: {
        const bool kv = c->terminal == SDB_TERM_BUILD_KV;
        if (!c->ht_out || c->ht_len <= 0) { why = "a build needs ht_out and ht_len > 0"; goto bad; }
        if (kv && !sdb::aligned(c->ht_out, 8)) { why = "key/value table must be 8-byte aligned"; goto bad; }
        if (c->ht_log2 < 0 || c->ht_log2 > 31) { why = "ht_log2 outside [0,31]"; goto bad; }
        if (c->ht_log2 && (!sdb::aligned(c->ht_out, 4) || c->ht_len == 0x7fffffff)) {
            why = "open-addressing build: table not aligned or 2^31 keys or more";
            goto bad;
        }
        if (!operand_ok(c->build_key, nregs, vec, &why)) goto bad;
        if (kv && !operand_ok(c->build_val, nregs, vec, &why)) goto bad;
        *term_out = T_BUILD;
        L.n_tests = range_tests(*c, L.tests);
        break;
    }
    default:
        why = "unknown terminal";
        goto bad;
    }
    L.vec = vec ? 1 : 0;
    std::memcpy(launch_out, &L, sizeof L);
    *nregs_out = nregs;
    return SDB_OK;
bad:
    return sdb_set_error(SDB_ERR_INVALID, "sdb_fused_chain: %s", why);
}

size_t sdb_chain_launch_bytes() { return sizeof(ChainLaunch); }

static int fused_chain_impl(const sdb_chain_desc *chain, int variant, sdb_stream_t stream)
{
    ChainLaunch L;
    int nregs = 1, term = 0;
    int st = sdb_chain_prepare(chain, &L, sizeof L, &nregs, &term);
    if (st != SDB_OK) return st;
    if (L.d.n == 0) return SDB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (term == T_BUILD) return launch_build(L, nregs, s);
    if (variant < 0) {
        variant = tune_entry(term, nregs, op_class(L.d), L.d.n);
        if (variant < 0) variant = kCompact2Variant;  // shape-specialised pass when one exists
    }
    if (variant >= kDenseVariant) {
        const int st2 = dense::dispatch(L, nregs, term, variant != kDenseVariant, variant_stages(variant),
                                        variant_carry(variant), s);
        if (st2 != SDB_ERR_UNSUPPORTED) return st2;
        variant = default_variant(nregs);
    }
    switch (term) {
    case T_FLAGS: return launch_regs<T_FLAGS>(L, nregs, variant, s);
    case T_SUM: return launch_regs<T_SUM>(L, nregs, variant, s);
    default: return launch_regs<T_GROUP>(L, nregs, variant, s);
    }
}

// ---- batched form -----------------------------------------------------------

struct sdb_chain_batch {
    struct Group {
        int term, compact, stages;
        int carry;
        bool bound;                      // every chain takes its shape's bound pass
        dense::Launch first;             // host copy, picks the instantiation
        const dense::Launch *launches;   // device
        const dense::Span *spans;        // device
        uint32_t n_spans;
        uint32_t *head;                  // device work-queue head
        uint32_t bitmap_words;
    };
    std::vector<Group> groups;
    std::vector<sdb_chain_desc> singles;  // chains with no batched instantiation
    uint32_t *heads = nullptr;
    size_t n_heads = 0;
    // hash-table builds, launched before everything else
    const ChainLaunch *builds = nullptr;   // device
    const uint32_t *build_tiles = nullptr; // device, n_builds + 1 tile offsets
    int n_builds = 0;
    uint32_t build_total = 0;
    int build_nregs = 0;
};

namespace {

// Host-side layout of a batch: groups of chains sharing one instantiation,
// their spans, and the device bytes they take.
struct BatchPlan {
    struct G {
        int term, compact, stages, shape;
        int carry = 0;
        bool bound = false;
        std::vector<dense::Launch> launches;
        std::vector<dense::Span> spans;
        uint32_t bitmap_words = 0;
    };
    std::vector<G> groups;
    std::vector<sdb_chain_desc> singles;
    std::vector<ChainLaunch> builds;
    std::vector<uint32_t> build_tiles;  // builds.size() + 1 offsets
    int build_nregs = 0;                // 0: every build in interval-test form
    size_t bytes = 0;
};

size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

int plan_batch(const sdb_chain_desc *chains, int n_chains, BatchPlan &bp)
{
    if (n_chains < 0 || (n_chains > 0 && !chains)) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch: bad chain list");
    constexpr uint64_t kTile = (uint64_t)kThreads * dense::kItems;
    // chains grouped by the shape-specialised instantiation they map to
    struct Item {
        int index;
        dense::Launch D;
        uint64_t tiles;
    };
    struct Family {
        int shape, term, nregs, opc;
        uint64_t rows = 0;
        std::vector<Item> items;
    };
    std::vector<Family> fams;
    uint64_t build_tiles = 0;
    bp.build_tiles.assign(1, 0);
    for (int i = 0; i < n_chains; i++) {
        ChainLaunch L;
        int nregs = 1, term = 0;
        int st = sdb_chain_prepare(&chains[i], &L, sizeof L, &nregs, &term);
        if (st != SDB_OK) return st;
        if (L.d.n == 0) continue;
        if (term == T_BUILD) {
            constexpr uint64_t kBuildTile = (uint64_t)kThreads * kBuildItems;
            build_tiles += (L.d.n + kBuildTile - 1) / kBuildTile;
            if (build_tiles > 0xffffffffull) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch: build chains too large");
            bp.builds.push_back(L);
            bp.build_tiles.push_back((uint32_t)build_tiles);
            if (L.n_tests < 0) bp.build_nregs = std::max(bp.build_nregs, nregs);
            continue;
        }
        Item it;
        it.index = i;
        dense::ShapeProbe probe;
        if (!dense::convert(L, nregs, it.D) || dense::with_shape(it.D, term, 1, probe) != SDB_OK ||
            (L.d.n + kTile - 1) / kTile > 0xffffffffull) {
            bp.singles.push_back(chains[i]);
            continue;
        }
        it.tiles = (L.d.n + kTile - 1) / kTile;
        size_t f = 0;
        while (f < fams.size() && !(fams[f].shape == probe.id && fams[f].term == term)) f++;
        if (f == fams.size()) fams.push_back(Family{probe.id, term, nregs, op_class(L.d)});
        fams[f].nregs = std::max(fams[f].nregs, nregs);
        fams[f].rows += L.d.n;
        fams[f].items.push_back(it);
    }
    // one launch per family, its variant tuned on the family's total rows
    uint64_t total_tiles = 0;
    std::vector<BatchPlan::G> groups;
    std::vector<const Family *> of;
    for (const Family &F : fams) {
        int variant = g_tune_init ? tune_entry(F.term, F.nregs, F.opc, F.rows).load(std::memory_order_relaxed) : -1;
        if (variant < 0) variant = kCompact2Variant;
        if (variant < kDenseVariant) {  // the general pass: chain by chain
            for (const Item &it : F.items) bp.singles.push_back(chains[it.index]);
            continue;
        }
        BatchPlan::G g;
        g.term = F.term;
        g.compact = variant != kDenseVariant;
        g.stages = variant_stages(variant);
        g.carry = variant_carry(variant);
        g.shape = F.shape;
        groups.push_back(g);
        of.push_back(&F);
        for (const Item &it : F.items) total_tiles += it.tiles;
    }
    // spans of S tiles: about 8 per resident block over the whole batch
    const uint64_t target = (uint64_t)num_sms() * 5 * 8;
    uint64_t S = (total_tiles + target - 1) / std::max<uint64_t>(target, 1);
    S = std::min<uint64_t>(std::max<uint64_t>(S, 2), 64);
    for (size_t g = 0; g < groups.size(); g++) {
        BatchPlan::G &G = groups[g];
        for (const Item &it : of[g]->items) {
            if (G.carry && !dense::can_carry(it.D, G.term)) G.carry = 0;  // every chain of the launch must allow it
            G.launches.push_back(it.D);
            if (G.carry == 3 && !dense::prepare_late(G.launches.back(), G.term)) {
                G.carry = 2;  // as variant 7
                G.stages = 2;
            }
            if (it.D.bitmap_ht) G.bitmap_words = std::max<uint32_t>(G.bitmap_words, (it.D.bitmap_len + 31) / 32);
        }
        if (G.carry != 3)  // chains readied for carry 3 before the group fell back
            for (dense::Launch &x : G.launches) dense::run_all_staged(x);
        // spans in the launch's tiles (carry 3: 8 rows per thread, spans of half
        // as many tiles)
        const uint64_t tile = (uint64_t)kThreads * (G.carry == 3 ? dense::items_of<3>() : dense::kItems);
        const uint64_t span = G.carry == 3 ? std::max<uint64_t>(S / 2, 1) : S;
        for (uint32_t c = 0; c < (uint32_t)G.launches.size(); c++) {
            const uint64_t tiles = (G.launches[c].n + tile - 1) / tile;
            for (uint64_t t = 0; t < tiles; t += span)
                G.spans.push_back({c, (uint32_t)t, (uint32_t)std::min<uint64_t>(t + span, tiles), 0});
        }
        G.bound = G.carry == 3;
        for (const dense::Launch &x : G.launches) {
            dense::BoundProbe p;
            if (G.bound && dense::with_shape(x, G.term, 1, p, true) == SDB_OK) G.bound = p.bound;
            else G.bound = false;
        }
    }
    // all builds run in one launch before the other chains: none may probe a
    // table another build writes
    for (const ChainLaunch &B : bp.builds)
        for (int k = 0; k < B.d.n_ops; k++) {
            const sdb_chain_op &o = B.d.ops[k];
            if (o.kind != SDB_OP_SEMI_PROBE && o.kind != SDB_OP_FULL_PROBE) continue;
            for (const ChainLaunch &W : bp.builds)
                if (W.d.ht_out == o.ht)
                    return sdb_set_error(SDB_ERR_INVALID,
                                         "sdb_chain_batch: a build chain probes a table built in the same batch");
        }
    bp.groups = std::move(groups);
    bp.bytes = round256(bp.groups.size() * sizeof(uint32_t));
    for (const auto &G : bp.groups)
        bp.bytes += round256(G.launches.size() * sizeof(dense::Launch)) + round256(G.spans.size() * sizeof(dense::Span));
    if (!bp.builds.empty())
        bp.bytes += round256(bp.builds.size() * sizeof(ChainLaunch)) + round256(bp.build_tiles.size() * sizeof(uint32_t));
    return SDB_OK;
}

}  // namespace

extern "C" {

size_t sdb_chain_batch_scratch_bytes(const sdb_chain_desc *chains, int n_chains)
{
    BatchPlan bp;
    if (plan_batch(chains, n_chains, bp) != SDB_OK) return 0;
    return std::max<size_t>(bp.bytes, 256);
}

static int chain_batch_create(const sdb_chain_desc *chains, int n_chains, void *dev_scratch, size_t dev_bytes,
                              void *host_staging, size_t host_bytes, sdb_stream_t stream, sdb_chain_batch **out)
{
    if (!out) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_create: NULL out");
    *out = nullptr;
    BatchPlan bp;
    int st = plan_batch(chains, n_chains, bp);
    if (st != SDB_OK) return st;
    if (dev_bytes < bp.bytes || (bp.bytes && !dev_scratch))
        return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_create: scratch of %zu bytes, %zu needed", dev_bytes,
                             bp.bytes);
    if (!sdb::aligned(dev_scratch, 256)) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_create: scratch not 256-byte aligned");
    if (host_staging && host_bytes < bp.bytes)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_create_async: staging of %zu bytes, %zu needed",
                             host_bytes, bp.bytes);
    std::vector<char> own;
    char *host = static_cast<char *>(host_staging);
    if (!host) {
        own.assign(bp.bytes, 0);
        host = own.data();
    } else {
        std::memset(host, 0, bp.bytes);
    }
    auto *b = new sdb_chain_batch;
    char *dev = static_cast<char *>(dev_scratch);
    size_t off = round256(bp.groups.size() * sizeof(uint32_t));
    b->heads = reinterpret_cast<uint32_t *>(dev);
    b->n_heads = bp.groups.size();
    for (size_t g = 0; g < bp.groups.size(); g++) {
        const auto &G = bp.groups[g];
        sdb_chain_batch::Group o;
        o.term = G.term;
        o.compact = G.compact;
        o.stages = G.stages;
        o.carry = G.carry;
        o.bound = G.bound;
        o.first = G.launches[0];
        o.head = b->heads + g;
        o.bitmap_words = G.bitmap_words;
        std::memcpy(host + off, G.launches.data(), G.launches.size() * sizeof(dense::Launch));
        o.launches = reinterpret_cast<const dense::Launch *>(dev + off);
        off += round256(G.launches.size() * sizeof(dense::Launch));
        std::memcpy(host + off, G.spans.data(), G.spans.size() * sizeof(dense::Span));
        o.spans = reinterpret_cast<const dense::Span *>(dev + off);
        o.n_spans = (uint32_t)G.spans.size();
        off += round256(G.spans.size() * sizeof(dense::Span));
        b->groups.push_back(o);
    }
    b->singles = bp.singles;
    if (!bp.builds.empty()) {
        std::memcpy(host + off, bp.builds.data(), bp.builds.size() * sizeof(ChainLaunch));
        b->builds = reinterpret_cast<const ChainLaunch *>(dev + off);
        off += round256(bp.builds.size() * sizeof(ChainLaunch));
        std::memcpy(host + off, bp.build_tiles.data(), bp.build_tiles.size() * sizeof(uint32_t));
        b->build_tiles = reinterpret_cast<const uint32_t *>(dev + off);
        off += round256(bp.build_tiles.size() * sizeof(uint32_t));
        b->n_builds = (int)bp.builds.size();
        b->build_total = bp.build_tiles.back();
        b->build_nregs = bp.build_nregs;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (bp.bytes) {
        cudaError_t e = cudaMemcpyAsync(dev_scratch, host, bp.bytes, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && !host_staging) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            delete b;
            return sdb_set_error(SDB_ERR_CUDA, "sdb_chain_batch_create: %s", cudaGetErrorString(e));
        }
    }
    *out = b;
    return SDB_OK;
}

int sdb_chain_batch_create(const sdb_chain_desc *chains, int n_chains, void *dev_scratch, size_t dev_bytes,
                           sdb_stream_t stream, sdb_chain_batch **out)
{
    return chain_batch_create(chains, n_chains, dev_scratch, dev_bytes, nullptr, 0, stream, out);
}

int sdb_chain_batch_create_async(const sdb_chain_desc *chains, int n_chains, void *dev_scratch, size_t dev_bytes,
                                 void *host_staging, size_t host_bytes, sdb_stream_t stream, sdb_chain_batch **out)
{
    if (!host_staging) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_create_async: NULL staging");
    return chain_batch_create(chains, n_chains, dev_scratch, dev_bytes, host_staging, host_bytes, stream, out);
}

int sdb_chain_batch_launch_part(const sdb_chain_batch *b, int part, sdb_stream_t stream)
{
    if (!b) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_launch: NULL batch");
    if (part != 0 && part != 1) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_launch_part: part %d", part);
    cudaStream_t s = (cudaStream_t)stream;
    if (part == 0)
        return b->n_builds ? launch_build_batch(b->builds, b->build_tiles, b->n_builds, b->build_total, b->build_nregs, s)
                           : SDB_OK;
    if (b->n_heads) {
        cudaError_t e = cudaMemsetAsync(b->heads, 0, b->n_heads * sizeof(uint32_t), s);
        if (e != cudaSuccess) return sdb_set_error(SDB_ERR_CUDA, "sdb_chain_batch_launch: %s", cudaGetErrorString(e));
    }
    for (const auto &G : b->groups) {
        dense::BatchLauncher f{G.launches, G.spans, G.n_spans, G.head, G.bitmap_words, G.stages, G.carry, s};
        int st = dense::with_shape(G.first, G.term, G.compact, f, G.bound);
        if (st != SDB_OK) return st;
    }
    for (const auto &c : b->singles) {
        int st = fused_chain_impl(&c, -1, stream);
        if (st != SDB_OK) return st;
    }
    return SDB_OK;
}

int sdb_chain_batch_launch(const sdb_chain_batch *b, sdb_stream_t stream)
{
    const int st = sdb_chain_batch_launch_part(b, 0, stream);
    return st != SDB_OK ? st : sdb_chain_batch_launch_part(b, 1, stream);
}

int sdb_chain_batch_kernels(const sdb_chain_batch *b)
{
    if (!b) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_batch_kernels: NULL batch");
    return (int)(b->groups.size() + b->singles.size()) + (b->n_builds ? 1 : 0);
}

void sdb_chain_batch_destroy(sdb_chain_batch *b) { delete b; }

}  // extern "C"

extern "C" {

int sdb_fused_chain(const sdb_chain_desc *chain, sdb_stream_t stream) { return fused_chain_impl(chain, -1, stream); }

int sdb_fused_chain_variant(const sdb_chain_desc *chain, int variant, sdb_stream_t stream)
{
    if (variant < 0 || variant > kMaxVariant)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_fused_chain_variant: variant %d", variant);
    return fused_chain_impl(chain, variant, stream);
}

int sdb_chain_tune_set_op(int terminal, int nregs, int first_op, uint64_t rows, int variant)
{
    if (terminal < 0 || terminal > 2 || nregs < 1 || nregs > SDB_CHAIN_MAX_REGS || variant < -1 ||
        variant > kMaxVariant || first_op < -1 || first_op >= kOpClasses)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_tune_set: bad argument");
    for (int c = 0; c < kOpClasses; c++)
        if (first_op < 0 || c == first_op) tune_entry(terminal, nregs, c, rows) = variant;
    return SDB_OK;
}

int sdb_fused_launch_counts(uint64_t *specialised, uint64_t *bound)
{
    if (specialised) *specialised = dense::g_dense_launches.load(std::memory_order_relaxed);
    if (bound) *bound = dense::g_bound_launches.load(std::memory_order_relaxed);
    return SDB_OK;
}

int sdb_chain_tune_set(int terminal, int nregs, uint64_t rows, int variant)
{
    return sdb_chain_tune_set_op(terminal, nregs, -1, rows, variant);
}

int sdb_chain_tune_get_op(int terminal, int nregs, int first_op, uint64_t rows)
{
    if (terminal < 0 || terminal > 2 || nregs < 1 || nregs > SDB_CHAIN_MAX_REGS || first_op < 0 ||
        first_op >= kOpClasses)
        return -1;
    if (!g_tune_init) return kCompact2Variant;
    int v = tune_entry(terminal, nregs, first_op, rows);
    return v < 0 ? kCompact2Variant : v;
}

int sdb_chain_tune_get(int terminal, int nregs, uint64_t rows)
{
    return sdb_chain_tune_get_op(terminal, nregs, 7, rows);
}

int sdb_chain_registers(const sdb_chain_desc *chain)
{
    ChainLaunch L;
    int nregs = 1, term = 0;
    int st = sdb_chain_prepare(chain, &L, sizeof L, &nregs, &term);
    return st != SDB_OK ? st : nregs;
}

int sdb_chain_specialised(const sdb_chain_desc *chain)
{
    ChainLaunch L;
    int nregs = 1, term = 0;
    int st = sdb_chain_prepare(chain, &L, sizeof L, &nregs, &term);
    if (st != SDB_OK) return st;
    if (term == T_BUILD) return 0;
    dense::Launch D;
    if (!dense::convert(L, nregs, D)) return 0;
    dense::ShapeProbe probe;
    if (dense::with_shape(D, term, 1, probe) != SDB_OK) return 0;
    if (dense::can_carry(D, term) && dense::prepare_late(D, term)) {
        dense::BoundProbe bp;
        if (dense::with_shape(D, term, 1, bp, true) == SDB_OK && bp.bound) return 2;
    }
    return 1;
}

// The paired pass.  A chain takes part as the single-chain pass would run it
// under its tuned variant: only a carry-3 launch (variant 8) of a bound
// shape pairs, so each chain's results are those of its own launch.
static bool pair_launch_of(const sdb_chain_desc *c, dense::Launch &D, int &term)
{
    ChainLaunch L;
    int nregs = 1;
    term = 0;
    if (sdb_chain_prepare(c, &L, sizeof L, &nregs, &term) != SDB_OK) return false;
    if (L.d.n == 0 || term == T_BUILD || term == T_FLAGS) return false;
    int variant = tune_entry(term, nregs, op_class(L.d), L.d.n);
    if (variant < 0) variant = kCompact2Variant;
    if (variant < kDenseVariant || variant_carry(variant) != 3) return false;
    if (!dense::convert(L, nregs, D)) return false;
    return dense::can_carry(D, term) && dense::prepare_late(D, term);
}

int sdb_chain_pair_key(const sdb_chain_desc *c, uint64_t *key)
{
    if (!c || !key) return 0;
    dense::Launch D;
    int term = 0;
    if (!pair_launch_of(c, D, term)) return 0;
    dense::PairProbe pp;
    if (dense::with_shape(D, term, 1, pp, true) != SDB_OK || !pp.ok) return 0;
    dense::ShapeProbe sp;
    dense::with_shape(D, term, 1, sp, true);
    // FNV-1a over what pairable compares
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int i = 0; i < 8; i++) {
            h ^= (v >> (8 * i)) & 0xffu;
            h *= 1099511628211ull;
        }
    };
    mix((uint64_t)sp.id);
    mix((uint64_t)term);
    mix(D.n);
    mix(((uint64_t)D.nstaged << 32) | ((uint64_t)D.nslot << 16) | D.late_slots);
    for (int i = 0; i < D.nstaged; i++) mix((uint64_t)(uintptr_t)D.slot[i]);
    *key = h;
    return 1;
}

int sdb_chain_pairable(const sdb_chain_desc *a, const sdb_chain_desc *b)
{
    if (!a || !b) return 0;
    dense::Launch A, B;
    int ta = 0, tb = 0;
    if (!pair_launch_of(a, A, ta) || !pair_launch_of(b, B, tb)) return 0;
    return dense::pairable(A, B, ta, tb) ? 1 : 0;
}

int sdb_chain_launch_pair(const sdb_chain_desc *a, const sdb_chain_desc *b, sdb_stream_t stream)
{
    if (!a || !b) return sdb_set_error(SDB_ERR_INVALID, "sdb_chain_launch_pair: NULL chain");
    dense::LaunchPair P;
    std::memset(&P, 0, sizeof P);
    int ta = 0, tb = 0;
    if (!pair_launch_of(a, P.L[0], ta) || !pair_launch_of(b, P.L[1], tb) || !dense::pairable(P.L[0], P.L[1], ta, tb))
        return sdb_set_error(SDB_ERR_UNSUPPORTED, "sdb_chain_launch_pair: the chains do not share a paired pass");
    dense::PairLauncher f{P, (cudaStream_t)stream};
    return dense::with_shape(P.L[0], ta, 1, f, true);
}

}  // extern "C"
