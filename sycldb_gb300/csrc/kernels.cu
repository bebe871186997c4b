// Operator kernels K1-K16 of the C ABI (include/sycldb_gpu.h) for sm_103a.
//
// Every kernel streams HBM: int32 columns are read with 128-bit loads
// (two int4 per 8-row group) and bool flags 8 at a time (one 64-bit word),
// grids are a multiple of the SM count and loop grid-stride.  Pointers that
// are not 16-byte (columns) / 8-byte (flags) aligned take the scalar
// instantiation, which computes the same values.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <initializer_list>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "ssbgen.cuh"

namespace {

__device__ unsigned long long g_errors;  // out-of-range slots skipped

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
constexpr int kMaxBlock = 512;  // largest block an operator kernel is tuned to

// Launch shape of an operator kernel: threads per block and the resident
// blocks per SM its grid-stride grid is sized for.  Tuned per (operator,
// log2 rows) by the autotuner (sdb_op_tune_set); unset entries take the
// defaults (256 threads; 8 blocks per SM for the map kernels, 4 for the
// reductions).
struct LaunchShape {
    int block, per_sm;
};
std::atomic<int32_t> g_op_tune[SDB_OPK_COUNT][40];  // block << 8 | per_sm; 0: default

int op_bucket(uint64_t n)
{
    int b = 0;
    while (b < 39 && (1ull << (b + 1)) <= n) b++;
    return b;
}

LaunchShape op_shape(int opk, uint64_t rows, int default_per_sm)
{
    const int32_t e = g_op_tune[opk][op_bucket(rows)].load(std::memory_order_relaxed);
    if (e <= 0) return {kThreads, default_per_sm};
    return {e >> 8, e & 0xff};
}

// Grid of `work` items for a launch shape (grid-stride kernels).
unsigned grid_of(uint64_t work, const LaunchShape &sh) { return sdb::grid_for(work, sh.block, sh.per_sm); }

// ---------------------------------------------------------------- vector io
__device__ __forceinline__ void ld8(const int32_t *p, uint64_t r0, int32_t (&v)[8])
{
    const int4 *q = reinterpret_cast<const int4 *>(p + r0);
    int4 a = __ldcs(q), b = __ldcs(q + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

__device__ __forceinline__ void st8(int32_t *p, uint64_t r0, const int32_t (&v)[8])
{
    int4 *q = reinterpret_cast<int4 *>(p + r0);
    q[0] = make_int4(v[0], v[1], v[2], v[3]);
    q[1] = make_int4(v[4], v[5], v[6], v[7]);
}

__device__ __forceinline__ uint32_t nz_bits4(uint32_t w)
{
    uint32_t x = __vcmpne4(w, 0u);
    return ((x >> 7) & 1u) | ((x >> 14) & 2u) | ((x >> 21) & 4u) | ((x >> 28) & 8u);
}

__device__ __forceinline__ uint32_t ldf8(const uint8_t *p, uint64_t r0)
{
    uint2 w = __ldcs(reinterpret_cast<const uint2 *>(p + r0));
    return nz_bits4(w.x) | (nz_bits4(w.y) << 4);
}

__device__ __forceinline__ uint32_t bits_to_bytes4(uint32_t m)
{
    return (m & 1u) | ((m & 2u) << 7) | ((m & 4u) << 14) | ((m & 8u) << 21);
}

__device__ __forceinline__ void stf8(uint8_t *p, uint64_t r0, uint32_t m)
{
    uint2 w;
    w.x = bits_to_bytes4(m & 0xFu);
    w.y = bits_to_bytes4((m >> 4) & 0xFu);
    *reinterpret_cast<uint2 *>(p + r0) = w;
}

// Grid-stride driver: Op provides group(r0) for 8 rows (vector path) and
// row(r) for one row.  VEC=false walks rows one at a time.
template <bool VEC, class Op>
__global__ void __launch_bounds__(kMaxBlock) k_map(uint64_t n, Op op)
{
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (VEC) {
        const uint64_t groups = n >> 3;
        for (uint64_t g = tid; g < groups; g += stride) op.group(g << 3);
        for (uint64_t r = (groups << 3) + tid; r < n; r += stride) op.row(r);
    } else {
        for (uint64_t r = tid; r < n; r += stride) op.row(r);
    }
}

template <class Op>
int launch_map(uint64_t n, bool vec, const Op &op, cudaStream_t s, const char *what, int opk)
{
    if (n == 0) return SDB_OK;
    const LaunchShape sh = op_shape(opk, n, 8);
    if (vec)
        k_map<true, Op><<<grid_of((n + 7) / 8, sh), sh.block, 0, s>>>(n, op);
    else
        k_map<false, Op><<<grid_of(n, sh), sh.block, 0, s>>>(n, op);
    return sdb_check_launch(what);
}

// ---------------------------------------------------------------- K1, K5
struct FillU8 {
    uint8_t *f; uint8_t v;
    __device__ void group(uint64_t r0) const
    {
        uint32_t w = 0x01010101u * v;
        *reinterpret_cast<uint2 *>(f + r0) = make_uint2(w, w);
    }
    __device__ void row(uint64_t r) const { f[r] = v; }
};

struct FillI32 {
    int32_t *d; int32_t v;
    __device__ void group(uint64_t r0) const
    {
        int32_t x[8] = {v, v, v, v, v, v, v, v};
        st8(d, r0, x);
    }
    __device__ void row(uint64_t r) const { d[r] = v; }
};

// ---------------------------------------------------------------- K2, K3, K4
struct SelectLit {
    const int32_t *col; int32_t v; int cmp, logic; const uint8_t *in; uint8_t *out;
    __device__ void group(uint64_t r0) const
    {
        int32_t c[8];
        ld8(col, r0, c);
        uint32_t fin = ldf8(in, r0), m = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) m |= (uint32_t)sdb::compare(cmp, c[j], v) << j;
        uint32_t lo = sdb::logical4(logic, fin & 0xF, m & 0xF), hi = sdb::logical4(logic, fin >> 4, m >> 4);
        stf8(out, r0, lo | (hi << 4));
    }
    __device__ void row(uint64_t r) const { out[r] = sdb::logical(logic, in[r] != 0, sdb::compare(cmp, col[r], v)); }
};

struct SelectCols {
    const int32_t *a, *b; int cmp, logic; const uint8_t *in; uint8_t *out;
    __device__ void group(uint64_t r0) const
    {
        int32_t x[8], y[8];
        ld8(a, r0, x);
        ld8(b, r0, y);
        uint32_t fin = ldf8(in, r0), m = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) m |= (uint32_t)sdb::compare(cmp, x[j], y[j]) << j;
        uint32_t lo = sdb::logical4(logic, fin & 0xF, m & 0xF), hi = sdb::logical4(logic, fin >> 4, m >> 4);
        stf8(out, r0, lo | (hi << 4));
    }
    __device__ void row(uint64_t r) const { out[r] = sdb::logical(logic, in[r] != 0, sdb::compare(cmp, a[r], b[r])); }
};

struct Logical {
    int logic; const uint8_t *in, *local; uint8_t *out;
    __device__ void group(uint64_t r0) const
    {
        uint32_t a = ldf8(in, r0), b = ldf8(local, r0);
        uint32_t lo = sdb::logical4(logic, a & 0xF, b & 0xF), hi = sdb::logical4(logic, a >> 4, b >> 4);
        stf8(out, r0, lo | (hi << 4));
    }
    __device__ void row(uint64_t r) const { out[r] = sdb::logical(logic, in[r] != 0, local[r] != 0); }
};

// ---------------------------------------------------------------- K6
// mode 0: col op col, 1: lit op col, 2: col op lit
struct Binop {
    int32_t *res; const int32_t *a, *b; int32_t la, lb; int op, mode; const uint8_t *flags;
    __device__ int32_t A(uint64_t r) const { return mode == 1 ? la : a[r]; }
    __device__ int32_t B(uint64_t r) const { return mode == 2 ? lb : b[r]; }
    __device__ void group(uint64_t r0) const
    {
        uint32_t f = ldf8(flags, r0);
        if (f == 0) return;
        int32_t x[8], y[8];
        if (mode == 1) { for (int j = 0; j < 8; j++) x[j] = la; } else ld8(a, r0, x);
        if (mode == 2) { for (int j = 0; j < 8; j++) y[j] = lb; } else ld8(b, r0, y);
        if (f == 0xFFu) {
            int32_t z[8];
#pragma unroll
            for (int j = 0; j < 8; j++) z[j] = sdb::binop(x[j], y[j], op);
            st8(res, r0, z);
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (f & (1u << j)) res[r0 + j] = sdb::binop(x[j], y[j], op);
        }
    }
    __device__ void row(uint64_t r) const
    {
        if (flags[r]) res[r] = sdb::binop(A(r), B(r), op);
    }
};

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ uint64_t block_sum_u64(uint64_t v)
{
    __shared__ uint64_t part[kMaxBlock / 32];
    v = warp_sum_u64(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) part[wid] = v;
    __syncthreads();
    uint64_t t = 0;
    if (wid == 0) {
        t = lane < (int)(blockDim.x >> 5) ? part[lane] : 0;
        t = warp_sum_u64(t);
    }
    __syncthreads();
    return t;  // valid in thread 0
}

// K7: one 64-bit atomic per block.
template <bool VEC>
__global__ void __launch_bounds__(kMaxBlock) k_sum(const int32_t *col, const uint8_t *flags, uint64_t n, uint64_t *acc)
{
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t s = 0;
    uint64_t start = 0;
    if (VEC) {
        const uint64_t groups = n >> 3;
        for (uint64_t g = tid; g < groups; g += stride) {
            uint32_t f = ldf8(flags, g << 3);
            if (f == 0) continue;
            int32_t c[8];
            ld8(col, g << 3, c);
#pragma unroll
            for (int j = 0; j < 8; j++)
                if (f & (1u << j)) s += sdb::widen(c[j]);
        }
        start = groups << 3;
    }
    for (uint64_t r = start + tid; r < n; r += stride)
        if (flags[r]) s += sdb::widen(col[r]);
    s = block_sum_u64(s);
    if (threadIdx.x == 0 && s != 0) atomicAdd(reinterpret_cast<unsigned long long *>(acc), (unsigned long long)s);
}

// K16
template <bool VEC>
__global__ void __launch_bounds__(kMaxBlock) k_count(const uint8_t *flags, uint64_t n, uint64_t *out)
{
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t s = 0, start = 0;
    if (VEC) {
        const uint64_t groups = n >> 3;
        for (uint64_t g = tid; g < groups; g += stride) s += __popc(ldf8(flags, g << 3));
        start = groups << 3;
    }
    for (uint64_t r = start + tid; r < n; r += stride) s += flags[r] != 0;
    s = block_sum_u64(s);
    if (threadIdx.x == 0 && s != 0) atomicAdd(reinterpret_cast<unsigned long long *>(out), (unsigned long long)s);
}

// min/max at load
__global__ void k_minmax_init(int32_t *mm)
{
    mm[0] = INT32_MAX;
    mm[1] = INT32_MIN;
}

template <bool VEC>
__global__ void __launch_bounds__(kMaxBlock) k_minmax(const int32_t *col, uint64_t n, int32_t *mm)
{
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    int32_t lo = INT32_MAX, hi = INT32_MIN;
    uint64_t start = 0;
    if (VEC) {
        const uint64_t groups = n >> 3;
        for (uint64_t g = tid; g < groups; g += stride) {
            int32_t c[8];
            ld8(col, g << 3, c);
#pragma unroll
            for (int j = 0; j < 8; j++) { lo = min(lo, c[j]); hi = max(hi, c[j]); }
        }
        start = groups << 3;
    }
    for (uint64_t r = start + tid; r < n; r += stride) { lo = min(lo, col[r]); hi = max(hi, col[r]); }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], lo);
        atomicMax(&mm[1], hi);
    }
}

// ---------------------------------------------------------------- K8, K9
struct GroupArgs {
    const int32_t *keys[8];
    int32_t mins[8];
    uint32_t mults[8];
    int g;
    const int32_t *val;
    const uint8_t *flags;
    uint64_t n, P;
    int32_t *out_keys[8];
    uint64_t *out_sum;
    uint32_t *occ;
};

__device__ __forceinline__ int64_t row_slot(const GroupArgs &a, uint64_t r)
{
    uint32_t h = 0;
    for (int j = 0; j < a.g; j++) h += ((uint32_t)a.keys[j][r] - (uint32_t)a.mins[j]) * a.mults[j];
    return sdb::group_slot(h, a.P);
}

__device__ __forceinline__ void claim_keys(const GroupArgs &a, int64_t h, uint64_t r)
{
    if (atomicExch(&a.occ[h], 1u) == 0u)
        for (int j = 0; j < a.g; j++) a.out_keys[j][h] = a.keys[j][r];
}

// Shared-memory privatised slot sums; a block's first touch of a slot also
// runs the global first-writer exchange; sums flush once per touched slot.
// One flagged row's slot update (K8): the first writer of a slot stores its
// keys, the value goes into the slot's sum.
template <bool SMEM>
__device__ __forceinline__ void group_row(const GroupArgs &a, uint64_t r, uint64_t *s_sum, uint32_t *s_occ)
{
    const int64_t h = row_slot(a, r);
    if (h < 0 || (uint64_t)h >= a.P) {
        atomicAdd(&g_errors, 1ull);
        return;
    }
    const unsigned long long v = (unsigned long long)sdb::widen(a.val[r]);
    if (SMEM) {
        if (atomicExch(&s_occ[h], 1u) == 0u) claim_keys(a, h, r);
        atomicAdd(reinterpret_cast<unsigned long long *>(&s_sum[h]), v);
    } else {
        if (a.occ[h] == 0u) claim_keys(a, h, r);
        atomicAdd(reinterpret_cast<unsigned long long *>(&a.out_sum[h]), v);
    }
}

// Grid-stride over 16-row groups: a thread reads its group's 16 flags with
// one 16-byte load (VEC: the flags are 16-byte aligned); the warp then lists
// its flagged rows in shared memory (a warp prefix sum of the lanes' counts)
// and updates them one row per lane, so the key and value loads of up to 32
// flagged rows are in flight together instead of one row after another.
constexpr int kGroupList = 32 * 16;  // a warp's rows per iteration

template <bool SMEM, bool VEC>
__global__ void __launch_bounds__(kThreads) k_groupby(const GroupArgs a)
{
    extern __shared__ uint64_t s_sum[];
    uint32_t *s_occ = reinterpret_cast<uint32_t *>(s_sum + (SMEM ? a.P : 0));
    uint32_t *s_list = s_occ + (SMEM ? ((a.P + 1) & ~1ull) : 0);  // 8-byte aligned after the table
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t *list = s_list + warp * kGroupList;
    if (SMEM) {
        for (uint64_t i = threadIdx.x; i < a.P; i += blockDim.x) { s_sum[i] = 0; s_occ[i] = 0; }
        __syncthreads();
    }
    const uint64_t groups = (a.n + 15) / 16;
    const uint64_t wstride = (uint64_t)gridDim.x * (kThreads / 32);
    // warp-uniform walk over chunks of 32 groups (512 rows)
    for (uint64_t c = (uint64_t)blockIdx.x * (kThreads / 32) + warp; c * 32 < groups; c += wstride) {
        const uint64_t gi = c * 32 + lane;
        const uint64_t r0 = gi * 16;
        uint32_t m = 0;  // bit b: row r0 + b is flagged
        if (gi < groups) {
            if (VEC && r0 + 16 <= a.n) {
                const uint4 q = __ldcs(reinterpret_cast<const uint4 *>(a.flags + r0));
                const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int b = 0; b < 4; b++) m |= (uint32_t)(((w[j] >> (8 * b)) & 0xffu) != 0) << (4 * j + b);
            } else {
                for (int b = 0; b < 16 && r0 + b < a.n; b++) m |= (uint32_t)(a.flags[r0 + b] != 0) << b;
            }
        }
        // this lane's rows go to list[pos .. pos + popc(m))
        const uint32_t cnt = __popc(m);
        uint32_t pos = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, pos, o);
            if (lane >= (uint32_t)o) pos += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, pos, 31);
        pos -= cnt;
        if (total == 0) continue;
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            list[pos++] = lane * 16 + (uint32_t)b;
        }
        __syncwarp();
        const uint64_t base = c * 32 * 16;
        for (uint32_t i = lane; i < total; i += 32) group_row<SMEM>(a, base + list[i], s_sum, s_occ);
        __syncwarp();
    }
    if (SMEM) {
        __syncthreads();
        for (uint64_t i = threadIdx.x; i < a.P; i += blockDim.x)
            if (s_occ[i]) atomicAdd(reinterpret_cast<unsigned long long *>(&a.out_sum[i]), (unsigned long long)s_sum[i]);
    }
}

struct OccToFlags {
    const uint32_t *occ; uint8_t *f;
    __device__ void group(uint64_t r0) const
    {
        const uint4 *q = reinterpret_cast<const uint4 *>(occ + r0);
        uint4 a = q[0], b = q[1];
        uint32_t m = (a.x != 0) | ((a.y != 0) << 1) | ((a.z != 0) << 2) | ((a.w != 0) << 3) |
                     ((b.x != 0) << 4) | ((b.y != 0) << 5) | ((b.z != 0) << 6) | ((b.w != 0) << 7);
        stf8(f, r0, m);
    }
    __device__ void row(uint64_t r) const { f[r] = occ[r] != 0; }
};

// ---------------------------------------------------------------- K10 - K13
__global__ void __launch_bounds__(kMaxBlock) k_build_keys(const int32_t *key, const uint8_t *flags, uint64_t n,
                                                         uint8_t *ht, int32_t mn, int32_t len)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        int64_t h = sdb::ht_slot(key[r], len, mn);
        if (h < 0 || h >= len) { atomicAdd(&g_errors, 1ull); continue; }
        ht[h] = flags[r] ? 1 : 0;
    }
}

__global__ void __launch_bounds__(kMaxBlock) k_build_kv(const int32_t *key, const int32_t *val, const uint8_t *flags,
                                                       uint64_t n, int32_t *ht2, int32_t mn, int32_t len)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        int64_t h = sdb::ht_slot(key[r], len, mn);
        if (h < 0 || h >= len) { atomicAdd(&g_errors, 1ull); continue; }
        if (flags[r]) {
            ht2[2 * h] = 1;
            ht2[2 * h + 1] = val[r];
        } else {
            ht2[2 * h] = 0;
        }
    }
}

struct ProbeSemi {
    const int32_t *key; const uint8_t *in; uint8_t *out; const uint8_t *ht; int32_t mn, mx;
    __device__ bool one(int32_t k, bool fin) const
    {
        return fin && k >= mn && k <= mx && __ldg(ht + ((uint32_t)k - (uint32_t)mn)) != 0;
    }
    __device__ void group(uint64_t r0) const
    {
        uint32_t f = ldf8(in, r0), m = 0;
        if (f) {
            int32_t k[8];
            ld8(key, r0, k);
#pragma unroll
            for (int j = 0; j < 8; j++) m |= (uint32_t)one(k[j], (f >> j) & 1u) << j;
        }
        stf8(out, r0, m);
    }
    __device__ void row(uint64_t r) const { out[r] = in[r] ? one(key[r], true) : 0; }
};

template <bool HT8>
struct ProbeFull {
    const int32_t *key; int32_t *val_out; const uint8_t *in; uint8_t *out; const int32_t *ht2; int32_t mn, mx;
    __device__ bool one(int32_t k, bool fin, int32_t &v) const
    {
        if (!fin || k < mn || k > mx) return false;
        const uint32_t h = (uint32_t)k - (uint32_t)mn;
        int32_t occ, val;
        if (HT8) {
            int2 e = __ldg(reinterpret_cast<const int2 *>(ht2) + h);
            occ = e.x; val = e.y;
        } else {
            occ = __ldg(ht2 + 2 * (uint64_t)h);
            val = __ldg(ht2 + 2 * (uint64_t)h + 1);
        }
        v = val;
        return occ == 1;
    }
    __device__ void group(uint64_t r0) const
    {
        uint32_t f = ldf8(in, r0), m = 0;
        if (f) {
            int32_t k[8];
            ld8(key, r0, k);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                int32_t v;
                if (one(k[j], (f >> j) & 1u, v)) {
                    val_out[r0 + j] = v;
                    m |= 1u << j;
                }
            }
        }
        stf8(out, r0, m);
    }
    __device__ void row(uint64_t r) const
    {
        int32_t v;
        if (in[r] && one(key[r], true, v)) {
            val_out[r] = v;
            out[r] = 1;
        } else {
            out[r] = 0;
        }
    }
};

// ------------------------------------------- K10 - K13 on open-addressing tables
// The same builds and probes over a table of 2^lg slots (sdb::oa_put /
// oa_find): a build row writes its key's slot as the direct-address build
// writes key - min (live: hit and value, dead: miss); `fresh` (the table is
// all zero and no other build writes it) skips dead rows, whose miss the
// empty table already reads.
__global__ void __launch_bounds__(kMaxBlock) k_build_keys_oa(const int32_t *key, const uint8_t *flags, uint64_t n,
                                                            uint32_t *ht, int lg, int32_t mn, int32_t mx, int fresh)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        const bool live = flags[r] != 0;
        if (!live && fresh) continue;
        const int32_t k = key[r];
        if (k < mn || k > mx || sdb::oa_put<1>(ht, lg, sdb::oa_tag(k, mn), live) == -2) atomicAdd(&g_errors, 1ull);
    }
}

__global__ void __launch_bounds__(kMaxBlock) k_build_kv_oa(const int32_t *key, const int32_t *val, const uint8_t *flags,
                                                          uint64_t n, int32_t *ht2, int lg, int32_t mn, int32_t mx,
                                                          int fresh)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        const bool live = flags[r] != 0;
        if (!live && fresh) continue;
        const int32_t k = key[r];
        if (k < mn || k > mx) {
            atomicAdd(&g_errors, 1ull);
            continue;
        }
        const int64_t h = sdb::oa_put<2>(reinterpret_cast<uint32_t *>(ht2), lg, sdb::oa_tag(k, mn), live);
        if (h == -2) atomicAdd(&g_errors, 1ull);
        else if (h >= 0 && live) ht2[2 * h + 1] = val[r];
    }
}

struct ProbeSemiOA {
    const int32_t *key; const uint8_t *in; uint8_t *out; const uint32_t *ht; int lg; int32_t mn, mx;
    __device__ bool one(int32_t k, bool fin) const
    {
        if (!fin || k < mn || k > mx) return false;
        const int64_t h = sdb::oa_find<1>(ht, lg, sdb::oa_tag(k, mn));
        return h >= 0 && (__ldg(ht + h) & 1u);
    }
    __device__ void group(uint64_t r0) const
    {
        uint32_t f = ldf8(in, r0), m = 0;
        if (f) {
            int32_t k[8];
            ld8(key, r0, k);
#pragma unroll
            for (int j = 0; j < 8; j++) m |= (uint32_t)one(k[j], (f >> j) & 1u) << j;
        }
        stf8(out, r0, m);
    }
    __device__ void row(uint64_t r) const { out[r] = in[r] ? one(key[r], true) : 0; }
};

struct ProbeFullOA {
    const int32_t *key; int32_t *val_out; const uint8_t *in; uint8_t *out; const int32_t *ht2; int lg; int32_t mn, mx;
    __device__ bool one(int32_t k, bool fin, int32_t &v) const
    {
        if (!fin || k < mn || k > mx) return false;
        const int64_t h = sdb::oa_find<2>(reinterpret_cast<const uint32_t *>(ht2), lg, sdb::oa_tag(k, mn));
        if (h < 0) return false;
        const int2 e = __ldg(reinterpret_cast<const int2 *>(ht2) + h);
        v = e.y;
        return (e.x & 1) != 0;
    }
    __device__ void group(uint64_t r0) const
    {
        uint32_t f = ldf8(in, r0), m = 0;
        if (f) {
            int32_t k[8];
            ld8(key, r0, k);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                int32_t v;
                if (one(k[j], (f >> j) & 1u, v)) {
                    val_out[r0 + j] = v;
                    m |= 1u << j;
                }
            }
        }
        stf8(out, r0, m);
    }
    __device__ void row(uint64_t r) const
    {
        int32_t v;
        if (in[r] && one(key[r], true, v)) {
            val_out[r] = v;
            out[r] = 1;
        } else {
            out[r] = 0;
        }
    }
};

// ---------------------------------------------------------------- K14, K15
constexpr int kCompactRowsPerThread = 16;
constexpr int kCompactChunk = kThreads * kCompactRowsPerThread;  // rows per block-chunk

__device__ __forceinline__ uint32_t count16(const uint8_t *flags, uint64_t r0, uint64_t n)
{
    if (r0 + 16 <= n) {
        uint4 w = *reinterpret_cast<const uint4 *>(flags + r0);
        return __popc(nz_bits4(w.x)) + __popc(nz_bits4(w.y)) + __popc(nz_bits4(w.z)) + __popc(nz_bits4(w.w));
    }
    uint32_t c = 0;
    for (uint64_t r = r0; r < n; r++) c += flags[r] != 0;
    return c;
}

__device__ __forceinline__ uint32_t mask16(const uint8_t *flags, uint64_t r0, uint64_t n)
{
    if (r0 + 16 <= n) {
        uint4 w = *reinterpret_cast<const uint4 *>(flags + r0);
        return nz_bits4(w.x) | (nz_bits4(w.y) << 4) | (nz_bits4(w.z) << 8) | (nz_bits4(w.w) << 12);
    }
    uint32_t m = 0;
    for (uint64_t r = r0; r < n; r++) m |= (uint32_t)(flags[r] != 0) << (r - r0);
    return m;
}

// Exclusive block scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total)
{
    __shared__ uint32_t warp_tot[kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < kThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kThreads / 32) warp_tot[lane] = t;  // inclusive prefix of warps
    }
    __syncthreads();
    uint32_t base = wid ? warp_tot[wid - 1] : 0;
    *total = warp_tot[kThreads / 32 - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void __launch_bounds__(kThreads) k_compact_count(const uint8_t *flags, uint64_t n, uint32_t *block_counts,
                                                            uint64_t nchunks)
{
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint64_t r0 = c * kCompactChunk + (uint64_t)threadIdx.x * kCompactRowsPerThread;
        uint32_t v = r0 < n ? count16(flags, r0, n) : 0;
        uint32_t tot;
        block_exclusive_scan(v, &tot);
        if (threadIdx.x == 0) block_counts[c] = tot;
    }
}

// Single block: exclusive scan of the chunk counts in place; *count = total.
__global__ void __launch_bounds__(kThreads) k_compact_scan(uint32_t *block_counts, uint64_t nchunks, uint32_t *count)
{
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < nchunks; base += kThreads) {
        const uint64_t i = base + threadIdx.x;
        uint32_t v = i < nchunks ? block_counts[i] : 0;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, &tot);
        if (i < nchunks) block_counts[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = carry;
}

__global__ void __launch_bounds__(kThreads) k_compact_write(const uint8_t *flags, uint64_t n, const uint32_t *offsets,
                                                            uint64_t nchunks, int32_t *ids)
{
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint64_t r0 = c * kCompactChunk + (uint64_t)threadIdx.x * kCompactRowsPerThread;
        uint32_t m = r0 < n ? mask16(flags, r0, n) : 0;
        uint32_t tot;
        uint32_t pos = offsets[c] + block_exclusive_scan(__popc(m), &tot);
        while (m) {
            int j = __ffs(m) - 1;
            ids[pos++] = (int32_t)(r0 + j);
            m &= m - 1;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kMaxBlock) k_gather(const T *src, const int32_t *ids, const uint32_t *count, T *dst,
                                                     uint64_t cap)
{
    const uint64_t c = min((uint64_t)*count, cap);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < c; i += stride) dst[i] = src[ids[i]];
}

// Ordered compaction and the gathers of every result column of a small
// segment (a group-by result) in one block of 1024 threads: thread t owns
// rows [t*per, (t+1)*per), counts its flagged rows, a block scan gives its
// first output position, then it copies its rows' values in row order.
constexpr uint32_t kSmallCompactMax = 65536;
static_assert(kSmallCompactMax <= 1024u * 64u, "k_compact_gather_small keeps a thread's flags in a 64-bit mask");
constexpr int kSmallCompactCols = 8;
struct SmallCompact {
    const void *flags;  // uint8 flags, or uint32 occupancy words (flag = word != 0)
    uint32_t n;
    int32_t ncols;
    const void *src[kSmallCompactCols];
    void *dst[kSmallCompactCols];
    int32_t wide[kSmallCompactCols];  // 1: uint64 column
    uint32_t *count;
};

template <typename F>
__global__ void __launch_bounds__(1024) k_compact_gather_small(const __grid_constant__ SmallCompact a)
{
    const F *flags = static_cast<const F *>(a.flags);
    __shared__ uint32_t s_warp[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t per = (a.n + 1023u) / 1024u;  // at most 64: n <= kSmallCompactMax
    const uint32_t b = min(threadIdx.x * per, a.n), e = min(b + per, a.n);
    // the thread's run of flags as a bit mask, eight independent loads at a
    // time (one latency per eight flags instead of one per flag)
    uint64_t m = 0;
    for (uint32_t j = b; j < e; j += 8) {
        F f[8];
#pragma unroll
        for (int k = 0; k < 8; k++) f[k] = j + k < e ? flags[j + k] : F(0);
#pragma unroll
        for (int k = 0; k < 8; k++) m |= (uint64_t)(f[k] != 0) << (j - b + k);
    }
    const uint32_t cnt = __popcll(m);
    uint32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t pos = x - cnt + (warp ? s_warp[warp - 1] : 0);
    if (threadIdx.x == 1023) *a.count = pos + cnt;
    // two live rows per round, every column of both loaded before any store
    while (m) {
        const uint32_t i0 = b + (uint32_t)__ffsll((long long)m) - 1u;
        m &= m - 1;
        const bool two = m != 0;
        const uint32_t i1 = two ? b + (uint32_t)__ffsll((long long)m) - 1u : i0;
        if (two) m &= m - 1;
        uint64_t v0[kSmallCompactCols], v1[kSmallCompactCols];
#pragma unroll
        for (int c = 0; c < kSmallCompactCols; c++) {
            if (c < a.ncols) {
                if (a.wide[c]) {
                    v0[c] = static_cast<const uint64_t *>(a.src[c])[i0];
                    v1[c] = static_cast<const uint64_t *>(a.src[c])[i1];
                } else {
                    v0[c] = (uint32_t) static_cast<const int32_t *>(a.src[c])[i0];
                    v1[c] = (uint32_t) static_cast<const int32_t *>(a.src[c])[i1];
                }
            }
        }
#pragma unroll
        for (int c = 0; c < kSmallCompactCols; c++) {
            if (c < a.ncols) {
                if (a.wide[c]) {
                    static_cast<uint64_t *>(a.dst[c])[pos] = v0[c];
                    if (two) static_cast<uint64_t *>(a.dst[c])[pos + 1] = v1[c];
                } else {
                    static_cast<int32_t *>(a.dst[c])[pos] = (int32_t)(uint32_t)v0[c];
                    if (two) static_cast<int32_t *>(a.dst[c])[pos + 1] = (int32_t)(uint32_t)v1[c];
                }
            }
        }
        pos += two ? 2u : 1u;
    }
}

// ---------------------------------------------------------------- data gen
__global__ void __launch_bounds__(kThreads) k_gen_uniform(int32_t *dst, uint64_t n, uint64_t row0, uint64_t key,
                                                          int32_t lo, int32_t hi)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = sdb::uniform_from_key(key, row0 + i, lo, hi);
}

__global__ void __launch_bounds__(kThreads) k_gen_dates(int32_t *dst, uint64_t n, uint64_t row0, uint64_t key,
                                                        int32_t ndays)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = sdb::datekey_of_day(sdb::uniform_from_key(key, row0 + i, 0, ndays - 1));
}

template <class F>
void parallel_rows(uint64_t n, F f)
{
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    if (n < (1u << 16)) nt = 1;
    std::vector<std::thread> th;
    uint64_t per = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
        uint64_t a = t * per, b = std::min<uint64_t>(n, a + per);
        if (a >= b) break;
        th.emplace_back([=] { for (uint64_t i = a; i < b; i++) f(i); });
    }
    for (auto &x : th) x.join();
}

bool flags_ok(const uint8_t *p) { return sdb::aligned(p, 8); }
bool col_ok(const void *p) { return sdb::aligned(p, 16); }

// Natural alignment of every typed pointer (int32/uint32: 4, uint64: 8).  A
// misaligned typed access would fault the device, so the host rejects it.
bool nat4(std::initializer_list<const void *> ps)
{
    for (auto p : ps)
        if (!sdb::aligned(p, 4)) return false;
    return true;
}
bool nat8(const void *p) { return sdb::aligned(p, 8); }
#define SDB_REQUIRE_ALIGNED(cond, what) \
    if (!(cond)) return sdb_set_error(SDB_ERR_INVALID, "%s: pointer not naturally aligned", what)

}  // namespace

// ============================================================== C ABI
extern "C" {

int sdb_fill_u8(uint8_t *flags, uint64_t n, uint8_t v, sdb_stream_t stream)
{
    if (n && !flags) return sdb_set_error(SDB_ERR_INVALID, "sdb_fill_u8: NULL buffer");
    return launch_map(n, flags_ok(flags), FillU8{flags, v}, (cudaStream_t)stream, "sdb_fill_u8", SDB_OPK_FILL_U8);
}

int sdb_select_lit(const int32_t *col, int32_t v, int cmp_op, int logic_op, const uint8_t *in, uint8_t *out,
                   uint64_t n, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({col}), "sdb_select_lit");
    if (n && (!col || !in || !out)) return sdb_set_error(SDB_ERR_INVALID, "sdb_select_lit: NULL buffer");
    bool vec = col_ok(col) && flags_ok(in) && flags_ok(out);
    return launch_map(n, vec, SelectLit{col, v, cmp_op, logic_op, in, out}, (cudaStream_t)stream, "sdb_select_lit", SDB_OPK_SELECT_LIT);
}

int sdb_select_cols(const int32_t *a, const int32_t *b, int cmp_op, int logic_op, const uint8_t *in, uint8_t *out,
                    uint64_t n, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({a, b}), "sdb_select_cols");
    if (n && (!a || !b || !in || !out)) return sdb_set_error(SDB_ERR_INVALID, "sdb_select_cols: NULL buffer");
    bool vec = col_ok(a) && col_ok(b) && flags_ok(in) && flags_ok(out);
    return launch_map(n, vec, SelectCols{a, b, cmp_op, logic_op, in, out}, (cudaStream_t)stream, "sdb_select_cols", SDB_OPK_SELECT_COLS);
}

int sdb_logical(int logic_op, const uint8_t *in, const uint8_t *local, uint8_t *out, uint64_t n, sdb_stream_t stream)
{
    if (n && (!in || !local || !out)) return sdb_set_error(SDB_ERR_INVALID, "sdb_logical: NULL buffer");
    bool vec = flags_ok(in) && flags_ok(local) && flags_ok(out);
    return launch_map(n, vec, Logical{logic_op, in, local, out}, (cudaStream_t)stream, "sdb_logical", SDB_OPK_LOGICAL);
}

int sdb_fill_i32(int32_t *dst, int32_t v, uint64_t n, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({dst}), "sdb_fill_i32");
    if (n && !dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_fill_i32: NULL buffer");
    return launch_map(n, col_ok(dst), FillI32{dst, v}, (cudaStream_t)stream, "sdb_fill_i32", SDB_OPK_FILL_I32);
}

static int binop_common(int32_t *res, const int32_t *a, const int32_t *b, int32_t la, int32_t lb, int op, int mode,
                        const uint8_t *flags, uint64_t n, sdb_stream_t stream, const char *what)
{
    SDB_REQUIRE_ALIGNED(nat4({res, a, b}), what);
    if (op < SDB_MUL || op > SDB_SUB) return sdb_set_error(SDB_ERR_INVALID, "%s: unknown operation %d", what, op);
    if (n && (!res || !flags || (mode != 1 && !a) || (mode != 2 && !b)))
        return sdb_set_error(SDB_ERR_INVALID, "%s: NULL buffer", what);
    bool vec = col_ok(res) && col_ok(a) && col_ok(b) && flags_ok(flags);
    return launch_map(n, vec, Binop{res, a, b, la, lb, op, mode, flags}, (cudaStream_t)stream, what, SDB_OPK_BINOP);
}

int sdb_binop_cc(int32_t *res, const int32_t *a, const int32_t *b, int bin_op, const uint8_t *flags, uint64_t n,
                 sdb_stream_t stream)
{
    return binop_common(res, a, b, 0, 0, bin_op, 0, flags, n, stream, "sdb_binop_cc");
}

int sdb_binop_lc(int32_t *res, int32_t a, const int32_t *b, int bin_op, const uint8_t *flags, uint64_t n,
                 sdb_stream_t stream)
{
    return binop_common(res, nullptr, b, a, 0, bin_op, 1, flags, n, stream, "sdb_binop_lc");
}

int sdb_binop_cl(int32_t *res, const int32_t *a, int32_t b, int bin_op, const uint8_t *flags, uint64_t n,
                 sdb_stream_t stream)
{
    return binop_common(res, a, nullptr, 0, b, bin_op, 2, flags, n, stream, "sdb_binop_cl");
}

int sdb_sum_i32_u64(const int32_t *col, const uint8_t *flags, uint64_t n, uint64_t *acc, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({col}) && nat8(acc), "sdb_sum_i32_u64");
    if (!acc || (n && (!col || !flags))) return sdb_set_error(SDB_ERR_INVALID, "sdb_sum_i32_u64: NULL buffer");
    if (n == 0) return SDB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const LaunchShape sh = op_shape(SDB_OPK_SUM, n, 4);
    if (col_ok(col) && flags_ok(flags))
        k_sum<true><<<grid_of((n + 7) / 8, sh), sh.block, 0, s>>>(col, flags, n, acc);
    else
        k_sum<false><<<grid_of(n, sh), sh.block, 0, s>>>(col, flags, n, acc);
    return sdb_check_launch("sdb_sum_i32_u64");
}

int sdb_count_flags(const uint8_t *flags, uint64_t n, uint64_t *out, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat8(out), "sdb_count_flags");
    if (!out || (n && !flags)) return sdb_set_error(SDB_ERR_INVALID, "sdb_count_flags: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(out, 0, sizeof(uint64_t), s) != cudaSuccess) return sdb_check_launch("sdb_count_flags");
    if (n == 0) return SDB_OK;
    const LaunchShape sh = op_shape(SDB_OPK_COUNT_FLAGS, n, 4);
    if (flags_ok(flags))
        k_count<true><<<grid_of((n + 7) / 8, sh), sh.block, 0, s>>>(flags, n, out);
    else
        k_count<false><<<grid_of(n, sh), sh.block, 0, s>>>(flags, n, out);
    return sdb_check_launch("sdb_count_flags");
}

int sdb_min_max_i32(const int32_t *col, uint64_t n, int32_t *minmax, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({col, minmax}), "sdb_min_max_i32");
    if (n == 0 || !col || !minmax) return sdb_set_error(SDB_ERR_INVALID, "sdb_min_max_i32: empty column or NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    k_minmax_init<<<1, 1, 0, s>>>(minmax);
    const LaunchShape sh = op_shape(SDB_OPK_MIN_MAX, n, 4);
    if (col_ok(col))
        k_minmax<true><<<grid_of((n + 7) / 8, sh), sh.block, 0, s>>>(col, n, minmax);
    else
        k_minmax<false><<<grid_of(n, sh), sh.block, 0, s>>>(col, n, minmax);
    sdb_count_launches(1);
    return sdb_check_launch("sdb_min_max_i32");
}

int sdb_groupby_sum(const int32_t *const *keys, const int32_t *mins, const int32_t *maxs, int g, const int32_t *val,
                    const uint8_t *flags, uint64_t n, uint64_t P, int32_t *const *out_keys, uint64_t *out_sum,
                    uint32_t *occ, sdb_stream_t stream)
{
    if (g < 1 || g > 8) return sdb_set_error(SDB_ERR_INVALID, "sdb_groupby_sum: g=%d outside [1,8]", g);
    if (!keys || !mins || !maxs || !out_keys) return sdb_set_error(SDB_ERR_INVALID, "sdb_groupby_sum: NULL host array");
    if (P == 0) return sdb_set_error(SDB_ERR_INVALID, "sdb_groupby_sum: P == 0");
    if (n && (!val || !flags || !out_sum || !occ)) return sdb_set_error(SDB_ERR_INVALID, "sdb_groupby_sum: NULL buffer");
    SDB_REQUIRE_ALIGNED(nat4({val, occ}) && nat8(out_sum), "sdb_groupby_sum");
    for (int j = 0; j < g; j++) SDB_REQUIRE_ALIGNED(nat4({keys[j], out_keys[j]}), "sdb_groupby_sum");
    GroupArgs a{};
    uint32_t mult = 1;
    for (int j = 0; j < g; j++) {
        if (n && (!keys[j] || !out_keys[j])) return sdb_set_error(SDB_ERR_INVALID, "sdb_groupby_sum: NULL key column");
        a.keys[j] = keys[j];
        a.out_keys[j] = out_keys[j];
        a.mins[j] = mins[j];
        a.mults[j] = mult;
        mult *= (uint32_t)maxs[j] - (uint32_t)mins[j] + 1u;
    }
    a.g = g; a.val = val; a.flags = flags; a.n = n; a.P = P; a.out_sum = out_sum; a.occ = occ;
    if (n == 0) return SDB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    // the slot table (P <= 8192: 12 B per slot, the occupancy words padded to
    // 8 bytes) and every warp's row list
    const size_t list_bytes = (size_t)(kThreads / 32) * kGroupList * sizeof(uint32_t);
    const size_t smem = (P <= 8192 ? (size_t)P * sizeof(uint64_t) + ((P + 1) & ~1ull) * sizeof(uint32_t) : 0) + list_bytes;
    const uint64_t groups = (n + 15) / 16;
    const bool vec = sdb::aligned(flags, 16);
    static const bool attr_set = [] {  // once, thread-safe
        const int most = 8192 * 12 + (kThreads / 32) * kGroupList * 4;
        cudaFuncSetAttribute(k_groupby<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        cudaFuncSetAttribute(k_groupby<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        return true;
    }();
    (void)attr_set;
    // a block per 32 x 8 groups, capped at the resident blocks
    const uint64_t want = (groups + 32 * (kThreads / 32) - 1) / (32 * (kThreads / 32));
    if (P <= 8192) {
        const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)sdb::device_sms() * 2));
        if (vec)
            k_groupby<true, true><<<blocks, kThreads, smem, s>>>(a);
        else
            k_groupby<true, false><<<blocks, kThreads, smem, s>>>(a);
    } else {
        const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)sdb::device_sms() * 8));
        if (vec)
            k_groupby<false, true><<<blocks, kThreads, smem, s>>>(a);
        else
            k_groupby<false, false><<<blocks, kThreads, smem, s>>>(a);
    }
    return sdb_check_launch("sdb_groupby_sum");
}

int sdb_occ_to_flags(const uint32_t *occ, uint8_t *flags, uint64_t P, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({occ}), "sdb_occ_to_flags");
    if (P && (!occ || !flags)) return sdb_set_error(SDB_ERR_INVALID, "sdb_occ_to_flags: NULL buffer");
    return launch_map(P, col_ok(occ) && flags_ok(flags), OccToFlags{occ, flags}, (cudaStream_t)stream,
                      "sdb_occ_to_flags", SDB_OPK_OCC_TO_FLAGS);
}

int sdb_ht_build_keys(const int32_t *key, const uint8_t *flags, uint64_t n, uint8_t *ht, int32_t min, int32_t len,
                      sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key}), "sdb_ht_build_keys");
    if (n && (!key || !flags || !ht)) return sdb_set_error(SDB_ERR_INVALID, "sdb_ht_build_keys: NULL buffer");
    if (n == 0) return SDB_OK;
    const LaunchShape sh = op_shape(SDB_OPK_BUILD_KEYS, n, 8);
    k_build_keys<<<grid_of(n, sh), sh.block, 0, (cudaStream_t)stream>>>(key, flags, n, ht, min, len);
    return sdb_check_launch("sdb_ht_build_keys");
}

int sdb_probe_semi(const int32_t *key, const uint8_t *in, uint8_t *out, uint64_t n, const uint8_t *ht, int32_t min,
                   int32_t max, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key}), "sdb_probe_semi");
    if (n && (!key || !in || !out || !ht)) return sdb_set_error(SDB_ERR_INVALID, "sdb_probe_semi: NULL buffer");
    bool vec = col_ok(key) && flags_ok(in) && flags_ok(out);
    return launch_map(n, vec, ProbeSemi{key, in, out, ht, min, max}, (cudaStream_t)stream, "sdb_probe_semi", SDB_OPK_PROBE_SEMI);
}

int sdb_ht_build_kv(const int32_t *key, const int32_t *val, const uint8_t *flags, uint64_t n, int32_t *ht2,
                    int32_t min, int32_t len, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key, val, ht2}), "sdb_ht_build_kv");
    if (n && (!key || !val || !flags || !ht2)) return sdb_set_error(SDB_ERR_INVALID, "sdb_ht_build_kv: NULL buffer");
    if (n == 0) return SDB_OK;
    const LaunchShape sh = op_shape(SDB_OPK_BUILD_KV, n, 8);
    k_build_kv<<<grid_of(n, sh), sh.block, 0, (cudaStream_t)stream>>>(key, val, flags, n, ht2, min, len);
    return sdb_check_launch("sdb_ht_build_kv");
}

int sdb_probe_full(const int32_t *key, int32_t *val_out, const uint8_t *in, uint8_t *out, uint64_t n,
                   const int32_t *ht2, int32_t min, int32_t max, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key, val_out, ht2}), "sdb_probe_full");
    if (n && (!key || !val_out || !in || !out || !ht2))
        return sdb_set_error(SDB_ERR_INVALID, "sdb_probe_full: NULL buffer");
    bool vec = col_ok(key) && flags_ok(in) && flags_ok(out);
    cudaStream_t s = (cudaStream_t)stream;
    if (sdb::aligned(ht2, 8))
        return launch_map(n, vec, ProbeFull<true>{key, val_out, in, out, ht2, min, max}, s, "sdb_probe_full", SDB_OPK_PROBE_FULL);
    return launch_map(n, vec, ProbeFull<false>{key, val_out, in, out, ht2, min, max}, s, "sdb_probe_full", SDB_OPK_PROBE_FULL);
}

int sdb_oa_log2_slots(uint64_t build_rows)
{
    if (build_rows > (1ull << 30)) return sdb_set_error(SDB_ERR_INVALID, "sdb_oa_log2_slots: more than 2^30 rows");
    int lg = 4;
    while ((1ull << lg) < 2 * build_rows) lg++;
    return lg;
}

// Checks the arguments every open-addressing entry shares.
static int oa_check(const char *what, int lg, int32_t mn, int32_t mx, const void *ht, uintptr_t align)
{
    if (lg < 1 || lg > 31) return sdb_set_error(SDB_ERR_INVALID, "%s: log2_slots=%d outside [1,31]", what, lg);
    if (mn > mx || (uint32_t)mx - (uint32_t)mn >= 0x7fffffffu)
        return sdb_set_error(SDB_ERR_INVALID, "%s: key range [%d,%d] empty or 2^31 keys or more", what, mn, mx);
    if (!sdb::aligned(ht, align)) return sdb_set_error(SDB_ERR_INVALID, "%s: table not %d-byte aligned", what, (int)align);
    return SDB_OK;
}

int sdb_ht_build_keys_oa(const int32_t *key, const uint8_t *flags, uint64_t n, uint32_t *ht, int log2_slots,
                         int32_t min, int32_t max, int fresh, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key}), "sdb_ht_build_keys_oa");
    if (n && (!key || !flags || !ht)) return sdb_set_error(SDB_ERR_INVALID, "sdb_ht_build_keys_oa: NULL buffer");
    int st = oa_check("sdb_ht_build_keys_oa", log2_slots, min, max, ht, 4);
    if (st != SDB_OK || n == 0) return st;
    const LaunchShape sh = op_shape(SDB_OPK_BUILD_KEYS, n, 8);
    k_build_keys_oa<<<grid_of(n, sh), sh.block, 0, (cudaStream_t)stream>>>(key, flags, n, ht, log2_slots, min, max,
                                                                          fresh);
    return sdb_check_launch("sdb_ht_build_keys_oa");
}

int sdb_probe_semi_oa(const int32_t *key, const uint8_t *in, uint8_t *out, uint64_t n, const uint32_t *ht,
                      int log2_slots, int32_t min, int32_t max, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key}), "sdb_probe_semi_oa");
    if (n && (!key || !in || !out || !ht)) return sdb_set_error(SDB_ERR_INVALID, "sdb_probe_semi_oa: NULL buffer");
    int st = oa_check("sdb_probe_semi_oa", log2_slots, min, max, ht, 4);
    if (st != SDB_OK) return st;
    bool vec = col_ok(key) && flags_ok(in) && flags_ok(out);
    return launch_map(n, vec, ProbeSemiOA{key, in, out, ht, log2_slots, min, max}, (cudaStream_t)stream,
                      "sdb_probe_semi_oa", SDB_OPK_PROBE_SEMI);
}

int sdb_ht_build_kv_oa(const int32_t *key, const int32_t *val, const uint8_t *flags, uint64_t n, int32_t *ht2,
                       int log2_slots, int32_t min, int32_t max, int fresh, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key, val}), "sdb_ht_build_kv_oa");
    if (n && (!key || !val || !flags || !ht2)) return sdb_set_error(SDB_ERR_INVALID, "sdb_ht_build_kv_oa: NULL buffer");
    int st = oa_check("sdb_ht_build_kv_oa", log2_slots, min, max, ht2, 8);
    if (st != SDB_OK || n == 0) return st;
    const LaunchShape sh = op_shape(SDB_OPK_BUILD_KV, n, 8);
    k_build_kv_oa<<<grid_of(n, sh), sh.block, 0, (cudaStream_t)stream>>>(key, val, flags, n, ht2, log2_slots, min,
                                                                        max, fresh);
    return sdb_check_launch("sdb_ht_build_kv_oa");
}

int sdb_probe_full_oa(const int32_t *key, int32_t *val_out, const uint8_t *in, uint8_t *out, uint64_t n,
                      const int32_t *ht2, int log2_slots, int32_t min, int32_t max, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({key, val_out}), "sdb_probe_full_oa");
    if (n && (!key || !val_out || !in || !out || !ht2))
        return sdb_set_error(SDB_ERR_INVALID, "sdb_probe_full_oa: NULL buffer");
    int st = oa_check("sdb_probe_full_oa", log2_slots, min, max, ht2, 8);
    if (st != SDB_OK) return st;
    bool vec = col_ok(key) && flags_ok(in) && flags_ok(out);
    return launch_map(n, vec, ProbeFullOA{key, val_out, in, out, ht2, log2_slots, min, max}, (cudaStream_t)stream,
                      "sdb_probe_full_oa", SDB_OPK_PROBE_FULL);
}

size_t sdb_compact_scratch_bytes(uint64_t n)
{
    uint64_t nchunks = (n + kCompactChunk - 1) / kCompactChunk;
    return (size_t)((nchunks * sizeof(uint32_t) + 255) & ~(uint64_t)255);
}

int sdb_compact_row_ids(const uint8_t *flags, uint64_t n, int32_t *ids, uint32_t *count, void *scratch,
                        size_t scratch_bytes, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({ids, count, scratch}), "sdb_compact_row_ids");
    if (!count) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_row_ids: NULL count");
    if (n > (uint64_t)INT32_MAX + 1) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_row_ids: n too large for int32 ids");
    cudaStream_t s = (cudaStream_t)stream;
    if (n == 0) {
        if (cudaMemsetAsync(count, 0, sizeof(uint32_t), s) != cudaSuccess) return sdb_check_launch("sdb_compact_row_ids");
        return SDB_OK;
    }
    if (!flags || !ids) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_row_ids: NULL buffer");
    if (!sdb::aligned(flags, 16)) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_row_ids: flags must be 16-byte aligned");
    const uint64_t nchunks = (n + kCompactChunk - 1) / kCompactChunk;
    if (!scratch || scratch_bytes < sdb_compact_scratch_bytes(n))
        return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_row_ids: scratch needs %zu bytes", sdb_compact_scratch_bytes(n));
    uint32_t *bc = static_cast<uint32_t *>(scratch);
    const unsigned grid = (unsigned)std::min<uint64_t>(nchunks, (uint64_t)sdb::device_sms() * 8);
    k_compact_count<<<grid, kThreads, 0, s>>>(flags, n, bc, nchunks);
    k_compact_scan<<<1, kThreads, 0, s>>>(bc, nchunks, count);
    k_compact_write<<<grid, kThreads, 0, s>>>(flags, n, bc, nchunks, ids);
    sdb_count_launches(2);
    return sdb_check_launch("sdb_compact_row_ids");
}

}  // extern "C"

// ---------------------------------------------------------------- no-allocation compaction
// Scratch of sdb_compact_row_ids_noalloc: the per-chunk counts for one
// segment of up to SDB_COMPACT_NOALLOC_MAX_ROWS rows (256 KB).  It lives in
// the library's own device image, so every device that loads the library
// holds it until the process exits, and every call on that device shares it.
static_assert(SDB_COMPACT_NOALLOC_MAX_ROWS % kCompactChunk == 0,
              "the no-allocation scratch holds one count per whole chunk of the largest segment");
static __device__ __align__(256) uint32_t g_noalloc_compact_scratch[SDB_COMPACT_NOALLOC_MAX_ROWS / kCompactChunk];
// what sdb_compact_scratch_bytes(SDB_COMPACT_NOALLOC_MAX_ROWS) asks for must fit the array
static_assert(((SDB_COMPACT_NOALLOC_MAX_ROWS / kCompactChunk) * sizeof(uint32_t) + 255) / 256 * 256 <=
                  sizeof(g_noalloc_compact_scratch),
              "no-allocation scratch smaller than the compaction needs at the row limit");

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_scratch_ptr[kNoAllocMaxDevices];  // device address of the array, per device (set up once)
}  // namespace

extern "C" {

int sdb_compact_row_ids_noalloc(const uint8_t *flags, uint64_t n, int32_t *ids, uint32_t *count, sdb_stream_t stream)
{
    if (n > SDB_COMPACT_NOALLOC_MAX_ROWS)
        return sdb_set_error(SDB_ERR_INVALID,
                             "sdb_compact_row_ids_noalloc: %llu rows exceed the fixed scratch (at most %llu rows per call)",
                             (unsigned long long)n, (unsigned long long)SDB_COMPACT_NOALLOC_MAX_ROWS);
    if (n == 0) return sdb_compact_row_ids(flags, 0, ids, count, nullptr, 0, stream);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sdb_set_error(SDB_ERR_CUDA, "sdb_compact_row_ids_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_row_ids_noalloc: device %d beyond the supported %d", dev,
                             kNoAllocMaxDevices);
    void *scratch = nullptr;
    {
        // Set-up, once per device, with that device current: the host-side
        // name of the array is not a device address, so ask the runtime for it.
        // The address is kept for the life of the process; a cudaDeviceReset
        // destroys the module that holds the array, so the entry must not be
        // called on a device after it was reset.
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_scratch_ptr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_compact_scratch);
            if (e != cudaSuccess || !p)
                return sdb_set_error(SDB_ERR_CUDA, "sdb_compact_row_ids_noalloc: cudaGetSymbolAddress: %s",
                                     cudaGetErrorString(e));
            g_noalloc_scratch_ptr[dev] = p;
        }
        scratch = g_noalloc_scratch_ptr[dev];
    }
    // Every count the passes read is written first by k_compact_count, so the
    // array needs no clearing between calls.
    return sdb_compact_row_ids(flags, n, ids, count, scratch, sizeof(g_noalloc_compact_scratch), stream);
}

static int compact_gather(const void *flags, bool occ, uint64_t n, int ncols, const void *const *src, const int *wide,
                          void *const *dst, uint32_t *count, sdb_stream_t stream)
{
    if (n > kSmallCompactMax) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_gather: n=%llu exceeds %u",
                                                   (unsigned long long)n, kSmallCompactMax);
    if (ncols < 0 || ncols > kSmallCompactCols || (ncols && (!src || !wide || !dst)))
        return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_gather: 0..%d columns", kSmallCompactCols);
    if (!count || (n && !flags)) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_gather: NULL flags or count");
    if (occ && !sdb::aligned(flags, 4)) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_gather_occ: occ misaligned");
    if (!sdb::aligned(count, 4)) return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_gather: count misaligned");
    SmallCompact a;
    a.flags = flags;
    a.n = (uint32_t)n;
    a.ncols = ncols;
    a.count = count;
    for (int c = 0; c < ncols; c++) {
        const size_t w = wide[c] ? 8 : 4;
        if (!src[c] || !dst[c] || !sdb::aligned(src[c], w) || !sdb::aligned(dst[c], w))
            return sdb_set_error(SDB_ERR_INVALID, "sdb_compact_gather: column %d NULL or misaligned", c);
        a.src[c] = src[c];
        a.dst[c] = dst[c];
        a.wide[c] = wide[c] ? 1 : 0;
    }
    if (occ)
        k_compact_gather_small<uint32_t><<<1, 1024, 0, (cudaStream_t)stream>>>(a);
    else
        k_compact_gather_small<uint8_t><<<1, 1024, 0, (cudaStream_t)stream>>>(a);
    return sdb_check_launch("sdb_compact_gather");
}

int sdb_compact_gather(const uint8_t *flags, uint64_t n, int ncols, const void *const *src, const int *wide,
                       void *const *dst, uint32_t *count, sdb_stream_t stream)
{
    return compact_gather(flags, false, n, ncols, src, wide, dst, count, stream);
}

int sdb_compact_gather_occ(const uint32_t *occ, uint64_t n, int ncols, const void *const *src, const int *wide,
                           void *const *dst, uint32_t *count, sdb_stream_t stream)
{
    return compact_gather(occ, true, n, ncols, src, wide, dst, count, stream);
}

int sdb_gather_i32(const int32_t *src, const int32_t *ids, const uint32_t *count, int32_t *dst, uint64_t cap,
                   sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({src, ids, count, dst}), "sdb_gather_i32");
    if (cap == 0) return SDB_OK;
    if (!src || !ids || !count || !dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_gather_i32: NULL buffer");
    const LaunchShape sh = op_shape(SDB_OPK_GATHER, cap, 8);
    k_gather<int32_t><<<grid_of(cap, sh), sh.block, 0, (cudaStream_t)stream>>>(src, ids, count, dst, cap);
    return sdb_check_launch("sdb_gather_i32");
}

int sdb_gather_u64(const uint64_t *src, const int32_t *ids, const uint32_t *count, uint64_t *dst, uint64_t cap,
                   sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({ids, count}) && nat8(src) && nat8(dst), "sdb_gather_u64");
    if (cap == 0) return SDB_OK;
    if (!src || !ids || !count || !dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_gather_u64: NULL buffer");
    const LaunchShape sh = op_shape(SDB_OPK_GATHER, cap, 8);
    k_gather<uint64_t><<<grid_of(cap, sh), sh.block, 0, (cudaStream_t)stream>>>(src, ids, count, dst, cap);
    return sdb_check_launch("sdb_gather_u64");
}

int32_t sdb_gen_uniform_host(uint64_t seed, uint64_t stream_id, uint64_t row, int32_t lo, int32_t hi)
{
    return sdb::uniform_from_key(sdb::stream_key(seed, stream_id), row, lo, hi);
}

int sdb_gen_uniform(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id, int32_t lo,
                    int32_t hi, sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({dst}), "sdb_gen_uniform");
    if (hi < lo) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_uniform: hi < lo");
    if (n == 0) return SDB_OK;
    if (!dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_uniform: NULL buffer");
    k_gen_uniform<<<sdb::grid_for(n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        dst, n, row0, sdb::stream_key(seed, stream_id), lo, hi);
    return sdb_check_launch("sdb_gen_uniform");
}

int sdb_gen_uniform_cpu(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id, int32_t lo,
                        int32_t hi)
{
    if (hi < lo) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_uniform_cpu: hi < lo");
    if (n && !dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_uniform_cpu: NULL buffer");
    const uint64_t key = sdb::stream_key(seed, stream_id);
    parallel_rows(n, [=](uint64_t i) { dst[i] = sdb::uniform_from_key(key, row0 + i, lo, hi); });
    return SDB_OK;
}

int sdb_gen_datekeys_cpu(int32_t *dst, uint64_t n, int64_t day0)
{
    if (n && !dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_datekeys_cpu: NULL buffer");
    for (uint64_t i = 0; i < n; i++) dst[i] = sdb::datekey_of_day(day0 + (int64_t)i);
    return SDB_OK;
}

int sdb_gen_dates(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id, int32_t ndays,
                  sdb_stream_t stream)
{
    SDB_REQUIRE_ALIGNED(nat4({dst}), "sdb_gen_dates");
    if (ndays < 1) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_dates: ndays < 1");
    if (n == 0) return SDB_OK;
    if (!dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_dates: NULL buffer");
    k_gen_dates<<<sdb::grid_for(n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        dst, n, row0, sdb::stream_key(seed, stream_id), ndays);
    return sdb_check_launch("sdb_gen_dates");
}

int sdb_gen_dates_cpu(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id, int32_t ndays)
{
    if (ndays < 1) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_dates_cpu: ndays < 1");
    if (n && !dst) return sdb_set_error(SDB_ERR_INVALID, "sdb_gen_dates_cpu: NULL buffer");
    const uint64_t key = sdb::stream_key(seed, stream_id);
    parallel_rows(n, [=](uint64_t i) { dst[i] = sdb::datekey_of_day(sdb::uniform_from_key(key, row0 + i, 0, ndays - 1)); });
    return SDB_OK;
}

}  // extern "C"

extern "C" {

int sdb_op_tune_set(int op_kernel, uint64_t rows, int block, int blocks_per_sm)
{
    if (op_kernel < 0 || op_kernel >= SDB_OPK_COUNT) return sdb_set_error(SDB_ERR_INVALID, "sdb_op_tune_set: bad kernel");
    int32_t e = 0;
    if (block != 0 || blocks_per_sm != 0) {
        if (block != 128 && block != 256 && block != 512)
            return sdb_set_error(SDB_ERR_INVALID, "sdb_op_tune_set: block must be 128, 256 or 512");
        if (blocks_per_sm < 1 || blocks_per_sm > 32 || blocks_per_sm * block > 2048)
            return sdb_set_error(SDB_ERR_INVALID, "sdb_op_tune_set: blocks_per_sm must be 1..32 and fit 2048 threads");
        e = (block << 8) | blocks_per_sm;
    }
    g_op_tune[op_kernel][op_bucket(rows)].store(e, std::memory_order_relaxed);
    return SDB_OK;
}

int sdb_op_tune_get(int op_kernel, uint64_t rows, int *block, int *blocks_per_sm)
{
    if (op_kernel < 0 || op_kernel >= SDB_OPK_COUNT || !block || !blocks_per_sm)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_op_tune_get: bad argument");
    const int def = (op_kernel == SDB_OPK_SUM || op_kernel == SDB_OPK_COUNT_FLAGS || op_kernel == SDB_OPK_MIN_MAX) ? 4 : 8;
    const LaunchShape sh = op_shape(op_kernel, rows, def);
    *block = sh.block;
    *blocks_per_sm = sh.per_sm;
    return SDB_OK;
}

}  // extern "C"
