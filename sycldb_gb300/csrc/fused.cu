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
#include <cstring>

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

enum Term { T_FLAGS = 0, T_SUM = 1, T_GROUP_SMEM = 2, T_GROUP_GLOBAL = 3 };

struct ChainLaunch {
    sdb_chain_desc d;
    int32_t dead_from;   // ops at index >= dead_from cannot revive a dead row
    int32_t vec;         // all column pointers 16-byte aligned, flags 4-byte aligned
    uint32_t mults[SDB_CHAIN_MAX_KEYS];
};

template <int NREGS>
struct Regs {
    int32_t v[NREGS][4];
};

template <int NREGS>
__device__ __forceinline__ void reg_get(const Regs<NREGS> &R, int idx, int32_t (&out)[4])
{
#pragma unroll
    for (int j = 0; j < 4; j++) out[j] = R.v[0][j];
#pragma unroll
    for (int r = 1; r < NREGS; r++)
        if (idx == r) {
#pragma unroll
            for (int j = 0; j < 4; j++) out[j] = R.v[r][j];
        }
}

template <int NREGS>
__device__ __forceinline__ void reg_set(Regs<NREGS> &R, int idx, const int32_t (&in)[4], uint32_t mask)
{
#pragma unroll
    for (int r = 0; r < NREGS; r++)
        if (idx == r) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (mask & (1u << j)) R.v[r][j] = in[j];
        }
}

// Loads operand `o` for the rows of `need` (other rows are left unspecified).
template <int NREGS>
__device__ __forceinline__ void fetch(const sdb_operand &o, uint64_t r0, uint32_t need, bool full, bool vec,
                                      const Regs<NREGS> &R, int32_t (&v)[4])
{
    if (o.kind == SDB_SRC_COL) {
        if (need == 0) return;
        if (full && vec) {
            int4 q = __ldcs(reinterpret_cast<const int4 *>(o.col + r0));
            v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (need & (1u << j)) v[j] = __ldcs(o.col + r0 + j);
        }
    } else if (o.kind == SDB_SRC_REG) {
        reg_get(R, o.reg, v);
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = o.lit;
    }
}

__device__ __forceinline__ void store_masked(int32_t *col, uint64_t r0, const int32_t (&v)[4], uint32_t mask)
{
#pragma unroll
    for (int j = 0; j < 4; j++)
        if (mask & (1u << j)) col[r0 + j] = v[j];
}

__device__ __forceinline__ uint32_t load_flags4(const uint8_t *f, uint64_t r0, uint32_t valid, bool full, bool vec)
{
    if (full && vec) {
        uint32_t w = __ldcs(reinterpret_cast<const unsigned int *>(f + r0));
        uint32_t x = __vcmpne4(w, 0u);
        return ((x >> 7) & 1u) | ((x >> 14) & 2u) | ((x >> 21) & 4u) | ((x >> 28) & 8u);
    }
    uint32_t m = 0;
#pragma unroll
    for (int j = 0; j < 4; j++)
        if ((valid >> j) & 1u) m |= (uint32_t)(f[r0 + j] != 0) << j;
    return m;
}

__device__ __forceinline__ void store_flags4(uint8_t *f, uint64_t r0, uint32_t live, uint32_t valid, bool full, bool vec)
{
    if (full && vec) {
        uint32_t w = (live & 1u) | ((live & 2u) << 7) | ((live & 4u) << 14) | ((live & 8u) << 21);
        *reinterpret_cast<unsigned int *>(f + r0) = w;
        return;
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
        if ((valid >> j) & 1u) f[r0 + j] = (uint8_t)((live >> j) & 1u);
}

// Evaluates the op list on one 4-row group.  Returns the live mask; the
// registers hold the values the ops produced for live rows.
template <int NREGS, class L>
__device__ __forceinline__ uint32_t run_ops(const L &Lc, uint64_t r0, uint32_t valid, bool full, Regs<NREGS> &R)
{
    const sdb_chain_desc &d = Lc.d;
    const bool vec = Lc.vec != 0;
    uint32_t live = d.flags_in ? load_flags4(d.flags_in, r0, valid, full, vec) : valid;

#pragma unroll 1
    for (int k = 0; k < d.n_ops; k++) {
        if (live == 0 && k >= Lc.dead_from) break;
        const sdb_chain_op &op = d.ops[k];
        int32_t a[4], b[4];
        switch (op.kind) {
        case SDB_OP_SELECT: {
            const uint32_t need = op.logic_op == SDB_AND ? live : valid;
            fetch(op.a, r0, need, full, vec, R, a);
            fetch(op.b, r0, need, full, vec, R, b);
            uint32_t m = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) m |= (uint32_t)sdb::compare(op.cmp_op, a[j], b[j]) << j;
            live = sdb::logical4(op.logic_op, live, m & need) & valid;
            break;
        }
        case SDB_OP_SEARCH_RANGE:
        case SDB_OP_SEARCH_POINTS: {
            const uint32_t need = op.logic_op == SDB_AND ? live : valid;
            fetch(op.a, r0, need, full, vec, R, a);
            uint32_t m = 0;
            if (op.kind == SDB_OP_SEARCH_RANGE) {
#pragma unroll
                for (int j = 0; j < 4; j++) m |= (uint32_t)(a[j] >= op.lo && a[j] <= op.hi) << j;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) m |= (uint32_t)(a[j] == op.lo || a[j] == op.hi) << j;
            }
            live = sdb::logical4(op.logic_op, live, m & need) & valid;
            break;
        }
        case SDB_OP_SEMI_PROBE: {
            fetch(op.a, r0, live, full, vec, R, a);
            const uint8_t *ht = static_cast<const uint8_t *>(op.ht);
            uint32_t m = 0;
#pragma unroll
            for (int j = 0; j < 4; j++)
                if ((live >> j) & 1u) {
                    const int32_t key = a[j];
                    if (key >= op.lo && key <= op.hi && __ldg(ht + ((uint32_t)key - (uint32_t)op.lo)) != 0)
                        m |= 1u << j;
                }
            live = m;
            break;
        }
        case SDB_OP_FULL_PROBE: {
            fetch(op.a, r0, live, full, vec, R, a);
            const int2 *ht = static_cast<const int2 *>(op.ht);
            uint32_t m = 0;
            int32_t val[4] = {0, 0, 0, 0};
#pragma unroll
            for (int j = 0; j < 4; j++)
                if ((live >> j) & 1u) {
                    const int32_t key = a[j];
                    if (key >= op.lo && key <= op.hi) {
                        const int2 e = __ldg(ht + ((uint32_t)key - (uint32_t)op.lo));
                        if (e.x == 1) {
                            m |= 1u << j;
                            val[j] = e.y;
                        }
                    }
                }
            live = m;
            reg_set(R, op.out_reg, val, m);
            if (op.out_col && m) store_masked(op.out_col, r0, val, m);
            break;
        }
        case SDB_OP_BINOP: {
            fetch(op.a, r0, live, full, vec, R, a);
            fetch(op.b, r0, live, full, vec, R, b);
            int32_t c[4];
#pragma unroll
            for (int j = 0; j < 4; j++) c[j] = sdb::binop(a[j], b[j], op.bin_op);
            reg_set(R, op.out_reg, c, live);
            if (op.out_col && live) store_masked(op.out_col, r0, c, live);
            break;
        }
        case SDB_OP_FILL: {
            int32_t c[4] = {op.a.lit, op.a.lit, op.a.lit, op.a.lit};
            reg_set(R, op.out_reg, c, valid);
            if (op.out_col) store_masked(op.out_col, r0, c, valid);
            break;
        }
        default:
            break;
        }
    }
    return live;
}

template <int TERM, int NREGS>
__global__ void __launch_bounds__(kThreads) k_chain(const __grid_constant__ ChainLaunch L)
{
    const sdb_chain_desc &d = L.d;
    extern __shared__ uint64_t s_sum[];
    uint32_t *s_occ = reinterpret_cast<uint32_t *>(s_sum + (TERM == T_GROUP_SMEM ? d.P : 0));
    if (TERM == T_GROUP_SMEM) {
        for (uint64_t i = threadIdx.x; i < d.P; i += blockDim.x) { s_sum[i] = 0; s_occ[i] = 0; }
        __syncthreads();
    }

    const uint64_t groups = (d.n + 3) >> 2;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t acc = 0;
    Regs<NREGS> R;
#pragma unroll
    for (int r = 0; r < NREGS; r++)
#pragma unroll
        for (int j = 0; j < 4; j++) R.v[r][j] = 0;

    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += stride) {
        const uint64_t r0 = g << 2;
        const uint64_t left = d.n - r0;
        const bool full = left >= 4;
        const uint32_t valid = full ? 0xFu : ((1u << left) - 1u);
        uint32_t live = run_ops<NREGS>(L, r0, valid, full, R);

        if (TERM == T_FLAGS || d.flags_out) store_flags4(d.flags_out, r0, live, valid, full, L.vec != 0);
        if (live == 0) continue;

        if (TERM == T_SUM) {
            int32_t v[4];
            fetch(d.value, r0, live, full, L.vec != 0, R, v);
#pragma unroll
            for (int j = 0; j < 4; j++)
                if ((live >> j) & 1u) acc += sdb::widen(v[j]);
        } else if (TERM == T_GROUP_SMEM || TERM == T_GROUP_GLOBAL) {
            int32_t v[4];
            int32_t key[SDB_CHAIN_MAX_KEYS][4];
            fetch(d.value, r0, live, full, L.vec != 0, R, v);
            uint32_t h[4] = {0, 0, 0, 0};
#pragma unroll
            for (int kk = 0; kk < SDB_CHAIN_MAX_KEYS; kk++) {
                if (kk >= d.n_keys) break;
                fetch(d.keys[kk], r0, live, full, L.vec != 0, R, key[kk]);
#pragma unroll
                for (int j = 0; j < 4; j++)
                    h[j] += ((uint32_t)key[kk][j] - (uint32_t)d.key_min[kk]) * L.mults[kk];
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (!((live >> j) & 1u)) continue;
                const int64_t s = sdb::group_slot(h[j], d.P);
                if (s < 0 || (uint64_t)s >= d.P) { atomicAdd(&g_errors, 1ull); continue; }
                bool first;
                if (TERM == T_GROUP_SMEM) {
                    first = atomicExch(&s_occ[s], 1u) == 0u;
                    if (first) first = atomicExch(&d.occ[s], 1u) == 0u;
                    atomicAdd(reinterpret_cast<unsigned long long *>(&s_sum[s]), (unsigned long long)sdb::widen(v[j]));
                } else {
                    first = d.occ[s] == 0u && atomicExch(&d.occ[s], 1u) == 0u;
                    atomicAdd(reinterpret_cast<unsigned long long *>(&d.out_sum[s]), (unsigned long long)sdb::widen(v[j]));
                }
                if (first) {
#pragma unroll
                    for (int kk = 0; kk < SDB_CHAIN_MAX_KEYS; kk++)
                        if (kk < d.n_keys) d.out_keys[kk][s] = key[kk][j];
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
    } else if (TERM == T_GROUP_SMEM) {
        __syncthreads();
        for (uint64_t i = threadIdx.x; i < d.P; i += blockDim.x)
            if (s_occ[i]) atomicAdd(reinterpret_cast<unsigned long long *>(&d.out_sum[i]), (unsigned long long)s_sum[i]);
    }
}

constexpr uint64_t kSmemSlotsMax = 16384;  // 16 K slots x 12 B = 192 KB of shared memory

int num_sms()
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = sdb::kSMs;
    }
    return sms;
}

template <int TERM, int NREGS>
int launch_term(const ChainLaunch &L, cudaStream_t s)
{
    auto kern = k_chain<TERM, NREGS>;
    size_t smem = 0;
    if (TERM == T_GROUP_SMEM) {
        smem = (size_t)L.d.P * (sizeof(uint64_t) + sizeof(uint32_t));
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSmemSlotsMax * 12));
            attr = true;
        }
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    const uint64_t groups = (L.d.n + 3) / 4;
    uint64_t blocks = (groups + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)num_sms() * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(L);
    return sdb_check_launch("sdb_fused_chain");
}

template <int TERM>
int launch_regs(const ChainLaunch &L, int nregs, cudaStream_t s)
{
    if (nregs <= 2) return launch_term<TERM, 2>(L, s);
    if (nregs <= 4) return launch_term<TERM, 4>(L, s);
    return launch_term<TERM, 8>(L, s);
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
        *term_out = c->P <= kSmemSlotsMax ? T_GROUP_SMEM : T_GROUP_GLOBAL;
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

extern "C" int sdb_fused_chain(const sdb_chain_desc *chain, sdb_stream_t stream)
{
    ChainLaunch L;
    int nregs = 1, term = 0;
    int st = sdb_chain_prepare(chain, &L, sizeof L, &nregs, &term);
    if (st != SDB_OK) return st;
    if (L.d.n == 0) return SDB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    switch (term) {
    case T_FLAGS: return launch_regs<T_FLAGS>(L, nregs, s);
    case T_SUM: return launch_regs<T_SUM>(L, nregs, s);
    case T_GROUP_SMEM: return launch_regs<T_GROUP_SMEM>(L, nregs, s);
    default: return launch_regs<T_GROUP_GLOBAL>(L, nregs, s);
    }
}
