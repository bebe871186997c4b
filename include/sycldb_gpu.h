/*
 * sycldb_gpu.h -- C ABI of the GB300 (sm_103a) operator library.
 *
 * This is the drop-in boundary for the SYCLDB physical-operator path.  In the
 * reference the boundary is a C++ class interface: Segment::*_operator
 * factories build KernelDefinition objects (models/models.hpp:604-986), and
 * KernelData::execute switches on KernelType and submits one SYCL
 * parallel_for per kernel (models/execution.hpp:30-46, 260-497).  Each
 * sdb_* kernel entry below replaces one arm of that switch, or one of the
 * inline kernels that TransientTable submits itself; the comment on each
 * entry names the reference code it replaces.
 *
 * Conventions (all entries):
 *   - Every pointer argument is a device pointer unless stated otherwise.
 *     The caller owns every buffer; no kernel entry allocates.  Hash tables
 *     and group-by slot arrays must arrive zeroed, as the reference's
 *     memory_manager::alloc_zero regions do.
 *   - Work is enqueued on `stream` and returns without waiting (the reference
 *     waits after every KernelBundle, models/execution.hpp:628; results are
 *     the same).  A NULL stream is the legacy default stream.
 *   - Return value: SDB_OK (0) or a negative sdb_status.  sdb_last_error()
 *     gives the message of the last failure on the calling thread.
 *   - Enum values are the reference's: comp_op and logical_op
 *     (kernels/selection.hpp:7-21), BinaryOp (kernels/aggregation.hpp:11-17).
 *   - Integer semantics are the reference's: int32 columns, uint8 (bool)
 *     flags, uint64 sums of sign-extended int32 values, int32 arithmetic that
 *     wraps.  Division by zero yields 0 and INT_MIN / -1 yields INT_MIN (both
 *     undefined in the reference).
 *   - Out-of-range hash-table or group-by slots (which the reference would
 *     write out of bounds) are skipped and counted in a device error word;
 *     sdb_device_errors() reads and clears it.
 */
#ifndef SYCLDB_GPU_H
#define SYCLDB_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t / CUstream. */
typedef struct CUstream_st *sdb_stream_t;

typedef enum sdb_status {
    SDB_OK = 0,
    SDB_ERR_INVALID = -1,     /* bad argument (the reference throws std::invalid_argument / runtime_error) */
    SDB_ERR_CUDA = -2,        /* CUDA launch or API failure */
    SDB_ERR_NOMEM = -3,       /* allocator budget exceeded (the reference throws std::bad_alloc) */
    SDB_ERR_TIMEOUT = -4,     /* a bounded device or host wait ran out */
    SDB_ERR_UNSUPPORTED = -5, /* plan shape the executor does not handle */
    SDB_ERR_DEVICE = -6       /* device-side check failed (see sdb_device_errors) */
} sdb_status;

typedef enum sdb_comp_op { SDB_EQ = 0, SDB_NE = 1, SDB_LT = 2, SDB_LE = 3, SDB_GT = 4, SDB_GE = 5 } sdb_comp_op;
typedef enum sdb_logical_op { SDB_NONE = 0, SDB_AND = 1, SDB_OR = 2 } sdb_logical_op;
typedef enum sdb_binary_op { SDB_MUL = 0, SDB_DIV = 1, SDB_ADD = 2, SDB_SUB = 3 } sdb_binary_op;

/* ---------------------------------------------------------------- library */

/* Message of the last failed call on this thread ("" if none). */
const char *sdb_last_error(void);
/* Library version string. */
const char *sdb_version(void);
/* sizeof of an ABI struct by name ("sdb_operand", "sdb_chain_op",
 * "sdb_chain_desc", "sdb_engine_config"), 0 if unknown: lets bindings check
 * their layouts. */
size_t sdb_abi_sizeof(const char *type_name);
/* Number of kernels this library has launched in this process (host-side
 * counter; cudaMemset/cudaMemcpy calls are not counted). */
uint64_t sdb_launch_count(void);
/* Reads and clears the device-side error counter (out-of-range slots skipped
 * by the build and group-by kernels).  Synchronises `stream`. */
int sdb_device_errors(uint64_t *count, sdb_stream_t stream);

/* ------------------------------------------------- operator kernels (K1-K16) */

/* K1: flags[i] = v.  Replaces queue.fill<bool> of the flag buffers
 * (models/transient_table.hpp:86,105). */
int sdb_fill_u8(uint8_t *flags, uint64_t n, uint8_t v, sdb_stream_t stream);

/* K2: out[i] = logical(logic_op, in[i], compare(cmp_op, col[i], v)).
 * Replaces SelectionKernelLiteral (kernels/selection.hpp:157-186),
 * KernelData::execute arm at models/execution.hpp:305-321.
 * in and out may alias. */
int sdb_select_lit(const int32_t *col, int32_t v, int cmp_op, int logic_op,
                   const uint8_t *in, uint8_t *out, uint64_t n, sdb_stream_t stream);

/* K3: out[i] = logical(logic_op, in[i], compare(cmp_op, a[i], b[i])).
 * Replaces SelectionKernelColumns (kernels/selection.hpp:127-155). */
int sdb_select_cols(const int32_t *a, const int32_t *b, int cmp_op, int logic_op,
                    const uint8_t *in, uint8_t *out, uint64_t n, sdb_stream_t stream);

/* K4: out[i] = logical(logic_op, in[i], local[i]).
 * Replaces LogicalKernel (kernels/selection.hpp:106-125), the last step of
 * Segment::search_operator (models/models.hpp:704-715). */
int sdb_logical(int logic_op, const uint8_t *in, const uint8_t *local, uint8_t *out,
                uint64_t n, sdb_stream_t stream);

/* K5: dst[i] = v.  Replaces FillKernel (kernels/projection.hpp:7-21). */
int sdb_fill_i32(int32_t *dst, int32_t v, uint64_t n, sdb_stream_t stream);

/* K6: if (flags[i]) res[i] = a op b; other rows are left untouched.
 * Replaces PerformOperationKernelColumns / LiteralFirst / LiteralSecond
 * (kernels/aggregation.hpp:50-72, 102-125, 155-178). */
int sdb_binop_cc(int32_t *res, const int32_t *a, const int32_t *b, int bin_op,
                 const uint8_t *flags, uint64_t n, sdb_stream_t stream);
int sdb_binop_lc(int32_t *res, int32_t a, const int32_t *b, int bin_op,
                 const uint8_t *flags, uint64_t n, sdb_stream_t stream);
int sdb_binop_cl(int32_t *res, const int32_t *a, int32_t b, int bin_op,
                 const uint8_t *flags, uint64_t n, sdb_stream_t stream);

/* K7: *acc += sum over rows of (uint64)(int64)(flags[i] ? col[i] : 0).
 * Accumulates (does not overwrite), like the sycl::reduction without
 * initialize_to_identity of AggregateOperationKernel
 * (kernels/aggregation.hpp:208-228; models/execution.hpp:458-476). */
int sdb_sum_i32_u64(const int32_t *col, const uint8_t *flags, uint64_t n, uint64_t *acc,
                    sdb_stream_t stream);

/* K8: dense group-by SUM.  For each flagged row, slot
 *   h = (int)((uint64)(int)(sum_j (keys[j][i]-mins[j]) * prod_{l<j}(maxs[l]-mins[l]+1)) % P)
 * (int arithmetic that wraps); the first row to claim occ[h] writes its key
 * values to out_keys[j][h]; out_sum[h] += (uint64)(int64)val[i].
 * Replaces GroupByAggregateKernel (kernels/aggregation.hpp:278-344).
 * keys/out_keys are HOST arrays of g device pointers; mins/maxs are HOST
 * arrays of g ints; 1 <= g <= 8.  occ and out_sum must arrive zeroed. */
int sdb_groupby_sum(const int32_t *const *keys, const int32_t *mins, const int32_t *maxs, int g,
                    const int32_t *val, const uint8_t *flags, uint64_t n, uint64_t P,
                    int32_t *const *out_keys, uint64_t *out_sum, uint32_t *occ, sdb_stream_t stream);

/* K9: flags[s] = occ[s] != 0.  Replaces the group-by final-flags kernel
 * (models/transient_table.hpp:1544-1558). */
int sdb_occ_to_flags(const uint32_t *occ, uint8_t *flags, uint64_t P, sdb_stream_t stream);

/* K10: ht[key[i]-min] = flags[i] (bool, false written too).
 * Replaces BuildKeysHTKernel (kernels/join.hpp:17-33). */
int sdb_ht_build_keys(const int32_t *key, const uint8_t *flags, uint64_t n,
                      uint8_t *ht, int32_t min, int32_t len, sdb_stream_t stream);

/* K11: out[i] = in[i] && min <= key[i] <= max && ht[key[i]-min].
 * Replaces FilterJoinKernel (kernels/join.hpp:129-173). */
int sdb_probe_semi(const int32_t *key, const uint8_t *in, uint8_t *out, uint64_t n,
                   const uint8_t *ht, int32_t min, int32_t max, sdb_stream_t stream);

/* K12: interleaved {occ, val} table: ht2[2h] = flags[i]; if flags[i]
 * ht2[2h+1] = val[i], h = key[i]-min.
 * Replaces BuildKeyValsHTKernel (kernels/join.hpp:60-93). */
int sdb_ht_build_kv(const int32_t *key, const int32_t *val, const uint8_t *flags, uint64_t n,
                    int32_t *ht2, int32_t min, int32_t len, sdb_stream_t stream);

/* K13: if in[i] && min <= key[i] <= max && ht2[2h] == 1:
 * val_out[i] = ht2[2h+1], out[i] = 1; else out[i] = 0.
 * Replaces FullJoinKernel (kernels/join.hpp:256-312). */
int sdb_probe_full(const int32_t *key, int32_t *val_out, const uint8_t *in, uint8_t *out,
                   uint64_t n, const int32_t *ht2, int32_t min, int32_t max, sdb_stream_t stream);

/* K10-K13 on open-addressing tables, for join keys whose range [min, max] is
 * much wider than the build side's rows (the engine's choice; the reference
 * sizes its direct-address table by the range, models/models.hpp:1413-1452,
 * 1509-1548, which a sparse key range makes as large as the range).  The
 * table has 2^log2_slots slots (sdb_oa_log2_slots: at least twice the build
 * rows) and must be all zero before its first build.  A slot is a 32-bit
 * word tag << 1 | flag, tag = key - min + 1 (0 = empty), claimed with
 * atomicCAS and probed linearly; the key/value table pairs it with the value
 * (int32 pairs {word, value}, 8-byte aligned).  Builds write what K10/K12
 * write -- a live row its key's hit (and value), a dead row a miss; `fresh`
 * (the table is all zero and no other build writes it meanwhile) skips dead
 * rows, as ht_zeroed does for the fused build.  Probes give exactly the hits
 * and values of K11/K13 on the direct table.  The key range must hold fewer
 * than 2^31 keys; keys outside it miss (probe) or are counted as errors and
 * skipped (build). */
int sdb_oa_log2_slots(uint64_t build_rows); /* smallest lg >= 4 with 2^lg >= 2 rows; rows <= 2^30 */
int sdb_ht_build_keys_oa(const int32_t *key, const uint8_t *flags, uint64_t n, uint32_t *ht, int log2_slots,
                         int32_t min, int32_t max, int fresh, sdb_stream_t stream);
int sdb_probe_semi_oa(const int32_t *key, const uint8_t *in, uint8_t *out, uint64_t n, const uint32_t *ht,
                      int log2_slots, int32_t min, int32_t max, sdb_stream_t stream);
int sdb_ht_build_kv_oa(const int32_t *key, const int32_t *val, const uint8_t *flags, uint64_t n, int32_t *ht2,
                       int log2_slots, int32_t min, int32_t max, int fresh, sdb_stream_t stream);
int sdb_probe_full_oa(const int32_t *key, int32_t *val_out, const uint8_t *in, uint8_t *out, uint64_t n,
                      const int32_t *ht2, int log2_slots, int32_t min, int32_t max, sdb_stream_t stream);

/* K14: ids[0..count) = indices of set flags, in increasing order; *count
 * (device word) = how many.  Replaces build_row_ids
 * (models/transient_table.hpp:535-599), whose atomic append gives the same
 * set in an unspecified order.  `scratch` is device memory of at least
 * sdb_compact_scratch_bytes(n) bytes. */
size_t sdb_compact_scratch_bytes(uint64_t n);
int sdb_compact_row_ids(const uint8_t *flags, uint64_t n, int32_t *ids, uint32_t *count,
                        void *scratch, size_t scratch_bytes, sdb_stream_t stream);

/* K14 without any allocation -- no counterpart in the reference.
 * Some callers cannot allocate device memory for scratch: executors whose
 * device memory all belongs to a pool they manage themselves (as the
 * reference's memory_manager reserves every byte up front), serving loops that
 * must not call cudaMalloc/cudaFree because those calls can synchronise the
 * whole device, or callers already at their memory budget.  This entry takes
 * the same arguments as sdb_compact_row_ids minus the scratch and returns the
 * same ids and count; its scratch is a fixed 256 KB array inside the library
 * (resident on every device that loads the library until the process
 * exits), so n is limited to SDB_COMPACT_NOALLOC_MAX_ROWS (one 2^28-row
 * segment); larger n is refused with SDB_ERR_INVALID.  The first call on a
 * device looks up that array's device address (a one-time set-up per device,
 * done with the device current); make that first call before any stream
 * capture.  The address is kept for the rest of the process: a device reset
 * (cudaDeviceReset) after the first call is not supported, since it rebuilds
 * the context and the array may move.  All calls on a device share the
 * array, so calls that overlap on the GPU (different streams, no ordering
 * between them) race and must not be issued.  It calls no allocator. */
#define SDB_COMPACT_NOALLOC_MAX_ROWS 268435456ull
int sdb_compact_row_ids_noalloc(const uint8_t *flags, uint64_t n, int32_t *ids, uint32_t *count,
                                sdb_stream_t stream);

/* K15: dst[i] = src[ids[i]] for i < *count (count is a device word, cap
 * bounds it).  Replaces the gather of Segment::compress_sync
 * (models/models.hpp:1019-1063). */
int sdb_gather_i32(const int32_t *src, const int32_t *ids, const uint32_t *count,
                   int32_t *dst, uint64_t cap, sdb_stream_t stream);
int sdb_gather_u64(const uint64_t *src, const int32_t *ids, const uint32_t *count,
                   uint64_t *dst, uint64_t cap, sdb_stream_t stream);

/* K16: *out = number of set flags (overwrites).  Replaces
 * count_true_flags (kernels/common.hpp:30-110). */
int sdb_count_flags(const uint8_t *flags, uint64_t n, uint64_t *out, sdb_stream_t stream);

/* Segment statistics computed at load: minmax[0] = min, minmax[1] = max of
 * col[0..n) (n >= 1).  Replaces the host scan of the Segment constructor
 * (models/models.hpp:71-77). */
int sdb_min_max_i32(const int32_t *col, uint64_t n, int32_t *minmax, sdb_stream_t stream);

/* The flagged rows of a small segment (n <= 65536, e.g. a group-by result)
 * gathered from up to 8 columns in row order, in one launch: what
 * sdb_compact_row_ids and one sdb_gather_* per column give together
 * (dst[c][0..*count) = src[c][rows with flags != 0]).  src/dst/wide are HOST
 * arrays of ncols entries; wide[c] = 1 for a uint64 column, 0 for int32. */
int sdb_compact_gather(const uint8_t *flags, uint64_t n, int ncols, const void *const *src, const int *wide,
                       void *const *dst, uint32_t *count, sdb_stream_t stream);
/* Same, the flag of row i being occ[i] != 0: a group-by result compacted
 * straight from its occupancy words (K8's occ), what sdb_occ_to_flags (K9)
 * followed by sdb_compact_gather gives (transient_table.hpp:1544-1558). */
int sdb_compact_gather_occ(const uint32_t *occ, uint64_t n, int ncols, const void *const *src, const int *wide,
                           void *const *dst, uint32_t *count, sdb_stream_t stream);

/* ORDER BY: perm[0..n) = the row ids 0..n-1 ordered by keys[0], then keys[1],
 * ... (nkeys <= 16; key_types[k] 0 = int32 compared signed, 1 = uint64
 * compared unsigned, the comparisons of the reference's sort_table,
 * kernels/sort.hpp:7-103; descending[k] != 0 reverses key k).  Stable: equal
 * rows keep their order.  n <= 2^31.  A radix sort: 4 passes per int32 key,
 * 8 per uint64 key.  scratch: sdb_sort_scratch_bytes(n) bytes, 256-byte aligned.
 * The reference's executor itself treats SORT as a pass-through
 * (executor/ddor_executor.cpp:209-211). */
size_t sdb_sort_scratch_bytes(uint64_t n);
int sdb_sort_rows(const void *const *keys, const int *key_types, const int *descending, int nkeys, uint64_t n,
                  uint32_t *perm, void *scratch, size_t scratch_bytes, sdb_stream_t stream);

/* ------------------------------------------------------ fused operator chain */

/* One pass over a segment that applies a KernelBundle's kernels in order with
 * the row's flag held in a register.  It computes what the composed K2-K13 +
 * K7/K8 launches compute (the reference's disabled call-sequence fusion,
 * models/execution.hpp:546-615, had the same intent). */
#define SDB_CHAIN_MAX_OPS 16
#define SDB_CHAIN_MAX_REGS 8
#define SDB_CHAIN_MAX_KEYS 4

typedef enum sdb_operand_kind { SDB_SRC_COL = 0, SDB_SRC_REG = 1, SDB_SRC_LIT = 2 } sdb_operand_kind;

typedef struct sdb_operand {
    int32_t kind;        /* sdb_operand_kind */
    int32_t reg;         /* SDB_SRC_REG: register index */
    int32_t lit;         /* SDB_SRC_LIT: value */
    int32_t pad;
    const int32_t *col;  /* SDB_SRC_COL: column (device) */
} sdb_operand;

typedef enum sdb_chain_op_kind {
    SDB_OP_SELECT = 0,        /* flag = logical(logic_op, flag, compare(cmp_op, a, b)) */
    SDB_OP_SEARCH_RANGE = 1,  /* flag = logical(logic_op, flag, lo <= a && a <= hi) */
    SDB_OP_SEARCH_POINTS = 2, /* flag = logical(logic_op, flag, a == lo || a == hi) */
    SDB_OP_SEMI_PROBE = 3,    /* flag = flag && lo <= a <= hi && ht8[a-lo] */
    SDB_OP_FULL_PROBE = 4,    /* flag = flag && lo <= a <= hi && ht2[2(a-lo)] == 1; reg[out_reg] = ht2[2(a-lo)+1] */
    SDB_OP_BINOP = 5,         /* if flag: reg[out_reg] = a bin_op b */
    SDB_OP_FILL = 6           /* reg[out_reg] = a (a literal), every row */
} sdb_chain_op_kind;

typedef struct sdb_chain_op {
    int32_t kind;        /* sdb_chain_op_kind */
    int32_t cmp_op;
    int32_t logic_op;
    int32_t bin_op;
    sdb_operand a;
    sdb_operand b;
    int32_t lo, hi;      /* SEARCH bounds or probe min/max */
    int32_t out_reg;     /* FULL_PROBE / BINOP / FILL */
    int32_t ht_log2;     /* SEMI / FULL: 0 = direct-address table (below); n > 0 = open-addressing
                            table of 2^n slots (layout of sdb_probe_semi_oa / sdb_probe_full_oa) */
    const void *ht;      /* SEMI: uint8[hi-lo+1]; FULL: int32[2*(hi-lo+1)] */
    int32_t *out_col;    /* FULL_PROBE / BINOP / FILL: if non-NULL the register
                            is also stored where the composed kernel stores it */
} sdb_chain_op;

typedef enum sdb_chain_terminal {
    SDB_TERM_FLAGS = 0,   /* write the final flags to flags_out */
    SDB_TERM_SUM = 1,     /* *sum_out += sum of value over surviving rows (K7) */
    SDB_TERM_GROUPBY = 2, /* dense group-by SUM into out_keys/out_sum/occ (K8) */
    /* Hash-table builds (Column::build_keys_hash_table / build_key_vals_hash_table,
     * models/models.hpp:1413-1452, 1509-1548): every row of the segment writes
     * its slot (build_key - ht_min) % ht_len of ht_out, live rows a hit and
     * dead rows a miss, as K10/K12 (kernels/join.hpp:17-33, 60-93) do with
     * the final flags. */
    SDB_TERM_BUILD_KEYS = 3, /* uint8 ht_out[slot] = flag */
    SDB_TERM_BUILD_KV = 4    /* flag: int32 ht_out[2 slot] = 1, [2 slot + 1] = build_val; else [2 slot] = 0 */
} sdb_chain_terminal;

typedef struct sdb_chain_desc {
    uint64_t n;                 /* rows of this segment */
    const uint8_t *flags_in;    /* NULL: every row starts with flag = true */
    uint8_t *flags_out;         /* final flags (required for SDB_TERM_FLAGS, optional otherwise) */
    int32_t n_ops;
    int32_t terminal;           /* sdb_chain_terminal */
    sdb_chain_op ops[SDB_CHAIN_MAX_OPS];
    sdb_operand value;          /* SUM / GROUPBY value */
    uint64_t *sum_out;          /* SUM: accumulated */
    int32_t n_keys;             /* GROUPBY */
    int32_t pad;
    sdb_operand keys[SDB_CHAIN_MAX_KEYS];
    int32_t key_min[SDB_CHAIN_MAX_KEYS];
    int32_t key_max[SDB_CHAIN_MAX_KEYS];
    uint64_t P;
    int32_t *out_keys[SDB_CHAIN_MAX_KEYS];
    uint64_t *out_sum;
    uint32_t *occ;
    sdb_operand build_key;      /* BUILD_KEYS / BUILD_KV: the key of every row */
    sdb_operand build_val;      /* BUILD_KV: the value of live rows */
    void *ht_out;               /* BUILD: uint8[ht_len] (KEYS) or int32[2 ht_len] (KV) */
    int32_t ht_min, ht_len;
    int32_t ht_zeroed;          /* BUILD: 1 = ht_out is all zero before the chain runs and no other
                                   build writes it meanwhile: a dead row's miss (a zero written over a
                                   zero) is skipped, so dead rows cost no key load and no store.  With
                                   duplicate keys the table is the one the reference's unordered
                                   writes give when dead rows write first. */
    int32_t ht_log2;            /* BUILD: 0 = direct-address table (ht_len entries from ht_min);
                                   n > 0 = open-addressing table of 2^n slots over the keys
                                   ht_min .. ht_min + ht_len - 1 (sdb_ht_build_keys_oa layout) */
} sdb_chain_desc;

/* Launch one fused pass.  The descriptor is read on the host (copied into
 * the launch); its pointers are device pointers.  The kernel variant comes
 * from the tuning table (below), else a default. */
int sdb_fused_chain(const sdb_chain_desc *chain, sdb_stream_t stream);
/* Same, forcing a kernel variant.  0, 1, 2: the general pass with 4, 8 or
 * 16 rows per thread (chains needing more than 2 registers cap it: 4
 * registers at 8 rows, 8 at 4); each row loads a column only while its flag
 * can still change, so later columns cost only the sectors that hold live
 * rows.  3: a shape-specialised pass (straight-line code for the common
 * chain shapes; every chain column of the next tiles is staged in shared
 * memory by asynchronous copies while the current tile is probed).  4: as 3,
 * and after the first op each warp compacts its surviving rows so that the
 * remaining ops run one row per lane.  5: as 4 with a 2-stage copy ring (less
 * shared memory, more resident blocks).  6: as 5, and a warp's surviving rows
 * that do not fill a last group of 32 are carried (their column values) into
 * the next tile, so the one-row-per-lane ops run on full warps (chains whose
 * later ops write no column).  7: as 6, and the rows that survive the first
 * op after the compaction are compacted again, across lanes in registers,
 * so the later ops and the terminal run on full warps.  8: as 7, and the
 * columns that only the ops after that second compaction read are not
 * staged: a surviving row carries its row number and loads them there
 * (only the sectors holding such rows are read; chains under 2^31 rows,
 * else as 7).  Shapes without a
 * specialised pass fall back to the general pass.  Default (and an unset
 * tuning entry): 5. */
int sdb_fused_chain_variant(const sdb_chain_desc *chain, int variant, sdb_stream_t stream);
/* Tuning table used by sdb_fused_chain: variant for chains with this
 * terminal (sdb_chain_terminal), register count and row count (bucketed by
 * log2).  variant -1 restores the default.  _get returns the variant used. */
int sdb_chain_tune_set(int terminal, int nregs, uint64_t rows, int variant);
int sdb_chain_tune_get(int terminal, int nregs, uint64_t rows);
/* The same per kind of the chain's first op (SDB_OP_*, 7 = a chain without
 * ops), which tells shapes of one terminal apart; first_op -1 in _set_op sets
 * every kind (what sdb_chain_tune_set does). */
int sdb_chain_tune_set_op(int terminal, int nregs, int first_op, uint64_t rows, int variant);
int sdb_chain_tune_get_op(int terminal, int nregs, int first_op, uint64_t rows);
/* Launch shapes of the operator-at-a-time kernels (K1-K16): threads per
 * block (128, 256 or 512) and resident blocks per SM the grid-stride grid is
 * sized for, per kernel and row count (bucketed by log2).  No counterpart in
 * the reference (its parallel_for ranges leave the work-group size to the
 * SYCL runtime).  block = blocks_per_sm = 0 restores the default (256
 * threads; 8 blocks per SM, 4 for the reductions K7, K16 and min/max). */
typedef enum sdb_op_kernel {
    SDB_OPK_FILL_U8 = 0, SDB_OPK_SELECT_LIT, SDB_OPK_SELECT_COLS, SDB_OPK_LOGICAL, SDB_OPK_FILL_I32, SDB_OPK_BINOP,
    SDB_OPK_SUM, SDB_OPK_COUNT_FLAGS, SDB_OPK_MIN_MAX, SDB_OPK_OCC_TO_FLAGS, SDB_OPK_BUILD_KEYS, SDB_OPK_PROBE_SEMI,
    SDB_OPK_BUILD_KV, SDB_OPK_PROBE_FULL, SDB_OPK_GATHER, SDB_OPK_COUNT
} sdb_op_kernel;
int sdb_op_tune_set(int op_kernel, uint64_t rows, int block, int blocks_per_sm);
int sdb_op_tune_get(int op_kernel, uint64_t rows, int *block, int *blocks_per_sm);

/* Launches of the shape-specialised passes since the library loaded
 * (single-chain and batched), and how many of them ran a bound pass: a hot
 * shape (star join, date join, filter-project-sum) under variant 8 whose
 * operands sit where the shape's canonical binding puts them, so the pass
 * reads every operand at a place fixed at compile time.  Host counters;
 * either pointer may be NULL. */
int sdb_fused_launch_counts(uint64_t *specialised, uint64_t *bound);
/* Registers (1..8) a chain needs, or a negative status if it is invalid. */
int sdb_chain_registers(const sdb_chain_desc *chain);
/* 2 when the chain has a shape-specialised instantiation (variants 3-8) and
 * variant 8 runs it in a bound pass (see sdb_fused_launch_counts), 1 when it
 * has one but no bound pass, 0 when only the general pass runs it, or a
 * negative status if it is invalid.  Host-only. */
int sdb_chain_specialised(const sdb_chain_desc *chain);

/* ------------------------------------------------------------ paired pass
 * The shared scan of a batch: two aggregating chains that scan the same fact
 * rows in one pass.  No counterpart in the reference, which runs each
 * query's kernels on their own (models/execution.hpp:528-650,
 * executor/ddor_executor.cpp:22-245); the results are those of calling
 * sdb_fused_chain on each chain.  Two chains pair when the single-chain pass
 * would run both as the same bound variant-8 instantiation of a served shape
 * (star join, date join, filter-project-sum), with the same staged columns
 * (the columns the pass copies into shared memory) over the same rows and no
 * incoming or outgoing flags; their literals, tables, late columns and
 * outputs are their own.  Each tile is then copied once and both chains run
 * on it, each with its own group table and semi-join bitmap. */
/* 1 when a and b can share one paired pass, else 0.  Host-only. */
int sdb_chain_pairable(const sdb_chain_desc *a, const sdb_chain_desc *b);
/* 1 and *key when c can take part in a paired pass, else 0: chains that can
 * pair have equal keys (equal keys are then checked with
 * sdb_chain_pairable), so a batch groups its chains in one pass over them.
 * Host-only. */
int sdb_chain_pair_key(const sdb_chain_desc *c, uint64_t *key);
/* Runs a and b as one paired pass on `stream`; SDB_ERR_UNSUPPORTED (nothing
 * launched) when they cannot pair. */
int sdb_chain_launch_pair(const sdb_chain_desc *a, const sdb_chain_desc *b, sdb_stream_t stream);

/* ------------------------------------------------------------ chain batches
 * Many fused chains in one persistent launch per chain shape.  No counterpart
 * in the reference, which runs one plan at a time (executor/ddor_executor.cpp:
 * 22-245); the results are those of calling sdb_fused_chain on each chain in
 * turn.  Chains are grouped by the kernel instantiation they map to; each
 * group's (chain, tile range) spans go to one launch whose blocks pull spans
 * from a device work queue.  Chains without a batched instantiation are
 * launched one by one by sdb_chain_batch_launch.  Hash-table builds
 * (SDB_TERM_BUILD_*) go first, all of them in one persistent launch of the
 * general pass, so the other chains may probe the tables they build; a build
 * chain may not probe a table that another build chain of the batch writes.
 *
 * sdb_chain_batch_create checks every chain, writes the batch's tables into
 * `dev_scratch` (sdb_chain_batch_scratch_bytes(chains, n) bytes, 256-byte
 * aligned) and waits for that copy on `stream`, so it must not run under
 * stream capture.  sdb_chain_batch_launch issues one memset and the kernels,
 * nothing else; the chains' buffers must stay valid and their outputs be
 * zeroed (group-by slots, sums) before each launch.  Launches of one batch
 * must not overlap: they share the work-queue heads in `dev_scratch`. */
typedef struct sdb_chain_batch sdb_chain_batch;
size_t sdb_chain_batch_scratch_bytes(const sdb_chain_desc *chains, int n_chains);
int sdb_chain_batch_create(const sdb_chain_desc *chains, int n_chains, void *dev_scratch, size_t dev_bytes,
                           sdb_stream_t stream, sdb_chain_batch **out);
/* As sdb_chain_batch_create, without waiting: the tables are written into
 * `host_staging` (pinned host memory of at least the scratch size), copied
 * with one cudaMemcpyAsync on `stream`, and `host_staging` must stay
 * untouched until that copy has completed. */
int sdb_chain_batch_create_async(const sdb_chain_desc *chains, int n_chains, void *dev_scratch, size_t dev_bytes,
                                 void *host_staging, size_t host_bytes, sdb_stream_t stream, sdb_chain_batch **out);
int sdb_chain_batch_launch(const sdb_chain_batch *batch, sdb_stream_t stream);
/* One part of sdb_chain_batch_launch: part 0 launches the build chains (if
 * any), part 1 the rest (memset included); part 0 then part 1 on one stream is
 * sdb_chain_batch_launch.  Lets a caller time the two apart. */
int sdb_chain_batch_launch_part(const sdb_chain_batch *batch, int part, sdb_stream_t stream);
/* Kernel launches one sdb_chain_batch_launch makes (the memset excluded). */
int sdb_chain_batch_kernels(const sdb_chain_batch *batch);
void sdb_chain_batch_destroy(sdb_chain_batch *batch);

/* ------------------------------------------------------ synthetic SSB data */

/* Counter-based generator shared by host and device: value of row `row` of
 * stream `stream_id` under `seed`, uniform in [lo, hi]. */
int32_t sdb_gen_uniform_host(uint64_t seed, uint64_t stream_id, uint64_t row, int32_t lo, int32_t hi);
/* Fill dst[0..n) with rows [row0, row0+n) of a uniform stream (device). */
int sdb_gen_uniform(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id,
                    int32_t lo, int32_t hi, sdb_stream_t stream);
/* Same on the host (dst is host memory), multi-threaded. */
int sdb_gen_uniform_cpu(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id,
                        int32_t lo, int32_t hi);
/* dst[i] = YYYYMMDD of day (day0 + i) counted from 1992-01-01 (host). */
int sdb_gen_datekeys_cpu(int32_t *dst, uint64_t n, int64_t day0);
/* lo_orderdate-style column: YYYYMMDD of a uniform day in [0, ndays). */
int sdb_gen_dates(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id,
                  int32_t ndays, sdb_stream_t stream);
int sdb_gen_dates_cpu(int32_t *dst, uint64_t n, uint64_t row0, uint64_t seed, uint64_t stream_id,
                      int32_t ndays);

/* ------------------------------------------------------------ host executor */

/* The executor above the kernels: Table/Column/Segment storage, TransientTable
 * with its pending per-segment kernel phases, and the plan-node dispatch of
 * executor::execute_ddor_plan (executor/ddor_executor.cpp:22-245).  Plans are
 * JSON text in the shape of the Thrift PlanResult (server/thrift/
 * calciteserver.thrift:22-80): {"rels": [{"id":0, "relOp":"TABLE_SCAN",
 * "tables":["ssb","lineorder"]}, ...]}. */
typedef struct sdb_engine sdb_engine;
typedef struct sdb_result sdb_result;

typedef struct sdb_engine_config {
    uint64_t arena_bytes;       /* device budget for intermediates (memory_manager budget) */
    uint64_t segment_rows;      /* rows per segment; 0 = 2^28 (common.hpp:12) */
    int32_t fuse;               /* 1: run fusable kernel runs as one sdb_fused_chain pass */
    int32_t profile;            /* 1: time every launch with CUDA events */
    sdb_stream_t stream;        /* NULL: the engine creates its own stream */
    int32_t plan_cache;         /* > 0: prepared plans kept (see sdb_engine_execute); 0: none */
    int32_t order_by;           /* 1: sdb_engine_execute orders result rows by the plan's last SORT
                                   collation on the device (sdb_sort_rows); 0: rows in the order the
                                   reference gives them (its SORT is a pass-through) */
    int32_t join_tables;        /* 0: a join's table is direct-address over the build key range (the
                                   reference's), or open-addressing (sdb_ht_build_keys_oa) when the
                                   range is sparse: at least 2^20 keys and 8 x the open-addressing
                                   slots (16 x the build rows); 1: always direct-address; 2: always
                                   open-addressing.  Results are the same either way. */
    int32_t no_shared_scans;    /* 0: a batch (and a served batch) runs pairs of its plans' fact chains
                                   that scan the same rows as one paired pass each
                                   (sdb_chain_launch_pair); 1: every chain on its own.  Results are
                                   the same either way. */
} sdb_engine_config;

/* Plan text.  Every entry that takes plan_json reads two dialects: the
 * reference's Thrift IDL shape (PlanResult/RelNode/ExprType of
 * server/thrift/calciteserver.thrift:22-80, enums by name or number) and
 * Calcite's RelJson as the reference's planner emits it, which
 * SycldbJsonConverter turns into those structs
 * (server/src/main/java/com/eurecom/calcite/SycldbJsonConverter.java:31-163:
 * planner class names as relOp, "table", string ids and inputs,
 * {"name": ...} operators and aggregates, bare-number literals, Sarg
 * rangeSets). */

/* Parses a plan and derives its execution order and group-by columns
 * (operations/preprocessing.cpp:104-275) without touching a device.
 * *n_rels = number of plan nodes; order (optional, n_rels entries) = the DAG
 * execution order. */
int sdb_plan_check(const char *plan_json, int *n_rels, int *order, int order_cap);

/* The plan as parsed, written back in the IDL shape (what
 * SycldbJsonConverter hands the executor through Thrift): *len = its length
 * without the terminating NUL; the text is copied to out when cap > *len.
 * Replaces SycldbJsonConverter.getRels + the Thrift transfer
 * (SycldbJsonConverter.java:13-29). */
int sdb_plan_to_idl_json(const char *plan_json, char *out, size_t cap, size_t *len);

int sdb_engine_create(const sdb_engine_config *cfg, sdb_engine **out);
int sdb_engine_destroy(sdb_engine *eng);

/* Register a base table.  cols[c] points at nrows int32 values, or is NULL
 * for a column that is not loaded.  on_device = 1: device pointers used in
 * place (caller keeps them alive); 0: host pointers, copied to the device
 * (pinned memory gives full bandwidth).  Computes per-segment min/max
 * (synchronises the engine stream).  Re-registering a name replaces it. */
int sdb_engine_load_table(sdb_engine *eng, const char *name, int ncols, const int32_t *const *cols,
                          uint64_t nrows, int on_device);

/* Register a base table from the reference's columnar files (Table::Table,
 * models/models.hpp:1659-1708): one file per column, dir/<NAME><i> with the
 * table name upper-cased ("LINEORDER5"), raw int32 in the machine's byte
 * order.  column_mask: bit i loads column i; 0 = the reference loader's
 * column set (kernels/types.cpp:3-11).  The row count is the first loaded
 * column's; a missing file, or one of another length, leaves that column
 * unloaded with a warning on stderr, as the reference does.  Files are read
 * in 32 MB chunks through two pinned buffers so that reading overlaps the
 * copies to the device.  background = 1: returns at once; a loader thread
 * reads, copies and computes segment min/max on its own stream, and the
 * first execute that scans the table (or sdb_engine_sync_tables) waits for
 * it and installs it -- the whole-table counterpart of the reference's
 * background copy activated on first use (models/models.hpp:489-564).  A
 * failed background load reports its error at that point. */
int sdb_engine_load_dir(sdb_engine *eng, const char *dir, const char *name, uint64_t column_mask, int background);
/* Waits for every background load and installs the tables. */
int sdb_engine_sync_tables(sdb_engine *eng);

/* Execute one plan; on success *out holds the result rows (host memory).
 * With plan_cache > 0 (and profile = 0) the second execution of the same plan
 * text prepares it as a one-plan batch (sdb_engine_batch_prepare: recorded
 * once against an arena of its own, captured as a CUDA graph); later
 * executions replay the graph -- the same kernels on the same tables, without
 * the host work of planning.  Up to plan_cache plans stay prepared (least
 * recently used dropped); sdb_engine_load_table drops them all. */
int sdb_engine_execute(sdb_engine *eng, const char *plan_json, sdb_result **out);

/* Result: flagged rows of the final table in row order, non-null columns in
 * order (executor/result_writer.cpp:41-67).  Column type 0 = int32,
 * 1 = uint64. */
int sdb_result_shape(const sdb_result *r, int *ncols, uint64_t *nrows);
int sdb_result_column(const sdb_result *r, int c, int *type, const void **data);
/* Writes the rows as the reference's .res file does (space-separated, one
 * row per line). */
int sdb_result_write_res(const sdb_result *r, const char *path);
void sdb_result_free(sdb_result *r);

/* Per-kernel launch statistics of the last execute (profile = 1):
 * name of kernel kind k, launches, total milliseconds.  Returns the number of
 * kinds when k is out of range. */
int sdb_engine_kernel_stats(const sdb_engine *eng, int k, const char **name, uint64_t *launches,
                            double *total_ms);
/* Device milliseconds of the last execute (CUDA events around the plan). */
int sdb_engine_last_plan_ms(const sdb_engine *eng, double *ms);

/* ---------------------------------------------------------------- batches
 * Many plans prepared once and run together.  No counterpart in the
 * reference, whose executor runs one plan at a time
 * (executor/ddor_executor.cpp:22-245); each plan's result is the one
 * sdb_engine_execute gives for it alone.
 *
 * Prepare records every plan's device work without running it (a sizing pass,
 * then a pass against an arena of exactly the size needed, owned by the
 * batch), splits each plan at its aggregating fused chain and gathers those
 * chains into one sdb_chain_batch.  A run replays: the zeroed region is
 * cleared, the plans' work before their chains runs spread over up to 8
 * streams, then the chain batch (one persistent launch per chain shape), then
 * the plans' remaining work and the copies of their results at full capacity
 * into pinned host staging.  Unless SDB_BATCH_EAGER, the replay is captured
 * once as a CUDA graph and each run is one graph launch.  The base tables the
 * plans read must stay loaded, unchanged, while the batch lives.  Runs of one
 * batch must not overlap; different batches and plain executes may alternate
 * freely (each batch has its own arena). */
typedef struct sdb_batch sdb_batch;

#define SDB_BATCH_EAGER 1           /* replay the recorded launches on every run, no graph */
#define SDB_BATCH_NO_CHAIN_BATCH 2  /* launch every fused chain on its own */
#define SDB_BATCH_BUILDS_ONLY 4     /* batch only the hash-table builds (one launch); the aggregating
                                       chains run on their own, with the tuned single-chain kernel */

typedef struct sdb_batch_stats {
    int32_t n_plans;
    int32_t kernels_per_run;  /* library kernel launches one run makes */
    int32_t graph;            /* 1: runs are CUDA graph launches */
    int32_t chain_launches;   /* kernel launches of the chain batch (one per chain shape, one for all builds) */
    int32_t batched_chains;   /* aggregating chains that went into the chain batch */
    int32_t batched_builds;   /* hash-table build chains that went into its build launch */
    uint64_t arena_bytes;     /* the batch's device arena */
    uint64_t zero_bytes;      /* of it, the region cleared on each run */
    uint64_t host_bytes;      /* pinned staging */
    double last_run_ms;       /* device milliseconds of the last run */
    double last_chain_ms;     /* of it, the chain batch's aggregating chains (0: none) */
    double last_pre_ms;       /* zeroing and the plans' unbatched work before the aggregating chains */
    double last_post_ms;      /* after it: final flags, compaction, gathers, result copies */
    double last_build_ms;     /* the chain batch's hash-table builds (one launch; 0: none) */
    int32_t paired_chains;    /* fact chains run two by two in paired passes (sdb_chain_launch_pair) */
} sdb_batch_stats;

int sdb_engine_batch_prepare(sdb_engine *eng, const char *const *plans_json, int n_plans, int flags,
                             sdb_batch **out);
/* Runs the batch once and waits for it; results[i] (n_plans entries, may be
 * NULL to skip the unpacking) receives plan i's result, freed with
 * sdb_result_free. */
int sdb_batch_run(sdb_batch *batch, sdb_result **results);
int sdb_batch_info(const sdb_batch *batch, sdb_batch_stats *info);
void sdb_batch_free(sdb_batch *batch);
/* Results without unpacking (for bindings that build their own arrays): after
 * sdb_batch_run (results may be NULL), the batch's pinned result mirror
 * (sdb_batch_host, `bytes` long, valid until the next run) holds for each
 * plan and segment a uint32 row count at count_off and each result column
 * (capacity rows; the first `count` are the result, in row order) at
 * col_offs[c]; sdb_batch_layout gives a plan's column count and types (0 int32,
 * 1 uint64) and segments. */
int sdb_batch_layout(const sdb_batch *batch, int plan, int *ncols, int *types, int types_cap, int *nsegs);
int sdb_batch_segment(const sdb_batch *batch, int plan, int seg, uint64_t *count_off, uint64_t *col_offs, int cap,
                      uint64_t *capacity);
const void *sdb_batch_host(const sdb_batch *batch, size_t *bytes);

/* ----------------------------------------------------------------- server
 * Continuous batching of arriving plans over the engine's loaded tables.  No
 * counterpart in the reference, whose application runs one plan at a time
 * (app/application.cpp:37-48); every result equals what sdb_engine_execute
 * gives for the plan alone.
 *
 * One dispatcher thread owns the device work and keeps up to `slots` batches
 * in flight, each on its own streams.  Whenever a slot is free and requests
 * wait, it admits the longest first-come prefix (at most max_batch plans)
 * whose hash tables and intermediates fit the free part of the device budget,
 * records those plans against memory carved from the budget (exact sizes from
 * a sizing pass) and enqueues them as one batch (sdb_engine_batch_prepare's
 * phases, without a graph: each batch runs once).  Requests arriving while
 * batches run go into the next free slot, so their work overlaps on the
 * device.  A request whose plan is invalid, or needs more than the whole
 * budget, finishes with an error status.  While a server exists its engine
 * must not be used by any other call (sdb_engine_execute, load_table, ...). */
typedef struct sdb_server sdb_server;

typedef struct sdb_server_config {
    uint64_t budget_bytes;    /* device memory for admitted plans' tables and intermediates; 0 = 60 GB */
    uint64_t pinned_bytes;    /* pinned host staging of results; 0 = 1 GB */
    int32_t slots;            /* batches in flight; 0 = 4 */
    int32_t max_batch;        /* plans per batch; 0 = 64 */
    int32_t streams_per_slot; /* 0 = 4 */
    int32_t no_direct;        /* 0: while no batch is in flight and at most 4 requests wait, the
                                 oldest runs at once through the plain path (no sizing pass, no batch
                                 set-up; first come first served); a longer queue goes into batches;
                                 1: every request goes through a batch */
} sdb_server_config;

typedef struct sdb_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t batches, batched_plans;   /* batches launched, plans in them */
    uint64_t max_batch_plans;          /* largest batch */
    uint64_t max_inflight_plans;       /* most plans admitted and unfinished at once */
    uint64_t peak_device_bytes;        /* most budget bytes in use at once */
    uint64_t peak_pinned_bytes;
    uint64_t budget_bytes;
    uint64_t direct_plans;             /* requests run at once through the plain path (idle server) */
    uint64_t sizing_us;                /* dispatcher host time in sizing passes (microseconds) */
    uint64_t launch_us;                /* dispatcher host time recording and enqueueing batches */
    uint64_t paired_chains;            /* fact chains run two by two in paired passes */
} sdb_server_stats;

int sdb_server_create(sdb_engine *eng, const sdb_server_config *cfg, sdb_server **out);
/* Queues a plan (thread-safe, does not wait); *id identifies its result. */
int sdb_server_submit(sdb_server *server, const char *plan_json, int64_t *id);
/* Waits up to timeout_ms (< 0: without limit) for the next finished request:
 * its id, status (SDB_OK or the failure; sdb_last_error() then holds the
 * message), result (NULL on failure; free with sdb_result_free) and latency
 * (ms from submission to the result reaching the host).  SDB_ERR_TIMEOUT when
 * none finished in time. */
int sdb_server_next(sdb_server *server, int timeout_ms, int64_t *id, int *status, sdb_result **result,
                    double *latency_ms);
int sdb_server_stats_get(sdb_server *server, sdb_server_stats *out);
/* Finishes every queued request, then frees the server (unread results too). */
int sdb_server_destroy(sdb_server *server);

/* Load generator over an arrival trace: plan i is submitted arrival_s[i]
 * seconds after the start (open loop, from an internal thread) and its status,
 * latency (from its scheduled arrival) and, if `results` is not NULL, result
 * are stored at index i.  *wall_s = seconds from the start to the last
 * completion.  Nothing else may submit to the server meanwhile. */
int sdb_server_replay(sdb_server *server, const char *const *plans, const double *arrival_s, int n, int *status,
                      sdb_result **results, double *latency_ms, double *wall_s);
/* The same trace through the plain path: one plan at a time, in arrival
 * order, each started at its arrival or when the previous one finished. */
int sdb_engine_replay_plain(sdb_engine *eng, const char *const *plans, const double *arrival_s, int n, int *status,
                            sdb_result **results, double *latency_ms, double *wall_s);

#ifdef __cplusplus
}
#endif

#endif /* SYCLDB_GPU_H */
