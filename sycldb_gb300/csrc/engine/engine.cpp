// Host executor above the C ABI kernels.
//
// This restates the reference's operator API for one GPU:
//   memory_manager      operations/memory_manager.{hpp,cpp}   (bump regions, zeroed region)
//   Segment/Column/Table models/models.hpp:20-1802            (int32 segments of <= 2^28 rows, min/max stats)
//   KernelData/Bundle   models/execution.hpp:30-651           (KernelType switch -> one C ABI call)
//   TransientTable      models/transient_table.hpp:20-1928    (flags, pending phases, apply_*)
//   execute_ddor_plan   executor/ddor_executor.cpp:22-245     (plan-node dispatch)
//   parse_execution_info operations/preprocessing.cpp:14-275  (group-by columns, DAG order)
// SYCL queues and events become one CUDA stream; kernels of a segment run in
// phase order on that stream, so no host wait is needed between bundles (the
// reference waits after each one).  Everything lives on the device: the
// reference's host-side kernel paths (used when a segment is not on a
// device) are not needed, so LITERAL projections fill on the device.
//
// With fusion on, each segment's bundle is scanned for runs of fusable
// kernels (selections, SEARCH triples, semi/full probes, projections) ending
// optionally in a SUM or group-by; a run becomes one sdb_fused_chain pass that
// computes the same outputs (the reference's own call-sequence fusion,
// models/execution.hpp:546-615, is disabled).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <future>
#include <functional>
#include <map>
#include <memory>
#include <new>
#include <set>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <mutex>
#include <thread>

#include <cuda_runtime.h>

#include "batch_api.hpp"
#include "plan.hpp"
#include "sycldb_gpu.h"

int sdb_set_error(int status, const char *fmt, ...);

namespace sdb {

constexpr uint64_t kDefaultSegment = 1ull << 28;  // common.hpp:12
// Aggregating chains of at least this many rows are not put in a batch's
// chain batch: one launch of such a chain fills the GPU by itself (152 SMs x
// 5 blocks x 8 tiles of 1024 rows is 6.2 M rows), and the tuned single-chain
// kernel runs it faster than the persistent batched one.  Measured on the
// 64-plan star batch: 2^21 / 2^22 / 2^23 / 2^25 / never -> 21.8 / 22.0 /
// 22.3 / 21.1 / 21.0 thousand queries/s; the served SF50 mix gains 15 %.
constexpr uint64_t kSoloChainRows = 1ull << 23;

// kernels/types.cpp:3-21
const std::map<std::string, std::set<int>> &table_column_indices()
{
    static const std::map<std::string, std::set<int>> m = {
        {"lineorder", {2, 3, 4, 5, 8, 9, 11, 12, 13}},
        {"part", {0, 2, 3, 4}},
        {"supplier", {0, 3, 4, 5}},
        {"customer", {0, 3, 4, 5}},
        {"ddate", {0, 4, 5}},
    };
    return m;
}

const std::map<std::string, int> &table_column_numbers()
{
    static const std::map<std::string, int> m = {
        {"lineorder", 17}, {"part", 9}, {"supplier", 7}, {"customer", 8}, {"ddate", 17}};
    return m;
}

// Tables may be registered under "<schema table>@<tag>" (e.g. one fact
// partition per tag); the schema is that of the part before '@'.
std::string base_name(const std::string &name)
{
    size_t at = name.find('@');
    return at == std::string::npos ? name : name.substr(0, at);
}

#define SDB_CUDA(x)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) throw ::sdb::Error(SDB_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

inline void check(int st)
{
    if (st != SDB_OK) throw Error(st, sdb_last_error());
}

// ------------------------------------------------------------------ strings
// kernels/selection.hpp:23-49, kernels/aggregation.hpp:37-48
int get_comp_op(const std::string &op)
{
    if (op == "==") return SDB_EQ;
    if (op == ">=") return SDB_GE;
    if (op == "<=") return SDB_LE;
    if (op == "<") return SDB_LT;
    if (op == ">") return SDB_GT;
    if (op == "!=" || op == "<>") return SDB_NE;
    return SDB_EQ;
}

int get_logical_op(const std::string &op)
{
    if (op == "AND") return SDB_AND;
    if (op == "OR") return SDB_OR;
    return SDB_NONE;
}

bool is_filter_logical(const std::string &op)
{
    for (char c : op)
        if (!std::isalpha((unsigned char)c)) return false;
    return true;
}

int get_op_from_string(const std::string &op)
{
    if (op == "*") return SDB_MUL;
    if (op == "/") return SDB_DIV;
    if (op == "+") return SDB_ADD;
    if (op == "-") return SDB_SUB;
    throw Error(SDB_ERR_INVALID, "Unknown operation: " + op);
}

// std::stoi as the reference's Segment::search_operator uses it.
int32_t stoi_ref(const std::string &s)
{
    try {
        return (int32_t)std::stoi(s);
    } catch (const std::exception &) {
        throw Error(SDB_ERR_INVALID, "SEARCH bound is not an integer: '" + s + "'");
    }
}

// ------------------------------------------------------------------ memory
// Device bump allocator with a zeroed region of budget/64
// (operations/memory_manager.cpp:219-233); reset per query.  Allocations are
// 256-byte aligned (the reference aligns to 8).
class MemoryManager {
public:
    MemoryManager() = default;
    ~MemoryManager() { release(); }

    void init(uint64_t budget, cudaStream_t s) { init_sized(budget, std::max<uint64_t>(budget >> 6, 1u << 20), s); }
    // device bytes of the arena and its zeroed region
    uint64_t capacity() const { return size_ + zsize_; }

    void init_sized(uint64_t size, uint64_t zsize, cudaStream_t s)
    {
        release();
        size_ = std::max<uint64_t>(size, 256);
        zsize_ = std::max<uint64_t>(zsize, 256);
        SDB_CUDA(cudaMalloc(&base_, size_));
        SDB_CUDA(cudaMalloc(&zbase_, zsize_));
        SDB_CUDA(cudaMemsetAsync(zbase_, 0, zsize_, s));
        used_ = zused_ = zdirty_ = peak_ = 0;
    }

    // Hands out addresses that are never dereferenced: a sizing pass records
    // a batch's work without running it, to learn how much memory it needs.
    void init_virtual()
    {
        release();
        virtual_ = true;
        base_ = reinterpret_cast<char *>(uintptr_t(1) << 44);
        zbase_ = reinterpret_cast<char *>(uintptr_t(3) << 44);
        size_ = zsize_ = uint64_t(1) << 43;
        used_ = zused_ = zdirty_ = peak_ = 0;
    }

    // Carves the arena out of memory the caller owns (a server's pool); the
    // caller clears the zeroed region before the work that uses it.
    void init_external(char *base, uint64_t size, char *zbase, uint64_t zsize)
    {
        release();
        external_ = true;
        base_ = base;
        zbase_ = zbase;
        size_ = size;
        zsize_ = zsize;
        used_ = zused_ = zdirty_ = peak_ = 0;
    }

    void release()
    {
        if (!virtual_ && !external_) {
            if (base_) cudaFree(base_);
            if (zbase_) cudaFree(zbase_);
        }
        virtual_ = external_ = false;
        base_ = zbase_ = nullptr;
    }

    void swap(MemoryManager &o)
    {
        std::swap(base_, o.base_);
        std::swap(zbase_, o.zbase_);
        std::swap(size_, o.size_);
        std::swap(used_, o.used_);
        std::swap(peak_, o.peak_);
        std::swap(zsize_, o.zsize_);
        std::swap(zused_, o.zused_);
        std::swap(zdirty_, o.zdirty_);
        std::swap(virtual_, o.virtual_);
        std::swap(external_, o.external_);
    }

    uint64_t used() const { return used_; }
    uint64_t zused() const { return zused_; }
    uint64_t size() const { return size_; }
    uint64_t zsize() const { return zsize_; }
    char *zero_base() const { return zbase_; }
    char *base() const { return base_; }

    template <typename T>
    T *alloc(uint64_t count)
    {
        uint64_t bytes = (count * sizeof(T) + 255) & ~(uint64_t)255;
        if (bytes == 0) bytes = 256;
        if (used_ + bytes > size_)
            throw Error(SDB_ERR_NOMEM, "Memory manager out of memory: requested " + std::to_string(bytes) +
                                           " bytes, " + std::to_string(size_ - used_) + " bytes available");
        T *p = reinterpret_cast<T *>(base_ + used_);
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return p;
    }

    template <typename T>
    T *alloc_zero(uint64_t count)
    {
        uint64_t bytes = (count * sizeof(T) + 255) & ~(uint64_t)255;
        if (bytes == 0) bytes = 256;
        if (zused_ + bytes > zsize_)
            throw Error(SDB_ERR_NOMEM, "Memory manager out of zeroed memory: requested " + std::to_string(bytes) +
                                           " bytes, " + std::to_string(zsize_ - zused_) + " bytes available");
        T *p = reinterpret_cast<T *>(zbase_ + zused_);
        zused_ += bytes;
        zdirty_ = std::max(zdirty_, zused_);
        return p;
    }

    // memory_manager::reset (operations/memory_manager.cpp:71-90): rewind and
    // re-zero what the zeroed region handed out.
    void reset(cudaStream_t s)
    {
        used_ = 0;
        if (zdirty_) SDB_CUDA(cudaMemsetAsync(zbase_, 0, zdirty_, s));
        zused_ = zdirty_ = 0;
    }

    uint64_t peak() const { return peak_; }

private:
    char *base_ = nullptr, *zbase_ = nullptr;
    uint64_t size_ = 0, used_ = 0, peak_ = 0;
    uint64_t zsize_ = 0, zused_ = 0, zdirty_ = 0;
    bool virtual_ = false;
    bool external_ = false;
};

// ------------------------------------------------------------------ storage
struct Segment {
    int32_t *data = nullptr;   // int32 rows (device)
    uint64_t *agg = nullptr;   // uint64 rows of an aggregate result (device)
    uint64_t nrows = 0;
    int32_t min = 0, max = 0;
};

struct Column {
    std::vector<Segment> segments;
    bool is_aggregate_result = false;

    // models/models.hpp:1257-1272
    std::pair<int32_t, int32_t> get_min_max() const
    {
        if (is_aggregate_result) throw Error(SDB_ERR_INVALID, "can't get min/max of aggregate result column");
        if (segments.empty()) throw Error(SDB_ERR_INVALID, "column is not loaded");
        int32_t mn = segments[0].min, mx = segments[0].max;
        for (size_t i = 1; i < segments.size(); i++) {
            mn = std::min(mn, segments[i].min);
            mx = std::max(mx, segments[i].max);
        }
        return {mn, mx};
    }
};

std::vector<std::pair<uint64_t, uint64_t>> split_rows(uint64_t n, uint64_t seg)
{
    std::vector<std::pair<uint64_t, uint64_t>> out;
    for (uint64_t s = 0; s < n; s += seg) out.emplace_back(s, std::min(seg, n - s));
    return out;
}

struct Table {
    std::string name;
    std::vector<Column> columns;
    uint64_t nrows = 0;
    std::vector<int32_t *> owned;  // device copies made by load_table
};

// ------------------------------------------------------------------ kernels
enum class KernelType : uint8_t {  // models/execution.hpp:30-46
    EmptyKernel,
    LogicalKernel,
    SelectionKernelColumns,
    SelectionKernelLiteral,
    FillKernel,
    PerformOperationKernelColumns,
    PerformOperationKernelLiteralFirst,
    PerformOperationKernelLiteralSecond,
    BuildKeysHTKernel,
    FilterJoinKernel,
    BuildKeyValsHTKernel,
    FullJoinKernel,
    AggregateOperationKernel,
    GroupByAggregateKernel,
};

const char *kernel_name(KernelType t)
{
    switch (t) {
    case KernelType::EmptyKernel: return "empty";
    case KernelType::LogicalKernel: return "logical";
    case KernelType::SelectionKernelColumns: return "select_cols";
    case KernelType::SelectionKernelLiteral: return "select_lit";
    case KernelType::FillKernel: return "fill_i32";
    case KernelType::PerformOperationKernelColumns: return "binop_cc";
    case KernelType::PerformOperationKernelLiteralFirst: return "binop_lc";
    case KernelType::PerformOperationKernelLiteralSecond: return "binop_cl";
    case KernelType::BuildKeysHTKernel: return "ht_build_keys";
    case KernelType::FilterJoinKernel: return "probe_semi";
    case KernelType::BuildKeyValsHTKernel: return "ht_build_kv";
    case KernelType::FullJoinKernel: return "probe_full";
    case KernelType::AggregateOperationKernel: return "sum";
    case KernelType::GroupByAggregateKernel: return "groupby";
    }
    return "?";
}

// Type-erased operator: the fields a KernelDefinition subclass would hold.
struct KernelData {
    KernelType type = KernelType::EmptyKernel;
    uint64_t n = 0;
    int cmp = 0, logic = 0, bin = 0;
    const int32_t *a = nullptr, *b = nullptr;
    int32_t la = 0, lb = 0;
    const uint8_t *in = nullptr, *local = nullptr;
    uint8_t *out = nullptr;
    int32_t *res = nullptr;            // fill / perform result, full-join value output
    void *ht = nullptr;
    int32_t ht_min = 0, ht_max = 0, ht_len = 0;
    int ht_log2 = 0;        // 0: direct-address table; n: open-addressing table of 2^n slots
    bool ht_fresh = false;  // builds: the table is still all zero (the first segment's build)
    uint64_t *agg_res = nullptr;
    std::vector<const int32_t *> keys;  // group-by
    std::vector<int32_t> mins, maxs;
    std::vector<int32_t *> out_keys;
    uint64_t P = 0;
    uint32_t *occ = nullptr;

    // KernelData::execute (models/execution.hpp:260-497): one C ABI call.
    int execute(cudaStream_t s) const
    {
        auto st = (sdb_stream_t)s;
        switch (type) {
        case KernelType::EmptyKernel: return SDB_OK;
        case KernelType::LogicalKernel: return sdb_logical(logic, in, local, out, n, st);
        case KernelType::SelectionKernelColumns: return sdb_select_cols(a, b, cmp, logic, in, out, n, st);
        case KernelType::SelectionKernelLiteral: return sdb_select_lit(a, lb, cmp, logic, in, out, n, st);
        case KernelType::FillKernel: return sdb_fill_i32(res, la, n, st);
        case KernelType::PerformOperationKernelColumns: return sdb_binop_cc(res, a, b, bin, in, n, st);
        case KernelType::PerformOperationKernelLiteralFirst: return sdb_binop_lc(res, la, b, bin, in, n, st);
        case KernelType::PerformOperationKernelLiteralSecond: return sdb_binop_cl(res, a, lb, bin, in, n, st);
        case KernelType::BuildKeysHTKernel:
            if (ht_log2)
                return sdb_ht_build_keys_oa(a, in, n, static_cast<uint32_t *>(ht), ht_log2, ht_min,
                                            (int32_t)((uint32_t)ht_min + (uint32_t)ht_len - 1u), ht_fresh ? 1 : 0, st);
            return sdb_ht_build_keys(a, in, n, static_cast<uint8_t *>(ht), ht_min, ht_len, st);
        case KernelType::FilterJoinKernel:
            if (ht_log2)
                return sdb_probe_semi_oa(a, in, out, n, static_cast<const uint32_t *>(ht), ht_log2, ht_min, ht_max, st);
            return sdb_probe_semi(a, in, out, n, static_cast<const uint8_t *>(ht), ht_min, ht_max, st);
        case KernelType::BuildKeyValsHTKernel:
            if (ht_log2)
                return sdb_ht_build_kv_oa(a, b, in, n, static_cast<int32_t *>(ht), ht_log2, ht_min,
                                          (int32_t)((uint32_t)ht_min + (uint32_t)ht_len - 1u), ht_fresh ? 1 : 0, st);
            return sdb_ht_build_kv(a, b, in, n, static_cast<int32_t *>(ht), ht_min, ht_len, st);
        case KernelType::FullJoinKernel:
            if (ht_log2)
                return sdb_probe_full_oa(a, res, in, out, n, static_cast<const int32_t *>(ht), ht_log2, ht_min, ht_max,
                                         st);
            return sdb_probe_full(a, res, in, out, n, static_cast<const int32_t *>(ht), ht_min, ht_max, st);
        case KernelType::AggregateOperationKernel: return sdb_sum_i32_u64(a, in, n, agg_res, st);
        case KernelType::GroupByAggregateKernel:
            return sdb_groupby_sum(keys.data(), mins.data(), maxs.data(), (int)keys.size(), a, in, n, P,
                                   out_keys.data(), agg_res, occ, st);
        }
        return sdb_set_error(SDB_ERR_INVALID, "Unknown kernel type");
    }
};

struct KernelBundle {  // models/execution.hpp:500-651 (one device, no host wait)
    std::vector<KernelData> kernels;
    bool on_device = true;
    int device_index = 0;
    void add_kernel(KernelData k) { kernels.push_back(std::move(k)); }
};

// ------------------------------------------------------------------ profiling
struct Profiler {
    bool on = false;
    struct Rec { std::string name; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    std::map<std::string, std::pair<uint64_t, double>> stats;

    cudaEvent_t ev()
    {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        SDB_CUDA(cudaEventCreate(&e));
        return e;
    }
    void begin(cudaStream_t s, const std::string &name, cudaEvent_t &a)
    {
        if (!on) return;
        a = ev();
        SDB_CUDA(cudaEventRecord(a, s));
        recs.push_back({name, a, nullptr});
    }
    void end(cudaStream_t s)
    {
        if (!on) return;
        cudaEvent_t b = ev();
        SDB_CUDA(cudaEventRecord(b, s));
        recs.back().b = b;
    }
    void collect()
    {
        for (auto &r : recs) {
            float ms = 0;
            if (r.b && cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
                auto &st = stats[r.name];
                st.first += 1;
                st.second += ms;
            }
            pool.push_back(r.a);
            if (r.b) pool.push_back(r.b);
        }
        recs.clear();
    }
    ~Profiler()
    {
        for (auto e : pool) cudaEventDestroy(e);
    }
};

struct Engine;

// ------------------------------------------------------------------ fusion
// Turns runs of a segment's kernel list into sdb_fused_chain launches.
struct Fuser {
    static bool fusable(KernelType t)
    {
        switch (t) {
        case KernelType::SelectionKernelLiteral:
        case KernelType::SelectionKernelColumns:
        case KernelType::LogicalKernel:
        case KernelType::FilterJoinKernel:
        case KernelType::FullJoinKernel:
        case KernelType::PerformOperationKernelColumns:
        case KernelType::PerformOperationKernelLiteralFirst:
        case KernelType::PerformOperationKernelLiteralSecond:
        case KernelType::FillKernel:
        case KernelType::AggregateOperationKernel:
        case KernelType::GroupByAggregateKernel:
        case KernelType::BuildKeysHTKernel:
        case KernelType::BuildKeyValsHTKernel:
            return true;
        default:
            return false;
        }
    }

    static bool is_build(int32_t terminal)
    {
        return terminal == SDB_TERM_BUILD_KEYS || terminal == SDB_TERM_BUILD_KV;
    }

    // Builds a chain from ks[i..]; returns the index after the last kernel
    // consumed, or i when no chain could be formed (two or more kernels, or a
    // hash-table build on its own).
    static size_t build(const std::vector<const KernelData *> &ks, size_t i,
                        const std::set<const uint8_t *> &all_true, sdb_chain_desc &c,
                        const uint8_t **final_flags = nullptr)
    {
        std::memset(&c, 0, sizeof c);
        if (final_flags) *final_flags = nullptr;
        const KernelData &first = *ks[i];
        const uint8_t *cur = nullptr;
        std::unordered_map<const int32_t *, int> regmap;  // column produced in-chain -> register
        int nregs = 0;
        size_t j = i;
        bool terminal = false, flags_in_set = false;
        c.n = first.n;

        auto operand = [&](const int32_t *col) {
            sdb_operand o{};
            auto it = regmap.find(col);
            if (it != regmap.end()) {
                o.kind = SDB_SRC_REG;
                o.reg = it->second;
            } else {
                o.kind = SDB_SRC_COL;
                o.col = col;
            }
            return o;
        };
        auto lit = [](int32_t v) {
            sdb_operand o{};
            o.kind = SDB_SRC_LIT;
            o.lit = v;
            return o;
        };

        while (j < ks.size() && c.n_ops < SDB_CHAIN_MAX_OPS && !terminal) {
            const KernelData &k = *ks[j];
            if (k.n != c.n || !fusable(k.type)) break;
            sdb_chain_op op{};
            size_t consumed = 1;
            // The first kernel fixes the chain's input flags.
            const uint8_t *kin = k.in;
            if (k.type == KernelType::SelectionKernelLiteral && k.in == k.out) {
                // SEARCH: select(local,NONE) ; select(local,AND|OR) ; logical(in, local, out)
                if (j + 2 >= ks.size()) break;
                const KernelData &k2 = *ks[j + 1], &k3 = *ks[j + 2];
                if (k2.type != KernelType::SelectionKernelLiteral || k3.type != KernelType::LogicalKernel) break;
                if (k2.in != k.out || k2.out != k.out || k3.local != k.out || k.a != k2.a || k.logic != SDB_NONE ||
                    k2.n != c.n || k3.n != c.n)
                    break;
                if (k.cmp == SDB_GE && k2.cmp == SDB_LE && k2.logic == SDB_AND) {
                    op.kind = SDB_OP_SEARCH_RANGE;
                } else if (k.cmp == SDB_EQ && k2.cmp == SDB_EQ && k2.logic == SDB_OR) {
                    op.kind = SDB_OP_SEARCH_POINTS;
                } else {
                    break;
                }
                op.a = operand(k.a);
                op.lo = k.lb;
                op.hi = k2.lb;
                op.logic_op = k3.logic;
                kin = k3.in;
                if (cur && kin != cur) break;
                cur = k3.out;
                consumed = 3;
            } else {
                if (cur && kin != cur) break;
                switch (k.type) {
                case KernelType::SelectionKernelLiteral:
                    op.kind = SDB_OP_SELECT;
                    op.cmp_op = k.cmp;
                    op.logic_op = k.logic;
                    op.a = operand(k.a);
                    op.b = lit(k.lb);
                    cur = k.out;
                    break;
                case KernelType::SelectionKernelColumns:
                    op.kind = SDB_OP_SELECT;
                    op.cmp_op = k.cmp;
                    op.logic_op = k.logic;
                    op.a = operand(k.a);
                    op.b = operand(k.b);
                    cur = k.out;
                    break;
                case KernelType::FilterJoinKernel:
                    op.kind = SDB_OP_SEMI_PROBE;
                    op.a = operand(k.a);
                    op.lo = k.ht_min;
                    op.hi = k.ht_max;
                    op.ht = k.ht;
                    op.ht_log2 = k.ht_log2;
                    cur = k.out;
                    break;
                case KernelType::FullJoinKernel:
                    if (nregs >= SDB_CHAIN_MAX_REGS) goto done;
                    op.kind = SDB_OP_FULL_PROBE;
                    op.a = operand(k.a);
                    op.lo = k.ht_min;
                    op.hi = k.ht_max;
                    op.ht = k.ht;
                    op.ht_log2 = k.ht_log2;
                    op.out_reg = nregs;
                    op.out_col = k.res;
                    regmap[k.res] = nregs++;
                    cur = k.out;
                    break;
                case KernelType::PerformOperationKernelColumns:
                case KernelType::PerformOperationKernelLiteralFirst:
                case KernelType::PerformOperationKernelLiteralSecond:
                    if (nregs >= SDB_CHAIN_MAX_REGS) goto done;
                    op.kind = SDB_OP_BINOP;
                    op.bin_op = k.bin;
                    op.a = k.type == KernelType::PerformOperationKernelLiteralFirst ? lit(k.la) : operand(k.a);
                    op.b = k.type == KernelType::PerformOperationKernelLiteralSecond ? lit(k.lb) : operand(k.b);
                    op.out_reg = nregs;
                    op.out_col = k.res;
                    regmap[k.res] = nregs++;
                    if (!cur) cur = k.in;  // reads flags without changing them
                    break;
                case KernelType::FillKernel:
                    if (nregs >= SDB_CHAIN_MAX_REGS) goto done;
                    op.kind = SDB_OP_FILL;
                    op.a = lit(k.la);
                    op.out_reg = nregs;
                    op.out_col = k.res;
                    regmap[k.res] = nregs++;
                    break;
                case KernelType::AggregateOperationKernel:
                    if (!cur) cur = k.in;
                    c.terminal = SDB_TERM_SUM;
                    c.value = operand(k.a);
                    c.sum_out = k.agg_res;
                    terminal = true;
                    break;
                case KernelType::GroupByAggregateKernel:
                    if (k.keys.size() > SDB_CHAIN_MAX_KEYS) goto done;
                    if (!cur) cur = k.in;
                    c.terminal = SDB_TERM_GROUPBY;
                    c.value = operand(k.a);
                    c.n_keys = (int32_t)k.keys.size();
                    for (size_t q = 0; q < k.keys.size(); q++) {
                        c.keys[q] = operand(k.keys[q]);
                        c.key_min[q] = k.mins[q];
                        c.key_max[q] = k.maxs[q];
                        c.out_keys[q] = k.out_keys[q];
                    }
                    c.P = k.P;
                    c.out_sum = k.agg_res;
                    c.occ = k.occ;
                    terminal = true;
                    break;
                case KernelType::BuildKeysHTKernel:
                case KernelType::BuildKeyValsHTKernel:
                    // K10 / K12 with the chain's flags; nothing after the build
                    // reads them (the build side's table is consumed by the join)
                    if (!cur) cur = k.in;
                    c.terminal = k.type == KernelType::BuildKeysHTKernel ? SDB_TERM_BUILD_KEYS : SDB_TERM_BUILD_KV;
                    c.build_key = operand(k.a);
                    if (k.type == KernelType::BuildKeyValsHTKernel) c.build_val = operand(k.b);
                    c.ht_out = k.ht;
                    c.ht_min = k.ht_min;
                    c.ht_len = k.ht_len;
                    c.ht_log2 = k.ht_log2;
                    c.ht_zeroed = k.ht_fresh ? 1 : 0;
                    terminal = true;
                    break;
                default:
                    goto done;
                }
            }
            if (!flags_in_set && kin) {
                c.flags_in = kin;
                flags_in_set = true;
            }
            if (!terminal) c.ops[c.n_ops++] = op;
            j += consumed;
        }
    done:
        const size_t count = j - i;
        if (count < 1 || (count < 2 && !(terminal && is_build(c.terminal)))) return i;
        // The input flags are not read when they are an untouched all-true
        // buffer, or when the first op overwrites them (logic NONE).
        if (c.flags_in && all_true.count(c.flags_in)) c.flags_in = nullptr;
        if (c.n_ops > 0 &&
            (c.ops[0].kind == SDB_OP_SELECT || c.ops[0].kind == SDB_OP_SEARCH_RANGE ||
             c.ops[0].kind == SDB_OP_SEARCH_POINTS) &&
            c.ops[0].logic_op == SDB_NONE)
            c.flags_in = nullptr;
        // Terminal: flags for a plain run; aggregates leave every
        // intermediate dead (apply_aggregate replaces flags and columns).
        if (!terminal) {
            c.terminal = SDB_TERM_FLAGS;
            c.flags_out = const_cast<uint8_t *>(cur);
        } else {
            for (int q = 0; q < c.n_ops; q++) c.ops[q].out_col = nullptr;
            c.flags_out = nullptr;
        }
        if (!terminal && !c.flags_out) return i;
        if (final_flags) *final_flags = cur;
        return j;
    }

    // Distinct columns a chain reads (the specialised pass stages up to 4).
    static int columns(const sdb_chain_desc &c)
    {
        std::set<const int32_t *> cols;
        auto add = [&](const sdb_operand &o) {
            if (o.kind == SDB_SRC_COL) cols.insert(o.col);
        };
        for (int k = 0; k < c.n_ops; k++) {
            if (c.ops[k].kind != SDB_OP_FILL) add(c.ops[k].a);
            if (c.ops[k].kind == SDB_OP_SELECT || c.ops[k].kind == SDB_OP_BINOP) add(c.ops[k].b);
        }
        if (c.terminal == SDB_TERM_SUM || c.terminal == SDB_TERM_GROUPBY) add(c.value);
        for (int q = 0; q < c.n_keys && c.terminal == SDB_TERM_GROUPBY; q++) add(c.keys[q]);
        return (int)cols.size();
    }

    // An aggregating chain that reads more columns than the specialised pass
    // stages, split in two specialised passes: its flag-only ops (semi
    // probes, AND selections of columns against literals) first, writing the
    // flags to `scratch` (the chain's own final flag buffer, which nothing
    // reads after an aggregation), then the rest reading them.  Every op of
    // such a chain ANDs into the row's flag and the flag-only ops use no
    // register, so the order of the two groups does not change any live
    // row's registers or the aggregate.  False (a, b untouched) when the
    // chain does not qualify or either half has no specialised pass.
    static bool split(const sdb_chain_desc &c, uint8_t *scratch, sdb_chain_desc &a, sdb_chain_desc &b)
    {
        if ((c.terminal != SDB_TERM_SUM && c.terminal != SDB_TERM_GROUPBY) || !scratch) return false;
        if (columns(c) <= 4 || sdb_chain_specialised(&c) >= 1) return false;
        sdb_chain_desc A = c, B = c;
        A.n_ops = B.n_ops = 0;
        for (int k = 0; k < c.n_ops; k++) {
            const sdb_chain_op &o = c.ops[k];
            const bool sel = o.kind == SDB_OP_SELECT || o.kind == SDB_OP_SEARCH_RANGE || o.kind == SDB_OP_SEARCH_POINTS;
            if (sel && (o.logic_op != SDB_AND || o.a.kind != SDB_SRC_COL ||
                        (o.kind == SDB_OP_SELECT && o.b.kind == SDB_SRC_REG)))
                return false;  // a NONE / OR selection or one over a register: order matters
            if (sel || (o.kind == SDB_OP_SEMI_PROBE && o.a.kind == SDB_SRC_COL))
                A.ops[A.n_ops++] = o;
            else
                B.ops[B.n_ops++] = o;
        }
        if (A.n_ops == 0 || B.n_ops == 0) return false;
        A.terminal = SDB_TERM_FLAGS;
        A.flags_out = scratch;
        B.flags_in = scratch;
        if (sdb_chain_specialised(&A) < 1 || sdb_chain_specialised(&B) < 1) return false;
        a = A;
        b = B;
        return true;
    }
};

// ------------------------------------------------------------------ engine state
// Device work recorded instead of run: a batch records every plan's launches,
// split at the plan's batched chain into the work before it (`pre`) and after
// it (`post`), and replays them later (eagerly or inside a CUDA graph).
struct DevOp {
    const char *name;
    std::function<int(cudaStream_t)> fn;
    bool has_chain = false;  // an aggregating fused chain (`chain`), which a shared scan may pair
    sdb_chain_desc chain{};
};

// A batch runs every plan's `pre` work, then every batched hash-table build
// (one launch), then every plan's `mid` work, then the batched aggregating
// chains, then every plan's `post` work.
struct PlanRecord {
    std::vector<DevOp> pre, mid, post;
    bool after = false;  // the plan's batched aggregating chain has been recorded
    size_t builds = 0;   // the plan's builds in the batch's build launch
};

struct Recorder {
    std::vector<PlanRecord> plans;
    std::vector<DevOp> shared_pre;       // paired fact scans of leading pre chains, before the pre work
    std::vector<DevOp> shared;           // paired fact scans of leading mid chains, after the builds
    std::vector<sdb_chain_desc> chains;  // chains for sdb_chain_batch
    bool batch_chains = true;            // aggregating chains into the chain batch
    bool batch_builds = true;            // hash-table builds into its build launch
};

struct Engine {
    sdb_engine_config cfg{};
    Recorder *rec = nullptr;  // non-null: record device work, don't run it
    // non-null: where result counts and gathered result columns go (a batch's
    // contiguous result region, copied to the host in one piece)
    MemoryManager *rmm = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // table loads: a second stream for segment statistics, the event that
    // hands a copied column to it, and the statistics' device and pinned words
    cudaStream_t aux = nullptr;
    cudaEvent_t copied = nullptr;
    int32_t *stats_dev = nullptr, *stats_host = nullptr;
    size_t stats_cap = 0;

    void stats_reserve(size_t words)
    {
        if (!copied) SDB_CUDA(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming));
        if (words <= stats_cap) return;
        if (stats_dev) cudaFree(stats_dev);
        if (stats_host) cudaFreeHost(stats_host);
        stats_dev = stats_host = nullptr;
        stats_cap = 0;
        const size_t cap = std::max<size_t>(words, 1024);
        SDB_CUDA(cudaMalloc(&stats_dev, cap * sizeof(int32_t)));
        SDB_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&stats_host), cap * sizeof(int32_t), cudaHostAllocDefault));
        stats_cap = cap;
    }
    uint64_t seg = kDefaultSegment;
    MemoryManager mm;
    std::map<std::string, std::unique_ptr<Table>> tables;
    // Tables being loaded from column files in the background: installed by
    // the first plan that scans them (activate).
    std::map<std::string, std::future<std::unique_ptr<Table>>> pending;
    Profiler prof;
    double last_plan_ms = 0;
    cudaEvent_t plan_a = nullptr, plan_b = nullptr;
    // Segment flag buffers that hold all-true: a TransientTable's initial
    // flags (transient_table.hpp:86,105), not written since.  The fill itself
    // is deferred until some kernel reads the buffer (`unfilled`), so a fused
    // pass that treats the buffer as all-true never pays for it.
    std::set<const uint8_t *> all_true;
    std::map<const uint8_t *, uint64_t> unfilled;
    // Segment flag buffers of a group-by result still to be derived from its
    // occupancy words (transient_table.hpp:1544-1558): the conversion runs
    // when a kernel reads the buffer, and the final compaction reads the
    // words directly instead.
    std::map<const uint8_t *, std::pair<const uint32_t *, uint64_t>> from_occ;

    // Every device operation of a plan goes through here: run now on the
    // engine's stream, or recorded for a batch.
    void dev(const char *name, std::function<int(cudaStream_t)> fn, const sdb_chain_desc *chain = nullptr)
    {
        if (rec) {
            PlanRecord &pr = rec->plans.back();
            DevOp op{name, std::move(fn)};
            if (chain) {
                op.has_chain = true;
                op.chain = *chain;
            }
            (pr.after ? pr.post : (pr.builds ? pr.mid : pr.pre)).push_back(std::move(op));
            return;
        }
        cudaEvent_t a = nullptr;
        prof.begin(stream, name, a);
        check(fn(stream));
        prof.end(stream);
    }

    void ensure_filled(const uint8_t *p)
    {
        auto oc = from_occ.find(p);
        if (oc != from_occ.end()) {
            uint8_t *q = const_cast<uint8_t *>(p);
            const uint32_t *occ = oc->second.first;
            const uint64_t n = oc->second.second;
            dev("occ_to_flags", [occ, q, n](cudaStream_t s) { return sdb_occ_to_flags(occ, q, n, (sdb_stream_t)s); });
            from_occ.erase(oc);
            return;
        }
        auto it = unfilled.find(p);
        if (it == unfilled.end()) return;
        uint8_t *q = const_cast<uint8_t *>(p);
        const uint64_t n = it->second;
        dev("fill_flags", [q, n](cudaStream_t s) { return sdb_fill_u8(q, n, 1, (sdb_stream_t)s); });
        unfilled.erase(it);
    }

    void written(const uint8_t *p)
    {
        all_true.erase(p);
        unfilled.erase(p);
        from_occ.erase(p);
    }

    void run_kernel(const KernelData &k)
    {
        // A selection or logical combine with logic NONE overwrites its
        // input (selection.hpp:83-96), so it does not need the fill.
        const bool ignores_in = (k.type == KernelType::SelectionKernelLiteral ||
                                 k.type == KernelType::SelectionKernelColumns || k.type == KernelType::LogicalKernel) &&
                                k.logic == SDB_NONE;
        if (k.in && !ignores_in) ensure_filled(k.in);
        dev(kernel_name(k.type), [k](cudaStream_t s) { return k.execute(s); });
        if (k.out) written(k.out);
    }


    // Whether a build chain can join the batch's build launch: it probes no
    // table that launch writes, and writes no table another build of the
    // launch writes (segments of one build side stay in order).
    bool build_batchable(const sdb_chain_desc &c) const
    {
        for (const sdb_chain_desc &o : rec->chains) {
            if (!Fuser::is_build(o.terminal)) continue;
            if (o.ht_out == c.ht_out) return false;
            for (int k = 0; k < c.n_ops; k++)
                if ((c.ops[k].kind == SDB_OP_SEMI_PROBE || c.ops[k].kind == SDB_OP_FULL_PROBE) && c.ops[k].ht == o.ht_out)
                    return false;
        }
        return true;
    }

    void run_chain(const sdb_chain_desc &c)
    {
        if (c.flags_in) ensure_filled(c.flags_in);
        PlanRecord *pr = rec ? &rec->plans.back() : nullptr;
        const bool build = Fuser::is_build(c.terminal);
        if (pr && rec->batch_builds && build && !pr->after && pr->mid.empty() && build_batchable(c)) {
            // into the batch's build launch, after the plan's pre work and
            // before anything the plan records later (its mid work)
            rec->chains.push_back(c);
            pr->builds++;
        } else if (pr && rec->batch_chains && !build && c.terminal != SDB_TERM_FLAGS && pr->post.empty() &&
                   c.n < kSoloChainRows) {
            // an aggregating chain goes into the batch's shared launch; the
            // plan's later work waits for it
            rec->chains.push_back(c);
            pr->after = true;
        } else {
            dev(build ? "build_chain" : "fused_chain",
                [c](cudaStream_t s) { return sdb_fused_chain(&c, (sdb_stream_t)s); },
                build || c.terminal == SDB_TERM_FLAGS ? nullptr : &c);
        }
        if (c.flags_out) written(c.flags_out);
    }

    // KernelBundle::execute for one segment, fusing runs when enabled.
    void run_kernels(const std::vector<const KernelData *> &ks)
    {
        size_t i = 0;
        while (i < ks.size()) {
            if (cfg.fuse && Fuser::fusable(ks[i]->type)) {
                sdb_chain_desc c;
                const uint8_t *last = nullptr;
                size_t j = Fuser::build(ks, i, all_true, c, &last);
                if (j > i) {
                    sdb_chain_desc a, b;
                    if (Fuser::split(c, const_cast<uint8_t *>(last), a, b)) {
                        run_chain(a);
                        run_chain(b);
                    } else {
                        run_chain(c);
                    }
                    i = j;
                    continue;
                }
            }
            run_kernel(*ks[i]);
            i++;
        }
    }
};

// ------------------------------------------------------------------ TransientTable
class TransientTable {
public:
    Engine &E;
    uint64_t nrows;
    uint8_t *flags = nullptr;
    uint8_t *flags_secondary = nullptr;
    std::vector<Column *> current_columns;
    std::deque<Column> materialized_columns;
    Column *group_by_column = nullptr;
    uint64_t group_by_column_index = 0;
    std::vector<std::vector<KernelBundle>> pending_kernels;

    // models/transient_table.hpp:52-156: flags filled with true.
    TransientTable(Engine &e, Table *base) : E(e), nrows(base->nrows)
    {
        flags = E.mm.alloc<uint8_t>(nrows);
        for (auto [start, cnt] : split_rows(nrows, E.seg)) {
            E.all_true.insert(flags + start);
            E.unfilled[flags + start] = cnt;
        }
        for (Column &c : base->columns) current_columns.push_back(&c);
    }

    uint64_t seg() const { return E.seg; }
    std::vector<std::pair<uint64_t, uint64_t>> segs() const { return split_rows(nrows, E.seg); }

    void set_group_by_column(uint64_t col)
    {
        if (col >= current_columns.size()) throw Error(SDB_ERR_INVALID, "group-by column index out of range");
        group_by_column = current_columns[col];
        group_by_column_index = col;
    }

    void ensure_secondary()
    {
        if (!flags_secondary) flags_secondary = E.mm.alloc<uint8_t>(nrows);
    }

    void swap_flag_buffers()
    {
        if (flags_secondary) std::swap(flags, flags_secondary);
    }

    // models/transient_table.hpp:347-381
    void add_pending_kernels(const std::vector<KernelBundle> &ops)
    {
        if (pending_kernels.empty()) {
            pending_kernels.push_back(ops);
            return;
        }
        auto &last = pending_kernels.back();
        bool can_merge = last.size() == ops.size();
        for (size_t i = 0; i < ops.size() && can_merge; i++)
            if (last[i].on_device != ops[i].on_device || last[i].device_index != ops[i].device_index) can_merge = false;
        if (can_merge) {
            for (size_t i = 0; i < ops.size(); i++)
                for (const auto &k : ops[i].kernels) last[i].add_kernel(k);
        } else {
            pending_kernels.push_back(ops);
        }
    }

    // models/transient_table.hpp:383-506: segment by segment, phases in order.
    void execute_pending_kernels()
    {
        if (pending_kernels.empty()) return;
        const size_t nseg = segs().size();
        for (const auto &ph : pending_kernels)
            if (ph.size() != nseg) throw Error(SDB_ERR_INVALID, "Pending kernels segment number mismatch.");
        for (size_t s = 0; s < nseg; s++) {
            std::vector<const KernelData *> ks;
            for (const auto &ph : pending_kernels)
                for (const auto &k : ph[s].kernels) ks.push_back(&k);
            E.run_kernels(ks);
        }
        pending_kernels.clear();
    }

    Column &new_materialized(uint64_t n)
    {
        Column &c = materialized_columns.emplace_back();
        for (auto [start, cnt] : split_rows(n, E.seg)) {
            Segment s;
            s.data = E.mm.alloc<int32_t>(cnt);
            s.nrows = cnt;
            c.segments.push_back(s);
        }
        return c;
    }

    Column *col_at(int64_t idx, const char *what)
    {
        if (idx < 0 || (uint64_t)idx >= current_columns.size() || current_columns[idx] == nullptr)
            throw Error(SDB_ERR_INVALID, std::string(what) + ": column index " + std::to_string(idx) + " is not available");
        Column *c = current_columns[idx];
        if (c->segments.size() != segs().size())
            throw Error(SDB_ERR_INVALID, std::string(what) + ": column " + std::to_string(idx) + " is not loaded");
        return c;
    }

    // models/transient_table.hpp:750-981
    void apply_filter(const ExprType &expr, const std::string &parent_op)
    {
        if (expr.exprType != EXPR) return;  // the reference logs and returns
        std::vector<KernelBundle> ops;
        if (expr.op == "SEARCH") {
            if (expr.operands.size() < 2) throw Error(SDB_ERR_INVALID, "SEARCH needs a column and a range set");
            Column *col = col_at(expr.operands[0].input, "SEARCH");
            const auto &rs = expr.operands[1].literal.rangeSet;
            ensure_secondary();
            const int logic = get_logical_op(parent_op);
            int32_t lo, hi;
            bool range = rs.size() == 1;
            // Segment::search_operator: models/models.hpp:604-718
            if (range) {
                if (rs[0].size() < 3) throw Error(SDB_ERR_INVALID, "SEARCH range needs [kind, lower, upper]");
                lo = stoi_ref(rs[0][1]);
                hi = stoi_ref(rs[0][2]);
            } else {
                if (rs.size() < 2 || rs[0].size() < 2 || rs[1].size() < 2)
                    throw Error(SDB_ERR_INVALID, "SEARCH needs one range or two points");
                lo = stoi_ref(rs[0][1]);
                hi = stoi_ref(rs[1][1]);
            }
            auto sg = segs();
            for (size_t s = 0; s < sg.size(); s++) {
                const uint64_t off = sg[s].first, cnt = sg[s].second;
                uint8_t *local = E.mm.alloc<uint8_t>(cnt);
                KernelBundle bundle;
                KernelData k1;
                k1.type = KernelType::SelectionKernelLiteral;
                k1.n = cnt;
                k1.a = col->segments[s].data;
                k1.in = local;
                k1.out = local;
                k1.cmp = range ? SDB_GE : SDB_EQ;
                k1.logic = SDB_NONE;
                k1.lb = lo;
                KernelData k2 = k1;
                k2.cmp = range ? SDB_LE : SDB_EQ;
                k2.logic = range ? SDB_AND : SDB_OR;
                k2.lb = hi;
                KernelData k3;
                k3.type = KernelType::LogicalKernel;
                k3.n = cnt;
                k3.logic = logic;
                k3.in = flags + off;
                k3.local = local;
                k3.out = flags_secondary + off;
                bundle.add_kernel(k1);
                bundle.add_kernel(k2);
                bundle.add_kernel(k3);
                ops.push_back(bundle);
            }
            add_pending_kernels(ops);
            swap_flag_buffers();
        } else if (is_filter_logical(expr.op)) {
            bool parent_op_used = false;
            for (const ExprType &operand : expr.operands) {
                apply_filter(operand, parent_op_used ? expr.op : parent_op);
                parent_op_used = true;
            }
        } else {
            if (expr.operands.size() != 2) return;  // the reference logs and returns
            Column *cols[2] = {nullptr, nullptr};
            bool literal = false;
            int32_t literal_value = 0;
            for (int i = 0; i < 2; i++) {
                const ExprType &o = expr.operands[i];
                if (o.exprType == COLUMN) {
                    cols[i] = col_at(o.input, "filter");
                } else if (o.exprType == LITERAL) {
                    literal = true;
                    literal_value = (int32_t)o.literal.value;
                } else {
                    return;  // the reference logs and returns
                }
            }
            if (!cols[0])
                throw Error(SDB_ERR_UNSUPPORTED, "filter comparison needs a column as its first operand");
            ensure_secondary();
            const int cmp = get_comp_op(expr.op), logic = get_logical_op(parent_op);
            auto sg = segs();
            for (size_t s = 0; s < sg.size(); s++) {
                const uint64_t off = sg[s].first, cnt = sg[s].second;
                KernelBundle bundle;
                KernelData k;
                k.type = literal ? KernelType::SelectionKernelLiteral : KernelType::SelectionKernelColumns;
                k.n = cnt;
                k.cmp = cmp;
                k.logic = logic;
                k.a = cols[0]->segments[s].data;
                if (literal)
                    k.lb = literal_value;
                else
                    k.b = cols[1]->segments[s].data;
                k.in = flags + off;
                k.out = flags_secondary + off;
                bundle.add_kernel(k);
                ops.push_back(bundle);
            }
            add_pending_kernels(ops);
            swap_flag_buffers();
        }
    }

    // models/transient_table.hpp:983-1224
    void apply_project(const std::vector<ExprType> &exprs)
    {
        std::vector<Column *> new_columns;
        for (size_t i = 0; i < exprs.size(); i++) {
            const ExprType &expr = exprs[i];
            if (expr.exprType == COLUMN) {
                if (expr.input < 0 || (uint64_t)expr.input >= current_columns.size())
                    throw Error(SDB_ERR_INVALID, "project: column index out of range");
                new_columns.push_back(current_columns[expr.input]);
                if ((uint64_t)expr.input == group_by_column_index) group_by_column_index = i;
            } else if (expr.exprType == LITERAL) {
                const int32_t v = (int32_t)expr.literal.value;
                Column &nc = new_materialized(nrows);
                std::vector<KernelBundle> ops;
                for (auto &s : nc.segments) {  // Segment::fill_with_literal: models/models.hpp:293-326
                    s.min = s.max = v;
                    KernelBundle b;
                    KernelData k;
                    k.type = KernelType::FillKernel;
                    k.n = s.nrows;
                    k.res = s.data;
                    k.la = v;
                    b.add_kernel(k);
                    ops.push_back(b);
                }
                add_pending_kernels(ops);
                new_columns.push_back(&nc);
            } else {
                if (expr.operands.size() != 2) return;  // the reference logs and returns
                const int bop = get_op_from_string(expr.op);
                const ExprType &x = expr.operands[0], &y = expr.operands[1];
                Column *ca = nullptr, *cb = nullptr;
                KernelType kt;
                if (x.exprType == COLUMN && y.exprType == COLUMN) {
                    ca = col_at(x.input, "project");
                    cb = col_at(y.input, "project");
                    kt = KernelType::PerformOperationKernelColumns;
                } else if (x.exprType == LITERAL && y.exprType == COLUMN) {
                    cb = col_at(y.input, "project");
                    kt = KernelType::PerformOperationKernelLiteralFirst;
                } else if (x.exprType == COLUMN && y.exprType == LITERAL) {
                    ca = col_at(x.input, "project");
                    kt = KernelType::PerformOperationKernelLiteralSecond;
                } else {
                    return;  // the reference logs and returns
                }
                Column &nc = new_materialized(nrows);
                std::vector<KernelBundle> ops;
                auto sg = segs();
                for (size_t s = 0; s < sg.size(); s++) {
                    Segment &r = nc.segments[s];
                    // Segment::perform_operator: models/models.hpp:760-845 (min/max of the operands' stats)
                    if (kt == KernelType::PerformOperationKernelColumns) {
                        r.min = std::min(ca->segments[s].min, cb->segments[s].min);
                        r.max = std::max(ca->segments[s].max, cb->segments[s].max);
                    } else if (kt == KernelType::PerformOperationKernelLiteralSecond) {
                        r.min = ca->segments[s].min;
                        r.max = ca->segments[s].max;
                    } else {
                        r.min = cb->segments[s].min;
                        r.max = cb->segments[s].max;
                    }
                    KernelBundle b;
                    KernelData k;
                    k.type = kt;
                    k.n = sg[s].second;
                    k.res = r.data;
                    k.bin = bop;
                    k.a = ca ? ca->segments[s].data : nullptr;
                    k.b = cb ? cb->segments[s].data : nullptr;
                    k.la = (int32_t)x.literal.value;
                    k.lb = (int32_t)y.literal.value;
                    k.in = flags + sg[s].first;
                    b.add_kernel(k);
                    ops.push_back(b);
                }
                add_pending_kernels(ops);
                new_columns.push_back(&nc);
            }
        }
        current_columns = new_columns;
    }

    // models/transient_table.hpp:1226-1647
    void apply_aggregate(const AggType &agg, const std::vector<int64_t> &group)
    {
        if (agg.operands.empty()) throw Error(SDB_ERR_UNSUPPORTED, "aggregate without an operand (COUNT(*) is not supported)");
        Column *acol = col_at(agg.operands[0], "aggregate");
        if (acol->is_aggregate_result) throw Error(SDB_ERR_UNSUPPORTED, "aggregate over an aggregate result");
        auto sg = segs();
        std::vector<KernelBundle> bundles;
        if (group.empty()) {
            uint64_t *final_result = E.mm.alloc_zero<uint64_t>(1);
            for (size_t s = 0; s < sg.size(); s++) {
                KernelBundle b;
                KernelData k;
                k.type = KernelType::AggregateOperationKernel;
                k.n = sg[s].second;
                k.a = acol->segments[s].data;
                k.in = flags + sg[s].first;
                k.agg_res = final_result;
                b.add_kernel(k);
                bundles.push_back(b);
            }
            add_pending_kernels(bundles);
            execute_pending_kernels();
            nrows = 1;
            flags = E.mm.alloc<uint8_t>(1);
            uint8_t *f = flags;
            E.dev("fill_flags", [f](cudaStream_t s) { return sdb_fill_u8(f, 1, 1, (sdb_stream_t)s); });
            flags_secondary = nullptr;
            Column &rc = materialized_columns.emplace_back();
            rc.is_aggregate_result = true;
            Segment s;
            s.agg = final_result;
            s.nrows = 1;
            rc.segments.push_back(s);
            current_columns.clear();
            current_columns.push_back(&rc);
            return;
        }
        std::vector<Column *> gcols;
        std::vector<int32_t> mins, maxs;
        uint64_t P = 1;
        for (int64_t gi : group) {
            Column *c = col_at(gi, "group-by");
            auto mm = c->get_min_max();
            mins.push_back(mm.first);
            maxs.push_back(mm.second);
            P *= (uint64_t)(int64_t)(int32_t)((uint32_t)mm.second - (uint32_t)mm.first + 1u);
            gcols.push_back(c);
        }
        if (P == 0 || P > (1ull << 31)) throw Error(SDB_ERR_NOMEM, "group-by slot array too large: " + std::to_string(P));
        uint64_t *aggregate_result = E.mm.alloc_zero<uint64_t>(P);
        uint32_t *temp_flags = E.mm.alloc_zero<uint32_t>(P);
        std::vector<int32_t *> results;
        for (size_t i = 0; i < group.size(); i++) results.push_back(E.mm.alloc<int32_t>(P));
        for (size_t s = 0; s < sg.size(); s++) {
            KernelBundle b;
            KernelData k;
            k.type = KernelType::GroupByAggregateKernel;
            k.n = sg[s].second;
            k.a = acol->segments[s].data;
            k.in = flags + sg[s].first;
            for (Column *c : gcols) k.keys.push_back(c->segments[s].data);
            k.mins = mins;
            k.maxs = maxs;
            k.out_keys = results;
            k.P = P;
            k.agg_res = aggregate_result;
            k.occ = temp_flags;
            b.add_kernel(k);
            bundles.push_back(b);
        }
        add_pending_kernels(bundles);
        execute_pending_kernels();
        uint8_t *new_flags = E.mm.alloc<uint8_t>(P);
        for (auto [start, cnt] : split_rows(P, E.seg))  // K9, deferred to the first reader
            E.from_occ[new_flags + start] = {temp_flags + start, cnt};
        flags = new_flags;
        flags_secondary = nullptr;
        nrows = P;
        current_columns.clear();
        auto out_segs = split_rows(P, E.seg);
        for (size_t i = 0; i < group.size(); i++) {
            Column &c = materialized_columns.emplace_back();
            for (auto [start, cnt] : out_segs) {
                Segment s;
                s.data = results[i] + start;
                s.nrows = cnt;
                c.segments.push_back(s);
            }
            current_columns.push_back(&c);
        }
        Column &ac = materialized_columns.emplace_back();
        ac.is_aggregate_result = true;
        for (auto [start, cnt] : out_segs) {
            Segment s;
            s.agg = aggregate_result + start;
            s.nrows = cnt;
            ac.segments.push_back(s);
        }
        current_columns.push_back(&ac);
    }

    // models/transient_table.hpp:1649-1927
    void apply_join(TransientTable &right, const RelNode &rel)
    {
        if (rel.condition.operands.size() < 2) throw Error(SDB_ERR_INVALID, "join condition needs two operands");
        const int64_t left_column = rel.condition.operands[0].input;
        const int64_t right_column = rel.condition.operands[1].input - (int64_t)current_columns.size();
        if (left_column < 0 || (uint64_t)left_column >= current_columns.size() || right_column < 0 ||
            (uint64_t)right_column >= right.current_columns.size())
            throw Error(SDB_ERR_INVALID, "Invalid column indices in join condition.");
        Column *probe = col_at(left_column, "join probe");
        Column *build = right.col_at(right_column, "join build");
        auto mm = build->get_min_max();
        const int32_t mn = mm.first, mx = mm.second;
        const int32_t len = (int32_t)((uint32_t)mx - (uint32_t)mn + 1u);
        if (len <= 0) throw Error(SDB_ERR_NOMEM, "join key range too large");
        auto lsg = segs();
        auto rsg = right.segs();
        // table layout: the reference's direct-address table over [mn, mx], or
        // open addressing (2^lg slots, at least twice the build rows) for a
        // sparse key range; the probes see the same hits and values
        int lg = 0;
        if (E.cfg.join_tables != 1 && right.nrows <= (1ull << 30)) {
            const int cand = sdb_oa_log2_slots(std::max<uint64_t>(right.nrows, 1));
            const bool sparse = (uint64_t)len >= (1ull << 20) && (uint64_t)len >= 8 * (1ull << cand);
            if (cand > 0 && (E.cfg.join_tables == 2 || sparse)) lg = cand;
        }
        if (rel.joinType == "semi") {
            // Column::build_keys_hash_table: models/models.hpp:1413-1452
            void *ht = lg ? (void *)E.mm.alloc_zero<uint32_t>(1ull << lg) : (void *)E.mm.alloc_zero<uint8_t>((uint64_t)len);
            std::vector<KernelBundle> hb;
            for (size_t s = 0; s < rsg.size(); s++) {
                KernelBundle b;
                KernelData k;
                k.type = KernelType::BuildKeysHTKernel;
                k.n = rsg[s].second;
                k.a = build->segments[s].data;
                k.in = right.flags + rsg[s].first;
                k.ht = ht;
                k.ht_min = mn;
                k.ht_len = len;
                k.ht_log2 = lg;
                k.ht_fresh = s == 0;  // alloc_zero; later segments keep the reference's segment order
                b.add_kernel(k);
                hb.push_back(b);
            }
            right.add_pending_kernels(hb);
            right.execute_pending_kernels();
            ensure_secondary();
            std::vector<KernelBundle> ops;  // Column::semi_join: models/models.hpp:1454-1507
            for (size_t s = 0; s < lsg.size(); s++) {
                KernelBundle b;
                KernelData k;
                k.type = KernelType::FilterJoinKernel;
                k.n = lsg[s].second;
                k.a = probe->segments[s].data;
                k.in = flags + lsg[s].first;
                k.out = flags_secondary + lsg[s].first;
                k.ht = ht;
                k.ht_min = mn;
                k.ht_max = mx;
                k.ht_log2 = lg;
                b.add_kernel(k);
                ops.push_back(b);
            }
            add_pending_kernels(ops);
            swap_flag_buffers();
            for (size_t i = 0; i < right.current_columns.size(); i++) current_columns.push_back(nullptr);
        } else {
            Column *gb = right.group_by_column;
            if (!gb) throw Error(SDB_ERR_UNSUPPORTED, "inner join needs a group-by column on the build side");
            if (gb->segments.size() != rsg.size()) throw Error(SDB_ERR_INVALID, "build-side group-by column is not loaded");
            auto gmm = gb->get_min_max();
            Column &nc = new_materialized(nrows);
            const uint64_t gidx = current_columns.size() + right.group_by_column_index;
            for (size_t i = 0; i < right.current_columns.size(); i++) current_columns.push_back(nullptr);
            current_columns[gidx] = &nc;
            // Column::build_key_vals_hash_table: models/models.hpp:1509-1548
            int32_t *ht = E.mm.alloc_zero<int32_t>(2 * (lg ? (1ull << lg) : (uint64_t)len));
            std::vector<KernelBundle> hb;
            for (size_t s = 0; s < rsg.size(); s++) {
                KernelBundle b;
                KernelData k;
                k.type = KernelType::BuildKeyValsHTKernel;
                k.n = rsg[s].second;
                k.a = build->segments[s].data;
                k.b = gb->segments[s].data;
                k.in = right.flags + rsg[s].first;
                k.ht = ht;
                k.ht_min = mn;
                k.ht_len = len;
                k.ht_log2 = lg;
                k.ht_fresh = s == 0;  // alloc_zero; later segments keep the reference's segment order
                b.add_kernel(k);
                hb.push_back(b);
            }
            right.add_pending_kernels(hb);
            right.execute_pending_kernels();
            ensure_secondary();
            std::vector<KernelBundle> ops;  // Column::full_join_operation: models/models.hpp:1550-1648
            for (size_t s = 0; s < lsg.size(); s++) {
                KernelBundle b;
                KernelData k;
                k.type = KernelType::FullJoinKernel;
                k.n = lsg[s].second;
                k.a = probe->segments[s].data;
                k.res = nc.segments[s].data;
                k.in = flags + lsg[s].first;
                k.out = flags_secondary + lsg[s].first;
                k.ht = ht;
                k.ht_min = mn;
                k.ht_max = mx;
                k.ht_log2 = lg;
                nc.segments[s].min = gmm.first;
                nc.segments[s].max = gmm.second;
                b.add_kernel(k);
                ops.push_back(b);
            }
            add_pending_kernels(ops);
            swap_flag_buffers();
        }
    }
};

// ------------------------------------------------------------------ execution info
void parse_expression_columns(const ExprType &e, std::set<int64_t> &cols)
{
    if (e.exprType == COLUMN)
        cols.insert(e.input);
    else if (e.exprType == EXPR)
        for (const auto &o : e.operands) parse_expression_columns(o, cols);
}

// operations/preprocessing.cpp:14-102
std::vector<int> dag_topological_sort(const PlanResult &p)
{
    const size_t n = p.rels.size();
    std::vector<std::vector<char>> dag(n, std::vector<char>(n, 0));
    std::deque<int> S;
    for (const RelNode &r : p.rels) {
        switch (r.relOp) {
        case TABLE_SCAN: S.push_front((int)r.id); break;
        case FILTER:
        case PROJECT:
        case AGGREGATE:
        case SORT:
            if (r.id < 1) return {};
            dag[r.id - 1][r.id] = 1;
            break;
        case JOIN:
            if (r.inputs.size() != 2) return {};
            for (auto in : r.inputs)
                if (in < 0 || (size_t)in >= n) return {};
            dag[r.inputs[0]][r.id] = 1;
            dag[r.inputs[1]][r.id] = 1;
            break;
        default: return {};
        }
    }
    std::vector<int> sorted;
    while (!S.empty()) {
        int node = S.back();
        S.pop_back();
        if (!S.empty() && p.rels[node].relOp == TABLE_SCAN && p.rels[node].tables.size() > 1 &&
            base_name(p.rels[node].tables[1]) == "lineorder") {
            S.push_front(node);
            continue;
        }
        sorted.push_back(node);
        for (size_t i = 0; i < n; i++) {
            if (dag[node][i] == 1) {
                dag[node][i] = 0;
                bool inbound = false;
                for (size_t j = 0; j < n && !inbound; j++) inbound = dag[j][i] == 1;
                if (!inbound) S.push_front((int)i);
            }
        }
    }
    if (sorted.size() != n) return {};
    return sorted;
}

struct ExecutionInfo {
    std::map<std::string, std::set<int>> loaded_columns;
    std::map<std::string, int> group_by_columns;
    std::vector<int> dag_order;
};

// operations/preprocessing.cpp:104-275
ExecutionInfo parse_execution_info(const PlanResult &p)
{
    ExecutionInfo info;
    std::vector<std::vector<std::pair<std::string, int>>> ops_info;
    auto at = [](const std::vector<std::pair<std::string, int>> &v, int64_t i) -> const std::pair<std::string, int> & {
        if (i < 0 || (size_t)i >= v.size()) throw Error(SDB_ERR_INVALID, "plan: column index " + std::to_string(i) + " out of range");
        return v[i];
    };
    for (const RelNode &r : p.rels) {
        switch (r.relOp) {
        case TABLE_SCAN: {
            if (r.tables.size() < 2) throw Error(SDB_ERR_INVALID, "TABLE_SCAN needs tables [schema, name]");
            auto it = table_column_numbers().find(base_name(r.tables[1]));
            if (it == table_column_numbers().end()) throw Error(SDB_ERR_INVALID, "unknown table " + r.tables[1]);
            std::vector<std::pair<std::string, int>> t;
            for (int i = 0; i < it->second; i++) t.emplace_back(r.tables[1], i);
            ops_info.push_back(t);
            info.loaded_columns[r.tables[1]];
            break;
        }
        case FILTER: {
            if (ops_info.empty()) throw Error(SDB_ERR_INVALID, "FILTER without input");
            auto oi = ops_info.back();
            std::set<int64_t> cols;
            parse_expression_columns(r.condition, cols);
            for (auto c : cols) info.loaded_columns[at(oi, c).first].insert(at(oi, c).second);
            ops_info.push_back(oi);
            break;
        }
        case PROJECT: {
            if (ops_info.empty()) throw Error(SDB_ERR_INVALID, "PROJECT without input");
            auto last = ops_info.back();
            std::vector<std::pair<std::string, int>> oi;
            for (const auto &e : r.exprs) {
                std::set<int64_t> cols;
                parse_expression_columns(e, cols);
                for (auto c : cols) info.loaded_columns[at(last, c).first].insert(at(last, c).second);
                if (!cols.empty()) oi.push_back(at(last, *cols.begin()));
            }
            ops_info.push_back(oi);
            break;
        }
        case AGGREGATE: {
            if (ops_info.empty()) throw Error(SDB_ERR_INVALID, "AGGREGATE without input");
            auto last = ops_info.back();
            std::vector<std::pair<std::string, int>> oi;
            for (auto g : r.group) {
                const auto &tc = at(last, g);
                info.loaded_columns[tc.first].insert(tc.second);
                oi.push_back(tc);
                info.group_by_columns[tc.first] = tc.second;
            }
            for (const auto &a : r.aggs) {
                for (auto c : a.operands) info.loaded_columns[at(last, c).first].insert(at(last, c).second);
                if (!a.operands.empty()) oi.push_back(at(last, a.operands[0]));
            }
            ops_info.push_back(oi);
            break;
        }
        case JOIN: {
            if (r.inputs.size() != 2) throw Error(SDB_ERR_INVALID, "JOIN needs two inputs");
            for (auto in : r.inputs)
                if (in < 0 || (size_t)in >= ops_info.size()) throw Error(SDB_ERR_INVALID, "JOIN input out of range");
            const auto &left = ops_info[r.inputs[0]];
            const auto &right = ops_info[r.inputs[1]];
            std::set<int64_t> cols;
            parse_expression_columns(r.condition, cols);
            for (auto c : cols) {
                const auto &tc = (size_t)c < left.size() ? at(left, c) : at(right, c - (int64_t)left.size());
                info.loaded_columns[tc.first].insert(tc.second);
            }
            auto oi = left;
            oi.insert(oi.end(), right.begin(), right.end());
            ops_info.push_back(oi);
            break;
        }
        case SORT: {
            if (ops_info.empty()) throw Error(SDB_ERR_INVALID, "SORT without input");
            auto oi = ops_info.back();
            for (const auto &c : r.collation)
                if (c.field >= 0 && (size_t)c.field < oi.size()) info.loaded_columns[oi[c.field].first].insert(oi[c.field].second);
            ops_info.push_back(oi);
            break;
        }
        default:
            throw Error(SDB_ERR_UNSUPPORTED, "Unsupported RelNodeType " + std::to_string(r.relOp));
        }
    }
    info.dag_order = dag_topological_sort(p);
    if (info.dag_order.empty()) throw Error(SDB_ERR_INVALID, "DAG topological sort failed");
    return info;
}

// A plan's result after its last kernel, before it reaches the host: per
// segment of the final table the device count of qualifying rows and the
// gathered columns (capacity `cap` rows each).
struct PendingSeg {
    uint32_t *count;
    std::vector<void *> dev;
    uint64_t cap;
};

struct PendingResult {
    std::vector<int> types;  // 0 int32, 1 uint64
    std::vector<PendingSeg> segs;
    std::vector<std::pair<int, int>> order;  // ORDER BY: (result column, descending), first key first
};

}  // namespace sdb

// ====================================================================== results
struct sdb_result {
    std::vector<int> types;  // 0 int32, 1 uint64
    std::vector<std::vector<int32_t>> i32;
    std::vector<std::vector<uint64_t>> u64;
    uint64_t nrows = 0;
};

struct sdb_engine {
    sdb::Engine E;
    // Prepared plans (sdb_engine_config.plan_cache): plan text -> times seen,
    // last use, and the one-plan batch replayed for it once prepared.
    struct Cached {
        uint64_t uses = 0, last = 0;
        sdb_batch *batch = nullptr;
    };
    std::map<std::string, Cached> cache;
    uint64_t tick = 0;
};

// A prepared batch: every plan's device work recorded once against the
// batch's own arena, replayed per run (as one CUDA graph unless eager).
struct sdb_batch {
    sdb_engine *eng = nullptr;
    int flags = 0;
    sdb::MemoryManager mm;
    sdb::Recorder rec;
    std::vector<sdb::PendingResult> pend;
    sdb_chain_batch *cb = nullptr;
    char *host = nullptr;  // pinned staging of counts and result columns
    size_t host_bytes = 0;
    struct Stage {
        size_t count_off;
        std::vector<size_t> col_off;
    };
    std::vector<std::vector<Stage>> stage;  // [plan][segment]
    sdb::MemoryManager rmm;  // result region: counts and result columns of every plan
    char *rbase = nullptr;   // its base; B.host mirrors it byte for byte
    size_t rbytes = 0;
    cudaStream_t bs = nullptr;              // the stream the graph is captured on
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr, ev_a = nullptr, ev_b = nullptr;
    // around the chain batch: before its builds, after them, before the
    // aggregating chains (after the plans' mid work), after them
    cudaEvent_t ev_c0 = nullptr, ev_cb = nullptr, ev_cm = nullptr, ev_c1 = nullptr;
    double last_chain_ms = 0, last_pre_ms = 0, last_post_ms = 0, last_build_ms = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
    int chain_groups = 0;
    int paired = 0;  // fact chains run in paired passes (two per pass)
    double last_ms = 0;
    // false: streams, events, staging and arena belong to the caller (a
    // server slot), the batch runs once
    bool owns = true;
    // false: no timing events around the chain batch (a prepared plan: one
    // plan, where the event nodes would cost more than they tell)
    bool timed = true;

    ~sdb_batch()
    {
        if (cb) sdb_chain_batch_destroy(cb);
        if (!owns) return;
        if (bs) cudaStreamSynchronize(bs);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto s : side) cudaStreamDestroy(s);
        for (auto e : join) cudaEventDestroy(e);
        for (auto e : {fork, ev_a, ev_b, ev_c0, ev_cb, ev_cm, ev_c1})
            if (e) cudaEventDestroy(e);
        if (bs) cudaStreamDestroy(bs);
        if (host) cudaFreeHost(host);
    }
};

namespace sdb {

// ------------------------------------------------------------------ table installation
// Replaces (or adds) table `name`: the old table's device buffers are freed
// once the engine's stream is idle.
void install_table(Engine &E, const std::string &name, std::unique_ptr<Table> t)
{
    auto old = E.tables.find(name);
    if (old != E.tables.end()) {
        SDB_CUDA(cudaStreamSynchronize(E.stream));
        for (auto p : old->second->owned) cudaFree(p);
        E.tables.erase(old);
    }
    E.tables[name] = std::move(t);
}

// Waits for a background load of `name`, if one is pending, and installs it
// (Segment::activate_background_buffer, models/models.hpp:541-550, for a
// whole table).
void activate_table(Engine &E, const std::string &name)
{
    auto it = E.pending.find(name);
    if (it == E.pending.end()) return;
    auto fut = std::move(it->second);
    E.pending.erase(it);
    install_table(E, name, fut.get());  // rethrows the loader's error
}

// Reads table `name` from the reference's columnar files -- one file per
// column, dir/<NAME><i> with the table name upper-cased, raw int32 in the
// machine's byte order (Table::Table, models/models.hpp:1659-1708) -- into
// new device buffers, and computes per-segment min/max.  Only the columns of
// `mask` (bit i = column i) are read; the row count is the first read
// column's; a missing file or one of another length leaves that column
// unloaded, as the reference does.  The files are read in 8 MB chunks by
// several threads, each alternating between two pinned buffers so that its
// reads overlap its copies; the chunks go to the device on one stream.
std::unique_ptr<Table> load_columns(const std::string &dir, const std::string &name, int ncols, uint64_t mask,
                                    uint64_t seg_rows, cudaStream_t s, std::vector<std::string> *warnings)
{
    constexpr size_t kChunk = 8u << 20;
    std::string upper = base_name(name);
    std::transform(upper.begin(), upper.end(), upper.begin(), [](unsigned char ch) { return (char)std::toupper(ch); });
    std::string prefix = dir;
    if (!prefix.empty() && prefix.back() != '/') prefix += '/';
    auto t = std::make_unique<Table>();
    t->name = name;
    t->columns.resize(ncols);
    bool nrows_set = false;
    int device = 0;
    SDB_CUDA(cudaGetDevice(&device));
    struct Job {
        int fd;
        uint64_t off;
        size_t len;
        char *dst;
    };
    std::vector<int> fds;
    std::vector<Job> jobs;
    auto close_fds = [&]() {
        for (int fd : fds) close(fd);
        fds.clear();
    };
    std::vector<std::pair<int, int32_t *>> dev_cols;
    try {
        for (int c = 0; c < ncols && c < 64; c++) {
            if (!((mask >> c) & 1u)) continue;
            const std::string file = prefix + upper + std::to_string(c);
            const int fd = open(file.c_str(), O_RDONLY);
            if (fd < 0) {
                if (warnings) warnings->push_back("column file missing: " + file);
                continue;
            }
            struct stat stt;
            if (fstat(fd, &stt) != 0) {
                close(fd);
                throw Error(SDB_ERR_INVALID, "cannot stat " + file);
            }
            const uint64_t bytes = (uint64_t)stt.st_size;
            const uint64_t n = bytes / sizeof(int32_t);
            if (!nrows_set) {
                if (n == 0) {
                    close(fd);
                    throw Error(SDB_ERR_INVALID, "empty column file " + file);
                }
                t->nrows = n;
                nrows_set = true;
            }
            if (n != t->nrows || bytes % sizeof(int32_t)) {
                close(fd);
                if (warnings)
                    warnings->push_back("column length mismatch in " + file + ": expected " + std::to_string(t->nrows) +
                                        ", got " + std::to_string(n));
                continue;
            }
            fds.push_back(fd);
            int32_t *d = nullptr;
            SDB_CUDA(cudaMalloc(&d, bytes));
            t->owned.push_back(d);
            for (uint64_t off = 0; off < bytes; off += kChunk)
                jobs.push_back({fd, off, (size_t)std::min<uint64_t>(kChunk, bytes - off), reinterpret_cast<char *>(d) + off});
            dev_cols.emplace_back(c, d);
        }
        if (!nrows_set) throw Error(SDB_ERR_INVALID, "no column file of table " + name + " under " + dir);
        // readers: each takes the next chunk, reads it into one of its two
        // pinned buffers (once that buffer's previous copy is done) and
        // queues the copy
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const size_t nthreads = std::max<size_t>(1, std::min<size_t>({(size_t)4, (size_t)hw, jobs.size()}));
        std::atomic<size_t> next{0};
        std::mutex err_mu;
        std::string err;
        auto reader = [&]() {
            char *pin[2] = {nullptr, nullptr};
            cudaEvent_t done[2] = {nullptr, nullptr};
            auto fail = [&](const std::string &m) {
                std::lock_guard<std::mutex> g(err_mu);
                if (err.empty()) err = m;
            };
            bool ok = cudaSetDevice(device) == cudaSuccess;
            for (int b = 0; b < 2 && ok; b++)
                ok = cudaHostAlloc(reinterpret_cast<void **>(&pin[b]), kChunk, cudaHostAllocDefault) == cudaSuccess &&
                     cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming) == cudaSuccess;
            if (!ok) fail("load_dir: pinned staging or event");
            int b = 0;
            for (size_t j = next++; ok && j < jobs.size(); j = next++) {
                {
                    std::lock_guard<std::mutex> g(err_mu);
                    if (!err.empty()) break;
                }
                const Job &jb = jobs[j];
                if (cudaEventSynchronize(done[b]) != cudaSuccess) {  // the buffer's previous copy is done
                    fail("load_dir: copy failed");
                    break;
                }
                size_t got = 0;
                while (got < jb.len) {
                    const ssize_t r = pread(jb.fd, pin[b] + got, jb.len - got, (off_t)(jb.off + got));
                    if (r <= 0) break;
                    got += (size_t)r;
                }
                if (got != jb.len) {
                    fail("load_dir: read failed");
                    break;
                }
                if (cudaMemcpyAsync(jb.dst, pin[b], jb.len, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                    cudaEventRecord(done[b], s) != cudaSuccess) {
                    fail("load_dir: copy failed");
                    break;
                }
                b ^= 1;
            }
            for (int q = 0; q < 2; q++) {
                if (done[q]) cudaEventSynchronize(done[q]), cudaEventDestroy(done[q]);
                if (pin[q]) cudaFreeHost(pin[q]);
            }
        };
        std::vector<std::thread> pool;
        for (size_t i = 1; i < nthreads; i++) pool.emplace_back(reader);
        reader();
        for (auto &th : pool) th.join();
        close_fds();
        if (!err.empty()) throw Error(SDB_ERR_INVALID, err);
        // Segment statistics (models/models.hpp:71-77), on the device.
        auto sg = split_rows(t->nrows, seg_rows);
        const size_t nmm = dev_cols.size() * sg.size() * 2;
        int32_t *mm = nullptr;
        SDB_CUDA(cudaMalloc(&mm, std::max<size_t>(nmm, 2) * sizeof(int32_t)));
        size_t q = 0;
        int st = SDB_OK;
        for (auto &dc : dev_cols)
            for (auto [start, cnt] : sg)
                if (st == SDB_OK) st = sdb_min_max_i32(dc.second + start, cnt, mm + 2 * (q++), (sdb_stream_t)s);
        std::vector<int32_t> host(nmm);
        cudaError_t e1 = st == SDB_OK ? cudaMemcpyAsync(host.data(), mm, nmm * sizeof(int32_t), cudaMemcpyDeviceToHost, s)
                                      : cudaSuccess;
        cudaError_t e2 = cudaStreamSynchronize(s);
        cudaFree(mm);
        check(st);
        if (e1 != cudaSuccess || e2 != cudaSuccess)
            throw Error(SDB_ERR_CUDA, std::string("load_dir: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
        q = 0;
        for (auto &dc : dev_cols) {
            Column &col = t->columns[dc.first];
            for (auto [start, cnt] : sg) {
                Segment sgm;
                sgm.data = dc.second + start;
                sgm.nrows = cnt;
                sgm.min = host[2 * q];
                sgm.max = host[2 * q + 1];
                col.segments.push_back(sgm);
                q++;
            }
        }
    } catch (...) {
        close_fds();
        cudaStreamSynchronize(s);
        for (auto p : t->owned) cudaFree(p);
        throw;
    }
    return t;
}

// execute_ddor_plan (executor/ddor_executor.cpp:22-245) up to the result
// materialisation of save_result (executor/result_writer.cpp:12-68): every
// device operation goes through Engine::dev.  The caller resets the arena.
PendingResult run_plan(Engine &E, const std::string &plan_text)
{
    PlanResult plan = plan_from_json(plan_text);
    ExecutionInfo info = parse_execution_info(plan);
    E.all_true.clear();
    E.unfilled.clear();
    E.from_occ.clear();

    std::deque<TransientTable> tts;
    std::vector<int> output_table(plan.rels.size(), -1);
    for (const RelNode &rel : plan.rels)
        if (rel.relOp == TABLE_SCAN) activate_table(E, rel.tables[1]);
    for (const RelNode &rel : plan.rels) {
        if (rel.relOp != TABLE_SCAN) continue;
        const std::string &name = rel.tables[1];
        auto it = E.tables.find(name);
        if (it == E.tables.end()) throw Error(SDB_ERR_INVALID, "Table " + name + " not found among loaded tables.");
        for (int c : info.loaded_columns[name])
            if ((size_t)c >= it->second->columns.size() || it->second->columns[c].segments.empty())
                throw Error(SDB_ERR_INVALID, "column " + std::to_string(c) + " of table " + name + " is not loaded");
        tts.emplace_back(E, it->second.get());
        auto g = info.group_by_columns.find(name);
        if (g != info.group_by_columns.end()) tts.back().set_group_by_column(g->second);
        output_table[rel.id] = (int)tts.size() - 1;
    }

    for (int id : info.dag_order) {
        const RelNode &rel = plan.rels[id];
        auto prev = [&]() {
            if (id < 1 || output_table[id - 1] < 0) throw Error(SDB_ERR_INVALID, "node has no input table");
            return output_table[id - 1];
        };
        switch (rel.relOp) {
        case TABLE_SCAN: break;
        case FILTER: {
            int t = prev();
            tts[t].apply_filter(rel.condition, "");
            output_table[id] = t;
            break;
        }
        case PROJECT: {
            int t = prev();
            tts[t].apply_project(rel.exprs);
            output_table[id] = t;
            break;
        }
        case AGGREGATE: {
            int t = prev();
            if (rel.aggs.empty()) throw Error(SDB_ERR_INVALID, "AGGREGATE without aggs");
            tts[t].apply_aggregate(rel.aggs[0], rel.group);
            output_table[id] = t;
            break;
        }
        case JOIN: {
            int l = output_table[rel.inputs[0]], r = output_table[rel.inputs[1]];
            if (l < 0 || r < 0) throw Error(SDB_ERR_INVALID, "JOIN input has no table");
            tts[l].apply_join(tts[r], rel);
            output_table[id] = l;
            break;
        }
        case SORT: output_table[id] = prev(); break;
        default: break;
        }
    }

    TransientTable &fin = tts[output_table[plan.rels.size() - 1]];
    fin.execute_pending_kernels();

    // Compact the flagged rows of the non-null columns, in row order.
    PendingResult pr;
    std::vector<Column *> cols;
    for (Column *c : fin.current_columns)
        if (c) {
            if (c->segments.size() != fin.segs().size()) throw Error(SDB_ERR_INVALID, "result column is not loaded");
            cols.push_back(c);
        }
    for (Column *c : cols) pr.types.push_back(c->is_aggregate_result ? 1 : 0);
    // ORDER BY: the collation of the plan's last SORT node, its fields being
    // positions in the final table's columns
    for (auto k = info.dag_order.rbegin(); k != info.dag_order.rend(); ++k) {
        const RelNode &rel = plan.rels[*k];
        if (rel.relOp != SORT || rel.collation.empty()) continue;
        for (const CollationType &c : rel.collation) {
            if (c.field < 0 || (size_t)c.field >= fin.current_columns.size() || !fin.current_columns[c.field])
                throw Error(SDB_ERR_UNSUPPORTED, "ORDER BY field " + std::to_string(c.field) + " is not a result column");
            const Column *col = fin.current_columns[c.field];
            const int pos = (int)(std::find(cols.begin(), cols.end(), col) - cols.begin());
            pr.order.emplace_back(pos, c.direction == 0 ? 1 : 0);
        }
        break;
    }
    auto sg = fin.segs();
    for (size_t s = 0; s < sg.size(); s++) {
        const uint64_t cnt = sg[s].second;
        PendingSeg o;
        o.cap = cnt;
        MemoryManager &R = E.rmm ? *E.rmm : E.mm;
        const uint8_t *fl0 = fin.flags + sg[s].first;
        if (cnt <= 65536 && cols.size() <= 8) {  // small result: compaction and gathers in one launch
            uint32_t *count = R.alloc<uint32_t>(1);
            o.count = count;
            std::vector<const void *> src;
            std::vector<void *> dst;
            std::vector<int> wide;
            for (Column *c : cols) {
                const Segment &seg = c->segments[s];
                if (c->is_aggregate_result) {
                    src.push_back(seg.agg);
                    dst.push_back(R.alloc<uint64_t>(cnt));
                    wide.push_back(1);
                } else {
                    src.push_back(seg.data);
                    dst.push_back(R.alloc<int32_t>(cnt));
                    wide.push_back(0);
                }
            }
            o.dev = dst;
            auto oc = E.from_occ.find(fl0);
            if (oc != E.from_occ.end()) {  // a group-by result: straight from its occupancy words
                const uint32_t *occ = oc->second.first;
                E.dev("compact_gather", [occ, cnt, src, wide, dst, count](cudaStream_t st) {
                    return sdb_compact_gather_occ(occ, cnt, (int)src.size(), src.data(), wide.data(), dst.data(), count,
                                                  (sdb_stream_t)st);
                });
            } else {
                E.ensure_filled(fl0);
                E.dev("compact_gather", [fl0, cnt, src, wide, dst, count](cudaStream_t st) {
                    return sdb_compact_gather(fl0, cnt, (int)src.size(), src.data(), wide.data(), dst.data(), count,
                                              (sdb_stream_t)st);
                });
            }
            pr.segs.push_back(o);
            continue;
        }
        int32_t *ids = E.mm.alloc<int32_t>(cnt);
        uint32_t *count = R.alloc<uint32_t>(1);
        o.count = count;
        size_t sb = sdb_compact_scratch_bytes(cnt);
        void *scratch = E.mm.alloc<uint8_t>(sb);
        const uint8_t *fl = fin.flags + sg[s].first;
        E.ensure_filled(fl);
        E.dev("compact_row_ids", [fl, cnt, ids, count, scratch, sb](cudaStream_t st) {
            return sdb_compact_row_ids(fl, cnt, ids, count, scratch, sb, (sdb_stream_t)st);
        });
        for (Column *c : cols) {
            const Segment &seg = c->segments[s];
            if (c->is_aggregate_result) {
                uint64_t *d = R.alloc<uint64_t>(cnt);
                const uint64_t *src = seg.agg;
                E.dev("gather", [src, ids, count, d, cnt](cudaStream_t st) {
                    return sdb_gather_u64(src, ids, count, d, cnt, (sdb_stream_t)st);
                });
                o.dev.push_back(d);
            } else {
                int32_t *d = R.alloc<int32_t>(cnt);
                const int32_t *src = seg.data;
                E.dev("gather", [src, ids, count, d, cnt](cudaStream_t st) {
                    return sdb_gather_i32(src, ids, count, d, cnt, (sdb_stream_t)st);
                });
                o.dev.push_back(d);
            }
        }
        pr.segs.push_back(o);
    }
    return pr;
}

// ORDER BY on the device: the result rows of all segments are laid end to
// end, sorted by the collation keys (sdb_sort_rows, stable) and gathered in
// that order; pr then describes one segment of `total` rows.
void sort_result(Engine &E, PendingResult &pr, std::vector<uint32_t> &counts, uint64_t total)
{
    const size_t ncols = pr.types.size();
    cudaStream_t st = E.stream;
    std::vector<void *> flat(ncols);
    for (size_t c = 0; c < ncols; c++) {
        const size_t w = pr.types[c] == 1 ? 8 : 4;
        if (pr.segs.size() == 1) {
            flat[c] = pr.segs[0].dev[c];
            continue;
        }
        char *d = E.mm.alloc<char>(total * w);
        uint64_t at = 0;
        for (size_t s = 0; s < pr.segs.size(); s++) {
            if (counts[s]) SDB_CUDA(cudaMemcpyAsync(d + at * w, pr.segs[s].dev[c], counts[s] * w, cudaMemcpyDeviceToDevice, st));
            at += counts[s];
        }
        flat[c] = d;
    }
    std::vector<const void *> keys;
    std::vector<int> types, desc;
    for (auto &o : pr.order) {
        keys.push_back(flat[o.first]);
        types.push_back(pr.types[o.first]);
        desc.push_back(o.second);
    }
    uint32_t *perm = E.mm.alloc<uint32_t>(total);
    const size_t sb = sdb_sort_scratch_bytes(total);
    void *scratch = E.mm.alloc<uint8_t>(sb);
    E.dev("sort_rows", [&](cudaStream_t s) {
        return sdb_sort_rows(keys.data(), types.data(), desc.data(), (int)keys.size(), total, perm, scratch, sb,
                             (sdb_stream_t)s);
    });
    uint32_t *count = E.mm.alloc<uint32_t>(1);
    const uint32_t t32 = (uint32_t)total;
    SDB_CUDA(cudaMemcpyAsync(count, &t32, sizeof t32, cudaMemcpyHostToDevice, st));
    PendingSeg one;
    one.count = count;
    one.cap = total;
    for (size_t c = 0; c < ncols; c++) {
        if (pr.types[c] == 1) {
            uint64_t *d = E.mm.alloc<uint64_t>(total);
            check(sdb_gather_u64(static_cast<const uint64_t *>(flat[c]), reinterpret_cast<const int32_t *>(perm), count, d,
                                 total, (sdb_stream_t)st));
            one.dev.push_back(d);
        } else {
            int32_t *d = E.mm.alloc<int32_t>(total);
            check(sdb_gather_i32(static_cast<const int32_t *>(flat[c]), reinterpret_cast<const int32_t *>(perm), count, d,
                                 total, (sdb_stream_t)st));
            one.dev.push_back(d);
        }
    }
    SDB_CUDA(cudaStreamSynchronize(st));  // t32 lives on this frame
    pr.segs.assign(1, one);
    counts.assign(1, (uint32_t)total);
}

std::unique_ptr<sdb_result> execute_plan(Engine &E, const std::string &plan_text)
{
    E.mm.reset(E.stream);
    if (E.cfg.profile) E.prof.stats.clear();
    SDB_CUDA(cudaEventRecord(E.plan_a, E.stream));
    PendingResult pr = run_plan(E, plan_text);

    auto res = std::make_unique<sdb_result>();
    res->types = pr.types;
    const size_t ncols = pr.types.size();
    res->i32.resize(ncols);
    res->u64.resize(ncols);
    std::vector<uint32_t> counts(pr.segs.size());
    for (size_t s = 0; s < pr.segs.size(); s++)
        SDB_CUDA(cudaMemcpyAsync(&counts[s], pr.segs[s].count, sizeof(uint32_t), cudaMemcpyDeviceToHost, E.stream));
    SDB_CUDA(cudaStreamSynchronize(E.stream));
    uint64_t total = 0;
    for (auto c : counts) total += c;
    for (size_t ci = 0; ci < ncols; ci++) {
        if (res->types[ci] == 1)
            res->u64[ci].resize(total);
        else
            res->i32[ci].resize(total);
    }
    if (E.cfg.order_by && !pr.order.empty() && total > 1) sort_result(E, pr, counts, total);
    uint64_t base = 0;
    for (size_t s = 0; s < pr.segs.size(); s++) {
        for (size_t ci = 0; ci < ncols; ci++) {
            if (!counts[s]) continue;
            if (res->types[ci] == 1)
                SDB_CUDA(cudaMemcpyAsync(res->u64[ci].data() + base, pr.segs[s].dev[ci], counts[s] * sizeof(uint64_t),
                                         cudaMemcpyDeviceToHost, E.stream));
            else
                SDB_CUDA(cudaMemcpyAsync(res->i32[ci].data() + base, pr.segs[s].dev[ci], counts[s] * sizeof(int32_t),
                                         cudaMemcpyDeviceToHost, E.stream));
        }
        base += counts[s];
    }
    SDB_CUDA(cudaEventRecord(E.plan_b, E.stream));
    SDB_CUDA(cudaStreamSynchronize(E.stream));
    res->nrows = total;
    float ms = 0;
    SDB_CUDA(cudaEventElapsedTime(&ms, E.plan_a, E.plan_b));
    E.last_plan_ms = ms;
    E.prof.collect();
    return res;
}

// Returns true when the table replaced one of the same name whose device
// buffers it reuses column for column and whose per-segment min/max it
// reproduces exactly: plans prepared against the old table then still hold.
bool load_table(Engine &E, const char *name, int ncols, const int32_t *const *cols, uint64_t nrows, int on_device)
{
    if (!name) throw Error(SDB_ERR_INVALID, "table name is NULL");
    activate_table(E, name);  // a background load of the same name finishes first
    auto it = table_column_numbers().find(base_name(name));
    if (it == table_column_numbers().end()) throw Error(SDB_ERR_INVALID, std::string("unknown table ") + name);
    if (ncols != it->second)
        throw Error(SDB_ERR_INVALID, std::string("table ") + name + " has " + std::to_string(it->second) + " columns");
    if (!cols) throw Error(SDB_ERR_INVALID, "cols is NULL");
    if (nrows == 0) throw Error(SDB_ERR_INVALID, "empty table");
    auto old = E.tables.find(name);
    std::vector<int32_t *> reuse;
    // the old table's column layout and statistics, to tell whether it changed
    bool comparable = false;
    std::vector<const int32_t *> old_data(ncols, nullptr);
    std::vector<std::pair<int32_t, int32_t>> old_stats;
    if (old != E.tables.end()) {
        SDB_CUDA(cudaStreamSynchronize(E.stream));
        const Table &o = *old->second;
        comparable = o.nrows == nrows && !on_device && (int)o.columns.size() == ncols;
        if (comparable)
            for (int c = 0; c < ncols; c++)
                if (!o.columns[c].segments.empty()) {
                    old_data[c] = o.columns[c].segments[0].data;
                    for (const Segment &sg : o.columns[c].segments) old_stats.emplace_back(sg.min, sg.max);
                }
        if (o.nrows == nrows) reuse = o.owned;
        else
            for (auto p : o.owned) cudaFree(p);
        E.tables.erase(old);
    }
    auto t = std::make_unique<Table>();
    t->name = name;
    t->nrows = nrows;
    t->columns.resize(ncols);
    auto sg = split_rows(nrows, E.seg);
    std::vector<std::pair<int, int32_t *>> dev_cols;
    size_t reuse_i = 0;
    for (int c = 0; c < ncols; c++) {
        if (!cols[c]) continue;
        int32_t *d;
        if (on_device) {
            d = const_cast<int32_t *>(cols[c]);
        } else {
            if (reuse_i < reuse.size()) {
                d = reuse[reuse_i++];
            } else {
                SDB_CUDA(cudaMalloc(&d, nrows * sizeof(int32_t)));
            }
            t->owned.push_back(d);
        }
        dev_cols.emplace_back(c, d);
    }
    for (; reuse_i < reuse.size(); reuse_i++) cudaFree(reuse[reuse_i]);
    // Segment statistics (models/models.hpp:71-77), computed on the device:
    // a column's min/max run on the engine's second stream while the next
    // column is still being copied on the first.
    const size_t nmm = dev_cols.size() * sg.size() * 2;
    E.stats_reserve(nmm);
    if (!E.aux) SDB_CUDA(cudaStreamCreateWithFlags(&E.aux, cudaStreamNonBlocking));
    size_t q = 0;
    for (auto &dc : dev_cols) {
        if (!on_device)
            SDB_CUDA(cudaMemcpyAsync(dc.second, cols[dc.first], nrows * sizeof(int32_t), cudaMemcpyHostToDevice,
                                     E.stream));
        SDB_CUDA(cudaEventRecord(E.copied, E.stream));
        SDB_CUDA(cudaStreamWaitEvent(E.aux, E.copied, 0));
        for (auto [start, cnt] : sg) {
            check(sdb_min_max_i32(dc.second + start, cnt, E.stats_dev + 2 * q, (sdb_stream_t)E.aux));
            q++;
        }
    }
    if (nmm) SDB_CUDA(cudaMemcpyAsync(E.stats_host, E.stats_dev, nmm * sizeof(int32_t), cudaMemcpyDeviceToHost, E.aux));
    SDB_CUDA(cudaStreamSynchronize(E.aux));
    SDB_CUDA(cudaStreamSynchronize(E.stream));
    q = 0;
    bool same = comparable;
    size_t oq = 0;
    for (int c = 0; c < ncols && same; c++) same = (cols[c] != nullptr) == (old_data[c] != nullptr);
    for (auto &dc : dev_cols) {
        Column &col = t->columns[dc.first];
        if (same && old_data[dc.first] != dc.second) same = false;
        for (auto [start, cnt] : sg) {
            Segment s;
            s.data = dc.second + start;
            s.nrows = cnt;
            s.min = E.stats_host[2 * q];
            s.max = E.stats_host[2 * q + 1];
            if (same && (oq >= old_stats.size() || old_stats[oq] != std::make_pair(s.min, s.max))) same = false;
            oq++;
            col.segments.push_back(s);
            q++;
        }
    }
    E.tables[name] = std::move(t);
    return same && oq == old_stats.size();
}

// ------------------------------------------------------------------ batches
// Records `plans` into B.rec against arena `mm` (swapped into the engine for
// the duration).
void record_plans(Engine &E, sdb_batch &B, MemoryManager &mm, MemoryManager &rmm,
                  const std::vector<std::string> &plans)
{
    struct Swap {  // the engine records into B against mm (results in rmm) until scope exit
        Engine &E;
        MemoryManager &mm;
        Swap(Engine &e, MemoryManager &m, MemoryManager &r, Recorder *rec) : E(e), mm(m)
        {
            E.mm.swap(mm);
            E.rec = rec;
            E.rmm = &r;
        }
        ~Swap()
        {
            E.mm.swap(mm);
            E.rec = nullptr;
            E.rmm = nullptr;
        }
    };
    B.rec = Recorder();
    B.rec.batch_chains = !(B.flags & (SDB_BATCH_NO_CHAIN_BATCH | SDB_BATCH_BUILDS_ONLY));
    B.rec.batch_builds = !(B.flags & SDB_BATCH_NO_CHAIN_BATCH);
    B.pend.clear();
    Swap guard(E, mm, rmm, &B.rec);
    for (const std::string &pt : plans) {
        B.rec.plans.emplace_back();
        B.pend.push_back(run_plan(E, pt));
    }
}

// Shared scans: plans of the batch whose fact chains scan the same rows in
// the same bound pass run those chains two by two, one paired pass each
// (sdb_chain_launch_pair: each tile copied once, both chains evaluated on it),
// on the main stream.  Only a plan's leading chains of a phase move -- none
// of the plan's work in that phase runs before them -- into a paired stage
// right before the phase: the pre phase (plans without batched builds) or
// the mid phase (after the builds).  Never two chains of one plan.  Results
// are those of the chains run apart.
void pair_phase(sdb_batch &B, std::vector<DevOp> PlanRecord::*list, std::vector<DevOp> &out)
{
    struct Cand {
        uint64_t key;
        size_t plan, idx;
        bool used;
    };
    // whether chain c reads a column that one of the plan's earlier leading
    // chains writes (a moved chain runs before those)
    auto reads_any = [](const sdb_chain_desc &c, const std::vector<const int32_t *> &cols) {
        auto hit = [&](const sdb_operand &o) {
            return o.kind == SDB_SRC_COL && std::find(cols.begin(), cols.end(), o.col) != cols.end();
        };
        for (int k = 0; k < c.n_ops; k++)
            if (hit(c.ops[k].a) || hit(c.ops[k].b)) return true;
        if (hit(c.value)) return true;
        for (int k = 0; k < c.n_keys; k++)
            if (hit(c.keys[k])) return true;
        return false;
    };
    std::vector<Cand> cands;
    for (size_t p = 0; p < B.rec.plans.size(); p++) {
        const std::vector<DevOp> &ops = B.rec.plans[p].*list;
        std::vector<const int32_t *> written;
        for (size_t i = 0; i < ops.size() && ops[i].has_chain; i++) {
            const sdb_chain_desc &c = ops[i].chain;
            uint64_t key = 0;
            if (!reads_any(c, written) && sdb_chain_pair_key(&c, &key) == 1) cands.push_back({key, p, i, false});
            for (int k = 0; k < c.n_ops; k++)
                if (c.ops[k].out_col) written.push_back(c.ops[k].out_col);
        }
    }
    // equal keys side by side, in plan order within a key
    std::stable_sort(cands.begin(), cands.end(), [](const Cand &a, const Cand &b) { return a.key < b.key; });
    int paired = 0;
    for (size_t a = 0; a < cands.size(); a++) {
        if (cands[a].used) continue;
        const sdb_chain_desc &x = (B.rec.plans[cands[a].plan].*list)[cands[a].idx].chain;
        for (size_t b = a + 1; b < cands.size() && cands[b].key == cands[a].key; b++) {
            if (cands[b].used || cands[b].plan == cands[a].plan) continue;
            const sdb_chain_desc &y = (B.rec.plans[cands[b].plan].*list)[cands[b].idx].chain;
            if (sdb_chain_pairable(&x, &y) != 1) continue;
            cands[a].used = cands[b].used = true;
            const sdb_chain_desc cx = x, cy = y;
            out.push_back({"paired_chains", [cx, cy](cudaStream_t s) {
                               return sdb_chain_launch_pair(&cx, &cy, (sdb_stream_t)s);
                           }});
            paired += 2;
            break;
        }
    }
    if (!paired) return;
    B.paired += paired;
    std::vector<std::vector<char>> moved(B.rec.plans.size());
    for (const Cand &c : cands)
        if (c.used) {
            auto &m = moved[c.plan];
            if (m.size() <= c.idx) m.resize(c.idx + 1, 0);
            m[c.idx] = 1;
        }
    for (size_t p = 0; p < B.rec.plans.size(); p++) {
        if (moved[p].empty()) continue;
        std::vector<DevOp> keep;
        std::vector<DevOp> &ops = B.rec.plans[p].*list;
        for (size_t i = 0; i < ops.size(); i++)
            if (i >= moved[p].size() || !moved[p][i]) keep.push_back(std::move(ops[i]));
        ops = std::move(keep);
    }
}

void pair_chains(Engine &E, sdb_batch &B)
{
    B.rec.shared_pre.clear();
    B.rec.shared.clear();
    B.paired = 0;
    if (E.cfg.no_shared_scans) return;
    pair_phase(B, &PlanRecord::pre, B.rec.shared_pre);
    pair_phase(B, &PlanRecord::mid, B.rec.shared);
}

void replay(sdb_batch &B, cudaStream_t main)
{
    if (B.mm.zused()) SDB_CUDA(cudaMemsetAsync(B.mm.zero_base(), 0, B.mm.zused(), main));
    const size_t K = B.side.size();
    // one phase: each plan's list on a side stream (plan p on p % K), joined
    // back into main; nothing when every list is empty
    auto phase = [&](std::vector<DevOp> PlanRecord::*list) {
        bool any = false;
        for (const PlanRecord &pr : B.rec.plans) any |= !(pr.*list).empty();
        if (!any) return;
        SDB_CUDA(cudaEventRecord(B.fork, main));
        for (size_t i = 0; i < K; i++) SDB_CUDA(cudaStreamWaitEvent(B.side[i], B.fork, 0));
        for (size_t p = 0; p < B.rec.plans.size(); p++) {
            cudaStream_t s = B.side[p % K];
            for (const DevOp &op : B.rec.plans[p].*list) check(op.fn(s));
        }
        for (size_t i = 0; i < K; i++) {
            SDB_CUDA(cudaEventRecord(B.join[i], B.side[i]));
            SDB_CUDA(cudaStreamWaitEvent(main, B.join[i], 0));
        }
    };
    // under capture, external records: they stay timing events in the graph
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SDB_CUDA(cudaStreamIsCapturing(main, &cs));
    const unsigned rf = cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    auto mark = [&](cudaEvent_t e) {
        if (B.cb && e && B.timed) SDB_CUDA(cudaEventRecordWithFlags(e, main, rf));
    };
    for (const DevOp &op : B.rec.shared_pre) check(op.fn(main));  // paired fact scans
    phase(&PlanRecord::pre);
    mark(B.ev_c0);
    if (B.cb) check(sdb_chain_batch_launch_part(B.cb, 0, (sdb_stream_t)main));  // builds
    mark(B.ev_cb);
    for (const DevOp &op : B.rec.shared) check(op.fn(main));  // paired fact scans
    phase(&PlanRecord::mid);
    mark(B.ev_cm);
    if (B.cb) check(sdb_chain_batch_launch_part(B.cb, 1, (sdb_stream_t)main));  // aggregating chains
    mark(B.ev_c1);
    phase(&PlanRecord::post);
    // every plan's count and result columns, in one copy to the pinned mirror
    if (B.rbytes) SDB_CUDA(cudaMemcpyAsync(B.host, B.rbase, B.rbytes, cudaMemcpyDeviceToHost, main));
}

// Where each plan's count and result columns sit in the result region (and
// so in its pinned mirror B.host).
void layout_results(sdb_batch &B, const char *rbase)
{
    B.stage.assign(B.pend.size(), {});
    for (size_t p = 0; p < B.pend.size(); p++)
        for (const PendingSeg &sg : B.pend[p].segs) {
            sdb_batch::Stage st;
            st.count_off = (size_t)(reinterpret_cast<const char *>(sg.count) - rbase);
            for (void *d : sg.dev) st.col_off.push_back((size_t)(static_cast<const char *>(d) - rbase));
            B.stage[p].push_back(st);
        }
}

// Plan p's result from the staging of a finished run.
sdb_result *unpack_result(const sdb_batch &B, size_t p)
{
    const PendingResult &pr = B.pend[p];
    auto res = std::make_unique<sdb_result>();
    res->types = pr.types;
    const size_t ncols = pr.types.size();
    res->i32.resize(ncols);
    res->u64.resize(ncols);
    std::vector<uint32_t> counts(pr.segs.size());
    uint64_t total = 0;
    for (size_t s = 0; s < pr.segs.size(); s++) {
        std::memcpy(&counts[s], B.host + B.stage[p][s].count_off, 4);
        if (counts[s] > pr.segs[s].cap) throw Error(SDB_ERR_DEVICE, "batch result count exceeds its capacity");
        total += counts[s];
    }
    for (size_t c = 0; c < ncols; c++) {
        if (pr.types[c] == 1)
            res->u64[c].resize(total);
        else
            res->i32[c].resize(total);
    }
    uint64_t base = 0;
    for (size_t s = 0; s < pr.segs.size(); s++) {
        for (size_t c = 0; c < ncols; c++) {
            const char *src = B.host + B.stage[p][s].col_off[c];
            if (pr.types[c] == 1)
                std::memcpy(res->u64[c].data() + base, src, counts[s] * sizeof(uint64_t));
            else
                std::memcpy(res->i32[c].data() + base, src, counts[s] * sizeof(int32_t));
        }
        base += counts[s];
    }
    res->nrows = total;
    return res.release();
}

void batch_prepare(Engine &E, sdb_batch &B, const std::vector<std::string> &plans)
{
    // sizing pass: addresses only
    MemoryManager vm, vr;
    vm.init_virtual();
    vr.init_virtual();
    record_plans(E, B, vm, vr, plans);
    const uint64_t used = vm.used(), zused = vm.zused(), rused = vr.used();
    const size_t cb_bytes = B.rec.chains.empty()
                                ? 0
                                : sdb_chain_batch_scratch_bytes(B.rec.chains.data(), (int)B.rec.chains.size());
    vm.release();

    // real pass against an arena of exactly that size
    B.mm.init_sized(used + cb_bytes + 256, zused, E.stream);
    B.rmm.init_sized(rused, 256, E.stream);
    record_plans(E, B, B.mm, B.rmm, plans);
    pair_chains(E, B);
    if (!B.rec.chains.empty()) {
        void *scratch = B.mm.alloc<uint8_t>(cb_bytes);
        check(sdb_chain_batch_create(B.rec.chains.data(), (int)B.rec.chains.size(), scratch, cb_bytes,
                                     (sdb_stream_t)E.stream, &B.cb));
        B.chain_groups = sdb_chain_batch_kernels(B.cb);
    }

    B.rbase = B.rmm.base();
    B.rbytes = B.rmm.used();
    layout_results(B, B.rbase);
    B.host_bytes = std::max<size_t>(B.rbytes, 64);
    SDB_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&B.host), B.host_bytes, cudaHostAllocDefault));

    // streams and events; the plans' work is spread over up to 8 streams
    SDB_CUDA(cudaStreamCreateWithFlags(&B.bs, cudaStreamNonBlocking));
    const size_t K = std::min<size_t>(std::max<size_t>(plans.size(), 1), 16);
    for (size_t i = 0; i < K; i++) {
        cudaStream_t s;
        SDB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        B.side.push_back(s);
        cudaEvent_t e;
        SDB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        B.join.push_back(e);
    }
    SDB_CUDA(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming));
    SDB_CUDA(cudaEventCreate(&B.ev_a));
    SDB_CUDA(cudaEventCreate(&B.ev_b));
    SDB_CUDA(cudaEventCreate(&B.ev_c0));
    SDB_CUDA(cudaEventCreate(&B.ev_cb));
    SDB_CUDA(cudaEventCreate(&B.ev_cm));
    SDB_CUDA(cudaEventCreate(&B.ev_c1));
    SDB_CUDA(cudaStreamSynchronize(E.stream));

    const uint64_t l0 = sdb_launch_count();
    if (!(B.flags & SDB_BATCH_EAGER)) {
        SDB_CUDA(cudaStreamBeginCapture(B.bs, cudaStreamCaptureModeThreadLocal));
        try {
            replay(B, B.bs);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(B.bs, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        SDB_CUDA(cudaStreamEndCapture(B.bs, &B.graph));
        SDB_CUDA(cudaGraphInstantiate(&B.exec, B.graph, 0));
        B.kernels = (int)(sdb_launch_count() - l0);
    } else {
        B.kernels = -1;  // counted on the first run
    }
}

void batch_run(Engine &E, sdb_batch &B, sdb_result **out)
{
    // in the engine's own stream order (the graph was captured on B.bs; a
    // graph launches into any stream), so no cross-stream event sits before it
    cudaStream_t s = E.stream;
    SDB_CUDA(cudaEventRecord(B.ev_a, s));
    if (B.exec) {
        SDB_CUDA(cudaGraphLaunch(B.exec, s));
    } else {
        const uint64_t l0 = sdb_launch_count();
        replay(B, s);
        B.kernels = (int)(sdb_launch_count() - l0);
    }
    SDB_CUDA(cudaEventRecord(B.ev_b, s));
    SDB_CUDA(cudaEventSynchronize(B.ev_b));
    float ms = 0;
    SDB_CUDA(cudaEventElapsedTime(&ms, B.ev_a, B.ev_b));
    B.last_ms = ms;
    if (B.cb && B.timed) {
        float cms = 0;
        B.last_chain_ms = cudaEventElapsedTime(&cms, B.ev_cm, B.ev_c1) == cudaSuccess ? cms : -1.0;
        float bms = 0;
        B.last_build_ms = cudaEventElapsedTime(&bms, B.ev_c0, B.ev_cb) == cudaSuccess ? bms : -1.0;
        float pre = 0, mid = 0, post = 0;
        B.last_pre_ms = cudaEventElapsedTime(&pre, B.ev_a, B.ev_c0) == cudaSuccess &&
                                cudaEventElapsedTime(&mid, B.ev_cb, B.ev_cm) == cudaSuccess
                            ? pre + mid
                            : -1.0;
        B.last_post_ms = cudaEventElapsedTime(&post, B.ev_c1, B.ev_b) == cudaSuccess ? post : -1.0;
    }
    if (!out) return;
    for (size_t p = 0; p < B.pend.size(); p++) out[p] = unpack_result(B, p);
}

// Drops every prepared plan (their batches read the loaded tables).
void plan_cache_clear(sdb_engine &eng)
{
    for (auto &c : eng.cache)
        if (c.second.batch) delete c.second.batch;
    eng.cache.clear();
}

// sdb_engine_execute with the plan cache: the second execution of a plan text
// prepares it as a one-plan batch (recorded once against its own arena,
// captured as a CUDA graph, fused chains launched on their own); from then on
// an execution is one graph launch and the unpacking of its result.  The
// device work is the plain path's, kernel for kernel.
std::unique_ptr<sdb_result> execute_cached(sdb_engine &eng, const std::string &text)
{
    Engine &E = eng.E;
    const uint64_t now = ++eng.tick;
    auto it = eng.cache.find(text);
    if (it == eng.cache.end()) {
        if (eng.cache.size() >= 4096) {  // forget plans seen once
            for (auto c = eng.cache.begin(); c != eng.cache.end();)
                c = c->second.batch ? std::next(c) : eng.cache.erase(c);
        }
        it = eng.cache.emplace(text, sdb_engine::Cached{}).first;
    }
    sdb_engine::Cached &c = it->second;
    c.last = now;
    if (!c.batch && ++c.uses < 2) return execute_plan(E, text);
    if (!c.batch) {
        size_t prepared = 0;
        for (auto &o : eng.cache) prepared += o.second.batch != nullptr;
        while (prepared >= (size_t)E.cfg.plan_cache) {  // least recently used goes
            auto lru = eng.cache.end();
            for (auto o = eng.cache.begin(); o != eng.cache.end(); ++o)
                if (o->second.batch && (lru == eng.cache.end() || o->second.last < lru->second.last)) lru = o;
            delete lru->second.batch;
            lru->second.batch = nullptr;
            prepared--;
        }
        auto B = std::make_unique<sdb_batch>();
        B->eng = &eng;
        B->flags = SDB_BATCH_BUILDS_ONLY;
        B->timed = false;
        batch_prepare(E, *B, {text});
        c.batch = B.release();
    }
    sdb_result *r = nullptr;
    batch_run(E, *c.batch, &r);
    E.last_plan_ms = c.batch->last_ms;
    return std::unique_ptr<sdb_result>(r);
}

// ------------------------------------------------------------------ batches on caller memory
// Used by the request server: a batch sized from a sizing pass, built on
// memory carved from the server's pools and run once, eagerly, on a slot's
// streams.

BatchSize batch_size(sdb_engine *eng, const std::vector<std::string> &plans)
{
    Engine &E = eng->E;
    sdb_batch B;
    MemoryManager vm, vr;
    vm.init_virtual();
    vr.init_virtual();
    record_plans(E, B, vm, vr, plans);
    BatchSize z;
    z.arena = vm.used();
    z.zero = vm.zused();
    z.staging = vr.used();
    z.chains = B.rec.chains;
    return z;
}

size_t batch_chain_bytes(const std::vector<sdb_chain_desc> &chains)
{
    return chains.empty() ? 0 : sdb_chain_batch_scratch_bytes(chains.data(), (int)chains.size());
}

sdb_batch *batch_launch_external(sdb_engine *eng, const std::vector<std::string> &plans, const BatchSize &z,
                                 char *dev, size_t dev_bytes, char *pinned, size_t pinned_bytes, const SlotStreams &ss)
{
    Engine &E = eng->E;
    auto Bp = std::make_unique<sdb_batch>();
    sdb_batch &B = *Bp;
    B.eng = eng;
    B.owns = false;
    const uint64_t arena = (z.arena + 255) & ~uint64_t(255), zero = (z.zero + 255) & ~uint64_t(255);
    const uint64_t results = (z.staging + 255) & ~uint64_t(255);
    const size_t cb_bytes = batch_chain_bytes(z.chains);
    if (arena + zero + results + cb_bytes > dev_bytes) throw Error(SDB_ERR_INVALID, "batch region too small");
    B.mm.init_external(dev, arena, dev + arena, zero);
    B.rmm.init_external(dev + arena + zero, results, nullptr, 0);
    record_plans(E, B, B.mm, B.rmm, plans);
    if (B.mm.used() != z.arena || B.mm.zused() != z.zero || B.rmm.used() != z.staging)
        throw Error(SDB_ERR_INVALID, "batch sizing mismatch");
    pair_chains(E, B);
    if (cb_bytes + z.staging > pinned_bytes) throw Error(SDB_ERR_INVALID, "batch staging too small");
    B.host = pinned + cb_bytes;
    B.host_bytes = z.staging;
    B.rbase = dev + arena + zero;
    B.rbytes = z.staging;
    layout_results(B, B.rbase);
    B.side = ss.side;
    B.join = ss.join;
    B.fork = ss.fork;
    if (!B.rec.chains.empty())
        check(sdb_chain_batch_create_async(B.rec.chains.data(), (int)B.rec.chains.size(), dev + arena + zero + results,
                                           cb_bytes, pinned, cb_bytes, (sdb_stream_t)ss.main, &B.cb));
    replay(B, ss.main);
    return Bp.release();
}

sdb_result *batch_take_result(const sdb_batch *B, size_t p) { return unpack_result(*B, p); }

int batch_paired_chains(const sdb_batch *B) { return B->paired; }

sdb_result *execute_plain(sdb_engine *eng, const std::string &plan) { return execute_plan(eng->E, plan).release(); }

uint64_t engine_memory_bytes(const sdb_engine *eng) { return eng->E.mm.capacity(); }

void batch_destroy(sdb_batch *B)
{
    if (B && !B->owns) {
        // the slot's streams and events are not the batch's
        B->side.clear();
        B->join.clear();
        B->fork = nullptr;
        B->host = nullptr;
    }
    delete B;
}

template <class F>
int guarded(F f)
{
    try {
        f();
        return SDB_OK;
    } catch (const Error &e) {
        return sdb_set_error(e.status, "%s", e.what());
    } catch (const std::bad_alloc &) {
        return sdb_set_error(SDB_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception &e) {
        return sdb_set_error(SDB_ERR_INVALID, "%s", e.what());
    }
}

}  // namespace sdb

// ====================================================================== C ABI
extern "C" {

int sdb_plan_check(const char *plan_json, int *n_rels, int *order, int order_cap)
{
    if (!plan_json) return sdb_set_error(SDB_ERR_INVALID, "sdb_plan_check: NULL plan");
    return sdb::guarded([&] {
        sdb::PlanResult p = sdb::plan_from_json(plan_json);
        sdb::ExecutionInfo info = sdb::parse_execution_info(p);
        if (n_rels) *n_rels = (int)p.rels.size();
        if (order)
            for (size_t i = 0; i < info.dag_order.size() && (int)i < order_cap; i++) order[i] = info.dag_order[i];
    });
}

int sdb_plan_to_idl_json(const char *plan_json, char *out, size_t cap, size_t *len)
{
    if (!plan_json || !len) return sdb_set_error(SDB_ERR_INVALID, "sdb_plan_to_idl_json: NULL argument");
    return sdb::guarded([&] {
        const std::string text = sdb::plan_to_json(sdb::plan_from_json(plan_json));
        *len = text.size();
        if (out && cap > text.size()) std::memcpy(out, text.c_str(), text.size() + 1);
    });
}

int sdb_engine_create(const sdb_engine_config *cfg, sdb_engine **out)
{
    if (!out) return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_create: out is NULL");
    *out = nullptr;
    auto eng = std::make_unique<sdb_engine>();
    int st = sdb::guarded([&] {
        sdb::Engine &E = eng->E;
        if (cfg) E.cfg = *cfg;
        if (E.cfg.segment_rows) {
            if (E.cfg.segment_rows % 256 != 0) throw sdb::Error(SDB_ERR_INVALID, "segment_rows must be a multiple of 256");
            E.seg = E.cfg.segment_rows;
        }
        if (E.cfg.stream) {
            E.stream = (cudaStream_t)E.cfg.stream;
        } else {
            SDB_CUDA(cudaStreamCreateWithFlags(&E.stream, cudaStreamNonBlocking));
            E.own_stream = true;
        }
        uint64_t budget = E.cfg.arena_bytes;
        if (budget == 0) {
            // runtime/runtime.cpp:278-285: min(max(8 GB, mem/2), 10.5 GB)
            size_t fr = 0, tot = 0;
            SDB_CUDA(cudaMemGetInfo(&fr, &tot));
            budget = std::min<uint64_t>(std::max<uint64_t>(8ull << 30, tot / 2), (10ull << 30) + (512ull << 20));
        }
        E.mm.init(budget, E.stream);
        E.prof.on = E.cfg.profile != 0;
        if (E.cfg.plan_cache < 0) throw sdb::Error(SDB_ERR_INVALID, "plan_cache must be >= 0");
        if (E.cfg.join_tables < 0 || E.cfg.join_tables > 2) throw sdb::Error(SDB_ERR_INVALID, "join_tables must be 0, 1 or 2");
        SDB_CUDA(cudaEventCreate(&E.plan_a));
        SDB_CUDA(cudaEventCreate(&E.plan_b));
        SDB_CUDA(cudaStreamSynchronize(E.stream));
    });
    if (st == SDB_OK) *out = eng.release();
    return st;
}

int sdb_engine_destroy(sdb_engine *eng)
{
    if (!eng) return SDB_OK;
    sdb::Engine &E = eng->E;
    cudaStreamSynchronize(E.stream);
    sdb::plan_cache_clear(*eng);
    for (auto &pl : E.pending) {  // finish background loads, then free them
        try {
            auto t = pl.second.get();
            for (auto p : t->owned) cudaFree(p);
        } catch (...) {
        }
    }
    E.pending.clear();
    for (auto &t : E.tables)
        for (auto p : t.second->owned) cudaFree(p);
    E.tables.clear();
    E.mm.release();
    if (E.plan_a) cudaEventDestroy(E.plan_a);
    if (E.plan_b) cudaEventDestroy(E.plan_b);
    if (E.aux) cudaStreamDestroy(E.aux);
    if (E.copied) cudaEventDestroy(E.copied);
    if (E.stats_dev) cudaFree(E.stats_dev);
    if (E.stats_host) cudaFreeHost(E.stats_host);
    if (E.own_stream) cudaStreamDestroy(E.stream);
    delete eng;
    return SDB_OK;
}

int sdb_engine_load_table(sdb_engine *eng, const char *name, int ncols, const int32_t *const *cols, uint64_t nrows,
                          int on_device)
{
    if (!eng) return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_load_table: engine is NULL");
    return sdb::guarded([&] {
        // prepared plans stay when the table comes back in the same buffers
        // with the same statistics (a re-load of the same data)
        bool same = false;
        try {
            same = sdb::load_table(eng->E, name, ncols, cols, nrows, on_device);
        } catch (...) {
            sdb::plan_cache_clear(*eng);
            throw;
        }
        if (!same) sdb::plan_cache_clear(*eng);
    });
}

int sdb_engine_load_dir(sdb_engine *eng, const char *dir, const char *name, uint64_t column_mask, int background)
{
    if (!eng || !dir || !name) return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_load_dir: NULL argument");
    return sdb::guarded([&] {
        sdb::Engine &E = eng->E;
        const std::string tname = name;
        auto it = sdb::table_column_numbers().find(sdb::base_name(tname));
        if (it == sdb::table_column_numbers().end()) throw sdb::Error(SDB_ERR_INVALID, "unknown table " + tname);
        const int ncols = it->second;
        uint64_t mask = column_mask;
        if (mask == 0)
            for (int c : sdb::table_column_indices().at(sdb::base_name(tname))) mask |= 1ull << c;
        if (ncols < 64 && (mask >> ncols))
            throw sdb::Error(SDB_ERR_INVALID, "column_mask names columns beyond the table's " + std::to_string(ncols));
        sdb::plan_cache_clear(*eng);
        sdb::activate_table(E, tname);
        const uint64_t seg = E.seg;
        const std::string d = dir;
        auto work = [d, tname, ncols, mask, seg](int device) {
            cudaSetDevice(device);
            cudaStream_t s = nullptr;
            SDB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            std::vector<std::string> warn;
            std::unique_ptr<sdb::Table> t;
            try {
                t = sdb::load_columns(d, tname, ncols, mask, seg, s, &warn);
            } catch (...) {
                cudaStreamDestroy(s);
                throw;
            }
            cudaStreamDestroy(s);
            for (auto &w : warn) std::fprintf(stderr, "sycldb: %s\n", w.c_str());
            return t;
        };
        int device = 0;
        SDB_CUDA(cudaGetDevice(&device));
        if (background)
            E.pending[tname] = std::async(std::launch::async, work, device);
        else
            sdb::install_table(E, tname, work(device));
    });
}

int sdb_engine_sync_tables(sdb_engine *eng)
{
    if (!eng) return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_sync_tables: engine is NULL");
    return sdb::guarded([&] {
        std::vector<std::string> names;
        for (auto &p : eng->E.pending) names.push_back(p.first);
        for (auto &n : names) sdb::activate_table(eng->E, n);
    });
}

int sdb_engine_execute(sdb_engine *eng, const char *plan_json, sdb_result **out)
{
    if (!eng || !plan_json || !out) return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_execute: NULL argument");
    *out = nullptr;
    return sdb::guarded([&] {
        auto r = (eng->E.cfg.plan_cache > 0 && !eng->E.prof.on && !eng->E.cfg.order_by)
                     ? sdb::execute_cached(*eng, plan_json)
                     : sdb::execute_plan(eng->E, plan_json);
        *out = r.release();
    });
}

int sdb_result_shape(const sdb_result *r, int *ncols, uint64_t *nrows)
{
    if (!r) return sdb_set_error(SDB_ERR_INVALID, "sdb_result_shape: NULL result");
    if (ncols) *ncols = (int)r->types.size();
    if (nrows) *nrows = r->nrows;
    return SDB_OK;
}

int sdb_result_column(const sdb_result *r, int c, int *type, const void **data)
{
    if (!r || c < 0 || (size_t)c >= r->types.size()) return sdb_set_error(SDB_ERR_INVALID, "sdb_result_column: bad column");
    if (type) *type = r->types[c];
    if (data) *data = r->types[c] == 1 ? (const void *)r->u64[c].data() : (const void *)r->i32[c].data();
    return SDB_OK;
}

int sdb_result_write_res(const sdb_result *r, const char *path)
{
    if (!r || !path) return sdb_set_error(SDB_ERR_INVALID, "sdb_result_write_res: NULL argument");
    std::ofstream f(path);
    if (!f.is_open()) return sdb_set_error(SDB_ERR_INVALID, "Could not open result file for writing: %s", path);
    for (uint64_t row = 0; row < r->nrows; row++) {
        for (size_t c = 0; c < r->types.size(); c++) {
            if (c) f << ' ';
            if (r->types[c] == 1)
                f << r->u64[c][row];
            else
                f << r->i32[c][row];
        }
        f << '\n';
    }
    return f.good() ? SDB_OK : sdb_set_error(SDB_ERR_INVALID, "write failed: %s", path);
}

void sdb_result_free(sdb_result *r) { delete r; }

int sdb_engine_kernel_stats(const sdb_engine *eng, int k, const char **name, uint64_t *launches, double *total_ms)
{
    if (!eng) return 0;
    const auto &st = eng->E.prof.stats;
    if (k < 0 || (size_t)k >= st.size()) return (int)st.size();
    auto it = st.begin();
    std::advance(it, k);
    if (name) *name = it->first.c_str();
    if (launches) *launches = it->second.first;
    if (total_ms) *total_ms = it->second.second;
    return (int)st.size();
}

int sdb_engine_last_plan_ms(const sdb_engine *eng, double *ms)
{
    if (!eng || !ms) return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_last_plan_ms: NULL argument");
    *ms = eng->E.last_plan_ms;
    return SDB_OK;
}

int sdb_engine_batch_prepare(sdb_engine *eng, const char *const *plans_json, int n_plans, int flags, sdb_batch **out)
{
    if (!eng || !out || n_plans < 1 || !plans_json)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_batch_prepare: bad argument");
    if (flags & ~(SDB_BATCH_EAGER | SDB_BATCH_NO_CHAIN_BATCH | SDB_BATCH_BUILDS_ONLY))
        return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_batch_prepare: unknown flags 0x%x", flags);
    *out = nullptr;
    std::vector<std::string> plans;
    for (int i = 0; i < n_plans; i++) {
        if (!plans_json[i]) return sdb_set_error(SDB_ERR_INVALID, "sdb_engine_batch_prepare: plan %d is NULL", i);
        plans.emplace_back(plans_json[i]);
    }
    auto B = std::make_unique<sdb_batch>();
    B->eng = eng;
    B->flags = flags;
    int st = sdb::guarded([&] { sdb::batch_prepare(eng->E, *B, plans); });
    if (st != SDB_OK) return st;
    *out = B.release();
    return SDB_OK;
}

int sdb_batch_run(sdb_batch *b, sdb_result **results)
{
    if (!b) return sdb_set_error(SDB_ERR_INVALID, "sdb_batch_run: NULL batch");
    return sdb::guarded([&] { sdb::batch_run(b->eng->E, *b, results); });
}

int sdb_batch_info(const sdb_batch *b, sdb_batch_stats *info)
{
    if (!b || !info) return sdb_set_error(SDB_ERR_INVALID, "sdb_batch_info: NULL argument");
    info->n_plans = (int32_t)b->pend.size();
    info->kernels_per_run = b->kernels;
    info->graph = b->exec ? 1 : 0;
    info->chain_launches = b->chain_groups;
    int32_t builds = 0;
    for (const sdb_chain_desc &c : b->rec.chains) builds += sdb::Fuser::is_build(c.terminal) ? 1 : 0;
    info->batched_chains = (int32_t)b->rec.chains.size() - builds;
    info->batched_builds = builds;
    info->arena_bytes = b->mm.size();
    info->zero_bytes = b->mm.zused();
    info->host_bytes = b->host_bytes;
    info->last_run_ms = b->last_ms;
    info->last_chain_ms = b->last_chain_ms;
    info->last_pre_ms = b->last_pre_ms;
    info->last_post_ms = b->last_post_ms;
    info->last_build_ms = b->last_build_ms;
    info->paired_chains = b->paired;
    return SDB_OK;
}

int sdb_batch_layout(const sdb_batch *b, int plan, int *ncols, int *types, int types_cap, int *nsegs)
{
    if (!b || plan < 0 || (size_t)plan >= b->pend.size() || !ncols || !nsegs)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_batch_layout: bad argument");
    const auto &pr = b->pend[plan];
    *ncols = (int)pr.types.size();
    *nsegs = (int)pr.segs.size();
    for (int c = 0; c < *ncols && c < types_cap && types; c++) types[c] = pr.types[c];
    return SDB_OK;
}

int sdb_batch_segment(const sdb_batch *b, int plan, int seg, uint64_t *count_off, uint64_t *col_offs, int cap,
                      uint64_t *capacity)
{
    if (!b || plan < 0 || (size_t)plan >= b->pend.size() || seg < 0 || (size_t)seg >= b->pend[plan].segs.size() ||
        !count_off || !capacity)
        return sdb_set_error(SDB_ERR_INVALID, "sdb_batch_segment: bad argument");
    const auto &st = b->stage[plan][seg];
    *count_off = st.count_off;
    *capacity = b->pend[plan].segs[seg].cap;
    for (size_t c = 0; c < st.col_off.size() && (int)c < cap && col_offs; c++) col_offs[c] = st.col_off[c];
    return SDB_OK;
}

const void *sdb_batch_host(const sdb_batch *b, size_t *bytes)
{
    if (!b) return nullptr;
    if (bytes) *bytes = b->rbytes;
    return b->host;
}

void sdb_batch_free(sdb_batch *b) { delete b; }

}  // extern "C"
