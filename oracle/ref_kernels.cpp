// Reference kernel functors, compiled from the SYCLDB sources where they lie
// and run on the CPU through the host SYCL shim (oracle/ref_shim).
//
// TEST INFRASTRUCTURE ONLY: the oracle tests compare the C restatement in
// sdb_oracle.c against these functions.  Nothing here is product code.
//
// Each ref_* entry builds the reference's KernelDefinition object and submits
// it the way KernelData::execute does (models/execution.hpp:260-497):
// queue.submit -> parallel_for(kernel.get_col_len(), kernel), or with
// sycl::reduction(agg_res, plus<uint64_t>) for AggregateOperationKernel.
#include <sycl/sycl.hpp>

#include "kernels/common.hpp"
#include "kernels/selection.hpp"
#include "kernels/projection.hpp"
#include "kernels/aggregation.hpp"
#include "kernels/join.hpp"
#include "kernels/types.hpp"

namespace {
sycl::queue q;

template <typename K>
void run(const K &k)
{
    q.submit([&](sycl::handler &cgh) { cgh.parallel_for(k.get_col_len(), k); });
}

const bool *b(const uint8_t *p) { return reinterpret_cast<const bool *>(p); }
bool *b(uint8_t *p) { return reinterpret_cast<bool *>(p); }
}  // namespace

extern "C" {

void ref_select_lit(const int32_t *col, int32_t v, int cmp, int logic, const uint8_t *in, uint8_t *out, uint64_t n)
{
    run(SelectionKernelLiteral((comp_op)cmp, (logical_op)logic, b(in), b(out), col, v, (int)n));
}

void ref_select_lit_str(const int32_t *col, int32_t v, const char *op, const char *parent,
                        const uint8_t *in, uint8_t *out, uint64_t n)
{
    run(SelectionKernelLiteral(b(in), b(out), col, std::string(op), v, std::string(parent), (int)n));
}

void ref_select_cols(const int32_t *a, const int32_t *c, int cmp, int logic, const uint8_t *in, uint8_t *out, uint64_t n)
{
    run(SelectionKernelColumns((comp_op)cmp, (logical_op)logic, b(in), b(out), a, c, (int)n));
}

void ref_logical(int logic, const uint8_t *in, const uint8_t *local, uint8_t *out, uint64_t n)
{
    run(LogicalKernel((logical_op)logic, b(in), b(local), b(out), (int)n));
}

void ref_fill_i32(int32_t *dst, int32_t v, uint64_t n)
{
    run(FillKernel(dst, v, (int)n));
}

void ref_binop_cc(int32_t *res, const int32_t *a, const int32_t *c, int op, const uint8_t *flags, uint64_t n)
{
    run(PerformOperationKernelColumns(res, a, c, b(flags), (BinaryOp)op, (int)n));
}

void ref_binop_lc(int32_t *res, int32_t lit, const int32_t *c, int op, const uint8_t *flags, uint64_t n)
{
    run(PerformOperationKernelLiteralFirst(res, lit, c, b(flags), (BinaryOp)op, (int)n));
}

void ref_binop_cl(int32_t *res, const int32_t *a, int32_t lit, int op, const uint8_t *flags, uint64_t n)
{
    run(PerformOperationKernelLiteralSecond(res, a, lit, b(flags), (BinaryOp)op, (int)n));
}

void ref_sum_i32_u64(const int32_t *col, const uint8_t *flags, uint64_t n, uint64_t *acc)
{
    AggregateOperationKernel k(col, b(flags), (int)n, acc);
    uint64_t *agg_res_ptr = k.get_agg_res();
    q.submit([&](sycl::handler &cgh) {
        cgh.parallel_for(k.get_col_len(), sycl::reduction(agg_res_ptr, sycl::plus<uint64_t>()), k);
    });
}

void ref_groupby_sum(const int32_t *const *keys, const int32_t *mins, const int32_t *maxs, int g,
                     const int32_t *val, const uint8_t *flags, uint64_t n, uint64_t P,
                     int32_t *const *out_keys, uint64_t *out_sum, uint32_t *occ)
{
    run(GroupByAggregateKernel(const_cast<const int **>(reinterpret_cast<const int *const *>(keys)), val,
                               maxs, mins, b(flags), g, (int)n, const_cast<int **>(reinterpret_cast<int *const *>(out_keys)),
                               out_sum, occ, P));
}

void ref_ht_build_keys(const int32_t *key, const uint8_t *flags, uint64_t n, uint8_t *ht, int32_t mn, int32_t len)
{
    run(BuildKeysHTKernel(b(ht), key, b(flags), len, mn, (int)n));
}

void ref_probe_semi(const int32_t *key, const uint8_t *in, uint8_t *out, uint64_t n, const uint8_t *ht, int32_t mn, int32_t mx)
{
    run(FilterJoinKernel(key, b(in), b(out), b(ht), mn, mx, (int)n));
}

void ref_ht_build_kv(const int32_t *key, const int32_t *val, const uint8_t *flags, uint64_t n, int32_t *ht2,
                     int32_t mn, int32_t len)
{
    run(BuildKeyValsHTKernel(ht2, key, val, b(flags), len, mn, (int)n));
}

void ref_probe_full(const int32_t *key, int32_t *val_out, const uint8_t *in, uint8_t *out, uint64_t n,
                    const int32_t *ht2, int32_t mn, int32_t mx)
{
    run(FullJoinKernel(key, val_out, b(in), b(out), ht2, mn, mx, (int)n));
}

uint64_t ref_count_flags(const uint8_t *flags, uint64_t n)
{
    return count_true_flags(b(flags), (int)n, q);
}

int ref_get_comp_op(const char *op) { return (int)get_comp_op(op); }
int ref_get_logical_op(const char *op) { return (int)get_logical_op(op); }
int ref_is_filter_logical(const char *op) { return is_filter_logical(op) ? 1 : 0; }
int ref_get_binop(const char *op)
{
    try {
        return (int)get_op_from_string(op);
    } catch (const std::invalid_argument &) {
        return -1;
    }
}

// Column maps of the base-table loader (kernels/types.cpp:3-21).
int ref_table_column_number(const char *table)
{
    auto it = table_column_numbers.find(table);
    return it == table_column_numbers.end() ? -1 : it->second;
}

int ref_table_column_loaded(const char *table, int col)
{
    auto it = table_column_indices.find(table);
    if (it == table_column_indices.end()) return -1;
    return it->second.count(col) ? 1 : 0;
}

}  // extern "C"

// operations/memory_manager.hpp declares these out of line; the kernels never
// allocate through them here, so the shim build only needs them to link.
memory_region::memory_region(sycl::queue &queue, uint64_t size, bool, bool zero)
    : size(size), queue(queue), zero(zero)
{
    throw std::runtime_error("memory_region is not available in the host shim build");
}
memory_region::~memory_region() {}
