// Runs the reference's own executor on the CPU.
//
// TEST INFRASTRUCTURE ONLY (an oracle: tests call it, nothing in the product
// links it).  build_oracle.py compiles this file together with the
// reference's executor sources where they lie (executor/ddor_executor.cpp,
// executor/result_writer.cpp, operations/preprocessing.cpp,
// operations/memory_manager.cpp, runtime/runtime.cpp, kernels/types.cpp,
// kernels/jit_kernels.cpp, app/query_utils.cpp,
// gen-cpp/calciteserver_types.cpp) against the host shims of
// oracle/ref_shim (SYCL work-items one at a time, Thrift types without
// serialisation, the disabled JIT), with the reference's correctness mode
// (PERFORMANCE_MEASUREMENT_ACTIVE 0, so execute_ddor_plan writes its .res
// result).  What this file adds is only the glue the reference's client
// would be: a plan in the IDL's JSON shape turned into the Thrift
// PlanResult (server/thrift/calciteserver.thrift:22-80), and the call
// sequence of app/application.cpp:91-122 -- build the runtime (one device),
// the allocators, execute_ddor_plan, wait.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "executor/ddor_executor.hpp"
#include "kernels/jit_kernels.hpp"
#include "gen-cpp/calciteserver_types.h"
#include "runtime/runtime.hpp"

namespace {

// ---- a small JSON reader (objects, arrays, strings, numbers, booleans, null)
struct Json {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    long long num = 0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json *get(const char *key) const
    {
        for (const auto &kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

class Reader {
public:
    explicit Reader(const char *s) : p_(s) {}

    Json value()
    {
        ws();
        Json j;
        if (*p_ == '{') {
            j.kind = Json::Obj;
            ++p_;
            ws();
            if (*p_ == '}') { ++p_; return j; }
            for (;;) {
                ws();
                std::string k = string();
                ws();
                expect(':');
                j.obj.emplace_back(k, value());
                ws();
                if (*p_ == ',') { ++p_; continue; }
                expect('}');
                return j;
            }
        }
        if (*p_ == '[') {
            j.kind = Json::Arr;
            ++p_;
            ws();
            if (*p_ == ']') { ++p_; return j; }
            for (;;) {
                j.arr.push_back(value());
                ws();
                if (*p_ == ',') { ++p_; continue; }
                expect(']');
                return j;
            }
        }
        if (*p_ == '"') {
            j.kind = Json::Str;
            j.str = string();
            return j;
        }
        if (!std::strncmp(p_, "true", 4)) { p_ += 4; j.kind = Json::Bool; j.b = true; return j; }
        if (!std::strncmp(p_, "false", 5)) { p_ += 5; j.kind = Json::Bool; return j; }
        if (!std::strncmp(p_, "null", 4)) { p_ += 4; return j; }
        char *end = nullptr;
        j.num = std::strtoll(p_, &end, 10);
        if (end == p_) throw std::runtime_error("plan JSON: unexpected character");
        p_ = end;
        j.kind = Json::Num;
        return j;
    }

private:
    const char *p_;
    void ws()
    {
        while (*p_ && std::isspace((unsigned char)*p_)) ++p_;
    }
    void expect(char c)
    {
        if (*p_ != c) throw std::runtime_error(std::string("plan JSON: expected '") + c + "'");
        ++p_;
    }
    std::string string()
    {
        expect('"');
        std::string s;
        while (*p_ && *p_ != '"') {
            if (*p_ == '\\' && p_[1]) ++p_;
            s += *p_++;
        }
        expect('"');
        return s;
    }
};

// Enum fields: by name (the IDL's identifiers) or by number.
int enum_of(const Json &j, const std::vector<const char *> &names)
{
    if (j.kind == Json::Num) return (int)j.num;
    for (size_t i = 0; i < names.size(); i++)
        if (j.str == names[i]) return (int)i;
    throw std::runtime_error("plan JSON: unknown enum value " + j.str);
}

std::vector<int64_t> ints(const Json &j)
{
    std::vector<int64_t> v;
    for (const Json &x : j.arr) v.push_back(x.num);
    return v;
}

std::vector<std::string> strings(const Json &j)
{
    std::vector<std::string> v;
    for (const Json &x : j.arr) v.push_back(x.str);
    return v;
}

ExprType expr_of(const Json &j)
{
    ExprType e;
    if (const Json *x = j.get("exprType")) e.__set_exprType((ExprOption::type)enum_of(*x, {"LITERAL", "COLUMN", "EXPR"}));
    if (const Json *x = j.get("input")) e.__set_input(x->num);
    if (const Json *x = j.get("name")) e.__set_name(x->str);
    if (const Json *x = j.get("op")) e.__set_op(x->str);
    if (const Json *x = j.get("operands")) {
        std::vector<ExprType> ops;
        for (const Json &o : x->arr) ops.push_back(expr_of(o));
        e.__set_operands(ops);
    }
    if (const Json *x = j.get("literal")) {
        LiteralType l;
        if (const Json *y = x->get("literalOption")) l.__set_literalOption((LiteralOption::type)enum_of(*y, {"LITERAL", "RANGE"}));
        if (const Json *y = x->get("value")) l.__set_value(y->num);
        if (const Json *y = x->get("rangeSet")) {
            std::vector<std::vector<std::string>> rs;
            for (const Json &r : y->arr) rs.push_back(strings(r));
            l.__set_rangeSet(rs);
        }
        e.__set_literal(l);
    }
    if (const Json *x = j.get("type")) e.__set_type(x->str);
    return e;
}

PlanResult plan_of(const Json &root)
{
    PlanResult pr;
    std::vector<RelNode> rels;
    const Json *rj = root.get("rels");
    if (!rj) throw std::runtime_error("plan JSON: no rels");
    for (const Json &r : rj->arr) {
        RelNode n;
        if (const Json *x = r.get("id")) n.__set_id(x->num);
        if (const Json *x = r.get("relOp"))
            n.__set_relOp((RelNodeType::type)enum_of(*x, {"TABLE_SCAN", "FILTER", "JOIN", "PROJECT", "AGGREGATE", "SORT"}));
        if (const Json *x = r.get("tables")) n.__set_tables(strings(*x));
        if (const Json *x = r.get("inputs")) n.__set_inputs(ints(*x));
        if (const Json *x = r.get("condition")) n.__set_condition(expr_of(*x));
        if (const Json *x = r.get("joinType")) n.__set_joinType(x->str);
        if (const Json *x = r.get("fields")) n.__set_fields(strings(*x));
        if (const Json *x = r.get("exprs")) {
            std::vector<ExprType> es;
            for (const Json &e : x->arr) es.push_back(expr_of(e));
            n.__set_exprs(es);
        }
        if (const Json *x = r.get("group")) n.__set_group(ints(*x));
        if (const Json *x = r.get("aggs")) {
            std::vector<AggType> as;
            for (const Json &a : x->arr) {
                AggType t;
                if (const Json *y = a.get("agg")) t.__set_agg(y->str);
                if (const Json *y = a.get("operands")) t.__set_operands(ints(*y));
                if (const Json *y = a.get("name")) t.__set_name(y->str);
                if (const Json *y = a.get("type")) t.__set_type(y->str);
                if (const Json *y = a.get("distinct")) t.__set_distinct(y->b);
                as.push_back(t);
            }
            n.__set_aggs(as);
        }
        if (const Json *x = r.get("collation")) {
            std::vector<CollationType> cs;
            for (const Json &c : x->arr) {
                CollationType t;
                if (const Json *y = c.get("field")) t.__set_field(y->num);
                if (const Json *y = c.get("direction"))
                    t.__set_direction((DirectionOption::type)enum_of(*y, {"DESCENDING", "ASCENDING"}));
                if (const Json *y = c.get("nulls")) t.__set_nulls((NullsOption::type)enum_of(*y, {"FIRST", "LAST"}));
                cs.push_back(t);
            }
            n.__set_collation(cs);
        }
        rels.push_back(n);
    }
    pr.__set_rels(rels);
    return pr;
}

}  // namespace

// The reference's timing counters (declared in common.hpp; its application
// defines them, app/application.cpp).
double g_total_jit_ms = 0, g_total_kernel_ms = 0, g_total_internal_kernel_ms = 0, g_total_load_ms = 0;

extern "C" {

// The call sequence the reference's JIT would generate for a fused bundle
// (kernels/jit_kernels.hpp); its fusion is switched off
// (models/execution.hpp: disable_fusion), so this is never called.
void execute_sycldb_ops_agg(sycl::item<1>, SYCLDBContext, bool &, uint64_t &)
{
    std::fprintf(stderr, "ref_exec: the JIT call sequence is not available\n");
    std::abort();
}

// Loads the tables from data_dir (the reference's columnar files,
// <NAME><i>), runs plan_json through execute_ddor_plan and leaves the result
// in <stem>.res in the current directory.  on_device: 1 = the runtime's
// primary device (the shim's one device), 0 = primary device -1 (the
// reference's host placement).  Returns 0, or -1 with the reason in err.
int ref_exec_run(const char *data_dir, const char *plan_json, const char *stem, int on_device, char *err,
                 size_t errcap)
{
    try {
        DATA_DIR = std::string(data_dir) + "/";
        Reader rd(plan_json);
        const PlanResult plan = plan_of(rd.value());
        runtime_setup::RuntimeEnvironment runtime = runtime_setup::build_runtime_environment("");
        memory_manager cpu_allocator = runtime_setup::build_cpu_allocator(runtime);
        std::vector<memory_manager> device_allocators = runtime_setup::build_device_allocators(runtime);
        executor::execute_ddor_plan(plan, std::string(stem) + ".sql", runtime.tables, runtime.queues, cpu_allocator,
                                    device_allocators, on_device ? runtime.config.primary_device_index : -1,
                                    std::cout);
        runtime_setup::wait_for_all_queues_and_throw(runtime.queues);
        return 0;
    } catch (const std::exception &e) {
        if (err && errcap) std::snprintf(err, errcap, "%s", e.what());
        return -1;
    }
}

}  // extern "C"
