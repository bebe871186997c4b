// Plan structures in the shape of the reference's Thrift IDL
// (server/thrift/calciteserver.thrift:3-80; generated C++ in
// gen-cpp/calciteserver_types.h), as plain C++ structs, and their loader from
// JSON text.  Enum values are the IDL's.  A JSON plan may give enums either
// by name ("TABLE_SCAN") or by number (0).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "json.hpp"

namespace sdb {

enum RelNodeType { TABLE_SCAN = 0, FILTER = 1, JOIN = 2, PROJECT = 3, AGGREGATE = 4, SORT = 5 };
enum ExprOption { LITERAL = 0, COLUMN = 1, EXPR = 2 };
enum LiteralOption { LIT_LITERAL = 0, LIT_RANGE = 1 };

struct LiteralType {
    int literalOption = LIT_LITERAL;
    int64_t value = 0;
    std::vector<std::vector<std::string>> rangeSet;
};

struct ExprType {
    int exprType = LITERAL;
    int64_t input = 0;
    std::string name;
    std::string op;
    std::vector<ExprType> operands;
    LiteralType literal;
    std::string type;
};

struct AggType {
    std::string agg;
    std::vector<int64_t> operands;
    std::string name;
    std::string type;
    bool distinct = false;
};

struct CollationType {
    int64_t field = 0;
    int direction = 1;  // ASCENDING
    int nulls = 1;      // LAST
};

struct RelNode {
    int64_t id = 0;
    int relOp = TABLE_SCAN;
    std::vector<std::string> tables;
    std::vector<int64_t> inputs;
    ExprType condition;
    std::string joinType;
    std::vector<std::string> fields;
    std::vector<ExprType> exprs;
    std::vector<int64_t> group;
    std::vector<AggType> aggs;
    std::vector<CollationType> collation;
};

struct PlanResult {
    std::vector<RelNode> rels;
    std::string oldJson;
};

namespace detail {

inline int enum_of(const json::Value &v, const char *const *names, int count, const char *what)
{
    if (v.is_number()) return (int)v.as_int();
    const std::string &s = v.as_string();
    for (int i = 0; i < count; i++)
        if (s == names[i]) return i;
    throw std::invalid_argument(std::string("plan: unknown ") + what + " '" + s + "'");
}

inline ExprType expr_from(const json::Value &v)
{
    static const char *const kExpr[] = {"LITERAL", "COLUMN", "EXPR"};
    static const char *const kLit[] = {"LITERAL", "RANGE"};
    ExprType e;
    if (!v.is_object()) throw std::invalid_argument("plan: expression must be an object");
    if (const json::Value *t = v.find("exprType")) e.exprType = enum_of(*t, kExpr, 3, "exprType");
    if (v.has("input")) e.input = v.find("input")->as_int();
    if (v.has("name")) e.name = v.find("name")->as_string();
    if (v.has("op")) e.op = v.find("op")->as_string();
    if (v.has("type")) e.type = v.find("type")->as_string();
    if (const json::Value *ops = v.find("operands"))
        for (const auto &o : ops->arr) e.operands.push_back(expr_from(o));
    if (const json::Value *l = v.find("literal")) {
        if (l->has("literalOption")) e.literal.literalOption = enum_of(*l->find("literalOption"), kLit, 2, "literalOption");
        if (l->has("value")) e.literal.value = l->find("value")->as_int();
        if (const json::Value *rs = l->find("rangeSet")) {
            e.literal.literalOption = LIT_RANGE;
            for (const auto &r : rs->arr) {
                std::vector<std::string> row;
                for (const auto &x : r.arr) row.push_back(x.is_string() ? x.s : std::to_string(x.as_int()));
                e.literal.rangeSet.push_back(std::move(row));
            }
        }
    }
    return e;
}

inline std::vector<int64_t> ints_from(const json::Value *v)
{
    std::vector<int64_t> out;
    if (v)
        for (const auto &x : v->arr) out.push_back(x.as_int());
    return out;
}

}  // namespace detail

inline PlanResult plan_from_json(const std::string &text)
{
    static const char *const kRel[] = {"TABLE_SCAN", "FILTER", "JOIN", "PROJECT", "AGGREGATE", "SORT"};
    static const char *const kDir[] = {"DESCENDING", "ASCENDING"};
    static const char *const kNulls[] = {"FIRST", "LAST"};
    json::Value root = json::parse(text);
    const json::Value *rels = root.find("rels");
    if (!rels || !rels->is_array()) throw std::invalid_argument("plan: missing \"rels\" array");
    PlanResult plan;
    for (const auto &r : rels->arr) {
        RelNode n;
        n.id = r.find("id") ? r.find("id")->as_int() : (int64_t)plan.rels.size();
        if (!r.find("relOp")) throw std::invalid_argument("plan: rel without relOp");
        n.relOp = detail::enum_of(*r.find("relOp"), kRel, 6, "relOp");
        if (const json::Value *t = r.find("tables"))
            for (const auto &x : t->arr) n.tables.push_back(x.as_string());
        n.inputs = detail::ints_from(r.find("inputs"));
        if (r.has("condition")) n.condition = detail::expr_from(*r.find("condition"));
        if (r.has("joinType")) n.joinType = r.find("joinType")->as_string();
        if (const json::Value *f = r.find("fields"))
            for (const auto &x : f->arr) n.fields.push_back(x.as_string());
        if (const json::Value *ex = r.find("exprs"))
            for (const auto &x : ex->arr) n.exprs.push_back(detail::expr_from(x));
        n.group = detail::ints_from(r.find("group"));
        if (const json::Value *ag = r.find("aggs"))
            for (const auto &x : ag->arr) {
                AggType a;
                if (x.has("agg")) a.agg = x.find("agg")->is_string() ? x.find("agg")->s : "";
                a.operands = detail::ints_from(x.find("operands"));
                if (x.has("name")) a.name = x.find("name")->as_string();
                if (x.has("type")) a.type = x.find("type")->is_string() ? x.find("type")->s : "";
                if (x.has("distinct")) a.distinct = x.find("distinct")->as_bool();
                n.aggs.push_back(a);
            }
        if (const json::Value *co = r.find("collation"))
            for (const auto &x : co->arr) {
                CollationType c;
                if (x.has("field")) c.field = x.find("field")->as_int();
                if (x.has("direction")) c.direction = detail::enum_of(*x.find("direction"), kDir, 2, "direction");
                if (x.has("nulls")) c.nulls = detail::enum_of(*x.find("nulls"), kNulls, 2, "nulls");
                n.collation.push_back(c);
            }
        plan.rels.push_back(std::move(n));
    }
    for (size_t i = 0; i < plan.rels.size(); i++)
        if (plan.rels[i].id != (int64_t)i) throw std::invalid_argument("plan: rel ids must be 0..n-1 in order");
    return plan;
}

}  // namespace sdb
