// Plan structures in the shape of the reference's Thrift IDL
// (server/thrift/calciteserver.thrift:3-80; generated C++ in
// gen-cpp/calciteserver_types.h), as plain C++ structs, and their loader from
// JSON text.  Enum values are the IDL's.  Two JSON dialects are read:
//
//  * the IDL shape: "relOp" an IDL name ("TABLE_SCAN") or number, "tables",
//    numeric ids and inputs, expressions tagged with "exprType", "op" a
//    string, literals {"literalOption", "value" | "rangeSet"};
//  * Calcite's RelJson as the reference's planner emits it and
//    SycldbJsonConverter turns into the IDL structs
//    (server/src/main/java/com/eurecom/calcite/SycldbJsonConverter.java:31-163):
//    "relOp" a planner class name ("com.eurecom.calcite.SycldbTableScan"),
//    "table", string ids and inputs, expressions told apart by their keys
//    (a column has "input", a call has "op": {"name": ...}, anything else
//    is a literal: a bare number, or {"rangeSet": ...} for a Sarg),
//    "type": {"type": ...}, aggregates with "agg": {"name": ...}.
//
// Both give the same PlanResult; plan_to_json writes one back in the IDL
// shape.
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
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

// An integer given as a JSON number or as a decimal string (RelJson writes
// rel ids and inputs as strings, SycldbJsonConverter.java:33,55-58).
inline int64_t int_of(const json::Value &v, const char *what)
{
    if (v.kind == json::Value::Int) return v.i;
    if (v.kind == json::Value::String) {
        const std::string &s = v.s;
        size_t k = (!s.empty() && (s[0] == '-' || s[0] == '+')) ? 1 : 0;
        if (k == s.size()) throw std::invalid_argument(std::string("plan: ") + what + " '" + s + "' is not an integer");
        for (size_t j = k; j < s.size(); j++)
            if (s[j] < '0' || s[j] > '9')
                throw std::invalid_argument(std::string("plan: ") + what + " '" + s + "' is not an integer");
        try {
            return std::stoll(s);
        } catch (const std::out_of_range &) {
            throw std::invalid_argument(std::string("plan: ") + what + " '" + s + "' out of range");
        }
    }
    throw std::invalid_argument(std::string("plan: ") + what + " must be an integer");
}

// A name given as a string or as an object {"name": ...} (RelJson's
// operators and aggregate functions) or {"type": ...} (RelJson's types).
inline std::string name_of(const json::Value &v, const char *key, const char *what)
{
    if (v.is_string()) return v.s;
    if (v.is_object())
        if (const json::Value *n = v.find(key))
            if (n->is_string()) return n->s;
    throw std::invalid_argument(std::string("plan: ") + what + " must be a string or an object with \"" + key + "\"");
}

inline void range_set_from(const json::Value &rs, LiteralType &lit)
{
    if (!rs.is_array()) throw std::invalid_argument("plan: rangeSet must be an array");
    lit.literalOption = LIT_RANGE;
    for (const auto &r : rs.arr) {
        if (!r.is_array()) throw std::invalid_argument("plan: rangeSet entries must be arrays");
        std::vector<std::string> row;
        for (const auto &x : r.arr) row.push_back(x.is_string() ? x.s : std::to_string(x.as_int()));
        lit.rangeSet.push_back(std::move(row));
    }
}

inline ExprType expr_from(const json::Value &v)
{
    static const char *const kExpr[] = {"LITERAL", "COLUMN", "EXPR"};
    static const char *const kLit[] = {"LITERAL", "RANGE"};
    ExprType e;
    if (!v.is_object()) throw std::invalid_argument("plan: expression must be an object");
    if (v.has("type")) e.type = name_of(*v.find("type"), "type", "expression type");
    if (const json::Value *t = v.find("exprType")) {
        // IDL shape
        e.exprType = enum_of(*t, kExpr, 3, "exprType");
        if (v.has("input")) e.input = int_of(*v.find("input"), "input");
        if (v.has("name")) e.name = v.find("name")->as_string();
        if (v.has("op")) e.op = name_of(*v.find("op"), "name", "op");
        if (const json::Value *ops = v.find("operands"))
            for (const auto &o : ops->arr) e.operands.push_back(expr_from(o));
        if (const json::Value *l = v.find("literal")) {
            if (!l->is_object()) throw std::invalid_argument("plan: IDL literal must be an object");
            if (l->has("literalOption")) e.literal.literalOption = enum_of(*l->find("literalOption"), kLit, 2, "literalOption");
            if (l->has("value")) e.literal.value = l->find("value")->as_int();
            if (const json::Value *rs = l->find("rangeSet")) range_set_from(*rs, e.literal);
        }
        return e;
    }
    // RelJson (SycldbJsonConverter.parseExpr, SycldbJsonConverter.java:121-162)
    if (v.has("input")) {
        e.exprType = COLUMN;
        e.input = int_of(*v.find("input"), "input");
        if (v.has("name")) e.name = v.find("name")->as_string();
    } else if (v.has("op")) {
        e.exprType = EXPR;
        e.op = name_of(*v.find("op"), "name", "op");
        const json::Value *ops = v.find("operands");
        if (!ops || !ops->is_array()) throw std::invalid_argument("plan: call \"" + e.op + "\" without operands");
        for (const auto &o : ops->arr) e.operands.push_back(expr_from(o));
    } else {
        e.exprType = LITERAL;
        const json::Value *l = v.find("literal");
        if (!l || l->is_null()) throw std::invalid_argument("plan: NULL literals are not supported");
        if (l->kind == json::Value::Int) {
            e.literal.literalOption = LIT_LITERAL;
            e.literal.value = l->i;
        } else if (l->is_object() && l->find("rangeSet")) {
            range_set_from(*l->find("rangeSet"), e.literal);
        } else {
            throw std::invalid_argument("plan: literal must be an integer or a Sarg with a rangeSet");
        }
    }
    return e;
}

inline std::vector<int64_t> ints_from(const json::Value *v, const char *what)
{
    std::vector<int64_t> out;
    if (v) {
        if (!v->is_array()) throw std::invalid_argument(std::string("plan: ") + what + " must be an array");
        for (const auto &x : v->arr) out.push_back(int_of(x, what));
    }
    return out;
}

// relOp: an IDL name or number, or the planner class that
// SycldbJsonConverter.parseRel maps to it (SycldbJsonConverter.java:36-44).
inline int rel_op_of(const json::Value &v)
{
    static const char *const kRel[] = {"TABLE_SCAN", "FILTER", "JOIN", "PROJECT", "AGGREGATE", "SORT"};
    static const char *const kClass[] = {"com.eurecom.calcite.SycldbTableScan", "com.eurecom.calcite.SycldbFilter",
                                         "com.eurecom.calcite.SycldbJoin",      "com.eurecom.calcite.SycldbProject",
                                         "com.eurecom.calcite.SycldbAggregate", "com.eurecom.calcite.SycldbSort"};
    if (v.is_string())
        for (int i = 0; i < 6; i++)
            if (v.s == kClass[i]) return i;
    return enum_of(v, kRel, 6, "relOp");
}

}  // namespace detail

inline PlanResult plan_from_json(const std::string &text)
{
    static const char *const kDir[] = {"DESCENDING", "ASCENDING"};
    static const char *const kNulls[] = {"FIRST", "LAST"};
    json::Value root = json::parse(text);
    const json::Value *rels = root.find("rels");
    if (!rels || !rels->is_array()) throw std::invalid_argument("plan: missing \"rels\" array");
    PlanResult plan;
    for (const auto &r : rels->arr) {
        RelNode n;
        if (!r.is_object()) throw std::invalid_argument("plan: rel must be an object");
        n.id = r.find("id") ? detail::int_of(*r.find("id"), "id") : (int64_t)plan.rels.size();
        if (!r.find("relOp")) throw std::invalid_argument("plan: rel without relOp");
        n.relOp = detail::rel_op_of(*r.find("relOp"));
        // "tables" in the IDL shape, "table" in RelJson (SycldbJsonConverter.java:50-52)
        const json::Value *t = r.find("tables");
        if (!t) t = r.find("table");
        if (t) {
            if (!t->is_array()) throw std::invalid_argument("plan: tables must be an array");
            for (const auto &x : t->arr) n.tables.push_back(x.as_string());
        }
        n.inputs = detail::ints_from(r.find("inputs"), "inputs");
        if (r.has("condition")) n.condition = detail::expr_from(*r.find("condition"));
        if (r.has("joinType")) n.joinType = r.find("joinType")->as_string();
        if (const json::Value *f = r.find("fields"))
            for (const auto &x : f->arr) n.fields.push_back(x.as_string());
        if (const json::Value *ex = r.find("exprs"))
            for (const auto &x : ex->arr) n.exprs.push_back(detail::expr_from(x));
        n.group = detail::ints_from(r.find("group"), "group");
        if (const json::Value *ag = r.find("aggs"))
            for (const auto &x : ag->arr) {
                AggType a;
                if (x.has("agg")) a.agg = detail::name_of(*x.find("agg"), "name", "agg");
                a.operands = detail::ints_from(x.find("operands"), "agg operands");
                if (x.has("name")) a.name = x.find("name")->as_string();
                if (x.has("type")) a.type = detail::name_of(*x.find("type"), "type", "agg type");
                if (x.has("distinct")) a.distinct = x.find("distinct")->as_bool();
                n.aggs.push_back(a);
            }
        if (const json::Value *co = r.find("collation"))
            for (const auto &x : co->arr) {
                CollationType c;
                if (x.has("field")) c.field = detail::int_of(*x.find("field"), "collation field");
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

namespace detail {

inline void put_str(std::string &o, const std::string &s)
{
    o += '"';
    for (char c : s) {
        if (c == '"' || c == '\\') {
            o += '\\';
            o += c;
        } else if ((unsigned char)c < 0x20) {
            char b[8];
            snprintf(b, sizeof b, "\\u%04x", (unsigned)(unsigned char)c);
            o += b;
        } else {
            o += c;
        }
    }
    o += '"';
}

inline void put_expr(std::string &o, const ExprType &e)
{
    static const char *const kExpr[] = {"LITERAL", "COLUMN", "EXPR"};
    o += "{\"exprType\": \"";
    o += kExpr[e.exprType >= 0 && e.exprType < 3 ? e.exprType : 0];
    o += '"';
    if (e.exprType == COLUMN) {
        o += ", \"input\": " + std::to_string(e.input) + ", \"name\": ";
        put_str(o, e.name);
    } else if (e.exprType == EXPR) {
        o += ", \"op\": ";
        put_str(o, e.op);
        o += ", \"operands\": [";
        for (size_t i = 0; i < e.operands.size(); i++) {
            if (i) o += ", ";
            put_expr(o, e.operands[i]);
        }
        o += ']';
    } else {
        o += ", \"literal\": {\"literalOption\": ";
        if (e.literal.literalOption == LIT_RANGE) {
            o += "\"RANGE\", \"rangeSet\": [";
            for (size_t i = 0; i < e.literal.rangeSet.size(); i++) {
                if (i) o += ", ";
                o += '[';
                for (size_t j = 0; j < e.literal.rangeSet[i].size(); j++) {
                    if (j) o += ", ";
                    put_str(o, e.literal.rangeSet[i][j]);
                }
                o += ']';
            }
            o += "]}";
        } else {
            o += "\"LITERAL\", \"value\": " + std::to_string(e.literal.value) + "}";
        }
    }
    if (!e.type.empty()) {
        o += ", \"type\": ";
        put_str(o, e.type);
    }
    o += '}';
}

inline void put_ints(std::string &o, const std::vector<int64_t> &v)
{
    o += '[';
    for (size_t i = 0; i < v.size(); i++) o += (i ? ", " : "") + std::to_string(v[i]);
    o += ']';
}

}  // namespace detail

// The plan in the IDL shape (the form plans.py builds): every field of every
// rel that its relOp uses, enums by name.
inline std::string plan_to_json(const PlanResult &p)
{
    static const char *const kRel[] = {"TABLE_SCAN", "FILTER", "JOIN", "PROJECT", "AGGREGATE", "SORT"};
    std::string o = "{\"rels\": [";
    for (size_t i = 0; i < p.rels.size(); i++) {
        const RelNode &n = p.rels[i];
        if (i) o += ", ";
        o += "{\"id\": " + std::to_string(n.id) + ", \"relOp\": \"" +
             kRel[n.relOp >= 0 && n.relOp < 6 ? n.relOp : 0] + "\"";
        if (n.relOp == TABLE_SCAN) {
            o += ", \"tables\": [";
            for (size_t j = 0; j < n.tables.size(); j++) {
                if (j) o += ", ";
                detail::put_str(o, n.tables[j]);
            }
            o += ']';
        }
        if (n.relOp == TABLE_SCAN || n.relOp == JOIN) {
            o += ", \"inputs\": ";
            detail::put_ints(o, n.inputs);
        }
        if (n.relOp == FILTER || n.relOp == JOIN) {
            o += ", \"condition\": ";
            detail::put_expr(o, n.condition);
        }
        if (n.relOp == JOIN) {
            o += ", \"joinType\": ";
            detail::put_str(o, n.joinType);
        }
        if (n.relOp == PROJECT) {
            o += ", \"fields\": [";
            for (size_t j = 0; j < n.fields.size(); j++) {
                if (j) o += ", ";
                detail::put_str(o, n.fields[j]);
            }
            o += "], \"exprs\": [";
            for (size_t j = 0; j < n.exprs.size(); j++) {
                if (j) o += ", ";
                detail::put_expr(o, n.exprs[j]);
            }
            o += ']';
        }
        if (n.relOp == AGGREGATE) {
            o += ", \"group\": ";
            detail::put_ints(o, n.group);
            o += ", \"aggs\": [";
            for (size_t j = 0; j < n.aggs.size(); j++) {
                const AggType &a = n.aggs[j];
                if (j) o += ", ";
                o += "{\"agg\": ";
                detail::put_str(o, a.agg);
                o += ", \"operands\": ";
                detail::put_ints(o, a.operands);
                o += ", \"name\": ";
                detail::put_str(o, a.name);
                o += ", \"type\": ";
                detail::put_str(o, a.type);
                o += std::string(", \"distinct\": ") + (a.distinct ? "true" : "false") + "}";
            }
            o += ']';
        }
        if (n.relOp == SORT) {
            o += ", \"collation\": [";
            for (size_t j = 0; j < n.collation.size(); j++) {
                const CollationType &c = n.collation[j];
                if (j) o += ", ";
                o += "{\"field\": " + std::to_string(c.field) + ", \"direction\": \"" +
                     (c.direction == 0 ? "DESCENDING" : "ASCENDING") + "\", \"nulls\": \"" +
                     (c.nulls == 0 ? "FIRST" : "LAST") + "\"}";
            }
            o += ']';
        }
        o += '}';
    }
    o += "]}";
    return o;
}

}  // namespace sdb
