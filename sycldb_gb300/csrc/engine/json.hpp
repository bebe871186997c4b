// Minimal JSON reader for plan text (objects, arrays, strings, integers,
// doubles, true/false/null).  Errors throw std::invalid_argument with the
// byte offset.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace sdb {
namespace json {

struct Value {
    enum Kind { Null, Bool, Int, Double, String, Array, Object } kind = Null;
    bool b = false;
    int64_t i = 0;
    double d = 0;
    std::string s;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;

    bool is_null() const { return kind == Null; }
    bool is_object() const { return kind == Object; }
    bool is_array() const { return kind == Array; }
    bool is_string() const { return kind == String; }
    bool is_number() const { return kind == Int || kind == Double; }

    const Value *find(const std::string &key) const
    {
        if (kind != Object) return nullptr;
        for (const auto &kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    bool has(const std::string &key) const { return find(key) != nullptr && !find(key)->is_null(); }

    int64_t as_int() const
    {
        if (kind == Int) return i;
        if (kind == Double) return (int64_t)d;
        if (kind == Bool) return b ? 1 : 0;
        if (kind == String) return std::stoll(s);
        throw std::invalid_argument("json: expected a number");
    }
    const std::string &as_string() const
    {
        if (kind != String) throw std::invalid_argument("json: expected a string");
        return s;
    }
    bool as_bool() const
    {
        if (kind == Bool) return b;
        if (kind == Int) return i != 0;
        throw std::invalid_argument("json: expected a boolean");
    }
};

class Parser {
public:
    explicit Parser(const std::string &t) : t_(t) {}

    Value parse()
    {
        Value v = value();
        ws();
        if (p_ != t_.size()) fail("trailing characters");
        return v;
    }

private:
    const std::string &t_;
    size_t p_ = 0;

    [[noreturn]] void fail(const char *what)
    {
        throw std::invalid_argument(std::string("json: ") + what + " at offset " + std::to_string(p_));
    }
    void ws()
    {
        while (p_ < t_.size() && (t_[p_] == ' ' || t_[p_] == '\n' || t_[p_] == '\r' || t_[p_] == '\t')) p_++;
    }
    char peek()
    {
        ws();
        if (p_ >= t_.size()) fail("unexpected end");
        return t_[p_];
    }
    void expect(char c)
    {
        if (peek() != c) fail("unexpected character");
        p_++;
    }
    bool lit(const char *w)
    {
        size_t n = std::char_traits<char>::length(w);
        if (t_.compare(p_, n, w) == 0) {
            p_ += n;
            return true;
        }
        return false;
    }

    Value value()
    {
        char c = peek();
        Value v;
        if (c == '{') {
            p_++;
            v.kind = Value::Object;
            if (peek() == '}') { p_++; return v; }
            for (;;) {
                if (peek() != '"') fail("expected a key");
                std::string k = str();
                expect(':');
                Value x = value();
                v.obj.emplace_back(std::move(k), std::move(x));
                char d = peek();
                p_++;
                if (d == '}') break;
                if (d != ',') fail("expected , or }");
            }
        } else if (c == '[') {
            p_++;
            v.kind = Value::Array;
            if (peek() == ']') { p_++; return v; }
            for (;;) {
                v.arr.push_back(value());
                char d = peek();
                p_++;
                if (d == ']') break;
                if (d != ',') fail("expected , or ]");
            }
        } else if (c == '"') {
            v.kind = Value::String;
            v.s = str();
        } else if (lit("true")) {
            v.kind = Value::Bool;
            v.b = true;
        } else if (lit("false")) {
            v.kind = Value::Bool;
        } else if (lit("null")) {
            v.kind = Value::Null;
        } else {
            number(v);
        }
        return v;
    }

    std::string str()
    {
        expect('"');
        std::string out;
        while (p_ < t_.size() && t_[p_] != '"') {
            char c = t_[p_++];
            if (c == '\\') {
                if (p_ >= t_.size()) fail("bad escape");
                char e = t_[p_++];
                switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    if (p_ + 4 > t_.size()) fail("bad \\u escape");
                    unsigned cp = (unsigned)std::strtoul(t_.substr(p_, 4).c_str(), nullptr, 16);
                    p_ += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                    else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: fail("bad escape");
                }
            } else {
                out += c;
            }
        }
        if (p_ >= t_.size()) fail("unterminated string");
        p_++;
        return out;
    }

    void number(Value &v)
    {
        size_t s = p_;
        if (p_ < t_.size() && (t_[p_] == '-' || t_[p_] == '+')) p_++;
        bool is_double = false;
        while (p_ < t_.size()) {
            char c = t_[p_];
            if (c >= '0' && c <= '9') { p_++; continue; }
            if (c == '.' || c == 'e' || c == 'E' || c == '-' || c == '+') { is_double = true; p_++; continue; }
            break;
        }
        if (s == p_) fail("unexpected character");
        std::string num = t_.substr(s, p_ - s);
        if (is_double) {
            v.kind = Value::Double;
            v.d = std::strtod(num.c_str(), nullptr);
        } else {
            v.kind = Value::Int;
            v.i = std::strtoll(num.c_str(), nullptr, 10);
        }
    }
};

inline Value parse(const std::string &text) { return Parser(text).parse(); }

}  // namespace json
}  // namespace sdb
