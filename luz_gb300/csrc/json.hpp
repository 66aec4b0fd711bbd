// json.hpp — a small JSON DOM for the scene files (.luz projects, glTF): parse and
// write. Integers that fit in 64 bits keep every digit (the .luz format stores
// 62-bit UUIDs as plain JSON integers); other numbers are doubles. Object members
// keep their order of appearance; lookups are linear (objects here are small).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace luz {
namespace json {

struct Value {
    enum Kind { Null, Bool, Int, UInt, Real, String, Array, Object } kind = Null;
    bool b = false;
    int64_t i = 0;       // Int (negative)
    uint64_t u = 0;      // UInt (non-negative integer)
    double d = 0.0;      // Real
    std::string s;
    std::vector<Value> items;                              // Array
    std::vector<std::pair<std::string, Value>> members;    // Object

    static Value object() { Value v; v.kind = Object; return v; }
    static Value array() { Value v; v.kind = Array; return v; }
    static Value of(double x) { Value v; v.kind = Real; v.d = x; return v; }
    static Value of_u64(uint64_t x) { Value v; v.kind = UInt; v.u = x; return v; }
    static Value of_i64(int64_t x) {
        Value v;
        if (x >= 0) { v.kind = UInt; v.u = (uint64_t)x; } else { v.kind = Int; v.i = x; }
        return v;
    }
    static Value of_bool(bool x) { Value v; v.kind = Bool; v.b = x; return v; }
    static Value of_str(std::string x) { Value v; v.kind = String; v.s = std::move(x); return v; }

    bool is_num() const { return kind == Int || kind == UInt || kind == Real; }
    bool is_obj() const { return kind == Object; }
    bool is_arr() const { return kind == Array; }

    const Value* find(const char* key) const {
        if (kind != Object) return nullptr;
        for (const auto& m : members)
            if (m.first == key) return &m.second;
        return nullptr;
    }
    bool has(const char* key) const { return find(key) != nullptr; }
    const Value& at(const char* key) const {
        const Value* v = find(key);
        if (!v) throw std::runtime_error(std::string("missing field '") + key + "'");
        return *v;
    }
    Value& set(const std::string& key, Value v) {
        for (auto& m : members)
            if (m.first == key) { m.second = std::move(v); return m.second; }
        members.emplace_back(key, std::move(v));
        return members.back().second;
    }
    Value& push(Value v) { items.push_back(std::move(v)); return items.back(); }

    double num() const {
        switch (kind) {
            case Int: return (double)i;
            case UInt: return (double)u;
            case Real: return d;
            case Bool: return b ? 1.0 : 0.0;
            default: throw std::runtime_error("number expected");
        }
    }
    float f32() const { return (float)num(); }
    // Integers: a value the target type cannot hold (negative for u64, beyond the
    // range, NaN) is an error, not a wrapped or undefined conversion.
    int64_t i64() const {
        switch (kind) {
            case Int: return i;
            case UInt:
                if (u > (uint64_t)INT64_MAX) throw std::runtime_error("integer out of range");
                return (int64_t)u;
            case Real:
                if (!(d >= -0x1p63 && d < 0x1p63)) throw std::runtime_error("integer out of range");
                return (int64_t)d;
            case Bool: return b ? 1 : 0;
            default: throw std::runtime_error("integer expected");
        }
    }
    uint64_t u64() const {
        switch (kind) {
            case UInt: return u;
            case Int:
                if (i < 0) throw std::runtime_error("non-negative integer expected");
                return (uint64_t)i;
            case Real:
                if (!(d >= 0.0 && d < 0x1p64)) throw std::runtime_error("non-negative integer expected");
                return (uint64_t)d;
            default: throw std::runtime_error("integer expected");
        }
    }
    const std::string& str() const {
        if (kind != String) throw std::runtime_error("string expected");
        return s;
    }
    size_t size() const { return kind == Array ? items.size() : kind == Object ? members.size() : 0; }
    const Value& operator[](size_t k) const { return items.at(k); }
};

class Parser {
public:
    Parser(const char* p, size_t n) : p_(p), end_(p + n) {}
    Value parse() {
        Value v = value(0);
        ws();
        if (p_ != end_) fail("trailing characters");
        return v;
    }

private:
    const char* p_;
    const char* end_;

    [[noreturn]] void fail(const char* what) { throw std::runtime_error(std::string("JSON: ") + what); }
    void ws() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool lit(const char* w) {
        size_t n = strlen(w);
        if ((size_t)(end_ - p_) >= n && memcmp(p_, w, n) == 0) { p_ += n; return true; }
        return false;
    }
    Value value(int depth) {
        if (depth > 256) fail("nesting too deep");
        ws();
        if (p_ >= end_) fail("unexpected end");
        char c = *p_;
        if (c == '{') return object(depth);
        if (c == '[') return array(depth);
        if (c == '"') { Value v; v.kind = Value::String; v.s = string(); return v; }
        if (lit("true")) return Value::of_bool(true);
        if (lit("false")) return Value::of_bool(false);
        if (lit("null")) return Value();
        return number();
    }
    Value object(int depth) {
        ++p_;
        Value v = Value::object();
        ws();
        if (p_ < end_ && *p_ == '}') { ++p_; return v; }
        for (;;) {
            ws();
            if (p_ >= end_ || *p_ != '"') fail("member name expected");
            std::string k = string();
            ws();
            if (p_ >= end_ || *p_ != ':') fail("':' expected");
            ++p_;
            v.members.emplace_back(std::move(k), value(depth + 1));
            ws();
            if (p_ < end_ && *p_ == ',') { ++p_; continue; }
            if (p_ < end_ && *p_ == '}') { ++p_; return v; }
            fail("',' or '}' expected");
        }
    }
    Value array(int depth) {
        ++p_;
        Value v = Value::array();
        ws();
        if (p_ < end_ && *p_ == ']') { ++p_; return v; }
        for (;;) {
            v.items.push_back(value(depth + 1));
            ws();
            if (p_ < end_ && *p_ == ',') { ++p_; continue; }
            if (p_ < end_ && *p_ == ']') { ++p_; return v; }
            fail("',' or ']' expected");
        }
    }
    static void utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) out += (char)cp;
        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
        else if (cp < 0x10000) {
            out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F));
        } else {
            out += (char)(0xF0 | (cp >> 18)); out += (char)(0x80 | ((cp >> 12) & 0x3F));
            out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F));
        }
    }
    uint32_t hex4() {
        if (end_ - p_ < 4) fail("bad \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; ++k) {
            char c = *p_++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else fail("bad \\u escape");
        }
        return v;
    }
    std::string string() {
        ++p_;
        std::string out;
        while (p_ < end_ && *p_ != '"') {
            char c = *p_++;
            if (c != '\\') { out += c; continue; }
            if (p_ >= end_) fail("bad escape");
            char e = *p_++;
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
                    uint32_t cp = hex4();
                    if (cp >= 0xD800 && cp < 0xDC00 && end_ - p_ >= 6 && p_[0] == '\\' && p_[1] == 'u') {
                        p_ += 2;
                        uint32_t lo = hex4();
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(out, cp);
                    break;
                }
                default: fail("bad escape");
            }
        }
        if (p_ >= end_) fail("unterminated string");
        ++p_;
        return out;
    }
    Value number() {
        const char* s = p_;
        bool neg = false, integral = true;
        if (p_ < end_ && *p_ == '-') { neg = true; ++p_; }
        if (p_ >= end_ || !(*p_ >= '0' && *p_ <= '9')) fail("number expected");
        while (p_ < end_ && *p_ >= '0' && *p_ <= '9') ++p_;
        if (p_ < end_ && *p_ == '.') {
            integral = false;
            ++p_;
            while (p_ < end_ && *p_ >= '0' && *p_ <= '9') ++p_;
        }
        if (p_ < end_ && (*p_ == 'e' || *p_ == 'E')) {
            integral = false;
            ++p_;
            if (p_ < end_ && (*p_ == '+' || *p_ == '-')) ++p_;
            while (p_ < end_ && *p_ >= '0' && *p_ <= '9') ++p_;
        }
        std::string tok(s, p_);
        if (integral) {
            // exact 64-bit integers; fall back to double beyond that range
            const char* digits = tok.c_str() + (neg ? 1 : 0);
            uint64_t acc = 0;
            bool overflow = false;
            for (const char* q = digits; *q; ++q) {
                uint64_t dgt = (uint64_t)(*q - '0');
                if (acc > (UINT64_MAX - dgt) / 10) { overflow = true; break; }
                acc = acc * 10 + dgt;
            }
            if (!overflow) {
                if (!neg) return Value::of_u64(acc);
                if (acc <= (uint64_t)INT64_MAX + 1) {
                    Value v;
                    v.kind = acc == 0 ? Value::UInt : Value::Int;
                    v.i = acc == 0 ? 0 : (int64_t)(0 - acc);
                    return v;
                }
            }
        }
        return Value::of(strtod(tok.c_str(), nullptr));
    }
};

inline Value parse(const std::string& text) { return Parser(text.data(), text.size()).parse(); }

// Writes numbers so that a float32 read back is the same float: 9 significant digits
// for values that are floats, 17 for other doubles; integers exactly.
inline void write_number(std::string& out, double d) {
    char buf[40];
    if (std::isfinite(d) && d == std::floor(d) && std::fabs(d) < 9.007199254740992e15) {
        snprintf(buf, sizeof buf, "%.1f", d);
    } else if (std::isfinite(d) && (double)(float)d == d) {
        snprintf(buf, sizeof buf, "%.9g", d);
    } else if (std::isfinite(d)) {
        snprintf(buf, sizeof buf, "%.17g", d);
    } else {
        snprintf(buf, sizeof buf, "null");
    }
    out += buf;
}

inline void write_string(std::string& out, const std::string& s) {
    out += '"';
    for (unsigned char c : s) {
        switch (c) {
            case '"': out += "\\\""; break;
            case '\\': out += "\\\\"; break;
            case '\n': out += "\\n"; break;
            case '\r': out += "\\r"; break;
            case '\t': out += "\\t"; break;
            default:
                if (c < 0x20) {
                    char b[8];
                    snprintf(b, sizeof b, "\\u%04x", c);
                    out += b;
                } else {
                    out += (char)c;
                }
        }
    }
    out += '"';
}

inline void write(std::string& out, const Value& v) {
    switch (v.kind) {
        case Value::Null: out += "null"; break;
        case Value::Bool: out += v.b ? "true" : "false"; break;
        case Value::Int: out += std::to_string(v.i); break;
        case Value::UInt: out += std::to_string(v.u); break;
        case Value::Real: write_number(out, v.d); break;
        case Value::String: write_string(out, v.s); break;
        case Value::Array:
            out += '[';
            for (size_t k = 0; k < v.items.size(); ++k) {
                if (k) out += ',';
                write(out, v.items[k]);
            }
            out += ']';
            break;
        case Value::Object:
            out += '{';
            for (size_t k = 0; k < v.members.size(); ++k) {
                if (k) out += ',';
                write_string(out, v.members[k].first);
                out += ':';
                write(out, v.members[k].second);
            }
            out += '}';
            break;
    }
}

inline std::string dump(const Value& v) {
    std::string out;
    write(out, v);
    return out;
}

}  // namespace json
}  // namespace luz
