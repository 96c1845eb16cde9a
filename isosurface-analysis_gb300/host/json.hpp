// json.hpp -- a small JSON value with a strict parser and a writer, for the
// module configs (SingleConfig, ScriptingInput, MultiVarConfig) and the
// meta.json run ledger (RunInformation).  Objects keep insertion order, so a
// written ledger lists fields in the same order as the reference's.
#pragma once

#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace isojson {

class Value {
public:
    enum Type { Null, Bool, Number, String, Array, Object };

    Value() : type_(Null) {}
    Value(bool b) : type_(Bool), b_(b) {}
    Value(double d) : type_(Number), d_(d) {}
    Value(int i) : type_(Number), d_(i) {}
    Value(long long i) : type_(Number), d_((double)i) {}
    Value(const char *s) : type_(String), s_(s) {}
    Value(std::string s) : type_(String), s_(std::move(s)) {}
    static Value array() { Value v; v.type_ = Array; return v; }
    static Value object() { Value v; v.type_ = Object; return v; }

    Type type() const { return type_; }
    bool is_null() const { return type_ == Null; }
    bool has(const std::string &k) const
    {
        for (auto &kv : obj_) if (kv.first == k) return true;
        return false;
    }
    const Value &at(const std::string &k) const
    {
        for (auto &kv : obj_) if (kv.first == k) return kv.second;
        throw std::runtime_error("json: missing field '" + k + "'");
    }
    Value &set(const std::string &k, Value v)
    {
        for (auto &kv : obj_)
            if (kv.first == k) { kv.second = std::move(v); return kv.second; }
        obj_.emplace_back(k, std::move(v));
        return obj_.back().second;
    }
    void push(Value v) { arr_.push_back(std::move(v)); }
    const std::vector<Value> &items() const { expect(Array); return arr_; }
    const std::vector<std::pair<std::string, Value>> &fields() const { expect(Object); return obj_; }

    double num() const { expect(Number); return d_; }
    int integer() const { expect(Number); return (int)std::llround(d_); }
    const std::string &str() const { expect(String); return s_; }
    bool boolean() const { expect(Bool); return b_; }

    std::string dump(int indent = 2) const
    {
        std::ostringstream os;
        write(os, indent, 0);
        return os.str();
    }

    static Value parse(const std::string &text)
    {
        size_t pos = 0;
        Value v = parse_value(text, pos);
        skip_ws(text, pos);
        if (pos != text.size()) fail(text, pos, "trailing characters");
        return v;
    }

private:
    Type type_;
    bool b_ = false;
    double d_ = 0;
    std::string s_;
    std::vector<Value> arr_;
    std::vector<std::pair<std::string, Value>> obj_;

    void expect(Type t) const
    {
        if (type_ != t) throw std::runtime_error("json: unexpected value type");
    }

    static void fail(const std::string &t, size_t pos, const char *what)
    {
        size_t line = 1;
        for (size_t i = 0; i < pos && i < t.size(); ++i) line += t[i] == '\n';
        throw std::runtime_error(std::string("json: ") + what + " at line " + std::to_string(line));
    }
    static void skip_ws(const std::string &t, size_t &p)
    {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\n' || t[p] == '\r' || t[p] == '\t')) ++p;
    }
    static Value parse_value(const std::string &t, size_t &p)
    {
        skip_ws(t, p);
        if (p >= t.size()) fail(t, p, "unexpected end");
        char c = t[p];
        if (c == '{') {
            Value v = object();
            ++p;
            skip_ws(t, p);
            if (p < t.size() && t[p] == '}') { ++p; return v; }
            for (;;) {
                skip_ws(t, p);
                if (p >= t.size() || t[p] != '"') fail(t, p, "expected a key");
                std::string k = parse_string(t, p);
                skip_ws(t, p);
                if (p >= t.size() || t[p] != ':') fail(t, p, "expected ':'");
                ++p;
                v.obj_.emplace_back(k, parse_value(t, p));
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',') { ++p; continue; }
                if (p < t.size() && t[p] == '}') { ++p; return v; }
                fail(t, p, "expected ',' or '}'");
            }
        }
        if (c == '[') {
            Value v = array();
            ++p;
            skip_ws(t, p);
            if (p < t.size() && t[p] == ']') { ++p; return v; }
            for (;;) {
                v.arr_.push_back(parse_value(t, p));
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',') { ++p; continue; }
                if (p < t.size() && t[p] == ']') { ++p; return v; }
                fail(t, p, "expected ',' or ']'");
            }
        }
        if (c == '"') return Value(parse_string(t, p));
        if (t.compare(p, 4, "true") == 0) { p += 4; return Value(true); }
        if (t.compare(p, 5, "false") == 0) { p += 5; return Value(false); }
        if (t.compare(p, 4, "null") == 0) { p += 4; return Value(); }
        size_t start = p;
        if (t[p] == '-' || t[p] == '+') ++p;
        while (p < t.size() && (isdigit((unsigned char)t[p]) || t[p] == '.' || t[p] == 'e' || t[p] == 'E' ||
                                t[p] == '-' || t[p] == '+'))
            ++p;
        if (start == p) fail(t, p, "unexpected character");
        char *end = nullptr;
        std::string num = t.substr(start, p - start);
        double d = strtod(num.c_str(), &end);
        if (!end || *end) fail(t, start, "bad number");
        return Value(d);
    }
    static std::string parse_string(const std::string &t, size_t &p)
    {
        std::string out;
        ++p;  // opening quote
        while (p < t.size() && t[p] != '"') {
            char c = t[p++];
            if (c == '\\') {
                if (p >= t.size()) break;
                char e = t[p++];
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    unsigned cp = (unsigned)strtoul(t.substr(p, 4).c_str(), nullptr, 16);
                    p += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                    else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (p >= t.size()) fail(t, p, "unterminated string");
        ++p;
        return out;
    }
    static void write_string(std::ostream &os, const std::string &s)
    {
        os << '"';
        for (char c : s) {
            switch (c) {
            case '"': os << "\\\""; break;
            case '\\': os << "\\\\"; break;
            case '\n': os << "\\n"; break;
            case '\t': os << "\\t"; break;
            case '\r': os << "\\r"; break;
            default: os << c;
            }
        }
        os << '"';
    }
    void write(std::ostream &os, int indent, int level) const
    {
        std::string pad(indent * (level + 1), ' '), pad0(indent * level, ' ');
        const char *nl = indent ? "\n" : "";
        switch (type_) {
        case Null: os << "null"; break;
        case Bool: os << (b_ ? "true" : "false"); break;
        case Number: {
            if (std::isfinite(d_) && d_ == std::floor(d_) && std::fabs(d_) < 9.0e15) {
                os << (long long)d_;
            } else {
                char buf[40];
                snprintf(buf, sizeof buf, "%.9g", d_);
                os << buf;
            }
            break;
        }
        case String: write_string(os, s_); break;
        case Array:
            if (arr_.empty()) { os << "[]"; break; }
            os << "[" << nl;
            for (size_t i = 0; i < arr_.size(); ++i) {
                os << pad;
                arr_[i].write(os, indent, level + 1);
                os << (i + 1 < arr_.size() ? "," : "") << nl;
            }
            os << pad0 << "]";
            break;
        case Object:
            if (obj_.empty()) { os << "{}"; break; }
            os << "{" << nl;
            for (size_t i = 0; i < obj_.size(); ++i) {
                os << pad;
                write_string(os, obj_[i].first);
                os << (indent ? ": " : ":");
                obj_[i].second.write(os, indent, level + 1);
                os << (i + 1 < obj_.size() ? "," : "") << nl;
            }
            os << pad0 << "}";
            break;
        }
    }
};

}  // namespace isojson
