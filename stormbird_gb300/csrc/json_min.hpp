// Minimal JSON document reader used by the setup parser.
//
// Stormbird's simulation setup is a serde_json document (stormbird/src/lifting_line/
// simulation_builder.rs:81-88). This header turns such a document into a small DOM of
// tagged values; the schema (field names, defaults, externally tagged enums) is applied
// by sb_setup.hpp. No third-party JSON library is available to the C-ABI library, so the
// grammar of RFC 8259 is implemented directly: objects, arrays, strings with escapes,
// numbers (parsed with strtod), true, false and null.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace sbjson {

struct Value;
using Object = std::vector<std::pair<std::string, Value>>;
using Array = std::vector<Value>;

struct Value {
    enum Kind { Null, Bool, Number, String, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::shared_ptr<Array> arr;
    std::shared_ptr<Object> obj;

    bool is_null() const { return kind == Null; }
    bool is_obj() const { return kind == Obj; }
    bool is_arr() const { return kind == Arr; }
    bool is_str() const { return kind == String; }
    bool is_num() const { return kind == Number; }
    bool is_bool() const { return kind == Bool; }
};

struct ParseError : std::runtime_error {
    explicit ParseError(const std::string& m) : std::runtime_error(m) {}
};

class Parser {
public:
    explicit Parser(const std::string& text) : s_(text), i_(0) {}

    Value parse_document() {
        skip_ws();
        Value v = parse_value(0);
        skip_ws();
        if (i_ != s_.size()) fail("trailing characters after the JSON document");
        return v;
    }

private:
    const std::string& s_;
    size_t i_;

    [[noreturn]] void fail(const std::string& what) const {
        throw ParseError("JSON parse error at offset " + std::to_string(i_) + ": " + what);
    }

    void skip_ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\n' || s_[i_] == '\r' || s_[i_] == '\t')) ++i_;
    }

    bool consume(char c) {
        skip_ws();
        if (i_ < s_.size() && s_[i_] == c) { ++i_; return true; }
        return false;
    }

    void expect(char c) {
        if (!consume(c)) fail(std::string("expected '") + c + "'");
    }

    Value parse_value(int depth) {
        if (depth > 256) fail("nesting too deep");
        skip_ws();
        if (i_ >= s_.size()) fail("unexpected end of input");
        char c = s_[i_];
        Value v;
        if (c == '{') {
            ++i_;
            v.kind = Value::Obj;
            v.obj = std::make_shared<Object>();
            if (consume('}')) return v;
            do {
                skip_ws();
                if (i_ >= s_.size() || s_[i_] != '"') fail("expected object key");
                std::string key = parse_string();
                expect(':');
                Value item = parse_value(depth + 1);
                v.obj->emplace_back(std::move(key), std::move(item));
            } while (consume(','));
            expect('}');
        } else if (c == '[') {
            ++i_;
            v.kind = Value::Arr;
            v.arr = std::make_shared<Array>();
            if (consume(']')) return v;
            do {
                v.arr->push_back(parse_value(depth + 1));
            } while (consume(','));
            expect(']');
        } else if (c == '"') {
            v.kind = Value::String;
            v.str = parse_string();
        } else if (c == 't') {
            literal("true");
            v.kind = Value::Bool;
            v.b = true;
        } else if (c == 'f') {
            literal("false");
            v.kind = Value::Bool;
            v.b = false;
        } else if (c == 'n') {
            literal("null");
            v.kind = Value::Null;
        } else if (c == '-' || (c >= '0' && c <= '9')) {
            v.kind = Value::Number;
            v.num = parse_number();
        } else {
            fail(std::string("unexpected character '") + c + "'");
        }
        return v;
    }

    void literal(const char* word) {
        size_t n = 0;
        while (word[n]) ++n;
        if (s_.compare(i_, n, word) != 0) fail(std::string("expected ") + word);
        i_ += n;
    }

    double parse_number() {
        size_t start = i_;
        if (s_[i_] == '-') ++i_;
        auto digits = [&]() {
            size_t d0 = i_;
            while (i_ < s_.size() && s_[i_] >= '0' && s_[i_] <= '9') ++i_;
            if (i_ == d0) fail("malformed number");
        };
        digits();
        if (i_ < s_.size() && s_[i_] == '.') { ++i_; digits(); }
        if (i_ < s_.size() && (s_[i_] == 'e' || s_[i_] == 'E')) {
            ++i_;
            if (i_ < s_.size() && (s_[i_] == '+' || s_[i_] == '-')) ++i_;
            digits();
        }
        std::string tok = s_.substr(start, i_ - start);
        char* end = nullptr;
        double d = std::strtod(tok.c_str(), &end);
        if (end == tok.c_str()) fail("malformed number");
        return d;
    }

    static void append_utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) {
            out.push_back(static_cast<char>(cp));
        } else if (cp < 0x800) {
            out.push_back(static_cast<char>(0xC0 | (cp >> 6)));
            out.push_back(static_cast<char>(0x80 | (cp & 0x3F)));
        } else if (cp < 0x10000) {
            out.push_back(static_cast<char>(0xE0 | (cp >> 12)));
            out.push_back(static_cast<char>(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back(static_cast<char>(0x80 | (cp & 0x3F)));
        } else {
            out.push_back(static_cast<char>(0xF0 | (cp >> 18)));
            out.push_back(static_cast<char>(0x80 | ((cp >> 12) & 0x3F)));
            out.push_back(static_cast<char>(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back(static_cast<char>(0x80 | (cp & 0x3F)));
        }
    }

    uint32_t hex4() {
        if (i_ + 4 > s_.size()) fail("truncated \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; ++k) {
            char c = s_[i_++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= static_cast<uint32_t>(c - '0');
            else if (c >= 'a' && c <= 'f') v |= static_cast<uint32_t>(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= static_cast<uint32_t>(c - 'A' + 10);
            else fail("bad hex digit in \\u escape");
        }
        return v;
    }

    std::string parse_string() {
        // caller guarantees s_[i_] == '"'
        ++i_;
        std::string out;
        while (true) {
            if (i_ >= s_.size()) fail("unterminated string");
            char c = s_[i_++];
            if (c == '"') break;
            if (c != '\\') { out.push_back(c); continue; }
            if (i_ >= s_.size()) fail("unterminated escape");
            char e = s_[i_++];
            switch (e) {
                case '"': out.push_back('"'); break;
                case '\\': out.push_back('\\'); break;
                case '/': out.push_back('/'); break;
                case 'b': out.push_back('\b'); break;
                case 'f': out.push_back('\f'); break;
                case 'n': out.push_back('\n'); break;
                case 'r': out.push_back('\r'); break;
                case 't': out.push_back('\t'); break;
                case 'u': {
                    uint32_t cp = hex4();
                    if (cp >= 0xD800 && cp <= 0xDBFF) {
                        if (i_ + 2 <= s_.size() && s_[i_] == '\\' && s_[i_ + 1] == 'u') {
                            i_ += 2;
                            uint32_t lo = hex4();
                            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                        }
                    }
                    append_utf8(out, cp);
                    break;
                }
                default: fail("unknown escape");
            }
        }
        return out;
    }
};

inline Value parse(const std::string& text) { return Parser(text).parse_document(); }

// Serialises a value back to JSON text: numbers with 17 significant digits (they parse back
// to the same double), strings with the escapes the parser reads.
inline void dump_to(const Value& v, std::string& out) {
    switch (v.kind) {
        case Value::Null: out += "null"; return;
        case Value::Bool: out += v.b ? "true" : "false"; return;
        case Value::Number: {
            char buf[40];
            std::snprintf(buf, sizeof(buf), "%.17g", v.num);
            out += buf;
            return;
        }
        case Value::String: {
            out += '"';
            for (unsigned char c : v.str) {
                if (c == '"') out += "\\\"";
                else if (c == '\\') out += "\\\\";
                else if (c < 0x20) {
                    char buf[8];
                    std::snprintf(buf, sizeof(buf), "\\u%04x", c);
                    out += buf;
                } else out += static_cast<char>(c);
            }
            out += '"';
            return;
        }
        case Value::Arr: {
            out += '[';
            for (size_t i = 0; i < v.arr->size(); ++i) {
                if (i) out += ',';
                dump_to((*v.arr)[i], out);
            }
            out += ']';
            return;
        }
        case Value::Obj: {
            out += '{';
            for (size_t i = 0; i < v.obj->size(); ++i) {
                if (i) out += ',';
                Value key;
                key.kind = Value::String;
                key.str = (*v.obj)[i].first;
                dump_to(key, out);
                out += ':';
                dump_to((*v.obj)[i].second, out);
            }
            out += '}';
            return;
        }
    }
}
inline std::string dump(const Value& v) {
    std::string s;
    dump_to(v, s);
    return s;
}

}  // namespace sbjson
