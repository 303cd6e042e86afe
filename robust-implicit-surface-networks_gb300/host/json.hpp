// Minimal JSON reader and number formatting for the host layer (configs, function files, tet-mesh
// files, mesh.json).  The reference uses nlohmann-json (absent here); this reader covers the
// documents the reference reads: objects, arrays, strings, numbers, booleans and null.
#pragma once
#include <cctype>
#include <charconv>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ria_host {

struct Json {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool contains(const std::string& k) const { return type == Object && obj.count(k) > 0; }
    const Json& operator[](const std::string& k) const {
        auto it = obj.find(k);
        if (type != Object || it == obj.end()) throw std::runtime_error("missing JSON key: " + k);
        return it->second;
    }
    const Json& operator[](size_t i) const {
        if (type != Array || i >= arr.size()) throw std::runtime_error("JSON index out of range");
        return arr[i];
    }
    size_t size() const { return type == Array ? arr.size() : (type == Object ? obj.size() : 0); }
    double as_double() const {
        if (type != Number) throw std::runtime_error("JSON value is not a number");
        return num;
    }
    bool as_bool() const {
        if (type == Bool) return b;
        if (type == Number) return num != 0.0;
        throw std::runtime_error("JSON value is not a boolean");
    }
    const std::string& as_string() const {
        if (type != String) throw std::runtime_error("JSON value is not a string");
        return str;
    }
};

class JsonParser {
   public:
    explicit JsonParser(const std::string& s) : s_(s) {}
    Json parse() {
        Json v = value();
        ws();
        if (p_ != s_.size()) fail("trailing characters");
        return v;
    }

   private:
    const std::string& s_;
    size_t p_ = 0;

    [[noreturn]] void fail(const char* what) {
        throw std::runtime_error(std::string("JSON parse error (") + what + ") at offset " + std::to_string(p_));
    }
    void ws() {
        while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\n' || s_[p_] == '\r' || s_[p_] == '\t')) ++p_;
    }
    bool lit(const char* w) {
        size_t n = std::char_traits<char>::length(w);
        if (s_.compare(p_, n, w) == 0) {
            p_ += n;
            return true;
        }
        return false;
    }
    Json value() {
        ws();
        if (p_ >= s_.size()) fail("unexpected end");
        Json v;
        char c = s_[p_];
        if (c == '{') {
            v.type = Json::Object;
            ++p_;
            ws();
            if (p_ < s_.size() && s_[p_] == '}') {
                ++p_;
                return v;
            }
            for (;;) {
                ws();
                Json k = value();
                if (k.type != Json::String) fail("object key");
                ws();
                if (p_ >= s_.size() || s_[p_] != ':') fail("expected ':'");
                ++p_;
                v.obj[k.str] = value();
                ws();
                if (p_ < s_.size() && s_[p_] == ',') {
                    ++p_;
                    continue;
                }
                if (p_ < s_.size() && s_[p_] == '}') {
                    ++p_;
                    return v;
                }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.type = Json::Array;
            ++p_;
            ws();
            if (p_ < s_.size() && s_[p_] == ']') {
                ++p_;
                return v;
            }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (p_ < s_.size() && s_[p_] == ',') {
                    ++p_;
                    continue;
                }
                if (p_ < s_.size() && s_[p_] == ']') {
                    ++p_;
                    return v;
                }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.type = Json::String;
            ++p_;
            while (p_ < s_.size() && s_[p_] != '"') {
                if (s_[p_] == '\\') {
                    ++p_;
                    if (p_ >= s_.size()) fail("escape");
                    char e = s_[p_];
                    v.str.push_back(e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e);
                } else {
                    v.str.push_back(s_[p_]);
                }
                ++p_;
            }
            if (p_ >= s_.size()) fail("unterminated string");
            ++p_;
            return v;
        }
        if (lit("true")) {
            v.type = Json::Bool;
            v.b = true;
            return v;
        }
        if (lit("false")) {
            v.type = Json::Bool;
            return v;
        }
        if (lit("null")) return v;
        size_t q = p_;
        while (q < s_.size() && (std::isdigit((unsigned char)s_[q]) || s_[q] == '-' || s_[q] == '+' || s_[q] == '.' ||
                                 s_[q] == 'e' || s_[q] == 'E'))
            ++q;
        if (q == p_) fail("unexpected character");
        v.type = Json::Number;
        auto r = std::from_chars(s_.data() + p_, s_.data() + q, v.num);
        if (r.ec != std::errc()) fail("number");
        p_ = q;
        return v;
    }
};

// A double as the reference's JSON library prints it: the shortest round-trip digits d1..dk with
// decimal exponent n (value = 0.d1..dk x 10^n), written
//   d1..dk 0..0 ".0"      if k <= n <= 15
//   d1..dn "." dn+1..dk   if 0 < n <= 15
//   "0." 0..0 d1..dk      if -4 < n <= 0
//   d1 "." d2..dk "e" +-XX   otherwise (exponent n-1, at least two digits; no "." when k = 1)
// and "null" for a NaN or an infinity.  Writes into `out` (room for kJsonDoubleMax characters) and
// returns the end.
constexpr int kJsonDoubleMax = 32;

inline char* json_double_to(char* out, double x) {
    if (x != x || x - x != 0.0) {
        std::memcpy(out, "null", 4);
        return out + 4;
    }
    char sci[40];
    const char* end = std::to_chars(sci, sci + sizeof(sci), x, std::chars_format::scientific).ptr;
    const char* p = sci;
    if (*p == '-') {
        *out++ = '-';
        ++p;
    }
    char digits[24];
    int k = 0;
    for (; *p != 'e'; ++p)
        if (*p != '.') digits[k++] = *p;
    ++p;
    const bool eneg = *p == '-';
    if (*p == '-' || *p == '+') ++p;
    int e10 = 0;
    for (; p < end; ++p) e10 = e10 * 10 + (*p - '0');
    const int n = (eneg ? -e10 : e10) + 1;
    auto put = [&](const char* src, int len) {
        std::memcpy(out, src, (size_t)len);
        out += len;
    };
    if (k == 1 && digits[0] == '0') {
        put("0.0", 3);
    } else if (k <= n && n <= 15) {
        put(digits, k);
        for (int i = k; i < n; ++i) *out++ = '0';
        put(".0", 2);
    } else if (0 < n && n <= 15) {
        put(digits, n);
        *out++ = '.';
        put(digits + n, k - n);
    } else if (-4 < n && n <= 0) {
        put("0.", 2);
        for (int i = 0; i < -n; ++i) *out++ = '0';
        put(digits, k);
    } else {
        *out++ = digits[0];
        if (k > 1) {
            *out++ = '.';
            put(digits + 1, k - 1);
        }
        const int ex = n - 1;
        *out++ = 'e';
        *out++ = ex < 0 ? '-' : '+';
        const int a = ex < 0 ? -ex : ex;
        if (a < 10) *out++ = '0';
        out = std::to_chars(out, out + 4, a).ptr;
    }
    return out;
}

inline std::string json_double(double x) {
    char buf[kJsonDoubleMax];
    return std::string(buf, json_double_to(buf, x));
}

// JSON text under construction: numbers formatted in place, without stream state or temporaries
struct JsonBuf {
    std::string s;
    void c(char ch) { s.push_back(ch); }
    void str(const char* p) { s.append(p); }
    void str(const std::string& p) { s.append(p); }
    void u(uint64_t v) {
        char b[24];
        s.append(b, std::to_chars(b, b + sizeof(b), v).ptr);
    }
    void d(double x) {
        char b[kJsonDoubleMax];
        s.append(b, json_double_to(b, x));
    }
};

}  // namespace ria_host
