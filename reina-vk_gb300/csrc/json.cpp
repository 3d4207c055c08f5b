// Minimal JSON reader (see json.h).
#include "json.h"

#include <cstdlib>
#include <cstring>

#include "errors.h"

namespace rt {

namespace {

const Json& null_json() {
    static const Json j;
    return j;
}

struct Parser {
    const char* p;
    const char* end;
    const char* begin;
    int depth = 0;

    [[noreturn]] void bad(const char* what) const {
        fail(REINA_ERR_IO, std::string("JSON: ") + what + " at byte " + std::to_string(p - begin));
    }
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool lit(const char* s) {
        const size_t n = std::strlen(s);
        if ((size_t)(end - p) >= n && std::memcmp(p, s, n) == 0) {
            p += n;
            return true;
        }
        return false;
    }
    static void put_utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) {
            out += (char)cp;
        } else if (cp < 0x800) {
            out += (char)(0xC0 | (cp >> 6));
            out += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += (char)(0xE0 | (cp >> 12));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        } else {
            out += (char)(0xF0 | (cp >> 18));
            out += (char)(0x80 | ((cp >> 12) & 0x3F));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        }
    }
    uint32_t hex4() {
        if (end - p < 4) bad("truncated \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; ++k) {
            const char c = *p++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else bad("bad \\u escape");
        }
        return v;
    }
    std::string string() {
        ++p;   // opening quote
        std::string out;
        while (true) {
            if (p >= end) bad("unterminated string");
            const char c = *p++;
            if (c == '"') break;
            if ((unsigned char)c < 0x20) bad("control character in string");
            if (c != '\\') {
                out += c;
                continue;
            }
            if (p >= end) bad("unterminated escape");
            const char e = *p++;
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
                    if (cp >= 0xD800 && cp < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                        p += 2;
                        const uint32_t lo = hex4();
                        if (lo >= 0xDC00 && lo < 0xE000) cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    put_utf8(out, cp);
                    break;
                }
                default: bad("bad escape");
            }
        }
        return out;
    }
    Json value() {
        if (++depth > 512) bad("nesting too deep");
        ws();
        if (p >= end) bad("unexpected end");
        Json j;
        const char c = *p;
        if (c == '{') {
            j.type = Json::Object;
            ++p;
            ws();
            if (p < end && *p == '}') {
                ++p;
            } else {
                while (true) {
                    ws();
                    if (p >= end || *p != '"') bad("expected a key");
                    std::string k = string();
                    ws();
                    if (p >= end || *p != ':') bad("expected ':'");
                    ++p;
                    j.obj[k] = value();
                    ws();
                    if (p < end && *p == ',') { ++p; continue; }
                    if (p < end && *p == '}') { ++p; break; }
                    bad("expected ',' or '}'");
                }
            }
        } else if (c == '[') {
            j.type = Json::Array;
            ++p;
            ws();
            if (p < end && *p == ']') {
                ++p;
            } else {
                while (true) {
                    j.arr.push_back(value());
                    ws();
                    if (p < end && *p == ',') { ++p; continue; }
                    if (p < end && *p == ']') { ++p; break; }
                    bad("expected ',' or ']'");
                }
            }
        } else if (c == '"') {
            j.type = Json::String;
            j.str = string();
        } else if (lit("true")) {
            j.type = Json::Bool;
            j.b = true;
        } else if (lit("false")) {
            j.type = Json::Bool;
        } else if (lit("null")) {
            j.type = Json::Null;
        } else if (c == '-' || (c >= '0' && c <= '9')) {
            std::string tok;
            while (p < end && (std::strchr("+-.eE", *p) || (*p >= '0' && *p <= '9'))) tok += *p++;
            char* stop = nullptr;
            j.type = Json::Number;
            j.num = std::strtod(tok.c_str(), &stop);
            if (stop != tok.c_str() + tok.size()) bad("malformed number");
        } else {
            bad("unexpected character");
        }
        --depth;
        return j;
    }
};

}  // namespace

const Json& Json::operator[](const std::string& k) const {
    if (type != Object) return null_json();
    auto it = obj.find(k);
    return it == obj.end() ? null_json() : it->second;
}

const Json& Json::operator[](size_t i) const {
    return (type == Array && i < arr.size()) ? arr[i] : null_json();
}

Json parse_json(const char* data, size_t size) {
    Parser ps{data, data + size, data};
    Json j = ps.value();
    ps.ws();
    if (ps.p != ps.end) ps.bad("trailing characters");
    return j;
}

}  // namespace rt
