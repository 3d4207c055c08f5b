// Minimal JSON reader for glTF 2.0 documents (RFC 8259: objects, arrays, strings with escapes, numbers,
// true/false/null).  Numbers are kept as double.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace rt {

struct Json {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool has(const std::string& k) const { return type == Object && obj.count(k) != 0; }
    const Json& operator[](const std::string& k) const;   // missing keys give a shared null
    const Json& operator[](size_t i) const;
    size_t size() const { return type == Array ? arr.size() : (type == Object ? obj.size() : 0); }
    double number(double dflt) const { return type == Number ? num : dflt; }
    int64_t integer(int64_t dflt) const { return type == Number ? (int64_t)num : dflt; }
    bool boolean(bool dflt) const { return type == Bool ? b : dflt; }
    const std::string& string(const std::string& dflt) const { return type == String ? str : dflt; }
};

// Parses a whole document; throws Error(REINA_ERR_IO) with the byte offset on malformed input.
Json parse_json(const char* data, size_t size);

}  // namespace rt
