// Minimal JSON reader/writer for the reference's scene, mesh and result files (include/assembly.h:885-935,
// cpp/grid.cpp:9-78, include/assembly.h:953-978).  Numbers are kept as double.
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace nsfhost {

struct Json {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool has(const std::string& k) const { return type == Object && obj.count(k) != 0; }
    const Json& operator[](const std::string& k) const;
    const Json& operator[](size_t i) const { return arr.at(i); }
    size_t size() const { return type == Array ? arr.size() : type == Object ? obj.size() : 0; }
    bool is_number() const { return type == Number; }
    bool is_string() const { return type == String; }
};

// Throws std::runtime_error with the byte offset on malformed input.
Json parse_json(const std::string& text);
Json parse_json_file(const std::string& path);

// Shortest round-trip text of a double, with ".0" appended to integral values (the way nlohmann::json prints).
std::string json_number(double v);

}  // namespace nsfhost
