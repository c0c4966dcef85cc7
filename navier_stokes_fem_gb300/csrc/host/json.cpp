#include "json.h"

#include <charconv>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace nsfhost {

const Json& Json::operator[](const std::string& k) const {
    static const Json null;
    if (type != Object) return null;
    auto it = obj.find(k);
    return it == obj.end() ? null : it->second;
}

namespace {

struct Parser {
    const char* p;
    const char* begin;
    const char* end;

    [[noreturn]] void fail(const char* what) {
        throw std::runtime_error(std::string("JSON parse error at byte ") + std::to_string(p - begin) + ": " + what);
    }
    void ws() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    bool lit(const char* s) {
        const size_t n = strlen(s);
        if ((size_t)(end - p) >= n && memcmp(p, s, n) == 0) { p += n; return true; }
        return false;
    }
    std::string string() {
        if (*p != '"') fail("expected string");
        ++p;
        std::string out;
        while (p < end && *p != '"') {
            if (*p == '\\') {
                ++p;
                if (p >= end) fail("bad escape");
                switch (*p) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (end - p < 5) fail("bad \\u escape");
                        const unsigned cp = (unsigned)strtoul(std::string(p + 1, p + 5).c_str(), nullptr, 16);
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                        p += 4;
                        break;
                    }
                    default: out += *p;
                }
                ++p;
            } else {
                out += *p++;
            }
        }
        if (p >= end) fail("unterminated string");
        ++p;
        return out;
    }
    Json value() {
        ws();
        if (p >= end) fail("unexpected end");
        Json j;
        if (*p == '{') {
            ++p;
            j.type = Json::Object;
            ws();
            if (*p == '}') { ++p; return j; }
            while (true) {
                ws();
                std::string k = string();
                ws();
                if (*p != ':') fail("expected ':'");
                ++p;
                j.obj[k] = value();
                ws();
                if (*p == ',') { ++p; continue; }
                if (*p == '}') { ++p; break; }
                fail("expected ',' or '}'");
            }
        } else if (*p == '[') {
            ++p;
            j.type = Json::Array;
            ws();
            if (*p == ']') { ++p; return j; }
            while (true) {
                j.arr.push_back(value());
                ws();
                if (*p == ',') { ++p; continue; }
                if (*p == ']') { ++p; break; }
                fail("expected ',' or ']'");
            }
        } else if (*p == '"') {
            j.type = Json::String;
            j.str = string();
        } else if (lit("true")) {
            j.type = Json::Bool; j.b = true;
        } else if (lit("false")) {
            j.type = Json::Bool; j.b = false;
        } else if (lit("null")) {
            j.type = Json::Null;
        } else {
            char* e = nullptr;
            j.num = strtod(p, &e);
            if (e == p) fail("unexpected character");
            j.type = Json::Number;
            p = e;
        }
        return j;
    }
};

}  // namespace

Json parse_json(const std::string& text) {
    Parser ps{text.data(), text.data(), text.data() + text.size()};
    Json j = ps.value();
    ps.ws();
    if (ps.p != ps.end) ps.fail("trailing characters");
    return j;
}

Json parse_json_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("Cannot open JSON file: " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return parse_json(ss.str());
}

std::string json_number(double v) {
    char buf[64];
    auto res = std::to_chars(buf, buf + sizeof(buf), v);
    std::string s(buf, res.ptr);
    if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
    return s;
}

}  // namespace nsfhost
