// Minimal JSON reader for Lumen scene files (the subset RFC 8259 describes: objects, arrays, strings with
// the standard escapes, numbers, true/false/null). Enough for the keys LumenScene::load_lumen_scene reads
// (src/RayTracer/LumenScene.cpp:231-513); written here because the reference's vendored parser is not ours.
#pragma once
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace lgbh {

struct Json {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool is_null() const { return type == Null; }
    // obj[key] that yields a null value for absent keys (Lumen's loader tests `.is_null()` the same way)
    const Json& operator[](const std::string& key) const {
        static const Json null_value;
        if (type != Object) return null_value;
        auto it = obj.find(key);
        return it == obj.end() ? null_value : it->second;
    }
    const Json& operator[](size_t i) const {
        static const Json null_value;
        return (type == Array && i < arr.size()) ? arr[i] : null_value;
    }
    size_t size() const { return type == Array ? arr.size() : (type == Object ? obj.size() : 0); }
    double as_number() const {
        if (type == Number) return num;
        if (type == Bool) return b ? 1.0 : 0.0;
        throw std::runtime_error("JSON value is not a number");
    }
    float f(float def) const { return is_null() ? def : (float)as_number(); }
    const std::string& as_string() const {
        if (type != String) throw std::runtime_error("JSON value is not a string");
        return str;
    }
};

class JsonParser {
  public:
    explicit JsonParser(const std::string& text) : s_(text) {}
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
        throw std::runtime_error(std::string("JSON parse error at offset ") + std::to_string(p_) + ": " + what);
    }
    void ws() {
        while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\n' || s_[p_] == '\r')) p_++;
    }
    bool eat(char c) {
        ws();
        if (p_ < s_.size() && s_[p_] == c) { p_++; return true; }
        return false;
    }
    Json value() {
        ws();
        if (p_ >= s_.size()) fail("unexpected end");
        char c = s_[p_];
        if (c == '{') return object();
        if (c == '[') return array();
        if (c == '"') { Json j; j.type = Json::String; j.str = string(); return j; }
        if (c == 't' || c == 'f' || c == 'n') return literal();
        return number();
    }
    Json object() {
        Json j;
        j.type = Json::Object;
        p_++;
        if (eat('}')) return j;
        do {
            ws();
            if (p_ >= s_.size() || s_[p_] != '"') fail("expected a key");
            std::string k = string();
            if (!eat(':')) fail("expected ':'");
            j.obj[k] = value();
        } while (eat(','));
        if (!eat('}')) fail("expected '}'");
        return j;
    }
    Json array() {
        Json j;
        j.type = Json::Array;
        p_++;
        if (eat(']')) return j;
        do {
            j.arr.push_back(value());
        } while (eat(','));
        if (!eat(']')) fail("expected ']'");
        return j;
    }
    std::string string() {
        std::string out;
        p_++;  // opening quote
        while (p_ < s_.size() && s_[p_] != '"') {
            char c = s_[p_++];
            if (c == '\\') {
                if (p_ >= s_.size()) fail("bad escape");
                char e = s_[p_++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (p_ + 4 > s_.size()) fail("bad \\u escape");
                        unsigned cp = (unsigned)std::strtoul(s_.substr(p_, 4).c_str(), nullptr, 16);
                        p_ += 4;
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
        if (p_ >= s_.size()) fail("unterminated string");
        p_++;
        return out;
    }
    Json literal() {
        Json j;
        if (s_.compare(p_, 4, "true") == 0) { j.type = Json::Bool; j.b = true; p_ += 4; }
        else if (s_.compare(p_, 5, "false") == 0) { j.type = Json::Bool; j.b = false; p_ += 5; }
        else if (s_.compare(p_, 4, "null") == 0) { p_ += 4; }
        else fail("bad literal");
        return j;
    }
    Json number() {
        const char* start = s_.c_str() + p_;
        char* end = nullptr;
        double v = std::strtod(start, &end);
        if (end == start) fail("bad number");
        p_ += (size_t)(end - start);
        Json j;
        j.type = Json::Number;
        j.num = v;
        return j;
    }
};

inline Json parse_json(const std::string& text) { return JsonParser(text).parse(); }

}  // namespace lgbh
