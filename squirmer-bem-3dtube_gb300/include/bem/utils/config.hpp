// config.hpp -- the "key = value" input files of the command-line modes
// (interface of src/utils/config.hpp, which the reference's main.cpp and tests
// call: Config::load, parse_line, has, str, num, integer, list, all).
//
// Input format, as the reference's inputs/*.in use it:
//   * a '#' and everything after it on a line is a comment;
//   * a line without '=' carries no setting;
//   * "key = value" sets key to value (both without surrounding blanks), the
//     first '=' splits the line, a later setting of the same key wins (so
//     command-line "key=value" arguments parsed after the file override it);
//   * a list value holds numbers separated by blanks and/or commas.
// Failures throw std::runtime_error with the reference's wording: "cannot open
// input file: <path>" and "missing required input: <key>".
#pragma once
#include <cstdlib>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

namespace bem {

namespace config_detail {

inline bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n'; }

// the text without leading and trailing blanks
inline std::string_view strip(std::string_view t) {
    size_t b = 0, e = t.size();
    while (b < e && is_blank(t[b])) ++b;
    while (e > b && is_blank(t[e - 1])) --e;
    return t.substr(b, e - b);
}

// every number in a blank- or comma-separated list, up to the first token that
// does not read as a number
inline std::vector<double> numbers(const std::string& text) {
    std::vector<double> out;
    const char* p = text.c_str();
    for (;;) {
        while (*p && (is_blank(*p) || *p == ',')) ++p;
        if (!*p) break;
        char* end = nullptr;
        const double v = std::strtod(p, &end);
        if (end == p) break;
        out.push_back(v);
        p = end;
    }
    return out;
}

}  // namespace config_detail

class Config {
public:
    Config() = default;

    static Config load(const std::string& path) {
        std::ifstream file(path);
        if (!file.is_open()) throw std::runtime_error("cannot open input file: " + path);
        Config cfg;
        std::string line;
        while (std::getline(file, line)) cfg.parse_line(line);
        return cfg;
    }

    void parse_line(std::string line) {
        std::string_view t(line);
        t = t.substr(0, t.find('#'));
        const size_t eq = t.find('=');
        if (eq == std::string_view::npos) return;
        const std::string_view name = config_detail::strip(t.substr(0, eq));
        if (name.empty()) return;
        table_[std::string(name)] = std::string(config_detail::strip(t.substr(eq + 1)));
    }

    bool has(const std::string& key) const { return table_.find(key) != table_.end(); }

    std::string str(const std::string& key, const std::string& fallback = "") const {
        const std::string* v = find(key);
        return v ? *v : fallback;
    }
    double num(const std::string& key, double fallback) const {
        const std::string* v = find(key);
        return v ? std::stod(*v) : fallback;
    }
    double num(const std::string& key) const { return std::stod(required(key)); }
    int integer(const std::string& key, int fallback) const {
        const std::string* v = find(key);
        return v ? std::stoi(*v) : fallback;
    }
    std::vector<double> list(const std::string& key, std::vector<double> fallback = {}) const {
        const std::string* v = find(key);
        return v ? config_detail::numbers(*v) : fallback;
    }
    const std::map<std::string, std::string>& all() const { return table_; }

private:
    std::map<std::string, std::string> table_;

    const std::string* find(const std::string& key) const {
        const auto it = table_.find(key);
        return it == table_.end() ? nullptr : &it->second;
    }
    const std::string& required(const std::string& key) const {
        const std::string* v = find(key);
        if (!v) throw std::runtime_error("missing required input: " + key);
        return *v;
    }
};

}  // namespace bem
