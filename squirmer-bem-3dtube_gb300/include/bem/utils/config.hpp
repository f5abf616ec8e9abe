// config.hpp -- "key = value" input files, drop-in for src/utils/config.hpp:19-70.
//
// Format: "#" starts a comment, "key = value" sets a key (keys and values are
// trimmed), list values are separated by commas or whitespace; values given on
// the command line as key=value override the file.  Same member functions and
// error messages as the reference.
#pragma once
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace bem {

class Config {
public:
    Config() = default;

    static Config load(const std::string& path) {
        std::ifstream in(path);
        if (!in) throw std::runtime_error("cannot open input file: " + path);
        Config c;
        for (std::string line; std::getline(in, line);) c.parse_line(line);
        return c;
    }
    void parse_line(std::string line) {
        const auto hash = line.find('#');
        if (hash != std::string::npos) line.erase(hash);
        const auto eq = line.find('=');
        if (eq == std::string::npos) return;
        const std::string key = trim(line.substr(0, eq));
        if (!key.empty()) values_[key] = trim(line.substr(eq + 1));
    }
    bool has(const std::string& k) const { return values_.count(k) != 0; }
    std::string str(const std::string& k, const std::string& def = "") const {
        const auto it = values_.find(k);
        return it == values_.end() ? def : it->second;
    }
    double num(const std::string& k, double def) const { return has(k) ? std::stod(values_.at(k)) : def; }
    double num(const std::string& k) const {
        if (!has(k)) throw std::runtime_error("missing required input: " + k);
        return std::stod(values_.at(k));
    }
    int integer(const std::string& k, int def) const { return has(k) ? std::stoi(values_.at(k)) : def; }
    std::vector<double> list(const std::string& k, std::vector<double> def = {}) const {
        if (!has(k)) return def;
        std::string s = values_.at(k);
        for (char& ch : s)
            if (ch == ',') ch = ' ';
        std::istringstream is(s);
        std::vector<double> out;
        for (double x; is >> x;) out.push_back(x);
        return out;
    }
    const std::map<std::string, std::string>& all() const { return values_; }

private:
    std::map<std::string, std::string> values_;
    static std::string trim(const std::string& s) {
        const auto b = s.find_first_not_of(" \t\r\n");
        if (b == std::string::npos) return "";
        const auto e = s.find_last_not_of(" \t\r\n");
        return s.substr(b, e - b + 1);
    }
};

}  // namespace bem
