// ini.hpp -- reader for the reference's configuration files.
//
// Follows the conventions of the INI parser the reference is built with
// (CUDA_week2/INIReader.cuh, the inih library): "[section]" headers,
// "name = value" (or "name: value") pairs with surrounding whitespace
// stripped, whole-line comments starting with ';' or '#', inline ';' comments
// only when preceded by whitespace, section and name case-insensitive, and a
// repeated name keeping its first value for numbers.  GetInteger / GetReal
// read the leading number of the value (strtol base 0 / strtod) and fall back
// to the default when there is none, so "601;   int" reads as 601.  Vectors
// "{a, b, c}" are read like the reference's parse_string_to_vector
// (util.cu:141-163): whitespace removed, everything from the first '}' on
// cut, the leading brace dropped, comma-separated atof.
#pragma once

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <map>
#include <string>
#include <vector>

class IniFile {
  public:
    explicit IniFile(const std::string& path) {
        std::ifstream in(path);
        if (!in) {
            error_ = -1;
            return;
        }
        std::string line, section;
        int lineno = 0;
        while (std::getline(in, line)) {
            lineno++;
            std::string s = trim(line);
            if (lineno == 1 && s.size() >= 3 && (unsigned char)s[0] == 0xEF && (unsigned char)s[1] == 0xBB &&
                (unsigned char)s[2] == 0xBF)
                s = trim(s.substr(3));  // UTF-8 byte-order mark
            if (s.empty() || s[0] == ';' || s[0] == '#') continue;
            if (s[0] == '[') {
                const size_t e = s.find(']');
                if (e == std::string::npos) {
                    if (!error_) error_ = lineno;
                    continue;
                }
                section = lower(trim(s.substr(1, e - 1)));
                continue;
            }
            size_t d = s.find_first_of("=:");
            if (d == std::string::npos) {
                if (!error_) error_ = lineno;
                continue;
            }
            std::string name = lower(trim(s.substr(0, d)));
            std::string value = strip_inline_comment(s.substr(d + 1));
            const std::string key = section + "=" + name;
            if (!values_.count(key)) values_[key] = trim(value);
        }
    }

    // 0 = parsed, -1 = file not found, > 0 = first line with an error
    int ParseError() const { return error_; }

    std::string Get(const std::string& sec, const std::string& name, const std::string& def) const {
        auto it = values_.find(lower(sec) + "=" + lower(name));
        return it == values_.end() ? def : it->second;
    }
    bool Has(const std::string& sec, const std::string& name) const {
        return values_.count(lower(sec) + "=" + lower(name)) != 0;
    }
    long GetInteger(const std::string& sec, const std::string& name, long def) const {
        const std::string v = Get(sec, name, "");
        const char* b = v.c_str();
        char* e = nullptr;
        const long n = std::strtol(b, &e, 0);
        return e > b ? n : def;
    }
    double GetReal(const std::string& sec, const std::string& name, double def) const {
        const std::string v = Get(sec, name, "");
        const char* b = v.c_str();
        char* e = nullptr;
        const double n = std::strtod(b, &e);
        return e > b ? n : def;
    }
    std::vector<double> GetVector(const std::string& sec, const std::string& name, const std::string& def) const {
        std::string s = Get(sec, name, def);
        std::string t;
        for (char c : s)
            if (!std::isspace((unsigned char)c)) t += c;
        const size_t close = t.find('}');
        if (close != std::string::npos) t.erase(close);
        if (!t.empty()) t.erase(0, 1);
        std::vector<double> out;
        size_t pos;
        while ((pos = t.find(',')) != std::string::npos) {
            out.push_back(std::atof(t.substr(0, pos).c_str()));
            t.erase(0, pos + 1);
        }
        out.push_back(std::atof(t.c_str()));
        return out;
    }

  private:
    static std::string trim(const std::string& s) {
        size_t a = 0, b = s.size();
        while (a < b && std::isspace((unsigned char)s[a])) a++;
        while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
        return s.substr(a, b - a);
    }
    static std::string lower(std::string s) {
        for (char& c : s) c = (char)std::tolower((unsigned char)c);
        return s;
    }
    static std::string strip_inline_comment(const std::string& v) {
        for (size_t i = 1; i < v.size(); i++)
            if (v[i] == ';' && std::isspace((unsigned char)v[i - 1])) return v.substr(0, i);
        return v;
    }
    std::map<std::string, std::string> values_;
    int error_ = 0;
};
