// config.h -- input-file reader of the calcqpi CLI.
//
// Same syntax and lookup rules as the reference's loadconfig (include/parser.h:24-197):
//  - one 'key=value;' per line; '#' starts a comment; a line with only one of '='
//    and ';' is reported as incorrect syntax;
//  - the key is the text before '=' verbatim (not trimmed), the value the text
//    between '=' and the first ';', trimmed of blanks and tabs when read;
//  - when a key appears twice the last value wins;
//  - lists are '(a, b, ...)', strings are quoted; atof/atoi number parsing;
//  - keys never read are reported as "Unused line i: key" at the end.
#pragma once

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

class InputFile {
    std::vector<std::string> names_, fields_;
    std::vector<size_t> used_;
    bool ok_ = true;

    static std::string unquote(const std::string &v)
    {
        size_t f = v.find_first_of('"'), l = v.find_last_of('"');
        if (f != std::string::npos && l != std::string::npos) return v.substr(f + 1, l - f - 1);
        return std::string();
    }

public:
    explicit InputFile(const std::string &path, std::ostream &err)
    {
        std::ifstream in(path.c_str());
        if (!in) {
            err << "Error while opening file " << path << " for reading." << std::endl;
            ok_ = false;
            return;
        }
        std::string line;
        size_t lineno = 0;
        while (std::getline(in, line)) {
            if (line.empty()) continue;
            lineno++;
            size_t h = line.find('#');
            if (h != std::string::npos) line.erase(h);
            size_t eq = line.find('='), sc = line.find(';');
            if (eq != std::string::npos && sc != std::string::npos) {
                names_.push_back(line.substr(0, eq));
                fields_.push_back(sc > eq ? line.substr(eq + 1, sc - eq - 1) : std::string());
            } else if (eq != std::string::npos || sc != std::string::npos) {
                err << "Incorrect syntax, '=' or ';' missing." << std::endl << "Line " << lineno << ": " << line << std::endl;
            }
        }
        used_.assign(names_.size(), 0);
    }
    bool ok() const { return ok_; }

    bool has(const std::string &key)
    {
        for (size_t i = 0; i < names_.size(); i++)
            if (names_[i] == key) {
                used_[i]++;
                return true;
            }
        return false;
    }
    std::string field(const std::string &key)
    {
        std::string v;
        for (size_t i = 0; i < names_.size(); i++)
            if (names_[i] == key) {
                used_[i]++;
                v = fields_[i];
            }
        if (v.empty()) return v;
        size_t s = v.find_first_not_of(" \t"), e = v.find_last_not_of(" \t");
        if (s == std::string::npos) return std::string();
        return v.substr(s, e - s + 1);
    }
    std::string str(const std::string &key) { return unquote(field(key)); }
    double value(const std::string &key)
    {
        std::string v = field(key);
        return v.empty() ? NAN : atof(v.c_str());
    }
    int ivalue(const std::string &key)
    {
        std::string v = field(key);
        return v.empty() ? 0 : atoi(v.c_str());
    }
    std::vector<std::string> list(const std::string &key)
    {
        std::string v = field(key);
        std::vector<std::string> out;
        size_t f = v.find_first_of('('), l = v.find_last_of(')');
        if (f == std::string::npos || l == std::string::npos) return out;
        size_t idx = f + 1, nidx;
        do {
            nidx = v.find_first_of(",)", idx);
            if (nidx == std::string::npos) break;
            std::string item = v.substr(idx, nidx - idx);
            size_t s = item.find_first_not_of(" \t"), e = item.find_last_not_of(" \t");
            out.push_back(s == std::string::npos ? std::string() : item.substr(s, e - s + 1));
            idx = nidx + 1;
        } while (nidx != l);
        return out;
    }
    std::vector<double> vec(const std::string &key)
    {
        std::vector<double> out;
        for (auto &s : list(key)) out.push_back(atof(s.c_str()));
        return out;
    }
    std::vector<std::string> strlist(const std::string &key)
    {
        std::vector<std::string> out;
        for (auto &s : list(key)) out.push_back(unquote(s));
        return out;
    }
    void report_unused(std::ostream &os) const
    {
        for (size_t i = 0; i < used_.size(); i++)
            if (!used_[i]) os << "Unused line " << i << ": " << names_[i] << std::endl;
    }
};
