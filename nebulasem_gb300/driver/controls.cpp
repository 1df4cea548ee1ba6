#include "controls.h"

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace nsem_driver {

namespace {

std::string upper(std::string s) {
    for (auto& c : s) c = (char)std::toupper((unsigned char)c);
    return s;
}

/* whitespace-separated tokens of one line with the `#` comment removed;
 * braces are tokens of their own */
std::vector<std::string> tokens(const std::string& line) {
    std::string t = line.substr(0, line.find('#'));
    std::string spaced;
    for (char c : t) {
        if (c == '{' || c == '}') {
            spaced += ' ';
            spaced += c;
            spaced += ' ';
        } else {
            spaced += c;
        }
    }
    std::istringstream is(spaced);
    std::vector<std::string> out;
    std::string w;
    while (is >> w) out.push_back(w);
    return out;
}

}  // namespace

Controls::Controls(const std::string& path) : path_(path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open controls file " + path);
    std::string line, block, pending;
    int depth = 0, lineno = 0;
    while (std::getline(in, line)) {
        lineno++;
        const std::vector<std::string> tk = tokens(line);
        size_t i = 0;
        while (i < tk.size()) {
            const std::string& w = tk[i];
            if (w == "{") {
                if (depth == 0) {
                    if (pending.empty())
                        throw std::runtime_error(path + ":" + std::to_string(lineno) +
                                                 ": block without a name");
                    block = pending;
                    pending.clear();
                }
                depth++;
                i++;
            } else if (w == "}") {
                if (depth == 0)
                    throw std::runtime_error(path + ":" + std::to_string(lineno) + ": unmatched '}'");
                depth--;
                if (depth == 0) block.clear();
                i++;
            } else if (depth == 0) {
                pending = w;
                i++;
            } else if (depth == 1) {
                /* key and the rest of the line up to a brace */
                std::vector<std::string> vals;
                size_t j = i + 1;
                while (j < tk.size() && tk[j] != "{" && tk[j] != "}") vals.push_back(tk[j++]);
                blocks_[block][w] = vals;
                i = j;
            } else {
                i++;   /* nested blocks are not used by the euler app */
            }
        }
    }
    if (depth != 0) throw std::runtime_error(path + ": unbalanced braces");
}

bool Controls::has(const std::string& block, const std::string& key) const {
    auto b = blocks_.find(block);
    return b != blocks_.end() && b->second.count(key);
}

const std::vector<std::string>& Controls::values(const std::string& block,
                                                 const std::string& key) const {
    auto b = blocks_.find(block);
    if (b == blocks_.end() || !b->second.count(key))
        throw std::runtime_error(path_ + ": " + block + "." + key + " is not set");
    return b->second.at(key);
}

std::string Controls::str(const std::string& block, const std::string& key,
                          const std::string& def) const {
    if (!has(block, key)) return def;
    const auto& v = values(block, key);
    if (v.empty()) throw std::runtime_error(path_ + ": " + block + "." + key + " has no value");
    return v[0];
}

double Controls::num(const std::string& block, const std::string& key, double def) const {
    if (!has(block, key)) return def;
    const std::string s = str(block, key, "");
    char* end = nullptr;
    const double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || *end)
        throw std::runtime_error(path_ + ": " + block + "." + key + " is not a number: " + s);
    return v;
}

long Controls::integer(const std::string& block, const std::string& key, long def) const {
    if (!has(block, key)) return def;
    const std::string s = str(block, key, "");
    char* end = nullptr;
    const long v = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || *end)
        throw std::runtime_error(path_ + ": " + block + "." + key + " is not an integer: " + s);
    return v;
}

bool Controls::flag(const std::string& block, const std::string& key, bool def) const {
    if (!has(block, key)) return def;
    const std::string s = upper(str(block, key, ""));
    if (s == "YES" || s == "1" || s == "TRUE") return true;
    if (s == "NO" || s == "0" || s == "FALSE") return false;
    throw std::runtime_error(path_ + ": " + block + "." + key + " must be YES or NO, not " + s);
}

std::vector<double> Controls::vec(const std::string& block, const std::string& key, size_t n,
                                  const std::vector<double>& def) const {
    if (!has(block, key)) return def;
    const auto& v = values(block, key);
    if (v.size() != n)
        throw std::runtime_error(path_ + ": " + block + "." + key + " needs " + std::to_string(n) +
                                 " values");
    std::vector<double> out(n);
    for (size_t i = 0; i < n; i++) {
        char* end = nullptr;
        out[i] = std::strtod(v[i].c_str(), &end);
        if (end == v[i].c_str() || *end)
            throw std::runtime_error(path_ + ": " + block + "." + key + " is not numeric");
    }
    return out;
}

}  // namespace nsem_driver
