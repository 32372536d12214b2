// plan_cache.h -- the autotuner's plan cache file.  Host-only, no CUDA.
//
// The file holds one JSON object per line, each a flat map of string and
// number fields: the device it was tuned on (name, SM count, compute
// capability, driver and runtime versions, library version), the key of
// the tuned object (image size and count, or a batch plan's size histogram
// and flags) and the choice with its timings.  A lookup returns the LAST
// line whose fields equal every field asked for, so a later tuning of the
// same key overrides an earlier one; lines that do not parse (a torn write,
// a hand edit) are skipped.  An append is one fwrite of one line to a file
// opened for appending.
#pragma once
#include <cctype>
#include <cstdio>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace glsfft {
namespace plan_cache {

using Fields = std::map<std::string, std::string>;  // name -> value (strings unescaped)
using Pairs = std::vector<std::pair<std::string, std::string>>;  // name -> JSON value text

// JSON string literal of v
inline std::string quote(const std::string &v) {
    std::string o = "\"";
    for (unsigned char c : v) {
        if (c == '"' || c == '\\') {
            o += '\\';
            o += (char)c;
        } else if (c < 0x20) {
            char b[8];
            std::snprintf(b, sizeof b, "\\u%04x", c);
            o += b;
        } else {
            o += (char)c;
        }
    }
    return o + "\"";
}

// one line (no newline) from name / JSON-value pairs, in the given order
inline std::string format_line(const Pairs &kv) {
    std::string o = "{";
    for (size_t i = 0; i < kv.size(); i++) {
        if (i) o += ", ";
        o += quote(kv[i].first) + ": " + kv[i].second;
    }
    return o + "}";
}

namespace detail {
inline void skip_ws(const std::string &s, size_t &i) {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r' || s[i] == '\n')) i++;
}
inline int hexval(char c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'f') return c - 'a' + 10;
    if (c >= 'A' && c <= 'F') return c - 'A' + 10;
    return -1;
}
// a JSON string at s[i] == '"'; only \uXXXX below 0x80 is decoded
inline bool parse_string(const std::string &s, size_t &i, std::string &out) {
    if (i >= s.size() || s[i] != '"') return false;
    out.clear();
    for (i++; i < s.size(); i++) {
        const char c = s[i];
        if (c == '"') {
            i++;
            return true;
        }
        if (c != '\\') {
            out += c;
            continue;
        }
        if (++i >= s.size()) return false;
        switch (s[i]) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'n': out += '\n'; break;
        case 't': out += '\t'; break;
        case 'r': out += '\r'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'u': {
            if (i + 4 >= s.size()) return false;
            int v = 0;
            for (int k = 1; k <= 4; k++) {
                const int h = hexval(s[i + k]);
                if (h < 0) return false;
                v = v * 16 + h;
            }
            if (v >= 0x80) return false;
            out += (char)v;
            i += 4;
            break;
        }
        default: return false;
        }
    }
    return false;
}
}  // namespace detail

// Parse one flat object of string / number / true / false / null values.
inline bool parse_line(const std::string &s, Fields &out) {
    using namespace detail;
    out.clear();
    size_t i = 0;
    skip_ws(s, i);
    if (i >= s.size() || s[i] != '{') return false;
    i++;
    skip_ws(s, i);
    if (i < s.size() && s[i] == '}') {
        i++;
    } else {
        for (;;) {
            std::string key, val;
            skip_ws(s, i);
            if (!parse_string(s, i, key)) return false;
            skip_ws(s, i);
            if (i >= s.size() || s[i] != ':') return false;
            i++;
            skip_ws(s, i);
            if (i >= s.size()) return false;
            if (s[i] == '"') {
                if (!parse_string(s, i, val)) return false;
            } else {
                const size_t b = i;
                while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '-' ||
                                        s[i] == '+' || s[i] == '.'))
                    i++;
                if (i == b) return false;  // objects and arrays are not part of the format
                val = s.substr(b, i - b);
            }
            out[key] = val;
            skip_ws(s, i);
            if (i < s.size() && s[i] == ',') {
                i++;
                continue;
            }
            if (i < s.size() && s[i] == '}') {
                i++;
                break;
            }
            return false;
        }
    }
    skip_ws(s, i);
    return i == s.size();
}

// The fields of name / JSON-value pairs as parse_line returns them.
inline Fields as_fields(const Pairs &kv) {
    Fields f;
    parse_line(format_line(kv), f);
    return f;
}

// The last line of `path` whose fields include every (name, value) of match.
inline bool lookup(const char *path, const Fields &match, Fields &out) {
    if (!path || !*path) return false;
    std::FILE *f = std::fopen(path, "r");
    if (!f) return false;
    bool found = false;
    std::string line;
    Fields cur;
    char buf[4096];
    auto finish_line = [&]() {
        if (!line.empty() && parse_line(line, cur)) {
            bool ok = true;
            for (const auto &m : match) {
                const auto it = cur.find(m.first);
                if (it == cur.end() || it->second != m.second) {
                    ok = false;
                    break;
                }
            }
            if (ok) {
                out = cur;
                found = true;
            }
        }
        line.clear();
    };
    while (std::fgets(buf, sizeof buf, f)) {
        line += buf;
        if (!line.empty() && line.back() == '\n') {
            line.pop_back();
            finish_line();
        }
    }
    finish_line();
    std::fclose(f);
    return found;
}

// Append one line; false when the file cannot be opened or written.
inline bool append(const char *path, const Pairs &kv) {
    if (!path || !*path) return false;
    std::FILE *f = std::fopen(path, "a");
    if (!f) return false;
    const std::string line = format_line(kv) + "\n";
    const bool ok = std::fwrite(line.data(), 1, line.size(), f) == line.size();
    return (std::fclose(f) == 0) && ok;
}

}  // namespace plan_cache
}  // namespace glsfft
