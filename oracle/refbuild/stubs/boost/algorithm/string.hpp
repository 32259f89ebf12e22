// Stand-in for Boost.StringAlgo to_lower_copy / trim_copy (oracle build only).
#pragma once
#include <string>
#include <algorithm>
#include <cctype>
namespace boost { namespace algorithm {
inline std::string to_lower_copy(std::string s) {
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    return s;
}
inline std::string trim_copy(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\n\r"), b = s.find_last_not_of(" \t\n\r");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}
}
using algorithm::to_lower_copy;
using algorithm::trim_copy;
}
#include <vector>
namespace boost {
struct is_any_of_t { std::string chars; bool operator()(char c) const { return chars.find(c) != std::string::npos; } };
inline is_any_of_t is_any_of(const std::string& c) { return {c}; }
inline void split(std::vector<std::string>& out, const std::string& in, is_any_of_t p) {
    out.clear();
    std::string cur;
    for (char c : in) {
        if (p(c)) { out.push_back(cur); cur.clear(); } else cur += c;
    }
    out.push_back(cur);
}
namespace algorithm {
inline std::string join(const std::vector<std::string>& v, const std::string& sep) {
    std::string r;
    for (size_t i = 0; i < v.size(); ++i) { if (i) r += sep; r += v[i]; }
    return r;
}
}
}
