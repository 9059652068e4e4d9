#include "params.h"

#include <cctype>
#include <cstdlib>
#include <fstream>

namespace iss {

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) b++;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) e--;
    return s.substr(b, e - b);
}

std::string to_lower(std::string s) {
    for (char& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

double string_to_double(const std::string& s) {
    const char* p = s.c_str();
    char* end = nullptr;
    const double v = std::strtod(p, &end);
    return end == p ? 0.0 : v;
}

long ParamStore::find(const std::string& key) const {
    const std::string k = to_lower(trim(key));
    for (size_t i = 0; i < items_.size(); i++) {
        if (items_[i].first == k) return static_cast<long>(i);
    }
    return -1;
}

void ParamStore::set(const std::string& key, double value) {
    const long i = find(key);
    if (i < 0) {
        items_.emplace_back(to_lower(trim(key)), value);
    } else {
        items_[static_cast<size_t>(i)].second = value;
    }
}

bool ParamStore::has(const std::string& key) const { return find(key) >= 0; }

void ParamStore::erase(const std::string& key) {
    const long i = find(key);
    if (i >= 0) items_.erase(items_.begin() + i);
}

bool ParamStore::get(const std::string& key, double* value) const {
    const long i = find(key);
    if (i < 0) return false;
    *value = items_[static_cast<size_t>(i)].second;
    return true;
}

double ParamStore::get_or(const std::string& key, double fallback) const {
    double v;
    return get(key, &v) ? v : fallback;
}

void ParamStore::parse_line(const std::string& line) {
    const std::string no_comment = line.substr(0, line.find('#'));
    if (trim(no_comment).empty()) return;
    const size_t eq = no_comment.find('=');
    if (eq == std::string::npos) return;
    set(no_comment.substr(0, eq), string_to_double(trim(no_comment.substr(eq + 1))));
}

bool ParamStore::read_file(const std::string& filename) {
    std::ifstream f(filename);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) parse_line(line);
    return true;
}

}  // namespace iss
