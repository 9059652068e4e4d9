// Parameter store with the semantics of the reference's ParameterReader
// (src/ParameterReader.cpp:33-175): "key = value  # comment" lines, keys
// trimmed and lower-cased, later assignments overwrite earlier ones, values
// parsed as doubles, lookups case-insensitive.
#pragma once

#include <string>
#include <utility>
#include <vector>

namespace iss {

class ParamStore {
 public:
    // ParameterReader::readFromFile (src/ParameterReader.cpp:87-106);
    // returns false if the file cannot be opened.
    bool read_file(const std::string& filename);
    // ParameterReader::phraseOneLine (src/ParameterReader.cpp:76-83): a line
    // without '=' is ignored, as in the reference.
    void parse_line(const std::string& line);
    // ParameterReader::setVal (src/ParameterReader.cpp:130-144).
    void set(const std::string& key, double value);
    // ParameterReader::exist / getVal.
    bool has(const std::string& key) const;
    bool get(const std::string& key, double* value) const;
    double get_or(const std::string& key, double fallback) const;
    // removes a key (a temporary setting put back to "not set")
    void erase(const std::string& key);
    const std::vector<std::pair<std::string, double>>& items() const { return items_; }

 private:
    long find(const std::string& key) const;
    std::vector<std::pair<std::string, double>> items_;
};

std::string trim(const std::string& s);
std::string to_lower(std::string s);
// stringToDouble of src/arsenal.cpp: the leading numeric prefix, 0 if none.
double string_to_double(const std::string& s);

}  // namespace iss
