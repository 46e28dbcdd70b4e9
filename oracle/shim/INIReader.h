// INIReader API stand-in -- TEST INFRASTRUCTURE ONLY.
//
// The reference includes "INIReader.h" from the jtilly/inih header-only fork
// (an empty, unpinned submodule).  This restates the published behaviour of
// that parser and of the four getters SimInfo.h:170-294 calls:
//   - one "[section]" / "name = value" (or "name : value") per line; leading
//     and trailing whitespace stripped; ';' or '#' at line start is a comment;
//     ';' preceded by whitespace starts an inline comment; an indented line
//     continues the previous value; a UTF-8 BOM on line 1 is skipped;
//   - section and key names are case-insensitive, values are not; a repeated
//     key appends "\n" + value;
//   - GetInteger: strtol(base 0), GetReal: strtod, GetFloat: strtof (single
//     precision, returned as float), GetBoolean: true/yes/on/1 and
//     false/no/off/0 (case-insensitive); a value that does not parse gives
//     the default.
#pragma once

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

class INIReader {
 public:
  explicit INIReader(const std::string& filename) {
    std::ifstream in(filename, std::ios::binary);
    if (!in) {
      error_ = -1;
      return;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    Parse(ss.str());
  }
  int ParseError() const { return error_; }

  std::string Get(const std::string& section, const std::string& name,
                  const std::string& default_value) const {
    auto it = values_.find(MakeKey(section, name));
    return it == values_.end() ? default_value : it->second;
  }
  long GetInteger(const std::string& section, const std::string& name, long default_value) const {
    std::string v = Get(section, name, "");
    const char* s = v.c_str();
    char* end = nullptr;
    long n = std::strtol(s, &end, 0);
    return end > s ? n : default_value;
  }
  double GetReal(const std::string& section, const std::string& name, double default_value) const {
    std::string v = Get(section, name, "");
    const char* s = v.c_str();
    char* end = nullptr;
    double n = std::strtod(s, &end);
    return end > s ? n : default_value;
  }
  float GetFloat(const std::string& section, const std::string& name, float default_value) const {
    std::string v = Get(section, name, "");
    const char* s = v.c_str();
    char* end = nullptr;
    float n = std::strtof(s, &end);
    return end > s ? n : default_value;
  }
  bool GetBoolean(const std::string& section, const std::string& name, bool default_value) const {
    std::string v = Get(section, name, "");
    std::transform(v.begin(), v.end(), v.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (v == "true" || v == "yes" || v == "on" || v == "1") return true;
    if (v == "false" || v == "no" || v == "off" || v == "0") return false;
    return default_value;
  }

 private:
  static std::string MakeKey(const std::string& section, const std::string& name) {
    std::string key = section + "=" + name;
    std::transform(key.begin(), key.end(), key.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    return key;
  }
  static bool IsSpace(char c) { return std::isspace((unsigned char)c) != 0; }
  static std::string RStrip(const std::string& s) {
    size_t e = s.size();
    while (e > 0 && IsSpace(s[e - 1])) --e;
    return s.substr(0, e);
  }
  static size_t LSkip(const std::string& s, size_t p) {
    while (p < s.size() && IsSpace(s[p])) ++p;
    return p;
  }
  // Index of the first char of `chars` or of an inline ';' comment (which must
  // follow whitespace), or s.size().
  static size_t FindCharsOrComment(const std::string& s, size_t p, const char* chars) {
    bool was_space = false;
    for (; p < s.size(); ++p) {
      const char c = s[p];
      if (chars && std::strchr(chars, c) && c != '\0') return p;
      if (was_space && c == ';') return p;
      was_space = IsSpace(c);
    }
    return s.size();
  }
  void Handle(const std::string& section, const std::string& name, const std::string& value) {
    std::string& slot = values_[MakeKey(section, name)];
    if (!slot.empty()) slot += "\n";
    slot += value;
  }
  void Parse(const std::string& text) {
    std::string section, prev_name;
    int lineno = 0;
    size_t pos = 0;
    while (pos < text.size()) {
      size_t nl = text.find('\n', pos);
      std::string raw = text.substr(pos, nl == std::string::npos ? std::string::npos : nl - pos);
      pos = (nl == std::string::npos) ? text.size() : nl + 1;
      ++lineno;
      if (lineno == 1 && raw.size() >= 3 && (unsigned char)raw[0] == 0xEF &&
          (unsigned char)raw[1] == 0xBB && (unsigned char)raw[2] == 0xBF)
        raw = raw.substr(3);
      std::string line = RStrip(raw);
      size_t start = LSkip(line, 0);
      if (start >= line.size()) continue;
      const char c0 = line[start];
      if (c0 == ';' || c0 == '#') continue;
      if (!prev_name.empty() && start > 0) {  // continuation line
        Handle(section, prev_name, line.substr(start));
        continue;
      }
      if (c0 == '[') {
        size_t end = FindCharsOrComment(line, start + 1, "]");
        if (end < line.size() && line[end] == ']') {
          section = line.substr(start + 1, end - start - 1);
          prev_name.clear();
        } else if (!error_) {
          error_ = lineno;
        }
        continue;
      }
      size_t end = FindCharsOrComment(line, start, "=:");
      if (end < line.size() && (line[end] == '=' || line[end] == ':')) {
        std::string name = RStrip(line.substr(start, end - start));
        size_t vstart = LSkip(line, end + 1);
        std::string value = line.substr(vstart);
        size_t cend = FindCharsOrComment(value, 0, nullptr);
        value = RStrip(value.substr(0, cend));
        prev_name = name;
        Handle(section, name, value);
      } else if (!error_) {
        error_ = lineno;
      }
    }
  }

  int error_ = 0;
  std::map<std::string, std::string> values_;
};
