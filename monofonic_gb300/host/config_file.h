// INI configuration in monofonIC's format (include/config_file.hh:39-381):
// "[section]" headers, "key = value" lines, comments from the first of '#',
// ';' or '%' to the end of the line, keys addressed as "section/key".
#pragma once
#include <algorithm>
#include <cctype>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>

namespace mfx {

class config_file {
 public:
  struct item_not_found : std::runtime_error {
    using std::runtime_error::runtime_error;
  };

  config_file() = default;

  // parses INI text (the reference reads the same text from a file,
  // config_file.hh:96-164)
  static config_file from_text(const std::string &text) {
    config_file cf;
    std::istringstream is(text);
    std::string line, section;
    while (std::getline(is, line)) {
      if (line.empty()) continue;
      const auto c = line.find_first_of("#;%");
      if (c != std::string::npos) line.erase(c);
      if (!line.empty() && line[0] == '[') {
        section = trim(line.substr(1, line.find(']') - 1));
        continue;
      }
      const auto eq = line.find('=');
      if (eq == std::string::npos) continue;
      const std::string name = trim(line.substr(0, eq)), value = trim(line.substr(eq + 1));
      if (name.empty() || value.empty()) continue;
      cf.items_[section + '/' + name] = value;
    }
    return cf;
  }

  bool contains_key(const std::string &section, const std::string &key) const {
    return items_.count(section + '/' + key) != 0;
  }
  bool contains_key(const std::string &path) const { return items_.count(path) != 0; }

  void insert_value(const std::string &section, const std::string &key, const std::string &value) {
    items_[section + '/' + key] = value;
  }

  template <class T> T get_value(const std::string &section, const std::string &key) const {
    auto it = items_.find(section + '/' + key);
    if (it == items_.end()) throw item_not_found("'" + section + '/' + key + "' not found.");
    return convert<T>(it->second, key);
  }

  template <class T> T get_value_safe(const std::string &section, const std::string &key, T def) const {
    auto it = items_.find(section + '/' + key);
    if (it == items_.end()) return def;
    try {
      return convert<T>(it->second, key);
    } catch (const std::exception &) {
      return def;
    }
  }

 private:
  std::map<std::string, std::string> items_;

  static std::string trim(const std::string &s) {
    const auto a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const auto b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
  }

  template <class T> static T convert(const std::string &v, const std::string &key) {
    std::istringstream is(v);
    T r{};
    is >> r;
    if (is.fail()) throw std::runtime_error("conversion error for '" + key + "' = '" + v + "'");
    return r;
  }
};

template <> inline std::string config_file::convert<std::string>(const std::string &v, const std::string &) {
  return v;
}

// bool conversion of get_value / get_value_safe (config_file.hh:344-381)
template <> inline bool config_file::convert<bool>(const std::string &v, const std::string &key) {
  std::string u = v;
  std::transform(u.begin(), u.end(), u.begin(), ::toupper);
  if (u == "YAY" || u == "TRUE" || u == "YES" || u == "ON" || u == "1") return true;
  if (u == "NAY" || u == "FALSE" || u == "NO" || u == "OFF" || u == "0") return false;
  throw std::runtime_error("Illegal identifier '" + v + "' in '" + key + "'.");
}

}  // namespace mfx
