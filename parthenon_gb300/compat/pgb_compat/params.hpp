// Package-facing compatibility layer: Params (typed package parameters) and
// ParameterInput (the input deck).
//
// Reference: src/interface/params.hpp (Params::Add/Get/GetMutable/Update/hasKey/reset),
// src/parameter_input.hpp (ParameterInput: <block> sections of `key = value` lines,
// `#` comments, `&` continuation lines; Get*/GetOrAdd*/Set*/CheckRequired/CheckDesired;
// command-line overrides `block/key=value`).
#pragma once

#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <typeindex>
#include <typeinfo>
#include <utility>
#include <vector>

#include "core.hpp"

namespace parthenon {

class Params {
 public:
  enum class Mutability { Immutable, Mutable, Restart };
  template <class T>
  void Add(const std::string &key, T value, Mutability m = Mutability::Immutable) {
    PARTHENON_REQUIRE_THROWS(!hasKey(key), "Key " + key + " already exists");
    entries_.emplace(key, Entry{std::make_shared<T>(std::move(value)), std::type_index(typeid(T)), m});
  }
  template <class T>
  void Add(const std::string &key, T value, bool is_mutable) {
    Add(key, std::move(value), is_mutable ? Mutability::Mutable : Mutability::Immutable);
  }
  template <class T>
  const T &Get(const std::string &key) const {
    return *typed<T>(key);
  }
  template <class T>
  const T &Get(const std::string &key, const T &fallback) const {
    return hasKey(key) ? Get<T>(key) : fallback;
  }
  template <class T>
  T *GetMutable(const std::string &key) const {
    auto it = entries_.find(key);
    PARTHENON_REQUIRE_THROWS(it != entries_.end(), "Key " + key + " doesn't exist");
    PARTHENON_REQUIRE_THROWS(it->second.m != Mutability::Immutable, "Parameter " + key + " must be marked as mutable");
    return typed<T>(key);
  }
  template <class T>
  void Update(const std::string &key, T value) {
    *GetMutable<T>(key) = std::move(value);
  }
  bool hasKey(const std::string &key) const { return entries_.count(key) > 0; }
  // removes every parameter (params.hpp Params::reset)
  void reset() { entries_.clear(); }

 private:
  struct Entry {
    std::shared_ptr<void> p;
    std::type_index type;
    Mutability m;
  };
  template <class T>
  T *typed(const std::string &key) const {
    auto it = entries_.find(key);
    PARTHENON_REQUIRE_THROWS(it != entries_.end(), "Key " + key + " doesn't exist");
    PARTHENON_REQUIRE_THROWS(it->second.type == std::type_index(typeid(T)),
                             "Parameter " + key + " requested with the wrong type");
    return static_cast<T *>(it->second.p.get());
  }
  std::map<std::string, Entry> entries_;
};

class ParameterInput {
 public:
  ParameterInput() = default;
  explicit ParameterInput(const std::string &deck_text) { LoadFromString(deck_text); }

  void LoadFromString(const std::string &text) {
    std::istringstream is(text);
    LoadFromStream(is);
  }
  void LoadFromFile(const std::string &path) {
    std::ifstream f(path);
    PARTHENON_REQUIRE_THROWS(f.good(), "cannot open input file " + path);
    LoadFromStream(f);
  }
  // parameter_input.cpp LoadFromStream: a value continues on the next line after a
  // trailing '&' (text after the '&' is an error); a line whose comment is the marker
  // GetOrAdd* writes ("Default value added at run time") holds a code default, which
  // CheckRequired does not accept
  void LoadFromStream(std::istream &is) {
    std::string line, block, pending;
    while (std::getline(is, line)) {
      const auto hash = line.find('#');
      bool is_default = false;
      if (hash != std::string::npos) {
        is_default = trim(line.substr(hash + 1)) == kDefaultMarker;
        line = line.substr(0, hash);
      }
      line = trim(line);
      if (line.empty()) continue;
      if (!pending.empty()) {  // continuation of the previous value
        line = pending + " " + line;
        pending.clear();
      }
      if (line.front() == '<') {
        const auto close = line.find('>');
        PARTHENON_REQUIRE_THROWS(close != std::string::npos, "malformed block line " + line);
        block = trim(line.substr(1, close - 1));
        continue;
      }
      const auto amp = line.find('&');
      if (amp != std::string::npos) {
        PARTHENON_REQUIRE_THROWS(amp == line.size() - 1, "text after '&' in the input line " + line);
        pending = trim(line.substr(0, line.size() - 1));
        continue;
      }
      const auto eq = line.find('=');
      PARTHENON_REQUIRE_THROWS(eq != std::string::npos && !block.empty(), "malformed input line " + line);
      Set(block, trim(line.substr(0, eq)), trim(line.substr(eq + 1)));
      if (is_default) defaults_.insert(block + "/" + trim(line.substr(0, eq)));
    }
  }
  // "block/key=value" overrides (ParthenonManager's command line)
  void ModifyFromCmdline(int argc, char *argv[]) {
    for (int i = 1; i < argc; ++i) {
      const std::string a = argv[i];
      const auto slash = a.find('/'), eq = a.find('=');
      if (slash == std::string::npos || eq == std::string::npos || eq < slash) continue;
      const auto last = a.rfind('/', eq);
      Set(a.substr(0, last), a.substr(last + 1, eq - last - 1), a.substr(eq + 1));
    }
  }

  bool DoesBlockExist(const std::string &b) const { return blocks_.count(b) > 0; }
  bool DoesParameterExist(const std::string &b, const std::string &k) const {
    auto it = blocks_.find(b);
    return it != blocks_.end() && it->second.count(k) > 0;
  }
  std::string GetString(const std::string &b, const std::string &k) const { return raw(b, k); }
  double GetReal(const std::string &b, const std::string &k) const { return std::stod(raw(b, k)); }
  int GetInteger(const std::string &b, const std::string &k) const { return std::stoi(raw(b, k)); }
  bool GetBoolean(const std::string &b, const std::string &k) const {
    const std::string v = raw(b, k);
    return v == "true" || v == "1" || v == "yes" || v == "on";
  }
  std::string GetOrAddString(const std::string &b, const std::string &k, const std::string &d) {
    if (!DoesParameterExist(b, k)) SetDefault(b, k, d);
    return GetString(b, k);
  }
  double GetOrAddReal(const std::string &b, const std::string &k, double d) {
    if (!DoesParameterExist(b, k)) SetDefault(b, k, num(d));
    return GetReal(b, k);
  }
  int GetOrAddInteger(const std::string &b, const std::string &k, int d) {
    if (!DoesParameterExist(b, k)) SetDefault(b, k, std::to_string(d));
    return GetInteger(b, k);
  }
  bool GetOrAddBoolean(const std::string &b, const std::string &k, bool d) {
    if (!DoesParameterExist(b, k)) SetDefault(b, k, d ? "true" : "false");
    return GetBoolean(b, k);
  }
  void SetString(const std::string &b, const std::string &k, const std::string &v) { Set(b, k, v); }
  void SetReal(const std::string &b, const std::string &k, double v) { Set(b, k, num(v)); }
  void SetInteger(const std::string &b, const std::string &k, int v) { Set(b, k, std::to_string(v)); }
  void SetBoolean(const std::string &b, const std::string &k, bool v) { Set(b, k, v ? "true" : "false"); }
  // parameter_input.cpp CheckRequired / CheckDesired: a code default does not count as
  // provided; a missing desired field prints a warning on stdout
  void CheckRequired(const std::string &b, const std::string &k) const {
    PARTHENON_REQUIRE_THROWS(DoesParameterExist(b, k) && !defaults_.count(b + "/" + k),
                             "Parameter file missing required field <" + b + ">/" + k);
  }
  void CheckDesired(const std::string &b, const std::string &k) const {
    if (!DoesParameterExist(b, k) || defaults_.count(b + "/" + k))
      std::cout << std::endl
                << "### WARNING in CheckDesired:" << std::endl
                << "Parameter file missing desired field <" << b << ">/" << k << std::endl;
  }

 private:
  static std::string trim(const std::string &s) {
    const auto a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    return s.substr(a, s.find_last_not_of(" \t\r\n") - a + 1);
  }
  static std::string num(double d) {
    std::ostringstream os;
    os.precision(17);
    os << d;
    return os.str();
  }
  static constexpr const char *kDefaultMarker = "Default value added at run time";
  void Set(const std::string &b, const std::string &k, const std::string &v) {
    blocks_[b][k] = v;
    defaults_.erase(b + "/" + k);
  }
  void SetDefault(const std::string &b, const std::string &k, const std::string &v) {
    Set(b, k, v);
    defaults_.insert(b + "/" + k);
  }
  std::string raw(const std::string &b, const std::string &k) const {
    auto it = blocks_.find(b);
    PARTHENON_REQUIRE_THROWS(it != blocks_.end() && it->second.count(k),
                             "Parameter " + b + "/" + k + " not found in the input");
    return it->second.at(k);
  }
  std::map<std::string, std::map<std::string, std::string>> blocks_;
  std::set<std::string> defaults_;  // "block/key" of the values a code default set
};

}  // namespace parthenon
