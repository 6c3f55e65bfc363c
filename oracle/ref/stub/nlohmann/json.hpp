// Inert stand-in for the nlohmann::json interface that the reference's
// headers name (its JSON read and write paths are not used by the oracle's
// pinning library): a json value that accepts and returns anything and
// stores nothing, and a NLOHMANN_DEFINE_TYPE_INTRUSIVE whose
// to_json / from_json do nothing.  Written for
// the oracle build only; it is not nlohmann_json.
#pragma once
#include <cstddef>
#include <initializer_list>
#include <istream>
#include <ostream>
#include <string>

namespace nlohmann {
template <typename T, typename SFINAE = void> struct adl_serializer;

struct json {
  json() = default;
  json(const json &) = default;
  json &operator=(const json &) = default;
  json(std::initializer_list<json>) {}
  template <typename T> json(const T &) {}
  static json array() { return json(); }
  static json object() { return json(); }
  template <typename T> void push_back(const T &) {}
  std::size_t size() const { return 0; }
  const json &at(std::size_t) const { return *this; }
  const json &at(const std::string &) const { return *this; }
  template <typename K> json &operator[](const K &) { return *this; }
  template <typename K> const json &operator[](const K &) const { return *this; }
  template <typename T> T get() const { return T(); }
  template <typename T> void get_to(T &) const {}
  template <typename T> operator T() const { return T(); }
};
inline std::ostream &operator<<(std::ostream &o, const json &) { return o; }
inline std::istream &operator>>(std::istream &i, json &) { return i; }
}  // namespace nlohmann

#define NLOHMANN_DEFINE_TYPE_INTRUSIVE(Type, ...)                    \
  friend void to_json(nlohmann::json &, const Type &) {}              \
  friend void from_json(const nlohmann::json &, Type &) {}
