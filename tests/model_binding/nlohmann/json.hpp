// A small stand-in for nlohmann/json (the reference's JSON dependency, absent here): just
// enough of nlohmann::ordered_json for physics/Model.hpp, utils/Parameters.hpp and the
// Physics::Model subclasses to compile and run their JSON reads.  TEST INFRASTRUCTURE ONLY.
// Values are null, boolean, number, string, array or object (keys in insertion order); a
// brace list of [string, value] pairs makes an object, any other brace list an array.
#pragma once

#include <cstddef>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define NLOHMANN_JSON_SERIALIZE_ENUM(ENUM_TYPE, ...)

namespace nlohmann
{
class ordered_json
{
  public:
  enum class kind { null, boolean, number, string, array, object };

  ordered_json() = default;
  ordered_json(std::nullptr_t) {}
  ordered_json(bool b) : m_kind(kind::boolean), m_num(b ? 1.0 : 0.0) {}
  template <typename T, typename std::enable_if<std::is_arithmetic<T>::value && !std::is_same<T, bool>::value, int>::type = 0>
  ordered_json(T v) : m_kind(kind::number), m_num((double)v) {}
  ordered_json(const char* s) : m_kind(kind::string), m_str(s) {}
  ordered_json(const std::string& s) : m_kind(kind::string), m_str(s) {}
  ordered_json(std::initializer_list<ordered_json> list)
  {
    bool pairs = list.size() > 0;
    for (const auto& e : list)
      pairs = pairs && e.m_kind == kind::array && e.m_items.size() == 2 && e.m_items[0].m_kind == kind::string;
    if (pairs) {
      m_kind = kind::object;
      for (const auto& e : list) m_members.emplace_back(e.m_items[0].m_str, e.m_items[1]);
    } else if (list.size() > 0) {
      m_kind = kind::array;
      m_items.assign(list.begin(), list.end());
    }
  }
  bool empty() const
  {
    return m_kind == kind::null || (m_kind == kind::array && m_items.empty()) ||
           (m_kind == kind::object && m_members.empty());
  }

  ordered_json& operator[](const std::string& key)
  {
    if (m_kind == kind::null) m_kind = kind::object;
    if (m_kind != kind::object) throw std::domain_error("not an object");
    for (auto& m : m_members)
      if (m.first == key) return m.second;
    m_members.emplace_back(key, ordered_json());
    return m_members.back().second;
  }
  ordered_json& operator[](const char* key) { return (*this)[std::string(key)]; }
  const ordered_json& at(const std::string& key) const
  {
    if (m_kind == kind::object)
      for (const auto& m : m_members)
        if (m.first == key) return m.second;
    throw std::out_of_range("key not found: " + key);
  }
  ordered_json& operator[](std::size_t i)
  {
    if (m_kind != kind::array || i >= m_items.size()) throw std::out_of_range("index");
    return m_items[i];
  }
  ordered_json& operator[](int i) { return (*this)[(std::size_t)i]; }

  template <typename T>
  T get() const
  {
    if (m_kind != kind::number && m_kind != kind::boolean) throw std::domain_error("not a number");
    return (T)m_num;
  }
  template <typename T, typename std::enable_if<std::is_arithmetic<T>::value, int>::type = 0>
  explicit operator T() const { return get<T>(); }

  friend bool operator==(const ordered_json& a, bool b) { return a.m_kind == kind::boolean && (a.m_num != 0.0) == b; }

  static ordered_json diff(const ordered_json& a, const ordered_json& b)
  {
    return same(a, b) ? ordered_json() : ordered_json{1};
  }
  void merge_patch(const ordered_json& patch)
  {
    if (patch.m_kind != kind::object) {
      *this = patch;
      return;
    }
    if (m_kind != kind::object) *this = ordered_json();
    for (const auto& m : patch.m_members) (*this)[m.first].merge_patch(m.second);
  }

  private:
  static bool same(const ordered_json& a, const ordered_json& b)
  {
    if (a.m_kind != b.m_kind || a.m_num != b.m_num || a.m_str != b.m_str || a.m_items.size() != b.m_items.size() ||
        a.m_members.size() != b.m_members.size())
      return false;
    for (std::size_t i = 0; i < a.m_items.size(); ++i)
      if (!same(a.m_items[i], b.m_items[i])) return false;
    for (std::size_t i = 0; i < a.m_members.size(); ++i)
      if (a.m_members[i].first != b.m_members[i].first || !same(a.m_members[i].second, b.m_members[i].second))
        return false;
    return true;
  }

  kind m_kind = kind::null;
  double m_num = 0.0;
  std::vector<ordered_json> m_items;
  std::vector<std::pair<std::string, ordered_json>> m_members;
  std::string m_str;
};
using json = ordered_json;
} // namespace nlohmann
