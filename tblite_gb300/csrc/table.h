// Data tables of the C API (reference include/tblite/table.h; src/tblite/api/table.f90 over
// toml-f): nested key/value tables whose values are booleans, 64-bit integers, doubles,
// strings, arrays of those, or sub-tables.  Keys keep their insertion order.
//
// The nodes are shared: a handle holds a reference, so a handle to a sub-table (from
// tblite_table_add_table / tblite_table_get_table) stays valid after the parent's handle is
// deleted, and deleting any handle only drops its own reference.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace tb {

struct TTable;
struct TArray;

enum TType { T_NONE = 0, T_BOOL = 1, T_INT = 2, T_DOUBLE = 3, T_CHAR = 4, T_ARRAY = 5, T_TABLE = 6 };

struct TValue {
  int type = T_NONE;
  bool b = false;
  int64_t i = 0;
  double d = 0.0;
  std::string s;
  std::shared_ptr<TArray> a;
  std::shared_ptr<TTable> t;
  static TValue of(bool v) { TValue x; x.type = T_BOOL; x.b = v; return x; }
  static TValue of(int64_t v) { TValue x; x.type = T_INT; x.i = v; return x; }
  static TValue of(double v) { TValue x; x.type = T_DOUBLE; x.d = v; return x; }
  static TValue of(const std::string& v) { TValue x; x.type = T_CHAR; x.s = v; return x; }
};

struct TArray {
  std::vector<TValue> v;
};

struct TTable {
  std::vector<std::pair<std::string, TValue>> kv;
  TValue* find(const std::string& key) {
    for (auto& e : kv)
      if (e.first == key) return &e.second;
    return nullptr;
  }
  const TValue* find(const std::string& key) const {
    for (const auto& e : kv)
      if (e.first == key) return &e.second;
    return nullptr;
  }
  // replaces an existing key in place (keeps its position) or appends
  TValue& set(const std::string& key, TValue v) {
    if (TValue* x = find(key)) {
      *x = std::move(v);
      return *x;
    }
    kv.emplace_back(key, std::move(v));
    return kv.back().second;
  }
  std::shared_ptr<TTable> add_table(const std::string& key) {
    TValue v;
    v.type = T_TABLE;
    v.t = std::make_shared<TTable>();
    return set(key, v).t;
  }
  std::shared_ptr<TArray> add_array(const std::string& key) {
    TValue v;
    v.type = T_ARRAY;
    v.a = std::make_shared<TArray>();
    return set(key, v).a;
  }
};

// TOML text of a table (tblite_dump_table)
std::string toml_dump(const TTable& t);

}  // namespace tb

struct _tblite_table {
  std::shared_ptr<tb::TTable> p;
};
struct _tblite_array {
  std::shared_ptr<tb::TArray> p;
};
