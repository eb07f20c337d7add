// C API of the data tables (reference include/tblite/table.h, src/tblite/api/table.f90).
// Errors follow the reference: a call with a null error handle does nothing, a missing table or
// array handle or a failed conversion sets the error.  Indices into arrays and the key list are
// 1-based, as in the reference.
#include "table.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>

#include "api_internal.h"

using tb::TArray;
using tb::TTable;
using tb::TValue;

namespace {

void fail(tblite_error error, const char* msg) {
  error->msg = msg;
  error->set = true;
}

// copy a NUL-terminated string into a caller buffer of n bytes (truncated, always terminated)
void put_string(const std::string& s, char* out, int n) {
  if (!out || n <= 0) return;
  const size_t m = std::min(s.size(), (size_t)n - 1);
  std::memcpy(out, s.data(), m);
  out[m] = '\0';
}

bool read_double(const TValue& v, double* out) {
  if (v.type == tb::T_DOUBLE) *out = v.d;
  else if (v.type == tb::T_INT) *out = (double)v.i;
  else return false;
  return true;
}

// the scalar types of an array entry, for tblite_table_set_array
TValue scalar_copy(const TValue& v) {
  TValue x;
  x.type = v.type;
  x.b = v.b;
  x.i = v.i;
  x.d = v.d;
  x.s = v.s;
  return x;
}

// -------- TOML text ----------------------------------------------------------------------
std::string quote(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
  }
  return o + "\"";
}
std::string key_text(const std::string& k) {
  for (char c : k)
    if (!(std::isalnum((unsigned char)c) || c == '_' || c == '-')) return quote(k);
  return k.empty() ? quote(k) : k;
}
std::string scalar_text(const TValue& v) {
  char buf[64];
  switch (v.type) {
    case tb::T_BOOL: return v.b ? "true" : "false";
    case tb::T_INT: return std::to_string(v.i);
    case tb::T_DOUBLE:
      if (std::isnan(v.d)) return "nan";
      if (std::isinf(v.d)) return v.d > 0 ? "inf" : "-inf";
      std::snprintf(buf, sizeof(buf), "%.17g", v.d);
      if (!std::strpbrk(buf, ".eE")) std::strcat(buf, ".0");
      return buf;
    case tb::T_CHAR: return quote(v.s);
    default: return "\"\"";
  }
}
void dump_table(const TTable& t, const std::string& path, std::ostringstream& out) {
  bool header_written = path.empty();
  auto header = [&]() {
    if (!header_written) {
      out << "\n[" << path << "]\n";
      header_written = true;
    }
  };
  for (const auto& [k, v] : t.kv) {
    if (v.type == tb::T_TABLE) continue;
    header();
    out << key_text(k) << " = ";
    if (v.type == tb::T_ARRAY) {
      out << "[";
      for (size_t i = 0; i < v.a->v.size(); ++i) out << (i ? ", " : "") << scalar_text(v.a->v[i]);
      out << "]\n";
    } else {
      out << scalar_text(v) << "\n";
    }
  }
  for (const auto& [k, v] : t.kv)
    if (v.type == tb::T_TABLE)
      dump_table(*v.t, path.empty() ? key_text(k) : path + "." + key_text(k), out);
}

}  // namespace

namespace tb {
std::string toml_dump(const TTable& t) {
  std::ostringstream out;
  dump_table(t, "", out);
  std::string s = out.str();
  if (!s.empty() && s[0] == '\n') s.erase(0, 1);
  return s;
}
}  // namespace tb

extern "C" {

tblite_table tblite_new_table(tblite_table* table) {
  // the reference passes an existing handle by value: a new reference to the same table
  auto* h = new _tblite_table();
  auto* other = reinterpret_cast<_tblite_table*>(table);
  h->p = other ? other->p : std::make_shared<TTable>();
  return h;
}

void tblite_delete_table(tblite_table* table) {
  if (table && *table) {
    delete *table;
    *table = nullptr;
  }
}

#define TABLE_GUARD(ret)                                \
  if (!error) return ret;                               \
  if (!table) {                                         \
    fail(error, "Data table object is missing");        \
    return ret;                                         \
  }

void tblite_table_set_double(tblite_error error, tblite_table table, char key[], double* value,
                             int n) {
  TABLE_GUARD();
  if (n > 0) {
    auto a = table->p->add_array(key);
    for (int i = 0; i < n; ++i) a->v.push_back(TValue::of(value[i]));
  } else {
    table->p->set(key, TValue::of(value[0]));
  }
}
void tblite_table_set_int64_t(tblite_error error, tblite_table table, char key[], int64_t* value,
                              int n) {
  TABLE_GUARD();
  if (n > 0) {
    auto a = table->p->add_array(key);
    for (int i = 0; i < n; ++i) a->v.push_back(TValue::of(value[i]));
  } else {
    table->p->set(key, TValue::of(value[0]));
  }
}
void tblite_table_set_bool(tblite_error error, tblite_table table, char key[], bool* value,
                           int n) {
  TABLE_GUARD();
  if (n > 0) {
    auto a = table->p->add_array(key);
    for (int i = 0; i < n; ++i) a->v.push_back(TValue::of(value[i]));
  } else {
    table->p->set(key, TValue::of(value[0]));
  }
}
// value: n strings of the same (unknown) buffer length would need the length; the reference
// reads consecutive NUL-terminated strings, which is what this does for n > 0
void tblite_table_set_char(tblite_error error, tblite_table table, char key[], char (*value)[],
                           int n) {
  TABLE_GUARD();
  const char* p = reinterpret_cast<const char*>(value);
  if (n > 0) {
    auto a = table->p->add_array(key);
    for (int i = 0; i < n; ++i) {
      a->v.push_back(TValue::of(std::string(p)));
      p += std::strlen(p) + 1;
    }
  } else {
    table->p->set(key, TValue::of(std::string(p)));
  }
}

tblite_table tblite_table_add_table(tblite_error error, tblite_table table, char key[]) {
  TABLE_GUARD(nullptr);
  auto* h = new _tblite_table();
  h->p = table->p->add_table(key);
  return h;
}

tblite_array tblite_new_array(void) {
  auto* h = new _tblite_array();
  h->p = std::make_shared<TArray>();
  return h;
}
void tblite_delete_array(tblite_array* array) {
  if (array && *array) {
    delete *array;
    *array = nullptr;
  }
}

#define ARRAY_GUARD(ret)                                \
  if (!error) return ret;                               \
  if (!array) {                                         \
    fail(error, "Data array object is missing");        \
    return ret;                                         \
  }

void tblite_array_push_back_double(tblite_error error, tblite_array array, double value) {
  ARRAY_GUARD();
  array->p->v.push_back(TValue::of(value));
}
void tblite_array_push_back_int64_t(tblite_error error, tblite_array array, int64_t value) {
  ARRAY_GUARD();
  array->p->v.push_back(TValue::of(value));
}
void tblite_array_push_back_bool(tblite_error error, tblite_array array, bool value) {
  ARRAY_GUARD();
  array->p->v.push_back(TValue::of(value));
}
void tblite_array_push_back_char(tblite_error error, tblite_array array, char value[]) {
  ARRAY_GUARD();
  array->p->v.push_back(TValue::of(std::string(value ? value : "")));
}
int tblite_array_size(tblite_error error, tblite_array array) {
  ARRAY_GUARD(0);
  return (int)array->p->v.size();
}
int tblite_array_get_type(tblite_error error, tblite_array array, int index) {
  ARRAY_GUARD(0);
  if (index < 1 || index > (int)array->p->v.size()) return tb::T_NONE;
  return array->p->v[(size_t)index - 1].type;
}
static const TValue* array_at(tblite_array array, int index) {
  return (index >= 1 && index <= (int)array->p->v.size()) ? &array->p->v[(size_t)index - 1]
                                                           : nullptr;
}
void tblite_array_get_double(tblite_error error, tblite_array array, int index, double* value) {
  ARRAY_GUARD();
  const TValue* v = array_at(array, index);
  if (!v || !read_double(*v, value)) fail(error, "Failed to read double value from data array");
}
void tblite_array_get_int64_t(tblite_error error, tblite_array array, int index, int64_t* value) {
  ARRAY_GUARD();
  const TValue* v = array_at(array, index);
  if (!v || v->type != tb::T_INT) fail(error, "Failed to read integer value from data array");
  else *value = v->i;
}
void tblite_array_get_bool(tblite_error error, tblite_array array, int index, bool* value) {
  ARRAY_GUARD();
  const TValue* v = array_at(array, index);
  if (!v || v->type != tb::T_BOOL) fail(error, "Failed to read boolean value from data array");
  else *value = v->b;
}
void tblite_array_get_char(tblite_error error, tblite_array array, int index, char value[],
                           int n) {
  ARRAY_GUARD();
  const TValue* v = array_at(array, index);
  if (!v || v->type != tb::T_CHAR) fail(error, "Failed to read character value from data array");
  else put_string(v->s, value, n);
}

void tblite_table_set_array(tblite_error error, tblite_table table, char key[],
                            tblite_array array) {
  TABLE_GUARD();
  if (!array) {
    fail(error, "Data array object is missing");
    return;
  }
  auto a = table->p->add_array(key);
  for (const TValue& v : array->p->v) {
    if (v.type == tb::T_ARRAY || v.type == tb::T_TABLE || v.type == tb::T_NONE) {
      fail(error, "Failed to push back array value(s) to data table");
      return;
    }
    a->v.push_back(scalar_copy(v));
  }
}

int tblite_table_get_type(tblite_error error, tblite_table table, char key[]) {
  TABLE_GUARD(tb::T_NONE);
  const TValue* v = table->p->find(key);
  return v ? v->type : tb::T_NONE;
}
void tblite_table_get_bool(tblite_error error, tblite_table table, char key[], bool* value) {
  TABLE_GUARD();
  const TValue* v = table->p->find(key);
  if (!v || v->type != tb::T_BOOL) fail(error, "Failed to read boolean value from data table");
  else *value = v->b;
}
void tblite_table_get_int64_t(tblite_error error, tblite_table table, char key[],
                              int64_t* value) {
  TABLE_GUARD();
  const TValue* v = table->p->find(key);
  if (!v || v->type != tb::T_INT) fail(error, "Failed to read integer value from data table");
  else *value = v->i;
}
void tblite_table_get_double(tblite_error error, tblite_table table, char key[], double* value) {
  TABLE_GUARD();
  const TValue* v = table->p->find(key);
  if (!v || !read_double(*v, value)) fail(error, "Failed to read double value from data table");
}
void tblite_table_get_char(tblite_error error, tblite_table table, char key[], char value[],
                           int n) {
  TABLE_GUARD();
  const TValue* v = table->p->find(key);
  if (!v || v->type != tb::T_CHAR) fail(error, "Failed to read character value from data table");
  else put_string(v->s, value, n);
}
tblite_table tblite_table_get_table(tblite_error error, tblite_table table, char key[]) {
  TABLE_GUARD(nullptr);
  TValue* v = table->p->find(key);
  if (!v || v->type != tb::T_TABLE) {
    fail(error, "Failed to read subtable from data table");
    return nullptr;
  }
  auto* h = new _tblite_table();
  h->p = v->t;
  return h;
}
tblite_array tblite_table_get_array(tblite_error error, tblite_table table, char key[]) {
  TABLE_GUARD(nullptr);
  TValue* v = table->p->find(key);
  if (!v || v->type != tb::T_ARRAY) {
    fail(error, "Failed to read array from data table");
    return nullptr;
  }
  auto* h = new _tblite_array();
  h->p = v->a;
  return h;
}
int tblite_table_get_n_keys(tblite_error error, tblite_table table) {
  TABLE_GUARD(0);
  return (int)table->p->kv.size();
}
void tblite_table_get_key(tblite_error error, tblite_table table, int index, char key[], int n) {
  TABLE_GUARD();
  if (index < 1 || index > (int)table->p->kv.size()) {
    fail(error, "Table key index out of range");
    return;
  }
  put_string(table->p->kv[(size_t)index - 1].first, key, n);
}
void tblite_dump_table(tblite_error error, tblite_table table, char filename[]) {
  TABLE_GUARD();
  std::FILE* f = std::fopen(filename ? filename : "", "w");
  if (!f) {
    fail(error, "Could not open file for writing the data table");
    return;
  }
  const std::string text = tb::toml_dump(*table->p);
  const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
  if (std::fclose(f) != 0 || !ok) fail(error, "Could not write the data table");
}

}  // extern "C"
