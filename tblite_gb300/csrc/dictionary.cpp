// Post-processing results as a dictionary of FP64 arrays, and the post-processing list of a
// calculator (reference include/tblite/double_dictionary.h, result.h:243-246,
// calculator.h:270-291; src/tblite/api/double_dictionary.f90, api/result.f90:572-595,
// api/calculator.f90:727-806, post_processing/list.f90:179-256).
//
// A dictionary is a snapshot of one result's post-processing entries, owned by the caller and
// freed with tblite_delete_double_dictionary.  Entries are addressed by label or by a 1-based
// index (the reference's Fortran indices pass through its C API unchanged); arrays come out in
// Fortran order with up to three dimensions, unused trailing dimensions reported as 0.
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"

struct _tblite_double_dictionary {
  struct Entry {
    std::string label;
    std::vector<double> data;
    int dims[3] = {0, 0, 0};
  };
  std::vector<Entry> entries;
  const Entry* at(int index) const {  // 1-based
    return index >= 1 && index <= (int)entries.size() ? &entries[(size_t)index - 1] : nullptr;
  }
  const Entry* find(const char* label) const {
    if (!label) return nullptr;
    for (const auto& e : entries)
      if (e.label == label) return &e;
    return nullptr;
  }
};

namespace {

void fail(tblite_error error, const char* msg) {
  if (error) {
    error->msg = msg;
    error->set = true;
  }
}

// Null error handles are ignored by the reference (check_dict returns before any access).
bool dict_ok(tblite_error error, tblite_double_dictionary dict) {
  if (!error) return false;
  if (!dict) {
    fail(error, "Dictionary is missing.");
    return false;
  }
  return true;
}

void sizes(const _tblite_double_dictionary::Entry& e, int* d1, int* d2, int* d3) {
  *d1 = e.dims[0];
  *d2 = e.dims[1];
  *d3 = e.dims[2];
}

}  // namespace

extern "C" {

tblite_double_dictionary tblite_get_post_processing_dict(tblite_error error, tblite_result res) {
  if (!res) {
    fail(error, "Result container is missing");
    return nullptr;
  }
  if (!res->has_energy || res->pp.empty()) {
    fail(error, "Result does not contain post processing dictionary.");
    return nullptr;
  }
  auto* d = new _tblite_double_dictionary();
  for (const auto& label : res->pp) {
    _tblite_double_dictionary::Entry e;
    e.label = label;
    if (label == "bond-orders") {
      e.data = res->wbo;
      e.dims[0] = res->nat;
      e.dims[1] = res->nat;
      e.dims[2] = res->wbo_channels;
    } else if (label == "molecular-dipole") {
      e.data.assign(res->dipole, res->dipole + 3);
      e.dims[0] = 3;
    } else if (label == "molecular-quadrupole") {
      e.data.assign(res->quadrupole, res->quadrupole + 6);
      e.dims[0] = 6;
    } else {
      continue;
    }
    d->entries.push_back(std::move(e));
  }
  return d;
}

int tblite_get_n_entries_dict(tblite_error error, tblite_double_dictionary dict) {
  if (!dict_ok(error, dict)) return 0;
  return (int)dict->entries.size();
}

void tblite_get_array_size_index(tblite_error error, tblite_double_dictionary dict,
                                 const int* index, int* dim1, int* dim2, int* dim3) {
  if (dim1) *dim1 = 0;
  if (dim2) *dim2 = 0;
  if (dim3) *dim3 = 0;
  if (!dict_ok(error, dict)) return;
  const auto* e = index ? dict->at(*index) : nullptr;
  if (!e) {
    fail(error, "Index is not a key in the dictionary.");
    return;
  }
  sizes(*e, dim1, dim2, dim3);
}

void tblite_get_array_entry_index(tblite_error error, tblite_double_dictionary dict,
                                  const int* index, double* array) {
  if (!dict_ok(error, dict)) return;
  const auto* e = index ? dict->at(*index) : nullptr;
  if (!e) {
    fail(error, "Index is not a key in the dictionary.");
    return;
  }
  if (!e->data.empty()) std::memcpy(array, e->data.data(), sizeof(double) * e->data.size());
}

void tblite_get_array_size_label(tblite_error error, tblite_double_dictionary dict, char* label,
                                 int* dim1, int* dim2, int* dim3) {
  if (dim1) *dim1 = 0;
  if (dim2) *dim2 = 0;
  if (dim3) *dim3 = 0;
  if (!dict_ok(error, dict)) return;
  const auto* e = dict->find(label);
  if (!e) {
    fail(error, "Label is not a key in the dictionary.");
    return;
  }
  sizes(*e, dim1, dim2, dim3);
}

void tblite_get_array_entry_label(tblite_error error, tblite_double_dictionary dict, char* label,
                                  double* array) {
  if (!dict_ok(error, dict)) return;
  const auto* e = dict->find(label);
  if (!e) {
    fail(error, "Label is not a key in the dictionary.");
    return;
  }
  if (!e->data.empty()) std::memcpy(array, e->data.data(), sizeof(double) * e->data.size());
}

void tblite_get_label_entry_index(tblite_error error, tblite_double_dictionary dict,
                                  const int* index, char* label, const int* buffersize) {
  if (!dict_ok(error, dict)) return;
  const auto* e = index ? dict->at(*index) : nullptr;
  if (!e) {
    fail(error, "Index is not a key in the dictionary.");
    return;
  }
  if (!label) return;
  // the label and its terminating NUL, truncated to the buffer (no size: as long as needed)
  size_t n = e->label.size();
  if (buffersize) {
    if (*buffersize <= 0) return;
    n = std::min(n, (size_t)*buffersize - 1);
  }
  std::memcpy(label, e->label.data(), n);
  label[n] = '\0';
}

void tblite_delete_double_dictionary(tblite_double_dictionary* dict) {
  if (dict && *dict) {
    delete *dict;
    *dict = nullptr;
  }
}

// Post-processing methods by name: "bond-orders" (Wiberg/Mayer bond orders) and "molmom"
// (molecular dipole and quadrupole moments), computed with every single point in the order they
// were added.  The reference's machine-learning descriptors ("xtbml", "xtbml-xyz") and
// post-processing read from a TOML file are not available and are refused with an error.
void tblite_push_back_post_processing_str(tblite_context ctx, tblite_calculator calc,
                                          tblite_structure mol, char* charptr) {
  if (!ctx) return;
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  if (!mol) {
    ctx->push("Molecular structure data is missing");
    return;
  }
  const std::string name = charptr ? charptr : "";
  if (name == "bond-orders" || name == "molmom") {
    calc->post_proc.push_back(name);
  } else if (name == "xtbml" || name == "xtbml-xyz" || name == "xtbml_xyz") {
    ctx->push("Post processing '" + name + "' (xtbml descriptors) is not available in this "
              "library");
  } else {
    ctx->push("Post processing from '" + name + "' is not available in this library: only "
              "'bond-orders' and 'molmom' are supported");
  }
}

}  // extern "C"
