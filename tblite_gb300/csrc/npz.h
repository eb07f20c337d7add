// NumPy .npz archives of FP64 arrays (stored zip members), for the wavefunction restart files
#pragma once

#include <map>
#include <string>
#include <utility>
#include <vector>

namespace tb {

struct NpyArray {
  std::vector<size_t> shape;  // Fortran order: shape[0] varies fastest in data
  std::vector<double> data;
};

// write the arrays as "<name>.npy" members; throws std::runtime_error on failure
void npz_write(const std::string& file, const std::vector<std::pair<std::string, NpyArray>>& arrays);
// read every member (float64, stored); names without ".npy"; throws on failure
std::map<std::string, NpyArray> npz_read(const std::string& file);

}  // namespace tb
