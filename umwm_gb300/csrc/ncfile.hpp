// Minimal netCDF classic-format files (64-bit offset variant, "CDF\2"),
// written and read without the netCDF library: the restart files
// (restart/umwmrst_<time>.nc, umwm_restart.F90:19-154) and the gridded
// output (output/umwmout_<time>.nc, umwm_io.F90:317-854) in the reference's
// layouts, and the spectrum output (output/umwmspc_<id>_<time>.nc,
// umwm_io.F90:150-314).  Only what those files use: fixed-size dimensions and
// one record (unlimited) dimension, float and 32-bit integer variables, text
// attributes.  Values are stored big-endian as the format
// requires; the host byte order does not matter.
#pragma once
#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <utility>
#include <vector>

namespace umwm {
namespace nc {

struct Var {
  std::string name;
  std::vector<int> dims;                                   // dimension ids, slowest first (C order)
  std::vector<std::pair<std::string, std::string>> atts;  // text attributes
  // fills out[0..count) with elements [first, first+count) of the variable
  std::function<bool(size_t first, size_t count, float* out)> fill;
  bool is_int = false;  // stored as 32-bit integers (the fill values are converted)
};

// Write a file with the given dimensions (name, length) and variables.  A
// dimension of length 0 is the record (unlimited) dimension; it must be a
// variable's first (slowest) dimension, and the file holds numrecs records
// (a record variable's fill sees its elements over all records, record
// slowest).
bool write(const std::string& path, const std::vector<std::pair<std::string, size_t>>& dims,
           const std::vector<Var>& vars, std::string& err, size_t numrecs = 1);

// Read float variable `name` of a classic or 64-bit-offset file: its
// dimension lengths (slowest first) and values.
bool read_float(const std::string& path, const std::string& name, std::vector<size_t>& shape,
                std::vector<float>& values, std::string& err);

}  // namespace nc
}  // namespace umwm
