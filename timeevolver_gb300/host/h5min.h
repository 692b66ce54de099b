// h5min.h -- a small writer of HDF5 files for the result layout of
// TimeEvolver's saveResult / saveMatrix / saveSparseMatrix
// (helper/krylovHelper.cpp:27-92, :112-203), with no HDF5 library.
//
// The file follows the published HDF5 format specification with the
// structures the HDF5 library writes by default for such files: a version 0
// superblock, a root group stored as a symbol table (a version 1 B-tree of
// group nodes, one symbol-table node and a local heap of link names), and one
// version 1 object header per dataset holding the dataspace (rank 1, current
// and maximum size), the datatype (little-endian IEEE double, or a
// little-endian two's-complement integer), the fill-value message, a
// contiguous layout, the modification time and one attribute message per
// parameter (a one-element double or int32 array).  The dataset values are
// stored contiguously after each header.  Datasets are linked in name order
// (the order of the B-tree), as the library does.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace h5min {

struct Attribute {
  std::string name;
  bool is_double = true;  // else int32
  double d = 0.0;
  int32_t i = 0;
};

enum class Type { F64, U64 };

struct Dataset {
  std::string name;
  Type type = Type::F64;
  std::vector<uint8_t> bytes;  // little-endian values
  uint64_t count = 0;
  std::vector<Attribute> attributes;
};

class File {
 public:
  void add(const std::string& name, const double* values, uint64_t count, std::vector<Attribute> attrs = {});
  void add(const std::string& name, const uint64_t* values, uint64_t count, std::vector<Attribute> attrs = {});
  // Write the file (truncating); mtime is stored in every dataset's
  // modification-time message.  Throws std::runtime_error on failure.
  void write(const std::string& path, uint32_t mtime) const;

 private:
  std::vector<Dataset> sets_;
};

}  // namespace h5min
