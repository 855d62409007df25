// TEST INFRASTRUCTURE: stand-in for the HDF5 C++ API surface used by PeriDEM's
// src/read/rw_hdf5.h and src/particle/timeloop.h (H5File, DataSet, DataSpace, PredType,
// createGroup). Files live in an in-process store (h5mem.cpp) that the test harness fills
// with the setup datasets and reads the outputs back from. Reads convert between the
// stored element type and the requested native type, like HDF5's conversion path.
#ifndef PD_SHIM_H5CPP_H
#define PD_SHIM_H5CPP_H
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

typedef unsigned long long hsize_t;
#define H5F_ACC_RDONLY 0u
#define H5F_ACC_TRUNC 2u

namespace H5 {

// element type codes shared with h5mem.cpp
enum ShimType { SHIM_F64 = 1, SHIM_I32 = 2, SHIM_U32 = 3, SHIM_I64 = 4, SHIM_U64 = 5, SHIM_F32 = 6 };

class PredType {
 public:
  int code;
  explicit PredType(int c) : code(c) {}
  static const PredType NATIVE_DOUBLE;
  static const PredType NATIVE_INT;
  static const PredType NATIVE_UINT;
};

class DataSpace {
 public:
  std::vector<hsize_t> dims;
  DataSpace() {}
  DataSpace(int rank, const hsize_t *d) : dims(d, d + rank) {}
  int getSimpleExtentDims(hsize_t *d, hsize_t *maxdims) const {
    for (size_t i = 0; i < dims.size(); ++i) {
      d[i] = dims[i];
      if (maxdims) maxdims[i] = dims[i];
    }
    return (int)dims.size();
  }
};

struct ShimDataset;
struct ShimFile;

class DataSet {
 public:
  std::shared_ptr<ShimDataset> ds;
  DataSet() {}
  explicit DataSet(std::shared_ptr<ShimDataset> d) : ds(d) {}
  void write(const void *buf, const PredType &t) const;
  void read(void *buf, const PredType &t, const DataSpace &s) const;
  void read(void *buf, const PredType &t) const { read(buf, t, getSpace()); }
  DataSpace getSpace() const;
};

class H5File {
 public:
  std::shared_ptr<ShimFile> f;
  H5File(const char *name, unsigned flags);
  H5File(const std::string &name, unsigned flags) : H5File(name.c_str(), flags) {}
  void createGroup(const char *name);
  void createGroup(const std::string &name) { createGroup(name.c_str()); }
  DataSet createDataSet(const char *name, const PredType &t, const DataSpace &s);
  DataSet createDataSet(const std::string &name, const PredType &t, const DataSpace &s) {
    return createDataSet(name.c_str(), t, s);
  }
  DataSet openDataSet(const char *name);
  DataSet openDataSet(const std::string &name) { return openDataSet(name.c_str()); }
  void close() {}
};

}  // namespace H5
#endif
