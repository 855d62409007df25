// h5lite.h -- a small HDF5 reader/writer for the files of PeriDEM's boundary: the setup schema
// (exp_dict.py:2119-2185) and the output frames (timeloop.h:321-350, 801-964).
//
// Writer: superblock version 0, version-1 object headers, groups as symbol tables (one
// local heap, a single-leaf v1 B-tree and one symbol-table node per group, leaf K sized to the
// largest group), contiguous datasets of little-endian IEEE f32/f64 or 32/64-bit integers.
// Reader: superblock versions 0-3; version-1 and version-2 object headers (with continuation
// blocks); groups stored as symbol tables (any B-tree depth) or as compact link messages;
// contiguous and compact layouts; fixed-point and floating-point element types of either byte
// order, converted on read to the requested type (like HDF5's read conversion).
#ifndef PD_H5LITE_H
#define PD_H5LITE_H
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

namespace h5lite {

enum DType { F64 = 1, I32 = 2, U32 = 3, I64 = 4, U64 = 5, F32 = 6 };
size_t dtype_size(int t);

class Writer {
 public:
  // path like "P_00000/Pos" or "/wall/allow_wall"; groups are created implicitly
  void add(const std::string &path, int dtype, const std::vector<uint64_t> &dims, const void *data);
  void add_group(const std::string &path);
  bool write(const std::string &filename, std::string &err) const;

 private:
  struct DS {
    int dtype;
    std::vector<uint64_t> dims;
    std::vector<uint8_t> bytes;
  };
  std::map<std::string, DS> sets_;
  std::vector<std::string> groups_;
};

struct Info {
  int rank = 0;
  std::vector<uint64_t> dims;
  int cls = 0;       // 0 fixed-point, 1 floating-point
  int size = 0;      // element bytes
  bool is_signed = false;
  bool big_endian = false;
  int layout = 1;    // 0 compact, 1 contiguous
  uint64_t addr = 0, nbytes = 0;
  std::vector<uint8_t> compact;
};

class Reader {
 public:
  bool open(const std::string &filename, std::string &err);
  bool has(const std::string &path) const;
  const Info *info(const std::string &path) const;
  // element count and data converted to dtype; dims returned
  bool read(const std::string &path, int dtype, std::vector<uint8_t> &out, std::vector<uint64_t> &dims,
            std::string &err) const;
  template <typename T>
  bool read_vec(const std::string &path, int dtype, std::vector<T> &out, std::vector<uint64_t> &dims,
                std::string &err) const {
    std::vector<uint8_t> b;
    if (!read(path, dtype, b, dims, err)) return false;
    out.resize(b.size() / sizeof(T));
    if (!b.empty()) memcpy_(out.data(), b.data(), b.size());
    return true;
  }
  std::vector<std::string> paths() const;

 private:
  static void memcpy_(void *d, const void *s, size_t n);
  bool walk_object(uint64_t addr, const std::string &prefix, int depth, std::string &err);
  bool read_header_messages(uint64_t addr, std::vector<std::pair<int, std::vector<uint8_t>>> &msgs,
                            std::string &err);
  bool walk_symbol_table(uint64_t btree, uint64_t heap, const std::string &prefix, int depth, std::string &err);
  bool walk_btree(uint64_t addr, uint64_t heap_data, const std::string &prefix, int depth, std::string &err);
  std::vector<uint8_t> file_;
  int so_ = 8, sl_ = 8;  // size of offsets / lengths
  uint64_t base_ = 0;
  std::map<std::string, Info> sets_;
};

}  // namespace h5lite
#endif
