// TEST INFRASTRUCTURE: in-process file store behind the H5Cpp.h stand-in, plus the C
// entry points the test harness uses to put setup datasets in and take outputs out, and
// pd_ref_run(), which calls the reference's own main() (compiled with -Dmain=pd_ref_main).
#include "H5Cpp.h"

#include <getopt.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <mutex>
#include <string>

namespace H5 {

const PredType PredType::NATIVE_DOUBLE(SHIM_F64);
const PredType PredType::NATIVE_INT(SHIM_I32);
const PredType PredType::NATIVE_UINT(SHIM_U32);

struct ShimDataset {
  int type = SHIM_F64;
  std::vector<hsize_t> dims;
  std::vector<unsigned char> bytes;
};

struct ShimFile {
  std::map<std::string, std::shared_ptr<ShimDataset>> sets;
  std::vector<std::string> groups;
};

static std::map<std::string, std::shared_ptr<ShimFile>> &store() {
  static std::map<std::string, std::shared_ptr<ShimFile>> s;
  return s;
}

static size_t type_size(int t) {
  switch (t) {
    case SHIM_F64: case SHIM_I64: case SHIM_U64: return 8;
    default: return 4;
  }
}

static std::string norm_path(const char *p) {
  std::string s(p);
  while (!s.empty() && s[0] == '/') s.erase(0, 1);
  return s;
}

static double load_as_double(const unsigned char *src, int t) {
  switch (t) {
    case SHIM_F64: { double v; std::memcpy(&v, src, 8); return v; }
    case SHIM_F32: { float v; std::memcpy(&v, src, 4); return v; }
    case SHIM_I32: { int32_t v; std::memcpy(&v, src, 4); return (double)v; }
    case SHIM_U32: { uint32_t v; std::memcpy(&v, src, 4); return (double)v; }
    case SHIM_I64: { int64_t v; std::memcpy(&v, src, 8); return (double)v; }
    case SHIM_U64: { uint64_t v; std::memcpy(&v, src, 8); return (double)v; }
  }
  return 0;
}
static int64_t load_as_int(const unsigned char *src, int t) {
  switch (t) {
    case SHIM_F64: { double v; std::memcpy(&v, src, 8); return (int64_t)v; }
    case SHIM_F32: { float v; std::memcpy(&v, src, 4); return (int64_t)v; }
    case SHIM_I32: { int32_t v; std::memcpy(&v, src, 4); return v; }
    case SHIM_U32: { uint32_t v; std::memcpy(&v, src, 4); return v; }
    case SHIM_I64: { int64_t v; std::memcpy(&v, src, 8); return v; }
    case SHIM_U64: { uint64_t v; std::memcpy(&v, src, 8); return (int64_t)v; }
  }
  return 0;
}

static void convert(const unsigned char *src, int st, unsigned char *dst, int dt, size_t n) {
  size_t ss = type_size(st), ds = type_size(dt);
  if (st == dt) {
    std::memcpy(dst, src, n * ss);
    return;
  }
  for (size_t i = 0; i < n; ++i) {
    const unsigned char *s = src + i * ss;
    unsigned char *d = dst + i * ds;
    switch (dt) {
      case SHIM_F64: { double v = load_as_double(s, st); std::memcpy(d, &v, 8); break; }
      case SHIM_F32: { float v = (float)load_as_double(s, st); std::memcpy(d, &v, 4); break; }
      case SHIM_I32: { int32_t v = (int32_t)load_as_int(s, st); std::memcpy(d, &v, 4); break; }
      case SHIM_U32: { uint32_t v = (uint32_t)load_as_int(s, st); std::memcpy(d, &v, 4); break; }
      case SHIM_I64: { int64_t v = load_as_int(s, st); std::memcpy(d, &v, 8); break; }
      case SHIM_U64: { uint64_t v = (uint64_t)load_as_int(s, st); std::memcpy(d, &v, 8); break; }
    }
  }
}

static size_t count_of(const std::vector<hsize_t> &dims) {
  size_t n = 1;
  for (hsize_t d : dims) n *= (size_t)d;
  return n;
}

H5File::H5File(const char *name, unsigned flags) {
  auto &s = store();
  if (flags == H5F_ACC_TRUNC) {
    f = std::make_shared<ShimFile>();
    s[name] = f;
  } else {
    auto it = s.find(name);
    if (it == s.end()) throw std::runtime_error(std::string("shim H5File: no such file ") + name);
    f = it->second;
  }
}

void H5File::createGroup(const char *name) { f->groups.push_back(norm_path(name)); }

DataSet H5File::createDataSet(const char *name, const PredType &t, const DataSpace &sp) {
  auto d = std::make_shared<ShimDataset>();
  d->type = t.code;
  d->dims = sp.dims;
  d->bytes.assign(count_of(sp.dims) * type_size(t.code), 0);
  f->sets[norm_path(name)] = d;
  return DataSet(d);
}

DataSet H5File::openDataSet(const char *name) {
  auto it = f->sets.find(norm_path(name));
  if (it == f->sets.end()) throw std::runtime_error(std::string("shim H5File: no dataset ") + name);
  return DataSet(it->second);
}

void DataSet::write(const void *buf, const PredType &t) const {
  size_t n = count_of(ds->dims);
  convert((const unsigned char *)buf, t.code, ds->bytes.data(), ds->type, n);
}

void DataSet::read(void *buf, const PredType &t, const DataSpace &) const {
  size_t n = count_of(ds->dims);
  convert(ds->bytes.data(), ds->type, (unsigned char *)buf, t.code, n);
}

DataSpace DataSet::getSpace() const {
  DataSpace s;
  s.dims = ds->dims;
  return s;
}

}  // namespace H5

int pd_ref_main(int argc, char *argv[]);

extern "C" {

void h5mem_clear(void) { H5::store().clear(); }

void h5mem_drop(const char *file) { H5::store().erase(file); }

int h5mem_put(const char *file, const char *path, int type, int rank, const uint64_t *dims,
              const void *data) {
  auto &s = H5::store();
  auto it = s.find(file);
  std::shared_ptr<H5::ShimFile> f;
  if (it == s.end()) {
    f = std::make_shared<H5::ShimFile>();
    s[file] = f;
  } else {
    f = it->second;
  }
  auto d = std::make_shared<H5::ShimDataset>();
  d->type = type;
  d->dims.assign(dims, dims + rank);
  size_t nb = H5::count_of(d->dims) * H5::type_size(type);
  d->bytes.resize(nb);
  if (nb) std::memcpy(d->bytes.data(), data, nb);
  f->sets[H5::norm_path(path)] = d;
  return 0;
}

// Returns rank (>= 0) and fills type/dims, or -1 if absent.
int h5mem_info(const char *file, const char *path, int *type, uint64_t *dims) {
  auto &s = H5::store();
  auto it = s.find(file);
  if (it == s.end()) return -1;
  auto jt = it->second->sets.find(H5::norm_path(path));
  if (jt == it->second->sets.end()) return -1;
  *type = jt->second->type;
  for (size_t i = 0; i < jt->second->dims.size(); ++i) dims[i] = jt->second->dims[i];
  return (int)jt->second->dims.size();
}

int h5mem_get(const char *file, const char *path, int type, void *out) {
  auto &s = H5::store();
  auto it = s.find(file);
  if (it == s.end()) return -1;
  auto jt = it->second->sets.find(H5::norm_path(path));
  if (jt == it->second->sets.end()) return -1;
  H5::convert(jt->second->bytes.data(), jt->second->type, (unsigned char *)out, type,
              H5::count_of(jt->second->dims));
  return 0;
}

// Newline-separated list of the file names in the store; returns the needed length.
size_t h5mem_files(char *buf, size_t cap) {
  std::string all;
  for (auto &kv : H5::store()) all += kv.first + "\n";
  if (buf && cap) {
    size_t n = all.size() < cap - 1 ? all.size() : cap - 1;
    std::memcpy(buf, all.data(), n);
    buf[n] = 0;
  }
  return all.size() + 1;
}

// Runs the reference's main() with the given argv; stdout goes to `log_path` when given.
int pd_ref_run(int argc, char **argv, const char *log_path) {
  optind = 0;  // re-initialise getopt for repeated calls in one process
  std::streambuf *old = nullptr;
  std::ofstream log;
  if (log_path && log_path[0]) {
    log.open(log_path);
    old = std::cout.rdbuf(log.rdbuf());
  }
  int rc = 1;
  try {
    rc = pd_ref_main(argc, argv);
  } catch (const std::exception &e) {
    std::cerr << "pd_ref_run: " << e.what() << std::endl;
    rc = 2;
  }
  if (old) std::cout.rdbuf(old);
  return rc;
}

}  // extern "C"
