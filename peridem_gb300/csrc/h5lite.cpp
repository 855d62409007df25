// h5lite.cpp -- see h5lite.h. Written from the HDF5 file format specification (superblock,
// object headers, symbol-table groups, local heaps, version-1 B-trees, symbol table nodes,
// dataspace/datatype/layout messages); it implements only the subset described there.
#include "h5lite.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <set>

namespace h5lite {

namespace {

const uint64_t UNDEF = ~0ull;
const uint8_t SIG[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
const int kInternalK = 16;  // group internal node K (B-tree fan-out 2K)

std::string norm(const std::string &p) {
  std::string s = p;
  while (!s.empty() && s[0] == '/') s.erase(0, 1);
  while (!s.empty() && s.back() == '/') s.pop_back();
  return s;
}
inline uint64_t align8(uint64_t x) { return (x + 7) & ~7ull; }

struct Buf {
  std::vector<uint8_t> b;
  void resize(uint64_t n) { b.resize(n, 0); }
  void u8(uint64_t at, uint8_t v) { b[at] = v; }
  void u16(uint64_t at, uint16_t v) { std::memcpy(&b[at], &v, 2); }
  void u32(uint64_t at, uint32_t v) { std::memcpy(&b[at], &v, 4); }
  void u64(uint64_t at, uint64_t v) { std::memcpy(&b[at], &v, 8); }
  void raw(uint64_t at, const void *p, uint64_t n) {
    if (n) std::memcpy(&b[at], p, n);
  }
};

// datatype message body (class bits, size, properties) for our element types
std::vector<uint8_t> dtype_message(int t) {
  std::vector<uint8_t> m;
  auto put32 = [&](uint32_t v) {
    for (int i = 0; i < 4; ++i) m.push_back((uint8_t)(v >> (8 * i)));
  };
  auto put16 = [&](uint16_t v) {
    m.push_back((uint8_t)v);
    m.push_back((uint8_t)(v >> 8));
  };
  if (t == F64 || t == F32) {
    const bool d = t == F64;
    m.push_back(0x11);                   // version 1, class 1 (floating point)
    m.push_back(0x20);                   // little endian, implied-msb mantissa normalisation
    m.push_back(d ? 63 : 31);            // sign bit location
    m.push_back(0);
    put32(d ? 8 : 4);                    // element size
    put16(0);                            // bit offset
    put16(d ? 64 : 32);                  // bit precision
    m.push_back(d ? 52 : 23);            // exponent location
    m.push_back(d ? 11 : 8);             // exponent size
    m.push_back(0);                      // mantissa location
    m.push_back(d ? 52 : 23);            // mantissa size
    put32(d ? 1023 : 127);               // exponent bias
  } else {
    const bool sgn = (t == I32 || t == I64);
    const uint32_t sz = (t == I64 || t == U64) ? 8 : 4;
    m.push_back(0x10);                   // version 1, class 0 (fixed point)
    m.push_back(sgn ? 0x08 : 0x00);      // little endian, signed bit
    m.push_back(0);
    m.push_back(0);
    put32(sz);
    put16(0);
    put16((uint16_t)(8 * sz));
  }
  return m;
}

}  // namespace

size_t dtype_size(int t) {
  switch (t) {
    case F64: case I64: case U64: return 8;
    default: return 4;
  }
}

void Writer::add(const std::string &path, int dtype, const std::vector<uint64_t> &dims, const void *data) {
  DS d;
  d.dtype = dtype;
  d.dims = dims;
  uint64_t n = 1;
  for (uint64_t x : dims) n *= x;
  d.bytes.resize(n * dtype_size(dtype));
  if (n && data) std::memcpy(d.bytes.data(), data, d.bytes.size());
  sets_[norm(path)] = std::move(d);
}

void Writer::add_group(const std::string &path) { groups_.push_back(norm(path)); }

bool Writer::write(const std::string &filename, std::string &err) const {
  // group tree: group path -> sorted child names (groups and datasets)
  std::map<std::string, std::set<std::string>> children;
  std::set<std::string> is_group;
  children[""];
  is_group.insert("");
  auto add_path = [&](const std::string &p, bool leaf_is_group) {
    std::string parent;
    size_t pos = 0;
    std::string cur;
    while (true) {
      size_t s = p.find('/', pos);
      std::string name = p.substr(pos, s == std::string::npos ? std::string::npos : s - pos);
      std::string full = cur.empty() ? name : cur + "/" + name;
      children[cur].insert(name);
      if (s == std::string::npos) {
        if (leaf_is_group) {
          is_group.insert(full);
          children[full];
        }
        break;
      }
      is_group.insert(full);
      children[full];
      cur = full;
      pos = s + 1;
    }
  };
  for (auto &kv : sets_) add_path(kv.first, false);
  for (auto &g : groups_)
    if (!g.empty()) add_path(g, true);
  size_t maxc = 1;
  for (auto &kv : children) maxc = std::max(maxc, kv.second.size());
  const int leafK = (int)std::max<size_t>(4, (maxc + 1) / 2);

  // ---- address assignment
  struct GroupLay {
    uint64_t ohdr, heap, heap_data, heap_size, btree, snod;
    std::map<std::string, uint64_t> name_off;
  };
  struct SetLay {
    uint64_t ohdr, ohdr_size, data;
  };
  std::map<std::string, GroupLay> gl;
  std::map<std::string, SetLay> sl;
  uint64_t at = 96;  // superblock v0
  const uint64_t group_ohdr_size = 256;
  const uint64_t btree_size = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
  const uint64_t snod_size = 8 + (uint64_t)2 * leafK * 40;
  for (auto &kv : children) {
    if (!is_group.count(kv.first)) continue;
    GroupLay g;
    g.ohdr = at;
    at += group_ohdr_size;
    g.heap = at;
    at += 32;
    g.heap_data = at;
    uint64_t hs = 8;  // offset 0: the empty name
    for (auto &nm : kv.second) {
      g.name_off[nm] = hs;
      hs += align8(nm.size() + 1);
    }
    g.heap_size = hs;
    at += hs;
    g.btree = at;
    at += btree_size;
    g.snod = kv.second.empty() ? UNDEF : at;
    if (!kv.second.empty()) at += snod_size;
    gl[kv.first] = g;
  }
  for (auto &kv : sets_) {
    SetLay s;
    s.ohdr = at;
    const uint64_t rank = kv.second.dims.size();
    const uint64_t dspace = 8 + align8(8 + 8 * rank);
    const uint64_t dtype = 8 + align8(dtype_message(kv.second.dtype).size());
    const uint64_t fill = 8 + 8;
    const uint64_t layout = 8 + 24;
    s.ohdr_size = 16 + dspace + dtype + fill + layout;
    at += s.ohdr_size;
    at = align8(at);
    s.data = kv.second.bytes.empty() ? UNDEF : at;
    at += align8(kv.second.bytes.size());
    sl[kv.first] = s;
  }
  const uint64_t eof = at;

  // ---- serialisation
  Buf f;
  f.resize(eof);
  f.raw(0, SIG, 8);
  f.u8(8, 0);   // superblock version
  f.u8(9, 0);   // free-space version
  f.u8(10, 0);  // root symbol table entry version
  f.u8(11, 0);
  f.u8(12, 0);  // shared header message format version
  f.u8(13, 8);  // size of offsets
  f.u8(14, 8);  // size of lengths
  f.u8(15, 0);
  f.u16(16, (uint16_t)leafK);
  f.u16(18, (uint16_t)kInternalK);
  f.u32(20, 0);
  f.u64(24, 0);      // base address
  f.u64(32, UNDEF);  // free-space info
  f.u64(40, eof);
  f.u64(48, UNDEF);  // driver info
  auto sym_entry = [&](uint64_t pos, uint64_t name_off, uint64_t ohdr, const GroupLay *g) {
    f.u64(pos, name_off);
    f.u64(pos + 8, ohdr);
    f.u32(pos + 16, g ? 1 : 0);
    f.u32(pos + 20, 0);
    if (g) {
      f.u64(pos + 24, g->btree);
      f.u64(pos + 32, g->heap);
    }
  };
  sym_entry(56, 0, gl[""].ohdr, &gl[""]);

  for (auto &kv : children) {
    if (!is_group.count(kv.first)) continue;
    const GroupLay &g = gl[kv.first];
    // object header v1: symbol table message + NIL padding
    uint64_t o = g.ohdr;
    f.u8(o, 1);
    f.u8(o + 1, 0);
    f.u16(o + 2, 2);
    f.u32(o + 4, 1);
    f.u32(o + 8, (uint32_t)(group_ohdr_size - 16));
    uint64_t m = o + 16;
    f.u16(m, 0x11);
    f.u16(m + 2, 16);
    f.u8(m + 4, 0);
    f.u64(m + 8, g.btree);
    f.u64(m + 16, g.heap);
    m += 24;
    f.u16(m, 0x0);  // NIL message filling the rest
    f.u16(m + 2, (uint16_t)(group_ohdr_size - 16 - 24 - 8));
    // local heap
    f.raw(g.heap, "HEAP", 4);
    f.u8(g.heap + 4, 0);
    f.u64(g.heap + 8, g.heap_size);
    f.u64(g.heap + 16, UNDEF);
    f.u64(g.heap + 24, g.heap_data);
    for (auto &nm : kv.second) f.raw(g.heap_data + g.name_off.at(nm), nm.c_str(), nm.size() + 1);
    // B-tree (group node, leaf level) with one child: the symbol table node
    f.raw(g.btree, "TREE", 4);
    f.u8(g.btree + 4, 0);
    f.u8(g.btree + 5, 0);
    f.u16(g.btree + 6, kv.second.empty() ? 0 : 1);
    f.u64(g.btree + 8, UNDEF);
    f.u64(g.btree + 16, UNDEF);
    f.u64(g.btree + 24, 0);  // key 0: the empty name
    if (!kv.second.empty()) {
      f.u64(g.btree + 32, g.snod);
      f.u64(g.btree + 40, g.name_off.at(*kv.second.rbegin()));  // key 1: the largest name
      f.raw(g.snod, "SNOD", 4);
      f.u8(g.snod + 4, 1);
      f.u8(g.snod + 5, 0);
      f.u16(g.snod + 6, (uint16_t)kv.second.size());
      uint64_t e = g.snod + 8;
      for (auto &nm : kv.second) {  // std::set keeps names sorted
        const std::string full = kv.first.empty() ? nm : kv.first + "/" + nm;
        if (is_group.count(full)) {
          sym_entry(e, g.name_off.at(nm), gl[full].ohdr, &gl[full]);
        } else {
          sym_entry(e, g.name_off.at(nm), sl[full].ohdr, nullptr);
        }
        e += 40;
      }
    }
  }
  for (auto &kv : sets_) {
    const SetLay &s = sl[kv.first];
    const DS &d = kv.second;
    uint64_t o = s.ohdr;
    f.u8(o, 1);
    f.u8(o + 1, 0);
    f.u16(o + 2, 4);
    f.u32(o + 4, 1);
    f.u32(o + 8, (uint32_t)(s.ohdr_size - 16));
    uint64_t m = o + 16;
    // dataspace v1
    const uint64_t rank = d.dims.size();
    const uint64_t dsz = align8(8 + 8 * rank);
    f.u16(m, 0x01);
    f.u16(m + 2, (uint16_t)dsz);
    f.u8(m + 8, 1);
    f.u8(m + 9, (uint8_t)rank);
    f.u8(m + 10, 0);
    for (uint64_t i = 0; i < rank; ++i) f.u64(m + 16 + 8 * i, d.dims[i]);
    m += 8 + dsz;
    // datatype
    std::vector<uint8_t> dt = dtype_message(d.dtype);
    const uint64_t tsz = align8(dt.size());
    f.u16(m, 0x03);
    f.u16(m + 2, (uint16_t)tsz);
    f.u8(m + 4, 1);  // constant
    f.raw(m + 8, dt.data(), dt.size());
    m += 8 + tsz;
    // fill value v2: allocation time late, written if set, not defined
    f.u16(m, 0x05);
    f.u16(m + 2, 8);
    f.u8(m + 4, 1);
    f.u8(m + 8, 2);
    f.u8(m + 9, 2);
    f.u8(m + 10, 2);
    f.u8(m + 11, 0);
    m += 16;
    // layout v3 contiguous
    f.u16(m, 0x08);
    f.u16(m + 2, 24);
    f.u8(m + 8, 3);
    f.u8(m + 9, 1);
    f.u64(m + 10, s.data);
    f.u64(m + 18, d.bytes.size());
    if (!d.bytes.empty()) f.raw(s.data, d.bytes.data(), d.bytes.size());
  }
  std::ofstream out(filename, std::ios::binary | std::ios::trunc);
  if (!out) {
    err = "cannot open " + filename + " for writing";
    return false;
  }
  out.write(reinterpret_cast<const char *>(f.b.data()), (std::streamsize)f.b.size());
  if (!out) {
    err = "write failed: " + filename;
    return false;
  }
  return true;
}

// ----------------------------------------------------------------------------------------
// Reader

void Reader::memcpy_(void *d, const void *s, size_t n) { std::memcpy(d, s, n); }

namespace {
struct Cur {
  const std::vector<uint8_t> &f;
  bool ok = true;
  uint64_t get(uint64_t at, int n) {
    if (at + n > f.size()) {
      ok = false;
      return 0;
    }
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= (uint64_t)f[at + i] << (8 * i);
    return v;
  }
};
}  // namespace

bool Reader::open(const std::string &filename, std::string &err) {
  std::ifstream in(filename, std::ios::binary);
  if (!in) {
    err = "cannot open " + filename;
    return false;
  }
  file_.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
  sets_.clear();
  if (file_.size() < 48 || std::memcmp(file_.data(), SIG, 8) != 0) {
    err = filename + ": not an HDF5 file (signature)";
    return false;
  }
  Cur c{file_};
  const int ver = (int)c.get(8, 1);
  uint64_t root = 0;
  if (ver == 0 || ver == 1) {
    so_ = (int)c.get(13, 1);
    sl_ = (int)c.get(14, 1);
    uint64_t p = 24 + (ver == 1 ? 4 : 0);
    base_ = c.get(p, so_);
    p += 4 * so_;  // base, free space, eof, driver
    root = c.get(p + so_, so_);  // root symbol table entry: name offset, object header
  } else if (ver == 2 || ver == 3) {
    so_ = (int)c.get(9, 1);
    sl_ = (int)c.get(10, 1);
    uint64_t p = 12;
    base_ = c.get(p, so_);
    root = c.get(p + 3 * so_, so_);
  } else {
    err = filename + ": unsupported superblock version " + std::to_string(ver);
    return false;
  }
  if (!c.ok || (so_ != 8 && so_ != 4) || (sl_ != 8 && sl_ != 4)) {
    err = filename + ": corrupt superblock";
    return false;
  }
  return walk_object(root, "", 0, err);
}

bool Reader::read_header_messages(uint64_t addr, std::vector<std::pair<int, std::vector<uint8_t>>> &msgs,
                                  std::string &err) {
  Cur c{file_};
  addr += base_;
  std::vector<std::pair<uint64_t, uint64_t>> blocks;
  bool v2 = false;
  uint64_t nmsgs = ~0ull;
  int v2flags = 0;
  if (addr + 4 <= file_.size() && std::memcmp(&file_[addr], "OHDR", 4) == 0) {
    v2 = true;
    v2flags = (int)c.get(addr + 5, 1);
    uint64_t p = addr + 6;
    if (v2flags & 0x20) p += 16;
    if (v2flags & 0x10) p += 4;
    const int szb = 1 << (v2flags & 3);
    const uint64_t chunk = c.get(p, szb);
    p += szb;
    blocks.push_back({p, chunk});
  } else {
    if (c.get(addr, 1) != 1) {
      err = "unsupported object header version at " + std::to_string(addr);
      return false;
    }
    nmsgs = c.get(addr + 2, 2);
    const uint64_t size = c.get(addr + 8, 4);
    blocks.push_back({addr + 16, size});
  }
  uint64_t seen = 0;
  for (size_t bi = 0; bi < blocks.size() && bi < 4096; ++bi) {
    uint64_t p = blocks[bi].first, end = p + blocks[bi].second;
    if (v2 && bi > 0) {
      if (p + 4 > file_.size() || std::memcmp(&file_[p], "OCHK", 4) != 0) {
        err = "bad continuation block";
        return false;
      }
      p += 4;
      end -= 4;  // checksum
    }
    const uint64_t hdr = v2 ? 4 + ((v2flags & 0x04) ? 2 : 0) : 8;
    while (p + hdr <= end && seen < nmsgs) {
      int type;
      uint64_t size;
      if (v2) {
        type = (int)c.get(p, 1);
        size = c.get(p + 1, 2);
      } else {
        type = (int)c.get(p, 2);
        size = c.get(p + 2, 2);
      }
      p += hdr;
      if (p + size > file_.size()) {
        err = "object header message out of file";
        return false;
      }
      std::vector<uint8_t> data(file_.begin() + p, file_.begin() + p + size);
      if (type == 0x10) {  // continuation
        Cur d{data};
        blocks.push_back({d.get(0, so_) + base_, d.get(so_, sl_)});
      }
      msgs.push_back({type, std::move(data)});
      p += size;
      ++seen;
    }
    if (v2 && bi == 0) {
      // v2 chunk #0 ends with a 4-byte checksum inside the chunk size
    }
  }
  if (!c.ok) {
    err = "truncated object header";
    return false;
  }
  return true;
}

bool Reader::walk_object(uint64_t addr, const std::string &prefix, int depth, std::string &err) {
  if (depth > 32) {
    err = "group nesting too deep";
    return false;
  }
  std::vector<std::pair<int, std::vector<uint8_t>>> msgs;
  if (!read_header_messages(addr, msgs, err)) return false;
  bool is_set = false, has_links = false;
  Info info;
  for (auto &m : msgs) {
    Cur d{m.second};
    switch (m.first) {
      case 0x11: {  // symbol table
        if (!walk_symbol_table(d.get(0, so_), d.get(so_, so_), prefix, depth, err)) return false;
        break;
      }
      case 0x06: {  // link message (compact group storage)
        has_links = true;
        const int flags = (int)d.get(1, 1);
        uint64_t p = 2;
        int ltype = 0;
        if (flags & 0x08) ltype = (int)d.get(p++, 1);
        if (flags & 0x04) p += 8;
        if (flags & 0x10) p += 1;
        const int lsz = 1 << (flags & 3);
        const uint64_t nlen = d.get(p, lsz);
        p += lsz;
        if (p + nlen > m.second.size()) {
          err = "bad link message";
          return false;
        }
        std::string name(m.second.begin() + p, m.second.begin() + p + nlen);
        p += nlen;
        if (ltype == 0) {
          const uint64_t obj = d.get(p, so_);
          if (!walk_object(obj, prefix.empty() ? name : prefix + "/" + name, depth + 1, err)) return false;
        }
        break;
      }
      case 0x02: {  // link info: dense storage is not handled
        const int flags = (int)d.get(1, 1);
        uint64_t p = 2 + ((flags & 1) ? 8 : 0);
        const uint64_t heap = d.get(p, so_);
        if (heap != UNDEF && (so_ == 8 || heap != 0xFFFFFFFFull)) {
          err = "group '" + prefix + "' uses dense link storage (fractal heap), not supported";
          return false;
        }
        break;
      }
      case 0x01: {  // dataspace
        const int ver = (int)d.get(0, 1);
        info.rank = (int)d.get(1, 1);
        uint64_t p = (ver == 1) ? 8 : 4;
        if (ver == 2 && d.get(3, 1) == 0) info.rank = 0;
        info.dims.clear();
        for (int i = 0; i < info.rank; ++i) info.dims.push_back(d.get(p + (uint64_t)i * sl_, sl_));
        break;
      }
      case 0x03: {  // datatype
        const int cls = (int)(d.get(0, 1) & 0x0F);
        const int b0 = (int)d.get(1, 1);
        info.cls = cls;
        info.size = (int)d.get(4, 4);
        info.big_endian = (b0 & 1) != 0;
        info.is_signed = (cls == 0) && (b0 & 0x08);
        if (cls != 0 && cls != 1) {
          err = "dataset '" + prefix + "': unsupported datatype class " + std::to_string(cls);
          return false;
        }
        break;
      }
      case 0x08: {  // data layout
        is_set = true;
        const int ver = (int)d.get(0, 1);
        if (ver == 3 || ver == 4) {
          const int cls = (int)d.get(1, 1);
          if (cls == 0) {
            info.layout = 0;
            const uint64_t n = d.get(2, 2);
            info.compact.assign(m.second.begin() + 4, m.second.begin() + 4 + std::min<uint64_t>(n, m.second.size() - 4));
          } else if (cls == 1) {
            info.layout = 1;
            info.addr = d.get(2, so_);
            info.nbytes = d.get(2 + so_, sl_);
          } else {
            err = "dataset '" + prefix + "': chunked/virtual layout not supported";
            return false;
          }
        } else if (ver == 1 || ver == 2) {
          const int nd = (int)d.get(1, 1);
          const int cls = (int)d.get(2, 1);
          if (cls == 1) {
            info.layout = 1;
            info.addr = d.get(8, so_);
            info.nbytes = ~0ull;
          } else if (cls == 0) {
            info.layout = 0;
            const uint64_t p = 8 + 4ull * nd;
            const uint64_t n = d.get(p, 4);
            info.compact.assign(m.second.begin() + p + 4, m.second.begin() + std::min<uint64_t>(p + 4 + n, m.second.size()));
          } else {
            err = "dataset '" + prefix + "': chunked layout not supported";
            return false;
          }
        }
        break;
      }
      default:
        break;
    }
  }
  (void)has_links;
  if (is_set) sets_[prefix] = info;
  return true;
}

bool Reader::walk_symbol_table(uint64_t btree, uint64_t heap, const std::string &prefix, int depth,
                               std::string &err) {
  Cur c{file_};
  const uint64_t h = heap + base_;
  if (h + 4 > file_.size() || std::memcmp(&file_[h], "HEAP", 4) != 0) {
    err = "bad local heap for group '" + prefix + "'";
    return false;
  }
  const uint64_t heap_data = c.get(h + 8 + 2 * sl_, so_) + base_;
  return walk_btree(btree, heap_data, prefix, depth, err);
}

bool Reader::walk_btree(uint64_t addr, uint64_t heap_data, const std::string &prefix, int depth, std::string &err) {
  Cur c{file_};
  const uint64_t a = addr + base_;
  if (a + 8 > file_.size() || std::memcmp(&file_[a], "TREE", 4) != 0) {
    err = "bad B-tree node in group '" + prefix + "'";
    return false;
  }
  const int level = (int)c.get(a + 5, 1);
  const uint64_t used = c.get(a + 6, 2);
  uint64_t p = a + 8 + 2 * so_;  // after siblings
  for (uint64_t i = 0; i < used; ++i) {
    p += sl_;  // key i
    const uint64_t child = c.get(p, so_);
    p += so_;
    if (level > 0) {
      if (!walk_btree(child, heap_data, prefix, depth, err)) return false;
      continue;
    }
    const uint64_t s = child + base_;
    if (s + 8 > file_.size() || std::memcmp(&file_[s], "SNOD", 4) != 0) {
      err = "bad symbol table node in group '" + prefix + "'";
      return false;
    }
    const uint64_t n = c.get(s + 6, 2);
    const uint64_t esz = 2 * so_ + 24;
    for (uint64_t e = 0; e < n; ++e) {
      const uint64_t ep = s + 8 + e * esz;
      const uint64_t noff = c.get(ep, so_);
      const uint64_t ohdr = c.get(ep + so_, so_);
      const uint64_t np = heap_data + noff;
      if (np >= file_.size()) {
        err = "name out of heap";
        return false;
      }
      std::string name(reinterpret_cast<const char *>(&file_[np]));
      const std::string full = prefix.empty() ? name : prefix + "/" + name;
      if (!walk_object(ohdr, full, depth + 1, err)) return false;
    }
  }
  if (!c.ok) {
    err = "truncated B-tree";
    return false;
  }
  return true;
}

bool Reader::has(const std::string &path) const { return sets_.count(norm(path)) != 0; }

const Info *Reader::info(const std::string &path) const {
  auto it = sets_.find(norm(path));
  return it == sets_.end() ? nullptr : &it->second;
}

std::vector<std::string> Reader::paths() const {
  std::vector<std::string> v;
  for (auto &kv : sets_) v.push_back(kv.first);
  return v;
}

bool Reader::read(const std::string &path, int dtype, std::vector<uint8_t> &out, std::vector<uint64_t> &dims,
                  std::string &err) const {
  const Info *in = info(path);
  if (!in) {
    err = "dataset '" + path + "' not found";
    return false;
  }
  dims = in->dims;
  uint64_t n = 1;
  for (uint64_t d : dims) n *= d;
  const uint64_t need = n * (uint64_t)in->size;
  const uint8_t *src = nullptr;
  std::vector<uint8_t> zeros;
  if (in->layout == 0) {
    if (in->compact.size() < need) {
      err = "compact dataset '" + path + "' too short";
      return false;
    }
    src = in->compact.data();
  } else if (in->addr == UNDEF || (so_ == 4 && in->addr == 0xFFFFFFFFull) || need == 0) {
    zeros.assign(need, 0);
    src = zeros.data();
  } else {
    const uint64_t a = in->addr + base_;
    if (a + need > file_.size()) {
      err = "dataset '" + path + "' extends past the end of the file";
      return false;
    }
    src = file_.data() + a;
  }
  const size_t osz = dtype_size(dtype);
  out.assign(n * osz, 0);
  for (uint64_t i = 0; i < n; ++i) {
    uint8_t e[8];
    const uint8_t *s = src + i * in->size;
    if (in->size > 8) {
      err = "element size above 8 bytes in '" + path + "'";
      return false;
    }
    for (int b = 0; b < in->size; ++b) e[b] = in->big_endian ? s[in->size - 1 - b] : s[b];
    double dv = 0;
    int64_t iv = 0;
    bool isf = in->cls == 1;
    if (isf) {
      if (in->size == 8) {
        std::memcpy(&dv, e, 8);
      } else if (in->size == 4) {
        float fv;
        std::memcpy(&fv, e, 4);
        dv = fv;
      } else {
        err = "unsupported float size in '" + path + "'";
        return false;
      }
    } else {
      uint64_t u = 0;
      for (int b = 0; b < in->size; ++b) u |= (uint64_t)e[b] << (8 * b);
      if (in->is_signed && in->size < 8 && (u >> (8 * in->size - 1)) & 1) u |= ~0ull << (8 * in->size);
      iv = (int64_t)u;
      if (!in->is_signed && in->size == 8) dv = (double)u; else dv = (double)iv;
    }
    uint8_t *d = out.data() + i * osz;
    switch (dtype) {
      case F64: { double v = isf ? dv : (in->is_signed ? (double)iv : (double)(uint64_t)iv); std::memcpy(d, &v, 8); break; }
      case F32: { float v = (float)(isf ? dv : (double)iv); std::memcpy(d, &v, 4); break; }
      case I32: { int32_t v = isf ? (int32_t)dv : (int32_t)iv; std::memcpy(d, &v, 4); break; }
      case U32: { uint32_t v = isf ? (uint32_t)dv : (uint32_t)iv; std::memcpy(d, &v, 4); break; }
      case I64: { int64_t v = isf ? (int64_t)dv : iv; std::memcpy(d, &v, 8); break; }
      case U64: { uint64_t v = isf ? (uint64_t)dv : (uint64_t)iv; std::memcpy(d, &v, 8); break; }
    }
  }
  return true;
}

}  // namespace h5lite
