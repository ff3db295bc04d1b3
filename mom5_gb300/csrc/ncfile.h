// netCDF classic files, the subset the restart files of fms_io use: CDF-1 and
// CDF-2 (64-bit offset) headers, fixed and record variables, numeric and text
// attributes.  Written by save_restart through mpp_io (mpp_io_connect.inc:654
// creates them with NF_64BIT_OFFSET).  Host code only; every value is
// big-endian on disk, assembled byte by byte so the same code runs on x86-64
// and aarch64 hosts.
#pragma once

#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

namespace mom5 {
namespace nc {

enum Type { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };
enum Tag { TAG_DIMENSION = 10, TAG_VARIABLE = 11, TAG_ATTRIBUTE = 12 };

inline int type_size(int t) {
  switch (t) {
    case NC_BYTE:
    case NC_CHAR: return 1;
    case NC_SHORT: return 2;
    case NC_INT:
    case NC_FLOAT: return 4;
    case NC_DOUBLE: return 8;
  }
  return 0;
}

inline uint64_t pad4(uint64_t n) { return (n + 3) & ~(uint64_t)3; }

struct Attr {
  std::string name;
  int type = NC_CHAR;
  uint64_t nelems = 0;
  std::vector<uint8_t> raw;  // big-endian values, unpadded
  std::string text() const { return type == NC_CHAR ? std::string(raw.begin(), raw.end()) : std::string(); }
  static Attr make_text(const std::string& n, const std::string& v) {
    Attr a;
    a.name = n;
    a.type = NC_CHAR;
    a.nelems = v.size();
    a.raw.assign(v.begin(), v.end());
    return a;
  }
};

struct Dim {
  std::string name;
  uint64_t len = 0;  // 0: the unlimited (record) dimension
};

struct Var {
  std::string name;
  std::vector<int> dimids;
  std::vector<Attr> atts;
  int type = NC_DOUBLE;
  uint64_t vsize = 0;  // bytes of the variable (of one record for a record variable), padded
  uint64_t begin = 0;  // file offset of the data (of record 0)
  bool record = false;
  const Attr* att(const char* n) const {
    for (const Attr& a : atts)
      if (a.name == n) return &a;
    return nullptr;
  }
};

struct File {
  int version = 2;
  uint64_t numrecs = 0;
  std::vector<Dim> dims;
  std::vector<Attr> gatts;
  std::vector<Var> vars;
  uint64_t recsize = 0;  // bytes between two records of one record variable
  int find(const std::string& n) const {
    for (size_t i = 0; i < vars.size(); ++i)
      if (vars[i].name == n) return (int)i;
    return -1;
  }
  int find_dim(const std::string& n) const {
    for (size_t i = 0; i < dims.size(); ++i)
      if (dims[i].name == n) return (int)i;
    return -1;
  }
  // elements of one record (record variable) or of the variable
  uint64_t count(const Var& v) const {
    uint64_t c = 1;
    for (int id : v.dimids)
      if (dims[id].len) c *= dims[id].len;
    return c;
  }
};

// ---- encoding -------------------------------------------------------------
struct Out {
  std::vector<uint8_t> b;
  void u32(uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
  }
  void u64(uint64_t v) {
    for (int s = 56; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
  }
  void bytes(const uint8_t* p, size_t n) {
    b.insert(b.end(), p, p + n);
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string& s) {
    u32((uint32_t)s.size());
    bytes((const uint8_t*)s.data(), s.size());
  }
  void atts(const std::vector<Attr>& a) {
    if (a.empty()) {
      u32(0);
      u32(0);
      return;
    }
    u32(TAG_ATTRIBUTE);
    u32((uint32_t)a.size());
    for (const Attr& x : a) {
      name(x.name);
      u32((uint32_t)x.type);
      u32((uint32_t)x.nelems);
      bytes(x.raw.data(), x.raw.size());
    }
  }
};

inline void be_double(double v, uint8_t* p) {
  uint64_t u;
  memcpy(&u, &v, 8);
  for (int q = 0; q < 8; ++q) p[q] = (uint8_t)(u >> (56 - 8 * q));
}
inline double double_be(const uint8_t* p) {
  uint64_t u = 0;
  for (int q = 0; q < 8; ++q) u = (u << 8) | p[q];
  double v;
  memcpy(&v, &u, 8);
  return v;
}
inline uint32_t u32_be(const uint8_t* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

// Header bytes of f (version 2: 64-bit offsets).
inline std::vector<uint8_t> encode_header(const File& f) {
  Out o;
  const uint8_t magic[4] = {'C', 'D', 'F', (uint8_t)f.version};
  o.b.insert(o.b.end(), magic, magic + 4);
  o.u32((uint32_t)f.numrecs);
  if (f.dims.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(TAG_DIMENSION);
    o.u32((uint32_t)f.dims.size());
    for (const Dim& d : f.dims) {
      o.name(d.name);
      o.u32((uint32_t)d.len);
    }
  }
  o.atts(f.gatts);
  if (f.vars.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(TAG_VARIABLE);
    o.u32((uint32_t)f.vars.size());
    for (const Var& v : f.vars) {
      o.name(v.name);
      o.u32((uint32_t)v.dimids.size());
      for (int id : v.dimids) o.u32((uint32_t)id);
      o.atts(v.atts);
      o.u32((uint32_t)v.type);
      o.u32(v.vsize > 0xFFFFFFFCull ? 0xFFFFFFFFu : (uint32_t)v.vsize);
      if (f.version == 1) o.u32((uint32_t)v.begin);
      else o.u64(v.begin);
    }
  }
  return o.b;
}

// Sizes and offsets of every variable: fixed variables first in definition
// order, then the records.  A single record variable is not padded.
inline void layout(File& f) {
  int nrec = 0;
  for (Var& v : f.vars) {
    v.record = !v.dimids.empty() && f.dims[v.dimids[0]].len == 0;
    nrec += v.record;
  }
  for (Var& v : f.vars) {
    uint64_t n = f.count(v) * type_size(v.type);
    v.vsize = (v.record && nrec == 1) ? n : pad4(n);
  }
  uint64_t off = encode_header(f).size();
  for (Var& v : f.vars)
    if (!v.record) {
      v.begin = off;
      off += v.vsize;
    }
  f.recsize = 0;
  for (Var& v : f.vars)
    if (v.record) {
      v.begin = off + f.recsize;
      f.recsize += v.vsize;
    }
}

// ---- decoding -------------------------------------------------------------
struct In {
  const uint8_t* p;
  size_t n, at = 0;
  bool ok = true;
  uint32_t u32() {
    if (at + 4 > n) return ok = false, 0;
    uint32_t v = u32_be(p + at);
    at += 4;
    return v;
  }
  uint64_t u64() {
    uint64_t hi = u32(), lo = u32();
    return (hi << 32) | lo;
  }
  std::string name() {
    uint32_t len = u32();
    if (!ok || at + len > n) return ok = false, std::string();
    std::string s((const char*)p + at, len);
    at += pad4(len);
    return s;
  }
  bool atts(std::vector<Attr>& out) {
    uint32_t tag = u32(), cnt = u32();
    if (!ok) return false;
    if (tag == 0 && cnt == 0) return true;
    if (tag != TAG_ATTRIBUTE) return ok = false;
    for (uint32_t q = 0; q < cnt && ok; ++q) {
      Attr a;
      a.name = name();
      a.type = (int)u32();
      a.nelems = u32();
      uint64_t bytes = a.nelems * (uint64_t)type_size(a.type);
      if (!ok || type_size(a.type) == 0 || at + bytes > n) return ok = false;
      a.raw.assign(p + at, p + at + bytes);
      at += pad4(bytes);
      out.push_back(a);
    }
    return ok;
  }
};

// Parse the header from the first bytes of a file; false on anything that is
// not a CDF-1/CDF-2 header (or a header longer than the bytes given).
inline bool decode_header(const uint8_t* p, size_t n, File& f) {
  In in{p, n};
  if (n < 8 || p[0] != 'C' || p[1] != 'D' || p[2] != 'F' || (p[3] != 1 && p[3] != 2)) return false;
  f = File();
  f.version = p[3];
  in.at = 4;
  f.numrecs = in.u32();
  uint32_t tag = in.u32(), cnt = in.u32();
  if (!in.ok || !(tag == TAG_DIMENSION || (tag == 0 && cnt == 0))) return false;
  for (uint32_t q = 0; q < cnt && in.ok; ++q) {
    Dim d;
    d.name = in.name();
    d.len = in.u32();
    f.dims.push_back(d);
  }
  if (!in.atts(f.gatts)) return false;
  tag = in.u32(), cnt = in.u32();
  if (!in.ok || !(tag == TAG_VARIABLE || (tag == 0 && cnt == 0))) return false;
  for (uint32_t q = 0; q < cnt && in.ok; ++q) {
    Var v;
    v.name = in.name();
    uint32_t nd = in.u32();
    if (!in.ok || nd > 64) return false;
    for (uint32_t r = 0; r < nd; ++r) {
      uint32_t id = in.u32();
      if (id >= f.dims.size()) return false;
      v.dimids.push_back((int)id);
    }
    if (!in.atts(v.atts)) return false;
    v.type = (int)in.u32();
    v.vsize = in.u32();
    v.begin = f.version == 1 ? in.u32() : in.u64();
    v.record = !v.dimids.empty() && f.dims[v.dimids[0]].len == 0;
    if (type_size(v.type) == 0) return false;
    f.vars.push_back(v);
  }
  if (!in.ok) return false;
  int nrec = 0;
  f.recsize = 0;
  for (Var& v : f.vars)
    if (v.record) {
      ++nrec;
      v.vsize = f.count(v) * type_size(v.type);  // the stored vsize may be clipped for huge variables
      f.recsize += pad4(v.vsize);
    }
  if (nrec == 1)
    for (Var& v : f.vars)
      if (v.record) f.recsize = v.vsize;
  return true;
}

// Read a whole header from an open file (grows the read until it parses).
inline bool read_header(FILE* fp, File& f) {
  std::vector<uint8_t> buf;
  for (size_t want = 4096; want <= ((size_t)1 << 28); want *= 4) {
    buf.resize(want);
    if (fseeko(fp, 0, SEEK_SET) != 0) return false;
    size_t got = fread(buf.data(), 1, want, fp);
    if (decode_header(buf.data(), got, f)) return true;
    if (got < want) return false;
  }
  return false;
}

}  // namespace nc
}  // namespace mom5
