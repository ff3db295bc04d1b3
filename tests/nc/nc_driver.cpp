// Test driver (CPU): the netCDF classic encoder and decoder of
// mom5_gb300/csrc/ncfile.h, exposed to ctypes so the tests can check them
// against scipy.io.netcdf_file in both directions.
#include "../../mom5_gb300/csrc/ncfile.h"

using namespace mom5::nc;

extern "C" {

// a file laid out like an fms restart: xaxis_1, yaxis_1, zaxis_1, Time and
// nvar 3-D double fields of one record, each with a text attribute
int nc_write_fields(const char* path, int ni, int nj, int nk, int nvar, const double* data) {
  File f;
  f.version = 2;
  f.numrecs = 1;
  f.dims = {{"xaxis_1", (uint64_t)ni}, {"yaxis_1", (uint64_t)nj}, {"zaxis_1", (uint64_t)nk}, {"Time", 0}};
  f.gatts = {Attr::make_text("filename", "test.res.nc")};
  const char* ax[3] = {"xaxis_1", "yaxis_1", "zaxis_1"};
  for (int a = 0; a < 3; ++a) {
    Var v;
    v.name = ax[a];
    v.dimids = {a};
    v.atts = {Attr::make_text("long_name", ax[a]), Attr::make_text("units", "none")};
    f.vars.push_back(v);
  }
  Var t;
  t.name = "Time";
  t.dimids = {3};
  t.atts = {Attr::make_text("long_name", "Time"), Attr::make_text("units", "time level")};
  f.vars.push_back(t);
  for (int q = 0; q < nvar; ++q) {
    Var v;
    v.name = "field" + std::to_string(q);
    v.dimids = {3, 2, 1, 0};
    v.atts = {Attr::make_text("long_name", v.name), Attr::make_text("checksum", "       0")};
    f.vars.push_back(v);
  }
  layout(f);
  FILE* fp = fopen(path, "wb");
  if (!fp) return -1;
  std::vector<uint8_t> h = encode_header(f);
  fwrite(h.data(), 1, h.size(), fp);
  size_t n3 = (size_t)ni * nj * nk;
  for (const Var& v : f.vars) {
    std::vector<uint8_t> b(v.vsize, 0);
    if (v.name == "xaxis_1" || v.name == "yaxis_1" || v.name == "zaxis_1" || v.name == "Time") {
      for (uint64_t e = 0; e < f.count(v); ++e) be_double((double)(e + 1), b.data() + 8 * e);
    } else {
      int q = atoi(v.name.c_str() + 5);
      for (size_t e = 0; e < n3; ++e) be_double(data[q * n3 + e], b.data() + 8 * e);
    }
    if (fseeko(fp, (off_t)v.begin, SEEK_SET) != 0) return -2;
    fwrite(b.data(), 1, b.size(), fp);
  }
  return fclose(fp) == 0 ? 0 : -3;
}

// read record `rec` (or the fixed data) of variable `name` as doubles; returns
// the element count, or < 0
long nc_read_var(const char* path, const char* name, long rec, double* out, long cap) {
  FILE* fp = fopen(path, "rb");
  if (!fp) return -1;
  File f;
  if (!read_header(fp, f)) return fclose(fp), -2;
  int vi = f.find(name);
  if (vi < 0) return fclose(fp), -3;
  const Var& v = f.vars[vi];
  uint64_t cnt = f.count(v), ts = type_size(v.type);
  if ((long)cnt > cap) return fclose(fp), -4;
  std::vector<uint8_t> b(cnt * ts);
  if (fseeko(fp, (off_t)(v.begin + (v.record ? rec * f.recsize : 0)), SEEK_SET) != 0 ||
      fread(b.data(), 1, b.size(), fp) != b.size())
    return fclose(fp), -5;
  for (uint64_t e = 0; e < cnt; ++e) {
    if (v.type == NC_DOUBLE) {
      out[e] = double_be(b.data() + 8 * e);
    } else if (v.type == NC_FLOAT) {
      uint32_t u = u32_be(b.data() + 4 * e);
      float x;
      memcpy(&x, &u, 4);
      out[e] = x;
    } else if (v.type == NC_INT) {
      out[e] = (double)(int32_t)u32_be(b.data() + 4 * e);
    } else {
      return fclose(fp), -6;
    }
  }
  fclose(fp);
  return (long)cnt;
}

// text attribute of a variable (or a global one with name == "")
int nc_read_text_att(const char* path, const char* var, const char* att, char* out, int cap) {
  FILE* fp = fopen(path, "rb");
  if (!fp) return -1;
  File f;
  bool ok = read_header(fp, f);
  fclose(fp);
  if (!ok) return -2;
  const std::vector<Attr>* list = &f.gatts;
  if (var && *var) {
    int vi = f.find(var);
    if (vi < 0) return -3;
    list = &f.vars[vi].atts;
  }
  for (const Attr& a : *list)
    if (a.name == att) {
      std::string s = a.text();
      if ((int)s.size() >= cap) return -4;
      memcpy(out, s.c_str(), s.size() + 1);
      return (int)s.size();
    }
  return -5;
}

}  // extern "C"
