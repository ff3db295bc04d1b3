// Restart files of the path's prognostic state in the layout fms_io writes
// (save_restart, fms_io.F90:2996-3260; axis and field metadata by
// mpp_write_meta, mpp_io_write.inc:440-520 and :677-890):
//   - dimensions xaxis_1, yaxis_1[, zaxis_1] and the unlimited Time;
//   - axis variables 1..n (double) with long_name, units "none", cartesian_axis;
//     Time (double) with long_name "Time", units "time level", cartesian_axis "T";
//   - one double variable per field, dimensions (Time, zaxis_1, yaxis_1, xaxis_1)
//     over the compute domain, attributes long_name (the field name), units
//     "none" and checksum: the sum of the fields' 64-bit patterns written with
//     Fortran's Z16 edit descriptor (mpp_chksum, mpp_chksum.h; checked again on
//     read as restore_state does, fms_io.F90:3737-3776).
// Files: the tracers by T_prog(n)%restart_file (ocean_tracer.F90:1670-1686,
// :2658-2681), ocean_barotropic.res.nc (ocean_barotropic.F90:5240-5294,
// two-level fields) and ocean_psom_moments.res.nc (psom_init,
// ocean_tracer_advect.F90:1795-1843).
#include <errno.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "internal.h"
#include "ncfile.h"

using namespace mom5;

namespace {

struct Field {
  std::string name;
  int id, n, level;
};

struct FileSpec {
  std::string file;
  bool three_d;
  std::vector<Field> fields;
};

const char* kPsomSuffix[10] = {"s0", "sx", "sxx", "sy", "syy", "sz", "szz", "sxy", "sxz", "syz"};

bool is_psom(const mom5gpu_domain* d, int n) { return d->scheme[n - 1].horz == MOM5GPU_ADVECT_PSOM; }

// the files and fields this domain holds at time level `level`
std::vector<FileSpec> plan(mom5gpu_domain* d, int level, bool for_read) {
  std::vector<FileSpec> out;
  std::map<std::string, size_t> byfile;
  int ntr = d->dims.num_prog_tracers;
  for (int n = 1; n <= ntr; ++n) {
    const std::string& f = d->tracer_file[n - 1];
    if (!byfile.count(f)) {
      byfile[f] = out.size();
      out.push_back({f, true, {}});
    }
    out[byfile[f]].fields.push_back({d->tracer_name[n - 1], MOM5GPU_TRACER, n, level});
  }
  if (for_read || fptr_if_set(d, MOM5GPU_ETA_T, 0, level)) {
    FileSpec b{"ocean_barotropic.res.nc", false, {}};
    b.fields = {{"eta_t", MOM5GPU_ETA_T, 0, level},       {"conv_rho_ud_t", MOM5GPU_CONV_RHO_UD_T, 0, level},
                {"eta_t_bar", MOM5GPU_ETA_T_BAR, 0, level}, {"eta_u", MOM5GPU_ETA_U, 0, level},
                {"patm_t", MOM5GPU_PATM, 0, 0},             {"udrho", MOM5GPU_UDRHO_U, 0, level},
                {"vdrho", MOM5GPU_UDRHO_V, 0, level},        {"forcing_u_bt", MOM5GPU_FORCING_BT_U, 0, 0},
                {"forcing_v_bt", MOM5GPU_FORCING_BT_V, 0, 0}};
    out.push_back(b);
  }
  FileSpec p{"ocean_psom_moments.res.nc", true, {}};
  for (int n = 1; n <= ntr; ++n)
    if (is_psom(d, n))
      for (int q = 0; q < 10; ++q)
        p.fields.push_back({d->tracer_name[n - 1] + "_prather_" + kPsomSuffix[q], MOM5GPU_PSOM_S0 + q, n, 0});
  if (!p.fields.empty()) out.push_back(p);
  return out;
}

std::string z16(uint64_t v) {
  char buf[17];
  snprintf(buf, sizeof(buf), "%16llX", (unsigned long long)v);
  return buf;
}

std::string path_join(const char* dir, const std::string& f) {
  std::string p = dir ? dir : ".";
  if (!p.empty() && p.back() != '/') p += '/';
  return p + f;
}

nc::Var axis_var(const std::string& name, int dim, const char* units, const char* cart) {
  nc::Var v;
  v.name = name;
  v.dimids = {dim};
  v.type = nc::NC_DOUBLE;
  v.atts = {nc::Attr::make_text("long_name", name == "Time" ? "Time" : name), nc::Attr::make_text("units", units),
            nc::Attr::make_text("cartesian_axis", cart)};
  return v;
}

// compute domain of a data-domain field, x fastest, then y, then z
void compute_domain(const Geo& g, const std::vector<double>& h, int nlev, std::vector<double>& c) {
  c.resize((size_t)g.ni * g.nj * nlev);
  size_t q = 0;
  for (int k = 0; k < nlev; ++k)
    for (int j = 1; j <= g.nj; ++j) {
      const double* row = h.data() + ((size_t)k * g.nyd + j) * g.nxd + 1;
      memcpy(c.data() + q, row, sizeof(double) * g.ni);
      q += g.ni;
    }
}

// data-domain field from compute values: halos hold the periodic images
// (corners when both directions are periodic), else 0
void data_domain(const Geo& g, const std::vector<double>& c, int nlev, std::vector<double>& h) {
  h.assign((size_t)g.nxd * g.nyd * nlev, 0.0);
  auto at = [&](int i, int j, int k) -> double& { return h[((size_t)k * g.nyd + j) * g.nxd + i]; };
  size_t q = 0;
  for (int k = 0; k < nlev; ++k)
    for (int j = 1; j <= g.nj; ++j)
      for (int i = 1; i <= g.ni; ++i) at(i, j, k) = c[q++];
  for (int k = 0; k < nlev; ++k) {
    if (g.cx)
      for (int j = 1; j <= g.nj; ++j) {
        at(0, j, k) = at(g.ni, j, k);
        at(g.ni + 1, j, k) = at(1, j, k);
      }
    if (g.cy)
      for (int i = 1; i <= g.ni; ++i) {
        at(i, 0, k) = at(i, g.nj, k);
        at(i, g.nj + 1, k) = at(i, 1, k);
      }
    if (g.cx && g.cy) {
      at(0, 0, k) = at(g.ni, g.nj, k);
      at(g.ni + 1, 0, k) = at(1, g.nj, k);
      at(0, g.nj + 1, k) = at(g.ni, 1, k);
      at(g.ni + 1, g.nj + 1, k) = at(1, 1, k);
    }
  }
}

uint64_t chksum(const std::vector<double>& c) {
  uint64_t s = 0;
  for (double v : c) {
    uint64_t u;
    memcpy(&u, &v, 8);
    s += u;  // two's-complement sum, wrapping as integer(8) does
  }
  return s;
}

int write_file(mom5gpu_domain* d, const char* dir, const FileSpec& fs) {
  const Geo& g = d->geo;
  int nk = fs.three_d ? g.nk : 1;
  nc::File f;
  f.version = 2;
  f.numrecs = 1;
  f.dims = {{"xaxis_1", (uint64_t)g.ni}, {"yaxis_1", (uint64_t)g.nj}};
  if (fs.three_d) f.dims.push_back({"zaxis_1", (uint64_t)g.nk});
  int tdim = (int)f.dims.size();
  f.dims.push_back({"Time", 0});
  f.gatts = {nc::Attr::make_text("filename", fs.file)};
  f.vars.push_back(axis_var("xaxis_1", 0, "none", "X"));
  f.vars.push_back(axis_var("yaxis_1", 1, "none", "Y"));
  if (fs.three_d) f.vars.push_back(axis_var("zaxis_1", 2, "none", "Z"));
  f.vars.push_back(axis_var("Time", tdim, "time level", "T"));
  size_t first_field = f.vars.size();
  for (const Field& fl : fs.fields) {
    nc::Var v;
    v.name = fl.name;
    v.dimids = fs.three_d ? std::vector<int>{tdim, 2, 1, 0} : std::vector<int>{tdim, 1, 0};
    v.type = nc::NC_DOUBLE;
    v.atts = {nc::Attr::make_text("long_name", fl.name), nc::Attr::make_text("units", "none"),
              nc::Attr::make_text("checksum", z16(0))};
    f.vars.push_back(v);
  }
  nc::layout(f);
  std::string path = path_join(dir, fs.file);
  FILE* fp = fopen(path.c_str(), "wb");
  if (!fp) return fail(d, MOM5GPU_EINVAL, "write_restart: cannot create %s: %s", path.c_str(), strerror(errno));
  std::vector<uint8_t> hdr = nc::encode_header(f), bytes;
  bool ok = fwrite(hdr.data(), 1, hdr.size(), fp) == hdr.size();
  auto put = [&](const std::vector<double>& vals, uint64_t vsize) {
    bytes.assign(vsize, 0);
    for (size_t q = 0; q < vals.size(); ++q) nc::be_double(vals[q], bytes.data() + 8 * q);
    ok = ok && fwrite(bytes.data(), 1, bytes.size(), fp) == bytes.size();
  };
  // axis values 1..n, then the record: Time = 1, the fields
  for (size_t v = 0; v < first_field; ++v) {
    const nc::Var& av = f.vars[v];
    std::vector<double> vals(av.name == "Time" ? 1 : f.dims[av.dimids[0]].len);
    for (size_t q = 0; q < vals.size(); ++q) vals[q] = (double)(q + 1);
    put(vals, av.vsize);
  }
  std::vector<double> h, c;
  int rc = MOM5GPU_OK;
  for (size_t q = 0; q < fs.fields.size() && ok; ++q) {
    const Field& fl = fs.fields[q];
    h.resize(mom5gpu_field_count(d, fl.id));
    if (!fptr_if_set(d, fl.id, fl.n, fl.level)) {
      std::fill(h.begin(), h.end(), 0.0);  // never set: the zero it would hold
    } else if ((rc = mom5gpu_get_field(d, fl.id, fl.n, fl.level, h.data(), 0))) {
      break;
    }
    compute_domain(g, h, nk, c);
    nc::Var& v = f.vars[first_field + q];
    v.atts[2] = nc::Attr::make_text("checksum", z16(chksum(c)));
    put(c, v.vsize);
  }
  if (rc == MOM5GPU_OK && ok) {
    std::vector<uint8_t> hdr2 = nc::encode_header(f);  // same size: the checksums are 16 characters
    ok = hdr2.size() == hdr.size() && fseeko(fp, 0, SEEK_SET) == 0 &&
         fwrite(hdr2.data(), 1, hdr2.size(), fp) == hdr2.size();
  }
  if (fclose(fp) != 0) ok = false;
  if (rc) return rc;
  if (!ok) return fail(d, MOM5GPU_EINVAL, "write_restart: writing %s failed", path.c_str());
  return MOM5GPU_OK;
}

bool parse_checksum(const std::string& text, size_t rec, uint64_t& out) {
  std::vector<std::string> parts;
  std::string cur;
  for (char ch : text) {
    if (ch == ',') {
      parts.push_back(cur);
      cur.clear();
    } else if (ch != ' ') {
      cur += ch;
    }
  }
  parts.push_back(cur);
  const std::string& s = parts[rec < parts.size() ? rec : 0];
  if (s.empty() || s.size() > 16) return false;
  uint64_t v = 0;
  for (char ch : s) {
    int x = (ch >= '0' && ch <= '9') ? ch - '0' : (ch >= 'A' && ch <= 'F') ? ch - 'A' + 10
                                                : (ch >= 'a' && ch <= 'f') ? ch - 'a' + 10 : -1;
    if (x < 0) return false;
    v = (v << 4) | (uint64_t)x;
  }
  out = v;
  return true;
}

// required: a missing variable is an error (else the field is left as it is)
int read_file(mom5gpu_domain* d, const char* dir, const FileSpec& fs, bool file_required,
              const std::vector<bool>& required) {
  const Geo& g = d->geo;
  int nk = fs.three_d ? g.nk : 1;
  std::string path = path_join(dir, fs.file);
  FILE* fp = fopen(path.c_str(), "rb");
  if (!fp) {
    if (file_required) return fail(d, MOM5GPU_ESTATE, "read_restart: %s: %s", path.c_str(), strerror(errno));
    return MOM5GPU_OK;
  }
  nc::File f;
  if (!nc::read_header(fp, f)) {
    fclose(fp);
    return fail(d, MOM5GPU_EINVAL, "read_restart: %s is not a netCDF classic file", path.c_str());
  }
  int rc = MOM5GPU_OK;
  std::vector<uint8_t> bytes;
  std::vector<double> c, h;
  for (size_t q = 0; q < fs.fields.size() && rc == MOM5GPU_OK; ++q) {
    const Field& fl = fs.fields[q];
    int vi = f.find(fl.name);
    if (vi < 0) {
      if (required[q]) rc = fail(d, MOM5GPU_ESTATE, "read_restart: %s has no field %s", path.c_str(), fl.name.c_str());
      continue;
    }
    const nc::Var& v = f.vars[vi];
    // spatial dimensions, x fastest: (ni, nj[, nk])
    std::vector<uint64_t> sp;
    for (int id : v.dimids)
      if (f.dims[id].len) sp.push_back(f.dims[id].len);
    bool shape_ok = sp.size() == (size_t)(fs.three_d ? 3 : 2) && sp.back() == (uint64_t)g.ni &&
                    sp[sp.size() - 2] == (uint64_t)g.nj && (!fs.three_d || sp[0] == (uint64_t)g.nk);
    if (!shape_ok || (v.type != nc::NC_DOUBLE && v.type != nc::NC_FLOAT)) {
      rc = fail(d, MOM5GPU_EINVAL, "read_restart: %s:%s does not match the domain (%dx%dx%d doubles)", path.c_str(),
                fl.name.c_str(), g.ni, g.nj, nk);
      break;
    }
    uint64_t rec = v.record ? (f.numrecs ? f.numrecs - 1 : 0) : 0;
    if (v.record && f.numrecs == 0) {
      rc = fail(d, MOM5GPU_EINVAL, "read_restart: %s:%s has no record", path.c_str(), fl.name.c_str());
      break;
    }
    uint64_t cnt = (uint64_t)g.ni * g.nj * nk, ts = nc::type_size(v.type);
    bytes.resize(cnt * ts);
    if (fseeko(fp, (off_t)(v.begin + rec * f.recsize), SEEK_SET) != 0 ||
        fread(bytes.data(), 1, bytes.size(), fp) != bytes.size()) {
      rc = fail(d, MOM5GPU_EINVAL, "read_restart: %s:%s is truncated", path.c_str(), fl.name.c_str());
      break;
    }
    c.resize(cnt);
    for (uint64_t e = 0; e < cnt; ++e) {
      if (ts == 8) {
        c[e] = nc::double_be(bytes.data() + 8 * e);
      } else {
        uint32_t u = nc::u32_be(bytes.data() + 4 * e);
        float x;
        memcpy(&x, &u, 4);
        c[e] = x;
      }
    }
    const nc::Attr* ck = v.att("checksum");
    uint64_t want;
    if (ck && ts == 8 && parse_checksum(ck->text(), rec, want) && want != chksum(c)) {
      rc = fail(d, MOM5GPU_ENUMERIC, "read_restart: checksum of input field %s (%s) does not match %s stored in %s",
                fl.name.c_str(), z16(chksum(c)).c_str(), z16(want).c_str(), path.c_str());
      break;
    }
    data_domain(g, c, nk, h);
    rc = mom5gpu_set_field(d, fl.id, fl.n, fl.level, h.data(), 0);
  }
  fclose(fp);
  return rc;
}

}  // namespace

extern "C" {

int mom5gpu_set_tracer_name(mom5gpu_domain* d, int n, const char* name, const char* restart_file) {
  if (!d) return MOM5GPU_EINVAL;
  if (n < 1 || n > d->dims.num_prog_tracers) return fail(d, MOM5GPU_EINVAL, "set_tracer_name: tracer %d", n);
  if (!name || !*name || strlen(name) > 120) return fail(d, MOM5GPU_EINVAL, "set_tracer_name: name must be 1..120 characters");
  d->tracer_name[n - 1] = name;
  if (restart_file && *restart_file) {
    if (strchr(restart_file, '/')) return fail(d, MOM5GPU_EINVAL, "set_tracer_name: restart_file is a file name, not a path");
    d->tracer_file[n - 1] = restart_file;
  }
  return MOM5GPU_OK;
}

int mom5gpu_write_restart(mom5gpu_domain* d, const char* dir, int level) {
  if (!d) return MOM5GPU_EINVAL;
  if (level < 1 || level > 3) return fail(d, MOM5GPU_EINVAL, "write_restart: time level %d", level);
  struct stat st;
  if (dir && *dir && (stat(dir, &st) != 0 || !S_ISDIR(st.st_mode)))
    return fail(d, MOM5GPU_EINVAL, "write_restart: %s is not a directory", dir);
  for (const FileSpec& fs : plan(d, level, false)) {
    int rc = write_file(d, dir, fs);
    if (rc) return rc;
  }
  return MOM5GPU_OK;
}

int mom5gpu_read_restart(mom5gpu_domain* d, const char* dir, int level) {
  if (!d) return MOM5GPU_EINVAL;
  if (level < 1 || level > 3) return fail(d, MOM5GPU_EINVAL, "read_restart: time level %d", level);
  for (const FileSpec& fs : plan(d, level, true)) {
    bool baro = fs.file == "ocean_barotropic.res.nc", psom = fs.file == "ocean_psom_moments.res.nc";
    std::vector<bool> req(fs.fields.size(), !psom);
    if (baro)  // patm_t and the forcing are optional here; eta_t .. vdrho mandatory as in read_barotropic
      for (size_t q = 0; q < fs.fields.size(); ++q)
        req[q] = fs.fields[q].id != MOM5GPU_PATM && fs.fields[q].id != MOM5GPU_FORCING_BT_U &&
                 fs.fields[q].id != MOM5GPU_FORCING_BT_V;
    // tracer files are required; the barotropic file only if the domain steps the barotropic mode;
    // PSOM moments start from zero without a file (psom_init)
    bool file_required = !psom && (!baro || d->baro_ready);
    int rc = read_file(d, dir, fs, file_required, req);
    if (rc) return rc;
  }
  return MOM5GPU_OK;
}

}  // extern "C"
