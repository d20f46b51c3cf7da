// Init-file parser and NetCDF classic-format reader (see oak_io.h). The NetCDF reader follows
// the published classic / 64-bit-offset / CDF-5 format specification (Unidata, "NetCDF
// Classic Format Specification"): a big-endian header (magic, record count, dimension,
// global-attribute and variable lists) followed by the variables' data, record variables
// interleaved record by record.
#include "oak_io.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <memory>

namespace oakg {
namespace io {

namespace {

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n'; }

bool parse_number(const std::string& tok, double& out) {
  std::string t = tok;
  for (char& ch : t)
    if (ch == 'd' || ch == 'D') ch = 'e';
  const char* b = t.c_str();
  char* e = nullptr;
  out = strtod(b, &e);
  if (e == b) return false;
  while (*e && is_space(*e)) e++;
  return *e == '\0';
}

}  // namespace

bool InitFile::load(const std::string& fname, std::string& err) {
  FILE* f = fopen(fname.c_str(), "r");
  if (!f) {
    err = "cannot read init file '" + fname + "'";
    return false;
  }
  kv_.clear();
  quoted_.clear();
  is_list_.clear();
  char buf[1 << 14];
  int lineno = 0;
  while (fgets(buf, sizeof buf, f)) {
    lineno++;
    std::string line(buf);
    size_t i = 0;
    auto skip = [&]() {
      while (i < line.size() && is_space(line[i])) i++;
    };
    skip();
    if (i >= line.size() || line[i] == '#' || line[i] == '!') continue;
    size_t k0 = i;
    while (i < line.size() && !is_space(line[i]) && line[i] != '=') i++;
    std::string key = line.substr(k0, i - k0);
    skip();
    if (i >= line.size() || line[i] != '=') {
      fclose(f);
      err = fname + ":" + std::to_string(lineno) + ": expected 'key = value'";
      return false;
    }
    i++;
    std::vector<std::string> items;
    std::vector<char> quoted;
    bool list = false, ok = true;
    auto read_item = [&](bool in_list) -> bool {
      skip();
      if (i >= line.size()) return false;
      if (line[i] == '\'') {
        std::string s;
        i++;
        for (;;) {
          if (i >= line.size()) return false;  // unterminated
          if (line[i] == '\'') {
            if (i + 1 < line.size() && line[i + 1] == '\'') {
              s += '\'';
              i += 2;
              continue;
            }
            i++;
            break;
          }
          s += line[i++];
        }
        items.push_back(s);
        quoted.push_back(1);
        return true;
      }
      size_t t0 = i;
      while (i < line.size() && !is_space(line[i]) && line[i] != ',' &&
             !(in_list && line[i] == ']') && line[i] != '#' && line[i] != '!')
        i++;
      if (i == t0) return false;
      items.push_back(line.substr(t0, i - t0));
      quoted.push_back(0);
      return true;
    };
    skip();
    if (i < line.size() && line[i] == '[') {
      list = true;
      i++;
      skip();
      if (i < line.size() && line[i] == ']') {
        i++;
      } else {
        for (;;) {
          if (!read_item(true)) {
            ok = false;
            break;
          }
          skip();
          if (i < line.size() && line[i] == ',') {
            i++;
            continue;
          }
          if (i < line.size() && line[i] == ']') {
            i++;
            break;
          }
          ok = false;
          break;
        }
      }
    } else {
      ok = read_item(false);
    }
    if (ok) {
      skip();
      ok = i >= line.size() || line[i] == '#' || line[i] == '!';
    }
    if (!ok) {
      fclose(f);
      err = fname + ":" + std::to_string(lineno) + ": cannot parse the value of '" + key + "'";
      return false;
    }
    if (!kv_.count(key)) {
      kv_[key] = items;
      quoted_[key] = quoted;
      is_list_[key] = list;
    }
  }
  fclose(f);
  return true;
}

bool InitFile::str(const std::string& key, std::string& out, std::string& err) const {
  auto it = kv_.find(key);
  if (it == kv_.end() || it->second.size() != 1) {
    err = "init file: '" + key + "' must be one value";
    return false;
  }
  out = it->second[0];
  return true;
}

bool InitFile::num(const std::string& key, double& out, std::string& err) const {
  std::string s;
  if (!str(key, s, err)) return false;
  if (quoted_.at(key)[0] || !parse_number(s, out)) {
    err = "init file: '" + key + "' must be a number";
    return false;
  }
  return true;
}

bool InitFile::strs(const std::string& key, std::vector<std::string>& out,
                    std::string& err) const {
  auto it = kv_.find(key);
  if (it == kv_.end()) {
    err = "init file: '" + key + "' is missing";
    return false;
  }
  out = it->second;
  return true;
}

bool InitFile::nums(const std::string& key, std::vector<double>& out, std::string& err) const {
  auto it = kv_.find(key);
  if (it == kv_.end()) {
    err = "init file: '" + key + "' is missing";
    return false;
  }
  out.clear();
  for (size_t q = 0; q < it->second.size(); q++) {
    double v;
    if (quoted_.at(key)[q] || !parse_number(it->second[q], v)) {
      err = "init file: '" + key + "' must hold numbers";
      return false;
    }
    out.push_back(v);
  }
  return true;
}

std::string InitFile::str_or(const std::string& key, const std::string& dflt) const {
  auto it = kv_.find(key);
  return (it == kv_.end() || it->second.size() != 1) ? dflt : it->second[0];
}

double InitFile::num_or(const std::string& key, double dflt) const {
  std::string e;
  double v;
  return (has(key) && num(key, v, e)) ? v : dflt;
}

// ureadfull_srepmat (ufileformat.F90:980-1035): a file whose shape differs from the
// variable's is replicated along the dimensions it lacks (each file dimension 1 or equal to
// the variable's, after padding with trailing ones; else matched in order by length).
bool replicate(const Array& a, const std::vector<int64_t>& t, std::vector<double>& out,
               std::string& err) {
  int64_t nt = 1;
  for (int64_t x : t) nt *= x;
  if ((int64_t)a.v.size() == nt) {
    out = a.v;
    return true;
  }
  const size_t nd = t.size();
  std::vector<int64_t> map(nd, -1);  // target dim -> file dim (or -1: replicated)
  const std::vector<int64_t>& s = a.shape;
  bool ok = s.size() <= nd;
  if (ok) {
    for (size_t k = 0; k < s.size() && ok; k++) ok = s[k] == t[k] || s[k] == 1;
    if (ok)
      for (size_t k = 0; k < s.size(); k++) map[k] = s[k] == 1 ? -1 : (int64_t)k;
  }
  if (!ok) {
    std::fill(map.begin(), map.end(), -1);
    size_t k = 0;
    ok = true;
    for (size_t q = 0; q < s.size() && ok; q++) {
      if (s[q] == 1) continue;
      while (k < nd && t[k] != s[q]) k++;
      ok = k < nd;
      if (ok) map[k++] = (int64_t)q;
    }
  }
  if (!ok) {
    err = "file shape does not fit the variable's shape";
    return false;
  }
  std::vector<int64_t> fstride(s.size(), 1);
  for (size_t q = 1; q < s.size(); q++) fstride[q] = fstride[q - 1] * s[q - 1];
  out.assign((size_t)nt, 0.0);
  std::vector<int64_t> idx(nd, 0);
  for (int64_t e = 0; e < nt; e++) {
    int64_t f = 0;
    for (size_t k = 0; k < nd; k++)
      if (map[k] >= 0) f += idx[k] * fstride[map[k]];
    out[e] = a.v[f];
    for (size_t k = 0; k < nd; k++) {
      if (++idx[k] < t[k]) break;
      idx[k] = 0;
    }
  }
  return true;
}

// Fortran edit descriptors of the ensemble file formats, e.g. ("Ens",I3.3,"/m.nc#v"): quoted
// literals and Iw / Iw.m integers (loadVectorSpace, assimilation.F90:1214-1220)
bool fortran_format(const std::string& fmt, int k, std::string& out, std::string& err) {
  std::string f = fmt;
  while (!f.empty() && f.front() == ' ') f.erase(f.begin());
  while (!f.empty() && f.back() == ' ') f.pop_back();
  out.clear();
  if (f.size() < 2 || f.front() != '(' || f.back() != ')') {
    err = "format '" + fmt + "': expected (...)";
    return false;
  }
  f = f.substr(1, f.size() - 2);
  size_t i = 0;
  while (i < f.size()) {
    const char c = f[i];
    if (c == ' ' || c == ',') {
      i++;
    } else if (c == '"' || c == '\'') {
      const size_t j = f.find(c, i + 1);
      if (j == std::string::npos) {
        err = "format '" + fmt + "': unterminated text";
        return false;
      }
      out += f.substr(i + 1, j - i - 1);
      i = j + 1;
    } else if (c == 'I' || c == 'i') {
      size_t j = i + 1;
      int w = 0, m = 0;
      while (j < f.size() && isdigit((unsigned char)f[j])) w = w * 10 + (f[j++] - '0');
      if (j < f.size() && f[j] == '.') {
        j++;
        while (j < f.size() && isdigit((unsigned char)f[j])) m = m * 10 + (f[j++] - '0');
      }
      if (w <= 0) {
        err = "format '" + fmt + "': I needs a width";
        return false;
      }
      std::string d = std::to_string(k);
      while ((int)d.size() < m) d = "0" + d;
      if ((int)d.size() > w) d = std::string(w, '*');
      while ((int)d.size() < w) d = " " + d;
      out += d;
      i = j;
    } else {
      err = "format '" + fmt + "': only quoted text and I edits are supported";
      return false;
    }
  }
  return true;
}

// ------------------------------------------------------------------------------ NetCDF

namespace {

enum : int32_t {
  NC_DIMENSION = 10,
  NC_VARIABLE = 11,
  NC_ATTRIBUTE = 12,
};

int type_size(int t) {
  switch (t) {
    case 1: case 2: case 7: return 1;  // byte, char, ubyte
    case 3: case 8: return 2;          // short, ushort
    case 4: case 5: case 9: return 4;  // int, float, uint
    case 6: case 10: case 11: return 8;  // double, int64, uint64
    default: return 0;
  }
}

uint64_t be(const unsigned char* p, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}

double decode(const unsigned char* p, int t) {
  switch (t) {
    case 1: return (double)(int8_t)p[0];
    case 2: return (double)p[0];
    case 7: return (double)p[0];
    case 3: return (double)(int16_t)(uint16_t)be(p, 2);
    case 8: return (double)(uint16_t)be(p, 2);
    case 4: return (double)(int32_t)(uint32_t)be(p, 4);
    case 9: return (double)(uint32_t)be(p, 4);
    case 10: return (double)(int64_t)be(p, 8);
    case 11: return (double)be(p, 8);
    case 5: {
      uint32_t u = (uint32_t)be(p, 4);
      float f;
      memcpy(&f, &u, 4);
      return (double)f;
    }
    case 6: {
      uint64_t u = be(p, 8);
      double d;
      memcpy(&d, &u, 8);
      return d;
    }
    default: return NAN;
  }
}

struct Reader {
  FILE* f = nullptr;
  int version = 1;
  bool fail = false;
  bool bytes(unsigned char* p, size_t n) {
    if (fail || fread(p, 1, n, f) != n) fail = true;
    return !fail;
  }
  uint64_t u(int n) {
    unsigned char b[8] = {0};
    bytes(b, n);
    return be(b, n);
  }
  uint64_t count() { return u(version == 5 ? 8 : 4); }
  std::string name() {
    const uint64_t n = count();
    if (fail || n > 4096) {
      fail = true;
      return "";
    }
    std::string s(n, '\0');
    bytes(reinterpret_cast<unsigned char*>(&s[0]), n);
    const size_t pad = (4 - n % 4) % 4;
    unsigned char b[4];
    bytes(b, pad);
    return s;
  }
};

struct Att {
  std::string name;
  int type = 0;
  std::vector<double> vals;
};

bool read_atts(Reader& r, std::vector<Att>& atts) {
  const uint64_t tag = r.u(4);
  const uint64_t n = r.count();
  if (r.fail) return false;
  if (tag == 0 && n == 0) return true;
  if (tag != NC_ATTRIBUTE || n > 100000) return false;
  for (uint64_t a = 0; a < n; a++) {
    Att at;
    at.name = r.name();
    at.type = (int)r.u(4);
    const uint64_t ne = r.count();
    const int ts = type_size(at.type);
    if (r.fail || ts == 0 || ne > (1u << 24)) return false;
    const size_t nb = ne * ts, pad = (4 - nb % 4) % 4;
    std::vector<unsigned char> buf(nb + pad);
    if (!r.bytes(buf.data(), nb + pad)) return false;
    if (at.type != 2)
      for (uint64_t q = 0; q < ne; q++) at.vals.push_back(decode(buf.data() + q * ts, at.type));
    atts.push_back(at);
  }
  return true;
}

}  // namespace

// GHER binary file (ufileformat.F90: UREADC, :1072-1160): Fortran unformatted sequential
// records with 4-byte length markers in either byte order (the reference's FORMAT=big_endian
// build writes big-endian): KBLANC = 10 records skipped, the header record (imax, jmax, kmax,
// iprec, nbmots as int32, valex as float32), then the values in records of nbmots words of
// iprec bytes. A negative extent marks the compact form: four values c0, dci, dcj, dck.
bool read_gher(const std::string& file, Array& out, std::string& err) {
  std::unique_ptr<FILE, int (*)(FILE*)> fp(fopen(file.c_str(), "rb"), fclose);
  if (!fp) {
    err = "cannot open '" + file + "'";
    return false;
  }
  std::vector<unsigned char> buf;
  {
    unsigned char chunk[1 << 16];
    size_t got;
    while ((got = fread(chunk, 1, sizeof chunk, fp.get())) > 0) {
      buf.insert(buf.end(), chunk, chunk + got);
      if (buf.size() > ((size_t)1 << 36)) {
        err = "'" + file + "' is too large";
        return false;
      }
    }
  }
  auto marker = [&](size_t off, bool big) -> int64_t {
    if (off + 4 > buf.size()) return -1;
    const unsigned char* p = buf.data() + off;
    return big ? (int64_t)be(p, 4)
               : (int64_t)((uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
                           ((uint32_t)p[3] << 24));
  };
  // records: (payload offset, length); the byte order whose first 11 records are consistent
  // and whose 11th is the 24-byte header
  std::vector<std::pair<size_t, size_t>> recs;
  bool big = false, ok = false;
  for (int order = 0; order < 2 && !ok; order++) {
    big = order == 1;
    recs.clear();
    size_t off = 0;
    ok = true;
    while (off < buf.size()) {
      const int64_t len = marker(off, big);
      if (len < 0 || off + 8 + (size_t)len > buf.size() ||
          marker(off + 4 + (size_t)len, big) != len) {
        ok = false;
        break;
      }
      recs.emplace_back(off + 4, (size_t)len);
      off += 8 + (size_t)len;
    }
    ok = ok && recs.size() >= 12 && recs[10].second == 24;
  }
  if (!ok) {
    err = "'" + file + "' is neither a NetCDF variable (file.nc#var) nor a GHER binary file";
    return false;
  }
  auto i32 = [&](size_t off) {
    const int64_t v = marker(off, big);
    return (int32_t)(uint32_t)v;
  };
  const size_t h = recs[10].first;
  const int32_t imax = i32(h), jmax = i32(h + 4), kmax = i32(h + 8), iprec = i32(h + 12);
  const uint32_t vx = (uint32_t)marker(h + 20, big);
  float valex4;
  memcpy(&valex4, &vx, 4);
  if (iprec != 4 && iprec != 8) {
    err = "'" + file + "': precision " + std::to_string(iprec) + " (expected 4 or 8)";
    return false;
  }
  const bool degen = imax < 0 || jmax < 0 || kmax < 0;
  const int64_t ni = imax < 0 ? -(int64_t)imax : imax, nj = jmax < 0 ? -(int64_t)jmax : jmax,
                nk = kmax < 0 ? -(int64_t)kmax : kmax;
  const int64_t total = ni * nj * nk, want = degen ? 4 : total;
  if (total <= 0 || total > ((int64_t)1 << 34)) {
    err = "'" + file + "': bad extents";
    return false;
  }
  std::vector<double> vals;
  vals.reserve((size_t)want);
  for (size_t r = 11; r < recs.size() && (int64_t)vals.size() < want; r++)
    for (size_t q = 0; q + iprec <= recs[r].second && (int64_t)vals.size() < want; q += iprec) {
      const unsigned char* p = buf.data() + recs[r].first + q;
      unsigned char tmp[8];
      for (int b = 0; b < iprec; b++) tmp[b] = big ? p[b] : p[iprec - 1 - b];  // to big-endian
      vals.push_back(decode(tmp, iprec == 4 ? 5 : 6));
    }
  if ((int64_t)vals.size() < want) {
    err = "'" + file + "': truncated data";
    return false;
  }
  // the extents as uread_prim reads them: trailing unit extents dropped
  out.shape = {ni};
  if (nk != 1) out.shape = {ni, nj, nk};
  else if (nj != 1) out.shape = {ni, nj};
  out.valex = (double)valex4;
  if (degen) {
    // uexplo (:2300-2337), 1-based indices
    const size_t nd = out.shape.size();
    out.v.assign((size_t)total, 0.0);
    for (int64_t e = 0; e < total; e++) {
      int64_t rem = e;
      double x = vals[0];
      for (size_t k = 0; k < nd; k++) {
        const int64_t ik = rem % out.shape[k];
        rem /= out.shape[k];
        x += vals[k + 1] * (double)(ik + 1);
      }
      out.v[e] = x;
    }
  } else {
    out.v.swap(vals);
  }
  return true;
}

bool read_array(const std::string& path, const std::string& spec, Array& out, std::string& err) {
  const size_t hash = spec.rfind('#');
  if (hash == std::string::npos) return read_gher(path + spec, out, err);
  const std::string file = path + spec.substr(0, hash), var = spec.substr(hash + 1);
  std::unique_ptr<FILE, int (*)(FILE*)> fp(fopen(file.c_str(), "rb"), fclose);
  if (!fp) {
    err = "cannot open '" + file + "'";
    return false;
  }
  Reader r;
  r.f = fp.get();
  unsigned char magic[4];
  if (!r.bytes(magic, 4) || memcmp(magic, "CDF", 3) != 0 ||
      (magic[3] != 1 && magic[3] != 2 && magic[3] != 5)) {
    err = "'" + file + "' is not a NetCDF classic-format file (NetCDF-4/HDF5 is not read)";
    return false;
  }
  r.version = magic[3];
  const uint64_t numrecs = r.count();
  // dimensions
  std::vector<std::string> dname;
  std::vector<uint64_t> dlen;
  int recdim = -1;
  {
    const uint64_t tag = r.u(4), n = r.count();
    if (!(tag == 0 && n == 0)) {
      if (tag != NC_DIMENSION || n > 100000) r.fail = true;
      for (uint64_t d = 0; d < n && !r.fail; d++) {
        dname.push_back(r.name());
        dlen.push_back(r.count());
        if (dlen.back() == 0) recdim = (int)d;
      }
    }
  }
  std::vector<Att> gatts;
  if (r.fail || !read_atts(r, gatts)) {
    err = "'" + file + "': damaged header";
    return false;
  }
  struct Var {
    std::string name;
    std::vector<uint64_t> dims;
    std::vector<Att> atts;
    int type = 0;
    uint64_t vsize = 0, begin = 0;
  };
  std::vector<Var> vars;
  {
    const uint64_t tag = r.u(4), n = r.count();
    if (!(tag == 0 && n == 0)) {
      if (tag != NC_VARIABLE || n > 100000) r.fail = true;
      for (uint64_t q = 0; q < n && !r.fail; q++) {
        Var v;
        v.name = r.name();
        const uint64_t nd = r.count();
        if (nd > 64) r.fail = true;
        for (uint64_t d = 0; d < nd && !r.fail; d++) v.dims.push_back(r.count());
        if (!r.fail && !read_atts(r, v.atts)) r.fail = true;
        v.type = (int)r.u(4);
        v.vsize = r.count();
        v.begin = r.u(r.version == 1 ? 4 : 8);
        vars.push_back(v);
      }
    }
  }
  if (r.fail) {
    err = "'" + file + "': damaged header";
    return false;
  }
  const Var* vp = nullptr;
  uint64_t recsize = 0;
  int nrecvars = 0;
  for (const Var& v : vars) {
    const bool rec = !v.dims.empty() && (int)v.dims[0] == recdim;
    if (rec) {
      recsize += v.vsize;
      nrecvars++;
    }
    if (v.name == var) vp = &v;
  }
  if (!vp) {
    err = "'" + file + "' has no variable '" + var + "'";
    return false;
  }
  const int ts = type_size(vp->type);
  if (ts == 0) {
    err = "'" + file + "#" + var + "': unsupported type";
    return false;
  }
  const bool rec = !vp->dims.empty() && (int)vp->dims[0] == recdim;
  std::vector<uint64_t> cshape;  // C order
  for (uint64_t d : vp->dims) {
    if (d >= dlen.size()) {
      err = "'" + file + "': bad dimension id";
      return false;
    }
    cshape.push_back((int)d == recdim ? numrecs : dlen[d]);
  }
  uint64_t per_rec = 1;
  for (size_t d = rec ? 1 : 0; d < cshape.size(); d++) per_rec *= cshape[d];
  const uint64_t nrec = rec ? numrecs : 1;
  if (rec && nrecvars == 1) recsize = per_rec * ts;  // a lone record variable is not padded
  // attributes of the variable
  double scale = 1.0, offset = 0.0;
  out.valex = -9999.0;
  std::vector<double> compact_shape;
  for (const Att& a : vp->atts) {
    if (a.vals.empty()) continue;
    if (a.name == "missing_value" || a.name == "_FillValue") out.valex = a.vals[0];
    else if (a.name == "scale_factor") scale = a.vals[0];
    else if (a.name == "add_offset") offset = a.vals[0];
    else if (a.name == "shape") compact_shape = a.vals;
  }
  const uint64_t total = per_rec * nrec;
  if (total > ((uint64_t)1 << 34)) {
    err = "'" + file + "#" + var + "' is too large";
    return false;
  }
  std::vector<unsigned char> raw((size_t)(total * ts));
  for (uint64_t q = 0; q < nrec; q++) {
    const uint64_t off = vp->begin + (rec ? q * recsize : 0);
    if (fseek(fp.get(), (long)off, SEEK_SET) != 0 ||
        fread(raw.data() + q * per_rec * ts, 1, per_rec * ts, fp.get()) != per_rec * ts) {
      err = "'" + file + "#" + var + "': truncated data";
      return false;
    }
  }
  std::vector<double> vals((size_t)total);
  for (uint64_t q = 0; q < total; q++) vals[q] = decode(raw.data() + q * ts, vp->type);
  if (!compact_shape.empty()) {
    // the compact regular form (uexplo, ufileformat.F90:2300-2337): with 1-based indices,
    // x(i_1..i_n) = c(0) + sum_k c(k) i_k; the shape in the attribute (Fortran order)
    const size_t nd = compact_shape.size();
    if (vals.size() < nd + 1) {
      err = "'" + file + "#" + var + "': compact form needs " + std::to_string(nd + 1) + " values";
      return false;
    }
    out.shape.clear();
    uint64_t cnt = 1;
    for (double s : compact_shape) {
      out.shape.push_back((int64_t)s);
      cnt *= (uint64_t)s;
    }
    out.v.assign((size_t)cnt, 0.0);
    for (uint64_t e = 0; e < cnt; e++) {
      uint64_t rem = e;
      double x = vals[0];
      for (size_t k = 0; k < nd; k++) {
        const uint64_t ik = rem % (uint64_t)out.shape[k];
        rem /= (uint64_t)out.shape[k];
        x += vals[k + 1] * (double)(ik + 1);
      }
      out.v[e] = x;
    }
    return true;
  }
  out.shape.assign(cshape.rbegin(), cshape.rend());
  if (out.shape.empty()) out.shape.push_back(1);
  if (scale != 1.0 || offset != 0.0)
    for (double& x : vals)
      if (x != out.valex) x = x * scale + offset;
  out.v.swap(vals);
  return true;
}

}  // namespace io
}  // namespace oakg
