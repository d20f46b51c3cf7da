// Host-side readers for OAK's configuration and data files: the init file (key = value lines,
// initfile.F90), NetCDF classic-format variables (the "file.nc#variable" specifications of
// ufileformat.F90) and GHER binary files (names without '#'). Used by the oak_init /
// oak_assim driver.
#pragma once
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

namespace oakg {
namespace io {

// OAK init file (initfile.F90): one "key = value" per line; '#' or '!' starts a comment
// outside strings; values are numbers (Fortran exponents d/D accepted), 'strings' ('' escapes
// a quote) or one-line lists [a, b, ...] of either. The first definition of a key counts.
class InitFile {
 public:
  bool load(const std::string& fname, std::string& err);
  bool has(const std::string& key) const { return kv_.count(key) != 0; }
  bool str(const std::string& key, std::string& out, std::string& err) const;
  bool num(const std::string& key, double& out, std::string& err) const;
  bool strs(const std::string& key, std::vector<std::string>& out, std::string& err) const;
  bool nums(const std::string& key, std::vector<double>& out, std::string& err) const;
  // typed getters with a default when the key is absent
  std::string str_or(const std::string& key, const std::string& dflt) const;
  double num_or(const std::string& key, double dflt) const;

 private:
  std::map<std::string, std::vector<std::string>> kv_;  // raw items (strings unquoted)
  std::map<std::string, std::vector<char>> quoted_;     // per item: was a quoted string
  std::map<std::string, bool> is_list_;
};

// One variable of a data file, as ufileformat's uload returns it: values in Fortran order
// (first dimension fastest), the shape in Fortran order, the missing value (the variable's
// missing_value or _FillValue attribute, else -9999), scale_factor / add_offset applied to the
// other values, and the "shape" attribute's compact regular form expanded.
struct Array {
  std::vector<double> v;
  std::vector<int64_t> shape;
  double valex = -9999.0;
};

// The values of a file whose shape is smaller than the variable's shape t, replicated along the
// missing dimensions (ureadfull_srepmat, ufileformat.F90:980-1035); false when they do not fit.
bool replicate(const Array& a, const std::vector<int64_t>& t, std::vector<double>& out,
               std::string& err);

// A file name from a Fortran format of quoted text and Iw / Iw.m edits applied to k, e.g.
// ("Ens",I3.3,"/model.nc#var1") -> Ens007/model.nc#var1; false for other edits.
bool fortran_format(const std::string& fmt, int k, std::string& out, std::string& err);

// spec "file.nc#var" (NetCDF classic, 64-bit-offset or CDF-5 format) or "file" (GHER binary);
// path prefixed
bool read_array(const std::string& path, const std::string& spec, Array& out, std::string& err);

}  // namespace io
}  // namespace oakg
