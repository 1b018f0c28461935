// cdf_io.h -- the column files of the reference's Cl_run_cdf / Cl_run_cdl
// drivers: netCDF classic binary files (CDF-1 and CDF-2, as written by the
// netCDF library) and their CDL text form.  Every variable is held as
// float64 values in the file's order (the last dimension varies fastest).
#pragma once

#include <cstddef>
#include <string>
#include <utility>
#include <vector>

namespace socgpu {

struct NcVar {
  std::string name;
  std::vector<int> dims;                                     // indices into NcFile::dims
  int type = 5;                                              // nc_type: 4 int, 5 float, 6 double
  std::vector<std::pair<std::string, std::string>> text_atts;
  std::vector<double> data;
};

struct NcFile {
  std::string name;                                          // CDL "netcdf <name>"
  std::vector<std::pair<std::string, size_t>> dims;
  std::vector<NcVar> vars;

  int dim_index(const std::string &n) const;
  const NcVar *var(const std::string &n) const;
  size_t dim_len(const std::string &n) const;                // 0 if absent
};

// Read a file in either form (detected from its first bytes).
bool read_nc(const std::string &path, NcFile &f, std::string &err);
bool read_cdl(const std::string &path, NcFile &f, std::string &err);
bool read_cdf(const std::string &path, NcFile &f, std::string &err);
bool write_cdl(const std::string &path, const NcFile &f, std::string &err);
bool write_cdf(const std::string &path, const NcFile &f, std::string &err);

}  // namespace socgpu
