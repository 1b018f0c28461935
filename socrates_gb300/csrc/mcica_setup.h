// mcica_setup.h -- the McICA data file and set_cld_mcica, shared by the
// column driver (socgpu_run) and runes.  Host code over the public C-ABI
// (socgpu_spectrum_k_terms, socgpu_cloud_gen).
#pragma once

#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/socgpu.h"

namespace socgpu {

// The McICA data file (read_mcica_data.F90): subcolumn counts, the long-wave
// reorderings, the per-(band, k-term) subcolumns of optimal sampling and
// the generator's condensate table xcw (n1, n2).
struct McicaData {
  int gen = 0, req_single = 0, req_optimal = 0, ipph = 0, n1 = 0, n2 = 0;
  std::vector<int> reorder_single, reorder_optimal;
  std::map<std::pair<int, int>, int> sw_subcol_k, lw_subcol_k;
  std::vector<double> xcw;
};

bool read_mcica_data(const std::string &path, McicaData &m, std::string &err);

// What set_cld_mcica leaves in cld (socrates_set_cld_mcica.F90:82-228).
struct McicaState {
  int gen = 1, n_subcol_req = 1, nd_k = 1;
  std::vector<int> subcol_k, first_subcol_k, subcol_reorder, n_subcol_cld;
  std::vector<double> c_sub, frac_cloudy;
  void attach(socgpu_cld &cld);
};

// Sampling tables for bands first..last of the spectrum, the generator's
// subcolumns (np columns, layers id_cloud_top..nl) with the condensate
// variability cond_rsd and the cloud fractions w_cloud (both (np,
// id_cloud_top..nl)), the layer pressures p (np, nl), the decorrelation
// pressure dp_corr (Pa; half of it for the condensate) and per-column
// seeds, then frac_cloudy.
// c_cloud and c_ratio (convective fraction and its share of the condensate,
// (np, id_cloud_top..nl)) may be NULL (zero).
int set_cld_mcica(socgpu_spectrum_handle h, const McicaData &md, int isolir, int sampling, int ioverlap, int first,
                  int last, int np, int nl, int id_cloud_top, const int *seeds, double dp_corr,
                  const double *cond_rsd, const double *w_cloud, const double *p, McicaState &out, char *msg,
                  size_t msg_len, const double *c_cloud = nullptr, const double *c_ratio = nullptr);

}  // namespace socgpu
