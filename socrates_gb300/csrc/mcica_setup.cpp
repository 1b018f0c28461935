// mcica_setup.cpp -- the McICA data file (read_mcica_data.F90) and
// set_cld_mcica (socrates_set_cld_mcica.F90:82-228) for the column driver
// and runes.
#include "mcica_setup.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace socgpu {

bool read_mcica_data(const std::string &path, McicaData &m, std::string &err) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) { err = "McICA data file " + path + " could not be opened"; return false; }
  std::vector<std::string> lines;
  char buf[4096];
  while (std::fgets(buf, sizeof(buf), f)) {
    std::string s(buf);
    while (!s.empty() && (s.back() == '\n' || s.back() == '\r' || s.back() == ' ')) s.pop_back();
    lines.push_back(s);
  }
  std::fclose(f);
  size_t i = 0;
  while (i < lines.size() && lines[i].rfind("*DATA", 0) != 0) ++i;
  if (i == lines.size()) { err = "No *DATA block present in McICA data file"; return false; }
  ++i;
  // the next n values (integers or reals) from line i on
  auto values = [&](size_t n, std::vector<double> &out) {
    out.clear();
    while (out.size() < n && i < lines.size()) {
      const char *c = lines[i++].c_str();
      char *end = nullptr;
      for (double v = std::strtod(c, &end); end != c; v = std::strtod(c, &end)) {
        out.push_back(v);
        c = end;
      }
    }
    return out.size() == n;
  };
  std::vector<double> v;
  while (i < lines.size() && lines[i].rfind("*END", 0) != 0) {
    std::string key = lines[i++];
    key.erase(0, key.find_first_not_of(' '));
    bool ok = true;
    if (key == "tot_subcol_gen" || key == "n_subcol_gen") { ok = values(1, v); m.gen = (int)v[0]; }
    else if (key == "subcol_need_single" || key == "n_subcol_req_single") { ok = values(1, v); m.req_single = (int)v[0]; }
    else if (key == "subcol_need_optimal" || key == "n_subcol_req_optimal") { ok = values(1, v); m.req_optimal = (int)v[0]; }
    else if (key == "ipph") { ok = values(1, v); m.ipph = (int)v[0]; }
    else if (key == "n1") { ok = values(1, v); m.n1 = (int)v[0]; }
    else if (key == "n2") { ok = values(1, v); m.n2 = (int)v[0]; }
    else if (key == "lw_subcol_reorder_single" || key == "lw_subcol_reorder_optimal") {
      const bool single = key == "lw_subcol_reorder_single";
      ok = values((size_t)(single ? m.req_single : m.req_optimal), v);
      (single ? m.reorder_single : m.reorder_optimal).assign(v.begin(), v.end());
    } else if (key == "sw_subcol_k" || key == "lw_subcol_k") {
      auto &tab = key == "sw_subcol_k" ? m.sw_subcol_k : m.lw_subcol_k;
      for (;;) {
        if (!values(3, v)) { ok = false; break; }
        if ((int)v[0] == -99) break;
        tab[{(int)v[0], (int)v[1]}] = (int)v[2];
      }
    } else if (key == "xcw") {
      ok = values((size_t)m.n1 * (size_t)m.n2, v);
      m.xcw = v;
    }
    if (!ok) { err = "Error reading data from McICA data file (" + key + ")"; return false; }
  }
  if (m.gen < 1 || m.xcw.empty()) { err = "McICA data file without subcolumn count or xcw"; return false; }
  return true;
}


void McicaState::attach(socgpu_cld &cld) {
  cld.n_subcol_gen = gen;
  cld.n_subcol_req = n_subcol_req;
  cld.c_sub = c_sub.data();
  cld.frac_cloudy = frac_cloudy.data();
  cld.n_subcol_cld = n_subcol_cld.data();
  cld.subcol_k = subcol_k.data();
  cld.first_subcol_k = first_subcol_k.data();
  cld.subcol_reorder = subcol_reorder.data();
}

int set_cld_mcica(socgpu_spectrum_handle h, const McicaData &md, int isolir, int sampling, int ioverlap, int first,
                  int last, int np, int nl, int id_cloud_top, const int *seeds, double dp_corr,
                  const double *cond_rsd, const double *w_cloud, const double *p, McicaState &out, char *msg,
                  size_t msg_len, const double *c_cloud, const double *c_ratio) {
  auto fail = [&](int st, const char *m) {
    if (msg && msg_len) std::snprintf(msg, msg_len, "%s", m);
    return st;
  };
  if (sampling < SOCGPU_IP_MCICA_FULL_SAMPLING || sampling > SOCGPU_IP_MCICA_OPTIMAL_SAMPLING)
    return fail(SOCGPU_I_ERR_FATAL, "The value of i_mcica_sampling is not valid.");
  const int gen = md.gen;
  if (gen < 1 || gen > SOCGPU_MAX_SUBCOL) return fail(SOCGPU_I_ERR_RANGE, "McICA subcolumns outside the solver's range");
  int n_band = 0, nd_k = 1;
  if (socgpu_spectrum_k_terms(h, 0, &n_band, &nd_k, nullptr) != SOCGPU_I_NORMAL)
    return fail(SOCGPU_I_ERR_EXIST, "spectrum lookup failed");
  if (first < 1 || last > n_band || last < first) return fail(SOCGPU_I_ERR_RANGE, "band range outside the spectrum");
  std::vector<int> n_k_major(std::max(n_band, 1), 0);
  socgpu_spectrum_k_terms(h, n_band, &n_band, &nd_k, n_k_major.data());
  McicaState s;
  s.gen = gen;
  s.nd_k = nd_k;
  // sampling tables (socrates_set_cld_mcica.F90:106-160)
  s.subcol_k.assign((size_t)n_band * nd_k, 1);
  if (sampling == SOCGPU_IP_MCICA_FULL_SAMPLING) {
    s.n_subcol_req = gen;
    std::fill(s.subcol_k.begin(), s.subcol_k.end(), gen);
  } else if (sampling == SOCGPU_IP_MCICA_SINGLE_SAMPLING) {
    s.n_subcol_req = md.req_single;
  } else {
    s.n_subcol_req = md.req_optimal;
    for (const auto &kv : isolir == SOCGPU_IP_SOLAR ? md.sw_subcol_k : md.lw_subcol_k) {
      const int b = kv.first.first, k = kv.first.second;
      if (b >= 1 && b <= n_band && k >= 1 && k <= nd_k) s.subcol_k[(size_t)(b - 1) + (size_t)n_band * (k - 1)] = kv.second;
    }
  }
  if (s.n_subcol_req < 1) return fail(SOCGPU_I_ERR_FATAL, "the McICA data file gives no subcolumns for this sampling");
  s.first_subcol_k.assign((size_t)n_band * (nd_k + 1), 0);
  auto fs = [&](int b, int k) -> int & { return s.first_subcol_k[(size_t)b + (size_t)n_band * k]; };
  fs(first - 1, 0) = 1;
  for (int b = first - 1; b < last; ++b) {
    const int n_k = n_k_major[b];
    for (int k = 0; k < n_k; ++k) fs(b, k + 1) = fs(b, k) + s.subcol_k[(size_t)b + (size_t)n_band * k];
    if (b < last - 1) fs(b + 1, 0) = fs(b, n_k);
  }
  s.subcol_reorder.assign(s.n_subcol_req, 0);
  for (int l = 1; l <= s.n_subcol_req; ++l) {
    int v2;
    if (isolir == SOCGPU_IP_SOLAR) v2 = l % gen;
    else if (sampling == SOCGPU_IP_MCICA_FULL_SAMPLING) v2 = l;
    else {
      const std::vector<int> &src = sampling == SOCGPU_IP_MCICA_SINGLE_SAMPLING ? md.reorder_single : md.reorder_optimal;
      if ((int)src.size() < s.n_subcol_req) return fail(SOCGPU_I_ERR_FATAL, "McICA data file: short subcolumn reorder list");
      v2 = src[l - 1] % gen;
    }
    s.subcol_reorder[l - 1] = v2 == 0 ? gen : v2;
  }
  // the generator (cloud_gen with the decorrelation scales of
  // socrates_set_cld_mcica.F90:185-206), then frac_cloudy
  const size_t ncl = (size_t)(nl - id_cloud_top + 1), cells = (size_t)np * ncl;
  std::vector<double> dp_cloud(cells, dp_corr), dp_cond(cells, 0.5 * dp_corr), zero(cells, 0.0);
  s.c_sub.assign(cells * (size_t)gen, 0.0);
  s.n_subcol_cld.assign(np, 0);
  int st = socgpu_cloud_gen(nl, id_cloud_top, nl, np, 1, np, gen, md.n1, md.n2, md.ipph, ioverlap, seeds,
                            dp_cloud.data(), dp_cond.data(), cond_rsd, w_cloud, c_cloud ? c_cloud : zero.data(),
                            c_ratio ? c_ratio : zero.data(), p,
                            md.xcw.data(), s.n_subcol_cld.data(), s.c_sub.data(), SOCGPU_RNG_LCG, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  s.frac_cloudy.assign(np, 1.0);
  if (sampling != SOCGPU_IP_MCICA_FULL_SAMPLING)
    for (int l = 0; l < np; ++l) s.frac_cloudy[l] = (double)s.n_subcol_cld[l] / (double)gen;
  out = std::move(s);
  return SOCGPU_I_NORMAL;
}

}  // namespace socgpu
