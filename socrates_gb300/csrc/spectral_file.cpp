// spectral_file.cpp -- reading the reference's text spectral files into a
// socgpu_spectrum_desc, and socgpu_spectrum_load (the file-reading part of
// set_spectrum, src/interface_core/socrates_set_spectrum.F90:90-121).
//
// Record layouts of read_spectrum.F90 (blocks 0-13): block 0 summary
// (versions 1 and 2), 1 band limits, 2 solar spectrum, 3 Rayleigh, 4
// absorbers per band, 5 k-terms (fixed columns: (2(3x,1pe16.9), i3, :,
// (t42, 1pe16.9, 3x, 1pe16.9))), 6 Planck polynomial, 8 and 9 continua, 13
// Doppler broadening, 10 and 12 Pade droplet and ice parameters (schemes 5
// and 20).  Other blocks are skipped.  Lookup tables come from the '_k' file.
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "host_internal.h"

namespace socgpu {
namespace {

// Parameters of each scaling function (rad_pcf.F90 n_scale_variable).
int n_scale_variable(int fnc) {
  static const int n[] = {0, 2, 3, 4, 0, 0, 6, 8, 10, 0, 0};
  return (fnc >= 0 && fnc <= 10) ? n[fnc] : 0;
}

std::string upper(std::string s) {
  for (char &c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

std::vector<std::string> split(const std::string &s) {
  std::istringstream in(s);
  std::vector<std::string> out;
  std::string w;
  while (in >> w) out.push_back(w);
  return out;
}

bool is_int(const std::string &w) {
  if (w.empty()) return false;
  for (char c : w)
    if (!std::isdigit((unsigned char)c) && c != '-' && c != '+') return false;
  return true;
}

// a Fortran real or integer literal (1.0E+00, 1.0D-03, -5, .5)
bool is_number(const std::string &w) {
  if (w.empty()) return false;
  bool digit = false;
  for (char c : w) {
    if (std::isdigit((unsigned char)c)) digit = true;
    else if (c != '-' && c != '+' && c != '.' && c != 'E' && c != 'e' && c != 'D' && c != 'd') return false;
  }
  return digit;
}

double num(const std::string &w) {
  std::string t = w;
  for (char &c : t)
    if (c == 'D' || c == 'd') c = 'E';
  return std::strtod(t.c_str(), nullptr);
}

// the first integer after '=' in a line
int int_after_eq(const std::string &line, int which = 0) {
  size_t p = 0;
  for (int k = 0; k <= which; ++k) {
    p = line.find('=', p);
    if (p == std::string::npos) return 0;
    ++p;
  }
  return std::atoi(line.c_str() + p);
}

double fixed(const std::string &line, size_t a, size_t b, bool &present) {
  present = line.size() > a && line.find_first_not_of(' ', a) < std::min(b, line.size());
  if (!present) return 0.0;
  return num(line.substr(a, b - a));
}

struct Block {
  int type = 0, subtype = 0, version = 0;
  std::vector<std::string> lines;
};

// The 1PE13.6 fields of one record of a '_k' file.
std::vector<double> fields13(const std::string &line) {
  std::vector<double> v;
  size_t end = line.find_last_not_of(" \r");
  if (end == std::string::npos) return v;
  for (size_t i = 0; i <= end; i += 13) {
    const std::string f = line.substr(i, 13);
    if (f.find_first_not_of(' ') != std::string::npos) v.push_back(std::strtod(f.c_str(), nullptr));
  }
  return v;
}

}  // namespace

// Owned arrays of one spectral file, in the layouts of socgpu_spectrum_desc.
struct SpectralFile {
  int n_band = 0, n_abs = 0, nd_k = 1, nsv = 4, ndc = 1;
  std::vector<double> wl_s, wl_l, solar, rayleigh;
  std::vector<int> type_absorb, n_band_absorb, band_overlap, index_absorb, i_band_k, i_scale_k, i_scale_fnc;
  std::vector<double> k, w, scale, p_ref, t_ref;
  std::vector<int> l_doppler;
  std::vector<double> doppler_cor;
  int n_deg_fit = 0;
  double t_ref_planck = 0.0;
  std::vector<double> thermal;
  std::vector<int> n_band_cont, index_cont, fnc_cont;
  std::vector<double> k_cont, scale_cont, p_ref_cont, t_ref_cont;
  int index_water = 0;
  // blocks 10 and 12: (ncp, n_band, n_type) at the file's type numbers
  int ncp = 0;
  std::vector<double> drop_parm, ice_parm, drop_lo, drop_hi, ice_lo, ice_hi;
  std::vector<int> drop_ids, ice_ids, drop_on, ice_on;
  // lookup tables of the '_k' file
  int n_pre = 0, n_tmp = 0, n_gf = 0, nsb = 0, nd_t = 0;
  std::vector<double> p_lookup, t_lookup, k_lookup, gf_lookup, k_lookup_sb, molar_weight;
  std::vector<int> index_sb, n_t_gas;
  std::vector<double> t_gas, k_t_gas;
  // Wen-Yi tables
  std::vector<double> wy_plg, wy_ttb, wy_tto, wy_gk250b, wy_gk4, wy_gk6;
  // block 11: classic aerosol species
  int n_aer = 0, nd_hum = 1, nd_phf = 1;
  std::vector<int> aer_type, aer_parm, aer_nhum, aer_nphf;
  std::vector<double> aer_hum, aer_abs, aer_scat, aer_phf;

  socgpu_spectrum_desc desc() const {
    socgpu_spectrum_desc d{};
    d.nd_band = n_band;
    d.nd_species = std::max(1, n_abs);
    d.nd_k_term = nd_k;
    d.nd_scale_variable = nsv;
    d.n_band = n_band;
    d.wavelength_short = wl_s.data();
    d.wavelength_long = wl_l.data();
    d.solar_flux_band = solar.empty() ? nullptr : solar.data();
    d.i_rayleigh_scheme = SOCGPU_IP_RAYLEIGH_TOTAL;
    d.rayleigh_coeff = rayleigh.empty() ? nullptr : rayleigh.data();
    d.n_absorb = n_abs;
    d.type_absorb = type_absorb.data();
    d.n_band_absorb = n_band_absorb.data();
    d.i_overlap = band_overlap.data();
    d.index_absorb = index_absorb.data();
    d.i_band_k = i_band_k.data();
    d.i_scale_k = i_scale_k.data();
    d.i_scale_fnc = i_scale_fnc.data();
    d.k = k.data();
    d.w = w.data();
    d.scale = scale.data();
    d.p_ref = p_ref.data();
    d.t_ref = t_ref.data();
    d.l_doppler = l_doppler.empty() ? nullptr : l_doppler.data();
    d.doppler_cor = doppler_cor.empty() ? nullptr : doppler_cor.data();
    if (!thermal.empty()) {
      d.n_deg_fit = n_deg_fit;
      d.t_ref_planck = t_ref_planck;
      d.nd_thermal_coeff = n_deg_fit + 1;
      d.thermal_coeff = thermal.data();
    }
    if (!drop_ids.empty()) {
      d.nd_cloud_parameter = ncp;
      d.nd_drop_type = (int)drop_ids.size();
      d.drop_parm_list = drop_parm.data();
      d.i_drop_parm = drop_ids.data();
      d.l_drop_type = drop_on.data();
      d.drop_parm_min_dim = drop_lo.data();
      d.drop_parm_max_dim = drop_hi.data();
    }
    if (!ice_ids.empty()) {
      d.nd_cloud_parameter = ncp;
      d.nd_ice_type = (int)ice_ids.size();
      d.ice_parm_list = ice_parm.data();
      d.i_ice_parm = ice_ids.data();
      d.l_ice_type = ice_on.data();
      d.ice_parm_min_dim = ice_lo.data();
      d.ice_parm_max_dim = ice_hi.data();
    }
    if (!k_lookup.empty()) {
      d.n_pre = n_pre; d.n_tmp = n_tmp;
      d.p_lookup = p_lookup.data(); d.t_lookup = t_lookup.data(); d.k_lookup = k_lookup.data();
    }
    if (!k_lookup_sb.empty()) {
      d.index_sb = index_sb.data(); d.nd_species_sb = nsb; d.n_gas_frac = n_gf;
      d.gf_lookup = gf_lookup.data(); d.k_lookup_sb = k_lookup_sb.data();
    }
    d.molar_weight = molar_weight.empty() ? nullptr : molar_weight.data();
    if (!k_t_gas.empty()) {
      d.nd_t_lookup_gas = nd_t; d.n_t_lookup_gas = n_t_gas.data();
      d.t_lookup_gas = t_gas.data(); d.k_t_lookup_gas = k_t_gas.data();
    }
    if (!wy_plg.empty()) {
      d.wenyi_plg = wy_plg.data(); d.wenyi_ttb = wy_ttb.data(); d.wenyi_tto = wy_tto.data();
      d.wenyi_gk250b = wy_gk250b.data(); d.wenyi_gk4 = wy_gk4.data(); d.wenyi_gk6 = wy_gk6.data();
      d.wenyi_n_term4 = (int)wy_gk250b.size(); d.wenyi_n_term6 = (int)(wy_gk6.size() / 234);
    }
    if (n_aer > 0) {
      d.n_aerosol = d.nd_aerosol_species = n_aer;
      d.nd_humidity = nd_hum; d.nd_phase_term = nd_phf;
      d.type_aerosol = aer_type.data(); d.i_aerosol_parm = aer_parm.data();
      d.nhumidity = aer_nhum.data(); d.n_aerosol_phf_term = aer_nphf.data();
      d.aerosol_humidities = aer_hum.data(); d.aerosol_abs = aer_abs.data();
      d.aerosol_scat = aer_scat.data(); d.aerosol_phf = aer_phf.data();
    }
    if (!n_band_cont.empty()) {
      d.nd_continuum = ndc;
      d.n_band_continuum = n_band_cont.data();
      d.index_continuum = index_cont.data();
      d.index_water = index_water;
      d.i_scale_fnc_cont = fnc_cont.data();
      d.k_cont = k_cont.data();
      d.scale_cont = scale_cont.data();
      d.p_ref_cont = p_ref_cont.data();
      d.t_ref_cont = t_ref_cont.data();
    }
    return d;
  }
};

// Molar weights [g/mol] of the absorbers by gas identifier (the published
// values of J. A. Duffy, General Inorganic Chemistry (1970), and NIST, as
// gas_list_pcf.F90:303-330 lists them); used for self-broadened gas fractions.
double molar_weight_of(int type) {
  static const double mw[] = {0.0, 18.0153, 44.0100, 47.9982, 44.0128, 28.0106, 16.0430, 31.9988, 30.0061,
                              64.0628, 46.0055, 17.0306, 63.0129, 28.0134, 137.3686, 120.9140, 187.3765,
                              86.46892, 120.02227, 102.03184, 170.921, 63.866, 66.9409, 2.01588, 4.002602,
                              60.075};
  return (type >= 1 && type < (int)(sizeof(mw) / sizeof(mw[0]))) ? mw[type] : 0.0;
}

// The lookup tables of a '_k' file in the order read_spectrum.F90:1420-1560
// reads them: the P/T grid, the gas fractions of self-broadened absorbers,
// one table per (band, absorber) record of block 5 (recs: band, absorber,
// scaling function, 0-based), then the temperature-only tables.
bool read_k_file(const std::string &path, SpectralFile &s, const std::vector<std::array<int, 3>> &recs,
                 std::string &err) {
  std::ifstream in(path);
  if (!in) { err = "the k-term lookup tables of block 5 are in " + path + ", which cannot be read"; return false; }
  std::vector<std::string> text;
  std::string line;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    text.push_back(line);
  }
  auto values = [&](size_t &q, size_t n, std::vector<double> &out) -> bool {
    out.clear();
    while (out.size() < n) {
      if (q >= text.size()) return false;
      for (double v : fields13(text[q++])) out.push_back(v);
    }
    out.resize(n);
    return true;
  };
  auto block = [&](const std::string &title, size_t &q) -> bool {
    for (q = 0; q < text.size(); ++q)
      if (text[q].rfind("*BLOCK", 0) == 0 && text[q].compare(8, title.size(), title) == 0) return true;
    return false;
  };
  const int nb = s.n_band, na = std::max(1, s.n_abs), ndk = s.nd_k;
  auto nk_of = [&](int b, int g) { return s.i_band_k[(size_t)b + (size_t)nb * g]; };
  std::vector<double> v;
  bool any_pt = false, any_t = false;
  for (auto &r : recs) { any_pt |= r[2] == SOCGPU_IP_SCALE_LOOKUP; any_t |= r[2] == SOCGPU_IP_SCALE_T_LOOKUP; }
  if (any_pt) {
    size_t q = 0;
    if (!block("k-table", q)) { err = path + ": no k-table block"; return false; }
    q += 3;
    const int npre = s.n_pre, ntmp = s.n_tmp;
    if (npre < 2 || ntmp < 2) { err = path + ": bad P/T table extents"; return false; }
    s.p_lookup.assign(npre, 0.0);
    s.t_lookup.assign((size_t)ntmp * npre, 0.0);
    for (int ip = 0; ip < npre; ++ip) {
      if (!values(q, 1 + ntmp, v)) { err = path + ": P/T grid truncated"; return false; }
      s.p_lookup[ip] = std::log(v[0]);
      for (int it = 0; it < ntmp; ++it) s.t_lookup[(size_t)it + (size_t)ntmp * ip] = v[1 + it];
    }
    bool sb = false;
    for (int x : s.index_sb) { sb |= x > 0; s.nsb = std::max(s.nsb, x); }
    if (sb) {
      if (q + 1 >= text.size()) { err = path + ": gas-fraction table missing"; return false; }
      s.n_gf = std::atoi(text[q + 1].substr(std::min<size_t>(14, text[q + 1].size())).c_str());
      q += 2;
      if (s.n_gf < 1 || !values(q, s.n_gf, s.gf_lookup)) { err = path + ": bad gas-fraction table"; return false; }
      s.k_lookup_sb.assign((size_t)ntmp * npre * s.n_gf * ndk * s.nsb * nb, 0.0);
    } else {
      s.index_sb.clear();
    }
    s.k_lookup.assign((size_t)ntmp * npre * ndk * na * nb, 0.0);
    for (auto &r : recs) {
      if (r[2] != SOCGPU_IP_SCALE_LOOKUP) continue;
      const int b = r[0], g = r[1], nk = nk_of(b, g);
      q += 2;
      const int jsb = sb ? s.index_sb[g] - 1 : -1;
      for (int t = 0; t < nk; ++t) {
        const int ngf = jsb >= 0 ? s.n_gf : 1;
        for (int ig = 0; ig < ngf; ++ig)
          for (int ip = 0; ip < npre; ++ip) {
            if (!values(q, ntmp, v)) { err = path + ": k table truncated"; return false; }
            for (int it = 0; it < ntmp; ++it) {
              if (jsb >= 0)
                s.k_lookup_sb[(size_t)it + (size_t)ntmp * ((size_t)ip + (size_t)npre * ((size_t)ig + (size_t)s.n_gf *
                    ((size_t)t + (size_t)ndk * ((size_t)jsb + (size_t)s.nsb * b))))] = v[it];
              else
                s.k_lookup[(size_t)it + (size_t)ntmp * ((size_t)ip + (size_t)npre * ((size_t)t + (size_t)ndk *
                    ((size_t)g + (size_t)na * b)))] = v[it];
            }
          }
      }
    }
  }
  if (any_t) {
    size_t q = 0;
    if (!block("temperature k-tables", q)) { err = path + ": no temperature k-tables block"; return false; }
    if (q + 2 >= text.size()) { err = path + ": bad temperature tables"; return false; }
    s.nd_t = std::atoi(text[q + 2].substr(std::min<size_t>(9, text[q + 2].size())).c_str());
    q += 3;
    s.n_t_gas.assign(na, 0);
    s.t_gas.assign((size_t)s.nd_t * na, 0.0);
    std::vector<int> t_gases;
    for (auto &r : recs)
      if (r[2] == SOCGPU_IP_SCALE_T_LOOKUP && std::find(t_gases.begin(), t_gases.end(), r[1]) == t_gases.end())
        t_gases.push_back(r[1]);
    std::sort(t_gases.begin(), t_gases.end());
    for (int g : t_gases) {
      if (q + 1 >= text.size()) { err = path + ": temperature grid missing"; return false; }
      s.n_t_gas[g] = std::atoi(text[q + 1].substr(std::min<size_t>(27, text[q + 1].size())).c_str());
      q += 2;
      if (s.n_t_gas[g] < 2 || s.n_t_gas[g] > s.nd_t || !values(q, s.n_t_gas[g], v)) {
        err = path + ": bad temperature grid";
        return false;
      }
      for (int k = 0; k < s.n_t_gas[g]; ++k) s.t_gas[(size_t)k + (size_t)s.nd_t * g] = v[k];
    }
    s.k_t_gas.assign((size_t)s.nd_t * ndk * na * nb, 0.0);
    for (int b = 0; b < nb; ++b)
      for (int j = 0; j < s.n_band_absorb[b]; ++j) {
        const int g = s.index_absorb[(size_t)j + (size_t)na * b] - 1;
        bool is_t = false;
        for (auto &r : recs) is_t |= r[0] == b && r[1] == g && r[2] == SOCGPU_IP_SCALE_T_LOOKUP;
        if (!is_t) continue;
        q += 2;
        for (int t = 0; t < nk_of(b, g); ++t) {
          if (!values(q, s.n_t_gas[g], v)) { err = path + ": temperature k table truncated"; return false; }
          for (int k = 0; k < s.n_t_gas[g]; ++k)
            s.k_t_gas[(size_t)k + (size_t)s.nd_t * ((size_t)t + (size_t)ndk * ((size_t)g + (size_t)na * b))] = v[k];
        }
      }
  }
  return true;
}

// Wen-Yi Zhong's CO2 (band 4) and O3 (band 6) tables from their data file
// (socrates_gb300/wenyi.py writes it from the reference's scale_wenyi
// module): a header line "socgpu-wenyi-tables 1", then the arrays plg (26),
// ttb (10), tto (9), gk250b (n4), gk4 (10 x 26 x n4) and gk6 (9 x 26 x n6),
// each as "<name> <dims...>" followed by its values, first index fastest.
bool read_wenyi(const std::string &path, SpectralFile &s, std::string &err) {
  std::ifstream in(path);
  if (!in) { err = "cannot open the Wen-Yi tables " + path; return false; }
  std::string magic, version;
  in >> magic >> version;
  if (magic != "socgpu-wenyi-tables" || version != "1") {
    err = path + ": not a Wen-Yi tables file (no 'socgpu-wenyi-tables 1' header)";
    return false;
  }
  struct Want { const char *name; int ndim; std::vector<double> *dst; std::vector<long> dims; };
  Want want[] = {{"plg", 1, &s.wy_plg, {}}, {"ttb", 1, &s.wy_ttb, {}}, {"tto", 1, &s.wy_tto, {}},
                 {"gk250b", 1, &s.wy_gk250b, {}}, {"gk4", 3, &s.wy_gk4, {}}, {"gk6", 3, &s.wy_gk6, {}}};
  for (Want &w : want) {
    std::string name;
    in >> name;
    if (name != w.name) { err = path + ": expected the array '" + w.name + "'"; return false; }
    size_t n = 1;
    for (int d = 0; d < w.ndim; ++d) {
      long v = 0;
      in >> v;
      if (!in || v < 1 || v > 4096) { err = path + ": bad dimensions of '" + name + "'"; return false; }
      w.dims.push_back(v);
      n *= (size_t)v;
    }
    w.dst->assign(n, 0.0);
    for (size_t q = 0; q < n; ++q) in >> (*w.dst)[q];
    if (!in) { err = path + ": '" + name + "' is short of values"; return false; }
  }
  const bool ok = want[0].dims[0] == 26 && want[1].dims[0] == 10 && want[2].dims[0] == 9 &&
                  want[4].dims[0] == 10 && want[4].dims[1] == 26 && want[4].dims[2] == want[3].dims[0] &&
                  want[5].dims[0] == 9 && want[5].dims[1] == 26;
  if (!ok) { err = path + ": the Wen-Yi tables have the wrong shapes"; return false; }
  return true;
}

bool read_spectral_file(const std::string &path, const std::string &k_path, const std::string &wenyi_path,
                        SpectralFile &sf, std::string &err) {
  std::ifstream in(path);
  if (!in) { err = "cannot open spectral file " + path; return false; }
  std::vector<Block> blocks;
  Block *cur = nullptr;
  std::string line;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.rfind("*BLOCK", 0) == 0) {
      std::string t = line;
      for (char &c : t)
        if (c == ':' || c == '=') c = ' ';
      auto w = split(t);
      blocks.emplace_back();
      cur = &blocks.back();
      cur->type = w.size() > 2 ? std::atoi(w[2].c_str()) : -1;
      cur->subtype = w.size() > 4 ? std::atoi(w[4].c_str()) : 0;
      cur->version = w.size() > 6 ? std::atoi(w[6].c_str()) : 0;
    } else if (line.rfind("*END", 0) == 0) {
      cur = nullptr;
    } else if (cur) {
      cur->lines.push_back(line);
    }
  }
  auto first = [&](int t) -> const Block * {
    for (const Block &b : blocks)
      if (b.type == t) return &b;
    return nullptr;
  };
  const Block *b0 = first(0), *b1 = first(1), *b4 = first(4), *b5 = first(5);
  if (!b0 || !b1) { err = path + ": summary or band limits missing"; return false; }
  SpectralFile s;
  for (size_t q = 0; q < b0->lines.size(); ++q) {
    std::string u = upper(b0->lines[q]);
    if (u.find("SPECTRAL BANDS") != std::string::npos) s.n_band = int_after_eq(u);
    else if (u.find("GASEOUS ABSORBERS") != std::string::npos) s.n_abs = int_after_eq(u);
    else if (u.find("INDEXING NUMBERS") != std::string::npos && u.find("ABSORBER") != std::string::npos &&
             u.find("AEROSOL") == std::string::npos) {
      for (int i = 0; i < s.n_abs && q + 2 + i < b0->lines.size(); ++i) {
        auto w = split(b0->lines[q + 2 + i]);
        if (w.size() < 2) { err = path + ": bad absorber list"; return false; }
        s.type_absorb.push_back(std::atoi(w[1].c_str()));
      }
    }
  }
  if (s.n_band < 1 || (int)s.type_absorb.size() != s.n_abs) { err = path + ": bad summary block"; return false; }
  const int nb = s.n_band, na = std::max(1, s.n_abs);
  s.wl_s.assign(nb, 0.0);
  s.wl_l.assign(nb, 0.0);
  for (size_t q = 3; q < b1->lines.size(); ++q) {
    auto w = split(b1->lines[q]);
    if (w.size() >= 3 && is_int(w[0])) {
      int b = std::atoi(w[0].c_str()) - 1;
      if (b >= 0 && b < nb) { s.wl_s[b] = num(w[1]); s.wl_l[b] = num(w[2]); }
    }
  }
  auto band_values = [&](int t, std::vector<double> &out) {
    const Block *bl = first(t);
    if (!bl) return;
    out.assign(nb, 0.0);
    for (const std::string &l : bl->lines) {
      auto w = split(l);
      if (w.size() >= 2 && is_int(w[0])) {
        int b = std::atoi(w[0].c_str()) - 1;
        if (b >= 0 && b < nb) out[b] = num(w[1]);
      }
    }
  };
  band_values(2, s.solar);
  band_values(3, s.rayleigh);
  // block 4
  s.n_band_absorb.assign(nb, 0);
  s.band_overlap.assign(nb, 0);
  s.index_absorb.assign((size_t)na * nb, 0);
  if (b4) {
    std::vector<std::string> tok;
    for (size_t q = 5; q < b4->lines.size(); ++q)
      for (auto &w : split(b4->lines[q])) tok.push_back(w);
    size_t q = 0;
    const bool with_overlap = b4->version >= 1;   // each band's overlap method follows its count
    for (int i = 0; i < nb && q + 1 < tok.size(); ++i) {
      int b = std::atoi(tok[q].c_str()) - 1, n = std::atoi(tok[q + 1].c_str());
      const int ov = with_overlap && q + 2 < tok.size() ? std::atoi(tok[q + 2].c_str()) : 0;
      q += with_overlap ? 3 : 2;
      if (b < 0 || b >= nb || n < 0 || n > na) { err = path + ": bad block 4"; return false; }
      s.n_band_absorb[b] = n;
      s.band_overlap[b] = ov;
      for (int j = 0; j < n && q < tok.size(); ++j) s.index_absorb[(size_t)j + (size_t)na * b] = std::atoi(tok[q++].c_str());
    }
  }
  // block 5: first pass for sizes
  struct Term { double k, w; std::vector<double> sc; };
  struct Rec { int b, g, nk, sk, fnc; double p, t; std::vector<Term> terms; };
  std::vector<Rec> recs;
  if (b5) {
    const auto &L = b5->lines;
    size_t q = 4;
    // version 1: the self-broadened indices of all absorbers may come first
    // (read_spectrum.F90:1268-1300)
    for (size_t h = 0; h < L.size(); ++h) {
      if (L[h].find("Self-broadened indexing numbers") != std::string::npos) {
        size_t r = h + 2;
        while ((int)s.index_sb.size() < s.n_abs && r < L.size())
          for (auto &x : split(L[r++])) s.index_sb.push_back(std::atoi(x.c_str()));
      }
      if (L[h].rfind("Band        Gas, Number of k-terms", 0) == 0) { q = h + 3; break; }
    }
    while (q < L.size()) {
      auto w = split(L[q]);
      if (w.size() < 5 || !is_int(w[0])) { ++q; continue; }
      Rec r{std::atoi(w[0].c_str()) - 1, std::atoi(w[1].c_str()) - 1, std::atoi(w[2].c_str()),
            std::atoi(w[3].c_str()), std::atoi(w[4].c_str()), 0.0, 0.0, {}};
      if (q + 1 >= L.size()) break;
      auto pt = split(L[q + 1]);
      if (r.fnc == SOCGPU_IP_SCALE_LOOKUP) {
        if (pt.size() < 2) { err = path + ": bad block 5 table extents"; return false; }
        s.n_pre = std::atoi(pt[0].c_str());
        s.n_tmp = std::atoi(pt[1].c_str());
      } else if (r.fnc != SOCGPU_IP_SCALE_T_LOOKUP) {
        if (pt.size() < 2) { err = path + ": bad block 5"; return false; }
        r.p = num(pt[0]);
        r.t = num(pt[1]);
      }
      q += 2;
      const int nsv = n_scale_variable(r.fnc);
      for (int t = 0; t < r.nk && q < L.size(); ++t) {
        Term tm;
        bool pr = false;
        tm.k = fixed(L[q], 3, 19, pr);
        tm.w = fixed(L[q], 22, 38, pr);
        std::string col = L[q];
        while ((int)tm.sc.size() < nsv) {
          const size_t starts[2] = {41, 60};
          for (size_t a : starts)
            if ((int)tm.sc.size() < nsv) {
              double v = fixed(col, a, a + 16, pr);
              if (pr) tm.sc.push_back(v);
            }
          if ((int)tm.sc.size() < nsv) {
            if (++q >= L.size()) break;
            col = L[q];
          }
        }
        ++q;
        r.terms.push_back(tm);
      }
      s.nd_k = std::max(s.nd_k, r.nk);
      s.nsv = std::max(s.nsv, nsv);
      recs.push_back(std::move(r));
    }
  }
  const size_t ndk = s.nd_k, nsv = s.nsv;
  s.i_band_k.assign((size_t)nb * na, 0);
  s.i_scale_k.assign((size_t)nb * na, 0);
  s.i_scale_fnc.assign((size_t)nb * na, 0);
  s.k.assign(ndk * nb * na, 0.0);
  s.w.assign(ndk * nb * na, 0.0);
  s.scale.assign(nsv * ndk * nb * na, 0.0);
  s.p_ref.assign((size_t)na * nb, 0.0);
  s.t_ref.assign((size_t)na * nb, 0.0);
  for (const Rec &r : recs) {
    if (r.b < 0 || r.b >= nb || r.g < 0 || r.g >= na) { err = path + ": bad band/gas in block 5"; return false; }
    const size_t bg = (size_t)r.b + (size_t)nb * r.g;
    s.i_band_k[bg] = r.nk;
    s.i_scale_k[bg] = r.sk;
    s.i_scale_fnc[bg] = r.fnc;
    s.p_ref[(size_t)r.g + (size_t)na * r.b] = r.p;
    s.t_ref[(size_t)r.g + (size_t)na * r.b] = r.t;
    for (size_t t = 0; t < r.terms.size(); ++t) {
      const size_t tbg = t + ndk * ((size_t)r.b + (size_t)nb * r.g);
      s.k[tbg] = r.terms[t].k;
      s.w[tbg] = r.terms[t].w;
      for (size_t v = 0; v < r.terms[t].sc.size(); ++v) s.scale[v + nsv * tbg] = r.terms[t].sc[v];
    }
  }
  // the lookup tables (read_spectrum.F90:1420-1560)
  {
    std::vector<std::array<int, 3>> lrecs;
    bool any = false;
    for (const Rec &r : recs) {
      lrecs.push_back({r.b, r.g, r.fnc});
      any |= r.fnc == SOCGPU_IP_SCALE_LOOKUP || r.fnc == SOCGPU_IP_SCALE_T_LOOKUP;
    }
    if (any && !read_k_file(k_path.empty() ? path + "_k" : k_path, s, lrecs, err)) return false;
  }
  if (!wenyi_path.empty() && !read_wenyi(wenyi_path, s, err)) return false;
  s.molar_weight.assign(na, 0.0);
  for (int g = 0; g < s.n_abs; ++g) s.molar_weight[g] = molar_weight_of(s.type_absorb[g]);
  // block 6
  if (const Block *b6 = first(6)) {
    size_t h = 0;
    while (h < b6->lines.size() && b6->lines[h].find('=') == std::string::npos) ++h;
    if (h >= b6->lines.size()) { err = path + ": bad block 6"; return false; }
    s.n_deg_fit = int_after_eq(b6->lines[h]);
    const size_t eq2 = b6->lines[h].find('=', b6->lines[h].find('=') + 1);
    s.t_ref_planck = num(b6->lines[h].substr(eq2 + 1));
    std::vector<std::string> tok;
    for (size_t q = h + 3; q < b6->lines.size(); ++q)
      for (auto &w : split(b6->lines[q])) tok.push_back(w);
    s.thermal.assign((size_t)(s.n_deg_fit + 1) * nb, 0.0);
    size_t q = 0;
    for (int i = 0; i < nb && q < tok.size(); ++i) {
      int b = std::atoi(tok[q++].c_str()) - 1;
      for (int j = 0; j <= s.n_deg_fit && q < tok.size(); ++j)
        if (b >= 0 && b < nb) s.thermal[(size_t)j + (size_t)(s.n_deg_fit + 1) * b] = num(tok[q++]);
    }
  }
  // blocks 8 and 9
  if (const Block *b8 = first(8)) {
    std::vector<std::string> tok;
    for (size_t q = 5; q < b8->lines.size(); ++q) {
      const std::string &l = b8->lines[q];
      if (l.find('=') != std::string::npos) s.index_water = int_after_eq(l);
      else {
        auto w = split(l);
        if (!w.empty() && is_int(w[0]))
          for (auto &x : w) tok.push_back(x);
      }
    }
    std::vector<std::vector<int>> idx(nb);
    size_t q = 0;
    int maxc = 1;
    while (q + 1 < tok.size()) {
      int b = std::atoi(tok[q].c_str()) - 1, n = std::atoi(tok[q + 1].c_str());
      q += 2;
      if (b < 0 || b >= nb || n < 0) { err = path + ": bad block 8"; return false; }
      for (int j = 0; j < n && q < tok.size(); ++j) idx[b].push_back(std::atoi(tok[q++].c_str()));
      maxc = std::max(maxc, n);
    }
    s.ndc = maxc;
    const size_t ndc = s.ndc;
    s.n_band_cont.assign(nb, 0);
    s.index_cont.assign((size_t)nb * ndc, 0);
    s.fnc_cont.assign((size_t)nb * ndc, 0);
    s.k_cont.assign((size_t)nb * ndc, 0.0);
    s.scale_cont.assign(nsv * nb * ndc, 0.0);
    s.p_ref_cont.assign(ndc * nb, 0.0);
    s.t_ref_cont.assign(ndc * nb, 0.0);
    for (int b = 0; b < nb; ++b) {
      s.n_band_cont[b] = (int)idx[b].size();
      for (size_t j = 0; j < idx[b].size(); ++j) s.index_cont[(size_t)b + (size_t)nb * j] = idx[b][j];
    }
    if (const Block *b9 = first(9)) {
      std::vector<std::string> t9;
      for (size_t q9 = 3; q9 < b9->lines.size(); ++q9)
        for (auto &x : split(b9->lines[q9])) t9.push_back(x);
      size_t r = 0;
      while (r + 5 < t9.size()) {
        int b = std::atoi(t9[r].c_str()) - 1, ci = std::atoi(t9[r + 1].c_str()), fnc = std::atoi(t9[r + 2].c_str());
        if (b < 0 || b >= nb) { err = path + ": bad block 9"; return false; }
        size_t j = 0;
        while (j < idx[b].size() && idx[b][j] != ci) ++j;
        if (j == idx[b].size()) { err = path + ": continuum of block 9 not listed in block 8"; return false; }
        const size_t bj = (size_t)b + (size_t)nb * j;
        s.fnc_cont[bj] = fnc;
        s.p_ref_cont[j + ndc * b] = num(t9[r + 3]);
        s.t_ref_cont[j + ndc * b] = num(t9[r + 4]);
        s.k_cont[bj] = num(t9[r + 5]);
        const int nv = n_scale_variable(fnc);
        for (int v = 0; v < nv && r + 6 + v < t9.size(); ++v) s.scale_cont[(size_t)v + nsv * bj] = num(t9[r + 6 + v]);
        r += 6 + nv;
      }
    }
  }
  // block 13
  if (const Block *b13 = first(13)) {
    s.l_doppler.assign(na, 0);
    s.doppler_cor.assign(na, 0.0);
    for (size_t q = 2; q < b13->lines.size(); ++q) {
      auto w = split(b13->lines[q]);
      if (w.size() >= 3 && is_int(w[0])) {
        int i = std::atoi(w[0].c_str()) - 1;
        if (i >= 0 && i < na) {
          s.l_doppler[i] = (std::toupper((unsigned char)w[1][0]) == 'T') ? 1 : 0;
          s.doppler_cor[i] = num(w[2]);
        }
      }
    }
  }
  // blocks 10 and 12 (read_block_10_0_2 / read_block_12_0_2 of
  // read_spectrum.F90): every parameter set at its type number, with its
  // scheme and range of validity
  struct CloudSet { int type, scheme, npar; double lo, hi; std::vector<double> v; };
  auto cloud_sets = [&](int t) {
    std::vector<CloudSet> out;
    for (const Block &bl : blocks) {
      if (bl.type != t) continue;
      size_t h = 0, ht = bl.lines.size();
      for (size_t q = 0; q < bl.lines.size(); ++q) {
        const std::string u = upper(bl.lines[q]);
        if (u.find("TYPE NUMBER") != std::string::npos) ht = q;
      }
      while (h < bl.lines.size() &&
             !(bl.lines[h].find('=') != std::string::npos && upper(bl.lines[h]).find("PARAMETERS") != std::string::npos))
        ++h;
      if (h >= bl.lines.size() || ht >= bl.lines.size()) continue;
      CloudSet cs{int_after_eq(bl.lines[ht]), int_after_eq(bl.lines[h]), int_after_eq(bl.lines[h], 1), 0.0, 0.0, {}};
      if (cs.type < 1 || cs.npar < 1) continue;
      std::vector<std::string> tok;
      for (size_t q = h + 1; q < bl.lines.size(); ++q) {
        const std::string &l = bl.lines[q];
        const std::string u = upper(l);
        bool digit = false;
        for (char c : l) digit |= (bool)std::isdigit((unsigned char)c);
        if (u.find("MOMENTS") != std::string::npos || !digit) continue;
        if (u.find("RANGE") != std::string::npos) {
          const size_t e = l.find('='), dd = l.find("--");
          if (e != std::string::npos && dd != std::string::npos && dd > e) {
            cs.lo = num(l.substr(e + 1, dd - e - 1));
            cs.hi = num(l.substr(dd + 2));
          }
          continue;
        }
        if (u.find("BAND") != std::string::npos && l.find('=') != std::string::npos) tok.push_back(std::to_string(int_after_eq(l)));
        else
          for (auto &x : split(l)) tok.push_back(x);
      }
      cs.v.assign((size_t)cs.npar * nb, 0.0);
      size_t q = 0;
      for (int i = 0; i < nb && q < tok.size(); ++i) {
        int b = std::atoi(tok[q++].c_str()) - 1;
        for (int v = 0; v < cs.npar && q < tok.size(); ++v)
          if (b >= 0 && b < nb) cs.v[(size_t)v + (size_t)cs.npar * b] = num(tok[q++]);
      }
      out.push_back(std::move(cs));
    }
    return out;
  };
  const std::vector<CloudSet> drops = cloud_sets(10), ices = cloud_sets(12);
  for (const auto &c : drops) s.ncp = std::max(s.ncp, c.npar);
  for (const auto &c : ices) s.ncp = std::max(s.ncp, c.npar);
  auto place = [&](const std::vector<CloudSet> &sets, std::vector<double> &parm, std::vector<int> &ids,
                   std::vector<int> &on, std::vector<double> &lo, std::vector<double> &hi) {
    int nt = 0;
    for (const auto &c : sets) nt = std::max(nt, c.type);
    if (nt == 0) return;
    parm.assign((size_t)s.ncp * nb * nt, 0.0);
    ids.assign(nt, 0); on.assign(nt, 0); lo.assign(nt, 0.0); hi.assign(nt, 0.0);
    for (const auto &c : sets) {
      const int t = c.type - 1;
      ids[t] = c.scheme; on[t] = 1; lo[t] = c.lo; hi[t] = c.hi;
      for (int b = 0; b < nb; ++b)
        for (int v = 0; v < c.npar; ++v)
          parm[(size_t)v + (size_t)s.ncp * ((size_t)b + (size_t)nb * t)] = c.v[(size_t)v + (size_t)c.npar * b];
    }
  };
  place(drops, s.drop_parm, s.drop_ids, s.drop_on, s.drop_lo, s.drop_hi);
  place(ices, s.ice_parm, s.ice_ids, s.ice_on, s.ice_lo, s.ice_hi);
  // block 11 (read_spectrum.F90:2335-2640): the species' number and type
  // numbers come from block 0; each block gives one species, dry (subtype 0:
  // per band the band index, absorption, scattering and the phase-function
  // moments) or moist (subtype 1: per band one row per humidity of humidity,
  // absorption, scattering and moments), the values as numeric records after
  // the header lines
  for (size_t q = 0; q < b0->lines.size(); ++q) {
    const std::string u = upper(b0->lines[q]);
    if (u.find("NUMBER OF AEROSOLS") != std::string::npos) s.n_aer = int_after_eq(u);
    else if (u.find("INDEXING NUMBERS OF AEROSOLS") != std::string::npos)
      for (int i = 0; i < s.n_aer && q + 2 + i < b0->lines.size(); ++i) {
        auto w = split(b0->lines[q + 2 + i]);
        s.aer_type.push_back(w.size() >= 2 ? std::atoi(w[1].c_str()) : 0);
      }
  }
  if (s.n_aer > 0) {
    struct Species { bool moist; int rows, nphf; std::vector<double> v; };
    std::map<int, Species> found;
    for (const Block &bl : blocks) {
      if (bl.type != 11) continue;
      int idx = -1, nh = 1, nphf = 1;
      std::vector<double> v;
      for (const std::string &l : bl.lines) {
        const std::string u = upper(l);
        if (u.find("INDEX OF SPECIES") != std::string::npos) idx = int_after_eq(u);
        else if (u.find("NUMBER OF HUMIDITY") != std::string::npos) nh = int_after_eq(u);
        else if (u.find("NUMBER OF TERMS IN PHASE FUNCTION") != std::string::npos) nphf = int_after_eq(u);
        auto w = split(l);
        bool all = !w.empty();
        for (auto &x : w) all = all && is_number(x);
        if (all)
          for (auto &x : w) v.push_back(num(x));
      }
      const bool moist = bl.subtype == 1;
      const int rows = moist ? nh : 1;
      if (idx < 1 || idx > s.n_aer || rows < 1 || nphf < 1 || v.size() < (size_t)nb * rows * (3 + nphf)) {
        err = path + ": bad aerosol block (species " + std::to_string(idx) + ")";
        return false;
      }
      found[idx] = Species{moist, rows, nphf, v};
      s.nd_hum = std::max(s.nd_hum, rows);
      s.nd_phf = std::max(s.nd_phf, nphf);
    }
    const int na_ = s.n_aer, ndh = s.nd_hum, ndf = s.nd_phf;
    s.aer_parm.assign(na_, SOCGPU_IP_AEROSOL_UNPARAMETRIZED);
    s.aer_nhum.assign(na_, 0);
    s.aer_nphf.assign(na_, 1);
    s.aer_hum.assign((size_t)ndh * na_, 0.0);
    s.aer_abs.assign((size_t)ndh * na_ * nb, 0.0);
    s.aer_scat.assign((size_t)ndh * na_ * nb, 0.0);
    s.aer_phf.assign((size_t)ndh * ndf * na_ * nb, 0.0);
    for (const auto &kv : found) {
      const int j = kv.first - 1;
      const Species &sp = kv.second;
      s.aer_nphf[j] = sp.nphf;
      s.aer_nhum[j] = sp.moist ? sp.rows : 0;
      s.aer_parm[j] = sp.moist ? (sp.nphf == 1 ? SOCGPU_IP_AEROSOL_PARAM_MOIST : SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST)
                               : (sp.nphf == 1 ? SOCGPU_IP_AEROSOL_PARAM_DRY : SOCGPU_IP_AEROSOL_PARAM_PHF_DRY);
      const int per = 3 + sp.nphf;
      for (int b = 0; b < nb; ++b)
        for (int h = 0; h < sp.rows; ++h) {
          const double *r = &sp.v[((size_t)b * sp.rows + h) * per];
          const size_t q = (size_t)h + (size_t)ndh * ((size_t)j + (size_t)na_ * b);
          if (sp.moist) s.aer_hum[(size_t)h + (size_t)ndh * j] = r[0];
          s.aer_abs[q] = r[1];
          s.aer_scat[q] = r[2];
          for (int m = 0; m < sp.nphf; ++m)
            s.aer_phf[(size_t)h + (size_t)ndh * ((size_t)m + (size_t)ndf * ((size_t)j + (size_t)na_ * b))] = r[3 + m];
        }
    }
  }
  sf = std::move(s);
  return true;
}

}  // namespace socgpu

using namespace socgpu;

extern "C" int socgpu_spectrum_load(const char *name, const char *path, socgpu_spectrum_handle *handle, char *msg,
                                    size_t msg_len) {
  return socgpu_spectrum_load_ext(name, path, nullptr, nullptr, handle, msg, msg_len);
}

extern "C" int socgpu_spectrum_load_ext(const char *name, const char *path, const char *k_path,
                                        const char *wenyi_path, socgpu_spectrum_handle *handle, char *msg,
                                        size_t msg_len) {
  if (!name || !path || !handle) { set_msg(msg, msg_len, "null argument"); return SOCGPU_I_ERR_FATAL; }
  SpectralFile sf;
  std::string err;
  if (!read_spectral_file(path, k_path ? k_path : "", wenyi_path ? wenyi_path : "", sf, err)) {
    set_msg(msg, msg_len, "%s", err.c_str());
    return SOCGPU_I_ERR_IO;
  }
  socgpu_spectrum_desc d = sf.desc();
  return socgpu_spectrum_register(name, &d, handle, msg, msg_len);
}
