// run_main.cpp -- socgpu_run: the reference's Cl_run_cdf / Cl_run_cdl column
// driver (src/aux/l_run_cdf.F90, l_run_cdl.F90; options of sbin/Cl_run_cdl)
// over the socgpu C-ABI.  Inputs are <base>.<suffix> files in netCDF classic
// or CDL form; outputs are written in the form of the temperature file.
//
//   socgpu_run -s <spectral file> -R <first band> <last band> (-I | -S) -B <base>
//              [-g <gas overlap>] [-c] [-r] [+R] [-q] [-t <two-stream scheme>]
//              [-v <solver>] [-C <cloud scheme>] [-z <scatter method>]
//              [-ds <direct tau>] [-P fp64|mixed] [-W <Wen-Yi tables file>]
//              [-C 10 -K <cloud representation> -d <droplet type> -i <ice type>
//               -m <condensate relative std. deviation> +m <sampling> -dp <decorrelation scale>]
//              [-C 6 -K 3|4 -d <droplet type> -i <ice type> +d <convective droplet type>
//               +i <convective ice type>]
//              [-C 7 | -C 8 (partially correlated regions) -dp <stratiform decorrelation scale>
//               +dp <convective decorrelation scale>]
//              [-a [+A]]
//   socgpu_run --convert <in> <out.cdf|out.cdl>
//
// Inputs: .t (layer temperatures on the layer pressures `plev`), .tl (level
// temperatures on the level pressures), optional .p and .pl (pressures per
// column), one file per absorber of the spectral file (suffixes of
// gas_list_pcf.F90: q, co2, o3, ...; an absent file means none of that
// gas), .tstar (infra-red), .szen and .stoa (solar), .surf (albedo weights).
// Outputs: .uflx, .dflx, .nflx, .hrts, and in the solar .vflx (direct) and
// .sflx (diffuse down).  The two-stream path is driven clear (-C 5), with
// clouds in a clear and a cloudy region (-C 2 maximum-random, -C 4 random
// overlap; solver 16 unless -v 11) or with McICA (-C 10): clouds of one
// homogeneous type (-K 1: .clfr) or of water and
// ice types (-K 2: .wclfr, .iclfr), droplets from .lwm and .re with the
// spectral file's droplet type -d, ice from .iwm and .ire with ice type -i
// (input_cloud_cdf.f:340-790), and the subcolumns of set_cld_mcica from the
// McICA data file beside the spectral file (l_run_cdf.F90:998-1010,
// 1281-1296).  Three regions (-C 6, solver 17 unless -v is given) take
// stratiform and convective cloud: -K 3 with .clfr and .ccfr, or -K 4 with
// .wclfr, .iclfr, .wccfr and .iccfr; convective droplets from .lwmcv and
// .recv (type +d), convective ice from .iwmcv and .irecv (type +i).
// 1281-1296).  With -a the spectral file's aerosol species are included:
// mixing ratios from <base>.<species suffix> (wtsol, dust, ocn, soot, ...;
// none without a file) and, with +A, prescribed optical properties from
// <base>.op_<species suffix> in place of the species' parametrization.
// Moist species take the clear-sky mean relative humidity of the layers.
// Lookup tables are read from the spectral file's '_k' companion; spectral
// files with Wen-Yi CO2 terms (GA7 and GA9 long wave) need -W, the data file
// of those tables (the reference compiles them in; socrates_gb300/wenyi.py
// converts them from a SOCRATES source tree once).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../../include/socgpu.h"
#include "cdf_io.h"
#include "mcica_setup.h"

using socgpu::McicaData;
using socgpu::McicaState;
using socgpu::NcFile;
using socgpu::NcVar;
using socgpu::read_mcica_data;
using socgpu::set_cld_mcica;

namespace {

// physical constants (rad_ccf.F90:42-58, gas_list_pcf.F90:303)
const double kGrav = 9.80665, kRGasDry = 287.026, kMolWeightAir = 28.966e-03, kCpAirDry = 1.005e+03;
const double kMolarWeightH2O = 18.0153;

const char *gas_suffix(int type) {
  static const char *s[] = {"",       "q",      "co2",    "o3",      "n2o",    "co",   "ch4",  "o2",
                            "no",     "so2",    "no2",    "nh3",     "hno3",   "n2",   "cfc11", "cfc12",
                            "cfc113", "hcfc22", "hfc125", "hfc134a", "cfc114", "tio",  "vo",   "h2",
                            "he",     "ocs",    "na",     "k",       "feh",    "crh",  "li",   "rb",
                            "cs",     "ph3",    "c2h2",   "hcn",     "h2s",    "ar"};
  return (type >= 1 && type < (int)(sizeof(s) / sizeof(s[0]))) ? s[type] : nullptr;
}

// File suffixes of the aerosol species by type number (the names
// l_run_cdf's input_aerosol_cdf.f looks for: <base>.<suffix> holds mixing
// ratios, <base>.op_<suffix> prescribed optical properties)
const char *aerosol_suffix(int type) {
  static const char *s[] = {"",         "wtsol",    "dust",     "ocn",      "soot",     "ash",     "sulph",
                            "nh4so4",   "aunch",    "sahara",   "accum",    "aitken",   "frsoot",  "agsoot",
                            "nacl",     "naclflm",  "nacljet",  "dustdiv1", "dustdiv2", "dustdiv3", "dustdiv4",
                            "dustdiv5", "dustdiv6", "bioms1",   "bioms2",   "biogenic", "frocff",  "agocff",
                            "delta",    "",         "nitrate",  "dust2bin1", "dust2bin2"};
  return (type >= 1 && type < (int)(sizeof(s) / sizeof(s[0])) && s[type][0]) ? s[type] : nullptr;
}

// Saturation mixing ratio over water [kg/kg] at temperature t [K] and
// pressure p [Pa]: the Goff-Gratch saturation vapour pressure over a plane
// water surface (WMO), t held to 183.15-338.15 K, times Gill's (1982,
// A4.7) factor for vapour in air, then the mixing ratio with the pressure
// floored at the vapour pressure (the role of qsat_wat.F90 in
// set_moist_aerosol_properties.F90; that routine interpolates a 0.1 K table
// of the same formula instead).
double qsat_water(double t, double p) {
  const double ts = 373.16, tt = std::min(std::max(t, 183.15), 338.15);
  const double r = ts / tt;
  const double log10_hpa = -7.90298 * (r - 1.0) + 5.02808 * std::log10(r) -
                           1.3816e-7 * (std::pow(10.0, 11.344 * (1.0 - 1.0 / r)) - 1.0) +
                           8.1328e-3 * (std::pow(10.0, -3.49149 * (r - 1.0)) - 1.0) + std::log10(1013.246);
  const double fsubw = 1.0 + 1.0e-8 * p * (4.5 + 6.0e-4 * (t - 273.15) * (t - 273.15));
  const double e = 100.0 * std::pow(10.0, log10_hpa) * fsubw;
  const double eps = kMolarWeightH2O * 1.0e-03 / kMolWeightAir;
  return eps * e / (std::max(p, e) - (1.0 - eps) * e);
}

int die(const std::string &m) {
  std::fprintf(stderr, "socgpu_run: %s\n", m.c_str());
  return 1;
}

bool exists(const std::string &p) {
  FILE *f = std::fopen(p.c_str(), "rb");
  if (f) std::fclose(f);
  return f != nullptr;
}

// The one field of a column file, mapped to (profile, level) with
// profiles enumerated latitude-major over the (lat, lon) grid.
struct Field {
  size_t n_lat = 1, n_lon = 1, n_lev = 1;
  std::vector<double> coord;   // the vertical coordinate (plev), if any
  std::vector<double> v;       // v[l + n_prof * k]
  size_t n_prof() const { return n_lat * n_lon; }
};

bool read_field(const std::string &path, Field &out, std::string &err) {
  NcFile f;
  if (!socgpu::read_nc(path, f, err)) return false;
  const NcVar *var = nullptr;
  for (const NcVar &v : f.vars)
    if (v.name != "lat" && v.name != "lon" && v.name != "plev" && v.name != "basis" && v.name != "band") var = &v;
  if (!var) { err = path + ": no data variable"; return false; }
  Field r;
  int ilat = -1, ilon = -1, ilev = -1;
  std::vector<size_t> len(var->dims.size()), stride(var->dims.size(), 1);
  for (size_t d = 0; d < var->dims.size(); ++d) {
    const std::string &dn = f.dims[var->dims[d]].first;
    len[d] = f.dims[var->dims[d]].second;
    if (dn == "lat") ilat = (int)d;
    else if (dn == "lon") ilon = (int)d;
    else ilev = (int)d;          // plev, basis or band
  }
  for (int d = (int)var->dims.size() - 2; d >= 0; --d) stride[d] = stride[d + 1] * len[d + 1];
  r.n_lat = ilat >= 0 ? len[ilat] : 1;
  r.n_lon = ilon >= 0 ? len[ilon] : 1;
  r.n_lev = ilev >= 0 ? len[ilev] : 1;
  if (const NcVar *c = f.var("plev")) r.coord = c->data;
  r.v.resize(r.n_prof() * r.n_lev);
  for (size_t a = 0; a < r.n_lat; ++a)
    for (size_t o = 0; o < r.n_lon; ++o)
      for (size_t k = 0; k < r.n_lev; ++k) {
        size_t at = (ilat >= 0 ? a * stride[ilat] : 0) + (ilon >= 0 ? o * stride[ilon] : 0) +
                    (ilev >= 0 ? k * stride[ilev] : 0);
        if (at >= var->data.size()) { err = path + ": short data"; return false; }
        r.v[(a * r.n_lon + o) + r.n_prof() * k] = var->data[at];
      }
  out = std::move(r);
  return true;
}

// Write one output field (plev, lat, lon) in the reference's layout.
bool write_field(const std::string &path, bool cdf, const std::string &name, const std::string &title,
                 const std::string &units, const std::vector<double> &plev, size_t n_lat, size_t n_lon,
                 const std::vector<double> &v, std::string &err) {
  NcFile f;
  f.name = path.substr(path.find_last_of('/') + 1);
  f.dims = {{"lon", n_lon}, {"lat", n_lat}, {"plev", plev.size()}};
  NcVar lon, lat, pl, d;
  lon.name = "lon"; lon.dims = {0}; lon.data.assign(n_lon, 0.0);
  lon.text_atts = {{"units", "degree"}, {"title", "longitude"}};
  lat.name = "lat"; lat.dims = {1}; lat.data.assign(n_lat, 0.0);
  lat.text_atts = {{"units", "degree"}, {"title", "latitude"}};
  pl.name = "plev"; pl.dims = {2}; pl.data = plev;
  pl.text_atts = {{"units", "pa"}, {"title", "pressure"}};
  d.name = name; d.dims = {2, 1, 0};
  d.text_atts = {{"units", units}, {"title", title}};
  const size_t np = n_lat * n_lon;
  d.data.resize(plev.size() * np);
  for (size_t k = 0; k < plev.size(); ++k)
    for (size_t l = 0; l < np; ++l) d.data[k * np + l] = v[l + np * k];
  f.vars = {lon, lat, pl, d};
  return cdf ? socgpu::write_cdf(path, f, err) : socgpu::write_cdl(path, f, err);
}

// Blocks 10 and 12 of a spectral file: the scheme and range of validity of
// each droplet or ice type (read_spectrum.F90 read_block_10_0_2 and 12_0_2).
struct CloudTypeInfo {
  int scheme = 0;
  double lo = 0.0, hi = 0.0;
};

bool read_cloud_types(const std::string &path, std::map<int, CloudTypeInfo> &drop,
                      std::map<int, CloudTypeInfo> &ice) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) return false;
  char line[512];
  int blk = -1, type = 0;
  CloudTypeInfo cur;
  auto flush = [&]() {
    if ((blk == 10 || blk == 12) && type > 0) (blk == 10 ? drop : ice)[type] = cur;
    type = 0;
    cur = CloudTypeInfo{};
  };
  while (std::fgets(line, sizeof(line), f)) {
    std::string s(line), u = s;
    for (char &c : u) c = (char)std::toupper((unsigned char)c);
    if (s.rfind("*BLOCK", 0) == 0) {
      flush();
      const size_t e = s.find('=');
      blk = e == std::string::npos ? -1 : std::atoi(s.c_str() + e + 1);
      continue;
    }
    if (s.rfind("*END", 0) == 0) { flush(); blk = -1; continue; }
    if (blk != 10 && blk != 12) continue;
    const size_t e = s.find('=');
    if (e == std::string::npos) continue;
    if (u.find("TYPE NUMBER") != std::string::npos) type = std::atoi(s.c_str() + e + 1);
    else if (u.find("PARAMETRIZATION SCHEME") != std::string::npos) cur.scheme = std::atoi(s.c_str() + e + 1);
    else if (u.find("RANGE OF VALIDITY") != std::string::npos) {
      const size_t dd = s.find("--", e);
      if (dd != std::string::npos) {
        cur.lo = std::strtod(s.c_str() + e + 1, nullptr);
        cur.hi = std::strtod(s.c_str() + dd + 2, nullptr);
      }
    }
  }
  flush();
  std::fclose(f);
  return true;
}

// The McICA data file (read_mcica_data, def_mcica.F90): keyword records of
// the *DATA block, each followed by its values.
}  // namespace

int main(int argc, char **argv) {
  std::vector<std::string> a(argv + 1, argv + argc);
  if (a.size() == 3 && a[0] == "--convert") {
    NcFile f;
    std::string err;
    if (!socgpu::read_nc(a[1], f, err)) return die(err);
    const bool to_cdf = a[2].size() > 4 && a[2].compare(a[2].size() - 4, 4, ".cdf") == 0;
    if (!(to_cdf ? socgpu::write_cdf(a[2], f, err) : socgpu::write_cdl(a[2], f, err))) return die(err);
    return 0;
  }
  std::string sp_file, base, wenyi_file;   // -W: the Wen-Yi tables' data file
  int first = 0, last = 0, isolir = 0, overlap = 0, two_stream = 0, solver = 0, cloud = SOCGPU_IP_CLOUD_CLEAR;
  int scatter = SOCGPU_IP_SCATTER_FULL, direct_tau = SOCGPU_IP_DIRECT_DELTA_SCALING;
  bool cont = false, rayleigh = false, rescale = false, quad = false, gas = false;
  int precision = SOCGPU_PRECISION_FP64;
  // clouds (-K, -d, -i) and McICA (-m, +m, -dp)
  int representation = 0, drop_type = 0, ice_type = 0, sampling = 2;
  int conv_drop_type = 0, conv_ice_type = 0;   // +d, +i: convective particles (three regions)
  bool aerosol = false, overlay = false;   // -a: classic aerosols; +A: overlay of optical properties
  double mcica_sigma = 0.0, dp_corr_strat = 0.0, dp_corr_conv = 0.0;
  for (size_t i = 0; i < a.size(); ++i) {
    const std::string &o = a[i];
    auto need = [&](size_t n) { return i + n < a.size(); };
    if (o == "-s" && need(1)) sp_file = a[++i];
    else if (o == "-W" && need(1)) wenyi_file = a[++i];
    else if (o == "-B" && need(1)) base = a[++i];
    else if (o == "-R" && need(2)) { first = std::atoi(a[i + 1].c_str()); last = std::atoi(a[i + 2].c_str()); i += 2; }
    else if (o == "-I") isolir = SOCGPU_IP_INFRA_RED;
    else if (o == "-S") isolir = SOCGPU_IP_SOLAR;
    else if (o == "-g" && need(1)) { gas = true; overlap = std::atoi(a[++i].c_str()); }
    else if (o == "-c") cont = true;
    else if (o == "-r") rayleigh = true;
    else if (o == "-a") aerosol = true;
    else if (o == "+A") overlay = true;
    else if (o == "+R") rescale = true;
    else if (o == "-q") quad = true;
    else if (o == "-t" && need(1)) two_stream = std::atoi(a[++i].c_str());
    else if (o == "-v" && need(1)) solver = std::atoi(a[++i].c_str());
    else if (o == "-C" && need(1)) cloud = std::atoi(a[++i].c_str());
    else if (o == "-z" && need(1)) scatter = std::atoi(a[++i].c_str());
    else if (o == "-ds" && need(1)) direct_tau = std::atoi(a[++i].c_str());
    else if (o == "-K" && need(1)) representation = std::atoi(a[++i].c_str());
    else if (o == "-d" && need(1)) drop_type = std::atoi(a[++i].c_str());
    else if (o == "-i" && need(1)) ice_type = std::atoi(a[++i].c_str());
    else if (o == "+d" && need(1)) conv_drop_type = std::atoi(a[++i].c_str());
    else if (o == "+i" && need(1)) conv_ice_type = std::atoi(a[++i].c_str());
    else if (o == "-m" && need(1)) mcica_sigma = std::atof(a[++i].c_str());
    else if (o == "+m" && need(1)) sampling = std::atoi(a[++i].c_str());
    else if (o == "-dp" && need(1)) dp_corr_strat = std::atof(a[++i].c_str());
    else if (o == "+dp" && need(1)) dp_corr_conv = std::atof(a[++i].c_str());
    else if (o == "-P" && need(1)) {
      std::string p = a[++i];
      precision = (p == "mixed") ? SOCGPU_PRECISION_MIXED : SOCGPU_PRECISION_FP64;
    } else return die("unknown or incomplete option " + o);
  }
  if (sp_file.empty()) return die("Spectral file not set.");
  if (base.empty()) return die("Base name not set.");
  if (!isolir) return die("Spectral region not set.");
  if (first < 1 || last < first) return die("Range of bands not set");
  if (overlay && !aerosol) return die("+A overlays aerosol optical properties: it needs -a");
  const bool triple = cloud == SOCGPU_IP_CLOUD_TRIPLE || cloud == SOCGPU_IP_CLOUD_PART_CORR_CNV;
  const bool region = cloud == SOCGPU_IP_CLOUD_MIX_MAX || cloud == SOCGPU_IP_CLOUD_MIX_RANDOM ||
                      cloud == SOCGPU_IP_CLOUD_PART_CORR || triple;
  if (cloud != SOCGPU_IP_CLOUD_CLEAR && cloud != SOCGPU_IP_CLOUD_MCICA && !region)
    return die("cloud scheme " + std::to_string(cloud) +
               " is not driven (clear sky -C 5, cloud regions -C 2, 4 or 7, three regions -C 6 or 8, McICA -C 10)");
  const bool mcica = cloud == SOCGPU_IP_CLOUD_MCICA;
  const bool clouds = mcica || region;
  const bool conv = representation == SOCGPU_IP_CLOUD_CONV_STRAT || representation == SOCGPU_IP_CLOUD_CSIW;
  if (clouds && !triple && representation != 1 && representation != SOCGPU_IP_CLOUD_ICE_WATER)
    return die("clouds need the cloud representation -K 1 (homogeneous) or -K 2 (ice and water)");
  if (triple && !conv)
    return die("three regions need the cloud representation -K 3 (convective and stratiform) or -K 4 "
               "(convective and stratiform ice and water)");
  if (clouds && !drop_type && !ice_type) return die("Clouds are specified, but no cloudy processes are included.");
  // sbin/Cl_run_cdf:218-260: a convective type for each stratiform process
  if (conv && ((drop_type && !conv_drop_type) || (ice_type && !conv_ice_type)))
    return die("Types of convective particles have not been set.");
  if (mcica && (sampling < 0 || sampling > 2)) return die("The value of i_mcica_sampling is not valid.");
  if (!two_stream) two_stream = isolir == SOCGPU_IP_INFRA_RED ? 12 : 16;
  // the solver Cl_run_cdf picks for the cloud scheme (sbin/Cl_run_cdf:293-310)
  if (!solver)
    solver = triple ? SOCGPU_IP_SOLVER_TRIPLE_HOGAN : region ? SOCGPU_IP_SOLVER_MIX_DIRECT_HOGAN
                    : scatter == SOCGPU_IP_SCATTER_FULL ? SOCGPU_IP_SOLVER_HOMOGEN_DIRECT : SOCGPU_IP_SOLVER_NO_SCAT;

  char msg[512] = "";
  socgpu_spectrum_handle h = 0;
  int st = socgpu_spectrum_load_ext(sp_file.c_str(), sp_file.c_str(), nullptr,
                                    wenyi_file.empty() ? nullptr : wenyi_file.c_str(), &h, msg, sizeof(msg));
  if (st != SOCGPU_I_NORMAL) return die(msg);

  // the spectral file's absorbers (for the gas files)
  std::string err;
  Field t, tl;
  const std::string t_path = base + ".t";
  if (!read_field(t_path, t, err) || !read_field(base + ".tl", tl, err)) return die(err);
  bool cdf_out = false;
  {
    FILE *f = std::fopen(t_path.c_str(), "rb");
    char m[3] = {0, 0, 0};
    if (f) { cdf_out = std::fread(m, 1, 3, f) == 3 && m[0] == 'C' && m[1] == 'D' && m[2] == 'F'; std::fclose(f); }
  }
  const size_t np = t.n_prof(), nl = t.n_lev;
  if (tl.n_prof() != np || tl.n_lev != nl + 1) return die("levels of .tl do not bracket the layers of .t");
  std::vector<double> p(np * nl), p_level(np * (nl + 1));
  Field pf, plf;
  if (exists(base + ".p")) {
    if (!read_field(base + ".p", pf, err)) return die(err);
    p = pf.v;
  } else {
    if (t.coord.size() != nl) return die(".t has no pressure coordinate");
    for (size_t k = 0; k < nl; ++k)
      for (size_t l = 0; l < np; ++l) p[l + np * k] = t.coord[k];
  }
  if (exists(base + ".pl")) {
    if (!read_field(base + ".pl", plf, err)) return die(err);
    p_level = plf.v;
  } else {
    if (tl.coord.size() != nl + 1) return die(".tl has no pressure coordinate");
    for (size_t k = 0; k <= nl; ++k)
      for (size_t l = 0; l < np; ++l) p_level[l + np * k] = tl.coord[k];
  }
  // the band count and absorber list of the spectral file (its summary block)
  std::vector<int> types;
  int n_band = 0;
  {
    FILE *f = std::fopen(sp_file.c_str(), "r");
    if (!f) return die("cannot open " + sp_file);
    char line[512];
    int n_abs = 0;
    bool in0 = false, list = false;
    while (std::fgets(line, sizeof(line), f)) {
      std::string s(line);
      if (s.rfind("*BLOCK", 0) == 0) { in0 = s.find("TYPE =    0") != std::string::npos; continue; }
      if (s.rfind("*END", 0) == 0) { if (in0) break; continue; }
      if (!in0) continue;
      std::string u = s;
      for (char &c : u) c = (char)std::toupper((unsigned char)c);
      if (u.find("SPECTRAL BANDS") != std::string::npos) n_band = std::atoi(s.c_str() + s.find('=') + 1);
      else if (u.find("GASEOUS ABSORBERS") != std::string::npos) n_abs = std::atoi(s.c_str() + s.find('=') + 1);
      else if (u.find("INDEXING NUMBERS") != std::string::npos && u.find("ABSORBER") != std::string::npos &&
               u.find("AEROSOL") == std::string::npos) list = true;
      else if (list && (int)types.size() < n_abs) {
        int idx = 0, ty = 0;
        if (std::sscanf(line, "%d %d", &idx, &ty) == 2) types.push_back(ty);
      }
    }
    std::fclose(f);
  }
  const size_t ns = std::max<size_t>(1, types.size());
  std::vector<double> gas_mr(np * nl * ns, 0.0);
  int i_water = -1;
  for (size_t j = 0; j < types.size(); ++j) {
    if (types[j] == 1) i_water = (int)j;
    const char *suf = gas_suffix(types[j]);
    std::string path = suf ? base + "." + suf : "";
    if (path.empty() || !exists(path)) {
      std::fprintf(stderr, "socgpu_run: no file for absorber type %d: taken as absent\n", types[j]);
      continue;
    }
    Field g;
    if (!read_field(path, g, err)) return die(err);
    if (g.n_prof() != np || g.n_lev != nl) return die(path + ": not on the layers of .t");
    for (size_t q = 0; q < np * nl; ++q) gas_mr[q + np * nl * j] = g.v[q];
  }
  // layer mass and density (l_run_cdl.F90:1017-1045)
  std::vector<double> mass(np * nl), density(np * nl), t_level = tl.v;
  for (size_t k = 0; k < nl; ++k)
    for (size_t l = 0; l < np; ++l) {
      const size_t q = l + np * k;
      mass[q] = (p_level[l + np * (k + 1)] - p_level[l + np * k]) / kGrav;
      const double w = i_water >= 0 ? gas_mr[q + np * nl * (size_t)i_water] : 0.0;
      density[q] = i_water >= 0 ? p[q] / (kRGasDry * t.v[q] * (1.0 + (kMolWeightAir / (kMolarWeightH2O * 1.0e-03) - 1.0) * w))
                                : p[q] / (kRGasDry * t.v[q]);
    }
  // boundary: rho_alb (nd_profile, 2, n_band) over all bands of the file
  if (last > n_band) return die("band range beyond the spectral file's bands");
  const int nb_total = n_band;
  std::vector<double> rho_alb(np * 2 * (size_t)nb_total, 0.0), t_ground(np, 0.0), zen_0(np, 1.0), irrad(np, 0.0);
  if (exists(base + ".surf")) {
    // albedo weights per basis function, and per band where the file has a
    // band dimension (assign_surface_char_cdf.f:150-350): in the two-stream
    // the first is the diffuse albedo and the second the direct one, which
    // is the diffuse one when only one is given
    NcFile sfile;
    if (!socgpu::read_nc(base + ".surf", sfile, err)) return die(err);
    const NcVar *alb = sfile.var("alb");
    if (!alb) return die(base + ".surf: no variable alb");
    size_t len[4] = {1, 1, 1, 1}, stride[4] = {0, 0, 0, 0};
    int id[4] = {-1, -1, -1, -1};    // lat, lon, basis, band
    for (size_t q = 0; q < alb->dims.size(); ++q) {
      const std::string &dn = sfile.dims[alb->dims[q]].first;
      // a dimension whose name starts with "band" (assign_surface_char_cdf.f:213-218)
      const int k = dn == "lat" ? 0 : dn == "lon" ? 1 : dn == "basis" ? 2 : dn.compare(0, 4, "band") == 0 ? 3 : -1;
      if (k < 0) return die(base + ".surf: unexpected dimension " + dn);
      id[k] = (int)q;
      len[k] = sfile.dims[alb->dims[q]].second;
    }
    if (id[2] < 0 || len[2] < 1 || len[2] > 2) return die(base + ".surf: one or two basis functions expected");
    if (id[3] >= 0 && (int)len[3] != nb_total) return die(base + ".surf: band dimension differs from the spectral file");
    if (len[0] * len[1] != np) return die(base + ".surf: not on the columns of .t");
    std::vector<size_t> dstride(alb->dims.size(), 1);
    for (int q = (int)alb->dims.size() - 2; q >= 0; --q)
      dstride[q] = dstride[q + 1] * sfile.dims[alb->dims[q + 1]].second;
    for (int k = 0; k < 4; ++k) stride[k] = id[k] >= 0 ? dstride[id[k]] : 0;
    for (size_t a = 0; a < len[0]; ++a)
      for (size_t o = 0; o < len[1]; ++o) {
        const size_t l = a * len[1] + o;
        for (int b = 0; b < nb_total; ++b)
          for (int k = 0; k < 2; ++k) {
            const size_t basis = std::min<size_t>((size_t)k, len[2] - 1);
            const size_t at = a * stride[0] + o * stride[1] + basis * stride[2] + (size_t)b * stride[3];
            if (at >= alb->data.size()) return die(base + ".surf: short data");
            rho_alb[l + np * ((size_t)k + 2 * (size_t)b)] = alb->data[at];
          }
      }
  }
  if (isolir == SOCGPU_IP_INFRA_RED) {
    Field ts;
    if (!read_field(base + ".tstar", ts, err)) return die(err);
    t_ground = ts.v;
  } else {
    Field sz, so;
    if (!read_field(base + ".szen", sz, err) || !read_field(base + ".stoa", so, err)) return die(err);
    for (size_t l = 0; l < np; ++l) {
      zen_0[l] = 1.0 / std::cos(sz.v[l] * std::acos(-1.0) / 180.0);   // secant of the zenith angle
      irrad[l] = so.v[l];
    }
  }

  // clouds and McICA (input_cloud_cdf.f:340-790; l_run_cdf.F90:1281-1296 with
  // socrates_set_cld_mcica.F90:82-228)
  int nc = 0, n_cloud_type = 1;
  std::vector<int> type_condensed, i_cloud_type, i_condensed_param, i_condensed_type;
  std::vector<double> cmr, dim, w_cloud, frac_cloud;
  McicaState mst;
  if (clouds) {
    std::map<int, CloudTypeInfo> drops, ices;
    if (!read_cloud_types(sp_file, drops, ices)) return die("cannot open " + sp_file);
    // components in the order of input_cloud_cdf.f (stratiform water and
    // ice, then convective water and ice) with their ip_clcmp codes and the
    // cloud type of each under the representation (input_cloud_cdf.f:640-760)
    struct Comp { int clcmp, phase, type, cloud_type; const char *mr, *dim; };
    std::vector<Comp> comps;
    const bool csiw = representation == SOCGPU_IP_CLOUD_CSIW;
    if (drop_type)
      comps.push_back({SOCGPU_IP_CLCMP_ST_WATER, SOCGPU_IP_PHASE_WATER, drop_type, 1, "lwm", "re"});
    if (ice_type)
      comps.push_back({SOCGPU_IP_CLCMP_ST_ICE, SOCGPU_IP_PHASE_ICE, ice_type,
                       representation == 1 || representation == SOCGPU_IP_CLOUD_CONV_STRAT ? 1 : 2, "iwm", "ire"});
    if (conv && drop_type)
      comps.push_back({SOCGPU_IP_CLCMP_CNV_WATER, SOCGPU_IP_PHASE_WATER, conv_drop_type, csiw ? 3 : 2, "lwmcv", "recv"});
    if (conv && ice_type)
      comps.push_back({SOCGPU_IP_CLCMP_CNV_ICE, SOCGPU_IP_PHASE_ICE, conv_ice_type, csiw ? 4 : 2, "iwmcv", "irecv"});
    nc = (int)comps.size();
    n_cloud_type = representation == 1 ? 1 : csiw ? 4 : 2;
    cmr.assign(np * nl * nc, 0.0);
    dim.assign(np * nl * nc, 0.0);
    for (int k = 0; k < nc; ++k) {
      const Comp &cp = comps[k];
      auto &tab = cp.phase == SOCGPU_IP_PHASE_WATER ? drops : ices;
      auto it = tab.find(cp.type);
      if (it == tab.end() || it->second.scheme == 0)
        return die(std::string(cp.phase == SOCGPU_IP_PHASE_WATER ? "droplet" : "ice") + " type " +
                   std::to_string(cp.type) + " is not in the spectral file");
      type_condensed.push_back(cp.clcmp);
      i_cloud_type.push_back(cp.cloud_type);
      i_condensed_param.push_back(it->second.scheme);
      i_condensed_type.push_back(cp.type);
      Field fm, fd;
      if (!read_field(base + "." + cp.mr, fm, err) || !read_field(base + "." + cp.dim, fd, err)) return die(err);
      if (fm.n_prof() != np || fm.n_lev != nl || fd.n_prof() != np || fd.n_lev != nl)
        return die(std::string(cp.mr) + "/" + cp.dim + ": not on the layers of .t");
      for (size_t q = 0; q < np * nl; ++q) {
        cmr[q + np * nl * k] = fm.v[q];
        dim[q + np * nl * k] = std::min(std::max(fd.v[q], it->second.lo), it->second.hi);
      }
    }
    // cloud fractions of each type, normalised by their sum (input_cloud_cdf.f:760-790)
    const char *frac_suffix[4] = {representation == 1 ? "clfr" : "wclfr", "iclfr", "wccfr", "iccfr"};
    if (representation == SOCGPU_IP_CLOUD_CONV_STRAT) { frac_suffix[0] = "clfr"; frac_suffix[1] = "ccfr"; }
    frac_cloud.assign(np * nl * n_cloud_type, 0.0);
    w_cloud.assign(np * nl, 0.0);
    for (int t2 = 0; t2 < n_cloud_type; ++t2) {
      Field ff;
      if (!read_field(base + "." + frac_suffix[t2], ff, err)) return die(err);
      if (ff.n_prof() != np || ff.n_lev != nl) return die(std::string(frac_suffix[t2]) + ": not on the layers of .t");
      for (size_t q = 0; q < np * nl; ++q) frac_cloud[q + np * nl * t2] = ff.v[q];
    }
    for (size_t q = 0; q < np * nl; ++q) {
      for (int t2 = 0; t2 < n_cloud_type; ++t2) w_cloud[q] += frac_cloud[q + np * nl * t2];
      if (w_cloud[q] > 0.0)
        for (int t2 = 0; t2 < n_cloud_type; ++t2) frac_cloud[q + np * nl * t2] /= w_cloud[q];
    }
  }
  if (mcica) {
    // McICA data beside the spectral file, then set_cld_mcica
    const size_t slash = sp_file.find_last_of('/');
    const std::string mcica_path = (slash == std::string::npos ? std::string() : sp_file.substr(0, slash + 1)) +
                                   "mcica_data";
    McicaData md;
    if (!read_mcica_data(mcica_path, md, err)) return die(err);
    // the generator's inputs: condensate variability weighted by the
    // grid-box condensate, decorrelation scales, seeds 10 + profile
    std::vector<double> cond_rsd(np * nl);
    const double eps = std::numeric_limits<double>::epsilon();
    for (size_t q = 0; q < np * nl; ++q) {
      double num = 0.0, den = 0.0;
      for (int k = 0; k < nc; ++k) {
        const double wgt = std::max(eps, cmr[q + np * nl * k] * frac_cloud[q + np * nl * (i_cloud_type[k] - 1)]);
        num += mcica_sigma * wgt;
        den += wgt;
      }
      cond_rsd[q] = num / den;
    }
    std::vector<int> seeds(np);
    for (size_t l = 0; l < np; ++l) seeds[l] = 10 + (int)l + 1;
    st = set_cld_mcica(h, md, isolir, sampling, SOCGPU_IP_EXPONENTIAL, first, last, (int)np, (int)nl, 1,
                       seeds.data(), dp_corr_strat, cond_rsd.data(), w_cloud.data(), p.data(), mst, msg,
                       sizeof(msg));
    if (st != SOCGPU_I_NORMAL) return die(msg);
  }
  // classic aerosols (-a; l_run_cdf.F90:847-920 with input_aerosol_cdf.f):
  // for each species of the spectral file, with +A a file of optical
  // properties <base>.op_<suffix> overlays it (the species becomes
  // unparametrized), otherwise its mixing ratios come from <base>.<suffix>
  // (none without a file); moist species need the clear-sky mean relative
  // humidity (set_moist_aerosol_properties.F90)
  int n_aer = 0, nd_lev_prsc = 1, nd_mom_prsc = 1;
  std::vector<int> aer_type, aer_parm, aer_nhum, mr_index, mr_source, nlev_prsc, nmom_prsc;
  std::vector<double> aer_mr, mrh, p_prsc, abs_prsc, scat_prsc, phf_prsc;
  if (aerosol) {
    if (socgpu_spectrum_aerosols(h, 0, &n_aer, nullptr, nullptr, nullptr) != SOCGPU_I_NORMAL || n_aer < 1)
      return die("The spectral file contains no aerosol data.");
    aer_type.resize(n_aer); aer_parm.resize(n_aer); aer_nhum.resize(n_aer);
    socgpu_spectrum_aerosols(h, n_aer, &n_aer, aer_type.data(), aer_parm.data(), aer_nhum.data());
    aer_mr.assign(np * nl * (size_t)n_aer, 0.0);
    nlev_prsc.assign(n_aer, 1);
    nmom_prsc.assign(n_aer, 1);
    struct Opt { size_t nlev, nmom; std::vector<double> lev, ab, sc, ph; };   // ab, sc: (band, lev, profile)
    std::map<int, Opt> opt;
    for (int i = 0; i < n_aer; ++i) {
      const char *suf = aerosol_suffix(aer_type[i]);
      if (!suf) continue;
      const std::string op_path = base + ".op_" + suf;
      if (overlay && exists(op_path)) {
        // assign_input_opt_cdf.f: abs and scat (band, plev, lat, lon), phf
        // (band, mom, plev, lat, lon) on the pressures of plev
        NcFile f;
        if (!socgpu::read_nc(op_path, f, err)) return die(err);
        const NcVar *va = f.var("abs"), *vs = f.var("scat"), *vp = f.var("phf"), *lev = f.var("plev");
        const size_t nlev = f.dim_len("plev"), nmom = std::max<size_t>(1, f.dim_len("mom"));
        if (!va || !vs || !vp || !lev || nlev < 1) return die(op_path + ": abs, scat, phf and plev expected");
        auto dims_are = [&](const NcVar *v, std::vector<std::string> want) {
          if (v->dims.size() != want.size()) return false;
          for (size_t q = 0; q < want.size(); ++q)
            if (f.dims[v->dims[q]].first != want[q]) return false;
          return true;
        };
        if (!dims_are(va, {"band", "plev", "lat", "lon"}) || !dims_are(vs, {"band", "plev", "lat", "lon"}) ||
            !dims_are(vp, {"band", "mom", "plev", "lat", "lon"}))
          return die(op_path + ": dimensions (band, [mom,] plev, lat, lon) expected");
        if ((int)f.dim_len("band") != nb_total) return die(op_path + ": band dimension differs from the spectral file");
        if (f.dim_len("lat") * std::max<size_t>(1, f.dim_len("lon")) != np) return die(op_path + ": not on the columns of .t");
        for (size_t k = 1; k < nlev; ++k)
          if (!(lev->data[k] > lev->data[k - 1])) return die(op_path + ": pressures must increase");
        if (va->data.size() != (size_t)nb_total * nlev * np || vs->data.size() != va->data.size() ||
            vp->data.size() != (size_t)nb_total * nmom * nlev * np)
          return die(op_path + ": short data");
        Opt o{nlev, nmom, lev->data, va->data, vs->data, vp->data};
        opt[i] = std::move(o);
        if (socgpu_spectrum_set_aerosol_parm(h, i + 1, SOCGPU_IP_AEROSOL_UNPARAMETRIZED, msg, sizeof(msg)) !=
            SOCGPU_I_NORMAL)
          return die(msg);
        aer_parm[i] = SOCGPU_IP_AEROSOL_UNPARAMETRIZED;
        nlev_prsc[i] = (int)nlev;
        nmom_prsc[i] = (int)nmom;
        nd_lev_prsc = std::max(nd_lev_prsc, (int)nlev);
        nd_mom_prsc = std::max(nd_mom_prsc, (int)nmom);
        continue;
      }
      const std::string mr_path = base + "." + suf;
      if (!exists(mr_path)) continue;
      Field fm;
      if (!read_field(mr_path, fm, err)) return die(err);
      if (fm.n_prof() != np || fm.n_lev != nl) return die(mr_path + ": not on the layers of .t");
      for (size_t q = 0; q < np * nl; ++q) aer_mr[q + np * nl * (size_t)i] = fm.v[q];
    }
    for (int i = 0; i < n_aer; ++i) {
      mr_index.push_back(i + 1);
      mr_source.push_back(SOCGPU_IP_AERSRC_CLASSIC_RON);
    }
    if (!opt.empty()) {
      const size_t ndl = (size_t)nd_lev_prsc, ndm = (size_t)nd_mom_prsc, na = (size_t)n_aer, nbt = (size_t)nb_total;
      p_prsc.assign(np * ndl * na, 0.0);
      abs_prsc.assign(np * ndl * na * nbt, 0.0);
      scat_prsc.assign(np * ndl * na * nbt, 0.0);
      phf_prsc.assign(np * ndl * ndm * na * nbt, 0.0);
      for (const auto &kv : opt) {
        const size_t j = (size_t)kv.first;
        const Opt &o = kv.second;
        for (size_t k = 0; k < o.nlev; ++k)
          for (size_t l = 0; l < np; ++l) {
            p_prsc[l + np * (k + ndl * j)] = o.lev[k];
            for (size_t b = 0; b < nbt; ++b) {
              abs_prsc[l + np * (k + ndl * (j + na * b))] = o.ab[(b * o.nlev + k) * np + l];
              scat_prsc[l + np * (k + ndl * (j + na * b))] = o.sc[(b * o.nlev + k) * np + l];
              for (size_t m = 0; m < o.nmom; ++m)
                phf_prsc[l + np * (k + ndl * (m + ndm * (j + na * b)))] = o.ph[((b * o.nmom + m) * o.nlev + k) * np + l];
            }
          }
      }
    }
    bool moist = false;
    for (int i = 0; i < n_aer; ++i)
      moist = moist || aer_parm[i] == SOCGPU_IP_AEROSOL_PARAM_MOIST || aer_parm[i] == SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST;
    if (moist) {
      if (i_water < 0) return die("Water vapour must be included in the spectral file to treat moist aerosols.");
      mrh.assign(np * nl, 0.0);
      for (size_t q = 0; q < np * nl; ++q) {
        const double qw = gas_mr[q + np * nl * (size_t)i_water];
        const double qs = qsat_water(t.v[q], p[q]);
        const double wc = clouds ? w_cloud[q] : 0.0;
        double clr = (qw - wc * qs) / std::max(1.0 - wc, 0.001);
        clr = std::max(std::min(clr, qw), 0.0);
        const double rh = clr * (1.0 - qs) / ((1.0 - clr) * qs);
        mrh[q] = std::max(std::min(rh, 0.99999), 0.0);
      }
    }
  }

  socgpu_control c{};
  c.isolir = isolir;
  c.i_angular_integration = SOCGPU_IP_TWO_STREAM;
  c.i_2stream = two_stream;
  c.i_scatter_method = scatter;
  c.i_solver = solver;
  c.i_cloud = cloud;
  c.i_cloud_representation = representation ? representation : SOCGPU_IP_CLOUD_ICE_WATER;
  c.i_gas_overlap = gas ? overlap : SOCGPU_IP_OVERLAP_RANDOM;
  c.i_direct_tau = direct_tau;
  c.l_rescale = rescale;
  c.n_order_forward = 2;
  c.l_ir_source_quad = quad;
  c.l_rayleigh = rayleigh;
  c.l_gas = gas;
  c.l_flux_div = 0;
  c.first_band = first;
  c.last_band = last;
  c.precision = precision;
  c.l_continuum = cont;
  // two-stream with rescaling: Henyey-Greenstein phase functions
  // (angular_control_cdf.f:236-246)
  c.l_aerosol = aerosol;
  c.l_henyey_greenstein_pf = rescale;
  socgpu_dimen d{};
  d.nd_profile = (int)np;
  d.nd_layer = (int)nl;
  d.id_cloud_top = 1;
  d.nd_aerosol_mode = 1;
  d.nd_cloud_component = std::max(1, nc);
  d.nd_cloud_type = n_cloud_type;
  d.nd_subcol_gen = mcica ? mst.gen : 1;
  d.nd_subcol_req = mcica ? mst.n_subcol_req : 1;
  d.nd_aerosol_mr = std::max(1, n_aer);
  d.nd_profile_aerosol_prsc = p_prsc.empty() ? 1 : (int)np;
  d.nd_opt_level_aerosol_prsc = nd_lev_prsc;
  d.nd_phf_term_aerosol_prsc = nd_mom_prsc;
  socgpu_atm atm{};
  atm.n_profile = (int)np;
  atm.n_layer = (int)nl;
  atm.p = p.data();
  atm.t = t.v.data();
  atm.p_level = p_level.data();
  atm.t_level = t_level.data();
  atm.mass = mass.data();
  atm.gas_mix_ratio = gas_mr.data();
  atm.density = density.data();
  socgpu_bound bd{};
  bd.rho_alb = rho_alb.data();
  if (isolir == SOCGPU_IP_INFRA_RED) bd.t_ground = t_ground.data();
  else { bd.zen_0 = zen_0.data(); bd.solar_irrad = irrad.data(); }
  std::vector<double> up(np * (nl + 1)), down(np * (nl + 1)), direct(np * (nl + 1)), hr(np * nl);
  socgpu_radout out{};
  out.flux_up = up.data();
  out.flux_down = down.data();
  out.flux_direct = isolir == SOCGPU_IP_SOLAR ? direct.data() : nullptr;
  socgpu_aer aer{};
  if (aerosol) {
    aer.n_aerosol_mr = n_aer;
    aer.mix_ratio = aer_mr.data();
    aer.mr_type_index = mr_index.data();
    aer.mr_source = mr_source.data();
    aer.mean_rel_humidity = mrh.empty() ? nullptr : mrh.data();
    if (!p_prsc.empty()) {
      aer.n_opt_level_prsc = nlev_prsc.data();
      aer.n_phase_term_prsc = nmom_prsc.data();
      aer.pressure_prsc = p_prsc.data();
      aer.absorption_prsc = abs_prsc.data();
      aer.scattering_prsc = scat_prsc.data();
      aer.phase_fnc_prsc = phf_prsc.data();
    }
  }
  socgpu_cld cld{};
  if (clouds) {
    cld.n_condensed = nc;
    cld.type_condensed = type_condensed.data();
    cld.i_cloud_type = i_cloud_type.data();
    cld.i_condensed_param = i_condensed_param.data();
    cld.i_condensed_type = i_condensed_type.data();
    cld.condensed_mix_ratio = cmr.data();
    cld.condensed_dim_char = dim.data();
    cld.n_cloud_type = n_cloud_type;
    cld.w_cloud = w_cloud.data();
    cld.frac_cloud = frac_cloud.data();
    // decorrelation scales of like regions (l_run_cdf.F90:984-996: -dp, +dp)
    cld.dp_corr_strat = dp_corr_strat;
    cld.dp_corr_conv = dp_corr_conv;
  }
  if (mcica) mst.attach(cld);
  const auto t0 = std::chrono::steady_clock::now();
  st = socgpu_radiance_calc(&c, &d, h, &atm, &cld, &aer, &bd, &out, msg, sizeof(msg));
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (st != SOCGPU_I_NORMAL) return die(msg);

  // outputs (l_run_cdl.F90:1100-1160): net flux and heating rate in K/day
  std::vector<double> net(np * (nl + 1)), diffuse(np * (nl + 1));
  for (size_t q = 0; q < net.size(); ++q) {
    net[q] = down[q] - up[q];
    diffuse[q] = down[q] - direct[q];
  }
  for (size_t k = 0; k < nl; ++k)
    for (size_t l = 0; l < np; ++l)
      hr[l + np * k] = 8.64e+04 * ((net[l + np * k] - net[l + np * (k + 1)]) / (mass[l + np * k] * kCpAirDry));
  std::vector<double> plev_levels(nl + 1), plev_layers(nl);
  for (size_t k = 0; k <= nl; ++k) plev_levels[k] = p_level[np * k];
  for (size_t k = 0; k < nl; ++k) plev_layers[k] = p[np * k];
  struct Out { const char *suffix, *title, *units; const std::vector<double> *v; bool levels; bool sw_only; };
  const Out outs[] = {
      {"uflx", "upward flux", "WM-2", &up, true, false},
      {"dflx", "total downward flux", "WM-2", &down, true, false},
      {"nflx", "net downward flux", "WM-2", &net, true, false},
      {"hrts", "heating rates", "K.D-1", &hr, false, false},
      {"vflx", "direct flux", "WM-2", &direct, true, true},
      {"sflx", "diffuse downward flux", "WM-2", &diffuse, true, true},
  };
  for (const Out &o : outs) {
    if (o.sw_only && isolir != SOCGPU_IP_SOLAR) continue;
    if (!write_field(base + "." + o.suffix, cdf_out, o.suffix, o.title, o.units, o.levels ? plev_levels : plev_layers,
                     t.n_lat, t.n_lon, *o.v, err))
      return die(err);
  }
  std::fprintf(stderr, "socgpu_run: %zu columns x %zu layers, bands %d-%d, %.3f ms in socgpu_radiance_calc\n", np, nl,
               first, last, ms);
  return 0;
}
