// run_main.cpp -- socgpu_run: the reference's Cl_run_cdf / Cl_run_cdl column
// driver (src/aux/l_run_cdf.F90, l_run_cdl.F90; options of sbin/Cl_run_cdl)
// over the socgpu C-ABI.  Inputs are <base>.<suffix> files in netCDF classic
// or CDL form; outputs are written in the form of the temperature file.
//
//   socgpu_run -s <spectral file> -R <first band> <last band> (-I | -S) -B <base>
//              [-g <gas overlap>] [-c] [-r] [+R] [-q] [-t <two-stream scheme>]
//              [-v <solver>] [-C <cloud scheme>] [-z <scatter method>]
//              [-ds <direct tau>] [-P fp64|mixed] [-W <scale_wenyi source>]
//   socgpu_run --convert <in> <out.cdf|out.cdl>
//
// Inputs: .t (layer temperatures on the layer pressures `plev`), .tl (level
// temperatures on the level pressures), optional .p and .pl (pressures per
// column), one file per absorber of the spectral file (suffixes of
// gas_list_pcf.F90: q, co2, o3, ...; an absent file means none of that
// gas), .tstar (infra-red), .szen and .stoa (solar), .surf (albedo weights).
// Outputs: .uflx, .dflx, .nflx, .hrts, and in the solar .vflx (direct) and
// .sflx (diffuse down).  Only the clear-sky two-stream path is driven.
// Lookup tables are read from the spectral file's '_k' companion; spectral
// files with Wen-Yi CO2 terms (GA7 and GA9 long wave) need -W, the SOCRATES
// source file that defines those tables (the reference compiles them in).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/socgpu.h"
#include "cdf_io.h"

using socgpu::NcFile;
using socgpu::NcVar;

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
  std::string sp_file, base, wenyi_file;   // -W: the Wen-Yi tables (SOCRATES's scale_wenyi source)
  int first = 0, last = 0, isolir = 0, overlap = 0, two_stream = 0, solver = 0, cloud = SOCGPU_IP_CLOUD_CLEAR;
  int scatter = SOCGPU_IP_SCATTER_FULL, direct_tau = SOCGPU_IP_DIRECT_DELTA_SCALING;
  bool cont = false, rayleigh = false, rescale = false, quad = false, gas = false;
  int precision = SOCGPU_PRECISION_FP64;
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
    else if (o == "+R") rescale = true;
    else if (o == "-q") quad = true;
    else if (o == "-t" && need(1)) two_stream = std::atoi(a[++i].c_str());
    else if (o == "-v" && need(1)) solver = std::atoi(a[++i].c_str());
    else if (o == "-C" && need(1)) cloud = std::atoi(a[++i].c_str());
    else if (o == "-z" && need(1)) scatter = std::atoi(a[++i].c_str());
    else if (o == "-ds" && need(1)) direct_tau = std::atoi(a[++i].c_str());
    else if (o == "-P" && need(1)) {
      std::string p = a[++i];
      precision = (p == "mixed") ? SOCGPU_PRECISION_MIXED : SOCGPU_PRECISION_FP64;
    } else return die("unknown or incomplete option " + o);
  }
  if (sp_file.empty()) return die("Spectral file not set.");
  if (base.empty()) return die("Base name not set.");
  if (!isolir) return die("Spectral region not set.");
  if (first < 1 || last < first) return die("Range of bands not set");
  if (cloud != SOCGPU_IP_CLOUD_CLEAR) return die("only clear-sky runs (-C 5) are driven");
  if (!two_stream) two_stream = isolir == SOCGPU_IP_INFRA_RED ? 12 : 16;
  if (!solver) solver = scatter == SOCGPU_IP_SCATTER_FULL ? SOCGPU_IP_SOLVER_HOMOGEN_DIRECT : SOCGPU_IP_SOLVER_NO_SCAT;

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
    Field sf;
    if (!read_field(base + ".surf", sf, err)) return die(err);
    for (size_t l = 0; l < np; ++l)
      for (int b = 0; b < nb_total; ++b) {
        const double alb = sf.v[l + np * std::min<size_t>((size_t)b, sf.n_lev - 1) * (sf.n_lev > 1 ? 1 : 0)];
        rho_alb[l + np * (0 + 2 * (size_t)b)] = alb;
        rho_alb[l + np * (1 + 2 * (size_t)b)] = alb;
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

  socgpu_control c{};
  c.isolir = isolir;
  c.i_angular_integration = SOCGPU_IP_TWO_STREAM;
  c.i_2stream = two_stream;
  c.i_scatter_method = scatter;
  c.i_solver = solver;
  c.i_cloud = SOCGPU_IP_CLOUD_CLEAR;
  c.i_cloud_representation = SOCGPU_IP_CLOUD_ICE_WATER;
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
  socgpu_dimen d{};
  d.nd_profile = (int)np;
  d.nd_layer = (int)nl;
  d.id_cloud_top = 1;
  d.nd_aerosol_mode = 1;
  d.nd_cloud_component = 1;
  d.nd_cloud_type = 1;
  d.nd_subcol_gen = 1;
  d.nd_subcol_req = 1;
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
  socgpu_cld cld{};
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
