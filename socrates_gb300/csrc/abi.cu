// abi.cu -- the extern "C" boundary of libsocgpu (include/socgpu.h).
//
// Host-side work only: spectrum registry keyed by name, option validation
// with the reference's error codes, per-thread device workspace and
// stream, host<->device staging for the host-pointer entry points, and
// the choice of kernel tile shape.  No computation of the flux path runs
// on the host: an unsupported request returns SOCGPU_I_ERR_FATAL.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "host_internal.h"

namespace socgpu {

// The equivalent-extinction overlaps (rad_pcf.F90:432-436), all solved by
// solve_band_k_eqv_scl.
// three regions (clear, stratiform, convective), and any region scheme
bool triple_cloud(int i_cloud) { return i_cloud == SOCGPU_IP_CLOUD_TRIPLE || i_cloud == SOCGPU_IP_CLOUD_PART_CORR_CNV; }
bool region_cloud(int i_cloud) {
  return i_cloud == SOCGPU_IP_CLOUD_MIX_MAX || i_cloud == SOCGPU_IP_CLOUD_MIX_RANDOM ||
         i_cloud == SOCGPU_IP_CLOUD_PART_CORR || triple_cloud(i_cloud);
}

int gas_overlap(const socgpu_control *c, const SpectrumEntry *sp) {
  if (c->i_gas_overlap != SOCGPU_IP_OVERLAP_HYBRID) return c->i_gas_overlap;
  const int nb = (int)sp->band_overlap.size();
  const int b0 = std::max(c->first_band, 1), b1 = std::min(c->last_band, nb);
  int ov = b0 <= b1 ? sp->band_overlap[b0 - 1] : 0;
  for (int b = b0; b <= b1; ++b)
    if (sp->band_overlap[b - 1] != ov) return 0;
  return ov == SOCGPU_IP_OVERLAP_HYBRID ? 0 : ov;
}

bool is_keqv(const socgpu_control *c, const SpectrumEntry *sp) {
  const int ov = gas_overlap(c, sp);
  return ov == SOCGPU_IP_OVERLAP_K_EQV_SCL || ov == SOCGPU_IP_OVERLAP_K_EQV || ov == SOCGPU_IP_OVERLAP_K_EQV_MOD;
}

int launch_cloud_gen(int nd_layer, int cloud_top, int n_layer, int nd_profile, int il1, int il2,
                     int n_subcol, int n1, int n2, int ipph, int ioverlap, const int *rand_seed,
                     const double *rlc_cf, const double *rlc_cw, const double *sigma_qcw,
                     const double *avg_cf, const double *c_cloud, const double *c_ratio,
                     const double *zf, const double *xcw, int *n_subcol_cld, double *c_sub, int rng,
                     int *range_dev, cudaStream_t st, char *msg, size_t len);
int launch_cloud_gen_noalloc(int nd_layer, int cloud_top, int n_layer, int nd_profile, int il1, int il2,
                             int n_subcol, int n1, int n2, int ipph, int ioverlap, const int *rand_seed,
                             const double *rlc_cf, const double *rlc_cw, const double *sigma_qcw,
                             const double *avg_cf, const double *c_cloud, const double *c_ratio,
                             const double *zf, const double *xcw, int *n_subcol_cld, double *c_sub, int rng,
                             cudaStream_t st, char *msg, size_t len);

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_msg(char *msg, size_t len, const char *fmt, ...) {
  if (!msg || len == 0) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, len, fmt, ap);
  va_end(ap);
}

namespace {

// ---------------------------------------------------------------------------
// Spectrum registry.
std::mutex g_reg_mutex;
std::map<int, std::unique_ptr<SpectrumEntry>> g_spectra;
std::map<std::string, int> g_names;
int g_next_handle = 1;

template <class T>
T fget2(const T *a, int i, int j, int nd1) { return a[(size_t)i + (size_t)nd1 * (size_t)j]; }

int build_spectrum(const socgpu_spectrum_desc *d, SpectrumEntry &e, char *msg, size_t msg_len) {
  if (d->n_band < 1 || d->n_band > SOCGPU_MAX_BAND || d->n_band > d->nd_band) {
    set_msg(msg, msg_len, "number of bands %d outside 1..%d", d->n_band, SOCGPU_MAX_BAND);
    return SOCGPU_I_ERR_RANGE;
  }
  if (d->n_absorb > SOCGPU_MAX_SPECIES) {
    set_msg(msg, msg_len, "too many absorbers (%d)", d->n_absorb);
    return SOCGPU_I_ERR_RANGE;
  }
  if (d->thermal_coeff && (d->n_deg_fit < 0 || d->n_deg_fit + 1 > kMaxPlanckCoeff)) {
    set_msg(msg, msg_len, "Planck polynomial degree %d unsupported", d->n_deg_fit);
    return SOCGPU_I_ERR_RANGE;
  }
  e.bands_host.assign(d->n_band, BandInfo{});
  e.gpoints_host.clear();
  e.type_absorb.assign(d->type_absorb, d->type_absorb + d->n_absorb);
  e.n_k_major.assign(d->n_band, 0);
  std::vector<BandInfo> bands_keqv;
  std::vector<GPoint> gpoints_keqv;
  std::vector<TermK> minor;
  bool random_ok = true;
  // lookup tables, gathered into one compact array: one block per (band,
  // absorber, k-term) that uses them (P/T: n_tmp x n_pre, or with gas
  // fractions n_tmp x n_pre x n_gf; temperature only: n_t)
  const int n_pre = d->n_pre, n_tmp = d->n_tmp;
  const bool sb_tables = d->index_sb && d->nd_species_sb > 0 && d->n_gas_frac >= 1 && d->gf_lookup && d->k_lookup_sb;
  std::vector<double> k_lk;
  std::map<std::tuple<int, int, int>, int> lk_of;
  auto lookup_block = [&](int b, int g, int iex, int fnc) -> int {
    if (fnc != SOCGPU_IP_SCALE_LOOKUP && fnc != SOCGPU_IP_SCALE_T_LOOKUP) return -1;
    auto key = std::make_tuple(b, g, iex);
    auto it = lk_of.find(key);
    if (it != lk_of.end()) return it->second;
    const int off = (int)k_lk.size();
    if (fnc == SOCGPU_IP_SCALE_T_LOOKUP) {
      const size_t src = (size_t)d->nd_t_lookup_gas * ((size_t)iex + (size_t)d->nd_k_term * ((size_t)g + (size_t)d->nd_species * b));
      for (int q = 0; q < d->n_t_lookup_gas[g]; ++q) k_lk.push_back(d->k_t_lookup_gas[src + q]);
    } else if (sb_tables && d->index_sb[g] > 0) {
      const size_t n = (size_t)n_tmp * n_pre * d->n_gas_frac;
      const size_t src = n * ((size_t)iex + (size_t)d->nd_k_term * ((size_t)(d->index_sb[g] - 1) + (size_t)d->nd_species_sb * b));
      k_lk.insert(k_lk.end(), d->k_lookup_sb + src, d->k_lookup_sb + src + n);
    } else {
      const size_t n = (size_t)n_tmp * n_pre;
      const size_t src = n * ((size_t)iex + (size_t)d->nd_k_term * ((size_t)g + (size_t)d->nd_species * b));
      k_lk.insert(k_lk.end(), d->k_lookup + src, d->k_lookup + src + n);
    }
    lk_of[key] = off;
    return off;
  };
  bool any_lookup = false;
  for (int b = 0; b < d->n_band; ++b) {
    BandInfo &bi = e.bands_host[b];
    bi.solar_flux_band = d->solar_flux_band ? d->solar_flux_band[b] : 0.0;
    bi.rayleigh_coeff = d->rayleigh_coeff ? d->rayleigh_coeff[b] : 0.0;
    if (d->thermal_coeff)
      for (int j = 0; j <= d->n_deg_fit; ++j) {
        bi.planck[j] = d->thermal_coeff[(size_t)j + (size_t)d->nd_thermal_coeff * b];
        bi.planck_f[j] = (float)bi.planck[j];
      }
    bi.rayleigh_f = (float)bi.rayleigh_coeff;
    bi.solar_flux_band_f = (float)bi.solar_flux_band;
    // continua of the band (blocks 8 and 9)
    if (d->n_band_continuum) {
      const int nc = d->n_band_continuum[b];
      if (nc < 0 || nc > kMaxContPerBand || nc > d->nd_continuum) {
        set_msg(msg, msg_len, "band %d has %d continua; at most %d supported", b + 1, nc, kMaxContPerBand);
        return SOCGPU_I_ERR_RANGE;
      }
      bi.n_cont = nc;
      for (int j = 0; j < nc; ++j) {
        BandCont &c = bi.cont[j];
        const size_t bj = (size_t)b + (size_t)d->nd_band * j;
        c.type = d->index_continuum[bj];
        c.fnc = d->i_scale_fnc_cont[bj];
        if ((c.type != SOCGPU_IP_SELF_CONTINUUM && c.type != SOCGPU_IP_FRN_CONTINUUM) ||
            (c.fnc != SOCGPU_IP_SCALE_POWER_LAW && c.fnc != SOCGPU_IP_SCALE_POWER_QUAD)) {
          set_msg(msg, msg_len, "band %d: continuum type %d with scaling %d unsupported", b + 1, c.type, c.fnc);
          return SOCGPU_I_ERR_FATAL;
        }
        c.p_ref = d->p_ref_cont[(size_t)j + (size_t)d->nd_continuum * b];
        c.t_ref = d->t_ref_cont[(size_t)j + (size_t)d->nd_continuum * b];
        c.k = d->k_cont[bj];
        for (int v = 0; v < 3; ++v)
          c.scale[v] = v < d->nd_scale_variable ? d->scale_cont[(size_t)v + (size_t)d->nd_scale_variable * bj] : 0.0;
        c.p_ref_f = (float)c.p_ref; c.t_ref_f = (float)c.t_ref; c.k_f = (float)c.k;
        for (int v = 0; v < 3; ++v) c.scale_f[v] = (float)c.scale[v];
      }
    }
    int n_abs = d->n_band_absorb ? d->n_band_absorb[b] : 0;
    if (n_abs > kMaxAbsPerBand) {
      set_msg(msg, msg_len, "band %d has %d absorbers; at most %d supported", b + 1, n_abs, kMaxAbsPerBand);
      return SOCGPU_I_ERR_RANGE;
    }
    bi.n_abs = n_abs;
    int nk[kMaxAbsPerBand];
    long long n_term = 1;
    for (int j = 0; j < n_abs; ++j) {
      int g = fget2(d->index_absorb, j, b, d->nd_species) - 1;
      if (g < 0 || g >= d->n_absorb) {
        set_msg(msg, msg_len, "band %d lists absorber index %d outside the spectrum", b + 1, g + 1);
        return SOCGPU_I_ERR_RANGE;
      }
      BandGas &gs = bi.gas[j];
      gs.species = g;
      gs.i_scale_k = fget2(d->i_scale_k, b, g, d->nd_band);
      gs.i_scale_fnc = fget2(d->i_scale_fnc, b, g, d->nd_band);
      gs.l_doppler = d->l_doppler ? d->l_doppler[g] : 0;
      gs.doppler_cor = d->doppler_cor ? d->doppler_cor[g] : 0.0;
      gs.p_ref = fget2(d->p_ref, g, b, d->nd_species);
      gs.t_ref = fget2(d->t_ref, g, b, d->nd_species);
      gs.sb = -1;
      gs.n_t = 0;
      if (gs.i_scale_k != SOCGPU_IP_SCALE_NULL && gs.i_scale_k != SOCGPU_IP_SCALE_BAND &&
          gs.i_scale_k != SOCGPU_IP_SCALE_TERM) {
        set_msg(msg, msg_len, "band %d absorber %d: illegal type of scaling %d", b + 1, g + 1, gs.i_scale_k);
        return SOCGPU_I_ERR_FATAL;
      }
      const int fnc = gs.i_scale_fnc;
      if (gs.i_scale_k != SOCGPU_IP_SCALE_NULL) {
        const bool table = fnc == SOCGPU_IP_SCALE_LOOKUP || fnc == SOCGPU_IP_SCALE_T_LOOKUP;
        if (fnc != SOCGPU_IP_SCALE_FNC_NULL && fnc != SOCGPU_IP_SCALE_POWER_LAW && fnc != SOCGPU_IP_SCALE_POWER_QUAD &&
            fnc != SOCGPU_IP_SCALE_DOPPLER_QUAD && fnc != SOCGPU_IP_SCALE_WENYI && !table) {
          set_msg(msg, msg_len, "band %d absorber %d: scaling function %d is not supported on the device path "
                  "(double power laws are not implemented)", b + 1, g + 1, fnc);
          return SOCGPU_I_ERR_FATAL;
        }
        if (table && gs.i_scale_k != SOCGPU_IP_SCALE_TERM) {
          set_msg(msg, msg_len, "band %d absorber %d: lookup tables need per-term scaling", b + 1, g + 1);
          return SOCGPU_I_ERR_FATAL;
        }
        if (fnc == SOCGPU_IP_SCALE_LOOKUP) {
          if (n_pre < 2 || n_tmp < 2 || n_tmp > 255 || n_pre > 255 || !d->p_lookup || !d->t_lookup || !d->k_lookup) {
            set_msg(msg, msg_len, "band %d absorber %d: P/T lookup tables missing or outside 2..255 entries",
                    b + 1, g + 1);
            return SOCGPU_I_ERR_FATAL;
          }
          if (sb_tables && d->index_sb[g] > 0) {
            gs.sb = d->index_sb[g] - 1;
            if (gs.sb >= kMaxSb || gs.sb >= d->nd_species_sb || d->n_gas_frac > 255) {
              set_msg(msg, msg_len, "absorber %d: self-broadened index %d outside 1..%d", g + 1, gs.sb + 1, kMaxSb);
              return SOCGPU_I_ERR_RANGE;
            }
          }
          any_lookup = true;
        }
        if (fnc == SOCGPU_IP_SCALE_T_LOOKUP) {
          if (!d->n_t_lookup_gas || !d->t_lookup_gas || !d->k_t_lookup_gas || d->n_t_lookup_gas[g] < 2 ||
              d->n_t_lookup_gas[g] > d->nd_t_lookup_gas) {
            set_msg(msg, msg_len, "band %d absorber %d: temperature lookup tables missing", b + 1, g + 1);
            return SOCGPU_I_ERR_FATAL;
          }
          gs.n_t = d->n_t_lookup_gas[g];
        }
        if (fnc == SOCGPU_IP_SCALE_WENYI &&
            (!d->wenyi_plg || !((b == 3 && d->wenyi_gk4 && d->wenyi_gk250b && d->wenyi_ttb) ||
                                (b == 5 && d->wenyi_gk6 && d->wenyi_tto)))) {
          set_msg(msg, msg_len, "band %d absorber %d: Wen-Yi scaling needs band 4 or 6 and its tables", b + 1, g + 1);
          return SOCGPU_I_ERR_FATAL;
        }
      }
      int nv = d->nd_scale_variable < 4 ? d->nd_scale_variable : 4;
      for (int v = 0; v < nv; ++v) {
        gs.scale[v] = d->scale[(size_t)v + (size_t)d->nd_scale_variable *
                                              ((size_t)0 + (size_t)d->nd_k_term * ((size_t)b + (size_t)d->nd_band * g))];
        gs.scale_f[v] = (float)gs.scale[v];
      }
      gs.p_ref_f = (float)gs.p_ref;
      gs.t_ref_f = (float)gs.t_ref;
      gs.doppler_cor_f = (float)gs.doppler_cor;
      nk[j] = fget2(d->i_band_k, b, g, d->nd_band);
      if (nk[j] < 1 || nk[j] > d->nd_k_term ||
          (fnc == SOCGPU_IP_SCALE_WENYI && nk[j] > (b == 3 ? d->wenyi_n_term4 : d->wenyi_n_term6))) {
        set_msg(msg, msg_len, "band %d absorber %d: %d k-terms", b + 1, g + 1, nk[j]);
        return SOCGPU_I_ERR_RANGE;
      }
      if (j == 0) e.n_k_major[b] = nk[0];
      if (n_term <= SOCGPU_MAX_GPOINT) n_term *= nk[j];
    }
    // one k-term of absorber j as a g-point entry; returns its weight
    auto set_term = [&](GPoint &gp, int j, int iex) {
      const int g = bi.gas[j].species;
      const size_t q = (size_t)iex + (size_t)d->nd_k_term * ((size_t)b + (size_t)d->nd_band * g);
      gp.k[j] = d->k[q];
      gp.kf[j] = (float)d->k[q];
      gp.iex[j] = (short)iex;
      gp.lk_off[j] = lookup_block(b, g, iex, bi.gas[j].i_scale_fnc);
      const int nv = d->nd_scale_variable < 4 ? d->nd_scale_variable : 4;
      for (int v = 0; v < nv; ++v) {
        gp.term_scale[j][v] = d->scale[(size_t)v + (size_t)d->nd_scale_variable * q];
        gp.term_scale_f[j][v] = (float)gp.term_scale[j][v];
      }
      return d->w[q];
    };
    // k-term products of random overlap (solve_band_random_overlap.F90:533-560)
    bi.g_first = (int)e.gpoints_host.size();
    if (n_abs == 0) n_term = 1;
    if ((long long)e.gpoints_host.size() + n_term > SOCGPU_MAX_GPOINT) random_ok = false;
    for (long long kt = 0; random_ok && kt < n_term; ++kt) {
      GPoint gp{};
      gp.band = b;
      gp.n_abs = n_abs;
      gp.weight = 1.0;
      long long step_prod = 1;
      for (int j = 0; j < n_abs; ++j) {
        step_prod *= nk[j];
        long long step = n_term / step_prod;
        int iex = (int)((kt / step) % nk[j]);
        double wj = set_term(gp, j, iex);
        gp.weight = (j == 0) ? wj : gp.weight * wj;
        if (j == 0) gp.iex_major = iex;
      }
      gp.weight_f = (float)gp.weight;
      if (n_abs > 0 && !(gp.weight > 0.0)) continue;   // n_term_reduced
      e.gpoints_host.push_back(gp);
    }
    bi.g_count = random_ok ? (int)e.gpoints_host.size() - bi.g_first : 0;
    // equivalent extinction (solve_band_k_eqv_scl.F90:1043-1100): the major
    // absorber's terms are solved, the minor absorbers' terms weighted
    BandInfo bk = bi;
    bk.g_first = (int)gpoints_keqv.size();
    const int n_major = n_abs > 0 ? nk[0] : 1;
    for (int iex = 0; iex < n_major; ++iex) {
      GPoint gp{};
      gp.band = b;
      gp.n_abs = n_abs > 0 ? 1 : 0;
      gp.weight = n_abs > 0 ? set_term(gp, 0, iex) : 1.0;
      gp.iex_major = iex;
      gp.weight_f = (float)gp.weight;
      gpoints_keqv.push_back(gp);
    }
    bk.g_count = n_major;
    for (int j = 1; j < n_abs; ++j) {
      bk.minor_first[j] = (int)minor.size();
      bk.minor_count[j] = nk[j];
      const int g = bi.gas[j].species;
      for (int iex = 0; iex < nk[j]; ++iex) {
        TermK t{};
        const size_t q = (size_t)iex + (size_t)d->nd_k_term * ((size_t)b + (size_t)d->nd_band * g);
        t.iex = iex;
        t.k = d->k[q]; t.w = d->w[q];
        t.kf = (float)t.k; t.wf = (float)t.w;
        t.lk_off = lookup_block(b, g, iex, bi.gas[j].i_scale_fnc);
        const int nv = d->nd_scale_variable < 4 ? d->nd_scale_variable : 4;
        for (int v = 0; v < nv; ++v) {
          t.scale[v] = d->scale[(size_t)v + (size_t)d->nd_scale_variable * q];
          t.scale_f[v] = (float)t.scale[v];
        }
        minor.push_back(t);
      }
    }
    bands_keqv.push_back(bk);
  }
  if ((long long)gpoints_keqv.size() > SOCGPU_MAX_GPOINT) {
    set_msg(msg, msg_len, "more than %d k-terms of major absorbers", SOCGPU_MAX_GPOINT);
    return SOCGPU_I_ERR_RANGE;
  }
  if (!random_ok) {
    e.gpoints_host.clear();
    for (auto &bb : e.bands_host) { bb.g_first = 0; bb.g_count = 0; }
  }
  SpectrumDev &s = e.dev;
  s.n_band = d->n_band;
  s.n_gpoint = (int)e.gpoints_host.size();
  s.n_species = d->n_absorb;
  s.n_deg_fit = d->n_deg_fit;
  s.nd_band = d->nd_band;
  s.nd_k_term = d->nd_k_term;
  s.t_ref_planck = d->t_ref_planck;
  s.has_solar = d->solar_flux_band != nullptr;
  s.has_planck = d->thermal_coeff != nullptr;
  s.has_rayleigh = d->rayleigh_coeff != nullptr;
  s.has_continuum = d->n_band_continuum != nullptr;
  s.index_water = d->index_water;
  for (int b = 0; b < d->n_band; ++b) s.host_first_g[b] = e.bands_host[b].g_first;
  s.host_first_g[d->n_band] = s.n_gpoint;
  s.random_ok = random_ok;
  s.n_gpoint_keqv = (int)gpoints_keqv.size();
  for (int b = 0; b < d->n_band; ++b) s.host_first_g_keqv[b] = bands_keqv[b].g_first;
  s.host_first_g_keqv[d->n_band] = s.n_gpoint_keqv;
  // lookup grids: ln p [n_pre], T [n_pre][n_tmp], gas fractions [n_gf]
  std::vector<double> grid;
  s.has_lookup = any_lookup;
  if (any_lookup) {
    s.lk_n_pre = n_pre; s.lk_n_tmp = n_tmp;
    grid.assign(d->p_lookup, d->p_lookup + n_pre);
    grid.insert(grid.end(), d->t_lookup, d->t_lookup + (size_t)n_tmp * n_pre);
    if (sb_tables) {
      s.lk_n_gf = d->n_gas_frac;
      grid.insert(grid.end(), d->gf_lookup, d->gf_lookup + d->n_gas_frac);
      // gas fractions (inter_pt_lookup.F90:198-230): molar weights of the
      // self-broadened absorbers and of water vapour
      s.n_sb = 0;
      s.l_water = 0;
      int iw = -1;
      for (int g = 0; g < d->n_absorb; ++g)
        if (d->type_absorb[g] == 1) { s.l_water = 1; if (iw < 0) iw = g; }
      const double mw_air = 28.966e-03;
      const double mw_w = (iw >= 0 && d->molar_weight && d->molar_weight[iw] > 0.0) ? d->molar_weight[iw] : 18.0153;
      s.ratio_water = mw_air / (mw_w * 1.0e-03);
      for (int g = 0; g < d->n_absorb; ++g) {
        const int jsb = d->index_sb[g] - 1;
        if (jsb < 0) continue;
        if (jsb >= kMaxSb || !d->molar_weight || !(d->molar_weight[g] > 0.0)) {
          set_msg(msg, msg_len, "self-broadened absorber %d: index above %d or no molar weight", g + 1, kMaxSb);
          return SOCGPU_I_ERR_RANGE;
        }
        s.sb_species[jsb] = g;
        s.sb_ratio_gas[jsb] = mw_air / (d->molar_weight[g] * 1.0e-03);
        s.n_sb = std::max(s.n_sb, jsb + 1);
      }
    }
  }
  std::vector<double> tgas;
  bool any_t = false;
  for (int g = 0; g < d->n_absorb && d->n_t_lookup_gas; ++g) any_t |= d->n_t_lookup_gas[g] > 1;
  if (any_t) {
    s.nd_t_lookup_gas = d->nd_t_lookup_gas;
    tgas.assign(d->t_lookup_gas, d->t_lookup_gas + (size_t)d->nd_t_lookup_gas * d->n_absorb);
  }
  // Wen-Yi tables: plg[26], ttb[10], tto[9], gk250b[n4], gk4[10][26][n4] (Fortran order), gk6[9][26][n6]
  std::vector<double> wy;
  if (d->wenyi_plg) {
    s.wenyi_n4 = (d->wenyi_gk4 && d->wenyi_gk250b && d->wenyi_ttb) ? d->wenyi_n_term4 : 0;
    s.wenyi_n6 = (d->wenyi_gk6 && d->wenyi_tto) ? d->wenyi_n_term6 : 0;
    wy.assign(d->wenyi_plg, d->wenyi_plg + 26);
    for (int q = 0; q < 10; ++q) wy.push_back(s.wenyi_n4 ? d->wenyi_ttb[q] : 0.0);
    for (int q = 0; q < 9; ++q) wy.push_back(s.wenyi_n6 ? d->wenyi_tto[q] : 0.0);
    for (int q = 0; q < s.wenyi_n4; ++q) wy.push_back(d->wenyi_gk250b[q]);
    if (s.wenyi_n4) wy.insert(wy.end(), d->wenyi_gk4, d->wenyi_gk4 + (size_t)260 * s.wenyi_n4);
    if (s.wenyi_n6) wy.insert(wy.end(), d->wenyi_gk6, d->wenyi_gk6 + (size_t)234 * s.wenyi_n6);
  }
  // cloud parameter sets
  std::vector<double> drop, ice;
  s.n_drop_type = (d->drop_parm_list && d->nd_drop_type > 0) ? d->nd_drop_type : 0;
  s.n_ice_type = (d->ice_parm_list && d->nd_ice_type > 0) ? d->nd_ice_type : 0;
  // each set at its type number (read_spectrum.F90 blocks 10 and 12), the
  // first kCloudParm coefficients; the scheme of each type stays on the host
  const int ncp = std::min(d->nd_cloud_parameter, kCloudParm);
  e.n_cloud_parameter = d->nd_cloud_parameter;
  e.drop_scheme.assign(s.n_drop_type, 0);
  e.ice_scheme.assign(s.n_ice_type, 0);
  e.drop_min_dim.clear(); e.drop_max_dim.clear(); e.ice_min_dim.clear(); e.ice_max_dim.clear();
  e.band_overlap.assign(d->n_band, 0);
  if (d->i_overlap) e.band_overlap.assign(d->i_overlap, d->i_overlap + d->n_band);
  if (d->drop_parm_min_dim && d->drop_parm_max_dim) {
    e.drop_min_dim.assign(d->drop_parm_min_dim, d->drop_parm_min_dim + s.n_drop_type);
    e.drop_max_dim.assign(d->drop_parm_max_dim, d->drop_parm_max_dim + s.n_drop_type);
  }
  if (d->ice_parm_min_dim && d->ice_parm_max_dim) {
    e.ice_min_dim.assign(d->ice_parm_min_dim, d->ice_parm_min_dim + s.n_ice_type);
    e.ice_max_dim.assign(d->ice_parm_max_dim, d->ice_parm_max_dim + s.n_ice_type);
  }
  for (int t = 0; t < s.n_drop_type; ++t)
    if ((!d->l_drop_type || d->l_drop_type[t]) && d->i_drop_parm) e.drop_scheme[t] = d->i_drop_parm[t];
  for (int t = 0; t < s.n_ice_type; ++t)
    if ((!d->l_ice_type || d->l_ice_type[t]) && d->i_ice_parm) e.ice_scheme[t] = d->i_ice_parm[t];
  drop.assign((size_t)std::max(1, s.n_drop_type) * d->n_band * kCloudParm, 0.0);
  ice.assign((size_t)std::max(1, s.n_ice_type) * d->n_band * kCloudParm, 0.0);
  for (int t = 0; t < s.n_drop_type; ++t)
    for (int b = 0; b < d->n_band; ++b)
      for (int c = 0; c < ncp; ++c)
        drop[((size_t)t * d->n_band + b) * kCloudParm + c] =
            d->drop_parm_list[(size_t)c + (size_t)d->nd_cloud_parameter * ((size_t)b + (size_t)d->nd_band * t)];
  for (int t = 0; t < s.n_ice_type; ++t)
    for (int b = 0; b < d->n_band; ++b)
      for (int c = 0; c < ncp; ++c)
        ice[((size_t)t * d->n_band + b) * kCloudParm + c] =
            d->ice_parm_list[(size_t)c + (size_t)d->nd_cloud_parameter * ((size_t)b + (size_t)d->nd_band * t)];
  std::vector<float> drop_f(drop.begin(), drop.end()), ice_f(ice.begin(), ice.end());
  // classic aerosol species (block 11): one row per (band, species,
  // humidity) of absorption, scattering and the phase-function moments
  std::vector<double> aer_tab, aer_hum;
  e.aer_parm.clear(); e.aer_nhum.clear(); e.aer_nphf.clear(); e.aer_type.clear();
  if (d->n_aerosol > 0 && d->i_aerosol_parm && d->aerosol_abs && d->aerosol_scat && d->aerosol_phf) {
    if (d->n_aerosol > d->nd_aerosol_species || d->nd_humidity < 1 || d->nd_phase_term < 1) {
      set_msg(msg, msg_len, "aerosol extents inconsistent (%d species, %d allocated)", d->n_aerosol,
              d->nd_aerosol_species);
      return SOCGPU_I_ERR_RANGE;
    }
    const int nsp = d->n_aerosol;
    int nh = 1, nphf = 1;
    for (int j = 0; j < nsp; ++j) {
      const int hj = d->nhumidity ? d->nhumidity[j] : 0, fj = d->n_aerosol_phf_term ? d->n_aerosol_phf_term[j] : 1;
      if (hj > d->nd_humidity || fj > d->nd_phase_term) {
        set_msg(msg, msg_len, "aerosol species %d: %d humidities or %d moments exceed the allocation", j + 1, hj, fj);
        return SOCGPU_I_ERR_RANGE;
      }
      e.aer_parm.push_back(d->i_aerosol_parm[j]);
      e.aer_type.push_back(d->type_aerosol ? d->type_aerosol[j] : 0);
      e.aer_nhum.push_back(hj);
      e.aer_nphf.push_back(std::max(1, fj));
      nh = std::max(nh, hj);
      nphf = std::max(nphf, fj);
    }
    s.aer_n_species = nsp; s.aer_nh = nh; s.aer_nphf = nphf;
    e.aer_nd_species = d->nd_aerosol_species;
    e.aer_parm_file = e.aer_parm;
    const int row = 2 + nphf, ndh = d->nd_humidity, ndf = d->nd_phase_term, nda = d->nd_aerosol_species;
    aer_tab.assign((size_t)d->n_band * nsp * nh * row, 0.0);
    aer_hum.assign((size_t)nsp * nh, 0.0);
    for (int j = 0; j < nsp; ++j)
      for (int h = 0; h < std::max(1, e.aer_nhum[j]); ++h)
        if (d->aerosol_humidities && e.aer_nhum[j] > 0) aer_hum[(size_t)j * nh + h] = d->aerosol_humidities[h + (size_t)ndh * j];
    for (int b = 0; b < d->n_band; ++b)
      for (int j = 0; j < nsp; ++j)
        for (int h = 0; h < std::max(1, e.aer_nhum[j]); ++h) {
          double *r = &aer_tab[(((size_t)b * nsp + j) * nh + h) * row];
          const size_t q = (size_t)h + (size_t)ndh * ((size_t)j + (size_t)nda * b);
          r[0] = d->aerosol_abs[q];
          r[1] = d->aerosol_scat[q];
          for (int m = 0; m < e.aer_nphf[j]; ++m)
            r[2 + m] = d->aerosol_phf[(size_t)h + (size_t)ndh * ((size_t)m + (size_t)ndf * ((size_t)j + (size_t)nda * b))];
        }
  }
  std::vector<float> aer_tab_f(aer_tab.begin(), aer_tab.end()), aer_hum_f(aer_hum.begin(), aer_hum.end());
  cudaGetDevice(&e.device);
  // the tables of lookup scaling, equivalent extinction and Wen-Yi scaling
  auto up = [&](auto *&dst, const auto &v) -> bool {
    using T = typename std::decay_t<decltype(v)>::value_type;
    if (v.empty()) { dst = nullptr; return true; }
    if (cudaMalloc((void **)&dst, sizeof(T) * v.size()) != cudaSuccess) return false;
    return cudaMemcpy(dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  };
  std::vector<float> grid_f(grid.begin(), grid.end()), k_lk_f(k_lk.begin(), k_lk.end());
  std::vector<float> tgas_f(tgas.begin(), tgas.end()), wy_f(wy.begin(), wy.end());
  if (!up(s.bands_keqv, bands_keqv) || !up(s.gpoints_keqv, gpoints_keqv) || !up(s.minor_terms, minor) ||
      !up(s.lk_grid, grid) || !up(s.lk_grid_f, grid_f) || !up(s.k_lookup, k_lk) || !up(s.k_lookup_f, k_lk_f) ||
      !up(s.t_lookup_gas, tgas) || !up(s.t_lookup_gas_f, tgas_f) || !up(s.wenyi, wy) || !up(s.wenyi_f, wy_f) ||
      !up(s.aer_tab, aer_tab) || !up(s.aer_tab_f, aer_tab_f) || !up(s.aer_hum, aer_hum) ||
      !up(s.aer_hum_f, aer_hum_f)) {
    cudaGetLastError();
    set_msg(msg, msg_len, "device allocation or upload of lookup and overlap tables failed");
    return SOCGPU_I_ABORT_CALCULATION;
  }
  if (cudaMalloc(&s.bands, sizeof(BandInfo) * s.n_band) != cudaSuccess ||
      cudaMalloc(&s.gpoints, sizeof(GPoint) * std::max(1, s.n_gpoint)) != cudaSuccess ||
      cudaMalloc(&s.drop_parm, sizeof(double) * drop.size()) != cudaSuccess ||
      cudaMalloc(&s.ice_parm, sizeof(double) * ice.size()) != cudaSuccess ||
      cudaMalloc(&s.drop_parm_f, sizeof(float) * drop_f.size()) != cudaSuccess ||
      cudaMalloc(&s.ice_parm_f, sizeof(float) * ice_f.size()) != cudaSuccess) {
    set_msg(msg, msg_len, "device allocation for spectral tables failed");
    return SOCGPU_I_ABORT_CALCULATION;
  }
  cudaError_t err = cudaMemcpy(s.bands, e.bands_host.data(), sizeof(BandInfo) * s.n_band, cudaMemcpyHostToDevice);
  if (err == cudaSuccess && s.n_gpoint > 0)
    err = cudaMemcpy(s.gpoints, e.gpoints_host.data(), sizeof(GPoint) * s.n_gpoint, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(s.drop_parm, drop.data(), sizeof(double) * drop.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(s.ice_parm, ice.data(), sizeof(double) * ice.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(s.drop_parm_f, drop_f.data(), sizeof(float) * drop_f.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(s.ice_parm_f, ice_f.data(), sizeof(float) * ice_f.size(), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    set_msg(msg, msg_len, "upload of spectral tables failed: %s", cudaGetErrorString(err));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return SOCGPU_I_NORMAL;
}

void free_spectrum(SpectrumEntry &e) {
  cudaFree(e.dev.bands_keqv);
  cudaFree(e.dev.gpoints_keqv);
  cudaFree(e.dev.minor_terms);
  cudaFree(e.dev.lk_grid);
  cudaFree(e.dev.lk_grid_f);
  cudaFree(e.dev.k_lookup);
  cudaFree(e.dev.k_lookup_f);
  cudaFree(e.dev.t_lookup_gas);
  cudaFree(e.dev.t_lookup_gas_f);
  cudaFree(e.dev.wenyi);
  cudaFree(e.dev.wenyi_f);
  cudaFree(e.dev.aer_tab);
  cudaFree(e.dev.aer_tab_f);
  cudaFree(e.dev.aer_hum);
  cudaFree(e.dev.aer_hum_f);
  cudaFree(e.dev.bands);
  cudaFree(e.dev.gpoints);
  cudaFree(e.dev.drop_parm);
  cudaFree(e.dev.ice_parm);
  cudaFree(e.dev.drop_parm_f);
  cudaFree(e.dev.ice_parm_f);
}

}  // namespace

SpectrumEntry *find_spectrum(int h) {
  std::lock_guard<std::mutex> lk(g_reg_mutex);
  auto it = g_spectra.find(h);
  return it == g_spectra.end() ? nullptr : it->second.get();
}

// ---------------------------------------------------------------------------
// Kernel variants and tile choice.
namespace {
#define SOCGPU_VARIANT(p, m, l) \
  {p, m, l, launch_flux_##p##_##m##_##l, prepare_flux_##p##_##m##_##l, preload_flux_##p##_##m##_##l}
const FluxVariant kVariants[] = {
    SOCGPU_VARIANT(0, 0, 16), SOCGPU_VARIANT(0, 0, 32), SOCGPU_VARIANT(0, 1, 16), SOCGPU_VARIANT(0, 1, 32),
    SOCGPU_VARIANT(0, 2, 16), SOCGPU_VARIANT(0, 2, 32), SOCGPU_VARIANT(1, 0, 8),  SOCGPU_VARIANT(1, 0, 16),
    SOCGPU_VARIANT(1, 0, 32), SOCGPU_VARIANT(1, 1, 8),  SOCGPU_VARIANT(1, 1, 16), SOCGPU_VARIANT(1, 1, 32),
    SOCGPU_VARIANT(1, 2, 8),  SOCGPU_VARIANT(1, 2, 16), SOCGPU_VARIANT(1, 2, 32),
    // the phased kernel: single-batch launches only
    {0, 0, 1, launch_phased_0_0, nullptr, nullptr}, {0, 1, 1, launch_phased_0_1, nullptr, nullptr},
    {1, 0, 1, launch_phased_1_0, nullptr, nullptr}, {1, 1, 1, launch_phased_1_1, nullptr, nullptr},
};
#undef SOCGPU_VARIANT
}  // namespace

const FluxVariant *find_variant(int precision, int mode, int lanes) {
  for (const FluxVariant &v : kVariants)
    if (v.precision == precision && v.mode == mode && v.lanes == lanes) return &v;
  return nullptr;
}

int preload_kernels() {
  static std::mutex m;
  static std::set<int> loaded;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return SOCGPU_I_ABORT_CALCULATION; }
  std::lock_guard<std::mutex> lk(m);
  if (loaded.count(dev)) return SOCGPU_I_NORMAL;
  for (const FluxVariant &v : kVariants)
    if (v.preload) {
      const int st = v.preload();
      if (st != 0) return st;
    }
  loaded.insert(dev);
  return SOCGPU_I_NORMAL;
}

// Tile overrides (socgpu_set_tile_config) and the tuner's table, keyed by
// (precision, mode, n_layer).
std::mutex g_tile_mutex;
int g_tile[2][3][2] = {};   // [precision][mode][lanes, warps]
std::map<std::tuple<int, int, int>, TileConfig> g_tuned;

// The built-in scan tile: 32 lanes above 64 layers (mixed) or above 128
// layers (FP64), else 16; 8 warps; the smallest chunk covering the column.
TileConfig scan_tile(int precision, int n_layer) {
  TileConfig t{};
  t.lanes_per_solve = precision == SOCGPU_PRECISION_MIXED ? (n_layer <= 64 ? 16 : 32) : (n_layer <= 128 ? 16 : 32);
  t.warps_per_cta = 8;
  while (t.lanes_per_solve < 32 && smallest_chunk(precision, t.lanes_per_solve, n_layer) == 0) t.lanes_per_solve *= 2;
  t.chunk = smallest_chunk(precision, t.lanes_per_solve, n_layer);
  return t;
}

TileConfig choose_tile(int precision, int mode, int n_layer) {
  TileConfig t{};
  bool tuned = false;
  {
    std::lock_guard<std::mutex> lk(g_tile_mutex);
    t.lanes_per_solve = g_tile[precision][mode][0];
    t.warps_per_cta = g_tile[precision][mode][1];
    if (t.lanes_per_solve <= 0 && t.warps_per_cta <= 0) {
      auto it = g_tuned.find(std::make_tuple(precision, mode, n_layer));
      if (it != g_tuned.end()) { t = it->second; tuned = true; }
    }
  }
  if (!tuned) {
    if (t.lanes_per_solve <= 0) {
      // measured on GB300: short chunks (few layers per lane) win over long
      // ones -- fewer live registers and more resident warps
      if (precision == SOCGPU_PRECISION_MIXED) t.lanes_per_solve = n_layer <= 64 ? 16 : 32;
      else t.lanes_per_solve = n_layer <= 128 ? 16 : 32;
    }
    if (t.warps_per_cta <= 0) t.warps_per_cta = 8;
    t.chunk = 0;
  }
  // the phased kernel's chunk is its k-term batch (0: the launcher's default)
  if (t.lanes_per_solve == 1) return t;
  // the chunk must cover the column
  while (t.lanes_per_solve < 32 && smallest_chunk(precision, t.lanes_per_solve, n_layer) == 0)
    t.lanes_per_solve *= 2;
  if (t.chunk == 0 || t.lanes_per_solve * t.chunk < n_layer)
    t.chunk = smallest_chunk(precision, t.lanes_per_solve, n_layer);
  return t;
}

// The phase of a condensed component (rad_pcf.F90:187-193): stratiform or
// convective water (ip_clcmp_st_water 1, ip_clcmp_cnv_water 3) or ice (2, 4).
int condensed_phase(int type_condensed) {
  if (type_condensed == SOCGPU_IP_CLCMP_ST_WATER || type_condensed == SOCGPU_IP_CLCMP_CNV_WATER)
    return SOCGPU_IP_PHASE_WATER;
  if (type_condensed == SOCGPU_IP_CLCMP_ST_ICE || type_condensed == SOCGPU_IP_CLCMP_CNV_ICE) return SOCGPU_IP_PHASE_ICE;
  return type_condensed;
}

// ---------------------------------------------------------------------------
// Validation (mirrors the checks the reference makes before and during
// radiance_calc; unsupported options are fatal, never a CPU fallback).
int validate(const socgpu_control *c, const socgpu_dimen *dm, const SpectrumEntry *sp, const socgpu_atm *atm,
             const socgpu_cld *cld, const socgpu_aer *aer, const socgpu_bound *bd, const socgpu_radout *out,
             char *msg, size_t msg_len) {
  if (!c || !dm || !atm || !bd || !out) { set_msg(msg, msg_len, "null argument"); return SOCGPU_I_ERR_FATAL; }
  if (!sp) { set_msg(msg, msg_len, "unknown spectrum handle"); return SOCGPU_I_ERR_EXIST; }
  if (c->i_angular_integration != SOCGPU_IP_TWO_STREAM) {
    set_msg(msg, msg_len, "only two-stream angular integration is supported"); return SOCGPU_I_ERR_FATAL; }
  if (c->isolir != SOCGPU_IP_SOLAR && c->isolir != SOCGPU_IP_INFRA_RED) {
    set_msg(msg, msg_len, "isolir must be solar or infra-red"); return SOCGPU_I_ERR_FATAL; }
  const int ovl = gas_overlap(c, sp);
  if (c->i_gas_overlap == SOCGPU_IP_OVERLAP_HYBRID && ovl == 0) {
    set_msg(msg, msg_len, "ip_overlap_hybrid: bands %d..%d of the spectral file do not name one overlap method "
            "(bands of several methods in one call are not built)", c->first_band, c->last_band);
    return SOCGPU_I_ERR_FATAL;
  }
  if (ovl != SOCGPU_IP_OVERLAP_RANDOM && !is_keqv(c, sp)) {
    set_msg(msg, msg_len, "only random and equivalent-extinction gas overlaps are supported");
    return SOCGPU_I_ERR_FATAL;
  }
  if (ovl == SOCGPU_IP_OVERLAP_RANDOM && !sp->dev.random_ok) {
    set_msg(msg, msg_len, "random overlap of this spectrum needs more than %d k-term products; "
            "use equivalent extinction (i_gas_overlap 4)", SOCGPU_MAX_GPOINT);
    return SOCGPU_I_ERR_RANGE;
  }
  switch (c->i_2stream) {
    case SOCGPU_IP_EDDINGTON: case SOCGPU_IP_ELSASSER: case SOCGPU_IP_DISCRETE_ORD: case SOCGPU_IP_PIFM85:
    case SOCGPU_IP_2S_TEST: case SOCGPU_IP_HEMI_MEAN: case SOCGPU_IP_PIFM80: break;
    default:
      if (c->i_scatter_method == SOCGPU_IP_SCATTER_FULL) {
        set_msg(msg, msg_len, "unrecognised or unimplemented two-stream scheme %d", c->i_2stream);
        return SOCGPU_I_ERR_FATAL;
      }
  }
  const bool triple = triple_cloud(c->i_cloud);
  const bool region = region_cloud(c->i_cloud);
  if (c->i_scatter_method == SOCGPU_IP_SCATTER_FULL) {
    if (!region && c->i_solver != SOCGPU_IP_SOLVER_HOMOGEN_DIRECT) {
      set_msg(msg, msg_len, "scattering requires solver_homogen_direct"); return SOCGPU_I_ERR_FATAL; }
    if (triple && c->i_solver != SOCGPU_IP_SOLVER_TRIPLE_HOGAN) {
      set_msg(msg, msg_len, "three cloud regions require solver_triple_hogan"); return SOCGPU_I_ERR_FATAL; }
    if (triple && c->i_cloud_representation != SOCGPU_IP_CLOUD_CONV_STRAT &&
        c->i_cloud_representation != SOCGPU_IP_CLOUD_CSIW && c->i_cloud_representation != SOCGPU_IP_CLOUD_SPLIT_HOMOGEN &&
        c->i_cloud_representation != SOCGPU_IP_CLOUD_SPLIT_ICE_WATER) {
      // aggregate_cloud.F90:155-160
      set_msg(msg, msg_len, "This representation of clouds is not compatible with separate convective and "
                            "stratiform overlap.");
      return SOCGPU_I_ERR_FATAL; }
    if (region && !triple && c->i_solver != SOCGPU_IP_SOLVER_MIX_DIRECT &&
        c->i_solver != SOCGPU_IP_SOLVER_MIX_DIRECT_HOGAN) {
      set_msg(msg, msg_len, "cloud regions require solver_mix_direct or solver_mix_direct_hogan");
      return SOCGPU_I_ERR_FATAL; }
  } else if (c->i_scatter_method == SOCGPU_IP_NO_SCATTER_ABS || c->i_scatter_method == SOCGPU_IP_NO_SCATTER_EXT) {
    if (c->i_solver != SOCGPU_IP_SOLVER_NO_SCAT) {
      set_msg(msg, msg_len, "no-scattering methods require solver_no_scat"); return SOCGPU_I_ERR_FATAL; }
    if (c->isolir == SOCGPU_IP_SOLAR) {
      set_msg(msg, msg_len, "the solar path requires scattering"); return SOCGPU_I_ERR_FATAL; }
    if (c->i_cloud == SOCGPU_IP_CLOUD_MCICA || region) {
      set_msg(msg, msg_len, "clouds require full scattering on the device path"); return SOCGPU_I_ERR_FATAL; }
  } else {
    set_msg(msg, msg_len, "unsupported scattering method %d", c->i_scatter_method); return SOCGPU_I_ERR_FATAL; }
  if (c->isolir == SOCGPU_IP_SOLAR && c->i_direct_tau != SOCGPU_IP_DIRECT_DELTA_SCALING &&
      c->i_direct_tau != SOCGPU_IP_DIRECT_NOSCALING) {
    set_msg(msg, msg_len, "only delta-scaled (i_direct_tau=1) and unscaled (0) direct optical depths are supported");
    return SOCGPU_I_ERR_FATAL;
  }
  if (c->l_rescale && c->n_order_forward < 1) {
    set_msg(msg, msg_len, "n_order_forward must be positive"); return SOCGPU_I_ERR_FATAL; }
  if (c->i_cloud != SOCGPU_IP_CLOUD_CLEAR && c->i_cloud != SOCGPU_IP_CLOUD_MCICA && !region) {
    set_msg(msg, msg_len, "only clear-sky, McICA and two- and three-region cloud schemes are supported");
    return SOCGPU_I_ERR_FATAL; }
  if (c->precision != SOCGPU_PRECISION_FP64 && c->precision != SOCGPU_PRECISION_MIXED) {
    set_msg(msg, msg_len, "unknown precision %d", c->precision); return SOCGPU_I_ERR_FATAL; }
  if (c->first_band < 1 || c->last_band > sp->dev.n_band || c->first_band > c->last_band) {
    set_msg(msg, msg_len, "band range %d..%d outside the spectrum's 1..%d", c->first_band, c->last_band, sp->dev.n_band);
    return SOCGPU_I_ERR_RANGE;
  }
  if (atm->n_profile < 0 || atm->n_profile > dm->nd_profile) {
    set_msg(msg, msg_len, "n_profile %d exceeds nd_profile %d", atm->n_profile, dm->nd_profile); return SOCGPU_I_ERR_RANGE; }
  if (atm->n_layer < 1 || atm->n_layer > dm->nd_layer || atm->n_layer > SOCGPU_MAX_LAYER) {
    set_msg(msg, msg_len, "n_layer %d outside 1..min(nd_layer=%d, %d)", atm->n_layer, dm->nd_layer, SOCGPU_MAX_LAYER);
    return SOCGPU_I_ERR_RANGE;
  }
  if (c->isolir == SOCGPU_IP_INFRA_RED && !sp->dev.has_planck) {
    set_msg(msg, msg_len, "infra-red calculation without Planck data"); return SOCGPU_I_ERR_FATAL; }
  if (c->isolir == SOCGPU_IP_SOLAR && !sp->dev.has_solar) {
    set_msg(msg, msg_len, "solar calculation without solar spectrum"); return SOCGPU_I_ERR_FATAL; }
  if (c->l_rayleigh && !sp->dev.has_rayleigh) {
    set_msg(msg, msg_len, "Rayleigh scattering requested without Rayleigh coefficients"); return SOCGPU_I_ERR_FATAL; }
  if (c->isolir == SOCGPU_IP_SOLAR && (!bd->zen_0 || !bd->solar_irrad)) {
    set_msg(msg, msg_len, "solar calculation without zen_0/solar_irrad"); return SOCGPU_I_ERR_FATAL; }
  if (c->isolir == SOCGPU_IP_INFRA_RED && !bd->t_ground && !bd->flux_ground) {
    set_msg(msg, msg_len, "infra-red calculation without t_ground or flux_ground"); return SOCGPU_I_ERR_FATAL; }
  if (c->l_continuum && sp->dev.has_continuum &&
      (!atm->density || !atm->gas_mix_ratio || sp->dev.index_water < 1 || sp->dev.index_water > sp->dev.n_species)) {
    set_msg(msg, msg_len, "continuum absorption needs the layer density, the gas mixing ratios and water vapour");
    return SOCGPU_I_ERR_FATAL;
  }
  // t_level feeds only the Planck terms of the infra-red
  if (!bd->rho_alb || !atm->p || !atm->t || !atm->mass || (c->l_gas && !atm->gas_mix_ratio) ||
      (c->isolir == SOCGPU_IP_INFRA_RED && !atm->t_level)) {
    set_msg(msg, msg_len, "missing atmospheric or surface field"); return SOCGPU_I_ERR_FATAL; }
  if (!out->flux_up || !out->flux_down) { set_msg(msg, msg_len, "missing output arrays"); return SOCGPU_I_ERR_FATAL; }
  if (out->flux_up_band || out->flux_down_band) {
    set_msg(msg, msg_len, "per-band flux diagnostics are not supported on the device path"); return SOCGPU_I_ERR_FATAL; }
  if (c->l_aerosol_mode && aer && aer->n_mode > 0) {
    if (aer->n_mode > SOCGPU_MAX_MODE || aer->n_mode > dm->nd_aerosol_mode) {
      set_msg(msg, msg_len, "aerosol modes %d exceed limits", aer->n_mode); return SOCGPU_I_ERR_RANGE; }
    if (!aer->mode_mix_ratio || !aer->mode_absorption || !aer->mode_scattering || !aer->mode_asymmetry) {
      set_msg(msg, msg_len, "missing aerosol mode fields"); return SOCGPU_I_ERR_FATAL; }
  }
  if (c->l_aerosol) {
    // classic aerosol species (radiance_calc.F90:603-626, opt_prop_aerosol.F90)
    const int nsp = (int)sp->aer_parm.size();
    if (nsp == 0) {
      set_msg(msg, msg_len, "aerosols requested but the spectral file has no aerosol species (block 11)");
      return SOCGPU_I_ERR_FATAL;
    }
    if (!aer || aer->n_aerosol_mr < 0 || aer->n_aerosol_mr > dm->nd_aerosol_mr) {
      set_msg(msg, msg_len, "aerosol mixing-ratio entries %d outside 0..nd_aerosol_mr", aer ? aer->n_aerosol_mr : -1);
      return SOCGPU_I_ERR_RANGE;
    }
    if (aer->n_aerosol_mr > 0 && (!aer->mix_ratio || !aer->mr_type_index)) {
      set_msg(msg, msg_len, "missing aerosol mixing ratios or their species"); return SOCGPU_I_ERR_FATAL; }
    int active = 0;
    bool moist = false;
    for (int k = 0; k < aer->n_aerosol_mr; ++k) {
      const int src = aer->mr_source ? aer->mr_source[k] : SOCGPU_IP_AERSRC_CLASSIC_RON;
      if (src < SOCGPU_IP_AERSRC_CUSACK_RON || src > SOCGPU_IP_AERSRC_ARCL_RON) continue;   // radiatively inactive
      const int j = aer->mr_type_index[k];
      if (j < 1 || j > nsp) {
        set_msg(msg, msg_len, "aerosol entry %d: species %d is not in the spectral file", k + 1, j);
        return SOCGPU_I_ERR_RANGE;
      }
      const int parm = sp->aer_parm[j - 1];
      if (parm == SOCGPU_IP_AEROSOL_UNPARAMETRIZED) {
        // prescribed optical properties (prsc_opt_prop.F90)
        if (!aer->n_opt_level_prsc || !aer->n_phase_term_prsc || !aer->pressure_prsc || !aer->absorption_prsc ||
            !aer->scattering_prsc || !aer->phase_fnc_prsc) {
          set_msg(msg, msg_len, "aerosol species %d is unparametrized but its prescribed properties are missing", j);
          return SOCGPU_I_ERR_FATAL;
        }
        const int nl = aer->n_opt_level_prsc[j - 1], nm = aer->n_phase_term_prsc[j - 1];
        const int need = (c->l_henyey_greenstein_pf || !c->l_rescale) ? 1 : std::max(1, c->n_order_forward);
        if (nl < 1 || nl > dm->nd_opt_level_aerosol_prsc || dm->nd_profile_aerosol_prsc < atm->n_profile ||
            nm < need || nm > dm->nd_phf_term_aerosol_prsc) {
          set_msg(msg, msg_len,
                  "aerosol species %d: %d prescribed levels and %d moments (%d needed) do not fit the extents "
                  "(%d profiles, %d levels, %d moments)", j, nl, nm, need, dm->nd_profile_aerosol_prsc,
                  dm->nd_opt_level_aerosol_prsc, dm->nd_phf_term_aerosol_prsc);
          return SOCGPU_I_ERR_RANGE;
        }
        if (!atm->density) {
          set_msg(msg, msg_len, "prescribed aerosol properties need the air density"); return SOCGPU_I_ERR_FATAL; }
        if (++active > kMaxAerMr) {
          set_msg(msg, msg_len, "more than %d active aerosol entries", kMaxAerMr); return SOCGPU_I_ERR_RANGE; }
        continue;
      }
      if (parm != SOCGPU_IP_AEROSOL_PARAM_DRY && parm != SOCGPU_IP_AEROSOL_PARAM_MOIST &&
          parm != SOCGPU_IP_AEROSOL_PARAM_PHF_DRY && parm != SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST) {
        set_msg(msg, msg_len, "aerosol species %d: parametrization %d is not supported", j, parm);
        return SOCGPU_I_ERR_FATAL;
      }
      if (parm == SOCGPU_IP_AEROSOL_PARAM_MOIST || parm == SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST) {
        moist = true;
        if (sp->aer_nhum[j - 1] < 2) {
          set_msg(msg, msg_len, "moist aerosol species %d has fewer than two humidities", j); return SOCGPU_I_ERR_FATAL; }
      }
      if ((parm == SOCGPU_IP_AEROSOL_PARAM_PHF_DRY || parm == SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST) && c->l_rescale &&
          !c->l_henyey_greenstein_pf && c->n_order_forward > sp->aer_nphf[j - 1]) {
        set_msg(msg, msg_len, "aerosol species %d has %d phase-function moments; forward scattering needs %d", j,
                sp->aer_nphf[j - 1], c->n_order_forward);
        return SOCGPU_I_ERR_FATAL;
      }
      if (++active > kMaxAerMr) {
        set_msg(msg, msg_len, "more than %d active aerosol entries", kMaxAerMr); return SOCGPU_I_ERR_RANGE; }
    }
    if (moist && !aer->mean_rel_humidity) {
      set_msg(msg, msg_len, "moist aerosols need the mean relative humidity"); return SOCGPU_I_ERR_FATAL; }
  }
  if (c->i_cloud == SOCGPU_IP_CLOUD_MCICA || region) {
    if (!cld || !cld->type_condensed || !cld->i_cloud_type || !cld->i_condensed_param || !cld->i_condensed_type ||
        !cld->condensed_mix_ratio || !cld->condensed_dim_char || !cld->w_cloud || !cld->frac_cloud) {
      set_msg(msg, msg_len, "clouds require cloud fields"); return SOCGPU_I_ERR_FATAL; }
    if (cld->n_condensed < 1 || cld->n_condensed > kMaxCloudComp || cld->n_cloud_type < 1 ||
        cld->n_cloud_type > (triple_cloud(c->i_cloud) ? 4 : 2)) {
      set_msg(msg, msg_len, "cloud components/types outside the supported range"); return SOCGPU_I_ERR_RANGE; }
    if (dm->id_cloud_top < 1 || dm->id_cloud_top > atm->n_layer) {
      set_msg(msg, msg_len, "id_cloud_top outside the column"); return SOCGPU_I_ERR_RANGE; }
    if (!region && (cld->n_subcol_gen < 1 || cld->n_subcol_gen > SOCGPU_MAX_SUBCOL || cld->n_subcol_req < 1)) {
      set_msg(msg, msg_len, "subcolumn counts outside 1..%d", SOCGPU_MAX_SUBCOL); return SOCGPU_I_ERR_RANGE; }
    if (!region && (!cld->c_sub || !cld->frac_cloudy || !cld->subcol_k || !cld->first_subcol_k || !cld->subcol_reorder)) {
      set_msg(msg, msg_len, "McICA requires the subcolumn fields"); return SOCGPU_I_ERR_FATAL; }
    for (int k = 0; k < cld->n_condensed; ++k) {
      int ph = condensed_phase(cld->type_condensed[k]), parm = cld->i_condensed_param[k], ty = cld->i_condensed_type[k];
      if (ph == SOCGPU_IP_PHASE_WATER) {
        if ((parm != SOCGPU_IP_SLINGO_SCHRECKER && parm != SOCGPU_IP_DROP_PADE_2) || ty < 1 ||
            ty > sp->dev.n_drop_type) {
          set_msg(msg, msg_len, "droplet parametrization %d (type %d) unsupported", parm, ty); return SOCGPU_I_ERR_FATAL; }
        if (sp->drop_scheme[ty - 1] != parm) {
          set_msg(msg, msg_len, "droplet type %d of the spectrum has scheme %d, not %d", ty, sp->drop_scheme[ty - 1],
                  parm);
          return SOCGPU_I_ERR_FATAL;
        }
      } else if (ph == SOCGPU_IP_PHASE_ICE) {
        if ((parm != SOCGPU_IP_SLINGO_SCHRECKER_ICE && parm != SOCGPU_IP_ICE_FU_PHF &&
             parm != SOCGPU_IP_ICE_PADE_2_PHF) || ty < 1 || ty > sp->dev.n_ice_type) {
          set_msg(msg, msg_len, "ice parametrization %d (type %d) unsupported", parm, ty); return SOCGPU_I_ERR_FATAL; }
        if (sp->ice_scheme[ty - 1] != parm) {
          set_msg(msg, msg_len, "ice type %d of the spectrum has scheme %d, not %d", ty, sp->ice_scheme[ty - 1], parm);
          return SOCGPU_I_ERR_FATAL;
        }
      } else {
        set_msg(msg, msg_len, "unknown condensed phase %d", ph); return SOCGPU_I_ERR_FATAL; }
      const int need = (parm == SOCGPU_IP_DROP_PADE_2 || parm == SOCGPU_IP_ICE_PADE_2_PHF) ? 16
                       : parm == SOCGPU_IP_ICE_FU_PHF ? 14 : 6;
      if (sp->n_cloud_parameter < need) {
        set_msg(msg, msg_len, "cloud scheme %d needs %d coefficients, the spectrum holds %d", parm, need,
                sp->n_cloud_parameter);
        return SOCGPU_I_ERR_RANGE;
      }
      if (cld->i_cloud_type[k] < 1 || cld->i_cloud_type[k] > cld->n_cloud_type) {
        set_msg(msg, msg_len, "component cloud type out of range"); return SOCGPU_I_ERR_RANGE; }
    }
    if (c->l_rescale && c->n_order_forward != 2) {
      set_msg(msg, msg_len, "McICA cloud optics need n_order_forward=2 (forward scattering k_scat g^2)");
      return SOCGPU_I_ERR_FATAL; }
  }
  return SOCGPU_I_NORMAL;
}

// Fill FluxParams from device pointers.
void fill_params(FluxParams &p, const socgpu_control *c, const socgpu_dimen *dm, const SpectrumEntry *sp,
                 const socgpu_atm *atm, const socgpu_cld *cld, const socgpu_aer *aer, const socgpu_bound *bd,
                 socgpu_radout *out, const double *weight_band_dev) {
  std::memset(&p, 0, sizeof(p));
  p.isolir = c->isolir; p.i_2stream = c->i_2stream; p.i_scatter_method = c->i_scatter_method;
  {
    // sum = A - omega (B g + C), diff = D (1 - omega), ksi_0 = K g / sec_0
    // (two_coeff_basic.F90:99-160, solar_coefficient_basic.F90:171-182)
    const float r3 = 1.7320508f;
    float a = 2.0f, b = 1.5f, cc = 0.5f, d = 2.0f, k = 1.5f;          // ip_pifm80
    switch (c->i_2stream) {
      case SOCGPU_IP_EDDINGTON: a = 1.5f; b = 1.5f; cc = 0.0f; d = 2.0f; break;
      case SOCGPU_IP_ELSASSER: a = 1.66f; b = 1.5f; cc = 0.0f; d = 1.66f; break;
      case SOCGPU_IP_DISCRETE_ORD: a = r3; b = r3; cc = 0.0f; d = r3; k = r3; break;
      case SOCGPU_IP_PIFM85: a = 2.0f; b = 1.5f; cc = 0.0f; d = 2.0f; break;
      case SOCGPU_IP_2S_TEST: a = 1.5f; b = 1.5f; cc = 0.0f; d = 1.5f; break;
      case SOCGPU_IP_HEMI_MEAN: a = 2.0f; b = 2.0f; cc = 0.0f; d = 2.0f; break;
      default: break;
    }
    p.scheme_f[0] = a; p.scheme_f[1] = b; p.scheme_f[2] = cc; p.scheme_f[3] = d; p.scheme_f[4] = k;
  }
  p.i_direct_tau = c->i_direct_tau; p.l_rescale = c->l_rescale; p.n_order_forward = c->n_order_forward;
  p.l_ir_source_quad = c->l_ir_source_quad; p.l_rayleigh = c->l_rayleigh; p.l_gas = c->l_gas;
  p.l_aerosol_mode = c->l_aerosol_mode && aer && aer->n_mode > 0; p.l_flux_div = c->l_flux_div;
  p.first_band = c->first_band; p.last_band = c->last_band;
  p.triple = triple_cloud(c->i_cloud);
  p.region = region_cloud(c->i_cloud);
  p.mcica = c->i_cloud == SOCGPU_IP_CLOUD_MCICA || p.region;
  p.solver_hogan = c->i_solver == SOCGPU_IP_SOLVER_MIX_DIRECT_HOGAN || c->i_solver == SOCGPU_IP_SOLVER_TRIPLE_HOGAN;
  // the correlation of like regions at an interface (overlap_coupled.F90:
  // 190-236): 1 under mix_max and triple, 0 under mix_random, and under the
  // partially correlated schemes exp(dp / dp_corr) with the clear region's
  // scale 1 Pa, the stratiform region's dp_corr_strat and the convective
  // region's dp_corr_conv
  p.corr_mode = (c->i_cloud == SOCGPU_IP_CLOUD_MIX_MAX || c->i_cloud == SOCGPU_IP_CLOUD_TRIPLE) ? 1
              : (c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR || c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR_CNV) ? 2 : 0;
  p.dp_corr[0] = 1.0;
  p.dp_corr[1] = cld ? cld->dp_corr_strat : 0.0;
  p.dp_corr[2] = cld ? cld->dp_corr_conv : 0.0;
  // aggregate_cloud (aggregate_cloud.F90:107-155): stratiform water and
  // ice then convective water and ice, or stratiform then convective
  for (int t = 0; t < 4; ++t) {
    const bool four = c->i_cloud_representation == SOCGPU_IP_CLOUD_CSIW ||
                      c->i_cloud_representation == SOCGPU_IP_CLOUD_SPLIT_ICE_WATER;
    p.type_region[t] = four ? (t < 2 ? 2 : 3) : (t == 0 ? 2 : 3);
  }
  p.l_continuum = c->l_continuum && sp->dev.has_continuum;
  p.l_mixing_ratio = c->l_mixing_ratio;
  p.i_water = sp->dev.index_water - 1;
  p.n_profile = atm->n_profile; p.n_layer = atm->n_layer;
  p.nd_profile = dm->nd_profile; p.nd_layer = dm->nd_layer;
  p.id_ct = (p.mcica ? dm->id_cloud_top : 1) - 1;
  p.keqv = is_keqv(c, sp);
  p.l_grey_single = c->l_grey_single;
  const int *first_g = p.keqv ? sp->dev.host_first_g_keqv : sp->dev.host_first_g;
  p.g_begin = first_g[c->first_band - 1];
  p.g_end = first_g[c->last_band];
  p.max_abs = 1;
  for (int b = c->first_band - 1; b < c->last_band; ++b)
    p.max_abs = std::max(p.max_abs, c->l_gas ? sp->bands_host[b].n_abs : 0);
  p.bands = p.keqv ? sp->dev.bands_keqv : sp->dev.bands;
  p.gpoints = p.keqv ? sp->dev.gpoints_keqv : sp->dev.gpoints;
  p.minor_terms = sp->dev.minor_terms;
  // lookup tables (staged per column only when a band of the range uses them)
  const SpectrumDev &sd = sp->dev;
  bool lk = false;
  if (c->l_gas && sd.has_lookup)
    for (int b = c->first_band - 1; b < c->last_band; ++b)
      for (int j = 0; j < sp->bands_host[b].n_abs; ++j)
        lk |= sp->bands_host[b].gas[j].i_scale_fnc == SOCGPU_IP_SCALE_LOOKUP;
  p.lk_on = lk;
  bool term = p.keqv;
  if (c->l_gas)
    for (int b = c->first_band - 1; b < c->last_band; ++b)
      for (int j = 0; j < sp->bands_host[b].n_abs; ++j)
        term |= sp->bands_host[b].gas[j].i_scale_k == SOCGPU_IP_SCALE_TERM;
  p.term_scr = term;
  p.lk_n_pre = sd.lk_n_pre; p.lk_n_tmp = sd.lk_n_tmp; p.lk_n_gf = sd.lk_n_gf; p.n_sb = lk ? sd.n_sb : 0;
  p.lk_grid = sd.lk_grid; p.lk_grid_f = sd.lk_grid_f; p.k_lookup = sd.k_lookup; p.k_lookup_f = sd.k_lookup_f;
  for (int q = 0; q < kMaxSb; ++q) { p.sb_species[q] = sd.sb_species[q]; p.sb_ratio_gas[q] = sd.sb_ratio_gas[q]; }
  p.ratio_water = sd.ratio_water; p.l_water = sd.l_water;
  p.nd_t_lookup_gas = sd.nd_t_lookup_gas; p.t_lookup_gas = sd.t_lookup_gas; p.t_lookup_gas_f = sd.t_lookup_gas_f;
  p.wenyi_n4 = sd.wenyi_n4; p.wenyi_n6 = sd.wenyi_n6; p.wenyi = sd.wenyi; p.wenyi_f = sd.wenyi_f;
  p.drop_parm = sp->dev.drop_parm; p.ice_parm = sp->dev.ice_parm;
  p.drop_parm_f = sp->dev.drop_parm_f; p.ice_parm_f = sp->dev.ice_parm_f;
  p.n_band = sp->dev.n_band; p.n_deg_fit = sp->dev.n_deg_fit; p.t_ref_planck = sp->dev.t_ref_planck;
  p.t_ref_planck_f = (float)sp->dev.t_ref_planck;
  p.weight_band = weight_band_dev;
  p.p = atm->p; p.t = atm->t; p.t_level = atm->t_level; p.mass = atm->mass; p.gas_mix_ratio = atm->gas_mix_ratio;
  p.density = atm->density;
  p.nd_species = sp->dev.n_species;
  p.zen_0 = bd->zen_0; p.solar_irrad = bd->solar_irrad; p.rho_alb = bd->rho_alb; p.t_ground = bd->t_ground;
  p.flux_ground = bd->flux_ground;
  if (p.l_aerosol_mode) {
    p.n_mode = aer->n_mode; p.nd_mode = dm->nd_aerosol_mode;
    p.mode_mix_ratio = aer->mode_mix_ratio; p.mode_absorption = aer->mode_absorption;
    p.mode_scattering = aer->mode_scattering; p.mode_asymmetry = aer->mode_asymmetry;
  }
  if (c->l_aerosol && aer && aer->n_aerosol_mr > 0 && !sp->aer_parm.empty()) {
    // the active entries, in order (opt_prop_aerosol.F90:273-283)
    for (int k = 0; k < aer->n_aerosol_mr && p.n_aer_mr < kMaxAerMr; ++k) {
      const int src = aer->mr_source ? aer->mr_source[k] : SOCGPU_IP_AERSRC_CLASSIC_RON;
      if (src < SOCGPU_IP_AERSRC_CUSACK_RON || src > SOCGPU_IP_AERSRC_ARCL_RON) continue;
      const int j = aer->mr_type_index[k] - 1;
      if (sp->aer_parm[j] == SOCGPU_IP_AEROSOL_UNPARAMETRIZED) {
        // prescribed: once per species, counted per entry
        int s = 0;
        while (s < p.n_prsc && p.prsc_species[s] != j) ++s;
        if (s == p.n_prsc) {
          p.prsc_species[s] = j;
          p.prsc_count[s] = 0;
          p.prsc_nlev[s] = aer->n_opt_level_prsc[j];
          ++p.n_prsc;
        }
        ++p.prsc_count[s];
        continue;
      }
      p.aer_entry[p.n_aer_mr] = k;
      p.aer_species[p.n_aer_mr] = j;
      p.aer_parm[p.n_aer_mr] = sp->aer_parm[j];
      ++p.n_aer_mr;
    }
    p.l_aerosol = p.n_aer_mr > 0;
    p.l_aer_prsc = p.n_prsc > 0;
    if (p.l_aer_prsc) {
      p.prsc_nq = (c->l_henyey_greenstein_pf || !c->l_rescale) ? 1 : std::max(1, c->n_order_forward);
      p.nd_prof_prsc = dm->nd_profile_aerosol_prsc;
      p.nd_lev_prsc = dm->nd_opt_level_aerosol_prsc;
      p.nd_phf_prsc = dm->nd_phf_term_aerosol_prsc;
      p.nd_sp_prsc = sp->aer_nd_species;
      p.prsc_p = aer->pressure_prsc; p.prsc_abs = aer->absorption_prsc;
      p.prsc_scat = aer->scattering_prsc; p.prsc_phf = aer->phase_fnc_prsc;
    }
    p.l_hg = c->l_henyey_greenstein_pf;
    p.aer_n_species = sp->dev.aer_n_species; p.aer_nh = sp->dev.aer_nh; p.aer_nphf = sp->dev.aer_nphf;
    // one humidity table for all moist species: that of the last one
    // (radiance_calc.F90:606-623)
    p.aer_nh_common = 0;
    for (size_t j = 0; j < sp->aer_parm.size(); ++j)
      if (sp->aer_parm[j] == SOCGPU_IP_AEROSOL_PARAM_MOIST || sp->aer_parm[j] == SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST)
        p.aer_nh_common = sp->aer_nhum[j];
    p.aer_dhum = p.aer_nh_common > 1 ? 1.0 / ((double)p.aer_nh_common - 1.0) : 0.0;
    p.aer_dhum_f = (float)p.aer_dhum;
    p.aer_mix_ratio = aer->mix_ratio;
    p.mean_rel_humidity = aer->mean_rel_humidity;
    p.aer_tab = sp->dev.aer_tab; p.aer_tab_f = sp->dev.aer_tab_f;
    p.aer_hum = sp->dev.aer_hum; p.aer_hum_f = sp->dev.aer_hum_f;
  }
  if (p.mcica) {
    p.n_condensed = cld->n_condensed; p.n_cloud_type = cld->n_cloud_type;
    for (int k = 0; k < cld->n_condensed; ++k) {
      p.comp_type[k] = cld->i_cloud_type[k];
      p.comp_phase[k] = condensed_phase(cld->type_condensed[k]);
      p.comp_parm_index[k] = cld->i_condensed_type[k] - 1;
      p.comp_scheme[k] = cld->i_condensed_param[k];
    }
    p.condensed_mix_ratio = cld->condensed_mix_ratio; p.condensed_dim_char = cld->condensed_dim_char;
    p.w_cloud = cld->w_cloud; p.frac_cloud = cld->frac_cloud; p.c_sub = cld->c_sub;
    p.frac_cloudy = cld->frac_cloudy; p.n_subcol_cld = cld->n_subcol_cld;
    p.subcol_k = cld->subcol_k; p.first_subcol_k = cld->first_subcol_k; p.subcol_reorder = cld->subcol_reorder;
    p.n_subcol_gen = p.region ? 0 : cld->n_subcol_gen;
    p.n_subcol_req = p.region ? 0 : cld->n_subcol_req;
    p.nd_band_sp = sp->dev.nd_band;
  }
  p.flux_up = out->flux_up; p.flux_down = out->flux_down;
  p.flux_direct = c->isolir == SOCGPU_IP_SOLAR ? out->flux_direct : nullptr;
  p.flux_div = out->flux_div; p.heating_rate = out->heating_rate;
}

int mode_index(const socgpu_control *c) {
  // McICA and cloud regions share the kernels that stage cloud optics
  if (c->i_cloud == SOCGPU_IP_CLOUD_MCICA || region_cloud(c->i_cloud))
    return 2;
  return c->i_scatter_method == SOCGPU_IP_SCATTER_FULL ? 1 : 0;
}

namespace {
int launch_flux(const FluxParams &p, const socgpu_control *c, cudaStream_t st, char *msg, size_t msg_len);
}

int launch(const FluxParams &p, const socgpu_control *c, cudaStream_t st, char *msg, size_t msg_len) {
  if (!p.l_aer_prsc) return launch_flux(p, c, st, msg, msg_len);
  // prescribed aerosol properties: their per-layer sums in stream-ordered
  // scratch memory, then the flux kernel
  void *scratch = nullptr;
  if (cudaMallocAsync(&scratch, std::max<size_t>(prsc_bytes(p), 256), st) != cudaSuccess) {
    cudaGetLastError();
    set_msg(msg, msg_len, "no device memory for the prescribed aerosol properties");
    return SOCGPU_I_ABORT_CALCULATION;
  }
  FluxParams q = p;
  q.aer_prsc = (const double *)scratch;
  int st_ = launch_prsc(q, (double *)scratch, st, msg, msg_len);
  if (st_ == SOCGPU_I_NORMAL) st_ = launch_flux(q, c, st, msg, msg_len);
  cudaFreeAsync(scratch, st);
  return st_;
}

namespace {
int launch_flux(const FluxParams &p, const socgpu_control *c, cudaStream_t st, char *msg, size_t msg_len) {
  const int mode = mode_index(c);
  TileConfig t = choose_tile(c->precision, mode, p.n_layer);
  // options the phased kernel does not cover run on the scan kernels
  if (t.lanes_per_solve == 1 && !phased_supported(p)) t = scan_tile(c->precision, p.n_layer);
  const FluxVariant *v = find_variant(c->precision, mode, t.lanes_per_solve);
  if (v && t.lanes_per_solve == 1) return v->launch(p, t, st, msg, msg_len);
  if (!v || t.chunk == 0) {
    set_msg(msg, msg_len, "no kernel built for %d lanes per solve and %d layers", t.lanes_per_solve, p.n_layer);
    return SOCGPU_I_ERR_RANGE;
  }
  return v->launch(p, t, st, msg, msg_len);
}
}  // namespace

// ---------------------------------------------------------------------------
// Staging of a host-pointer call.
void StagedCall::stage(const socgpu_control *c, const socgpu_dimen *dm, const SpectrumEntry *s, const socgpu_atm *a,
                       const socgpu_cld *cl, const socgpu_aer *ae, const socgpu_bound *b, socgpu_radout *r) {
  control = c; dimen = dm; sp = s; atm = a; cld = cl; aer = ae; bound = b; radout = r;
  plan = Plan{};
  const size_t ndp = dm->nd_profile, ndl = dm->nd_layer, np = a->n_profile, nl = a->n_layer;
  const size_t nb = s->dev.n_band, ns = std::max(1, s->dev.n_species);
  sw = c->isolir == SOCGPU_IP_SOLAR;
  mc = c->i_cloud == SOCGPU_IP_CLOUD_MCICA || region_cloud(c->i_cloud);
  aero = c->l_aerosol_mode && ae && ae->n_mode > 0;
  const size_t D = sizeof(double), none = (size_t)-1;
  // inputs: (nd_profile, rows) arrays copied with their valid profiles only;
  // t_level feeds only the infra-red Planck terms, t_ground only the IR surface
  o_p = plan.add(a->p, D, ndp, np, nl);
  o_t = plan.add(a->t, D, ndp, np, nl);
  o_tl = !sw ? plan.add(a->t_level, D, ndp, np, nl + 1) : none;
  o_m = plan.add(a->mass, D, ndp, np, nl);
  const bool cont = c->l_continuum && s->dev.has_continuum;
  o_g = (c->l_gas || cont) ? plan.add(a->gas_mix_ratio, D, ndp, np, ndl * ns) : none;
  // prescribed aerosol properties: species whose spectral parametrization is
  // unparametrized, named by an active entry
  prsc = false;
  if (c->l_aerosol && ae && ae->n_aerosol_mr > 0 && ae->mr_type_index)
    for (int k = 0; k < ae->n_aerosol_mr; ++k) {
      const int src = ae->mr_source ? ae->mr_source[k] : SOCGPU_IP_AERSRC_CLASSIC_RON;
      const int j = ae->mr_type_index[k] - 1;
      if (src >= SOCGPU_IP_AERSRC_CUSACK_RON && src <= SOCGPU_IP_AERSRC_ARCL_RON && j >= 0 &&
          j < (int)s->aer_parm.size() && s->aer_parm[j] == SOCGPU_IP_AEROSOL_UNPARAMETRIZED)
        prsc = true;
    }
  o_rho = (cont || prsc) ? plan.add(a->density, D, ndp, np, nl) : none;
  o_z = sw ? plan.add(b->zen_0, D, ndp, np, 1) : none;
  o_si = sw ? plan.add(b->solar_irrad, D, ndp, np, 1) : none;
  o_alb = plan.add(b->rho_alb, D, ndp, np, 2 * nb);
  o_tg = !sw ? plan.add(b->t_ground, D, ndp, np, 1) : none;
  o_fg = !sw ? plan.add(b->flux_ground, D, ndp, np, nb) : none;
  o_amr = o_aab = o_asc = o_aas = none;
  const size_t ndm = dm->nd_aerosol_mode;
  if (aero) {
    o_amr = plan.add(ae->mode_mix_ratio, D, ndp, np, ndl * ndm);
    o_aab = plan.add(ae->mode_absorption, D, ndp, np, ndl * ndm * nb);
    o_asc = plan.add(ae->mode_scattering, D, ndp, np, ndl * ndm * nb);
    o_aas = plan.add(ae->mode_asymmetry, D, ndp, np, ndl * ndm * nb);
  }
  // classic aerosol: the mixing ratios of every entry, and the humidity
  o_xmr = o_mrh = none;
  classic = c->l_aerosol && ae && ae->n_aerosol_mr > 0 && ae->mix_ratio;
  if (classic) {
    o_xmr = plan.add(ae->mix_ratio, D, ndp, np, ndl * (size_t)ae->n_aerosol_mr);
    if (ae->mean_rel_humidity) o_mrh = plan.add(ae->mean_rel_humidity, D, ndp, np, nl);
  }
  o_pp = o_pab = o_psc = o_pph = none;
  if (prsc) {
    const size_t ndpp = dm->nd_profile_aerosol_prsc, nlv = dm->nd_opt_level_aerosol_prsc;
    const size_t nsp = s->aer_nd_species, nph = dm->nd_phf_term_aerosol_prsc, ndb = s->dev.nd_band;
    o_pp = plan.add(ae->pressure_prsc, D, ndpp, np, nlv * nsp);
    o_pab = plan.add(ae->absorption_prsc, D, ndpp, np, nlv * nsp * ndb);
    o_psc = plan.add(ae->scattering_prsc, D, ndpp, np, nlv * nsp * ndb);
    o_pph = plan.add(ae->phase_fnc_prsc, D, ndpp, np, nlv * nph * nsp * ndb);
  }
  o_wb = c->weight_band ? plan.add(c->weight_band, D, nb, nb, 1, false, nullptr, false) : none;
  o_cmr = o_cdc = o_wc = o_fc = o_cs = o_fcl = o_nsc = o_sk = o_fsk = o_sro = none;
  if (mc) {
    const size_t ndc = ndl - (dm->id_cloud_top - 1);
    const size_t ncc = std::max(1, dm->nd_cloud_component), nct = std::max(1, dm->nd_cloud_type);
    o_cmr = plan.add(cl->condensed_mix_ratio, D, ndp, np, ndc * ncc);
    o_cdc = plan.add(cl->condensed_dim_char, D, ndp, np, ndc * ncc);
    o_wc = plan.add(cl->w_cloud, D, ndp, np, ndc);
    o_fc = plan.add(cl->frac_cloud, D, ndp, np, ndc * nct);
    o_cs = plan.add(cl->c_sub, D, ndp, np, ndc * cl->n_subcol_gen);
    o_fcl = plan.add(cl->frac_cloudy, D, ndp, np, 1);
    if (cl->n_subcol_cld) o_nsc = plan.add(cl->n_subcol_cld, sizeof(int), ndp, np, 1);
    const size_t ndb = s->dev.nd_band, ndk = s->dev.nd_k_term;
    o_sk = plan.add(cl->subcol_k, sizeof(int), ndb * ndk, ndb * ndk, 1, false, nullptr, false);
    o_fsk = plan.add(cl->first_subcol_k, sizeof(int), ndb * (ndk + 1), ndb * (ndk + 1), 1, false, nullptr, false);
    o_sro = plan.add(cl->subcol_reorder, sizeof(int), cl->n_subcol_req, cl->n_subcol_req, 1, false, nullptr, false);
  }
  n_inputs = plan.slots.size();
  o_fu = plan.add(nullptr, D, ndp, np, nl + 1, true, r->flux_up);
  o_fd = plan.add(nullptr, D, ndp, np, nl + 1, true, r->flux_down);
  o_fdir = (sw && r->flux_direct) ? plan.add(nullptr, D, ndp, np, nl + 1, true, r->flux_direct) : none;
  o_div = r->flux_div ? plan.add(nullptr, D, ndp, np, nl, true, r->flux_div) : none;
  o_hr = r->heating_rate ? plan.add(nullptr, D, ndp, np, nl, true, r->heating_rate) : none;
}

int StagedCall::copy_in(char *base, cudaStream_t s, char *msg, size_t msg_len) const {
  for (size_t k = 0; k < n_inputs; ++k) {
    const Slot &sl = plan.slots[k];
    if (sl.row_bytes == 0) continue;
    CUDA_TRY(cudaMemcpy2DAsync(base + sl.off, sl.dev_pitch, sl.host, sl.host_pitch, sl.row_bytes, sl.rows,
                               cudaMemcpyHostToDevice, s));
  }
  return SOCGPU_I_NORMAL;
}

int StagedCall::copy_out(char *base, cudaStream_t s, char *msg, size_t msg_len) const {
  for (size_t k = n_inputs; k < plan.slots.size(); ++k) {
    const Slot &sl = plan.slots[k];
    if (sl.row_bytes == 0) continue;
    CUDA_TRY(cudaMemcpy2DAsync(sl.out_host, sl.host_pitch, base + sl.off, sl.dev_pitch, sl.row_bytes, sl.rows,
                               cudaMemcpyDeviceToHost, s));
  }
  return SOCGPU_I_NORMAL;
}

int StagedCall::copy_in_window(char *base, cudaStream_t s, size_t c0, size_t n, bool shared, char *msg,
                               size_t msg_len) const {
  for (size_t k = 0; k < n_inputs; ++k) {
    const Slot &sl = plan.slots[k];
    if (sl.row_bytes == 0) continue;
    if (!sl.per_profile) {
      if (shared)
        CUDA_TRY(cudaMemcpy2DAsync(base + sl.off, sl.dev_pitch, sl.host, sl.host_pitch, sl.row_bytes, sl.rows,
                                   cudaMemcpyHostToDevice, s));
      continue;
    }
    const size_t es = sl.row_bytes / (size_t)atm->n_profile;   // element size
    if (n == 0) continue;
    CUDA_TRY(cudaMemcpy2DAsync(base + sl.off + c0 * es, sl.dev_pitch, (const char *)sl.host + c0 * es, sl.host_pitch,
                               n * es, sl.rows, cudaMemcpyHostToDevice, s));
  }
  return SOCGPU_I_NORMAL;
}

int StagedCall::copy_out_window(char *base, cudaStream_t s, size_t c0, size_t n, char *msg, size_t msg_len) const {
  for (size_t k = n_inputs; k < plan.slots.size(); ++k) {
    const Slot &sl = plan.slots[k];
    if (sl.row_bytes == 0 || n == 0) continue;
    const size_t es = sl.row_bytes / (size_t)atm->n_profile;
    CUDA_TRY(cudaMemcpy2DAsync((char *)sl.out_host + c0 * es, sl.host_pitch, base + sl.off + c0 * es, sl.dev_pitch,
                               n * es, sl.rows, cudaMemcpyDeviceToHost, s));
  }
  return SOCGPU_I_NORMAL;
}

void window_params(FluxParams &p, int c0, int n) {
  auto mv = [&](auto &ptr) { if (ptr) ptr += c0; };
  mv(p.p); mv(p.t); mv(p.t_level); mv(p.mass); mv(p.gas_mix_ratio); mv(p.density);
  mv(p.zen_0); mv(p.solar_irrad); mv(p.rho_alb); mv(p.t_ground); mv(p.flux_ground);
  mv(p.mode_mix_ratio); mv(p.mode_absorption); mv(p.mode_scattering); mv(p.mode_asymmetry);
  mv(p.aer_mix_ratio); mv(p.mean_rel_humidity);
  mv(p.prsc_p); mv(p.prsc_abs); mv(p.prsc_scat); mv(p.prsc_phf);
  mv(p.condensed_mix_ratio); mv(p.condensed_dim_char); mv(p.w_cloud); mv(p.frac_cloud);
  mv(p.c_sub); mv(p.frac_cloudy); mv(p.n_subcol_cld);
  mv(p.flux_up); mv(p.flux_down); mv(p.flux_direct); mv(p.flux_div); mv(p.heating_rate);
  p.n_profile = n;
}

void StagedCall::params(char *base, FluxParams &p) const {
  auto dptr = [&](size_t off) -> void * { return off == (size_t)-1 ? nullptr : (void *)(base + off); };
  socgpu_atm a2 = *atm;
  a2.p = (const double *)dptr(o_p); a2.t = (const double *)dptr(o_t); a2.t_level = (const double *)dptr(o_tl);
  a2.mass = (const double *)dptr(o_m); a2.gas_mix_ratio = (const double *)dptr(o_g); a2.p_level = nullptr;
  a2.density = (const double *)dptr(o_rho);
  socgpu_bound b2 = *bound;
  b2.zen_0 = (const double *)dptr(o_z); b2.solar_irrad = (const double *)dptr(o_si);
  b2.rho_alb = (const double *)dptr(o_alb); b2.t_ground = (const double *)dptr(o_tg);
  b2.flux_ground = (const double *)dptr(o_fg);
  socgpu_aer e2{};
  if (aero || classic) {
    e2 = *aer;    // the entries' species and sources stay host arrays
    e2.mode_mix_ratio = (const double *)dptr(o_amr); e2.mode_absorption = (const double *)dptr(o_aab);
    e2.mode_scattering = (const double *)dptr(o_asc); e2.mode_asymmetry = (const double *)dptr(o_aas);
    if (!aero) e2.n_mode = 0;
    e2.mix_ratio = (const double *)dptr(o_xmr);
    e2.mean_rel_humidity = (const double *)dptr(o_mrh);
    e2.pressure_prsc = (const double *)dptr(o_pp); e2.absorption_prsc = (const double *)dptr(o_pab);
    e2.scattering_prsc = (const double *)dptr(o_psc); e2.phase_fnc_prsc = (const double *)dptr(o_pph);
  }
  socgpu_cld c2{};
  if (mc) {
    c2 = *cld;
    c2.condensed_mix_ratio = (const double *)dptr(o_cmr); c2.condensed_dim_char = (const double *)dptr(o_cdc);
    c2.w_cloud = (const double *)dptr(o_wc); c2.frac_cloud = (const double *)dptr(o_fc);
    c2.c_sub = (const double *)dptr(o_cs); c2.frac_cloudy = (const double *)dptr(o_fcl);
    c2.n_subcol_cld = (const int *)dptr(o_nsc);
    c2.subcol_k = (const int *)dptr(o_sk); c2.first_subcol_k = (const int *)dptr(o_fsk);
    c2.subcol_reorder = (const int *)dptr(o_sro);
  }
  socgpu_radout r2{};
  r2.flux_up = (double *)dptr(o_fu); r2.flux_down = (double *)dptr(o_fd);
  r2.flux_direct = (double *)dptr(o_fdir); r2.flux_div = (double *)dptr(o_div);
  r2.heating_rate = (double *)dptr(o_hr);
  fill_params(p, control, dimen, sp, &a2, mc ? &c2 : nullptr, (aero || classic) ? &e2 : nullptr, &b2, &r2,
              (const double *)dptr(o_wb));
}

long long StagedCall::column_gpoints() const {
  const int *first_g = is_keqv(control, sp) ? sp->dev.host_first_g_keqv : sp->dev.host_first_g;
  const int g0 = first_g[control->first_band - 1], g1 = first_g[control->last_band];
  return (long long)atm->n_profile * (g1 - g0);
}

namespace {

// ---------------------------------------------------------------------------
// Per-thread device workspace for the host-pointer entry points.
// The host-pointer call pipelines column chunks over kPipe streams: the
// inputs of one chunk copy in while another computes and a third copies out.
constexpr int kPipe = 3;
struct Workspace {
  int device = -1;
  cudaStream_t stream = nullptr;
  cudaStream_t aux[kPipe - 1] = {};
  cudaEvent_t shared_done = nullptr;
  void *buf = nullptr;
  size_t cap = 0;
  char *pinned = nullptr;          // page-locked staging for pageable caller arrays
  size_t pinned_cap = 0;
  int *range = nullptr;
  std::vector<cudaEvent_t> events;  // per-chunk hand-offs of the pinned pipeline
  ~Workspace() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    if (pinned) cudaFreeHost(pinned);
    if (buf) cudaFree(buf);
    if (range) cudaFree(range);
    if (stream) cudaStreamDestroy(stream);
    for (cudaStream_t a : aux)
      if (a) cudaStreamDestroy(a);
    if (shared_done) cudaEventDestroy(shared_done);
  }
};
thread_local Workspace tl_ws;

int ensure_workspace(size_t bytes, char *msg, size_t msg_len) {
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (tl_ws.device != dev) {
    if (tl_ws.buf) cudaFree(tl_ws.buf);
    if (tl_ws.range) cudaFree(tl_ws.range);
    tl_ws.buf = nullptr; tl_ws.cap = 0; tl_ws.range = nullptr;
    if (tl_ws.stream) cudaStreamDestroy(tl_ws.stream);
    tl_ws.stream = nullptr;
    for (cudaStream_t &a : tl_ws.aux) {
      if (a) cudaStreamDestroy(a);
      a = nullptr;
    }
    if (tl_ws.shared_done) cudaEventDestroy(tl_ws.shared_done);
    tl_ws.shared_done = nullptr;
    for (cudaEvent_t e : tl_ws.events) cudaEventDestroy(e);
    tl_ws.events.clear();
    CUDA_TRY(cudaStreamCreateWithFlags(&tl_ws.stream, cudaStreamNonBlocking));
    for (cudaStream_t &a : tl_ws.aux) CUDA_TRY(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&tl_ws.shared_done, cudaEventDisableTiming));
    CUDA_TRY(cudaMalloc(&tl_ws.range, 2 * sizeof(int)));
    tl_ws.device = dev;
  }
  if (bytes > tl_ws.cap) {
    if (tl_ws.buf) CUDA_TRY(cudaFree(tl_ws.buf));
    tl_ws.buf = nullptr;
    size_t want = bytes + bytes / 4;
    CUDA_TRY(cudaMalloc(&tl_ws.buf, want));
    tl_ws.cap = want;
  }
  return SOCGPU_I_NORMAL;
}

// Bytes of one column chunk of the host-pointer pipeline: 24 MB unless the
// environment variable SOCGPU_CHUNK_MB sets another size (a tuning knob,
// read once).
size_t pipeline_chunk_bytes() {
  static const size_t bytes = [] {
    const char *e = std::getenv("SOCGPU_CHUNK_MB");
    const long mb = e ? std::atol(e) : 0;
    return (size_t)(mb > 0 ? mb : 24) << 20;
  }();
  return bytes;
}

// Host-pointer call from pageable caller arrays: column chunks are packed
// into page-locked staging (one region per stream, reused once the stream's
// previous chunk is done), copied in, computed and copied out; the results
// are unpacked into the caller's arrays after the chunk's stream is synchronised.
int staged_radiance_calc(const StagedCall &call, const socgpu_control *control, char *base,
                         cudaStream_t *streams, char *msg, size_t msg_len) {
  const size_t np = (size_t)call.atm->n_profile;
  const auto &slots = call.plan.slots;
  // the arrays shared by all columns (small): synchronous copies
  for (size_t k = 0; k < call.n_inputs; ++k) {
    const Slot &sl = slots[k];
    if (sl.per_profile || sl.row_bytes == 0) continue;
    CUDA_TRY(cudaMemcpy2D(base + sl.off, sl.dev_pitch, sl.host, sl.host_pitch, sl.row_bytes, sl.rows,
                          cudaMemcpyHostToDevice));
  }
  size_t per_col = 0;
  for (const Slot &sl : slots)
    if (sl.per_profile && sl.row_bytes) per_col += sl.rows * (sl.row_bytes / np);
  const size_t target = std::max<size_t>(pipeline_chunk_bytes(), (size_t)64 << 20);
  size_t cols = std::max<size_t>(256, target / std::max<size_t>(per_col, 1));
  cols = std::min(cols, np);
  const size_t region = (cols * per_col + 255) & ~(size_t)255;
  if (tl_ws.pinned_cap < region * kPipe) {
    if (tl_ws.pinned) cudaFreeHost(tl_ws.pinned);
    tl_ws.pinned = nullptr;
    tl_ws.pinned_cap = 0;
    CUDA_TRY(cudaMallocHost((void **)&tl_ws.pinned, region * kPipe));
    tl_ws.pinned_cap = region * kPipe;
  }
  FluxParams p;
  call.params(base, p);
  const size_t n_chunk = (np + cols - 1) / cols;
  std::vector<size_t> chunk_c0(n_chunk), chunk_n(n_chunk);
  auto unpack = [&](size_t k) {
    char *r = tl_ws.pinned + region * (k % kPipe);
    const size_t c0 = chunk_c0[k], n = chunk_n[k];
    size_t pos = 0;
    for (const Slot &sl : slots) {
      if (!sl.per_profile || sl.row_bytes == 0) continue;
      const size_t es = sl.row_bytes / np, w = n * es;
      if (sl.output)
        for (size_t row = 0; row < sl.rows; ++row)
          std::memcpy((char *)sl.out_host + c0 * es + row * sl.host_pitch, r + pos + row * w, w);
      pos += sl.rows * w;
    }
  };
  for (size_t k = 0; k < n_chunk; ++k) {
    const size_t c0 = k * cols, n = std::min(cols, np - c0);
    chunk_c0[k] = c0;
    chunk_n[k] = n;
    cudaStream_t sk = streams[k % kPipe];
    if (k >= (size_t)kPipe) {        // the region's previous chunk must be done and unpacked
      CUDA_TRY(cudaStreamSynchronize(sk));
      unpack(k - kPipe);
    }
    char *r = tl_ws.pinned + region * (k % kPipe);
    size_t pos = 0;
    for (const Slot &sl : slots) {
      if (!sl.per_profile || sl.row_bytes == 0) continue;
      const size_t es = sl.row_bytes / np, w = n * es;
      if (!sl.output) {
        for (size_t row = 0; row < sl.rows; ++row)
          std::memcpy(r + pos + row * w, (const char *)sl.host + c0 * es + row * sl.host_pitch, w);
        CUDA_TRY(cudaMemcpy2DAsync(base + sl.off + c0 * es, sl.dev_pitch, r + pos, w, w, sl.rows,
                                   cudaMemcpyHostToDevice, sk));
      }
      pos += sl.rows * w;
    }
    FluxParams pk = p;
    window_params(pk, (int)c0, (int)n);
    int st = launch(pk, control, sk, msg, msg_len);
    if (st != SOCGPU_I_NORMAL) return st;
    pos = 0;
    for (const Slot &sl : slots) {
      if (!sl.per_profile || sl.row_bytes == 0) continue;
      const size_t es = sl.row_bytes / np, w = n * es;
      if (sl.output)
        CUDA_TRY(cudaMemcpy2DAsync(r + pos, w, base + sl.off + c0 * es, sl.dev_pitch, w, sl.rows,
                                   cudaMemcpyDeviceToHost, sk));
      pos += sl.rows * w;
    }
  }
  for (size_t k = (n_chunk > (size_t)kPipe ? n_chunk - kPipe : 0); k < n_chunk; ++k) {
    CUDA_TRY(cudaStreamSynchronize(streams[k % kPipe]));
    unpack(k);
  }
  return SOCGPU_I_NORMAL;
}

}  // namespace
}  // namespace socgpu

using namespace socgpu;

// ---------------------------------------------------------------------------
// Multi-batch launches (socgpu_batch_*): the batches are grouped into kernel
// classes (precision, mode, tile); each class runs as one persistent launch
// over all its columns, and the launches are captured in one CUDA graph.
struct socgpu_batch_s {
  int device = 0;
  std::vector<FluxParams> params;      // one per batch
  std::vector<int> precision, mode;
  std::vector<BatchGroup> groups;
  std::vector<std::vector<FluxParams>> group_items;
  std::vector<std::vector<long long>> group_start;
  std::vector<FluxParams *> d_items;
  std::vector<long long *> d_start;
  char *dbuf = nullptr;
  cudaStream_t capture = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long n_columns = 0, n_colg = 0;
  ~socgpu_batch_s() {
    if (exec) cudaGraphExecDestroy(exec);
    if (dbuf) cudaFree(dbuf);
    if (capture) cudaStreamDestroy(capture);
  }
};

namespace {

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// One group (kernel class) over the given batches with tile t: items copied,
// column offsets, then the variant's prepare step.
int make_group(socgpu_batch_s &b, const std::vector<int> &idx, int precision, int mode, const TileConfig &t,
               BatchGroup &g, std::vector<FluxParams> &items, std::vector<long long> &start, char *msg,
               size_t msg_len) {
  const FluxVariant *v = find_variant(precision, mode, t.lanes_per_solve);
  if (!v) { set_msg(msg, msg_len, "no kernel built for %d lanes per solve", t.lanes_per_solve); return SOCGPU_I_ERR_RANGE; }
  items.clear();
  start.assign(1, 0);
  for (int i : idx) {
    if (b.params[i].l_aer_prsc) {
      set_msg(msg, msg_len, "batch %d: prescribed aerosol properties run through socgpu_radiance_calc and "
                            "socgpu_radiance_calc_device, not multi-batch launches", i);
      return SOCGPU_I_ERR_FATAL;
    }
    items.push_back(b.params[i]);
    start.push_back(start.back() + b.params[i].n_profile);
  }
  g = BatchGroup{};
  g.precision = precision; g.mode = mode; g.tile = t;
  g.items = items.data(); g.col_start = start.data();
  g.n_items = (int)items.size(); g.total = start.back();
  return v->prepare(g, msg, msg_len);
}

// Copy groups' tables to one device buffer (device pointers returned per group).
int upload_groups(std::vector<BatchGroup> &groups, char *&dbuf, std::vector<FluxParams *> &d_items,
                  std::vector<long long *> &d_start, char *msg, size_t msg_len) {
  size_t bytes = 0;
  for (const BatchGroup &g : groups)
    bytes += align256(sizeof(FluxParams) * g.n_items) + align256(sizeof(long long) * (g.n_items + 1));
  if (dbuf) { cudaFree(dbuf); dbuf = nullptr; }
  CUDA_TRY(cudaMalloc(&dbuf, std::max<size_t>(bytes, 256)));
  size_t off = 0;
  d_items.clear(); d_start.clear();
  for (const BatchGroup &g : groups) {
    FluxParams *di = (FluxParams *)(dbuf + off);
    off += align256(sizeof(FluxParams) * g.n_items);
    long long *ds = (long long *)(dbuf + off);
    off += align256(sizeof(long long) * (g.n_items + 1));
    CUDA_TRY(cudaMemcpy(di, g.items, sizeof(FluxParams) * g.n_items, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(ds, g.col_start, sizeof(long long) * (g.n_items + 1), cudaMemcpyHostToDevice));
    d_items.push_back(di);
    d_start.push_back(ds);
  }
  return SOCGPU_I_NORMAL;
}

// `count`: a real launch (not one recorded into a graph).
int launch_group(const BatchGroup &g, FluxParams *di, long long *ds, cudaStream_t st, bool count = true) {
  if (g.total <= 0) return 0;
  int n_items = g.n_items;
  long long total = g.total;
  void *args[] = {&di, &ds, &n_items, &total};
  cudaError_t e = cudaLaunchKernel(g.kernel, dim3(g.grid), dim3(g.threads), args, g.smem, st);
  if (count) count_launch();
  return e == cudaSuccess ? 0 : -1;
}

// Group the batches by the tile each one is given (tuner table, overrides or
// heuristic), prepare, upload and capture the graph.
int build_plan(socgpu_batch_s &b, char *msg, size_t msg_len) {
  std::map<std::tuple<int, int, int, int, int, int>, std::vector<int>> classes;
  for (size_t i = 0; i < b.params.size(); ++i) {
    TileConfig t = choose_tile(b.precision[i], b.mode[i], b.params[i].n_layer);
    // the phased kernel has no persistent multi-batch form
    if (t.lanes_per_solve == 1) t = scan_tile(b.precision[i], b.params[i].n_layer);
    classes[std::make_tuple(b.precision[i], b.mode[i], t.lanes_per_solve, t.chunk, t.warps_per_cta,
                            b.params[i].isolir)].push_back((int)i);
  }
  b.groups.assign(classes.size(), BatchGroup{});
  b.group_items.assign(classes.size(), {});
  b.group_start.assign(classes.size(), {});
  size_t k = 0;
  for (auto &kv : classes) {
    TileConfig t{std::get<2>(kv.first), std::get<4>(kv.first), std::get<3>(kv.first)};
    int st = make_group(b, kv.second, std::get<0>(kv.first), std::get<1>(kv.first), t, b.groups[k],
                        b.group_items[k], b.group_start[k], msg, msg_len);
    if (st != SOCGPU_I_NORMAL) return st;
    ++k;
  }
  int st = upload_groups(b.groups, b.dbuf, b.d_items, b.d_start, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  if (b.exec) { cudaGraphExecDestroy(b.exec); b.exec = nullptr; }
  CUDA_TRY(cudaStreamBeginCapture(b.capture, cudaStreamCaptureModeThreadLocal));
  int bad = 0;
  for (size_t g = 0; g < b.groups.size(); ++g) bad |= launch_group(b.groups[g], b.d_items[g], b.d_start[g], b.capture, false);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(b.capture, &graph);
  if (bad || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    set_msg(msg, msg_len, "capture of the batch launches failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  e = cudaGraphInstantiate(&b.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_msg(msg, msg_len, "graph instantiation failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return SOCGPU_I_NORMAL;
}

}  // namespace

extern "C" {

int socgpu_abi_version(void) { return SOCGPU_ABI_VERSION; }

long long socgpu_kernel_launch_count(void) { return g_launches.load(); }

int socgpu_set_device(int device) { return cudaSetDevice(device) == cudaSuccess ? SOCGPU_I_NORMAL : SOCGPU_I_ERR_FATAL; }

int socgpu_set_tile_config(int precision, int mode, int lanes_per_solve, int warps_per_cta) {
  if (precision < 0 || precision > 1 || mode < 0 || mode > 2) return SOCGPU_I_ERR_RANGE;
  if (lanes_per_solve != 0 && lanes_per_solve != 1 && lanes_per_solve != 8 && lanes_per_solve != 16 &&
      lanes_per_solve != 32)
    return SOCGPU_I_ERR_RANGE;
  if (precision == SOCGPU_PRECISION_FP64 && lanes_per_solve == 8) return SOCGPU_I_ERR_RANGE;
  if (lanes_per_solve == 1 && mode == 2) return SOCGPU_I_ERR_RANGE;   // the phased kernel is clear-sky only
  if (warps_per_cta < 0 || warps_per_cta > 8) return SOCGPU_I_ERR_RANGE;
  std::lock_guard<std::mutex> lk(g_tile_mutex);
  g_tile[precision][mode][0] = lanes_per_solve;
  g_tile[precision][mode][1] = warps_per_cta;
  return SOCGPU_I_NORMAL;
}

int socgpu_spectrum_register(const char *name, const socgpu_spectrum_desc *desc, socgpu_spectrum_handle *handle,
                             char *msg, size_t msg_len) {
  if (!name || !desc || !handle) { set_msg(msg, msg_len, "null argument"); return SOCGPU_I_ERR_FATAL; }
  {
    std::lock_guard<std::mutex> lk(g_reg_mutex);
    auto it = g_names.find(name);
    if (it != g_names.end()) { *handle = it->second; return SOCGPU_I_NORMAL; }
  }
  auto e = std::make_unique<SpectrumEntry>();
  e->name = name;
  int st = build_spectrum(desc, *e, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) { free_spectrum(*e); return st; }
  std::lock_guard<std::mutex> lk(g_reg_mutex);
  auto it = g_names.find(name);
  if (it != g_names.end()) { free_spectrum(*e); *handle = it->second; return SOCGPU_I_NORMAL; }
  int h = g_next_handle++;
  g_names[name] = h;
  g_spectra[h] = std::move(e);
  *handle = h;
  return SOCGPU_I_NORMAL;
}

int socgpu_spectrum_lookup(const char *name, socgpu_spectrum_handle *handle) {
  if (!name || !handle) return SOCGPU_I_ERR_FATAL;
  std::lock_guard<std::mutex> lk(g_reg_mutex);
  auto it = g_names.find(name);
  if (it == g_names.end()) return SOCGPU_I_ERR_EXIST;
  *handle = it->second;
  return SOCGPU_I_NORMAL;
}

int socgpu_spectrum_n_gpoint(socgpu_spectrum_handle handle) {
  SpectrumEntry *e = find_spectrum(handle);
  return e ? e->dev.n_gpoint : -1;
}

int socgpu_spectrum_k_terms(socgpu_spectrum_handle handle, int n_band_max, int *n_band, int *nd_k_term,
                            int *n_k_major) {
  SpectrumEntry *e = find_spectrum(handle);
  if (!e) return SOCGPU_I_ERR_EXIST;
  if (n_band) *n_band = e->dev.n_band;
  if (nd_k_term) *nd_k_term = e->dev.nd_k_term;
  if (n_k_major)
    for (int b = 0; b < e->dev.n_band && b < n_band_max; ++b) n_k_major[b] = e->n_k_major[b];
  return SOCGPU_I_NORMAL;
}

int socgpu_spectrum_aerosols(socgpu_spectrum_handle handle, int n_max, int *n_aerosol, int *type_aerosol,
                             int *i_aerosol_parm, int *nhumidity) {
  SpectrumEntry *e = find_spectrum(handle);
  if (!e) return SOCGPU_I_ERR_EXIST;
  const int n = (int)e->aer_parm.size();
  if (n_aerosol) *n_aerosol = n;
  for (int j = 0; j < n && j < n_max; ++j) {
    if (type_aerosol) type_aerosol[j] = e->aer_type[j];
    if (i_aerosol_parm) i_aerosol_parm[j] = e->aer_parm[j];
    if (nhumidity) nhumidity[j] = e->aer_nhum[j];
  }
  return SOCGPU_I_NORMAL;
}

int socgpu_spectrum_set_aerosol_parm(socgpu_spectrum_handle handle, int species, int parm, char *msg,
                                     size_t msg_len) {
  SpectrumEntry *e = find_spectrum(handle);
  if (!e) { set_msg(msg, msg_len, "no spectrum with handle %d", handle); return SOCGPU_I_ERR_EXIST; }
  if (species < 1 || species > (int)e->aer_parm.size()) {
    set_msg(msg, msg_len, "aerosol species %d is not in the spectrum", species); return SOCGPU_I_ERR_RANGE; }
  if (parm != SOCGPU_IP_AEROSOL_UNPARAMETRIZED && parm != e->aer_parm_file[species - 1]) {
    set_msg(msg, msg_len, "aerosol species %d: parametrization %d is neither prescribed nor the file's %d", species,
            parm, e->aer_parm_file[species - 1]);
    return SOCGPU_I_ERR_RANGE;
  }
  std::lock_guard<std::mutex> lk(g_reg_mutex);
  e->aer_parm[species - 1] = parm;
  return SOCGPU_I_NORMAL;
}

int socgpu_spectrum_release(socgpu_spectrum_handle handle) {
  std::unique_ptr<SpectrumEntry> e;
  {
    std::lock_guard<std::mutex> lk(g_reg_mutex);
    auto it = g_spectra.find(handle);
    if (it == g_spectra.end()) return SOCGPU_I_ERR_EXIST;
    e = std::move(it->second);
    g_spectra.erase(it);
    g_names.erase(e->name);
  }
  cudaDeviceSynchronize();
  free_spectrum(*e);
  return SOCGPU_I_NORMAL;
}

int socgpu_radiance_calc_device(const socgpu_control *control, const socgpu_dimen *dimen,
                                socgpu_spectrum_handle spectrum, const socgpu_atm *atm, const socgpu_cld *cld,
                                const socgpu_aer *aer, const socgpu_bound *bound, socgpu_radout *radout,
                                void *stream, char *msg, size_t msg_len) {
  SpectrumEntry *sp = find_spectrum(spectrum);
  int st = validate(control, dimen, sp, atm, cld, aer, bound, radout, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  FluxParams p;
  fill_params(p, control, dimen, sp, atm, cld, aer, bound, radout, control->weight_band);
  return launch(p, control, (cudaStream_t)stream, msg, msg_len);
}

int socgpu_radiance_calc(const socgpu_control *control, const socgpu_dimen *dimen, socgpu_spectrum_handle spectrum,
                         const socgpu_atm *atm, const socgpu_cld *cld, const socgpu_aer *aer,
                         const socgpu_bound *bound, socgpu_radout *radout, char *msg, size_t msg_len) {
  SpectrumEntry *sp = find_spectrum(spectrum);
  int st = validate(control, dimen, sp, atm, cld, aer, bound, radout, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  if (atm->n_profile == 0) return SOCGPU_I_NORMAL;
  StagedCall call;
  call.stage(control, dimen, sp, atm, cld, aer, bound, radout);
  st = ensure_workspace(call.plan.bytes, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  char *base = (char *)tl_ws.buf;
  cudaStream_t streams[kPipe] = {tl_ws.stream, tl_ws.aux[0], tl_ws.aux[1]};
  auto sync_all = [&] {
    for (cudaStream_t x : streams) cudaStreamSynchronize(x);
  };
  // Caller arrays that are not page-locked never go to the copy engines
  // directly: they are packed chunk by chunk into page-locked staging.
  bool all_pinned = true;
  for (const Slot &sl : call.plan.slots) {
    const void *hp = sl.output ? sl.out_host : sl.host;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, hp) != cudaSuccess) { cudaGetLastError(); all_pinned = false; break; }
    if (at.type != cudaMemoryTypeHost) { all_pinned = false; break; }
  }
  if (!all_pinned) {
    st = staged_radiance_calc(call, control, base, streams, msg, msg_len);
    if (st != SOCGPU_I_NORMAL) sync_all();
    return st;
  }
  // Column chunks of about pipeline_chunk_bytes() (at least 256 columns).
  // Each stream has one role: the first copies every chunk in, back to back;
  // the second runs a chunk's kernel once its copy has landed; the third
  // copies a chunk's outputs back once its kernel is done.  Every column
  // has its own place in the workspace, so no chunk waits for a buffer and
  // the host link stays busy from the first copy to the last.
  const int np = atm->n_profile;
  size_t per_col = 0;
  for (const Slot &sl : call.plan.slots)
    if (sl.per_profile && sl.row_bytes) per_col += sl.rows * (sl.row_bytes / (size_t)np);
  const size_t want = std::max<size_t>(256, pipeline_chunk_bytes() / std::max<size_t>(per_col, 1));
  const int chunk = (int)std::min<size_t>((size_t)np, want);
  const int n_chunk = (np + chunk - 1) / chunk;
  while (tl_ws.events.size() < 2 * (size_t)n_chunk) {
    cudaEvent_t e = nullptr;
    CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    tl_ws.events.push_back(e);
  }
  cudaStream_t s_in = streams[0], s_run = streams[1], s_out = streams[2];
  // the arrays shared by all columns go first, ahead of chunk 0's columns
  st = call.copy_in_window(base, s_in, 0, 0, true, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) { sync_all(); return st; }
  FluxParams p;
  call.params(base, p);
  for (int k = 0; k < n_chunk; ++k) {
    const int c0 = k * chunk, n = std::min(chunk, np - c0);
    if (n <= 0) break;
    cudaEvent_t landed = tl_ws.events[2 * k], done = tl_ws.events[2 * k + 1];
    st = call.copy_in_window(base, s_in, c0, n, false, msg, msg_len);
    if (st != SOCGPU_I_NORMAL) { sync_all(); return st; }
    CUDA_TRY(cudaEventRecord(landed, s_in));
    CUDA_TRY(cudaStreamWaitEvent(s_run, landed, 0));
    FluxParams pk = p;
    window_params(pk, c0, n);
    st = launch(pk, control, s_run, msg, msg_len);
    if (st != SOCGPU_I_NORMAL) { sync_all(); return st; }
    CUDA_TRY(cudaEventRecord(done, s_run));
    CUDA_TRY(cudaStreamWaitEvent(s_out, done, 0));
    st = call.copy_out_window(base, s_out, c0, n, msg, msg_len);
    if (st != SOCGPU_I_NORMAL) { sync_all(); return st; }
  }
  for (cudaStream_t x : streams) CUDA_TRY(cudaStreamSynchronize(x));
  return SOCGPU_I_NORMAL;
}

int socgpu_cloud_gen_device(int nd_layer, int cloud_top, int n_layer, int nd_profile, int il1, int il2, int n_subcol,
                            int n1, int n2, int ipph, int ioverlap, const int *rand_seed, const double *rlc_cf,
                            const double *rlc_cw, const double *sigma_qcw, const double *avg_cf,
                            const double *c_cloud, const double *c_ratio, const double *zf, const double *xcw,
                            int *n_subcol_cld, double *c_sub, int rng, void *stream, char *msg, size_t msg_len) {
  if (ioverlap < 0 || ioverlap > 3) {
    set_msg(msg, msg_len, "Choice of overlap not compatible with cloud generator");
    return SOCGPU_I_ERR_FATAL;
  }
  if (rng != SOCGPU_RNG_LCG && rng != SOCGPU_RNG_PHILOX) { set_msg(msg, msg_len, "unknown rng %d", rng); return SOCGPU_I_ERR_FATAL; }
  if (cloud_top < 1 || n_layer > nd_layer || il1 < 1 || il2 > nd_profile || n_subcol < 1) {
    set_msg(msg, msg_len, "cloud_gen dimensions out of range"); return SOCGPU_I_ERR_RANGE; }
  if (ipph != 0 && (!xcw || !sigma_qcw || n1 < 2 || n2 < 2)) {
    set_msg(msg, msg_len, "ipph needs the xcw table and sigma_qcw"); return SOCGPU_I_ERR_FATAL; }
  if (!rand_seed || !rlc_cf || !rlc_cw || !avg_cf || !zf || !n_subcol_cld || !c_sub) {
    set_msg(msg, msg_len, "missing cloud_gen argument"); return SOCGPU_I_ERR_FATAL; }
  int st = ensure_workspace(1, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  return launch_cloud_gen(nd_layer, cloud_top, n_layer, nd_profile, il1, il2, n_subcol, n1, n2, ipph, ioverlap,
                          rand_seed, rlc_cf, rlc_cw, sigma_qcw, avg_cf, c_cloud, c_ratio, zf, xcw, n_subcol_cld,
                          c_sub, rng, tl_ws.range, (cudaStream_t)stream, msg, msg_len);
}

// Same checks as socgpu_cloud_gen_device, then the allocation-free launcher:
// no workspace, no allocation of any kind on this path.
int socgpu_cloud_gen_device_noalloc(int nd_layer, int cloud_top, int n_layer, int nd_profile, int il1, int il2,
                                    int n_subcol, int n1, int n2, int ipph, int ioverlap, const int *rand_seed,
                                    const double *rlc_cf, const double *rlc_cw, const double *sigma_qcw,
                                    const double *avg_cf, const double *c_cloud, const double *c_ratio,
                                    const double *zf, const double *xcw, int *n_subcol_cld, double *c_sub,
                                    int rng, void *stream, char *msg, size_t msg_len) {
  if (ioverlap < 0 || ioverlap > 3) {
    set_msg(msg, msg_len, "Choice of overlap not compatible with cloud generator");
    return SOCGPU_I_ERR_FATAL;
  }
  if (rng != SOCGPU_RNG_LCG && rng != SOCGPU_RNG_PHILOX) { set_msg(msg, msg_len, "unknown rng %d", rng); return SOCGPU_I_ERR_FATAL; }
  if (cloud_top < 1 || n_layer > nd_layer || il1 < 1 || il2 > nd_profile || n_subcol < 1) {
    set_msg(msg, msg_len, "cloud_gen dimensions out of range"); return SOCGPU_I_ERR_RANGE; }
  if (n_layer - cloud_top + 1 > SOCGPU_NOALLOC_MAX_CLOUD_LAYERS) {
    set_msg(msg, msg_len, "%d cloud layers exceed the allocation-free limit of %d (SOCGPU_NOALLOC_MAX_CLOUD_LAYERS)",
            n_layer - cloud_top + 1, SOCGPU_NOALLOC_MAX_CLOUD_LAYERS);
    return SOCGPU_I_ERR_RANGE;
  }
  if (ipph != 0 && (!xcw || !sigma_qcw || n1 < 2 || n2 < 2)) {
    set_msg(msg, msg_len, "ipph needs the xcw table and sigma_qcw"); return SOCGPU_I_ERR_FATAL; }
  if (!rand_seed || !rlc_cf || !rlc_cw || !avg_cf || !zf || !n_subcol_cld || !c_sub) {
    set_msg(msg, msg_len, "missing cloud_gen argument"); return SOCGPU_I_ERR_FATAL; }
  return launch_cloud_gen_noalloc(nd_layer, cloud_top, n_layer, nd_profile, il1, il2, n_subcol, n1, n2, ipph,
                                  ioverlap, rand_seed, rlc_cf, rlc_cw, sigma_qcw, avg_cf, c_cloud, c_ratio, zf, xcw,
                                  n_subcol_cld, c_sub, rng, (cudaStream_t)stream, msg, msg_len);
}

int socgpu_cloud_gen(int nd_layer, int cloud_top, int n_layer, int nd_profile, int il1, int il2, int n_subcol,
                     int n1, int n2, int ipph, int ioverlap, const int *rand_seed, const double *rlc_cf,
                     const double *rlc_cw, const double *sigma_qcw, const double *avg_cf, const double *c_cloud,
                     const double *c_ratio, const double *zf, const double *xcw, int *n_subcol_cld, double *c_sub,
                     int rng, char *msg, size_t msg_len) {
  if (cloud_top < 1 || n_layer > nd_layer || il1 < 1 || il2 > nd_profile || n_subcol < 1 || ioverlap < 0 || ioverlap > 3) {
    set_msg(msg, msg_len, "cloud_gen arguments out of range"); return SOCGPU_I_ERR_RANGE; }
  const size_t ndp = nd_profile, ndc = nd_layer - cloud_top + 1, D = sizeof(double);
  Plan plan;
  size_t o_seed = plan.add(rand_seed, sizeof(int), ndp, ndp, 1);
  size_t o_cf = plan.add(rlc_cf, D, ndp, ndp, ndc);
  size_t o_cw = plan.add(rlc_cw, D, ndp, ndp, ndc);
  size_t o_sq = sigma_qcw ? plan.add(sigma_qcw, D, ndp, ndp, ndc) : (size_t)-1;
  size_t o_av = plan.add(avg_cf, D, ndp, ndp, ndc);
  size_t o_cc = c_cloud ? plan.add(c_cloud, D, ndp, ndp, ndc) : (size_t)-1;
  size_t o_cr = c_ratio ? plan.add(c_ratio, D, ndp, ndp, ndc) : (size_t)-1;
  size_t o_zf = plan.add(zf, D, ndp, ndp, nd_layer);
  size_t o_x = (xcw && ipph != 0) ? plan.add(xcw, D, (size_t)n1, (size_t)n1, (size_t)n2) : (size_t)-1;
  const size_t n_inputs = plan.slots.size();
  size_t o_n = plan.add(nullptr, sizeof(int), ndp, ndp, 1, true, n_subcol_cld);
  size_t o_cs = plan.add(nullptr, D, ndp, ndp, ndc * n_subcol, true, c_sub);
  int st = ensure_workspace(plan.bytes, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  char *base = (char *)tl_ws.buf;
  cudaStream_t s = tl_ws.stream;
  for (size_t k = 0; k < n_inputs; ++k) {
    const Slot &sl = plan.slots[k];
    CUDA_TRY(cudaMemcpy2DAsync(base + sl.off, sl.dev_pitch, sl.host, sl.host_pitch, sl.row_bytes, sl.rows,
                               cudaMemcpyHostToDevice, s));
  }
  auto dptr = [&](size_t off) -> void * { return off == (size_t)-1 ? nullptr : (void *)(base + off); };
  st = socgpu_cloud_gen_device(nd_layer, cloud_top, n_layer, nd_profile, il1, il2, n_subcol, n1, n2, ipph, ioverlap,
                               (const int *)dptr(o_seed), (const double *)dptr(o_cf), (const double *)dptr(o_cw),
                               (const double *)dptr(o_sq),
                               (const double *)dptr(o_av),
                               (const double *)(o_cc == (size_t)-1 ? nullptr : dptr(o_cc)),
                               (const double *)(o_cr == (size_t)-1 ? nullptr : dptr(o_cr)),
                               (const double *)dptr(o_zf), (const double *)dptr(o_x), (int *)dptr(o_n),
                               (double *)dptr(o_cs), rng, s, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) { cudaStreamSynchronize(s); return st; }
  for (size_t k = n_inputs; k < plan.slots.size(); ++k) {
    const Slot &sl = plan.slots[k];
    CUDA_TRY(cudaMemcpy2DAsync(sl.out_host, sl.host_pitch, base + sl.off, sl.dev_pitch, sl.row_bytes, sl.rows,
                               cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  return SOCGPU_I_NORMAL;
}

int socgpu_batch_create(const socgpu_batch_item *items, int n_items, socgpu_batch *batch, char *msg,
                        size_t msg_len) {
  if (!items || n_items < 1 || !batch) { set_msg(msg, msg_len, "no batches"); return SOCGPU_I_ERR_FATAL; }
  std::unique_ptr<socgpu_batch_s> b(new socgpu_batch_s);
  CUDA_TRY(cudaGetDevice(&b->device));
  for (int i = 0; i < n_items; ++i) {
    const socgpu_batch_item &it = items[i];
    SpectrumEntry *sp = find_spectrum(it.spectrum);
    char sub[256] = "";
    int st = validate(it.control, it.dimen, sp, it.atm, it.cld, it.aer, it.bound, it.radout, sub, sizeof(sub));
    if (st != SOCGPU_I_NORMAL) { set_msg(msg, msg_len, "batch %d: %s", i, sub); return st; }
    FluxParams p;
    fill_params(p, it.control, it.dimen, sp, it.atm, it.cld, it.aer, it.bound, it.radout, it.control->weight_band);
    b->params.push_back(p);
    b->precision.push_back(it.control->precision);
    b->mode.push_back(mode_index(it.control));
    b->n_columns += p.n_profile;
    b->n_colg += (long long)p.n_profile * (p.g_end - p.g_begin);
  }
  CUDA_TRY(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
  int st = build_plan(*b, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  *batch = b.release();
  return SOCGPU_I_NORMAL;
}

int socgpu_batch_run(socgpu_batch batch, void *stream, char *msg, size_t msg_len) {
  if (!batch || !batch->exec) { set_msg(msg, msg_len, "invalid batch"); return SOCGPU_I_ERR_FATAL; }
  CUDA_TRY(cudaGraphLaunch(batch->exec, (cudaStream_t)stream));
  for (const BatchGroup &g : batch->groups)
    if (g.total > 0) count_launch();
  return SOCGPU_I_NORMAL;
}

int socgpu_batch_tune(socgpu_batch batch, void *stream, int reps, char *msg, size_t msg_len) {
  if (!batch) { set_msg(msg, msg_len, "invalid batch"); return SOCGPU_I_ERR_FATAL; }
  socgpu_batch_s &b = *batch;
  if (reps < 1) reps = 3;
  cudaStream_t st = (cudaStream_t)stream;
  // tuning sets: (precision, mode, layers); each set is timed per source
  // (solar and infra-red run different kernels) and the times summed
  std::map<std::tuple<int, int, int>, std::vector<int>> keys;
  for (size_t i = 0; i < b.params.size(); ++i)
    keys[std::make_tuple(b.precision[i], b.mode[i], b.params[i].n_layer)].push_back((int)i);
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  int status = SOCGPU_I_NORMAL;
  for (auto &kv : keys) {
    const int prec = std::get<0>(kv.first), mode = std::get<1>(kv.first), L = std::get<2>(kv.first);
    float best = 1e30f;
    TileConfig best_t{};
    const int lanes_opts[] = {8, 16, 32};
    for (int lanes : lanes_opts) {
      const int chunk = smallest_chunk(prec, lanes, L);
      if (!find_variant(prec, mode, lanes) || chunk == 0) continue;
      for (int warps : {4, 8}) {
        TileConfig t{lanes, warps, chunk};
        // one group per source
        std::vector<std::vector<int>> by_src(2);
        for (int i : kv.second) by_src[b.params[i].isolir == SOCGPU_IP_SOLAR ? 0 : 1].push_back(i);
        std::vector<BatchGroup> groups;
        std::vector<std::vector<FluxParams>> items;
        std::vector<std::vector<long long>> starts;
        groups.reserve(2); items.reserve(2); starts.reserve(2);
        bool fits = true;
        for (auto &idx : by_src) {
          if (idx.empty()) continue;
          groups.emplace_back(); items.emplace_back(); starts.emplace_back();
          char sub[256] = "";
          if (make_group(b, idx, prec, mode, t, groups.back(), items.back(), starts.back(), sub, sizeof(sub)) !=
              SOCGPU_I_NORMAL)
            fits = false;
        }
        if (!fits) continue;   // this tile does not fit (shared memory): not a candidate
        char *tbuf = nullptr;
        std::vector<FluxParams *> di;
        std::vector<long long *> ds;
        char sub[256] = "";
        if (upload_groups(groups, tbuf, di, ds, sub, sizeof(sub)) != SOCGPU_I_NORMAL) {
          if (tbuf) cudaFree(tbuf);
          status = SOCGPU_I_ABORT_CALCULATION;
          set_msg(msg, msg_len, "tuning upload failed: %s", sub);
          break;
        }
        float ms = 1e30f;
        int bad = 0;
        for (size_t q = 0; q < groups.size(); ++q) bad |= launch_group(groups[q], di[q], ds[q], st);   // warm-up
        for (int r = 0; r < reps && !bad; ++r) {
          cudaEventRecord(e0, st);
          for (size_t q = 0; q < groups.size(); ++q) bad |= launch_group(groups[q], di[q], ds[q], st);
          cudaEventRecord(e1, st);
          if (cudaEventSynchronize(e1) != cudaSuccess) { bad = 1; break; }
          float m = 0.f;
          cudaEventElapsedTime(&m, e0, e1);
          ms = std::min(ms, m);
        }
        cudaStreamSynchronize(st);
        cudaFree(tbuf);
        if (bad) {
          cudaGetLastError();
          status = SOCGPU_I_ABORT_CALCULATION;
          set_msg(msg, msg_len, "tuning launch failed for %d lanes x %d layers, %d warps", lanes, chunk, warps);
          break;
        }
        if (ms < best) { best = ms; best_t = t; }
      }
      if (status != SOCGPU_I_NORMAL) break;
    }
    if (status != SOCGPU_I_NORMAL) break;
    if (best_t.lanes_per_solve) {
      std::lock_guard<std::mutex> lk(g_tile_mutex);
      g_tuned[kv.first] = best_t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status != SOCGPU_I_NORMAL) return status;
  return build_plan(b, msg, msg_len);
}

int socgpu_batch_info(socgpu_batch batch, int *n_groups, long long *n_columns, long long *n_column_gpoints) {
  if (!batch) return SOCGPU_I_ERR_FATAL;
  if (n_groups) *n_groups = (int)batch->groups.size();
  if (n_columns) *n_columns = batch->n_columns;
  if (n_column_gpoints) *n_column_gpoints = batch->n_colg;
  return SOCGPU_I_NORMAL;
}

int socgpu_batch_destroy(socgpu_batch batch) {
  if (!batch) return SOCGPU_I_NORMAL;
  cudaStreamSynchronize(batch->capture);
  cudaDeviceSynchronize();
  delete batch;
  return SOCGPU_I_NORMAL;
}

int socgpu_tune_get(int precision, int mode, int n_layer, int *lanes_per_solve, int *layers_per_lane,
                    int *warps_per_cta) {
  std::lock_guard<std::mutex> lk(g_tile_mutex);
  auto it = g_tuned.find(std::make_tuple(precision, mode, n_layer));
  if (it == g_tuned.end()) return SOCGPU_I_ERR_EXIST;
  if (lanes_per_solve) *lanes_per_solve = it->second.lanes_per_solve;
  if (layers_per_lane) *layers_per_lane = it->second.chunk;
  if (warps_per_cta) *warps_per_cta = it->second.warps_per_cta;
  return SOCGPU_I_NORMAL;
}

int socgpu_tune_set(int precision, int mode, int n_layer, int lanes_per_solve, int layers_per_lane,
                    int warps_per_cta) {
  if (precision < 0 || precision > 1 || mode < 0 || mode > 2 || n_layer < 1 || n_layer > SOCGPU_MAX_LAYER)
    return SOCGPU_I_ERR_RANGE;
  std::lock_guard<std::mutex> lk(g_tile_mutex);
  if (lanes_per_solve == 0) { g_tuned.erase(std::make_tuple(precision, mode, n_layer)); return SOCGPU_I_NORMAL; }
  if (lanes_per_solve == 1) {
    // the phased kernel: layers_per_lane is its k-term batch
    if (mode == 2 || n_layer > kPhasedMaxLayers || layers_per_lane < 1 || layers_per_lane > 32 || warps_per_cta < 2 ||
        warps_per_cta > 8)
      return SOCGPU_I_ERR_RANGE;
    g_tuned[std::make_tuple(precision, mode, n_layer)] = TileConfig{1, warps_per_cta, layers_per_lane};
    return SOCGPU_I_NORMAL;
  }
  const int *c = nullptr;
  const int n = chunk_list(precision, lanes_per_solve, &c);
  bool ok = false;
  for (int i = 0; i < n; ++i) ok |= (c[i] == layers_per_lane);
  if (!ok || lanes_per_solve * layers_per_lane < n_layer || warps_per_cta < 1 || warps_per_cta > 8 ||
      (warps_per_cta * 32) % lanes_per_solve != 0)
    return SOCGPU_I_ERR_RANGE;
  g_tuned[std::make_tuple(precision, mode, n_layer)] = TileConfig{lanes_per_solve, warps_per_cta, layers_per_lane};
  return SOCGPU_I_NORMAL;
}

}  // extern "C"
