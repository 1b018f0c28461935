// runes.cpp -- socgpu_runes: the model-facing interface of the reference
// (src/interface_core/socrates_runes.F90:47-1079) over socgpu_radiance_calc.
//
// The argument mapping follows the reference's set_* routines: set_control's
// defaults (socrates_set_control.F90:232-300: PIFM80 or Elsasser with a
// quadratic source, full scattering, delta rescaling, continuum,
// equivalent-extinction overlap, clear sky), set_atm's absorbers
// (socrates_set_atm.F90:535-622), set_bound's surface
// (socrates_set_bound.F90:138-640) with the surface Planck flux of
// diff_planck_source_mod.F90:123-190, and set_diag's diagnostics
// (socrates_set_diag.F90:140-220).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "host_internal.h"
#include "mcica_setup.h"

namespace socgpu {
namespace {

// planck_flux_band (planck_flux_band_mod.F90:33-48), polynomial branch.
double planck_band(const SpectrumEntry &e, int b, double t) {
  const double x = t / e.dev.t_ref_planck;
  const double *c = e.bands_host[b].planck;
  double v = c[e.dev.n_deg_fit];
  for (int j = e.dev.n_deg_fit - 1; j >= 0; --j) v = v * x + c[j];
  return v;
}

}  // namespace
}  // namespace socgpu

using namespace socgpu;

extern "C" int socgpu_runes(const socgpu_runes_args *a, socgpu_runes_diag *diag, char *msg, size_t msg_len) {
  if (!a || !diag || !a->spectrum_name) { set_msg(msg, msg_len, "null argument"); return SOCGPU_I_ERR_FATAL; }
  const int np = a->n_profile, nl = a->n_layer;
  if (np < 0 || nl < 1) { set_msg(msg, msg_len, "n_profile %d / n_layer %d out of range", np, nl); return SOCGPU_I_ERR_RANGE; }
  socgpu_spectrum_handle h = 0;
  if (socgpu_spectrum_lookup(a->spectrum_name, &h) != SOCGPU_I_NORMAL) {
    set_msg(msg, msg_len, "spectrum '%s' has not been set", a->spectrum_name);
    return SOCGPU_I_ERR_EXIST;
  }
  const SpectrumEntry *e = find_spectrum(h);
  if (!e) { set_msg(msg, msg_len, "spectrum '%s' has not been set", a->spectrum_name); return SOCGPU_I_ERR_EXIST; }
  const bool solar = a->i_source == SOCGPU_IP_SOURCE_ILLUMINATE;
  if (!solar && a->i_source != SOCGPU_IP_SOURCE_THERMAL) {
    set_msg(msg, msg_len, "Radiative source option unrecognised.");
    return SOCGPU_I_ERR_FATAL;
  }
  if (!a->p_layer || !a->t_layer || !a->mass) {
    set_msg(msg, msg_len, "p_layer, t_layer and mass are required");
    return SOCGPU_I_ERR_FATAL;
  }
  if (!solar && !a->t_level) { set_msg(msg, msg_len, "the thermal source needs t_level"); return SOCGPU_I_ERR_FATAL; }
  if (solar && (!a->cos_zenith_angle || !a->solar_irrad)) {
    set_msg(msg, msg_len, "the solar source needs cos_zenith_angle and solar_irrad");
    return SOCGPU_I_ERR_FATAL;
  }
  const int nb = e->dev.n_band, ns = std::max(1, (int)e->type_absorb.size());
  const size_t NP = (size_t)std::max(np, 1);
  // vertical order (set_atm: layer_offset, level_offset): the reference's
  // layer i is the caller's layer lay(i), its level i the caller's lev(i)
  auto lay = [&](int i) { return a->l_invert ? nl - 1 - i : i; };
  auto lev = [&](int i) { return a->l_invert ? nl - i : i; };
  auto layer_field = [&](const double *src, std::vector<double> &dst) {
    dst.assign(NP * nl, 0.0);
    if (!src) return;
    for (int i = 0; i < nl; ++i)
      for (int l = 0; l < np; ++l) dst[l + NP * i] = src[l + (size_t)np * lay(i)];
  };
  std::vector<double> p, t, mass, density, t_level, p_level;
  layer_field(a->p_layer, p);
  layer_field(a->t_layer, t);
  layer_field(a->mass, mass);
  if (a->density) layer_field(a->density, density);
  auto level_field = [&](const double *src, std::vector<double> &dst) {
    dst.assign(NP * (nl + 1), 0.0);
    if (!src) return;
    for (int i = 0; i <= nl; ++i)
      for (int l = 0; l < np; ++l) dst[l + NP * i] = src[l + (size_t)np * lev(i)];
  };
  level_field(a->t_level, t_level);
  // absorbers of the spectrum (set_gas_mix_ratio, socrates_set_atm.F90:535-622)
  std::vector<double> gas(NP * nl * ns, 0.0);
  for (size_t g = 0; g < e->type_absorb.size(); ++g) {
    const int ty = e->type_absorb[g];
    if (ty < 1 || ty >= SOCGPU_RUNES_N_GAS) continue;
    const bool mix = a->has_mix_ratio[ty] != 0;
    const bool well_mixed = (mix && a->gas_well_mixed[ty]) || (!a->gas[ty] && mix);
    double *dst = gas.data() + NP * nl * g;
    if (well_mixed) {
      for (size_t q = 0; q < NP * nl; ++q) dst[q] = a->gas_mix_ratio[ty];
    } else if (a->gas[ty]) {
      for (int i = 0; i < nl; ++i)
        for (int l = 0; l < np; ++l) dst[l + NP * i] = std::max(a->gas[ty][l + (size_t)np * lay(i)], 0.0);
    }
  }
  // surface (set_bound)
  std::vector<double> rho_alb(NP * 2 * nb, 0.0), zen_0(NP, 1.0), solar_irrad(NP, 0.0), t_ground(NP, 0.0);
  for (int b = 0; b < nb; ++b)
    for (int l = 0; l < np; ++l) {
      double ad, ar;
      if (a->l_grey_albedo) {
        ad = ar = a->grey_albedo;
      } else {
        ad = a->albedo_diff ? a->albedo_diff[l + (size_t)np * b] : 0.0;
        ar = a->albedo_dir ? a->albedo_dir[l + (size_t)np * b] : 0.0;
      }
      rho_alb[l + NP * (0 + 2 * (size_t)b)] = ad;
      rho_alb[l + NP * (1 + 2 * (size_t)b)] = ar;
    }
  const bool tiles = a->l_tile && a->n_tile > 0;
  const int nt = tiles ? a->n_tile : 0;
  if (tiles && !a->frac_tile) { set_msg(msg, msg_len, "tiles need frac_tile"); return SOCGPU_I_ERR_FATAL; }
  // tile albedos: the grid box takes their fraction-weighted mean; else the
  // tiles take the grid box's
  std::vector<double> alb_tile((size_t)NP * 2 * std::max(nt, 1) * nb, 0.0);
  auto at = [&](int l, int k, int s, int b) -> double & {
    return alb_tile[l + NP * ((size_t)s + 2 * ((size_t)k + (size_t)nt * b))];
  };
  for (int s = 0; s < 2 && tiles; ++s) {
    const double *src = s == 0 ? a->albedo_diff_tile : a->albedo_dir_tile;
    for (int b = 0; b < nb; ++b)
      for (int l = 0; l < np; ++l) {
        if (src) {
          double sum = 0.0;
          for (int k = 0; k < nt; ++k) {
            at(l, k, s, b) = src[l + (size_t)np * ((size_t)k + (size_t)nt * b)];
            sum += at(l, k, s, b) * a->frac_tile[l + (size_t)np * k];
          }
          rho_alb[l + NP * ((size_t)s + 2 * (size_t)b)] = sum;
        } else {
          for (int k = 0; k < nt; ++k) at(l, k, s, b) = rho_alb[l + NP * ((size_t)s + 2 * (size_t)b)];
        }
      }
  }
  if (solar)
    for (int l = 0; l < np; ++l)
      if (a->cos_zenith_angle[l] > 0.0) {
        solar_irrad[l] = a->solar_irrad[l];
        zen_0[l] = 1.0 / a->cos_zenith_angle[l];
      }
  if (a->t_ground)
    for (int l = 0; l < np; ++l) t_ground[l] = a->t_ground[l];
  // the surface's Planck flux per band (diff_planck_source_mod.F90:123-190)
  std::vector<double> flux_ground;
  const bool given = !solar && a->l_flux_ground;
  if (!solar && (given || tiles)) {
    if (given && !a->flux_ground) { set_msg(msg, msg_len, "l_flux_ground needs flux_ground"); return SOCGPU_I_ERR_FATAL; }
    if (tiles && (!a->t_tile && !a->flux_tile)) {
      set_msg(msg, msg_len, "tiles need t_tile or flux_tile");
      return SOCGPU_I_ERR_FATAL;
    }
    flux_ground.assign(NP * nb, 0.0);
    for (int b = 0; b < nb; ++b)
      for (int l = 0; l < np; ++l) {
        double fg;
        if (given) fg = a->flux_ground[l + (size_t)np * b] / (1.0 - rho_alb[l + NP * (2 * (size_t)b)]);
        else fg = planck_band(*e, b, t_ground[l]);
        if (tiles) {
          fg = 0.0;
          for (int k = 0; k < nt; ++k) {
            const double f = a->frac_tile[l + (size_t)np * k];
            const bool flux_k = a->l_flux_tile && a->l_flux_tile[k] && a->flux_tile;
            double ft = 0.0;
            if (flux_k && f > 2.2250738585072014e-308)
              ft = a->flux_tile[l + (size_t)np * ((size_t)k + (size_t)nt * b)] / (1.0 - at(l, k, 0, b));
            else if (f > 2.2250738585072014e-308)
              ft = planck_band(*e, b, a->t_tile ? a->t_tile[l + (size_t)np * k] : 0.0);
            fg = (k == 0) ? f * ft : fg + f * ft;
          }
        }
        flux_ground[l + NP * b] = fg;
      }
  }
  // clouds (socrates_set_control.F90:291-370, socrates_set_cld.F90,
  // socrates_set_cld_dim.F90, socrates_set_cld_mcica.F90)
  int rep = a->i_cloud_representation ? a->i_cloud_representation : SOCGPU_IP_CLOUD_OFF;
  if (rep < SOCGPU_IP_CLOUD_HOMOGEN || rep > SOCGPU_IP_CLOUD_SPLIT_ICE_WATER) {
    set_msg(msg, msg_len, "cloud representation %d unrecognised", rep);
    return SOCGPU_I_ERR_FATAL;
  }
  const bool clouds = rep != SOCGPU_IP_CLOUD_OFF;
  // separate convective cloud runs in clear, stratiform and convective
  // regions; the split representations combine the two clouds and split the
  // total into an optically thin and a thick part (socrates_set_cld.F90:215-229)
  const bool split = rep == SOCGPU_IP_CLOUD_SPLIT_HOMOGEN || rep == SOCGPU_IP_CLOUD_SPLIT_ICE_WATER;
  const bool conv_sep = split || rep == SOCGPU_IP_CLOUD_CONV_STRAT || rep == SOCGPU_IP_CLOUD_CSIW;
  const bool four_types = rep == SOCGPU_IP_CLOUD_CSIW || rep == SOCGPU_IP_CLOUD_SPLIT_ICE_WATER;
  // McICA does not take separate convective cloud (socrates_set_control.F90:336)
  const int inhom = (conv_sep && a->i_inhom == SOCGPU_IP_MCICA) ? SOCGPU_IP_HOMOGENEOUS : a->i_inhom;
  const bool mcica = clouds && inhom == SOCGPU_IP_MCICA;
  const bool homogen = rep == SOCGPU_IP_CLOUD_HOMOGEN || rep == SOCGPU_IP_CLOUD_COMBINE_HOMOGEN;
  const bool combine = split || rep == SOCGPU_IP_CLOUD_COMBINE_HOMOGEN || rep == SOCGPU_IP_CLOUD_COMBINE_ICE_WATER;
  const int scatter = a->i_scatter_method ? a->i_scatter_method : SOCGPU_IP_SCATTER_FULL;
  int i_cloud = SOCGPU_IP_CLOUD_CLEAR, solver = scatter == SOCGPU_IP_SCATTER_FULL ? SOCGPU_IP_SOLVER_HOMOGEN_DIRECT
                                                                               : SOCGPU_IP_SOLVER_NO_SCAT;
  if (clouds && !mcica) {
    if (inhom != SOCGPU_IP_HOMOGENEOUS && inhom != SOCGPU_IP_SCALING && inhom != SOCGPU_IP_TRIPLECLOUDS_2019) {
      set_msg(msg, msg_len, "condensate inhomogeneity %d is not built for cloud regions", inhom);
      return SOCGPU_I_ERR_RANGE;
    }
    if (scatter != SOCGPU_IP_SCATTER_FULL) {
      set_msg(msg, msg_len, "cloud regions need the full scattering treatment");
      return SOCGPU_I_ERR_RANGE;
    }
    if (conv_sep) {
      if (a->i_overlap != SOCGPU_IP_MAX_RAND && a->i_overlap != SOCGPU_IP_EXPONENTIAL_RAND) {
        // random overlap keeps two regions, whose solver (mix_column.F90:438-530)
        // does not take solver_triple_hogan
        set_msg(msg, msg_len, "***Error: The solver specified is not valid here.");
        return SOCGPU_I_ERR_FATAL;
      }
      if (a->i_cloud_entrapment == SOCGPU_IP_MAX_ENTRAPMENT) {
        set_msg(msg, msg_len, "maximal entrapment in three regions (solver_triple) is not built");
        return SOCGPU_I_ERR_RANGE;
      }
      i_cloud = a->i_overlap == SOCGPU_IP_EXPONENTIAL_RAND ? SOCGPU_IP_CLOUD_PART_CORR_CNV : SOCGPU_IP_CLOUD_TRIPLE;
      solver = SOCGPU_IP_SOLVER_TRIPLE_HOGAN;
    } else {
      i_cloud = a->i_overlap == SOCGPU_IP_MAX_RAND ? SOCGPU_IP_CLOUD_MIX_MAX
              : a->i_overlap == SOCGPU_IP_EXPONENTIAL_RAND ? SOCGPU_IP_CLOUD_PART_CORR : SOCGPU_IP_CLOUD_MIX_RANDOM;
      solver = a->i_cloud_entrapment == SOCGPU_IP_MAX_ENTRAPMENT ? SOCGPU_IP_SOLVER_MIX_DIRECT
                                                                  : SOCGPU_IP_SOLVER_MIX_DIRECT_HOGAN;
    }
  } else if (mcica) {
    i_cloud = SOCGPU_IP_CLOUD_MCICA;
  }
  const int ict = (clouds && a->n_cloud_layer > 0) ? nl + 1 - std::min(a->n_cloud_layer, nl) : 1;
  const size_t ncl = (size_t)(nl - ict + 1), NC = NP * ncl;
  const int nct = homogen ? 1 : (four_types ? 4 : 2);
  std::vector<double> cmr, cdim, w_cloud, frac_cloud, c_cloud, c_ratio, rsd_w;
  std::vector<int> type_condensed, i_cloud_type, i_condensed_param, i_condensed_type;
  McicaState mst;
  if (clouds) {
    const double eps = std::numeric_limits<double>::epsilon(), min_cloud_fraction = 0.001;
    // a (n_profile, n_layer) argument on the cloudy layers, floored at zero
    auto cfield = [&](const double *src, std::vector<double> &dst, bool floor0) {
      dst.assign(NC, 0.0);
      for (size_t k = 0; k < ncl; ++k)
        for (int l = 0; l < np; ++l) {
          const double v = src[l + (size_t)np * lay(ict - 1 + (int)k)];
          dst[l + NP * k] = floor0 ? std::max(v, 0.0) : v;
        }
    };
    // condensed components (socrates_set_cld.F90:175-212): stratiform water
    // and ice, then convective water and ice where convective cloud is separate
    struct Comp { int clcmp, phase, type; bool conv; };
    std::vector<Comp> comps = {{SOCGPU_IP_CLCMP_ST_WATER, SOCGPU_IP_PHASE_WATER, a->i_st_water, false},
                               {SOCGPU_IP_CLCMP_ST_ICE, SOCGPU_IP_PHASE_ICE, a->i_st_ice, false}};
    if (conv_sep) {
      comps.push_back({SOCGPU_IP_CLCMP_CNV_WATER, SOCGPU_IP_PHASE_WATER, a->i_cnv_water, true});
      comps.push_back({SOCGPU_IP_CLCMP_CNV_ICE, SOCGPU_IP_PHASE_ICE, a->i_cnv_ice, true});
    }
    const int nc = (int)comps.size();
    cmr.assign(NC * nc, 0.0);
    cdim.assign(NC * nc, 0.0);
    rsd_w.assign(NC * nc, 0.0);
    c_cloud.assign(NC, 0.0);
    c_ratio.assign(NC, 0.0);
    std::vector<double> tmp, rsd;
    for (int k = 0; k < nc; ++k) {
      const bool water = comps[k].phase == SOCGPU_IP_PHASE_WATER, conv = comps[k].conv;
      const int ty = comps[k].type;
      const std::vector<int> &schemes = water ? e->drop_scheme : e->ice_scheme;
      if (ty <= 0) {
        set_msg(msg, msg_len, water ? "Prescribed liquid cloud not yet implemented." : "Prescribed ice cloud not yet implemented.");
        return SOCGPU_I_ERR_FATAL;
      }
      if (ty > (int)schemes.size() || schemes[ty - 1] == 0) {
        set_msg(msg, msg_len, water ? "Liquid cloud type not in spectral file." : "Ice cloud type not in spectral file.");
        return SOCGPU_I_ERR_FATAL;
      }
      type_condensed.push_back(comps[k].clcmp);
      i_condensed_param.push_back(schemes[ty - 1]);
      i_condensed_type.push_back(ty);
      // the component's cloud type (socrates_set_cld.F90:475-660)
      int ct;
      if (homogen) ct = 1;
      else if (four_types) ct = water ? (conv ? SOCGPU_IP_CLOUD_TYPE_CW : SOCGPU_IP_CLOUD_TYPE_SW)
                                      : (conv ? SOCGPU_IP_CLOUD_TYPE_CI : SOCGPU_IP_CLOUD_TYPE_SI);
      else if (conv_sep) ct = conv ? SOCGPU_IP_CLOUD_TYPE_CONV : SOCGPU_IP_CLOUD_TYPE_STRAT;
      else ct = water ? SOCGPU_IP_CLOUD_TYPE_WATER : SOCGPU_IP_CLOUD_TYPE_ICE;
      i_cloud_type.push_back(ct);
      // grid-box mixing ratios; combined cloud adds the other part's condensate
      const double *st = water ? a->liq_mmr : a->ice_mmr, *cv = water ? a->liq_conv_mmr : a->ice_conv_mmr;
      double *dst = cmr.data() + NC * k;
      if (!conv) {
        if (!st) { set_msg(msg, msg_len, water ? "Liquid MMR not provided." : "Ice MMR not provided."); return SOCGPU_I_ERR_FATAL; }
        cfield(st, tmp, true);
        std::copy(tmp.begin(), tmp.end(), dst);
        if (combine && cv) {
          cfield(cv, tmp, true);
          for (size_t q = 0; q < NC; ++q) { dst[q] += tmp[q]; c_ratio[q] += tmp[q]; }
        }
      } else {
        if (cv) {
          cfield(cv, tmp, true);
          std::copy(tmp.begin(), tmp.end(), dst);
        } else if (!split) {
          set_msg(msg, msg_len, water ? "Convective liquid MMR not provided." : "Convective ice MMR not provided.");
          return SOCGPU_I_ERR_FATAL;
        }
        if (combine && st) {
          cfield(st, tmp, true);
          for (size_t q = 0; q < NC; ++q) dst[q] += tmp[q];
        }
      }
      const double *rsd_src = conv ? (water ? a->liq_conv_rsd : a->ice_conv_rsd) : (water ? a->liq_rsd : a->ice_rsd);
      if (rsd_src) cfield(rsd_src, rsd, true);
      else rsd.assign(NC, a->has_cloud_horizontal_rsd ? a->cloud_horizontal_rsd : 0.0);
      for (size_t q = 0; q < NC; ++q) {
        if (inhom == SOCGPU_IP_SCALING) dst[q] /= (1.0 + rsd[q] * rsd[q]);
        rsd_w[q + NC * k] = rsd[q];
      }
    }
    // fractions (socrates_set_cld.F90:475-790)
    frac_cloud.assign(NC * nct, 0.0);
    auto fr = [&](int type) { return frac_cloud.data() + NC * (size_t)(type - 1); };
    auto put = [&](int type, const std::vector<double> &v) { std::copy(v.begin(), v.end(), fr(type)); };
    // split a mixed-phase fraction between ice and liquid by the ratio of
    // their in-cloud mixing ratios (split_mix_phase, socrates_set_cld.F90:905-935),
    // then share the total out in proportion
    auto split_phase = [&](std::vector<double> &fl, std::vector<double> &fi, const std::vector<double> &f, int tw,
                           int ti) {
      for (size_t q = 0; q < NC; ++q) {
        if (fl[q] + fi[q] > eps) {
          const double mix = fl[q] + fi[q] - f[q];
          if (mix > eps && fl[q] > eps && fi[q] > eps) {
            double lm = 0.0, im = 0.0;
            for (int k = 0; k < nc; ++k) {
              if (i_cloud_type[k] == tw) lm += cmr[q + NC * k] / fl[q];
              else if (i_cloud_type[k] == ti) im += cmr[q + NC * k] / fi[q];
            }
            if (lm + im > eps) {
              fl[q] = std::max(fl[q] - mix * im / (lm + im), 0.0);
              fi[q] = std::max(fi[q] - mix * lm / (lm + im), 0.0);
            }
          }
          const double s2 = fl[q] + fi[q];
          const double nl_ = f[q] * fl[q] / s2, ni_ = f[q] * fi[q] / s2;
          fl[q] = nl_;
          fi[q] = ni_;
        } else {
          fl[q] = 0.0;
          fi[q] = 0.0;
        }
      }
    };
    if (homogen) {
      if (!a->cloud_frac) { set_msg(msg, msg_len, "Cloud fraction not provided."); return SOCGPU_I_ERR_FATAL; }
      cfield(a->cloud_frac, tmp, true);
      put(1, tmp);
      if (combine && a->conv_frac) {
        cfield(a->conv_frac, c_cloud, true);
        for (size_t q = 0; q < NC; ++q) frac_cloud[q] += c_cloud[q];
      }
    } else if (!conv_sep) {
      std::vector<double> fl, fi, f;
      if (a->liq_frac && a->ice_frac && a->cloud_frac) {
        cfield(a->liq_frac, fl, true); cfield(a->ice_frac, fi, true); cfield(a->cloud_frac, f, true);
        split_phase(fl, fi, f, 1, 2);
      } else if (a->liq_frac && a->ice_frac) {
        cfield(a->liq_frac, fl, true); cfield(a->ice_frac, fi, true);
      } else {
        set_msg(msg, msg_len, "Liquid and ice cloud fractions not provided.");
        return SOCGPU_I_ERR_FATAL;
      }
      put(1, fl);
      put(2, fi);
      if (combine && a->liq_conv_frac && a->ice_conv_frac) {
        std::vector<double> cl, ci, cf;
        cfield(a->liq_conv_frac, cl, true); cfield(a->ice_conv_frac, ci, true);
        if (a->conv_frac) {
          cfield(a->conv_frac, cf, true);
          // the convective split keeps its fractions where both are zero
          for (size_t q = 0; q < NC; ++q) {
            if (cl[q] + ci[q] > eps) {
              const double mix = cl[q] + ci[q] - cf[q];
              if (mix > eps && cl[q] > eps && ci[q] > eps) {
                double lm = 0.0, im = 0.0;
                for (int k = 0; k < nc; ++k) {
                  if (i_cloud_type[k] == 1) lm += cmr[q + NC * k] / cl[q];
                  else if (i_cloud_type[k] == 2) im += cmr[q + NC * k] / ci[q];
                }
                if (lm + im > eps) {
                  cl[q] = std::max(cl[q] - mix * im / (lm + im), 0.0);
                  ci[q] = std::max(ci[q] - mix * lm / (lm + im), 0.0);
                }
              }
              // in sequence, as socrates_set_cld.F90:548-551 updates them
              cl[q] = cf[q] * cl[q] / (cl[q] + ci[q]);
              ci[q] = cf[q] * ci[q] / (cl[q] + ci[q]);
            }
          }
        }
        for (size_t q = 0; q < NC; ++q) {
          frac_cloud[q] += cl[q];
          frac_cloud[q + NC] += ci[q];
          c_cloud[q] = cl[q] + ci[q];
        }
      }
    } else if (!four_types) {
      // stratiform and convective types (socrates_set_cld.F90:567-600)
      if (a->cloud_frac && a->conv_frac) {
        cfield(a->cloud_frac, tmp, true);
        put(SOCGPU_IP_CLOUD_TYPE_STRAT, tmp);
        cfield(a->conv_frac, tmp, true);
        put(SOCGPU_IP_CLOUD_TYPE_CONV, tmp);
      } else if (split && a->cloud_frac) {
        cfield(a->cloud_frac, tmp, true);
        put(SOCGPU_IP_CLOUD_TYPE_STRAT, tmp);
      } else {
        set_msg(msg, msg_len, "Cloud fractions not provided.");
        return SOCGPU_I_ERR_FATAL;
      }
    } else {
      // stratiform and convective water and ice (socrates_set_cld.F90:642-747)
      std::vector<double> fl, fi, f;
      if (a->liq_frac && a->ice_frac && a->cloud_frac) {
        cfield(a->liq_frac, fl, true); cfield(a->ice_frac, fi, true); cfield(a->cloud_frac, f, true);
        split_phase(fl, fi, f, SOCGPU_IP_CLOUD_TYPE_SW, SOCGPU_IP_CLOUD_TYPE_SI);
      } else if (a->liq_frac && a->ice_frac) {
        cfield(a->liq_frac, fl, true); cfield(a->ice_frac, fi, true);
      } else {
        set_msg(msg, msg_len, "Liquid and ice cloud fractions not provided.");
        return SOCGPU_I_ERR_FATAL;
      }
      put(SOCGPU_IP_CLOUD_TYPE_SW, fl);
      put(SOCGPU_IP_CLOUD_TYPE_SI, fi);
      if (a->liq_conv_frac && a->ice_conv_frac && a->conv_frac) {
        cfield(a->liq_conv_frac, fl, true); cfield(a->ice_conv_frac, fi, true); cfield(a->conv_frac, f, true);
        split_phase(fl, fi, f, SOCGPU_IP_CLOUD_TYPE_CW, SOCGPU_IP_CLOUD_TYPE_CI);
      } else if (a->liq_conv_frac && a->ice_conv_frac) {
        cfield(a->liq_conv_frac, fl, true); cfield(a->ice_conv_frac, fi, true);
      } else if (split) {
        fl.assign(NC, 0.0);
        fi.assign(NC, 0.0);
      } else {
        set_msg(msg, msg_len, "Liquid and ice convective cloud fractions not provided.");
        return SOCGPU_I_ERR_FATAL;
      }
      put(SOCGPU_IP_CLOUD_TYPE_CW, fl);
      put(SOCGPU_IP_CLOUD_TYPE_CI, fi);
    }
    if (split) {
      // the combined cloud split into an optically thin and a thick part
      // (socrates_set_cld.F90:602-640, 749-790): by the condensate RSD with
      // equations A1 and A2 of Hogan et al. (2019), else in equal halves
      for (int ph = 0; ph < (four_types ? 2 : 1); ++ph) {
        const int thin = four_types ? (ph == 0 ? SOCGPU_IP_CLOUD_TYPE_SW : SOCGPU_IP_CLOUD_TYPE_SI)
                                    : SOCGPU_IP_CLOUD_TYPE_STRAT;
        const int thick = four_types ? (ph == 0 ? SOCGPU_IP_CLOUD_TYPE_CW : SOCGPU_IP_CLOUD_TYPE_CI)
                                     : SOCGPU_IP_CLOUD_TYPE_CONV;
        double *ft = fr(thin), *fk = fr(thick);
        for (size_t q = 0; q < NC; ++q) {
          const double frac = ft[q] + fk[q];
          if (inhom != SOCGPU_IP_TRIPLECLOUDS_2019) {
            ft[q] = 0.5 * frac;
            fk[q] = 0.5 * frac;
            continue;
          }
          // one RSD per part: the thin type's own (water and ice apart), or
          // the condensate-weighted mean over the stratiform components
          double r = 0.0;
          if (four_types) {
            for (int k = 0; k < nc; ++k)
              if (i_cloud_type[k] == thin) r = rsd_w[q + NC * k];
          } else {
            double num = 0.0, den = 0.0;
            for (int k = 0; k < nc; ++k)
              if (i_cloud_type[k] == thin) { num += rsd_w[q + NC * k] * cmr[q + NC * k]; den += cmr[q + NC * k]; }
            r = num / std::max(den, eps);
          }
          const double f_thin = std::max(0.5, std::min(0.9, r * (0.4 / 2.25) + 0.525 / 2.25));
          ft[q] = frac * f_thin;
          fk[q] = frac * (1.0 - f_thin);
          const double ratio = 0.025 + 0.975 * std::exp(-r - r * r / 2.0 - r * r * r / 4.0);
          for (int k = 0; k < nc; ++k) {
            if (i_cloud_type[k] == thin) cmr[q + NC * k] *= ratio * f_thin;
            else if (i_cloud_type[k] == thick) cmr[q + NC * k] *= 1.0 - ratio * f_thin;
          }
        }
      }
      if (inhom != SOCGPU_IP_TRIPLECLOUDS_2019)
        for (double &v : cmr) v *= 0.5;
    }
    std::vector<double> cond_total;
    if (combine) {
      cond_total.assign(NC, 0.0);
      for (size_t q = 0; q < NC; ++q) {
        c_ratio[q] = c_ratio[q] / std::max(c_cloud[q], eps);
        for (int k = 0; k < nc; ++k) cond_total[q] += cmr[q + NC * k];
      }
    }
    // in-cloud mixing ratios, then normalised fractions
    for (int k = 0; k < nc; ++k)
      for (size_t q = 0; q < NC; ++q) {
        const double f = frac_cloud[q + NC * (i_cloud_type[k] - 1)];
        cmr[q + NC * k] = f > eps ? cmr[q + NC * k] / f : 0.0;
      }
    w_cloud.assign(NC, 0.0);
    for (size_t q = 0; q < NC; ++q) {
      double w = 0.0;
      for (int t2 = 0; t2 < nct; ++t2) w += frac_cloud[q + NC * t2];
      if (w > min_cloud_fraction) {
        for (int t2 = 0; t2 < nct; ++t2) frac_cloud[q + NC * t2] /= w;
        if (combine) c_ratio[q] = c_ratio[q] * w / std::max(cond_total[q], eps);
      } else {
        w = 0.0;
        for (int t2 = 0; t2 < nct; ++t2) frac_cloud[q + NC * t2] = 0.0;
        if (combine) { c_cloud[q] = 0.0; c_ratio[q] = 0.0; }
      }
      if (w > 1.0 + min_cloud_fraction) { set_msg(msg, msg_len, "Cloud fraction greater than 1."); return SOCGPU_I_ERR_FATAL; }
      w_cloud[q] = std::min(w, 1.0);
    }
    // effective dimensions (socrates_set_cld_dim.F90:155-230); the split
    // representations size and bound their convective part as the stratiform one
    for (int k = 0; k < nc; ++k) {
      const bool water = comps[k].phase == SOCGPU_IP_PHASE_WATER, own = comps[k].conv && !split;
      double *dst = cdim.data() + NC * k;
      const double *ice_src = own ? a->ice_conv_dim : a->ice_dim;
      if (water) {
        const int re = a->i_drop_re ? a->i_drop_re : SOCGPU_IP_RE_EXTERNAL;
        const double *src = own ? a->liq_conv_dim : a->liq_dim;
        const bool has_c = own ? a->has_liq_conv_dim_constant : a->has_liq_dim_constant;
        if (re == SOCGPU_IP_RE_EXTERNAL && src) {
          cfield(src, tmp, false);
          std::copy(tmp.begin(), tmp.end(), dst);
        } else if (re == SOCGPU_IP_RE_CONSTANT && has_c) {
          std::fill(dst, dst + NC, own ? a->liq_conv_dim_constant : a->liq_dim_constant);
        } else if (re == SOCGPU_IP_RE_LIU) {
          set_msg(msg, msg_len, "droplet radii from droplet numbers (ip_re_liu) are not mapped; give liq_dim");
          return SOCGPU_I_ERR_RANGE;
        } else {
          std::fill(dst, dst + NC, 7.0e-6);
        }
      } else if (ice_src) {
        cfield(ice_src, tmp, false);
        std::copy(tmp.begin(), tmp.end(), dst);
      } else {
        // set_ice_dim: sizes from the layer temperature
        const int scheme = i_condensed_param[k];
        for (size_t kk = 0; kk < ncl; ++kk)
          for (int l = 0; l < np; ++l) {
            const double tk = t[l + NP * (ict - 1 + kk)];
            double dge;
            switch (scheme) {
              case 6:    // ip_ice_adt
                dst[l + NP * kk] = std::min(7.198755e-04, std::exp(5.522e-02 * (tk - 2.7965e+02)) / 9.702e+02);
                break;
              case 12: case 16:   // ip_ice_agg_de, ip_ice_agg_de_sun
                dge = tk < 216.208 ? 7.5094588e-04 * std::exp(0.05 * (tk - 279.5)) + 5.0830326e-07
                                   : 1.3505403e-04 * std::exp(0.05 * (tk - 279.5)) + 2.6517429e-05;
                dst[l + NP * kk] = (3.0 / 2.0) * (3.0 / (2.0 * std::sqrt(3.0))) * std::min(1.24e-04, std::max(8.0e-06, dge));
                break;
              case 19:   // ip_ice_baran
                dst[l + NP * kk] = 1.868e-6 * tk - 353.613e-6;
                break;
              case 20:   // ip_ice_pade_2_phf: from ice crystal numbers
                set_msg(msg, msg_len, "ice sizes from crystal numbers (ip_ice_pade_2_phf) are not mapped; give ice_dim");
                return SOCGPU_I_ERR_RANGE;
              default:
                dst[l + NP * kk] = 30.0e-6;
            }
          }
      }
      const std::vector<double> &lo = water ? e->drop_min_dim : e->ice_min_dim, &hi = water ? e->drop_max_dim : e->ice_max_dim;
      const int ty = own ? comps[k].type : (water ? a->i_st_water : a->i_st_ice);
      if (ty <= (int)lo.size() && ty <= (int)hi.size())
        for (size_t q = 0; q < NC; ++q) dst[q] = std::min(std::max(dst[q], lo[ty - 1]), hi[ty - 1]);
    }
    if (mcica) {
      if (!a->mcica_data) { set_msg(msg, msg_len, "McICA needs the McICA data file (mcica_data)"); return SOCGPU_I_ERR_FATAL; }
      McicaData md;
      std::string err;
      if (!read_mcica_data(a->mcica_data, md, err)) { set_msg(msg, msg_len, "%s", err.c_str()); return SOCGPU_I_ERR_IO; }
      // the condensate RSD weighted by each component's grid-box condensate
      std::vector<double> cond_rsd(NC, 0.0);
      for (size_t q = 0; q < NC; ++q) {
        double num = 0.0, den = 0.0;
        for (int k = 0; k < nc; ++k) {
          const double wgt = std::max(eps, cmr[q + NC * k] * frac_cloud[q + NC * (i_cloud_type[k] - 1)]);
          num += rsd_w[q + NC * k] * wgt;
          den += wgt;
        }
        cond_rsd[q] = num / den;
      }
      std::vector<int> seeds(NP);
      for (int l = 0; l < np; ++l) seeds[l] = a->rand_seed ? a->rand_seed[l] : 10 + l + 1;
      const int sampling = a->i_mcica_sampling >= 0 ? a->i_mcica_sampling : SOCGPU_IP_MCICA_OPTIMAL_SAMPLING;
      const int st_m = set_cld_mcica(h, md, solar ? SOCGPU_IP_SOLAR : SOCGPU_IP_INFRA_RED, sampling, a->i_overlap, 1, nb,
                                     np, nl, ict, seeds.data(), a->has_cloud_vertical_decorr ? a->cloud_vertical_decorr : 0.0,
                                     cond_rsd.data(), w_cloud.data(), p.data(), mst, msg, msg_len,
                                     combine ? c_cloud.data() : nullptr, combine ? c_ratio.data() : nullptr);
      if (st_m != SOCGPU_I_NORMAL) return st_m;
    }
  }
  // classic aerosol species (set_aer): every species an entry, active where
  // its mixing ratios are given
  const int n_aer_sp = (int)e->aer_parm.size();
  std::vector<double> aer_mr, mrh;
  std::vector<int> mr_index, mr_source;
  bool classic = false;
  for (int j = 0; j < n_aer_sp; ++j) {
    const int ty = e->aer_type[j];
    classic = classic || (ty > 0 && ty < SOCGPU_RUNES_N_AER && a->aerosol[ty]);
  }
  if (classic) {
    aer_mr.assign(NP * nl * n_aer_sp, 0.0);
    for (int j = 0; j < n_aer_sp; ++j) {
      const int ty = e->aer_type[j];
      const double *src = (ty > 0 && ty < SOCGPU_RUNES_N_AER) ? a->aerosol[ty] : nullptr;
      mr_index.push_back(j + 1);
      mr_source.push_back(src ? SOCGPU_IP_AERSRC_CLASSIC_RON : SOCGPU_IP_AERSRC_CLASSIC_RON + 10);
      if (src)
        for (int i = 0; i < nl; ++i)
          for (int l = 0; l < np; ++l) aer_mr[l + NP * (i + (size_t)nl * j)] = src[l + (size_t)np * lay(i)];
    }
    if (a->mean_rel_humidity) layer_field(a->mean_rel_humidity, mrh);
  }
  // control (set_control's defaults for the two-stream path)
  socgpu_control c{};
  c.isolir = solar ? SOCGPU_IP_SOLAR : SOCGPU_IP_INFRA_RED;
  c.i_angular_integration = SOCGPU_IP_TWO_STREAM;
  c.i_2stream = solar ? SOCGPU_IP_PIFM80 : SOCGPU_IP_ELSASSER;
  c.i_scatter_method = scatter;
  c.i_solver = solver;
  c.i_cloud = i_cloud;
  c.i_cloud_representation = !clouds ? 0 : conv_sep ? rep : (homogen ? SOCGPU_IP_CLOUD_HOMOGEN : SOCGPU_IP_CLOUD_ICE_WATER);
  c.i_gas_overlap = a->i_gas_overlap ? a->i_gas_overlap : SOCGPU_IP_OVERLAP_K_EQV_SCL;
  c.i_direct_tau = SOCGPU_IP_DIRECT_DELTA_SCALING;
  c.l_rescale = 1;
  c.n_order_forward = 2;
  c.l_ir_source_quad = solar ? 0 : 1;
  c.l_rayleigh = a->l_rayleigh;
  c.l_gas = 1;
  c.l_continuum = 1;
  c.l_mixing_ratio = a->l_mixing_ratio;
  c.l_grey_single = c.i_scatter_method != SOCGPU_IP_SCATTER_FULL;
  c.l_aerosol_mode = a->l_aerosol_mode && a->n_aer_mode > 0;
  c.l_aerosol = classic;
  c.l_flux_div = 0;
  c.first_band = 1;
  c.last_band = nb;
  c.precision = a->precision;
  socgpu_dimen dm{};
  dm.nd_profile = (int)NP;
  dm.nd_layer = nl;
  dm.id_cloud_top = ict;
  dm.nd_aerosol_mode = std::max(1, a->n_aer_mode);
  dm.nd_cloud_component = std::max(2, (int)type_condensed.size());
  dm.nd_cloud_type = nct;
  dm.nd_subcol_gen = mcica ? mst.gen : 1;
  dm.nd_subcol_req = mcica ? mst.n_subcol_req : 1;
  dm.nd_aerosol_mr = std::max(1, n_aer_sp);
  dm.nd_profile_aerosol_prsc = dm.nd_opt_level_aerosol_prsc = dm.nd_phf_term_aerosol_prsc = 1;
  socgpu_atm atm{};
  atm.n_profile = np;
  atm.n_layer = nl;
  atm.p = p.data(); atm.t = t.data(); atm.mass = mass.data();
  atm.t_level = solar ? nullptr : t_level.data();
  atm.gas_mix_ratio = gas.data();
  atm.density = a->density ? density.data() : nullptr;
  atm.p_level = nullptr;
  (void)p_level;
  socgpu_bound bd{};
  bd.zen_0 = zen_0.data(); bd.solar_irrad = solar_irrad.data(); bd.rho_alb = rho_alb.data();
  bd.t_ground = t_ground.data();
  bd.flux_ground = flux_ground.empty() ? nullptr : flux_ground.data();
  // modal aerosol optical properties, reordered vertically
  std::vector<double> amr, aab, asc, aas;
  socgpu_aer aer{};
  if (c.l_aerosol_mode) {
    const int nm = a->n_aer_mode;
    if (!a->aer_mix_ratio || !a->aer_absorption || !a->aer_scattering || !a->aer_asymmetry) {
      set_msg(msg, msg_len, "l_aerosol_mode needs aer_mix_ratio, aer_absorption, aer_scattering and aer_asymmetry");
      return SOCGPU_I_ERR_FATAL;
    }
    amr.assign(NP * nl * nm, 0.0);
    aab.assign(NP * nl * nm * nb, 0.0);
    asc.assign(aab.size(), 0.0);
    aas.assign(aab.size(), 0.0);
    for (int m = 0; m < nm; ++m)
      for (int i = 0; i < nl; ++i)
        for (int l = 0; l < np; ++l) {
          amr[l + NP * (i + (size_t)nl * m)] = a->aer_mix_ratio[l + (size_t)np * (lay(i) + (size_t)nl * m)];
          for (int b = 0; b < nb; ++b) {
            const size_t qd = l + NP * (i + (size_t)nl * (m + (size_t)nm * b));
            const size_t qs = l + (size_t)np * (lay(i) + (size_t)nl * (m + (size_t)nm * b));
            aab[qd] = a->aer_absorption[qs];
            asc[qd] = a->aer_scattering[qs];
            aas[qd] = a->aer_asymmetry[qs];
          }
        }
    aer.n_mode = nm;
    aer.mode_mix_ratio = amr.data(); aer.mode_absorption = aab.data();
    aer.mode_scattering = asc.data(); aer.mode_asymmetry = aas.data();
  }
  if (classic) {
    aer.n_aerosol_mr = n_aer_sp;
    aer.mix_ratio = aer_mr.data();
    aer.mr_type_index = mr_index.data();
    aer.mr_source = mr_source.data();
    aer.mean_rel_humidity = mrh.empty() ? nullptr : mrh.data();
  }
  socgpu_cld cld{};
  if (clouds) {
    cld.n_condensed = (int)type_condensed.size();
    cld.type_condensed = type_condensed.data();
    cld.i_cloud_type = i_cloud_type.data();
    cld.i_condensed_param = i_condensed_param.data();
    cld.i_condensed_type = i_condensed_type.data();
    cld.condensed_mix_ratio = cmr.data();
    cld.condensed_dim_char = cdim.data();
    cld.n_cloud_type = nct;
    cld.w_cloud = w_cloud.data();
    cld.frac_cloud = frac_cloud.data();
    // decorrelation scales of like regions (socrates_set_cld.F90:454-465)
    cld.dp_corr_strat = a->has_cloud_vertical_decorr ? a->cloud_vertical_decorr : 0.0;
    cld.dp_corr_conv = a->has_conv_vertical_decorr ? a->conv_vertical_decorr : 0.0;
    if (mcica) mst.attach(cld);
  }
  std::vector<double> fu(NP * (nl + 1)), fd(NP * (nl + 1)), fdir(NP * (nl + 1)), hr(NP * nl);
  socgpu_radout out{};
  out.flux_up = fu.data(); out.flux_down = fd.data();
  out.flux_direct = solar ? fdir.data() : nullptr;
  out.heating_rate = hr.data();
  if (np == 0) return SOCGPU_I_NORMAL;
  int st = socgpu_radiance_calc(&c, &dm, h, &atm, clouds ? &cld : nullptr,
                                (c.l_aerosol_mode || c.l_aerosol) ? &aer : nullptr, &bd, &out, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  // diagnostics (set_diag): levels and layers back in the caller's order
  for (int i = 0; i <= nl; ++i)
    for (int l = 0; l < np; ++l) {
      const size_t src = l + NP * i, dst = l + (size_t)np * lev(i);
      if (diag->flux_up) diag->flux_up[dst] = fu[src];
      if (diag->flux_down) diag->flux_down[dst] = fd[src];
      if (diag->flux_direct) diag->flux_direct[dst] = solar ? fdir[src] : 0.0;
    }
  for (int l = 0; l < np; ++l) {
    const size_t top = l, sfc = l + NP * nl;
    if (diag->flux_up_toa) diag->flux_up_toa[l] = fu[top];
    if (diag->flux_down_toa) diag->flux_down_toa[l] = fd[top];
    if (diag->flux_direct_toa) diag->flux_direct_toa[l] = solar ? fdir[top] : 0.0;
    if (diag->flux_up_surf) diag->flux_up_surf[l] = fu[sfc];
    if (diag->flux_down_surf) diag->flux_down_surf[l] = fd[sfc];
    if (diag->flux_direct_surf) diag->flux_direct_surf[l] = solar ? fdir[sfc] : 0.0;
  }
  if (diag->heating_rate)
    for (int i = 1; i <= nl; ++i)
      for (int l = 0; l < np; ++l) {
        // socrates_set_diag.F90:150-158: the divergence from the level
        // fluxes; in mixed precision the kernel's own layer divergence (its
        // heating rate times the layer's heat capacity), which differencing
        // FP32-accurate level fluxes across thin layers would spoil
        const double div = c.precision == SOCGPU_PRECISION_MIXED
                               ? hr[l + NP * (i - 1)] * (mass[l + NP * (i - 1)] * 1.005e+03) / 8.64e+04
                               : fd[l + NP * (i - 1)] - fd[l + NP * i] + fu[l + NP * i] - fu[l + NP * (i - 1)];
        const size_t dst = l + (size_t)np * lay(i - 1);
        diag->heating_rate[dst] = a->layer_heat_capacity ? div / a->layer_heat_capacity[dst] : div;
      }
  return SOCGPU_I_NORMAL;
}
