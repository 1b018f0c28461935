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
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "host_internal.h"

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
  // control (set_control's defaults for the two-stream path)
  socgpu_control c{};
  c.isolir = solar ? SOCGPU_IP_SOLAR : SOCGPU_IP_INFRA_RED;
  c.i_angular_integration = SOCGPU_IP_TWO_STREAM;
  c.i_2stream = solar ? SOCGPU_IP_PIFM80 : SOCGPU_IP_ELSASSER;
  c.i_scatter_method = a->i_scatter_method ? a->i_scatter_method : SOCGPU_IP_SCATTER_FULL;
  c.i_solver = c.i_scatter_method == SOCGPU_IP_SCATTER_FULL ? SOCGPU_IP_SOLVER_HOMOGEN_DIRECT : SOCGPU_IP_SOLVER_NO_SCAT;
  c.i_cloud = SOCGPU_IP_CLOUD_CLEAR;
  c.i_cloud_representation = 0;
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
  c.l_flux_div = 0;
  c.first_band = 1;
  c.last_band = nb;
  c.precision = a->precision;
  socgpu_dimen dm{};
  dm.nd_profile = (int)NP;
  dm.nd_layer = nl;
  dm.id_cloud_top = 1;
  dm.nd_aerosol_mode = std::max(1, a->n_aer_mode);
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
  std::vector<double> fu(NP * (nl + 1)), fd(NP * (nl + 1)), fdir(NP * (nl + 1)), hr(NP * nl);
  socgpu_radout out{};
  out.flux_up = fu.data(); out.flux_down = fd.data();
  out.flux_direct = solar ? fdir.data() : nullptr;
  out.heating_rate = hr.data();
  if (np == 0) return SOCGPU_I_NORMAL;
  int st = socgpu_radiance_calc(&c, &dm, h, &atm, nullptr, c.l_aerosol_mode ? &aer : nullptr, &bd, &out, msg,
                                msg_len);
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
