// flux_kernel.cuh -- fused two-stream flux kernel for sm_103a.
//
// One CTA per column.  The CTA first stages the column's per-band grey
// optics, gas amounts, Planck terms and boundary values in shared memory
// (the band loop of radiance_calc.F90:883-1600), then its lanes solve the
// monochromatic problems of every g-point (k-term product):
//
//   * a "group" of P consecutive lanes owns one (column, g-point) solve;
//     lane r of the group holds layers [r*CH, r*CH+CH) in registers;
//   * the per-layer physics (single_scattering, rescale_tau_omega,
//     two_coeff, sources) is computed for all layers in parallel;
//   * the direct beam (solar_source.F90:105-176) is a product scan over the
//     group's lanes, and the adding-method solve
//     (solver_homogen_direct.F90:94-131) becomes an associative scan of
//     layer "composites" (reflection/transmission/source of a stack of
//     layers) down and up the group, followed by the reference's
//     elimination and back-substitution inside each lane's chunk;
//   * solver_no_scat (solver_no_scat.F90:75-94) is two affine scans;
//   * each group accumulates its fluxes in its own shared-memory slice
//     (augment_channel_mod.F90:158-235); slices are summed in a fixed order
//     at the end, so results are deterministic.
//
// Per-layer shared arrays use a permuted slot order: layer i lives in slot
// (i % CH) * P + i / CH, so lane r's j-th layer is slot j*P + r and the P
// lanes of a group touch P consecutive words (no bank conflicts).
//
// The mixed-precision instantiation (R = float) does all of its arithmetic
// in FP32: FP64 inputs are narrowed once while staging (on the integer
// pipe), table constants come from FP32 copies, and results are widened on
// the way out.  On GB300 the FP64 pipe runs at 1/64 of FP32.
//
// McICA (mcica_sample.F90:453-925, mcica_column.F90:261-602): a group loops
// over the subcolumns assigned to its g-point plus the clear solve and adds
// each with its blending weight.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include "socgpu_internal.h"
#include "twostream_math.cuh"

namespace socgpu {

constexpr int kNumAcc = 4;     // up, down, direct (per level), divergence (per layer)
constexpr int kBandScal = 6;   // f_inc_down, f_inc_dir, alb_diff, alb_dir, dB_surf, weight_band

// Column-major (Fortran) element access with leading extent nd.
__device__ __forceinline__ double ld2(const double *a, int l, int i, int nd) {
  return __ldg(a + (size_t)l + (size_t)nd * (size_t)i);
}

// FP64 -> FP32 narrowing with round-to-nearest-even on the integer pipe
// (the F2F instruction issues on the FP64 pipe).  Results below the FP32
// normal range flush to zero, as the mixed kernels run with FTZ; NaN stays
// NaN and overflow gives infinity.
__device__ __forceinline__ float narrow(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  const unsigned rem = lo & 0x1FFFFFFFu;
  unsigned bits = ((unsigned)e << 23) + m;
  bits += (rem > 0x10000000u) | ((rem == 0x10000000u) & (m & 1u));
  if (e <= 0) bits = 0u;
  if (e >= 255) bits = ((hi & 0x7FFFFFFFu) > 0x7FF00000u || ((hi & 0x7FFFFFFFu) == 0x7FF00000u && lo))
                           ? 0x7FC00000u : 0x7F800000u;
  return __uint_as_float(sign | bits);
}

// FP32 -> FP64 widening (exact) on the integer pipe; FP32 subnormals are
// already flushed.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u, e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  unsigned hi, lo;
  if (e == 0u) { hi = sign; lo = 0u; }
  else if (e == 255u) { hi = sign | 0x7FF00000u | (m >> 3); lo = m << 29; }
  else { hi = sign | ((e + 896u) << 20) | (m >> 3); lo = m << 29; }
  return __hiloint2double((int)hi, (int)lo);
}

template <class R>
__device__ __forceinline__ R load_in(const double *a) {
  if constexpr (sizeof(R) == 8) return __ldg(a);
  else return narrow(__ldg(a));
}
// A raw FP64 input already in shared memory, in R.
template <class R>
__device__ __forceinline__ R raw_in(double v) {
  if constexpr (sizeof(R) == 8) return v;
  else return narrow(v);
}
// One asynchronous 8-byte copy from global to shared memory (cp.async).
__device__ __forceinline__ void cp_async8(double *dst, const double *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
template <class R>
__device__ __forceinline__ double store_out(R v) {
  if constexpr (sizeof(R) == 8) return v;
  else return widen(v);
}

template <class R>
struct Comp {     // composite of a stack of layers
  R R1, R2, Td, Tu, Su, Sd;
};

template <class R>
__device__ __forceinline__ Comp<R> comp_identity() {
  Comp<R> c; c.R1 = R(0); c.R2 = R(0); c.Td = R(1); c.Tu = R(1); c.Su = R(0); c.Sd = R(0); return c;
}

// Stack A (above) on B (below).  Derived from the adding equations of
// solver_homogen_direct: interface fluxes x (down) and y (up) satisfy
// x = A.Sd + A.R2 y, y = B.Su + B.R1 x.
template <class R>
__device__ __forceinline__ Comp<R> stack(const Comp<R> &A, const Comp<R> &B) {
  R D = R(1) / (R(1) - A.R2 * B.R1);
  Comp<R> o;
  R dTd = D * A.Td, dTu = D * B.Tu;
  o.R1 = A.R1 + A.Tu * B.R1 * dTd;
  o.R2 = B.R2 + B.Td * A.R2 * dTu;
  o.Td = B.Td * dTd;
  o.Tu = A.Tu * dTu;
  o.Su = A.Su + A.Tu * D * (B.Su + B.R1 * A.Sd);
  o.Sd = B.Sd + B.Td * D * (A.Sd + A.R2 * B.Su);
  return o;
}

template <class R>
__device__ __forceinline__ Comp<R> shfl_up_comp(const Comp<R> &c, int d, int width) {
  Comp<R> o;
  o.R1 = __shfl_up_sync(0xffffffffu, c.R1, d, width);
  o.R2 = __shfl_up_sync(0xffffffffu, c.R2, d, width);
  o.Td = __shfl_up_sync(0xffffffffu, c.Td, d, width);
  o.Tu = __shfl_up_sync(0xffffffffu, c.Tu, d, width);
  o.Su = __shfl_up_sync(0xffffffffu, c.Su, d, width);
  o.Sd = __shfl_up_sync(0xffffffffu, c.Sd, d, width);
  return o;
}
template <class R>
__device__ __forceinline__ Comp<R> shfl_down_comp(const Comp<R> &c, int d, int width) {
  Comp<R> o;
  o.R1 = __shfl_down_sync(0xffffffffu, c.R1, d, width);
  o.R2 = __shfl_down_sync(0xffffffffu, c.R2, d, width);
  o.Td = __shfl_down_sync(0xffffffffu, c.Td, d, width);
  o.Tu = __shfl_down_sync(0xffffffffu, c.Tu, d, width);
  o.Su = __shfl_down_sync(0xffffffffu, c.Su, d, width);
  o.Sd = __shfl_down_sync(0xffffffffu, c.Sd, d, width);
  return o;
}

// ---------------------------------------------------------------------------
// Shared-memory layout of one column (identical on host and device).  LP is
// the padded layer count P*CH; level arrays hold LP+1 entries (slot LP is
// level 0).
struct SmemLayout {
  int LP, nb, max_abs, n_comp, n_sub, n_groups, acc_stride;
  size_t off_p, off_t, off_mass, off_kgt, off_kes, off_kabs, off_asym, off_fwd, off_amt, off_bscal;
  size_t off_planck, off_dB, off_dB2;
  size_t off_phf_nc, off_fwd_nc, off_c_ke, off_c_ks, off_c_ka, off_c_phf, off_c_fwd;
  size_t off_wcld, off_frac, off_csub;
  size_t off_aux, off_lkf, off_lki, off_sbf, off_sbj, off_kscr;
  size_t off_ovl, off_reg, off_regd, off_nct, off_t0d, off_frr;
  int reg_rows, regd_rows;            // rows per group of the region solves (two or three regions)
  size_t off_acc;
  // the column's FP64 inputs, fetched into shared memory ahead of staging
  // (offsets in doubles from off_acc, whose space they share); raw_on false
  // leaves staging on direct global loads
  int raw_on, raw_n;
  int r_p, r_t, r_mass, r_gas, r_mmr, r_mabs, r_msca, r_masy, r_sol, r_zen, r_alb, r_tg, r_fg, r_tl;
  size_t bytes;
};

// Rows of a group's scratch for the two-region solve (cloud regions): the
// clear (free) and cloudy coefficients of each layer, the elimination
// coefficients of the solver, the level fluxes and the layer divergence.
enum RegRow {
  kRgFT, kRgFR, kRgFT0, kRgFC1, kRgFC2, kRgFOM,
  kRgCT, kRgCR, kRgCT0, kRgCC1, kRgCC2, kRgCOM,
  kRgFT0D, kRgCT0D,          // unscaled direct transmissions (i_direct_tau = ip_direct_noscaling)
  kRgFU, kRgFD, kRgFDIR, kRgDIV, kRegRows,
  // three regions: the convective region's coefficients after the rows
  // above (the stratiform region uses the cloudy rows)
  kRgVT = kRegRows, kRgVR, kRgVT0, kRgVC1, kRgVC2, kRgVOM, kRgVT0D, kRegRows3
};
// The solver's elimination coefficients, kept in FP64 in every build: the
// serial solve runs on one lane in FP64 from the coefficients of the layers.
enum RegDRow { kRgB11, kRgB21, kRgB22, kRgG11, kRgG12, kRgG21, kRgG22, kRgH1, kRgH2, kRegDRows,
               // three regions (Hogan's form): the convective region's
               // elimination coefficients and its solar sources in FP64
               kRgB33 = kRegDRows, kRgG33, kRgH3, kRgSUV, kRgSDV, kRegDRows3 };

// The layout of a column of batch p: nb bands staged at a time, n_groups
// solve groups of P lanes, LP = P*CH layer slots.
template <class R>
__host__ __device__ inline SmemLayout make_layout(const FluxParams &p, int LP, int P, int nb, int n_groups,
                                                  bool mcica, bool raw_ok = false) {
  const int max_abs = p.max_abs, n_comp = mcica ? p.n_condensed : 0, n_sub = mcica ? p.n_subcol_gen : 0;
  const bool lw = p.isolir == SOCGPU_IP_INFRA_RED;
  SmemLayout s{};
  s.LP = LP; s.nb = nb; s.max_abs = max_abs; s.n_comp = n_comp; s.n_sub = n_sub; s.n_groups = n_groups;
  size_t o = 0;
  auto take = [&](size_t elems) { size_t r = (o + 15) & ~(size_t)15; o = r + elems * sizeof(R); return r; };
  auto take_int = [&](size_t elems) { size_t r = (o + 15) & ~(size_t)15; o = r + elems * sizeof(int); return r; };
  auto take_dbl = [&](size_t elems) { size_t r = (o + 15) & ~(size_t)15; o = r + elems * sizeof(double); return r; };
  s.off_p = take(LP);
  s.off_t = take(LP);
  s.off_mass = take(LP);
  s.off_kgt = take((size_t)nb * LP);
  s.off_kes = take((size_t)nb * LP);
  s.off_kabs = take((size_t)nb * LP);
  s.off_asym = take((size_t)nb * LP);
  s.off_fwd = take((size_t)nb * LP);
  s.off_amt = take((size_t)nb * max_abs * LP);
  s.off_bscal = take((size_t)nb * kBandScal);
  s.off_planck = lw ? take((size_t)nb * (LP + 1)) : o;
  s.off_dB = lw ? take((size_t)nb * LP) : o;
  s.off_dB2 = lw ? take((size_t)nb * LP) : o;
  if (mcica) {
    s.off_phf_nc = take((size_t)nb * LP);
    s.off_fwd_nc = take((size_t)nb * LP);
    s.off_c_ke = take((size_t)nb * n_comp * LP);
    s.off_c_ks = take((size_t)nb * n_comp * LP);
    s.off_c_ka = take((size_t)nb * n_comp * LP);
    s.off_c_phf = take((size_t)nb * n_comp * LP);
    s.off_c_fwd = take((size_t)nb * n_comp * LP);
    s.off_wcld = take(LP);
    s.off_frac = take((size_t)(p.n_cloud_type > 2 ? p.n_cloud_type : 2) * LP);
    s.off_csub = take((size_t)n_sub * LP);
  }
  // equivalent extinction, solar: each minor absorber's direct-beam factor
  s.off_aux = (p.keqv && !lw) ? take((size_t)nb * max_abs * LP) : o;
  // lookup tables: interpolation factors and packed indices of each slot
  s.off_lkf = p.lk_on ? take((size_t)4 * LP) : o;
  s.off_lki = p.lk_on ? take_int(LP) : o;
  s.off_sbf = p.n_sb > 0 ? take((size_t)p.n_sb * LP) : o;
  s.off_sbj = p.n_sb > 0 ? take_int((size_t)p.n_sb * LP) : o;
  // per-group scratch row for k of per-term scaled absorbers
  s.off_kscr = p.term_scr ? take((size_t)n_groups * LP) : o;
  // cloud regions: the column's interface coefficients and cloud top, and
  // each group's rows for the serial two-region solve
  const bool region = mcica && p.region;
  const bool triple = region && p.triple;
  s.reg_rows = triple ? kRegRows3 : kRegRows;
  s.regd_rows = triple ? kRegDRows3 : kRegDRows;
  s.off_ovl = region ? take((size_t)(triple ? 18 : 8) * (LP + 1)) : o;
  s.off_reg = region ? take((size_t)n_groups * s.reg_rows * (LP + 1)) : o;
  s.off_regd = region ? take_dbl((size_t)n_groups * s.regd_rows * (LP + 1)) : o;
  s.off_nct = region ? take_int(4) : o;
  // three regions: the stratiform and convective shares of each layer's
  // cloud (frac_region), by layer
  s.off_frr = triple ? take((size_t)2 * LP) : o;
  // the direct beam without delta-scaling: each group's row of the layers'
  // unscaled direct transmissions
  s.off_t0d = (!lw && p.i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING && !region) ? take((size_t)n_groups * LP) : o;
  // per-group accumulator slices, offset by P words mod 32 so that the
  // groups of one warp land on different banks
  const int words = (int)(sizeof(R) / 4);
  int stride = kNumAcc * (LP + 1);
  int rem = (stride * words) % 32;
  int want = (P * words) % 32;
  while (rem != want) { ++stride; rem = (stride * words) % 32; }
  s.acc_stride = stride;
  s.off_acc = take((size_t)n_groups * stride);
  // The raw inputs of the column: layer fields, gas mixing ratios (up to
  // kMaxRawGas species), modal aerosol and the surface values, when the
  // whole band range is staged at once.  They are read only by the staging,
  // before the accumulators are cleared, so they share their space.
  s.raw_on = 0; s.raw_n = 0;
  if (raw_ok && nb == p.last_band - p.first_band + 1) {
    const int L = p.n_layer;
    int n = 0;
    auto seg = [&](int len) { int r = n; n += len; return r; };
    s.r_p = seg(L); s.r_t = seg(L); s.r_mass = seg(L);
    s.r_gas = seg((p.l_gas && p.nd_species <= kMaxRawGas) ? p.nd_species * L : 0);
    const bool aer = p.l_aerosol_mode && p.n_mode > 0;
    s.r_mmr = seg(aer ? p.n_mode * L : 0);
    s.r_mabs = seg(aer ? p.n_mode * nb * L : 0);
    s.r_msca = seg(aer ? p.n_mode * nb * L : 0);
    s.r_masy = seg(aer ? p.n_mode * nb * L : 0);
    s.r_sol = seg(!lw && p.solar_irrad ? 1 : 0);
    s.r_zen = seg(!lw && p.zen_0 ? 1 : 0);
    s.r_alb = seg(2 * nb);
    s.r_tg = seg(lw && p.t_ground ? 1 : 0);
    s.r_fg = seg(lw && p.flux_ground ? nb : 0);
    s.r_tl = seg(lw && p.t_level ? L + 1 : 0);
    s.raw_on = 1; s.raw_n = n;
    const size_t need = s.off_acc + (size_t)n * sizeof(double);
    if (need > o) o = need;
  }
  s.bytes = (o + 15) & ~(size_t)15;
  return s;
}

// Pressure/temperature scaling of a k-term (scale_absorb.F90:110-224).
__device__ __forceinline__ double scale_factor_ref(int fnc, double p, double t, double p_ref, double t_ref,
                                                   const double *sp, int l_doppler, double dop) {
  double off = l_doppler ? dop : 0.0;
  if (fnc == SOCGPU_IP_SCALE_POWER_LAW) {
    double t_inv = 1.0 / t_ref, p_ref_off_inv = 1.0 / (p_ref + off);
    return pow((p + off) * p_ref_off_inv, sp[0]) * pow(t * t_inv, sp[1]);
  } else if (fnc == SOCGPU_IP_SCALE_POWER_QUAD) {
    double p_ref_off_inv = 1.0 / (p_ref + off), t_inv = 1.0 / t_ref;
    double pwk = pow((p + off) * p_ref_off_inv, sp[0]);
    double tmp = t * t_inv - 1.0;
    return pwk * (1.0 + tmp * sp[1] + sp[2] * tmp * tmp);
  } else if (fnc == SOCGPU_IP_SCALE_DOPPLER_QUAD) {
    double pwk = pow((p + sp[1]) / (p_ref + sp[1]), sp[0]);
    double tmp = t * (1.0 / t_ref) - 1.0;
    return pwk * (1.0 + tmp * sp[2] + sp[3] * tmp * tmp);
  }
  return 1.0;
}
__device__ __forceinline__ float scale_factor_mix(int fnc, float p, float t, float p_ref, float t_ref,
                                                  const float *sp, int l_doppler, float dop) {
  float off = l_doppler ? dop : 0.0f;
  if (fnc == SOCGPU_IP_SCALE_POWER_LAW) {
    return exp2f(sp[0] * __log2f((p + off) / (p_ref + off)) + sp[1] * __log2f(t / t_ref));
  } else if (fnc == SOCGPU_IP_SCALE_POWER_QUAD) {
    float pwk = exp2f(sp[0] * __log2f((p + off) / (p_ref + off)));
    float tmp = t / t_ref - 1.0f;
    return pwk * (1.0f + tmp * sp[1] + sp[2] * tmp * tmp);
  } else if (fnc == SOCGPU_IP_SCALE_DOPPLER_QUAD) {
    float pwk = exp2f(sp[0] * __log2f((p + sp[1]) / (p_ref + sp[1])));
    float tmp = t / t_ref - 1.0f;
    return pwk * (1.0f + tmp * sp[2] + sp[3] * tmp * tmp);
  }
  return 1.0f;
}

// Band Planck flux (planck_flux_band_mod.F90:33-48), Horner in T/T_ref.
__device__ __forceinline__ double planck_ref(const double *c, int n_deg, double t_ratio) {
  double f = c[n_deg];
  for (int j = n_deg - 1; j >= 0; --j) f = f * t_ratio + c[j];
  return f;
}
__device__ __forceinline__ float planck_mix(const float *c, int n_deg, float x) {
  float f = c[n_deg];
  for (int j = n_deg - 1; j >= 0; --j) f = f * x + c[j];
  return f;
}
// B(x1) - B(x0) without cancellation: x1^j - x0^j = (x1 - x0) d_j with
// d_j = x1 d_{j-1} + x0^(j-1).
__device__ __forceinline__ float planck_diff_mix(const float *c, int n_deg, float x1, float x0) {
  float d = 0.0f, p0 = 1.0f, sum = 0.0f;
  for (int j = 1; j <= n_deg; ++j) {
    d = x1 * d + p0;
    p0 *= x0;
    sum += c[j] * d;
  }
  return (x1 - x0) * sum;
}

// ---------------------------------------------------------------------------
// SRC: the source of the radiation, SOCGPU_IP_SOLAR or SOCGPU_IP_INFRA_RED,
// fixed at compile time so that each kernel carries only its own paths (the
// solar kernel without the Planck terms and the IR coefficients, and the
// reverse): a smaller body keeps the hot loop in the instruction cache.
template <class R, bool MIX, int P, int CH, bool NOSCAT, bool MCICA, int SRC>
struct FluxKernel {
  using Acc = R;
  static constexpr bool kFP64 = (sizeof(R) == 8);
  static constexpr int LP = P * CH;

  // Fetch the column's raw inputs ahead of staging (fetch_raw) for tiles of
  // at most 16 lanes per solve.  Measured on GB300: their CTAs have few warps
  // (long chunks hold many registers), so each CTA's staging round trips
  // stalled most of its warps; the 32-lane tiles' 8-warp CTAs hide them, and
  // the prefetch cost them 8 %.
  static constexpr bool kRawFetch = P <= 16;
  __device__ static __forceinline__ int slot(int i) { return (i % CH) * P + i / CH; }
  __device__ static __forceinline__ int layer_of_slot(int s) { return (s % P) * CH + s / P; }
  __device__ static __forceinline__ int level_slot(int lev) { return lev == 0 ? LP : slot(lev - 1); }

  // Single scattering + delta rescaling + two-stream coefficients of a cell.
  // kgt/kes/kabs: grey extinction, scattering, absorption; asym/fwd: g' and f.
  __device__ static __forceinline__ void cell_coef(const FluxParams &p, R kgt, R kes, R kabs, R kgas,
                                                   R dm, R asym, R fwd, R sec0,
                                                   R &T, R &Rf, R &T0, R &c1, R &c2, R &omtr) {
    if constexpr (kFP64) {
      // single_scattering.F90:119-164, rescale_tau_omega.F90:73-80
      double tau, om;
      if (p.i_scatter_method == SOCGPU_IP_SCATTER_FULL) {
        double k_total = kgt + kgas;
        tau = k_total * dm;
        om = kes / (k_total + kTiny64);
        double cap = 1.0 - 3.2e1 * kEps64;
        if (om > cap) om = cap;
      } else if (p.i_scatter_method == SOCGPU_IP_NO_SCATTER_ABS) {
        tau = (kgt + kgas - kes) * dm; om = 0.0;
      } else {
        tau = (kgt + kgas) * dm; om = 0.0;
      }
      if (p.l_rescale) {
        tau = tau * (1.0 - om * fwd);
        om = om * (1.0 - fwd) / (1.0 - om * fwd);
      }
      Coef c = NOSCAT ? fast_lw_ref(p.l_ir_source_quad, tau)
                      : two_coeff_ref(SRC, p.i_2stream, p.l_ir_source_quad, asym, om, tau, sec0);
      T = c.T; Rf = c.R; T0 = c.T0; c1 = c.c1; c2 = c.c2; omtr = R(0);
    } else {
      float tau, om, omc;
      if (p.i_scatter_method == SOCGPU_IP_SCATTER_FULL) {
        float k_total = kgt + kgas;
        float inv = 1.0f / fmaxf(k_total, 1.0e-30f);
        tau = k_total * dm;
        om = kes * inv;
        omc = (kabs + kgas) * inv;                 // 1 - omega without cancellation
        const float floor_c = (float)(3.2e1 * kEps64);
        if (!(omc > floor_c)) { omc = floor_c; om = 1.0f - floor_c; }
      } else if (p.i_scatter_method == SOCGPU_IP_NO_SCATTER_ABS) {
        tau = (kabs + kgas) * dm; om = 0.0f; omc = 1.0f;
      } else {
        tau = (kgt + kgas) * dm; om = 0.0f; omc = 1.0f;
      }
      if (p.l_rescale) {
        float den = fmaf(-om, fwd, 1.0f);
        tau = tau * den;
        float inv = 1.0f / den;
        om = om * (1.0f - fwd) * inv;
        omc = omc * inv;                            // 1 - omega' = (1-omega)/(1-omega f)
      }
      const SchemeF sc{p.scheme_f[0], p.scheme_f[1], p.scheme_f[2], p.scheme_f[3], p.scheme_f[4]};
      CoefF c = NOSCAT ? fast_lw_mix(p.l_ir_source_quad, tau)
                       : two_coeff_mix(SRC, sc, p.l_ir_source_quad, asym, om, omc, tau, sec0);
      T = c.T; Rf = c.R; T0 = c.T0; c1 = c.c1; c2 = c.c2; omtr = c.omtr;
    }
  }

  struct Smem {
    R *p, *t, *mass, *kgt, *kes, *kabs, *asym, *fwd, *amt, *bscal, *planck, *dB, *dB2;
    R *phf_nc, *fwd_nc, *c_ke, *c_ks, *c_ka, *c_phf, *c_fwd, *wcld, *frac, *csub;
    R *aux, *lkf, *sbf, *kscr;
    int *lki, *sbj;
    R *ovl, *reg, *t0d, *frr;
    double *regd;
    int *nct;
    Acc *acc;
    // the column's raw inputs (null: read them from global memory)
    const double *raw;
    int r_p, r_t, r_mass, r_gas, r_mmr, r_mabs, r_msca, r_masy, r_sol, r_zen, r_alb, r_tg, r_fg, r_tl;
  };

  __device__ static Smem bind(unsigned char *smem, const SmemLayout &l) {
    Smem s;
    s.p = (R *)(smem + l.off_p); s.t = (R *)(smem + l.off_t); s.mass = (R *)(smem + l.off_mass);
    s.kgt = (R *)(smem + l.off_kgt); s.kes = (R *)(smem + l.off_kes); s.kabs = (R *)(smem + l.off_kabs);
    s.asym = (R *)(smem + l.off_asym); s.fwd = (R *)(smem + l.off_fwd); s.amt = (R *)(smem + l.off_amt);
    s.bscal = (R *)(smem + l.off_bscal);
    s.planck = (R *)(smem + l.off_planck); s.dB = (R *)(smem + l.off_dB); s.dB2 = (R *)(smem + l.off_dB2);
    s.phf_nc = (R *)(smem + l.off_phf_nc); s.fwd_nc = (R *)(smem + l.off_fwd_nc);
    s.c_ke = (R *)(smem + l.off_c_ke); s.c_ks = (R *)(smem + l.off_c_ks); s.c_ka = (R *)(smem + l.off_c_ka);
    s.c_phf = (R *)(smem + l.off_c_phf); s.c_fwd = (R *)(smem + l.off_c_fwd);
    s.wcld = (R *)(smem + l.off_wcld); s.frac = (R *)(smem + l.off_frac); s.csub = (R *)(smem + l.off_csub);
    s.aux = (R *)(smem + l.off_aux);
    s.lkf = (R *)(smem + l.off_lkf); s.lki = (int *)(smem + l.off_lki);
    s.sbf = (R *)(smem + l.off_sbf); s.sbj = (int *)(smem + l.off_sbj);
    s.kscr = (R *)(smem + l.off_kscr);
    s.ovl = (R *)(smem + l.off_ovl); s.reg = (R *)(smem + l.off_reg); s.nct = (int *)(smem + l.off_nct);
    s.regd = (double *)(smem + l.off_regd);
    s.t0d = (R *)(smem + l.off_t0d);
    s.frr = (R *)(smem + l.off_frr);
    s.acc = (Acc *)(smem + l.off_acc);
    s.raw = l.raw_on ? (const double *)(smem + l.off_acc) : nullptr;
    s.r_p = l.r_p; s.r_t = l.r_t; s.r_mass = l.r_mass; s.r_gas = l.r_gas; s.r_mmr = l.r_mmr;
    s.r_mabs = l.r_mabs; s.r_msca = l.r_msca; s.r_masy = l.r_masy; s.r_sol = l.r_sol; s.r_zen = l.r_zen;
    s.r_alb = l.r_alb; s.r_tg = l.r_tg; s.r_fg = l.r_fg; s.r_tl = l.r_tl;
    return s;
  }

  // ---------------- lookup-table k scaling ----------------------------------
  // The staged interpolation factors of the column (passed on their own so
  // that calls need not spill the whole shared-memory map).
  struct Lk {
    const R *f;                 // fac00, fac10, fac01, fac11 of each slot
    const int *idx;             // jp | jt << 8 | jtt << 16
    const R *sbf;               // gas-fraction weight of each self-broadened index and slot
    const int *sbj;             // its indices jgf | jgfp1 << 8
  };
  __device__ static __forceinline__ Lk lk_of(const Smem &S) { return Lk{S.lkf, S.lki, S.sbf, S.sbj}; }
  __device__ static __forceinline__ const R *lk_grid(const FluxParams &p) {
    if constexpr (kFP64) return p.lk_grid; else return p.lk_grid_f;
  }
  __device__ static __forceinline__ const R *lk_table(const FluxParams &p) {
    if constexpr (kFP64) return p.k_lookup; else return p.k_lookup_f;
  }
  // Largest index k in 0..n-2 with tab[k] <= x (MINLOC of the non-negative
  // differences in inter_pt_lookup.F90, for increasing tables).
  __device__ static __forceinline__ int below(const R *tab, int n, R x) {
    int lo = 0, hi = n - 2;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
  }
  // Interpolation factors of slot s (inter_pt_lookup.F90:146-268): pressure
  // and temperature weights and indices, and the gas fractions of the
  // self-broadened absorbers.
  __device__ static __forceinline__ void lookup_slot(const FluxParams &p, R *lkf, int *lki, R *sbf, int *sbj, R pv,
                                                  R tv, int col, int s, int i) {
    const R eps = kFP64 ? (R)kEps64 : R(0);
    const int npre = p.lk_n_pre, ntmp = p.lk_n_tmp;
    const R *g = lk_grid(p), *tt = g + npre;
    const R lo_p = g[0] + fmax(fabs(g[0]) * eps, eps), hi_p = g[npre - 1] - fmax(fabs(g[npre - 1]) * eps, eps);
    R x = log(pv);
    x = fmin(fmax(x, lo_p), hi_p);
    const int jp = below(g, npre, x);
    const R fp = (x - g[jp]) / (g[jp + 1] - g[jp]);
    const R *t0 = tt + (size_t)ntmp * jp, *t1 = t0 + ntmp;
    R tl = fmin(fmax(tv, t0[0] * (R(1) + eps)), t0[ntmp - 1] * (R(1) - eps));
    const int jt = below(t0, ntmp, tl);
    const R ft = (tl - t0[jt]) / (t0[jt + 1] - t0[jt]);
    tl = fmin(fmax(tv, t1[0] * (R(1) + eps)), t1[ntmp - 1] * (R(1) - eps));
    const int jtt = below(t1, ntmp, tl);
    const R ftt = (tl - t1[jtt]) / (t1[jtt + 1] - t1[jtt]);
    const R compfp = R(1) - fp;
    lkf[s] = compfp * (R(1) - ft);
    lkf[LP + s] = fp * (R(1) - ftt);
    lkf[2 * LP + s] = compfp * ft;
    lkf[3 * LP + s] = fp * ftt;
    lki[s] = jp | (jt << 8) | (jtt << 16);
    if (p.n_sb > 0) {
      const int ngf = p.lk_n_gf;
      const R *gf = tt + (size_t)ntmp * npre;
      const R lo_g = gf[0] + fmax(gf[0] * eps, eps), hi_g = gf[ngf - 1] - fmax(gf[ngf - 1] * eps, eps);
      const size_t base = (size_t)col + (size_t)p.nd_profile * i;
      const size_t stride = (size_t)p.nd_profile * p.nd_layer;
      const R q = p.l_water ? load_in<R>(p.gas_mix_ratio + base + stride * (p.i_water >= 0 ? p.i_water : 0)) : R(0);
      for (int k = 0; k < p.n_sb; ++k) {
        const R mr = load_in<R>(p.gas_mix_ratio + base + stride * p.sb_species[k]);
        const R rg = (R)p.sb_ratio_gas[k], rw = (R)p.ratio_water;
        R v;
        if (!p.l_water) v = mr * rg;
        else if (p.l_mixing_ratio) v = mr * rg / (R(1) + q * rw);
        else v = mr * rg / (R(1) + q * (rw - R(1)));
        if (ngf == 1) {
          sbf[(size_t)k * LP + s] = R(1);
          sbj[(size_t)k * LP + s] = 0;
        } else {
          v = fmin(fmax(v, lo_g), hi_g);
          const int jg = below(gf, ngf, v);
          sbf[(size_t)k * LP + s] = R(1) - (v - gf[jg]) / (gf[jg + 1] - gf[jg]);
          sbj[(size_t)k * LP + s] = jg | ((jg + 1) << 8);
        }
      }
    }
  }
  // k of one term from the P/T tables (radiance_calc.F90:1097-1145), times
  // the absorber amount a.
  __device__ static __forceinline__ R lookup_k(const FluxParams &p, Lk lk, int off, int sb, int s, R a) {
    const R *K = lk_table(p) + off;
    const int nt = p.lk_n_tmp, idx = lk.idx[s];
    const int jp = idx & 255, jt = (idx >> 8) & 255, jtt = idx >> 16;
    const R f00 = lk.f[s], f10 = lk.f[LP + s], f01 = lk.f[2 * LP + s], f11 = lk.f[3 * LP + s];
    const int i00 = jt + nt * jp, i10 = jtt + nt * (jp + 1), i01 = jt + 1 + nt * jp, i11 = jtt + 1 + nt * (jp + 1);
    R ke;
    if (sb < 0) {
      ke = f00 * K[i00] + f10 * K[i10] + f01 * K[i01] + f11 * K[i11];
    } else {
      const int jj = lk.sbj[(size_t)sb * LP + s];
      const R fg = lk.sbf[(size_t)sb * LP + s];
      const R *K0 = K + (size_t)nt * p.lk_n_pre * (jj & 255), *K1 = K + (size_t)nt * p.lk_n_pre * (jj >> 8);
      ke = fg * (f00 * K0[i00] + f10 * K0[i10] + f01 * K0[i01] + f11 * K0[i11])
         + (R(1) - fg) * (f00 * K1[i00] + f10 * K1[i10] + f01 * K1[i01] + f11 * K1[i11]);
    }
    ke = ke > R(0) ? ke : R(0);
    R v = ke * a;
    v = v > R(0) ? v : R(0);
    // unfilled table entries (about 1e37) would overflow FP32 optical depths;
    // any k this large already makes the layer opaque
    if constexpr (!kFP64) v = fminf(v, 1.0e30f);
    return v;
  }
  // k of one term from a temperature-only table (inter_t_lookup.F90:70-86,
  // radiance_calc.F90:1154-1166), times the absorber amount a.
  __device__ static __forceinline__ R t_lookup_k(const FluxParams &p, const BandGas &gs, int off, R tl, R a) {
    const R eps = kFP64 ? (R)kEps64 : R(0);
    const R *tg;
    const R *K;
    if constexpr (kFP64) { tg = p.t_lookup_gas; K = p.k_lookup; } else { tg = p.t_lookup_gas_f; K = p.k_lookup_f; }
    tg += (size_t)p.nd_t_lookup_gas * gs.species;
    K += off;
    const int n = gs.n_t;
    const R t = fmin(fmax(tl, tg[0] * (R(1) + eps)), tg[n - 1] * (R(1) - eps));
    const int jt = below(tg, n, t);
    const R wt = R(1) - (t - tg[jt]) / (tg[jt + 1] - tg[jt]);
    R ke = wt * K[jt] + (R(1) - wt) * K[jt + 1];
    ke = ke > R(0) ? ke : R(0);
    const R v = ke * a;
    return v > R(0) ? v : R(0);
  }
  // Wen-Yi Zhong's scaling of the CO2 (band 4) and O3 (band 6) terms
  // (scale_absorb.F90:238-281); b is the 0-based band.
  __device__ static __forceinline__ R wenyi_factor(const FluxParams &p, int b, int iex, R pl, R tl) {
    const R *W;
    if constexpr (kFP64) W = p.wenyi; else W = p.wenyi_f;
    const R *plg = W, *ttb = W + 26, *tto = W + 36, *gk250b = W + 45;
    const R *gk4 = gk250b + p.wenyi_n4, *gk6 = gk4 + (size_t)260 * p.wenyi_n4;
    R cgp = log(pl / R(100));
    if (cgp < R(-5.5)) cgp = R(-5.5);
    int jp = (int)((R(5.5) + cgp) * R(2)) + 1;
    jp = jp < 1 ? 1 : (jp > 26 ? 26 : jp);
    const int jp1 = jp + 1 < 26 ? jp + 1 : 26;
    const bool b4 = (b == 3);
    const int n_t = b4 ? 10 : 9;
    const R *gk = b4 ? gk4 : gk6, *tref = b4 ? ttb : tto;
    int jt = (int)((tl - R(240)) / R(20) + (b4 ? R(7) : R(5)));
    jt = jt < 1 ? 1 : (jt > n_t ? n_t : jt);
    const int jt1 = jt + 1 < n_t ? jt + 1 : n_t;
    auto G = [&](int a, int c) { return gk[(size_t)(a - 1) + (size_t)n_t * ((size_t)(c - 1) + (size_t)26 * iex)]; };
    const R dp = (cgp - plg[jp - 1]) * R(2);
    const R gkpb = G(jt, jp) + (G(jt, jp1) - G(jt, jp)) * dp;
    const R gkpc = G(jt1, jp) + (G(jt1, jp1) - G(jt1, jp)) * dp;
    const R v = gkpb + (gkpc - gkpb) * (tl - tref[jt - 1]) / R(20);
    return b4 ? v / gk250b[iex] : v;
  }
  // k of one term of absorber gs at slot s (k_abs_layer of
  // radiance_calc.F90:1330-1470): a is the staged amount (the scaled amount
  // under ip_scale_band, the mixing ratio otherwise), kj the term's k, sc its
  // scaling parameters, lk_off its lookup table, iex the term.
  __device__ static __forceinline__ R term_k(const FluxParams &p, Lk lk, const BandGas &gs, int b, R kj, const R *sc,
                             int lk_off, int iex, R a, int s, R pl, R tl) {
    if (gs.i_scale_k != SOCGPU_IP_SCALE_TERM) return kj * a;
    const int fnc = gs.i_scale_fnc;
    if (fnc == SOCGPU_IP_SCALE_LOOKUP) return lookup_k(p, lk, lk_off, gs.sb, s, a);
    if (fnc == SOCGPU_IP_SCALE_T_LOOKUP) return t_lookup_k(p, gs, lk_off, tl, a);
    R gf;
    if (fnc == SOCGPU_IP_SCALE_WENYI) gf = wenyi_factor(p, b, iex, pl, tl);
    else if constexpr (kFP64) gf = scale_factor_ref(fnc, pl, tl, gs.p_ref, gs.t_ref, sc, gs.l_doppler, gs.doppler_cor);
    else gf = scale_factor_mix(fnc, pl, tl, gs.p_ref_f, gs.t_ref_f, sc, gs.l_doppler, gs.doppler_cor_f);
    const R v = gf * a;
    return kj * (v > R(0) ? v : R(0));
  }


  // The temperature at level lev, in T.
  template <class T>
  __device__ static __forceinline__ T t_lev(const FluxParams &p, const Smem &S, int col, int lev) {
    if (S.raw) return raw_in<T>(S.raw[S.r_tl + lev]);
    return load_in<T>(p.t_level + (size_t)col + (size_t)p.nd_profile * lev);
  }

  // The column's raw FP64 inputs into shared memory (layout of make_layout):
  // one asynchronous 8-byte copy per element, all in flight together, so
  // that staging waits for one round trip to memory instead of one per
  // dependent load.  Every source is an element the staging would read.
  __device__ static void fetch_raw(const FluxParams &p, const SmemLayout &l, double *raw, int col, int bstart) {
    const int L = p.n_layer, ndp = p.nd_profile, ndl = p.nd_layer, nt = blockDim.x, nb = l.nb;
    const size_t c = (size_t)col;
    for (int k = threadIdx.x; k < L; k += nt) {
      cp_async8(raw + l.r_p + k, p.p + c + (size_t)ndp * k);
      cp_async8(raw + l.r_t + k, p.t + c + (size_t)ndp * k);
      cp_async8(raw + l.r_mass + k, p.mass + c + (size_t)ndp * k);
    }
    for (int k = threadIdx.x; k < l.r_mmr - l.r_gas; k += nt) {
      const int sp = k / L, i = k - sp * L;
      cp_async8(raw + l.r_gas + k, p.gas_mix_ratio + c + (size_t)ndp * ((size_t)i + (size_t)ndl * sp));
    }
    for (int k = threadIdx.x; k < l.r_mabs - l.r_mmr; k += nt) {
      const int m = k / L, i = k - m * L;
      cp_async8(raw + l.r_mmr + k, p.mode_mix_ratio + c + (size_t)ndp * ((size_t)i + (size_t)ndl * m));
    }
    for (int k = threadIdx.x; k < l.r_msca - l.r_mabs; k += nt) {
      const int mb = k / L, i = k - mb * L, m = mb / nb, b = bstart + (mb - m * nb);
      const size_t q4 = c + (size_t)ndp * ((size_t)i + (size_t)ndl * ((size_t)m + (size_t)p.nd_mode * b));
      cp_async8(raw + l.r_mabs + k, p.mode_absorption + q4);
      cp_async8(raw + l.r_msca + k, p.mode_scattering + q4);
      cp_async8(raw + l.r_masy + k, p.mode_asymmetry + q4);
    }
    if (threadIdx.x == 0) {
      if (l.r_zen > l.r_sol) cp_async8(raw + l.r_sol, p.solar_irrad + c);
      if (l.r_alb > l.r_zen) cp_async8(raw + l.r_zen, p.zen_0 + c);
      if (l.r_fg > l.r_tg) cp_async8(raw + l.r_tg, p.t_ground + c);
    }
    for (int k = threadIdx.x; k < 2 * nb; k += nt)
      cp_async8(raw + l.r_alb + k, p.rho_alb + c + (size_t)ndp * ((size_t)(k & 1) + 2 * (size_t)(bstart + (k >> 1))));
    for (int k = threadIdx.x; k < l.r_tl - l.r_fg; k += nt)
      cp_async8(raw + l.r_fg + k, p.flux_ground + c + (size_t)ndp * (size_t)(bstart + k));
    for (int k = threadIdx.x; k < l.raw_n - l.r_tl; k += nt)
      cp_async8(raw + l.r_tl + k, p.t_level + c + (size_t)ndp * k);
    asm volatile("cp.async.wait_all;\n" ::: "memory");
  }

  __device__ static void run(const FluxParams &p, const int col) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int L = p.n_layer;
    const int nb_all = p.last_band - p.first_band + 1;
    const int nbat = p.band_batch;             // bands staged at a time
    const int nthreads = blockDim.x;
    const int n_groups = nthreads / P;
    constexpr bool lw = (SRC == SOCGPU_IP_INFRA_RED);
    const int max_abs = p.max_abs;
    const SmemLayout lay = make_layout<R>(p, LP, P, nbat, n_groups, MCICA, kRawFetch);
    const Smem S = bind(smem, lay);
    const int ndp = p.nd_profile;
    if (lay.raw_on) {
      fetch_raw(p, lay, (double *)(smem + lay.off_acc), col, p.first_band - 1);
      __syncthreads();
    }

    // ---------------- column fields and accumulators ------------------------
    for (int s = threadIdx.x; s < LP; s += nthreads) {
      const int i = layer_of_slot(s);
      if (i < L) {
        if (S.raw) {
          S.p[s] = raw_in<R>(S.raw[S.r_p + i]);
          S.t[s] = raw_in<R>(S.raw[S.r_t + i]);
          S.mass[s] = raw_in<R>(S.raw[S.r_mass + i]);
        } else {
          S.p[s] = load_in<R>(p.p + (size_t)col + (size_t)ndp * i);
          S.t[s] = load_in<R>(p.t + (size_t)col + (size_t)ndp * i);
          S.mass[s] = load_in<R>(p.mass + (size_t)col + (size_t)ndp * i);
        }
        if (p.lk_on) lookup_slot(p, S.lkf, S.lki, S.sbf, S.sbj, S.p[s], S.t[s], col, s, i);
      }
    }
    if (!S.raw)
      for (int q = threadIdx.x; q < n_groups * lay.acc_stride; q += nthreads) S.acc[q] = Acc(0);
    if (MCICA) stage_cloud_column(p, S, col);
    if (MCICA && p.region) {
      if (p.triple) stage_regions3(p, S, col, LP);
      else stage_regions(p, S, col, LP);
    }
    const int gid = threadIdx.x / P;
    const int r = threadIdx.x % P;
    const R sec0 = !p.zen_0 ? R(1) : (S.raw && S.r_alb > S.r_zen) ? raw_in<R>(S.raw[S.r_zen]) : load_in<R>(p.zen_0 + col);
    Acc *acc = S.acc + (size_t)gid * lay.acc_stride;
    __syncthreads();

    for (int bb = 0; bb < nb_all; bb += nbat) {
      const int nb = min(nbat, nb_all - bb);
      const int bstart = p.first_band - 1 + bb;
      stage_bands(p, S, col, bstart, nb, lw);
      if (MCICA) stage_cloud_bands(p, S, col, bstart, nb);
      __syncthreads();
      stage_boundary(p, S, col, bstart, nb, lw);
      __syncthreads();
      if (S.raw) {
        // the raw inputs are consumed: their space becomes the accumulators
        // (the whole band range is staged at once, so this runs once)
        for (int q = threadIdx.x; q < n_groups * lay.acc_stride; q += nthreads) S.acc[q] = Acc(0);
        __syncthreads();
      }
      if (p.keqv) {
        stage_keqv(p, S, bstart, nb, sec0);
        __syncthreads();
        fold_keqv(p, S, bstart, nb, sec0);
        __syncthreads();
      }
      // g-point solves.  Every group of every warp runs the same number of
      // rounds so that the full-warp shuffles of the scans always see all
      // 32 lanes; a group with no g-point left in the last round solves the
      // first g-point of the batch and discards it.
      const int g_lo = p.bands[bstart].g_first;
      const int g_hi = p.bands[bstart + nb - 1].g_first + p.bands[bstart + nb - 1].g_count;
      const int rounds = (g_hi - g_lo + n_groups - 1) / n_groups;
      for (int rd = 0; rd < rounds; ++rd) {
        int g = g_lo + rd * n_groups + gid;
        const bool active = g < g_hi;
        if (!active) g = g_lo;
        solve_gpoint(p, S, col, g, bstart, max_abs, sec0, r, acc, lw, active);
      }
      __syncthreads();
      if (lw) {
        // adjust_ir_radiance.F90:75-95: add the band Planck flux back, into
        // the first group's slice
        for (int s = threadIdx.x; s <= LP; s += nthreads) {
          const int lev = (s == LP) ? 0 : layer_of_slot(s) + 1;
          if (lev > L) continue;
          Acc add = Acc(0);
          for (int bi = 0; bi < nb; ++bi) add += S.planck[bi * (LP + 1) + s] * S.bscal[bi * kBandScal + 5];
          S.acc[s] += add;
          S.acc[(LP + 1) + s] += add;
        }
        __syncthreads();
      }
    }

    // ---------------- reduce over groups, write ------------------------------
    for (int lev = threadIdx.x; lev <= L; lev += nthreads) {
      const int s = level_slot(lev);
      Acc up = Acc(0), dn = Acc(0), dir = Acc(0);
      for (int q = 0; q < n_groups; ++q) {
        const Acc *a = S.acc + (size_t)q * lay.acc_stride;
        up += a[s]; dn += a[(LP + 1) + s]; dir += a[2 * (LP + 1) + s];
      }
      const size_t o = (size_t)col + (size_t)ndp * lev;
      p.flux_up[o] = store_out<R>(up);
      p.flux_down[o] = store_out<R>(dn);
      if (p.flux_direct) p.flux_direct[o] = lw ? 0.0 : store_out<R>(dir);
      if (lev < L) {
        // the divergence of layer lev sits at its bottom level's slot
        Acc dlay = Acc(0);
        const int sl = slot(lev);
        for (int q = 0; q < n_groups; ++q) dlay += S.acc[(size_t)q * lay.acc_stride + 3 * (LP + 1) + sl];
        if (p.flux_div) p.flux_div[(size_t)col + (size_t)ndp * lev] = store_out<R>(dlay);
        if (p.heating_rate) {
          // heating rate (l_run_cdf.F90:1340-1380); without l_flux_div the
          // FP64 rate is filled below from the net fluxes
          double hr;
          if constexpr (kFP64) hr = p.l_flux_div ? 8.64e4 * dlay / (ld2(p.mass, col, lev, ndp) * 1.005e3) : 0.0;
          else hr = store_out<R>(8.64e4f * dlay / (S.mass[sl] * 1.005e3f));
          p.heating_rate[(size_t)col + (size_t)ndp * lev] = hr;
        }
      }
    }
    if (kFP64 && p.heating_rate && !p.l_flux_div) {
      __syncthreads();
      for (int i = threadIdx.x; i < L; i += nthreads) {
        double hc = ld2(p.mass, col, i, ndp) * 1.005e3;
        double fn0 = p.flux_down[(size_t)col + (size_t)ndp * i] - p.flux_up[(size_t)col + (size_t)ndp * i];
        double fn1 = p.flux_down[(size_t)col + (size_t)ndp * (i + 1)] - p.flux_up[(size_t)col + (size_t)ndp * (i + 1)];
        p.heating_rate[(size_t)col + (size_t)ndp * i] = 8.64e4 * ((fn0 - fn1) / hc);
      }
    }
  }

  // Grey optics, gas amounts and Planck terms of bands bstart..bstart+nb-1
  // (radiance_calc.F90:883-1600 band loop; slot order).
  __device__ static void stage_bands(const FluxParams &p, const Smem &S, int col, int bstart, int nb, bool lw) {
    const int L = p.n_layer, ndp = p.nd_profile, ndl = p.nd_layer, nthreads = blockDim.x;
    const int max_abs = p.max_abs;
    for (int q = threadIdx.x; q < nb * LP; q += nthreads) {
      const int bi = q / LP, s = q - bi * LP, b = bstart + bi;
      const int i = layer_of_slot(s);
      if (i >= L) continue;
      const BandInfo &bd = p.bands[b];
      // grey optics: grey_opt_prop.F90:470-790 (Rayleigh, modal aerosol)
      R kes = p.l_rayleigh ? (kFP64 ? (R)bd.rayleigh_coeff : (R)bd.rayleigh_f) : R(0);
      R kabs = R(0), phf = R(0), fwd = R(0);
      if (p.l_aerosol) classic_aerosol(p, col, i, b, kabs, kes, phf, fwd);
      if (p.l_aer_prsc) {
        // prescribed species: the sums of the prescribed-property kernel
        const size_t plane = (size_t)(p.last_band - p.first_band + 1) * L;
        const size_t q0 = ((size_t)col * 4 * (p.last_band - p.first_band + 1) + (b - (p.first_band - 1))) * L + i;
        kabs = kabs + load_in<R>(p.aer_prsc + q0);
        kes = kes + load_in<R>(p.aer_prsc + plane + q0);
        phf = phf + load_in<R>(p.aer_prsc + 2 * plane + q0);
        if (p.l_rescale) fwd = fwd + load_in<R>(p.aer_prsc + 3 * plane + q0);
      }
      if (p.l_aerosol_mode) {
        for (int j = 0; j < p.n_mode; ++j) {
          R mmr, g, ka, ksc;
          if (S.raw && S.r_mabs > S.r_mmr) {
            const int qr = (j * nb + bi) * L + i;
            mmr = raw_in<R>(S.raw[S.r_mmr + j * L + i]);
            g = raw_in<R>(S.raw[S.r_masy + qr]);
            ka = raw_in<R>(S.raw[S.r_mabs + qr]);
            ksc = raw_in<R>(S.raw[S.r_msca + qr]);
          } else {
            mmr = load_in<R>(p.mode_mix_ratio + (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * j));
            size_t q4 = (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * ((size_t)j + (size_t)p.nd_mode * b));
            g = load_in<R>(p.mode_asymmetry + q4);
            ka = load_in<R>(p.mode_absorption + q4);
            ksc = load_in<R>(p.mode_scattering + q4);
          }
          kabs = kabs + mmr * ka;
          R ks = mmr * ksc;
          kes = kes + ks;
          phf = phf + ks * g;
          if (p.l_rescale) {
            R ks_phf = ks * g;
            if (p.n_order_forward == 1) fwd = fwd + ks_phf;
            else if (p.n_order_forward == 2) fwd = fwd + ks_phf * g;
            else {
              R gp = R(1);
              for (int o = 0; o < p.n_order_forward; ++o) gp *= g;
              fwd = fwd + ks * gp;
            }
          }
        }
      }
      if (p.l_continuum) {
        // continuum absorption (grey_opt_prop.F90:801-817), amounts as
        // rescale_continuum.F90 (self: molar density of water x water;
        // foreign: air density x water / molar weight of air)
        const R water = load_in<R>(p.gas_mix_ratio + (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * p.i_water));
        const R rho = load_in<R>(p.density + (size_t)col + (size_t)ndp * i);
        for (int j = 0; j < bd.n_cont; ++j) {
          const BandCont &c = bd.cont[j];
          R a;
          if constexpr (kFP64) {
            a = pow(S.p[s] / c.p_ref, c.scale[0]);
            if (c.fnc == SOCGPU_IP_SCALE_POWER_LAW) {
              a = a * pow(S.t[s] / c.t_ref, c.scale[1]);
            } else if (c.fnc == SOCGPU_IP_SCALE_POWER_QUAD) {
              const double x = S.t[s] / c.t_ref - 1.0;
              a = a * (1.0 + c.scale[1] * x + c.scale[2] * (x * x));
            }
            if (c.type == SOCGPU_IP_SELF_CONTINUUM) {
              a = a * (rho * water / ((18.0153 / 28.966) * 28.966e-03)) * water;
            } else if (c.type == SOCGPU_IP_FRN_CONTINUUM) {
              a = p.l_mixing_ratio ? a * rho * water / 28.966e-03 : a * rho * water * (1.0 - water) / 28.966e-03;
            }
            kabs = kabs + c.k * a;
          } else {
            a = __powf(S.p[s] / c.p_ref_f, c.scale_f[0]);
            if (c.fnc == SOCGPU_IP_SCALE_POWER_LAW) {
              a = a * __powf(S.t[s] / c.t_ref_f, c.scale_f[1]);
            } else if (c.fnc == SOCGPU_IP_SCALE_POWER_QUAD) {
              const float x = S.t[s] / c.t_ref_f - 1.0f;
              a = a * (1.0f + c.scale_f[1] * x + c.scale_f[2] * (x * x));
            }
            if (c.type == SOCGPU_IP_SELF_CONTINUUM) {
              a = a * (rho * water * (1.0f / 0.0180153f)) * water;
            } else if (c.type == SOCGPU_IP_FRN_CONTINUUM) {
              a = p.l_mixing_ratio ? a * rho * water * (1.0f / 0.028966f)
                                   : a * rho * water * (1.0f - water) * (1.0f / 0.028966f);
            }
            kabs = kabs + c.k_f * a;
          }
        }
      }
      R kgt = kabs + kes;     // grey_opt_prop.F90:773-790
      if (MCICA) { S.phf_nc[q] = phf; S.fwd_nc[q] = fwd; }
      R asym = phf, f = fwd;
      if (kFP64 ? ((double)kes > kTiny64) : (kes > R(0))) {   // normalisation, grey_opt_prop.F90:840-880
        if (p.l_rescale) { R tinv = R(1) / kes; f = fwd * tinv; asym = phf * tinv; }
        else asym = phf / kes;
      }
      if (p.l_rescale) asym = (asym - f) / (R(1) - f);   // rescale_phase_fnc.F90:120-128
      S.kgt[q] = kgt; S.kes[q] = kes; S.kabs[q] = kabs; S.asym[q] = asym; S.fwd[q] = f;
      // gas amounts (radiance_calc.F90:1330-1470)
      const int n_abs_b = p.l_gas ? min(bd.n_abs, max_abs) : 0;
      for (int j = 0; j < n_abs_b; ++j) {
        const BandGas &gs = bd.gas[j];
        R mmr = (S.raw && S.r_mmr > S.r_gas)
                    ? raw_in<R>(S.raw[S.r_gas + gs.species * L + i])
                    : load_in<R>(p.gas_mix_ratio + (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * gs.species));
        R amt;
        if (gs.i_scale_k == SOCGPU_IP_SCALE_BAND) {
          R gf;
          if constexpr (kFP64)
            gf = scale_factor_ref(gs.i_scale_fnc, S.p[s], S.t[s], gs.p_ref, gs.t_ref, gs.scale, gs.l_doppler,
                                  gs.doppler_cor);
          else
            gf = scale_factor_mix(gs.i_scale_fnc, S.p[s], S.t[s], gs.p_ref_f, gs.t_ref_f, gs.scale_f,
                                  gs.l_doppler, gs.doppler_cor_f);
          R v = gf * mmr;
          amt = v > R(0) ? v : R(0);
        } else {
          amt = mmr;   // ip_scale_null, or ip_scale_term (scaled per term below)
        }
        S.amt[((size_t)bi * max_abs + j) * LP + s] = amt;
      }
    }
    if (lw) {
      // diff_planck_source (diff_planck_source_mod.F90:102-136)
      for (int q = threadIdx.x; q < nb * (LP + 1); q += nthreads) {
        const int bi = q / (LP + 1), s = q - bi * (LP + 1);
        const int lev = (s == LP) ? 0 : layer_of_slot(s) + 1;
        if (lev > L) continue;
        const BandInfo &bd = p.bands[bstart + bi];
        if constexpr (kFP64)
          S.planck[q] = planck_ref(bd.planck, p.n_deg_fit, t_lev<double>(p, S, col, lev) / p.t_ref_planck);
        else
          S.planck[q] = planck_mix(bd.planck_f, p.n_deg_fit,
                                   t_lev<float>(p, S, col, lev) / p.t_ref_planck_f);
      }
      for (int q = threadIdx.x; q < nb * LP; q += nthreads) {
        const int bi = q / LP, s = q - bi * LP;
        const int i = layer_of_slot(s);
        if (i >= L) continue;
        const BandInfo &bd = p.bands[bstart + bi];
        if constexpr (kFP64) {
          double b1 = planck_ref(bd.planck, p.n_deg_fit, t_lev<double>(p, S, col, i + 1) / p.t_ref_planck);
          double bm = planck_ref(bd.planck, p.n_deg_fit, t_lev<double>(p, S, col, i) / p.t_ref_planck);
          S.dB[q] = b1 - bm;
          if (p.l_ir_source_quad) {
            double bl = planck_ref(bd.planck, p.n_deg_fit,
                                   (S.raw ? S.raw[S.r_t + i] : ld2(p.t, col, i, ndp)) / p.t_ref_planck);
            S.dB2[q] = 2.0 * (b1 + bm - 2.0 * bl);
          }
        } else {
          const float x1 = t_lev<float>(p, S, col, i + 1) / p.t_ref_planck_f;
          const float x0 = t_lev<float>(p, S, col, i) / p.t_ref_planck_f;
          S.dB[q] = planck_diff_mix(bd.planck_f, p.n_deg_fit, x1, x0);
          if (p.l_ir_source_quad) {
            const float xl = S.t[s] / p.t_ref_planck_f;
            S.dB2[q] = 2.0f * (planck_diff_mix(bd.planck_f, p.n_deg_fit, x1, xl) +
                               planck_diff_mix(bd.planck_f, p.n_deg_fit, x0, xl));
          }
        }
      }
    }
  }

  // Classic aerosol species in cell (col, i) of band b (opt_prop_aerosol.F90:
  // 273-640 for two-stream phase functions): each active mixing-ratio entry
  // adds its absorption and scattering, interpolated in the layer's mean
  // relative humidity for moist species (radiance_calc.F90:617-623 for the
  // pointer into the common humidity table, clamped to the table here), the
  // first phase-function moment (the asymmetry) and, with rescaling, the
  // forward-scattering moment: a power of the asymmetry for Henyey-Greenstein
  // species, the tabulated moment n_order_forward otherwise.
  __device__ static __forceinline__ void classic_aerosol(const FluxParams &p, int col, int i, int b, R &kabs,
                                                         R &kes, R &phf, R &fwd) {
    const int ndp = p.nd_profile, ndl = p.nd_layer;
    const int row = 2 + p.aer_nphf;
    const R *tab, *hum;
    if constexpr (kFP64) { tab = p.aer_tab; hum = p.aer_hum; } else { tab = p.aer_tab_f; hum = p.aer_hum_f; }
    const R dhum = kFP64 ? (R)p.aer_dhum : (R)p.aer_dhum_f;
    for (int e = 0; e < p.n_aer_mr; ++e) {
      const int j = p.aer_species[e], parm = p.aer_parm[e];
      const R mmr = load_in<R>(p.aer_mix_ratio + (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * p.aer_entry[e]));
      const R *t0 = tab + ((size_t)b * p.aer_n_species + j) * p.aer_nh * row;
      const bool moist = parm == SOCGPU_IP_AEROSOL_PARAM_MOIST || parm == SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST;
      R wu = R(0);
      const R *t1 = t0;
      if (moist) {
        const R mrh = load_in<R>(p.mean_rel_humidity + (size_t)col + (size_t)ndp * i);
        int ip = 1 + (int)(mrh * (R)(p.aer_nh_common - 1));
        ip = ip < 1 ? 1 : (ip > p.aer_nh_common - 1 ? p.aer_nh_common - 1 : ip);
        wu = (mrh - hum[(size_t)j * p.aer_nh + ip - 1]) / dhum;
        t0 = t0 + (size_t)(ip - 1) * row;
        t1 = t0 + row;
      }
      auto at = [&](int c) { return moist ? t0[c] + wu * (t1[c] - t0[c]) : t0[c]; };
      kabs = kabs + mmr * at(0);
      const R ks = mmr * at(1);
      kes = kes + ks;
      const R g = at(2);
      phf = phf + ks * g;
      if (p.l_rescale) {
        const bool hg = p.l_hg || parm == SOCGPU_IP_AEROSOL_PARAM_DRY || parm == SOCGPU_IP_AEROSOL_PARAM_MOIST;
        const int nof = p.n_order_forward;
        if (!hg) {
          fwd = fwd + ks * at(1 + nof);
        } else if (nof == 1) {
          fwd = fwd + ks * g;
        } else if (nof == 2) {
          fwd = fwd + ks * g * g;
        } else {
          R gp = R(1);
          for (int o = 0; o < nof; ++o) gp *= g;
          fwd = fwd + ks * gp;
        }
      }
    }
  }

  // Per-band boundary values (solve_band_random_overlap.F90:565-600,
  // column_solver.F90): incident fluxes, surface albedos and emission.
  __device__ static void stage_boundary(const FluxParams &p, const Smem &S, int col, int bstart, int nb, bool lw) {
    const int L = p.n_layer, ndp = p.nd_profile;
    for (int bi = threadIdx.x; bi < nb; bi += blockDim.x) {
      const int b = bstart + bi;
      const BandInfo &bd = p.bands[b];
      R *v = S.bscal + bi * kBandScal;
      if (S.raw) {
        v[2] = raw_in<R>(S.raw[S.r_alb + 2 * bi]);
        v[3] = raw_in<R>(S.raw[S.r_alb + 2 * bi + 1]);
      } else {
        v[2] = load_in<R>(p.rho_alb + (size_t)col + (size_t)ndp * (0 + 2 * (size_t)b));
        v[3] = load_in<R>(p.rho_alb + (size_t)col + (size_t)ndp * (1 + 2 * (size_t)b));
      }
      v[5] = p.weight_band ? load_in<R>(p.weight_band + b) : R(1);
      if (lw) {
        v[0] = -S.planck[bi * (LP + 1) + LP];
        v[1] = R(0);
        if (p.flux_ground) {
          // the surface's Planck flux given per band (l_flux_ground, tiles)
          v[4] = (S.raw ? raw_in<R>(S.raw[S.r_fg + bi]) : load_in<R>(p.flux_ground + (size_t)col + (size_t)ndp * b)) -
                 S.planck[bi * (LP + 1) + level_slot(L)];
        } else if constexpr (kFP64) {
          double bg = planck_ref(bd.planck, p.n_deg_fit,
                                 (S.raw ? S.raw[S.r_tg] : ld2(p.t_ground, col, 0, ndp)) / p.t_ref_planck);
          v[4] = bg - S.planck[bi * (LP + 1) + level_slot(L)];
        } else {
          const float tg = S.raw ? raw_in<float>(S.raw[S.r_tg]) : load_in<float>(p.t_ground + col);
          v[4] = planck_diff_mix(bd.planck_f, p.n_deg_fit, tg / p.t_ref_planck_f,
                                 t_lev<float>(p, S, col, L) / p.t_ref_planck_f);
        }
      } else {
        if constexpr (kFP64) {
          double sib = (S.raw ? S.raw[S.r_sol] : ld2(p.solar_irrad, col, 0, ndp)) * bd.solar_flux_band;
          v[0] = sib / (S.raw ? S.raw[S.r_zen] : ld2(p.zen_0, col, 0, ndp));
        } else {
          const float sol = S.raw ? raw_in<float>(S.raw[S.r_sol]) : load_in<float>(p.solar_irrad + col);
          const float zen = S.raw ? raw_in<float>(S.raw[S.r_zen]) : load_in<float>(p.zen_0 + col);
          v[0] = sol * bd.solar_flux_band_f / zen;
        }
        v[1] = v[0];
        v[4] = R(0);
      }
    }
  }

  // Cloud-component optics of bands bstart..bstart+nb-1: opt_prop_pade_2
  // (opt_prop_pade_2_mod.F90:99-140), Slingo and Schrecker's fits
  // (opt_prop_water_cloud.F90:231-247, opt_prop_ice_cloud.F90:278-294) and
  // Fu's ice fits (opt_prop_fu_phf_mod.F90:92-130).  Forward scattering is
  // k_scat g^2 (n_order_forward 2) for all of them.
  __device__ static void stage_cloud_bands(const FluxParams &p, const Smem &S, int col, int bstart, int nb) {
    const int L = p.n_layer, ndp = p.nd_profile, ndl = p.nd_layer, ict = p.id_ct;
    const int ndc = ndl - ict, nc = p.n_condensed;
    for (int q = threadIdx.x; q < nb * nc * LP; q += blockDim.x) {
      const int s = q % LP, k = (q / LP) % nc, bi = q / (LP * nc);
      const int i = layer_of_slot(s);
      R vke = R(0), vks = R(0), vka = R(0), vph = R(0), vfw = R(0);
      if (i < L && i >= ict) {
        const size_t qc = (size_t)col + (size_t)ndp * (size_t)(i - ict);
        R re = load_in<R>(p.condensed_dim_char + qc + (size_t)ndp * ndc * k);
        if (load_in<R>(p.w_cloud + qc) > R(0) && re > R(0)) {
          const size_t po = ((size_t)p.comp_parm_index[k] * p.n_band + (bstart + bi)) * kCloudParm;
          R qm = load_in<R>(p.condensed_mix_ratio + qc + (size_t)ndp * ndc * k);
          R cp[kCloudParm];
          if constexpr (kFP64) {
            const double *c = (p.comp_phase[k] == SOCGPU_IP_PHASE_WATER ? p.drop_parm : p.ice_parm) + po;
            for (int m = 0; m < kCloudParm; ++m) cp[m] = c[m];
          } else {
            const float *c = (p.comp_phase[k] == SOCGPU_IP_PHASE_WATER ? p.drop_parm_f : p.ice_parm_f) + po;
            for (int m = 0; m < kCloudParm; ++m) cp[m] = c[m];
          }
          const int scheme = p.comp_scheme[k];
          R kext, coalb, g;
          if (scheme == SOCGPU_IP_SLINGO_SCHRECKER) {
            // the droplet and ice forms are the same (both schemes are 1)
            kext = qm * (cp[0] + cp[1] / re);
            coalb = cp[2] + cp[3] * re;
            g = cp[4] + cp[5] * re;
          } else if (scheme == SOCGPU_IP_ICE_FU_PHF && p.comp_phase[k] == SOCGPU_IP_PHASE_ICE) {
            R x = cp[3] / re;
            kext = qm * ((cp[2] * x + cp[1]) * x + cp[0]);
            x = re / cp[8];
            coalb = cp[4] + x * (cp[5] + x * (cp[6] + x * cp[7]));
            x = re / cp[13];
            g = cp[9] + x * (cp[10] + x * (cp[11] + x * cp[12]));
          } else {
            kext = qm * (cp[0] + re * (cp[1] + re * cp[2])) / (R(1) + re * (cp[3] + re * (cp[4] + re * cp[5])));
            coalb = (cp[6] + re * (cp[7] + re * cp[8])) / (R(1) + re * (cp[9] + re * cp[10]));
            g = (cp[11] + re * (cp[12] + re * cp[13])) / (R(1) + re * (cp[14] + re * cp[15]));
          }
          const R kscat = kext * (R(1) - coalb);
          vke = kext; vks = kscat; vka = kext * coalb; vph = kscat * g; vfw = kscat * g * g;
        }
      }
      S.c_ke[q] = vke; S.c_ks[q] = vks; S.c_ka[q] = vka; S.c_phf[q] = vph; S.c_fwd[q] = vfw;
    }
  }

  // The column's cloud fractions and subcolumn scalings.
  __device__ static void stage_cloud_column(const FluxParams &p, const Smem &S, int col) {
    const int L = p.n_layer, ndp = p.nd_profile, ndl = p.nd_layer, ict = p.id_ct;
    const int ndc = ndl - ict;
    for (int s = threadIdx.x; s < LP; s += blockDim.x) {
      const int i = layer_of_slot(s);
      R w = R(0), f[4] = {R(0), R(0), R(0), R(0)};
      if (i < L && i >= ict) {
        size_t qc = (size_t)col + (size_t)ndp * (size_t)(i - ict);
        w = load_in<R>(p.w_cloud + qc);
        for (int t = 0; t < p.n_cloud_type && t < 4; ++t) f[t] = load_in<R>(p.frac_cloud + qc + (size_t)ndp * ndc * t);
      }
      S.wcld[s] = w;
      const int nt = p.n_cloud_type > 2 ? p.n_cloud_type : 2;
      for (int t = 0; t < nt && t < 4; ++t) S.frac[(size_t)t * LP + s] = f[t];
    }
    for (int q = threadIdx.x; q < p.n_subcol_gen * LP; q += blockDim.x) {
      const int s = q % LP, sub = q / LP;
      const int i = layer_of_slot(s);
      R v = R(0);
      if (i < L && i >= ict) v = load_in<R>(p.c_sub + (size_t)col + (size_t)ndp * ((size_t)(i - ict) + (size_t)ndc * sub));
      S.csub[q] = v;
    }
  }

  // Per-g-point gas data held in registers for the layer loop.
  struct GasTerm {
    int n_abs;
    bool any_term;          // some absorber scaled per term (ip_scale_term)
    R k[kMaxAbsPerBand];
  };

  __device__ static __forceinline__ GasTerm load_gas(const GPoint &gp, const BandInfo &bd, int max_abs) {
    GasTerm t;
    t.n_abs = min(gp.n_abs, max_abs);
    t.any_term = false;
#pragma unroll
    for (int j = 0; j < kMaxAbsPerBand; ++j) {
      if (j < t.n_abs) {
        if constexpr (kFP64) t.k[j] = gp.k[j];
        else t.k[j] = gp.kf[j];
        t.any_term |= (bd.gas[j].i_scale_k == SOCGPU_IP_SCALE_TERM);
      } else {
        t.k[j] = R(0);
      }
    }
    return t;
  }

  // Gas absorption of a g-point at slot s (gas_optical_properties.F90:80-95)
  // when no absorber of the band is scaled per term.
  __device__ static __forceinline__ R gas_k(const GasTerm &gt, const R *amt, int s) {
    // one absorber (the common case) without the guarded loop
    if (gt.n_abs == 1) return gt.k[0] * amt[s];
    R kg = R(0);
#pragma unroll
    for (int j = 0; j < kMaxAbsPerBand; ++j)
      if (j < gt.n_abs) {
        R kal = gt.k[j] * amt[(size_t)j * LP + s];
        kg = (j == 0) ? kal : kg + kal;
      }
    return kg;
  }

  // Gas absorption of a g-point in the lane's layers when an absorber is
  // scaled per term (power laws per term, Wen-Yi or lookup tables), written
  // to the group's scratch row.  The layer loop stays rolled so that the
  // table code appears once, without calls.
  __device__ static __forceinline__ void gas_k_terms(const FluxParams &p, const Smem &S, const GPoint &gp,
                                                     const BandInfo &bd, int n_abs, const R *amt, int r, int L,
                                                     R *scr) {
    const Lk lk = lk_of(S);
#pragma unroll 1
    for (int jj = 0; jj < CH; ++jj) {
      const int i = r * CH + jj, s = jj * P + r;
      R kg = R(0);
      if (i < L) {
        for (int j = 0; j < n_abs; ++j) {
          const R kj = kFP64 ? (R)gp.k[j] : (R)gp.kf[j];
          const R *sc;
          if constexpr (kFP64) sc = gp.term_scale[j]; else sc = gp.term_scale_f[j];
          const R kal = term_k(p, lk, bd.gas[j], gp.band, kj, sc, gp.lk_off[j], gp.iex[j], amt[(size_t)j * LP + s],
                               s, S.p[s], S.t[s]);
          kg = (j == 0) ? kal : kg + kal;
        }
      }
      scr[s] = kg;
    }
  }

  // The gas absorption of a g-point in the lane's layers.
  __device__ static __forceinline__ void gas_k_lane(const FluxParams &p, const Smem &S, const GasTerm &gt,
                                                    const GPoint &gp, const BandInfo &bd, const R *amt, int r, int L,
                                                    R (&kgv)[CH]) {
    if (p.l_gas && gt.any_term) {
      R *scr = S.kscr + (size_t)(threadIdx.x / P) * LP;
      gas_k_terms(p, S, gp, bd, gt.n_abs, amt, r, L, scr);
#pragma unroll
      for (int jj = 0; jj < CH; ++jj) kgv[jj] = scr[jj * P + r];
    } else {
#pragma unroll
      for (int jj = 0; jj < CH; ++jj) {
        const int i = r * CH + jj, s = jj * P + r;
        kgv[jj] = (i < L && p.l_gas) ? gas_k(gt, amt, s) : R(0);
      }
    }
  }

  // k of one k-term of one absorber in the lane's layers, into registers
  // through the group's scratch row (as gas_k_terms).
  __device__ static __forceinline__ void term_k_lane(const FluxParams &p, const Smem &S, const BandGas &gs, int b,
                                                     R kj, const R *sc, int lk_off, int iex, const R *amt, int r,
                                                     int L, R (&kk)[CH]) {
    R *scr = S.kscr + (size_t)(threadIdx.x / P) * LP;
    const Lk lk = lk_of(S);
#pragma unroll 1
    for (int jj = 0; jj < CH; ++jj) {
      const int i = r * CH + jj, s = jj * P + r;
      scr[s] = (i < L) ? term_k(p, lk, gs, b, kj, sc, lk_off, iex, amt[s], s, S.p[s], S.t[s]) : R(0);
    }
#pragma unroll
    for (int jj = 0; jj < CH; ++jj) kk[jj] = scr[jj * P + r];
  }

  // ---------------- equivalent extinction (k_eqv_scl) ------------------------
  // Minor absorber j of staged band bi, solved by one group of P lanes
  // (solve_band_k_eqv_scl.F90:560-1040, two-stream, plane parallel).  Its
  // k-terms are weighted by the fluxes they leave: the direct flux reaching
  // the surface (solar), or the fluxes incident on each layer from a
  // scattering-free solve with diffusivity 1.66 (monochromatic_gas_flux.F90,
  // infra-red).  The absorber's share of k_eqv replaces its staged amount;
  // under the solar source its direct-beam factor goes to aux.  gm is the
  // group's lane mask: groups of one warp may run different absorbers.
  __device__ static __forceinline__ void minor_gas(const FluxParams &p, const Smem &S, int bi, int b, int j, R sec0,
                                                int r, unsigned gm) {
    constexpr bool lw = (SRC == SOCGPU_IP_INFRA_RED);
    const int L = p.n_layer, max_abs = p.max_abs;
    const BandInfo &bd = p.bands[b];
    const BandGas &gs = bd.gas[j];
    R *amt = S.amt + ((size_t)bi * max_abs + j) * LP;
    const int t0 = bd.minor_first[j], nt = bd.minor_count[j];
    // infra-red: sfl, the flux weights; solar: fg, the direct flux of the
    // absorber alone at each layer's bottom, and (FP32, in the absorber's
    // aux row) the flux it loses in each layer, summed without cancellation
    R skf[CH], sfl[CH], kmin[CH], fg[CH];
    R sfs = R(0);
    R *loss = S.aux + ((size_t)bi * max_abs + j) * LP;
#pragma unroll
    for (int jj = 0; jj < CH; ++jj) {
      skf[jj] = R(0); sfl[jj] = R(0); fg[jj] = R(0); kmin[jj] = R(3.0e38);
      if constexpr (!lw && !kFP64) loss[jj * P + r] = R(0);
    }
    if (lw && nt == 1 && p.l_grey_single) {
      // a single-term minor absorber as a grey absorber (l_grey_single)
      const TermK &tk = p.minor_terms[t0];
      const R *sc;
      if constexpr (kFP64) sc = tk.scale; else sc = tk.scale_f;
      R kk[CH];
      term_k_lane(p, S, gs, b, kFP64 ? (R)tk.k : (R)tk.kf, sc, tk.lk_off, tk.iex, amt, r, L, kk);
#pragma unroll
      for (int jj = 0; jj < CH; ++jj) {
        const int i = r * CH + jj, s = jj * P + r;
        if (i < L) amt[s] = kk[jj];
      }
      return;
    }
    const R *bs = S.bscal + bi * kBandScal;
    const R *dB_b = S.dB + (size_t)bi * LP;
    for (int t = 0; t < nt; ++t) {
      const TermK &tk = p.minor_terms[t0 + t];
      const R kj = kFP64 ? (R)tk.k : (R)tk.kf, we = kFP64 ? (R)tk.w : (R)tk.wf;
      const R *sc;
      if constexpr (kFP64) sc = tk.scale; else sc = tk.scale_f;
      R kk[CH];
      term_k_lane(p, S, gs, b, kj, sc, tk.lk_off, tk.iex, amt, r, L, kk);
#pragma unroll
      for (int jj = 0; jj < CH; ++jj)
        if (r * CH + jj < L) kmin[jj] = kk[jj] < kmin[jj] ? kk[jj] : kmin[jj];
      if constexpr (!lw) {
        // direct beam of this term alone: an exclusive product scan
        R e[CH], prod = R(1);
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) {
          const int i = r * CH + jj, s = jj * P + r;
          if (i < L) {
            if constexpr (kFP64) e[jj] = exp(-kk[jj] * S.mass[s] * sec0);
            else e[jj] = expf(-kk[jj] * S.mass[s] * sec0);
          } else {
            e[jj] = R(1);
          }
          prod *= e[jj];
        }
        R incl = prod;
#pragma unroll
        for (int d = 1; d < P; d <<= 1) {
          const R y = __shfl_up_sync(gm, incl, d, P);
          if (r >= d) incl = y * incl;
        }
        R f = __shfl_up_sync(gm, incl, 1, P);
        if (r == 0) f = R(1);
        f = we * f;
        const R f_surf = we * __shfl_sync(gm, incl, P - 1, P);
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) {
          if constexpr (!kFP64) {
            const int s = jj * P + r;
            if (r * CH + jj < L) loss[s] += f * -expm1f(-kk[jj] * S.mass[s] * sec0);
          }
          f = f * e[jj];
          fg[jj] += f;
          skf[jj] += kk[jj] * f_surf;
        }
        sfs += f_surf;
      } else {
        // monochromatic_gas_flux.F90:100-197: downward then upward affine scans
        R T[CH], su[CH];
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) {
          const int i = r * CH + jj, s = jj * P + r;
          if (i < L) {
            R c1;
            if constexpr (kFP64) { Coef c = fast_lw_ref(0, kk[jj] * S.mass[s]); T[jj] = c.T; c1 = c.c1; }
            else { CoefF c = fast_lw_mix(0, kk[jj] * S.mass[s]); T[jj] = c.T; c1 = c.c1; }
            su[jj] = c1 * dB_b[s];
          } else {
            T[jj] = R(1); su[jj] = R(0);
          }
        }
        R A = R(1), B = R(0);
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) { A = T[jj] * A; B = T[jj] * B - su[jj]; }
        R iA = A, iB = B;
#pragma unroll
        for (int d = 1; d < P; d <<= 1) {
          const R yA = __shfl_up_sync(gm, iA, d, P), yB = __shfl_up_sync(gm, iB, d, P);
          if (r >= d) { iB = iA * yB + iB; iA = iA * yA; }
        }
        R eA = __shfl_up_sync(gm, iA, 1, P), eB = __shfl_up_sync(gm, iB, 1, P);
        if (r == 0) { eA = R(1); eB = R(0); }
        const R f_top = bs[0];
        const R fdn_top = eA * f_top + eB;
        const R fdn_surf = __shfl_sync(gm, iA, P - 1, P) * f_top + __shfl_sync(gm, iB, P - 1, P);
        const R fup_surf = bs[4] + bs[2] * fdn_surf;
        R C = R(1), E = R(0);
#pragma unroll
        for (int jj = CH - 1; jj >= 0; --jj) { C = T[jj] * C; E = su[jj] + T[jj] * E; }
        R sC = C, sE = E;
#pragma unroll
        for (int d = 1; d < P; d <<= 1) {
          const R yC = __shfl_down_sync(gm, sC, d, P), yE = __shfl_down_sync(gm, sE, d, P);
          if (r + d < P) { sE = sC * yE + sE; sC = sC * yC; }
        }
        R xC = __shfl_down_sync(gm, sC, 1, P), xE = __shfl_down_sync(gm, sE, 1, P);
        if (r == P - 1) { xC = R(1); xE = R(0); }
        R fu = xC * fup_surf + xE;         // F_up at the bottom of this lane's chunk
        R fub[CH];
#pragma unroll
        for (int jj = CH - 1; jj >= 0; --jj) { fub[jj] = fu; fu = su[jj] + T[jj] * fu; }
        R fd = fdn_top;
#pragma unroll
        for (int jj = 0; jj < CH; ++jj) {
          const R a = fabs(fd) + fabs(fub[jj]);
          skf[jj] += kk[jj] * we * a;
          sfl[jj] += we * a;
          fd = T[jj] * fd - su[jj];
        }
      }
    }
    // this absorber's share of k_eqv (and its direct-beam factor)
    R fg_above = __shfl_up_sync(gm, fg[CH - 1], 1, P);
    if (r == 0) fg_above = R(1);
#pragma unroll
    for (int jj = 0; jj < CH; ++jj) {
      const int i = r * CH + jj, s = jj * P + r;
      if (i < L) {
        if constexpr (!lw) {
          amt[s] = sfs > R(0) ? skf[jj] / sfs : kmin[jj];
          // FP64: the ratio of the absorber's direct flux across the layer;
          // FP32: its logarithm log1p(-loss / flux above), so that the factor
          // can be formed as f - 1 without cancellation
          R v;
          if constexpr (kFP64) v = fg_above > R(0) ? fg[jj] / fg_above : R(1);
          else v = fg_above > R(0) ? log1pf(-fminf(loss[s] / fg_above, 1.0f)) : R(0);
          loss[s] = v;
        } else {
          amt[s] = sfl[jj] > R(0) ? skf[jj] / sfl[jj] : kmin[jj];
        }
      }
      fg_above = fg[jj];
    }
  }

  // The minor absorbers of the staged bands, one (band, absorber) per group.
  __device__ static void stage_keqv(const FluxParams &p, const Smem &S, int bstart, int nb, R sec0) {
    const int n_groups = blockDim.x / P, gid = threadIdx.x / P, r = threadIdx.x % P;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned gm = (P == 32) ? 0xffffffffu : (((1u << P) - 1u) << (lane & ~(unsigned)(P - 1)));
    int item = 0;
    for (int bi = 0; bi < nb; ++bi) {
      const int na = p.l_gas ? min(p.bands[bstart + bi].n_abs, p.max_abs) : 0;
      for (int j = 1; j < na; ++j, ++item)
        if (item % n_groups == gid) minor_gas(p, S, bi, bstart + bi, j, sec0, r, gm);
    }
  }

  // k_eqv of every slot into the grey absorption, and the solar direct-beam
  // factor adjust_solar_ke (solve_band_k_eqv_scl.F90:975-1040), summed over
  // the minor absorbers in their order.
  __device__ static void fold_keqv(const FluxParams &p, const Smem &S, int bstart, int nb, R sec0) {
    constexpr bool lw = (SRC == SOCGPU_IP_INFRA_RED);
    const int L = p.n_layer, max_abs = p.max_abs;
    for (int q = threadIdx.x; q < nb * LP; q += blockDim.x) {
      const int bi = q / LP, s = q - bi * LP;
      if (layer_of_slot(s) >= L) continue;
      const int na = p.l_gas ? min(p.bands[bstart + bi].n_abs, max_abs) : 0;
      // FP64: adj is the product of the absorbers' ratios; FP32: the sum of
      // their logarithms
      R keq = R(0), adj = kFP64 ? R(1) : R(0);
      for (int j = 1; j < na; ++j) {
        keq += S.amt[((size_t)bi * max_abs + j) * LP + s];
        if (!lw) {
          if constexpr (kFP64) adj *= S.aux[((size_t)bi * max_abs + j) * LP + s];
          else adj += S.aux[((size_t)bi * max_abs + j) * LP + s];
        }
      }
      S.kgt[q] += keq;
      S.kabs[q] += keq;
      if constexpr (!lw) {
        const R tmax = R(36.04365338911715);   // ln(1 / epsilon) of FP64
        const R x = keq * S.mass[s] * sec0;
        // FP64: the factor f itself; FP32: f - 1
        if constexpr (kFP64) S.aux[(size_t)bi * max_abs * LP + s] = adj * exp(x < tmax ? x : tmax);
        else S.aux[(size_t)bi * max_abs * LP + s] = expm1f(adj + (x < tmax ? x : tmax));
      }
    }
  }

  // The direct-beam factor folded into the layer coefficients
  // (solar_source.F90:115-130 with l_scale_solar): T0' = T0 f and
  // c2' = c2 + T0 (f - 1).  The staged value is f in FP64 and f - 1 in FP32.
  __device__ static __forceinline__ void fold_direct(const Smem &S, int bi, int max_abs, int r, int L,
                                                     R (&T0)[CH], R (&c2)[CH]) {
    const R *a = S.aux + (size_t)bi * max_abs * LP;
#pragma unroll
    for (int jj = 0; jj < CH; ++jj) {
      const int i = r * CH + jj, s = jj * P + r;
      if (i < L) {
        const R fm1 = kFP64 ? a[s] - R(1) : a[s];
        c2[jj] = c2[jj] + T0[jj] * fm1;
        T0[jj] = kFP64 ? T0[jj] * a[s] : T0[jj] + T0[jj] * fm1;
      }
    }
  }

  // The direct transmission of a cell before delta-rescaling, exp(-tau sec0)
  // (two_coeff.F90 trans_0_dir for ip_direct_noscaling).
  __device__ static __forceinline__ R t0_unscaled(R kgt, R kg, R dm, R sec0) {
    if constexpr (kFP64) return exp(-(kgt + kg) * dm * sec0);
    else return expf(-(kgt + kg) * dm * sec0);
  }
  // adjust_solar_ke on a row of unscaled transmissions (k_eqv_scl, solar)
  __device__ static __forceinline__ void fold_direct_row(const Smem &S, int bi, int max_abs, int r, int L, R *row) {
    const R *a = S.aux + (size_t)bi * max_abs * LP;
#pragma unroll
    for (int jj = 0; jj < CH; ++jj) {
      const int i = r * CH + jj, s = jj * P + r;
      if (i < L) row[s] = row[s] * (kFP64 ? a[s] : R(1) + a[s]);
    }
  }

  // One g-point of one column (all its subcolumns under McICA).
  __device__ static void solve_gpoint(const FluxParams &p, const Smem &S, int col, int g, int bstart, int max_abs,
                                      R sec0, int r, Acc *acc, bool lw, bool active) {
    const int L = p.n_layer;
    const GPoint &gp = p.gpoints[g];
    const int b = gp.band, bi = b - bstart;
    const BandInfo &bd = p.bands[b];
    const R *bs = S.bscal + bi * kBandScal;
    const R w_g = kFP64 ? (R)(bs[5] * gp.weight) : (R)(bs[5] * gp.weight_f);
    const GasTerm gt = load_gas(gp, bd, max_abs);
    const R *kgt_b = S.kgt + (size_t)bi * LP, *kes_b = S.kes + (size_t)bi * LP;
    const R *kabs_b = S.kabs + (size_t)bi * LP, *asym_b = S.asym + (size_t)bi * LP;
    const R *fwd_b = S.fwd + (size_t)bi * LP, *amt_b = S.amt + (size_t)bi * max_abs * LP;
    const R *dB_b = S.dB + (size_t)bi * LP, *dB2_b = S.dB2 + (size_t)bi * LP;
    const R f_inc_down = bs[0], f_inc_dir = bs[1], alb_diff = bs[2], alb_dir = bs[3], dB_surf = bs[4];

    // the unscaled direct transmissions (i_direct_tau = ip_direct_noscaling)
    R *t0d = (!lw && p.i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING && !p.region)
                 ? S.t0d + (size_t)(threadIdx.x / P) * LP : nullptr;
    if (!MCICA) {
      // the gas absorption of the lane's layers first, while few registers
      // are live, then the coefficients
      R kgv[CH];
      gas_k_lane(p, S, gt, gp, bd, amt_b, r, L, kgv);
      R T[CH], Rf[CH], T0[CH], c1[CH], c2[CH], om[CH];
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j, s = j * P + r;
        if (i < L) {
          cell_coef(p, kgt_b[s], kes_b[s], kabs_b[s], kgv[j], S.mass[s], asym_b[s], fwd_b[s], sec0,
                    T[j], Rf[j], T0[j], c1[j], c2[j], om[j]);
        } else {
          T[j] = R(1); Rf[j] = R(0); T0[j] = R(1); c1[j] = R(0); c2[j] = R(0); om[j] = R(0);
        }
      }
      if (t0d) {
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          const int i = r * CH + j, s = j * P + r;
          t0d[s] = i < L ? t0_unscaled(kgt_b[s], kgv[j], S.mass[s], sec0) : R(1);
        }
      }
      if constexpr (SRC == SOCGPU_IP_SOLAR)
        if (p.keqv) {
          fold_direct(S, bi, max_abs, r, L, T0, c2);
          if (t0d) fold_direct_row(S, bi, max_abs, r, L, t0d);
        }
      solve_column(p, T, Rf, T0, c1, c2, om, r, L, lw, dB_b, dB2_b, f_inc_down, f_inc_dir,
                   alb_diff, alb_dir, dB_surf, w_g, acc, active, t0d);
    } else if (p.region) {
      solve_region(p, g, bstart, sec0, r, lw, active);
    } else {
      solve_mcica(p, S, col, gp, gt, bd, bi, b, r, L, lw, sec0, dB_b, dB2_b, f_inc_down, f_inc_dir,
                  alb_diff, alb_dir, dB_surf, w_g, acc, max_abs, active);
    }
  }

  // the correlation of like region k (0 clear, 1 stratiform, 2 convective)
  // at interface i (overlap_coupled.F90:190-236): 1 under mix_max and triple,
  // 0 under mix_random, and under part_corr and part_corr_cnv
  // exp((p(i) - p(i+1)) / dp_corr) between layers 1 < i < n_layer (1 at the
  // ends), in FP64
  __device__ static R like_corr(const FluxParams &p, int col, int i, int k) {
    if (p.corr_mode != 2) return p.corr_mode == 1 ? R(1) : R(0);
    if (!(i < p.n_layer && i > 1)) return R(1);
    const size_t q = (size_t)col + (size_t)p.nd_profile * (size_t)(i - 1);
    return (R)exp((p.p[q] - p.p[q + (size_t)p.nd_profile]) / p.dp_corr[k]);
  }

  // set_cloud_geometry and overlap_coupled (set_cloud_geometry.F90:76-96,
  // overlap_coupled.F90:120-440) for the column, by one thread: the first
  // cloudy layer (1-based, at most n_layer) and, at each interface i (0: the
  // top), the fractions of each upper region (clear, cloudy) over each lower
  // one (ovl rows 2 j + k) and of each lower region under each upper one
  // (rows 4 + 2 j + k).  The interfaces above the cloud top keep the identity.
  __device__ static void stage_regions(const FluxParams &p, const Smem &S, int col, int LP_) {
    if (threadIdx.x != 0) return;
    const int L = p.n_layer, ndp = p.nd_profile, ict = p.id_ct;
    auto wc = [&](int i1) -> R {
      return (i1 - 1 >= ict) ? load_in<R>(p.w_cloud + (size_t)col + (size_t)ndp * (size_t)(i1 - 1 - ict)) : R(0);
    };
    int nct = ict + 1;
    while (nct < L && !(wc(nct) > R(0))) ++nct;
    S.nct[0] = nct;
    const R tol = (R)(1.0e+02 * kEps64);
    for (int i = 0; i < nct - 1; ++i)
      for (int m = 0; m < 8; ++m) S.ovl[(size_t)m * (LP_ + 1) + i] = (m == 0 || m == 3 || m == 4 || m == 7) ? R(1) : R(0);
    R au0 = R(1), au1 = R(0);
    for (int i = nct - 1; i <= L; ++i) {
      R al0, al1;
      if (i < L) { const R w = wc(i + 1); al0 = R(1) - w; al1 = w; }
      else { al0 = R(1); al1 = R(0); }
      R a00 = like_corr(p, col, i, 0) * (al0 < au0 ? al0 : au0), a11 = like_corr(p, col, i, 1) * (al1 < au1 ? al1 : au1);
      R a01 = R(0), a10 = R(0);
      R art = R(1) - a00;
      art = art - a11;
      const R ru0 = au0 - a00, ru1 = au1 - a11, rl0 = al0 - a00, rl1 = al1 - a11;
      if (art > tol) {
        a00 = a00 + ru0 * rl0 / art; a01 = a01 + ru0 * rl1 / art;
        a10 = a10 + ru1 * rl0 / art; a11 = a11 + ru1 * rl1 / art;
      }
      R v[8] = {R(1), R(0), R(0), R(1), R(1), R(0), R(0), R(1)};
      if (au0 > tol) { v[0] = a00 / au0; v[2] = a01 / au0; }
      if (au1 > tol) { v[1] = a10 / au1; v[3] = a11 / au1; }
      if (al0 > tol) { v[4] = a00 / al0; v[6] = a10 / al0; }
      if (al1 > tol) { v[5] = a01 / al1; v[7] = a11 / al1; }
      for (int m = 0; m < 8; ++m) S.ovl[(size_t)m * (LP_ + 1) + i] = v[m];
      if (i < L) { au0 = al0; au1 = al1; }
    }
  }

  // set_cloud_geometry, aggregate_cloud and overlap_coupled for three
  // regions, clear (0), stratiform (1) and convective (2), with like regions
  // maximally overlapped (aggregate_cloud.F90:107-155, overlap_coupled.F90:
  // 150-450), by one thread: the cloud top, each layer's stratiform and
  // convective shares of its cloud (frr rows), and at each interface i the
  // fraction v_jk of upper region k going into lower region j (ovl row
  // 3 j + k) and the fraction u_jk of lower region k going into upper region
  // j (row 9 + 3 j + k).  The interfaces above the cloud top keep the
  // identity.
  __device__ static void stage_regions3(const FluxParams &p, const Smem &S, int col, int LP_) {
    if (threadIdx.x != 0) return;
    const int L = p.n_layer, ndp = p.nd_profile, ict = p.id_ct, ndc = p.nd_layer - ict;
    auto wc = [&](int i1) -> R {
      return (i1 - 1 >= ict) ? load_in<R>(p.w_cloud + (size_t)col + (size_t)ndp * (size_t)(i1 - 1 - ict)) : R(0);
    };
    int nct = ict + 1;
    while (nct < L && !(wc(nct) > R(0))) ++nct;
    S.nct[0] = nct;
    for (int i = 0; i < L; ++i) {
      R f2 = R(0), f3 = R(0);
      if (i >= ict)
        for (int t = 0; t < p.n_cloud_type; ++t) {
          const R fc = load_in<R>(p.frac_cloud + (size_t)col + (size_t)ndp * ((size_t)(i - ict) + (size_t)ndc * t));
          if (p.type_region[t] == 2) f2 = f2 + fc; else f3 = f3 + fc;
        }
      S.frr[i] = f2; S.frr[LP_ + i] = f3;
    }
    const R tol = (R)(1.0e+02 * kEps64);
    for (int i = 0; i < nct - 1; ++i)
      for (int m = 0; m < 18; ++m) S.ovl[(size_t)m * (LP_ + 1) + i] = (m == 0 || m == 4 || m == 8 || m == 9 || m == 13 || m == 17) ? R(1) : R(0);
    R au[3] = {R(1), R(0), R(0)};
    for (int i = nct - 1; i <= L; ++i) {
      R al[3], ao[3][3];
      if (i < L) { const R w = wc(i + 1); al[0] = R(1) - w; al[1] = w * S.frr[i]; al[2] = w * S.frr[LP_ + i]; }
      else { al[0] = R(1); al[1] = R(0); al[2] = R(0); }
      for (int k = 0; k < 3; ++k) ao[k][k] = like_corr(p, col, i, k) * (al[k] < au[k] ? al[k] : au[k]);
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < k; ++j) { ao[k][j] = R(0); ao[j][k] = R(0); }
      R art = R(1) - ao[0][0];
      for (int k = 1; k < 3; ++k) art = art - ao[k][k];
      R aru[3], arl[3];
      for (int k = 0; k < 3; ++k) { aru[k] = au[k] - ao[k][k]; arl[k] = al[k] - ao[k][k]; }
      if (art > tol)
        for (int k = 0; k < 3; ++k)
          for (int j = 0; j < 3; ++j) ao[k][j] = ao[k][j] + aru[k] * arl[j] / art;
      R v[18];
      for (int m = 0; m < 18; ++m) v[m] = R(0);
      for (int k = 0; k < 3; ++k) { v[3 * k + k] = R(1); v[9 + 3 * k + k] = R(1); }
      for (int k = 0; k < 3; ++k)
        if (au[k] > tol)
          for (int j = 0; j < 3; ++j) v[3 * j + k] = ao[k][j] / au[k];
      for (int k = 0; k < 3; ++k)
        if (al[k] > tol)
          for (int j = 0; j < 3; ++j) v[9 + 3 * j + k] = ao[j][k] / al[k];
      for (int m = 0; m < 18; ++m) S.ovl[(size_t)m * (LP_ + 1) + i] = v[m];
      if (i < L) { au[0] = al[0]; au[1] = al[1]; au[2] = al[2]; }
    }
  }

  // One g-point of a column in a clear and a cloudy region (mix_column.F90:
  // 150-460).  The lanes of the group compute the clear coefficients and the
  // frac_cloud-weighted coefficients of the cloud types (two_coeff_cloud.F90)
  // of their layers, and the infra-red sources; lane 0 then runs the serial
  // parts from the group's scratch rows: the direct beam through both regions
  // (mixed_solar_source.F90), solver_mix_direct.F90 or
  // solver_mix_direct_hogan.F90 and the back-substitution; the lanes add the
  // level fluxes to the group's accumulators.
  // Called out of line with scalars only, so that the McICA kernels it
  // shares keep their registers: the shared-memory view, the g-point and
  // the group's accumulators are rebuilt here as the column loop builds them.
  __device__ static __noinline__ void solve_region(const FluxParams &p, int g, int bstart, R sec0, int r, bool lw,
                                                   bool active) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int n_groups = blockDim.x / P, L = p.n_layer, max_abs = p.max_abs;
    const SmemLayout lay = make_layout<R>(p, LP, P, p.band_batch, n_groups, MCICA);
    const Smem S = bind(smem, lay);
    const GPoint &gp = p.gpoints[g];
    const int b = gp.band, bi = b - bstart;
    const BandInfo &bd = p.bands[b];
    const GasTerm gt = load_gas(gp, bd, max_abs);
    const R *bs = S.bscal + bi * kBandScal;
    const R w_g = kFP64 ? (R)(bs[5] * gp.weight) : (R)(bs[5] * gp.weight_f);
    const R f_inc_down = bs[0], f_inc_dir = bs[1], alb_diff = bs[2], alb_dir = bs[3], dB_surf = bs[4];
    const R *dB_b = S.dB + (size_t)bi * LP, *dB2_b = S.dB2 + (size_t)bi * LP;
    const int nc = p.n_condensed;
    const int gid = threadIdx.x / P;
    Acc *acc = S.acc + (size_t)gid * lay.acc_stride;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned gm = (P == 32) ? 0xffffffffu : (((1u << P) - 1u) << (lane & ~(unsigned)(P - 1)));
    const R *kgt_b = S.kgt + (size_t)bi * LP, *kes_b = S.kes + (size_t)bi * LP;
    const R *kabs_b = S.kabs + (size_t)bi * LP, *asym_b = S.asym + (size_t)bi * LP;
    const R *fwd_b = S.fwd + (size_t)bi * LP, *amt_b = S.amt + (size_t)bi * max_abs * LP;
    const R *phf_nc = S.phf_nc + (size_t)bi * LP, *fwd_nc = S.fwd_nc + (size_t)bi * LP;
    const R *c_ke = S.c_ke + (size_t)bi * nc * LP, *c_ks = S.c_ks + (size_t)bi * nc * LP;
    const R *c_ka = S.c_ka + (size_t)bi * nc * LP, *c_ph = S.c_phf + (size_t)bi * nc * LP;
    const R *c_fw = S.c_fwd + (size_t)bi * nc * LP;
    R *X = S.reg + (size_t)gid * lay.reg_rows * (LP + 1);
    auto row = [&](int k) { return X + (size_t)k * (LP + 1); };
    const int nct = S.nct[0];
    const bool triple = p.triple;

    R kgv[CH];
    gas_k_lane(p, S, gt, gp, bd, amt_b, r, L, kgv);
    R Tf[CH], Rff[CH], T0f[CH], c1f[CH], c2f[CH], omf[CH];
    R Tc[CH], Rc[CH], T0c[CH], c1c[CH], c2c[CH], omc[CH];
    // three regions: the convective region's coefficients are summed in its
    // rows of the group's scratch (the stratiform region uses Tc..), so the
    // McICA kernels this function shares keep their registers
    R *VT = row(kRgVT), *VR = row(kRgVR), *VT0 = row(kRgVT0), *VC1 = row(kRgVC1), *VC2 = row(kRgVC2);
    R *VOM = row(kRgVOM);
    // the direct beam without delta-scaling (two_coeff.F90 trans_0_dir):
    // exp(-tau sec0) of the optical depth before rescaling, per region
    const bool dir_unscaled = !lw && p.i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING;
    auto t0_unscaled = [&](R kgt, R kg, R dm) -> R {
      if constexpr (kFP64) return exp(-(kgt + kg) * dm * sec0);
      else return expf(-(kgt + kg) * dm * sec0);
    };
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int i = r * CH + j, s = j * P + r;
      Tc[j] = R(0); Rc[j] = R(0); T0c[j] = R(0); c1c[j] = R(0); c2c[j] = R(0); omc[j] = R(0);
      if (triple && i < L) { VT[i] = R(0); VR[i] = R(0); VT0[i] = R(0); VC1[i] = R(0); VC2[i] = R(0); VOM[i] = R(0); }
      if (i < L && dir_unscaled) {
        row(kRgFT0D)[i] = t0_unscaled(kgt_b[s], kgv[j], S.mass[s]); row(kRgCT0D)[i] = R(0);
        if (triple) row(kRgVT0D)[i] = R(0);
      }
      if (i < L) {
        cell_coef(p, kgt_b[s], kes_b[s], kabs_b[s], kgv[j], S.mass[s], asym_b[s], fwd_b[s], sec0,
                  Tf[j], Rff[j], T0f[j], c1f[j], c2f[j], omf[j]);
        if (S.wcld[s] > R(0)) {
          for (int t = 0; t < p.n_cloud_type; ++t) {
            const R fc = S.frac[(size_t)t * LP + s];
            if (!(fc > R(0))) continue;
            // the type's optical properties (grey_opt_prop.F90:980-1000,
            // 1195-1240, 1475-1500; rescale_phase_fnc.F90)
            R kgt = kgt_b[s], kes = kes_b[s], kab = kabs_b[s], fw = fwd_nc[s], ph = phf_nc[s];
            for (int k = 0; k < nc; ++k) {
              if (p.comp_type[k] - 1 != t) continue;
              const size_t qk = (size_t)k * LP + s;
              kgt = kgt + c_ke[qk]; kes = kes + c_ks[qk]; kab = kab + c_ka[qk];
              fw = fw + c_fw[qk]; ph = ph + c_ph[qk];
            }
            R asym = ph, fwd = R(0);
            if (kes > (R)kTiny64) {
              const R inv = R(1) / kes;
              if (p.l_rescale) {
                fwd = fw * inv;
                asym = (ph * inv - fwd) / (R(1) - fwd);
              } else {
                asym = ph * inv;
              }
            }
            R tT, tR, tT0, t1, t2, tO;
            cell_coef(p, kgt, kes, kab, kgv[j], S.mass[s], asym, fwd, sec0, tT, tR, tT0, t1, t2, tO);
            if (triple && p.type_region[t] == 3) {
              // a convective type (aggregate_cloud.F90:107-155)
              VT[i] = VT[i] + fc * tT; VR[i] = VR[i] + fc * tR; VT0[i] = VT0[i] + fc * tT0;
              if (dir_unscaled) row(kRgVT0D)[i] = row(kRgVT0D)[i] + fc * t0_unscaled(kgt, kgv[j], S.mass[s]);
              VC1[i] = VC1[i] + fc * t1; VC2[i] = VC2[i] + fc * t2; VOM[i] = VOM[i] + fc * tO;
            } else {
              Tc[j] = Tc[j] + fc * tT; Rc[j] = Rc[j] + fc * tR; T0c[j] = T0c[j] + fc * tT0;
              if (dir_unscaled) row(kRgCT0D)[i] = row(kRgCT0D)[i] + fc * t0_unscaled(kgt, kgv[j], S.mass[s]);
              c1c[j] = c1c[j] + fc * t1; c2c[j] = c2c[j] + fc * t2; omc[j] = omc[j] + fc * tO;
            }
          }
          if (triple) {
            // each cloudy region's weighted sums over its share of the cloud
            // (two_coeff_region.F90:383-440)
            const R f2 = S.frr[i], f3 = S.frr[LP + i];
            if (f2 > (R)kTiny64) {
              const R inv = R(1) / f2;
              Tc[j] = Tc[j] * inv; Rc[j] = Rc[j] * inv; T0c[j] = T0c[j] * inv;
              c1c[j] = c1c[j] * inv; c2c[j] = c2c[j] * inv; omc[j] = omc[j] * inv;
              if (dir_unscaled) row(kRgCT0D)[i] = row(kRgCT0D)[i] * inv;
            }
            if (f3 > (R)kTiny64) {
              const R inv = R(1) / f3;
              VT[i] = VT[i] * inv; VR[i] = VR[i] * inv; VT0[i] = VT0[i] * inv;
              VC1[i] = VC1[i] * inv; VC2[i] = VC2[i] * inv; VOM[i] = VOM[i] * inv;
              if (dir_unscaled) row(kRgVT0D)[i] = row(kRgVT0D)[i] * inv;
            }
          }
        }
      } else {
        Tf[j] = R(1); Rff[j] = R(0); T0f[j] = R(1); c1f[j] = R(0); c2f[j] = R(0); omf[j] = R(0);
      }
    }
    if constexpr (SRC == SOCGPU_IP_SOLAR)
      if (p.keqv) {
        fold_direct(S, bi, max_abs, r, L, T0f, c2f);
        fold_direct(S, bi, max_abs, r, L, T0c, c2c);
        if (triple) {
          // the same correction on the convective rows (fold_direct)
          const R *a = S.aux + (size_t)bi * max_abs * LP;
#pragma unroll
          for (int j = 0; j < CH; ++j) {
            const int i = r * CH + j, s = j * P + r;
            if (i < L) {
              const R fm1 = kFP64 ? a[s] - R(1) : a[s];
              VC2[i] = VC2[i] + VT0[i] * fm1;
              VT0[i] = kFP64 ? VT0[i] * a[s] : VT0[i] + VT0[i] * fm1;
            }
          }
        }
        if (dir_unscaled) {
          // adjust_solar_ke on the unscaled beam too (mixed_solar_source.F90:130-140)
          const R *a = S.aux + (size_t)bi * max_abs * LP;
#pragma unroll
          for (int j = 0; j < CH; ++j) {
            const int i = r * CH + j, s = j * P + r;
            if (i < L) {
              const R f = kFP64 ? a[s] : R(1) + a[s];
              row(kRgFT0D)[i] = row(kRgFT0D)[i] * f;
              row(kRgCT0D)[i] = row(kRgCT0D)[i] * f;
              if (triple) row(kRgVT0D)[i] = row(kRgVT0D)[i] * f;
            }
          }
        }
      }
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int i = r * CH + j, s = j * P + r;
      if (i >= L) continue;
      if (lw) {
        // ir_source.F90:93-119 in each region, weighted by its area in the
        // cloudy layers (mix_column.F90:185-230)
        const R dB = dB_b[s];
        R su, sd, suc, sdc, suv = R(0), sdv = R(0);
        if (p.l_ir_source_quad) {
          su = c1f[j] * dB + c2f[j] * dB2_b[s]; sd = -c1f[j] * dB + c2f[j] * dB2_b[s];
          suc = c1c[j] * dB + c2c[j] * dB2_b[s]; sdc = -c1c[j] * dB + c2c[j] * dB2_b[s];
          if (triple) { suv = VC1[i] * dB + VC2[i] * dB2_b[s]; sdv = -VC1[i] * dB + VC2[i] * dB2_b[s]; }
        } else {
          su = c1f[j] * dB; sd = -su; suc = c1c[j] * dB; sdc = -suc;
          if (triple) { suv = VC1[i] * dB; sdv = -suv; }
        }
        if (i + 1 >= nct) {
          const R wc = S.wcld[s], wf = R(1) - wc;
          su = wf * su; sd = wf * sd;
          if (triple) {
            // the areas of the three regions (triple_column.F90:320-350)
            const R a2 = wc * S.frr[i], a3 = wc * S.frr[LP + i];
            suc = a2 * suc; sdc = a2 * sdc; suv = a3 * suv; sdv = a3 * sdv;
          } else {
            suc = wc * suc; sdc = wc * sdc;
          }
        }
        c1f[j] = su; c2f[j] = sd; c1c[j] = suc; c2c[j] = sdc;
        if (triple) { VC1[i] = suv; VC2[i] = sdv; }
      }
      row(kRgFT)[i] = Tf[j]; row(kRgFR)[i] = Rff[j]; row(kRgFT0)[i] = T0f[j];
      row(kRgFC1)[i] = c1f[j]; row(kRgFC2)[i] = c2f[j]; row(kRgFOM)[i] = omf[j];
      row(kRgCT)[i] = Tc[j]; row(kRgCR)[i] = Rc[j]; row(kRgCT0)[i] = T0c[j];
      row(kRgCC1)[i] = c1c[j]; row(kRgCC2)[i] = c2c[j]; row(kRgCOM)[i] = omc[j];
    }
    __syncwarp(gm);
    if (r == 0) {
      double *Y = S.regd + (size_t)gid * lay.regd_rows * (LP + 1);
      if (triple) region_serial3(p, S, X, Y, nct, L, lw, f_inc_down, f_inc_dir, alb_diff, alb_dir, dB_surf);
      else region_serial(p, S, X, Y, nct, L, lw, f_inc_down, f_inc_dir, alb_diff, alb_dir, dB_surf);
    }
    __syncwarp(gm);
    // accumulate the level fluxes and the layer divergence
    const int L_acc = active ? L : -1;
    Acc *acc_up = acc, *acc_dn = acc + (LP + 1), *acc_dir = acc + 2 * (LP + 1), *acc_div = acc + 3 * (LP + 1);
    const R *fu = row(kRgFU), *fd = row(kRgFD), *fdir = row(kRgFDIR), *dv = row(kRgDIV);
    if (r == 0 && active) {
      acc_up[LP] += w_g * fu[0]; acc_dn[LP] += w_g * fd[0];
      if (!lw) acc_dir[LP] += w_g * fdir[0];
    }
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int i = r * CH + j, s = j * P + r;
      if (i < L_acc) {
        acc_up[s] += w_g * fu[i + 1];
        acc_dn[s] += w_g * fd[i + 1];
        if (!lw) acc_dir[s] += w_g * fdir[i + 1];
        acc_div[s] += w_g * dv[i];
      }
    }
    __syncwarp(gm);
  }

  // The serial part of the two-region solve, on one lane, in FP64 in every
  // build (the FP32 coefficients of the layers are its inputs): rows as
  // solve_region leaves them; writes the level fluxes (diffuse in the
  // solar), the direct flux and the layer divergence.  Layers i are 0-based
  // here; interface i lies below layer i-1 (0: the top).
  __device__ static __noinline__ void region_serial(const FluxParams &p, const Smem &S, R *X, double *Y, int nct,
                                                    int L, bool lw, R f_inc_down_r, R f_inc_dir_r, R alb_diff_r,
                                                    R alb_dir_r, R dB_surf_r) {
    using D = double;
    auto row = [&](int k) { return X + (size_t)k * (LP + 1); };
    auto drow = [&](int k) { return Y + (size_t)k * (LP + 1); };
    auto ov = [&](int m, int i) -> D { return (D)S.ovl[(size_t)m * (LP + 1) + i]; };
    const D f_inc_down = f_inc_down_r, f_inc_dir = f_inc_dir_r, alb_diff = alb_diff_r, alb_dir = alb_dir_r;
    const D dB_surf = dB_surf_r;
    R *FT = row(kRgFT), *FR = row(kRgFR), *FT0 = row(kRgFT0), *FC1 = row(kRgFC1), *FC2 = row(kRgFC2);
    R *CT = row(kRgCT), *CR = row(kRgCR), *CT0 = row(kRgCT0), *CC1 = row(kRgCC1), *CC2 = row(kRgCC2);
    R *FOM = row(kRgFOM), *COM = row(kRgCOM);
    D *B11 = drow(kRgB11), *B21 = drow(kRgB21), *B22 = drow(kRgB22), *G11 = drow(kRgG11), *G12 = drow(kRgG12);
    D *G21 = drow(kRgG21), *G22 = drow(kRgG22), *H1 = drow(kRgH1), *H2 = drow(kRgH2);
    R *FU = row(kRgFU), *FD = row(kRgFD), *FDIR = row(kRgFDIR), *DV = row(kRgDIV);
    const bool hogan = p.solver_hogan;
    // the solar sources of each region in FP64 (mixed_solar_source.F90:
    // 95-250), held in four of the elimination rows until the elimination
    // (which reads a layer's sources before it writes that layer's row)
    // takes them over
    D *SU = G21, *SD = G22, *SUC = G12, *SDC = B21;
    D bc = 0.0;
    if (!lw) {
      D f = f_inc_dir;
      FDIR[0] = (R)f;
      for (int i1 = 1; i1 <= nct - 1; ++i1) {
        const int ii = i1 - 1;
        SU[ii] = (D)FC1[ii] * f;
        SD[ii] = (D)FC2[ii] * f;
        f = f * (D)FT0[ii];
        FDIR[i1] = (R)f;
      }
      D bf = f;
      for (int i1 = nct; i1 <= L; ++i1) {
        const int ii = i1 - 1;
        const D tc = ov(3, i1 - 1) * bc + ov(2, i1 - 1) * bf;
        const D tf = ov(0, i1 - 1) * bf + ov(1, i1 - 1) * bc;
        SU[ii] = (D)FC1[ii] * tf; SD[ii] = (D)FC2[ii] * tf;
        SUC[ii] = (D)CC1[ii] * tc; SDC[ii] = (D)CC2[ii] * tc;
        bf = tf * (D)FT0[ii];
        bc = tc * (D)CT0[ii];
        FDIR[i1] = (R)(bf + bc);
      }
      if (p.i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING) {
        // the direct flux without delta-scaling, which the outputs and the
        // ground's direct reflection take (mixed_solar_source.F90:200-240)
        const R *FT0D = row(kRgFT0D), *CT0D = row(kRgCT0D);
        D fdd = f_inc_dir;
        for (int i1 = 1; i1 <= nct - 1; ++i1) { fdd = fdd * (D)FT0D[i1 - 1]; FDIR[i1] = (R)fdd; }
        D df = fdd, dc = 0.0;
        for (int i1 = nct; i1 <= L; ++i1) {
          const int ii = i1 - 1;
          const D tc = ov(3, i1 - 1) * dc + ov(2, i1 - 1) * df;
          const D tf = ov(0, i1 - 1) * df + ov(1, i1 - 1) * dc;
          df = tf * (D)FT0D[ii];
          dc = tc * (D)CT0D[ii];
          FDIR[i1] = (R)(df + dc);
        }
        bc = dc;
      }
      // the layers' source rows now hold the sources themselves
      for (int ii = 0; ii < L; ++ii) {
        FC1[ii] = (R)SU[ii]; FC2[ii] = (R)SD[ii];
        if (ii + 1 >= nct) { CC1[ii] = (R)SUC[ii]; CC2[ii] = (R)SDC[ii]; }
      }
    }
    auto su_of = [&](int ii) -> D { return lw ? (D)FC1[ii] : SU[ii]; };
    auto sd_of = [&](int ii) -> D { return lw ? (D)FC2[ii] : SD[ii]; };
    auto suc_of = [&](int ii) -> D { return lw ? (D)CC1[ii] : SUC[ii]; };
    auto sdc_of = [&](int ii) -> D { return lw ? (D)CC2[ii] : SDC[ii]; };
    // ground sources (mix_column.F90:365-385)
    D sgf, sgc;
    if (!lw) { sgf = (alb_dir - alb_diff) * ((D)FDIR[L] - bc); sgc = (alb_dir - alb_diff) * bc; }
    else { sgf = ov(4, L) * (1.0 - alb_diff) * dB_surf; sgc = ov(6, L) * (1.0 - alb_diff) * dB_surf; }
    // elimination, from the ground up (solver_mix_direct.F90:88-180,
    // solver_mix_direct_hogan.F90:78-140); the solar sources of layer ii are
    // read before row ii of the coefficients is written
    D a11 = alb_diff, a22 = alb_diff, a12 = 0.0, a21 = 0.0, g1 = sgf, g2 = sgc;
    for (int i1 = L; i1 >= 1; --i1) {
      const int ii = i1 - 1;
      const D r = FR[ii], t = FT[ii], sd = sd_of(ii), su = su_of(ii);
      if (i1 >= nct) {
        const D rcl = CR[ii], tcl = CT[ii], sdc = sdc_of(ii), suc = suc_of(ii);
        const D v11 = ov(0, i1), v21 = ov(2, i1), v12 = ov(1, i1), v22 = ov(3, i1);
        const D u11 = ov(4, i1 - 1), u12 = ov(5, i1 - 1), u21 = ov(6, i1 - 1), u22 = ov(7, i1 - 1);
        if (!hogan) {
          const D th11 = a11 * v11 + a12 * v21, th12 = a11 * v12 + a12 * v22;
          const D th21 = a21 * v11 + a22 * v21, th22 = a21 * v12 + a22 * v22;
          const D b21 = -th21 * r, b22 = 1.0 / (1.0 - th22 * rcl);
          const D gm21 = th21 * t, gm22 = th22 * tcl;
          const D hh2 = g2 + th21 * sd + th22 * sdc;
          D lam = th12 * rcl * b22;
          const D b11 = 1.0 / (1.0 - th11 * r + lam * b21);
          const D gm11 = th11 * t + lam * gm21, gm12 = th12 * tcl + lam * gm22;
          const D hh1 = g1 + th11 * sd + th12 * sdc + lam * hh2;
          B11[ii] = b11; B21[ii] = b21; B22[ii] = b22; G11[ii] = gm11; G12[ii] = gm12; G21[ii] = gm21;
          G22[ii] = gm22; H1[ii] = hh1; H2[ii] = hh2;
          lam = u22 * tcl * b22;
          D lamb = (u21 * t + lam * b21) * b11;
          const D n21 = u21 * r + lam * gm21 + lamb * gm11;
          const D n22 = u22 * rcl + lam * gm22 + lamb * gm12;
          const D ng2 = u21 * su + u22 * suc + lam * hh2 + lamb * hh1;
          lam = u12 * tcl * b22;
          lamb = (u11 * t + lam * b21) * b11;
          a11 = u11 * r + lam * gm21 + lamb * gm11;
          a12 = u12 * rcl + lam * gm22 + lamb * gm12;
          g1 = u11 * su + u12 * suc + lam * hh2 + lamb * hh1;
          a21 = n21; a22 = n22; g2 = ng2;
        } else {
          const D th11 = a11 * v11 + a22 * v21, th22 = a11 * v12 + a22 * v22;
          const D b11 = 1.0 / (1.0 - th11 * r), gm11 = th11 * t, hh1 = g1 + th11 * sd;
          const D b22 = 1.0 / (1.0 - th22 * rcl), gm22 = th22 * tcl, hh2 = g2 + th22 * sdc;
          const D l1 = su + hh1 * t * b11, l2 = suc + hh2 * tcl * b22;
          B11[ii] = b11; G11[ii] = gm11; H1[ii] = hh1; B22[ii] = b22; G22[ii] = gm22; H2[ii] = hh2;
          a11 = r + th11 * t * t * b11;
          a22 = rcl + th22 * tcl * tcl * b22;
          g1 = u11 * l1 + u12 * l2;
          g2 = u21 * l1 + u22 * l2;
        }
      } else {
        D th11 = a11;
        if (i1 == nct - 1 && nct < L) th11 = hogan ? a11 * ov(0, i1) + a22 * ov(2, i1) : a11 * ov(0, i1) + a12 * ov(2, i1);
        const D b11 = 1.0 / (1.0 - th11 * r), gm11 = th11 * t, hh1 = g1 + th11 * sd;
        B11[ii] = b11; G11[ii] = gm11; H1[ii] = hh1;
        const D lam = t * b11;
        a11 = r + lam * gm11;
        g1 = su + lam * hh1;
      }
    }
    // back-substitution (solver_mix_direct.F90:182-300); the sources are
    // read back from the rows, which hold them rounded to the build's type
    D fd_prev = f_inc_down, fu_prev;
    FD[0] = (R)f_inc_down;
    if (nct > 1) fu_prev = a11 * f_inc_down + g1;
    else fu_prev = g1 + f_inc_down * (ov(0, 0) * a11 + ov(2, 0) * (hogan ? a22 : a12));
    FU[0] = (R)fu_prev;
    for (int i1 = 1; i1 <= nct - 1; ++i1) {
      const int ii = i1 - 1;
      const D fdt = fd_prev;
      const D fub = (G11[ii] * fdt + H1[ii]) * B11[ii];
      const D fdb = (D)FT[ii] * fdt + (D)FR[ii] * fub + (D)FC2[ii];
      FU[i1] = (R)fub; FD[i1] = (R)fdb;
      if constexpr (kFP64) DV[ii] = fub - fu_prev + fdt - fdb;
      else DV[ii] = (R)((D)FOM[ii] * (fdt + fub) - ((D)FC1[ii] + (D)FC2[ii]));
      fu_prev = fub; fd_prev = fdb;
    }
    D fd1 = 0.0, fd2 = 0.0;
    for (int i1 = nct; i1 <= L; ++i1) {
      const int ii = i1 - 1;
      if (i1 > nct) {
        const D d1 = fd1, d2 = fd2;
        fd1 = ov(0, i1 - 1) * d1 + ov(1, i1 - 1) * d2;
        fd2 = ov(2, i1 - 1) * d1 + ov(3, i1 - 1) * d2;
      } else {
        fd1 = ov(0, i1 - 1) * fd_prev;
        fd2 = ov(2, i1 - 1) * fd_prev;
      }
      D fu1, fu2;
      if (!hogan) {
        fu1 = (G11[ii] * fd1 + G12[ii] * fd2 + H1[ii]) * B11[ii];
        fu2 = (G21[ii] * fd1 + G22[ii] * fd2 - B21[ii] * fu1 + H2[ii]) * B22[ii];
      } else {
        fu1 = (G11[ii] * fd1 + H1[ii]) * B11[ii];
        fu2 = (G22[ii] * fd2 + H2[ii]) * B22[ii];
      }
      const D nd1 = (D)FT[ii] * fd1 + (D)FR[ii] * fu1 + (D)FC2[ii];
      const D nd2 = (D)CT[ii] * fd2 + (D)CR[ii] * fu2 + (D)CC2[ii];
      const D fdt = fd_prev, fut = fu_prev;
      fu_prev = fu1 + fu2; fd_prev = nd1 + nd2;
      FU[i1] = (R)fu_prev; FD[i1] = (R)fd_prev;
      // the layer's divergence: from the level fluxes of the FP64 solve, or
      // in the mixed build under Hogan's form from each region's absorption,
      // whose region fluxes close each region's layer equations (those of
      // solver_mix_direct close only in their sum over the regions)
      if (kFP64 || !hogan) DV[ii] = (R)(fu_prev - fut + fdt - fd_prev);
      else
        DV[ii] = (R)((D)FOM[ii] * (fd1 + fu1) - ((D)FC1[ii] + (D)FC2[ii]) + (D)COM[ii] * (fd2 + fu2) -
                     ((D)CC1[ii] + (D)CC2[ii]));
      fd1 = nd1; fd2 = nd2;
    }
  }

  // The serial part of the three-region solve (clear, stratiform and
  // convective) on one lane, in FP64 in every build: triple_solar_source.F90:
  // 160-400, the ground sources of triple_column.F90:380-410 and
  // solver_triple_hogan.F90:200-410.  Rows as solve_region leaves them, the
  // interface coefficients of stage_regions3 (v_jk row 3 j + k, u_jk row
  // 9 + 3 j + k); writes the level fluxes (diffuse in the solar), the direct
  // flux and the layer divergence.  Layers i are 0-based here; interface i
  // lies below layer i-1 (0: the top).
  __device__ static __noinline__ void region_serial3(const FluxParams &p, const Smem &S, R *X, double *Y, int nct,
                                                     int L, bool lw, R f_inc_down_r, R f_inc_dir_r, R alb_diff_r,
                                                     R alb_dir_r, R dB_surf_r) {
    using D = double;
    auto row = [&](int k) { return X + (size_t)k * (LP + 1); };
    auto drow = [&](int k) { return Y + (size_t)k * (LP + 1); };
    auto ov = [&](int m, int i) -> D { return (D)S.ovl[(size_t)m * (LP + 1) + i]; };
    const D f_inc_down = f_inc_down_r, f_inc_dir = f_inc_dir_r, alb_diff = alb_diff_r, alb_dir = alb_dir_r;
    const D dB_surf = dB_surf_r;
    // region k's rows: 0 the clear, 1 the stratiform, 2 the convective
    R *T[3] = {row(kRgFT), row(kRgCT), row(kRgVT)}, *RR[3] = {row(kRgFR), row(kRgCR), row(kRgVR)};
    R *T0[3] = {row(kRgFT0), row(kRgCT0), row(kRgVT0)}, *C1[3] = {row(kRgFC1), row(kRgCC1), row(kRgVC1)};
    R *C2[3] = {row(kRgFC2), row(kRgCC2), row(kRgVC2)}, *OM[3] = {row(kRgFOM), row(kRgCOM), row(kRgVOM)};
    D *B[3] = {drow(kRgB11), drow(kRgB22), drow(kRgB33)}, *G[3] = {drow(kRgG11), drow(kRgG22), drow(kRgG33)};
    D *H[3] = {drow(kRgH1), drow(kRgH2), drow(kRgH3)};
    // the solar sources of each region in FP64 (Hogan's form leaves the
    // coupling rows free)
    D *SU[3] = {drow(kRgG21), drow(kRgG12), drow(kRgSUV)}, *SD[3] = {drow(kRgB21), drow(kRgH2), drow(kRgSDV)};
    R *FU = row(kRgFU), *FD = row(kRgFD), *FDIR = row(kRgFDIR), *DV = row(kRgDIV);
    D base[3] = {0.0, 0.0, 0.0};
    if (!lw) {
      D f = f_inc_dir;
      FDIR[0] = (R)f;
      for (int i1 = 1; i1 <= nct - 1; ++i1) {
        const int ii = i1 - 1;
        SU[0][ii] = (D)C1[0][ii] * f;
        SD[0][ii] = (D)C2[0][ii] * f;
        f = f * (D)T0[0][ii];
        FDIR[i1] = (R)f;
      }
      base[0] = f;
      for (int i1 = nct; i1 <= L; ++i1) {
        const int ii = i1 - 1;
        D top[3];
        for (int j = 0; j < 3; ++j)
          top[j] = ov(3 * j, i1 - 1) * base[0] + ov(3 * j + 1, i1 - 1) * base[1] + ov(3 * j + 2, i1 - 1) * base[2];
        for (int k = 0; k < 3; ++k) {
          base[k] = top[k] * (D)T0[k][ii];
          SU[k][ii] = (D)C1[k][ii] * top[k];
          SD[k][ii] = (D)C2[k][ii] * top[k];
        }
        FDIR[i1] = (R)(base[0] + base[1] + base[2]);
      }
      if (p.i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING) {
        // the direct flux without delta-scaling, which the outputs and the
        // ground's direct reflection take (triple_solar_source.F90:300-350)
        const R *T0D[3] = {row(kRgFT0D), row(kRgCT0D), row(kRgVT0D)};
        D fdd = f_inc_dir;
        for (int i1 = 1; i1 <= nct - 1; ++i1) { fdd = fdd * (D)T0D[0][i1 - 1]; FDIR[i1] = (R)fdd; }
        D db[3] = {fdd, 0.0, 0.0};
        for (int i1 = nct; i1 <= L; ++i1) {
          const int ii = i1 - 1;
          D top[3];
          for (int j = 0; j < 3; ++j)
            top[j] = ov(3 * j, i1 - 1) * db[0] + ov(3 * j + 1, i1 - 1) * db[1] + ov(3 * j + 2, i1 - 1) * db[2];
          for (int k = 0; k < 3; ++k) db[k] = top[k] * (D)T0D[k][ii];
          FDIR[i1] = (R)(db[0] + db[1] + db[2]);
        }
        for (int k = 0; k < 3; ++k) base[k] = db[k];
      }
      // the layers' source rows now hold the sources themselves
      for (int ii = 0; ii < L; ++ii)
        for (int k = 0; k < 3; ++k)
          if (k == 0 || ii + 1 >= nct) { C1[k][ii] = (R)SU[k][ii]; C2[k][ii] = (R)SD[k][ii]; }
    }
    auto su_of = [&](int k, int ii) -> D { return lw ? (D)C1[k][ii] : SU[k][ii]; };
    auto sd_of = [&](int k, int ii) -> D { return lw ? (D)C2[k][ii] : SD[k][ii]; };
    // ground sources (triple_column.F90:380-410)
    D sg[3];
    for (int k = 0; k < 3; ++k)
      sg[k] = lw ? ov(9 + 3 * k, L) * (1.0 - alb_diff) * dB_surf : (alb_dir - alb_diff) * base[k];
    // elimination from the ground up (solver_triple_hogan.F90:200-320); the
    // solar sources of layer ii are read before its coefficient rows are
    // written
    D a[3] = {alb_diff, alb_diff, alb_diff}, g[3] = {sg[0], sg[1], sg[2]};
    for (int i1 = L; i1 >= 1; --i1) {
      const int ii = i1 - 1;
      if (i1 >= nct) {
        D th[3], lam[3];
        for (int k = 0; k < 3; ++k) th[k] = a[0] * ov(k, i1) + a[1] * ov(3 + k, i1) + a[2] * ov(6 + k, i1);
        for (int k = 0; k < 3; ++k) {
          const D r = RR[k][ii], t = T[k][ii], sd = sd_of(k, ii), su = su_of(k, ii);
          const D b = 1.0 / (1.0 - th[k] * r);
          const D hh = g[k] + th[k] * sd;
          B[k][ii] = b; G[k][ii] = th[k] * t; H[k][ii] = hh;
          lam[k] = su + hh * t * b;
          a[k] = r + th[k] * t * t * b;
        }
        for (int j = 0; j < 3; ++j)
          g[j] = ov(9 + 3 * j, i1 - 1) * lam[0] + ov(9 + 3 * j + 1, i1 - 1) * lam[1] + ov(9 + 3 * j + 2, i1 - 1) * lam[2];
      } else {
        const D r = RR[0][ii], t = T[0][ii], sd = sd_of(0, ii), su = su_of(0, ii);
        D th11 = a[0];
        if (i1 == nct - 1 && nct < L) th11 = a[0] * ov(0, i1) + a[1] * ov(3, i1) + a[2] * ov(6, i1);
        const D b11 = 1.0 / (1.0 - th11 * r), gm11 = th11 * t, hh1 = g[0] + th11 * sd;
        B[0][ii] = b11; G[0][ii] = gm11; H[0][ii] = hh1;
        const D lam = t * b11;
        a[0] = r + lam * gm11;
        g[0] = su + lam * hh1;
      }
    }
    // back-substitution (solver_triple_hogan.F90:320-410); the sources are
    // read back from the rows, which hold them rounded to the build's type
    D fd_prev = f_inc_down, fu_prev;
    FD[0] = (R)f_inc_down;
    if (nct > 1) fu_prev = a[0] * f_inc_down + g[0];
    else fu_prev = g[0] + f_inc_down * (ov(0, 0) * a[0] + ov(3, 0) * a[1] + ov(6, 0) * a[2]);
    FU[0] = (R)fu_prev;
    for (int i1 = 1; i1 <= nct - 1; ++i1) {
      const int ii = i1 - 1;
      const D fdt = fd_prev;
      const D fub = (G[0][ii] * fdt + H[0][ii]) * B[0][ii];
      const D fdb = (D)T[0][ii] * fdt + (D)RR[0][ii] * fub + (D)C2[0][ii];
      FU[i1] = (R)fub; FD[i1] = (R)fdb;
      if constexpr (kFP64) DV[ii] = fub - fu_prev + fdt - fdb;
      else DV[ii] = (R)((D)OM[0][ii] * (fdt + fub) - ((D)C1[0][ii] + (D)C2[0][ii]));
      fu_prev = fub; fd_prev = fdb;
    }
    D fdk[3] = {0.0, 0.0, 0.0};
    for (int i1 = nct; i1 <= L; ++i1) {
      const int ii = i1 - 1;
      D d[3];
      if (i1 > nct) {
        for (int j = 0; j < 3; ++j)
          d[j] = ov(3 * j, i1 - 1) * fdk[0] + ov(3 * j + 1, i1 - 1) * fdk[1] + ov(3 * j + 2, i1 - 1) * fdk[2];
      } else {
        for (int j = 0; j < 3; ++j) d[j] = ov(3 * j, i1 - 1) * fd_prev;
      }
      const D fdt = fd_prev, fut = fu_prev;
      D fu_sum = 0.0, fd_sum = 0.0, div = 0.0;
      for (int k = 0; k < 3; ++k) {
        const D fu = (G[k][ii] * d[k] + H[k][ii]) * B[k][ii];
        fdk[k] = (D)T[k][ii] * d[k] + (D)RR[k][ii] * fu + (D)C2[k][ii];
        fu_sum = fu_sum + fu;
        fd_sum = fd_sum + fdk[k];
        // each region's absorption closes its own layer equations under
        // Hogan's form: the mixed build forms the divergence from it
        div = div + ((D)OM[k][ii] * (d[k] + fu) - ((D)C1[k][ii] + (D)C2[k][ii]));
      }
      fu_prev = fu_sum; fd_prev = fd_sum;
      FU[i1] = (R)fu_prev; FD[i1] = (R)fd_prev;
      if constexpr (kFP64) DV[ii] = (R)(fu_prev - fut + fdt - fd_prev);
      else DV[ii] = (R)div;
    }
  }

  __device__ static void solve_mcica(const FluxParams &p, const Smem &S, int col, const GPoint &gp,
                                     const GasTerm &gt, const BandInfo &bd, int bi, int b, int r, int L, bool lw,
                                     R sec0, const R *dB_b, const R *dB2_b, R f_inc_down, R f_inc_dir,
                                     R alb_diff, R alb_dir, R dB_surf, R w_g, Acc *acc, int max_abs,
                                     bool active) {
    const int ndp = p.nd_profile, nc = p.n_condensed;
    R *t0d = (!lw && p.i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING) ? S.t0d + (size_t)(threadIdx.x / P) * LP : nullptr;
    const R *kgt_b = S.kgt + (size_t)bi * LP, *kes_b = S.kes + (size_t)bi * LP;
    const R *kabs_b = S.kabs + (size_t)bi * LP, *asym_b = S.asym + (size_t)bi * LP;
    const R *fwd_b = S.fwd + (size_t)bi * LP, *amt_b = S.amt + (size_t)bi * max_abs * LP;
    const R *phf_nc = S.phf_nc + (size_t)bi * LP, *fwd_nc = S.fwd_nc + (size_t)bi * LP;
    const R *c_ke = S.c_ke + (size_t)bi * nc * LP, *c_ks = S.c_ks + (size_t)bi * nc * LP;
    const R *c_ka = S.c_ka + (size_t)bi * nc * LP, *c_ph = S.c_phf + (size_t)bi * nc * LP;
    const R *c_fw = S.c_fwd + (size_t)bi * nc * LP;

    const int iex = gp.iex_major;
    const int first = __ldg(p.first_subcol_k + b + (size_t)p.nd_band_sp * iex);
    const int last = __ldg(p.first_subcol_k + b + (size_t)p.nd_band_sp * (iex + 1)) - 1;
    const int nsub = __ldg(p.subcol_k + b + (size_t)p.nd_band_sp * iex);
    const R fcl = load_in<R>(p.frac_cloudy + col);
    const int ncld = p.n_subcol_cld ? __ldg(p.n_subcol_cld + col) : 0;
    const int nfill = min(p.n_subcol_req, p.n_subcol_gen);
    // blending weights (mcica_sample.F90:862-925)
    const R w_sub = w_g * fcl / (R)(nsub > 0 ? nsub : 1);
    const R w_clr = w_g * (R(1) - fcl);
    (void)ndp;

    // Solve index it = 0 is the clear solve, it = 1.. the subcolumns
    // first..last.  The count is made uniform over the warp (all groups
    // take part in every shuffle); surplus iterations are discarded.
    // the gas absorption of the lane's layers is the same for every subcolumn
    R kgv[CH];
    gas_k_lane(p, S, gt, gp, bd, amt_b, r, L, kgv);
    const int n_iter = last - first + 2;
    const int n_iter_warp = __reduce_max_sync(0xffffffffu, n_iter);
    for (int it = 0; it < n_iter_warp; ++it) {
      const bool clear = (it == 0);
      const int m = first + it - 1;
      bool use = active && it < n_iter && (clear ? (w_clr != R(0)) : (w_sub != R(0)));
      int slot_sub = -1;
      if (!clear) {
        int idx = (it < n_iter ? m : first) % p.n_subcol_req;
        if (idx == 0) idx = p.n_subcol_req;
        int j = __ldg(p.subcol_reorder + (idx - 1));
        if (p.n_subcol_cld && ncld > 0 && j > ncld && j <= nfill) j = (j - 1) % ncld + 1;
        slot_sub = j - 1;
        if (slot_sub < 0 || slot_sub >= p.n_subcol_gen) {   // out-of-range table entry: report, skip
          if (p.error_flag) atomicOr(p.error_flag, 1);
          slot_sub = -1;
          use = false;
        }
      }
      R T[CH], Rf[CH], T0[CH], c1[CH], c2[CH], om[CH];
#pragma unroll
      for (int jj = 0; jj < CH; ++jj) {
        const int i = r * CH + jj, s = jj * P + r;
        if (i < L) {
          const R kg = kgv[jj];
          R cs_i = (slot_sub >= 0) ? S.csub[(size_t)slot_sub * LP + s] : R(0);
          bool cloudy = false;
          if (slot_sub >= 0 && S.wcld[s] > R(0)) {
            for (int t = 0; t < p.n_cloud_type; ++t) cloudy |= (cs_i * S.frac[(size_t)t * LP + s] > R(0));
          }
          if (!cloudy) {
            cell_coef(p, kgt_b[s], kes_b[s], kabs_b[s], kg, S.mass[s], asym_b[s], fwd_b[s], sec0,
                      T[jj], Rf[jj], T0[jj], c1[jj], c2[jj], om[jj]);
            if (t0d) t0d[s] = t0_unscaled(kgt_b[s], kg, S.mass[s], sec0);
          } else {
            // mcica_sample.F90:472-700 then mcica_column.F90:336-470: each
            // cloud type is the clear cell plus its components in order,
            // scaled by c_sub (one component per type for ice/water clouds,
            // both in type 1 for homogeneous clouds)
            R sT = R(0), sR = R(0), sT0 = R(0), s1 = R(0), s2 = R(0), sO = R(0), sT0d = R(0);
            for (int t = 0; t < p.n_cloud_type; ++t) {
              const R fc = S.frac[(size_t)t * LP + s];
              if (!(cs_i * fc > R(0))) continue;
              R kgt = kgt_b[s], kes = kes_b[s], kab = kabs_b[s], fw = fwd_nc[s], ph = phf_nc[s];
              for (int k = 0; k < nc; ++k) {
                if (p.comp_type[k] - 1 != t) continue;
                const size_t qk = (size_t)k * LP + s;
                kgt = kgt + c_ke[qk] * cs_i;
                kes = kes + c_ks[qk] * cs_i;
                kab = kab + c_ka[qk] * cs_i;
                fw = fw + c_fw[qk] * cs_i;
                ph = ph + c_ph[qk] * cs_i;
              }
              R asym, fwd;
              const R eps = (R)kEps64;
              if (p.l_rescale) {
                R den = kes - fw;
                asym = (ph - fw) / (den > eps ? den : eps);
                fwd = fw / (kes > eps ? kes : eps);
              } else {
                asym = ph / (kes > eps ? kes : eps);
                fwd = R(0);
              }
              R tT, tR, tT0, t1, t2, tO;
              cell_coef(p, kgt, kes, kab, kg, S.mass[s], asym, fwd, sec0, tT, tR, tT0, t1, t2, tO);
              sT = sT + fc * tT; sR = sR + fc * tR; sT0 = sT0 + fc * tT0;
              s1 = s1 + fc * t1; s2 = s2 + fc * t2; sO = sO + fc * tO;
              if (t0d) sT0d = sT0d + fc * t0_unscaled(kgt, kg, S.mass[s], sec0);
            }
            T[jj] = sT; Rf[jj] = sR; T0[jj] = lw ? R(1) : sT0; c1[jj] = s1; c2[jj] = s2; om[jj] = sO;
            if (t0d) t0d[s] = sT0d;
          }
        } else {
          T[jj] = R(1); Rf[jj] = R(0); T0[jj] = R(1); c1[jj] = R(0); c2[jj] = R(0); om[jj] = R(0);
          if (t0d) t0d[s] = R(1);
        }
      }
      if constexpr (SRC == SOCGPU_IP_SOLAR)
        if (p.keqv) {
          fold_direct(S, bi, max_abs, r, L, T0, c2);
          if (t0d) fold_direct_row(S, bi, max_abs, r, L, t0d);
        }
      solve_column(p, T, Rf, T0, c1, c2, om, r, L, lw, dB_b, dB2_b, f_inc_down, f_inc_dir,
                   alb_diff, alb_dir, dB_surf, clear ? w_clr : w_sub, acc, use, t0d);
    }
  }

  // Sources, direct beam, solve and accumulation of one monochromatic
  // problem held in the group's registers.
  __device__ static void solve_column(const FluxParams &p, R (&T)[CH], R (&Rf)[CH], R (&T0)[CH],
                                      R (&c1)[CH], R (&c2)[CH], R (&om)[CH], int r, int L, bool lw,
                                      const R *dB_b, const R *dB2_b, R f_inc_down, R f_inc_dir,
                                      R alb_diff, R alb_dir, R dB_surf, R w, Acc *acc, bool active,
                                      const R *t0d = nullptr) {
    // the last layer a lane accumulates into: none when the solve is discarded
    const int L_acc = active ? L : -1;
    Acc *acc_up = acc, *acc_dn = acc + (LP + 1), *acc_dir = acc + 2 * (LP + 1), *acc_div = acc + 3 * (LP + 1);
    // --- sources -------------------------------------------------------------
    // ssum = s_up + s_down of each layer: with om = 1 - T - R it gives the
    // layer's flux divergence (1-T-R)(F_dn(top) + F_up(bottom)) - ssum, the
    // form the mixed kernel uses instead of differencing FP32 level fluxes
    R ssum[CH];
    R fdir_bottom = R(0);
    if (!lw) {
      // direct beam: exclusive product scan of the chunks' transmissions
      R prod = R(1);
#pragma unroll
      for (int j = 0; j < CH; ++j) prod *= T0[j];
      R incl = prod;
#pragma unroll
      for (int d = 1; d < P; d <<= 1) {
        R y = __shfl_up_sync(0xffffffffu, incl, d, P);
        if (r >= d) incl = y * incl;
      }
      R excl = __shfl_up_sync(0xffffffffu, incl, 1, P);
      if (r == 0) excl = R(1);
      R fd = f_inc_dir * excl;
      fdir_bottom = f_inc_dir * __shfl_sync(0xffffffffu, incl, P - 1, P);
      if (r == 0 && active) acc_dir[LP] += w * fd;
      // the reported direct flux: the scaled beam here, or the unscaled one
      // below (ip_direct_noscaling)
      const int L_dir = t0d ? -1 : L_acc;
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j;
        R su = c1[j] * fd, sd = c2[j] * fd;   // solar_source.F90:146-155
        c1[j] = su; c2[j] = sd;
        ssum[j] = su + sd;
        fd = fd * T0[j];
        if (i < L_dir) acc_dir[j * P + r] += w * fd;
      }
      if (t0d) {
        // ip_direct_noscaling (solar_source.F90:157-176): the reported direct
        // flux and the ground's direct reflection take the unscaled beam,
        // the sources the scaled one
        R pd = R(1);
#pragma unroll
        for (int j = 0; j < CH; ++j) pd *= t0d[j * P + r];
        R incd = pd;
#pragma unroll
        for (int d = 1; d < P; d <<= 1) {
          R y = __shfl_up_sync(0xffffffffu, incd, d, P);
          if (r >= d) incd = y * incd;
        }
        R exd = __shfl_up_sync(0xffffffffu, incd, 1, P);
        if (r == 0) exd = R(1);
        R fdd = f_inc_dir * exd;
        fdir_bottom = f_inc_dir * __shfl_sync(0xffffffffu, incd, P - 1, P);
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          const int i = r * CH + j;
          fdd = fdd * t0d[j * P + r];
          if (i < L_acc) acc_dir[j * P + r] += w * fdd;
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j, s = j * P + r;
        if (i < L) {
          R dB = dB_b[s];
          R su, sd;
          if (p.l_ir_source_quad) {       // ir_source.F90:93-119
            su = c1[j] * dB + c2[j] * dB2_b[s];
            sd = -c1[j] * dB + c2[j] * dB2_b[s];
            ssum[j] = R(2) * c2[j] * dB2_b[s];
          } else {
            su = c1[j] * dB; sd = -su;
            ssum[j] = R(0);
          }
          c1[j] = su; c2[j] = sd;
        } else {
          c1[j] = R(0); c2[j] = R(0); ssum[j] = R(0);
        }
      }
    }
    R src_ground = lw ? (R(1) - alb_diff) * dB_surf : (alb_dir - alb_diff) * fdir_bottom;

    if (NOSCAT) {
      // solver_no_scat.F90:75-94: downward affine scan then upward.
      R A = R(1), B = R(0);                // F_dn(bottom) = A*F_dn(top) + B over the chunk
#pragma unroll
      for (int j = 0; j < CH; ++j) { A = T[j] * A; B = c2[j] + T[j] * B; }
      R iA = A, iB = B;
#pragma unroll
      for (int d = 1; d < P; d <<= 1) {
        R yA = __shfl_up_sync(0xffffffffu, iA, d, P), yB = __shfl_up_sync(0xffffffffu, iB, d, P);
        if (r >= d) { iB = iA * yB + iB; iA = iA * yA; }
      }
      R eA = __shfl_up_sync(0xffffffffu, iA, 1, P), eB = __shfl_up_sync(0xffffffffu, iB, 1, P);
      if (r == 0) { eA = R(1); eB = R(0); }
      R fdn_top = eA * f_inc_down + eB;
      R fdn_surf = __shfl_sync(0xffffffffu, iA, P - 1, P) * f_inc_down + __shfl_sync(0xffffffffu, iB, P - 1, P);
      R fup_surf = (R(1) - alb_diff) * dB_surf + alb_diff * fdn_surf;
      // upward: F_up(top) = C*F_up(bottom) + E over the chunk
      R C = R(1), E = R(0);
#pragma unroll
      for (int j = CH - 1; j >= 0; --j) { C = T[j] * C; E = c1[j] + T[j] * E; }
      R sC = C, sE = E;
#pragma unroll
      for (int d = 1; d < P; d <<= 1) {
        R yC = __shfl_down_sync(0xffffffffu, sC, d, P), yE = __shfl_down_sync(0xffffffffu, sE, d, P);
        if (r + d < P) { sE = sC * yE + sE; sC = sC * yC; }
      }
      R xC = __shfl_down_sync(0xffffffffu, sC, 1, P), xE = __shfl_down_sync(0xffffffffu, sE, 1, P);
      if (r == P - 1) { xC = R(1); xE = R(0); }
      R fup_bot = xC * fup_surf + xE;      // F_up at the bottom of this chunk
      // per-level fluxes of the chunk: first the upward sweep, storing F_up in c1
      R fu = fup_bot;
#pragma unroll
      for (int j = CH - 1; j >= 0; --j) {
        R top = c1[j] + T[j] * fu;
        c1[j] = fu;                        // F_up at the bottom of layer j
        fu = top;
      }
      R fd = fdn_top;
      if (r == 0 && active) { acc_up[LP] += w * fu; acc_dn[LP] += w * fd; }
      R fu_prev = fu;
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j, s = j * P + r;
        R fdn = c2[j] + T[j] * fd;
        if (i < L_acc) {
          acc_up[s] += w * c1[j];
          acc_dn[s] += w * fdn;
          if constexpr (kFP64) acc_div[s] += w * (c1[j] - fu_prev + fd - fdn);
          else acc_div[s] += w * (om[j] * (fd + c1[j]) - ssum[j]);
        }
        fu_prev = c1[j];
        fd = fdn;
      }
      return;
    }

    // --- adding method (solver_homogen_direct.F90:94-131), eliminated from
    // the top down: at each level F_dn = rho F_up + sig, and across layer j
    // F_up(top) = a_j F_up(bottom) + b_j.  The chunks' states from above come
    // from a prefix scan of their layer composites; the upward fluxes at the
    // chunk bottoms from a suffix scan of the chunks' affine maps (a, b).
    // the chunk's composite, stacked pairwise (a tree of depth log2 CH, so
    // that the divisions of independent pairs overlap)
    Comp<R> cc;
    {
      Comp<R> lv[CH];
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        lv[j].R1 = Rf[j]; lv[j].R2 = Rf[j]; lv[j].Td = T[j]; lv[j].Tu = T[j]; lv[j].Su = c1[j]; lv[j].Sd = c2[j];
      }
#pragma unroll
      for (int w = 1; w < CH; w <<= 1)
#pragma unroll
        for (int j = 0; j + w < CH; j += 2 * w) lv[j] = stack(lv[j], lv[j + w]);
      cc = lv[0];
    }
    // above: inclusive prefix C_0 .. C_r, then the exclusive one
    Comp<R> pre = cc;
#pragma unroll
    for (int d = 1; d < P; d <<= 1) {
      Comp<R> y = shfl_up_comp(pre, d, P);
      if (r >= d) pre = stack(y, pre);
    }
    Comp<R> ex = shfl_up_comp(pre, 1, P);
    R rho, sig;            // the state at the top of this chunk
    if (r == 0) { rho = R(0); sig = f_inc_down; }
    else { rho = ex.R2; sig = ex.Sd + ex.Td * f_inc_down; }
    // elimination through the chunk.  The arrays now hold, per layer,
    // a (T), b (Rf) and the state at its top, rho (c1) and sig (c2);
    // F_up(chunk top) = A F_up(chunk bottom) + B.  Padding layers (T = 1,
    // R = 0, no sources) are the identity.
    R A = R(1), B = R(0);
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const R q = R(1) / (R(1) - Rf[j] * rho);
      const R a = T[j] * q;
      const R b = (Rf[j] * sig + c1[j]) * q;
      const R rho_n = Rf[j] + (T[j] * T[j] * rho) * q;     // T^2 rho formed beside the division
      const R sig_n = c2[j] + a * (sig + rho * c1[j]);
      T[j] = a; Rf[j] = b; c1[j] = rho; c2[j] = sig;
      B = B + A * b; A = A * a;
      rho = rho_n; sig = sig_n;
    }
    // the surface closes the last chunk: F_up = alb F_dn + src_ground with
    // F_dn = rho F_up + sig; that chunk's map becomes the constant F_up(top)
    R fu_surf = R(0);
    if (r == P - 1) {
      fu_surf = (alb_diff * sig + src_ground) / (R(1) - alb_diff * rho);
      B = A * fu_surf + B; A = R(0);
    }
    // suffix scan of the affine maps: F_up at the top of every chunk
#pragma unroll
    for (int d = 1; d < P; d <<= 1) {
      R yA = __shfl_down_sync(0xffffffffu, A, d, P), yB = __shfl_down_sync(0xffffffffu, B, d, P);
      if (r + d < P) { B = A * yB + B; A = A * yA; }
    }
    R fu = __shfl_down_sync(0xffffffffu, B, 1, P);     // F_up at the bottom of this chunk
    if (r == P - 1) fu = fu_surf;
    R fd = rho * fu + sig;
    // back-substitution from the chunk bottom up, accumulating the level
    // below each layer and the layer's divergence
#pragma unroll
    for (int j = CH - 1; j >= 0; --j) {
      const int i = r * CH + j, s = j * P + r;
      const R fu_top = T[j] * fu + Rf[j];
      const R fd_top = c1[j] * fu_top + c2[j];
      if (i < L_acc) {
        acc_up[s] += w * fu;
        acc_dn[s] += w * fd;
        if constexpr (kFP64) acc_div[s] += w * (fu - fu_top + fd_top - fd);
        else acc_div[s] += w * (om[j] * (fd_top + fu) - ssum[j]);
      }
      fu = fu_top; fd = fd_top;
    }
    if (r == 0 && active) { acc_up[LP] += w * fu; acc_dn[LP] += w * fd; }
  }
};

// Resident CTAs asked of the register allocator for the single-batch kernel:
// short chunks of the clear-sky kernels keep 4 CTAs of 256 threads (64
// registers) per SM, which the shared memory of a 100-layer solar column
// also allows; the McICA kernels would spill at 64 registers.
constexpr int single_min_ctas(int ch, bool mcica) { return (ch <= 4 && !mcica) ? 4 : (ch <= 13 && !mcica ? 2 : 1); }

template <class R, bool MIX, int P, int CH, bool NOSCAT, bool MCICA, int SRC>
__global__ void __launch_bounds__(256, single_min_ctas(CH, MCICA)) flux_kernel(const __grid_constant__ FluxParams p) {
  FluxKernel<R, MIX, P, CH, NOSCAT, MCICA, SRC>::run(p, blockIdx.x);
}

// Persistent form over many column batches: items[i] describes one batch
// (its own spectrum, layer count, options and arrays); batch i owns the work
// indices col_start[i] .. col_start[i+1]-1, one per column.  Each CTA strides
// over the work indices, finds the batch by binary search and keeps the
// batch's parameters in shared memory while consecutive indices stay in it.
// Resident CTAs the batched kernel asks the register allocator for: its
// parameters sit in shared memory, not in the constant bank, so without a
// bound it keeps about twice the registers of flux_kernel (measured with
// -Xptxas -v: 3 CTAs of 256 threads fit without spills up to 4 layers per
// lane).
constexpr int batched_min_ctas(int ch) { return ch <= 4 ? 3 : (ch <= 9 ? 2 : 1); }

template <class R, bool MIX, int P, int CH, bool NOSCAT, bool MCICA, int SRC>
__global__ void __launch_bounds__(256, batched_min_ctas(CH))
flux_kernel_batched(const FluxParams *__restrict__ items, const long long *__restrict__ col_start, int n_items,
                    long long total) {
  __shared__ __align__(16) FluxParams sp;
  __shared__ int s_item;
  static_assert(sizeof(FluxParams) % 4 == 0, "FluxParams is copied as words");
  int cur = -1;
  for (long long w = blockIdx.x; w < total; w += gridDim.x) {
    if (threadIdx.x == 0) {
      int lo = 0, hi = n_items - 1;   // last batch whose first index is <= w
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (col_start[mid] <= w) lo = mid; else hi = mid - 1;
      }
      s_item = lo;
    }
    __syncthreads();
    const int it = s_item;
    if (it != cur) {
      const int *src = reinterpret_cast<const int *>(items + it);
      int *dst = reinterpret_cast<int *>(&sp);
      for (int q = threadIdx.x; q < (int)(sizeof(FluxParams) / 4); q += blockDim.x) dst[q] = src[q];
      cur = it;
    }
    __syncthreads();
    FluxKernel<R, MIX, P, CH, NOSCAT, MCICA, SRC>::run(sp, (int)(w - col_start[it]));
    __syncthreads();
  }
}

}  // namespace socgpu
