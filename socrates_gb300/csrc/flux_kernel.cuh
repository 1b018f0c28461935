// flux_kernel.cuh -- fused two-stream flux kernel for sm_103a.
//
// One CTA per column.  The CTA first stages the column's per-band grey
// optics, gas amounts and Planck terms in shared memory (the band loop of
// radiance_calc.F90:883-1600), then its lanes solve the monochromatic
// problems of every g-point (k-term product) of the band range:
//
//   * a "group" of P consecutive lanes owns one (column, g-point) solve;
//     lane r of the group holds layers [r*CH, r*CH+CH) in registers;
//   * the per-layer physics (single_scattering, rescale_tau_omega,
//     two_coeff, sources) is computed for all layers in parallel;
//   * the direct beam (solar_source.F90:105-176) is a product scan over
//     the group's lanes, and the adding-method solve
//     (solver_homogen_direct.F90:94-131) becomes an associative scan of
//     layer "composites" (reflection/transmission/source of a stack of
//     layers) down and up the group, followed by the reference's
//     elimination and back-substitution inside each lane's chunk;
//   * solver_no_scat (solver_no_scat.F90:75-94) is two affine scans;
//   * each group accumulates its fluxes in its own shared-memory slice
//     (augment_channel_mod.F90:158-235); slices are summed in a fixed order
//     at the end, so results are deterministic.
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

constexpr int kNumAcc = 4;   // up, down, direct (per level), divergence (per layer)

// Column-major (Fortran) element access with leading extent nd.
__device__ __forceinline__ double ld2(const double *a, int l, int i, int nd) {
  return __ldg(a + (size_t)l + (size_t)nd * (size_t)i);
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
// Shared-memory layout of one column (identical on host and device).
struct SmemLayout {
  int L, nb, max_abs, n_comp, n_sub, n_groups;
  size_t off_p, off_t, off_mass, off_kgt, off_kes, off_kabs, off_asym, off_fwd, off_amt;
  size_t off_planck, off_dB, off_dB2;
  size_t off_phf_nc, off_fwd_nc, off_c_ke, off_c_ks, off_c_ka, off_c_phf, off_c_fwd;
  size_t off_wcld, off_frac, off_csub;
  size_t off_acc;
  size_t bytes;
};

template <class R, class Acc>
__host__ __device__ inline SmemLayout make_layout(int L, int nb, int max_abs, int n_comp, int n_sub,
                                                  int n_groups, bool lw, bool mcica) {
  SmemLayout s{};
  s.L = L; s.nb = nb; s.max_abs = max_abs; s.n_comp = n_comp; s.n_sub = n_sub; s.n_groups = n_groups;
  size_t o = 0;
  auto take = [&](size_t elems, size_t esz) { size_t r = (o + 15) & ~(size_t)15; o = r + elems * esz; return r; };
  s.off_p = take(L, sizeof(R));
  s.off_t = take(L, sizeof(R));
  s.off_mass = take(L, sizeof(R));
  s.off_kgt = take((size_t)nb * L, sizeof(R));
  s.off_kes = take((size_t)nb * L, sizeof(R));
  s.off_kabs = take((size_t)nb * L, sizeof(R));
  s.off_asym = take((size_t)nb * L, sizeof(R));
  s.off_fwd = take((size_t)nb * L, sizeof(R));
  s.off_amt = take((size_t)nb * max_abs * L, sizeof(R));
  s.off_planck = lw ? take((size_t)nb * (L + 1), sizeof(R)) : o;
  s.off_dB = lw ? take((size_t)nb * L, sizeof(R)) : o;
  s.off_dB2 = lw ? take((size_t)nb * L, sizeof(R)) : o;
  if (mcica) {
    s.off_phf_nc = take((size_t)nb * L, sizeof(R));
    s.off_fwd_nc = take((size_t)nb * L, sizeof(R));
    s.off_c_ke = take((size_t)nb * n_comp * L, sizeof(R));
    s.off_c_ks = take((size_t)nb * n_comp * L, sizeof(R));
    s.off_c_ka = take((size_t)nb * n_comp * L, sizeof(R));
    s.off_c_phf = take((size_t)nb * n_comp * L, sizeof(R));
    s.off_c_fwd = take((size_t)nb * n_comp * L, sizeof(R));
    s.off_wcld = take(L, sizeof(R));
    s.off_frac = take((size_t)2 * L, sizeof(R));
    s.off_csub = take((size_t)n_sub * L, sizeof(R));
  }
  s.off_acc = take((size_t)n_groups * (L + 1) * kNumAcc, sizeof(Acc));
  s.bytes = (o + 15) & ~(size_t)15;
  return s;
}

// Powers used by scale_absorb (scale_absorb.F90:122-224).
template <class R>
__device__ __forceinline__ R scale_factor(int fnc, R p, R t, R p_ref, R t_ref, const double *sp,
                                          int l_doppler, R dop) {
  if constexpr (sizeof(R) == 8) {
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
  } else {
    float off = l_doppler ? (float)dop : 0.0f;
    if (fnc == SOCGPU_IP_SCALE_POWER_LAW) {
      return exp2f((float)sp[0] * __log2f((p + off) / (p_ref + off)) + (float)sp[1] * __log2f(t / t_ref));
    } else if (fnc == SOCGPU_IP_SCALE_POWER_QUAD) {
      float pwk = exp2f((float)sp[0] * __log2f((p + off) / (p_ref + off)));
      float tmp = t / t_ref - 1.0f;
      return pwk * (1.0f + tmp * (float)sp[1] + (float)sp[2] * tmp * tmp);
    } else if (fnc == SOCGPU_IP_SCALE_DOPPLER_QUAD) {
      float pwk = exp2f((float)sp[0] * __log2f((p + (float)sp[1]) / (p_ref + (float)sp[1])));
      float tmp = t / t_ref - 1.0f;
      return pwk * (1.0f + tmp * (float)sp[2] + (float)sp[3] * tmp * tmp);
    }
    return 1.0f;
  }
}

// Band Planck flux (planck_flux_band_mod.F90:33-48), Horner in T/T_ref.
__device__ __forceinline__ double planck_ref(const double *c, int n_deg, double t_ratio) {
  double f = c[n_deg];
  for (int j = n_deg - 1; j >= 0; --j) f = f * t_ratio + c[j];
  return f;
}

// Difference B(t1) - B(t0) of the polynomial without cancellation:
// t1^j - t0^j = (t1 - t0) * sum_{m<j} t1^m t0^(j-1-m), accumulated in FP32.
__device__ __forceinline__ float planck_diff_mix(const double *c, int n_deg, float x1, float x0) {
  float dx = x1 - x0;
  float d = 0.0f;            // d_j = (x1^j - x0^j) / dx
  float p0 = 1.0f;           // x0^(j-1)
  float sum = 0.0f;
  for (int j = 1; j <= n_deg; ++j) {
    d = x1 * d + p0;         // d_j = x1 d_{j-1} + x0^{j-1}
    p0 *= x0;
    sum += (float)c[j] * d;
  }
  return dx * sum;
}

// ---------------------------------------------------------------------------
template <class R, bool MIX, int P, int CH, bool NOSCAT, bool MCICA>
struct FluxKernel {
  using Acc = R;
  static constexpr bool kFP64 = (sizeof(R) == 8);

  // Single scattering + delta rescaling + two-stream coefficients of a cell.
  // kgt/kes/kabs: grey extinction, scattering, absorption; asym/fwd: g' and f.
  __device__ static __forceinline__ void cell_coef(const FluxParams &p, R kgt, R kes, R kabs, R kgas,
                                                   R dm, R asym, R fwd, R sec0,
                                                   R &T, R &Rf, R &T0, R &c1, R &c2, R &omtr) {
    if constexpr (kFP64) {
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
                      : two_coeff_ref(p.isolir, p.i_2stream, p.l_ir_source_quad, asym, om, tau, sec0);
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
        float of = om * fwd;
        float den = 1.0f - of;
        tau = tau * den;
        float inv = 1.0f / den;
        om = om * (1.0f - fwd) * inv;
        omc = omc * inv;                            // 1 - omega' = (1-omega)/(1-omega f)
      }
      CoefF c = NOSCAT ? fast_lw_mix(p.l_ir_source_quad, tau)
                       : two_coeff_mix(p.isolir, p.i_2stream, p.l_ir_source_quad, asym, om, omc, tau, sec0);
      T = c.T; Rf = c.R; T0 = c.T0; c1 = c.c1; c2 = c.c2; omtr = c.omtr;
    }
  }

  __device__ static void run(const FluxParams &p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int col = blockIdx.x;
    const int L = p.n_layer;
    const int nb = p.last_band - p.first_band + 1;
    const int b0 = p.first_band - 1;
    const int nthreads = blockDim.x;
    const int n_groups = nthreads / P;
    const bool lw = (p.isolir == SOCGPU_IP_INFRA_RED);
    const int max_abs = p.max_abs;
    const SmemLayout lay = make_layout<R, Acc>(L, nb, max_abs, MCICA ? p.n_condensed : 0,
                                               MCICA ? p.n_subcol_gen : 0, n_groups, lw, MCICA);
    R *s_p = (R *)(smem + lay.off_p), *s_t = (R *)(smem + lay.off_t), *s_mass = (R *)(smem + lay.off_mass);
    R *s_kgt = (R *)(smem + lay.off_kgt), *s_kes = (R *)(smem + lay.off_kes);
    R *s_kabs = (R *)(smem + lay.off_kabs), *s_asym = (R *)(smem + lay.off_asym);
    R *s_fwd = (R *)(smem + lay.off_fwd), *s_amt = (R *)(smem + lay.off_amt);
    R *s_planck = (R *)(smem + lay.off_planck), *s_dB2 = (R *)(smem + lay.off_dB2);
    R *s_dB = (R *)(smem + lay.off_dB);
    Acc *s_acc = (Acc *)(smem + lay.off_acc);
    const int ndp = p.nd_profile, ndl = p.nd_layer;

    // ---------------- phase 1: stage the column ----------------------------
    for (int i = threadIdx.x; i < L; i += nthreads) {
      s_p[i] = (R)ld2(p.p, col, i, ndp);
      s_t[i] = (R)ld2(p.t, col, i, ndp);
      s_mass[i] = (R)ld2(p.mass, col, i, ndp);
    }
    for (size_t q = threadIdx.x; q < (size_t)n_groups * (L + 1) * kNumAcc; q += nthreads) s_acc[q] = Acc(0);
    __syncthreads();
    for (int q = threadIdx.x; q < nb * L; q += nthreads) {
      const int bi = q / L, i = q - bi * L, b = b0 + bi;
      const BandInfo &bd = p.bands[b];
      // grey optics: grey_opt_prop.F90:470-790 (Rayleigh, modal aerosol),
      // computed in the kernel's working precision R
      R kes = p.l_rayleigh ? (R)bd.rayleigh_coeff : R(0);
      R kabs = R(0), phf = R(0), fwd = R(0);
      if (p.l_aerosol_mode) {
        for (int j = 0; j < p.n_mode; ++j) {
          R mmr = (R)__ldg(p.mode_mix_ratio + (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * j));
          size_t q4 = (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * ((size_t)j + (size_t)p.nd_mode * b));
          R g = (R)__ldg(p.mode_asymmetry + q4);
          kabs = kabs + mmr * (R)__ldg(p.mode_absorption + q4);
          R ks = mmr * (R)__ldg(p.mode_scattering + q4);
          kes = kes + ks;
          phf = phf + ks * g;
          if (p.l_rescale) {
            R ks_phf = ks * g;
            if (p.n_order_forward == 1) fwd = fwd + ks_phf;
            else if (p.n_order_forward == 2) fwd = fwd + ks_phf * g;
            else fwd = fwd + ks * (R)pow((double)g, (double)p.n_order_forward);
          }
        }
      }
      R kgt = kabs + kes;     // grey_opt_prop.F90:773-790
      if (MCICA) {
        R *s_phf_nc = (R *)(smem + lay.off_phf_nc), *s_fwd_nc = (R *)(smem + lay.off_fwd_nc);
        s_phf_nc[q] = phf;
        s_fwd_nc[q] = fwd;
      }
      R asym = phf, f = fwd;
      if ((double)kes > kTiny64) {   // normalisation, grey_opt_prop.F90:840-880
        if (p.l_rescale) { R tinv = R(1) / kes; f = fwd * tinv; asym = phf * tinv; }
        else asym = phf / kes;
      }
      if (p.l_rescale) asym = (asym - f) / (R(1) - f);   // rescale_phase_fnc.F90:120-128
      s_kgt[q] = kgt; s_kes[q] = kes; s_kabs[q] = kabs;
      s_asym[q] = asym; s_fwd[q] = f;
      // gas amounts (radiance_calc.F90:1330-1470)
      const int n_abs_b = p.l_gas ? min(bd.n_abs, max_abs) : 0;
      for (int j = 0; j < n_abs_b; ++j) {
        const BandGas &gs = bd.gas[j];
        R mmr = (R)__ldg(p.gas_mix_ratio + (size_t)col + (size_t)ndp * ((size_t)i + (size_t)ndl * gs.species));
        R amt;
        if (gs.i_scale_k == SOCGPU_IP_SCALE_BAND) {
          R gf = scale_factor<R>(gs.i_scale_fnc, s_p[i] , s_t[i], (R)gs.p_ref, (R)gs.t_ref, gs.scale,
                                 gs.l_doppler, (R)gs.doppler_cor);
          R v = gf * mmr;
          amt = v > R(0) ? v : R(0);
        } else {
          amt = mmr;   // ip_scale_null, or ip_scale_term (scaled per term below)
        }
        s_amt[((size_t)bi * max_abs + j) * L + i] = amt;
      }
    }
    if (lw) {
      // diff_planck_source (diff_planck_source_mod.F90:102-136)
      for (int q = threadIdx.x; q < nb * (L + 1); q += nthreads) {
        const int bi = q / (L + 1), i = q - bi * (L + 1);
        const double *c = p.bands[b0 + bi].planck;
        if constexpr (kFP64) {
          s_planck[q] = planck_ref(c, p.n_deg_fit, ld2(p.t_level, col, i, ndp) / p.t_ref_planck);
        } else {
          float x = (float)(ld2(p.t_level, col, i, ndp) / p.t_ref_planck);
          float f = (float)c[p.n_deg_fit];
          for (int j = p.n_deg_fit - 1; j >= 0; --j) f = f * x + (float)c[j];
          s_planck[q] = f;
        }
      }
      for (int q = threadIdx.x; q < nb * L; q += nthreads) {
        const int bi = q / L, i = q - bi * L;
        const double *c = p.bands[b0 + bi].planck;
        if constexpr (kFP64) {
          double b1 = planck_ref(c, p.n_deg_fit, ld2(p.t_level, col, i + 1, ndp) / p.t_ref_planck);
          double bm = planck_ref(c, p.n_deg_fit, ld2(p.t_level, col, i, ndp) / p.t_ref_planck);
          s_dB[q] = b1 - bm;
          if (p.l_ir_source_quad) {
            double bl = planck_ref(c, p.n_deg_fit, ld2(p.t, col, i, ndp) / p.t_ref_planck);
            s_dB2[q] = 2.0 * (b1 + bm - 2.0 * bl);
          }
        } else {
          // differences of the polynomial without cancellation
          float x1 = (float)(ld2(p.t_level, col, i + 1, ndp) / p.t_ref_planck);
          float x0 = (float)(ld2(p.t_level, col, i, ndp) / p.t_ref_planck);
          s_dB[q] = planck_diff_mix(c, p.n_deg_fit, x1, x0);
          if (p.l_ir_source_quad) {
            float xl = (float)(ld2(p.t, col, i, ndp) / p.t_ref_planck);
            s_dB2[q] = 2.0f * (planck_diff_mix(c, p.n_deg_fit, x1, xl) + planck_diff_mix(c, p.n_deg_fit, x0, xl));
          }
        }
      }
    }
    if (MCICA) stage_clouds(p, lay, smem, col, nb, b0);
    __syncthreads();

    // ---------------- phase 2: g-point solves ---------------------------------
    const int gid = threadIdx.x / P;
    const int r = threadIdx.x % P;
    const R sec0 = p.zen_0 ? (R)ld2(p.zen_0, col, 0, ndp) : R(1);
    Acc *acc = s_acc + (size_t)gid * (L + 1) * kNumAcc;
    // Every group of every warp runs the same number of rounds so that the
    // full-warp shuffles of the scans always see all 32 lanes; a group with
    // no g-point left in the last round solves g_begin and discards it.
    const int rounds = (p.g_end - p.g_begin + n_groups - 1) / n_groups;
    for (int rd = 0; rd < rounds; ++rd) {
      int g = p.g_begin + rd * n_groups + gid;
      const bool active = g < p.g_end;
      if (!active) g = p.g_begin;
      solve_gpoint(p, lay, smem, col, g, b0, max_abs, sec0, r, acc, lw, active);
    }
    __syncthreads();

    // ---------------- phase 3: reduce over groups, write ------------------------
    for (int lev = threadIdx.x; lev <= L; lev += nthreads) {
      Acc up = Acc(0), dn = Acc(0), dir = Acc(0), dv = Acc(0);
      for (int q = 0; q < n_groups; ++q) {
        const Acc *a = s_acc + ((size_t)q * (L + 1) + lev) * kNumAcc;
        up += a[0]; dn += a[1]; dir += a[2]; dv += a[3];
      }
      if (lw) {    // adjust_ir_radiance.F90:75-95
        for (int bi = 0; bi < nb; ++bi) {
          Acc wb = p.weight_band ? (Acc)p.weight_band[b0 + bi] : Acc(1);
          Acc bw = s_planck[bi * (L + 1) + lev] * wb;
          up += bw; dn += bw;
        }
      }
      size_t o = (size_t)col + (size_t)ndp * lev;
      p.flux_up[o] = (double)up;
      p.flux_down[o] = (double)dn;
      if (p.flux_direct) p.flux_direct[o] = lw ? 0.0 : (double)dir;
      if (lev < L && p.flux_div) p.flux_div[(size_t)col + (size_t)ndp * lev] = (double)dv;
    }
    if (p.heating_rate) {
      __syncthreads();
      for (int i = threadIdx.x; i < L; i += nthreads) {
        double hc = ld2(p.mass, col, i, ndp) * 1.005e3;
        double hr;
        if (p.l_flux_div && p.flux_div) {
          hr = 8.64e4 * p.flux_div[(size_t)col + (size_t)ndp * i] / hc;
        } else {
          double fn0 = p.flux_down[(size_t)col + (size_t)ndp * i] - p.flux_up[(size_t)col + (size_t)ndp * i];
          double fn1 = p.flux_down[(size_t)col + (size_t)ndp * (i + 1)] - p.flux_up[(size_t)col + (size_t)ndp * (i + 1)];
          hr = 8.64e4 * ((fn0 - fn1) / hc);
        }
        p.heating_rate[(size_t)col + (size_t)ndp * i] = hr;
      }
    }
  }

  // Cloud-component optics of every (band, layer) of the column through
  // opt_prop_pade_2 (opt_prop_pade_2_mod.F90:99-140), plus the column's
  // cloud fractions and subcolumn scalings.
  __device__ static void stage_clouds(const FluxParams &p, const SmemLayout &lay, unsigned char *smem,
                                      int col, int nb, int b0) {
    const int L = p.n_layer, ndp = p.nd_profile, ndl = p.nd_layer, ict = p.id_ct;
    const int ndc = ndl - ict, nc = p.n_condensed;
    R *ke = (R *)(smem + lay.off_c_ke), *ks = (R *)(smem + lay.off_c_ks), *ka = (R *)(smem + lay.off_c_ka);
    R *ph = (R *)(smem + lay.off_c_phf), *fw = (R *)(smem + lay.off_c_fwd);
    R *wc = (R *)(smem + lay.off_wcld), *fr = (R *)(smem + lay.off_frac), *cs = (R *)(smem + lay.off_csub);
    for (int q = threadIdx.x; q < nb * nc * L; q += blockDim.x) {
      const int i = q % L, k = (q / L) % nc, bi = q / (L * nc);
      double vke = 0.0, vks = 0.0, vka = 0.0, vph = 0.0, vfw = 0.0;
      if (i >= ict) {
        size_t qc = (size_t)col + (size_t)ndp * (size_t)(i - ict);
        double w = __ldg(p.w_cloud + qc);
        if (w > 0.0) {
          const double *cp = (p.comp_phase[k] == SOCGPU_IP_PHASE_WATER ? p.drop_parm : p.ice_parm)
                             + ((size_t)p.comp_parm_index[k] * p.n_band + (b0 + bi)) * kPadeParm;
          double qm = __ldg(p.condensed_mix_ratio + qc + (size_t)ndp * ndc * k);
          double re = __ldg(p.condensed_dim_char + qc + (size_t)ndp * ndc * k);
          double kext = qm * (cp[0] + re * (cp[1] + re * cp[2]))
                        / (1.0e+00 + re * (cp[3] + re * (cp[4] + re * cp[5])));
          double coalb = (cp[6] + re * (cp[7] + re * cp[8])) / (1.0e+00 + re * (cp[9] + re * cp[10]));
          double kscat = kext * (1.0e+00 - coalb);
          double g = (cp[11] + re * (cp[12] + re * cp[13])) / (1.0e+00 + re * (cp[14] + re * cp[15]));
          vke = kext; vks = kscat; vka = kext * coalb; vph = kscat * g; vfw = kscat * g * g;
        }
      }
      ke[q] = (R)vke; ks[q] = (R)vks; ka[q] = (R)vka; ph[q] = (R)vph; fw[q] = (R)vfw;
    }
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      double w = 0.0, f1 = 0.0, f2 = 0.0;
      if (i >= ict) {
        size_t qc = (size_t)col + (size_t)ndp * (size_t)(i - ict);
        w = __ldg(p.w_cloud + qc);
        f1 = __ldg(p.frac_cloud + qc);
        if (p.n_cloud_type > 1) f2 = __ldg(p.frac_cloud + qc + (size_t)ndp * ndc);
      }
      wc[i] = (R)w; fr[i] = (R)f1; fr[L + i] = (R)f2;
    }
    for (int q = threadIdx.x; q < p.n_subcol_gen * L; q += blockDim.x) {
      const int i = q % L, s = q / L;
      double v = 0.0;
      if (i >= ict) v = __ldg(p.c_sub + (size_t)col + (size_t)ndp * ((size_t)(i - ict) + (size_t)ndc * s));
      cs[q] = (R)v;
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

  // Gas absorption of a g-point at layer i (gas_optical_properties.F90:80-95).
  __device__ static __forceinline__ R gas_k(const GasTerm &gt, const GPoint &gp, const BandInfo &bd,
                                            const R *amt, int L, int i, R pl, R tl) {
    R kg = R(0);
    if (!gt.any_term) {
#pragma unroll
      for (int j = 0; j < kMaxAbsPerBand; ++j)
        if (j < gt.n_abs) {
          R kal = gt.k[j] * amt[(size_t)j * L + i];
          kg = (j == 0) ? kal : kg + kal;
        }
      return kg;
    }
    for (int j = 0; j < gt.n_abs; ++j) {
      R a = amt[(size_t)j * L + i];
      R kal;
      if (bd.gas[j].i_scale_k == SOCGPU_IP_SCALE_TERM) {
        R gf = scale_factor<R>(bd.gas[j].i_scale_fnc, pl, tl, (R)bd.gas[j].p_ref, (R)bd.gas[j].t_ref,
                               gp.term_scale[j], bd.gas[j].l_doppler, (R)bd.gas[j].doppler_cor);
        R v = gf * a;
        kal = gt.k[j] * (v > R(0) ? v : R(0));
      } else {
        kal = gt.k[j] * a;
      }
      kg = (j == 0) ? kal : kg + kal;
    }
    return kg;
  }

  // One g-point of one column (all its subcolumns under McICA).
  __device__ static void solve_gpoint(const FluxParams &p, const SmemLayout &lay, unsigned char *smem,
                                      int col, int g, int b0, int max_abs, R sec0, int r, Acc *acc,
                                      bool lw, bool active) {
    const int L = p.n_layer, ndp = p.nd_profile;
    const GPoint &gp = p.gpoints[g];
    const int b = gp.band, bi = b - b0;
    const BandInfo &bd = p.bands[b];
    const double wb = p.weight_band ? p.weight_band[b] : 1.0;
    const R w_g = (R)(wb * gp.weight);
    const GasTerm gt = load_gas(gp, bd, max_abs);
    const R *s_p = (const R *)(smem + lay.off_p), *s_t = (const R *)(smem + lay.off_t);
    const R *s_mass = (const R *)(smem + lay.off_mass);
    const R *kgt_b = (const R *)(smem + lay.off_kgt) + (size_t)bi * L;
    const R *kes_b = (const R *)(smem + lay.off_kes) + (size_t)bi * L;
    const R *kabs_b = (const R *)(smem + lay.off_kabs) + (size_t)bi * L;
    const R *asym_b = (const R *)(smem + lay.off_asym) + (size_t)bi * L;
    const R *fwd_b = (const R *)(smem + lay.off_fwd) + (size_t)bi * L;
    const R *amt_b = (const R *)(smem + lay.off_amt) + (size_t)bi * max_abs * L;
    const R *planck_b = (const R *)(smem + lay.off_planck) + (size_t)bi * (L + 1);
    const R *dB2_b = (const R *)(smem + lay.off_dB2) + (size_t)bi * L;
    const R *dB_b = (const R *)(smem + lay.off_dB) + (size_t)bi * L;

    // boundary conditions (solve_band_random_overlap.F90:565-600, column_solver.F90)
    R f_inc_down, f_inc_dir, alb_diff, alb_dir, dB_surf = R(0);
    alb_diff = (R)__ldg(p.rho_alb + (size_t)col + (size_t)ndp * (0 + 2 * (size_t)b));
    alb_dir = (R)__ldg(p.rho_alb + (size_t)col + (size_t)ndp * (1 + 2 * (size_t)b));
    if (lw) {
      f_inc_dir = R(0);
      f_inc_down = -planck_b[0];
      double bg = planck_ref(bd.planck, p.n_deg_fit, ld2(p.t_ground, col, 0, ndp) / p.t_ref_planck);
      if constexpr (kFP64) dB_surf = bg - planck_b[L];
      else dB_surf = (R)planck_diff_mix(bd.planck, p.n_deg_fit,
                                        (float)(ld2(p.t_ground, col, 0, ndp) / p.t_ref_planck),
                                        (float)(ld2(p.t_level, col, L, ndp) / p.t_ref_planck));
    } else {
      double sib = ld2(p.solar_irrad, col, 0, ndp) * bd.solar_flux_band;
      f_inc_down = (R)(sib / (double)sec0);
      f_inc_dir = f_inc_down;
    }

    if (!MCICA) {
      R T[CH], Rf[CH], T0[CH], c1[CH], c2[CH], om[CH];
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j;
        if (i < L) {
          R kg = p.l_gas ? gas_k(gt, gp, bd, amt_b, L, i, s_p[i], s_t[i]) : R(0);
          cell_coef(p, kgt_b[i], kes_b[i], kabs_b[i], kg, s_mass[i], asym_b[i], fwd_b[i], sec0,
                    T[j], Rf[j], T0[j], c1[j], c2[j], om[j]);
        } else {
          T[j] = R(1); Rf[j] = R(0); T0[j] = R(1); c1[j] = R(0); c2[j] = R(0); om[j] = R(0);
        }
      }
      solve_column(p, T, Rf, T0, c1, c2, om, r, L, lw, dB_b, dB2_b, f_inc_down, f_inc_dir,
                   alb_diff, alb_dir, dB_surf, w_g, acc, active);
    } else {
      solve_mcica(p, lay, smem, col, gp, gt, bd, bi, b, r, L, lw, sec0, dB_b, dB2_b, f_inc_down, f_inc_dir,
                  alb_diff, alb_dir, dB_surf, w_g, acc, max_abs, active);
    }
  }

  __device__ static void solve_mcica(const FluxParams &p, const SmemLayout &lay, unsigned char *smem,
                                     int col, const GPoint &gp, const GasTerm &gt, const BandInfo &bd,
                                     int bi, int b, int r,
                                     int L, bool lw, R sec0, const R *dB_b, const R *dB2_b,
                                     R f_inc_down, R f_inc_dir, R alb_diff, R alb_dir, R dB_surf,
                                     R w_g, Acc *acc, int max_abs, bool active) {
    const int ndp = p.nd_profile, nc = p.n_condensed;
    const R *s_p = (const R *)(smem + lay.off_p), *s_t = (const R *)(smem + lay.off_t);
    const R *s_mass = (const R *)(smem + lay.off_mass);
    const R *kgt_b = (const R *)(smem + lay.off_kgt) + (size_t)bi * L;
    const R *kes_b = (const R *)(smem + lay.off_kes) + (size_t)bi * L;
    const R *kabs_b = (const R *)(smem + lay.off_kabs) + (size_t)bi * L;
    const R *asym_b = (const R *)(smem + lay.off_asym) + (size_t)bi * L;
    const R *fwd_b = (const R *)(smem + lay.off_fwd) + (size_t)bi * L;
    const R *amt_b = (const R *)(smem + lay.off_amt) + (size_t)bi * max_abs * L;
    const R *phf_nc = (const R *)(smem + lay.off_phf_nc) + (size_t)bi * L;
    const R *fwd_nc = (const R *)(smem + lay.off_fwd_nc) + (size_t)bi * L;
    const R *c_ke = (const R *)(smem + lay.off_c_ke) + (size_t)bi * nc * L;
    const R *c_ks = (const R *)(smem + lay.off_c_ks) + (size_t)bi * nc * L;
    const R *c_ka = (const R *)(smem + lay.off_c_ka) + (size_t)bi * nc * L;
    const R *c_ph = (const R *)(smem + lay.off_c_phf) + (size_t)bi * nc * L;
    const R *c_fw = (const R *)(smem + lay.off_c_fwd) + (size_t)bi * nc * L;
    const R *wc = (const R *)(smem + lay.off_wcld), *fr = (const R *)(smem + lay.off_frac);
    const R *cs = (const R *)(smem + lay.off_csub);

    const int iex = gp.iex_major;
    const int first = __ldg(p.first_subcol_k + b + (size_t)p.nd_band_sp * iex);
    const int last = __ldg(p.first_subcol_k + b + (size_t)p.nd_band_sp * (iex + 1)) - 1;
    const int nsub = __ldg(p.subcol_k + b + (size_t)p.nd_band_sp * iex);
    const R fcl = (R)ld2(p.frac_cloudy, col, 0, ndp);
    const int ncld = p.n_subcol_cld ? __ldg(p.n_subcol_cld + col) : 0;
    const int nfill = min(p.n_subcol_req, p.n_subcol_gen);
    // blending weights (mcica_sample.F90:862-925)
    const R w_sub = w_g * fcl / (R)nsub;
    const R w_clr = w_g * (R(1) - fcl);

    // Solve index it = 0 is the clear solve, it = 1.. the subcolumns
    // first..last.  The count is made uniform over the warp (all groups
    // take part in every shuffle); surplus iterations are discarded.
    const int n_iter = last - first + 2;
    const int n_iter_warp = __reduce_max_sync(0xffffffffu, n_iter);
    for (int it = 0; it < n_iter_warp; ++it) {
      const bool clear = (it == 0);
      const int m = first + it - 1;
      bool use = active && it < n_iter && (clear ? (w_clr != R(0)) : (w_sub != R(0)));
      int slot = -1;
      if (!clear) {
        int idx = (it < n_iter ? m : first) % p.n_subcol_req;
        if (idx == 0) idx = p.n_subcol_req;
        int j = __ldg(p.subcol_reorder + (idx - 1));
        if (p.n_subcol_cld && ncld > 0 && j > ncld && j <= nfill) j = (j - 1) % ncld + 1;
        slot = j - 1;
        if (slot < 0 || slot >= p.n_subcol_gen) {   // out-of-range table entry: report, solve clear
          if (p.error_flag) atomicOr(p.error_flag, 1);
          slot = -1;
          use = false;
        }
      }
      R T[CH], Rf[CH], T0[CH], c1[CH], c2[CH], om[CH];
#pragma unroll
      for (int jj = 0; jj < CH; ++jj) {
        const int i = r * CH + jj;
        if (i < L) {
          R kg = p.l_gas ? gas_k(gt, gp, bd, amt_b, L, i, s_p[i], s_t[i]) : R(0);
          R cs_i = (slot >= 0) ? cs[(size_t)slot * L + i] : R(0);
          bool cloudy = false;
          if (slot >= 0 && wc[i] > R(0)) {
            for (int t = 0; t < p.n_cloud_type; ++t) cloudy |= (cs_i * fr[(size_t)t * L + i] > R(0));
          }
          if (!cloudy) {
            cell_coef(p, kgt_b[i], kes_b[i], kabs_b[i], kg, s_mass[i], asym_b[i], fwd_b[i], sec0,
                      T[jj], Rf[jj], T0[jj], c1[jj], c2[jj], om[jj]);
          } else {
            // mcica_sample.F90:472-560 then mcica_column.F90:336-470
            R sT = R(0), sR = R(0), sT0 = R(0), s1 = R(0), s2 = R(0), sO = R(0);
            for (int k = 0; k < nc; ++k) {
              const int t = p.comp_type[k] - 1;
              const R fc = fr[(size_t)t * L + i];
              if (!(cs_i * fc > R(0))) continue;
              const size_t qk = (size_t)k * L + i;
              R kgt = kgt_b[i] + c_ke[qk] * cs_i;
              R kes = kes_b[i] + c_ks[qk] * cs_i;
              R kab = kabs_b[i] + c_ka[qk] * cs_i;
              R asym, fwd;
              const R eps = kFP64 ? (R)kEps64 : (R)kEps64;
              if (p.l_rescale) {
                R fw = fwd_nc[i] + c_fw[qk] * cs_i;
                R den = kes - fw;
                asym = (phf_nc[i] + c_ph[qk] * cs_i - fw) / (den > eps ? den : eps);
                fwd = fw / (kes > eps ? kes : eps);
              } else {
                asym = (phf_nc[i] + c_ph[qk] * cs_i) / (kes > eps ? kes : eps);
                fwd = R(0);
              }
              R tT, tR, tT0, t1, t2, tO;
              cell_coef(p, kgt, kes, kab, kg, s_mass[i], asym, fwd, sec0, tT, tR, tT0, t1, t2, tO);
              sT = sT + fc * tT; sR = sR + fc * tR; sT0 = sT0 + fc * tT0;
              s1 = s1 + fc * t1; s2 = s2 + fc * t2; sO = sO + fc * tO;
            }
            T[jj] = sT; Rf[jj] = sR; T0[jj] = lw ? R(1) : sT0; c1[jj] = s1; c2[jj] = s2; om[jj] = sO;
          }
        } else {
          T[jj] = R(1); Rf[jj] = R(0); T0[jj] = R(1); c1[jj] = R(0); c2[jj] = R(0); om[jj] = R(0);
        }
      }
      solve_column(p, T, Rf, T0, c1, c2, om, r, L, lw, dB_b, dB2_b, f_inc_down, f_inc_dir,
                   alb_diff, alb_dir, dB_surf, clear ? w_clr : w_sub, acc, use);
    }
  }

  // Sources, direct beam, solve and accumulation of one monochromatic
  // problem held in the group's registers.
  __device__ static void solve_column(const FluxParams &p, R (&T)[CH], R (&Rf)[CH], R (&T0)[CH],
                                      R (&c1)[CH], R (&c2)[CH], R (&om)[CH], int r, int L, bool lw,
                                      const R *dB_b, const R *dB2_b, R f_inc_down, R f_inc_dir,
                                      R alb_diff, R alb_dir, R dB_surf, R w, Acc *acc, bool active) {
    // the last level a lane accumulates into: none when the solve is discarded
    const int L_acc = active ? L : -1;
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
      if (r == 0 && active) acc[0 * kNumAcc + 2] += w * fd;
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j;
        R su = c1[j] * fd, sd = c2[j] * fd;   // solar_source.F90:146-155
        c1[j] = su; c2[j] = sd;
        ssum[j] = su + sd;
        fd = fd * T0[j];
        if (i < L_acc) acc[(size_t)(i + 1) * kNumAcc + 2] += w * fd;
      }
    } else {
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j;
        if (i < L) {
          R dB = dB_b[i];
          R su, sd;
          if (p.l_ir_source_quad) {       // ir_source.F90:93-119
            su = c1[j] * dB + c2[j] * dB2_b[i];
            sd = -c1[j] * dB + c2[j] * dB2_b[i];
            ssum[j] = R(2) * c2[j] * dB2_b[i];
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
      if (r == 0 && active) { acc[0] += w * fu; acc[1] += w * fd; }
      R fu_prev = fu;
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int i = r * CH + j;
        R fdn = c2[j] + T[j] * fd;
        if (i < L_acc) {
          acc[(size_t)(i + 1) * kNumAcc + 0] += w * c1[j];
          acc[(size_t)(i + 1) * kNumAcc + 1] += w * fdn;
          if constexpr (kFP64) acc[(size_t)i * kNumAcc + 3] += w * (c1[j] - fu_prev + fd - fdn);
          else acc[(size_t)i * kNumAcc + 3] += w * (om[j] * (fd + c1[j]) - ssum[j]);
        }
        fu_prev = c1[j];
        fd = fdn;
      }
      return;
    }

    // --- adding-method solve as a scan of composites ---------------------------
    Comp<R> cc = comp_identity<R>();
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      Comp<R> lj; lj.R1 = Rf[j]; lj.R2 = Rf[j]; lj.Td = T[j]; lj.Tu = T[j]; lj.Su = c1[j]; lj.Sd = c2[j];
      cc = (j == 0) ? lj : stack(cc, lj);
    }
    // above: inclusive prefix C_0 .. C_r
    Comp<R> pre = cc;
#pragma unroll
    for (int d = 1; d < P; d <<= 1) {
      Comp<R> y = shfl_up_comp(pre, d, P);
      if (r >= d) pre = stack(y, pre);
    }
    Comp<R> ex = shfl_up_comp(pre, 1, P);
    // state above this chunk: rho (reflection back down), sigma (downward flux source)
    R rho, sigma;
    if (r == 0) { rho = R(0); sigma = f_inc_down; }
    else { rho = ex.R2; sigma = ex.Sd + ex.Td * f_inc_down; }
    // below: inclusive suffix C_r .. C_{P-1}
    Comp<R> suf = cc;
#pragma unroll
    for (int d = 1; d < P; d <<= 1) {
      Comp<R> y = shfl_down_comp(suf, d, P);
      if (r + d < P) suf = stack(suf, y);
    }
    Comp<R> bx = shfl_down_comp(suf, 1, P);
    R alpha, S;     // albedo and upward source at the bottom of this chunk
    if (r == P - 1) { alpha = alb_diff; S = src_ground; }
    else {
      R D = R(1) / (R(1) - bx.R2 * alb_diff);
      alpha = bx.R1 + bx.Tu * alb_diff * D * bx.Td;
      S = bx.Su + bx.Tu * D * (src_ground + alb_diff * bx.Sd);
    }
    // elimination inside the chunk (solver_homogen_direct.F90:94-110);
    // beta, gamma, h overwrite T0, c1 and a copy kept in Rf-sized arrays.
    R (&beta)[CH] = T0;   // the direct transmission is no longer needed
    R gam[CH];
#pragma unroll
    for (int j = CH - 1; j >= 0; --j) {
      R bt = R(1) / (R(1) - alpha * Rf[j]);
      R gm = alpha * T[j];
      R h = S + alpha * c2[j];
      alpha = Rf[j] + bt * gm * T[j];
      S = c1[j] + bt * T[j] * h;
      beta[j] = bt; gam[j] = gm; c1[j] = h;
    }
    // fluxes at the chunk top, then back-substitution (solver_homogen_direct.F90:112-128)
    R fdn = (sigma + rho * S) / (R(1) - rho * alpha);
    R fup = alpha * fdn + S;
    if (r == 0) {
      fdn = f_inc_down; fup = alpha * fdn + S;
      if (active) { acc[0] += w * fup; acc[1] += w * fdn; }
    }
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int i = r * CH + j;
      R fu = beta[j] * (c1[j] + gam[j] * fdn);
      R fd = c2[j] + T[j] * fdn + Rf[j] * fu;
      if (i < L_acc) {
        acc[(size_t)(i + 1) * kNumAcc + 0] += w * fu;
        acc[(size_t)(i + 1) * kNumAcc + 1] += w * fd;
        if constexpr (kFP64) acc[(size_t)i * kNumAcc + 3] += w * (fu - fup + fdn - fd);
        else acc[(size_t)i * kNumAcc + 3] += w * (om[j] * (fdn + fu) - ssum[j]);
      }
      fup = fu; fdn = fd;
    }
  }
};

template <class R, bool MIX, int P, int CH, bool NOSCAT, bool MCICA>
__global__ void __launch_bounds__(256) flux_kernel(const __grid_constant__ FluxParams p) {
  FluxKernel<R, MIX, P, CH, NOSCAT, MCICA>::run(p);
}

}  // namespace socgpu
