// twostream_math.cuh -- per-cell two-stream physics for the device kernels.
//
// Two flavours of every formula:
//   * Ref  (double): the reference's FP64 expressions in the reference's
//     operation order, so the FP64 device path agrees with the reference to
//     rounding (two_coeff_basic.F90:99-160, two_coeff.F90:148-188,
//     solar_coefficient_basic.F90:124-219, trans_source_coeff.F90:144-263,
//     two_coeff_fast_lw.F90:112-154, single_scattering.F90:119-164,
//     rescale_tau_omega.F90:73-80).
//   * Mix  (float): the same quantities rearranged so that no step cancels
//     catastrophically in FP32 -- 1-omega carried from the absorption
//     coefficient, 1-gamma = 2 lambda/(sum+lambda), 1-exp via expm1, and
//     (1-T), (1-T-R) in factored form -- with the FP64 clamps of the
//     reference kept as constants.  Next to the solar singularity
//     lambda = sec_0 the coefficients are interpolated across it.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/socgpu.h"

namespace socgpu {

// EPSILON/TINY of the reference's working precision (FP64).
constexpr double kEps64 = 2.220446049250313e-16;
constexpr double kTiny64 = 2.2250738585072014e-308;
constexpr double kSqEps64 = 1.4901161193847656e-08;      // SQRT(EPSILON(1.0_RealK))
constexpr double kTolQuad64 = 1.220703125e-04;            // SQRT(SQRT(EPSILON))
constexpr double kElsasser = 1.66;                        // diffusivity_factor.F90:16
constexpr double kRoot3 = 1.7320508075688772;             // two_coeff_basic.F90:87

struct Coef {
  // trans, reflect, direct transmission, two source coefficients
  // (solar: up/down per unit direct flux at the layer top;
  //  IR: 1d/2d of ir_source)
  double T, R, T0, c1, c2;
};
struct CoefF {
  float T, R, T0, c1, c2;
  float omtr;          // 1 - T - R, formed without cancellation
};

// ---- scheme coefficients (two_coeff_basic.F90:99-160) --------------------
__device__ __forceinline__ void sum_diff_ref(int scheme, double om, double g, double &sum, double &diff) {
  switch (scheme) {
    case SOCGPU_IP_EDDINGTON: sum = 1.5 * (1.0 - om * g); diff = 2.0 * (1.0 - om); break;
    case SOCGPU_IP_ELSASSER: sum = kElsasser - 1.5 * om * g; diff = kElsasser * (1.0 - om); break;
    case SOCGPU_IP_DISCRETE_ORD: sum = kRoot3 * (1.0 - om * g); diff = kRoot3 * (1.0 - om); break;
    case SOCGPU_IP_PIFM85: sum = 2.0 - 1.5 * om * g; diff = 2.0 * (1.0 - om); break;
    case SOCGPU_IP_2S_TEST: sum = 1.5 - 1.5 * om * g; diff = 1.5 * (1.0 - om); break;
    case SOCGPU_IP_HEMI_MEAN: sum = 2.0 * (1.0 - om * g); diff = 2.0 * (1.0 - om); break;
    default: /* ip_pifm80 */ sum = 2.0 - 1.5 * om * g - 0.5 * om; diff = 2.0 * (1.0 - om); break;
  }
}

// ---- full two-stream coefficients, reference form -------------------------
__device__ __forceinline__ Coef two_coeff_ref(int isolir, int scheme, int l_quad,
                                              double g, double om, double tau, double sec0) {
  Coef c;
  double sum, diff;
  sum_diff_ref(scheme, om, g, sum, diff);
  double lambda = sqrt(sum * diff);
  double gam_up = 0.0, gam_dn = 0.0;
  if (isolir == SOCGPU_IP_SOLAR) {
    const double tol_perturb = 3.2e1 * kEps64;
    if (fabs(lambda - sec0) < tol_perturb) {
      sum = (1.0 + tol_perturb) * sum;
      diff = (1.0 + tol_perturb) * diff;
      lambda = (1.0 + tol_perturb) * lambda;
    }
    double ksi0 = (scheme == SOCGPU_IP_DISCRETE_ORD) ? kRoot3 * g / sec0 : 1.5 * g / sec0;
    double factor = 0.5 * om * sec0 / ((lambda - sec0) * (lambda + sec0));
    gam_up = factor * (sum - sec0 - ksi0 * (diff - sec0));
    gam_dn = factor * (sum + sec0 + ksi0 * (diff + sec0));
  }
  double e = exp(-lambda * tau);
  double e2 = e * e;
  double gamma = (sum - lambda) / (sum + lambda);
  double gamma2 = gamma * gamma;
  double tmp_inv = 1.0 / (1.0 - e2 * gamma2);
  c.T = e * (1.0 - gamma2) * tmp_inv;
  c.R = gamma * (1.0 - e2) * tmp_inv;
  c.T0 = 1.0;
  c.c2 = 0.0;
  if (isolir == SOCGPU_IP_SOLAR) {
    c.T0 = exp(-tau * sec0);
    c.c1 = (gam_up - c.R * (1.0 + gam_dn)) - gam_up * c.T * c.T0;
    c.c2 = c.T0 * (1.0 + gam_dn - gam_up * c.R) - (1.0 + gam_dn) * c.T;
  } else {
    c.c1 = (1.0 - c.T + c.R + kSqEps64) / (kSqEps64 + tau * sum);
    if (l_quad) {
      double s2;
      if (tau > kTolQuad64) s2 = -2.0 * (1.0 - c.T - c.R + kSqEps64) / (diff * tau + kSqEps64);
      else s2 = -2.0 + diff * tau;
      c.c2 = -(1.0 + c.R + c.T + s2) / (sum * tau + kSqEps64);
    }
  }
  return c;
}

// two_coeff_fast_lw, reference form.
__device__ __forceinline__ Coef fast_lw_ref(int l_quad, double tau) {
  Coef c;
  c.T = exp(-1.66 * tau);
  c.R = 0.0; c.T0 = 1.0; c.c2 = 0.0;
  c.c1 = (1.0 - c.T + kSqEps64) / (1.66 * tau + kSqEps64);
  if (l_quad) {
    if (tau > kTolQuad64) c.c2 = -(1.0 + c.T - 2.0 * c.c1) / (1.66 * tau + kSqEps64);
    else c.c2 = -(1.0 + c.T - 2.0 + 1.66 * tau) / (1.66 * tau + kSqEps64);
  }
  return c;
}

// ---- mixed-precision forms -------------------------------------------------
// Scheme constants of the mixed kernels (two_coeff_basic.F90:99-160,
// solar_coefficient_basic.F90:171-182): sum = A - omega (B g + C),
// diff = D (1 - omega), ksi_0 = K g / sec_0.  The host fills them once per
// call (FluxParams::scheme_f), so the per-cell code has no switch.
struct SchemeF { float A, B, C, D, K; };

// 1 - exp(-x) given e = exp(-x): below x = 0.25 the Taylor series to x^6
// (relative truncation error under 5e-8), above it 1 - e (which then loses
// at most a factor 1/0.22 of FP32 rounding).  Branch-free.
__device__ __forceinline__ float one_minus_exp(float x, float e) {
  const float p = x * fmaf(x, fmaf(x, fmaf(x, fmaf(x, fmaf(x, -1.0f / 720.0f, 1.0f / 120.0f), -1.0f / 24.0f),
                                             1.0f / 6.0f), -0.5f), 1.0f);
  return x < 0.25f ? p : 1.0f - e;
}
// phi(x) = x - (1 - exp(-x)) = x^2/2 - x^3/6 + ...
__device__ __forceinline__ float phi_exp(float x, float em1) {
  if (x < 0.25f)
    return x * x * 0.5f * (1.0f - x * (1.0f / 3.0f) * (1.0f - x * 0.25f * (1.0f - x * 0.2f *
           (1.0f - x * (1.0f / 6.0f) * (1.0f - x * (1.0f / 7.0f))))));
  return x - em1;
}
// psi(x) = exp(-x) (1 + x) - 1 = -x^2/2 + x^3/3 - x^4/8 + x^5/30 - x^6/144 + x^7/840 - ...
__device__ __forceinline__ float psi_exp(float x, float e) {
  if (x < 0.25f)
    return -x * x * (0.5f - x * ((1.0f / 3.0f) - x * (0.125f - x * ((1.0f / 30.0f) - x * ((1.0f / 144.0f) -
           x * (1.0f / 840.0f))))));
  return e * (1.0f + x) - 1.0f;
}

// Relative distance of lambda from sec_0 inside which the solar
// coefficients are interpolated across the removable singularity.
constexpr float kSolarSingularTol = 3.0e-3f;

// Reflection and transmission of a homogeneous layer (trans_source_coeff.F90:
// 144-200) regrouped around 1 - e, 1 - gamma = 2 lambda/(sum + lambda) and
// 1 - e gamma = (1 - e) + e (1 - gamma), so that none cancels; with 1 - T and
// 1 - T - R in factored form.
struct LayerF { float x, e, em1, gamma, omg, eg, T, R, omt, omtr; };
__device__ __forceinline__ LayerF layer_mix(float sum, float lambda, float tau) {
  LayerF l;
  l.x = lambda * tau;
  l.e = __expf(-l.x);
  l.em1 = one_minus_exp(l.x, l.e);
  const float inv_sl = 1.0f / (sum + lambda);
  l.gamma = (sum - lambda) * inv_sl;
  l.omg = 2.0f * lambda * inv_sl;
  l.eg = l.e * l.gamma;
  const float u = fmaf(l.e, l.omg, l.em1);                  // 1 - e gamma
  const float inv_den = 1.0f / (u * (1.0f + l.eg));          // 1 / (1 - e^2 gamma^2)
  l.T = l.e * l.omg * (1.0f + l.gamma) * inv_den;
  l.R = l.gamma * l.em1 * (1.0f + l.e) * inv_den;
  l.omt = l.em1 * fmaf(l.eg, l.gamma, 1.0f) * inv_den;       // 1 - T
  l.omtr = l.em1 * l.omg * u * inv_den;                      // 1 - T - R = em1 (1 - gamma) / (1 + e gamma)
  return l;
}

// Solar source coefficients (solar_coefficient_basic.F90:124-219,
// trans_source_coeff.F90:144-263): c1 = gam_up - R(1+gam_dn) - gam_up T T0
// and c2 = T0(1+gam_dn-gam_up R) - (1+gam_dn) T, regrouped with
// 1 - T T0 = (1-T0) + T0 (1-T) and T0 - T = (1-T) - (1-T0).
__device__ __forceinline__ void solar_c12(float K, float sum, float diff, float lambda, float om, float g,
                                          float sec0, float T0, float omt0, float R, float omt,
                                          float &c1, float &c2) {
  const float ksi0 = K * g / sec0;
  const float factor = 0.5f * om * sec0 / ((lambda - sec0) * (lambda + sec0));
  const float gam_up = factor * (sum - sec0 - ksi0 * (diff - sec0));
  const float gam_dn = factor * (sum + sec0 + ksi0 * (diff + sec0));
  const float opd = 1.0f + gam_dn;
  c1 = gam_up * fmaf(T0, omt, omt0) - R * opd;
  c2 = opd * (omt - omt0) - gam_up * R * T0;
}

// The solar source coefficients where lambda lies within kSolarSingularTol of
// sec_0.  They are smooth through lambda = sec_0, where the particular
// solution's 1/(lambda^2 - sec_0^2) cancels: evaluate at (sum, diff, lambda)
// scaled by rho_a, rho_b placed a safe distance either side of the
// singularity and interpolate linearly to rho = 1 (error ~ tol^2 + FP32
// eps / tol).  Out of line: few cells take it, and the hot loop stays small.
static __device__ __noinline__ float2 solar_c12_singular(float K, float sum, float diff, float lambda, float om,
                                                  float g, float tau, float sec0, float T0, float omt0) {
  const float ra = sec0 * (1.0f - kSolarSingularTol) / lambda;
  const float rb = sec0 * (1.0f + kSolarSingularTol) / lambda;
  float a1, a2, b1, b2;
  const LayerF la = layer_mix(ra * sum, ra * lambda, tau);
  solar_c12(K, ra * sum, ra * diff, ra * lambda, om, g, sec0, T0, omt0, la.R, la.omt, a1, a2);
  const LayerF lb = layer_mix(rb * sum, rb * lambda, tau);
  solar_c12(K, rb * sum, rb * diff, rb * lambda, om, g, sec0, T0, omt0, lb.R, lb.omt, b1, b2);
  const float w = (1.0f - ra) / (rb - ra);
  return make_float2(a1 + w * (b1 - a1), a2 + w * (b2 - a2));
}

__device__ __forceinline__ CoefF two_coeff_mix(int isolir, const SchemeF &sc, int l_quad,
                                               float g, float om, float one_m_om,
                                               float tau, float sec0) {
  CoefF c;
  const float sum = fmaf(-om, fmaf(sc.B, g, sc.C), sc.A);
  const float diff = sc.D * one_m_om;
  const float lambda = sqrtf(sum * diff);
  const LayerF l = layer_mix(sum, lambda, tau);
  c.T = l.T; c.R = l.R; c.omtr = l.omtr;
  if (isolir == SOCGPU_IP_SOLAR) {
    const float x0 = tau * sec0;
    const float T0 = __expf(-x0);
    const float omt0 = one_minus_exp(x0, T0);
    solar_c12(sc.K, sum, diff, lambda, om, g, sec0, T0, omt0, l.R, l.omt, c.c1, c.c2);
    if (fabsf(lambda - sec0) < kSolarSingularTol * sec0) {
      const float2 v = solar_c12_singular(sc.K, sum, diff, lambda, om, g, tau, sec0, T0, omt0);
      c.c1 = v.x; c.c2 = v.y;
    }
    c.T0 = T0;
    return c;
  }
  // infra-red (trans_source_coeff.F90:200-257)
  const float sq = (float)kSqEps64;
  c.T0 = 1.0f;
  c.c1 = (l.omt + l.R + sq) / fmaf(tau, sum, sq);
  c.c2 = 0.0f;
  if (l_quad) {
    // the numerator 1 + R + T + s2 equals d tau - (1-T-R) (thin layers) or
    // 2 (d tau - (1-T-R))/(d tau + sq) - (1-T-R);
    // d tau - (1-T-R) = (1-gamma)(phi(x) + gamma psi(x)) / ((1+gamma)(1+e gamma))
    const float dmo = l.omg * (phi_exp(l.x, l.em1) + l.gamma * psi_exp(l.x, l.e)) /
                      ((1.0f + l.gamma) * (1.0f + l.eg));
    const float num = (tau > (float)kTolQuad64) ? 2.0f * dmo / fmaf(diff, tau, sq) - l.omtr : dmo;
    c.c2 = -num / fmaf(sum, tau, sq);
  }
  return c;
}

__device__ __forceinline__ CoefF fast_lw_mix(int l_quad, float tau) {
  CoefF c;
  const float sq = (float)kSqEps64;
  const float x = 1.66f * tau;
  const float e = __expf(-x);
  const float em1 = one_minus_exp(x, e);     // 1 - T
  c.T = e;
  c.omtr = em1;
  c.R = 0.0f; c.T0 = 1.0f; c.c2 = 0.0f;
  c.c1 = (em1 + sq) / (x + sq);
  if (l_quad) {
    // two_coeff_fast_lw.F90:138-152 with 1 + T - 2 c1 = 2 phi(x)/(x + sq) - (1-T)
    const float ph = phi_exp(x, em1);
    const float num = (tau > (float)kTolQuad64) ? 2.0f * ph / (x + sq) - em1 : ph;
    c.c2 = -num / (x + sq);
  }
  return c;
}

}  // namespace socgpu
