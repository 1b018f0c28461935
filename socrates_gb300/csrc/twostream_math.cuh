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
//     reference kept as constants.  Cells next to the solar singularity
//     lambda = sec_0 fall back to the FP64 expressions.
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
  float one_minus_T;   // accurate 1-T (IR source) -- informational
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

// Same in FP32, taking 1-omega directly (no cancellation in diff).
__device__ __forceinline__ void sum_diff_mix(int scheme, float om, float one_m_om, float g,
                                             float &sum, float &diff) {
  switch (scheme) {
    case SOCGPU_IP_EDDINGTON: sum = 1.5f * (1.0f - om * g); diff = 2.0f * one_m_om; break;
    case SOCGPU_IP_ELSASSER: sum = 1.66f - 1.5f * om * g; diff = 1.66f * one_m_om; break;
    case SOCGPU_IP_DISCRETE_ORD: sum = 1.7320508f * (1.0f - om * g); diff = 1.7320508f * one_m_om; break;
    case SOCGPU_IP_PIFM85: sum = 2.0f - 1.5f * om * g; diff = 2.0f * one_m_om; break;
    case SOCGPU_IP_2S_TEST: sum = 1.5f - 1.5f * om * g; diff = 1.5f * one_m_om; break;
    case SOCGPU_IP_HEMI_MEAN: sum = 2.0f * (1.0f - om * g); diff = 2.0f * one_m_om; break;
    default: sum = 2.0f - 1.5f * om * g - 0.5f * om; diff = 2.0f * one_m_om; break;
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
// Distance to the solar singularity below which the FP64 expressions are used.
constexpr float kSolarSingularTol = 2.0e-3f;

__device__ __forceinline__ CoefF two_coeff_mix(int isolir, int scheme, int l_quad,
                                               float g, float om, float one_m_om,
                                               float tau, float sec0) {
  CoefF c;
  float sum, diff;
  sum_diff_mix(scheme, om, one_m_om, g, sum, diff);
  float lambda = sqrtf(sum * diff);
  if (isolir == SOCGPU_IP_SOLAR && fabsf(lambda - sec0) < kSolarSingularTol * sec0) {
    // near lambda = sec_0 the particular solution cancels: FP64 reference form
    Coef d = two_coeff_ref(isolir, scheme, l_quad, (double)g, 1.0 - (double)one_m_om,
                           (double)tau, (double)sec0);
    c.T = (float)d.T; c.R = (float)d.R; c.T0 = (float)d.T0; c.c1 = (float)d.c1; c.c2 = (float)d.c2;
    c.one_minus_T = (float)(1.0 - d.T);
    return c;
  }
  float lt = lambda * tau;
  float em1 = -expm1f(-lt);                  // 1 - e, accurate for small lambda*tau
  float e = 1.0f - em1;
  float inv_sl = 1.0f / (sum + lambda);
  float gamma = (sum - lambda) * inv_sl;
  float one_m_gamma = 2.0f * lambda * inv_sl;          // 1 - gamma
  float one_m_gamma2 = one_m_gamma * (1.0f + gamma);   // 1 - gamma^2
  float eg = e * gamma;
  float one_m_eg = em1 + e * one_m_gamma;              // 1 - e*gamma
  float den = one_m_eg * (1.0f + eg);                  // 1 - e^2 gamma^2
  float inv_den = 1.0f / den;
  float one_m_e2 = em1 * (1.0f + e);                   // 1 - e^2
  c.T = e * one_m_gamma2 * inv_den;
  c.R = gamma * one_m_e2 * inv_den;
  c.T0 = 1.0f;
  c.c2 = 0.0f;
  // 1 - T = (1-e)(1+e gamma^2)/(1-e^2 gamma^2)
  c.one_minus_T = em1 * (1.0f + eg * gamma) * inv_den;
  if (isolir == SOCGPU_IP_SOLAR) {
    float ksi0 = ((scheme == SOCGPU_IP_DISCRETE_ORD) ? 1.7320508f : 1.5f) * g / sec0;
    float factor = 0.5f * om * sec0 / ((lambda - sec0) * (lambda + sec0));
    float gam_up = factor * (sum - sec0 - ksi0 * (diff - sec0));
    float gam_dn = factor * (sum + sec0 + ksi0 * (diff + sec0));
    c.T0 = __expf(-tau * sec0);
    c.c1 = (gam_up - c.R * (1.0f + gam_dn)) - gam_up * c.T * c.T0;
    c.c2 = c.T0 * (1.0f + gam_dn - gam_up * c.R) - (1.0f + gam_dn) * c.T;
  } else {
    const float sq = (float)kSqEps64;
    c.c1 = (c.one_minus_T + c.R + sq) / (sq + tau * sum);
    if (l_quad) {
      // 1 - T - R = (1-e)(1-gamma)/(1+e gamma)
      float one_m_t_m_r = em1 * one_m_gamma / (1.0f + eg);
      float s2;
      if (tau > (float)kTolQuad64) s2 = -2.0f * (one_m_t_m_r + sq) / (diff * tau + sq);
      else s2 = -2.0f + diff * tau;
      c.c2 = -(1.0f + c.R + c.T + s2) / (sum * tau + sq);
    }
  }
  return c;
}

__device__ __forceinline__ CoefF fast_lw_mix(int l_quad, float tau) {
  CoefF c;
  const float sq = (float)kSqEps64;
  float x = 1.66f * tau;
  float em1 = -expm1f(-x);     // 1 - T
  c.T = 1.0f - em1;
  c.one_minus_T = em1;
  c.R = 0.0f; c.T0 = 1.0f; c.c2 = 0.0f;
  c.c1 = (em1 + sq) / (x + sq);
  if (l_quad) {
    if (tau > (float)kTolQuad64) c.c2 = -(2.0f - em1 - 2.0f * c.c1) / (x + sq);
    else c.c2 = -(x - em1) / (x + sq);
  }
  return c;
}

}  // namespace socgpu
