// aerosol_prsc.cu -- prescribed aerosol optical properties
// (prsc_opt_prop.F90, prsc_gather_spline.F90, spline_fit.F90,
// spline_evaluate.F90, called from opt_prop_aerosol.F90:714-790 for species
// whose parametrization is ip_aerosol_unparametrized).
//
// Each species gives absorption, scattering and phase-function moments on
// its own pressure levels, per profile and band.  One CTA per (column, band)
// fits a natural cubic spline in pressure to every quantity of every
// prescribed species (one thread per spline; x, y, second derivatives and the
// elimination's scratch in shared memory), then evaluates the splines at the
// layer pressures and writes four per-layer sums that the flux kernel adds
// to its grey optics: absorption and scattering (the volume coefficients
// divided by the air density, floored at zero), scattering x asymmetry and
// scattering x forward-scattering moment.  A layer pressure outside a
// species' levels gives zero for that quantity, as the reference's range
// error does; a species of one level has constant properties.
#include <cstdio>
#include "socgpu_internal.h"

namespace socgpu {
namespace {

constexpr int kThreads = 128;

// Natural cubic spline through (x[k], y[k]), k < n: second derivatives y2,
// u as scratch (the tridiagonal elimination of spline_fit.F90).
__device__ void spline_fit(int n, const double *x, const double *y, double *y2, double *u) {
  if (n == 1) { y2[0] = 0.0; return; }
  y2[0] = 0.0;
  u[0] = 0.0;
  for (int i = 1; i < n - 1; ++i) {
    const double sigma = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    const double rho = sigma * y2[i - 1] + 2.0;
    y2[i] = (sigma - 1.0) / rho;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) -
            sigma * u[i - 1]) / rho;
  }
  y2[n - 1] = 0.0;
  for (int i = n - 2; i >= 0; --i) y2[i] = y2[i] * y2[i + 1] + u[i];
}

// The spline's value at xp in the interval (lo, hi) found by bisection
// (spline_evaluate.F90).
__device__ __forceinline__ double spline_at(const double *x, const double *y, const double *y2, int lo, int hi,
                                            double xp) {
  const double delta = x[hi] - x[lo];
  const double a = (x[hi] - xp) / delta, b = (xp - x[lo]) / delta, c = delta * delta / 6.0;
  return a * (y[lo] + (a * a - 1.0) * y2[lo] * c) + b * (y[hi] + (b * b - 1.0) * y2[hi] * c);
}

__global__ void __launch_bounds__(kThreads) prsc_kernel(const FluxParams p, double *out) {
  extern __shared__ double sm[];
  const int col = blockIdx.x, bi = blockIdx.y, b = p.first_band - 1 + bi;
  const int nbc = gridDim.y, L = p.n_layer, n = p.n_profile;
  const size_t ndpp = (size_t)p.nd_prof_prsc, ndlv = (size_t)p.nd_lev_prsc, ndf = (size_t)p.nd_phf_prsc;
  const size_t nsp = (size_t)p.nd_sp_prsc;
  const int nq = 2 + p.prsc_nq;   // absorption, scattering, moments 1..prsc_nq
  // species s: x[nlev], then per quantity y[nlev], y2[nlev], u[nlev]
  auto base = [&](int s) {
    size_t o = 0;
    for (int t = 0; t < s; ++t) o += (size_t)p.prsc_nlev[t] * (1 + 3 * nq);
    return o;
  };
  for (int s = 0; s < p.n_prsc; ++s) {
    const int nl = p.prsc_nlev[s];
    const size_t j = (size_t)p.prsc_species[s];
    double *x = sm + base(s);
    for (int k = threadIdx.x; k < nl * nq; k += blockDim.x) {
      const int q = k / nl, lev = k - q * nl;
      if (q == 0) x[lev] = p.prsc_p[col + ndpp * (lev + ndlv * j)];
      double v;
      if (q == 0) v = p.prsc_abs[col + ndpp * (lev + ndlv * (j + nsp * b))];
      else if (q == 1) v = p.prsc_scat[col + ndpp * (lev + ndlv * (j + nsp * b))];
      else v = p.prsc_phf[col + ndpp * (lev + ndlv * ((q - 2) + ndf * (j + nsp * b)))];
      x[nl * (1 + 3 * q) + lev] = v;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < p.n_prsc * nq; t += blockDim.x) {
    const int s = t / nq, q = t - s * nq, nl = p.prsc_nlev[s];
    double *x = sm + base(s), *y = x + nl * (1 + 3 * q);
    spline_fit(nl, x, y, y + nl, y + 2 * nl);
  }
  __syncthreads();
  const int ndp = p.nd_profile, nof = p.n_order_forward;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const double pr = p.p[col + (size_t)ndp * i], rho = p.density[col + (size_t)ndp * i];
    double kabs = 0.0, ks = 0.0, kg = 0.0, kf = 0.0;
    for (int s = 0; s < p.n_prsc; ++s) {
      const int nl = p.prsc_nlev[s];
      const double *x = sm + base(s);
      const bool in = nl == 1 || (pr <= x[nl - 1] && pr >= x[0]);
      int lo = 0, hi = nl - 1;
      while (nl > 1 && hi - lo > 1) {
        const int m = (lo + hi) / 2;
        if (pr > x[m]) lo = m; else hi = m;
      }
      auto val = [&](int q) -> double {
        if (!in) return 0.0;
        const double *y = x + nl * (1 + 3 * q);
        return nl == 1 ? y[0] : spline_at(x, y, y + nl, lo, hi, pr);
      };
      const double a = fmax(0.0, val(0) / rho), sc = fmax(0.0, val(1) / rho);
      const double g = val(2), cnt = (double)p.prsc_count[s];
      kabs += cnt * a;
      ks += cnt * sc;
      kg += cnt * (sc * g);
      if (p.l_rescale) {
        double f;
        if (!p.l_hg) f = sc * val(1 + nof);
        else if (nof == 1) f = sc * g;
        else if (nof == 2) f = (sc * g) * g;
        else f = sc * pow(g, (double)nof);
        kf += cnt * f;
      }
    }
    const size_t plane = (size_t)nbc * L * n, q0 = ((size_t)bi * L + i) * n + col;
    out[q0] = kabs;
    out[plane + q0] = ks;
    out[2 * plane + q0] = kg;
    out[3 * plane + q0] = kf;
  }
}

}  // namespace

size_t prsc_bytes(const FluxParams &p) {
  return 4 * sizeof(double) * (size_t)(p.last_band - p.first_band + 1) * p.n_layer * p.n_profile;
}

int launch_prsc(const FluxParams &p, double *out, cudaStream_t st, char *msg, size_t len) {
  size_t smem = 0;
  for (int s = 0; s < p.n_prsc; ++s) smem += (size_t)p.prsc_nlev[s] * (1 + 3 * (2 + p.prsc_nq)) * sizeof(double);
  int dev = 0, max_smem = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if ((long long)smem > max_smem) {
    snprintf(msg, len, "prescribed aerosol levels need %zu bytes of shared memory (limit %d)", smem, max_smem);
    return SOCGPU_I_ERR_RANGE;
  }
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(prsc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    snprintf(msg, len, "shared memory request of %zu bytes refused", smem);
    return SOCGPU_I_ERR_RANGE;
  }
  if (p.n_profile <= 0 || p.n_layer <= 0) return SOCGPU_I_NORMAL;
  const dim3 grid(p.n_profile, p.last_band - p.first_band + 1);
  prsc_kernel<<<grid, kThreads, smem, st>>>(p, out);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, len, "prescribed aerosol kernel launch failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return SOCGPU_I_NORMAL;
}

}  // namespace socgpu
