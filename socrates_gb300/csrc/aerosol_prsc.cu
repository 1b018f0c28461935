// aerosol_prsc.cu -- prescribed aerosol optical properties
// (prsc_opt_prop.F90, prsc_gather_spline.F90, spline_fit.F90,
// spline_evaluate.F90, called from opt_prop_aerosol.F90:714-790 for species
// whose parametrization is ip_aerosol_unparametrized).
//
// Each species gives absorption, scattering and phase-function moments on
// its own pressure levels, per profile and band; every quantity is fitted by
// a natural cubic spline in pressure and evaluated at the layer pressures.
// One CTA per column.  The parts of the fit and of the evaluation that
// depend on the pressures only are computed once per column and species:
// the elimination's coefficients (sigma, 1/rho, the back-substitution
// factor, the reciprocal level spacings) and, for each layer, its interval
// and interpolation weights.  What is left per (band, quantity) is the
// right-hand side of the tridiagonal system and the back-substitution, and
// per (band, layer) a few fused multiply-adds -- the GPU has few FP64
// units, so the divisions of the per-point formulas are hoisted out.  Bands
// are staged through shared memory in chunks.  The kernel writes, per
// column, four per-layer sums that the flux kernel adds to its grey optics:
// absorption and scattering (the volume coefficients divided by the air
// density, floored at zero), scattering x asymmetry and scattering x
// forward-scattering moment.  A layer pressure outside a species' levels
// gives zero for that quantity, as the reference's range error does; a
// species of one level has constant properties.
#include <algorithm>
#include <cstdio>
#include "socgpu_internal.h"

namespace socgpu {
namespace {

constexpr int kThreads = 128;
constexpr size_t kChunkBytes = 48 * 1024;   // shared memory for the staged bands

// Shared-memory layout of one column.
struct PrscLayout {
  int nq, nbc;                 // quantities per band (2 + moments), bands per chunk
  size_t geo[kMaxAerMr];       // per species: x, hinv, winv, sig, rinv, c2 (6 nl doubles)
  size_t wts;                  // per (species, layer): a, b, c (doubles); lo in `lo`
  size_t lo;                   // ints: per (species, layer) lower level, -1 outside, -2 one level
  size_t rho;                  // per layer: 1 / density
  size_t ytab[kMaxAerMr];      // per species: (band of chunk, quantity) x (y, y2, u) x nl
  size_t bytes;
};

inline PrscLayout prsc_layout(const FluxParams &p, int nb_total, size_t chunk_bytes) {
  PrscLayout s{};
  s.nq = 2 + p.prsc_nq;
  size_t o = 0, ylev = 0;
  for (int k = 0; k < p.n_prsc; ++k) {
    s.geo[k] = o;
    o += 6 * (size_t)p.prsc_nlev[k];
    ylev += (size_t)p.prsc_nlev[k];
  }
  s.wts = o;
  o += 3 * (size_t)p.n_prsc * p.n_layer;
  s.rho = o;
  o += (size_t)p.n_layer;
  const size_t per_band = 3 * (size_t)s.nq * ylev * sizeof(double);
  s.nbc = (int)std::max<size_t>(1, std::min<size_t>((size_t)nb_total, chunk_bytes / std::max<size_t>(per_band, 1)));
  for (int k = 0, acc = 0; k < p.n_prsc; ++k) {
    s.ytab[k] = o + (size_t)acc * 3 * s.nq * s.nbc;
    acc += p.prsc_nlev[k];
  }
  o += 3 * (size_t)s.nq * ylev * s.nbc;
  s.lo = o * sizeof(double);
  s.bytes = s.lo + sizeof(int) * (size_t)p.n_prsc * p.n_layer;
  return s;
}

__global__ void __launch_bounds__(kThreads) prsc_kernel(const FluxParams p, PrscLayout lay, double *out) {
  extern __shared__ double sm[];
  int *lo_tab = (int *)((char *)sm + lay.lo);
  const int col = blockIdx.x, L = p.n_layer, ns = p.n_prsc, nq = lay.nq;
  const int b0 = p.first_band - 1, nb = p.last_band - p.first_band + 1;
  const size_t ndpp = (size_t)p.nd_prof_prsc, ndlv = (size_t)p.nd_lev_prsc, ndf = (size_t)p.nd_phf_prsc;
  const size_t nsp = (size_t)p.nd_sp_prsc;
  const int ndp = p.nd_profile, nof = p.n_order_forward;
  // levels of every species
  for (int s = 0; s < ns; ++s) {
    const size_t j = (size_t)p.prsc_species[s];
    for (int k = threadIdx.x; k < p.prsc_nlev[s]; k += blockDim.x)
      sm[lay.geo[s] + k] = p.prsc_p[col + ndpp * (k + ndlv * j)];
  }
  __syncthreads();
  // the elimination's coefficients of each species (spline_fit.F90): they
  // depend on the levels only
  for (int s = threadIdx.x; s < ns; s += blockDim.x) {
    const int nl = p.prsc_nlev[s];
    double *x = sm + lay.geo[s], *hinv = x + nl, *winv = x + 2 * nl, *sig = x + 3 * nl, *rinv = x + 4 * nl,
           *c2 = x + 5 * nl;
    for (int i = 0; i < nl - 1; ++i) hinv[i] = 1.0 / (x[i + 1] - x[i]);
    c2[0] = 0.0;
    for (int i = 1; i < nl - 1; ++i) {
      winv[i] = 1.0 / (x[i + 1] - x[i - 1]);
      sig[i] = (x[i] - x[i - 1]) * winv[i];
      const double rho = sig[i] * c2[i - 1] + 2.0;
      rinv[i] = 1.0 / rho;
      c2[i] = (sig[i] - 1.0) * rinv[i];
    }
    if (nl > 1) c2[nl - 1] = 0.0;
  }
  // each layer's interval and weights for each species (spline_evaluate.F90)
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const double pr = p.p[col + (size_t)ndp * i];
    sm[lay.rho + i] = 1.0 / p.density[col + (size_t)ndp * i];
    for (int s = 0; s < ns; ++s) {
      const int nl = p.prsc_nlev[s];
      const double *x = sm + lay.geo[s];
      double *w = sm + lay.wts + 3 * ((size_t)s * L + i);
      int &lo = lo_tab[(size_t)s * L + i];
      if (nl == 1) { lo = -2; continue; }
      if (pr > x[nl - 1] || pr < x[0]) { lo = -1; continue; }
      int l0 = 0, h0 = nl - 1;
      while (h0 - l0 > 1) {
        const int m = (l0 + h0) / 2;
        if (pr > x[m]) l0 = m; else h0 = m;
      }
      const double delta = x[h0] - x[l0], dinv = 1.0 / delta;
      w[0] = (x[h0] - pr) * dinv;
      w[1] = (pr - x[l0]) * dinv;
      w[2] = delta * delta * (1.0 / 6.0);
      lo = l0;
    }
  }
  for (int c0 = 0; c0 < nb; c0 += lay.nbc) {
    const int nbc = min(lay.nbc, nb - c0);
    __syncthreads();
    // stage the chunk's values: y of (band, quantity) rows
    for (int s = 0; s < ns; ++s) {
      const int nl = p.prsc_nlev[s];
      const size_t j = (size_t)p.prsc_species[s];
      double *yt = sm + lay.ytab[s];
      for (int k = threadIdx.x; k < nbc * nq * nl; k += blockDim.x) {
        const int lev = k % nl, r = k / nl, q = r % nq, bc = r / nq, b = b0 + c0 + bc;
        double v;
        if (q == 0) v = p.prsc_abs[col + ndpp * (lev + ndlv * (j + nsp * b))];
        else if (q == 1) v = p.prsc_scat[col + ndpp * (lev + ndlv * (j + nsp * b))];
        else v = p.prsc_phf[col + ndpp * (lev + ndlv * ((q - 2) + ndf * (j + nsp * b)))];
        yt[(size_t)r * 3 * nl + lev] = v;
      }
    }
    __syncthreads();
    // second derivatives of every (species, band, quantity) spline
    for (int t = threadIdx.x; t < ns * nbc * nq; t += blockDim.x) {
      const int s = t / (nbc * nq), r = t - s * nbc * nq, nl = p.prsc_nlev[s];
      const double *x = sm + lay.geo[s], *hinv = x + nl, *winv = x + 2 * nl, *sig = x + 3 * nl,
                   *rinv = x + 4 * nl, *c2 = x + 5 * nl;
      double *y = sm + lay.ytab[s] + (size_t)r * 3 * nl, *y2 = y + nl, *u = y + 2 * nl;
      if (nl == 1) { y2[0] = 0.0; continue; }
      u[0] = 0.0;
      for (int i = 1; i < nl - 1; ++i)
        u[i] = (6.0 * ((y[i + 1] - y[i]) * hinv[i] - (y[i] - y[i - 1]) * hinv[i - 1]) * winv[i] -
                sig[i] * u[i - 1]) * rinv[i];
      y2[nl - 1] = 0.0;
      for (int i = nl - 2; i >= 0; --i) y2[i] = c2[i] * y2[i + 1] + u[i];
    }
    __syncthreads();
    // the sums of every (band, layer) of the chunk
    for (int t = threadIdx.x; t < nbc * L; t += blockDim.x) {
      const int bc = t / L, i = t - bc * L;
      const double rinv_air = sm[lay.rho + i];
      double kabs = 0.0, ks = 0.0, kg = 0.0, kf = 0.0;
      for (int s = 0; s < ns; ++s) {
        const int nl = p.prsc_nlev[s], lo = lo_tab[(size_t)s * L + i];
        if (lo == -1) continue;
        const double *yb = sm + lay.ytab[s] + (size_t)bc * nq * 3 * nl;
        const double *w = sm + lay.wts + 3 * ((size_t)s * L + i);
        auto val = [&](int q) -> double {
          const double *y = yb + (size_t)q * 3 * nl, *y2 = y + nl;
          if (lo == -2) return y[0];
          const double a = w[0], bb = w[1], c = w[2];
          return a * (y[lo] + (a * a - 1.0) * y2[lo] * c) + bb * (y[lo + 1] + (bb * bb - 1.0) * y2[lo + 1] * c);
        };
        const double a = fmax(0.0, val(0) * rinv_air), sc = fmax(0.0, val(1) * rinv_air);
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
      // column-major output: the flux kernel's CTA for this column reads
      // consecutive layers
      const size_t q0 = (((size_t)col * 4) * nb + (c0 + bc)) * L + i, plane = (size_t)nb * L;
      out[q0] = kabs;
      out[plane + q0] = ks;
      out[2 * plane + q0] = kg;
      out[3 * plane + q0] = kf;
    }
  }
}

}  // namespace

size_t prsc_bytes(const FluxParams &p) {
  return 4 * sizeof(double) * (size_t)(p.last_band - p.first_band + 1) * p.n_layer * p.n_profile;
}

int launch_prsc(const FluxParams &p, double *out, cudaStream_t st, char *msg, size_t len) {
  const PrscLayout lay = prsc_layout(p, p.last_band - p.first_band + 1, kChunkBytes);
  const size_t smem = lay.bytes;
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
  prsc_kernel<<<p.n_profile, kThreads, smem, st>>>(p, lay, out);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, len, "prescribed aerosol kernel launch failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return SOCGPU_I_NORMAL;
}

}  // namespace socgpu
