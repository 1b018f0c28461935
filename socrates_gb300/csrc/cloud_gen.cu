// cloud_gen.cu -- McICA stochastic subcolumn generator for sm_103a.
//
// Restates cloud_gen (src/interface_core/socrates_cloud_gen.F90:8-470) with
// one thread per column.  The reference generator is sequential per column
// (its LCG stream is advanced a data-dependent number of times per layer),
// so columns, not layers, are the parallel axis; consecutive threads own
// consecutive columns and every store of c_sub(nd_profile, k, s) is
// coalesced.  The reference's FP64 arithmetic is kept where it decides a
// branch (the LCG modulo via int(real(temp)*rm), the overlap parameters and
// the uniform deviates), so masks are bit-identical to the CPU restatement.
// The Philox mode replaces the two LCG streams by Philox4x32-10 keyed by
// (column seed, subcolumn, layer): four deviates per cell, so a column's
// masks depend only on its own seed and inputs.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include "socgpu_internal.h"

namespace socgpu {

namespace {

constexpr int kM = 86436, kA = 1093, kC = 18257;   // socrates_cloud_gen.F90:48-50
constexpr double kEps64 = 2.220446049250313e-16;

__device__ __forceinline__ int lcg_next(int x) {
  const double rm = 1.0 / (double)kM;
  int temp = x * kA + kC;
  return temp - (int)(__dmul_rn((double)temp, rm)) * kM;
}

__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

__device__ __forceinline__ double u01(uint32_t w) { return (double)w * (1.0 / 4294967296.0); }

struct GenArgs {
  int nd_layer, cloud_top, n_layer, nd_profile, il1, il2, n_subcol, n1, n2, ipph, ioverlap, rng;
  const int *rand_seed;
  const double *rlc_cf, *rlc_cw, *sigma_qcw, *avg_cf, *c_cloud, *c_ratio, *zf, *xcw;
  int *n_subcol_cld;
  double *c_sub;
  int *range;   // [0] = k_top, [1] = k_base (device)
};

// First and last layer holding cloud in any column (socrates_cloud_gen.F90:225-250).
__global__ void cloud_range_kernel(GenArgs a) {
  const int ndc = a.nd_layer - a.cloud_top + 1;
  const int ncol = a.il2 - a.il1 + 1;
  const long long total = (long long)ncol * (a.n_layer - a.cloud_top + 1);
  const double cut = kEps64;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    int il = a.il1 + (int)(q % ncol);
    int k = a.cloud_top + (int)(q / ncol);
    double cf = a.avg_cf[(size_t)(il - 1) + (size_t)a.nd_profile * (size_t)(k - a.cloud_top)];
    if (cf > cut) atomicMin(&a.range[0], k);
    if (cf >= cut) atomicMax(&a.range[1], k);
  }
  (void)ndc;
}

__global__ void cloud_gen_kernel(GenArgs a) {
  const int il = a.il1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (il > a.il2) return;
  const int ndp = a.nd_profile, ct = a.cloud_top, ndc = a.nd_layer - ct + 1;
  const double rm = 1.0 / (double)kM;
#define CLD(arr, k) __ldg((arr) + (size_t)(il - 1) + (size_t)ndp * (size_t)((k) - ct))
#define CSUB(k, s) a.c_sub[(size_t)(il - 1) + (size_t)ndp * ((size_t)((k) - ct) + (size_t)ndc * (size_t)((s) - 1))]
  for (int s = 1; s <= a.n_subcol; ++s)
    for (int k = ct; k <= a.nd_layer; ++k) CSUB(k, s) = 0.0;
  const int k_top = a.range[0], k_base = a.range[1];
  if (k_top > a.n_layer || k_base < k_top) { a.n_subcol_cld[il - 1] = 0; return; }

  // seed streams (socrates_cloud_gen.F90:180-203): advance n_subcol times,
  // then n_subcol x seeds, then n_subcol y seeds.  Each subcolumn's seeds
  // are recomputed from the column seed when needed.
  const int rand_seed_max = (2147483647 - kC) / kA;
  int seed = a.rand_seed[il - 1];
  int rd0 = (seed < 0 ? -seed : seed) % rand_seed_max;
  for (int i = 0; i < a.n_subcol; ++i) rd0 = lcg_next(rd0);
  int rd_x = rd0;                       // state before the first x seed
  int rd_y = rd0;
  for (int i = 0; i < a.n_subcol; ++i) rd_y = lcg_next(rd_y);   // state before the first y seed
  const uint32_t key0 = (uint32_t)seed, key1 = 0x534F4352u;

  int i_loc = 1;
  double x = 0.0, y = 0.0;     // persist across subcolumns like x(il), y(il)
  for (int i = 1; i <= a.n_subcol; ++i) {
    rd_x = lcg_next(rd_x);
    rd_y = lcg_next(rd_y);
    int int_x = rd_x, int_y = rd_y;
    bool l_cld = false;
    for (int k = k_top; k <= k_base; ++k) {
      const double cf = CLD(a.avg_cf, k);
      if (!(cf > 0.0)) continue;
      uint32_t u[4] = {0u, 0u, 0u, 0u};
      if (a.rng == SOCGPU_RNG_PHILOX) philox4x32_10((uint32_t)k, (uint32_t)i, 0u, 0u, key0, key1, u);
      if (a.ioverlap == SOCGPU_IP_MAX_RAND) {
        // socrates_cloud_gen.F90:263-330
        if (a.rng == SOCGPU_RNG_PHILOX) { x = u01(u[0]); y = u01(u[1]); }
        else {
          int_x = lcg_next(int_x); x = __dmul_rn((double)int_x, rm);
          int_y = lcg_next(int_y); y = __dmul_rn((double)int_y, rm);
        }
        if (k == ct) {
          if (a.rng == SOCGPU_RNG_PHILOX) { x = u01(u[2]); y = u01(u[3]); }
          else {
            int_x = lcg_next(int_x); x = __dmul_rn((double)int_x, rm);
            int_y = lcg_next(int_y); y = __dmul_rn((double)int_y, rm);
          }
        } else {
          const double cfm = CLD(a.avg_cf, k - 1);
          if (x < (1.0 - cfm)) {
            double x1, y1;
            if (a.rng == SOCGPU_RNG_PHILOX) { x1 = u01(u[2]); y1 = u01(u[3]); }
            else {
              int_x = lcg_next(int_x); x1 = __dmul_rn((double)int_x, rm);
              int_y = lcg_next(int_y); y1 = __dmul_rn((double)int_y, rm);
            }
            x = __dmul_rn(x1, 1.0 - cfm);
            y = y1;
          }
        }
      } else {
        // socrates_cloud_gen.F90:338-460; alpha/rcorr of layer k-1
        double alpha = 0.0, rcorr = 0.0;
        const int km = k - 1;
        if (!(a.ioverlap == SOCGPU_IP_RAND || km < ct)) {
          if (a.ioverlap == SOCGPU_IP_EXPONENTIAL || CLD(a.avg_cf, km) > 0.0) {
            double dz = __dsub_rn(__ldg(a.zf + (size_t)(il - 1) + (size_t)ndp * (size_t)(km - 1)),
                                  __ldg(a.zf + (size_t)(il - 1) + (size_t)ndp * (size_t)km));
            double lcf = CLD(a.rlc_cf, km), lcw = CLD(a.rlc_cw, km);
            alpha = lcf > 0.0 ? exp(__ddiv_rn(dz, lcf)) : 0.0;
            rcorr = lcw > 0.0 ? exp(__ddiv_rn(dz, lcw)) : 0.0;
          }
        }
        double x1, y1;
        if (a.rng == SOCGPU_RNG_PHILOX) { x1 = u01(u[0]); y1 = u01(u[1]); }
        else {
          int_x = lcg_next(int_x); x1 = __dmul_rn((double)int_x, rm);
          int_y = lcg_next(int_y); y1 = __dmul_rn((double)int_y, rm);
        }
        if (x1 >= alpha) {
          if (a.rng == SOCGPU_RNG_PHILOX) x = u01(u[2]);
          else { int_x = lcg_next(int_x); x = __dmul_rn((double)int_x, rm); }
        }
        if (y1 >= rcorr) {
          if (a.rng == SOCGPU_RNG_PHILOX) y = u01(u[3]);
          else { int_y = lcg_next(int_y); y = __dmul_rn((double)int_y, rm); }
        }
      }
      if (x < cf) {
        double zcw = 1.0;
        if (a.ipph != 0) {
          double ratio = 1.0;
          if (a.ioverlap != SOCGPU_IP_MAX_RAND) {
            const double cc = a.c_cloud ? CLD(a.c_cloud, k) : 0.0;
            const double cr = a.c_ratio ? CLD(a.c_ratio, k) : 0.0;
            if (x < cc) ratio = cr;
            else if (cc > 0.0 && cc < cf) {
              double num = cf - cr * cc;
              ratio = (num > 0.0 ? num : 0.0) / (cf - cc);
            }
          }
          double rind1 = y * (a.n1 - 1) + 1.0;
          int ind1 = (int)rind1; ind1 = ind1 > a.n1 - 1 ? a.n1 - 1 : ind1; ind1 = ind1 < 1 ? 1 : ind1;
          rind1 = rind1 - (double)ind1; rind1 = rind1 > 1.0 ? 1.0 : (rind1 < 0.0 ? 0.0 : rind1);
          double rind2 = 40.0 * CLD(a.sigma_qcw, k) - 3.0;
          int ind2 = (int)rind2; ind2 = ind2 > a.n2 - 1 ? a.n2 - 1 : ind2; ind2 = ind2 < 1 ? 1 : ind2;
          rind2 = rind2 - (double)ind2; rind2 = rind2 > 1.0 ? 1.0 : (rind2 < 0.0 ? 0.0 : rind2);
#define XCW(p, q) __ldg(a.xcw + (size_t)((p) - 1) + (size_t)a.n1 * (size_t)((q) - 1))
          zcw = (1.0 - rind1) * (1.0 - rind2) * XCW(ind1, ind2)
              + (1.0 - rind1) * rind2 * XCW(ind1, ind2 + 1)
              + rind1 * (1.0 - rind2) * XCW(ind1 + 1, ind2)
              + rind1 * rind2 * XCW(ind1 + 1, ind2 + 1);
#undef XCW
          zcw = zcw * ratio;
        }
        l_cld = true;
        CSUB(k, i_loc) = zcw;
      }
    }
    if (l_cld) ++i_loc;
  }
  a.n_subcol_cld[il - 1] = i_loc - 1;
#undef CLD
#undef CSUB
}

}  // namespace

// Threads per CTA of the generator (one thread per column): as few as a
// warp, so that the columns spread over every SM -- each thread's work is a
// serial chain of FP64 arithmetic and random draws, and the FP64 units of an
// SM are shared by its warps -- up to 128 once there are two CTAs per SM.
static int gen_block(int ncol) {
  int n_sm = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    n_sm = 1;
  }
  const int per = (ncol + 2 * n_sm - 1) / (2 * n_sm);
  return std::min(128, std::max(32, (per + 31) / 32 * 32));
}

int launch_cloud_gen(int nd_layer, int cloud_top, int n_layer, int nd_profile, int il1, int il2,
                     int n_subcol, int n1, int n2, int ipph, int ioverlap, const int *rand_seed,
                     const double *rlc_cf, const double *rlc_cw, const double *sigma_qcw,
                     const double *avg_cf, const double *c_cloud, const double *c_ratio,
                     const double *zf, const double *xcw, int *n_subcol_cld, double *c_sub, int rng,
                     int *range_dev, cudaStream_t st, char *msg, size_t len) {
  GenArgs a{nd_layer, cloud_top, n_layer, nd_profile, il1, il2, n_subcol, n1, n2, ipph, ioverlap, rng,
            rand_seed, rlc_cf, rlc_cw, sigma_qcw, avg_cf, c_cloud, c_ratio, zf, xcw, n_subcol_cld, c_sub,
            range_dev};
  const int ncol = il2 - il1 + 1;
  if (ncol <= 0) return SOCGPU_I_NORMAL;
  int init[2] = {n_layer + 1, cloud_top - 1};
  cudaMemcpyAsync(range_dev, init, sizeof(init), cudaMemcpyHostToDevice, st);
  long long cells = (long long)ncol * (n_layer - cloud_top + 1);
  int blocks = (int)((cells + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  cloud_range_kernel<<<blocks, 256, 0, st>>>(a);
  count_launch();
  const int bs = gen_block(ncol);
  cloud_gen_kernel<<<(ncol + bs - 1) / bs, bs, 0, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, len, "cloud_gen launch failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return SOCGPU_I_NORMAL;
}

// ---------------------------------------------------------------------------
// Allocation-free variant (socgpu_cloud_gen_device_noalloc).
//
// Some callers cannot allocate device memory where they generate subcolumns:
// a host model that gives the radiation scheme a fixed device-memory budget at
// start-up and treats any later allocation as an error, or a time step whose
// concurrent streams must not be serialised by the device-wide
// synchronisation that cudaFree implies.  This variant keeps its scratch in a
// fixed array of the library's own device memory instead of the per-thread
// workspace, and makes no allocation of any kind.
//
// Layout of the scratch (ints), n = SOCGPU_NOALLOC_MAX_CLOUD_LAYERS:
//   [0, n)       layer cloud_top + j holds cloud fraction >  cut in some column
//   [n, 2n)      layer cloud_top + j holds cloud fraction >= cut in some column
//   [2n, 2n + 2) k_top, k_base of the batch (read by cloud_gen_kernel)
// The flags of the call's layers must be zero when cloud_layer_flag_kernel
// runs: every call clears them itself on its own stream first, so no state
// carries over from one call to the next.  The range slots are always written
// by cloud_layer_range_kernel before cloud_gen_kernel reads them.  All calls on
// one device share this array: calls that overlap in time (different streams
// or host threads without ordering between them) race on it.
namespace {

constexpr int kNoAllocLayers = SOCGPU_NOALLOC_MAX_CLOUD_LAYERS;
static __device__ __align__(256) int g_noalloc_scratch[2 * kNoAllocLayers + 2];

// Which cloud layers hold cloud anywhere in the batch
// (socrates_cloud_gen.F90:225-250, as flags instead of atomic min/max).
__global__ void cloud_layer_flag_kernel(GenArgs a, int *flags, int ncl) {
  const int ncol = a.il2 - a.il1 + 1;
  const long long total = (long long)ncol * ncl;
  const double cut = kEps64;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int il = a.il1 + (int)(q % ncol);
    const int kk = (int)(q / ncol);
    const double cf = a.avg_cf[(size_t)(il - 1) + (size_t)a.nd_profile * (size_t)kk];
    if (cf > cut) flags[kk] = 1;
    if (cf >= cut) flags[kNoAllocLayers + kk] = 1;
  }
}

// Reduce the flags to the batch's first and last cloudy layer.
__global__ void cloud_layer_range_kernel(const int *flags, int ncl, int cloud_top, int n_layer, int *range) {
  __shared__ int s_top, s_base;
  if (threadIdx.x == 0) { s_top = n_layer + 1; s_base = cloud_top - 1; }
  __syncthreads();
  for (int kk = threadIdx.x; kk < ncl; kk += blockDim.x) {
    if (flags[kk]) atomicMin(&s_top, cloud_top + kk);
    if (flags[kNoAllocLayers + kk]) atomicMax(&s_base, cloud_top + kk);
  }
  __syncthreads();
  if (threadIdx.x == 0) { range[0] = s_top; range[1] = s_base; }
}

std::mutex g_noalloc_mutex;
constexpr int kMaxDevices = 64;
int *g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (the first call on a device does this setup).  The address holds for
// the life of the device's primary context; the header tells callers not to
// use this entry point after destroying that context (cudaDeviceReset).
int noalloc_scratch(int **out, char *msg, size_t len) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    snprintf(msg, len, "no usable CUDA device: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      snprintf(msg, len, "address of the allocation-free scratch not available: %s", cudaGetErrorString(e));
      return SOCGPU_I_ABORT_CALCULATION;
    }
    g_noalloc_addr[dev] = (int *)p;
  }
  *out = g_noalloc_addr[dev];
  return SOCGPU_I_NORMAL;
}

}  // namespace

int launch_cloud_gen_noalloc(int nd_layer, int cloud_top, int n_layer, int nd_profile, int il1, int il2,
                             int n_subcol, int n1, int n2, int ipph, int ioverlap, const int *rand_seed,
                             const double *rlc_cf, const double *rlc_cw, const double *sigma_qcw,
                             const double *avg_cf, const double *c_cloud, const double *c_ratio,
                             const double *zf, const double *xcw, int *n_subcol_cld, double *c_sub, int rng,
                             cudaStream_t st, char *msg, size_t len) {
  const int ncl = n_layer - cloud_top + 1;
  if (ncl > kNoAllocLayers) {
    snprintf(msg, len, "%d cloud layers exceed the allocation-free limit of %d (SOCGPU_NOALLOC_MAX_CLOUD_LAYERS)",
             ncl, kNoAllocLayers);
    return SOCGPU_I_ERR_RANGE;
  }
  int *scratch = nullptr;
  int stat = noalloc_scratch(&scratch, msg, len);
  if (stat != SOCGPU_I_NORMAL) return stat;
  int *range = scratch + 2 * kNoAllocLayers;
  GenArgs a{nd_layer, cloud_top, n_layer, nd_profile, il1, il2, n_subcol, n1, n2, ipph, ioverlap, rng,
            rand_seed, rlc_cf, rlc_cw, sigma_qcw, avg_cf, c_cloud, c_ratio, zf, xcw, n_subcol_cld, c_sub,
            range};
  const int ncol = il2 - il1 + 1;
  if (ncol <= 0) return SOCGPU_I_NORMAL;
  if (ncl > 0) {
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(int) * ncl, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch + kNoAllocLayers, 0, sizeof(int) * ncl, st);
    if (e != cudaSuccess) {
      snprintf(msg, len, "clearing the cloud layer flags failed: %s", cudaGetErrorString(e));
      return SOCGPU_I_ABORT_CALCULATION;
    }
    long long cells = (long long)ncol * ncl;
    int blocks = (int)((cells + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    cloud_layer_flag_kernel<<<blocks, 256, 0, st>>>(a, scratch, ncl);
    count_launch();
  }
  cloud_layer_range_kernel<<<1, 256, 0, st>>>(scratch, ncl > 0 ? ncl : 0, cloud_top, n_layer, range);
  count_launch();
  const int bs = gen_block(ncol);
  cloud_gen_kernel<<<(ncol + bs - 1) / bs, bs, 0, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, len, "cloud_gen launch failed: %s", cudaGetErrorString(e));
    return SOCGPU_I_ABORT_CALCULATION;
  }
  return SOCGPU_I_NORMAL;
}

}  // namespace socgpu
