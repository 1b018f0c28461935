// host_internal.h -- host-side pieces shared by the C-ABI entry points
// (abi.cu) and the request server (server.cu): the spectrum registry entry,
// option validation, the staging plan of a host-pointer call and the kernel
// dispatch.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <string>
#include <vector>

#include "socgpu_internal.h"

namespace socgpu {

void set_msg(char *msg, size_t len, const char *fmt, ...);

#define CUDA_TRY(expr)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      set_msg(msg, msg_len, "%s failed: %s", #expr, cudaGetErrorString(e_));            \
      return SOCGPU_I_ABORT_CALCULATION;                                                \
    }                                                                                   \
  } while (0)

// A registered spectrum: device tables plus the host copies validation reads.
struct SpectrumEntry {
  std::string name;
  SpectrumDev dev{};
  std::vector<BandInfo> bands_host;
  std::vector<GPoint> gpoints_host;
  std::vector<int> type_absorb;       // gas identifier of each absorber (runes maps gases by name)
  std::vector<int> drop_scheme, ice_scheme;   // scheme of each droplet / ice type, 0 where undefined
  std::vector<double> drop_min_dim, drop_max_dim, ice_min_dim, ice_max_dim;   // their ranges of validity [m]
  int n_cloud_parameter = 0;          // coefficients per parameter set in the spectrum
  std::vector<int> n_k_major;         // k-terms of each band's first absorber (McICA tables)
  std::vector<int> band_overlap;      // the gas overlap method each band names, 0 where none
  // classic aerosol species (block 11): parametrization, humidities and
  // phase-function moments of each, for validation
  std::vector<int> aer_parm, aer_nhum, aer_nphf;
  std::vector<int> aer_type;          // type numbers of the species
  std::vector<int> aer_parm_file;     // parametrizations as the spectral file gives them
  int aer_nd_species = 0;             // the species extent of the aerosol arrays
  int device = 0;
};

SpectrumEntry *find_spectrum(int handle);
// the gas overlap of a call: the control's, or under ip_overlap_hybrid the
// method every band of the call names in the spectral file (0 when they
// differ or name none; radiance_calc.F90:888-893)
int gas_overlap(const socgpu_control *c, const SpectrumEntry *sp);
bool triple_cloud(int i_cloud);
bool region_cloud(int i_cloud);
bool is_keqv(const socgpu_control *c, const SpectrumEntry *sp);

int validate(const socgpu_control *c, const socgpu_dimen *dm, const SpectrumEntry *sp, const socgpu_atm *atm,
             const socgpu_cld *cld, const socgpu_aer *aer, const socgpu_bound *bd, const socgpu_radout *out,
             char *msg, size_t msg_len);
void fill_params(FluxParams &p, const socgpu_control *c, const socgpu_dimen *dm, const SpectrumEntry *sp,
                 const socgpu_atm *atm, const socgpu_cld *cld, const socgpu_aer *aer, const socgpu_bound *bd,
                 socgpu_radout *out, const double *weight_band_dev);
int mode_index(const socgpu_control *c);
TileConfig choose_tile(int precision, int mode, int n_layer);
// The built-in tile of the scan kernels (flux_kernel), for launches the
// phased kernel does not take (persistent multi-batch classes).
TileConfig scan_tile(int precision, int n_layer);

using LaunchFn = int (*)(const FluxParams &, const TileConfig &, cudaStream_t, char *, size_t);
using PrepareFn = int (*)(BatchGroup &, char *, size_t);
struct FluxVariant {
  int precision, mode, lanes;
  LaunchFn launch;
  PrepareFn prepare;
  int (*preload)();
};
const FluxVariant *find_variant(int precision, int mode, int lanes);
// Loads every scan-kernel variant onto the current device (once per process
// and device); returns 0 or a SOCGPU_I_* status.
int preload_kernels();

// The kernel parameters of columns c0 .. c0+n-1 of a launch (every
// per-column pointer moved by c0; the leading extents stay).
void window_params(FluxParams &p, int c0, int n);

// One launch of a single batch (tile from choose_tile).
int launch(const FluxParams &p, const socgpu_control *c, cudaStream_t st, char *msg, size_t msg_len);

// A plan of device copies: each host array gets a 256-byte aligned slot.
struct Slot {
  const void *host;
  void *out_host;
  size_t off, rows, row_bytes, host_pitch, dev_pitch;
  bool output;
  bool per_profile;   // rows of (profile) columns, split by column windows
};

struct Plan {
  std::vector<Slot> slots;
  size_t bytes = 0;
  // Add an array of `rows` rows of `n_valid` elements each, with leading
  // (Fortran) extent nd in host memory; on the device the same extent is kept.
  size_t add(const void *host, size_t esize, size_t nd, size_t n_valid, size_t rows, bool output = false,
             void *out_host = nullptr, bool per_profile = true) {
    if (!host && !out_host) return (size_t)-1;
    size_t off = (bytes + 255) & ~(size_t)255;
    Slot s{host, out_host, off, rows, n_valid * esize, nd * esize, nd * esize, output, per_profile};
    slots.push_back(s);
    bytes = off + nd * esize * rows;
    return off;
  }
};

// A host-pointer radiance_calc staged through device memory: which arrays
// the chosen path reads (the plan), their copy in, the kernel parameters
// over the device copies, and the copy out of the results.  The structs
// passed to stage() must outlive the object.
struct StagedCall {
  Plan plan;
  size_t n_inputs = 0;
  const socgpu_control *control = nullptr;
  const socgpu_dimen *dimen = nullptr;
  const SpectrumEntry *sp = nullptr;
  const socgpu_atm *atm = nullptr;
  const socgpu_cld *cld = nullptr;
  const socgpu_aer *aer = nullptr;
  const socgpu_bound *bound = nullptr;
  socgpu_radout *radout = nullptr;
  bool sw = false, mc = false, aero = false, classic = false;
  size_t o_p, o_t, o_tl, o_m, o_g, o_rho, o_z, o_si, o_alb, o_tg, o_amr, o_aab, o_asc, o_aas, o_wb, o_fg = (size_t)-1;
  size_t o_xmr = (size_t)-1, o_mrh = (size_t)-1;   // classic aerosol mixing ratios, mean relative humidity
  bool prsc = false;                                // prescribed aerosol properties
  size_t o_pp = (size_t)-1, o_pab = (size_t)-1, o_psc = (size_t)-1, o_pph = (size_t)-1;
  size_t o_cmr, o_cdc, o_wc, o_fc, o_cs, o_fcl, o_nsc, o_sk, o_fsk, o_sro;
  size_t o_fu, o_fd, o_fdir, o_div, o_hr;

  void stage(const socgpu_control *c, const socgpu_dimen *dm, const SpectrumEntry *s, const socgpu_atm *a,
             const socgpu_cld *cl, const socgpu_aer *ae, const socgpu_bound *b, socgpu_radout *r);
  int copy_in(char *base, cudaStream_t s, char *msg, size_t msg_len) const;
  void params(char *base, FluxParams &p) const;
  int copy_out(char *base, cudaStream_t s, char *msg, size_t msg_len) const;
  // Copies of the column window c0 .. c0+n-1 only; `shared`: the arrays
  // that are not per column (copied once).
  int copy_in_window(char *base, cudaStream_t s, size_t c0, size_t n, bool shared, char *msg,
                     size_t msg_len) const;
  int copy_out_window(char *base, cudaStream_t s, size_t c0, size_t n, char *msg, size_t msg_len) const;
  long long column_gpoints() const;
};

}  // namespace socgpu
