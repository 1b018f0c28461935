/*
 * socrates_oracle.h -- FP64 CPU restatement of the SOCRATES two-stream flux
 * path.  TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the
 * CPU-baseline leg of bench.py as the checker.  The product path never links
 * or calls it.
 *
 * Parity status: pinned to the reference's own known-good outputs.  The
 * reference (Fortran) cannot be compiled here, but its example runs ship
 * printed results, and this restatement reproduces them to half a unit of
 * the printed last digit (tests/test_oracle.py): ICRCCM case 27 (HadCM3
 * long wave, random overlap, continuum), CIRC case 6 with the GA7 long-wave
 * file (lookup-table k, Wen-Yi terms, k_eqv_scl), the runes test with the
 * GA9 files (solar and three thermal surfaces), the McICA example 5118_142
 * (GA3.0 and GA7, long and short wave) and the cloud-region example 7460_28
 * (HadGEM1 and GA9).  Parts no example exercises (the modal aerosol, the
 * synthetic power-law spectra) are checked against analytic known answers
 * and by reading against the reference source.
 */
#ifndef SOCRATES_ORACLE_H
#define SOCRATES_ORACLE_H

#include "socgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* radiance_calc restated for the clear-sky and McICA two-stream paths. */
int oracle_radiance_calc(const socgpu_control *control, const socgpu_dimen *dimen,
                         const socgpu_spectrum_desc *spec, const socgpu_atm *atm,
                         const socgpu_cld *cld, const socgpu_aer *aer,
                         const socgpu_bound *bound, socgpu_radout *radout,
                         char *msg, size_t msg_len);

/* Same, parallel over contiguous column segments with OpenMP (the way the
 * host model calls radiance_calc per segment).  n_threads <= 0: default. */
int oracle_radiance_calc_segmented(const socgpu_control *control, const socgpu_dimen *dimen,
                                   const socgpu_spectrum_desc *spec, const socgpu_atm *atm,
                                   const socgpu_cld *cld, const socgpu_aer *aer,
                                   const socgpu_bound *bound, socgpu_radout *radout,
                                   int n_threads, char *msg, size_t msg_len);

/* cloud_gen restated (socrates_cloud_gen.F90:8-470); rng selects the
 * reference LCG or the Philox stream. */
int oracle_cloud_gen(int nd_layer, int cloud_top, int n_layer, int nd_profile,
                     int il1, int il2, int n_subcol, int n1, int n2,
                     int ipph, int ioverlap, const int *rand_seed,
                     const double *rlc_cf, const double *rlc_cw,
                     const double *sigma_qcw, const double *avg_cf,
                     const double *c_cloud, const double *c_ratio,
                     const double *zf, const double *xcw,
                     int *n_subcol_cld, double *c_sub, int rng);

/* Philox4x32-10 block: counter (4 words) and key (2 words) -> 4 words. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif

#endif
