/*
 * socrates_oracle.c -- FP64 CPU restatement of the SOCRATES two-stream flux
 * path (clear sky and McICA).  TEST INFRASTRUCTURE ONLY: the checker for the
 * CUDA path and the CPU baseline of the benchmark.  Nothing in the product
 * library links it.
 *
 * Each function restates one reference routine and cites it; paths are
 * relative to the SOCRATES source tree.  Loop order follows the reference
 * (band -> k-term -> [subcolumn] -> layer -> profile, profile innermost) so
 * that FP64 results agree to rounding.  Build with -ffp-contract=off: the
 * reference is compiled without fused multiply-add contraction on x86.
 *
 * Parity is unpinned against reference-produced numbers (no Fortran
 * compiler here; the reference's own fixtures need lookup-table scaling,
 * continua and k_eqv_scl overlap).  See socrates_oracle.h.
 */
#include "socrates_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EPS_R  DBL_EPSILON   /* EPSILON(1.0_RealK) */
#define TINY_R DBL_MIN       /* TINY(1.0_RealK) */

/* rad_ccf.F90:44,50,56 */
static const double seconds_per_day = 8.64e4;
static const double cp_air_dry = 1.005e3;
/* diffusivity_factor.F90:16 */
static const double elsasser_factor = 1.66;
/* two_coeff_basic.F90:87 */
static const double root_3 = 1.7320508075688772;

/* Fortran-layout index helpers (1-based in the reference, 0-based here). */
#define IX2(a, l, i, nd1) ((a)[(size_t)(l) + (size_t)(nd1) * (size_t)(i)])
#define IX3(a, l, i, j, nd1, nd2) \
    ((a)[(size_t)(l) + (size_t)(nd1) * ((size_t)(i) + (size_t)(nd2) * (size_t)(j))])

static void set_msg(char *msg, size_t len, const char *text)
{
    if (msg && len > 0) {
        strncpy(msg, text, len - 1);
        msg[len - 1] = '\0';
    }
}

/* --------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of the
 * 4x32 bijection with the published multipliers and Weyl key steps.      */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* --------------------------------------------------------------------- */
/* Spectral accessors on the flat Fortran arrays of socgpu_spectrum_desc. */
static int sp_index_absorb(const socgpu_spectrum_desc *d, int j, int b)
{   /* index_absorb(nd_species, nd_band): 1-based species -> 0-based */
    return IX2(d->index_absorb, j, b, d->nd_species) - 1;
}
static int sp_bg(const int *a, const socgpu_spectrum_desc *d, int b, int g) { return IX2(a, b, g, d->nd_band); }
static double sp_kw(const double *a, const socgpu_spectrum_desc *d, int k, int b, int g)
{ return IX3(a, k, b, g, d->nd_k_term, d->nd_band); }
static const double *sp_scale(const socgpu_spectrum_desc *d, int k, int b, int g)
{
    return d->scale + (size_t)d->nd_scale_variable *
        ((size_t)k + (size_t)d->nd_k_term * ((size_t)b + (size_t)d->nd_band * (size_t)g));
}

/* --------------------------------------------------------------------- */
/* scale_absorb (scale_absorb.F90:110-281): pressure/temperature scaling
 * factor of one absorber for all cells of the segment.                  */
static int scale_absorb(int n_profile, int n_layer, int ndp_in, int ndp_w,
                        const double *p, const double *t, double *gfr,
                        int i_fnc, double p_reference, double t_reference,
                        const double *sp, int l_doppler, double doppler_correction,
                        const socgpu_spectrum_desc *d, int iex, int i_band)
{
    double pressure_offset = l_doppler ? doppler_correction : 0.0;
    if (i_fnc == SOCGPU_IP_SCALE_WENYI) {
        /* scale_absorb.F90:238-281: bilinear interpolation in ln(p/100 Pa)
         * and T of the CO2 (band 4) or O3 (band 6) tables; iex is the
         * 0-based k-term, i_band the 1-based band */
        if (!d->wenyi_plg) return SOCGPU_I_ERR_FATAL;
        int n_t, t_shift, nterm;
        const double *gk, *tt;
        if (i_band == 4) { n_t = 10; t_shift = 7; gk = d->wenyi_gk4; tt = d->wenyi_ttb; nterm = d->wenyi_n_term4; }
        else if (i_band == 6) { n_t = 9; t_shift = 5; gk = d->wenyi_gk6; tt = d->wenyi_tto; nterm = d->wenyi_n_term6; }
        else return SOCGPU_I_ERR_FATAL;
        if (!gk || !tt || iex >= nterm || (i_band == 4 && !d->wenyi_gk250b)) return SOCGPU_I_ERR_FATAL;
#define GK(a, b) gk[(size_t)((a) - 1) + (size_t)n_t * ((size_t)((b) - 1) + 26u * (size_t)iex)]
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                double pl = IX2(p, l, i, ndp_in), tl = IX2(t, l, i, ndp_in);
                double cgp = log(pl / 100.0);
                if (cgp < -5.5) cgp = -5.5;
                int jp = (int)((5.5 + cgp) * 2.0) + 1;
                jp = jp < 1 ? 1 : (jp > 26 ? 26 : jp);
                int jp1 = jp + 1 < 26 ? jp + 1 : 26;
                int jt = (int)((tl - 240.0) / 20.0 + (double)t_shift);
                jt = jt < 1 ? 1 : (jt > n_t ? n_t : jt);
                int jt1 = jt + 1 < n_t ? jt + 1 : n_t;
                double dp = (cgp - d->wenyi_plg[jp - 1]) * 2.0;
                double gkpb = GK(jt, jp) + (GK(jt, jp1) - GK(jt, jp)) * dp;
                double gkpc = GK(jt1, jp) + (GK(jt1, jp1) - GK(jt1, jp)) * dp;
                double v = gkpb + (gkpc - gkpb) * (tl - tt[jt - 1]) / 20.0;
                IX2(gfr, l, i, ndp_w) = (i_band == 4) ? v / d->wenyi_gk250b[iex] : v;
            }
#undef GK
        return SOCGPU_I_NORMAL;
    }
    if (i_fnc == SOCGPU_IP_SCALE_POWER_LAW) {
        /* scale_absorb.F90:122-137: ((p+off)/(pref+off))**sp1 * (t/tref)**sp2 */
        double t_inv = 1.0 / t_reference;
        double p_ref_off_inv = 1.0 / (p_reference + pressure_offset);
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                double pwk_in = (IX2(p, l, i, ndp_in) + pressure_offset) * p_ref_off_inv;
                double twk_in = IX2(t, l, i, ndp_in) * t_inv;
                IX2(gfr, l, i, ndp_w) = pow(pwk_in, sp[0]) * pow(twk_in, sp[1]);
            }
    } else if (i_fnc == SOCGPU_IP_SCALE_FNC_NULL) {
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) IX2(gfr, l, i, ndp_w) = 1.0;
    } else if (i_fnc == SOCGPU_IP_SCALE_POWER_QUAD) {
        /* scale_absorb.F90:170-186 */
        double p_ref_off_inv = 1.0 / (p_reference + pressure_offset);
        double t_inv = 1.0 / t_reference;
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                double pwk = pow((IX2(p, l, i, ndp_in) + pressure_offset) * p_ref_off_inv, sp[0]);
                double tmp = IX2(t, l, i, ndp_in) * t_inv - 1.0;
                IX2(gfr, l, i, ndp_w) = pwk * (1.0 + tmp * sp[1] + sp[2] * tmp * tmp);
            }
    } else if (i_fnc == SOCGPU_IP_SCALE_DOPPLER_QUAD) {
        /* scale_absorb.F90:208-224 */
        double t_inv = 1.0 / t_reference;
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                double pwk = pow((IX2(p, l, i, ndp_in) + sp[1]) / (p_reference + sp[1]), sp[0]);
                double tmp = IX2(t, l, i, ndp_in) * t_inv - 1.0;
                IX2(gfr, l, i, ndp_w) = pwk * (1.0 + tmp * sp[2] + sp[3] * tmp * tmp);
            }
    } else {
        return SOCGPU_I_ERR_FATAL;
    }
    return SOCGPU_I_NORMAL;
}

/* planck_flux_band (planck_flux_band_mod.F90:33-48), polynomial branch. */
static double planck_flux_band(const socgpu_spectrum_desc *d, int b, double temperature)
{
    double t_ratio = temperature / d->t_ref_planck;
    const double *c = d->thermal_coeff + (size_t)d->nd_thermal_coeff * (size_t)b;
    double f = c[d->n_deg_fit];
    for (int j = d->n_deg_fit - 1; j >= 0; --j) f = f * t_ratio + c[j];
    return f;
}

/* --------------------------------------------------------------------- */
/* Two-stream coefficients of one cell.                                   */

/* two_coeff_basic (two_coeff_basic.F90:99-160). */
static int two_coeff_basic(int i_2stream, double omega, double asym, double *sum, double *diff)
{
    switch (i_2stream) {
    case SOCGPU_IP_EDDINGTON:
        *sum = 1.5 * (1.0 - omega * asym); *diff = 2.0 * (1.0 - omega); break;
    case SOCGPU_IP_ELSASSER:
        *sum = elsasser_factor - 1.5 * omega * asym; *diff = elsasser_factor * (1.0 - omega); break;
    case SOCGPU_IP_DISCRETE_ORD:
        *sum = root_3 * (1.0 - omega * asym); *diff = root_3 * (1.0 - omega); break;
    case SOCGPU_IP_PIFM85:
        *sum = 2.0 - 1.5 * omega * asym; *diff = 2.0 * (1.0 - omega); break;
    case SOCGPU_IP_2S_TEST:
        *sum = 1.5 - 1.5 * omega * asym; *diff = 1.5 * (1.0 - omega); break;
    case SOCGPU_IP_HEMI_MEAN:
        *sum = 2.0 * (1.0 - omega * asym); *diff = 2.0 * (1.0 - omega); break;
    case SOCGPU_IP_PIFM80:
        *sum = 2.0 - 1.5 * omega * asym - 0.5 * omega; *diff = 2.0 * (1.0 - omega); break;
    default:
        return SOCGPU_I_ERR_FATAL;
    }
    return SOCGPU_I_NORMAL;
}

typedef struct { double trans, reflect, trans_0, trans_0_dir, sc1, sc2; } coeffs;

/* two_coeff (two_coeff.F90:148-188) -> solar_coefficient_basic
 * (solar_coefficient_basic.F90:124-219) -> trans_source_coeff
 * (trans_source_coeff.F90:144-263).  sc1/sc2 are the solar (up, down) or
 * IR (1d, 2d) source coefficients. */
static void two_coeff_cell(int isolir, int i_2stream, int i_direct_tau, int l_ir_source_quad,
                           double asym, double omega, double tau_dir, double tau, double sec_0,
                           coeffs *o)
{
    double sum = 0.0, diff = 0.0;
    two_coeff_basic(i_2stream, omega, asym, &sum, &diff);
    double lambda = sqrt(sum * diff);
    double gamma_up = 0.0, gamma_down = 0.0;
    if (isolir == SOCGPU_IP_SOLAR) {
        double tol_perturb = 3.2e1 * EPS_R;
        if (fabs(lambda - sec_0) < tol_perturb) {
            sum = (1.0 + tol_perturb) * sum;
            diff = (1.0 + tol_perturb) * diff;
            lambda = (1.0 + tol_perturb) * lambda;
        }
        double ksi_0 = (i_2stream == SOCGPU_IP_DISCRETE_ORD) ? root_3 * asym / sec_0
                                                            : 1.5 * asym / sec_0;
        double factor = 0.5 * omega * sec_0 / ((lambda - sec_0) * (lambda + sec_0));
        gamma_up = factor * (sum - sec_0 - ksi_0 * (diff - sec_0));
        gamma_down = factor * (sum + sec_0 + ksi_0 * (diff + sec_0));
    }
    double sq_eps_r = sqrt(EPS_R), tol = sqrt(sq_eps_r);
    double exponential = exp(-lambda * tau);
    double exponential2 = exponential * exponential;
    double gamma = (sum - lambda) / (sum + lambda);
    double gamma2 = gamma * gamma;
    double tmp_inv = 1.0 / (1.0 - exponential2 * gamma2);
    o->trans = exponential * (1.0 - gamma2) * tmp_inv;
    o->reflect = gamma * (1.0 - exponential2) * tmp_inv;
    o->trans_0 = 0.0; o->trans_0_dir = 0.0; o->sc2 = 0.0;
    if (isolir == SOCGPU_IP_SOLAR) {
        o->trans_0 = exp(-tau * sec_0);
        if (i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING || i_direct_tau == SOCGPU_IP_DIRECT_CSR_SCALING)
            o->trans_0_dir = exp(-tau_dir * sec_0);
        o->sc1 = (gamma_up - o->reflect * (1.0 + gamma_down)) - gamma_up * o->trans * o->trans_0;
        o->sc2 = o->trans_0 * (1.0 + gamma_down - gamma_up * o->reflect) - (1.0 + gamma_down) * o->trans;
    } else {
        o->sc1 = (1.0 - o->trans + o->reflect + sq_eps_r) / (sq_eps_r + tau * sum);
        if (l_ir_source_quad) {
            double s2;
            if (tau > tol) s2 = -2.0 * (1.0 - o->trans - o->reflect + sq_eps_r) / (diff * tau + sq_eps_r);
            else s2 = -2.0 + diff * tau;
            o->sc2 = -(1.0 + o->reflect + o->trans + s2) / (sum * tau + sq_eps_r);
        }
    }
}

/* two_coeff_fast_lw (two_coeff_fast_lw.F90:112-154). */
static void two_coeff_fast_lw_cell(int l_ir_source_quad, double tau, coeffs *o)
{
    double sq_eps_r = sqrt(EPS_R), tol = sqrt(sq_eps_r);
    o->trans = exp(-1.66 * tau);
    o->reflect = 0.0; o->trans_0 = 0.0; o->trans_0_dir = 0.0; o->sc2 = 0.0;
    o->sc1 = (1.0 - o->trans + sq_eps_r) / (1.66 * tau + sq_eps_r);
    if (l_ir_source_quad) {
        if (tau > tol) o->sc2 = -(1.0 + o->trans - 2.0 * o->sc1) / (1.66 * tau + sq_eps_r);
        else o->sc2 = -(1.0 + o->trans - 2.0 + 1.66 * tau) / (1.66 * tau + sq_eps_r);
    }
}

/* single_scattering (single_scattering.F90:119-164), the direct-beam depth
 * (monochromatic_radiance.F90:459-475) and rescale_tau_omega
 * (rescale_tau_omega.F90:73-80) for one cell. */
static void single_scatter_cell(const socgpu_control *c, double k_grey_tot, double k_ext_scat,
                                double k_gas_abs, double d_mass, double fwd,
                                double *tau, double *tau_dir, double *omega)
{
    int m = c->i_scatter_method;
    if (m == SOCGPU_IP_SCATTER_FULL) {
        double k_total = k_grey_tot + k_gas_abs;
        *tau = k_total * d_mass;
        *omega = k_ext_scat / (k_total + TINY_R);
        double cap = 1.0 - 3.2e1 * EPS_R;
        if (*omega > cap) *omega = cap;
    } else if (m == SOCGPU_IP_NO_SCATTER_ABS) {
        *tau = (k_grey_tot + k_gas_abs - k_ext_scat) * d_mass;
        *omega = 0.0;
    } else {
        *tau = (k_grey_tot + k_gas_abs) * d_mass;
        *omega = 0.0;
    }
    *tau_dir = *tau;
    if (c->l_rescale) {
        *tau = *tau * (1.0 - *omega * fwd);
        *omega = *omega * (1.0 - fwd) / (1.0 - *omega * fwd);
    }
}

/* --------------------------------------------------------------------- */
/* Workspace of one column segment.  Work arrays use the segment's own
 * leading dimension `wp`; caller arrays keep dimen->nd_profile.          */
typedef struct {
    int wp, ndl, n_profile, n_layer;
    double *k_grey_tot, *k_ext_scat, *phase_fnc, *forward_scatter, *cont_amount;
    double *phase_fnc_nc, *forward_scatter_nc;
    double *k_ext_tot_cc, *k_ext_scat_cc, *phf_cc, *fwd_cc;   /* per cloud component */
    double *gfr;                                              /* per absorber of the band */
    double *k_gas_abs;
    double *planck_flux, *planck_diff, *planck_diff_2, *flux_ground;
    double *flux_inc_down, *flux_inc_direct, *d_planck_flux_surface;
    double *sec_0, *alb_diff, *alb_dir;
    double *tau, *tau_dir, *omega;
    double *trans, *reflect, *trans_0, *trans_0_dir, *sc1, *sc2;
    double *trans_clr, *reflect_clr, *trans_0_clr, *trans_0_dir_clr, *sc1_clr, *sc2_clr;
    double *s_up, *s_down, *source_ground;
    double *flux_direct, *flux_direct_dir, *flux_total;
    double *flux_direct_acc, *flux_total_acc, *flux_direct_clear, *flux_total_clear;
    double *alpha, *s_up_prime, *beta, *gam, *h;
    double *ty_tau[3], *ty_tau_dir[3], *ty_omega[3], *ty_asym[3];      /* cloud types 1..2 */
    double *ty_valid[3];
    /* cloud regions (mix_column): cloudy-region coefficients and sources,
     * the solver's elimination coefficients, the interface coefficients */
    double *tc, *rc, *t0c, *t0dc, *sc1c, *sc2c, *s_up_c, *s_down_c;
    double *b11, *b21, *b22, *g11, *g12, *g21, *g22, *h1, *h2, *ovl;
    /* three regions (triple_column): the convective region's coefficients
     * and sources (the stratiform region uses the cloudy-region arrays
     * above), its elimination coefficients, the regions' fractions of the
     * cloud, and the direct flux and sources at the ground of the two
     * cloudy regions */
    double *tv, *rv, *t0v, *t0dv, *sc1v, *sc2v, *s_up_v, *s_down_v;
    double *b33, *g33, *h3, *fr2, *fr3, *fdg2, *fdg3, *sg2, *sg3;
    int nct;                    /* n_cloud_top, 1-based */
    int *slot;
    const double *adj;          /* adjust_solar_ke of k_eqv_scl (solar), or NULL */
} work;

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* Interface coefficients kept per (profile, interface): two regions use
 * 8 (overlap_coupled2), three use 18 (overlap_coupled3). */
#define OVS 18

#define WORK_FIELDS(X) \
    X(k_grey_tot, pl) X(k_ext_scat, pl) X(phase_fnc, pl) X(forward_scatter, pl) \
    X(phase_fnc_nc, pl) X(forward_scatter_nc, pl) \
    X(k_ext_tot_cc, pl * nc) X(k_ext_scat_cc, pl * nc) X(phf_cc, pl * nc) X(fwd_cc, pl * nc) \
    X(gfr, pl * na) X(k_gas_abs, pl) \
    X(planck_flux, pl1) X(planck_diff, pl) X(planck_diff_2, pl) X(flux_ground, wp) \
    X(flux_inc_down, wp) X(flux_inc_direct, wp) X(d_planck_flux_surface, wp) \
    X(sec_0, wp) X(alb_diff, wp) X(alb_dir, wp) \
    X(tau, pl) X(tau_dir, pl) X(omega, pl) \
    X(trans, pl) X(reflect, pl) X(trans_0, pl) X(trans_0_dir, pl) X(sc1, pl) X(sc2, pl) \
    X(trans_clr, pl) X(reflect_clr, pl) X(trans_0_clr, pl) X(trans_0_dir_clr, pl) X(sc1_clr, pl) X(sc2_clr, pl) \
    X(s_up, pl) X(s_down, pl) X(source_ground, wp) \
    X(flux_direct, pl1) X(flux_direct_dir, pl1) X(flux_total, pl2) \
    X(flux_direct_acc, pl1) X(flux_total_acc, pl2) X(flux_direct_clear, pl1) X(flux_total_clear, pl2) \
    X(alpha, wp) X(s_up_prime, wp) X(beta, pl) X(gam, pl) X(h, pl) X(cont_amount, pl) \
    X(tc, pl) X(rc, pl) X(t0c, pl) X(t0dc, pl) X(sc1c, pl) X(sc2c, pl) X(s_up_c, pl) X(s_down_c, pl) \
    X(b11, pl) X(b21, pl) X(b22, pl) X(g11, pl) X(g12, pl) X(g21, pl) X(g22, pl) X(h1, pl) X(h2, pl) \
    X(ovl, pl1 * OVS) \
    X(tv, pl) X(rv, pl) X(t0v, pl) X(t0dv, pl) X(sc1v, pl) X(sc2v, pl) X(s_up_v, pl) X(s_down_v, pl) \
    X(b33, pl) X(g33, pl) X(h3, pl) X(fr2, pl) X(fr3, pl) X(fdg2, wp) X(fdg3, wp) X(sg2, wp) X(sg3, wp)

static void work_init(work *w, int wp, int ndl, int n_profile, int n_layer, int nc, int na)
{
    size_t pl = (size_t)wp * ndl, pl1 = (size_t)wp * (ndl + 1), pl2 = (size_t)wp * (2 * ndl + 2);
    memset(w, 0, sizeof(*w));
    w->wp = wp; w->ndl = ndl; w->n_profile = n_profile; w->n_layer = n_layer;
    if (nc < 1) nc = 1;
    if (na < 1) na = 1;
#define ALLOC_F(name, n) w->name = zalloc(n);
    WORK_FIELDS(ALLOC_F)
#undef ALLOC_F
    for (int t = 0; t < 3; ++t) {
        w->ty_tau[t] = zalloc(pl); w->ty_tau_dir[t] = zalloc(pl);
        w->ty_omega[t] = zalloc(pl); w->ty_asym[t] = zalloc(pl); w->ty_valid[t] = zalloc(pl);
    }
    w->slot = (int *)calloc((size_t)wp, sizeof(int));
}

static void work_free(work *w)
{
#define FREE_F(name, n) free(w->name); w->name = NULL;
    WORK_FIELDS(FREE_F)
#undef FREE_F
    for (int t = 0; t < 3; ++t) {
        free(w->ty_tau[t]); free(w->ty_tau_dir[t]); free(w->ty_omega[t]);
        free(w->ty_asym[t]); free(w->ty_valid[t]);
    }
    free(w->slot);
}

/* --------------------------------------------------------------------- */
/* Column solve of one monochromatic problem for all profiles of the
 * segment: ir_source (ir_source.F90:93-119), solar_source
 * (solar_source.F90:105-176), column_solver (column_solver.F90:160-243),
 * solver_homogen_direct (solver_homogen_direct.F90:94-131) and
 * solver_no_scat (solver_no_scat.F90:75-94).
 * flux_total(l, m) of the reference is IX2(flux_total, l, m-1, wp). */
static void column_solve(work *w, const socgpu_control *c, int no_scat)
{
    int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp;
    double *fd = w->flux_direct, *ft = w->flux_total;
    if (c->isolir == SOCGPU_IP_INFRA_RED) {
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                if (c->l_ir_source_quad) {
                    IX2(w->s_up, l, i, wp) = IX2(w->sc1, l, i, wp) * IX2(w->planck_diff, l, i, wp)
                        + IX2(w->sc2, l, i, wp) * IX2(w->planck_diff_2, l, i, wp);
                    IX2(w->s_down, l, i, wp) = -IX2(w->sc1, l, i, wp) * IX2(w->planck_diff, l, i, wp)
                        + IX2(w->sc2, l, i, wp) * IX2(w->planck_diff_2, l, i, wp);
                } else {
                    IX2(w->s_up, l, i, wp) = IX2(w->sc1, l, i, wp) * IX2(w->planck_diff, l, i, wp);
                    IX2(w->s_down, l, i, wp) = -IX2(w->s_up, l, i, wp);
                }
            }
        for (int l = 0; l < n_profile; ++l)
            w->source_ground[l] = (1.0 - w->alb_diff[l]) * w->d_planck_flux_surface[l];
        for (int i = 0; i <= n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) IX2(fd, l, i, wp) = 0.0;
    } else {
        int l_dir = (c->i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING ||
                     c->i_direct_tau == SOCGPU_IP_DIRECT_CSR_SCALING);
        for (int l = 0; l < n_profile; ++l) {
            IX2(fd, l, 0, wp) = w->flux_inc_direct[l];
            if (l_dir) IX2(w->flux_direct_dir, l, 0, wp) = w->flux_inc_direct[l];
        }
        if (w->adj) {
            /* l_scale_solar (solar_source.F90:115-130) */
            for (int i = 1; i <= n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    IX2(fd, l, i, wp) = IX2(fd, l, i - 1, wp) * IX2(w->trans_0, l, i - 1, wp) * IX2(w->adj, l, i - 1, wp);
                    IX2(w->s_up, l, i - 1, wp) = IX2(w->sc1, l, i - 1, wp) * IX2(fd, l, i - 1, wp);
                    IX2(w->s_down, l, i - 1, wp) = (IX2(w->sc2, l, i - 1, wp) - IX2(w->trans_0, l, i - 1, wp))
                        * IX2(fd, l, i - 1, wp) + IX2(fd, l, i, wp);
                }
        } else {
            for (int i = 1; i <= n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    IX2(fd, l, i, wp) = IX2(fd, l, i - 1, wp) * IX2(w->trans_0, l, i - 1, wp);
                    IX2(w->s_up, l, i - 1, wp) = IX2(w->sc1, l, i - 1, wp) * IX2(fd, l, i - 1, wp);
                    IX2(w->s_down, l, i - 1, wp) = IX2(w->sc2, l, i - 1, wp) * IX2(fd, l, i - 1, wp);
                }
        }
        if (l_dir) {
            for (int i = 1; i <= n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    IX2(w->flux_direct_dir, l, i, wp) =
                        IX2(w->flux_direct_dir, l, i - 1, wp) * IX2(w->trans_0_dir, l, i - 1, wp);
                    if (w->adj) IX2(w->flux_direct_dir, l, i, wp) = IX2(w->flux_direct_dir, l, i, wp) * IX2(w->adj, l, i - 1, wp);
                }
            for (int i = 0; i <= n_layer; ++i)
                for (int l = 0; l < n_profile; ++l)
                    IX2(fd, l, i, wp) = IX2(w->flux_direct_dir, l, i, wp);
        }
        for (int l = 0; l < n_profile; ++l)
            w->source_ground[l] = (w->alb_dir[l] - w->alb_diff[l]) * IX2(fd, l, n_layer, wp);
    }

    if (no_scat) {
        for (int l = 0; l < n_profile; ++l) IX2(ft, l, 1, wp) = w->flux_inc_down[l];
        for (int i = 1; i <= n_layer; ++i)
            for (int l = 0; l < n_profile; ++l)
                IX2(ft, l, 2 * i + 1, wp) = IX2(w->s_down, l, i - 1, wp)
                    + IX2(w->trans, l, i - 1, wp) * IX2(ft, l, 2 * i - 1, wp);
        for (int l = 0; l < n_profile; ++l)
            IX2(ft, l, 2 * n_layer, wp) = (1.0 - w->alb_diff[l]) * w->d_planck_flux_surface[l]
                + w->alb_diff[l] * IX2(ft, l, 2 * n_layer + 1, wp);
        for (int i = n_layer; i >= 1; --i)
            for (int l = 0; l < n_profile; ++l)
                IX2(ft, l, 2 * i - 2, wp) = IX2(w->s_up, l, i - 1, wp)
                    + IX2(w->trans, l, i - 1, wp) * IX2(ft, l, 2 * i, wp);
    } else {
        for (int l = 0; l < n_profile; ++l) {
            w->alpha[l] = w->alb_diff[l];
            w->s_up_prime[l] = w->source_ground[l];
        }
        for (int ii = n_layer - 1; ii >= 0; --ii)
            for (int l = 0; l < n_profile; ++l) {
                double r = IX2(w->reflect, l, ii, wp), t = IX2(w->trans, l, ii, wp);
                double beta = 1.0 / (1.0 - w->alpha[l] * r);
                double gam = w->alpha[l] * t;
                double h = w->s_up_prime[l] + w->alpha[l] * IX2(w->s_down, l, ii, wp);
                IX2(w->beta, l, ii, wp) = beta; IX2(w->gam, l, ii, wp) = gam; IX2(w->h, l, ii, wp) = h;
                w->alpha[l] = r + beta * gam * t;
                w->s_up_prime[l] = IX2(w->s_up, l, ii, wp) + beta * t * h;
            }
        for (int l = 0; l < n_profile; ++l) {
            IX2(ft, l, 1, wp) = w->flux_inc_down[l];
            IX2(ft, l, 0, wp) = w->alpha[l] * IX2(ft, l, 1, wp) + w->s_up_prime[l];
        }
        for (int i = 1; i <= n_layer; ++i) {
            int ii = i - 1;
            for (int l = 0; l < n_profile; ++l) {
                IX2(ft, l, 2 * i, wp) = IX2(w->beta, l, ii, wp)
                    * (IX2(w->h, l, ii, wp) + IX2(w->gam, l, ii, wp) * IX2(ft, l, 2 * i - 1, wp));
                IX2(ft, l, 2 * i + 1, wp) = IX2(w->s_down, l, ii, wp)
                    + IX2(w->trans, l, ii, wp) * IX2(ft, l, 2 * i - 1, wp)
                    + IX2(w->reflect, l, ii, wp) * IX2(ft, l, 2 * i, wp);
            }
        }
    }
}

/* Clear (type 0) optical properties and two-stream coefficients of one
 * k-term (monochromatic_radiance.F90:429-528, two_stream.F90:166-206 for the
 * coefficient part). */
static void clear_coefficients(work *w, const socgpu_control *c, const double *mass, int ndp_in)
{
    int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp;
    int no_scat = (c->i_scatter_method != SOCGPU_IP_SCATTER_FULL);
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < n_profile; ++l) {
            double tau, tau_dir, om;
            single_scatter_cell(c, IX2(w->k_grey_tot, l, i, wp), IX2(w->k_ext_scat, l, i, wp),
                                IX2(w->k_gas_abs, l, i, wp), IX2(mass, l, i, ndp_in),
                                IX2(w->forward_scatter, l, i, wp), &tau, &tau_dir, &om);
            IX2(w->tau, l, i, wp) = tau; IX2(w->tau_dir, l, i, wp) = tau_dir; IX2(w->omega, l, i, wp) = om;
        }
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < n_profile; ++l) {
            coeffs o;
            if (no_scat)
                two_coeff_fast_lw_cell(c->l_ir_source_quad, IX2(w->tau, l, i, wp), &o);
            else
                two_coeff_cell(c->isolir, c->i_2stream, c->i_direct_tau, c->l_ir_source_quad,
                               IX2(w->phase_fnc, l, i, wp), IX2(w->omega, l, i, wp),
                               IX2(w->tau_dir, l, i, wp), IX2(w->tau, l, i, wp), w->sec_0[l], &o);
            IX2(w->trans, l, i, wp) = o.trans; IX2(w->reflect, l, i, wp) = o.reflect;
            IX2(w->trans_0, l, i, wp) = o.trans_0; IX2(w->trans_0_dir, l, i, wp) = o.trans_0_dir;
            IX2(w->sc1, l, i, wp) = o.sc1; IX2(w->sc2, l, i, wp) = o.sc2;
        }
}

/* --------------------------------------------------------------------- */
/* Grey optical properties of one band (grey_opt_prop.F90:470-920,
 * 1010-1030, 1390-1450; opt_prop_ukca_aerosol.F90:128-208;
 * rescale_phase_fnc.F90:120-128 as called at radiance_calc.F90:996-1017).
 * Cloud-component optics through opt_prop_pade_2
 * (opt_prop_pade_2_mod.F90:99-140, the rescaled n_order_forward=2 path of
 * opt_prop_water_cloud.F90:212-219 and opt_prop_ice_cloud.F90:228-236),
 * Slingo and Schrecker's fits (opt_prop_water_cloud.F90:231-247,
 * opt_prop_ice_cloud.F90:278-294) and Fu's ice fits
 * (opt_prop_fu_phf_mod.F90:92-130). */
/* Physical constants (rad_ccf.F90:42-58, gas_list_pcf.F90:303-306). */
#define MOL_WEIGHT_AIR 28.966e-03
#define REPSILON (18.0153 / 28.966)

static int cloud_scheme_known(int phase, int scheme)
{
    if (phase == SOCGPU_IP_PHASE_WATER) return scheme == SOCGPU_IP_SLINGO_SCHRECKER || scheme == SOCGPU_IP_DROP_PADE_2;
    if (phase == SOCGPU_IP_PHASE_ICE)
        return scheme == SOCGPU_IP_SLINGO_SCHRECKER_ICE || scheme == SOCGPU_IP_ICE_FU_PHF ||
               scheme == SOCGPU_IP_ICE_PADE_2_PHF;
    return 0;
}

/* Extinction, scattering and asymmetry of one cloud component of mass
 * fraction q and characteristic dimension re under scheme `scheme` with the
 * coefficients cp of its type in this band; 0 when the scheme is not one of
 * these. */
static int cloud_component_optics(int phase, int scheme, const double *cp, double q, double re,
                                  double *ke, double *ks, double *g)
{
    if ((phase == SOCGPU_IP_PHASE_WATER && scheme == SOCGPU_IP_SLINGO_SCHRECKER) ||
        (phase == SOCGPU_IP_PHASE_ICE && scheme == SOCGPU_IP_SLINGO_SCHRECKER_ICE)) {
        *ke = q * (cp[0] + cp[1] / re);
        *ks = *ke * (1.0e+00 - cp[2] - cp[3] * re);
        *g = cp[4] + cp[5] * re;
        return 1;
    }
    if ((phase == SOCGPU_IP_PHASE_WATER && scheme == SOCGPU_IP_DROP_PADE_2) ||
        (phase == SOCGPU_IP_PHASE_ICE && scheme == SOCGPU_IP_ICE_PADE_2_PHF)) {
        *ke = q * (cp[0] + re * (cp[1] + re * cp[2])) / (1.0e+00 + re * (cp[3] + re * (cp[4] + re * cp[5])));
        *ks = *ke * (1.0e+00 - (cp[6] + re * (cp[7] + re * cp[8])) / (1.0e+00 + re * (cp[9] + re * cp[10])));
        *g = (cp[11] + re * (cp[12] + re * cp[13])) / (1.0e+00 + re * (cp[14] + re * cp[15]));
        return 1;
    }
    if (phase == SOCGPU_IP_PHASE_ICE && scheme == SOCGPU_IP_ICE_FU_PHF) {
        double x = cp[3] / re;
        *ke = q * ((cp[2] * x + cp[1]) * x + cp[0]);
        x = re / cp[8];
        *ks = *ke * (1.0e+00 - (cp[4] + x * (cp[5] + x * (cp[6] + x * cp[7]))));
        x = re / cp[13];
        *g = cp[9] + x * (cp[10] + x * (cp[11] + x * cp[12]));
        return 1;
    }
    return 0;
}

/* rescale_continuum (rescale_continuum.F90): amount of continuum j of band
 * b in every layer, from the p/T scaling and the water vapour. */
static void rescale_continuum(const socgpu_control *c, const socgpu_spectrum_desc *d, const socgpu_atm *atm,
                              int ndp, int ndl, int n_profile, int n_layer, int b, int j, double *amount, int wp)
{
    const int ndb = d->nd_band, ndc = d->nd_continuum;
    const int i_cont = d->index_continuum[b + ndb * j];
    const int fnc = d->i_scale_fnc_cont[b + ndb * j];
    const double p_ref = d->p_ref_cont[j + ndc * b], t_ref = d->t_ref_cont[j + ndc * b];
    const double *sc = d->scale_cont + (size_t)d->nd_scale_variable * ((size_t)b + (size_t)ndb * j);
    const int iw = d->index_water - 1;
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < n_profile; ++l) {
            double p = IX2(atm->p, l, i, ndp), t = IX2(atm->t, l, i, ndp);
            double a = pow(p / p_ref, sc[0]);
            if (fnc == SOCGPU_IP_SCALE_POWER_LAW) a = a * pow(t / t_ref, sc[1]);
            else if (fnc == SOCGPU_IP_SCALE_POWER_QUAD) {
                double x = t / t_ref - 1.0e+00;
                a = a * (1.0e+00 + sc[1] * x + sc[2] * (x * x));
            }
            double water = IX3(atm->gas_mix_ratio, l, i, iw, ndp, ndl);
            double rho = IX2(atm->density, l, i, ndp);
            if (i_cont == SOCGPU_IP_SELF_CONTINUUM) {
                double molar_density_water = rho * water / (REPSILON * MOL_WEIGHT_AIR);
                a = a * molar_density_water * water;
            } else if (i_cont == SOCGPU_IP_FRN_CONTINUUM) {
                if (c->l_mixing_ratio) a = a * rho * water / MOL_WEIGHT_AIR;
                else a = a * rho * water * (1.0 - water) / MOL_WEIGHT_AIR;
            }
            IX2(amount, l, i, wp) = a;
        }
}

/* spline_fit.F90: second derivatives of the natural cubic spline through
 * (x[k], y[k]) by tridiagonal elimination (the reference leaves y2 unset for
 * one point; spline_at never reads it then). */
static void spline_fit(int n, const double *x, const double *y, double *y2)
{
    if (n == 1) { y2[0] = 0.0; return; }
    double *u = (double *)malloc(sizeof(double) * (size_t)n);
    y2[0] = 0.0;
    u[0] = 0.0;
    for (int i = 1; i < n - 1; ++i) {
        const double sigma = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
        const double rho = sigma * y2[i - 1] + 2.0;
        y2[i] = (sigma - 1.0) / rho;
        u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]))
                / (x[i + 1] - x[i - 1]) - sigma * u[i - 1]) / rho;
    }
    y2[n - 1] = 0.0;
    for (int i = n - 2; i >= 0; --i) y2[i] = y2[i] * y2[i + 1] + u[i];
    free(u);
}

/* spline_evaluate.F90: the spline at xp (bisection for the interval); 1 when
 * xp lies outside [x[0], x[n-1]] (the reference's i_err_range). */
static int spline_at(int n, const double *x, const double *y, const double *y2, double xp, double *yp)
{
    if (n == 1) { *yp = y[0]; return 0; }
    if (xp > x[n - 1] || xp < x[0]) return 1;
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int m = (lo + hi) / 2;
        if (xp > x[m]) lo = m; else hi = m;
    }
    const double delta = x[hi] - x[lo];
    const double a = (x[hi] - xp) / delta, bb = (xp - x[lo]) / delta, cc = delta * delta / 6.0;
    *yp = a * (y[lo] + (a * a - 1.0) * y2[lo] * cc) + bb * (y[hi] + (bb * bb - 1.0) * y2[hi] * cc);
    return 0;
}

/* prsc_gather_spline.F90: one prescribed quantity of species j (values v of
 * stride `st` between levels, from the profile's first level) at the layer
 * pressures of profile l; zero outside the levels. */
static void prsc_gather(int nl, const double *x, const double *v, size_t st, const double *p, int ndp, int l,
                        int n_layer, double *out)
{
    double *y = (double *)malloc(sizeof(double) * (size_t)nl), *y2 = (double *)malloc(sizeof(double) * (size_t)nl);
    for (int k = 0; k < nl; ++k) y[k] = v[(size_t)k * st];
    spline_fit(nl, x, y, y2);
    for (int i = 0; i < n_layer; ++i)
        if (spline_at(nl, x, y, y2, IX2(p, l, i, ndp), &out[i])) out[i] = 0.0;
    free(y); free(y2);
}

/* prsc_opt_prop.F90:165-300 for two-stream phase functions: species j's
 * prescribed absorption and scattering (volume coefficients over the air
 * density, floored at zero) and its asymmetry or tabulated moments, added to
 * the grey optics of band b. */
static void prsc_opt_prop(work *w, const socgpu_control *c, const socgpu_dimen *dm, const socgpu_spectrum_desc *d,
                          const socgpu_atm *atm, const socgpu_aer *aer, int j, int b)
{
    const int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp, ndp = dm->nd_profile;
    const size_t ndpp = (size_t)dm->nd_profile_aerosol_prsc, ndlv = (size_t)dm->nd_opt_level_aerosol_prsc;
    const size_t ndf = (size_t)dm->nd_phf_term_aerosol_prsc, nsp = (size_t)d->nd_aerosol_species;
    const int nl = aer->n_opt_level_prsc[j], nof = c->n_order_forward;
    double *x = (double *)malloc(sizeof(double) * (size_t)nl);
    double *ka = (double *)malloc(sizeof(double) * (size_t)n_layer), *ks = (double *)malloc(sizeof(double) * (size_t)n_layer);
    double *g = (double *)malloc(sizeof(double) * (size_t)n_layer), *f = (double *)malloc(sizeof(double) * (size_t)n_layer);
#define PRSC_AT(a, l, k) (a)[(size_t)(l) + ndpp * ((size_t)(k) + ndlv * ((size_t)j + nsp * (size_t)b))]
#define PRSC_PHF(l, m) &aer->phase_fnc_prsc[(size_t)(l) + ndpp * (ndlv * ((size_t)(m) + ndf * ((size_t)j + nsp * (size_t)b)))]
    for (int l = 0; l < n_profile; ++l) {
        for (int k = 0; k < nl; ++k) x[k] = aer->pressure_prsc[(size_t)l + ndpp * ((size_t)k + ndlv * (size_t)j)];
        prsc_gather(nl, x, &PRSC_AT(aer->absorption_prsc, l, 0), ndpp, atm->p, ndp, l, n_layer, ka);
        prsc_gather(nl, x, &PRSC_AT(aer->scattering_prsc, l, 0), ndpp, atm->p, ndp, l, n_layer, ks);
        for (int i = 0; i < n_layer; ++i) {
            const double rho = IX2(atm->density, l, i, ndp);
            ks[i] = fmax(0.0, ks[i] / rho);
            ka[i] = fmax(0.0, ka[i] / rho);
        }
        prsc_gather(nl, x, PRSC_PHF(l, 0), ndpp, atm->p, ndp, l, n_layer, g);
        if (c->l_rescale && !c->l_henyey_greenstein_pf)
            prsc_gather(nl, x, PRSC_PHF(l, nof - 1), ndpp, atm->p, ndp, l, n_layer, f);
        for (int i = 0; i < n_layer; ++i) {
            IX2(w->k_grey_tot, l, i, wp) = IX2(w->k_grey_tot, l, i, wp) + ka[i];
            IX2(w->k_ext_scat, l, i, wp) = IX2(w->k_ext_scat, l, i, wp) + ks[i];
            const double phf1 = ks[i] * g[i];
            IX2(w->phase_fnc, l, i, wp) = IX2(w->phase_fnc, l, i, wp) + phf1;
            if (c->l_rescale) {
                double fw;
                if (!c->l_henyey_greenstein_pf) fw = ks[i] * f[i];
                else if (nof == 1) fw = phf1;
                else if (nof == 2) fw = phf1 * g[i];
                else fw = ks[i] * pow(g[i], (double)nof);
                IX2(w->forward_scatter, l, i, wp) = IX2(w->forward_scatter, l, i, wp) + fw;
            }
        }
    }
#undef PRSC_AT
#undef PRSC_PHF
    free(x); free(ka); free(ks); free(g); free(f);
}

/* opt_prop_aerosol (opt_prop_aerosol.F90:273-640), two-stream phase
 * functions (n_order_phase 1), for band b: every radiatively active entry of
 * the mixing ratios adds its species' absorption and scattering, interpolated
 * in the mean relative humidity for moist species, the asymmetry to the first
 * phase-function moment and, with rescaling, the forward-scattering moment.
 * The humidity pointer follows radiance_calc.F90:603-623 (one table, that of
 * the last moist species of the spectrum); it is clamped to the table, where
 * the reference would read past it for a humidity of 1. */
static int opt_prop_aerosol(work *w, const socgpu_control *c, const socgpu_dimen *dm,
                            const socgpu_spectrum_desc *d, const socgpu_atm *atm, const socgpu_aer *aer, int b)
{
    const int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp, ndl = w->ndl, ndp = dm->nd_profile;
    const int ndh = d->nd_humidity, nda = d->nd_aerosol_species, ndf = d->nd_phase_term;
    if (d->n_aerosol <= 0 || !d->i_aerosol_parm || !d->aerosol_abs || !d->aerosol_scat || !d->aerosol_phf)
        return SOCGPU_I_ERR_FATAL;
    int nhc = 0;
    for (int j = 0; j < d->n_aerosol; ++j)
        if (d->i_aerosol_parm[j] == SOCGPU_IP_AEROSOL_PARAM_MOIST ||
            d->i_aerosol_parm[j] == SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST)
            nhc = d->nhumidity[j];
    const double delta_humidity = nhc > 1 ? 1.0e+00 / ((double)nhc - 1.0e+00) : 0.0;
    for (int jm = 0; jm < aer->n_aerosol_mr; ++jm) {
        const int src = aer->mr_source ? aer->mr_source[jm] : SOCGPU_IP_AERSRC_CLASSIC_RON;
        if (src != SOCGPU_IP_AERSRC_CUSACK_RON && src != SOCGPU_IP_AERSRC_CLASSIC_RON && src != SOCGPU_IP_AERSRC_ARCL_RON)
            continue;
        const int j = aer->mr_type_index[jm] - 1;
        if (j < 0 || j >= d->n_aerosol) return SOCGPU_I_ERR_RANGE;
        const int parm = d->i_aerosol_parm[j];
        if (parm == SOCGPU_IP_AEROSOL_UNPARAMETRIZED) {
            /* opt_prop_aerosol.F90:714-790 */
            if (!aer->n_opt_level_prsc || !aer->n_phase_term_prsc || !aer->pressure_prsc || !aer->absorption_prsc ||
                !aer->scattering_prsc || !aer->phase_fnc_prsc || !atm->density)
                return SOCGPU_I_ERR_FATAL;
            const int need = (c->l_henyey_greenstein_pf || !c->l_rescale) ? 1 :
                             (c->n_order_forward > 1 ? c->n_order_forward : 1);
            if (aer->n_opt_level_prsc[j] < 1 || aer->n_opt_level_prsc[j] > dm->nd_opt_level_aerosol_prsc ||
                aer->n_phase_term_prsc[j] < need || aer->n_phase_term_prsc[j] > dm->nd_phf_term_aerosol_prsc ||
                dm->nd_profile_aerosol_prsc < n_profile)
                return SOCGPU_I_ERR_RANGE;
            prsc_opt_prop(w, c, dm, d, atm, aer, j, b);
            continue;
        }
        const int moist = parm == SOCGPU_IP_AEROSOL_PARAM_MOIST || parm == SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST;
        const int hg = c->l_henyey_greenstein_pf || parm == SOCGPU_IP_AEROSOL_PARAM_DRY ||
                       parm == SOCGPU_IP_AEROSOL_PARAM_MOIST;
        if (!hg && parm != SOCGPU_IP_AEROSOL_PARAM_PHF_DRY && parm != SOCGPU_IP_AEROSOL_PARAM_PHF_MOIST)
            return SOCGPU_I_ERR_FATAL;
        if (moist && (nhc < 2 || !aer->mean_rel_humidity || !d->aerosol_humidities)) return SOCGPU_I_ERR_FATAL;
#define AEROSOL_PHF(h, m) d->aerosol_phf[(size_t)(h) + (size_t)ndh * ((size_t)(m) + (size_t)ndf * ((size_t)j + (size_t)nda * b))]
#define AEROSOL_TAB(a, h) (a)[(size_t)(h) + (size_t)ndh * ((size_t)j + (size_t)nda * b)]
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                const double mmr = aer->mix_ratio[(size_t)l + (size_t)ndp * ((size_t)i + (size_t)ndl * jm)];
                int ip = 0;            /* 0-based i_pointer - 1 */
                double weight_upper = 0.0;
                if (moist) {
                    const double mrh = IX2(aer->mean_rel_humidity, l, i, ndp);
                    int i_pointer = 1 + (int)(mrh * (nhc - 1));
                    if (i_pointer < 1) i_pointer = 1;
                    if (i_pointer > nhc - 1) i_pointer = nhc - 1;
                    ip = i_pointer - 1;
                    weight_upper = (mrh - d->aerosol_humidities[(size_t)ip + (size_t)ndh * j]) / delta_humidity;
                }
                double ab = AEROSOL_TAB(d->aerosol_abs, ip), sc = AEROSOL_TAB(d->aerosol_scat, ip);
                double g = AEROSOL_PHF(ip, 0);
                if (moist) {
                    ab = ab + weight_upper * (AEROSOL_TAB(d->aerosol_abs, ip + 1) - AEROSOL_TAB(d->aerosol_abs, ip));
                    sc = sc + weight_upper * (AEROSOL_TAB(d->aerosol_scat, ip + 1) - AEROSOL_TAB(d->aerosol_scat, ip));
                    g = g + weight_upper * (AEROSOL_PHF(ip + 1, 0) - AEROSOL_PHF(ip, 0));
                }
                IX2(w->k_grey_tot, l, i, wp) = IX2(w->k_grey_tot, l, i, wp) + mmr * ab;
                const double k_scatter = mmr * sc;
                IX2(w->k_ext_scat, l, i, wp) = IX2(w->k_ext_scat, l, i, wp) + k_scatter;
                IX2(w->phase_fnc, l, i, wp) = IX2(w->phase_fnc, l, i, wp) + k_scatter * g;
                if (c->l_rescale) {
                    double f;
                    if (!hg) {
                        const int m = c->n_order_forward - 1;
                        f = AEROSOL_PHF(ip, m);
                        if (moist) f = f + weight_upper * (AEROSOL_PHF(ip + 1, m) - AEROSOL_PHF(ip, m));
                        f = k_scatter * f;
                    } else if (c->n_order_forward == 1) {
                        f = k_scatter * g;
                    } else if (c->n_order_forward == 2) {
                        f = k_scatter * g * g;
                    } else {
                        f = k_scatter * pow(g, (double)c->n_order_forward);
                    }
                    IX2(w->forward_scatter, l, i, wp) = IX2(w->forward_scatter, l, i, wp) + f;
                }
            }
#undef AEROSOL_PHF
#undef AEROSOL_TAB
    }
    return SOCGPU_I_NORMAL;
}

static int grey_opt_prop(work *w, const socgpu_control *c, const socgpu_dimen *dm,
                         const socgpu_spectrum_desc *d, const socgpu_atm *atm, const socgpu_aer *aer,
                         const socgpu_cld *cld, int b, int l_cloud)
{
    int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp, ndl = w->ndl;
    int ndp = dm->nd_profile;
    size_t pl = (size_t)wp * ndl;
    for (size_t q = 0; q < pl; ++q) {
        w->k_grey_tot[q] = 0.0; w->k_ext_scat[q] = 0.0;
        w->phase_fnc[q] = 0.0; w->forward_scatter[q] = 0.0;
    }
    if (c->l_rayleigh) {
        if (d->i_rayleigh_scheme != SOCGPU_IP_RAYLEIGH_TOTAL || !d->rayleigh_coeff) return SOCGPU_I_ERR_FATAL;
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) IX2(w->k_ext_scat, l, i, wp) = d->rayleigh_coeff[b];
    }
    if (c->l_aerosol && aer && aer->n_aerosol_mr > 0) {
        int st = opt_prop_aerosol(w, c, dm, d, atm, aer, b);
        if (st != SOCGPU_I_NORMAL) return st;
    }
    if (c->l_aerosol_mode && aer && aer->n_mode > 0) {
        int ndm = dm->nd_aerosol_mode;
        for (int j = 0; j < aer->n_mode; ++j)
            for (int i = 0; i < n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    double mmr = IX3(aer->mode_mix_ratio, l, i, j, ndp, ndl);
                    size_t q4 = (size_t)l + (size_t)ndp * ((size_t)i + (size_t)ndl *
                                                           ((size_t)j + (size_t)ndm * (size_t)b));
                    double g = aer->mode_asymmetry[q4];
                    IX2(w->k_grey_tot, l, i, wp) = IX2(w->k_grey_tot, l, i, wp) + mmr * aer->mode_absorption[q4];
                    double k_scatter = mmr * aer->mode_scattering[q4];
                    IX2(w->k_ext_scat, l, i, wp) = IX2(w->k_ext_scat, l, i, wp) + k_scatter;
                    IX2(w->phase_fnc, l, i, wp) = IX2(w->phase_fnc, l, i, wp) + k_scatter * g;
                    if (c->l_rescale) {
                        double ks_phf = k_scatter * g;
                        if (c->n_order_forward == 1)
                            IX2(w->forward_scatter, l, i, wp) = IX2(w->forward_scatter, l, i, wp) + ks_phf;
                        else if (c->n_order_forward == 2)
                            IX2(w->forward_scatter, l, i, wp) = IX2(w->forward_scatter, l, i, wp) + ks_phf * g;
                        else
                            IX2(w->forward_scatter, l, i, wp) = IX2(w->forward_scatter, l, i, wp)
                                + k_scatter * pow(g, (double)c->n_order_forward);
                    }
                }
    }
    /* continuum absorption (grey_opt_prop.F90:801-817) */
    if (c->l_continuum && d->n_band_continuum) {
        for (int j = 0; j < d->n_band_continuum[b]; ++j) {
            const double kc = d->k_cont[b + d->nd_band * j];
            rescale_continuum(c, d, atm, ndp, ndl, n_profile, n_layer, b, j, w->cont_amount, wp);
            for (int i = 0; i < n_layer; ++i)
                for (int l = 0; l < n_profile; ++l)
                    IX2(w->k_grey_tot, l, i, wp) = IX2(w->k_grey_tot, l, i, wp) + kc * IX2(w->cont_amount, l, i, wp);
        }
    }
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < n_profile; ++l)
            IX2(w->k_grey_tot, l, i, wp) = IX2(w->k_grey_tot, l, i, wp) + IX2(w->k_ext_scat, l, i, wp);

    if (l_cloud) {
        memcpy(w->phase_fnc_nc, w->phase_fnc, pl * sizeof(double));
        memcpy(w->forward_scatter_nc, w->forward_scatter, pl * sizeof(double));
    }
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < n_profile; ++l) {
            double ks = IX2(w->k_ext_scat, l, i, wp);
            if (ks > TINY_R) {
                if (c->l_rescale) {
                    double tmp_inv = 1.0 / ks;
                    IX2(w->forward_scatter, l, i, wp) = IX2(w->forward_scatter, l, i, wp) * tmp_inv;
                    IX2(w->phase_fnc, l, i, wp) = IX2(w->phase_fnc, l, i, wp) * tmp_inv;
                } else {
                    IX2(w->phase_fnc, l, i, wp) = IX2(w->phase_fnc, l, i, wp) / ks;
                }
            }
        }
    if (c->l_rescale)
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                double f = IX2(w->forward_scatter, l, i, wp);
                IX2(w->phase_fnc, l, i, wp) = (IX2(w->phase_fnc, l, i, wp) - f) / (1.0 - f);
            }

    if (l_cloud) {
        int ict = dm->id_cloud_top - 1, ndc = ndl - ict;
        for (int k = 0; k < cld->n_condensed; ++k) {
            const double *cp0;
            int ity = cld->i_condensed_type[k] - 1;
            /* stratiform or convective water (ip_clcmp 1, 3) or ice (2, 4), rad_pcf.F90:187-193 */
            const int tc = cld->type_condensed[k];
            const int phase = (tc == 1 || tc == 3) ? SOCGPU_IP_PHASE_WATER : (tc == 2 || tc == 4) ? SOCGPU_IP_PHASE_ICE : tc;
            const int scheme = cld->i_condensed_param[k];
            if (phase == SOCGPU_IP_PHASE_WATER) {
                if (!d->drop_parm_list || ity < 0 || ity >= d->nd_drop_type) return SOCGPU_I_ERR_FATAL;
                cp0 = d->drop_parm_list + (size_t)d->nd_cloud_parameter * ((size_t)b + (size_t)d->nd_band * (size_t)ity);
            } else {
                if (!d->ice_parm_list || ity < 0 || ity >= d->nd_ice_type) return SOCGPU_I_ERR_FATAL;
                cp0 = d->ice_parm_list + (size_t)d->nd_cloud_parameter * ((size_t)b + (size_t)d->nd_band * (size_t)ity);
            }
            if (!cloud_scheme_known(phase, scheme)) return SOCGPU_I_ERR_FATAL;
            double *kext = w->k_ext_tot_cc + pl * k, *kscat = w->k_ext_scat_cc + pl * k;
            double *phf = w->phf_cc + pl * k, *fwd = w->fwd_cc + pl * k;
            for (int i = ict; i < n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    size_t qc = (size_t)l + (size_t)ndp * (size_t)(i - ict);
                    double q = cld->condensed_mix_ratio[qc + (size_t)ndp * ndc * k];
                    double re = cld->condensed_dim_char[qc + (size_t)ndp * ndc * k];
                    double ke = 0.0, ks = 0.0, g = 0.0;
                    if (re > 0.0) cloud_component_optics(phase, scheme, cp0, q, re, &ke, &ks, &g);
                    IX2(kext, l, i, wp) = ke;
                    IX2(kscat, l, i, wp) = ks;
                    IX2(phf, l, i, wp) = ks * g;
                    IX2(fwd, l, i, wp) = ks * g * g;
                }
        }
    }
    return SOCGPU_I_NORMAL;
}

/* --------------------------------------------------------------------- */
/* McICA: one k-term of one band (mcica_sample.F90:453-925 with
 * mcica_column.F90:261-602).  Leaves the blended fluxes in flux_direct and
 * flux_total. */
static void solve_mcica_term(work *w, const socgpu_control *c, const socgpu_dimen *dm,
                             const socgpu_spectrum_desc *d, const double *mass,
                             const socgpu_cld *cld, int b, int iex)
{
    int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp, ndl = w->ndl;
    int ndp = dm->nd_profile;
    int no_scat = (c->i_scatter_method != SOCGPU_IP_SCATTER_FULL);
    int ict = dm->id_cloud_top - 1, ndc = ndl - ict;
    size_t pl = (size_t)wp * ndl, pl1 = (size_t)wp * (ndl + 1), pl2 = (size_t)wp * (2 * ndl + 2);
    const double eps = EPS_R;   /* mcica_sample.F90:440 */
    int first = IX2(cld->first_subcol_k, b, iex, d->nd_band);
    int last = IX2(cld->first_subcol_k, b, iex + 1, d->nd_band) - 1;
    double subcol_k_inv = 1.0 / (double)IX2(cld->subcol_k, b, iex, d->nd_band);

    /* clear coefficients (type 0): identical for every subcolumn */
    clear_coefficients(w, c, mass, ndp);
    memcpy(w->trans_clr, w->trans, pl * sizeof(double));
    memcpy(w->reflect_clr, w->reflect, pl * sizeof(double));
    memcpy(w->trans_0_clr, w->trans_0, pl * sizeof(double));
    memcpy(w->trans_0_dir_clr, w->trans_0_dir, pl * sizeof(double));
    memcpy(w->sc1_clr, w->sc1, pl * sizeof(double));
    memcpy(w->sc2_clr, w->sc2, pl * sizeof(double));

    for (int m = first; m <= last; ++m) {
        int index_subcol = m % cld->n_subcol_req;
        if (index_subcol == 0) index_subcol = cld->n_subcol_req;
        index_subcol = cld->subcol_reorder[index_subcol - 1];
        /* per-profile subcolumn slot, with the fill of set_cld_mcica
         * (socrates_set_cld_mcica.F90:206-220) applied on the fly when the
         * compacted cloud_gen output is given */
        for (int l = 0; l < n_profile; ++l) {
            int j = index_subcol;
            if (cld->n_subcol_cld) {
                int ncld = cld->n_subcol_cld[l];
                int nfill = cld->n_subcol_req < cld->n_subcol_gen ? cld->n_subcol_req : cld->n_subcol_gen;
                if (ncld > 0 && j > ncld && j <= nfill) j = (j - 1) % ncld + 1;
            }
            w->slot[l] = j - 1;
        }
#define CSUB_AT(qc, l) (cld->c_sub[(qc) + (size_t)ndp * ndc * (size_t)w->slot[l]])

        if (m == first) {
            /* the clear solve (mcica_column.F90:309-327, l_clear) */
            column_solve(w, c, no_scat);
            memcpy(w->flux_direct_clear, w->flux_direct, pl1 * sizeof(double));
            memcpy(w->flux_total_clear, w->flux_total, pl2 * sizeof(double));
        }
        /* cloudy-type optics (mcica_sample.F90:472-700): each type starts
         * from the clear-sky values and adds its components in order, scaled
         * by c_sub (one component per type under ip_cloud_ice_water, all of
         * them in type 1 under ip_cloud_homogen); then their optical depths
         * (single_scattering_all, rescale_tau_omega) */
        for (int t = 1; t <= 2; ++t)
            for (size_t q = 0; q < pl; ++q) w->ty_valid[t][q] = 0.0;
        for (int t = 1; t <= cld->n_cloud_type; ++t)
            for (int i = ict; i < n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    size_t qc = (size_t)l + (size_t)ndp * (size_t)(i - ict);
                    if (!(cld->w_cloud[qc] > 0.0)) continue;
                    double cs = CSUB_AT(qc, l);
                    double kgt = IX2(w->k_grey_tot, l, i, wp), kes = IX2(w->k_ext_scat, l, i, wp);
                    double fwd = IX2(w->forward_scatter_nc, l, i, wp), phf = IX2(w->phase_fnc_nc, l, i, wp);
                    for (int k = 0; k < cld->n_condensed; ++k) {
                        if (cld->i_cloud_type[k] != t) continue;
                        kgt = kgt + IX2(w->k_ext_tot_cc + pl * k, l, i, wp) * cs;
                        kes = kes + IX2(w->k_ext_scat_cc + pl * k, l, i, wp) * cs;
                        fwd = fwd + IX2(w->fwd_cc + pl * k, l, i, wp) * cs;
                        phf = phf + IX2(w->phf_cc + pl * k, l, i, wp) * cs;
                    }
                    double asym;
                    if (c->l_rescale) {
                        double den = kes - fwd;
                        asym = (phf - fwd) / (den > eps ? den : eps);
                        fwd = fwd / (kes > eps ? kes : eps);
                    } else {
                        fwd = 0.0;
                        asym = phf / (kes > eps ? kes : eps);
                    }
                    double tau, tau_dir, om;
                    single_scatter_cell(c, kgt, kes, IX2(w->k_gas_abs, l, i, wp),
                                        IX2(mass, l, i, ndp), fwd, &tau, &tau_dir, &om);
                    IX2(w->ty_tau[t], l, i, wp) = tau; IX2(w->ty_tau_dir[t], l, i, wp) = tau_dir;
                    IX2(w->ty_omega[t], l, i, wp) = om; IX2(w->ty_asym[t], l, i, wp) = asym;
                    IX2(w->ty_valid[t], l, i, wp) = 1.0;
                }
        /* mcica_column.F90:336-470: clear coefficients, then the cloudy
         * cells of this subcolumn get the frac_cloud-weighted cloudy ones */
        memcpy(w->trans, w->trans_clr, pl * sizeof(double));
        memcpy(w->reflect, w->reflect_clr, pl * sizeof(double));
        memcpy(w->trans_0, w->trans_0_clr, pl * sizeof(double));
        memcpy(w->trans_0_dir, w->trans_0_dir_clr, pl * sizeof(double));
        memcpy(w->sc1, w->sc1_clr, pl * sizeof(double));
        memcpy(w->sc2, w->sc2_clr, pl * sizeof(double));
        for (int t = 1; t <= cld->n_cloud_type; ++t)
            for (int i = ict; i < n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    size_t qc = (size_t)l + (size_t)ndp * (size_t)(i - ict);
                    double fc = cld->frac_cloud[qc + (size_t)ndp * ndc * (size_t)(t - 1)];
                    if (CSUB_AT(qc, l) * fc > 0.0) {
                        IX2(w->trans, l, i, wp) = 0.0; IX2(w->reflect, l, i, wp) = 0.0;
                        IX2(w->sc1, l, i, wp) = 0.0; IX2(w->sc2, l, i, wp) = 0.0;
                        if (c->isolir == SOCGPU_IP_SOLAR) {
                            IX2(w->trans_0, l, i, wp) = 0.0; IX2(w->trans_0_dir, l, i, wp) = 0.0;
                        }
                    }
                }
        for (int t = 1; t <= cld->n_cloud_type; ++t)
            for (int i = ict; i < n_layer; ++i)
                for (int l = 0; l < n_profile; ++l) {
                    size_t qc = (size_t)l + (size_t)ndp * (size_t)(i - ict);
                    double fc = cld->frac_cloud[qc + (size_t)ndp * ndc * (size_t)(t - 1)];
                    if (!(CSUB_AT(qc, l) * fc > 0.0) || IX2(w->ty_valid[t], l, i, wp) == 0.0) continue;
                    coeffs o;
                    if (no_scat)
                        two_coeff_fast_lw_cell(c->l_ir_source_quad, IX2(w->ty_tau[t], l, i, wp), &o);
                    else
                        two_coeff_cell(c->isolir, c->i_2stream, c->i_direct_tau, c->l_ir_source_quad,
                                       IX2(w->ty_asym[t], l, i, wp), IX2(w->ty_omega[t], l, i, wp),
                                       IX2(w->ty_tau_dir[t], l, i, wp), IX2(w->ty_tau[t], l, i, wp),
                                       w->sec_0[l], &o);
                    IX2(w->trans, l, i, wp) = IX2(w->trans, l, i, wp) + fc * o.trans;
                    IX2(w->reflect, l, i, wp) = IX2(w->reflect, l, i, wp) + fc * o.reflect;
                    IX2(w->sc1, l, i, wp) = IX2(w->sc1, l, i, wp) + fc * o.sc1;
                    if (c->isolir == SOCGPU_IP_SOLAR || c->l_ir_source_quad)
                        IX2(w->sc2, l, i, wp) = IX2(w->sc2, l, i, wp) + fc * o.sc2;
                    if (c->isolir == SOCGPU_IP_SOLAR) {
                        IX2(w->trans_0, l, i, wp) = IX2(w->trans_0, l, i, wp) + fc * o.trans_0;
                        if (c->i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING ||
                            c->i_direct_tau == SOCGPU_IP_DIRECT_CSR_SCALING)
                            IX2(w->trans_0_dir, l, i, wp) = IX2(w->trans_0_dir, l, i, wp) + fc * o.trans_0_dir;
                    }
                }
        column_solve(w, c, no_scat);
        /* mcica_sample.F90:793-860: accumulate the subcolumn fluxes */
        if (m == first) {
            memcpy(w->flux_direct_acc, w->flux_direct, pl1 * sizeof(double));
            memcpy(w->flux_total_acc, w->flux_total, pl2 * sizeof(double));
        } else {
            for (int i = 0; i <= n_layer; ++i)
                for (int l = 0; l < n_profile; ++l)
                    IX2(w->flux_direct_acc, l, i, wp) = IX2(w->flux_direct_acc, l, i, wp) + IX2(w->flux_direct, l, i, wp);
            for (int i = 0; i < 2 * n_layer + 2; ++i)
                for (int l = 0; l < n_profile; ++l)
                    IX2(w->flux_total_acc, l, i, wp) = IX2(w->flux_total_acc, l, i, wp) + IX2(w->flux_total, l, i, wp);
        }
    }
#undef CSUB_AT
    /* mcica_sample.F90:862-925: mean over subcolumns, blend with clear */
    if (c->isolir == SOCGPU_IP_SOLAR)
        for (int i = 0; i <= n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                double fc = cld->frac_cloudy[l];
                double v = IX2(w->flux_direct_acc, l, i, wp) * subcol_k_inv;
                IX2(w->flux_direct, l, i, wp) = fc * v + ((1.0 - fc) * IX2(w->flux_direct_clear, l, i, wp));
            }
    else
        for (int i = 0; i <= n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) IX2(w->flux_direct, l, i, wp) = 0.0;
    for (int i = 0; i < 2 * n_layer + 2; ++i)
        for (int l = 0; l < n_profile; ++l) {
            double fc = cld->frac_cloudy[l];
            double v = IX2(w->flux_total_acc, l, i, wp) * subcol_k_inv;
            IX2(w->flux_total, l, i, wp) = (fc * v) + ((1.0 - fc) * IX2(w->flux_total_clear, l, i, wp));
        }
}

/* --------------------------------------------------------------------- */
/* Lookup-table k scaling.  Interpolation factors of every cell of the
 * segment: inter_pt_lookup.F90:146-268 (pressure, temperature and gas
 * fraction) and inter_t_lookup.F90:70-86 (temperature only).  Indices are
 * stored 0-based. */
typedef struct {
    double *fac00, *fac01, *fac10, *fac11;   /* (wp, ndl) */
    int *jp, *jt, *jtt;                       /* (wp, ndl) */
    double *fgf; int *jgf, *jgfp1;            /* (wp, ndl, nd_species_sb) */
    double *wt_gas; int *jt_gas;              /* (wp, ndl, nd_species) */
} lookup_fac;

/* MINLOC(x - tab(1:n), MASK = x - tab >= 0): the first index of the smallest
 * non-negative difference, 0-based (0 when none qualifies; the clamps before
 * every call keep x inside the table). */
static int minloc_below(double x, const double *tab, int n)
{
    int best = -1;
    double dmin = 0.0;
    for (int k = 0; k < n; ++k) {
        double dd = x - tab[k];
        if (dd >= 0.0 && (best < 0 || dd < dmin)) { best = k; dmin = dd; }
    }
    return best < 0 ? 0 : best;
}

static void lookup_fac_free(lookup_fac *f)
{
    free(f->fac00); free(f->fac01); free(f->fac10); free(f->fac11);
    free(f->jp); free(f->jt); free(f->jtt);
    free(f->fgf); free(f->jgf); free(f->jgfp1); free(f->wt_gas); free(f->jt_gas);
    memset(f, 0, sizeof(*f));
}

static void lookup_fac_init(lookup_fac *f, const socgpu_control *c, const socgpu_spectrum_desc *d,
                            const socgpu_atm *atm, int np, int n_layer, int ndp, int wp, int ndl)
{
    memset(f, 0, sizeof(*f));
    int any_pt = 0, any_t = 0;
    for (int b = c->first_band - 1; b < c->last_band; ++b)
        for (int j = 0; j < d->n_band_absorb[b]; ++j) {
            int fnc = sp_bg(d->i_scale_fnc, d, b, sp_index_absorb(d, j, b));
            any_pt |= (fnc == SOCGPU_IP_SCALE_LOOKUP);
            any_t |= (fnc == SOCGPU_IP_SCALE_T_LOOKUP);
        }
    size_t pl = (size_t)wp * ndl;
    const double eps = EPS_R;
    if (any_pt && d->n_pre > 1 && d->n_tmp > 1 && d->p_lookup && d->t_lookup) {
        int npre = d->n_pre, ntmp = d->n_tmp;
        f->fac00 = zalloc(pl); f->fac01 = zalloc(pl); f->fac10 = zalloc(pl); f->fac11 = zalloc(pl);
        f->jp = (int *)calloc(pl, sizeof(int)); f->jt = (int *)calloc(pl, sizeof(int));
        f->jtt = (int *)calloc(pl, sizeof(int));
        double p_min = d->p_lookup[0] + fmax(fabs(d->p_lookup[0]) * eps, eps);
        double p_max = d->p_lookup[npre - 1] - fmax(fabs(d->p_lookup[npre - 1]) * eps, eps);
#define TL(it, ip) d->t_lookup[(size_t)(it) + (size_t)ntmp * (size_t)(ip)]
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < np; ++l) {
                double p_layer = fmin(fmax(log(IX2(atm->p, l, i, ndp)), p_min), p_max);
                int jp = minloc_below(p_layer, d->p_lookup, npre);
                double fp = (p_layer - d->p_lookup[jp]) / (d->p_lookup[jp + 1] - d->p_lookup[jp]);
                double t = IX2(atm->t, l, i, ndp);
                double t_layer = fmin(fmax(t, TL(0, jp) * (1.0 + eps)), TL(ntmp - 1, jp) * (1.0 - eps));
                int jt = minloc_below(t_layer, &TL(0, jp), ntmp);
                double ft = (t_layer - TL(jt, jp)) / (TL(jt + 1, jp) - TL(jt, jp));
                t_layer = fmin(fmax(t, TL(0, jp + 1) * (1.0 + eps)), TL(ntmp - 1, jp + 1) * (1.0 - eps));
                int jtt = minloc_below(t_layer, &TL(0, jp + 1), ntmp);
                double ftt = (t_layer - TL(jtt, jp + 1)) / (TL(jtt + 1, jp + 1) - TL(jtt, jp + 1));
                double compfp = 1.0 - fp;
                IX2(f->fac00, l, i, wp) = compfp * (1.0 - ft);
                IX2(f->fac10, l, i, wp) = fp * (1.0 - ftt);
                IX2(f->fac01, l, i, wp) = compfp * ft;
                IX2(f->fac11, l, i, wp) = fp * ftt;
                IX2(f->jp, l, i, wp) = jp; IX2(f->jt, l, i, wp) = jt; IX2(f->jtt, l, i, wp) = jtt;
            }
#undef TL
        /* gas fractions of the self-broadened absorbers (inter_pt_lookup.F90:198-266) */
        int nsb = d->nd_species_sb;
        if (d->index_sb && nsb > 0 && d->n_gas_frac >= 1 && d->gf_lookup) {
            int ngf = d->n_gas_frac;
            f->fgf = zalloc(pl * nsb);
            f->jgf = (int *)calloc(pl * nsb, sizeof(int));
            f->jgfp1 = (int *)calloc(pl * nsb, sizeof(int));
            double gf_min = d->gf_lookup[0] + fmax(d->gf_lookup[0] * eps, eps);
            double gf_max = d->gf_lookup[ngf - 1] - fmax(d->gf_lookup[ngf - 1] * eps, eps);
            int iw = d->index_water - 1;
            if (iw < 0) iw = 0;   /* i_pointer_water = MAX(index_water, 1) */
            int l_water = 0;
            double mw_w = 18.0153;
            for (int g = 0; g < d->n_absorb; ++g)
                if (d->type_absorb[g] == 1) {
                    l_water = 1;
                    if (d->molar_weight) mw_w = d->molar_weight[g];
                }
            for (int g = 0; g < d->n_absorb; ++g) {
                int jsb = d->index_sb[g] - 1;
                if (jsb < 0 || jsb >= nsb) continue;
                double mw_g = d->molar_weight ? d->molar_weight[g] : 0.0;
                double ratio_gas = MOL_WEIGHT_AIR / (mw_g * 1.0e-03);
                double ratio_water = MOL_WEIGHT_AIR / (mw_w * 1.0e-03);
                for (int i = 0; i < n_layer; ++i)
                    for (int l = 0; l < np; ++l) {
                        double mr = IX3(atm->gas_mix_ratio, l, i, g, ndp, ndl);
                        double gf;
                        if (l_water) {
                            double q = IX3(atm->gas_mix_ratio, l, i, iw, ndp, ndl);
                            gf = c->l_mixing_ratio ? mr * ratio_gas / (1.0 + q * ratio_water)
                                                   : mr * ratio_gas / (1.0 + q * (ratio_water - 1.0));
                        } else {
                            gf = mr * ratio_gas;
                        }
                        size_t q3 = (size_t)l + (size_t)wp * ((size_t)i + (size_t)ndl * jsb);
                        if (ngf == 1) {
                            f->jgf[q3] = 0; f->jgfp1[q3] = 0; f->fgf[q3] = 1.0;
                        } else {
                            double gl = fmin(fmax(gf, gf_min), gf_max);
                            int jg = minloc_below(gl, d->gf_lookup, ngf);
                            f->jgf[q3] = jg; f->jgfp1[q3] = jg + 1;
                            f->fgf[q3] = 1.0 - (gl - d->gf_lookup[jg]) / (d->gf_lookup[jg + 1] - d->gf_lookup[jg]);
                        }
                    }
            }
        }
    }
    if (any_t && d->n_t_lookup_gas && d->t_lookup_gas && d->nd_t_lookup_gas > 1) {
        int nsp = d->nd_species;
        f->wt_gas = zalloc(pl * nsp);
        f->jt_gas = (int *)calloc(pl * nsp, sizeof(int));
        for (int g = 0; g < d->n_absorb; ++g) {
            int n = d->n_t_lookup_gas[g];
            if (n < 2) continue;
            const double *tc = d->t_lookup_gas + (size_t)d->nd_t_lookup_gas * g;
            for (int i = 0; i < n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    double t_layer = fmin(fmax(IX2(atm->t, l, i, ndp), tc[0] * (1.0 + eps)), tc[n - 1] * (1.0 - eps));
                    int jt = minloc_below(t_layer, tc, n);
                    size_t q3 = (size_t)l + (size_t)wp * ((size_t)i + (size_t)ndl * g);
                    f->jt_gas[q3] = jt;
                    f->wt_gas[q3] = 1.0 - (t_layer - tc[jt]) / (tc[jt + 1] - tc[jt]);
                }
        }
    }
}

/* k_abs_layer(:, :, iex, j) of radiance_calc.F90:1330-1470 for absorber j
 * (species g) of band b: band-scaled amounts from gfr (ip_scale_band: the
 * scaled amount; ip_scale_null: the mixing ratio), per-term scaling through
 * scale_absorb, or the lookup tables (k_esft_layer of
 * radiance_calc.F90:1097-1170; k of block 5 is then unused).  tmp is a (wp,
 * ndl) scratch array. */
static int absorber_term_k(const lookup_fac *lf, const socgpu_spectrum_desc *d, const socgpu_atm *atm,
                           int np, int n_layer, int ndp, int wp, int ndl,
                           int b, int g, int iex, const double *gfr, double *tmp, double *kout)
{
    int isk = sp_bg(d->i_scale_k, d, b, g), fnc = sp_bg(d->i_scale_fnc, d, b, g);
    double kval = sp_kw(d->k, d, iex, b, g);
    if (isk != SOCGPU_IP_SCALE_TERM) {
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < np; ++l) IX2(kout, l, i, wp) = kval * IX2(gfr, l, i, wp);
        return SOCGPU_I_NORMAL;
    }
    if (fnc == SOCGPU_IP_SCALE_LOOKUP) {
        if (!lf->fac00) return SOCGPU_I_ERR_FATAL;
        int ntmp = d->n_tmp, npre = d->n_pre;
        int jsb = (d->index_sb && lf->fgf) ? d->index_sb[g] - 1 : -1;
        if (jsb < 0) {
            if (!d->k_lookup) return SOCGPU_I_ERR_FATAL;
            const double *K = d->k_lookup + (size_t)ntmp * npre *
                ((size_t)iex + (size_t)d->nd_k_term * ((size_t)g + (size_t)d->nd_species * b));
#define KL(it, ip) K[(size_t)(it) + (size_t)ntmp * (size_t)(ip)]
            for (int i = 0; i < n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    int jp = IX2(lf->jp, l, i, wp), jt = IX2(lf->jt, l, i, wp), jtt = IX2(lf->jtt, l, i, wp);
                    double ke = IX2(lf->fac00, l, i, wp) * KL(jt, jp) + IX2(lf->fac10, l, i, wp) * KL(jtt, jp + 1)
                        + IX2(lf->fac01, l, i, wp) * KL(jt + 1, jp) + IX2(lf->fac11, l, i, wp) * KL(jtt + 1, jp + 1);
                    ke = ke > 0.0 ? ke : 0.0;
                    double v = ke * IX3(atm->gas_mix_ratio, l, i, g, ndp, ndl);
                    IX2(kout, l, i, wp) = v > 0.0 ? v : 0.0;
                }
#undef KL
        } else {
            if (!d->k_lookup_sb) return SOCGPU_I_ERR_FATAL;
            int ngf = d->n_gas_frac;
            const double *K = d->k_lookup_sb + (size_t)ntmp * npre * ngf *
                ((size_t)iex + (size_t)d->nd_k_term * ((size_t)jsb + (size_t)d->nd_species_sb * b));
#define KS(it, ip, ig) K[(size_t)(it) + (size_t)ntmp * ((size_t)(ip) + (size_t)npre * (size_t)(ig))]
            for (int i = 0; i < n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    int jp = IX2(lf->jp, l, i, wp), jt = IX2(lf->jt, l, i, wp), jtt = IX2(lf->jtt, l, i, wp);
                    size_t q3 = (size_t)l + (size_t)wp * ((size_t)i + (size_t)ndl * jsb);
                    int g0 = lf->jgf[q3], g1 = lf->jgfp1[q3];
                    double f00 = IX2(lf->fac00, l, i, wp), f10 = IX2(lf->fac10, l, i, wp);
                    double f01 = IX2(lf->fac01, l, i, wp), f11 = IX2(lf->fac11, l, i, wp);
                    double fg = lf->fgf[q3];
                    double ke = fg * (f00 * KS(jt, jp, g0) + f10 * KS(jtt, jp + 1, g0)
                                      + f01 * KS(jt + 1, jp, g0) + f11 * KS(jtt + 1, jp + 1, g0))
                        + (1.0 - fg) * (f00 * KS(jt, jp, g1) + f10 * KS(jtt, jp + 1, g1)
                                        + f01 * KS(jt + 1, jp, g1) + f11 * KS(jtt + 1, jp + 1, g1));
                    ke = ke > 0.0 ? ke : 0.0;
                    double v = ke * IX3(atm->gas_mix_ratio, l, i, g, ndp, ndl);
                    IX2(kout, l, i, wp) = v > 0.0 ? v : 0.0;
                }
#undef KS
        }
        return SOCGPU_I_NORMAL;
    }
    if (fnc == SOCGPU_IP_SCALE_T_LOOKUP) {
        if (!lf->wt_gas || !d->k_t_lookup_gas) return SOCGPU_I_ERR_FATAL;
        const double *K = d->k_t_lookup_gas + (size_t)d->nd_t_lookup_gas *
            ((size_t)iex + (size_t)d->nd_k_term * ((size_t)g + (size_t)d->nd_species * b));
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < np; ++l) {
                size_t q3 = (size_t)l + (size_t)wp * ((size_t)i + (size_t)ndl * g);
                int jt = lf->jt_gas[q3];
                double wt = lf->wt_gas[q3];
                double ke = wt * K[jt] + (1.0 - wt) * K[jt + 1];
                ke = ke > 0.0 ? ke : 0.0;
                double v = ke * IX3(atm->gas_mix_ratio, l, i, g, ndp, ndl);
                IX2(kout, l, i, wp) = v > 0.0 ? v : 0.0;
            }
        return SOCGPU_I_NORMAL;
    }
    int st = scale_absorb(np, n_layer, ndp, wp, atm->p, atm->t, tmp, fnc,
                          IX2(d->p_ref, g, b, d->nd_species), IX2(d->t_ref, g, b, d->nd_species),
                          sp_scale(d, iex, b, g), d->l_doppler ? d->l_doppler[g] : 0,
                          d->doppler_cor ? d->doppler_cor[g] : 0.0, d, iex, b + 1);
    if (st != SOCGPU_I_NORMAL) return st;
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < np; ++l) {
            double v = IX2(tmp, l, i, wp) * IX3(atm->gas_mix_ratio, l, i, g, ndp, ndl);
            IX2(kout, l, i, wp) = kval * (v > 0.0 ? v : 0.0);
        }
    return SOCGPU_I_NORMAL;
}

/* Equivalent extinction of the minor gases (index_abs 2..n_abs) of band b
 * (solve_band_k_eqv_scl.F90:560-1040, the two-stream, non-spherical
 * branches).  Solar: each gas's k-terms are weighted by the direct flux
 * they transmit to the surface, and adjust_solar_ke corrects the direct
 * beam of the major gas's solve.  Infra-red: the weights are the fluxes
 * incident on each layer from monochromatic_gas_flux.F90:100-197 (no
 * scattering, diffusivity 1.66).  k_eqv + k_grey is added to the grey
 * extinction. */
static int k_eqv_minor(work *w, const socgpu_control *c, const lookup_fac *lf, const socgpu_spectrum_desc *d,
                       const socgpu_atm *atm, int np, int n_layer, int ndp, int b, int n_abs, const int *gas_of,
                       const int *nk, double *k_eqv, double *adj)
{
    int wp = w->wp, ndl = w->ndl;
    size_t pl = (size_t)wp * ndl, pl2 = (size_t)wp * (2 * ndl + 2);
    double *kab = zalloc(pl), *tmp = zalloc(pl), *k_min = zalloc(pl), *k_grey = zalloc(pl);
    double *skf = zalloc(pl2), *sfl = zalloc(pl2), *ft = zalloc(pl2), *trans = zalloc(pl), *su = zalloc(pl);
    double *fgas = zalloc((size_t)wp * (ndl + 1)), *fdt = zalloc((size_t)wp * (ndl + 1));
    int status = SOCGPU_I_NORMAL;
    const double *mass = atm->mass;
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < np; ++l) {
            IX2(k_eqv, l, i, wp) = 0.0; IX2(k_grey, l, i, wp) = 0.0;
            if (adj) IX2(adj, l, i, wp) = 1.0;
        }
    for (int j = 1; j < n_abs && status == SOCGPU_I_NORMAL; ++j) {
        int g = gas_of[j];
        const double *gfr = w->gfr + pl * j;
        if (c->isolir == SOCGPU_IP_SOLAR) {
            for (int l = 0; l < np; ++l) { IX2(fgas, l, 0, wp) = 1.0; IX2(sfl, l, 0, wp) = 0.0; }
            for (int i = 0; i < n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    IX2(fgas, l, i + 1, wp) = 0.0; IX2(skf, l, i, wp) = 0.0; IX2(k_min, l, i, wp) = HUGE_VAL;
                }
            for (int iex = 0; iex < nk[j]; ++iex) {
                double we = sp_kw(d->w, d, iex, b, g);
                status = absorber_term_k(lf, d, atm, np, n_layer, ndp, wp, ndl, b, g, iex, gfr, tmp, kab);
                if (status != SOCGPU_I_NORMAL) break;
                for (int l = 0; l < np; ++l) IX2(fdt, l, 0, wp) = we;
                for (int i = 1; i <= n_layer; ++i)
                    for (int l = 0; l < np; ++l) {
                        double e = exp(-IX2(kab, l, i - 1, wp) * IX2(mass, l, i - 1, ndp) * w->sec_0[l]);
                        IX2(fdt, l, i, wp) = IX2(fdt, l, i - 1, wp) * e;
                        IX2(fgas, l, i, wp) = IX2(fgas, l, i, wp) + IX2(fdt, l, i, wp);
                    }
                for (int i = 0; i < n_layer; ++i)
                    for (int l = 0; l < np; ++l) {
                        IX2(skf, l, i, wp) = IX2(skf, l, i, wp) + IX2(kab, l, i, wp) * IX2(fdt, l, n_layer, wp);
                        IX2(k_min, l, i, wp) = fmin(IX2(k_min, l, i, wp), IX2(kab, l, i, wp));
                    }
                for (int l = 0; l < np; ++l) IX2(sfl, l, 0, wp) = IX2(sfl, l, 0, wp) + IX2(fdt, l, n_layer, wp);
            }
            for (int i = 1; i <= n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    double sf = IX2(sfl, l, 0, wp);
                    if (sf > 0.0) IX2(k_eqv, l, i - 1, wp) = IX2(k_eqv, l, i - 1, wp) + IX2(skf, l, i - 1, wp) / sf;
                    else IX2(k_eqv, l, i - 1, wp) = IX2(k_eqv, l, i - 1, wp) + IX2(k_min, l, i - 1, wp);
                    if (IX2(fgas, l, i - 1, wp) > 0.0)
                        IX2(adj, l, i - 1, wp) = IX2(adj, l, i - 1, wp) * IX2(fgas, l, i, wp) / IX2(fgas, l, i - 1, wp);
                }
        } else {
            if (nk[j] == 1 && c->l_grey_single) {
                status = absorber_term_k(lf, d, atm, np, n_layer, ndp, wp, ndl, b, g, 0, gfr, tmp, kab);
                for (int i = 0; i < n_layer; ++i)
                    for (int l = 0; l < np; ++l) IX2(k_grey, l, i, wp) = IX2(k_grey, l, i, wp) + IX2(kab, l, i, wp);
                continue;
            }
            for (size_t q = 0; q < pl2; ++q) { skf[q] = 0.0; sfl[q] = 0.0; }
            for (size_t q = 0; q < pl; ++q) k_min[q] = HUGE_VAL;
            const double sq_eps = sqrt(EPS_R), dfac = 1.66;   /* diffusivity_factor_minor */
            for (int iex = 0; iex < nk[j]; ++iex) {
                double we = sp_kw(d->w, d, iex, b, g);
                status = absorber_term_k(lf, d, atm, np, n_layer, ndp, wp, ndl, b, g, iex, gfr, tmp, kab);
                if (status != SOCGPU_I_NORMAL) break;
                /* monochromatic_gas_flux.F90:100-197; ft as flux_total: 2i up, 2i+1 down at level i */
                for (int i = 0; i < n_layer; ++i)
                    for (int l = 0; l < np; ++l) {
                        double tau = IX2(kab, l, i, wp) * IX2(mass, l, i, ndp);
                        IX2(k_min, l, i, wp) = fmin(IX2(k_min, l, i, wp), IX2(kab, l, i, wp));
                        double t = exp(-dfac * tau);
                        IX2(trans, l, i, wp) = t;
                        IX2(su, l, i, wp) = (1.0 - t + sq_eps) * IX2(w->planck_diff, l, i, wp) / (dfac * tau + sq_eps);
                    }
                for (int l = 0; l < np; ++l) IX2(ft, l, 1, wp) = w->flux_inc_down[l];
                for (int i = 1; i <= n_layer; ++i)
                    for (int l = 0; l < np; ++l)
                        IX2(ft, l, 2 * i + 1, wp) = IX2(trans, l, i - 1, wp) * IX2(ft, l, 2 * i - 1, wp) - IX2(su, l, i - 1, wp);
                for (int l = 0; l < np; ++l)
                    IX2(ft, l, 2 * n_layer, wp) = w->d_planck_flux_surface[l] + w->alb_diff[l] * IX2(ft, l, 2 * n_layer + 1, wp);
                for (int i = n_layer; i >= 1; --i)
                    for (int l = 0; l < np; ++l)
                        IX2(ft, l, 2 * i - 2, wp) = IX2(trans, l, i - 1, wp) * IX2(ft, l, 2 * i, wp) + IX2(su, l, i - 1, wp);
                /* solve_band_k_eqv_scl.F90:993-1004 over flux_term(2 .. 2L+1), layer m/2 */
                for (int m = 2; m <= 2 * n_layer + 1; ++m)
                    for (int l = 0; l < np; ++l) {
                        double a = fabs(IX2(ft, l, m - 1, wp));
                        IX2(skf, l, m - 1, wp) = IX2(skf, l, m - 1, wp) + IX2(kab, l, m / 2 - 1, wp) * we * a;
                        IX2(sfl, l, m - 1, wp) = IX2(sfl, l, m - 1, wp) + we * a;
                    }
            }
            for (int i = 1; i <= n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    double kf = IX2(skf, l, 2 * i - 1, wp) + IX2(skf, l, 2 * i, wp);
                    double fl = IX2(sfl, l, 2 * i - 1, wp) + IX2(sfl, l, 2 * i, wp);
                    if (fl > 0.0) IX2(k_eqv, l, i - 1, wp) = IX2(k_eqv, l, i - 1, wp) + kf / fl;
                    else IX2(k_eqv, l, i - 1, wp) = IX2(k_eqv, l, i - 1, wp) + IX2(k_min, l, i - 1, wp);
                }
        }
    }
    if (status == SOCGPU_I_NORMAL && c->isolir == SOCGPU_IP_SOLAR) {
        const double temp_max = log(1.0 / EPS_R);
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < np; ++l)
                IX2(adj, l, i, wp) = IX2(adj, l, i, wp)
                    * exp(fmin(IX2(k_eqv, l, i, wp) * IX2(mass, l, i, ndp) * w->sec_0[l], temp_max));
    }
    /* solve_band_k_eqv_scl.F90:1024-1040 */
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < np; ++l)
            IX2(w->k_grey_tot, l, i, wp) = IX2(w->k_grey_tot, l, i, wp) + IX2(k_eqv, l, i, wp) + IX2(k_grey, l, i, wp);
    free(kab); free(tmp); free(k_min); free(k_grey); free(skf); free(sfl); free(ft); free(trans); free(su);
    free(fgas); free(fdt);
    return status;
}

/* --------------------------------------------------------------------- */
/* Clouds in two regions, clear and cloudy (mix_column.F90), for
 * ip_cloud_mix_max and ip_cloud_mix_random with ip_solver_mix_direct and
 * ip_solver_mix_direct_hogan.  Layers are 1-based in the comments and
 * 0-based in the arrays; interface i lies below layer i (0: the top). */

/* The cloud fraction of 1-based layer i of profile l. */
static double cloud_w(const socgpu_cld *cld, int ndp, int ict, int l, int i)
{
    return (i - 1 >= ict) ? cld->w_cloud[(size_t)l + (size_t)ndp * (size_t)(i - 1 - ict)] : 0.0;
}

/* set_cloud_geometry (set_cloud_geometry.F90:76-96): the first layer from
 * id_ct with a cloudy profile, at most n_layer. */
static int cloud_top(const socgpu_cld *cld, int ndp, int ict, int n_profile, int n_layer)
{
    int top = ict + 1;
    for (;;) {
        int any = 0;
        for (int l = 0; l < n_profile && !any; ++l) any = cloud_w(cld, ndp, ict, l, top) > 0.0;
        if (any || top >= n_layer) return top;
        ++top;
    }
}

/* overlap_coupled (overlap_coupled.F90:120-440) for the clear (region 1) and
 * the cloudy (region 2) region: at each interface i = nct-1 .. n_layer the
 * fractions of each upper region that lie over each lower one (ovl[0..3],
 * cloud_overlap(:, i, 1..4)) and of each lower region under each upper one
 * (ovl[4..7]).  0-based ovl index 2 j + k for region k above and j below,
 * 4 + 2 j + k for region k below and j above. */
/* The correlation of like region k (0 clear, 1 stratiform, 2 convective) at
 * interface i (overlap_coupled.F90:190-236): maximal (1) under mix_max and
 * triple, random (0) under mix_random; under part_corr and part_corr_cnv
 * exp((p(i) - p(i+1)) / dp_corr) between layers 1 < i < n_layer, with
 * dp_corr 1 Pa for the clear region and dp_corr_strat / dp_corr_conv for the
 * others, and 1 at the two ends. */
static double like_corr(int i_cloud, const socgpu_cld *cld, const double *p, int ndp, int l, int i, int n_layer,
                        int k)
{
    if (i_cloud == SOCGPU_IP_CLOUD_MIX_MAX || i_cloud == SOCGPU_IP_CLOUD_TRIPLE) return 1.0;
    if (i_cloud != SOCGPU_IP_CLOUD_PART_CORR && i_cloud != SOCGPU_IP_CLOUD_PART_CORR_CNV) return 0.0;
    if (!(i < n_layer && i > 1)) return 1.0;
    const double dp_corr = k == 0 ? 1.0 : (k == 1 ? cld->dp_corr_strat : cld->dp_corr_conv);
    return exp((p[(size_t)l + (size_t)ndp * (size_t)(i - 1)] - p[(size_t)l + (size_t)ndp * (size_t)i]) / dp_corr);
}

static void overlap_coupled2(work *w, const socgpu_cld *cld, const double *p, int ndp, int ict, int i_cloud)
{
    const int n_layer = w->n_layer, wp = w->wp, nct = w->nct;
    const double tol = 1.0e+02 * EPS_R;
    for (int l = 0; l < w->n_profile; ++l) {
        double au[2] = {1.0, 0.0};
        for (int i = nct - 1; i <= n_layer; ++i) {
            double al[2], ao[2][2];
            if (i < n_layer) {
                const double wc = cloud_w(cld, ndp, ict, l, i + 1);
                al[0] = 1.0 - wc;
                al[1] = wc * 1.0;
            } else {
                al[0] = 1.0;
                al[1] = 0.0;
            }
            for (int k = 0; k < 2; ++k)
                ao[k][k] = like_corr(i_cloud, cld, p, ndp, l, i, n_layer, k) * (al[k] < au[k] ? al[k] : au[k]);
            ao[0][1] = 0.0;
            ao[1][0] = 0.0;
            double art = 1.0 - ao[0][0];
            art = art - ao[1][1];
            double aru[2], arl[2];
            for (int k = 0; k < 2; ++k) {
                aru[k] = au[k] - ao[k][k];
                arl[k] = al[k] - ao[k][k];
            }
            for (int k = 0; k < 2; ++k)
                for (int j = 0; j < 2; ++j)
                    if (art > tol) ao[k][j] = ao[k][j] + aru[k] * arl[j] / art;
            double *cv = w->ovl + OVS * ((size_t)l + (size_t)wp * (size_t)i);
            for (int k = 0; k < 2; ++k) {
                cv[2 * k + k] = 1.0;
                for (int j = 0; j < k; ++j) { cv[2 * j + k] = 0.0; cv[2 * k + j] = 0.0; }
            }
            for (int k = 0; k < 2; ++k)
                if (au[k] > tol)
                    for (int j = 0; j < 2; ++j) cv[2 * j + k] = ao[k][j] / au[k];
            for (int k = 0; k < 2; ++k) {
                cv[4 + 2 * k + k] = 1.0;
                for (int j = 0; j < k; ++j) { cv[4 + 2 * j + k] = 0.0; cv[4 + 2 * k + j] = 0.0; }
            }
            for (int k = 0; k < 2; ++k)
                if (al[k] > tol)
                    for (int j = 0; j < 2; ++j) cv[4 + 2 * j + k] = ao[j][k] / al[k];
            if (i < n_layer) { au[0] = al[0]; au[1] = al[1]; }
        }
    }
}

/* The two-stream coefficients of cloud type t (1-based) in cell (l, i):
 * the clear grey optics plus the type's components, normalised and
 * rescaled (grey_opt_prop.F90:980-1000, 1195-1240, 1475-1500,
 * rescale_phase_fnc.F90), then single_scattering and two_coeff
 * (two_coeff_cloud.F90, two_coeff_region.F90:275-380). */
static void type_coeffs(const work *w, const socgpu_control *c, const double *mass, int ndp, const socgpu_cld *cld,
                        int l, int i, int t, coeffs *o)
{
    const int wp = w->wp;
    const size_t pl = (size_t)wp * w->ndl;
    double kgt = IX2(w->k_grey_tot, l, i, wp), kes = IX2(w->k_ext_scat, l, i, wp);
    double fwd = IX2(w->forward_scatter_nc, l, i, wp), phf = IX2(w->phase_fnc_nc, l, i, wp);
    for (int k = 0; k < cld->n_condensed; ++k) {
        if (cld->i_cloud_type[k] != t) continue;
        kgt = kgt + IX2(w->k_ext_tot_cc + pl * k, l, i, wp);
        kes = kes + IX2(w->k_ext_scat_cc + pl * k, l, i, wp);
        fwd = fwd + IX2(w->fwd_cc + pl * k, l, i, wp);
        phf = phf + IX2(w->phf_cc + pl * k, l, i, wp);
    }
    double asym = phf;
    if (kes > TINY_R) {
        const double inv = 1.0 / kes;
        if (c->l_rescale) {
            fwd = fwd * inv;
            asym = phf * inv;
            asym = (asym - fwd) / (1.0 - fwd);
        } else {
            asym = phf / kes;
        }
    }
    if (!c->l_rescale) fwd = 0.0;
    double tau, tau_dir, om;
    single_scatter_cell(c, kgt, kes, IX2(w->k_gas_abs, l, i, wp), IX2(mass, l, i, ndp), fwd, &tau, &tau_dir, &om);
    two_coeff_cell(c->isolir, c->i_2stream, c->i_direct_tau, c->l_ir_source_quad, asym, om, tau_dir, tau,
                   w->sec_0[l], o);
}

/* One k-term in two regions (mix_column.F90:150-460): the clear
 * coefficients of every layer, the frac_cloud-weighted coefficients of the
 * cloud types (two_coeff_cloud.F90), the sources (ir_source with w_free and
 * w_cloud, or mixed_solar_source.F90) and solver_mix_direct.F90 or
 * solver_mix_direct_hogan.F90.  Leaves flux_total and flux_direct as
 * column_solve does. */
static void solve_region_term(work *w, const socgpu_control *c, const socgpu_dimen *dm, const double *mass,
                              const socgpu_cld *cld)
{
    const int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp, ndp = dm->nd_profile;
    const int ict = dm->id_cloud_top - 1, ndc = w->ndl - ict, nct = w->nct;
    const int solar = (c->isolir == SOCGPU_IP_SOLAR);
    const int l_dir = (c->i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING || c->i_direct_tau == SOCGPU_IP_DIRECT_CSR_SCALING);
#define OV(l, i, m) (w->ovl[OVS * ((size_t)(l) + (size_t)wp * (size_t)(i)) + (m)])
    clear_coefficients(w, c, mass, ndp);
    /* two_coeff_cloud */
    for (int i = nct - 1; i < n_layer; ++i)
        for (int l = 0; l < n_profile; ++l) {
            IX2(w->tc, l, i, wp) = 0.0; IX2(w->rc, l, i, wp) = 0.0; IX2(w->t0c, l, i, wp) = 0.0;
            IX2(w->t0dc, l, i, wp) = 0.0; IX2(w->sc1c, l, i, wp) = 0.0; IX2(w->sc2c, l, i, wp) = 0.0;
        }
    for (int t = 1; t <= cld->n_cloud_type; ++t)
        for (int i = nct - 1; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                if (i < ict) continue;
                const size_t qc = (size_t)l + (size_t)ndp * (size_t)(i - ict);
                const double fc = cld->frac_cloud[qc + (size_t)ndp * ndc * (size_t)(t - 1)];
                if (!(fc > 0.0) || !(cld->w_cloud[qc] > 0.0)) continue;
                coeffs o;
                type_coeffs(w, c, mass, ndp, cld, l, i, t, &o);
                IX2(w->tc, l, i, wp) = IX2(w->tc, l, i, wp) + fc * o.trans;
                IX2(w->rc, l, i, wp) = IX2(w->rc, l, i, wp) + fc * o.reflect;
                IX2(w->sc1c, l, i, wp) = IX2(w->sc1c, l, i, wp) + fc * o.sc1;
                if (solar || c->l_ir_source_quad) IX2(w->sc2c, l, i, wp) = IX2(w->sc2c, l, i, wp) + fc * o.sc2;
                if (solar) {
                    IX2(w->t0c, l, i, wp) = IX2(w->t0c, l, i, wp) + fc * o.trans_0;
                    if (l_dir) IX2(w->t0dc, l, i, wp) = IX2(w->t0dc, l, i, wp) + fc * o.trans_0_dir;
                }
            }
    /* sources */
    double *fd = w->flux_direct;
    if (!solar) {
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                const double d1 = IX2(w->planck_diff, l, i, wp), d2 = IX2(w->planck_diff_2, l, i, wp);
                double su, sd, suc = 0.0, sdc = 0.0;
                if (c->l_ir_source_quad) {
                    su = IX2(w->sc1, l, i, wp) * d1 + IX2(w->sc2, l, i, wp) * d2;
                    sd = -IX2(w->sc1, l, i, wp) * d1 + IX2(w->sc2, l, i, wp) * d2;
                    suc = IX2(w->sc1c, l, i, wp) * d1 + IX2(w->sc2c, l, i, wp) * d2;
                    sdc = -IX2(w->sc1c, l, i, wp) * d1 + IX2(w->sc2c, l, i, wp) * d2;
                } else {
                    su = IX2(w->sc1, l, i, wp) * d1;
                    sd = -su;
                    suc = IX2(w->sc1c, l, i, wp) * d1;
                    sdc = -suc;
                }
                if (i >= nct - 1) {
                    const double wc = cloud_w(cld, ndp, ict, l, i + 1), wf = 1.0 - wc;
                    su = wf * su; sd = wf * sd;
                    suc = wc * suc; sdc = wc * sdc;
                }
                IX2(w->s_up, l, i, wp) = su; IX2(w->s_down, l, i, wp) = sd;
                IX2(w->s_up_c, l, i, wp) = suc; IX2(w->s_down_c, l, i, wp) = sdc;
            }
    } else {
        /* mixed_solar_source (mixed_solar_source.F90:95-250) */
        const double *adj = w->adj;
        for (int l = 0; l < n_profile; ++l) {
            IX2(fd, l, 0, wp) = w->flux_inc_direct[l];
            if (l_dir) IX2(w->flux_direct_dir, l, 0, wp) = w->flux_inc_direct[l];
        }
        for (int i = 1; i <= nct - 1; ++i)
            for (int l = 0; l < n_profile; ++l) {
                const int ii = i - 1;
                const double f0 = IX2(fd, l, i - 1, wp), t0 = IX2(w->trans_0, l, ii, wp);
                if (adj) {
                    IX2(fd, l, i, wp) = f0 * t0 * IX2(adj, l, ii, wp);
                    IX2(w->s_up, l, ii, wp) = IX2(w->sc1, l, ii, wp) * f0;
                    IX2(w->s_down, l, ii, wp) = (IX2(w->sc2, l, ii, wp) - t0) * f0 + IX2(fd, l, i, wp);
                } else {
                    IX2(fd, l, i, wp) = f0 * t0;
                    IX2(w->s_up, l, ii, wp) = IX2(w->sc1, l, ii, wp) * f0;
                    IX2(w->s_down, l, ii, wp) = IX2(w->sc2, l, ii, wp) * f0;
                }
                if (l_dir) {
                    double v = IX2(w->flux_direct_dir, l, i - 1, wp) * IX2(w->trans_0_dir, l, ii, wp);
                    if (adj) v = v * IX2(adj, l, ii, wp);
                    IX2(w->flux_direct_dir, l, i, wp) = v;
                }
            }
        for (int l = 0; l < n_profile; ++l) {
            double bf = IX2(fd, l, nct - 1, wp), bc = 0.0;
            for (int i = nct; i <= n_layer; ++i) {
                const int ii = i - 1;
                const double tc_ = OV(l, i - 1, 3) * bc + OV(l, i - 1, 2) * bf;
                const double tf_ = OV(l, i - 1, 0) * bf + OV(l, i - 1, 1) * bc;
                const double t0f = IX2(w->trans_0, l, ii, wp), t0c = IX2(w->t0c, l, ii, wp);
                if (adj) {
                    const double a = IX2(adj, l, ii, wp);
                    bf = tf_ * t0f * a;
                    bc = tc_ * t0c * a;
                    IX2(w->s_up, l, ii, wp) = IX2(w->sc1, l, ii, wp) * tf_;
                    IX2(w->s_down, l, ii, wp) = (IX2(w->sc2, l, ii, wp) - t0f) * tf_ + bf;
                    IX2(w->s_up_c, l, ii, wp) = IX2(w->sc1c, l, ii, wp) * tc_;
                    IX2(w->s_down_c, l, ii, wp) = (IX2(w->sc2c, l, ii, wp) - t0c) * tc_ + bc;
                } else {
                    bf = tf_ * t0f;
                    bc = tc_ * t0c;
                    IX2(w->s_up, l, ii, wp) = IX2(w->sc1, l, ii, wp) * tf_;
                    IX2(w->s_down, l, ii, wp) = IX2(w->sc2, l, ii, wp) * tf_;
                    IX2(w->s_up_c, l, ii, wp) = IX2(w->sc1c, l, ii, wp) * tc_;
                    IX2(w->s_down_c, l, ii, wp) = IX2(w->sc2c, l, ii, wp) * tc_;
                }
                IX2(fd, l, i, wp) = bf + bc;
            }
            w->alpha[l] = bc;          /* the direct flux reaching the ground under cloud */
            if (l_dir) {
                double df = IX2(w->flux_direct_dir, l, nct - 1, wp), dc = 0.0;
                for (int i = nct; i <= n_layer; ++i) {
                    const int ii = i - 1;
                    const double tc_ = OV(l, i - 1, 3) * dc + OV(l, i - 1, 2) * df;
                    const double tf_ = OV(l, i - 1, 0) * df + OV(l, i - 1, 1) * dc;
                    const double a = adj ? IX2(adj, l, ii, wp) : 1.0;
                    df = adj ? tf_ * IX2(w->trans_0_dir, l, ii, wp) * a : tf_ * IX2(w->trans_0_dir, l, ii, wp);
                    dc = adj ? tc_ * IX2(w->t0dc, l, ii, wp) * a : tc_ * IX2(w->t0dc, l, ii, wp);
                    IX2(w->flux_direct_dir, l, i, wp) = df + dc;
                }
                for (int i = 0; i <= n_layer; ++i) IX2(fd, l, i, wp) = IX2(w->flux_direct_dir, l, i, wp);
                w->alpha[l] = dc;
            }
        }
    }
    /* ground sources (mix_column.F90:365-385) */
    for (int l = 0; l < n_profile; ++l) {
        if (solar) {
            const double fdc = w->alpha[l];
            w->source_ground[l] = (w->alb_dir[l] - w->alb_diff[l]) * (IX2(fd, l, n_layer, wp) - fdc);
            w->s_up_prime[l] = (w->alb_dir[l] - w->alb_diff[l]) * fdc;
        } else {
            w->source_ground[l] = OV(l, n_layer, 4) * (1.0 - w->alb_diff[l]) * w->d_planck_flux_surface[l];
            w->s_up_prime[l] = OV(l, n_layer, 6) * (1.0 - w->alb_diff[l]) * w->d_planck_flux_surface[l];
        }
    }
    /* solver_mix_direct.F90:88-300 or solver_mix_direct_hogan.F90:78-260,
     * with v11 = ovl 0, v21 = ovl 2, v12 = ovl 1, v22 = ovl 3, u11 = ovl 4,
     * u12 = ovl 5, u21 = ovl 6, u22 = ovl 7 */
    const int hogan = (c->i_solver == SOCGPU_IP_SOLVER_MIX_DIRECT_HOGAN);
    double *ft = w->flux_total;
    for (int l = 0; l < n_profile; ++l) {
        double a11 = 0.0, a12 = 0.0, a21 = 0.0, a22 = 0.0, g1 = 0.0, g2 = 0.0;
        for (int i = n_layer + 1; i >= 1; --i) {
            const int ii = i - 1;
            if (i < n_layer + 1 && i >= nct) {
                const double r = IX2(w->reflect, l, ii, wp), t = IX2(w->trans, l, ii, wp);
                const double rcl = IX2(w->rc, l, ii, wp), tcl = IX2(w->tc, l, ii, wp);
                const double sd = IX2(w->s_down, l, ii, wp), su = IX2(w->s_up, l, ii, wp);
                const double sdc = IX2(w->s_down_c, l, ii, wp), suc = IX2(w->s_up_c, l, ii, wp);
                const double v11 = OV(l, i, 0), v21 = OV(l, i, 2), v12 = OV(l, i, 1), v22 = OV(l, i, 3);
                const double u11 = OV(l, i - 1, 4), u12 = OV(l, i - 1, 5), u21 = OV(l, i - 1, 6), u22 = OV(l, i - 1, 7);
                if (!hogan) {
                    const double th11 = a11 * v11 + a12 * v21, th12 = a11 * v12 + a12 * v22;
                    const double th21 = a21 * v11 + a22 * v21, th22 = a21 * v12 + a22 * v22;
                    const double b21 = -th21 * r;
                    const double b22 = 1.0 / (1.0 - th22 * rcl);
                    const double gm21 = th21 * t, gm22 = th22 * tcl;
                    const double hh2 = g2 + th21 * sd + th22 * sdc;
                    double lam = th12 * rcl * b22;
                    const double b11 = 1.0 / (1.0 - th11 * r + lam * b21);
                    const double gm11 = th11 * t + lam * gm21, gm12 = th12 * tcl + lam * gm22;
                    const double hh1 = g1 + th11 * sd + th12 * sdc + lam * hh2;
                    IX2(w->b21, l, ii, wp) = b21; IX2(w->b22, l, ii, wp) = b22; IX2(w->b11, l, ii, wp) = b11;
                    IX2(w->g11, l, ii, wp) = gm11; IX2(w->g12, l, ii, wp) = gm12;
                    IX2(w->g21, l, ii, wp) = gm21; IX2(w->g22, l, ii, wp) = gm22;
                    IX2(w->h1, l, ii, wp) = hh1; IX2(w->h2, l, ii, wp) = hh2;
                    lam = u22 * tcl * b22;
                    double lamb = (u21 * t + lam * b21) * b11;
                    a21 = u21 * r + lam * gm21 + lamb * gm11;
                    a22 = u22 * rcl + lam * gm22 + lamb * gm12;
                    const double ng2 = u21 * su + u22 * suc + lam * hh2 + lamb * hh1;
                    lam = u12 * tcl * b22;
                    lamb = (u11 * t + lam * b21) * b11;
                    a11 = u11 * r + lam * gm21 + lamb * gm11;
                    a12 = u12 * rcl + lam * gm22 + lamb * gm12;
                    g1 = u11 * su + u12 * suc + lam * hh2 + lamb * hh1;
                    g2 = ng2;
                } else {
                    const double th11 = a11 * v11 + a22 * v21, th22 = a11 * v12 + a22 * v22;
                    const double b11 = 1.0 / (1.0 - th11 * r), gm11 = th11 * t, hh1 = g1 + th11 * sd;
                    const double b22 = 1.0 / (1.0 - th22 * rcl), gm22 = th22 * tcl, hh2 = g2 + th22 * sdc;
                    const double l1 = su + hh1 * t * b11, l2 = suc + hh2 * tcl * b22;
                    IX2(w->b11, l, ii, wp) = b11; IX2(w->g11, l, ii, wp) = gm11; IX2(w->h1, l, ii, wp) = hh1;
                    IX2(w->b22, l, ii, wp) = b22; IX2(w->g22, l, ii, wp) = gm22; IX2(w->h2, l, ii, wp) = hh2;
                    a11 = r + th11 * t * t * b11;
                    g1 = u11 * l1 + u12 * l2;
                    a22 = rcl + th22 * tcl * tcl * b22;
                    g2 = u21 * l1 + u22 * l2;
                }
            } else if (i < nct - 1) {
                const double r = IX2(w->reflect, l, ii, wp), t = IX2(w->trans, l, ii, wp);
                const double b11 = 1.0 / (1.0 - a11 * r), gm11 = a11 * t;
                const double hh1 = g1 + a11 * IX2(w->s_down, l, ii, wp);
                IX2(w->b11, l, ii, wp) = b11; IX2(w->g11, l, ii, wp) = gm11; IX2(w->h1, l, ii, wp) = hh1;
                const double lam = t * b11;
                a11 = r + lam * gm11;
                g1 = IX2(w->s_up, l, ii, wp) + lam * hh1;
            } else if (i == nct - 1) {
                const double r = IX2(w->reflect, l, ii, wp), t = IX2(w->trans, l, ii, wp);
                const double th11 = (nct < n_layer) ? (hogan ? a11 * OV(l, i, 0) + a22 * OV(l, i, 2)
                                                             : a11 * OV(l, i, 0) + a12 * OV(l, i, 2))
                                                    : a11;
                const double b11 = 1.0 / (1.0 - th11 * r), gm11 = th11 * t;
                const double hh1 = g1 + th11 * IX2(w->s_down, l, ii, wp);
                IX2(w->b11, l, ii, wp) = b11; IX2(w->g11, l, ii, wp) = gm11; IX2(w->h1, l, ii, wp) = hh1;
                const double lam = t * b11;
                a11 = r + lam * gm11;
                g1 = IX2(w->s_up, l, ii, wp) + lam * hh1;
            } else if (i == n_layer + 1) {
                a11 = w->alb_diff[l];
                a22 = w->alb_diff[l];
                a21 = 0.0;
                a12 = 0.0;
                g1 = w->source_ground[l];
                g2 = w->s_up_prime[l];
            }
        }
        IX2(ft, l, 1, wp) = w->flux_inc_down[l];
        if (nct > 1) IX2(ft, l, 0, wp) = a11 * IX2(ft, l, 1, wp) + g1;
        else IX2(ft, l, 0, wp) = g1 + w->flux_inc_down[l] * (OV(l, 0, 0) * a11 + OV(l, 0, 2) * (hogan ? a22 : a12));
        for (int i = 1; i <= nct - 1; ++i) {
            const int ii = i - 1;
            IX2(ft, l, 2 * i, wp) = (IX2(w->g11, l, ii, wp) * IX2(ft, l, 2 * i - 1, wp) + IX2(w->h1, l, ii, wp))
                * IX2(w->b11, l, ii, wp);
            IX2(ft, l, 2 * i + 1, wp) = IX2(w->trans, l, ii, wp) * IX2(ft, l, 2 * i - 1, wp)
                + IX2(w->reflect, l, ii, wp) * IX2(ft, l, 2 * i, wp) + IX2(w->s_down, l, ii, wp);
        }
        double fd1 = 0.0, fd2 = 0.0;
        for (int i = nct; i <= n_layer; ++i) {
            const int ii = i - 1;
            if (i > nct) {
                const double d1 = fd1, d2 = fd2;
                fd1 = OV(l, i - 1, 0) * d1 + OV(l, i - 1, 1) * d2;
                fd2 = OV(l, i - 1, 2) * d1 + OV(l, i - 1, 3) * d2;
            } else {
                fd1 = OV(l, i - 1, 0) * IX2(ft, l, 2 * i - 1, wp);
                fd2 = OV(l, i - 1, 2) * IX2(ft, l, 2 * i - 1, wp);
            }
            double fu1, fu2;
            if (!hogan) {
                fu1 = (IX2(w->g11, l, ii, wp) * fd1 + IX2(w->g12, l, ii, wp) * fd2 + IX2(w->h1, l, ii, wp))
                    * IX2(w->b11, l, ii, wp);
                fu2 = (IX2(w->g21, l, ii, wp) * fd1 + IX2(w->g22, l, ii, wp) * fd2 - IX2(w->b21, l, ii, wp) * fu1
                       + IX2(w->h2, l, ii, wp)) * IX2(w->b22, l, ii, wp);
            } else {
                fu1 = (IX2(w->g11, l, ii, wp) * fd1 + IX2(w->h1, l, ii, wp)) * IX2(w->b11, l, ii, wp);
                fu2 = (IX2(w->g22, l, ii, wp) * fd2 + IX2(w->h2, l, ii, wp)) * IX2(w->b22, l, ii, wp);
            }
            fd1 = IX2(w->trans, l, ii, wp) * fd1 + IX2(w->reflect, l, ii, wp) * fu1 + IX2(w->s_down, l, ii, wp);
            fd2 = IX2(w->tc, l, ii, wp) * fd2 + IX2(w->rc, l, ii, wp) * fu2 + IX2(w->s_down_c, l, ii, wp);
            IX2(ft, l, 2 * i, wp) = fu1 + fu2;
            IX2(ft, l, 2 * i + 1, wp) = fd1 + fd2;
        }
    }
#undef OV
}

/* Clouds in three regions, clear (1), stratiform (2) and convective (3)
 * (triple_column.F90), for ip_cloud_triple with ip_solver_triple_hogan.
 * Layers are 1-based in the comments and 0-based in the arrays; interface
 * i lies below layer i (0: the top). */

/* aggregate_cloud (aggregate_cloud.F90:107-160): the region of cloud type t
 * (1-based).  Stratiform water and ice, then convective water and ice
 * (csiw, split_ice_water); or stratiform, then convective (conv_strat,
 * split_homogen). */
static int region_of_type(int rep, int t)
{
    if (rep == SOCGPU_IP_CLOUD_CSIW || rep == SOCGPU_IP_CLOUD_SPLIT_ICE_WATER)
        return (t == SOCGPU_IP_CLOUD_TYPE_SW || t == SOCGPU_IP_CLOUD_TYPE_SI) ? 2 : 3;
    return t == SOCGPU_IP_CLOUD_TYPE_STRAT ? 2 : 3;
}

/* The regions' shares of the cloud (frac_region, aggregate_cloud.F90) and
 * overlap_coupled (overlap_coupled.F90:150-450) for three regions with
 * like regions maximally overlapped (ip_cloud_triple): at each interface
 * i = nct-1 .. n_layer the fraction v_jk of upper region k going into lower
 * region j (ovl[3 j + k], cloud_overlap(:, i, 3 j + k + 1)) and the fraction
 * u_jk of lower region k going into upper region j (ovl[9 + 3 j + k]). */
static void overlap_coupled3(work *w, const socgpu_control *c, const socgpu_cld *cld, const double *p, int ndp,
                             int ict)
{
    const int n_layer = w->n_layer, wp = w->wp, nct = w->nct, ndc = w->ndl - ict;
    const double tol = 1.0e+02 * EPS_R;
    for (int i = 0; i < n_layer; ++i)
        for (int l = 0; l < w->n_profile; ++l) {
            double f2 = 0.0, f3 = 0.0;
            if (i >= ict)
                for (int t = 1; t <= cld->n_cloud_type; ++t) {
                    const double fc = cld->frac_cloud[(size_t)l + (size_t)ndp * ((size_t)(i - ict) + (size_t)ndc * (t - 1))];
                    if (region_of_type(c->i_cloud_representation, t) == 2) f2 = f2 + fc; else f3 = f3 + fc;
                }
            IX2(w->fr2, l, i, wp) = f2;
            IX2(w->fr3, l, i, wp) = f3;
        }
    for (int l = 0; l < w->n_profile; ++l) {
        double au[3] = {1.0, 0.0, 0.0};
        for (int i = nct - 1; i <= n_layer; ++i) {
            double al[3], ao[3][3];
            if (i < n_layer) {
                const double wc = cloud_w(cld, ndp, ict, l, i + 1);
                al[0] = 1.0 - wc;
                al[1] = wc * IX2(w->fr2, l, i, wp);
                al[2] = wc * IX2(w->fr3, l, i, wp);
            } else {
                al[0] = 1.0; al[1] = 0.0; al[2] = 0.0;
            }
            for (int k = 0; k < 3; ++k)
                ao[k][k] = like_corr(c->i_cloud, cld, p, ndp, l, i, n_layer, k) * (al[k] < au[k] ? al[k] : au[k]);
            for (int k = 0; k < 3; ++k)
                for (int j = 0; j < k; ++j) { ao[k][j] = 0.0; ao[j][k] = 0.0; }
            double art = 1.0 - ao[0][0];
            for (int k = 1; k < 3; ++k) art = art - ao[k][k];
            double aru[3], arl[3];
            for (int k = 0; k < 3; ++k) {
                aru[k] = au[k] - ao[k][k];
                arl[k] = al[k] - ao[k][k];
            }
            for (int k = 0; k < 3; ++k)
                for (int j = 0; j < 3; ++j)
                    if (art > tol) ao[k][j] = ao[k][j] + aru[k] * arl[j] / art;
            double *cv = w->ovl + OVS * ((size_t)l + (size_t)wp * (size_t)i);
            for (int k = 0; k < 3; ++k) {
                cv[3 * k + k] = 1.0;
                for (int j = 0; j < k; ++j) { cv[3 * j + k] = 0.0; cv[3 * k + j] = 0.0; }
            }
            for (int k = 0; k < 3; ++k)
                if (au[k] > tol)
                    for (int j = 0; j < 3; ++j) cv[3 * j + k] = ao[k][j] / au[k];
            for (int k = 0; k < 3; ++k) {
                cv[9 + 3 * k + k] = 1.0;
                for (int j = 0; j < k; ++j) { cv[9 + 3 * j + k] = 0.0; cv[9 + 3 * k + j] = 0.0; }
            }
            for (int k = 0; k < 3; ++k)
                if (al[k] > tol)
                    for (int j = 0; j < 3; ++j) cv[9 + 3 * j + k] = ao[j][k] / al[k];
            if (i < n_layer) { au[0] = al[0]; au[1] = al[1]; au[2] = al[2]; }
        }
    }
}

/* One k-term in three regions (triple_column.F90:260-560): the clear
 * coefficients of every layer, each cloudy region's coefficients as the
 * frac_cloud-weighted sum over its cloud types divided by its share
 * (two_coeff_region.F90:230-440), the infra-red sources weighted by the
 * regions' areas or triple_solar_source.F90, the ground sources and
 * solver_triple_hogan.F90.  Leaves flux_total and flux_direct as
 * column_solve does. */
static void solve_triple_term(work *w, const socgpu_control *c, const socgpu_dimen *dm, const double *mass,
                              const socgpu_cld *cld)
{
    const int n_profile = w->n_profile, n_layer = w->n_layer, wp = w->wp, ndp = dm->nd_profile;
    const int ict = dm->id_cloud_top - 1, ndc = w->ndl - ict, nct = w->nct;
    const int solar = (c->isolir == SOCGPU_IP_SOLAR);
    const int l_dir = (c->i_direct_tau == SOCGPU_IP_DIRECT_NOSCALING || c->i_direct_tau == SOCGPU_IP_DIRECT_CSR_SCALING);
#define OV3(l, i, m) (w->ovl[OVS * ((size_t)(l) + (size_t)wp * (size_t)(i)) + (m)])
    /* region k's arrays: 1 the clear, 2 the stratiform, 3 the convective */
    double *T[4] = {NULL, w->trans, w->tc, w->tv}, *Rr[4] = {NULL, w->reflect, w->rc, w->rv};
    double *T0[4] = {NULL, w->trans_0, w->t0c, w->t0v}, *T0D[4] = {NULL, w->trans_0_dir, w->t0dc, w->t0dv};
    double *S1[4] = {NULL, w->sc1, w->sc1c, w->sc1v}, *S2[4] = {NULL, w->sc2, w->sc2c, w->sc2v};
    double *SU[4] = {NULL, w->s_up, w->s_up_c, w->s_up_v}, *SD[4] = {NULL, w->s_down, w->s_down_c, w->s_down_v};
    double *FR[4] = {NULL, NULL, w->fr2, w->fr3};
    clear_coefficients(w, c, mass, ndp);
    for (int k = 2; k <= 3; ++k)
        for (int i = nct - 1; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                IX2(T[k], l, i, wp) = 0.0; IX2(Rr[k], l, i, wp) = 0.0; IX2(T0[k], l, i, wp) = 0.0;
                IX2(T0D[k], l, i, wp) = 0.0; IX2(S1[k], l, i, wp) = 0.0; IX2(S2[k], l, i, wp) = 0.0;
            }
    for (int t = 1; t <= cld->n_cloud_type; ++t) {
        const int k = region_of_type(c->i_cloud_representation, t);
        for (int i = nct - 1; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                if (i < ict) continue;
                const size_t qc = (size_t)l + (size_t)ndp * (size_t)(i - ict);
                const double fc = cld->frac_cloud[qc + (size_t)ndp * ndc * (size_t)(t - 1)];
                if (!(fc > TINY_R) || !(cld->w_cloud[qc] > 0.0)) continue;
                coeffs o;
                type_coeffs(w, c, mass, ndp, cld, l, i, t, &o);
                IX2(T[k], l, i, wp) = IX2(T[k], l, i, wp) + fc * o.trans;
                IX2(Rr[k], l, i, wp) = IX2(Rr[k], l, i, wp) + fc * o.reflect;
                IX2(S1[k], l, i, wp) = IX2(S1[k], l, i, wp) + fc * o.sc1;
                if (solar || c->l_ir_source_quad) IX2(S2[k], l, i, wp) = IX2(S2[k], l, i, wp) + fc * o.sc2;
                if (solar) {
                    IX2(T0[k], l, i, wp) = IX2(T0[k], l, i, wp) + fc * o.trans_0;
                    if (l_dir) IX2(T0D[k], l, i, wp) = IX2(T0D[k], l, i, wp) + fc * o.trans_0_dir;
                }
            }
    }
    for (int k = 2; k <= 3; ++k)
        for (int i = nct - 1; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                const double fr = IX2(FR[k], l, i, wp);
                if (!(fr > TINY_R)) continue;
                const double inv = 1.0 / fr;
                IX2(T[k], l, i, wp) = IX2(T[k], l, i, wp) * inv;
                IX2(Rr[k], l, i, wp) = IX2(Rr[k], l, i, wp) * inv;
                if (solar) {
                    IX2(T0[k], l, i, wp) = IX2(T0[k], l, i, wp) * inv;
                    if (l_dir) IX2(T0D[k], l, i, wp) = IX2(T0D[k], l, i, wp) * inv;
                }
                IX2(S1[k], l, i, wp) = IX2(S1[k], l, i, wp) * inv;
                if (solar || c->l_ir_source_quad) IX2(S2[k], l, i, wp) = IX2(S2[k], l, i, wp) * inv;
            }
    /* sources */
    double *fd = w->flux_direct;
    if (!solar) {
        /* ir_source per region, then weighted by the areas (triple_column.F90:296-350) */
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < n_profile; ++l) {
                const double d1 = IX2(w->planck_diff, l, i, wp), d2 = IX2(w->planck_diff_2, l, i, wp);
                for (int k = 1; k <= 3; ++k) {
                    if (k > 1 && i < nct - 1) continue;
                    double su, sd;
                    if (c->l_ir_source_quad) {
                        su = IX2(S1[k], l, i, wp) * d1 + IX2(S2[k], l, i, wp) * d2;
                        sd = -IX2(S1[k], l, i, wp) * d1 + IX2(S2[k], l, i, wp) * d2;
                    } else {
                        su = IX2(S1[k], l, i, wp) * d1;
                        sd = -su;
                    }
                    if (i >= nct - 1) {
                        const double wc = cloud_w(cld, ndp, ict, l, i + 1);
                        const double a = (k == 1) ? 1.0 - wc : wc * IX2(FR[k], l, i, wp);
                        su = a * su; sd = a * sd;
                    }
                    IX2(SU[k], l, i, wp) = su; IX2(SD[k], l, i, wp) = sd;
                }
            }
    } else {
        /* triple_solar_source (triple_solar_source.F90:160-400) */
        const double *adj = w->adj;
        for (int l = 0; l < n_profile; ++l) {
            IX2(fd, l, 0, wp) = w->flux_inc_direct[l];
            if (l_dir) IX2(w->flux_direct_dir, l, 0, wp) = w->flux_inc_direct[l];
        }
        for (int i = 1; i <= nct - 1; ++i)
            for (int l = 0; l < n_profile; ++l) {
                const int ii = i - 1;
                const double f0 = IX2(fd, l, i - 1, wp), t0 = IX2(w->trans_0, l, ii, wp);
                if (adj) {
                    IX2(fd, l, i, wp) = f0 * t0 * IX2(adj, l, ii, wp);
                    IX2(w->s_up, l, ii, wp) = IX2(w->sc1, l, ii, wp) * f0;
                    IX2(w->s_down, l, ii, wp) = (IX2(w->sc2, l, ii, wp) - t0) * f0 + IX2(fd, l, i, wp);
                } else {
                    IX2(fd, l, i, wp) = f0 * t0;
                    IX2(w->s_up, l, ii, wp) = IX2(w->sc1, l, ii, wp) * f0;
                    IX2(w->s_down, l, ii, wp) = IX2(w->sc2, l, ii, wp) * f0;
                }
                if (l_dir) {
                    double v = IX2(w->flux_direct_dir, l, i - 1, wp) * IX2(w->trans_0_dir, l, ii, wp);
                    if (adj) v = v * IX2(adj, l, ii, wp);
                    IX2(w->flux_direct_dir, l, i, wp) = v;
                }
            }
        for (int l = 0; l < n_profile; ++l) {
            double base[3] = {IX2(fd, l, nct - 1, wp), 0.0, 0.0};
            for (int i = nct; i <= n_layer; ++i) {
                const int ii = i - 1;
                double top[3];
                for (int j = 0; j < 3; ++j)
                    top[j] = OV3(l, i - 1, 3 * j) * base[0] + OV3(l, i - 1, 3 * j + 1) * base[1]
                           + OV3(l, i - 1, 3 * j + 2) * base[2];
                for (int k = 1; k <= 3; ++k) {
                    const double t0 = IX2(T0[k], l, ii, wp);
                    if (adj) {
                        base[k - 1] = top[k - 1] * t0 * IX2(adj, l, ii, wp);
                        IX2(SU[k], l, ii, wp) = IX2(S1[k], l, ii, wp) * top[k - 1];
                        IX2(SD[k], l, ii, wp) = (IX2(S2[k], l, ii, wp) - t0) * top[k - 1] + base[k - 1];
                    } else {
                        base[k - 1] = top[k - 1] * t0;
                        IX2(SU[k], l, ii, wp) = IX2(S1[k], l, ii, wp) * top[k - 1];
                        IX2(SD[k], l, ii, wp) = IX2(S2[k], l, ii, wp) * top[k - 1];
                    }
                }
                IX2(fd, l, i, wp) = base[0] + base[1] + base[2];
            }
            w->alpha[l] = base[0]; w->fdg2[l] = base[1]; w->fdg3[l] = base[2];
            if (l_dir) {
                double db[3] = {IX2(w->flux_direct_dir, l, nct - 1, wp), 0.0, 0.0};
                for (int i = nct; i <= n_layer; ++i) {
                    const int ii = i - 1;
                    double top[3];
                    for (int j = 0; j < 3; ++j)
                        top[j] = OV3(l, i - 1, 3 * j) * db[0] + OV3(l, i - 1, 3 * j + 1) * db[1]
                               + OV3(l, i - 1, 3 * j + 2) * db[2];
                    for (int k = 1; k <= 3; ++k) {
                        double v = top[k - 1] * IX2(T0D[k], l, ii, wp);
                        if (adj) v = v * IX2(adj, l, ii, wp);
                        db[k - 1] = v;
                    }
                    IX2(w->flux_direct_dir, l, i, wp) = db[0] + db[1] + db[2];
                }
                for (int i = 0; i <= n_layer; ++i) IX2(fd, l, i, wp) = IX2(w->flux_direct_dir, l, i, wp);
                w->alpha[l] = db[0]; w->fdg2[l] = db[1]; w->fdg3[l] = db[2];
            }
        }
    }
    /* ground sources (triple_column.F90:380-410) */
    for (int l = 0; l < n_profile; ++l) {
        if (solar) {
            const double a = w->alb_dir[l] - w->alb_diff[l];
            w->source_ground[l] = a * w->alpha[l];
            w->sg2[l] = a * w->fdg2[l];
            w->sg3[l] = a * w->fdg3[l];
        } else {
            const double e = (1.0 - w->alb_diff[l]) * w->d_planck_flux_surface[l];
            w->source_ground[l] = OV3(l, n_layer, 9) * e;
            w->sg2[l] = OV3(l, n_layer, 12) * e;
            w->sg3[l] = OV3(l, n_layer, 15) * e;
        }
    }
    /* solver_triple_hogan (solver_triple_hogan.F90:200-410), v_jk = ovl 3 j + k,
     * u_jk = ovl 9 + 3 j + k (0-based regions) */
    double *B[4] = {NULL, w->b11, w->b22, w->b33}, *G[4] = {NULL, w->g11, w->g22, w->g33};
    double *H[4] = {NULL, w->h1, w->h2, w->h3};
    double *ft = w->flux_total;
    for (int l = 0; l < n_profile; ++l) {
        double a[4] = {0.0, 0.0, 0.0, 0.0}, g[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = n_layer + 1; i >= 1; --i) {
            const int ii = i - 1;
            if (i < n_layer + 1 && i >= nct) {
                double th[4], lam[4];
                for (int k = 1; k <= 3; ++k)
                    th[k] = a[1] * OV3(l, i, k - 1) + a[2] * OV3(l, i, 3 + k - 1) + a[3] * OV3(l, i, 6 + k - 1);
                for (int k = 1; k <= 3; ++k) {
                    const double r = IX2(Rr[k], l, ii, wp), t = IX2(T[k], l, ii, wp);
                    const double b = 1.0 / (1.0 - th[k] * r);
                    IX2(B[k], l, ii, wp) = b;
                    IX2(G[k], l, ii, wp) = th[k] * t;
                    IX2(H[k], l, ii, wp) = g[k] + th[k] * IX2(SD[k], l, ii, wp);
                    lam[k] = IX2(SU[k], l, ii, wp) + IX2(H[k], l, ii, wp) * t * b;
                    a[k] = r + th[k] * t * t * b;
                }
                for (int j = 1; j <= 3; ++j)
                    g[j] = OV3(l, i - 1, 9 + 3 * (j - 1)) * lam[1] + OV3(l, i - 1, 9 + 3 * (j - 1) + 1) * lam[2]
                         + OV3(l, i - 1, 9 + 3 * (j - 1) + 2) * lam[3];
            } else if (i < nct - 1) {
                const double r = IX2(w->reflect, l, ii, wp), t = IX2(w->trans, l, ii, wp);
                const double b11 = 1.0 / (1.0 - a[1] * r), gm11 = a[1] * t;
                const double hh1 = g[1] + a[1] * IX2(w->s_down, l, ii, wp);
                IX2(w->b11, l, ii, wp) = b11; IX2(w->g11, l, ii, wp) = gm11; IX2(w->h1, l, ii, wp) = hh1;
                const double lam = t * b11;
                a[1] = r + lam * gm11;
                g[1] = IX2(w->s_up, l, ii, wp) + lam * hh1;
            } else if (i == nct - 1) {
                const double r = IX2(w->reflect, l, ii, wp), t = IX2(w->trans, l, ii, wp);
                const double th11 = (nct < n_layer) ? a[1] * OV3(l, i, 0) + a[2] * OV3(l, i, 3) + a[3] * OV3(l, i, 6)
                                                    : a[1];
                const double b11 = 1.0 / (1.0 - th11 * r), gm11 = th11 * t;
                const double hh1 = g[1] + th11 * IX2(w->s_down, l, ii, wp);
                IX2(w->b11, l, ii, wp) = b11; IX2(w->g11, l, ii, wp) = gm11; IX2(w->h1, l, ii, wp) = hh1;
                const double lam = t * b11;
                a[1] = r + lam * gm11;
                g[1] = IX2(w->s_up, l, ii, wp) + lam * hh1;
            } else if (i == n_layer + 1) {
                a[1] = a[2] = a[3] = w->alb_diff[l];
                g[1] = w->source_ground[l];
                g[2] = w->sg2[l];
                g[3] = w->sg3[l];
            }
        }
        IX2(ft, l, 1, wp) = w->flux_inc_down[l];
        if (nct > 1) IX2(ft, l, 0, wp) = a[1] * IX2(ft, l, 1, wp) + g[1];
        else IX2(ft, l, 0, wp) = g[1] + w->flux_inc_down[l] * (OV3(l, 0, 0) * a[1] + OV3(l, 0, 3) * a[2]
                                                              + OV3(l, 0, 6) * a[3]);
        for (int i = 1; i <= nct - 1; ++i) {
            const int ii = i - 1;
            IX2(ft, l, 2 * i, wp) = (IX2(w->g11, l, ii, wp) * IX2(ft, l, 2 * i - 1, wp) + IX2(w->h1, l, ii, wp))
                * IX2(w->b11, l, ii, wp);
            IX2(ft, l, 2 * i + 1, wp) = IX2(w->trans, l, ii, wp) * IX2(ft, l, 2 * i - 1, wp)
                + IX2(w->reflect, l, ii, wp) * IX2(ft, l, 2 * i, wp) + IX2(w->s_down, l, ii, wp);
        }
        double fdn[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = nct; i <= n_layer; ++i) {
            const int ii = i - 1;
            double d[4];
            if (i > nct) {
                for (int j = 1; j <= 3; ++j)
                    d[j] = OV3(l, i - 1, 3 * (j - 1)) * fdn[1] + OV3(l, i - 1, 3 * (j - 1) + 1) * fdn[2]
                         + OV3(l, i - 1, 3 * (j - 1) + 2) * fdn[3];
            } else {
                for (int j = 1; j <= 3; ++j) d[j] = OV3(l, i - 1, 3 * (j - 1)) * IX2(ft, l, 2 * i - 1, wp);
            }
            double fu_sum = 0.0, fd_sum = 0.0;
            for (int k = 1; k <= 3; ++k) {
                const double fu = (IX2(G[k], l, ii, wp) * d[k] + IX2(H[k], l, ii, wp)) * IX2(B[k], l, ii, wp);
                fdn[k] = IX2(T[k], l, ii, wp) * d[k] + IX2(Rr[k], l, ii, wp) * fu + IX2(SD[k], l, ii, wp);
                fu_sum = fu_sum + fu;
                fd_sum = fd_sum + fdn[k];
            }
            IX2(ft, l, 2 * i, wp) = fu_sum;
            IX2(ft, l, 2 * i + 1, wp) = fd_sum;
        }
    }
#undef OV3
}

/* --------------------------------------------------------------------- */
static int check_options(const socgpu_control *c, const socgpu_spectrum_desc *d,
                         const socgpu_atm *atm, const socgpu_dimen *dm, const socgpu_cld *cld,
                         char *msg, size_t msg_len)
{
    if (c->i_angular_integration != SOCGPU_IP_TWO_STREAM) {
        set_msg(msg, msg_len, "only two-stream angular integration is supported"); return SOCGPU_I_ERR_FATAL; }
    if (c->isolir != SOCGPU_IP_SOLAR && c->isolir != SOCGPU_IP_INFRA_RED) {
        set_msg(msg, msg_len, "isolir must be solar or infra-red"); return SOCGPU_I_ERR_FATAL; }
    if (c->i_gas_overlap != SOCGPU_IP_OVERLAP_RANDOM && c->i_gas_overlap != SOCGPU_IP_OVERLAP_K_EQV_SCL &&
        c->i_gas_overlap != SOCGPU_IP_OVERLAP_K_EQV && c->i_gas_overlap != SOCGPU_IP_OVERLAP_K_EQV_MOD) {
        set_msg(msg, msg_len, "only random and equivalent-extinction gas overlaps are supported");
        return SOCGPU_I_ERR_FATAL; }
    double s, t;
    if (c->i_scatter_method == SOCGPU_IP_SCATTER_FULL) {
        if (two_coeff_basic(c->i_2stream, 0.5, 0.5, &s, &t) != SOCGPU_I_NORMAL) {
            set_msg(msg, msg_len, "unrecognised or unimplemented two-stream scheme"); return SOCGPU_I_ERR_FATAL; }
        const int region = (c->i_cloud == SOCGPU_IP_CLOUD_MIX_MAX || c->i_cloud == SOCGPU_IP_CLOUD_MIX_RANDOM ||
                            c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR);
        const int triple = (c->i_cloud == SOCGPU_IP_CLOUD_TRIPLE || c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR_CNV);
        if (triple && c->i_solver != SOCGPU_IP_SOLVER_TRIPLE_HOGAN) {
            set_msg(msg, msg_len, "three cloud regions require solver_triple_hogan"); return SOCGPU_I_ERR_FATAL; }
        if (triple && c->i_cloud_representation != SOCGPU_IP_CLOUD_CONV_STRAT &&
            c->i_cloud_representation != SOCGPU_IP_CLOUD_CSIW && c->i_cloud_representation != SOCGPU_IP_CLOUD_SPLIT_HOMOGEN &&
            c->i_cloud_representation != SOCGPU_IP_CLOUD_SPLIT_ICE_WATER) {
            set_msg(msg, msg_len, "This representation of clouds is not compatible with separate convective and "
                                  "stratiform overlap.");
            return SOCGPU_I_ERR_FATAL; }
        if (!region && !triple && c->i_solver != SOCGPU_IP_SOLVER_HOMOGEN_DIRECT) {
            set_msg(msg, msg_len, "scattering requires solver_homogen_direct"); return SOCGPU_I_ERR_FATAL; }
        if (region && c->i_solver != SOCGPU_IP_SOLVER_MIX_DIRECT && c->i_solver != SOCGPU_IP_SOLVER_MIX_DIRECT_HOGAN) {
            set_msg(msg, msg_len, "cloud regions require solver_mix_direct or solver_mix_direct_hogan");
            return SOCGPU_I_ERR_FATAL; }
    } else if (c->i_scatter_method == SOCGPU_IP_NO_SCATTER_ABS || c->i_scatter_method == SOCGPU_IP_NO_SCATTER_EXT) {
        if (c->i_solver != SOCGPU_IP_SOLVER_NO_SCAT) {
            set_msg(msg, msg_len, "no-scattering methods require solver_no_scat"); return SOCGPU_I_ERR_FATAL; }
    } else {
        set_msg(msg, msg_len, "unsupported scattering method"); return SOCGPU_I_ERR_FATAL; }
    if (c->i_cloud != SOCGPU_IP_CLOUD_CLEAR && c->i_cloud != SOCGPU_IP_CLOUD_MCICA &&
        c->i_cloud != SOCGPU_IP_CLOUD_MIX_MAX && c->i_cloud != SOCGPU_IP_CLOUD_MIX_RANDOM &&
        c->i_cloud != SOCGPU_IP_CLOUD_TRIPLE && c->i_cloud != SOCGPU_IP_CLOUD_PART_CORR &&
        c->i_cloud != SOCGPU_IP_CLOUD_PART_CORR_CNV) {
        set_msg(msg, msg_len, "only clear-sky, McICA and two- and three-region cloud schemes are supported");
        return SOCGPU_I_ERR_FATAL; }
    if (c->i_cloud != SOCGPU_IP_CLOUD_CLEAR &&
        (!cld || cld->n_condensed < 1 || !cld->type_condensed || !cld->i_cloud_type || !cld->i_condensed_param ||
         !cld->i_condensed_type || !cld->condensed_mix_ratio || !cld->condensed_dim_char || !cld->w_cloud ||
         !cld->frac_cloud || cld->n_cloud_type < 1 ||
         cld->n_cloud_type > ((c->i_cloud == SOCGPU_IP_CLOUD_TRIPLE || c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR_CNV) ? 4 : 2))) {
        set_msg(msg, msg_len, "clouds require cloud fields"); return SOCGPU_I_ERR_FATAL; }
    if (c->i_cloud == SOCGPU_IP_CLOUD_MCICA &&
        (!cld->c_sub || !cld->frac_cloudy || !cld->subcol_k || !cld->first_subcol_k || !cld->subcol_reorder)) {
        set_msg(msg, msg_len, "McICA requires the subcolumn fields"); return SOCGPU_I_ERR_FATAL; }
    if ((c->i_cloud == SOCGPU_IP_CLOUD_MIX_MAX || c->i_cloud == SOCGPU_IP_CLOUD_MIX_RANDOM ||
         c->i_cloud == SOCGPU_IP_CLOUD_TRIPLE || c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR ||
         c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR_CNV) && c->i_scatter_method != SOCGPU_IP_SCATTER_FULL) {
        set_msg(msg, msg_len, "cloud regions require full scattering"); return SOCGPU_I_ERR_FATAL; }
    if (c->first_band < 1 || c->last_band > d->n_band || c->first_band > c->last_band) {
        set_msg(msg, msg_len, "band range outside the spectrum"); return SOCGPU_I_ERR_RANGE; }
    if (atm->n_profile < 0 || atm->n_profile > dm->nd_profile || atm->n_layer < 1 || atm->n_layer > dm->nd_layer) {
        set_msg(msg, msg_len, "profile/layer counts exceed their dimensions"); return SOCGPU_I_ERR_RANGE; }
    if (c->l_continuum && d->n_band_continuum &&
        (!atm->density || d->index_water < 1 || !d->k_cont || !d->scale_cont)) {
        set_msg(msg, msg_len, "continuum absorption needs the layer density and water vapour"); return SOCGPU_I_ERR_FATAL; }
    if (c->isolir == SOCGPU_IP_INFRA_RED && !d->thermal_coeff) {
        set_msg(msg, msg_len, "infra-red calculation without Planck data"); return SOCGPU_I_ERR_FATAL; }
    if (c->isolir == SOCGPU_IP_SOLAR && !d->solar_flux_band) {
        set_msg(msg, msg_len, "solar calculation without solar spectrum"); return SOCGPU_I_ERR_FATAL; }
    return SOCGPU_I_NORMAL;
}

/* radiance_calc (radiance_calc.F90:16-2160) for one column segment.  The
 * caller's arrays are viewed from profile p0 on; dimen->nd_profile stays
 * the leading dimension. */
static int segment_radiance_calc(const socgpu_control *c, const socgpu_dimen *dm,
                                 const socgpu_spectrum_desc *d, const socgpu_atm *atm0,
                                 const socgpu_cld *cld0, const socgpu_aer *aer0,
                                 const socgpu_bound *bd, socgpu_radout *out0,
                                 int p0, int np, char *msg, size_t msg_len)
{
    int status = check_options(c, d, atm0, dm, cld0, msg, msg_len);
    if (status != SOCGPU_I_NORMAL) return status;
    if (np <= 0) return SOCGPU_I_NORMAL;
    int ndp = dm->nd_profile, ndl = dm->nd_layer, n_layer = atm0->n_layer;
    int l_cloud = (c->i_cloud == SOCGPU_IP_CLOUD_MCICA);
    int l_triple = (c->i_cloud == SOCGPU_IP_CLOUD_TRIPLE || c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR_CNV);
    int l_region = (c->i_cloud == SOCGPU_IP_CLOUD_MIX_MAX || c->i_cloud == SOCGPU_IP_CLOUD_MIX_RANDOM ||
                    c->i_cloud == SOCGPU_IP_CLOUD_PART_CORR) || l_triple;
    int ict = dm->id_cloud_top - 1;

    /* views shifted to the first profile of the segment */
    socgpu_atm atm = *atm0;
    atm.p += p0; atm.t += p0; atm.t_level += p0; atm.mass += p0; atm.gas_mix_ratio += p0;
    if (atm.p_level) atm.p_level += p0;
    if (atm.density) atm.density += p0;
    socgpu_aer aerv, *aer = NULL;
    if (aer0) {
        aerv = *aer0; aer = &aerv;
        if (aerv.n_mode > 0) {
            aerv.mode_mix_ratio += p0; aerv.mode_absorption += p0;
            aerv.mode_scattering += p0; aerv.mode_asymmetry += p0;
        }
        if (aerv.n_aerosol_mr > 0 && aerv.mix_ratio) aerv.mix_ratio += p0;
        if (aerv.mean_rel_humidity) aerv.mean_rel_humidity += p0;
        if (aerv.pressure_prsc) aerv.pressure_prsc += p0;
        if (aerv.absorption_prsc) aerv.absorption_prsc += p0;
        if (aerv.scattering_prsc) aerv.scattering_prsc += p0;
        if (aerv.phase_fnc_prsc) aerv.phase_fnc_prsc += p0;
    }
    socgpu_cld cldv, *cld = NULL;
    if (cld0 && (l_cloud || l_region)) {
        cldv = *cld0; cld = &cldv;
        cldv.condensed_mix_ratio += p0; cldv.condensed_dim_char += p0;
        cldv.w_cloud += p0; cldv.frac_cloud += p0;
        if (cldv.c_sub) cldv.c_sub += p0;
        if (cldv.frac_cloudy) cldv.frac_cloudy += p0;
        if (cldv.n_subcol_cld) cldv.n_subcol_cld += p0;
    }
    socgpu_radout out = *out0;
    out.flux_up += p0; out.flux_down += p0;
    if (out.flux_direct) out.flux_direct += p0;
    if (out.flux_div) out.flux_div += p0;
    if (out.heating_rate) out.heating_rate += p0;
    if (out.flux_up_band) out.flux_up_band += p0;
    if (out.flux_down_band) out.flux_down_band += p0;

    int max_abs = 1;
    for (int b = c->first_band - 1; b < c->last_band; ++b)
        if (d->n_band_absorb[b] > max_abs) max_abs = d->n_band_absorb[b];
    work w;
    work_init(&w, np, ndl, np, n_layer, cld ? cld->n_condensed : 0, max_abs);
    int wp = np;
    lookup_fac lf;
    lookup_fac_init(&lf, c, d, &atm, np, n_layer, ndp, wp, ndl);
    double *kterm = zalloc((size_t)wp * ndl), *k_eqv = zalloc((size_t)wp * ndl), *adj = zalloc((size_t)wp * ndl);
    if (l_region) {
        /* set_cloud_geometry, aggregate_cloud and overlap_coupled
         * (radiance_calc.F90:640-700) */
        w.nct = cloud_top(cld, ndp, ict, np, n_layer);
        if (l_triple) overlap_coupled3(&w, c, cld, atm.p, ndp, ict);
        else overlap_coupled2(&w, cld, atm.p, ndp, ict, c->i_cloud);
    }

    /* zero the outputs (augment_radiance's l_initial branch is equivalent) */
    for (int i = 0; i <= n_layer; ++i)
        for (int l = 0; l < np; ++l) {
            IX2(out.flux_up, l, i, ndp) = 0.0;
            IX2(out.flux_down, l, i, ndp) = 0.0;
            if (out.flux_direct) IX2(out.flux_direct, l, i, ndp) = 0.0;
        }
    if (out.flux_div)
        for (int i = 0; i < n_layer; ++i)
            for (int l = 0; l < np; ++l) IX2(out.flux_div, l, i, ndp) = 0.0;
    for (int b = 0; b < d->n_band; ++b)
        for (int i = 0; i <= n_layer; ++i)
            for (int l = 0; l < np; ++l) {
                if (out.flux_up_band) IX3(out.flux_up_band, l, i, b, ndp, ndl + 1) = 0.0;
                if (out.flux_down_band) IX3(out.flux_down_band, l, i, b, ndp, ndl + 1) = 0.0;
            }

    for (int b = c->first_band - 1; b < c->last_band && status == SOCGPU_I_NORMAL; ++b) {
        double weight_band = c->weight_band ? c->weight_band[b] : 1.0;
        status = grey_opt_prop(&w, c, dm, d, &atm, aer, cld, b, l_cloud || l_region);
        if (status != SOCGPU_I_NORMAL) { set_msg(msg, msg_len, "unsupported optical property option"); break; }

        /* gas scaling of each absorber (radiance_calc.F90:1330-1470) */
        int n_abs = c->l_gas ? d->n_band_absorb[b] : 0;
        int gas_of[SOCGPU_MAX_SPECIES], nk[SOCGPU_MAX_SPECIES];
        for (int j = 0; j < n_abs; ++j) {
            int g = sp_index_absorb(d, j, b);
            gas_of[j] = g;
            nk[j] = sp_bg(d->i_band_k, d, b, g);
            int isk = sp_bg(d->i_scale_k, d, b, g);
            double *gfr = w.gfr + (size_t)wp * ndl * j;
            if (isk == SOCGPU_IP_SCALE_BAND) {
                status = scale_absorb(np, n_layer, ndp, wp, atm.p, atm.t, gfr, sp_bg(d->i_scale_fnc, d, b, g),
                                      IX2(d->p_ref, g, b, d->nd_species), IX2(d->t_ref, g, b, d->nd_species),
                                      sp_scale(d, 0, b, g), d->l_doppler ? d->l_doppler[g] : 0,
                                      d->doppler_cor ? d->doppler_cor[g] : 0.0, d, 0, b + 1);
                for (int i = 0; i < n_layer; ++i)
                    for (int l = 0; l < np; ++l) {
                        double v = IX2(gfr, l, i, wp) * IX3(atm.gas_mix_ratio, l, i, g, ndp, ndl);
                        IX2(gfr, l, i, wp) = v > 0.0 ? v : 0.0;
                    }
            } else if (isk == SOCGPU_IP_SCALE_NULL) {
                for (int i = 0; i < n_layer; ++i)
                    for (int l = 0; l < np; ++l) IX2(gfr, l, i, wp) = IX3(atm.gas_mix_ratio, l, i, g, ndp, ndl);
            } else if (isk != SOCGPU_IP_SCALE_TERM) {
                status = SOCGPU_I_ERR_FATAL;
            }
            if (status != SOCGPU_I_NORMAL) { set_msg(msg, msg_len, "illegal type of scaling"); break; }
        }
        if (status != SOCGPU_I_NORMAL) break;
        /* Planck terms (diff_planck_source_mod.F90:102-136) and boundary
         * fluxes (solve_band_random_overlap.F90:565-600) */
        for (int l = 0; l < np; ++l) {
            w.sec_0[l] = bd->zen_0 ? bd->zen_0[p0 + l] : 1.0;
            w.alb_diff[l] = IX3(bd->rho_alb, p0 + l, 0, b, ndp, 2);
            w.alb_dir[l] = IX3(bd->rho_alb, p0 + l, 1, b, ndp, 2);
        }
        if (c->isolir == SOCGPU_IP_INFRA_RED) {
            for (int l = 0; l < np; ++l)
                IX2(w.planck_flux, l, 0, wp) = planck_flux_band(d, b, IX2(atm.t_level, l, 0, ndp));
            for (int i = 1; i <= n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    IX2(w.planck_flux, l, i, wp) = planck_flux_band(d, b, IX2(atm.t_level, l, i, ndp));
                    IX2(w.planck_diff, l, i - 1, wp) = IX2(w.planck_flux, l, i, wp) - IX2(w.planck_flux, l, i - 1, wp);
                }
            if (c->l_ir_source_quad)
                for (int i = 1; i <= n_layer; ++i)
                    for (int l = 0; l < np; ++l) {
                        double bt = planck_flux_band(d, b, IX2(atm.t, l, i - 1, ndp));
                        IX2(w.planck_diff_2, l, i - 1, wp) = 2.0 * (IX2(w.planck_flux, l, i, wp)
                            + IX2(w.planck_flux, l, i - 1, wp) - 2.0 * bt);
                    }
            for (int l = 0; l < np; ++l) {
                /* the surface's Planck flux given per band (l_flux_ground and tiles,
                 * diff_planck_source_mod.F90:123-135), else that of t_ground */
                w.flux_ground[l] = bd->flux_ground ? IX2(bd->flux_ground, p0 + l, b, ndp)
                                                   : planck_flux_band(d, b, bd->t_ground[p0 + l]);
                w.flux_inc_direct[l] = 0.0;
                w.flux_inc_down[l] = -IX2(w.planck_flux, l, 0, wp);
                w.d_planck_flux_surface[l] = w.flux_ground[l] - IX2(w.planck_flux, l, n_layer, wp);
            }
        } else {
            for (int l = 0; l < np; ++l) {
                double solar_irrad_band = bd->solar_irrad[p0 + l] * d->solar_flux_band[b];
                w.d_planck_flux_surface[l] = 0.0;
                w.flux_inc_down[l] = solar_irrad_band / w.sec_0[l];
                w.flux_inc_direct[l] = solar_irrad_band / w.sec_0[l];
            }
        }

        int keqv = (c->i_gas_overlap == SOCGPU_IP_OVERLAP_K_EQV_SCL || c->i_gas_overlap == SOCGPU_IP_OVERLAP_K_EQV
                    || c->i_gas_overlap == SOCGPU_IP_OVERLAP_K_EQV_MOD) && n_abs > 0;
        w.adj = NULL;
        if (keqv) {
            status = k_eqv_minor(&w, c, &lf, d, &atm, np, n_layer, ndp, b, n_abs, gas_of, nk, k_eqv,
                                 c->isolir == SOCGPU_IP_SOLAR ? adj : NULL);
            if (status != SOCGPU_I_NORMAL) { set_msg(msg, msg_len, "illegal type of scaling"); break; }
            if (c->isolir == SOCGPU_IP_SOLAR) w.adj = adj;
        }

        /* k-terms: products over the absorbers under random overlap
         * (solve_band_random_overlap.F90:533-560), the major absorber's
         * terms under k_eqv_scl (solve_band_k_eqv_scl.F90:1043-1100) */
        int n_term = 1;
        if (keqv) n_term = nk[0];
        else for (int j = 0; j < n_abs; ++j) n_term *= nk[j];
        int n_sum = keqv ? 1 : n_abs;
        for (int kt = 0; kt < n_term; ++kt) {
            int iex_of[SOCGPU_MAX_SPECIES];
            double product_weight = 1.0;
            int step_prod = 1;
            for (int j = 0; j < n_sum; ++j) {
                step_prod *= nk[j];
                int step = n_term / step_prod;
                iex_of[j] = (kt / step) % nk[j];
                double wj = sp_kw(d->w, d, iex_of[j], b, gas_of[j]);
                product_weight = (j == 0) ? wj : product_weight * wj;
            }
            if (!keqv && n_abs > 0 && !(product_weight > 0.0)) continue;
            if (n_abs == 0) product_weight = 1.0;
            /* gas_optical_properties (gas_optical_properties.F90:80-95) */
            for (int i = 0; i < n_layer; ++i)
                for (int l = 0; l < np; ++l) IX2(w.k_gas_abs, l, i, wp) = 0.0;
            for (int j = 0; j < n_sum; ++j) {
                status = absorber_term_k(&lf, d, &atm, np, n_layer, ndp, wp, ndl, b, gas_of[j], iex_of[j],
                                         w.gfr + (size_t)wp * ndl * j, w.beta, kterm);
                if (status != SOCGPU_I_NORMAL) break;
                for (int i = 0; i < n_layer; ++i)
                    for (int l = 0; l < np; ++l)
                        IX2(w.k_gas_abs, l, i, wp) = (j == 0) ? IX2(kterm, l, i, wp)
                                                              : IX2(w.k_gas_abs, l, i, wp) + IX2(kterm, l, i, wp);
            }
            if (status != SOCGPU_I_NORMAL) { set_msg(msg, msg_len, "illegal type of scaling"); break; }
            if (l_cloud) {
                solve_mcica_term(&w, c, dm, d, atm.mass, cld, b, n_abs > 0 ? iex_of[0] : 0);
            } else if (l_triple) {
                solve_triple_term(&w, c, dm, atm.mass, cld);
            } else if (l_region) {
                solve_region_term(&w, c, dm, atm.mass, cld);
            } else {
                clear_coefficients(&w, c, atm.mass, ndp);
                column_solve(&w, c, c->i_scatter_method != SOCGPU_IP_SCATTER_FULL);
            }
            /* augment_radiance / augment_channel (augment_channel_mod.F90:158-235) */
            double wi = weight_band * product_weight;
            for (int i = 0; i <= n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    IX2(out.flux_up, l, i, ndp) = IX2(out.flux_up, l, i, ndp) + wi * IX2(w.flux_total, l, 2 * i, wp);
                    IX2(out.flux_down, l, i, ndp) = IX2(out.flux_down, l, i, ndp) + wi * IX2(w.flux_total, l, 2 * i + 1, wp);
                    if (out.flux_direct && c->isolir == SOCGPU_IP_SOLAR)
                        IX2(out.flux_direct, l, i, ndp) = IX2(out.flux_direct, l, i, ndp) + wi * IX2(w.flux_direct, l, i, wp);
                    if (out.flux_up_band)
                        IX3(out.flux_up_band, l, i, b, ndp, ndl + 1) += wi * IX2(w.flux_total, l, 2 * i, wp);
                    if (out.flux_down_band)
                        IX3(out.flux_down_band, l, i, b, ndp, ndl + 1) += wi * IX2(w.flux_total, l, 2 * i + 1, wp);
                }
            if (out.flux_div)
                for (int i = 1; i <= n_layer; ++i)
                    for (int l = 0; l < np; ++l)
                        IX2(out.flux_div, l, i - 1, ndp) = IX2(out.flux_div, l, i - 1, ndp) + wi
                            * (IX2(w.flux_total, l, 2 * i, wp) - IX2(w.flux_total, l, 2 * i - 2, wp)
                               + IX2(w.flux_total, l, 2 * i - 1, wp) - IX2(w.flux_total, l, 2 * i + 1, wp));
        }
        /* adjust_ir_radiance (adjust_ir_radiance.F90:75-95, adjust_ir_channel) */
        if (c->isolir == SOCGPU_IP_INFRA_RED)
            for (int i = 0; i <= n_layer; ++i)
                for (int l = 0; l < np; ++l) {
                    double bw = IX2(w.planck_flux, l, i, wp) * weight_band;
                    IX2(out.flux_up, l, i, ndp) = IX2(out.flux_up, l, i, ndp) + bw;
                    IX2(out.flux_down, l, i, ndp) = IX2(out.flux_down, l, i, ndp) + bw;
                    if (out.flux_up_band) IX3(out.flux_up_band, l, i, b, ndp, ndl + 1) += bw;
                    if (out.flux_down_band) IX3(out.flux_down_band, l, i, b, ndp, ndl + 1) += bw;
                }
    }
    /* heating rate (l_run_cdf.F90:1340-1380) */
    if (status == SOCGPU_I_NORMAL && out.heating_rate)
        for (int i = 1; i <= n_layer; ++i)
            for (int l = 0; l < np; ++l) {
                double hc = IX2(atm.mass, l, i - 1, ndp) * cp_air_dry;
                double hr;
                if (c->l_flux_div && out.flux_div) {
                    hr = seconds_per_day * IX2(out.flux_div, l, i - 1, ndp) / hc;
                } else {
                    double fn0 = IX2(out.flux_down, l, i - 1, ndp) - IX2(out.flux_up, l, i - 1, ndp);
                    double fn1 = IX2(out.flux_down, l, i, ndp) - IX2(out.flux_up, l, i, ndp);
                    hr = (fn0 - fn1) / hc;
                    hr = seconds_per_day * hr;
                }
                IX2(out.heating_rate, l, i - 1, ndp) = hr;
            }
    (void)ict;
    lookup_fac_free(&lf);
    free(kterm); free(k_eqv); free(adj);
    work_free(&w);
    return status;
}

int oracle_radiance_calc(const socgpu_control *c, const socgpu_dimen *dm,
                         const socgpu_spectrum_desc *d, const socgpu_atm *atm,
                         const socgpu_cld *cld, const socgpu_aer *aer,
                         const socgpu_bound *bd, socgpu_radout *out,
                         char *msg, size_t msg_len)
{
    return segment_radiance_calc(c, dm, d, atm, cld, aer, bd, out, 0, atm->n_profile, msg, msg_len);
}

int oracle_radiance_calc_segmented(const socgpu_control *c, const socgpu_dimen *dm,
                                   const socgpu_spectrum_desc *d, const socgpu_atm *atm,
                                   const socgpu_cld *cld, const socgpu_aer *aer,
                                   const socgpu_bound *bd, socgpu_radout *out,
                                   int n_threads, char *msg, size_t msg_len)
{
    int n = atm->n_profile;
    int status = check_options(c, d, atm, dm, cld, msg, msg_len);
    if (status != SOCGPU_I_NORMAL) return status;
#ifdef _OPENMP
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#else
    n_threads = 1;
#endif
    int n_seg = n_threads * 4;
    if (n_seg > n) n_seg = n > 0 ? n : 1;
    int worst = SOCGPU_I_NORMAL;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads) reduction(max:worst)
#endif
    for (int s = 0; s < n_seg; ++s) {
        int p0 = (int)((long long)n * s / n_seg), p1 = (int)((long long)n * (s + 1) / n_seg);
        char m[256] = {0};
        int st = segment_radiance_calc(c, dm, d, atm, cld, aer, bd, out, p0, p1 - p0, m, sizeof m);
        if (st > worst) worst = st;
    }
    if (worst != SOCGPU_I_NORMAL) set_msg(msg, msg_len, "a column segment failed");
    return worst;
}

/* --------------------------------------------------------------------- */
/* cloud_gen (socrates_cloud_gen.F90:8-470).  Cloud arrays are indexed
 * (nd_profile, cloud_top:nd_layer); zf and the column seeds by profile.  */
static const int lcg_m = 86436, lcg_a = 1093, lcg_c = 18257;   /* socrates_cloud_gen.F90:48-50 */

static inline int lcg_next(int x)
{   /* temp = x*a+c; x = temp - int(real(temp)*rm)*m  (socrates_cloud_gen.F90:180-203) */
    const double rm = 1.0 / (double)lcg_m;
    int temp = x * lcg_a + lcg_c;
    return temp - (int)((double)temp * rm) * lcg_m;
}

static inline double philox_u01(uint32_t word) { return (double)word * (1.0 / 4294967296.0); }

int oracle_cloud_gen(int nd_layer, int cloud_top, int n_layer, int nd_profile,
                     int il1, int il2, int n_subcol, int n1, int n2,
                     int ipph, int ioverlap, const int *rand_seed,
                     const double *rlc_cf, const double *rlc_cw,
                     const double *sigma_qcw, const double *avg_cf,
                     const double *c_cloud, const double *c_ratio,
                     const double *zf, const double *xcw,
                     int *n_subcol_cld, double *c_sub, int rng)
{
    const double rm = 1.0 / (double)lcg_m;
    const double cut = EPS_R;
    int ndc = nd_layer - cloud_top + 1;
    int rand_seed_max = (2147483647 - lcg_c) / lcg_a;
#define CLD(a, l, k) ((a)[(size_t)((l) - 1) + (size_t)nd_profile * (size_t)((k) - cloud_top)])
#define CSUB(l, k, s) (c_sub[(size_t)((l) - 1) + (size_t)nd_profile * ((size_t)((k) - cloud_top) + (size_t)ndc * (size_t)((s) - 1))])
    if (ioverlap < 0 || ioverlap > 3) return SOCGPU_I_ERR_FATAL;
    for (int il = il1; il <= il2; ++il)
        for (int k = cloud_top; k <= nd_layer; ++k)
            for (int s = 1; s <= n_subcol; ++s) CSUB(il, k, s) = 0.0;

    /* first and last cloudy layers over all columns */
    int k_top = 0, l_top = 0;
    for (int k = cloud_top; k <= n_layer && !l_top; ++k)
        for (int il = il1; il <= il2; ++il) { k_top = k; if (CLD(avg_cf, il, k) > cut) l_top = 1; }
    if (!l_top) k_top = 0;
    if (k_top == 0) {
        for (int il = il1; il <= il2; ++il) n_subcol_cld[il - 1] = 0;
        return SOCGPU_I_NORMAL;
    }
    int k_base = 0, l_bot = 0;
    for (int k = n_layer; k >= cloud_top && !l_bot; --k)
        for (int il = il1; il <= il2; ++il) { k_base = k; if (CLD(avg_cf, il, k) >= cut) l_bot = 1; }

    double *alpha = zalloc((size_t)(nd_layer + 2)), *rcorr = zalloc((size_t)(nd_layer + 2));
    int *seed_x = (int *)calloc((size_t)n_subcol, sizeof(int));
    int *seed_y = (int *)calloc((size_t)n_subcol, sizeof(int));
    for (int il = il1; il <= il2; ++il) {
        /* seed streams (socrates_cloud_gen.F90:180-203) */
        int rd = abs(rand_seed[il - 1]) % rand_seed_max;
        for (int i = 0; i < n_subcol; ++i) rd = lcg_next(rd);
        for (int i = 0; i < n_subcol; ++i) { rd = lcg_next(rd); seed_x[i] = rd; }
        for (int i = 0; i < n_subcol; ++i) { rd = lcg_next(rd); seed_y[i] = rd; }
        uint32_t key[2] = {(uint32_t)rand_seed[il - 1], 0x534F4352u};

        /* overlap parameters alpha/rcorr (socrates_cloud_gen.F90:338-375) */
        if (ioverlap >= 1)
            for (int k = k_top - 1; k <= k_base - 1; ++k) {
                double a = 0.0, r = 0.0;
                if (!(ioverlap == 1 || k < cloud_top)) {
                    if (ioverlap == 2 || CLD(avg_cf, il, k) > 0.0) {
                        double dz = zf[(size_t)(il - 1) + (size_t)nd_profile * (size_t)(k - 1)]
                                  - zf[(size_t)(il - 1) + (size_t)nd_profile * (size_t)k];
                        a = CLD(rlc_cf, il, k) > 0.0 ? exp(dz / CLD(rlc_cf, il, k)) : 0.0;
                        r = CLD(rlc_cw, il, k) > 0.0 ? exp(dz / CLD(rlc_cw, il, k)) : 0.0;
                    }
                }
                alpha[k] = a; rcorr[k] = r;
            }
        int i_loc = 1;
        /* x and y persist across the subcolumns of a column, as the
         * reference's per-column arrays x(il), y(il) do */
        double x = 0.0, y = 0.0, x1, y1;
        for (int i = 1; i <= n_subcol; ++i) {
            int int_x = seed_x[i - 1], int_y = seed_y[i - 1];
            int l_cld = 0;
            for (int k = k_top; k <= k_base; ++k) {
                double cf = CLD(avg_cf, il, k);
                if (!(cf > 0.0)) continue;
                uint32_t u[4] = {0, 0, 0, 0};
                if (rng == SOCGPU_RNG_PHILOX) {
                    uint32_t ctr[4] = {(uint32_t)k, (uint32_t)i, 0u, 0u};
                    oracle_philox4x32_10(ctr, key, u);
                }
                double zcw;
                if (ioverlap == 0) {
                    /* maximum-random (socrates_cloud_gen.F90:251-330) */
                    if (rng == SOCGPU_RNG_PHILOX) { x = philox_u01(u[0]); y = philox_u01(u[1]); }
                    else {
                        int_x = lcg_next(int_x); x = (double)int_x * rm;
                        int_y = lcg_next(int_y); y = (double)int_y * rm;
                    }
                    if (k == cloud_top) {
                        if (rng == SOCGPU_RNG_PHILOX) { x = philox_u01(u[2]); y = philox_u01(u[3]); }
                        else {
                            int_x = lcg_next(int_x); x = (double)int_x * rm;
                            int_y = lcg_next(int_y); y = (double)int_y * rm;
                        }
                    } else if (x < (1.0 - CLD(avg_cf, il, k - 1))) {
                        if (rng == SOCGPU_RNG_PHILOX) { x1 = philox_u01(u[2]); y1 = philox_u01(u[3]); }
                        else {
                            int_x = lcg_next(int_x); x1 = (double)int_x * rm;
                            int_y = lcg_next(int_y); y1 = (double)int_y * rm;
                        }
                        x = x1 * (1.0 - CLD(avg_cf, il, k - 1));
                        y = y1;
                    }
                } else {
                    /* random / exponential / exponential-random (socrates_cloud_gen.F90:376-460) */
                    if (rng == SOCGPU_RNG_PHILOX) { x1 = philox_u01(u[0]); y1 = philox_u01(u[1]); }
                    else {
                        int_x = lcg_next(int_x); x1 = (double)int_x * rm;
                        int_y = lcg_next(int_y); y1 = (double)int_y * rm;
                    }
                    if (x1 >= alpha[k - 1]) {
                        if (rng == SOCGPU_RNG_PHILOX) x = philox_u01(u[2]);
                        else { int_x = lcg_next(int_x); x = (double)int_x * rm; }
                    }
                    if (y1 >= rcorr[k - 1]) {
                        if (rng == SOCGPU_RNG_PHILOX) y = philox_u01(u[3]);
                        else { int_y = lcg_next(int_y); y = (double)int_y * rm; }
                    }
                }
                if (x < cf) {
                    if (ipph == 0) {
                        zcw = 1.0;
                    } else {
                        double sig = CLD(sigma_qcw, il, k);
                        double ratio = 1.0;
                        if (ioverlap != 0) {
                            if (x < CLD(c_cloud, il, k)) ratio = CLD(c_ratio, il, k);
                            else {
                                double cc = CLD(c_cloud, il, k);
                                ratio = (cc > 0.0 && cc < cf) ? (cf - CLD(c_ratio, il, k) * cc > 0.0 ?
                                         (cf - CLD(c_ratio, il, k) * cc) : 0.0) / (cf - cc) : 1.0;
                            }
                        }
                        double rind1 = y * (n1 - 1) + 1.0;
                        int ind1 = (int)rind1; if (ind1 > n1 - 1) ind1 = n1 - 1; if (ind1 < 1) ind1 = 1;
                        rind1 = rind1 - (double)ind1; if (rind1 > 1.0) rind1 = 1.0; if (rind1 < 0.0) rind1 = 0.0;
                        double rind2 = 40.0 * sig - 3.0;
                        int ind2 = (int)rind2; if (ind2 > n2 - 1) ind2 = n2 - 1; if (ind2 < 1) ind2 = 1;
                        rind2 = rind2 - (double)ind2; if (rind2 > 1.0) rind2 = 1.0; if (rind2 < 0.0) rind2 = 0.0;
#define XCW(a, b) xcw[(size_t)((a) - 1) + (size_t)n1 * (size_t)((b) - 1)]
                        zcw = (1.0 - rind1) * (1.0 - rind2) * XCW(ind1, ind2)
                            + (1.0 - rind1) * rind2 * XCW(ind1, ind2 + 1)
                            + rind1 * (1.0 - rind2) * XCW(ind1 + 1, ind2)
                            + rind1 * rind2 * XCW(ind1 + 1, ind2 + 1);
#undef XCW
                        zcw = zcw * ratio;
                    }
                    l_cld = 1;
                    CSUB(il, k, i_loc) = zcw;
                }
            }
            if (l_cld) i_loc = i_loc + 1;
        }
        n_subcol_cld[il - 1] = i_loc - 1;
    }
    free(alpha); free(rcorr); free(seed_x); free(seed_y);
#undef CLD
#undef CSUB
    return SOCGPU_I_NORMAL;
}
