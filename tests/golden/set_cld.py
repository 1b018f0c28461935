"""A numpy restatement of the cloud set-up runes does before radiance_calc
(socrates_set_control.F90:291-370, socrates_set_cld.F90:170-850,
socrates_set_cld_dim.F90:155-230 and 300-470), for the representations with
stratiform water and ice (ip_cloud_homogen, ip_cloud_ice_water and their
combinations with convective cloud).  Test infrastructure: it builds the
cloud fields that radiance.Marshal passes to the oracle, for comparison with
socgpu_runes, which maps the same arguments in C++.

Arrays are (n_profile, n_layer), top layer first, grid-box values as runes
takes them; the result holds full-height arrays with the cloudy layers
id_cloud_top..n_layer set."""
import numpy as np

from socrates_gb300 import abi

EPS = np.finfo(np.float64).eps
MIN_CLOUD_FRACTION = 0.001


def _split(fl, fi, f, cmr, types, tw, ti):
    """split_mix_phase (socrates_set_cld.F90:905-935) and the proportional
    fractions that follow it, elementwise; fl, fi are modified."""
    out_l, out_i = np.zeros_like(fl), np.zeros_like(fi)
    for q in np.ndindex(fl.shape):
        if fl[q] + fi[q] > EPS:
            mix = fl[q] + fi[q] - f[q]
            if mix > EPS and fl[q] > EPS and fi[q] > EPS:
                lm = sum(cmr[k][q] / fl[q] for k in range(len(types)) if types[k] == tw)
                im = sum(cmr[k][q] / fi[q] for k in range(len(types)) if types[k] == ti)
                if lm + im > EPS:
                    fl[q], fi[q] = max(fl[q] - mix * im / (lm + im), 0.0), max(fi[q] - mix * lm / (lm + im), 0.0)
            out_l[q] = f[q] * fl[q] / (fl[q] + fi[q])
            out_i[q] = f[q] * fi[q] / (fl[q] + fi[q])
    return out_l, out_i


def ice_dim_from_t(scheme, t):
    """set_ice_dim's temperature parametrizations (socrates_set_cld_dim.F90:385-445)."""
    if scheme == 6:
        return np.minimum(7.198755e-04, np.exp(5.522e-02 * (t - 2.7965e+02)) / 9.702e+02)
    if scheme in (12, 16):
        dge = np.where(t < 216.208, 7.5094588e-04 * np.exp(0.05 * (t - 279.5)) + 5.0830326e-07,
                       1.3505403e-04 * np.exp(0.05 * (t - 279.5)) + 2.6517429e-05)
        return (3.0 / 2.0) * (3.0 / (2.0 * np.sqrt(3.0))) * np.minimum(1.24e-04, np.maximum(8.0e-06, dge))
    if scheme == 19:
        return 1.868e-6 * t - 353.613e-6
    return np.full_like(t, 30.0e-6)


def set_cld(sp, t, rep, i_st_water, i_st_ice, n_cloud_layer=0, i_inhom=abi.IP_HOMOGENEOUS, cloud_frac=None,
            conv_frac=None, liq_frac=None, ice_frac=None, liq_conv_frac=None, ice_conv_frac=None, liq_mmr=None,
            ice_mmr=None, liq_conv_mmr=None, ice_conv_mmr=None, liq_dim=None, ice_dim=None, liq_rsd=None,
            ice_rsd=None, cloud_horizontal_rsd=None, i_drop_re=abi.IP_RE_EXTERNAL, liq_dim_constant=None):
    """col.cld for radiance.Marshal and the id_cloud_top runes uses."""
    n, L = t.shape
    ict = L + 1 - min(n_cloud_layer, L) if n_cloud_layer > 0 else 1
    cl = slice(ict - 1, L)
    homogen = rep in (abi.IP_CLOUD_HOMOGEN, abi.IP_CLOUD_COMBINE_HOMOGEN)
    combine = rep in (abi.IP_CLOUD_COMBINE_HOMOGEN, abi.IP_CLOUD_COMBINE_ICE_WATER)
    g = lambda a: np.maximum(np.asarray(a, dtype=np.float64)[:, cl], 0.0)
    types = [1, 1] if homogen else [abi.IP_CLOUD_TYPE_WATER, abi.IP_CLOUD_TYPE_ICE]
    nct = 1 if homogen else 2
    cmr, rsd = [], []
    c_ratio = np.zeros_like(g(t))
    for water, mmr, conv, r in ((True, liq_mmr, liq_conv_mmr, liq_rsd), (False, ice_mmr, ice_conv_mmr, ice_rsd)):
        m = g(mmr)
        if combine and conv is not None:
            m = m + g(conv)
            c_ratio = c_ratio + g(conv)
        rr = g(r) if r is not None else np.full_like(m, cloud_horizontal_rsd if cloud_horizontal_rsd else 0.0)
        if i_inhom == abi.IP_SCALING:
            m = m / (1.0 + rr ** 2)
        cmr.append(m)
        rsd.append(rr)
    c_cloud = np.zeros_like(c_ratio)
    if homogen:
        frac = [g(cloud_frac)]
        if combine and conv_frac is not None:
            c_cloud = g(conv_frac)
            frac[0] = frac[0] + c_cloud
    else:
        if cloud_frac is not None:
            fl, fi = _split(g(liq_frac), g(ice_frac), g(cloud_frac), cmr, types, 1, 2)
        else:
            fl, fi = g(liq_frac), g(ice_frac)
        frac = [fl, fi]
        if combine and liq_conv_frac is not None and ice_conv_frac is not None:
            cl_, ci_ = g(liq_conv_frac), g(ice_conv_frac)
            if conv_frac is not None:
                cf = g(conv_frac)
                for q in np.ndindex(cl_.shape):
                    if cl_[q] + ci_[q] > EPS:
                        # the reference updates them in sequence (set_cld.F90:548-551)
                        l0, i0 = _split_raw(cl_[q], ci_[q], cf[q], [c[q] for c in cmr], types)
                        cl_[q] = cf[q] * l0 / (l0 + i0)
                        ci_[q] = cf[q] * i0 / (cl_[q] + i0)
            frac = [frac[0] + cl_, frac[1] + ci_]
            c_cloud = cl_ + ci_
    if combine:
        c_ratio = c_ratio / np.maximum(c_cloud, EPS)
        cond_total = sum(cmr)
    for k in range(2):
        f = frac[types[k] - 1]
        cmr[k] = np.where(f > EPS, cmr[k] / np.where(f > EPS, f, 1.0), 0.0)
    w = sum(frac)
    big = w > MIN_CLOUD_FRACTION
    frac = [np.where(big, f / np.where(big, w, 1.0), 0.0) for f in frac]
    if combine:
        c_ratio = np.where(big, c_ratio * w / np.maximum(cond_total, EPS), 0.0)
        c_cloud = np.where(big, c_cloud, 0.0)
    w = np.minimum(np.where(big, w, 0.0), 1.0)
    # effective dimensions
    dims = []
    for k, water in enumerate((True, False)):
        ty = i_st_water if water else i_st_ice
        if water:
            if i_drop_re == abi.IP_RE_EXTERNAL and liq_dim is not None:
                d = np.asarray(liq_dim, dtype=np.float64)[:, cl]
            elif i_drop_re == abi.IP_RE_CONSTANT and liq_dim_constant is not None:
                d = np.full(w.shape, float(liq_dim_constant))
            else:
                d = np.full(w.shape, 7.0e-6)
            lo, hi = sp.drop_parm_min_dim[ty - 1], sp.drop_parm_max_dim[ty - 1]
            scheme = int(sp.i_drop_parm[ty - 1])
        else:
            scheme = int(sp.i_ice_parm[ty - 1])
            d = np.asarray(ice_dim, dtype=np.float64)[:, cl] if ice_dim is not None else ice_dim_from_t(scheme, t[:, cl])
            lo, hi = sp.ice_parm_min_dim[ty - 1], sp.ice_parm_max_dim[ty - 1]
        dims.append(np.minimum(np.maximum(d, lo), hi))
    full = lambda a: np.concatenate([np.zeros((n, ict - 1) + a.shape[2:]), a], axis=1)
    cld = dict(n_condensed=2, type_condensed=[abi.IP_PHASE_WATER, abi.IP_PHASE_ICE], i_cloud_type=types,
               n_cloud_type=nct,
               i_condensed_param=[int(sp.i_drop_parm[i_st_water - 1]), int(sp.i_ice_parm[i_st_ice - 1])],
               i_condensed_type=[i_st_water, i_st_ice],
               condensed_mix_ratio=np.asfortranarray(full(np.stack(cmr, axis=2))),
               condensed_dim_char=np.asfortranarray(full(np.stack(dims, axis=2))),
               w_cloud=np.asfortranarray(full(w)), frac_cloud=np.asfortranarray(full(np.stack(frac, axis=2))),
               # one relative standard deviation per component where uniform
               # (radiance.set_cld_mcica weights it by the condensate)
               rel_var_dens=[float(r.flat[0]) if np.all(r == r.flat[0]) else r for r in rsd],
               c_cloud=np.asfortranarray(full(c_cloud)), c_ratio=np.asfortranarray(full(c_ratio)))
    return cld, ict


def _split_raw(fl, fi, f, cmr, types):
    """split_mix_phase alone on scalars: the liquid and ice fractions after
    the mixed-phase part is shared out."""
    mix = fl + fi - f
    if mix > EPS and fl > EPS and fi > EPS:
        lm = sum(cmr[k] / fl for k in range(len(types)) if types[k] == 1)
        im = sum(cmr[k] / fi for k in range(len(types)) if types[k] == 2)
        if lm + im > EPS:
            return max(fl - mix * im / (lm + im), 0.0), max(fi - mix * lm / (lm + im), 0.0)
    return fl, fi
