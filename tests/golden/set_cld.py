"""A numpy restatement of the cloud set-up runes does before radiance_calc
(socrates_set_control.F90:291-370, socrates_set_cld.F90:170-850,
socrates_set_cld_dim.F90:155-230 and 300-470), for the representations with
stratiform water and ice (ip_cloud_homogen, ip_cloud_ice_water and their
combinations with convective cloud) and those with separate convective cloud
(ip_cloud_conv_strat, ip_cloud_csiw and their split forms).  Test infrastructure: it builds the
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
            ice_rsd=None, cloud_horizontal_rsd=None, i_drop_re=abi.IP_RE_EXTERNAL, liq_dim_constant=None,
            i_cnv_water=0, i_cnv_ice=0, liq_conv_dim=None, ice_conv_dim=None, liq_conv_rsd=None, ice_conv_rsd=None,
            liq_conv_dim_constant=None, cloud_vertical_decorr=None, conv_vertical_decorr=None):
    """col.cld for radiance.Marshal and the id_cloud_top runes uses."""
    n, L = t.shape
    ict = L + 1 - min(n_cloud_layer, L) if n_cloud_layer > 0 else 1
    cl = slice(ict - 1, L)
    split = rep in (abi.IP_CLOUD_SPLIT_HOMOGEN, abi.IP_CLOUD_SPLIT_ICE_WATER)
    conv_sep = split or rep in (abi.IP_CLOUD_CONV_STRAT, abi.IP_CLOUD_CSIW)
    four = rep in (abi.IP_CLOUD_CSIW, abi.IP_CLOUD_SPLIT_ICE_WATER)
    homogen = rep in (abi.IP_CLOUD_HOMOGEN, abi.IP_CLOUD_COMBINE_HOMOGEN)
    combine = split or rep in (abi.IP_CLOUD_COMBINE_HOMOGEN, abi.IP_CLOUD_COMBINE_ICE_WATER)
    if conv_sep and i_inhom == abi.IP_MCICA:                  # set_control.F90:336
        i_inhom = abi.IP_HOMOGENEOUS
    g = lambda a: np.maximum(np.asarray(a, dtype=np.float64)[:, cl], 0.0)
    # components (clcmp, water, convective, type): set_cld.F90:175-212
    comps = [(abi.IP_CLCMP_ST_WATER, True, False, i_st_water), (abi.IP_CLCMP_ST_ICE, False, False, i_st_ice)]
    if conv_sep:
        comps += [(abi.IP_CLCMP_CNV_WATER, True, True, i_cnv_water), (abi.IP_CLCMP_CNV_ICE, False, True, i_cnv_ice)]
    types = []
    for _, water, conv, _ in comps:
        if homogen:
            types.append(1)
        elif four:
            types.append({(True, False): abi.IP_CLOUD_TYPE_SW, (False, False): abi.IP_CLOUD_TYPE_SI,
                          (True, True): abi.IP_CLOUD_TYPE_CW, (False, True): abi.IP_CLOUD_TYPE_CI}[(water, conv)])
        elif conv_sep:
            types.append(abi.IP_CLOUD_TYPE_CONV if conv else abi.IP_CLOUD_TYPE_STRAT)
        else:
            types.append(abi.IP_CLOUD_TYPE_WATER if water else abi.IP_CLOUD_TYPE_ICE)
    nct = 1 if homogen else (4 if four else 2)
    zero = np.zeros_like(g(t))
    cmr, rsd = [], []
    c_ratio = zero.copy()
    for _, water, conv, _ in comps:
        st, cv = (liq_mmr, liq_conv_mmr) if water else (ice_mmr, ice_conv_mmr)
        if not conv:
            m = g(st)
            if combine and cv is not None:
                m = m + g(cv)
                c_ratio = c_ratio + g(cv)
        else:
            m = g(cv) if cv is not None else zero.copy()
            if combine and st is not None:
                m = m + g(st)
        r = (liq_conv_rsd if water else ice_conv_rsd) if conv else (liq_rsd if water else ice_rsd)
        rr = g(r) if r is not None else np.full_like(m, cloud_horizontal_rsd if cloud_horizontal_rsd else 0.0)
        if i_inhom == abi.IP_SCALING:
            m = m / (1.0 + rr ** 2)
        cmr.append(m)
        rsd.append(rr)
    c_cloud = zero.copy()
    if homogen:
        frac = [g(cloud_frac)]
        if combine and conv_frac is not None:
            c_cloud = g(conv_frac)
            frac[0] = frac[0] + c_cloud
    elif not conv_sep:
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
    elif not four:
        # stratiform and convective types (set_cld.F90:567-600)
        frac = [g(cloud_frac), g(conv_frac) if conv_frac is not None else zero.copy()]
    else:
        # stratiform and convective water and ice (set_cld.F90:642-747)
        if cloud_frac is not None:
            fl, fi = _split(g(liq_frac), g(ice_frac), g(cloud_frac), cmr, types, abi.IP_CLOUD_TYPE_SW,
                            abi.IP_CLOUD_TYPE_SI)
        else:
            fl, fi = g(liq_frac), g(ice_frac)
        cl_, ci_ = zero.copy(), zero.copy()
        if liq_conv_frac is not None and ice_conv_frac is not None:
            if conv_frac is not None:
                cl_, ci_ = _split(g(liq_conv_frac), g(ice_conv_frac), g(conv_frac), cmr, types,
                                  abi.IP_CLOUD_TYPE_CW, abi.IP_CLOUD_TYPE_CI)
            else:
                cl_, ci_ = g(liq_conv_frac), g(ice_conv_frac)
        frac = [fl, fi, cl_, ci_]
    if split:
        # thin and thick parts (set_cld.F90:602-640, 749-790; Hogan et al. 2019, A1 and A2)
        pairs = ([(abi.IP_CLOUD_TYPE_SW, abi.IP_CLOUD_TYPE_CW), (abi.IP_CLOUD_TYPE_SI, abi.IP_CLOUD_TYPE_CI)] if four
                 else [(abi.IP_CLOUD_TYPE_STRAT, abi.IP_CLOUD_TYPE_CONV)])
        for thin, thick in pairs:
            tot = frac[thin - 1] + frac[thick - 1]
            if i_inhom != abi.IP_TRIPLECLOUDS_2019:
                frac[thin - 1], frac[thick - 1] = 0.5 * tot, 0.5 * tot
                continue
            if four:
                r = zero.copy()
                for k in range(len(comps)):
                    if types[k] == thin:
                        r = rsd[k]
            else:
                num = sum(rsd[k] * cmr[k] for k in range(len(comps)) if types[k] == thin)
                den = sum(cmr[k] for k in range(len(comps)) if types[k] == thin)
                r = num / np.maximum(den, EPS)
            ft = np.maximum(0.5, np.minimum(0.9, r * (0.4 / 2.25) + 0.525 / 2.25))
            frac[thin - 1], frac[thick - 1] = tot * ft, tot * (1.0 - ft)
            ratio = 0.025 + 0.975 * np.exp(-r - r ** 2 / 2.0 - r ** 3 / 4.0)
            for k in range(len(comps)):
                if types[k] == thin:
                    cmr[k] = cmr[k] * ratio * ft
                elif types[k] == thick:
                    cmr[k] = cmr[k] * (1.0 - ratio * ft)
        if i_inhom != abi.IP_TRIPLECLOUDS_2019:
            cmr = [0.5 * m for m in cmr]
    if combine:
        c_ratio = c_ratio / np.maximum(c_cloud, EPS)
        cond_total = sum(cmr)
    for k in range(len(comps)):
        f = frac[types[k] - 1]
        cmr[k] = np.where(f > EPS, cmr[k] / np.where(f > EPS, f, 1.0), 0.0)
    w = sum(frac)
    big = w > MIN_CLOUD_FRACTION
    frac = [np.where(big, f / np.where(big, w, 1.0), 0.0) for f in frac]
    if combine:
        c_ratio = np.where(big, c_ratio * w / np.maximum(cond_total, EPS), 0.0)
        c_cloud = np.where(big, c_cloud, 0.0)
    w = np.minimum(np.where(big, w, 0.0), 1.0)
    # effective dimensions (set_cld_dim.F90:155-230); the split forms size and
    # bound their convective part as the stratiform one
    dims, params = [], []
    for _, water, conv, ty in comps:
        own = conv and not split
        bty = ty if own else (i_st_water if water else i_st_ice)
        if water:
            src, cst = (liq_conv_dim, liq_conv_dim_constant) if own else (liq_dim, liq_dim_constant)
            if i_drop_re == abi.IP_RE_EXTERNAL and src is not None:
                d = np.asarray(src, dtype=np.float64)[:, cl]
            elif i_drop_re == abi.IP_RE_CONSTANT and cst is not None:
                d = np.full(w.shape, float(cst))
            else:
                d = np.full(w.shape, 7.0e-6)
            lo, hi = sp.drop_parm_min_dim[bty - 1], sp.drop_parm_max_dim[bty - 1]
            params.append(int(sp.i_drop_parm[ty - 1]))
        else:
            scheme = int(sp.i_ice_parm[ty - 1])
            src = ice_conv_dim if own else ice_dim
            d = np.asarray(src, dtype=np.float64)[:, cl] if src is not None else ice_dim_from_t(scheme, t[:, cl])
            lo, hi = sp.ice_parm_min_dim[bty - 1], sp.ice_parm_max_dim[bty - 1]
            params.append(scheme)
        dims.append(np.minimum(np.maximum(d, lo), hi))
    full = lambda a: np.concatenate([np.zeros((n, ict - 1) + a.shape[2:]), a], axis=1)
    cld = dict(n_condensed=len(comps), type_condensed=[c[0] for c in comps], i_cloud_type=types,
               n_cloud_type=nct, i_condensed_param=params, i_condensed_type=[c[3] for c in comps],
               condensed_mix_ratio=np.asfortranarray(full(np.stack(cmr, axis=2))),
               condensed_dim_char=np.asfortranarray(full(np.stack(dims, axis=2))),
               w_cloud=np.asfortranarray(full(w)), frac_cloud=np.asfortranarray(full(np.stack(frac, axis=2))),
               # one relative standard deviation per component where uniform
               # (radiance.set_cld_mcica weights it by the condensate)
               rel_var_dens=[float(r.flat[0]) if np.all(r == r.flat[0]) else r for r in rsd],
               c_cloud=np.asfortranarray(full(c_cloud)), c_ratio=np.asfortranarray(full(c_ratio)),
               # decorrelation scales of like regions (set_cld.F90:454-465)
               dp_corr_strat=float(cloud_vertical_decorr or 0.0), dp_corr_conv=float(conv_vertical_decorr or 0.0))
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
