"""runes, the model-facing interface (socrates_runes.F90:47), through
socgpu_runes: the reference's runes test (src/aux/runes_driver.f90 with the
GA9 spectral files) reproduced on the GPU, the vertical inversion, the
surface options against the oracle, and the host-side argument checks."""
import numpy as np
import pytest

import runes_case as RC
from socrates_gb300 import abi, build
from socrates_gb300 import runes as RN
from socrates_gb300.radiance import RadianceError


@pytest.fixture(scope="module")
def ga9(gpu_lib):
    """Registers the two GA9 spectra under the names the driver uses."""
    sw, lw = RC.spectra()
    RN.set_spectrum("sw", spectrum=sw)
    RN.set_spectrum("lw", spectrum=lw)
    return RC.data(), sw, lw


@pytest.fixture(scope="module")
def O():
    import oracle
    return oracle


def _printed(diag, d):
    """The driver's printed columns: levels 1..32 and the K/day heating
    rate of layers 1..32 (runes_driver.f90)."""
    return np.stack([diag["flux_down"][0, 1:], diag["flux_up"][0, 1:], diag["heating_rate"][0] * RC.SECONDS_PER_DAY],
                    axis=1)


@pytest.mark.gpu
@pytest.mark.parametrize("section", RC.SECTIONS)
def test_runes_ga9_known_good_output_on_gpu(ga9, O, section):
    """FP64 through socgpu_runes: the driver's printed fluxes and heating
    rates (8 decimals) to 2e-8, and every level flux within 1e-10 of the
    largest flux of the oracle's radiance_calc on the set-up runes makes;
    mixed precision within 0.1 W/m2 and 0.05 K/day of the printed values."""
    d, sw, lw = ga9
    kw = RC.runes_kwargs(d, section)
    diag = RN.runes(**kw)
    kgo = d["kgo_" + section]
    err = np.abs(_printed(diag, d) - kgo)
    assert err.max() <= 2e-8, f"{section}: level {err.max(axis=1).argmax() + 1}, error {err.max():.2e}"
    ctl, sp, col = RC.direct_case(d, sw, lw, section)
    ref = O.radiance_calc(ctl, sp, col)
    scale = max(np.abs(ref["flux_down"]).max(), np.abs(ref["flux_up"]).max())
    for k in ("flux_down", "flux_up") + (("flux_direct",) if section == "sw" else ()):
        e = np.abs(diag[k] - ref[k]).max() / scale
        assert e <= 1e-10, f"{section} {k}: scaled error {e:.2e}"
    assert diag["flux_up_toa"][0] == diag["flux_up"][0, 0]
    assert diag["flux_down_surf"][0] == diag["flux_down"][0, -1]
    mixed = RN.runes(**kw, precision=abi.PRECISION_MIXED)
    m = _printed(mixed, d)
    assert np.abs(m[:, :2] - kgo[:, :2]).max() <= 0.1
    assert np.abs(m[:, 2] - kgo[:, 2]).max() <= 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("section", ["sw", "lw_tiles"])
def test_runes_invert(ga9, section):
    """l_invert: profiles given surface first give the same diagnostics,
    surface first, bit for bit (socrates_set_atm.F90 layer_offset)."""
    d, _, _ = ga9
    kw = RC.runes_kwargs(d, section)
    diag = RN.runes(**kw)
    flip = dict(kw, l_invert=True)
    for k, v in kw.items():
        if isinstance(v, np.ndarray) and v.ndim == 2 and v.shape[1] in (32, 33) and k not in ("frac_tile", "t_tile"):
            flip[k] = np.asfortranarray(v[:, ::-1])
    inv = RN.runes(**flip)
    for k in ("flux_down", "flux_up", "flux_direct", "heating_rate"):
        assert np.array_equal(inv[k][:, ::-1], diag[k]), k
    for k in ("flux_up_toa", "flux_down_surf", "flux_direct_surf"):
        assert np.array_equal(inv[k], diag[k]), k


@pytest.mark.gpu
def test_runes_surface_and_gas_options(ga9, O):
    """Profile and well-mixed gases (l_<gas>_well_mixed prefers the mixing
    ratio), per-band diffuse and direct albedos, a sun below the horizon,
    several profiles: FP64 against the oracle at 1e-10."""
    d, sw, _ = ga9
    kw = RC.runes_kwargs(d, "sw")
    n = 3
    for k in ("p_layer", "t_layer", "mass", "density", "layer_heat_capacity", "h2o", "o3"):
        kw[k] = np.asfortranarray(np.repeat(kw[k], n, axis=0))
    kw["o3"][1] *= 1.5
    kw["h2o"][2] *= 0.5
    kw["co2"] = np.asfortranarray(np.full((n, 32), 9.9))          # ignored: well mixed preferred
    kw["l_co2_well_mixed"] = True
    kw["cos_zenith_angle"] = np.array([0.3, -0.2, 0.9])
    kw["solar_irrad"] = np.full(n, float(d["solar_irrad"]))
    kw.update(l_grey_albedo=False, albedo_diff=np.asfortranarray(np.linspace(0.05, 0.3, n * sw.n_band).reshape(n, -1)),
              albedo_dir=np.asfortranarray(np.linspace(0.1, 0.2, n * sw.n_band).reshape(n, -1)))
    diag = RN.runes(n_profile=n, **{k: v for k, v in kw.items() if k != "n_profile"})
    ctl, sp, col = RC.direct_case(d, sw, None, "sw")
    from socrates_gb300.synth import Column
    gas = np.repeat(col.gas_mix_ratio, n, axis=0)
    ih2o, io3 = (int(np.where(sp.type_absorb == t)[0][0]) for t in (1, 3))
    gas[:, :, io3] = np.maximum(kw["o3"], 0.0)
    gas[:, :, ih2o] = np.maximum(kw["h2o"], 0.0)
    rep = lambda a: np.asfortranarray(np.repeat(a, n, axis=0))
    c = Column(n, 32, rep(col.p), rep(col.t), rep(col.p_level), rep(col.t_level), rep(col.mass),
               np.asfortranarray(gas), z=np.zeros((n, 32)), t_ground=np.repeat(col.t_ground, n), density=rep(col.density))
    c.rho_alb = np.asfortranarray(np.stack([kw["albedo_diff"], kw["albedo_dir"]], axis=1))
    cz = kw["cos_zenith_angle"]
    c.zen_0 = np.where(cz > 0, 1.0 / np.where(cz > 0, cz, 1.0), 1.0)
    c.solar_irrad = np.where(cz > 0, kw["solar_irrad"], 0.0)
    ref = O.radiance_calc(ctl, sp, c)
    assert np.all(diag["flux_down"][1] == 0.0)
    scale = np.abs(ref["flux_down"]).max()
    for k in ("flux_down", "flux_up", "flux_direct"):
        e = np.abs(diag[k] - ref[k]).max() / scale
        assert e <= 1e-10, f"{k}: scaled error {e:.2e}"


def _repeated(col, n):
    """The driver's single column repeated n times."""
    from socrates_gb300.synth import Column
    rep = lambda a: np.asfortranarray(np.repeat(a, n, axis=0))
    c = Column(n, col.n_layer, rep(col.p), rep(col.t), rep(col.p_level), rep(col.t_level), rep(col.mass),
               rep(col.gas_mix_ratio), z=np.zeros((n, col.n_layer)), t_ground=np.repeat(col.t_ground, n),
               density=rep(col.density))
    c.rho_alb = rep(col.rho_alb)
    for k in ("zen_0", "solar_irrad"):
        if getattr(col, k, None) is not None:
            setattr(c, k, np.repeat(getattr(col, k), n))
    return c


def _cloud_fields(n, L, seed):
    """Stratiform and convective cloud in the lower two thirds: fractions whose
    liquid and ice parts overlap (a mixed-phase share to split), grid-box
    mixing ratios, sizes and relative standard deviations, by the names of
    set_cld and set_cld_dim."""
    rng = np.random.default_rng(seed)
    cloudy = rng.uniform(size=(n, L)) < 0.6
    cloudy[:, : L // 3] = False
    u = lambda lo, hi: np.asfortranarray(np.where(cloudy, rng.uniform(lo, hi, size=(n, L)), 0.0))
    cf, cv = u(0.1, 0.6), u(0.0, 0.35)
    return dict(cloud_frac=cf, conv_frac=cv, liq_frac=cf * u(0.4, 1.0), ice_frac=cf * u(0.4, 1.0),
                liq_conv_frac=cv * u(0.4, 1.0), ice_conv_frac=cv * u(0.4, 1.0),
                liq_mmr=u(1e-5, 3e-4), ice_mmr=u(0.0, 1e-4), liq_conv_mmr=u(2e-5, 6e-4), ice_conv_mmr=u(0.0, 2e-4),
                liq_dim=u(5e-6, 1.5e-5), ice_dim=u(2e-5, 8e-5), liq_conv_dim=u(6e-6, 2e-5),
                ice_conv_dim=u(3e-5, 1e-4), liq_rsd=u(0.3, 1.5), ice_rsd=u(0.3, 1.5), liq_conv_rsd=u(0.3, 1.5),
                ice_conv_rsd=u(0.3, 1.5))


CLOUD_CASES = [
    (abi.IP_CLOUD_HOMOGEN, {}),
    (abi.IP_CLOUD_ICE_WATER, dict(i_inhom=abi.IP_SCALING)),
    (abi.IP_CLOUD_COMBINE_HOMOGEN, dict(i_overlap=abi.IP_RAND)),
    (abi.IP_CLOUD_COMBINE_ICE_WATER, dict(i_cloud_entrapment=abi.IP_MAX_ENTRAPMENT)),
    (abi.IP_CLOUD_CONV_STRAT, dict(ice_dim=None)),              # stratiform ice sizes from temperature
    (abi.IP_CLOUD_CSIW, dict(i_inhom=abi.IP_SCALING, n_cloud_layer=20)),
    (abi.IP_CLOUD_SPLIT_HOMOGEN, dict(i_inhom=abi.IP_TRIPLECLOUDS_2019)),
    (abi.IP_CLOUD_SPLIT_ICE_WATER, dict(liq_conv_mmr=None, ice_conv_mmr=None, liq_conv_frac=None,
                                        ice_conv_frac=None)),
    (abi.IP_CLOUD_SPLIT_ICE_WATER, dict(i_inhom=abi.IP_TRIPLECLOUDS_2019)),
    (abi.IP_CLOUD_ICE_WATER, dict(i_overlap=abi.IP_EXPONENTIAL_RAND, cloud_vertical_decorr=5000.0)),
    (abi.IP_CLOUD_CSIW, dict(i_overlap=abi.IP_EXPONENTIAL_RAND, cloud_vertical_decorr=4000.0,
                             conv_vertical_decorr=1500.0)),
]
THREE = (abi.IP_CLOUD_CONV_STRAT, abi.IP_CLOUD_CSIW, abi.IP_CLOUD_SPLIT_HOMOGEN, abi.IP_CLOUD_SPLIT_ICE_WATER)


@pytest.mark.gpu
@pytest.mark.parametrize("section", ["sw", "lw_tground"])
@pytest.mark.parametrize("case", range(len(CLOUD_CASES)))
def test_runes_clouds(ga9, O, section, case):
    """Every cloud representation through socgpu_runes (set_control's scheme
    and solver, set_cld's components, types, fractions, mixed-phase split
    and thin/thick split, set_cld_dim's sizes) on 4 columns against the
    oracle's radiance_calc on the fields a numpy restatement of set_cld
    makes: FP64 within 1e-10 of the largest flux.  The three-region
    representations use convective ice of another type (Pade, type 12)."""
    import set_cld as SC
    from dataclasses import replace
    d, sw, lw = ga9
    rep, opts = CLOUD_CASES[case]
    n = 4
    kw = RC.runes_kwargs(d, section)
    for k in ("p_layer", "t_layer", "mass", "density", "layer_heat_capacity", "h2o", "o3", "t_level"):
        if k in kw:
            kw[k] = np.asfortranarray(np.repeat(kw[k], n, axis=0))
    for k in ("cos_zenith_angle", "solar_irrad", "t_ground"):
        if k in kw:
            kw[k] = np.repeat(kw[k], n)
    fields = {**_cloud_fields(n, 32, seed=70 + case), **opts}
    types = dict(i_st_water=5, i_st_ice=8, i_cnv_water=5, i_cnv_ice=12)
    diag = RN.runes(n_profile=n, **{k: v for k, v in kw.items() if k != "n_profile"}, i_cloud_representation=rep,
                    **types, **{k: v for k, v in fields.items() if v is not None})
    ctl, sp, col = RC.direct_case(d, sw, lw, section)
    col = _repeated(col, n)
    arrays = {k: v for k, v in fields.items() if k not in ("i_inhom", "i_overlap", "i_cloud_entrapment")}
    cld, ict = SC.set_cld(sp, kw["t_layer"], rep, i_inhom=opts.get("i_inhom", abi.IP_HOMOGENEOUS), **types, **arrays)
    col.cld = cld
    expo = opts.get("i_overlap") == abi.IP_EXPONENTIAL_RAND
    if rep in THREE:
        ctl = replace(ctl, i_cloud=abi.IP_CLOUD_PART_CORR_CNV if expo else abi.IP_CLOUD_TRIPLE,
                      i_solver=abi.IP_SOLVER_TRIPLE_HOGAN, i_cloud_representation=rep)
    else:
        homogen = rep in (abi.IP_CLOUD_HOMOGEN, abi.IP_CLOUD_COMBINE_HOMOGEN)
        ctl = replace(ctl, i_cloud=abi.IP_CLOUD_MIX_RANDOM if opts.get("i_overlap") == abi.IP_RAND
                      else abi.IP_CLOUD_PART_CORR if expo else abi.IP_CLOUD_MIX_MAX,
                      i_solver=abi.IP_SOLVER_MIX_DIRECT if opts.get("i_cloud_entrapment") == abi.IP_MAX_ENTRAPMENT
                      else abi.IP_SOLVER_MIX_DIRECT_HOGAN,
                      i_cloud_representation=abi.IP_CLOUD_HOMOGEN if homogen else abi.IP_CLOUD_ICE_WATER)
    ref = O.radiance_calc(ctl, sp, col, id_cloud_top=ict)
    clear = O.radiance_calc(replace(ctl, i_cloud=abi.IP_CLOUD_CLEAR, i_solver=abi.IP_SOLVER_HOMOGEN_DIRECT), sp, col)
    assert np.abs(ref["flux_up"] - clear["flux_up"]).max() > 1.0          # the clouds matter
    scale = max(np.abs(ref["flux_down"]).max(), np.abs(ref["flux_up"]).max())
    for k in ("flux_down", "flux_up") + (("flux_direct",) if section == "sw" else ()):
        e = np.abs(diag[k] - ref[k]).max() / scale
        assert e <= 1e-10, f"{k}: scaled error {e:.2e}"


@pytest.mark.gpu
def test_runes_three_region_refusals(ga9):
    """Separate convective cloud: random overlap leaves two regions whose
    solver does not take solver_triple_hogan (mix_column.F90:526-530);
    maximal entrapment is not built; the convective mixing ratios are
    required unless the cloud is split."""
    d, _, _ = ga9
    kw = RC.runes_kwargs(d, "lw_tground")
    fields = _cloud_fields(1, 32, seed=5)
    base = dict(kw, i_cloud_representation=abi.IP_CLOUD_CSIW, i_st_water=5, i_st_ice=8, i_cnv_water=5, i_cnv_ice=8,
                **fields)
    for extra, status, words in ((dict(i_overlap=abi.IP_RAND), abi.I_ERR_FATAL, "solver specified is not valid"),
                                 (dict(i_cloud_entrapment=abi.IP_MAX_ENTRAPMENT), abi.I_ERR_RANGE, "solver_triple"),
                                 (dict(liq_conv_mmr=None), abi.I_ERR_FATAL, "Convective liquid MMR not provided"),
                                 (dict(i_cnv_ice=0), abi.I_ERR_FATAL, "Prescribed ice cloud")):
        args = {k: v for k, v in {**base, **extra}.items() if v is not None}
        with pytest.raises(RadianceError) as e:
            RN.runes(**args)
        assert e.value.status == status and words in str(e.value), (extra, str(e.value))


# ---------------------------------------------------------------------------
# host side (no GPU)

@pytest.fixture(scope="module")
def lib():
    build.build()
    return RN.load_library()


def test_gas_identifiers_follow_gas_list():
    """runes' gas arguments map to gas_list_pcf.F90's identifiers."""
    assert [RN.GAS_ID[g] for g in ("h2o", "co2", "o3", "n2o", "co", "ch4", "o2")] == [1, 2, 3, 4, 5, 6, 7]
    assert RN.GAS_ID["ar"] == 37 and RN.GAS_ID["o"] == 39 and RN.GAS_ID["ch3ono2"] == 67
    assert max(RN.GAS_ID.values()) < abi.RUNES_N_GAS


def _minimal(**kw):
    z = np.zeros((1, 4))
    return dict(n_profile=1, n_layer=4, spectrum_name="lw", i_source=abi.IP_SOURCE_THERMAL, p_layer=z, t_layer=z,
                mass=z, t_level=np.zeros((1, 5)), **kw)


def test_runes_unknown_gas_keyword(lib):
    with pytest.raises(TypeError, match="xenon"):
        RN.runes(**_minimal(xenon=np.zeros((1, 4))))
    with pytest.raises(TypeError, match="l_xenon_well_mixed"):
        RN.runes(**_minimal(l_xenon_well_mixed=True))


def test_runes_unset_spectrum(lib):
    """A spectrum that has not been set is an error found before any device
    work (socrates_runes.F90: the spectrum is looked up by name)."""
    with pytest.raises(RadianceError) as e:
        RN.runes(**dict(_minimal(), spectrum_name="no-such-spectrum"))
    assert e.value.status == abi.I_ERR_EXIST and "no-such-spectrum" in str(e.value)
