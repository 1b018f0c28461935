"""socgpu_run, the drop-in for the reference's Cl_run_cdl / Cl_run_cdf
column drivers: netCDF classic and CDL files in, the same files out.

CPU tests check the file formats (CDL -> CDF -> CDL through the driver's
converter, cross-checked with scipy's netCDF reader); GPU tests run the
reference's ICRCCM case 27 (examples/aer_cmp/run27) end to end from CDL and
from netCDF files and compare the written heating rates with the reference's
known-good output."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import icrccm27 as K
from cdl import field, read_cdl, write_cdl
from socrates_gb300 import build

ROOT = Path(__file__).resolve().parent.parent
SUFFIX = {1: "q", 2: "co2", 3: "o3", 4: "n2o", 6: "ch4", 7: "o2", 9: "so2", 14: "cfc11", 15: "cfc12",
          16: "cfc113", 17: "hcfc22", 18: "hfc125", 19: "hfc134a", 25: "ocs"}


def _tool():
    build.build()
    return str(build.TOOL)


def _column_files(tmp, name, d, sp, sp_name, to_cdf=False, gases=None, wenyi=False, digits=7, extra=None):
    """A case's inputs written as column files like the reference's, with the
    spectral file (and its '_k' tables) written beside them.  gases: the
    absorber types that have input files (default all); digits: significant
    digits of the CDL values; extra: {suffix: (coordinate, values)} of more
    fields (clouds, the solar zenith angle and irradiance)."""
    sp_path = tmp / sp_name
    sp.write_text(sp_path)
    if sp.k_lookup is not None or sp.k_t_lookup_gas is not None:
        sp.write_k_file(str(sp_path) + "_k")
    wy = None
    if wenyi:
        wy = tmp / "wenyi_tables.dat"
        sp.write_wenyi_data(wy)
    base = tmp / name
    coord = {"units": "degree", "title": "latitude"}

    def put(suffix, plev, values, vname, units="None"):
        dims = [("lat", 1), ("lon", 1), ("plev", len(plev))]
        variables = [("lat", ["lat"], [0.0], coord), ("lon", ["lon"], [0.0], {"units": "degree", "title": "longitude"}),
                     ("plev", ["plev"], plev, {"units": "Pa", "title": "PRESSURE"}),
                     (vname, ["plev", "lon", "lat"], np.reshape(values, (len(plev), 1, 1)), {"units": units})]
        path = tmp / f"{name}.{suffix}"
        write_cdl(path, f"{name}.{suffix}", dims, variables, digits)
        return path

    files = [put("t", d["p"], d["t"], "t", "K"), put("tl", d["p_level"], d["t_level"], "tl", "K")]
    for j, ty in enumerate(sp.type_absorb):
        if gases is None or int(ty) in gases:
            files.append(put(SUFFIX[int(ty)], d["p"], d["gas"][:, j], SUFFIX[int(ty)]))
    files.append(put("tstar", [1.013e5], d["t_ground"], "tstar", "K"))
    for suffix, (plev, values) in (extra or {}).items():
        files.append(put(suffix, plev, values, suffix))
    surf = tmp / f"{name}.surf"
    write_cdl(surf, f"{name}.surf", [("lat", 1), ("lon", 1), ("basis", 1)],
              [("lat", ["lat"], [1.0], {}), ("lon", ["lon"], [0.0], {}), ("basis", ["basis"], [1.0], {}),
               ("alb", ["basis", "lat", "lon"], np.reshape(d["alb"], (1, 1, 1)), {"title": "ALBEDO WEIGHTS"})])
    files.append(surf)
    if to_cdf:
        tool = _tool()
        for f in files:
            tmp_out = f.with_name(f.name + ".cdf")
            subprocess.run([tool, "--convert", str(f), str(tmp_out)], check=True)
            tmp_out.replace(f)
    return sp_path, base, wy


def _case27_files(tmp, to_cdf=False):
    from socrates_gb300.spectrum import Spectrum
    sp = Spectrum.load_npz(K.FIXTURE, prefix="sp_")
    sp_path, base, _ = _column_files(tmp, "laer27", np.load(K.FIXTURE), sp, "sp_lw_hadcm3", to_cdf)
    return sp_path, base


def test_cdl_cdf_round_trip(tmp_path):
    scipy_io = pytest.importorskip("scipy.io")
    tool = _tool()
    src = tmp_path / "x.t"
    plev = np.array([10.0, 200.0, 3000.5, 90000.0])
    write_cdl(src, "x.t", [("lat", 2), ("lon", 3), ("plev", 4)],
              [("lat", ["lat"], [0.0, 1.0], {"units": "degree"}), ("lon", ["lon"], [0.0, 1.0, 2.0], {}),
               ("plev", ["plev"], plev, {"units": "Pa"}),
               ("t", ["plev", "lon", "lat"], np.arange(24.0).reshape(4, 3, 2) + 200.25, {"units": "K"})])
    cdf = tmp_path / "x.cdf"
    subprocess.run([tool, "--convert", str(src), str(cdf)], check=True)
    with scipy_io.netcdf_file(str(cdf), "r", mmap=False) as nc:
        np.testing.assert_allclose(nc.variables["plev"][:], plev, rtol=1e-6)
        np.testing.assert_allclose(nc.variables["t"][:], np.arange(24.0).reshape(4, 3, 2) + 200.25, rtol=1e-6)
        assert nc.variables["t"].units in (b"K", "K")
    back = tmp_path / "y.cdl"
    subprocess.run([tool, "--convert", str(cdf), str(back)], check=True)
    dims, v = read_cdl(back)
    assert dims == {"lat": 2, "lon": 3, "plev": 4}
    np.testing.assert_allclose(v["t"], (np.arange(24.0) + 200.25), rtol=1e-6)


def test_driver_rejects_bad_options(tmp_path):
    tool = _tool()
    r = subprocess.run([tool, "-B", str(tmp_path / "none")], capture_output=True, text=True)
    assert r.returncode != 0 and "Spectral file not set" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("to_cdf", [False, True])
def test_driver_reproduces_icrccm27(gpu_lib, tmp_path, to_cdf):
    tool = _tool()
    sp, base = _case27_files(tmp_path, to_cdf)
    cmd = [tool, "-s", str(sp), "-R", "1", "8", "-I", "-g", "2", "-c", "-t", "12", "-v", "13", "-C", "5",
           "-B", str(base)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = str(base) + ".hrts"
    if to_cdf:
        scipy_io = pytest.importorskip("scipy.io")
        with scipy_io.netcdf_file(out, "r", mmap=False) as nc:
            hr = np.array(nc.variables["hrts"][:]).ravel()
    else:
        _, hr = field(out)
    kgo = K.load()[3]
    if to_cdf:
        # netCDF "float" variables hold single precision: inputs and outputs
        # rounded to float32 move the heating rates by up to about 1e-6 relative
        assert np.abs(hr - kgo).max() <= 2e-5 * np.abs(kgo).max()
    else:
        # CDL text carries 7 significant digits: the reference's 6 must match
        half_unit = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(kgo))) - 5)
        assert (np.abs(hr - kgo) / half_unit).max() <= 1.05
    r = subprocess.run(cmd + ["-P", "mixed"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, hr_mixed = field(out) if not to_cdf else (None, hr)
    assert np.abs(hr_mixed - kgo).max() <= 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("to_cdf", [False, True])
def test_driver_reproduces_circ6_ga7(gpu_lib, tmp_path, to_cdf):
    """CIRC case 6 with the GA7 long-wave file through the column driver
    (examples/netcdf/CIRC_case6/run_me: -R 1 9 -I -g 4 -c -C 5): the spectral
    file with its '_k' lookup tables and the Wen-Yi tables (-W) read by the
    C++ loader, absorbers without input files taken as absent."""
    import circ6 as K6
    from socrates_gb300.spectrum import Spectrum
    tool = _tool()
    d = np.load(K6.FIXTURE)
    sp = Spectrum.load_npz(K6.FIXTURE, prefix="sp_")
    # the case's inputs are single-precision netCDF values: CDL with 17 digits
    # carries them exactly
    sp_path, base, wy = _column_files(tmp_path, "case6", d, sp, "sp_lw_ga7", to_cdf,
                                      gases=set(int(x) for x in d["gases_present"]), wenyi=True, digits=17)
    cmd = [tool, "-s", str(sp_path), "-R", "1", "9", "-I", "-g", "4", "-c", "-C", "5", "-B", str(base),
           "-W", str(wy)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = str(base) + ".hrts"
    if to_cdf:
        scipy_io = pytest.importorskip("scipy.io")
        with scipy_io.netcdf_file(out, "r", mmap=False) as nc:
            hr = np.array(nc.variables["hrts"][:]).ravel()
    else:
        _, hr = field(out)
    kgo = d["kgo_hrts"]
    if to_cdf:
        assert np.abs(hr - kgo).max() <= 2e-5 * np.abs(kgo).max()
    else:
        half_unit = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(kgo))) - 5)
        assert (np.abs(hr - kgo) / half_unit).max() <= 1.05
    # without the Wen-Yi tables the band-4 CO2 terms cannot be scaled
    r = subprocess.run(cmd[:-2], capture_output=True, text=True)
    assert r.returncode != 0 and "Wen-Yi" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["self_broadened", "temperature_tables"])
def test_loader_reads_self_broadened_and_temperature_tables(gpu_lib, tmp_path, kind):
    """Self-broadened and temperature-only tables written in the '_k'
    layouts, read back by the C++ loader (socgpu_spectrum_load_ext) and
    solved on the GPU, match the oracle on the arrays they were written from."""
    import ctypes as C
    import oracle as O
    import test_lookup_gpu as T
    from socrates_gb300 import abi, synth
    from socrates_gb300 import radiance as R
    sp = (T._self_broadened if kind == "self_broadened" else T._temperature_tables)(T._ga7_lw())
    sp_path = tmp_path / "sp"
    sp.write_text(sp_path)
    sp.write_k_file(str(sp_path) + "_k")
    wy = tmp_path / "wy.dat"
    sp.write_wenyi_data(wy)
    lib = R.load_library()
    h = C.c_int(0)
    msg = C.create_string_buffer(512)
    name = f"loaded_{kind}".encode()
    st = lib.socgpu_spectrum_load_ext(name, str(sp_path).encode(), None, str(wy).encode(), C.byref(h), msg, 512)
    assert st == 0, msg.value.decode()
    col = synth.operational_case(sp, 33, 40, seed=51, solar=False)
    ctl = R.lw_control(l_continuum=True, i_gas_overlap=abi.IP_OVERLAP_K_EQV_SCL)
    m = R.Marshal(ctl, sp, col)
    st = lib.socgpu_radiance_calc(*m.args(h.value), msg, 512)
    assert st == 0, msg.value.decode()
    got = m.result()
    ref = O.radiance_calc(ctl, sp, col)
    fscale = np.abs(ref["flux_up"]).max()
    for k in ("flux_up", "flux_down"):
        assert np.abs(got[k] - ref[k]).max() <= 1e-10 * fscale, k


def _mcica5118_files(tmp, run, to_cdf):
    """The inputs of one run of examples/netcdf/mcica as column files, with
    its spectral file, the McICA data file beside it and the Wen-Yi tables;
    returns (spectral file, base name, Wen-Yi source, options)."""
    import mcica5118 as M
    from socrates_gb300.radiance import write_mcica_data
    d = np.load(M.FIXTURE)
    sps = M.spectra()
    solar, ga7 = run.startswith("sw"), run.endswith("ga7")
    sp = sps[("sw_" if solar else "lw_") + ("ga7" if ga7 else "ga3")]
    gases = {1: "q", 2: "co2", 3: "o3", 4: "n2o", 6: "ch4", 7: "o2"}
    gas = np.zeros((d["p"].size, sp.n_absorb))
    for j, ty in enumerate(sp.type_absorb):
        if int(ty) in gases:
            gas[:, j] = d[gases[int(ty)]]
    case = dict(p=d["p"], t=d["t"], p_level=d["p_level"], t_level=d["t_level"], gas=gas, t_ground=d["tstar"],
                alb=d["surfsw" if solar else "surflw"])
    extra = {k: (d["p"], d[k]) for k in ("clfr", "lwm", "iwm", "re", "ire")}
    if solar:
        extra.update(szen=([1.013e5], d["szen"]), stoa=([1.013e5], d["stoa"]))
    name = "sp_" + ("sw" if solar else "lw") + ("_ga7" if ga7 else "_ga3_0")
    sp_path, base, wy = _column_files(tmp, "5118_142", case, sp, name, to_cdf, gases=set(gases),
                                      wenyi=not solar, digits=17, extra=extra)
    write_mcica_data(tmp / "mcica_data", M.mcica_data(d, "ga7_" if ga7 else "ga3_"))
    opts = {"lw_avg": "-R 1 9 -I -t 12 +R -v 13 -g 5 -c -C 10 -K 1 -d 1 -i 1",
            "sw_avg": "-R 1 6 -S -t 2 +R -v 13 -g 5 -r -C 10 -K 1 -d 3 -i 3",
            "lw_ga7": "-R 1 9 -I +R -g 4 -c -C 10 -K 1 -d 5 -i 8",
            "sw_ga7": "-R 1 6 -S +R -g 4 -r -C 10 -K 1 -d 5 -i 8"}[run].split()
    opts += ["-m", "0.75", "+m", "2", "-dp", "10000"]
    return sp_path, base, wy, opts, np.asarray(d["kgo_" + run])


@pytest.mark.gpu
@pytest.mark.parametrize("run,to_cdf", [("lw_avg", False), ("sw_avg", True), ("lw_ga7", True), ("sw_ga7", False)])
def test_driver_reproduces_mcica5118(gpu_lib, tmp_path, run, to_cdf):
    """The reference's McICA example (examples/netcdf/mcica/run_me) through
    the column driver: cloud fields, droplet and ice types of the spectral
    file, the McICA data file beside it, cloud_gen's subcolumns and optimal
    sampling, from CDL or netCDF files; the written heating rates against
    the known-good output to half a unit of the 6th digit (CDL, which
    carries the single-precision inputs exactly) or 2e-5 of the largest
    (netCDF output, single precision)."""
    tool = _tool()
    sp_path, base, wy, opts, kgo = _mcica5118_files(tmp_path, run, to_cdf)
    cmd = [tool, "-s", str(sp_path)] + opts + ["-B", str(base)] + (["-W", str(wy)] if wy else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = str(base) + ".hrts"
    if to_cdf:
        scipy_io = pytest.importorskip("scipy.io")
        with scipy_io.netcdf_file(out, "r", mmap=False) as nc:
            hr = np.array(nc.variables["hrts"][:]).ravel()
        assert np.abs(hr - kgo).max() <= 2e-5 * np.abs(kgo).max()
    else:
        _, hr = field(out)
        half_unit = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(kgo))) - 5)
        assert (np.abs(hr - kgo) / half_unit).max() <= 1.05


def test_driver_refuses_clouds_without_processes(tmp_path):
    """-C 10 without a droplet or ice type: the reference's message, no run."""
    r = subprocess.run([_tool(), "-s", "x", "-R", "1", "1", "-I", "-C", "10", "-K", "1", "-B", "y"],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "no cloudy processes" in r.stderr


def _cld7460_files(tmp, run, to_cdf):
    """The inputs of one averaged-column run of examples/netcdf/7460_28 as
    column files, with its spectral file beside them and, for .surfsw2, a
    surface of two albedo weights (diffuse, direct)."""
    import cld7460 as K
    d = np.load(K.FIXTURE)
    sps = K.spectra()
    solar, ga9 = "sw" in run, "ga9" in run
    sp = sps[("ga9" if ga9 else "h") + ("sw" if solar else "lw")]
    gases = {1: "q", 2: "co2", 3: "o3", 4: "n2o", 6: "ch4", 7: "o2"}
    gas = np.zeros((d["avg_p"].size, sp.n_absorb))
    for j, ty in enumerate(sp.type_absorb):
        if int(ty) in gases:
            gas[:, j] = d["avg_" + gases[int(ty)]][:, 0]
    case = dict(p=d["avg_p"], t=d["avg_t"][:, 0], p_level=d["avg_p_level"], t_level=d["avg_t_level"][:, 0], gas=gas,
                t_ground=d["avg_tstar"], alb=d["avg_surfsw" if solar else "avg_surflw"])
    extra = {k: (d["avg_p"], d["avg_" + k][:, 0]) for k in ("clfr", "lwm", "iwm", "re", "ire")}
    if solar:
        extra.update(szen=([1.013e5], d["avg_szen"]), stoa=([1.013e5], d["avg_stoa"]))
    sp_path, base, wy = _column_files(tmp, "7460_28", case, sp, f"sp_{run}", False, gases=set(gases),
                                      wenyi=ga9 and not solar, digits=17, extra=extra)
    if run.startswith("sw2") or (ga9 and solar):
        surf = tmp / "7460_28.surf"
        write_cdl(surf, "7460_28.surf", [("lat", 1), ("lon", 1), ("basis", 2)],
                  [("lat", ["lat"], [1.0], {}), ("lon", ["lon"], [0.0], {}), ("basis", ["basis"], [1.0, 2.0], {}),
                   ("alb", ["basis", "lat", "lon"], np.reshape(d["avg_surfsw2"], (2, 1, 1)),
                    {"title": "ALBEDO WEIGHTS"})])
    if to_cdf:
        tool = _tool()
        for f in tmp.glob("7460_28.*"):
            tmp_out = f.with_name(f.name + ".cdf")
            subprocess.run([tool, "--convert", str(f), str(tmp_out)], check=True)
            tmp_out.replace(f)
    opts = {"lw_avg": "-R 1 9 -I -t 12 +R -v 11 -g 2 -c -C 2 -K 1 -d 1 -i 1",
            "sw2": "-R 1 6 -S -t 2 +R -v 11 -g 2 -r -C 2 -K 1 -d 3 -i 3",
            "sw_ga9_avg": "-R 1 6 -S +R -g 4 -c -r -C 2 -K 1 -d 5 -i 8"}[run].split()
    return sp_path, base, wy, opts, np.asarray(d["kgo_" + run]), ("nflx" if ga9 else "hrts")


@pytest.mark.gpu
@pytest.mark.parametrize("run,to_cdf", [("lw_avg", False), ("sw2", True), ("sw_ga9_avg", False)])
def test_driver_reproduces_cld7460(gpu_lib, tmp_path, run, to_cdf):
    """The reference's cloud-region example (examples/netcdf/7460_28/run_me)
    through the column driver: -C 2 with solver 11, or the default solver 16
    with the GA9 file; a surface of one albedo weight or of two (diffuse and
    direct); the written heating rates or net fluxes against the
    known-good output (half a unit of the 6th digit from CDL, 2e-5 of the
    largest from single-precision netCDF)."""
    import cld7460 as K
    tool = _tool()
    sp_path, base, wy, opts, kgo, kind = _cld7460_files(tmp_path, run, to_cdf)
    cmd = [tool, "-s", str(sp_path)] + opts + ["-B", str(base)] + (["-W", str(wy)] if wy else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = str(base) + "." + kind
    if to_cdf:
        scipy_io = pytest.importorskip("scipy.io")
        with scipy_io.netcdf_file(out, "r", mmap=False) as nc:
            got = np.array(nc.variables[kind][:]).ravel()
        assert np.abs(got - kgo).max() <= 2e-5 * np.abs(kgo).max()
    else:
        _, got = field(out)
        assert K.half_units(got, kgo).max() <= 1.05


@pytest.mark.gpu
@pytest.mark.parametrize("to_cdf", [False, True])
def test_driver_reproduces_circ6_sw_aerosol(gpu_lib, tmp_path, to_cdf):
    """CIRC case 6 in the short wave with the GA7 file, two-region clouds and
    the overlay of prescribed soot optical properties through the column
    driver (examples/netcdf/CIRC_case6/run_me: -R 1 6 -S +R -g 4 -c -r -a +A
    -C 2 -K 1 -d 5 -i 8): the driver reads the aerosol species of the
    spectral file (block 11), finds case6.op_soot, makes soot unparametrized
    and runs the others with zero mixing ratios (no files); the surface file
    has a 'bands' dimension (one albedo per band)."""
    import circ6_sw as K
    from socrates_gb300.spectrum import Spectrum
    tool = _tool()
    d = dict(np.load(K.FIXTURE))
    sp = Spectrum.load_npz(K.FIXTURE, prefix="sp_")
    d["t_ground"] = np.zeros(1)
    d["alb"] = np.zeros(1)
    extra = {k: (d["p"], d[k]) for k in ("clfr", "lwm", "iwm", "re", "ire")}
    extra.update(szen=([1.013e5], d["szen"]), stoa=([1.013e5], d["stoa"]))
    sp_path, base, _ = _column_files(tmp_path, "case6", d, sp, "sp_sw_ga7", False,
                                     gases=set(int(x) for x in d["gases_present"]), digits=17, extra=extra)
    nb = sp.n_band
    surf = tmp_path / "case6.surf"
    write_cdl(surf, "case6.surf", [("lon", 1), ("lat", 1), ("basis", 1), ("bands", nb)],
              [("lon", ["lon"], [0.0], {}), ("lat", ["lat"], [0.0], {}), ("basis", ["basis"], [1.0], {}),
               ("bands", ["bands"], np.arange(1, nb + 1), {}),
               ("alb", ["bands", "basis", "lat", "lon"], np.reshape(np.load(K.FIXTURE)["alb"], (nb, 1, 1, 1)), {})],
              digits=17)
    lev = d["soot_plev"]
    nl, nm = lev.size, d["soot_phf"].shape[1]
    op = tmp_path / "case6.op_soot"
    write_cdl(op, "case6.op_soot", [("lon", 1), ("lat", 1), ("plev", nl), ("mom", nm), ("band", nb)],
              [("lon", ["lon"], [0.0], {}), ("lat", ["lat"], [0.0], {}), ("plev", ["plev"], lev, {"units": "Pa"}),
               ("mom", ["mom"], np.arange(1, nm + 1), {}), ("band", ["band"], np.arange(1, nb + 1), {}),
               ("abs", ["band", "plev", "lat", "lon"], np.reshape(d["soot_abs"], (nb, nl, 1, 1)), {}),
               ("scat", ["band", "plev", "lat", "lon"], np.reshape(d["soot_scat"], (nb, nl, 1, 1)), {}),
               ("phf", ["band", "mom", "plev", "lat", "lon"], np.reshape(d["soot_phf"], (nb, nm, nl, 1, 1)), {})],
              digits=17)
    if to_cdf:
        for f in (surf, op):
            out = f.with_name(f.name + ".cdf")
            subprocess.run([tool, "--convert", str(f), str(out)], check=True)
            out.replace(f)
    cmd = [tool, "-s", str(sp_path), "-R", "1", str(nb), "-S", "+R", "-g", "4", "-c", "-r", "-a", "+A", "-C", "2",
           "-K", "1", "-d", "5", "-i", "8", "-B", str(base)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, hr = field(str(base) + ".hrts")
    kgo = d["kgo_hrts"]
    half_unit = 0.5 * 10.0 ** (np.floor(np.log10(np.abs(kgo))) - 5)
    err = np.abs(hr - kgo) / half_unit
    assert err.max() <= 1.05, f"layer {err.argmax()}: {hr[err.argmax()]} vs {kgo[err.argmax()]}"
    # without the overlay soot falls back to its parametrization with no
    # mixing ratio: the heating rates lose the aerosol
    r = subprocess.run([x for x in cmd if x != "+A"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, hr2 = field(str(base) + ".hrts")
    assert (np.abs(hr2 - kgo) / half_unit).max() > 1000.0


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["triple", "part_corr_cnv"])
def test_driver_three_regions(gpu_lib, tmp_path, scheme):
    """Three regions through the column driver (-C 6 -K 3, solver 17 by
    default; -C 8 with -dp 3000 +dp 1000 for partially correlated like
    regions): the 7460_28 long-wave column with 40 % of its cloud made
    convective (.ccfr) and denser convective water (.lwmcv), .clfr holding
    the stratiform rest.  The written heating rates match the oracle on the
    same clouds (set up as input_cloud_cdf.f does: stratiform water and ice
    of type 1, convective water and ice of type 2) to half a unit of their
    6th digit."""
    import cld7460 as K
    import oracle as O
    from dataclasses import replace
    from socrates_gb300 import abi
    tool = _tool()
    sp_path, base, wy, opts, _, _ = _cld7460_files(tmp_path, "lw_avg", False)
    lev, clfr = field(str(base) + ".clfr")
    _, lwm = field(str(base) + ".lwm")
    lev, clfr, lwm = (np.asarray(a, dtype=np.float64).ravel() for a in (lev, clfr, lwm))
    for suffix, vals in (("clfr", 0.6 * clfr), ("ccfr", 0.4 * clfr), ("lwmcv", 1.5 * lwm)):
        write_cdl(tmp_path / f"7460_28.{suffix}", f"7460_28.{suffix}", [("lat", 1), ("lon", 1), ("plev", lev.size)],
                  [("lat", ["lat"], [1.0], {}), ("lon", ["lon"], [0.0], {}),
                   ("plev", ["plev"], lev, {"units": "Pa", "title": "PRESSURE"}),
                   (suffix, ["plev", "lon", "lat"], np.reshape(vals, (lev.size, 1, 1)), {"units": "None"})], 17)
    for src, dst in (("re", "recv"), ("iwm", "iwmcv"), ("ire", "irecv")):
        text = (tmp_path / f"7460_28.{src}").read_text().replace(f"7460_28.{src}", f"7460_28.{dst}")
        (tmp_path / f"7460_28.{dst}").write_text(text)
    opts = "-R 1 9 -I -t 12 +R -g 2 -c -C 6 -K 3 -d 1 -i 1 +d 1 +i 1".split()
    if scheme == "part_corr_cnv":
        opts[opts.index("-C") + 1] = "8"
        opts += "-dp 3000 +dp 1000".split()
    r = subprocess.run([tool, "-s", str(sp_path)] + opts + ["-B", str(base)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, got = field(str(base) + ".hrts")
    ctl, sp, col, _, _ = K.setup("lw_avg", K.spectra())
    c = col.cld
    w = c["w_cloud"]
    mr, dc = c["condensed_mix_ratio"], c["condensed_dim_char"]
    col.cld = dict(c, n_condensed=4, type_condensed=[1, 2, 3, 4], i_cloud_type=[1, 1, 2, 2], n_cloud_type=2,
                   i_condensed_param=list(c["i_condensed_param"]) * 2, i_condensed_type=list(c["i_condensed_type"]) * 2,
                   condensed_mix_ratio=np.asfortranarray(np.concatenate([mr, mr * np.array([1.5, 1.0])], axis=2)),
                   condensed_dim_char=np.asfortranarray(np.concatenate([dc, dc], axis=2)),
                   frac_cloud=np.asfortranarray(np.stack([np.where(w > 0, 0.6, 0.0), np.where(w > 0, 0.4, 0.0)],
                                                         axis=2)))
    ctl = replace(ctl, i_cloud=abi.IP_CLOUD_TRIPLE if scheme == "triple" else abi.IP_CLOUD_PART_CORR_CNV,
                  i_solver=abi.IP_SOLVER_TRIPLE_HOGAN, i_cloud_representation=abi.IP_CLOUD_CONV_STRAT)
    col.cld.update(dp_corr_strat=3000.0, dp_corr_conv=1000.0)
    ref = K.printed(O.radiance_calc(ctl, sp, col), col, "hrts")[0]
    assert K.half_units(got, ref).max() <= 1.05
