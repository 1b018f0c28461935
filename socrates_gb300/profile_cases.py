"""One small case per kernel of the path, for profiling a single launch:

    python -m socrates_gb300.profile_cases <case>

Each case runs its kernel three times on `cuda:0` (inputs larger than the
L2 cache where the case allows) and prints "ok <case>".  Under ncu, capture
the second launch: `ncu --set full --clock-control none --kernel-name-base
demangled -k regex:<kernel> -s 1 -c 1 python -m socrates_gb300.profile_cases
<case>`.

  fp64_sw           FP64 solar kernel, 10000 columns x 100 layers, the bench's
                    shortwave configuration (flux_kernel<double ...>)
  lwns              mixed infra-red no-scattering kernel, 30000 x 60
  mcica_sw          mixed solar McICA kernel, 8192 x 85, 16 subcolumns
  batched           the multi-batch kernel over 256 mixed requests
  cloud_gen         the McICA subcolumn generator, 8192 x 85
  prsc              prescribed aerosol properties and the solar kernel after
                    them, 10000 x 100 through the host path (column windows)
  phased            the phased kernel, mixed solar, 10000 x 100
  fp64_lwns_phased  the phased kernel, FP64 infra-red no-scattering, 30000 x 60
"""
import sys

import torch

from . import abi, synth
from . import radiance as R
from .device import DeviceCase

CASES = ("fp64_sw", "lwns", "mcica_sw", "batched", "cloud_gen", "prsc", "phased", "fp64_lwns_phased")


def run(mode: str) -> None:
    s = torch.cuda.current_stream().cuda_stream
    lib = R.load_library()
    case = None
    if mode == "fp64_sw":
        sp, col = synth.config2(10000, 100, 2)
        case = DeviceCase(R.sw_control(l_aerosol_mode=True), sp, col)
    elif mode == "lwns":
        sp, col = synth.config1(30000, 60, 1)
        case = DeviceCase(R.lw_noscat_control(precision=abi.PRECISION_MIXED), sp, col)
    elif mode == "mcica_sw":
        _, sw, col = synth.config3(8192, 85, seed=3, n_subcol=16)
        synth.add_sw_surface(col, sw.n_band, 3)
        c_sub, nsc = R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
        mc = R.set_cld_mcica(sw, col, abi.IP_SOLAR, abi.IP_MCICA_SINGLE_SAMPLING, c_sub=c_sub, n_subcol_cld=nsc)
        case = DeviceCase(R.sw_control(i_cloud=abi.IP_CLOUD_MCICA, precision=abi.PRECISION_MIXED), sw, col, mc)
    elif mode == "batched":
        from .batch import Batch
        from .workload import Pools, request_specs
        specs = request_specs(256, 4)
        pools = Pools(specs, 4)
        b = Batch([DeviceCase(*pools.request(q, abi.PRECISION_MIXED), keep_host=False) for q in specs])
        for _ in range(3):
            b.run(s)
    elif mode == "cloud_gen":
        _, _, col = synth.config3(8192, 85, seed=3, n_subcol=16)
        for _ in range(3):
            R.cloud_gen(col, 16, abi.IP_EXPONENTIAL_RAND, abi.RNG_PHILOX)
    elif mode == "prsc":
        sp, col = synth.config2(10000, 100, seed=66)
        col.aer = None
        synth.add_density(col, 1)
        synth.add_aerosol_species(sp, 66, n_humidity=21, n_phf=3)
        synth.add_aerosol_mix(col, 66, entries=(1, 2, 3, 2, 4))
        sp, col = synth.add_prescribed_aerosol(sp, col, 66, species=(2,), n_phf=2)
        ctl = R.sw_control(l_aerosol=True, l_henyey_greenstein_pf=True, precision=abi.PRECISION_MIXED)
        for _ in range(3):
            R.radiance_calc(ctl, sp, col)
    elif mode == "phased":
        lib.socgpu_set_tile_config(1, 1, 1, 8)
        sp, col = synth.config2(10000, 100, 2)
        case = DeviceCase(R.sw_control(l_aerosol_mode=True, precision=abi.PRECISION_MIXED), sp, col)
    elif mode == "fp64_lwns_phased":
        lib.socgpu_set_tile_config(0, 0, 1, 8)
        sp, col = synth.config1(30000, 60, 1)
        case = DeviceCase(R.lw_noscat_control(), sp, col)
    else:
        raise SystemExit(f"unknown case {mode}; one of {', '.join(CASES)}")
    if case is not None:
        for _ in range(3):
            case.run(s)
    torch.cuda.synchronize()
    print("ok", mode)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    run(sys.argv[1])
