"""Reader of the CDL text files (netCDF's text form) that the reference's
Cl_run_cdl driver takes as input and writes as output
(src/aux/l_run_cdl.F90; read_cdl.f90 and output_flux_cdl layouts): the
dimensions and the data section's variables, as float64 arrays."""
import re

import numpy as np


def read_cdl(path):
    text = open(path).read()
    dims = {m.group(1): int(m.group(2)) for m in re.finditer(r"^\s*(\w+)\s*=\s*(\d+)\s*;", 
                                                                text.split("variables:")[0], re.M)}
    data = text.split("data:", 1)[1]
    out = {}
    for m in re.finditer(r"(\w+)\s*=\s*([^;]*);", data):
        vals = [float(x) for x in m.group(2).replace(",", " ").split()]
        out[m.group(1)] = np.array(vals)
    return dims, out


def field(path, coord="plev"):
    """(coordinate values, values of the one non-coordinate variable)."""
    dims, v = read_cdl(path)
    names = [k for k in v if k not in ("lat", "lon", "plev", "basis")]
    assert len(names) == 1, (path, names)
    return v.get(coord), v[names[0]]


def write_cdl(path, name, dims, variables, digits=7):
    """Write a CDL file like the reference's column files: `dims` is a list
    of (name, length); `variables` a list of (name, dim names, values,
    {attribute: text}) with values in C order, printed with `digits`
    significant digits (the reference's files carry 7)."""
    lines = [f"netcdf {name}{{", "", "dimensions:"]
    for d, n in dims:
        lines.append(f"    {d:<15s}= {n:3d};")
    lines += ["", "", "variables:"]
    for v, vd, _, atts in variables:
        lines.append(f"    float {v}({','.join(vd)});")
        for k, t in atts.items():
            lines.append(f'             {v}:{k} = "{t}";')
    lines += ["", "data:"]
    for v, _, vals, _ in variables:
        flat = [f"{x: .{digits - 1}E}" for x in np.ravel(vals)]
        body = ",\n                    ".join(", ".join(flat[i:i + 4]) for i in range(0, len(flat), 4))
        lines.append(f"{v:>17s} = {body};")
    lines += ["", "}"]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
