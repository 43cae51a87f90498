"""Arithmetic per zone-update of the hot path, counted by the oracle's
counting-scalar build (flopcount.cpp). TEST/MEASUREMENT INFRASTRUCTURE
ONLY: it writes roofline_constants.json at the repository root, which the
benchmark reads to turn step times into achieved FP64 FLOP/s.

Workloads: the 2x2x2-block periodic boxes of 16^3 cells of the hydro
(HLLC) and MHD (HLLD + CT) parity cases, one step each at CFL 0.8, and
the implicit heating/cooling of the MHD box's cells at that step's dt.

python oracle/flopcount.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# the script's own folder would shadow the oracle package by its module
sys.path[:] = [ROOT] + [q for q in sys.path if os.path.abspath(q or ".") != HERE]


def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle_fc.so"], check=True)
    L = C.CDLL(os.path.join(HERE, "liboracle_fc.so"))
    L.fc_read.argtypes = [C.c_void_p]
    L.fc_phase_read.argtypes = [C.c_void_p]
    L.fc_unsplit_blocks.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_double, C.c_double]
    L.fc_dt_blocks.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_double]
    L.fc_radheat_cells.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
    return L


def counts(L):
    out = np.zeros(5, np.uint64)
    L.fc_read(out.ctypes.data_as(C.c_void_p))
    a, m, d, s, t = (int(x) for x in out)
    return {"add": a, "mul": m, "div": d, "sqrt": s, "flops": a + m + d + s, "transcendental": t}


PHASES = ("recon", "flux", "emf", "update")


def phase_counts(L):
    out = np.zeros(20, np.uint64)
    L.fc_phase_read(out.ctypes.data_as(C.c_void_p))
    res = {}
    for k, name in enumerate(PHASES):
        a, m, d, s, t = (int(x) for x in out[5 * k:5 * k + 5])
        res[name] = {"add": a, "mul": m, "div": d, "sqrt": s, "flops": a + m + d + s, "transcendental": t}
    return res


def per(c, n):
    return {k: v / n for k, v in c.items()}


def main():
    from oracle import oracle as O
    from torch_gb300 import gbhydro as G
    from torch_gb300 import tables
    from torch_gb300 import workloads as W
    L = build()
    out = {"definition": "per interior zone-update; + - * / sqrt = 1 flop each (add, mul, div, sqrt), "
                         "exp/log/pow counted as transcendental; negation, fabs, min/max, compares not counted",
           "source": "oracle/flopcount.py (counting-scalar build of the oracle)",
           "phases": "*_phases: the same counts split by the step's phases (recon: reconstruction with the "
                     "hybrid-order divergence; flux: Riemann solves and artificial viscosity; emf: edge "
                     "electric fields; update: face field and cell update), per interior zone-update"}
    zones = 8 * 4096
    for name, mhd, mach, sig in (("hydro_hllc", False, 2.0, 0.5), ("mhd_hlld_ct", True, 5.0, 1.0)):
        ic = W.turbulent_box(2, 2, 2, seed=41 + int(mhd), sigma_ln=sig, mach=mach, mhd=mhd, nvar=10)
        p = O.hydro_params(mhd)
        u = ic["u"].copy()
        fx, fy, fz = (ic[k].copy() for k in ("fx", "fy", "fz")) if mhd else (None, None, None)
        O.fill_guards_periodic(p, 2, 2, 2, u, fx, fy, fz)
        dx = ic["dx"]
        L.fc_reset()
        L.fc_dt_blocks(C.byref(p), 8, u.ctypes.data_as(C.c_void_p), dx)
        out["dt_" + name] = per(counts(L), zones)
        dt = 0.8 * O.dt_limit(p, u, dx, dx, dx)
        ptr = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
        L.fc_reset()
        L.fc_unsplit_blocks(C.byref(p), 8, ptr(u), ptr(fx), ptr(fy), ptr(fz), dt, dx)
        out[name] = per(counts(L), zones)
        out[name + "_phases"] = {k: per(v, zones) for k, v in phase_counts(L).items()}
        if mhd:
            units = G.code_units()
            sl = (slice(None), slice(4, 20), slice(4, 20), slice(4, 20))
            rho = np.ascontiguousarray(u[:, 0][sl] * units["dens_unit"]).ravel()
            ei = np.ascontiguousarray(u[:, 6][sl] * units["vel_unit"] ** 2).ravel()
            T = ei * (2.0 / 3.0) * (24.0 / 11.0) * G.MP / G.KB
            td = np.full_like(T, 18.0)
            cp = O.cool_params()
            tab = O.table_from_ilog(*tables.read_compact())
            ener = ei.copy()
            L.fc_reset()
            L.fc_radheat_cells(C.byref(cp), C.byref(tab), len(rho), dt * units["time_unit"], ptr(rho), ptr(ener),
                               ptr(ei), ptr(T), ptr(td))
            out["cooling_implicit"] = per(counts(L), len(rho))
    m = out["mhd_hlld_ct"]
    out["mhd_cooling_step"] = {k: m[k] + out["dt_mhd_hlld_ct"][k] + out["cooling_implicit"][k] for k in m}
    path = os.path.join(ROOT, "roofline_constants.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
