"""Regenerate the golden fixtures in this directory from the reference tree.

Run here (the reference is not present where the GPU tests run):
    python tests/golden/make_golden.py /path/to/reference

Outputs
  dopr5_kat.json      - IntegratorModule/test.dat: the known-answer rows of
                        the DoPr5 driver on dx/dt = t (test.f95:17-38).
  gas_cool.json       - docs/torch_manual/gas_cool.py's own radloss and
                        dustloss evaluated on a temperature grid. Only the
                        module's function definitions are executed (the
                        file plots at import time).
  cool_table_check.json - checksums of the parsed cool.dat columns.
  eq_curve.json       - a subsample of hAc_b_2.0E-17_e_0.021_FUV_1.69.dat
                        (equilibrium n, T; columns per
                        utils/ic-generator/turb-sphere.py:505-506).
"""
from __future__ import annotations

import ast
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main(ref: str) -> None:
    # 1. DoPr5 known-answer vectors
    kat = os.path.join(ref, "src/flash/source/flashUtilities/IntegratorModule/test.dat")
    rows = [list(map(float, l.split())) for l in open(kat) if l.strip()]
    json.dump({"source": "src/flash/source/flashUtilities/IntegratorModule/test.dat",
               "columns": ["x", "t"], "rows": rows}, open(os.path.join(HERE, "dopr5_kat.json"), "w"))

    # 2. the Python restatement's radloss / dustloss
    src = open(os.path.join(ref, "docs/torch_manual/gas_cool.py")).read()
    tree = ast.parse(src)
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in ("radloss", "dustloss", "lin_interp")]
    ns = {"np": np}
    exec(compile(ast.Module(body=keep, type_ignores=[]), "gas_cool.py", "exec"), ns)
    T = np.logspace(0.5, 8.5, 801)
    rad = [ns["radloss"](float(t)) for t in T]
    td = 15.0
    dust = [ns["dustloss"](float(t), td) for t in T]
    json.dump({"source": "docs/torch_manual/gas_cool.py", "T": T.tolist(), "radloss": rad,
               "tdust": td, "dustloss": dust}, open(os.path.join(HERE, "gas_cool.json"), "w"))

    # 3. cool.dat column checksums (the compact table must decode to these)
    from torch_gb300 import tables
    logT, logn, logL = tables.parse_flash_cool_dat(os.path.join(ref, "cool.dat"))
    h = hashlib.sha256()
    for a in (logT, logn, logL):
        h.update(np.ascontiguousarray(a, "<i4").tobytes())
    json.dump({"source": "cool.dat", "sha256_ilog": h.hexdigest(),
               "logT_first_last": [int(logT[0]), int(logT[-1])],
               "logn_first_last": [int(logn[0]), int(logn[-1])],
               "logL_min_max": [int(logL.min()), int(logL.max())]},
              open(os.path.join(HERE, "cool_table_check.json"), "w"))

    # 4. equilibrium curve subsample
    eq = np.loadtxt(os.path.join(ref, "hAc_b_2.0E-17_e_0.021_FUV_1.69.dat"))
    sub = eq[::200]
    json.dump({"source": "hAc_b_2.0E-17_e_0.021_FUV_1.69.dat",
               "columns": ["time", "n", "T", "e", "P/k", "xHp", "mu", "Tdust"],
               "rows": sub.tolist()}, open(os.path.join(HERE, "eq_curve.json"), "w"))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("GBHYDRO_REFERENCE"):
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set GBHYDRO_REFERENCE)")
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["GBHYDRO_REFERENCE"])
