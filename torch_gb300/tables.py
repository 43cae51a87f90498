"""Molecular cooling table I/O.

FLASH reads ``cool.dat`` with ``get_cooling_data``
(src/flash/source/physics/sourceTerms/Heat/HeatMain/HeatCool/phenHeat/
mol_and_dust/get_cooling_data.F90:20-55): a header ``(2(2X,I4.4))`` with
TEMP_PTS=320 and DENS_PTS=190, then 60 800 records ``6(2X,F8.4)`` holding
log10 T, log10 n, three unused columns and log10 Lambda, temperature outer
and density inner. Every field is a multiple of 1e-4, so the table is stored
losslessly as int32 counts of 1e-4 in a compact binary ``cool_table.bin``
(magic ``GBCOOL01``, int32 TEMP_PTS, DENS_PTS, then logT[320], logn[190],
logL[320*190] with density fastest). The C library reads either format.
"""
from __future__ import annotations

import os
import struct

import numpy as np

TEMP_PTS, DENS_PTS = 320, 190
MAGIC = b"GBCOOL01"
DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
COMPACT_PATH = os.path.join(DATA_DIR, "cool_table.bin")


def parse_flash_cool_dat(path: str):
    """Return int32 (logT[320], logn[190], logL[320*190]) in units of 1e-4."""
    with open(path, "r") as f:
        head = f.readline().split()
        if len(head) != 2 or int(head[0]) != TEMP_PTS or int(head[1]) != DENS_PTS:
            raise ValueError(f"wrong number of data points in {path}: {head}")
        vals = np.empty((TEMP_PTS * DENS_PTS, 6), np.int64)
        for r in range(TEMP_PTS * DENS_PTS):
            line = f.readline()
            if len(line.rstrip("\n")) < 60:
                raise ValueError(f"read error at record {r + 1} of {path}")
            for c in range(6):
                fld = line[10 * c:10 * c + 10]
                vals[r, c] = int(round(float(fld) * 1e4))
    logT = vals[::DENS_PTS, 0].astype(np.int32)          # cool_dat(1, :, 1)
    logn = vals[:DENS_PTS, 1].astype(np.int32)           # cool_dat(:, 1, 2)
    logL = vals[:, 5].astype(np.int32)                   # cool_dat(:, :, 3)
    return logT, logn, logL


def write_compact(path: str, logT, logn, logL) -> None:
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<ii", TEMP_PTS, DENS_PTS))
        f.write(np.ascontiguousarray(logT, "<i4").tobytes())
        f.write(np.ascontiguousarray(logn, "<i4").tobytes())
        f.write(np.ascontiguousarray(logL, "<i4").tobytes())


def read_compact(path: str = COMPACT_PATH):
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: not a compact cooling table")
        nt, nd = struct.unpack("<ii", f.read(8))
        if (nt, nd) != (TEMP_PTS, DENS_PTS):
            raise ValueError(f"{path}: table shape {nt}x{nd}")
        logT = np.frombuffer(f.read(4 * nt), "<i4").copy()
        logn = np.frombuffer(f.read(4 * nd), "<i4").copy()
        logL = np.frombuffer(f.read(4 * nt * nd), "<i4").copy()
    return logT, logn, logL


def table_values(logT, logn, logL):
    """10**(k/1e4) as the Fortran computes ``10.e0**x``: scalar libm pow
    (numpy's vectorised power can differ from it in the last bit)."""
    import math
    T = np.array([math.pow(10.0, int(k) / 10000.0) for k in logT])
    n = np.array([math.pow(10.0, int(k) / 10000.0) for k in logn])
    L = np.array([math.pow(10.0, int(k) / 10000.0) for k in logL])
    return T, n, L


if __name__ == "__main__":
    import sys
    src = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else COMPACT_PATH
    write_compact(out, *parse_flash_cool_dat(src))
    print("wrote", out)
