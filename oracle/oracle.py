"""ctypes binding of the CPU oracle (oracle/liboracle.so).

Test infrastructure only: used by tests/, by ``__graft_entry__.smoke()`` to
compare GPU results against, and by ``bench.py`` for the timed CPU baseline. The product
library never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

TEMP_PTS, DENS_PTS = 320, 190
ORV = dict(DENS=0, VELX=1, VELY=2, VELZ=3, PRES=4, ENER=5, EINT=6, MAGX=7, MAGY=8, MAGZ=9)
ORV_NVAR = 10


class CoolParams(C.Structure):
    _fields_ = [
        ("tradmin", C.c_double), ("tradmax", C.c_double), ("dradmin", C.c_double),
        ("dradmax", C.c_double), ("theatmin", C.c_double), ("theatmax", C.c_double),
        ("absTmin", C.c_double), ("absTmax", C.c_double), ("Gzero", C.c_double),
        ("subfactor", C.c_double), ("smallp", C.c_double), ("use_cr_heating", C.c_int),
        ("crIonRate", C.c_double), ("crIonNH", C.c_double), ("crIonExp", C.c_double),
        ("crIonEnergy", C.c_double), ("dust_sputter_temp", C.c_double), ("pe_recipe", C.c_int),
        ("pe_norm", C.c_double), ("boltz", C.c_double), ("mp", C.c_double),
        ("T_cool_min", C.c_double), ("nd_cool_min", C.c_double), ("nd_cool_max", C.c_double),
        ("useDustCool", C.c_int), ("int_method", C.c_int), ("mu_mol", C.c_double),
    ]


class Table(C.Structure):
    _fields_ = [
        ("T", C.c_double * TEMP_PTS), ("n", C.c_double * DENS_PTS),
        ("lam", C.c_double * (TEMP_PTS * DENS_PTS)), ("T_min", C.c_double),
        ("nd_min", C.c_double),
    ]


class CoolVars(C.Structure):
    _fields_ = [(k, C.c_double) for k in
                ("ndens", "rho", "conf", "Gflux", "ephen", "tdust", "TtoEI", "xHp",
                 "strat_factor", "mu_mol")]


class HydroParams(C.Structure):
    _fields_ = [
        ("gamma", C.c_double), ("cvisc", C.c_double), ("use_avisc", C.c_int),
        ("eint_switch", C.c_double), ("smlrho", C.c_double), ("smallp", C.c_double),
        ("mhd", C.c_int), ("nxb", C.c_int), ("nguard", C.c_int), ("energy_fix", C.c_int), ("cfl_sum", C.c_int),
        ("hybrid_order", C.c_int), ("fallback_lower_cfl", C.c_int), ("hybrid_kappa", C.c_double),
        ("cfl_fallback_factor", C.c_double), ("cfl", C.c_double), ("cflc", C.c_void_p),
        ("emf_average", C.c_int),
    ]

    def keep_cfl_codes(self, nblocks: int):
        """Per-cell CFL codes for nblocks store blocks (the array stays
        alive with the params object)."""
        self._cflc = np.zeros((nblocks, 4096), np.uint8)
        self.cflc = self._cflc.ctypes.data_as(C.c_void_p)
        return self._cflc


_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.orc_cool_default_params.argtypes = [C.POINTER(CoolParams)]
        L.orc_table_load_flash.argtypes = [C.POINTER(Table), C.c_char_p]
        L.orc_table_load_flash.restype = C.c_int
        L.orc_table_from_ilog.argtypes = [C.POINTER(Table), ip, ip, ip]
        L.orc_find.argtypes = [dp, C.c_double, C.c_int]
        L.orc_find.restype = C.c_int
        L.orc_radloss.argtypes = [C.c_double]
        L.orc_radloss.restype = C.c_double
        L.orc_dust_cooling.argtypes = [C.POINTER(CoolParams), C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_dust_cooling.restype = C.c_double
        L.orc_heating_and_cooling.argtypes = [C.POINTER(CoolParams), C.POINTER(Table), C.POINTER(CoolVars),
                                              C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double),
                                              C.c_void_p]
        L.orc_dei_dt.argtypes = [C.POINTER(CoolParams), C.POINTER(Table), C.POINTER(CoolVars),
                                 C.c_double, C.c_double]
        L.orc_dei_dt.restype = C.c_double
        L.orc_dopr5_line_kat.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                         C.c_double, C.c_double, dp, dp, C.c_int]
        L.orc_dopr5_line_kat.restype = C.c_int
        optd = C.c_void_p
        L.orc_radheat_cells.argtypes = [C.POINTER(CoolParams), C.POINTER(Table), C.c_int64,
                                        C.c_double, optd, optd, optd, optd, optd, optd, optd,
                                        optd, optd, optd, optd, optd, optd]
        L.orc_radheat_cells.restype = C.c_int
        L.orc_radheat_cells_omp.argtypes = L.orc_radheat_cells.argtypes
        L.orc_radheat_cells_omp.restype = C.c_int
        L.orc_hydro_default_params.argtypes = [C.POINTER(HydroParams), C.c_int]
        L.orc_unsplit_block.argtypes = [C.POINTER(HydroParams), optd, optd, optd, optd,
                                        C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_unsplit_block.restype = C.c_int
        L.orc_unsplit_blocks.argtypes = [C.POINTER(HydroParams), C.c_int, optd, optd, optd, optd,
                                         C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_unsplit_blocks.restype = C.c_long
        L.orc_dt_limit_blocks.argtypes = [C.POINTER(HydroParams), C.c_int, optd, C.c_double,
                                          C.c_double, C.c_double]
        L.orc_dt_limit_blocks.restype = C.c_double
        L.orc_fill_guards_periodic.argtypes = [C.POINTER(HydroParams), C.c_int, C.c_int, C.c_int,
                                               optd, optd, optd, optd]
        L.orc_conserved_totals.argtypes = [C.POINTER(HydroParams), C.c_int, optd, optd, optd,
                                           optd, C.c_double, C.c_double, C.c_double, dp]
        L.orc_test_eig.argtypes = [C.c_int, C.c_double, dp, dp, dp, dp]
        L.orc_fill_guards_tree.argtypes = [C.POINTER(HydroParams), C.c_int, optd, optd, optd, optd, C.c_int,
                                           C.c_int, C.c_int, C.c_int, optd, optd, optd, optd]
        L.orc_fill_guards_list.argtypes = [C.POINTER(HydroParams), C.c_int, optd, optd, optd, optd, optd,
                                           C.c_int, C.c_int, C.c_int, C.c_int, optd, optd, optd, optd]
        L.orc_dt_limit_list.argtypes = [C.POINTER(HydroParams), C.c_int, optd, optd, optd, C.c_double]
        L.orc_dt_limit_list.restype = C.c_double
        L.orc_unsplit_list.argtypes = [C.POINTER(HydroParams), C.c_int, optd, optd, optd, optd, optd, optd,
                                       C.c_double, C.c_double]
        L.orc_unsplit_list.restype = C.c_long
        L.orc_unsplit_tree.argtypes = [C.POINTER(HydroParams), C.c_int, optd, optd, optd, optd, optd, C.c_int,
                                       C.c_int, C.c_int, C.c_int, optd, optd, optd, optd, C.c_double, C.c_double,
                                       C.c_int]
        L.orc_unsplit_tree.restype = C.c_long
        L.orc_face_links.argtypes = [C.c_int, optd, optd, optd, optd, C.c_int, C.c_int, C.c_int, C.c_int, optd, optd]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def cool_params(**over) -> CoolParams:
    p = CoolParams()
    lib().orc_cool_default_params(C.byref(p))
    for k, v in over.items():
        setattr(p, k, v)
    return p


def table_from_ilog(logT, logn, logL) -> Table:
    t = Table()
    lib().orc_table_from_ilog(C.byref(t), np.ascontiguousarray(logT, np.int32),
                              np.ascontiguousarray(logn, np.int32),
                              np.ascontiguousarray(logL, np.int32))
    return t


def table_load_flash(path: str) -> Table:
    t = Table()
    rc = lib().orc_table_load_flash(C.byref(t), path.encode())
    if rc != 0:
        raise IOError(f"cool.dat load failed ({rc}): {path}")
    return t


def radheat_cells(p: CoolParams, t: Table, dt: float, dens, ener, eint, temp, tdus,
                  velx=None, vely=None, velz=None, xhp=None, phhe=None, pefl=None,
                  threads: int | None = None):
    """Apply RadHeat's per-cell body in place; returns (iters, flags)."""
    n = dens.size
    iters = np.zeros(n, np.int32)
    flags = np.zeros(n, np.int32)
    args = (C.byref(p), C.byref(t), n, dt, _p(dens), _p(velx), _p(vely), _p(velz), _p(ener),
            _p(eint), _p(temp), _p(tdus), _p(xhp), _p(phhe), _p(pefl), _p(iters), _p(flags))
    if threads == 1:
        lib().orc_radheat_cells(*args)
    else:
        if threads:
            lib().orc_set_num_threads(threads)
        lib().orc_radheat_cells_omp(*args)
    return iters, flags


def hydro_params(mhd: bool, **over) -> HydroParams:
    p = HydroParams()
    lib().orc_hydro_default_params(C.byref(p), int(mhd))
    for k, v in over.items():
        setattr(p, k, v)
    return p


def unsplit_blocks(p: HydroParams, u, bx, by, bz, dt, dx, dy, dz, threads: int | None = None):
    if threads:
        lib().orc_set_num_threads(threads)
    nb = u.shape[0]
    return lib().orc_unsplit_blocks(C.byref(p), nb, _p(u), _p(bx), _p(by), _p(bz), dt, dx, dy, dz)


def fill_guards_periodic(p: HydroParams, nbx, nby, nbz, u, bx=None, by=None, bz=None):
    lib().orc_fill_guards_periodic(C.byref(p), nbx, nby, nbz, _p(u), _p(bx), _p(by), _p(bz))


def fill_guards_tree(p: HydroParams, tree: dict, u, bx=None, by=None, bz=None):
    """AMR guard fill over a torch_gb300.amr tree dict."""
    a = {k: np.ascontiguousarray(tree[k], np.int32) for k in ("level", "coord", "child", "root")}
    nr = tree["nr"]
    lib().orc_fill_guards_tree(C.byref(p), len(a["level"]), _p(a["level"]), _p(a["coord"]), _p(a["child"]),
                               _p(a["root"]), nr[0], nr[1], nr[2], int(tree["maxlevel"]), _p(u), _p(bx),
                               _p(by), _p(bz))


class TreeLists:
    """int32 copies of a block tree's arrays for the leaf-list drivers."""

    def __init__(self, tree: dict):
        self.a = {k: np.ascontiguousarray(tree[k], np.int32) for k in ("level", "coord", "child", "root")}
        self.nr = tree["nr"]
        self.maxlevel = int(tree["maxlevel"])


def fill_guards_list(p: HydroParams, tl: TreeLists, leaves, u, bx=None, by=None, bz=None):
    """OpenMP guard fill of the listed leaves (every leaf read must be up to date)."""
    a = tl.a
    ls = np.ascontiguousarray(leaves, np.int32)
    lib().orc_fill_guards_list(C.byref(p), len(ls), _p(ls), _p(a["level"]), _p(a["coord"]), _p(a["child"]),
                               _p(a["root"]), tl.nr[0], tl.nr[1], tl.nr[2], tl.maxlevel, _p(u), _p(bx), _p(by),
                               _p(bz))


def dt_limit_list(p: HydroParams, tl: TreeLists, leaves, u, root_dx) -> float:
    ls = np.ascontiguousarray(leaves, np.int32)
    return lib().orc_dt_limit_list(C.byref(p), len(ls), _p(ls), _p(tl.a["level"]), _p(u), root_dx)


def unsplit_list(p: HydroParams, tl: TreeLists, leaves, u, bx, by, bz, dt, root_dx):
    ls = np.ascontiguousarray(leaves, np.int32)
    return lib().orc_unsplit_list(C.byref(p), len(ls), _p(ls), _p(tl.a["level"]), _p(u), _p(bx), _p(by),
                                  _p(bz), dt, root_dx)


def unsplit_tree(p: HydroParams, tl: TreeLists, leaves, u, bx, by, bz, dt, root_dx, flux_correct=True):
    """One step of the listed leaves, finest level first, with flux
    conservation at fine-coarse faces when flux_correct."""
    a = tl.a
    ls = np.ascontiguousarray(leaves, np.int32)
    return lib().orc_unsplit_tree(C.byref(p), len(ls), _p(ls), _p(a["level"]), _p(a["coord"]), _p(a["child"]),
                                  _p(a["root"]), tl.nr[0], tl.nr[1], tl.nr[2], tl.maxlevel, _p(u), _p(bx), _p(by),
                                  _p(bz), dt, root_dx, int(flux_correct))


def face_links(tl: TreeLists, b: int):
    """(type[6], fine[6, 4]) of leaf b."""
    a = tl.a
    t = np.zeros(6, np.int32)
    f = np.zeros(24, np.int32)
    lib().orc_face_links(int(b), _p(a["level"]), _p(a["coord"]), _p(a["child"]), _p(a["root"]), tl.nr[0], tl.nr[1],
                         tl.nr[2], tl.maxlevel, _p(t), _p(f))
    return t, f.reshape(6, 4)


def dt_limit(p: HydroParams, u, dx, dy, dz) -> float:
    return lib().orc_dt_limit_blocks(C.byref(p), u.shape[0], _p(u), dx, dy, dz)


def totals(p: HydroParams, u, bx, by, bz, dx, dy, dz):
    out = np.zeros(6)
    lib().orc_conserved_totals(C.byref(p), u.shape[0], _p(u), _p(bx), _p(by), _p(bz), dx, dy,
                               dz, out)
    return out


def eig(mhd: bool, gam: float, q8):
    lam = np.zeros(7)
    R = np.zeros((7, 7))
    L = np.zeros((7, 7))
    lib().orc_test_eig(int(mhd), gam, np.ascontiguousarray(q8, np.float64), lam, R, L)
    return lam, R, L


def dopr5_kat(have_hmax=False, hmax=0.0, n_out=101):
    x = np.zeros(n_out)
    t = np.zeros(n_out)
    k = lib().orc_dopr5_line_kat(1e-3, 1e-4, 1e-10, int(have_hmax), hmax, 0.1, 10.0, x, t, n_out)
    return x[:max(k, 0)], t[:max(k, 0)], k
