"""Python host over libgbhydro.so (ctypes), with torch for device memory.

Mirrors the reference's per-step call surface for the hot path:

* ``Hydro(blockCount, blockList, timeEndAdv, dt, dtOld, sweepOrder)``
  (src/flash/source/physics/Hydro/HydroMain/unsplit/hy_uhd_interface.F90:472-479,
  called at src/flash/source/Driver/DriverMain/Unsplit/Couple_AMUSE/Driver_evolveFlash.F90:406)
* ``Heat(blockCount, blockList, dt, time)``
  (src/flash/source/physics/sourceTerms/Heat/HeatMain/HeatCool/phenHeat/Heat_interface.F90:10-16)
* ``Driver_computeDt`` reduced to the CFL minimum over leaf blocks
  (src/flash/source/Driver/DriverMain/Unsplit/Couple_AMUSE/Driver_computeDt.F90:327-335,514-515)

FLASH's block ids are 1-based; ``blockList`` here takes FLASH ids and
converts. Errors raise ``GBError`` (the reference aborts through
Driver_abortFlash). There is no CPU fallback: without the CUDA library
every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from . import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
NROLE = 15
ROLES = ["DENS", "VELX", "VELY", "VELZ", "PRES", "ENER", "EINT", "MAGX", "MAGY", "MAGZ", "TEMP",
         "TDUS", "PHHE", "PEFL", "IHP"]
R = {n: i for i, n in enumerate(ROLES)}
NB = 24
N3 = NB ** 3
FSZ = NB * NB * (NB + 1)

ST_NAMES = {0: "ok", 1: "negative density", 2: "pressure floored", 3: "non-finite state",
            4: "root finder not bracketed", 5: "root finder iteration cap", 6: "overheated (T > absTmax)",
            7: "copy wait timed out"}


class GBError(RuntimeError):
    pass


class GridDesc(C.Structure):
    _fields_ = [("nvar", C.c_int), ("maxblocks", C.c_int), ("slot", C.c_int * NROLE),
                ("unk", C.c_void_p), ("facex", C.c_void_p), ("facey", C.c_void_p),
                ("facez", C.c_void_p)]


class TreeDesc(C.Structure):
    _fields_ = [("nnodes", C.c_int), ("nrx", C.c_int), ("nry", C.c_int), ("nrz", C.c_int),
                ("maxlevel", C.c_int), ("level", C.c_void_p), ("coord", C.c_void_p),
                ("child", C.c_void_p), ("root", C.c_void_p), ("xmin", C.c_double * 3),
                ("root_dx", C.c_double * 3)]


class HydroParams(C.Structure):
    _fields_ = [("gamma", C.c_double), ("cfl", C.c_double), ("cvisc", C.c_double),
                ("use_avisc", C.c_int), ("mhd", C.c_int), ("eint_switch", C.c_double),
                ("smlrho", C.c_double), ("smallp", C.c_double), ("precision", C.c_int),
                ("energy_fix", C.c_int), ("hybrid_order", C.c_int), ("fallback_lower_cfl", C.c_int),
                ("hybrid_kappa", C.c_double), ("cfl_fallback_factor", C.c_double), ("cfl_sum", C.c_int),
                ("shock_detect", C.c_int)]


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
        ("xHp_const", C.c_double), ("dens_unit", C.c_double), ("vel_unit", C.c_double),
        ("time_unit", C.c_double), ("eos_abar", C.c_double),
    ]


class HostIO(C.Structure):
    """gb_host_io: a FLASH host's pinned unk and facevar arrays."""
    _fields_ = [("unk", C.c_void_p), ("nunk", C.c_int), ("host_slot", C.c_int * NROLE),
                ("facex", C.c_void_p), ("facey", C.c_void_p), ("facez", C.c_void_p)]


class Status(C.Structure):
    _fields_ = [("code", C.c_int), ("block", C.c_int), ("i", C.c_int), ("j", C.c_int),
                ("k", C.c_int), ("pad", C.c_int), ("value", C.c_double),
                ("n_fallback", C.c_ulonglong), ("n_bracket_fail", C.c_ulonglong),
                ("n_dust_noconv", C.c_ulonglong), ("n_clamped", C.c_ulonglong),
                ("n_eint_switch", C.c_ulonglong), ("n_surrogate", C.c_ulonglong),
                ("n_surrogate_reject", C.c_ulonglong), ("n_code", C.c_ulonglong * 8),
                ("n_rh_fallback", C.c_ulonglong)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("pad", "n_code")}
        d["n_code"] = {ST_NAMES[c]: int(self.n_code[c]) for c in ST_NAMES if self.n_code[c]}
        return d


def status_buffer(device="cuda"):
    """Zeroed device memory for one gb_status."""
    import torch
    return torch.zeros((C.sizeof(Status) + 7) // 8, dtype=torch.float64, device=device)


# every entry point the header declares: name -> (restype, argtypes)
_SIG = {
    "gb_register_grid": (C.c_int, [C.POINTER(GridDesc), C.POINTER(TreeDesc)]),
    "gb_fill_guardcells": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p]),
    "gb_hydro_init": (C.c_int, [C.POINTER(HydroParams)]),
    "gb_hydro_unsplit": (C.c_int, [C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_void_p]),
    "gb_set_chunk_blocks": (C.c_int, [C.c_int]),
    "gb_set_launch_config": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "gb_get_launch_config": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "gb_set_fused": (C.c_int, [C.c_int]),
    "gb_get_fused": (C.c_int, []),
    "gb_set_chunk_streams": (C.c_int, [C.c_int]),
    "gb_get_chunk_streams": (C.c_int, []),
    "gb_step_graph": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gb_step_graph_host": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p]),
    "gb_set_dt_limits": (C.c_int, [C.c_double, C.c_double, C.c_double]),
    "gb_cfl_codes_reset": (C.c_int, [C.c_void_p]),
    "gb_set_flux_correction": (C.c_int, [C.c_int]),
    "gb_measure_fp64_peak": (C.c_int, [C.POINTER(C.c_double)]),
    "gb_measure_fp32_peak": (C.c_int, [C.POINTER(C.c_double)]),
    "gb_check_bounded_wait": (C.c_int, [C.c_longlong, C.c_int, C.c_void_p, C.POINTER(C.c_int), C.c_void_p]),
    "gb_selfcheck_conversions": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gb_graph_reset": (C.c_int, []),
    "gb_graph_info": (C.c_int, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "gb_hydro_unsplit_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_void_p,
                                           C.c_void_p]),
    "gb_compute_dt": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gb_cool_init": (C.c_int, [C.c_char_p, C.POINTER(CoolParams)]),
    "gb_set_brent_tolerance": (C.c_int, [C.c_double]),
    "gb_set_rate_form": (C.c_int, [C.c_int]),
    "gb_cfl_codes_save": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p]),
    "gb_cfl_codes_load": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p]),
    "gb_heat": (C.c_int, [C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_void_p]),
    "gb_cool_cells": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    "gb_evolve_step": (C.c_int, [C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.c_void_p]),
    "gb_grid_upload_flash": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    "gb_grid_download_flash": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    "gb_grid_upload_flash_list": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "gb_grid_download_flash_list": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "gb_grid_upload_faces_list": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "gb_grid_upload_flash_interior_list": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                                     C.c_void_p]),
    "gb_grid_download_flash_interior_list": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                                       C.c_void_p]),
    "gb_grid_upload_faces_interior_list": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                                     C.c_void_p]),
    "gb_grid_download_faces_interior_list": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                                       C.c_void_p]),
    "gb_grid_download_faces_list": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                              C.c_void_p]),
    "gb_status_reset": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gb_status_read": (C.c_int, [C.c_void_p, C.POINTER(Status)]),
    "gb_mlp_init_random": (C.c_int, [C.c_uint64]),
    "gb_mlp_set_weights": (C.c_int, [C.c_void_p, C.c_int]),
    "gb_mlp_get_weights": (C.c_int, [C.c_void_p, C.c_int]),
    "gb_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gb_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_uint64,
                               C.c_void_p, C.c_void_p]),
    "gb_mlp_infer": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "gb_surrogate_samples": (C.c_int, [C.c_int64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gb_set_cooling_mode": (C.c_int, [C.c_int, C.c_double, C.c_int]),
    "gb_prof_enable": (C.c_int, [C.c_int]),
    "gb_prof_read": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "gb_last_error": (C.c_char_p, []),
    "gb_version": (C.c_int, []),
}

_lib = None


def lib(build: bool = True):
    """Load (building if needed) the CUDA library. Raises if it cannot."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build:
            path = _build.build()
        if not os.path.exists(path):
            raise GBError(f"CUDA library missing: {path}")
        L = C.CDLL(path)
        for name, (res, args) in _SIG.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise GBError(f"{what}: rc={rc}: {lib().gb_last_error().decode(errors='replace')}")


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


# ------------------------------------------------------------------ parameters
def hydro_params(mhd: bool, precision: int = 0, **over) -> HydroParams:
    """Values of flash.par.turbsph_standard (:33, :163-165, :197-198,
    :206-208, :213) in code units; floors are code-unit values. The CFL
    limit is the summed form (cfl_sum), the one the unsplit step is stable
    under at cfl 0.8."""
    p = HydroParams(gamma=5.0 / 3.0, cfl=0.8, cvisc=0.1, use_avisc=1, mhd=int(mhd),
                    eint_switch=1.0e-4, smlrho=1e-30, smallp=1e-30, precision=precision,
                    energy_fix=1, hybrid_order=1, fallback_lower_cfl=1, hybrid_kappa=0.0,
                    cfl_fallback_factor=0.9, cfl_sum=1, shock_detect=0)
    for k, v in over.items():
        setattr(p, k, v)
    return p


# CGS constants (CODATA 2006); FLASH's PhysicalConstants unit is not vendored
KB = 1.3806504e-16
MP = 1.672621637e-24
PC = 3.0856775807e18


def cool_params(**over) -> CoolParams:
    """flash.par.turbsph_standard:300-390 (+ phenHeat/Config defaults)."""
    p = CoolParams(
        tradmin=10.0, tradmax=1.0e15, dradmin=1e-99, dradmax=1e10, theatmin=1e-99, theatmax=2.0e4,
        absTmin=10.0, absTmax=1e9, Gzero=1.69, subfactor=0.3, smallp=1.3807e-19, use_cr_heating=1,
        crIonRate=2.0e-17, crIonNH=1e20, crIonExp=0.021, crIonEnergy=20.0 * 1.6022e-12,
        dust_sputter_temp=3e5, pe_recipe=0, pe_norm=1.3e-24, boltz=KB, mp=MP, T_cool_min=10.0,
        nd_cool_min=1e1, nd_cool_max=1e10, useDustCool=1, int_method=0, mu_mol=24.0 / 11.0,
        xHp_const=1e-4, dens_unit=1.0, vel_unit=1.0, time_unit=1.0, eos_abar=24.0 / 11.0)
    for k, v in over.items():
        setattr(p, k, v)
    return p


def code_units(n_mean: float = 10.0, T_mean: float = 100.0, box_pc: float = 1.0,
               mu: float = 24.0 / 11.0):
    """Code units of the turbulent-box workloads: mean density 1 <-> n_mean
    cm^-3 of mean molecular weight mu; pressure 1 <-> rho n k T_mean/mu-ish
    (v_unit^2 = k T_mean / (mu m_p)); box length 1 <-> box_pc parsec."""
    rho_u = n_mean * mu * MP
    v_u = np.sqrt(KB * T_mean / (mu * MP))
    L_u = box_pc * PC
    return dict(dens_unit=rho_u, vel_unit=float(v_u), time_unit=float(L_u / v_u), length_unit=L_u)


# ------------------------------------------------------------------ block trees
def uniform_tree(nbx: int, nby: int, nbz: int):
    """A periodic root grid of same-level leaf blocks (block id = bx +
    nbx*(by + nby*bz))."""
    n = nbx * nby * nbz
    ids = np.arange(n)
    coord = np.stack([ids % nbx, (ids // nbx) % nby, ids // (nbx * nby)], 1).astype(np.int32)
    return dict(level=np.zeros(n, np.int32), coord=coord, child=-np.ones((n, 8), np.int32),
                root=ids.astype(np.int32), nr=(nbx, nby, nbz), maxlevel=0, leaf=ids.astype(np.int32))


def check_leaf_ids(blockList, nblocks: int, leaf) -> np.ndarray:
    """0-based int32 copy of a list of FLASH (1-based) block ids, checked on
    the host before any launch: every id names a leaf block of the store and
    appears once. The C entry points take device lists and index the block
    store with them unchecked, so a bad id must not get that far: FLASH's
    own callers pass the leaf list of the local blocks, each once."""
    ids = np.asarray(blockList).reshape(-1)
    if ids.size and not np.issubdtype(ids.dtype, np.integer):
        raise GBError(f"block ids must be integers, not {ids.dtype}")
    ids = ids.astype(np.int64) - 1  # FLASH ids are 1-based
    bad = (ids < 0) | (ids >= nblocks)
    if bad.any():
        raise GBError(f"block id {int(ids[bad][0]) + 1} outside 1..{nblocks}")
    isleaf = np.zeros(nblocks, bool)
    isleaf[np.asarray(leaf, np.int64)] = True
    if not isleaf[ids].all():
        raise GBError(f"block id {int(ids[~isleaf[ids]][0]) + 1} is not a leaf block")
    u, n = np.unique(ids, return_counts=True)
    if (n > 1).any():
        raise GBError(f"block id {int(u[n > 1][0]) + 1} listed more than once")
    return ids.astype(np.int32)


class Grid:
    """Device block store + block tree registered with the library."""

    def __init__(self, nblocks: int, nvar: int, slots: dict, mhd: bool, tree: dict,
                 root_dx: float, device: str = "cuda"):
        import torch
        self.torch = torch
        self.nblocks, self.nvar, self.mhd = nblocks, nvar, mhd
        self.u = torch.zeros((nblocks, nvar, NB, NB, NB), dtype=torch.float64, device=device)
        if mhd:
            self.fx = torch.zeros((nblocks, NB, NB, NB + 1), dtype=torch.float64, device=device)
            self.fy = torch.zeros((nblocks, NB, NB + 1, NB), dtype=torch.float64, device=device)
            self.fz = torch.zeros((nblocks, NB + 1, NB, NB), dtype=torch.float64, device=device)
        else:
            self.fx = self.fy = self.fz = None
        self.slots = dict(slots)
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.int32), device=device)
        self.t_level = t(tree["level"])
        self.t_coord = t(tree["coord"])
        self.t_child = t(tree["child"])
        self.t_root = t(tree["root"])
        self.tree = tree
        self.root_dx = root_dx
        self.status = status_buffer(device)
        self.leaf = np.nonzero(tree["child"][:, 0] < 0)[0].astype(np.int32)
        self.t_leaf = t(self.leaf)
        self.register()

    def register(self):
        d = GridDesc()
        d.nvar, d.maxblocks = self.nvar, self.nblocks
        for r in range(NROLE):
            d.slot[r] = -1
        for name, s in self.slots.items():
            d.slot[R[name]] = s
        d.unk = self.u.data_ptr()
        if self.mhd:
            d.facex, d.facey, d.facez = self.fx.data_ptr(), self.fy.data_ptr(), self.fz.data_ptr()
        tr = TreeDesc()
        tr.nnodes = int(self.tree["level"].shape[0])
        tr.nrx, tr.nry, tr.nrz = self.tree["nr"]
        tr.maxlevel = int(self.tree["maxlevel"])
        tr.level, tr.coord = self.t_level.data_ptr(), self.t_coord.data_ptr()
        tr.child, tr.root = self.t_child.data_ptr(), self.t_root.data_ptr()
        for q in range(3):
            tr.root_dx[q] = self.root_dx
            tr.xmin[q] = 0.0
        self._desc, self._tree = d, tr
        check(lib().gb_register_grid(C.byref(d), C.byref(tr)), "gb_register_grid")

    # --------------------------------------------------------------- status
    def status_reset(self):
        check(lib().gb_status_reset(_ptr(self.status), _stream()), "gb_status_reset")

    def status_read(self) -> dict:
        self.torch.cuda.synchronize()
        s = Status()
        check(lib().gb_status_read(_ptr(self.status), C.byref(s)), "gb_status_read")
        return s.as_dict()

    # --------------------------------------------------------------- steps
    def list_tensor(self, blockList=None):
        if blockList is None:
            return self.t_leaf, len(self.leaf)
        ids = check_leaf_ids(blockList, self.nblocks, self.leaf)
        return self.torch.as_tensor(ids, device=self.u.device), len(ids)

    def fill_guardcells(self, blockList=None):
        lt, n = self.list_tensor(blockList)
        check(lib().gb_fill_guardcells(n, _ptr(lt), _stream()), "gb_fill_guardcells")

    def compute_dt(self, blockList=None):
        lt, n = self.list_tensor(blockList)
        out = self.torch.zeros(1, dtype=self.torch.float64, device=self.u.device)
        check(lib().gb_compute_dt(n, _ptr(lt), _ptr(out), _stream()), "gb_compute_dt")
        return out

    # device driver clock (gb_driver_state): sim_time, dt, dt_old, t_max, nstep
    DRV_TIME, DRV_DT, DRV_DTOLD, DRV_TMAX, DRV_NSTEP = range(5)

    @property
    def driver(self):
        if getattr(self, "_drv", None) is None:
            self._drv = self.torch.tensor([0.0, 0.0, 0.0, float("inf"), 0.0], dtype=self.torch.float64,
                                          device=self.u.device)
        return self._drv

    def step_graph(self, cool: bool, blockList=None):
        """One whole step (device dt, guard fill, hydro, cooling, clock
        advance) as a replayed CUDA graph; returns the device tensor view
        holding the step's dt."""
        lt, n = self.list_tensor(blockList)
        if blockList is not None:
            self._graph_list = lt  # the graph keeps the pointer
        drv = self.driver
        check(lib().gb_step_graph(n, _ptr(lt), int(cool), _ptr(drv), _ptr(self.status), _stream()),
              "gb_step_graph")
        return drv[self.DRV_DT:self.DRV_DT + 1]

    def step_graph_host(self, io: "HostIO", cool: bool, blockList=None):
        """step_graph for a host-resident state: uploads the listed blocks'
        interiors from the pinned host arrays in `io`, steps, and downloads
        each chunk's interiors while later chunks compute (one graph)."""
        lt, n = self.list_tensor(blockList)
        if blockList is not None:
            self._graph_list = lt
        drv = self.driver
        check(lib().gb_step_graph_host(n, _ptr(lt), int(cool), _ptr(drv), _ptr(self.status), C.byref(io),
                                       _stream()), "gb_step_graph_host")
        return drv[self.DRV_DT:self.DRV_DT + 1]

    def evolve_step(self, dt: float, cool: bool, blockList=None):
        lt, n = self.list_tensor(blockList)
        check(lib().gb_evolve_step(n, _ptr(lt), float(dt), int(cool), _ptr(self.status), _stream()),
              "gb_evolve_step")


# what the Python side last configured (keys of the autotuner's cache)
state = {"precision": None, "mhd": None, "surrogate": False}


def init_hydro(p: HydroParams) -> None:
    check(lib().gb_hydro_init(C.byref(p)), "gb_hydro_init")
    state["precision"], state["mhd"] = int(p.precision), int(p.mhd)


def init_cooling(p: CoolParams, table_path: str | None = None) -> None:
    from . import tables
    path = table_path or tables.COMPACT_PATH
    check(lib().gb_cool_init(path.encode(), C.byref(p)), "gb_cool_init")


def set_dt_limits(dtmin: float = 0.0, dtmax: float = float("inf"), change_factor: float = float("inf")) -> None:
    """Driver_computeDt's limits on every step's dt (code units)."""
    check(lib().gb_set_dt_limits(float(dtmin), float(dtmax), float(change_factor)), "gb_set_dt_limits")


def set_flux_correction(on: bool = True) -> None:
    """Flux conservation at fine-coarse faces (FLASH flux_correct)."""
    check(lib().gb_set_flux_correction(int(on)), "gb_set_flux_correction")


def measure_fp64_peak() -> float:
    """FP64 FMA throughput of this GPU, TFLOP/s."""
    v = C.c_double()
    check(lib().gb_measure_fp64_peak(C.byref(v)), "gb_measure_fp64_peak")
    return v.value


def check_bounded_wait(limit_cycles: int, arrive: bool):
    """Run the bounded-wait self-check: (1 completed or 2 gave up, the
    status it recorded as a dict)."""
    st = status_buffer()
    r = C.c_int(0)
    check(lib().gb_check_bounded_wait(int(limit_cycles), int(arrive), _ptr(st), C.byref(r), _stream()),
          "gb_check_bounded_wait")
    s = Status()
    check(lib().gb_status_read(_ptr(st), C.byref(s)), "gb_status_read")
    return r.value, s.as_dict()


def measure_fp32_peak() -> float:
    """FP32 FMA throughput of this GPU, TFLOP/s."""
    v = C.c_double()
    check(lib().gb_measure_fp32_peak(C.byref(v)), "gb_measure_fp32_peak")
    return v.value


def graph_info() -> tuple:
    """(captures, replays, kernel launches per replay of the current graph)."""
    a, b, k = C.c_longlong(), C.c_longlong(), C.c_longlong()
    check(lib().gb_graph_info(C.byref(a), C.byref(b), C.byref(k)), "gb_graph_info")
    return a.value, b.value, k.value


def set_brent_tolerance(kelvin: float = 1.0) -> None:
    """Brent tolerance floor of the plain implicit step (1 K = heatCool.F90)."""
    check(lib().gb_set_brent_tolerance(float(kelvin)), "gb_set_brent_tolerance")


def set_rate_form(form: int = 0) -> None:
    """Rate formulation gb_cool_cells integrates: 0 = heatCool.F90's terms
    as written, 1 = the same terms with shared transcendentals (the mixed
    hydro path's fused epilogue)."""
    check(lib().gb_set_rate_form(int(form)), "gb_set_rate_form")


def set_launch_config(chunk_blocks: int, recon_tile: int, recon_occupancy: int = 0) -> None:
    check(lib().gb_set_launch_config(int(chunk_blocks), int(recon_tile), int(recon_occupancy)),
          "gb_set_launch_config")


def get_launch_config() -> tuple:
    """(blocks per chunk, reconstruction tile, reconstruction occupancy bound)."""
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    check(lib().gb_get_launch_config(C.byref(a), C.byref(b), C.byref(c)), "gb_get_launch_config")
    return a.value, b.value, c.value


def set_fused(mode) -> None:
    """Reconstruction and Riemann solve fused per block (gb_set_fused): 0
    (False) two kernels, 1 (True) fused with the TMA window in the mixed
    path, 2 fused with the mixed path's stencils read through L1."""
    check(lib().gb_set_fused(int(mode)), "gb_set_fused")


def get_fused() -> int:
    return int(lib().gb_get_fused())


def set_chunk_streams(n: int) -> None:
    """Run consecutive chunks on 1 or 2 streams (bitwise the same results)."""
    check(lib().gb_set_chunk_streams(int(n)), "gb_set_chunk_streams")


def get_chunk_streams() -> int:
    return int(lib().gb_get_chunk_streams())


def set_chunk_blocks(n: int) -> None:
    check(lib().gb_set_chunk_blocks(int(n)), "gb_set_chunk_blocks")


# --------------------------------------------------------------- FLASH surface
_active: Grid | None = None


def use_grid(g: Grid) -> None:
    global _active
    _active = g


def Hydro(blockCount: int, blockList, timeEndAdv: float, dt: float, dtOld: float, sweepOrder: int = 0):
    """FLASH ``Hydro`` -> ``hy_uhd_unsplit(blockCount, blockList, dt, dtOld)``
    on the active grid: guard-cell fill, then one unsplit step of the
    listed (1-based) leaf blocks."""
    g = _require()
    lt, n = g.list_tensor(np.asarray(blockList)[:blockCount])
    check(lib().gb_fill_guardcells(n, _ptr(lt), _stream()), "Grid_fillGuardCells")
    check(lib().gb_hydro_unsplit(n, _ptr(lt), float(dt), float(dtOld), _ptr(g.status), _stream()),
          "hy_uhd_unsplit")


def Heat(blockCount: int, blockList, dt: float, time: float):
    """FLASH ``Heat`` -> ``RadHeat`` per-cell heating/cooling on the active
    grid (the ``he_int_method = "Implicit"`` integrator)."""
    g = _require()
    lt, n = g.list_tensor(np.asarray(blockList)[:blockCount])
    check(lib().gb_heat(n, _ptr(lt), float(dt), float(time), _ptr(g.status), _stream()), "RadHeat")


def Driver_computeDt(blockCount: int, blockList) -> float:
    """CFL minimum over the listed leaf blocks (the device reduction that
    replaces Hydro_computeDt + MPI_AllReduce MINLOC). With no blocks the
    local limit stays at its start value, huge(1.0) (Driver_computeDt.F90:114,
    222), as on a rank that holds no leaf blocks."""
    g = _require()
    if blockCount == 0:
        return float(np.finfo(np.float64).max)
    return float(g.compute_dt(np.asarray(blockList)[:blockCount]).item())


def _require() -> Grid:
    if _active is None:
        raise GBError("no active grid: call use_grid(Grid(...)) first")
    return _active


def cool_cells(dens, ei, temp, tdust, dt, xhp=None, phhe=None, gflux=None, status=None):
    """Per-cell solve on CGS device arrays (torch float64, updated in place)."""
    n = dens.numel()
    check(lib().gb_cool_cells(n, _ptr(dens), _ptr(ei), _ptr(temp), _ptr(tdust), _ptr(xhp), _ptr(phhe),
                              _ptr(gflux), float(dt), _ptr(status), _stream()), "gb_cool_cells")


def grid_from_workload(ic: dict, mhd: bool, cooling: bool, device: str = "cuda") -> Grid:
    """Build a registered Grid from a workloads.turbulent_box dict."""
    nbx, nby, nbz = ic["nbx"], ic["nby"], ic["nbz"]
    slots = {n: i for i, n in enumerate(["DENS", "VELX", "VELY", "VELZ", "PRES", "ENER", "EINT"])}
    nvar = 7
    if mhd:
        slots.update(MAGX=7, MAGY=8, MAGZ=9)
        nvar = 10
    if cooling:
        slots.update(TEMP=nvar, TDUS=nvar + 1)
        nvar += 2
    tree = uniform_tree(nbx, nby, nbz)
    g = Grid(nbx * nby * nbz, nvar, slots, mhd, tree, ic["dx"], device)
    import torch
    k = 10 if mhd else 7
    g.u[:, :k] = torch.as_tensor(ic["u"][:, :k], device=device)
    if mhd:
        g.fx.copy_(torch.as_tensor(ic["fx"], device=device))
        g.fy.copy_(torch.as_tensor(ic["fy"], device=device))
        g.fz.copy_(torch.as_tensor(ic["fz"], device=device))
    return g


# --------------------------------------------------------------- surrogate
NPARAM = 64 * 4 + 64 + 64 * 64 + 64 + 64 * 64 + 64 + 64 + 1


def surrogate_samples(n: int, seed: int, status=None):
    """n training samples from the plain integrator (device tensors)."""
    import torch
    feat = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    tgt = torch.empty(n, dtype=torch.float32, device="cuda")
    check(lib().gb_surrogate_samples(n, seed, _ptr(feat), _ptr(tgt), _ptr(status), _stream()),
          "gb_surrogate_samples")
    return feat, tgt


def mlp_init(seed: int = 0):
    check(lib().gb_mlp_init_random(seed), "gb_mlp_init_random")


def mlp_weights() -> np.ndarray:
    w = np.zeros(NPARAM, np.float32)
    check(lib().gb_mlp_get_weights(w.ctypes.data_as(C.c_void_p), NPARAM), "gb_mlp_get_weights")
    return w


def mlp_set_weights(w) -> None:
    w = np.ascontiguousarray(w, np.float32)
    check(lib().gb_mlp_set_weights(w.ctypes.data_as(C.c_void_p), NPARAM), "gb_mlp_set_weights")


def mlp_grad(feat, tgt):
    g = np.zeros(NPARAM, np.float32)
    loss = np.zeros(1, np.float32)
    check(lib().gb_mlp_grad(_ptr(feat), _ptr(tgt), feat.shape[0], g.ctypes.data_as(C.c_void_p),
                            loss.ctypes.data_as(C.c_void_p), _stream()), "gb_mlp_grad")
    return g, float(loss[0])


def mlp_train(feat, tgt, steps: int, batch: int = 8192, lr: float = 2e-3, seed: int = 1):
    losses = np.zeros(steps, np.float32)
    check(lib().gb_mlp_train(_ptr(feat), _ptr(tgt), feat.shape[0], steps, batch, lr, seed,
                             losses.ctypes.data_as(C.c_void_p), _stream()), "gb_mlp_train")
    return losses


def mlp_infer(feat, tensor_cores: bool = True):
    import torch
    y = torch.empty(feat.shape[0], dtype=torch.float32, device=feat.device)
    check(lib().gb_mlp_infer(feat.shape[0], _ptr(feat), _ptr(y), int(tensor_cores), _stream()), "gb_mlp_infer")
    return y


def set_cooling_mode(mode, rel_tol: float = 2e-3, check_fp64: bool = False):
    """Cooling of a step with cool=True: 0 (False) the plain integrator fused
    into the update, 1 (True) the learned surrogate with the plain
    integrator as fallback, 2 the plain integrator on FP32 rates (the mixed
    path; the FP64 path keeps its reference rates)."""
    m = int(mode)
    check(lib().gb_set_cooling_mode(m, rel_tol, int(check_fp64)), "gb_set_cooling_mode")
    state["surrogate"] = m == 1


PROF_NAMES = ["guard_fill", "recon", "flux", "emf", "faceb", "update", "dt", "heat", "sur_feat", "mlp_infer",
              "sur_accept", "sur_fallback", "layout_copy"]


def prof_enable(on: bool = True):
    check(lib().gb_prof_enable(int(on)), "gb_prof_enable")


def prof_read() -> dict:
    n = len(PROF_NAMES)
    ms = np.zeros(n)
    cnt = np.zeros(n, np.int64)
    check(lib().gb_prof_read(ms.ctypes.data_as(C.c_void_p), cnt.ctypes.data_as(C.c_void_p), n), "gb_prof_read")
    return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(PROF_NAMES) if cnt[i]}


def grid_from_amr(tree: dict, state: dict, mhd: bool = True, cooling: bool = True, device: str = "cuda") -> Grid:
    """Registered Grid over an amr.build_tree tree with an amr.amr_box state."""
    slots = {n: i for i, n in enumerate(["DENS", "VELX", "VELY", "VELZ", "PRES", "ENER", "EINT"])}
    nvar = 7
    if mhd:
        slots.update(MAGX=7, MAGY=8, MAGZ=9)
        nvar = 10
    if cooling:
        slots.update(TEMP=nvar, TDUS=nvar + 1)
        nvar += 2
    nn = len(tree["level"])
    g = Grid(nn, nvar, slots, mhd, tree, state["root_dx"], device)
    k = 10 if mhd else 7
    g.u[:, :k] = state["u"][:, :k].to(device)
    if mhd:
        g.fx.copy_(state["fx"])
        g.fy.copy_(state["fy"])
        g.fz.copy_(state["fz"])
    return g
