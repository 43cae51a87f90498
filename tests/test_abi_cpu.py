"""The C-ABI library builds, loads without a GPU and exports every symbol
include/gbhydro.h declares."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gbhydro.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(gb_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("gb_hydro_unsplit", "gb_heat", "gb_cool_init", "gb_register_grid",
                 "gb_compute_dt", "gb_evolve_step", "gb_fill_guardcells"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from torch_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.gb_version.restype = ctypes.c_int
    assert lib.gb_version() >= 1


def test_python_binding_covers_header():
    from torch_gb300 import gbhydro
    names = declared_functions()
    assert set(names) <= set(gbhydro._SIG), set(names) - set(gbhydro._SIG)


def test_entry_points_reject_bad_arguments_without_gpu():
    """Argument checks run before any device work: null descriptors and
    missing initialisation come back as error codes, not crashes."""
    from torch_gb300 import gbhydro as G
    L = G.lib()
    assert L.gb_register_grid(None, None) == -1
    assert L.gb_hydro_unsplit(1, None, 1.0, 1.0, None, None) == -3
    assert L.gb_heat(1, None, 1.0, 0.0, None, None) == -3
    assert b"gb_heat" in L.gb_last_error()
