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


def test_block_lists_are_checked_on_the_host():
    """FLASH block ids (1-based) are checked before any launch: ids outside
    the store, ids of refined (non-leaf) blocks and repeated ids are
    rejected; the empty list and any order of distinct leaves pass."""
    import numpy as np
    import pytest
    from torch_gb300 import gbhydro as G
    leaf = np.array([0, 2, 3, 5], np.int32)  # blocks 1, 4 (0-based) are refined
    assert G.check_leaf_ids([], 6, leaf).size == 0
    assert np.array_equal(G.check_leaf_ids([6, 1, 4], 6, leaf), [5, 0, 3])
    for bad, what in (([0], "outside"), ([7], "outside"), ([-2], "outside"), ([2], "not a leaf"),
                      ([5], "not a leaf"), ([1, 3, 1], "more than once"), ([1.0], "integers")):
        with pytest.raises(G.GBError, match=what):
            G.check_leaf_ids(bad, 6, leaf)


def test_mlp_and_wait_entries_reject_bad_arguments_without_gpu():
    """The surrogate MLP's entries and the bounded-wait self-check reject
    bad arguments before any device work: null or unaligned feature
    arrays, empty or oversized batches, an inference without weights, a
    wait limit outside 1e3 .. 4e9 cycles."""
    import ctypes as C
    from torch_gb300 import gbhydro as G
    L = G.lib()
    ERR_ARG = -1
    assert L.gb_mlp_train(None, None, 10, 1, 16, C.c_float(1e-3), 1, None, None) == ERR_ARG
    assert L.gb_mlp_train(C.c_void_p(16), C.c_void_p(16), 10, 0, 16, C.c_float(1e-3), 1, None, None) == ERR_ARG
    assert L.gb_mlp_train(C.c_void_p(16), C.c_void_p(16), 10, 1, (1 << 20) + 1, C.c_float(1e-3), 1, None,
                          None) == ERR_ARG
    assert L.gb_mlp_train(C.c_void_p(20), C.c_void_p(16), 10, 1, 16, C.c_float(1e-3), 1, None, None) == ERR_ARG
    assert L.gb_mlp_grad(None, None, 10, None, None, None) == ERR_ARG
    assert L.gb_mlp_grad(C.c_void_p(16), C.c_void_p(16), 0, None, None, None) == ERR_ARG
    assert L.gb_mlp_infer(-1, None, None, 1, None) == ERR_ARG
    assert L.gb_mlp_infer(4, C.c_void_p(20), C.c_void_p(16), 1, None) == ERR_ARG
    r = C.c_int(0)
    assert L.gb_check_bounded_wait(10, 0, None, C.byref(r), None) == ERR_ARG
    assert L.gb_check_bounded_wait(5_000_000_000, 0, None, C.byref(r), None) == ERR_ARG
    assert L.gb_check_bounded_wait(2_000_000, 0, None, None, None) == ERR_ARG
