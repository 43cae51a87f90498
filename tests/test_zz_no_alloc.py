"""The allocation-free FP64 unsplit step (gb_hydro_unsplit_noalloc), for
callers that cannot let the library allocate device memory, against the
allocating entry point gb_hydro_unsplit on the same inputs, two calls in a
row. Collected last so a failure here stops a -x run after everything else."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(gb):
    from torch_gb300 import workloads as W
    ic = W.turbulent_box(2, 2, 1, seed=21, sigma_ln=1.0, mach=3.0, mhd=True, nvar=10)
    return gb.grid_from_workload(ic, mhd=True, cooling=False), ic["dx"]


def test_noalloc_matches_allocating_entry_point(gb):
    import torch
    L = gb.lib()
    ga, dx = _grid(gb)
    gbb, _ = _grid(gb)
    gb.init_hydro(gb.hydro_params(True, precision=0))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        ga.register()
        dt = ga.compute_dt().item()
        ga.fill_guardcells()
        ga.status_reset()
        gb.check(L.gb_hydro_unsplit(4, C.c_void_p(ga.t_leaf.data_ptr()), dt, dt,
                                    C.c_void_p(ga.status.data_ptr()), stream), "gb_hydro_unsplit")
        gbb.register()
        gbb.fill_guardcells()
        gbb.status_reset()
        gb.check(L.gb_hydro_unsplit_noalloc(4, C.c_void_p(gbb.t_leaf.data_ptr()), dt, dt,
                                            C.c_void_p(gbb.status.data_ptr()), stream),
                 "gb_hydro_unsplit_noalloc")
        torch.cuda.synchronize()
        a = ga.u.cpu().numpy()[:, :, 4:20, 4:20, 4:20]
        b = gbb.u.cpu().numpy()[:, :, 4:20, 4:20, 4:20]
        rel = np.abs(a - b) / (np.abs(a) + 1e-300)
        assert rel.max() <= 1e-12, (call, rel.max())
        for fa, fb in ((ga.fx, gbb.fx), (ga.fy, gbb.fy), (ga.fz, gbb.fz)):
            d = np.abs(fa.cpu().numpy() - fb.cpu().numpy()).max()
            assert d <= 1e-12 * np.abs(fa.cpu().numpy()).max()
        assert ga.status_read()["code"] == 0 and gbb.status_read()["code"] == 0


def test_noalloc_rejects_more_blocks_than_its_scratch(gb):
    import torch
    g, _ = _grid(gb)
    gb.init_hydro(gb.hydro_params(True, precision=0))
    g.register()
    too_many = torch.zeros(5, dtype=torch.int32, device="cuda")
    rc = gb.lib().gb_hydro_unsplit_noalloc(5, C.c_void_p(too_many.data_ptr()), 1e-3, 1e-3, None, None)
    assert rc == -5
    assert b"outside 0..4" in gb.lib().gb_last_error()


def test_noalloc_argument_checks(gb):
    """Arguments are checked before any launch: no blocks is a no-op, a
    non-positive dt or a missing list with blocks is rejected."""
    import torch
    g, _ = _grid(gb)
    gb.init_hydro(gb.hydro_params(True, precision=0))
    g.register()
    L = gb.lib()
    lst = C.c_void_p(g.t_leaf.data_ptr())
    assert L.gb_hydro_unsplit_noalloc(0, None, 1e-3, 1e-3, None, None) == 0
    assert L.gb_hydro_unsplit_noalloc(4, lst, 0.0, 1e-3, None, None) == -1
    assert L.gb_hydro_unsplit_noalloc(4, lst, -1e-3, 1e-3, None, None) == -1
    assert L.gb_hydro_unsplit_noalloc(2, None, 1e-3, 1e-3, None, None) == -1
    torch.cuda.synchronize()
