"""Checkpoint and restart (IO_writeCheckpoint / IO_readCheckpoint's role):
a run restarted from a checkpoint continues bit for bit as the
uninterrupted run, driver clock and hybrid-order CFL codes included."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(gb):
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=7, device="cuda")
    g = gb.grid_from_amr(t, st, mhd=True, cooling=True)
    units = gb.code_units()
    g.u[:, g.slots["TEMP"]] = g.u[:, g.slots["EINT"]] * units["vel_unit"] ** 2 * (2.0 / 3.0) * (24.0 / 11.0) \
        * gb.MP / gb.KB
    g.u[:, g.slots["TDUS"]] = 18.0
    return g


@pytest.mark.parametrize("precision,surrogate", [(0, False), (1, True)])
def test_restart_continues_bit_for_bit(gb, tmp_path, precision, surrogate):
    import torch
    from torch_gb300 import checkpoint as CK
    units = gb.code_units()
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    if surrogate:
        gb.mlp_init(3)
    gb.init_hydro(gb.hydro_params(True, precision=precision))
    gb.set_cooling_mode(surrogate)
    path = str(tmp_path / "run.chk")
    try:
        a = _grid(gb)
        a.register()
        for _ in range(3):
            a.step_graph(cool=True)
        hdr = CK.write_checkpoint(path, a, surrogate=surrogate)
        n = a.nblocks * 3 * 16 ** 3
        codes_a = torch.empty(n, dtype=torch.uint8, device="cuda")
        gb.check(gb.lib().gb_cfl_codes_save(codes_a.data_ptr(), n, None), "save")
        for _ in range(3):
            a.step_graph(cool=True)
        torch.cuda.synchronize()
        assert a.status_read()["code"] == 0
        ref = [x.clone() for x in (a.u, a.fx, a.fy, a.fz, a.driver)]
        del a
        if surrogate:
            gb.mlp_init(11)  # other weights: the checkpoint's must come back
        b = CK.read_checkpoint(path, surrogate=surrogate)
        assert b.driver[b.DRV_NSTEP].item() == 3 and hdr["driver"]["nstep"] == 3
        codes_b = torch.empty(n, dtype=torch.uint8, device="cuda")
        gb.check(gb.lib().gb_cfl_codes_save(codes_b.data_ptr(), n, None), "save")
        torch.cuda.synchronize()
        assert torch.equal(codes_a, codes_b)
        for _ in range(3):
            b.step_graph(cool=True)
        torch.cuda.synchronize()
        out = [b.u, b.fx, b.fy, b.fz, b.driver]
        assert all(torch.equal(x, y) for x, y in zip(ref, out))
        with pytest.raises(Exception):
            gb.check(gb.lib().gb_cfl_codes_load(codes_b.data_ptr(), n - 1, None), "load")
    finally:
        gb.set_cooling_mode(False)
