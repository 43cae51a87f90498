"""The whole step as a replayed CUDA graph with dt on the device gives the
eager step's state bit for bit."""
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


@pytest.mark.parametrize("precision,mode", [(0, 0), (1, 0), (1, 1), (1, 2)])
def test_graph_step_matches_eager(gb, precision, mode):
    """mode: the cooling mode (plain integrator, learned surrogate, plain
    integrator on FP32 rates)."""
    import torch
    units = gb.code_units()
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    if mode == 1:
        gb.mlp_init(3)
    gb.init_hydro(gb.hydro_params(True, precision=precision))
    a, b = _grid(gb), _grid(gb)
    gb.set_chunk_blocks(16)
    dts = []
    a.register()
    gb.set_cooling_mode(mode)
    for _ in range(3):
        dt = a.compute_dt().item()
        dts.append(dt)
        a.evolve_step(dt, cool=True)
    b.register()
    c0, l0, _ = gb.graph_info()
    for q in range(3):
        d = b.step_graph(cool=True)
        torch.cuda.synchronize()
        assert d.item() == dts[q]
    c1, l1, kn = gb.graph_info()
    gb.set_cooling_mode(False)
    assert (c1 - c0, l1 - l0) == (1, 3)
    assert kn > 0
    assert torch.equal(a.u[a.t_leaf.long()], b.u[b.t_leaf.long()])
    for x, y in ((a.fx, b.fx), (a.fy, b.fy), (a.fz, b.fz)):
        assert torch.equal(x[a.t_leaf.long()], y[b.t_leaf.long()])


def test_graph_recaptured_on_configuration_change(gb):
    import torch
    units = gb.code_units()
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    gb.init_hydro(gb.hydro_params(True, precision=1))
    g = _grid(gb)
    c0, _, _ = gb.graph_info()
    g.step_graph(cool=True)
    g.step_graph(cool=True)
    gb.set_chunk_blocks(8)
    g.step_graph(cool=True)
    g.step_graph(cool=False)
    gb.set_chunk_blocks(16)
    torch.cuda.synchronize()
    c1, _, _ = gb.graph_info()
    assert c1 - c0 == 3
    assert g.status_read()["code"] == 0


@pytest.mark.parametrize("precision", [0, 1])
def test_launch_shapes_do_not_change_results(gb, precision):
    """Chunk size and reconstruction tile only change the launch grid: the
    state after a step is identical for every shape."""
    import torch
    gb.init_hydro(gb.hydro_params(True, precision=precision))
    out = []
    try:
        for chunk, tile, occ in ((16, 32, 0), (5, 64, 0), (64, 32, 1), (7, 64, 2), (9, 32, 2)):
            gb.set_launch_config(chunk, tile, occ)
            g = _grid(gb)
            dt = g.compute_dt().item()
            g.evolve_step(dt, cool=False)
            torch.cuda.synchronize()
            out.append(g.u[g.t_leaf.long()].clone())
            del g
    finally:
        gb.set_launch_config(16, 32)
    assert all(torch.equal(out[0], o) for o in out[1:])


@pytest.mark.parametrize("precision,surrogate", [(0, False), (1, True)])
def test_two_chunk_streams_match_one(gb, precision, surrogate):
    """Chunks alternating between two streams (with flux conservation across
    the three levels of the tree, so chunks wait on each other's flux
    registration) give the one-stream state bit for bit, eager and graph."""
    import torch
    units = gb.code_units()
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    if surrogate:
        gb.mlp_init(3)
    gb.init_hydro(gb.hydro_params(True, precision=precision))
    gb.set_flux_correction(True)
    gb.set_cooling_mode(surrogate)
    out = []
    try:
        for ns, graph in ((1, False), (2, False), (2, True)):
            gb.set_launch_config(7, 32, 1 if precision == 1 else 0)
            gb.set_chunk_streams(ns)
            assert gb.get_chunk_streams() == ns
            g = _grid(gb)
            g.register()
            for _ in range(2):
                if graph:
                    g.step_graph(cool=True)
                else:
                    g.evolve_step(g.compute_dt().item(), cool=True)
            torch.cuda.synchronize()
            assert g.status_read()["code"] == 0
            out.append([g.u[g.t_leaf.long()].clone()] + [x[g.t_leaf.long()].clone() for x in (g.fx, g.fy, g.fz)])
            del g
    finally:
        gb.set_chunk_streams(1)
        gb.set_launch_config(16, 32)
        gb.set_cooling_mode(False)
    for o in out[1:]:
        assert all(torch.equal(x, y) for x, y in zip(out[0], o))
    with pytest.raises(Exception):
        gb.set_chunk_streams(3)


def test_autotuner_picks_a_candidate_and_restores_state(gb, tmp_path, monkeypatch):
    import torch
    from torch_gb300 import autotune
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tune.json"))
    units = gb.code_units()
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    gb.init_hydro(gb.hydro_params(True, precision=1))
    g = _grid(gb)
    before = g.u.clone()
    try:
        r = autotune.tune(g, cool=True, chunks=(8, 16), tiles=(32, 64), steps=1)
        assert (r["chunk"], r["tile"]) in {(8, 32), (8, 64), (16, 32), (16, 64)} and r["occ"] in (0, 1, 2)
        assert gb.get_launch_config() == (r["chunk"], r["tile"], r["occ"])
        assert gb.get_chunk_streams() == r["streams"]
        # 2 chunks x 2 tiles x 3 bounds x 2 stream counts, and each of the
        # two fused modes once per chunk size and stream count
        assert len(r["trials"]) == 24 + 8 and not r["cached"]
        assert gb.get_fused() == r["fused"]
        assert torch.equal(g.u, before)
        r2 = autotune.tune(g, cool=True, chunks=(8, 16), tiles=(32, 64), steps=1)
        assert r2["cached"] and (r2["chunk"], r2["tile"], r2["occ"]) == (r["chunk"], r["tile"], r["occ"])
    finally:
        gb.set_launch_config(16, 32)
        gb.set_chunk_streams(1)
        gb.set_fused(False)


@pytest.mark.parametrize("streams", [1, 2])
def test_host_resident_step_matches_separate_transfers(gb, streams):
    """gb_step_graph_host (interior upload, step, per-chunk downloads
    overlapping later chunks, one graph) leaves the host arrays and the
    device store bit for bit as interior upload + step graph + interior
    download do."""
    import ctypes as C
    import torch
    units = gb.code_units()
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    gb.mlp_init(3)
    gb.init_hydro(gb.hydro_params(True, precision=1))
    gb.set_flux_correction(True)
    gb.set_cooling_mode(True)
    L = gb.lib()
    out = []
    try:
        gb.set_launch_config(7, 32, 1)
        gb.set_chunk_streams(streams)
        for fused in (False, True):
            g = _grid(gb)
            g.register()
            nunk, nn = g.nvar, g.nblocks
            host = torch.empty((nn, 24 ** 3, nunk), dtype=torch.float64).pin_memory()
            hf = [a.cpu().pin_memory() for a in (g.fx, g.fy, g.fz)]
            io = gb.HostIO()
            io.unk, io.nunk = host.data_ptr(), nunk
            for r in range(gb.NROLE):
                io.host_slot[r] = -1
            for name, s in g.slots.items():
                io.host_slot[gb.R[name]] = s
            io.facex, io.facey, io.facez = (h.data_ptr() for h in hf)
            gb.check(L.gb_grid_download_flash(C.c_void_p(host.data_ptr()), nunk, io.host_slot, nn, None), "init")
            torch.cuda.synchronize()
            leaves = np.ascontiguousarray(g.leaf, np.int32)
            lp = leaves.ctypes.data_as(C.c_void_p)
            fp = [C.c_void_p(h.data_ptr()) for h in hf]
            for _ in range(2):
                if fused:
                    g.step_graph_host(io, cool=True)
                else:
                    gb.check(L.gb_grid_upload_flash_interior_list(C.c_void_p(host.data_ptr()), nunk, io.host_slot,
                                                                  len(leaves), lp, None), "up")
                    gb.check(L.gb_grid_upload_faces_interior_list(*fp, len(leaves), lp, None), "up faces")
                    g.step_graph(cool=True)
                    gb.check(L.gb_grid_download_flash_interior_list(C.c_void_p(host.data_ptr()), nunk, io.host_slot,
                                                                    len(leaves), lp, None), "down")
                    gb.check(L.gb_grid_download_faces_interior_list(*fp, len(leaves), lp, None), "down faces")
            torch.cuda.synchronize()
            assert g.status_read()["code"] == 0
            out.append([host.clone()] + [h.clone() for h in hf] + [g.u[g.t_leaf.long()].clone()])
            del g
    finally:
        gb.set_chunk_streams(1)
        gb.set_launch_config(16, 32)
        gb.set_cooling_mode(False)
    assert all(torch.equal(a, b) for a, b in zip(out[0], out[1]))
