"""Reconstruction and Riemann solve fused per block (gb_set_fused): the
face states stay in shared memory, the mixed path stages its primitives
with the tensor memory accelerator. The same arithmetic as the two-kernel
path: FP64 equals the oracle, the mixed path equals the two-kernel mixed
path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def fused(gb):
    gb.set_fused(True)
    yield gb
    gb.set_fused(False)


def _rel(a, b, floor):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


@pytest.mark.parametrize("mhd", [False, True])
def test_fused_fp64_matches_oracle(fused, oracle, mhd):
    """FP64 box, three steps: the fused kernel's step equals the oracle's to
    1e-12 per cell."""
    gb = fused
    from torch_gb300 import workloads as W
    ic = W.turbulent_box(2, 2, 2, seed=43, sigma_ln=0.5, mach=2.0, mhd=mhd, nvar=10)
    g = gb.grid_from_workload(ic, mhd=mhd, cooling=False)
    gb.init_hydro(gb.hydro_params(mhd, precision=0))
    g.register()
    p = oracle.hydro_params(mhd)
    u, fx, fy, fz = (None if ic[k] is None else ic[k].copy() for k in ("u", "fx", "fy", "fz"))
    dx, nv = ic["dx"], (10 if mhd else 7)
    for step in range(3):
        oracle.fill_guards_periodic(p, 2, 2, 2, u, fx, fy, fz)
        dt = 0.8 * oracle.dt_limit(p, u, dx, dx, dx)
        g.evolve_step(dt, cool=False)
        oracle.unsplit_blocks(p, u, fx, fy, fz, dt, dx, dx, dx)
        gu = g.u.cpu().numpy()[:, :nv, 4:20, 4:20, 4:20]
        ou = u[:, :nv, 4:20, 4:20, 4:20]
        scale = np.abs(ou).max(axis=(0, 2, 3, 4), keepdims=True)
        assert np.all(np.abs(gu - ou) <= 1e-12 * np.maximum(np.abs(ou), 1e-2 * scale)), step
    assert g.status_read()["code"] == 0


def _tree_grid(gb, mhd, device="cuda"):
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=5, device=device)
    return gb.grid_from_amr(t, st, mhd=mhd, cooling=False)


@pytest.mark.parametrize("precision,mode", [(0, 1), (1, 1), (1, 2)])
def test_fused_equals_two_kernels_on_tree(gb, precision, mode):
    """Three MHD steps over the 3-level tree with flux conservation and two
    chunk streams: the fused step equals the two-kernel step (FP64 to the
    last bit; the mixed path, whose FP32 arithmetic the compiler may fuse
    differently in the two kernels, to 1e-5 of each field's scale)."""
    import torch
    out = []
    streams = gb.get_chunk_streams()
    try:
        gb.set_chunk_streams(2)
        gb.set_launch_config(16, 32, 0)
        for fused in (0, mode):
            gb.set_fused(fused)
            gb.init_hydro(gb.hydro_params(True, precision=precision))
            g = _tree_grid(gb, True)
            g.register()
            for _ in range(3):
                g.evolve_step(g.compute_dt().item(), cool=False)
            torch.cuda.synchronize()
            out.append(g.u[g.t_leaf.long(), :10, 4:20, 4:20, 4:20].cpu().numpy())
    finally:
        gb.set_fused(False)
        gb.set_chunk_streams(streams)
    a, b = out
    if precision == 0:
        assert np.array_equal(a, b)
    else:
        scale = np.abs(a).max(axis=(0, 2, 3, 4), keepdims=True)
        assert np.max(np.abs(a - b) / scale) < 1e-5


def test_fused_graph_matches_eager(fused):
    """The fused mixed step replayed as a CUDA graph equals it launched
    eagerly, bit for bit."""
    import torch
    gb = fused
    gb.init_hydro(gb.hydro_params(True, precision=1))
    a, b = _tree_grid(gb, True), _tree_grid(gb, True)
    a.register()
    for _ in range(2):
        a.evolve_step(a.compute_dt().item(), cool=False)
    b.register()
    try:
        for _ in range(2):
            b.step_graph(False)
    finally:
        gb.check(gb.lib().gb_graph_reset(), "gb_graph_reset")
    torch.cuda.synchronize()
    assert torch.equal(a.u[a.t_leaf.long()], b.u[b.t_leaf.long()])
