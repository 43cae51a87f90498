"""The step's safeguards against the oracle, and long runs at Mach 5.

- hybrid order (hy_uhd_dataReconstOneStep.F90:934-999, :1150-1218): where
  the flow compresses, face states that fail the Rankine-Hugoniot check
  fall back to first order and lower the cell's CFL for the next step;
- energyFix (flash.par.turbsph_standard:213): the gas energy from the
  flux-updated cell field;
- the summed CFL limit, under which the unsplit step stays stable at
  cfl 0.8 (its transverse terms vanish on grid-scale modes).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b) / (np.abs(b) + 1e-300))


@pytest.mark.parametrize("mhd", [False, True])
def test_hybrid_order_fallback_matches_oracle(gb, oracle, mhd):
    """Mach 5, sigma_ln 2 box at the per-direction CFL limit, where the
    hybrid-order check fires: 12 FP64 steps equal the oracle's to 1e-12,
    and every step's dt (scaled by the previous step's per-cell CFL codes)
    is the oracle's to the last bit."""
    from torch_gb300 import workloads as W
    ic = W.turbulent_box(2, 2, 2, seed=43, sigma_ln=2.0, mach=5.0, mhd=mhd, nvar=10)
    g = gb.grid_from_workload(ic, mhd=mhd, cooling=False)
    gb.init_hydro(gb.hydro_params(mhd, cfl_sum=0))
    g.register()
    p = oracle.hydro_params(mhd, cfl_sum=0)
    codes = p.keep_cfl_codes(8)
    u, fx, fy, fz = (None if ic[k] is None else ic[k].copy() for k in ("u", "fx", "fy", "fz"))
    dx = ic["dx"]
    nv = 10 if mhd else 7
    lowered = 0
    g.status_reset()
    for step in range(12):
        oracle.fill_guards_periodic(p, 2, 2, 2, u, fx, fy, fz)
        dt_o = 0.8 * oracle.dt_limit(p, u, dx, dx, dx)
        dt = g.compute_dt().item()
        assert dt == dt_o, (step, dt, dt_o)
        g.evolve_step(dt, cool=False)
        oracle.unsplit_blocks(p, u, fx, fy, fz, dt, dx, dx, dx)
        lowered += int(np.count_nonzero(codes))
        gu = g.u.cpu().numpy()[:, :nv, 4:20, 4:20, 4:20]
        assert _rel(gu, u[:, :nv, 4:20, 4:20, 4:20]) <= 1e-12, step
    st = g.status_read()
    assert lowered > 0 and st["n_rh_fallback"] > 0, (lowered, st)


def _tree_state(gb, mhd, mach=5.0, sigma_ln=1.0, device="cuda"):
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=11, mach=mach, sigma_ln=sigma_ln, device=device)
    return t, st


def test_mach5_tree_25_steps_matches_oracle(gb, oracle):
    """25 FP64 MHD steps of a Mach-5, sigma_ln-1 3-level tree with flux
    conservation, dt on the device each step: the state stays finite, no
    pressure is floored, and it equals the oracle's after every step to
    1e-12 (dt bit for bit)."""
    t, st = _tree_state(gb, True)
    g = gb.grid_from_amr(t, st, mhd=True, cooling=False)
    gb.init_hydro(gb.hydro_params(True))
    g.register()
    p = oracle.hydro_params(True)
    p.keep_cfl_codes(g.nblocks)
    tl = oracle.TreeLists(t)
    u = st["u"][:, :10].cpu().numpy().copy()
    fx, fy, fz = (st[k].cpu().numpy().copy() for k in ("fx", "fy", "fz"))
    leaf = t["leaf"]
    g.status_reset()
    for step in range(25):
        dt = g.compute_dt().item()
        oracle.fill_guards_tree(p, t, u, fx, fy, fz)
        assert dt == 0.8 * oracle.dt_limit_list(p, tl, leaf, u, st["root_dx"]), step
        g.evolve_step(dt, cool=False)
        oracle.unsplit_tree(p, tl, leaf, u, fx, fy, fz, dt, st["root_dx"], flux_correct=True)
        gu = g.u.cpu().numpy()[leaf, :10, 4:20, 4:20, 4:20]
        ou = u[leaf, :10, 4:20, 4:20, 4:20]
        r = np.abs(gu - ou) / (np.abs(ou) + 1e-300)
        w = np.unravel_index(np.argmax(r), r.shape)
        assert r[w] <= 1e-12, (step, w, gu[w], ou[w])
    s = g.status_read()
    assert s["code"] == 0, s
    assert np.all(np.isfinite(gu))


def test_fast_path_25_steps_stays_finite(gb):
    """The fast path (mixed hydro, learned cooling with the plain
    integrator as fallback) on a Mach-5 3-level tree with cooling, 25
    graph-replayed steps: finite temperatures everywhere, no floored
    pressure and no non-finite cell (status counters per code)."""
    import torch
    t, st = _tree_state(gb, True)
    g = gb.grid_from_amr(t, st, mhd=True, cooling=True)
    units = gb.code_units()
    e = g.u[:, g.slots["EINT"]]
    g.u[:, g.slots["TEMP"]] = e * units["vel_unit"] ** 2 * (2.0 / 3.0) * (24.0 / 11.0) * gb.MP / gb.KB
    g.u[:, g.slots["TDUS"]] = 18.0
    # the network learns from the plain integrator in CGS, then the step
    # cools the grid's code units
    gb.init_cooling(gb.cool_params())
    gb.mlp_init(7)
    feat, tgt = gb.surrogate_samples(200_000, 3)
    keep = torch.isfinite(tgt)
    gb.mlp_train(feat[keep].contiguous(), tgt[keep].contiguous(), steps=400, batch=4096, lr=3e-3, seed=5)
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    gb.init_hydro(gb.hydro_params(True, precision=1))
    gb.set_cooling_mode(True)
    try:
        g.register()
        g.status_reset()
        for _ in range(25):
            g.step_graph(True)
        s = g.status_read()
    finally:
        gb.set_cooling_mode(False)
        gb.check(gb.lib().gb_graph_reset(), "gb_graph_reset")
    leaf = torch.as_tensor(np.asarray(t["leaf"]), device="cuda").long()
    T = g.u[leaf, g.slots["TEMP"], 4:20, 4:20, 4:20]
    assert bool(torch.isfinite(T).all()) and float(T.min()) > 0.0
    assert s["code"] == 0, s
