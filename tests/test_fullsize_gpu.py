"""The bench's full-size AMR configurations through size-independent
properties, where the oracle would take minutes: 4101 leaf blocks over
levels 0-3 (16.8 M zones) and the largest, 16381 leaf blocks over levels
0-4 (67.1 M zones, 24 GB of cell state), both at Mach 5, sigma_ln 1,
beta 1. Graph-replayed steps of the plain FP64 path and of the mixed path
conserve mass and momentum to round-off over the periodic tree (flux
conservation at fine-coarse faces), keep div B at round-off in every leaf,
and leave a finite state with a clean status."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(config):
    from torch_gb300 import amr
    make, ts, ics = (amr.config3_tree, 45, 46) if config == 3 else (amr.config5_tree, 47, 48)
    tree, centres = make(ts)
    st = amr.amr_box(tree, centres, seed=ics, sigma_ln=1.0, mach=5.0, beta=1.0, dA=0.1, contrast=100.0,
                     fwhm_cells=4.0, nvar=10, device="cuda")
    return tree, st


@pytest.mark.parametrize("config,precision", [(3, 0), (3, 1), (5, 0), (5, 1)])
def test_fullsize_amr_conservation_and_divb(gb, config, precision):
    import torch
    tree, st = _state(config)
    assert len(tree["leaf"]) == (4101 if config == 3 else 16381)
    g = gb.grid_from_amr(tree, st, mhd=True, cooling=False)
    root_dx = st["root_dx"]
    del st
    gb.init_hydro(gb.hydro_params(True, precision=precision))
    g.register()
    leaf = g.t_leaf.long()
    lv = torch.as_tensor(np.asarray(tree["level"])[g.leaf], dtype=torch.float64, device="cuda")
    vol = (root_dx / 2 ** lv) ** 3
    s = g.slots
    # leaves in batches of 1024, so that no copy of the whole state is made
    batches = [slice(a, min(a + 1024, len(leaf))) for a in range(0, len(leaf), 1024)]

    def totals():
        tot = torch.zeros(4, dtype=torch.float64, device="cuda")
        mag = torch.zeros(4, dtype=torch.float64, device="cuda")
        for b in batches:
            u = g.u[leaf[b]][:, :, 4:20, 4:20, 4:20]
            rho = u[:, s["DENS"]]
            q = [rho, rho * u[:, s["VELX"]], rho * u[:, s["VELY"]], rho * u[:, s["VELZ"]]]
            tot += torch.stack([(x.sum(dim=(1, 2, 3)) * vol[b]).sum() for x in q])
            mag += torch.stack([(x.abs().sum(dim=(1, 2, 3)) * vol[b]).sum() for x in q])
        return tot.cpu().numpy(), mag.cpu().numpy()

    def divb():
        worst = 0.0
        for b in batches:
            fx, fy, fz = g.fx[leaf[b]], g.fy[leaf[b]], g.fz[leaf[b]]
            d = (fx[:, 4:20, 4:20, 5:21] - fx[:, 4:20, 4:20, 4:20]) + \
                (fy[:, 4:20, 5:21, 4:20] - fy[:, 4:20, 4:20, 4:20]) + (fz[:, 5:21, 4:20, 4:20] - fz[:, 4:20, 4:20, 4:20])
            bmax = torch.stack([fx[:, 4:20, 4:20, 4:21].abs().amax(dim=(1, 2, 3)),
                                fy[:, 4:20, 4:21, 4:20].abs().amax(dim=(1, 2, 3)),
                                fz[:, 4:21, 4:20, 4:20].abs().amax(dim=(1, 2, 3))]).amax(dim=0)
            worst = max(worst, float((d.abs().amax(dim=(1, 2, 3)) / bmax).max()))
        return worst

    def finite():
        return all(bool(torch.isfinite(g.u[leaf[b]][:, :10, 4:20, 4:20, 4:20]).all()) for b in batches)

    t0, m0 = totals()
    g.status_reset()
    for _ in range(2):
        g.step_graph(cool=False)
    torch.cuda.synchronize()
    t1, _ = totals()
    stt = g.status_read()
    assert stt["code"] == 0, stt
    assert finite()
    # mass to round-off; momentum against the total momentum magnitude
    assert abs(t1[0] - t0[0]) <= 1e-12 * t0[0], (t0[0], t1[0])
    assert np.all(np.abs(t1[1:] - t0[1:]) <= 1e-12 * m0[1:]), (t0, t1, m0)
    assert divb() <= 1e-12


def test_fullsize_amr_compliant_path_with_cooling(gb):
    """The metric-compliant path (mixed hydro, the plain integrator on FP32
    rates) with cooling on the 4101-leaf configuration: two graph-replayed
    steps keep mass and momentum to round-off (cooling changes neither), div B
    at round-off, a clean status (no root-finder failure, no floor), and
    finite temperatures inside the integrator's bounds."""
    import torch
    tree, st = _state(3)
    units = gb.code_units()
    gb.init_cooling(gb.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                   time_unit=units["time_unit"]))
    g = gb.grid_from_amr(tree, st, mhd=True, cooling=True)
    root_dx = st["root_dx"]
    del st
    s = g.slots
    g.u[:, s["TEMP"]] = g.u[:, s["EINT"]] * units["vel_unit"] ** 2 * (2.0 / 3.0) * (24.0 / 11.0) * gb.MP / gb.KB
    g.u[:, s["TDUS"]] = 18.0
    gb.init_hydro(gb.hydro_params(True, precision=1))
    gb.set_cooling_mode(2)
    try:
        g.register()
        leaf = g.t_leaf.long()
        lv = torch.as_tensor(np.asarray(tree["level"])[g.leaf], dtype=torch.float64, device="cuda")
        vol = (root_dx / 2 ** lv) ** 3

        def mass_mom():
            u = g.u[leaf][:, :, 4:20, 4:20, 4:20]
            rho = u[:, s["DENS"]]
            q = [rho, rho * u[:, s["VELX"]], rho * u[:, s["VELY"]], rho * u[:, s["VELZ"]]]
            return (torch.stack([(x.sum(dim=(1, 2, 3)) * vol).sum() for x in q]).cpu().numpy(),
                    torch.stack([(x.abs().sum(dim=(1, 2, 3)) * vol).sum() for x in q]).cpu().numpy())

        t0, m0 = mass_mom()
        g.status_reset()
        for _ in range(2):
            g.step_graph(cool=True)
        torch.cuda.synchronize()
        t1, _ = mass_mom()
        stt = g.status_read()
        assert stt["code"] == 0 and not stt["n_code"], stt
        T = g.u[leaf][:, s["TEMP"], 4:20, 4:20, 4:20]
        p = gb.cool_params()
        assert bool(torch.isfinite(T).all()) and float(T.min()) >= p.absTmin and float(T.max()) <= p.absTmax
        assert abs(t1[0] - t0[0]) <= 1e-12 * t0[0]
        assert np.all(np.abs(t1[1:] - t0[1:]) <= 1e-12 * m0[1:])
    finally:
        gb.set_cooling_mode(0)
