"""The bench's full-size AMR configuration (4101 leaf blocks over levels
0-3, 16.8 M zones, Mach 5, sigma_ln 1, beta 1) through size-independent
properties, where the oracle would take minutes: graph-replayed steps of
the plain FP64 path and of the mixed path conserve mass and momentum to
round-off over the periodic tree (flux conservation at fine-coarse faces),
keep div B at round-off in every leaf, and leave a finite state with a
clean status."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state():
    from torch_gb300 import amr
    tree, centres = amr.config3_tree(45)
    st = amr.amr_box(tree, centres, seed=46, sigma_ln=1.0, mach=5.0, beta=1.0, dA=0.1, contrast=100.0,
                     fwhm_cells=4.0, nvar=10, device="cuda")
    return tree, st


@pytest.mark.parametrize("precision", [0, 1])
def test_fullsize_amr_conservation_and_divb(gb, precision):
    import torch
    tree, st = _state()
    assert len(tree["leaf"]) == 4101
    g = gb.grid_from_amr(tree, st, mhd=True, cooling=False)
    gb.init_hydro(gb.hydro_params(True, precision=precision))
    g.register()
    leaf = g.t_leaf.long()
    lv = torch.as_tensor(np.asarray(tree["level"])[g.leaf], dtype=torch.float64, device="cuda")
    dx = st["root_dx"] / 2 ** lv
    vol = dx ** 3
    s = g.slots

    def totals():
        u = g.u[leaf][:, :, 4:20, 4:20, 4:20]
        rho = u[:, s["DENS"]]
        q = [rho, rho * u[:, s["VELX"]], rho * u[:, s["VELY"]], rho * u[:, s["VELZ"]]]
        tot = torch.stack([(x.sum(dim=(1, 2, 3)) * vol).sum() for x in q])
        mag = torch.stack([(x.abs().sum(dim=(1, 2, 3)) * vol).sum() for x in q])
        return tot.cpu().numpy(), mag.cpu().numpy()

    def divb():
        fx, fy, fz = g.fx[leaf], g.fy[leaf], g.fz[leaf]
        d = (fx[:, 4:20, 4:20, 5:21] - fx[:, 4:20, 4:20, 4:20]) + (fy[:, 4:20, 5:21, 4:20] - fy[:, 4:20, 4:20, 4:20]) \
            + (fz[:, 5:21, 4:20, 4:20] - fz[:, 4:20, 4:20, 4:20])
        bmax = torch.stack([fx[:, 4:20, 4:20, 4:21].abs().amax(dim=(1, 2, 3)),
                            fy[:, 4:20, 4:21, 4:20].abs().amax(dim=(1, 2, 3)),
                            fz[:, 4:21, 4:20, 4:20].abs().amax(dim=(1, 2, 3))]).amax(dim=0)
        return float((d.abs().amax(dim=(1, 2, 3)) / bmax).max())

    t0, m0 = totals()
    g.status_reset()
    for _ in range(2):
        g.step_graph(cool=False)
    torch.cuda.synchronize()
    t1, _ = totals()
    stt = g.status_read()
    assert stt["code"] == 0, stt
    assert bool(torch.isfinite(g.u[leaf][:, :10, 4:20, 4:20, 4:20]).all())
    # mass to round-off; momentum against the total momentum magnitude
    assert abs(t1[0] - t0[0]) <= 1e-12 * t0[0], (t0[0], t1[0])
    assert np.all(np.abs(t1[1:] - t0[1:]) <= 1e-12 * m0[1:]), (t0, t1, m0)
    assert divb() <= 1e-12
