"""The batched step over an AMR block list against the oracle: guard
filling across levels, the FP64 step with per-level cell sizes, and the
mixed-precision path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(gb, mhd):
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=5, device="cuda")
    g = gb.grid_from_amr(t, st, mhd=mhd, cooling=False)
    return t, st, g


def _oracle_arrays(st, mhd):
    u = st["u"][:, :10].cpu().numpy().copy()
    f = [st[k].cpu().numpy().copy() for k in ("fx", "fy", "fz")] if mhd else [None] * 3
    return u, f


@pytest.mark.parametrize("mhd", [False, True])
def test_amr_guard_fill_matches_oracle(gb, oracle, mhd):
    t, st, g = _state(gb, mhd)
    gb.init_hydro(gb.hydro_params(mhd))
    g.fill_guardcells()
    u, (fx, fy, fz) = _oracle_arrays(st, mhd)
    p = oracle.hydro_params(mhd)
    oracle.fill_guards_tree(p, t, u, fx, fy, fz)
    nv = 10 if mhd else 7
    leaf = t["leaf"]
    assert np.array_equal(g.u.cpu().numpy()[leaf, :nv], u[leaf, :nv])
    if mhd:
        for a, b in ((g.fx, fx), (g.fy, fy), (g.fz, fz)):
            assert np.array_equal(a.cpu().numpy()[leaf], b[leaf])


@pytest.mark.parametrize("mhd", [False, True])
def test_amr_fp64_step_matches_oracle(gb, oracle, mhd):
    t, st, g = _state(gb, mhd)
    gb.init_hydro(gb.hydro_params(mhd))
    u, (fx, fy, fz) = _oracle_arrays(st, mhd)
    p = oracle.hydro_params(mhd)
    dx0 = st["root_dx"]
    oracle.fill_guards_tree(p, t, u, fx, fy, fz)
    dt = g.compute_dt().item()
    g.evolve_step(dt, cool=False)
    fsz = 24 * 24 * 25
    for b in t["leaf"]:
        dx = dx0 / 2 ** t["level"][b]
        ub = u[b:b + 1]
        fb = [None if f is None else f[b:b + 1] for f in (fx, fy, fz)]
        oracle.unsplit_blocks(p, ub, *fb, dt, dx, dx, dx)
        if mhd:
            fx[b], fy[b], fz[b] = fb[0][0], fb[1][0], fb[2][0]
        u[b] = ub[0]
    nv = 10 if mhd else 7
    leaf = t["leaf"]
    gu = g.u.cpu().numpy()[leaf, :nv, 4:20, 4:20, 4:20]
    ou = u[leaf, :nv, 4:20, 4:20, 4:20]
    assert np.max(np.abs(gu - ou) / (np.abs(ou) + 1e-300)) <= 1e-12


@pytest.mark.parametrize("mhd", [False, True])
def test_amr_mixed_precision_l1(gb, mhd):
    t, st, g64 = _state(gb, mhd)
    _, _, g32 = _state(gb, mhd)
    dts = []
    gb.init_hydro(gb.hydro_params(mhd, precision=0))
    g64.register()
    for _ in range(10):
        dt = g64.compute_dt().item()
        dts.append(dt)
        g64.evolve_step(dt, cool=False)
    gb.init_hydro(gb.hydro_params(mhd, precision=1))
    g32.register()
    for dt in dts:
        g32.evolve_step(dt, cool=False)
    leaf = t["leaf"]
    a = g64.u.cpu().numpy()[leaf][:, :, 4:20, 4:20, 4:20]
    b = g32.u.cpu().numpy()[leaf][:, :, 4:20, 4:20, 4:20]
    for v in (0, 4):
        assert np.abs(a[:, v] - b[:, v]).sum() / np.abs(a[:, v]).sum() <= 1e-4
