"""The AMUSE-facing call surface over the device store."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _code(gb, cool=False):
    from torch_gb300 import amr
    from torch_gb300.amuse_flash import FlashCode
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=5, device="cuda")
    g = gb.grid_from_amr(t, st, mhd=True, cooling=False)
    gb.init_hydro(gb.hydro_params(True, precision=0))
    g.register()
    return g, FlashCode(g, cool=cool)


def test_grid_state_roundtrip(gb):
    g, f = _code(gb)
    rng = np.random.default_rng(0)
    n = 500
    blocks = rng.choice(np.asarray(g.leaf) + 1, n)
    i, j, k = (rng.integers(1, 17, n) for _ in range(3))
    p = np.zeros(n, int)
    rho, mx, my, mz, en, rc = f.get_grid_state(i, j, k, blocks, p)
    assert rc == 0
    u = g.u.cpu().numpy()
    ref = u[blocks - 1, 0, k + 3, j + 3, i + 3]
    assert np.array_equal(rho, ref)
    assert np.array_equal(mx, ref * u[blocks - 1, 1, k + 3, j + 3, i + 3])
    assert np.array_equal(en, ref * u[blocks - 1, 5, k + 3, j + 3, i + 3])
    # cells of another process stay zero
    r2 = f.get_grid_state(i[:3], j[:3], k[:3], blocks[:3], [1, 1, 1])
    assert not np.any(np.concatenate(r2[:5]))
    # set: unique cells, new values, then read back and check the EOS
    cells = np.unique(np.stack([blocks, k, j, i], 1), axis=0)
    b2, k2, j2, i2 = cells.T
    m = len(b2)
    assert f.set_grid_state(i2, j2, k2, b2, np.zeros(m, int), np.full(m, 2.0), np.full(m, 2.0),
                            np.zeros(m), np.zeros(m), np.full(m, 5.0)) == 0
    u = g.u.cpu().numpy()
    assert np.all(u[b2 - 1, 0, k2 + 3, j2 + 3, i2 + 3] == 2.0)
    assert np.all(u[b2 - 1, 1, k2 + 3, j2 + 3, i2 + 3] == 1.0)
    assert np.allclose(u[b2 - 1, 6, k2 + 3, j2 + 3, i2 + 3], 2.5 - 0.5)
    assert np.allclose(u[b2 - 1, 4, k2 + 3, j2 + 3, i2 + 3], (2.0 / 3.0) * 2.0 * 2.0)
    with pytest.raises(IndexError):
        f.get_grid_state([17], [1], [1], [1], [0])


def test_evolve_model_lands_on_the_end_time(gb):
    g, f = _code(gb)
    try:
        gb.set_dt_limits(0.0, float("inf"), 1.5)
        f.set_timestep(1e-5)
        dt0, _ = f.get_timestep()
        assert dt0 == 1e-5
        assert f.evolve_model(2.0e-5) == 0
        t, _ = f.get_time()
        assert t == 2.0e-5
        # first step limited by the change factor, second shortened to t_end
        d = g.driver.cpu().numpy()
        assert d[g.DRV_NSTEP] == 2
        assert d[g.DRV_DTOLD] == d[g.DRV_DT]
        assert abs(d[g.DRV_DT] - 0.5e-5) < 1e-18
        assert f.evolve_model(2.0e-5) == 0  # already there: no step
        assert g.driver.cpu().numpy()[g.DRV_NSTEP] == 2
    finally:
        gb.set_dt_limits()
