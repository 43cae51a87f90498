"""The CUDA unsplit hydro / MHD step against the CPU oracle, plus the
size-independent properties (conservation, div B, guard fill)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(gb, oracle, mhd, nb=2, seed=43, mach=2.0, sig=0.5, precision=0, **over):
    from torch_gb300 import workloads as W
    ic = W.turbulent_box(nb, nb, nb, seed=seed, sigma_ln=sig, mach=mach, mhd=mhd, nvar=10)
    g = gb.grid_from_workload(ic, mhd=mhd, cooling=False)
    gb.init_hydro(gb.hydro_params(mhd, precision=precision, **over))
    p = oracle.hydro_params(mhd, **over)
    return ic, g, p


def _oracle_arrays(ic):
    return ic["u"].copy(), *(None if ic[k] is None else ic[k].copy() for k in ("fx", "fy", "fz"))


def _interior(a):
    return a[..., 4:20, 4:20, 4:20]


@pytest.mark.parametrize("mhd", [False, True])
def test_guard_fill_matches_oracle(gb, oracle, mhd):
    ic, g, p = _setup(gb, oracle, mhd)
    g.fill_guardcells()
    u, fx, fy, fz = _oracle_arrays(ic)
    oracle.fill_guards_periodic(p, 2, 2, 2, u, fx, fy, fz)
    nv = 10 if mhd else 7
    assert np.array_equal(g.u.cpu().numpy()[:, :nv], u[:, :nv])
    if mhd:
        assert np.array_equal(g.fx.cpu().numpy(), fx)
        assert np.array_equal(g.fy.cpu().numpy(), fy)
        assert np.array_equal(g.fz.cpu().numpy(), fz)


@pytest.mark.parametrize("mhd", [False, True])
def test_fp64_step_matches_oracle(gb, oracle, mhd):
    """Plain FP64 on the 2x2x2-block box (the hydro case is the reference's
    first configuration: sigma_ln 0.5, Mach 2, 10 steps at CFL 0.8): every
    step equals the oracle to 1e-12 relative per cell, and the device's CFL
    limit is the oracle's bit for bit."""
    ic, g, p = _setup(gb, oracle, mhd)
    p.keep_cfl_codes(8)
    u, fx, fy, fz = _oracle_arrays(ic)
    dx = ic["dx"]
    nv = 10 if mhd else 7
    for step in range(10):
        oracle.fill_guards_periodic(p, 2, 2, 2, u, fx, fy, fz)
        dt = 0.8 * oracle.dt_limit(p, u, dx, dx, dx)
        assert g.compute_dt().item() == dt, step
        g.status_reset()
        g.evolve_step(dt, cool=False)
        oracle.unsplit_blocks(p, u, fx, fy, fz, dt, dx, dx, dx)
        gu = g.u.cpu().numpy()
        rel = np.abs(_interior(gu[:, :nv]) - _interior(u[:, :nv])) / (np.abs(_interior(u[:, :nv])) + 1e-300)
        scale = np.abs(_interior(u[:, :nv])).max(axis=(0, 2, 3, 4), keepdims=True)
        absd = np.abs(_interior(gu[:, :nv]) - _interior(u[:, :nv])) / scale
        assert np.all((rel <= 1e-12) | (absd <= 1e-14)), (step, rel.max(), absd.max())
        if mhd:
            for a, b in ((g.fx, fx), (g.fy, fy), (g.fz, fz)):
                d = np.abs(a.cpu().numpy()[:, 4:20, 4:20, 4:20] - b[:, 4:20, 4:20, 4:20])
                assert d.max() <= 1e-12 * np.abs(b).max()
        assert g.status_read()["code"] in (0,)


def test_cfl_dt_matches_oracle(gb, oracle):
    ic, g, p = _setup(gb, oracle, True)
    u, fx, fy, fz = _oracle_arrays(ic)
    dx = ic["dx"]
    dt_o = 0.8 * oracle.dt_limit(p, u, dx, dx, dx)
    assert g.compute_dt().item() == dt_o


@pytest.mark.parametrize("mhd,precision", [(False, 0), (True, 0), (False, 1), (True, 1)])
def test_conservation_and_divb(gb, oracle, mhd, precision):
    """Periodic box: mass, momentum, energy at round-off (Mach 1, no
    dual-energy switching) and div B at round-off after 5 steps, in FP64
    and in the mixed path (FP32 fluxes summed in double-float, one FP64
    scaling per cell). energyFix off: the strictly conservative form (with
    it, the reference's setting, the magnetic energy of the staggered field
    replaces the flux-updated one, which E does not conserve)."""
    ic, g, p = _setup(gb, oracle, mhd, seed=5, mach=1.0, sig=0.3, precision=precision, energy_fix=0)
    dx = ic["dx"]

    def totals():
        u = g.u.cpu().numpy()
        if mhd:
            return oracle.totals(p, np.ascontiguousarray(u), g.fx.cpu().numpy(), g.fy.cpu().numpy(),
                                 g.fz.cpu().numpy(), dx, dx, dx)
        uu = np.zeros((u.shape[0], 10) + u.shape[2:])
        uu[:, :7] = u
        return oracle.totals(p, uu, None, None, None, dx, dx, dx)
    t0 = totals()
    for _ in range(5):
        dt = g.compute_dt().item()
        g.status_reset()
        g.evolve_step(dt, cool=False)
        st = g.status_read()
        assert st["n_eint_switch"] == 0 and st["code"] == 0
    t1 = totals()
    scale = np.sqrt(t0[0] * t0[4])
    assert abs(t1[0] - t0[0]) < 1e-13 * t0[0]
    assert np.all(np.abs(t1[1:4] - t0[1:4]) < 1e-13 * scale)
    assert abs(t1[4] - t0[4]) < 1e-13 * t0[4]
    if mhd:
        assert t1[5] < 1e-12


@pytest.mark.parametrize("mhd", [False, True])
def test_mixed_precision_l1(gb, oracle, mhd):
    """FP32 reconstruction/Riemann + FP64 update against the all-FP64 path:
    density and pressure L1 relative error <= 1e-4 after 10 steps (same dt
    sequence)."""
    import torch
    from torch_gb300 import workloads as W
    ic = W.turbulent_box(2, 2, 2, seed=44, sigma_ln=1.0 if mhd else 0.5, mach=5.0 if mhd else 2.0,
                         mhd=mhd, nvar=10)
    g64 = gb.grid_from_workload(ic, mhd=mhd, cooling=False)
    g32 = gb.grid_from_workload(ic, mhd=mhd, cooling=False)
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
    torch.cuda.synchronize()
    a, b = g64.u.cpu().numpy(), g32.u.cpu().numpy()
    for v in (0, 4):
        l1 = np.abs(_interior(a[:, v]) - _interior(b[:, v])).sum() / np.abs(_interior(a[:, v])).sum()
        assert l1 <= 1e-4, (v, l1)


def test_integer_pipe_conversions_match_hardware(gb):
    """The mixed path's FP64 <-> FP32 conversions done with integer
    instructions equal the hardware conversions bit for bit: random bit
    patterns (all exponents, signs, ties), values of the workload's range,
    zeros, subnormals, the float range edges, inf and nan."""
    import torch
    rng = np.random.default_rng(0)
    n = 1 << 22
    d = rng.integers(0, 2 ** 63, n, dtype=np.int64).view(np.float64).copy()
    d[: n // 4] = rng.normal(0, 1, n // 4) * 10.0 ** rng.uniform(-40, 40, n // 4)
    # exact ties of the 29 dropped bits (round half to even)
    t = rng.integers(0, 2 ** 62, 4096, dtype=np.int64)
    d[n // 4:n // 4 + 4096] = ((t & ~np.int64((1 << 29) - 1)) | (1 << 28)).view(np.float64)
    edge = np.array([0.0, -0.0, 5e-324, -5e-324, 1e-45, 1.4e-45, 1.17549435e-38, 1.1754942e-38, 3.4028234e38,
                     3.4028235e38, 3.40282357e38, 1e39, -1e39, np.inf, -np.inf, np.nan, 1.0, -1.0])
    d[-len(edge):] = edge
    f = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32).view(np.float32).copy()
    with np.errstate(over="ignore"):
        f[: len(edge)] = edge.astype(np.float32)
    dd, fd = torch.as_tensor(d, device="cuda"), torch.as_tensor(f, device="cuda")
    bad = torch.zeros(2, dtype=torch.int64, device="cuda")
    gb.check(gb.lib().gb_selfcheck_conversions(n, dd.data_ptr(), fd.data_ptr(), bad.data_ptr(), None), "conv")
    torch.cuda.synchronize()
    assert bad.tolist() == [0, 0]
