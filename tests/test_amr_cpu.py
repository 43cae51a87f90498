"""Block trees and the oracle's guard fill across refinement levels (CPU)."""
import numpy as np


def test_config3_tree_counts_and_balance():
    from torch_gb300 import amr
    t, _ = amr.config3_tree()
    assert amr.leaf_counts(t) == [2057, 1020, 768, 256]
    assert len(t["leaf"]) * 4096 == 4101 * 4096  # 16.8 M zones, 256^3-equivalent
    assert amr.check_balance(t) == 0


def test_oracle_tree_fill_copies_injects_restricts(oracle):
    """Uniform fields stay uniform; a field linear in position is restored
    exactly in guard cells filled by restriction (mean of 8 fine cells) or
    same-level copy."""
    from torch_gb300 import amr
    t, _ = amr.small_tree()
    nn = len(t["level"])
    p = oracle.hydro_params(False)
    u = np.zeros((nn, 10, 24, 24, 24))
    u[:, 0] = 2.5
    oracle.fill_guards_tree(p, t, u)
    for b in t["leaf"]:
        assert np.all(u[b, 0] == 2.5)
    # linear field along x (cell centres in finest-cell units), away from the
    # periodic seam
    ml = t["maxlevel"]
    for b in t["leaf"]:
        s = 2 ** (ml - t["level"][b])
        x = (t["coord"][b][0] * 16 + np.arange(24) - 4 + 0.5) * s
        u[b, 1] = x[None, None, :]
    oracle.fill_guards_tree(p, t, u)
    N = 4 * 16 * 2 ** ml
    for b in t["leaf"]:
        s = 2 ** (ml - t["level"][b])
        x = (t["coord"][b][0] * 16 + np.arange(24) - 4 + 0.5) * s
        ok = (x > s) & (x < N - s)
        for i in np.nonzero(ok)[0]:
            col = u[b, 1, :, :, i]
            # every guard value is within one coarse cell of the exact value
            assert np.all(np.abs(col - x[i]) <= 2 * s)


def test_oracle_leaf_list_drivers_match_serial(oracle):
    """The OpenMP leaf-list drivers (the CPU baseline's step) give the
    serial per-leaf fill and step bit for bit."""
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=5, device="cpu")
    p = oracle.hydro_params(True)
    arrs = [st["u"][:, :10].numpy().copy()] + [st[k].numpy().copy() for k in ("fx", "fy", "fz")]
    u1, x1, y1, z1 = [a.copy() for a in arrs]
    u2, x2, y2, z2 = [a.copy() for a in arrs]
    leaves = t["leaf"][::3]
    oracle.fill_guards_tree(p, t, u1, x1, y1, z1)
    dt = 0.8 * min(oracle.dt_limit(p, u1[b:b + 1], *(3 * [st["root_dx"] / 2 ** t["level"][b]]))
                   for b in leaves)
    for b in leaves:
        dx = st["root_dx"] / 2 ** t["level"][b]
        oracle.unsplit_blocks(p, u1[b:b + 1], x1[b:b + 1], y1[b:b + 1], z1[b:b + 1], dt, dx, dx, dx)
    tl = oracle.TreeLists(t)
    oracle.fill_guards_list(p, tl, t["leaf"], u2, x2, y2, z2)
    dt2 = 0.8 * oracle.dt_limit_list(p, tl, leaves, u2, st["root_dx"])
    assert dt2 == dt
    oracle.unsplit_list(p, tl, leaves, u2, x2, y2, z2, dt, st["root_dx"])
    for a, b in zip((u1, x1, y1, z1), (u2, x2, y2, z2)):
        assert np.array_equal(a[leaves], b[leaves])
