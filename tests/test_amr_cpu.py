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
