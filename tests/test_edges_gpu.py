"""Block-list edge cases on the GPU: the empty list, any order of the
leaves, a ragged subset of them against the oracle, and ids that the host
rejects before any launch (FLASH's Hydro takes whatever leaf list its
caller holds: hy_uhd_interface.F90:472-479)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(gb, mhd, precision=0):
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=5, device="cuda")
    g = gb.grid_from_amr(t, st, mhd=mhd, cooling=False)
    gb.init_hydro(gb.hydro_params(mhd, precision=precision))
    gb.use_grid(g)
    return t, st, g


def _arrays(g):
    return [g.u] + ([g.fx, g.fy, g.fz] if g.mhd else [])


def _snapshot(g):
    return [a.clone() for a in _arrays(g)]


def _restore(g, snap):
    for a, b in zip(_arrays(g), snap):
        a.copy_(b)


def test_empty_block_list_is_a_no_op(gb):
    import torch
    t, st, g = _grid(gb, True)
    snap = _snapshot(g)
    gb.Hydro(0, [], 0.0, 1e-3, 1e-3)
    g.fill_guardcells([])
    torch.cuda.synchronize()
    assert all(torch.equal(a, b) for a, b in zip(_arrays(g), snap))
    # a rank without leaf blocks keeps the limit's start value
    assert gb.Driver_computeDt(0, []) == np.finfo(np.float64).max


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("mhd", [False, True])
def test_leaf_order_does_not_change_results(gb, mhd, precision):
    """The same step over the leaves in tree order and in a shuffled order,
    flux and edge-field matching on: the whole store (guards included) and
    the face fields bit-identical."""
    import torch
    t, st, g = _grid(gb, mhd, precision)
    snap = _snapshot(g)
    leaf = np.asarray(t["leaf"]) + 1
    dt = g.compute_dt().item()
    g.evolve_step(dt, cool=False, blockList=leaf)
    ref = _snapshot(g)
    _restore(g, snap)
    g.evolve_step(dt, cool=False, blockList=np.random.default_rng(11).permutation(leaf))
    torch.cuda.synchronize()
    assert all(torch.equal(a, b) for a, b in zip(_arrays(g), ref))


@pytest.mark.parametrize("mhd", [False, True])
def test_ragged_subset_matches_oracle(gb, oracle, mhd):
    """One FP64 step over every other leaf (all levels, shuffled), no
    fine-coarse matching (it pairs blocks of one call): the listed interiors
    match the oracle on the same list, the others do not change."""
    import torch
    t, st, g = _grid(gb, mhd)
    gb.set_flux_correction(False)
    try:
        u0 = g.u.cpu().numpy().copy()
        f0 = [a.cpu().numpy().copy() for a in (g.fx, g.fy, g.fz)] if mhd else [None] * 3
        leaf = np.asarray(t["leaf"])
        sub = np.random.default_rng(3).permutation(leaf[::2])
        rest = np.setdiff1d(leaf, sub)
        dt = g.compute_dt().item()
        g.evolve_step(dt, cool=False, blockList=sub + 1)
        torch.cuda.synchronize()
    finally:
        gb.set_flux_correction(True)
    p = oracle.hydro_params(mhd)
    u = st["u"][:, :10].cpu().numpy().copy()
    f = [st[k].cpu().numpy().copy() for k in ("fx", "fy", "fz")] if mhd else [None] * 3
    oracle.fill_guards_tree(p, t, u, *f)
    oracle.unsplit_tree(p, oracle.TreeLists(t), sub, u, *f, dt, st["root_dx"], flux_correct=False)
    nv = 10 if mhd else 7
    gu = g.u.cpu().numpy()
    I = (slice(None), slice(0, nv), slice(4, 20), slice(4, 20), slice(4, 20))
    ou, gs = u[sub][I], gu[sub][I]
    assert np.max(np.abs(gs - ou) / (np.abs(ou) + 1e-300)) <= 1e-12
    assert np.array_equal(gu[rest][I], u0[rest][I])
    if mhd:
        for a, b in zip((g.fx, g.fy, g.fz), f0):
            assert np.array_equal(a.cpu().numpy()[rest], b[rest])


def test_bad_block_ids_are_rejected_before_launch(gb):
    """Ids outside the store, of refined blocks, or repeated: GBError on the
    host, the state untouched."""
    import torch
    t, st, g = _grid(gb, True)
    snap = _snapshot(g)
    leaf = np.asarray(t["leaf"]) + 1
    parent = int(np.nonzero(np.asarray(t["child"])[:, 0] >= 0)[0][0]) + 1
    for bad in ([g.nblocks + 1], [0], [parent], [leaf[0], leaf[1], leaf[0]]):
        with pytest.raises(gb.GBError):
            gb.Hydro(len(bad), bad, 0.0, 1e-3, 1e-3)
        with pytest.raises(gb.GBError):
            g.evolve_step(1e-3, cool=False, blockList=bad)
    torch.cuda.synchronize()
    assert all(torch.equal(a, b) for a, b in zip(_arrays(g), snap))
