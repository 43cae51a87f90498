"""Morton-ordered leaf lists, equal-work splits and the cross-rank dt
minimum (gloo, two ranks on CPU)."""
import os
import socket

import numpy as np
import pytest


def test_morton_order_is_a_space_filling_permutation():
    from torch_gb300 import amr, blocklist
    t, _ = amr.small_tree()
    order = blocklist.morton_order(t)
    assert sorted(order.tolist()) == sorted(t["leaf"].tolist())
    keys = blocklist.morton_keys(t, order)
    assert np.all(np.diff(keys.astype(np.float64)) > 0)  # distinct and increasing
    # the 8 children of a refined block are consecutive on the curve
    pos = {b: q for q, b in enumerate(order)}
    for n in range(len(t["level"])):
        ch = t["child"][n]
        if ch[0] >= 0 and all(t["child"][c][0] < 0 for c in ch):
            q = sorted(pos[c] for c in ch)
            assert q[-1] - q[0] == 7


def test_split_is_contiguous_and_balanced():
    from torch_gb300 import amr, blocklist
    t, _ = amr.config3_tree()
    order = blocklist.morton_order(t)
    for n in (1, 2, 3, 8):
        parts = blocklist.split_blocks(order, n)
        assert np.array_equal(np.concatenate(parts), order)
        sizes = [len(p) for p in parts]
        assert max(sizes) - min(sizes) <= 1
    w = np.where(np.asarray(t["level"])[order] == 3, 2.0, 1.0)
    parts = blocklist.split_blocks(order, 4, w)
    loads = [w[np.isin(order, p)].sum() for p in parts]
    assert max(loads) - min(loads) <= 2.0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    from oracle import oracle as O
    from torch_gb300 import amr, blocklist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t, c = amr.small_tree()
        st = amr.amr_box(t, c, seed=5, device="cpu")
        p = O.hydro_params(True)
        u = st["u"][:, :10].numpy().copy()
        mine = blocklist.split_blocks(blocklist.morton_order(t), world)[rank]
        lim = [O.dt_limit(p, u[b:b + 1], *(3 * [st["root_dx"] / 2 ** t["level"][b]])) for b in mine]
        q = int(np.argmin(lim))
        dt, owner, blk = blocklist.global_dt(0.8 * lim[q], int(mine[q]))
        slow = blocklist.max_over_ranks(float(rank + 1))
        out.put((rank, dt, owner, blk, slow))
    finally:
        dist.destroy_process_group()


def test_global_dt_two_ranks_gloo(oracle):
    import torch.multiprocessing as mp
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=5, device="cpu")
    p = oracle.hydro_params(True)
    u = st["u"][:, :10].numpy().copy()
    lim = {int(b): oracle.dt_limit(p, u[b:b + 1], *(3 * [st["root_dx"] / 2 ** t["level"][b]])) for b in t["leaf"]}
    ref_blk = min(lim, key=lim.get)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = [q.get(timeout=240) for _ in range(2)]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for rank, dt, owner, blk, slow in res:
        assert dt == 0.8 * lim[ref_blk]
        assert blk == ref_blk
        assert slow == 2.0
    assert len({r[2] for r in res}) == 1
