"""Failure detection without a GPU fault: the bounded mbarrier wait of the
tcgen05 and TMA kernels gives up after its cycle limit, records
GB_ST_TIMEOUT in the status the host reads, and leaves the context usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_that_completes_records_nothing(gb):
    r, st = gb.check_bounded_wait(2_000_000, arrive=True)
    assert r == 1
    assert st["code"] == 0 and not st["n_code"]


def test_wait_that_runs_out_records_a_timeout_and_the_context_survives(gb):
    import torch
    # a barrier nothing arrives on, about a millisecond of waiting
    r, st = gb.check_bounded_wait(2_000_000, arrive=False)
    assert r == 2
    assert st["code"] == 7 and st["n_code"] == {gb.ST_NAMES[7]: 1}
    # the context still runs work: the tcgen05 inference on a few cells
    gb.mlp_init(3)
    x = torch.randn(1000, 4, device="cuda")
    y = gb.mlp_infer(x).cpu().numpy()
    assert np.isfinite(y).all()
