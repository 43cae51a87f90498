"""Checkpoint file format on the host: arrays and scalars round-trip, and a
damaged file is refused (bad magic, a flipped byte, a truncated array)."""
import numpy as np
import pytest


class _FakeGrid:
    """The attributes write_checkpoint reads from a gbhydro.Grid, on the CPU."""

    def __init__(self, nblocks=3, mhd=True, seed=0):
        import torch
        rng = np.random.default_rng(seed)
        nb = 24
        self.nblocks, self.nvar, self.mhd = nblocks, 10, mhd
        self.u = torch.as_tensor(rng.standard_normal((nblocks, 10, nb, nb, nb)))
        self.fx = torch.as_tensor(rng.standard_normal((nblocks, nb, nb, nb + 1)))
        self.fy = torch.as_tensor(rng.standard_normal((nblocks, nb, nb + 1, nb)))
        self.fz = torch.as_tensor(rng.standard_normal((nblocks, nb + 1, nb, nb)))
        self.slots = {"DENS": 0, "VELX": 1, "VELY": 2, "VELZ": 3, "PRES": 4, "ENER": 5, "EINT": 6,
                      "MAGX": 7, "MAGY": 8, "MAGZ": 9}
        self.tree = {"level": np.zeros(nblocks, np.int32), "coord": np.arange(3 * nblocks, dtype=np.int32).reshape(-1, 3),
                     "child": -np.ones((nblocks, 8), np.int32), "root": np.arange(nblocks, dtype=np.int32),
                     "nr": (nblocks, 1, 1), "maxlevel": 0}
        self.root_dx = 0.125
        self.driver = torch.tensor([1.5, 0.01, 0.02, float("inf"), 7.0], dtype=torch.float64)


def test_round_trip(tmp_path, monkeypatch):
    from torch_gb300 import checkpoint as CK
    monkeypatch.setattr(CK, "SLICE", 1 << 16)  # many slices per array
    g = _FakeGrid()
    p = str(tmp_path / "chk")
    hdr = CK.write_checkpoint(p, g, cfl_codes=False)
    h2, arr = CK.load_arrays(p)
    assert h2 == hdr
    assert h2["driver"] == {"sim_time": 1.5, "dt": 0.01, "dt_old": 0.02, "t_max": float("inf"), "nstep": 7.0}
    assert h2["grid"]["slots"] == g.slots and h2["grid"]["nblocks"] == 3
    for name, t in (("unk", g.u), ("facex", g.fx), ("facey", g.fy), ("facez", g.fz)):
        assert np.array_equal(arr[name], t.numpy()), name
    for k in ("level", "coord", "child", "root"):
        assert np.array_equal(arr["tree_" + k], g.tree[k])
    base = CK.read_header(p)[1]
    assert base % CK.ALIGN == 0 and all(a["offset"] % CK.ALIGN == 0 for a in hdr["arrays"])
    assert not (tmp_path / "chk.partial").exists()


def test_damaged_files_are_refused(tmp_path):
    from torch_gb300 import checkpoint as CK
    g = _FakeGrid(nblocks=2, mhd=False)
    p = tmp_path / "chk"
    hdr = CK.write_checkpoint(str(p), g, cfl_codes=False)
    good = p.read_bytes()
    base = CK.read_header(str(p))[1]
    unk = next(a for a in hdr["arrays"] if a["name"] == "unk")
    bad = bytearray(good)
    bad[base + unk["offset"] + 12345] ^= 0x10
    p.write_bytes(bytes(bad))
    with pytest.raises(CK.CheckpointError, match="CRC"):
        CK.load_arrays(str(p))
    p.write_bytes(good[: base + unk["offset"] + 1000])
    with pytest.raises(CK.CheckpointError):
        CK.load_arrays(str(p))
    p.write_bytes(b"NOTACKPT" + good[8:])
    with pytest.raises(CK.CheckpointError, match="not a gbhydro checkpoint"):
        CK.load_arrays(str(p))
    p.write_bytes(good)
    CK.load_arrays(str(p))
