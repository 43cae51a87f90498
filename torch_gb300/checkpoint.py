"""Checkpoint and restart of the device block store.

FLASH writes its checkpoints through IO_writeCheckpoint.F90 (HDF5: unk,
facevar{x,y,z}, the tree, the driver's scalars) and restarts from them with
IO_readCheckpoint.F90; Torch's Python side adds its own pickles
(torch_state.py:91-160). HDF5 is not part of this build, and the device
store is a plain array of blocks, so a checkpoint here is one file:

    "GBCKPT01"  (8 bytes)
    header length H (8 bytes, little-endian)
    header (H bytes of UTF-8 JSON)
    arrays, each starting on a 4096-byte boundary

The header lists every array (name, dtype, shape, offset, bytes, CRC-32) and
the scalars: the grid's shape and variable slots, the root block size, the
device driver clock (sim_time, dt, dt_old, t_max, nstep), and optionally the
cooling surrogate's weights. The per-cell CFL codes of the hybrid-order
fallback are saved too, so a restarted run takes the same next dt, and
therefore the same states, as the uninterrupted run. Large arrays move
through a pinned staging buffer in slices, so the host never holds a second
copy of the whole store.
"""
from __future__ import annotations

import json
import os
import zlib

import numpy as np

from . import gbhydro as G

MAGIC = b"GBCKPT01"
VERSION = 1
ALIGN = 4096
SLICE = 256 << 20  # bytes per staged copy


class CheckpointError(RuntimeError):
    pass


def _pad(n: int) -> int:
    return (n + ALIGN - 1) // ALIGN * ALIGN


def _stage(nbytes: int):
    import torch
    s = torch.empty(max(1, min(nbytes, SLICE)), dtype=torch.uint8)
    return s.pin_memory() if torch.cuda.is_available() else s


def _sync():
    import torch
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def _write_tensor(f, t, staging) -> int:
    """Device or host tensor -> file, in slices; returns the CRC-32."""
    import torch
    flat = t.contiguous().view(-1).view(torch.uint8)
    crc = 0
    for a in range(0, flat.numel(), staging.numel()):
        b = min(a + staging.numel(), flat.numel())
        s = staging[: b - a]
        s.copy_(flat[a:b])
        if flat.is_cuda:
            _sync()
        mv = memoryview(s.numpy())
        crc = zlib.crc32(mv, crc)
        f.write(mv)
    return crc


def _read_tensor(f, t, nbytes: int, staging) -> int:
    """File -> device or host tensor, in slices; returns the CRC-32."""
    import torch
    flat = t.view(-1).view(torch.uint8)
    if flat.numel() != nbytes:
        raise CheckpointError(f"array holds {flat.numel()} bytes, the file {nbytes}")
    crc = 0
    for a in range(0, nbytes, staging.numel()):
        b = min(a + staging.numel(), nbytes)
        s = staging[: b - a]
        mv = memoryview(s.numpy())
        if f.readinto(mv) != b - a:
            raise CheckpointError("file ends inside an array")
        crc = zlib.crc32(mv, crc)
        flat[a:b].copy_(s)
        if flat.is_cuda:
            _sync()
    return crc


def _arrays(grid, with_codes: bool, weights):
    import torch
    out = [("unk", grid.u)]
    if grid.mhd:
        out += [("facex", grid.fx), ("facey", grid.fy), ("facez", grid.fz)]
    tr = grid.tree
    for k in ("level", "coord", "child", "root"):
        out.append(("tree_" + k, torch.as_tensor(np.ascontiguousarray(tr[k], np.int32))))
    if with_codes:
        n = grid.nblocks * 3 * (G.NB - 8) ** 3  # 16^3 interior cells, 3 directions
        codes = torch.empty(n, dtype=torch.uint8, device=grid.u.device)
        G.check(G.lib().gb_cfl_codes_save(G._ptr(codes), n, G._stream()), "gb_cfl_codes_save")
        out.append(("cfl_codes", codes))
    if weights is not None:
        out.append(("mlp_weights", torch.as_tensor(np.ascontiguousarray(weights, np.float32))))
    return out


def write_checkpoint(path: str, grid, *, cfl_codes: bool = True, surrogate: bool = False) -> dict:
    """Write grid (a registered gbhydro.Grid) with its driver clock to path.
    cfl_codes: also the per-cell CFL codes (the grid must be the registered
    one); surrogate: also the cooling surrogate's weights. Returns the
    header. The file is written beside path and renamed into place, so a
    crash leaves the previous checkpoint intact."""
    _sync()
    weights = G.mlp_weights() if surrogate else None
    arrays = _arrays(grid, cfl_codes, weights)
    drv = grid.driver.cpu().tolist()
    hdr = {
        "format": "gbhydro-checkpoint", "version": VERSION,
        "grid": {"nblocks": grid.nblocks, "nvar": grid.nvar, "mhd": bool(grid.mhd), "slots": grid.slots,
                 "root_dx": float(grid.root_dx), "nr": [int(x) for x in grid.tree["nr"]],
                 "maxlevel": int(grid.tree["maxlevel"])},
        "driver": dict(zip(("sim_time", "dt", "dt_old", "t_max", "nstep"), drv)),
        "arrays": [],
    }
    off = 0
    for name, t in arrays:
        nb = t.numel() * t.element_size()
        hdr["arrays"].append({"name": name, "dtype": str(t.dtype).replace("torch.", ""), "shape": list(t.shape),
                              "offset": off, "bytes": nb, "crc32": 0})
        off = _pad(off + nb)
    # the header's size does not depend on the CRCs' values: reserve it with
    # the widest CRC and rewrite it in place once the arrays are written
    for a in hdr["arrays"]:
        a["crc32"] = 0xFFFFFFFF
    blob = json.dumps(hdr, sort_keys=True).encode()
    base = _pad(16 + len(blob))
    tmp = path + ".partial"
    staging = _stage(max(a["bytes"] for a in hdr["arrays"]))
    with open(tmp, "wb") as f:
        f.write(b"\0" * base)
        for (name, t), a in zip(arrays, hdr["arrays"]):
            f.seek(base + a["offset"])
            a["crc32"] = _write_tensor(f, t, staging)
        f.truncate(base + off)
        blob2 = json.dumps(hdr, sort_keys=True).encode().ljust(len(blob))
        f.seek(0)
        f.write(MAGIC + len(blob2).to_bytes(8, "little") + blob2)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)
    return hdr


def read_header(path: str) -> tuple[dict, int]:
    """(header, byte offset of the array section)."""
    with open(path, "rb") as f:
        head = f.read(16)
        if len(head) != 16 or head[:8] != MAGIC:
            raise CheckpointError(f"{path}: not a gbhydro checkpoint")
        n = int.from_bytes(head[8:], "little")
        if n <= 0 or n > (64 << 20):
            raise CheckpointError(f"{path}: bad header length {n}")
        blob = f.read(n)
    if len(blob) != n:
        raise CheckpointError(f"{path}: truncated header")
    hdr = json.loads(blob.decode())
    if hdr.get("format") != "gbhydro-checkpoint" or hdr.get("version") != VERSION:
        raise CheckpointError(f"{path}: format {hdr.get('format')} version {hdr.get('version')}")
    return hdr, _pad(16 + n)


def read_checkpoint(path: str, device: str = "cuda", *, surrogate: bool = False):
    """Rebuild the Grid a checkpoint holds, register it, restore its driver
    clock and (when saved) its CFL codes; surrogate: also load the saved
    surrogate weights into the library. Every array's CRC-32 is checked."""
    import torch
    hdr, base = read_header(path)
    gh = hdr["grid"]
    arrays = {a["name"]: a for a in hdr["arrays"]}
    size = os.path.getsize(path)
    for a in hdr["arrays"]:
        if base + a["offset"] + a["bytes"] > size:
            raise CheckpointError(f"{path}: array {a['name']} runs past the end of the file")
    staging = _stage(max(a["bytes"] for a in hdr["arrays"]))

    def load(f, name, out):
        a = arrays[name]
        if list(out.shape) != a["shape"] or str(out.dtype).replace("torch.", "") != a["dtype"]:
            raise CheckpointError(f"{path}: {name} is {a['dtype']}{a['shape']}")
        f.seek(base + a["offset"])
        crc = _read_tensor(f, out, a["bytes"], staging)
        if crc != a["crc32"]:
            raise CheckpointError(f"{path}: CRC mismatch in {name}")
        return out

    with open(path, "rb") as f:
        tree = {"nr": tuple(gh["nr"]), "maxlevel": gh["maxlevel"]}
        for k in ("level", "coord", "child", "root"):
            a = arrays["tree_" + k]
            tree[k] = load(f, "tree_" + k, torch.empty(a["shape"], dtype=torch.int32)).numpy()
        g = G.Grid(gh["nblocks"], gh["nvar"], gh["slots"], gh["mhd"], tree, gh["root_dx"], device=device)
        load(f, "unk", g.u)
        if gh["mhd"]:
            for k, t in (("facex", g.fx), ("facey", g.fy), ("facez", g.fz)):
                load(f, k, t)
        if "cfl_codes" in arrays:
            codes = load(f, "cfl_codes", torch.empty(arrays["cfl_codes"]["shape"], dtype=torch.uint8,
                                                     device=device))
            G.check(G.lib().gb_cfl_codes_load(G._ptr(codes), codes.numel(), G._stream()), "gb_cfl_codes_load")
            _sync()
        if surrogate:
            if "mlp_weights" not in arrays:
                raise CheckpointError(f"{path}: no surrogate weights saved")
            w = load(f, "mlp_weights", torch.empty(arrays["mlp_weights"]["shape"], dtype=torch.float32))
            G.mlp_set_weights(w.numpy())
    d = hdr["driver"]
    g.driver.copy_(torch.tensor([d["sim_time"], d["dt"], d["dt_old"], d["t_max"], d["nstep"]],
                                dtype=torch.float64))
    return g


def load_arrays(path: str) -> tuple[dict, dict]:
    """(header, {name: numpy array}) of a checkpoint, read on the host with
    every CRC-32 checked: for inspection and for tools that post-process a
    run without a GPU."""
    import torch
    hdr, base = read_header(path)
    size = os.path.getsize(path)
    out = {}
    with open(path, "rb") as f:
        for a in hdr["arrays"]:
            if base + a["offset"] + a["bytes"] > size:
                raise CheckpointError(f"{path}: array {a['name']} runs past the end of the file")
            t = torch.empty(a["shape"], dtype=getattr(torch, a["dtype"]))
            f.seek(base + a["offset"])
            if _read_tensor(f, t, a["bytes"], _stage(a["bytes"])) != a["crc32"]:
                raise CheckpointError(f"{path}: CRC mismatch in {a['name']}")
            out[a["name"]] = t.numpy()
    return hdr, out
