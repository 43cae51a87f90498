"""Autotuner for the launch shapes of the step.

Times the whole step (the replayed CUDA graph of gb_step_graph) for each
candidate (blocks per chunk, reconstruction tile, in the mixed path the
reconstruction's occupancy bound, the number of streams the chunks
alternate between, and reconstruction and Riemann solve fused per block or
not) on the registered grid,
restoring the grid's state after every trial so tuning does not advance the
simulation, and keeps the fastest. Results are cached per device, block
count, physics and precision in a JSON file beside this module (or the path
in GBHYDRO_TUNE_CACHE).
"""
from __future__ import annotations

import json
import os

CHUNKS = (32, 64, 128, 256, 512, 1024)
TILES = (32, 64)
OCCS = (0, 1, 2)
STREAMS = (1, 2)
FUSED = (0, 1, 2)
CACHE = os.environ.get("GBHYDRO_TUNE_CACHE",
                       os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tune_cache.json"))


def _key(grid, cool: bool) -> str:
    import torch
    from . import gbhydro as G
    st = G.state
    return (f"{torch.cuda.get_device_name()}|leaves={len(grid.leaf)}|mhd={int(grid.mhd)}|"
            f"precision={st['precision']}|cool={int(cool)}|surrogate={int(st['surrogate'])}")


def _load() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d: dict) -> None:
    tmp = CACHE + ".tmp"
    try:
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, CACHE)
    except OSError:
        pass


def time_config(grid, cool: bool, chunk: int, tile: int, steps: int = 3, warmup: int = 1, occ: int = 0,
                streams: int = 1, step_fn=None, fused: int = 0) -> float:
    """ms per step of the graph-replayed step at one launch shape (step_fn:
    the step to time, grid.step_graph(cool) by default)."""
    import torch
    from . import gbhydro as G
    G.set_launch_config(chunk, tile, occ)
    G.set_chunk_streams(streams)
    G.set_fused(int(fused))
    step = step_fn or (lambda: grid.step_graph(cool))
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        step()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(steps):
        step()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def tune(grid, cool: bool = True, chunks=CHUNKS, tiles=TILES, occs=OCCS, steps: int = 3,
         use_cache: bool = True, streams=STREAMS, step_fn=None, restore_fn=None, variant: str = "",
         fused=FUSED) -> dict:
    """Pick and set the fastest (chunk, tile, occ, streams) for `grid`
    (registered, with hydro/cooling configured; the occupancy bound only
    exists in the mixed path). step_fn replaces the timed step (for example
    the host-resident step) and restore_fn runs after each trial's device
    state is restored (for example to restore host arrays); variant names
    that choice in the cache key. Returns {"chunk", "tile", "occ",
    "streams", "fused", "ms", "trials", "cached"}. The fused kernel has no
    tile or occupancy choice: it is tried once per chunk size and stream
    count."""
    import torch
    from . import gbhydro as G
    key = _key(grid, cool) + (f"|{variant}" if variant else "")
    cache = _load() if use_cache else {}
    if key in cache:
        r = dict(cache[key], cached=True)
        G.set_launch_config(r["chunk"], r["tile"], r.get("occ", 0))
        G.set_chunk_streams(r.get("streams", 1))
        G.set_fused(int(r.get("fused", 0)))
        return r
    if G.state["precision"] != 1:
        occs = (0,)
    saved = [grid.u.clone()] + ([a.clone() for a in (grid.fx, grid.fy, grid.fz)] if grid.mhd else [])
    trials = []
    shapes = [(c, t, o, ns, 0) for c in chunks for t in tiles for o in occs for ns in streams if 0 in fused]
    for fu in (1, 2):
        # mode 2 differs from 1 only in the mixed path
        if fu in fused and (fu == 1 or G.state["precision"] == 1):
            shapes += [(c, tiles[0], 0, ns, fu) for c in chunks for ns in streams]
    try:
        for c, t, o, ns, fu in shapes:
            ms = time_config(grid, cool, c, t, steps=steps, occ=o, streams=ns, step_fn=step_fn, fused=fu)
            trials.append({"chunk": c, "tile": t, "occ": o, "streams": ns, "fused": fu, "ms": ms})
            grid.u.copy_(saved[0])
            if grid.mhd:
                for a, b in zip((grid.fx, grid.fy, grid.fz), saved[1:]):
                    a.copy_(b)
            G.lib().gb_cfl_codes_reset(None)
            if restore_fn:
                restore_fn()
    finally:
        del saved
        torch.cuda.synchronize()
    best = min(trials, key=lambda r: r["ms"])
    G.set_launch_config(best["chunk"], best["tile"], best["occ"])
    G.set_chunk_streams(best["streams"])
    G.set_fused(int(best["fused"]))
    r = {"chunk": best["chunk"], "tile": best["tile"], "occ": best["occ"], "streams": best["streams"],
         "fused": best["fused"], "ms": best["ms"], "trials": trials}
    if use_cache:
        cache[key] = r
        _save(cache)
    return dict(r, cached=False)
