"""Benchmark: zone-updates/s of the hydro/MHD + cooling step on one GB300.

A step is one pass of the hot path over the whole block list: CFL time step
(device min-reduction), guard-cell fill, unsplit MHD update, heating/cooling
source term. Two paths run on the same seeded input:
  plain : all-FP64 reconstruction/Riemann/update + the plain implicit
          cooling integrator
  fast  : FP32 reconstruction/Riemann, FP64 update/CT/energy recovery,
          learned cooling surrogate (tensor-core MLP guess + secant-Newton
          on the backward-Euler residual, plain integrator as fallback)
`value` is the fast path's device throughput; `plain_fp64` the plain one;
`e2e` is the fast path through the C ABI with host FLASH-layout buffers
copied in and out every step.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # 4101 leaf blocks over levels 0-3 (2057 / 1020 / 768 / 256) of a 13^3-root
    # periodic tree refined around 8 seeded Gaussian overdensities (contrast
    # 100, FWHM 4 finest cells): 16.8 M zones, 256^3-equivalent
    "amr": dict(name="amr_mhd_4101_leaf_blocks_cooling", kind="amr", tree_seed=45, ic_seed=46, sigma_ln=1.0,
                mach=5.0, beta=1.0, dA=0.1, contrast=100.0, fwhm_cells=4.0, cpu_stride=4),
    # 16381 leaf blocks over levels 0-4 of a 16^3-root tree (67.1 M zones):
    # the full-scale case, timed on the plain and fast paths only
    "amr16k": dict(name="amr_mhd_16381_leaf_blocks_5_levels_cooling", kind="amr5", tree_seed=47, ic_seed=48,
                   sigma_ln=1.0, mach=5.0, beta=1.0, dA=0.1, contrast=100.0, fwhm_cells=4.0, cpu_stride=16,
                   lite=True),
    # 8^3 blocks = 128^3 uniform periodic box
    "box128": dict(name="mhd_turbbox_128cubed_cooling", kind="box", nbx=8, nby=8, nbz=8, seed=44, sigma_ln=1.0,
                   mach=5.0, beta=1.0, dA=0.1, cpu_stride=1),
}
TDUST0 = 18.0  # initial dust temperature [K] (sim_tdust, flash.par.turbsph_standard:19)

# DRAM bytes (read + write) per interior zone of each profiler category of
# the fast path, from one-kernel ncu captures of the 128^3 box (one
# 512-block launch per kernel): "recon" = FP32 copy + velocity divergence +
# reconstruction, "emf" = time-n edge fields + edge fields, "guard_fill" =
# cells + faces. The roofline's traffic is this times the zones one launch
# covers.
TRAFFIC_B_PER_ZONE = {"recon": 764.0, "update": 398.0, "flux": 484.0, "guard_fill": 305.0, "mlp_infer": 16.0,
                      "sur_accept": 111.0, "emf": 151.0, "faceb": 81.0, "dt": 101.0}


def build_workload(wl, device):
    """(tree, state) of a workload: state = dict(u, fx, fy, fz, root_dx) with
    u[nnodes, 10, 24, 24, 24] (hydro + cell B) and face B, torch FP64."""
    import torch
    from torch_gb300 import amr
    from torch_gb300 import gbhydro as G
    from torch_gb300 import workloads as W
    if wl["kind"] in ("amr", "amr5"):
        tree, centres = (amr.config3_tree if wl["kind"] == "amr" else amr.config5_tree)(wl["tree_seed"])
        st = amr.amr_box(tree, centres, seed=wl["ic_seed"], sigma_ln=wl["sigma_ln"], mach=wl["mach"],
                         beta=wl["beta"], dA=wl["dA"], contrast=wl["contrast"], fwhm_cells=wl["fwhm_cells"],
                         nvar=10, device=device)
        return tree, st
    ic = W.turbulent_box(wl["nbx"], wl["nby"], wl["nbz"], seed=wl["seed"], sigma_ln=wl["sigma_ln"],
                         mach=wl["mach"], mhd=True, beta=wl["beta"], dA=wl["dA"], nvar=10)
    tree = G.uniform_tree(wl["nbx"], wl["nby"], wl["nbz"])
    st = {k: torch.as_tensor(ic[k], device=device) for k in ("u", "fx", "fy", "fz")}
    st["root_dx"] = ic["dx"]
    return tree, st


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def clocks_csv_path(args):
    """Where the sampled clocks go: --clocks-csv, else a file in the system's
    temporary directory (the JSON line carries their summary either way)."""
    import tempfile
    path = args.clocks_csv or os.path.join(tempfile.gettempdir(), "gbhydro_bench_clocks.csv")
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    return path


def current_gpu_id() -> str:
    """nvidia-smi's id of the GPU this process computes on: its PCI bus id
    (nvidia-smi ignores CUDA_VISIBLE_DEVICES, so an index would name
    another GPU of the machine), or "0" when torch cannot say."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(torch.cuda.current_device())
        return f"{pr.pci_domain_id:08x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
    except Exception:
        return "0"


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", current_gpu_id()], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path) if l.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def make_grid(G, tree, st, cooling=True):
    g = G.grid_from_amr(tree, st, mhd=True, cooling=cooling)
    units = G.code_units()
    gm1 = 2.0 / 3.0
    if cooling:
        e = g.u[:, g.slots["EINT"]]
        g.u[:, g.slots["TEMP"]] = e * units["vel_unit"] ** 2 * gm1 * (24.0 / 11.0) * G.MP / G.KB
        g.u[:, g.slots["TDUS"]] = TDUST0
    return g


def run_path(G, g, precision, steps, warmup, cool=True, surrogate=False, profile=False, ncu_range=False,
             graph=False, tune=False, tune_kw=None, cool_mode=None):
    """Time `steps` steps of one path after `warmup` untimed ones. Eager: dt
    read back by the host each step, then the step's launches; graph: the
    whole step (dt on the device) replayed as one CUDA graph. cool_mode
    overrides the cooling mode surrogate implies (2: the plain integrator
    on FP32 rates)."""
    import torch
    G.init_hydro(G.hydro_params(True, precision=precision))
    G.set_cooling_mode(surrogate if cool_mode is None else cool_mode)
    g.register()
    s = torch.cuda.current_stream()
    tuned = None
    if tune:
        from torch_gb300 import autotune
        tuned = autotune.tune(g, cool=cool, **(tune_kw or {}))

    def step():
        if graph:
            g.step_graph(cool)
        else:
            dt = g.compute_dt().item()
            g.evolve_step(dt, cool=cool)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    g.status_reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if profile:
        G.prof_enable(True)
    if ncu_range:
        torch.cuda.cudart().cudaProfilerStart()
    e0.record(s)
    for _ in range(steps):
        step()
    e1.record(s)
    torch.cuda.synchronize()
    if ncu_range:
        torch.cuda.cudart().cudaProfilerStop()
    prof = G.prof_read() if profile else None
    G.prof_enable(False)
    G.set_cooling_mode(False)
    if graph:
        prof = {"graph_kernels_per_step": G.graph_info()[2], "tuned": tuned}
    return e0.elapsed_time(e1) / steps, g.status_read(), prof


class CpuStep:
    """The oracle (C restatement of the reference's algorithm, OpenMP over
    leaf blocks, all host cores) on a fixed sample of the workload's leaves:
    one step = guard fill of the sampled leaves, CFL limit over them, one
    unsplit MHD step of each (cell size per level), implicit heating/cooling
    of their interior cells."""

    def __init__(self, wl, tree, st):
        from oracle import oracle as O
        from torch_gb300 import gbhydro as G
        from torch_gb300 import tables
        O.build()
        self.O, self.G = O, G
        self.p = O.hydro_params(True)
        self.tl = O.TreeLists(tree)
        self.sample = np.ascontiguousarray(tree["leaf"][::wl["cpu_stride"]], np.int32)
        self.u = np.ascontiguousarray(st["u"][:, :10].cpu().numpy())
        self.f = [np.ascontiguousarray(st[k].cpu().numpy()) for k in ("fx", "fy", "fz")]
        self.root_dx = st["root_dx"]
        self.units = G.code_units()
        self.cp = O.cool_params()
        self.tab = O.table_from_ilog(*tables.read_compact())
        self.cores = int(O.lib().orc_num_threads())
        self.zones = len(self.sample) * 4096
        self.desc = (f"{len(self.sample)} of {len(tree['leaf'])} leaf blocks (every {wl['cpu_stride']}th leaf, "
                     f"all levels) of the {wl['name']} workload")

    def step(self):
        O, G, u, (fx, fy, fz) = self.O, self.G, self.u, self.f
        sl = (self.sample[:, None, None, None], slice(4, 20), slice(4, 20), slice(4, 20))
        t0 = time.perf_counter()
        O.fill_guards_list(self.p, self.tl, self.sample, u, fx, fy, fz)
        dt = 0.8 * O.dt_limit_list(self.p, self.tl, self.sample, u, self.root_dx)
        O.unsplit_list(self.p, self.tl, self.sample, u, fx, fy, fz, dt, self.root_dx)
        rho = np.ascontiguousarray(u[:, 0][sl] * self.units["dens_unit"]).ravel()
        ei = np.ascontiguousarray(u[:, 6][sl] * self.units["vel_unit"] ** 2).ravel()
        T = ei * (2.0 / 3.0) * (24.0 / 11.0) * G.MP / G.KB
        td = np.full_like(T, TDUST0)
        O.radheat_cells(self.cp, self.tab, dt * self.units["time_unit"], rho, ei.copy(), ei, T, td)
        return time.perf_counter() - t0


def cpu_baseline(cs: CpuStep, steps=1):
    el = sum(cs.step() for _ in range(steps))
    return {"value": cs.zones * steps / el, "unit": "zone-updates/s", "cores": cs.cores, "kind": "port",
            "sample": f"{steps} step(s) of {cs.desc} on the oracle (C port, OpenMP over blocks), {el:.2f} s"}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]
    tree, st = build_workload(wl, "cpu")
    cs = CpuStep(wl, tree, st)
    del st
    for _ in range(args.warmup):
        cs.step()
    times = [cs.step() for _ in range(max(1, args.steps))]
    v = cs.zones * len(times) / sum(times)
    line = {"metric": "zone-updates/s", "value": v, "unit": "zone-updates/s", "n_gpus": args.gpus,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "impl": "reference", "dtype": "f64", "data": "synthetic",
            "scaling": "weak", "vs_baseline": None,
            "config": {"workload": wl["name"], "sampled_blocks": len(cs.sample), "block": "16^3+4gc"},
            "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": cs.cores, "kind": "port",
                             "sample": cs.desc + " per step"},
            "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "FLASH 4.6.2 (the reference's hydro) is not in the reference tree and no Fortran "
                    "compiler exists here; the timed reference is the oracle's C restatement of the "
                    "reference's algorithm on host cores"}
    print(json.dumps(line))


def host_link_gbs(nbytes=1 << 29, reps=3):
    """Bandwidth of the host link (pinned host memory <-> HBM) with plain
    copies of one large buffer, best of `reps`: the ceiling of the
    end-to-end path's transfers."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = [0.0, 0.0]
    for _ in range(reps):
        for k, (dst, src) in enumerate(((d, h), (h, d))):
            a.record()
            dst.copy_(src, non_blocking=True)
            b.record()
            torch.cuda.synchronize()
            best[k] = max(best[k], nbytes / (a.elapsed_time(b) * 1e-3) / 1e9)
    del h, d
    return best[0], best[1]


def e2e_run(G, g, steps, warmup, tune=False):
    """Fast path through the C ABI as a FLASH host would drive it: the host
    owns unk (FLASH order, variable fastest) and facevar{x,y,z} in pinned
    memory. Each step is one gb_step_graph_host call: upload of the leaf
    blocks' interiors (cells and owned faces; the step rebuilds guard cells
    and guard faces on the device), CFL dt, the step, and the download of
    each chunk's interiors while later chunks compute. One more step, run
    as separate interior upload / step graph / interior download calls,
    gives the parts."""
    import ctypes as C
    import torch
    G.init_hydro(G.hydro_params(True, precision=1))
    g.register()
    nunk, nn = g.nvar, g.nblocks
    host = torch.empty((nn, 24 ** 3, nunk), dtype=torch.float64).pin_memory()
    hf = [torch.empty(a.shape, dtype=torch.float64).pin_memory() for a in (g.fx, g.fy, g.fz)]
    io = G.HostIO()
    io.unk, io.nunk = host.data_ptr(), nunk
    for r in range(G.NROLE):
        io.host_slot[r] = -1
    for name, s in g.slots.items():
        io.host_slot[G.R[name]] = s
    io.facex, io.facey, io.facez = (h.data_ptr() for h in hf)
    L = G.lib()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    def host_from_device():
        G.check(L.gb_grid_download_flash(C.c_void_p(host.data_ptr()), nunk, io.host_slot, nn, st), "init")
        for h, d in zip(hf, (g.fx, g.fy, g.fz)):
            h.copy_(d.cpu())
        torch.cuda.synchronize()

    host_from_device()
    if tune:
        # the host-resident step picks its own chunk size: its downloads
        # overlap later chunks, so smaller chunks than the device-only
        # step's can win
        from torch_gb300 import autotune
        t0, o0, s0 = G.get_launch_config()[1], G.get_launch_config()[2], G.get_chunk_streams()
        autotune.tune(g, cool=True, chunks=(64, 128, 256, 512), tiles=(t0,), occs=(o0,), streams=(s0,),
                      step_fn=lambda: g.step_graph_host(io, cool=True), restore_fn=host_from_device,
                      variant="host")
    leaves = np.ascontiguousarray(g.leaf, np.int32)
    lp, nl = leaves.ctypes.data_as(C.c_void_p), len(leaves)
    hp = C.c_void_p(host.data_ptr())
    fp = [C.c_void_p(h.data_ptr()) for h in hf]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    parts = np.zeros(3)

    def separate():
        ev[0].record()
        G.check(L.gb_grid_upload_flash_interior_list(hp, nunk, io.host_slot, nl, lp, st), "upload")
        G.check(L.gb_grid_upload_faces_interior_list(*fp, nl, lp, st), "upload faces")
        ev[1].record()
        g.step_graph(cool=True)
        ev[2].record()
        G.check(L.gb_grid_download_flash_interior_list(hp, nunk, io.host_slot, nl, lp, st), "download")
        G.check(L.gb_grid_download_faces_interior_list(*fp, nl, lp, st), "download faces")
        ev[3].record()
        torch.cuda.synchronize()
        for q in range(3):
            parts[q] += ev[q].elapsed_time(ev[q + 1])

    for _ in range(warmup):
        g.step_graph_host(io, cool=True)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        g.step_graph_host(io, cool=True)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / steps
    nbytes = nl * (16 ** 3 * nunk + 3 * 17 * 16 * 16) * 8
    separate()
    c, t, o = G.get_launch_config()
    # the link's ceiling: the upload precedes the step (the guard fill needs
    # every leaf), the download can hide under the compute
    h2d, d2h = host_link_gbs()
    t_up, t_down = nbytes / (h2d * 1e9) * 1e3, nbytes / (d2h * 1e9) * 1e3
    bound = t_up + max(parts[1], t_down)
    return ms, nbytes, {"upload_ms": parts[0], "step_ms": parts[1], "download_ms": parts[2],
                        "link_h2d_gbs": h2d, "link_d2h_gbs": d2h,
                        "upload_gbs": nbytes / (parts[0] * 1e-3) / 1e9,
                        "download_gbs": nbytes / (parts[2] * 1e-3) / 1e9,
                        "bound_ms": bound, "frac_of_bound": bound / ms,
                        "launch_config": {"chunk": c, "tile": t, "occ": o, "streams": G.get_chunk_streams()},
                        "note": "parts from one step run as separate calls; the timed steps overlap the "
                                "download of each chunk with the compute of later chunks; bound_ms = the "
                                "bytes over the measured link rate for the upload, plus the larger of the "
                                "device step and the download"}


def rel_stats(x, ref):
    """Distribution of |x - ref| / ref over interior cells (torch tensors).
    Cells where either value is non-finite, or the reference is zero, are
    counted apart (n_bad) and left out of the quantiles."""
    import torch
    x, ref = x.flatten(), ref.flatten()
    ok = torch.isfinite(x) & torch.isfinite(ref) & (ref != 0)
    n_bad = int((~ok).sum())
    r = (x[ok] - ref[ok]).abs() / ref[ok].abs()
    if r.numel() == 0:
        return {"p50": None, "p99": None, "p999": None, "max": None, "frac_within_1pct": 0.0, "n_bad": n_bad}
    sub = r[torch.randperm(r.numel(), device=r.device)[:1 << 22]]
    q = torch.quantile(sub, torch.tensor([0.5, 0.99, 0.999], dtype=r.dtype, device=r.device)).tolist()
    return {"p50": q[0], "p99": q[1], "p999": q[2], "max": float(r.max()),
            "frac_within_1pct": float((r <= 0.01).double().sum()) / x.numel(), "n_bad": n_bad}


def cooling_one_step(G, grids, src, leaves):
    """One step from one common state (src's) under three cooling solvers,
    the hydro identical (mixed precision, same dt): the reference's plain
    implicit integrator (Brent stopped at 1 K), the same integrator stopped
    at 1e-3 K (the backward-Euler root to ~1e-3 K) and the learned path."""
    import torch
    g_plain, g_fast, g_tight = grids
    G.init_hydro(G.hydro_params(True, precision=1))
    src.register()
    dt = src.compute_dt().item()
    out = {}
    for name, g, sur, tol in (("plain", g_plain, False, 1.0), ("fast", g_fast, True, 1.0),
                              ("exact", g_tight, False, 1e-3)):
        g.u.copy_(src.u)
        for a, b in ((g.fx, src.fx), (g.fy, src.fy), (g.fz, src.fz)):
            a.copy_(b)
        G.set_brent_tolerance(tol)
        G.set_cooling_mode(sur)
        g.register()
        g.evolve_step(dt, cool=True)
        out[name] = g.u[leaves, g.slots["TEMP"], 4:20, 4:20, 4:20]
    G.set_brent_tolerance(1.0)
    G.set_cooling_mode(False)
    torch.cuda.synchronize()
    T0 = src.u[leaves, src.slots["TEMP"], 4:20, 4:20, 4:20]
    brent = (out["plain"] - out["fast"]).abs() <= 0.01 * out["plain"] + 2.0
    return {"fast_vs_plain": dict(rel_stats(out["fast"], out["plain"]),
                                  frac_within_1pct_or_2K=float(brent.double().mean())),
            "plain_vs_exact": rel_stats(out["plain"], out["exact"]),
            "fast_vs_exact": rel_stats(out["fast"], out["exact"]),
            "step_change": rel_stats(out["exact"], T0),
            "note": "one step from the same state; 'exact' = the plain integrator with Brent's "
                    "tolerance floor at 1e-3 K instead of 1 K"}


def l1(a, b, leaves, v):
    x = a[leaves, v, 4:20, 4:20, 4:20]
    y = b[leaves, v, 4:20, 4:20, 4:20]
    return float((x - y).abs().sum() / x.abs().sum())


def accuracy_condition(l1_fast, l1_mixed, l1_fast_exact, roundoff, v_fast, sp_fast, v_mixed, sp_mixed, bound=1e-4,
                       more=None):
    """Which path meets the metric's L1 <= 1e-4 (density and pressure after
    the run's steps): against the all-FP64 plain path, and for the learned
    path also against the backward-Euler root trajectory (the plain
    integrator with Brent's tolerance floor at 1e-3 K). more: further
    paths, name -> (l1, value, speedup), compared with the plain path."""
    ok = lambda d: d is not None and max(d.values()) <= bound
    paths = {
        "fast_vs_plain_fp64": {"l1": l1_fast, "meets": ok(l1_fast), "value": v_fast, "speedup_vs_plain_fp64": sp_fast},
        "fast_vs_backward_euler_root": {"l1": l1_fast_exact, "meets": ok(l1_fast_exact), "value": v_fast,
                                        "speedup_vs_plain_fp64": sp_fast},
        "mixed_plain_cooling_vs_plain_fp64": {"l1": l1_mixed, "meets": ok(l1_mixed), "value": v_mixed,
                                              "speedup_vs_plain_fp64": sp_mixed},
    }
    for name, (l1v, val, sp) in (more or {}).items():
        paths[name + "_vs_plain_fp64"] = {"l1": l1v, "meets": ok(l1v), "value": val, "speedup_vs_plain_fp64": sp}
    meeting = [(k, v) for k, v in paths.items() if v["meets"] and k.endswith("vs_plain_fp64")]
    best = max(meeting, key=lambda kv: kv[1]["value"]) if meeting else None
    return {"bound": bound, "paths": paths,
            "fastest_meeting_bound_vs_plain_fp64": ({"path": best[0], "value": best[1]["value"],
                                                     "speedup_vs_plain_fp64": best[1]["speedup_vs_plain_fp64"]}
                                                    if best else None),
            "plain_fp64_roundoff_drift_max": max(max(v.values()) for v in roundoff.values()) if roundoff else None,
            "note": "plain_fp64_roundoff_drift_max: L1 between two plain FP64 runs whose initial densities differ "
                    "by one ulp; a path cannot be held to a bound below its reference's own drift"}


def roundoff_divergence(G, tree, st, checkpoints=(10, 20)):
    """How far two plain FP64 runs drift apart from the same state when one
    of them starts with every density nudged by one ulp: density and
    pressure L1 (interior cells of the leaves) at each checkpoint step. The
    plain path's own sensitivity to round-off, against which a path's L1
    error after the same steps has to be read."""
    import torch
    ga = make_grid(G, tree, st)
    gbb = make_grid(G, tree, st)
    d = gbb.u[:, gbb.slots["DENS"]]
    d.copy_(torch.nextafter(d, torch.full_like(d, float("inf"))))
    G.init_hydro(G.hydro_params(True, precision=0))
    lv = torch.as_tensor(tree["leaf"].astype(np.int64), device="cuda")
    snap = {}
    for name, g in (("a", ga), ("b", gbb)):
        g.register()
        done = 0
        for n in checkpoints:
            for _ in range(n - done):
                g.step_graph(True)
            done = n
            snap[name, n] = [g.u[lv, v, 4:20, 4:20, 4:20].clone() for v in (0, 4)]
    out = {}
    for n in checkpoints:
        out[str(n)] = {v: float((snap["a", n][q] - snap["b", n][q]).abs().sum() / snap["a", n][q].abs().sum())
                       for q, v in enumerate(("dens", "pres"))}
    del ga, gbb, snap
    torch.cuda.empty_cache()
    return out


def lite_run(args, G, wl, tree, st, zones, world, rank, t_ic):
    """The full-scale workload: plain FP64 and fast paths only (each grid
    holds ~30 GB), both graph-replayed with tuned launch shapes."""
    import torch
    leaves = tree["leaf"]
    g_plain = make_grid(G, tree, st)
    g_fast = make_grid(G, tree, st)
    del st
    torch.cuda.empty_cache()
    clk = ClockSampler(clocks_csv_path(args))
    with clk:
        ms_plain, st_plain, pinfo = run_path(G, g_plain, 0, args.steps, args.warmup, graph=True,
                                             tune=not args.no_tune,
                                             tune_kw={"chunks": (16, 64), "tiles": (64,), "steps": 1})
        ms_fast, st_fast, ginfo = run_path(G, g_fast, 1, args.steps, args.warmup, surrogate=True, graph=True,
                                           tune=not args.no_tune)
    if world > 1:
        from torch_gb300.blocklist import max_over_ranks
        ms_plain, ms_fast = max_over_ranks(ms_plain), max_over_ranks(ms_fast)
    lv = torch.as_tensor(leaves.astype(np.int64), device="cuda")
    l1_fast = {v: l1(g_plain.u, g_fast.u, lv, i) for v, i in (("dens", 0), ("pres", 4))}
    if rank != 0:
        return
    lvl = np.bincount(tree["level"][leaves]).tolist()
    line = {
        "metric": "zone-updates/s", "value": zones * world / (ms_fast * 1e-3), "unit": "zone-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_fast,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": wl["name"], "leaf_blocks": len(leaves), "leaves_per_level": lvl, "zones": zones,
                   "block": "16^3+4gc", "physics": "MHD HLLD+CT, PPM, implicit heating/cooling",
                   "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (state %.1f GB)" % (g_fast.u.numel() * 8 / 1e9)},
        "plain_fp64": {"value": zones * world / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                       "launch_config": {k: pinfo["tuned"][k] for k in ("chunk", "tile", "streams", "fused")}
                       if pinfo["tuned"] else None},
        "speedup_vs_plain_fp64": ms_plain / ms_fast,
        # which accuracy the headline (the learned-cooling path) meets, and
        # the fastest path that meets the metric's bound against plain FP64
        "headline_accuracy": {
            "path": "mixed hydro + batched graph + learned cooling",
            "meets_l1_1e-4_vs_plain_fp64": max(l1_fast.values()) <= 1e-4,
            "meets_l1_1e-4_vs_backward_euler_root": max(l1_fast_exact.values()) <= 1e-4,
            "metric_compliant_path": {"path": "mixed hydro + batched graph + plain integrator on FP32 rates",
                                      "value": zones * world / (ms_m32 * 1e-3),
                                      "speedup_vs_plain_fp64": ms_plain / ms_m32,
                                      "l1_vs_plain_fp64": l1_m32,
                                      "frac_temps_within_1pct_of_plain": temp_m32["frac_within_1pct"]},
            "note": "the learned path solves the backward-Euler step to ~1e-8 of its root; the reference "
                    "integrator stops Brent at 1 K, which alone moves pressure L1 by "
                    "l1_reference_integrator_tolerance; the metric-compliant path keeps the reference "
                    "integrator's iterates"},
        "l1_err_vs_fp64": l1_fast,
        "launch_config": {k: ginfo["tuned"].get(k) for k in ("chunk", "tile", "occ", "streams")} if ginfo["tuned"] else None,
        "surrogate_fallback": st_fast["n_surrogate_reject"],
        "status": {"plain": st_plain["code"], "fast": st_fast["code"]},
        "gpu_launches": int(ginfo["graph_kernels_per_step"]) * args.steps,
        "clocks": clk.summary(),
        "ic_s": t_ic,
        "e2e": None,
        "note": "full-scale case: plain and fast paths only; the end-to-end, CPU-baseline and accuracy "
                "diagnostics run on the default 4101-block workload",
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb")
    ap.add_argument("--workload", default="amr", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (16 blocks, tile 32)")
    ap.add_argument("--weights", default=None, help="load surrogate weights (.npy) instead of training")
    ap.add_argument("--clocks-csv", default=None,
                    help="file for the nvidia-smi clock samples of the timed region (default: a temporary file)")
    # (--workload amr16k: the 16381-block, 5-level case; ~90 GB on the device)
    ap.add_argument("--save-weights", default=None)
    ap.add_argument("--ncu-range", action="store_true",
                    help="bracket the fast path's timed region with cudaProfilerStart/Stop")
    ap.add_argument("--only", choices=["plain", "fast", "eager", "e2e", "mixed", "mixed32"], default=None,
                    help="time one path alone and print a short line (for profiler captures)")
    ap.add_argument("--chunk", type=int, default=0, help="with --only: blocks per chunk (no autotuning)")
    ap.add_argument("--tile", type=int, default=32, help="with --chunk: reconstruction tile (32 or 64)")
    ap.add_argument("--occ", type=int, default=0, help="with --chunk: reconstruction occupancy bound (0, 1 or 2)")
    ap.add_argument("--streams", type=int, default=1, help="with --chunk: streams the chunks alternate between (1 or 2)")
    ap.add_argument("--fused", type=int, default=0, help="with --chunk: reconstruction and Riemann solve fused per block")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from torch_gb300 import gbhydro as G
    wl = WORKLOADS[args.workload]
    # replicas: every rank runs its own copy of the workload; the only
    # cross-rank exchange is the timing reduction (and the CFL minimum, when
    # ranks share one grid, in blocklist.global_dt)
    t0 = time.perf_counter()
    tree, st = build_workload(wl, "cuda")
    t_ic = time.perf_counter() - t0
    leaves = tree["leaf"]
    zones = len(leaves) * 4096
    units = G.code_units()
    # learned cooling: 1e7 samples from the plain integrator, then training
    # (outside the timed region; reported)
    if args.weights:
        G.init_cooling(G.cool_params())
        G.mlp_init(7)
        G.mlp_set_weights(np.load(args.weights))
        t_samples = t_train = 0.0
        losses = np.array([np.nan])
    else:
        t0 = time.perf_counter()
        G.init_cooling(G.cool_params())
        feat, tgt = G.surrogate_samples(10_000_000, 2024)
        keep = torch.isfinite(tgt)
        feat, tgt = feat[keep].contiguous(), tgt[keep].contiguous()
        torch.cuda.synchronize()
        t_samples = time.perf_counter() - t0
        t0 = time.perf_counter()
        G.mlp_init(7)
        losses = G.mlp_train(feat, tgt, steps=8000, batch=16384, lr=3e-3, seed=5)
        t_train = time.perf_counter() - t0
        del feat, tgt
    if args.save_weights:
        np.save(args.save_weights, G.mlp_weights())
    G.init_cooling(G.cool_params(dens_unit=units["dens_unit"], vel_unit=units["vel_unit"],
                                 time_unit=units["time_unit"]))
    if args.only:
        g = make_grid(G, tree, st)
        del st
        if args.chunk:
            G.set_launch_config(args.chunk, args.tile, args.occ)
            G.set_chunk_streams(args.streams)
            G.set_fused(int(args.fused))
        if args.only == "e2e":
            # the fast path (launch shapes as given) end to end from host arrays
            G.set_cooling_mode(True)
            ms, nbytes, parts = e2e_run(G, g, args.steps, args.warmup)
            if rank == 0:
                print(json.dumps({"path": "e2e", "workload": wl["name"], "ms_per_step": ms,
                                  "value": zones * world / (ms * 1e-3), "unit": "zone-updates/s",
                                  "h2d_bytes_per_step": nbytes, "parts": parts}))
            return
        prec, sur, graph, cm = {"plain": (0, False, True, None), "fast": (1, True, True, None),
                                "eager": (1, True, False, None), "mixed": (1, False, True, None),
                                "mixed32": (1, False, True, 2)}[args.only]
        ms, stt, info = run_path(G, g, prec, args.steps, args.warmup, surrogate=sur, graph=graph,
                                 tune=not args.no_tune and graph and not args.chunk, profile=not graph,
                                 ncu_range=args.ncu_range, cool_mode=cm)
        if rank == 0:
            print(json.dumps({"path": args.only, "workload": wl["name"], "ms_per_step": ms,
                              "value": zones * world / (ms * 1e-3), "unit": "zone-updates/s",
                              "status_code": stt["code"],
                              "kernels": {k: v[0] / args.steps for k, v in info.items()} if not graph else info}))
        return
    if wl.get("lite"):
        return lite_run(args, G, wl, tree, st, zones, world, rank, t_ic)
    g_plain = make_grid(G, tree, st)
    g_fast = make_grid(G, tree, st)
    g_mixed = make_grid(G, tree, st)
    g_m32 = make_grid(G, tree, st)
    g_tight = make_grid(G, tree, st)
    g_eager = make_grid(G, tree, st)
    cs = None
    if rank == 0 and not args.no_cpu_baseline:
        cs = CpuStep(wl, tree, st)
    clk = ClockSampler(clocks_csv_path(args))
    if world > 1:
        dist.barrier()
    with clk:
        ms_plain, st_plain, pinfo = run_path(G, g_plain, 0, args.steps, args.warmup, graph=True,
                                             tune=not args.no_tune,
                                             tune_kw={"chunks": (64, 256, 1024), "steps": 1})
        ms_fast, st_fast, ginfo = run_path(G, g_fast, 1, args.steps, args.warmup, surrogate=True, graph=True,
                                           tune=not args.no_tune, ncu_range=args.ncu_range)
        # the same path launched eagerly with the in-library profiler on:
        # per-kernel times (the profiler cannot time inside a graph)
        ms_eager, st_eager, prof = run_path(G, g_eager, 1, args.steps, args.warmup, surrogate=True, profile=True)
        # mixed hydro with the plain integrator (the path that keeps the
        # reference integrator's answers), at the fast path's launch shape
        if ginfo["tuned"]:
            G.set_launch_config(ginfo["tuned"]["chunk"], ginfo["tuned"]["tile"], ginfo["tuned"]["occ"])
            G.set_chunk_streams(ginfo["tuned"]["streams"])
            G.set_fused(int(ginfo["tuned"].get("fused", 0)))
        ms_mixed, st_mixed, _ = run_path(G, g_mixed, 1, args.steps, args.warmup, graph=True)
        # the same with the integrator's rate function in FP32 (Brent's
        # iterates in FP64)
        ms_m32, st_m32, _ = run_path(G, g_m32, 1, args.steps, args.warmup, graph=True, cool_mode=2)
    # diagnostic, untimed: the plain path's own drift under a one-ulp
    # nudge of the initial density (what an L1 error after 10 and 20 steps
    # can be read against)
    roundoff = roundoff_divergence(G, tree, st)
    del st
    # diagnostic, untimed: mixed hydro + the plain integrator with Brent's
    # tolerance floor at 1e-3 K (the backward-Euler trajectory)
    G.set_brent_tolerance(1e-3)
    run_path(G, g_tight, 1, args.steps, args.warmup)
    G.set_brent_tolerance(1.0)
    if world > 1:
        from torch_gb300.blocklist import max_over_ranks
        ms_plain, ms_fast = max_over_ranks(ms_plain), max_over_ranks(ms_fast)
        ms_mixed, ms_m32 = max_over_ranks(ms_mixed), max_over_ranks(ms_m32)
    # accuracy of the fast path against the plain one after the same steps
    lv = torch.as_tensor(leaves.astype(np.int64), device="cuda")
    a, b, c, d = g_plain.u, g_fast.u, g_mixed.u, g_tight.u
    fields = (("dens", 0), ("pres", 4))
    l1_fast = {v: l1(a, b, lv, i) for v, i in fields}
    l1_mixed = {v: l1(a, c, lv, i) for v, i in fields}
    l1_m32 = {v: l1(a, g_m32.u, lv, i) for v, i in fields}
    l1_tol = {v: l1(d, c, lv, i) for v, i in fields}
    l1_fast_exact = {v: l1(d, b, lv, i) for v, i in fields}
    sT = g_plain.slots["TEMP"]
    Ta, Tb = a[lv, sT, 4:20, 4:20, 4:20], b[lv, sT, 4:20, 4:20, 4:20]
    temp_steps = dict(rel_stats(Tb, Ta), frac_within_1pct_or_2K=float(((Ta - Tb).abs() <= 0.01 * Ta + 2.0)
                                                                        .double().mean()))
    # the metric-compliant path's cooled temperatures against the plain path's
    Tm = g_m32.u[lv, sT, 4:20, 4:20, 4:20]
    temp_m32 = rel_stats(Tm, Ta)
    del a, b, c, d, Ta, Tb, Tm
    one_step = cooling_one_step(G, (g_plain, g_fast, g_tight), g_mixed, lv)
    G.set_cooling_mode(True)
    e2e_ms, e2e_bytes, e2e_parts = e2e_run(G, g_fast, max(2, args.steps // 2), 3, tune=not args.no_tune)
    G.set_cooling_mode(False)
    hbm, hbm_kind = peaks()
    # FP64-pipe roofline of the plain path: flops per zone-update counted by
    # the oracle's counting build (roofline_constants.json) over the
    # measured FP64 FMA peak of this GPU
    fp64 = None
    step_roof = None
    rc = {}
    try:
        with open(os.path.join(ROOT, "roofline_constants.json")) as f:
            rc = json.load(f)
        fpz = rc["mhd_cooling_step"]["flops"]
        peak64 = G.measure_fp64_peak()
        peak32 = G.measure_fp32_peak()
        ach64 = zones * fpz / (ms_plain * 1e-3) / 1e12
        fp64 = {"path": "plain_fp64", "flops_per_zone": fpz, "achieved_tflops": ach64, "peak_tflops": peak64,
                "frac": ach64 / peak64, "peak_kind": "measured FP64 FMA loop on this GPU",
                "note": "flops = + - * / sqrt of the oracle's MHD step + CFL + implicit cooling per zone; "
                        "a division or sqrt issues several FP64 instructions, so the pipe is busier than "
                        "this fraction"}
        # the fast path: reconstruction, Riemann solve and edge fields in
        # FP32, the update in FP64 (the learned cooling's FP32 rate
        # evaluations are not counted); HBM: 216 B per zone-update
        ph = rc["mhd_hlld_ct_phases"]
        f32 = ph["recon"]["flops"] + ph["flux"]["flops"] + ph["emf"]["flops"]
        f64 = ph["update"]["flops"]
        t_fast = ms_fast * 1e-3
        step_roof = {
            "plain_fp64": {"pipe": "fp64", "frac": ach64 / peak64},
            "fast": {"fp32": {"flops_per_zone": f32, "achieved_tflops": zones * f32 / t_fast / 1e12,
                              "peak_tflops": peak32, "frac": zones * f32 / t_fast / 1e12 / peak32},
                     "fp64": {"flops_per_zone": f64, "achieved_tflops": zones * f64 / t_fast / 1e12,
                              "peak_tflops": peak64, "frac": zones * f64 / t_fast / 1e12 / peak64},
                     "hbm": {"bytes_per_zone": 216.0, "achieved_gbs": zones * 216.0 / t_fast / 1e9,
                             "peak_gbs": hbm, "frac": zones * 216.0 / t_fast / 1e9 / hbm}},
            "peak_kind": "FP32 and FP64: measured FMA loops on this GPU; HBM: " + hbm_kind,
            "note": "flops per zone from the oracle's counting build split by phase (roofline_constants.json)"}
    except (OSError, KeyError, ValueError, G.GBError):
        pass
    # dominant kernel: largest share of the fast path's timed region.
    # Algorithmic bytes = 216 B per unit (12 FP64 MHD words + 3 cooling
    # words, read once + written once) x the units a launch covers: zones,
    # or for the plain-integrator fallback the cells it was handed.
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom][0], prof[dom][1]
    units_total = zones * args.steps
    if dom == "sur_fallback":
        units_total = st_eager["n_surrogate_reject"]
    zones_per_launch = units_total / dom_n
    launch_s = dom_ms / dom_n * 1e-3
    ach = 216.0 * zones_per_launch / launch_s / 1e9
    compute = None
    phase = {"recon": "recon", "flux": "flux", "emf": "emf"}.get(dom)
    if phase and rc.get("mhd_hlld_ct_phases") and step_roof:
        fz = rc["mhd_hlld_ct_phases"][phase]["flops"]
        a32 = fz * zones_per_launch / launch_s / 1e12
        compute = {"pipe": "fp32", "flops_per_zone": fz, "achieved_tflops": a32,
                   "peak_tflops": step_roof["fast"]["fp32"]["peak_tflops"],
                   "frac": a32 / step_roof["fast"]["fp32"]["peak_tflops"],
                   "note": "algorithmic flops of this phase (the oracle's count, which includes products with "
                           "the eigenvectors' structural zeros that the kernel skips)"}
    launches = int(ginfo["graph_kernels_per_step"]) * args.steps
    if rank != 0:
        return
    lvl = np.bincount(tree["level"][leaves]).tolist()
    line = {
        "metric": "zone-updates/s", "value": zones * world / (ms_fast * 1e-3), "unit": "zone-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_fast,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": wl["name"], "leaf_blocks": len(leaves), "leaves_per_level": lvl,
                   "zones": zones, "block": "16^3+4gc",
                   "physics": "MHD HLLD+CT, PPM, implicit heating/cooling", "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (state %.1f GB)" % (g_fast.u.numel() * 8 / 1e9)},
        "plain_fp64": {"value": zones * world / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                       "launch_config": {k: pinfo["tuned"][k] for k in ("chunk", "tile", "streams", "fused")}
                       if pinfo["tuned"] else None},
        "speedup_vs_plain_fp64": ms_plain / ms_fast,
        "l1_err_vs_fp64": l1_fast,
        "l1_err_mixed_hydro_vs_fp64": l1_mixed,
        "l1_err_vs_backward_euler_root": l1_fast_exact,
        "l1_reference_integrator_tolerance": l1_tol,
        "l1_note": "after warmup+steps steps. l1_err_vs_fp64: fast path vs the all-FP64 path with the plain "
                   "integrator; l1_err_mixed_hydro_vs_fp64: FP32 reconstruction/Riemann + plain integrator vs "
                   "all-FP64; l1_reference_integrator_tolerance: the plain integrator with Brent stopped at 1 K "
                   "(the reference) vs at 1e-3 K, both on mixed hydro; l1_err_vs_backward_euler_root: fast "
                   "path vs the 1e-3 K run",
        "mixed_plain_cooling": {"value": zones * world / (ms_mixed * 1e-3), "ms_per_step": ms_mixed,
                                "speedup_vs_plain_fp64": ms_plain / ms_mixed,
                                "note": "mixed hydro; the plain integrator fused into the update, its rate "
                                        "function in FP64 with shared transcendentals"},
        "mixed_fp32_rates_cooling": {"value": zones * world / (ms_m32 * 1e-3), "ms_per_step": ms_m32,
                                     "speedup_vs_plain_fp64": ms_plain / ms_m32, "l1_err_vs_fp64": l1_m32,
                                     "temp_rel_err_vs_plain_after_steps": temp_m32,
                                     "note": "mixed hydro; the plain integrator as a pass of its own after the "
                                             "update, its rate function in FP32 (Brent's and the bracket search's "
                                             "iterates and the residual in FP64)"},
        "roundoff_divergence_plain_fp64": roundoff,
        "accuracy_condition": accuracy_condition(l1_fast, l1_mixed, l1_fast_exact, roundoff,
                                                 zones * world / (ms_fast * 1e-3), ms_plain / ms_fast,
                                                 zones * world / (ms_mixed * 1e-3), ms_plain / ms_mixed,
                                                 more={"mixed_fp32_rates_cooling": (
                                                     l1_m32, zones * world / (ms_m32 * 1e-3), ms_plain / ms_m32)}),
        "fast_eager": {"ms_per_step": ms_eager, "value": zones * world / (ms_eager * 1e-3),
                       "note": "the same fast path launched kernel by kernel with the host reading dt each step"},
        "launch_config": {k: ginfo["tuned"].get(k) for k in ("chunk", "tile", "occ", "streams", "fused", "cached")}
        if ginfo["tuned"] else {"chunk": 16, "tile": 32, "occ": 0, "streams": 1, "tuned": False},
        "kernel_ms_per_step_fast": {k: v[0] / args.steps for k, v in prof.items()},
        "kernel_launches_per_step_fast": {k: v[1] / args.steps for k, v in prof.items()},
        "temp_rel_err_vs_plain_after_steps": temp_steps,
        "cooling_one_step": one_step,
        "surrogate": {"samples": 10_000_000, "sample_s": t_samples, "train_s": t_train,
                      "train_loss_final": float(np.mean(losses[-200:])),
                      "accepted": st_fast["n_surrogate"], "fallback": st_fast["n_surrogate_reject"],
                      "fallback_frac": st_fast["n_surrogate_reject"] / max(1, st_fast["n_surrogate"] + st_fast["n_surrogate_reject"])},
        "status": {name: {k: stt[k] for k in ("code", "n_code", "n_fallback", "n_rh_fallback", "n_eint_switch",
                                                 "n_bracket_fail", "n_clamped")}
                   for name, stt in (("plain", st_plain), ("fast", st_fast), ("mixed_plain_cooling", st_mixed),
                                     ("mixed_fp32_rates_cooling", st_m32))},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s",
                     "frac": ach / hbm,
                     "traffic": TRAFFIC_B_PER_ZONE[dom] * zones_per_launch if dom in TRAFFIC_B_PER_ZONE else None,
                     "traffic_source": "ncu DRAM bytes per zone of the kernels this profiler bucket times (one-kernel "
                                       "captures on the 128^3 box, one 512-block launch each), times the zones of "
                                       "one launch here",
                     "peak_kind": hbm_kind, "launch_ms": dom_ms / dom_n,
                     "algo_bytes_per_launch": 216.0 * zones_per_launch, "compute": compute},
        "step_roofline": step_roof,
        "e2e": {"value": zones / (e2e_ms * 1e-3), "unit": "zone-updates/s", "h2d_bytes_per_step": e2e_bytes,
                "d2h_bytes_per_step": e2e_bytes, "parts": e2e_parts},
        "fp64_roofline": fp64,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "ic_s": t_ic,
    }
    if cs is not None:
        line["cpu_baseline"] = cpu_baseline(cs, 1)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
