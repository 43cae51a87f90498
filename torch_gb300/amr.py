"""Block-structured AMR trees and synthetic AMR workloads.

A FLASH/PARAMESH-style octree of 16^3 blocks: a periodic root grid of
nr^3 level-0 blocks, each refined block holding 8 children. The
refinement is driven by position (the distance to seeded overdensity
centres), level by level, with the counts of refined blocks chosen to give
the requested leaf counts per level; the result is checked for 2:1 balance
(face, edge and corner neighbours of a leaf differ by at most one level).

Node ids double as store block ids (every node has a slot; only leaves are
updated). Arrays follow gb_tree_desc: level[n], coord[n, 3] (lower corner
in units of the node's own block size), child[n, 8] (-1 for leaves; child c
has offset (c & 1, (c >> 1) & 1, (c >> 2) & 1)), root[rx + nr (ry + nr rz)].
"""
from __future__ import annotations

import numpy as np

NXB = 16


def build_tree(nr: int, centres: np.ndarray, refine_counts) -> dict:
    """Refine, at each level l, the refine_counts[l] blocks of level l whose
    centres lie closest to any of `centres` (unit-cube coordinates), taking
    only blocks whose 26 neighbouring regions are covered at level >= l so
    the tree stays 2:1 balanced."""
    level = [0] * nr ** 3
    coord = [(i % nr, (i // nr) % nr, i // (nr * nr)) for i in range(nr ** 3)]
    child = [[-1] * 8 for _ in range(nr ** 3)]
    root = np.arange(nr ** 3, dtype=np.int32)
    frontier = list(range(nr ** 3))
    for lev, count in enumerate(refine_counts):
        size = 1.0 / (nr * 2 ** lev)
        pos = np.array([[(coord[n][d] + 0.5) * size for d in range(3)] for n in frontier])
        dist = np.full(len(frontier), np.inf)
        for c in centres:
            dd = np.abs(pos - c)
            dd = np.minimum(dd, 1.0 - dd)  # periodic
            dist = np.minimum(dist, np.sqrt((dd ** 2).sum(1)))
        # blocks of this level by integer coordinate (level-lev units)
        nl = nr * 2 ** lev
        present = set(coord[n] for n in frontier)
        chosen = []
        for q in np.argsort(dist, kind="stable"):
            if len(chosen) == count:
                break
            c0 = coord[frontier[q]]
            ok = True
            for dz in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        nb = ((c0[0] + dx) % nl, (c0[1] + dy) % nl, (c0[2] + dz) % nl)
                        if nb not in present:  # covered by a coarser leaf
                            ok = False
            if ok:
                chosen.append(q)
        if len(chosen) < count:
            raise ValueError(f"only {len(chosen)} of {count} level-{lev} blocks can be refined")
        new_frontier = []
        for q in sorted(chosen):
            n = frontier[q]
            for c in range(8):
                off = (c & 1, (c >> 1) & 1, (c >> 2) & 1)
                level.append(lev + 1)
                coord.append(tuple(2 * coord[n][d] + off[d] for d in range(3)))
                child.append([-1] * 8)
                child[n][c] = len(level) - 1
                new_frontier.append(len(level) - 1)
        frontier = new_frontier
    t = dict(level=np.array(level, np.int32), coord=np.array(coord, np.int32),
             child=np.array(child, np.int32), root=root, nr=(nr, nr, nr),
             maxlevel=int(max(level)))
    t["leaf"] = np.nonzero(t["child"][:, 0] < 0)[0].astype(np.int32)
    return t


def leaf_counts(t: dict):
    lv = t["level"][t["leaf"]]
    return [int((lv == l).sum()) for l in range(t["maxlevel"] + 1)]


def leaf_at(t: dict, X) -> int:
    """Leaf containing the point X (integer coordinates in finest cells)."""
    S0 = NXB << t["maxlevel"]
    nr = t["nr"]
    r = [int(X[d] // S0) for d in range(3)]
    node = int(t["root"][r[0] + nr[0] * (r[1] + nr[1] * r[2])])
    lev = 0
    while t["child"][node, 0] >= 0:
        half = S0 >> (lev + 1)
        c = sum(((int(X[d]) // half) & 1) << d for d in range(3))
        node = int(t["child"][node, c])
        lev += 1
    return node


def check_balance(t: dict) -> int:
    """Number of leaf pairs (sharing a face, edge or corner) whose levels
    differ by more than one."""
    ml = t["maxlevel"]
    N = [n * NXB << ml for n in t["nr"]]
    bad = 0
    for n in t["leaf"]:
        L = int(t["level"][n])
        s = 1 << (ml - L)
        lo = t["coord"][n] * NXB * s
        size = NXB * s
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if dx == dy == dz == 0:
                        continue
                    # sample just outside each face/edge/corner at a few points
                    for f in (0.25, 0.75):
                        X = []
                        for d, o in enumerate((dx, dy, dz)):
                            if o < 0:
                                X.append((lo[d] - 1) % N[d])
                            elif o > 0:
                                X.append((lo[d] + size) % N[d])
                            else:
                                X.append(lo[d] + int(f * size))
                        m = leaf_at(t, X)
                        if abs(int(t["level"][m]) - L) > 1:
                            bad += 1
    return bad


def config3_tree(seed: int = 45):
    """4096-ish leaf blocks over 4 levels: 13^3 root blocks, refinement
    counts (140, 100, 32) -> leaves 2057 / 1020 / 768 / 256 (4101 blocks,
    16.8 M zones, 256^3-equivalent) around 8 seeded centres."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.1, 0.9, (8, 3))
    return build_tree(13, centres, [140, 100, 32]), centres


def config5_tree(seed: int = 47):
    """The full-scale tree: 16^3 root blocks refined (760, 600, 330, 65) ->
    leaves 3336 / 5480 / 4470 / 2575 / 520 over 5 levels (16381 blocks,
    67.1 M zones) around 8 seeded centres. (A cubic root grid cannot give
    exactly 16384 leaves: nr^3 + 7 * refined never equals it.)"""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.1, 0.9, (8, 3))
    return build_tree(16, centres, [760, 600, 330, 65]), centres


def _trilinear(base, pts):
    """Periodic trilinear sample of base[x, y, z] (cell-centred values on an
    N^3 grid of the unit cube) at pts[..., 3] in unit-cube coordinates."""
    import torch
    N = base.shape[0]
    q = pts * N - 0.5
    i0 = torch.floor(q)
    f = q - i0
    i0 = i0.long()
    out = 0.0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (f[..., 0] if dx else 1 - f[..., 0]) * (f[..., 1] if dy else 1 - f[..., 1]) * \
                    (f[..., 2] if dz else 1 - f[..., 2])
                ix = (i0[..., 0] + dx) % N
                iy = (i0[..., 1] + dy) % N
                iz = (i0[..., 2] + dz) % N
                out = out + w * base[ix, iy, iz]
    return out


def amr_box(tree: dict, centres, seed: int, sigma_ln=1.0, mach=5.0, beta=1.0, dA=0.1, contrast=100.0,
            fwhm_cells=4.0, gamma=5.0 / 3.0, nvar=12, device="cuda"):
    """Synthetic AMR MHD state on every leaf of `tree` (interior cells and
    interior faces; guard cells are left to the guard fill).

    Returns dict(u[nnodes, nvar, 24, 24, 24], fx, fy, fz, root_dx) as torch
    tensors on `device`. Slots: 0..6 hydro, 7..9 cell B, 10 TEMP (set by
    the caller from the EOS), 11 TDUS."""
    import torch
    from . import workloads as W
    rng = np.random.default_rng(seed)
    nr = tree["nr"][0]
    N0 = nr * NXB
    shape = (N0, N0, N0)
    g = torch.as_tensor(W.grf_scalar(shape, 1, 8, rng), device=device)
    vx, vy, vz = W.grf_vector(shape, 1, 8, rng, solenoidal=True)
    p0 = 1.0
    vrms = np.sqrt(np.mean(vx ** 2 + vy ** 2 + vz ** 2))
    sv = mach * np.sqrt(gamma * p0) / vrms
    vel = [torch.as_tensor(a * sv, device=device) for a in (vx, vy, vz)]
    B0 = np.sqrt(2.0 * p0 / beta)
    ax, ay, az = W.grf_vector(shape, 1, 8, rng)
    # scale A so that its discrete curl on the root grid has rms dA * B0
    h = 1.0 / N0
    d = lambda a, axis: (np.roll(a, -1, axis) - a) / h
    bxr, byr, bzr = d(az, 1) - d(ay, 2), d(ax, 2) - d(az, 0), d(ay, 0) - d(ax, 1)
    sa = dA * B0 / np.sqrt(np.mean(bxr ** 2 + byr ** 2 + bzr ** 2))
    A = [torch.as_tensor(a * sa, device=device) for a in (ax, ay, az)]
    cen = torch.as_tensor(np.asarray(centres), device=device)
    sig_b = fwhm_cells / (N0 * 2 ** tree["maxlevel"]) / 2.3548200450309493
    nn = len(tree["level"])
    NB = NXB + 8
    u = torch.zeros((nn, nvar, NB, NB, NB), dtype=torch.float64, device=device)
    fx = torch.zeros((nn, NB, NB, NB + 1), dtype=torch.float64, device=device)
    fy = torch.zeros((nn, NB, NB + 1, NB), dtype=torch.float64, device=device)
    fz = torch.zeros((nn, NB + 1, NB, NB), dtype=torch.float64, device=device)
    leaves = tree["leaf"]
    ar = torch.arange(NXB, dtype=torch.float64, device=device)
    ar1 = torch.arange(NXB + 1, dtype=torch.float64, device=device)
    for chunk in np.array_split(leaves, max(1, len(leaves) // 256)):
        lv = torch.as_tensor(tree["level"][chunk], device=device, dtype=torch.float64)
        co = torch.as_tensor(tree["coord"][chunk], device=device, dtype=torch.float64)
        dx = 1.0 / (nr * NXB * 2.0 ** lv)  # per block
        # cell centres [b, k, j, i, 3]
        def grid(ox, oy, oz, ni, nj, nk, sx, sy, sz):
            xs = (co[:, 0, None] * NXB + ox[None, :] + sx) * dx[:, None]
            ys = (co[:, 1, None] * NXB + oy[None, :] + sy) * dx[:, None]
            zs = (co[:, 2, None] * NXB + oz[None, :] + sz) * dx[:, None]
            X = xs[:, None, None, :].expand(-1, nk, nj, ni)
            Y = ys[:, None, :, None].expand(-1, nk, nj, ni)
            Z = zs[:, :, None, None].expand(-1, nk, nj, ni)
            return torch.stack([X, Y, Z], -1) % 1.0
        P = grid(ar, ar, ar, NXB, NXB, NXB, 0.5, 0.5, 0.5)
        rho = torch.exp(sigma_ln * _trilinear(g, P) - 0.5 * sigma_ln ** 2)
        bump = torch.zeros_like(rho)
        for c in cen:
            dd = torch.abs(P - c)
            dd = torch.minimum(dd, 1.0 - dd)
            bump = bump + torch.exp(-(dd ** 2).sum(-1) / (2 * sig_b ** 2))
        rho = rho * (1.0 + (contrast - 1.0) * bump)
        v3 = [_trilinear(vv, P) for vv in vel]
        # face fields: discrete curl of A sampled on the block's edges
        def edgeA(comp, sx, sy, sz, ni, nj, nk, ox, oy, oz):
            return _trilinear(A[comp], grid(ox, oy, oz, ni, nj, nk, sx, sy, sz))
        dxb = dx[:, None, None, None]
        # Bx on x-faces (i = 0..16, j, k = 0..15): dAz/dy - dAy/dz
        Az_x = edgeA(2, 0.0, 0.0, 0.5, NXB + 1, NXB + 1, NXB, ar1, ar1, ar)
        Ay_x = edgeA(1, 0.0, 0.5, 0.0, NXB + 1, NXB, NXB + 1, ar1, ar, ar1)
        Bx = (Az_x[:, :, 1:, :] - Az_x[:, :, :-1, :]) / dxb - (Ay_x[:, 1:, :, :] - Ay_x[:, :-1, :, :]) / dxb
        Ax_y = edgeA(0, 0.5, 0.0, 0.0, NXB, NXB + 1, NXB + 1, ar, ar1, ar1)
        Az_y = edgeA(2, 0.0, 0.0, 0.5, NXB + 1, NXB + 1, NXB, ar1, ar1, ar)
        By = (Ax_y[:, 1:, :, :] - Ax_y[:, :-1, :, :]) / dxb - (Az_y[:, :, :, 1:] - Az_y[:, :, :, :-1]) / dxb
        Ay_z = edgeA(1, 0.0, 0.5, 0.0, NXB + 1, NXB, NXB + 1, ar1, ar, ar1)
        Ax_z = edgeA(0, 0.5, 0.0, 0.0, NXB, NXB + 1, NXB + 1, ar, ar1, ar1)
        Bz = (Ay_z[:, :, :, 1:] - Ay_z[:, :, :, :-1]) / dxb - (Ax_z[:, :, 1:, :] - Ax_z[:, :, :-1, :]) / dxb + B0
        ids = torch.as_tensor(chunk.astype(np.int64), device=device)
        s = slice(4, 4 + NXB)
        s1 = slice(4, 4 + NXB + 1)
        eint = p0 / ((gamma - 1.0) * rho)
        vals = [rho, v3[0], v3[1], v3[2], torch.full_like(rho, p0), eint + 0.5 * (v3[0] ** 2 + v3[1] ** 2 + v3[2] ** 2),
                eint, 0.5 * (Bx[..., 1:] + Bx[..., :-1]), 0.5 * (By[:, :, 1:, :] + By[:, :, :-1, :]),
                0.5 * (Bz[:, 1:] + Bz[:, :-1])]
        for v, val in enumerate(vals):
            if v < nvar:
                u[ids, v, s, s, s] = val
        fx[ids, s, s, s1] = Bx
        fy[ids, s, s1, s] = By
        fz[ids, s1, s, s] = Bz
    return dict(u=u, fx=fx, fy=fy, fz=fz, root_dx=1.0 / N0)


def small_tree(seed: int = 3):
    """A 4^3-root tree with two refined levels around one centre (for
    parity tests): leaves 56 / 60 / 16."""
    rng = np.random.default_rng(seed)
    centres = 0.5 + rng.uniform(-0.02, 0.02, (1, 3))
    return build_tree(4, centres, [8, 2]), centres
