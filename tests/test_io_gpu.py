"""FLASH-layout host <-> device transfers of the block store."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(gb):
    from torch_gb300 import amr
    t, c = amr.small_tree()
    st = amr.amr_box(t, c, seed=5, device="cuda")
    return t, gb.grid_from_amr(t, st, mhd=True, cooling=True)


def _slots(gb, g):
    hs = (C.c_int * gb.NROLE)(*([-1] * gb.NROLE))
    for name, s in g.slots.items():
        hs[gb.R[name]] = s
    return hs


def test_flash_layout_roundtrip_whole_store(gb):
    import torch
    t, g = _grid(gb)
    L, nunk, nb = gb.lib(), g.nvar, g.nblocks
    ref = g.u.clone()
    host = torch.empty((nb, 24 ** 3, nunk), dtype=torch.float64).pin_memory()
    gb.check(L.gb_grid_download_flash(C.c_void_p(host.data_ptr()), nunk, _slots(gb, g), nb, None), "down")
    torch.cuda.synchronize()
    # variable-fastest order: host[b, cell, v] == store[b, v, cell]
    assert torch.equal(host, ref.reshape(nb, nunk, -1).transpose(1, 2).cpu())
    g.u.zero_()
    gb.check(L.gb_grid_upload_flash(C.c_void_p(host.data_ptr()), nunk, _slots(gb, g), nb, None), "up")
    torch.cuda.synchronize()
    assert torch.equal(g.u, ref)


def test_flash_layout_list_transfers(gb):
    """Leaf-list transfers move exactly the listed blocks, cells and faces,
    and agree with the whole-store transfer on them."""
    import torch
    t, g = _grid(gb)
    L, nunk, nb = gb.lib(), g.nvar, g.nblocks
    leaves = np.ascontiguousarray(t["leaf"][::2], np.int32)   # runs and gaps
    lp = leaves.ctypes.data_as(C.c_void_p)
    host = torch.zeros((nb, 24 ** 3, nunk), dtype=torch.float64).pin_memory()
    hf = [torch.zeros(a.shape, dtype=torch.float64).pin_memory() for a in (g.fx, g.fy, g.fz)]
    gb.check(L.gb_grid_download_flash_list(C.c_void_p(host.data_ptr()), nunk, _slots(gb, g), len(leaves), lp,
                                           None), "down list")
    gb.check(L.gb_grid_download_faces_list(*[C.c_void_p(h.data_ptr()) for h in hf], len(leaves), lp, None),
             "faces down")
    torch.cuda.synchronize()
    full = g.u.reshape(nb, nunk, -1).transpose(1, 2).cpu()
    mask = np.zeros(nb, bool)
    mask[leaves] = True
    assert torch.equal(host[mask], full[mask])
    assert not host[~mask].any()
    for h, d in zip(hf, (g.fx, g.fy, g.fz)):
        assert torch.equal(h[mask], d.cpu()[mask])
        assert not h[~mask].any()
    # upload a modified copy of the listed blocks into a cleared store
    ref_u, ref_f = g.u.clone(), [a.clone() for a in (g.fx, g.fy, g.fz)]
    host[mask] *= 2.0
    for h in hf:
        h[mask] += 1.0
    g.u.zero_()
    for a in (g.fx, g.fy, g.fz):
        a.zero_()
    gb.check(L.gb_grid_upload_flash_list(C.c_void_p(host.data_ptr()), nunk, _slots(gb, g), len(leaves), lp,
                                         None), "up list")
    gb.check(L.gb_grid_upload_faces_list(*[C.c_void_p(h.data_ptr()) for h in hf], len(leaves), lp, None),
             "faces up")
    torch.cuda.synchronize()
    m = torch.as_tensor(mask, device="cuda")
    assert torch.equal(g.u[m], 2.0 * ref_u[m])
    assert not g.u[~m].any()
    for a, r in zip((g.fx, g.fy, g.fz), ref_f):
        assert torch.equal(a[m], r[m] + 1.0)
        assert not a[~m].any()


def test_list_transfer_rejects_bad_ids(gb):
    t, g = _grid(gb)
    L = gb.lib()
    bad = np.array([0, g.nblocks], np.int32)
    host = np.zeros((2, 24 ** 3, g.nvar))
    rc = L.gb_grid_upload_flash_list(host.ctypes.data_as(C.c_void_p), g.nvar, _slots(gb, g), 2,
                                     bad.ctypes.data_as(C.c_void_p), None)
    assert rc != 0


def test_interior_transfers_move_interiors_only(gb):
    """Interior transfers move the 16^3 interior cells and the owned faces
    (4..20 along the normal) of the listed blocks, and leave guard cells and
    guard faces on both sides as they were."""
    import torch
    t, g = _grid(gb)
    L, nunk, nb = gb.lib(), g.nvar, g.nblocks
    leaves = np.ascontiguousarray(t["leaf"][::2], np.int32)
    lp = leaves.ctypes.data_as(C.c_void_p)
    host = torch.full((nb, 24, 24, 24, nunk), -7.0, dtype=torch.float64).pin_memory()
    hf = [torch.full(a.shape, -7.0, dtype=torch.float64).pin_memory() for a in (g.fx, g.fy, g.fz)]
    gb.check(L.gb_grid_download_flash_interior_list(C.c_void_p(host.data_ptr()), nunk, _slots(gb, g), len(leaves),
                                                    lp, None), "down")
    gb.check(L.gb_grid_download_faces_interior_list(*[C.c_void_p(h.data_ptr()) for h in hf], len(leaves), lp, None),
             "faces down")
    torch.cuda.synchronize()
    mask = np.zeros(nb, bool)
    mask[leaves] = True
    inner = (slice(4, 20),) * 3
    cells = torch.zeros((24, 24, 24), dtype=torch.bool)
    cells[inner] = True
    full = g.u.permute(0, 2, 3, 4, 1).cpu()   # [b, k, j, i, v]
    assert torch.equal(host[mask][:, cells], full[mask][:, cells])
    assert (host[mask][:, ~cells] == -7.0).all() and (host[~mask] == -7.0).all()
    owned = []
    for a, (h, d) in enumerate(zip(hf, (g.fx, g.fy, g.fz))):
        o = torch.zeros(d.shape[1:], dtype=torch.bool)
        sl = [slice(4, 20)] * 3
        sl[2 - a] = slice(4, 21)  # arrays are [k, j, i]: the normal axis of face a is 2 - a
        o[tuple(sl)] = True
        owned.append(o)
        assert torch.equal(h[mask][:, o], d.cpu()[mask][:, o])
        assert (h[mask][:, ~o] == -7.0).all() and (h[~mask] == -7.0).all()
    # upload changed interiors: the store's interiors change, its guards do not
    ref_u, ref_f = g.u.clone(), [a.clone() for a in (g.fx, g.fy, g.fz)]
    host[mask] *= 2.0
    for h in hf:
        h[mask] += 1.0
    gb.check(L.gb_grid_upload_flash_interior_list(C.c_void_p(host.data_ptr()), nunk, _slots(gb, g), len(leaves),
                                                  lp, None), "up")
    gb.check(L.gb_grid_upload_faces_interior_list(*[C.c_void_p(h.data_ptr()) for h in hf], len(leaves), lp, None),
             "faces up")
    torch.cuda.synchronize()
    m = torch.as_tensor(mask, device="cuda")
    cm = cells.cuda()
    after = g.u.permute(0, 2, 3, 4, 1)
    before = ref_u.permute(0, 2, 3, 4, 1)
    assert torch.equal(after[m][:, cm], 2.0 * before[m][:, cm])
    assert torch.equal(after[m][:, ~cm], before[m][:, ~cm])
    assert torch.equal(g.u[~m], ref_u[~m])
    for a, r, o in zip((g.fx, g.fy, g.fz), ref_f, owned):
        oc = o.cuda()
        assert torch.equal(a[m][:, oc], r[m][:, oc] + 1.0)
        assert torch.equal(a[m][:, ~oc], r[m][:, ~oc])
        assert torch.equal(a[~m], r[~m])
