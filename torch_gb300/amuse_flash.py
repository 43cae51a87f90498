"""The AMUSE-side call surface of Torch's FLASH worker over the device block
store.

Torch's Python host drives FLASH through AMUSE's legacy interface
(src/amuse/torch_amuse_flash/interface.py: evolve_model, get/set_grid_state,
get/set_timestep, ...; implemented in interface.F90 and
base_grid_interface.F90). `FlashCode` offers the same functions, with the
same argument meaning, on a registered `gbhydro.Grid`: each returns its
outputs followed by the int32 error code the legacy function returns (0 on
success). Cell indices are FLASH's: i, j, k 1-based inside the block's
interior, index_of_grid the 1-based block id, nproc the owning process (0
here: one process per GPU, and the entries of other processes stay 0, as
get_grid_state leaves them before its MPI_Reduce). Values are in code units.
"""
from __future__ import annotations

import numpy as np

from . import gbhydro as G


class FlashCode:
    def __init__(self, grid: "G.Grid", cool: bool = True, gamma: float = 5.0 / 3.0, nproc: int = 0):
        self.g = grid
        self.cool = bool(cool)
        self.gamma = gamma
        self.me = nproc
        self.t_end = float("inf")

    # ------------------------------------------------------------ lifecycle
    def initialize_code(self):
        return 0

    def cleanup_code(self):
        return 0

    # ------------------------------------------------------------ time
    def _clock(self):
        return self.g.driver.cpu().numpy()

    def get_time(self):
        """Driver_getSimTime (interface.F90:355-361)."""
        return float(self._clock()[G.Grid.DRV_TIME]), 0

    def get_timestep(self):
        """dr_dt, the last step's dt (interface.F90:371-383)."""
        return float(self._clock()[G.Grid.DRV_DT]), 0

    def set_timestep(self, value):
        """dr_dt = dr_dtInit = value (interface.F90:385-396): here it becomes
        the previous dt that the change-factor limit measures the next one
        against."""
        d = self.g.driver
        d[G.Grid.DRV_DT] = float(value)
        d[G.Grid.DRV_DTOLD] = float(value)
        return 0

    def get_end_time(self):
        return self.t_end, 0

    def set_end_time(self, value):
        self.t_end = float(value)
        return 0

    def evolve_model(self, value):
        """dr_tmax = value; Driver_evolveFlash (interface.F90:451-472):
        whole steps until the clock reaches value, the last one shortened to
        end on it. The clock is read back once per step."""
        d = self.g.driver
        d[G.Grid.DRV_TMAX] = float(value)
        self.t_end = float(value)
        while True:
            t = float(d[G.Grid.DRV_TIME].item())
            if not t < value:
                break
            self.g.step_graph(self.cool)
            if float(d[G.Grid.DRV_DT].item()) <= 0.0:
                return -1  # no progress: dt limited to zero
        return 0

    # ------------------------------------------------------------ grid state
    def _index(self, i, j, k, index_of_grid, nproc, slot):
        i, j, k, b, p = (np.atleast_1d(np.asarray(a, np.int64)) for a in (i, j, k, index_of_grid, nproc))
        mine = p == self.me
        ok = mine & (b >= 1) & (b <= self.g.nblocks) & (i >= 1) & (i <= 16) & (j >= 1) & (j <= 16) & \
            (k >= 1) & (k <= 16)
        if np.any(mine & ~ok):
            raise IndexError("cell index outside a block's interior or block id outside the store")
        N, ng = G.NB, 4
        flat = (((b - 1) * self.g.nvar + slot) * N + (k - 1 + ng)) * N + (j - 1 + ng)
        flat = flat * N + (i - 1 + ng)
        return flat, mine

    def _get(self, idx, slot):
        flat, mine = self._index(*idx, slot)
        out = np.zeros(len(flat))
        if mine.any():
            t = self.g.torch.as_tensor(flat[mine], device=self.g.u.device)
            out[mine] = self.g.u.view(-1)[t].cpu().numpy()
        return out

    def _put(self, idx, slot, vals):
        flat, mine = self._index(*idx, slot)
        if mine.any():
            t = self.g.torch.as_tensor(flat[mine], device=self.g.u.device)
            v = self.g.torch.as_tensor(np.broadcast_to(np.asarray(vals, np.float64), flat.shape)[mine],
                                       device=self.g.u.device)
            self.g.u.view(-1)[t] = v

    def _eos(self, idx):
        """Gamma-law EOS in MODE_DENS_EI on the touched cells: e_int from the
        total specific energy, then p and T."""
        s = self.g.slots
        rho, e = self._get(idx, s["DENS"]), self._get(idx, s["ENER"])
        v2 = sum(self._get(idx, s[n]) ** 2 for n in ("VELX", "VELY", "VELZ"))
        eint = e - 0.5 * v2
        self._put(idx, s["EINT"], eint)
        self._put(idx, s["PRES"], (self.gamma - 1.0) * rho * eint)
        if "TEMP" in s:
            u = G.code_units()
            self._put(idx, s["TEMP"], eint * u["vel_unit"] ** 2 * (self.gamma - 1.0) * (24.0 / 11.0) * G.MP / G.KB)

    def get_grid_state(self, i, j, k, index_of_grid, nproc):
        """(rho, rhovx, rhovy, rhovz, rhoen, 0) (base_grid_interface.F90:404-470)."""
        idx = (i, j, k, index_of_grid, nproc)
        s = self.g.slots
        rho = self._get(idx, s["DENS"])
        out = [rho] + [rho * self._get(idx, s[n]) for n in ("VELX", "VELY", "VELZ", "ENER")]
        return (*out, 0)

    def set_grid_state(self, i, j, k, index_of_grid, nproc, rho, rhovx, rhovy, rhovz, rhoen):
        """DENS, VEL = rhov / rho, ENER = rhoen / rho (base_grid_interface.F90:
        329-362), then the EOS on those cells."""
        idx = (i, j, k, index_of_grid, nproc)
        s = self.g.slots
        rho = np.asarray(rho, np.float64)
        self._put(idx, s["DENS"], rho)
        for n, q in (("VELX", rhovx), ("VELY", rhovy), ("VELZ", rhovz), ("ENER", rhoen)):
            self._put(idx, s[n], np.asarray(q, np.float64) / rho)
        self._eos(idx)
        return 0

    def get_grid_density(self, i, j, k, index_of_grid, nproc):
        return self._get((i, j, k, index_of_grid, nproc), self.g.slots["DENS"]), 0

    def get_grid_velocity(self, i, j, k, index_of_grid, nproc):
        idx = (i, j, k, index_of_grid, nproc)
        return (*[self._get(idx, self.g.slots[n]) for n in ("VELX", "VELY", "VELZ")], 0)

    def set_grid_velocity(self, i, j, k, index_of_grid, nproc, vx, vy, vz):
        idx = (i, j, k, index_of_grid, nproc)
        s = self.g.slots
        e = self._get(idx, s["EINT"])
        for n, q in (("VELX", vx), ("VELY", vy), ("VELZ", vz)):
            self._put(idx, s[n], q)
        v2 = sum(self._get(idx, s[n]) ** 2 for n in ("VELX", "VELY", "VELZ"))
        self._put(idx, s["ENER"], e + 0.5 * v2)
        return 0

    def get_grid_momentum_density(self, i, j, k, index_of_grid, nproc):
        idx = (i, j, k, index_of_grid, nproc)
        rho = self._get(idx, self.g.slots["DENS"])
        return (*[rho * self._get(idx, self.g.slots[n]) for n in ("VELX", "VELY", "VELZ")], 0)

    def get_grid_energy_density(self, i, j, k, index_of_grid, nproc):
        idx = (i, j, k, index_of_grid, nproc)
        return self._get(idx, self.g.slots["DENS"]) * self._get(idx, self.g.slots["ENER"]), 0

    # ------------------------------------------------------------ grid layout
    def get_number_of_grids(self):
        return len(self.g.leaf), 0

    def get_leaf_indices(self):
        """1-based ids of the leaf blocks."""
        return np.asarray(self.g.leaf) + 1, 0

    def get_grid_range(self, index_of_grid):
        return 1, 16, 1, 16, 1, 16, 0

    def get_max_refinement(self):
        return int(self.g.tree["maxlevel"]) + 1, 0
