"""Seeded synthetic inputs for the hydro/MHD + cooling step.

No dataset ships with the reference; its production ICs are generated at run
time by utils/ic-generator/turb-sphere.py. These generators follow the
k-space convention of utils/ic-generator/turb-velbox.py:12-45 (uniform
random complex coefficients, a mask (k^2)^(Eslp/4 - 1/2) on kmin <= |k| <=
kmax, inverse FFT, real part). A 3-D power spectrum P(k) ~ k^-4 is Eslp = -2,
i.e. a k^-2 amplitude per mode. Solenoidal fields are Helmholtz-projected in
k-space. Seeds are numpy.random.default_rng(42 + config_id).

Code units: box length 1, mean density 1, uniform pressure 1 (so the sound
speed is sqrt(gamma)), B in Heaviside-Lorentz units (magnetic pressure B^2/2,
plasma beta = 2p/B^2).
"""
from __future__ import annotations

import numpy as np

NXB = 16
NG = 4
NB = NXB + 2 * NG  # 24 cells per padded block side

# cell-variable slots of the block store
VARS = ["DENS", "VELX", "VELY", "VELZ", "PRES", "ENER", "EINT", "MAGX", "MAGY", "MAGZ", "TEMP", "TDUS"]
SLOT = {v: i for i, v in enumerate(VARS)}
NVAR_HYDRO = 7
NVAR_MHD = 10
NVAR_ALL = 12


def _mask(shape, kmin, kmax, eslp):
    axes = [n / 2 - np.abs(np.arange(n, dtype=np.float64) - n / 2) for n in shape]
    mx, my, mz = np.meshgrid(*axes, indexing="ij")
    k2 = mx * mx + my * my + mz * mz
    m = np.zeros_like(k2)
    sel = (k2 >= kmin * kmin) & (k2 <= kmax * kmax) & (k2 > 0)
    m[sel] = k2[sel] ** (0.25 * eslp - 0.5)
    return m


def _spectral(shape, rng):
    return np.sqrt(2.0) * (rng.random(shape) - 0.5) + 1j * np.sqrt(2.0) * (rng.random(shape) - 0.5)


def grf_vector(shape, kmin, kmax, rng, eslp=-2.0, solenoidal=False):
    """Three-component random field with the turb-velbox spectrum."""
    m = _mask(shape, kmin, kmax, eslp)
    s = [_spectral(shape, rng) * m for _ in range(3)]
    if solenoidal:
        kx = np.fft.fftfreq(shape[0]) * shape[0]
        ky = np.fft.fftfreq(shape[1]) * shape[1]
        kz = np.fft.fftfreq(shape[2]) * shape[2]
        KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
        k2 = KX * KX + KY * KY + KZ * KZ
        k2[0, 0, 0] = 1.0
        dot = (s[0] * KX + s[1] * KY + s[2] * KZ) / k2
        s = [s[0] - dot * KX, s[1] - dot * KY, s[2] - dot * KZ]
    return [np.fft.ifftn(c).real for c in s]


def grf_scalar(shape, kmin, kmax, rng, eslp=-2.0):
    f = np.fft.ifftn(_spectral(shape, rng) * _mask(shape, kmin, kmax, eslp)).real
    f -= f.mean()
    return f / f.std()


def global_to_blocks(arrs, nbx, nby, nbz, nvar):
    """Split global (NX, NY, NZ) arrays indexed [x, y, z] into padded block
    storage u[block, var, k, j, i] (guards left zero)."""
    nb = nbx * nby * nbz
    u = np.zeros((nb, nvar, NB, NB, NB))
    for b in range(nb):
        bx, by, bz = b % nbx, (b // nbx) % nby, b // (nbx * nby)
        sl = (slice(bx * NXB, (bx + 1) * NXB), slice(by * NXB, (by + 1) * NXB),
              slice(bz * NXB, (bz + 1) * NXB))
        for v, a in arrs.items():
            u[b, v, NG:NG + NXB, NG:NG + NXB, NG:NG + NXB] = a[sl].transpose(2, 1, 0)
    return u


def faces_to_blocks(bxf, byf, bzf, nbx, nby, nbz):
    """Global periodic face fields (bxf[i, j, k] = B_x on the low-x face of
    cell (i, j, k)) -> per-block face arrays with interior faces set."""
    nb = nbx * nby * nbz
    fx = np.zeros((nb, NB, NB, NB + 1))
    fy = np.zeros((nb, NB, NB + 1, NB))
    fz = np.zeros((nb, NB + 1, NB, NB))
    NX, NY, NZ = bxf.shape
    for b in range(nb):
        bx, by, bz = b % nbx, (b // nbx) % nby, b // (nbx * nby)
        ix = (np.arange(NXB + 1) + bx * NXB) % NX
        iy = (np.arange(NXB + 1) + by * NXB) % NY
        iz = (np.arange(NXB + 1) + bz * NXB) % NZ
        cy = np.arange(NXB) + by * NXB
        cz = np.arange(NXB) + bz * NXB
        cx = np.arange(NXB) + bx * NXB
        fx[b, NG:NG + NXB, NG:NG + NXB, NG:NG + NXB + 1] = bxf[np.ix_(ix, cy, cz)].transpose(2, 1, 0)
        fy[b, NG:NG + NXB, NG:NG + NXB + 1, NG:NG + NXB] = byf[np.ix_(cx, iy, cz)].transpose(2, 1, 0)
        fz[b, NG:NG + NXB + 1, NG:NG + NXB, NG:NG + NXB] = bzf[np.ix_(cx, cy, iz)].transpose(2, 1, 0)
    return fx, fy, fz


def turbulent_box(nbx, nby, nbz, seed, sigma_ln=0.5, mach=2.0, mhd=False, beta=1.0,
                  dA=0.1, kmin=1, kmax=8, gamma=5.0 / 3.0, solenoidal=None, nvar=None):
    """Periodic turbulent box of nbx*nby*nbz blocks.

    Returns dict(u=[nb, nvar, 24, 24, 24], fx, fy, fz (mhd) or None, dx).
    Density lognormal exp(sigma g - sigma^2/2), velocity P(k) ~ k^-4
    rescaled to rms Mach `mach`, uniform p = 1; MHD adds a uniform B_z with
    the given beta plus curl of a random edge-centred vector potential whose
    field has rms dA * B0 (divergence-free on faces to round-off)."""
    rng = np.random.default_rng(seed)
    NX, NY, NZ = nbx * NXB, nby * NXB, nbz * NXB
    shape = (NX, NY, NZ)
    if solenoidal is None:
        solenoidal = mhd
    g = grf_scalar(shape, kmin, kmax, rng)
    rho = np.exp(sigma_ln * g - 0.5 * sigma_ln * sigma_ln)
    vx, vy, vz = grf_vector(shape, kmin, kmax, rng, solenoidal=solenoidal)
    p0 = 1.0
    cs = np.sqrt(gamma * p0 / 1.0)
    vrms = np.sqrt(np.mean(vx * vx + vy * vy + vz * vz))
    s = mach * cs / vrms
    vx, vy, vz = vx * s, vy * s, vz * s
    pres = np.full(shape, p0)
    eint = pres / ((gamma - 1.0) * rho)
    ener = eint + 0.5 * (vx * vx + vy * vy + vz * vz)
    if nvar is None:
        nvar = NVAR_MHD if mhd else NVAR_HYDRO
    arrs = {0: rho, 1: vx, 2: vy, 3: vz, 4: pres, 5: ener, 6: eint}
    dx = 1.0 / NX
    out = dict(dx=dx, nbx=nbx, nby=nby, nbz=nbz, gamma=gamma, fx=None, fy=None, fz=None)
    if mhd:
        B0 = np.sqrt(2.0 * p0 / beta)
        ax, ay, az = grf_vector(shape, kmin, kmax, rng)
        # edge-centred A: ax on (i, j-1/2, k-1/2) etc.; faces from exact
        # discrete curl on the periodic lattice
        def d(a, axis):
            return (np.roll(a, -1, axis) - a) / dx
        bxf = d(az, 1) - d(ay, 2)
        byf = d(ax, 2) - d(az, 0)
        bzf = d(ay, 0) - d(ax, 1)
        brms = np.sqrt(np.mean(bxf ** 2 + byf ** 2 + bzf ** 2))
        sc = dA * B0 / brms
        bxf, byf, bzf = bxf * sc, byf * sc, bzf * sc + B0
        bcx = 0.5 * (bxf + np.roll(bxf, -1, 0))
        bcy = 0.5 * (byf + np.roll(byf, -1, 1))
        bcz = 0.5 * (bzf + np.roll(bzf, -1, 2))
        arrs.update({7: bcx, 8: bcy, 9: bcz})
        out["fx"], out["fy"], out["fz"] = faces_to_blocks(bxf, byf, bzf, nbx, nby, nbz)
    out["u"] = global_to_blocks(arrs, nbx, nby, nbz, nvar)
    return out
