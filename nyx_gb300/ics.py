"""Seeded cosmological initial conditions for the PM step.

One particle per lattice cell at the cell centre, displaced by the Zel'dovich
approximation from a Gaussian random field with power spectrum P(k) ~ k^slope,
velocities from linear growth.  This follows the placement and velocity
convention of Nyx's 1-particle-per-cell cosmological start
(Source/Particle/DarkMatterParticleContainer.cpp:370-397: pos = plo + (i+1/2)dx
+ displacement; Source/Initialization/Nyx_initcosmo.cpp:286-289: velocity =
displacement * a * H(a), H in km/s/Mpc), in Nyx code units (Mpc, M_sun, km/s).
The particle mass gives the mean matter density Omega_M * rho_crit.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# Source/Driver/constants_cosmo.H:7-16
_M_UNIT = 1.98848e33
_L_UNIT = 3.0856776e24
_V_UNIT = 1.0e5
_T_UNIT = _L_UNIT / _V_UNIT
GCONST = 6.67408e-8 * _M_UNIT * _T_UNIT * _T_UNIT / (_L_UNIT * _L_UNIT * _L_UNIT)
HUBBLE_CONST = 100.0


@dataclass
class Cosmology:
    OmM: float = 1.0
    OmR: float = 0.0
    h: float = 0.675

    @property
    def OmL(self) -> float:
        return 1.0 - self.OmM - self.OmR

    def hubble(self, a: float) -> float:
        """H(a) in km/s/Mpc."""
        return self.h * HUBBLE_CONST * math.sqrt(self.OmM / a ** 3 + self.OmR / a ** 4 + self.OmL)

    def rho_crit(self) -> float:
        H0 = self.h * HUBBLE_CONST
        return 3.0 * H0 * H0 / (8.0 * math.pi * GCONST)


@dataclass
class InitialConditions:
    pos: np.ndarray      # (np, 3) float64, in [0, L)
    vel: np.ndarray      # (np, 3) float64, km/s (a * dx/dt)
    mass: float          # M_sun, identical for all particles
    n: int               # grid cells per dimension
    L: float             # box length, Mpc
    a: float             # scale factor of the ICs
    lattice: np.ndarray  # (np, 3) float64, unperturbed lattice position


def displacement_field(n: int, L: float, slope: float, seed: int) -> np.ndarray:
    """Unit-normalised Zel'dovich displacement psi (3, n, n, n), div psi = -delta."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n, n, n))
    wk = np.fft.rfftn(white)
    kf = 2.0 * np.pi / L
    kx = np.fft.fftfreq(n, d=1.0 / n) * kf
    kz = np.fft.rfftfreq(n, d=1.0 / n) * kf
    KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
    k2 = KX * KX + KY * KY + KZ * KZ
    k2[0, 0, 0] = 1.0
    amp = np.power(np.sqrt(k2), 0.5 * slope)
    amp[0, 0, 0] = 0.0
    dk = wk * amp
    psi = np.empty((3, n, n, n))
    for d, K in enumerate((KX, KY, KZ)):
        psi[d] = np.fft.irfftn(1j * K / k2 * dk, s=(n, n, n), axes=(0, 1, 2))
    rms = math.sqrt(float(np.mean(np.sum(psi * psi, axis=0))))
    if rms > 0:
        psi /= rms
    # array axes are (x, y, z); the particle lattice below is x-fastest
    return psi


def _zeldovich_ics_on_device(n, L, slope, seed, a_init, rms_disp_cells, cosmo, device):
    """zeldovich_ics with the FFTs and the lattice arithmetic on a CUDA device
    (torch), for the large grids of the benchmark: the same white noise (numpy's
    generator, same seed) and the same steps, so the field equals the host
    path's up to the rounding of the FFTs."""
    import torch
    dev = torch.device(device)
    f64 = torch.float64
    rng = np.random.default_rng(seed)
    wk = torch.fft.rfftn(torch.from_numpy(rng.standard_normal((n, n, n))).to(dev))
    kf = 2.0 * np.pi / L
    kx = torch.fft.fftfreq(n, d=1.0 / n, dtype=f64, device=dev) * kf
    kz = torch.fft.rfftfreq(n, d=1.0 / n, dtype=f64, device=dev) * kf
    KX, KY, KZ = kx[:, None, None], kx[None, :, None], kz[None, None, :]
    k2 = KX * KX + KY * KY + KZ * KZ
    k2[0, 0, 0] = 1.0
    amp = torch.pow(torch.sqrt(k2), 0.5 * slope)
    amp[0, 0, 0] = 0.0
    dk = wk * amp
    del wk, amp
    psi = torch.empty((3, n, n, n), dtype=f64, device=dev)
    for d, K in enumerate((KX, KY, KZ)):
        psi[d] = torch.fft.irfftn(1j * K / k2 * dk, s=(n, n, n), dim=(0, 1, 2))
    del dk, k2
    rms = float(torch.sqrt(torch.mean(torch.sum(psi * psi, dim=0))))
    if rms > 0:
        psi *= (rms_disp_cells * L / n) / rms
    # array axes are (x, y, z); particles are x-fastest (z, y, x order of the axes)
    disp = psi.permute(0, 3, 2, 1).reshape(3, -1).t()
    del psi
    idx = (torch.arange(n, dtype=f64, device=dev) + 0.5) * (L / n)
    lattice = torch.stack(torch.meshgrid(idx, idx, idx, indexing="ij")[::-1], dim=-1).reshape(-1, 3)
    pos = torch.remainder(lattice + disp, L)
    pos[pos >= L] = 0.0
    vel = disp * (a_init * cosmo.hubble(a_init))
    mass = cosmo.OmM * cosmo.rho_crit() * L ** 3 / pos.shape[0]
    # (np, 3) arrays in row-major order, as the host path returns them
    out = InitialConditions(pos=np.ascontiguousarray(pos.cpu().numpy()),
                            vel=np.ascontiguousarray(vel.cpu().numpy()), mass=mass, n=n, L=L,
                            a=a_init, lattice=np.ascontiguousarray(lattice.cpu().numpy()))
    del pos, vel, lattice, disp
    torch.cuda.empty_cache()
    return out


def zeldovich_ics(n: int, L: float = 1.0, slope: float = -2.0, seed: int = 1,
                  a_init: float = 0.02, rms_disp_cells: float = 0.2,
                  cosmo: Cosmology | None = None, fraction: float = 1.0,
                  npart_1d: int | None = None, device: str | None = None) -> InitialConditions:
    """Zel'dovich ICs on an n^3 grid with rms displacement rms_disp_cells * dx.

    fraction < 1 keeps a seeded random subset of ceil(fraction * n^3) lattice
    sites; the particle mass rises so the mean density is unchanged.  device (a
    CUDA device, e.g. "cuda:0") runs the FFTs there (one particle per cell only).
    """
    cosmo = cosmo or Cosmology()
    if device is not None:
        if fraction != 1.0 or npart_1d not in (None, n):
            raise ValueError("the device path makes one particle per cell")
        return _zeldovich_ics_on_device(n, L, slope, seed, a_init, rms_disp_cells, cosmo, device)
    m = npart_1d or n
    psi = displacement_field(m, L, slope, seed) * (rms_disp_cells * L / n)
    dxp = L / m
    idx = np.arange(m, dtype=np.float64)
    # x fastest: lattice index q = i + m*(j + m*k)
    Z, Y, X = np.meshgrid(idx, idx, idx, indexing="ij")
    lattice = np.stack([(X.ravel() + 0.5) * dxp, (Y.ravel() + 0.5) * dxp, (Z.ravel() + 0.5) * dxp],
                       axis=1)
    disp = np.stack([psi[0].transpose(2, 1, 0).ravel(), psi[1].transpose(2, 1, 0).ravel(),
                     psi[2].transpose(2, 1, 0).ravel()], axis=1)
    if fraction < 1.0:
        rng = np.random.default_rng(seed + 7919)
        keep = np.sort(rng.choice(lattice.shape[0], size=int(math.ceil(fraction * lattice.shape[0])),
                                  replace=False))
        lattice = lattice[keep]
        disp = disp[keep]
    pos = np.mod(lattice + disp, L)
    pos[pos >= L] = 0.0
    vel = disp * (a_init * cosmo.hubble(a_init))
    mass = cosmo.OmM * cosmo.rho_crit() * L ** 3 / pos.shape[0]
    return InitialConditions(pos=np.ascontiguousarray(pos), vel=np.ascontiguousarray(vel),
                             mass=mass, n=n, L=L, a=a_init, lattice=lattice)
