"""Initial fields for periodic 2D decaying turbulence.

A divergence-free random velocity field whose energy spectrum is E(k) ~ k^4 exp(-2 (k/k0)^2)
(peak at |k| = k0 in integer wavenumbers of the periodic box), with seeded random phases,
scaled to a prescribed RMS speed.  The field is built in Fourier space: a random complex
stream function psi_hat with |psi_hat|^2 ~ E(k) / (pi k^3) gives u = (d psi/dy, -d psi/dx), which
is divergence-free by construction.  Host-side numpy; not part of any timed region.
"""
import numpy as np


def random_velocity(n: int, seed: int, k0: float = 8.0, u_rms: float = 0.04, ny: int = None):
    """(ux, uy) float64 arrays of shape (ny, n) on an n x ny periodic lattice."""
    ny = n if ny is None else ny
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(n, d=1.0 / n)
    ky = np.fft.fftfreq(ny, d=1.0 / ny)
    KX, KY = np.meshgrid(kx, ky)
    k = np.sqrt(KX ** 2 + KY ** 2)
    E = np.zeros_like(k)
    nz = k > 0
    E[nz] = k[nz] ** 4 * np.exp(-2.0 * (k[nz] / k0) ** 2)
    # shell energy E(k) dk spread over the ring of circumference 2 pi k; |u_hat| = k |psi_hat|
    amp = np.zeros_like(k)
    amp[nz] = np.sqrt(E[nz] / (2.0 * np.pi * k[nz])) / k[nz]
    phase = np.exp(2j * np.pi * rng.random(k.shape))
    psi_hat = amp * phase
    ux = np.real(np.fft.ifft2(2j * np.pi * KY / ny * psi_hat))
    uy = np.real(np.fft.ifft2(-2j * np.pi * KX / n * psi_hat))
    rms = np.sqrt(np.mean(ux ** 2 + uy ** 2))
    s = u_rms / rms if rms > 0 else 0.0
    return ux * s, uy * s


def pressure_density(ux: np.ndarray, uy: np.ndarray, rho0: float = 1.0, cs2: float = 1.0 / 3.0):
    """Density consistent with an incompressible velocity field: the pressure solves
    lap p = -d_i u_j d_j u_i (periodic, spectral), and rho = rho0 (1 + p / cs2)."""
    ny, nx = ux.shape
    kx = 2j * np.pi * np.fft.fftfreq(nx)
    ky = 2j * np.pi * np.fft.fftfreq(ny)
    KX, KY = np.meshgrid(kx, ky)
    U, V = np.fft.fft2(ux), np.fft.fft2(uy)
    ux_x, ux_y = np.real(np.fft.ifft2(KX * U)), np.real(np.fft.ifft2(KY * U))
    uy_x, uy_y = np.real(np.fft.ifft2(KX * V)), np.real(np.fft.ifft2(KY * V))
    src = -(ux_x * ux_x + 2.0 * ux_y * uy_x + uy_y * uy_y)
    k2 = -(KX * KX + KY * KY).real
    k2[0, 0] = 1.0
    ph = -np.fft.fft2(src) / k2
    ph[0, 0] = 0.0
    p = np.real(np.fft.ifft2(ph))
    return rho0 * (1.0 + p / cs2)


def coarse_grain(field: np.ndarray, factor: int) -> np.ndarray:
    """Block average of a (ny, nx) field over factor x factor blocks."""
    ny, nx = field.shape
    return field.reshape(ny // factor, factor, nx // factor, factor).mean(axis=(1, 3))


def energy_spectrum(ux: np.ndarray, uy: np.ndarray):
    """Shell-summed kinetic energy spectrum (k, E(k)) of a periodic field."""
    ny, nx = ux.shape
    uh = np.fft.fft2(ux) / (nx * ny)
    vh = np.fft.fft2(uy) / (nx * ny)
    e = 0.5 * (np.abs(uh) ** 2 + np.abs(vh) ** 2)
    kx = np.fft.fftfreq(nx, d=1.0 / nx)
    ky = np.fft.fftfreq(ny, d=1.0 / ny)
    k = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    kb = np.rint(k).astype(int)
    spec = np.bincount(kb.ravel(), weights=e.ravel())
    return np.arange(spec.size), spec
