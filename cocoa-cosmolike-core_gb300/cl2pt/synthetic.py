"""Seeded synthetic inputs with the shapes and value distributions of the
2-point workloads (the reference ships no data; every workload here is
synthetic).

Cosmology: flat LCDM, Eisenstein & Hu (1998) no-wiggle transfer function
(their eqs. 26-31, written from the paper), normalised to sigma_8 with an
R = 8 Mpc/h top-hat; linear growth from the exact LCDM integral
D(a) ~ H(a) int_0^a da' / (a' H(a'))^3; comoving distance
chi(z) = (c/H0) int_0^z dz'/E(z') in Mpc/h.

The tables follow the reference setter layouts
(cosmolike/generic_interface.cpp:1085-1267):
  * distances / growth: (z, chi[Mpc/h]) and (z, G = D/a) columns;
  * lnP: row-major [i_k * nz + j_z] on log10(k [h/Mpc]) x z axes;
  * n(z): rows (z, n_1 .. n_N) (cosmolike/generic_interface.cpp:1802-1988).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
from scipy import integrate, special

C_OVER_H0 = 2997.92458  # Mpc/h, cosmology.coverH0 in the reference
T_CMB = 2.7255


@dataclasses.dataclass
class Cosmo:
    omega_m: float = 0.3
    h: float = 0.7
    ns: float = 0.96
    sigma8: float = 0.8
    omega_b: float = 0.05


def eh_nowiggle_transfer(k_hmpc: np.ndarray, c: Cosmo) -> np.ndarray:
    """EH98 zero-baryon-oscillation transfer function, k in h/Mpc."""
    h = c.h
    om = c.omega_m * h * h
    ob = c.omega_b * h * h
    fb = c.omega_b / c.omega_m
    theta = T_CMB / 2.7
    s = 44.5 * np.log(9.83 / om) / np.sqrt(1.0 + 10.0 * ob ** 0.75)  # Mpc
    alpha = 1.0 - 0.328 * np.log(431.0 * om) * fb + 0.38 * np.log(22.3 * om) * fb * fb
    k_mpc = k_hmpc * h
    gamma_eff = c.omega_m * h * (alpha + (1.0 - alpha) / (1.0 + (0.43 * k_mpc * s) ** 4))
    q = k_hmpc * theta * theta / gamma_eff
    L0 = np.log(2.0 * math.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1.0 + 62.5 * q)
    return L0 / (L0 + C0 * q * q)


def _sigma8_raw(c: Cosmo) -> float:
    lnk = np.linspace(np.log(1e-5), np.log(1e3), 20001)
    k = np.exp(lnk)
    pk = k ** c.ns * eh_nowiggle_transfer(k, c) ** 2
    x = 8.0 * k
    w = 3.0 * (np.sin(x) - x * np.cos(x)) / x ** 3
    integrand = k ** 3 * pk * w * w / (2.0 * np.pi ** 2)
    return float(np.sqrt(integrate.trapezoid(integrand, lnk)))


def plin_z0(k_hmpc: np.ndarray, c: Cosmo) -> np.ndarray:
    """Linear P(k, z=0) in (Mpc/h)^3 normalised to sigma_8."""
    amp = (c.sigma8 / _sigma8_raw(c)) ** 2
    return amp * k_hmpc ** c.ns * eh_nowiggle_transfer(k_hmpc, c) ** 2


def efunc(z, c: Cosmo):
    return np.sqrt(c.omega_m * (1.0 + z) ** 3 + (1.0 - c.omega_m))


def growth_D(z: np.ndarray, c: Cosmo) -> np.ndarray:
    """Linear growth D(z) with D(0) = 1 (exact LCDM integral form)."""
    def unnorm(a):
        if a <= 0:
            return 0.0
        f = lambda ap: 1.0 / (ap * efunc(1.0 / ap - 1.0, c)) ** 3
        val, _ = integrate.quad(f, 0.0, a, epsabs=0, epsrel=1e-12, limit=200)
        return efunc(1.0 / a - 1.0, c) * val
    a = 1.0 / (1.0 + np.asarray(z, dtype=np.float64))
    d = np.array([unnorm(x) for x in np.atleast_1d(a)])
    return d / unnorm(1.0)


def chi_of_z(z: np.ndarray, c: Cosmo) -> np.ndarray:
    """Comoving distance in Mpc/h."""
    z = np.asarray(z, dtype=np.float64)
    zf = np.linspace(0.0, float(z.max()), 200001)
    integ = 1.0 / efunc(zf, c)
    cum = integrate.cumulative_trapezoid(integ, zf, initial=0.0)
    return C_OVER_H0 * np.interp(z, zf, cum)


def background_z_grid(z_max: float = 60.0) -> np.ndarray:
    """z grid for the distance and growth tables.  By default it runs to
    z = 60 so that every lookup the 2-point path makes (down to a_min = 1/41,
    z = 40) stays strictly inside the table; the CMB-lensing spectra need
    chi(z = 1090), so their tables run further (z_max)."""
    lo = np.linspace(0.0, 4.5, 1800)
    hi = np.geomspace(4.5, z_max, 201 if z_max <= 60.0 else 301)[1:]
    return np.concatenate([lo, hi])


@dataclasses.dataclass
class CosmoTables:
    omega_m: float
    h0: float  # H0 / 100
    chi_z: np.ndarray
    chi: np.ndarray  # Mpc/h
    G_z: np.ndarray
    G: np.ndarray  # D / a
    log10k: np.ndarray
    pk_z: np.ndarray
    lnP: np.ndarray  # [nk, nz]
    # linear table (identical to lnP unless made with nl_boost)
    lnPL: np.ndarray


def make_cosmo_tables(c: Cosmo = Cosmo(), nk: int = 600, nz: int = 200,
                      log10k_range=(-4.0, 2.0), z_range=(0.0, 4.0), nl_boost: bool = False,
                      z_max: float = 60.0) -> CosmoTables:
    """nl_boost: the nonlinear table is the linear one times a smooth
    small-scale boost 1 + 0.6 (k/k_nl)^1.5, k_nl = 0.25 (1+z)^1.2 h/Mpc
    (a halofit-like shape), so the two tables differ; otherwise they are
    the same."""
    zg = background_z_grid(z_max)
    chi = chi_of_z(zg, c)
    D = growth_D(zg, c)
    G = D * (1.0 + zg)
    log10k = np.linspace(log10k_range[0], log10k_range[1], nk)
    pz = np.linspace(z_range[0], z_range[1], nz)
    p0 = plin_z0(10.0 ** log10k, c)
    Dz = np.interp(pz, zg, D)
    lnPL = np.log(p0)[:, None] + 2.0 * np.log(Dz)[None, :]
    lnP = lnPL.copy()
    if nl_boost:
        x = 10.0 ** log10k[:, None] / (0.25 * (1.0 + pz[None, :]) ** 1.2)
        lnP += np.log1p(0.6 * x ** 1.5)
    return CosmoTables(c.omega_m, c.h, zg, chi, zg.copy(), G, log10k, pz,
                       np.ascontiguousarray(lnP), np.ascontiguousarray(lnPL))


def perturb_tables(base: CosmoTables, rng: np.random.Generator, amp_sigma=0.02) -> CosmoTables:
    """A walker's tables: the base cosmology with a random sigma_8-like
    amplitude and a small random tilt, so each point carries its own
    P(k, z) table."""
    dlnA = rng.normal(0.0, amp_sigma)
    tilt = rng.normal(0.0, 0.01)
    d = 2.0 * dlnA + tilt * (base.log10k[:, None] - 0.0) * math.log(10.0)
    return dataclasses.replace(base, lnP=np.ascontiguousarray(base.lnP + d),
                               lnPL=np.ascontiguousarray(base.lnPL + d))


NZ_ROWS = 300
NZ_ZMAX = 4.0


def _nz_grid():
    return np.arange(NZ_ROWS) * (NZ_ZMAX / NZ_ROWS)


def _window(z, zlo, zhi, sigma):
    s = np.sqrt(2.0) * sigma
    return 0.5 * (special.erf((zhi - z) / s) - special.erf((zlo - z) / s))


def source_nz(nbins: int, sigma0: float = 0.05) -> np.ndarray:
    """Source table rows (z, n_1..n_N): n(z) ~ z^2 exp(-(z/0.5)^1.5) split in
    equal-number true-z bins, each times a Gaussian photo-z window with
    sigma = sigma0 (1 + z)."""
    z = _nz_grid()
    zf = np.linspace(0.0, NZ_ZMAX, 40001)
    nf = zf ** 2 * np.exp(-((zf / 0.5) ** 1.5))
    cdf = integrate.cumulative_trapezoid(nf, zf, initial=0.0)
    cdf /= cdf[-1]
    edges = np.interp(np.linspace(0, 1, nbins + 1), cdf, zf)
    edges[0], edges[-1] = 0.0, NZ_ZMAX
    n = z ** 2 * np.exp(-((z / 0.5) ** 1.5))
    cols = [z]
    for i in range(nbins):
        cols.append(n * _window(z, edges[i], edges[i + 1], sigma0 * (1.0 + z)))
    return np.ascontiguousarray(np.stack(cols, axis=1))


def lens_nz(nbins: int, zlo=0.2, zhi=1.2, sigma0: float = 0.03) -> np.ndarray:
    """Lens table rows (z, n_1..n_N): equal-width top-hats in [zlo, zhi]
    convolved with a Gaussian of sigma = sigma0 (1 + z)."""
    z = _nz_grid()
    edges = np.linspace(zlo, zhi, nbins + 1)
    cols = [z]
    for i in range(nbins):
        cols.append(_window(z, edges[i], edges[i + 1], sigma0 * (1.0 + z)))
    return np.ascontiguousarray(np.stack(cols, axis=1))
