"""Named 2-point workloads with seeded synthetic inputs.

  cosmic_shear_fourier   5 source bins -> 15 shear spectra at 20 log-spaced
                         l in 20-3000; P(k,z) 400 x 100
  real_3x2pt             10 source + 5 lens bins -> 55 xi+/xi-, 50 gamma_t,
                         5 w(theta) spectra on 20 log theta bins in
                         2.5-250 arcmin, Legendre sums to l = 50000 from
                         1000 log-spaced C_l nodes; P(k,z) 600 x 200;
                         b1 ~ U(1.2, 2.2); non-Limber w(theta)
  real_3x2pt_small       a reduced real_3x2pt (4 + 3 bins, 10 theta bins,
                         l <= 5000, 200 nodes) for fast checks, whose
                         nonlinear table carries a small-scale boost over
                         the linear one (the reduced workloads pass both)
  cmb_lensing[_tatt]_small the 6x2pt CMB-lensing spectra C_gk, C_ks, C_kk of
                         real_3x2pt[_tatt]_small's samples at 16 log-spaced
                         l in 2-5000, on distance tables to z = 1100
  real_3x2pt_tatt[_small] the same with TATT intrinsic alignments
                         (redshift evolution: A1, A2, eta, b_TA) and
                         nonlinear galaxy bias (b2, bs2)
  fourier_serving        batched sampler serving: Fourier 3x2pt, 10 source
                         + 10 lens bins, 26 log-spaced l bins in 20-15000,
                         non-Limber clustering below l = 200 with the FFTLog
                         on 2048 log-chi points; per-point scale cuts
                         (scale_cuts) keep 40-100% of each data vector
  fourier_serving_small  a reduced serving workload (4 + 3 bins, 500 chi
                         points) for fast checks
  real_3x2pt_small_nla   real_3x2pt_small with NLA intrinsic alignments in
                         the redshift-evolution mode (A1 ~ U(0.3, 1),
                         eta ~ U(-1.5, 1.5)), lens photo-z stretch
                         ~ U(0.9, 1.1) and b1 evolving as (1+z)/(1+<z>)
                         (bias model 1)
  real_3x2pt_small_nlabin real_3x2pt_small with NLA in the redshift-binning
                         mode (A1 ~ U(-1, 1) per source bin), lens stretch
                         and the growth-scaled b1 of bias model 2
  real_3x2pt_small_hdi   real_3x2pt_small with high_def_integration = 1
                         (larger Gauss-Legendre sets) and the ggl pairs
                         (lens 0, source 3) and (lens 1, source 2) excluded
  real_3x2pt_small_lin   real_3x2pt_small in the linear run mode (every
                         spectrum from p_lin)

Per-point variation: every walker gets its own P(k,z) amplitude/tilt,
source photo-z shifts N(0, 0.02), shear calibration N(0, 0.01) and lens
biases, so each point carries distinct tables and nuisances.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import abi, synthetic

SEED0 = 20261203


@dataclasses.dataclass
class Workload:
    name: str
    cfg: abi.Config
    src: np.ndarray
    lens: np.ndarray
    base: synthetic.CosmoTables
    ell: np.ndarray | None = None  # Fourier multipoles
    tatt: bool = False             # TATT IA + nonlinear galaxy bias nuisances
    nla: bool = False              # NLA amplitudes and lens stretch drawn per point


def _fourier_ells(nell, lmin, lmax):
    # init_binning_fourier (generic_interface.cpp:448-456)
    logdl = (np.log(lmax) - np.log(lmin)) / nell
    return np.exp(np.log(lmin) + (np.arange(nell) + 0.5) * logdl)


def make(name: str) -> Workload:
    if name == "cosmic_shear_fourier":
        cfg = abi.make_config(n_source=5, n_lens=1, probes=abi.PROBE_XI)
        base = synthetic.make_cosmo_tables(nk=400, nz=100)
        return Workload(name, cfg, synthetic.source_nz(5), synthetic.lens_nz(1), base,
                        _fourier_ells(20, 20.0, 3000.0))
    if name == "real_3x2pt":
        cfg = abi.make_config(n_source=10, n_lens=5, ntheta=20, theta_min=2.5,
                              theta_max=250.0, lmax=50000, n_ell=1000)
        base = synthetic.make_cosmo_tables(nk=600, nz=200)
        return Workload(name, cfg, synthetic.source_nz(10), synthetic.lens_nz(5), base)
    if name == "real_3x2pt_limber":
        w = make("real_3x2pt")
        w.cfg.adopt_limber_gg = 1
        w.name = name
        return w
    if name == "real_3x2pt_small":
        cfg = abi.make_config(n_source=4, n_lens=3, ntheta=10, theta_min=2.5,
                              theta_max=250.0, lmax=5000, n_ell=200)
        base = synthetic.make_cosmo_tables(nk=400, nz=100, nl_boost=True)
        return Workload(name, cfg, synthetic.source_nz(4), synthetic.lens_nz(3), base)
    if name in ("cmb_lensing_small", "cmb_lensing_tatt_small"):
        # the 6x2pt CMB-lensing spectra: real_3x2pt_small's samples (with
        # TATT and one-loop galaxy bias in the _tatt case) on distance and
        # growth tables that reach the last-scattering surface
        w = make(name.replace("cmb_lensing", "real_3x2pt"))
        w.base = synthetic.make_cosmo_tables(nk=400, nz=100, nl_boost=True, z_max=1100.0)
        w.ell = _fourier_ells(16, 2.0, 5000.0)
        w.name = name
        return w
    if name == "real_3x2pt_small_limber":
        w = make("real_3x2pt_small")
        w.cfg.adopt_limber_gg = 1
        w.name = name
        return w
    if name == "fourier_serving":
        cfg = abi.make_config(n_source=10, n_lens=10, lmax_nolimber=200, nl_nchi=2048)
        base = synthetic.make_cosmo_tables(nk=600, nz=200)
        return Workload(name, cfg, synthetic.source_nz(10), synthetic.lens_nz(10), base,
                        _fourier_ells(26, 20.0, 15000.0))
    if name == "fourier_serving_small":
        cfg = abi.make_config(n_source=4, n_lens=3, lmax_nolimber=200, nl_nchi=500, lmax=20000,
                              n_ell=200)
        base = synthetic.make_cosmo_tables(nk=400, nz=100, nl_boost=True)
        return Workload(name, cfg, synthetic.source_nz(4), synthetic.lens_nz(3), base,
                        _fourier_ells(12, 20.0, 15000.0))
    if name in ("real_3x2pt_tatt", "real_3x2pt_tatt_small"):
        # the differentiable-3x2pt layout: real_3x2pt plus TATT intrinsic
        # alignments (redshift-evolution mode) and nonlinear galaxy bias
        w = make(name.replace("_tatt", ""))
        w.cfg.ia_model = abi.IA_TATT
        w.cfg.ia_mode = abi.IA_REDSHIFT_EVOLUTION
        w.cfg.one_loop_bias = 1
        w.name = name
        w.tatt = True
        return w
    if name == "real_3x2pt_small_hdi":
        w = make("real_3x2pt_small")
        w.cfg.high_def_integration = 1
        ex = [(0, 3), (1, 2)]
        w.cfg.n_ggl_exclude = len(ex)
        for i, (zl, zs) in enumerate(ex):
            w.cfg.ggl_exclude[2 * i] = zl
            w.cfg.ggl_exclude[2 * i + 1] = zs
        w.name = name
        return w
    if name == "real_3x2pt_small_lin":
        w = make("real_3x2pt_small")
        w.cfg.linear_pk = 1
        w.name = name
        return w
    if name in ("real_3x2pt_small_nla", "real_3x2pt_small_nlabin"):
        w = make("real_3x2pt_small")
        binned = name.endswith("bin")
        w.cfg.ia_model = abi.IA_NLA
        w.cfg.ia_mode = abi.IA_REDSHIFT_BINNING if binned else abi.IA_REDSHIFT_EVOLUTION
        w.cfg.bias_model[0] = 2 if binned else 1
        w.name = name
        w.nla = True
        return w
    raise KeyError(name)


def points(w: Workload, n: int, seed: int = 0, vary_cosmo: bool = True, bmag: bool = False):
    """n parameter points: (list of CosmoTables, list of abi.Nuisance).
    bmag: also draw a magnification bias bmag ~ U(-1, 3) per lens bin (from
    a stream of its own, so the other draws do not change)."""
    rng = np.random.default_rng(SEED0 + seed)
    rng_m = np.random.default_rng(SEED0 + 900 + seed)
    rng_a = np.random.default_rng(SEED0 + 950 + seed)
    ns, nl = w.cfg.n_source, w.cfg.n_lens
    tabs, nus = [], []
    for _ in range(n):
        t = synthetic.perturb_tables(w.base, rng) if vary_cosmo else w.base
        extra = {}
        if w.tatt:
            # A1 ~ U(-1, 1), A2 ~ U(-2, 2), eta ~ U(-2, 2) (both IA powers),
            # b_TA ~ U(0, 2); b2, bs2 ~ U(-1, 1) per lens bin
            eta = rng.uniform(-2.0, 2.0)
            extra = dict(ia=[[rng.uniform(-1.0, 1.0), eta], [rng.uniform(-2.0, 2.0), eta],
                             [rng.uniform(0.0, 2.0)]],
                         b2=rng.uniform(-1.0, 1.0, nl), bs2=rng.uniform(-1.0, 1.0, nl))
        nu = abi.make_nuisance(
            src_dz=rng.normal(0.0, 0.02, ns),
            lens_dz=rng.normal(0.0, 0.005, nl),
            shear_m=rng.normal(0.0, 0.01, ns),
            b1=rng.uniform(1.2, 2.2, nl),
            **extra,
        )
        if bmag:
            for q, v in enumerate(rng_m.uniform(-1.0, 3.0, nl)):
                nu.gb[4][q] = float(v)
        if w.nla:
            if w.cfg.ia_mode == abi.IA_REDSHIFT_BINNING:
                for s_, v in enumerate(rng_a.uniform(-1.0, 1.0, ns)):
                    nu.ia[0][s_] = float(v)
            else:
                nu.ia[0][0] = float(rng_a.uniform(0.3, 1.0))
                nu.ia[0][1] = float(rng_a.uniform(-1.5, 1.5))
            for q, v in enumerate(rng_a.uniform(0.9, 1.1, nl)):
                nu.lens_stretch[q] = float(v)
        tabs.append(t)
        nus.append(nu)
    return tabs, nus


def scale_cuts(w: Workload, n: int, seed: int = 0):
    """Per-point scale cuts of a Fourier workload as CSR lists (row_ptr
    [n+1], idx [nnz]): point i draws a kept fraction f ~ U(0.4, 1) and keeps
    the lowest round(f nell) (at least 1) multipole bins of every spectrum."""
    rng = np.random.default_rng(SEED0 + 50 + seed)
    pss, pgs, pgg = abi.n_pairs(w.cfg)
    nell = len(w.ell)
    nspec = pss + pgs + w.cfg.n_lens
    ptr, idx = [0], []
    for _ in range(n):
        m = max(1, int(round(rng.uniform(0.4, 1.0) * nell)))
        for sp in range(nspec):
            idx.extend(sp * nell + np.arange(m))
        ptr.append(len(idx))
    return np.asarray(ptr, dtype=np.int32), np.asarray(idx, dtype=np.int32)


def scale_cut_requests():
    """Requests of the scale-cut diagnostics tests: a (k, l) grid for
    dC_ss/dlnk, (kmax, l) pairs for RF_C_ss, a 60-node
    ln k grid on [1e-5, 1e2] h/Mpc for the real-space dlnxi/dlnk (the
    reference's Ntable.dCX_dlnk_* with 60 instead of 190 nodes), and kmax
    values for RF_xi."""
    return dict(k=np.exp(np.linspace(np.log(1e-3), np.log(30.0), 23)),
                l=np.array([2.0, 10.0, 37.5, 150.0, 800.0, 4000.0]),
                pairs=[(0, 0), (0, 3), (2, 3), (3, 3)],
                rf_kmax=np.array([0.05, 0.3, 1.0, 5.0]), rf_l=np.array([30.0, 200.0, 1000.0, 300.0]),
                nlnk=60, kmin=1e-5, kmax=1e2, xi_kmax=np.array([0.05, 0.3, 1.0, 5.0]))


def baryon_scenarios(n: int = 4):
    """n synthetic baryon-feedback scenarios standing in for the hydro
    simulations the reference reads (PkRatio_baryons tables): log10 of a
    smooth suppression 1 - A x(k) a^p with x(k) a tanh step at log10 k0
    and width w, per scenario (A, k0, w, p) spread over (0.1-0.3, -0.3-0.6,
    0.25-0.45, 0.3-1.2), plus a small seeded bump; on a (log10 k [h/Mpc], a)
    grid of 41 x 16 that the P(k, z) tables exceed on both sides."""
    lk = np.linspace(-2.5, 1.5, 41)
    a = np.linspace(0.25, 1.0, 16)
    rng = np.random.default_rng(SEED0 + 91)
    out = []
    for i in range(n):
        t = i / max(n - 1, 1)
        A, k0, wd, pw = 0.1 + 0.2 * t, -0.3 + 0.9 * t, 0.25 + 0.2 * (1 - t), 0.3 + 0.9 * t
        x = 0.5 * (1.0 + np.tanh((lk - k0) / wd))
        bump = 0.02 * rng.uniform(0.5, 1.0) * np.exp(-0.5 * ((lk - rng.uniform(-0.5, 0.5)) / 0.3) ** 2)
        out.append(np.log10(1.0 - A * x[None, :] * a[:, None] ** pw) + bump[None, :] * a[:, None])
    return lk, a, np.ascontiguousarray(np.stack(out))


def cmb_map_filter():
    """The CMB map filter of the real-space CMB-lensing cross-correlations
    (init_cmb_cross_correlation's arguments): l in [2, 3000], a 5 arcmin
    Gaussian beam, and a smooth stand-in for the HEALPix pixel window,
    exp(-(l / 4000)^2) for l < 4500 (the reference reads the window of the
    survey's nside from a file; none ships with it)."""
    return dict(lmin=2, lmax=3000, fwhm_arcmin=5.0,
                healpixwin=np.exp(-(np.arange(4500) / 4000.0) ** 2))


def cmb_kk_bandpowers():
    """A kk bandpower binning of the shape the reference reads from its
    binning-matrix file: 8 log-spaced top-hat bands over L = 8..2000 with
    weights 1/width, and a small seeded theory offset per band."""
    lminbp, lmaxbp, nbp = 8, 2000, 8
    edges = np.unique(np.round(np.geomspace(lminbp, lmaxbp + 1, nbp + 1)).astype(int))
    L = np.arange(lminbp, lmaxbp + 1)
    M = np.zeros((len(edges) - 1, len(L)))
    for j in range(len(edges) - 1):
        sel = (L >= edges[j]) & (L < edges[j + 1])
        M[j, sel] = 1.0 / sel.sum()
    off = np.random.default_rng(SEED0 + 77).normal(0.0, 1e-9, len(edges) - 1)
    return lminbp, lmaxbp, M, off


def stack_lin(tabs):
    """The points' linear tables lnPL, [n][nk * nz] (numpy)."""
    return np.stack([np.ascontiguousarray(t.lnPL).reshape(-1) for t in tabs])


def one_table(tabs):
    """The points with the nonlinear table replaced by the linear one (for
    callers that pass a single table, which then also feeds the FAST-PT
    tables)."""
    return [dataclasses.replace(t, lnP=np.ascontiguousarray(t.lnPL.copy())) for t in tabs]


def stack(tabs):
    """Per-point arrays of a batch: omega_m, h0, chi, G, lnP (numpy)."""
    om = np.array([t.omega_m for t in tabs])
    h0 = np.array([t.h0 for t in tabs])
    chi = np.stack([t.chi for t in tabs])
    G = np.stack([t.G for t in tabs])
    lnP = np.stack([t.lnP.reshape(-1) for t in tabs])
    return om, h0, chi, G, lnP


# ------------------------------------------------------------- FAST-PT batch
FASTPT_NK = 2048
FASTPT_KMIN, FASTPT_KMAX = 1e-5, 1e3  # h/Mpc


def fastpt_spectra(n: int, seed: int = 0, nk: int = FASTPT_NK):
    """Batched FAST-PT workload: n linear P(k, z=0) spectra (Eisenstein-Hu
    no-wiggle, sigma_8 normalised) on nk log-spaced k in 1e-5..1e3 h/Mpc,
    each with its own (Omega_m, h, n_s, sigma_8) drawn uniformly from
    [0.25, 0.35] x [0.6, 0.8] x [0.92, 1.0] x [0.7, 0.9].
    Returns (k [nk], P [n][nk], params [n][4])."""
    rng = np.random.default_rng(SEED0 + 3 + seed)
    k = np.geomspace(FASTPT_KMIN, FASTPT_KMAX, nk)
    lo = np.array([0.25, 0.6, 0.92, 0.7])
    hi = np.array([0.35, 0.8, 1.0, 0.9])
    par = lo + (hi - lo) * rng.uniform(size=(n, 4))
    P = np.empty((n, nk))
    for i, (om, h, ns, s8) in enumerate(par):
        P[i] = synthetic.plin_z0(k, synthetic.Cosmo(omega_m=om, h=h, ns=ns, sigma8=s8))
    return k, P, par
