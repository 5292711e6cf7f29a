"""ctypes mirrors of include/cl2pt_types.h and helpers that build them from
numpy arrays (the arrays are kept alive on the returned object)."""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

MAX_BINS = 20

IA_NLA, IA_TATT = 0, 1
NO_IA, IA_NLA_LF, IA_REDSHIFT_BINNING, IA_REDSHIFT_EVOLUTION = 0, 1, 2, 3
PROBE_XI, PROBE_GAMMAT, PROBE_WTHETA = 1, 2, 4

_dp = C.POINTER(C.c_double)


class Config(C.Structure):
    _fields_ = [
        ("n_source", C.c_int), ("n_lens", C.c_int), ("ntheta", C.c_int),
        ("theta_min_arcmin", C.c_double), ("theta_max_arcmin", C.c_double),
        ("lmax", C.c_int), ("n_ell", C.c_int), ("n_a", C.c_int),
        ("nl_nchi", C.c_int), ("high_def_integration", C.c_int),
        ("lmin_tab", C.c_int), ("lmax_nolimber", C.c_int),
        ("a_min", C.c_double), ("adopt_limber_gg", C.c_int),
        ("ia_model", C.c_int), ("ia_mode", C.c_int),
        ("bias_model", C.c_int * 6), ("linear_pk", C.c_int),
        ("probes", C.c_int), ("n_ggl_exclude", C.c_int),
        ("ggl_exclude", C.c_int * (2 * MAX_BINS * MAX_BINS)),
        ("one_loop_bias", C.c_int),
    ]


class Cosmo(C.Structure):
    _fields_ = [
        ("omega_m", C.c_double), ("h0", C.c_double),
        ("chi_nz", C.c_int), ("chi_z", _dp), ("chi", _dp),
        ("G_nz", C.c_int), ("G_z", _dp), ("G", _dp),
        ("pk_nk", C.c_int), ("pk_nz", C.c_int),
        ("pk_log10k", _dp), ("pk_z", _dp), ("lnP", _dp),
        ("pkl_nk", C.c_int), ("pkl_nz", C.c_int),
        ("pkl_log10k", _dp), ("pkl_z", _dp), ("lnPL", _dp),
    ]


class NZ(C.Structure):
    _fields_ = [("nzbins", C.c_int), ("ntomo", C.c_int), ("table", _dp)]


class Nuisance(C.Structure):
    _fields_ = [
        ("src_dz", C.c_double * MAX_BINS),
        ("lens_dz", C.c_double * MAX_BINS),
        ("lens_stretch", C.c_double * MAX_BINS),
        ("shear_m", C.c_double * MAX_BINS),
        ("gb", (C.c_double * MAX_BINS) * 6),
        ("ia", (C.c_double * MAX_BINS) * 3),
    ]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def make_config(n_source=5, n_lens=5, ntheta=20, theta_min=2.5, theta_max=250.0,
                lmax=50000, n_ell=300, n_a=225, nl_nchi=500, hdi=0,
                lmin_tab=20, lmax_nolimber=150, a_min=1.0 / 41.0,
                adopt_limber_gg=0, ia_model=IA_NLA, ia_mode=NO_IA,
                bias_model=(0, 0, 0, 0, 0, 0), linear_pk=0,
                probes=PROBE_XI | PROBE_GAMMAT | PROBE_WTHETA,
                ggl_exclude=(), one_loop_bias=0) -> Config:
    c = Config()
    c.n_source, c.n_lens, c.ntheta = n_source, n_lens, ntheta
    c.theta_min_arcmin, c.theta_max_arcmin = theta_min, theta_max
    c.lmax, c.n_ell, c.n_a, c.nl_nchi = lmax, n_ell, n_a, nl_nchi
    c.high_def_integration = hdi
    c.lmin_tab, c.lmax_nolimber, c.a_min = lmin_tab, lmax_nolimber, a_min
    c.adopt_limber_gg, c.ia_model, c.ia_mode = adopt_limber_gg, ia_model, ia_mode
    for i, b in enumerate(bias_model):
        c.bias_model[i] = b
    c.linear_pk, c.probes = linear_pk, probes
    c.one_loop_bias = one_loop_bias
    c.n_ggl_exclude = len(ggl_exclude)
    for i, (zl, zs) in enumerate(ggl_exclude):
        c.ggl_exclude[2 * i] = zl
        c.ggl_exclude[2 * i + 1] = zs
    return c


@dataclasses.dataclass
class CosmoHandle:
    """A Cosmo struct plus the arrays it points into."""
    struct: Cosmo
    arrays: tuple


def make_cosmo(t) -> CosmoHandle:
    """Build a Cosmo struct from a cl2pt.synthetic.CosmoTables-like object."""
    arrs = tuple(np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in
                 (t.chi_z, t.chi, t.G_z, t.G, t.log10k, t.pk_z, t.lnP, t.lnPL))
    chi_z, chi, G_z, G, lk, pz, lnP, lnPL = arrs
    s = Cosmo()
    s.omega_m, s.h0 = t.omega_m, t.h0
    s.chi_nz, s.chi_z, s.chi = len(chi_z), dptr(chi_z), dptr(chi)
    s.G_nz, s.G_z, s.G = len(G_z), dptr(G_z), dptr(G)
    s.pk_nk, s.pk_nz = len(lk), len(pz)
    s.pk_log10k, s.pk_z, s.lnP = dptr(lk), dptr(pz), dptr(lnP)
    s.pkl_nk, s.pkl_nz = len(lk), len(pz)
    s.pkl_log10k, s.pkl_z, s.lnPL = dptr(lk), dptr(pz), dptr(lnPL)
    return CosmoHandle(s, arrs)


@dataclasses.dataclass
class NZHandle:
    struct: NZ
    table: np.ndarray


def make_nz(table: np.ndarray) -> NZHandle:
    t = np.ascontiguousarray(table, dtype=np.float64)
    s = NZ()
    s.nzbins, s.ntomo, s.table = t.shape[0], t.shape[1] - 1, dptr(t)
    return NZHandle(s, t)


def make_nuisance(src_dz=(), lens_dz=(), lens_stretch=(), shear_m=(),
                  b1=(), b2=(), bs2=(), b3=(), bmag=(), bk=(),
                  ia=None) -> Nuisance:
    n = Nuisance()
    for i in range(MAX_BINS):
        n.lens_stretch[i] = 1.0
    for arr, name in ((src_dz, "src_dz"), (lens_dz, "lens_dz"),
                      (lens_stretch, "lens_stretch"), (shear_m, "shear_m")):
        dst = getattr(n, name)
        for i, v in enumerate(arr):
            dst[i] = float(v)
    for k, arr in enumerate((b1, b2, bs2, b3, bmag, bk)):
        for i, v in enumerate(arr):
            n.gb[k][i] = float(v)
    if ia is not None:
        for k, row in enumerate(ia):
            for i, v in enumerate(row):
                n.ia[k][i] = float(v)
    return n


def nuisance_to_array(n: Nuisance) -> np.ndarray:
    """Flat float64 view of a Nuisance struct (13 x MAX_BINS values)."""
    return np.frombuffer(bytes(n), dtype=np.float64).copy()


def n_pairs(cfg: Config):
    """(P_ss, P_gs, P_gg) in the reference's ordering conventions."""
    ns, nl = cfg.n_source, cfg.n_lens
    excl = {(cfg.ggl_exclude[2 * i], cfg.ggl_exclude[2 * i + 1]) for i in range(cfg.n_ggl_exclude)}
    pgs = sum(1 for i in range(nl) for j in range(ns) if (i, j) not in excl)
    return ns * (ns + 1) // 2, pgs, nl


def shear_pairs(ns):
    return [(i, j) for i in range(ns) for j in range(i, ns)]


def ggl_pairs(cfg: Config):
    excl = {(cfg.ggl_exclude[2 * i], cfg.ggl_exclude[2 * i + 1]) for i in range(cfg.n_ggl_exclude)}
    return [(i, j) for i in range(cfg.n_lens) for j in range(cfg.n_source) if (i, j) not in excl]
