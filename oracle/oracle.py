"""ctypes front end for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries share this interface:
  * liboracle.so              -- this project's C restatement ("orc_"),
  * _ref/libcosmolike_ref.so  -- the reference's own sources driven by
                                 ref_harness.c ("ref_"); it exists only where
                                 the reference tree was available to build it.
Both keep process-global state, so one process drives one configuration of
the reference library (its pair maps are built once per process).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "cocoa-cosmolike-core_gb300"))
from cl2pt import abi  # noqa: E402

ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcosmolike_ref.so")


def reference_tree() -> str:
    """Root of the reference source tree: $CL2PT_REFERENCE_TREE, else the
    recipe's default (the Makefile's REF)."""
    env = os.environ.get("CL2PT_REFERENCE_TREE")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip()

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """Build liboracle.so (and the reference library when its tree exists)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}"], check=True,
                   stdout=out)
    tree = reference_tree()
    if ref is None:
        ref = bool(tree) and os.path.isdir(os.path.join(tree, "cosmolike"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"-j{os.cpu_count() or 4}",
                        f"REF={tree}"], check=True, stdout=out)


def _p(a):
    return a.ctypes.data_as(_dp)


class Oracle:
    """One loaded oracle library with prefix 'orc' or 'ref'."""

    def __init__(self, which: str = "orc"):
        self.which = which
        path = ORACLE_SO if which == "orc" else REF_SO
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.cfg = None
        self._keep = []
        pre = which + "_"
        d = C.c_double
        for name, args in {
            "nz_source": [d, C.c_int], "nz_lens": [d, C.c_int], "g_tomo": [d, C.c_int],
            "g_lens": [d, C.c_int], "chi": [d], "a_chi": [d], "growfac": [d],
            "f_growth": [d], "p_nonlin": [d, d], "amin_lens": [C.c_int],
            "amax_lens": [C.c_int], "zmean_lens": [C.c_int],
            "C_ss_nointerp": [d, C.c_int, C.c_int, C.c_int],
            "C_gs_nointerp": [d, C.c_int, C.c_int],
            "C_gg_nointerp": [d, C.c_int, C.c_int],
            "C_ss_limber": [d, C.c_int, C.c_int, C.c_int],
            "C_gs_limber": [d, C.c_int, C.c_int], "C_gg_limber": [d, C.c_int],
        }.items():
            f = getattr(self.lib, pre + name)
            f.restype = C.c_double
            f.argtypes = args
            setattr(self, name, f)

    # ---- state
    def setup(self, cfg, src_table, lens_table):
        self.cfg = cfg
        self._src = abi.make_nz(src_table)
        self._lens = abi.make_nz(lens_table)
        st = getattr(self.lib, self.which + "_setup")(C.byref(cfg), C.byref(self._src.struct),
                                                      C.byref(self._lens.struct))
        if st != 0:
            raise RuntimeError(f"setup failed: {st}")

    def set_point(self, tables, nuisance):
        self._cosmo = abi.make_cosmo(tables)
        self._nu = nuisance
        st = getattr(self.lib, self.which + "_set_point")(C.byref(self._cosmo.struct),
                                                          C.byref(nuisance))
        if st != 0:
            raise RuntimeError(f"set_point failed: {st}")

    @property
    def npairs(self):
        return abi.n_pairs(self.cfg)

    # ---- outputs
    def xi_pm(self):
        pss = self.npairs[0]
        nt = self.cfg.ntheta
        xp = np.zeros(pss * nt)
        xm = np.zeros(pss * nt)
        getattr(self.lib, self.which + "_xi_pm")(_p(xp), _p(xm))
        return xp.reshape(pss, nt), xm.reshape(pss, nt)

    def w_gammat(self):
        pgs = self.npairs[1]
        out = np.zeros(pgs * self.cfg.ntheta + 1)
        getattr(self.lib, self.which + "_w_gammat")(_p(out))
        return out[:-1].reshape(pgs, self.cfg.ntheta)

    def w_gg(self):
        pgg = self.npairs[2]
        out = np.zeros(pgg * self.cfg.ntheta + 1)
        getattr(self.lib, self.which + "_w_gg")(_p(out))
        return out[:-1].reshape(pgg, self.cfg.ntheta)

    def C_cl_tomo(self):
        nl, L = self.cfg.n_lens, self.cfg.lmax_nolimber
        out = np.zeros(nl * L)
        f = getattr(self.lib, self.which + "_C_cl_tomo")
        if self.which == "orc":
            conv = np.zeros(nl, dtype=np.int32)
            f(_p(out), conv.ctypes.data_as(_ip))
            return out.reshape(nl, L), conv
        f(_p(out))
        return out.reshape(nl, L), None

    def data_vector_real(self, mask=None, pm=None):
        pss, pgs, pgg = self.npairs
        n = self.cfg.ntheta * (2 * pss + pgs + pgg)
        if mask is None:
            mask = np.ones(n, dtype=np.int32)
        mask = np.ascontiguousarray(mask, dtype=np.int32)
        dv = np.zeros(n)
        pmp = None
        if pm is not None:
            pm = np.ascontiguousarray(pm, dtype=np.float64)
            pmp = _p(pm)
        getattr(self.lib, self.which + "_data_vector_real")(mask.ctypes.data_as(_ip), pmp, _p(dv))
        return dv

    def data_vector_fourier(self, ell, lmax_shear=1e30, use_nonlimber=1, mask=None):
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        pss, pgs, pgg = self.npairs
        n = len(ell) * (pss + pgs + pgg)
        if mask is None:
            mask = np.ones(n, dtype=np.int32)
        mask = np.ascontiguousarray(mask, dtype=np.int32)
        dv = np.zeros(n)
        f = getattr(self.lib, "orc_data_vector_fourier")
        f.argtypes = [C.c_int, _dp, C.c_double, C.c_int, _ip, _dp]
        f(len(ell), _p(ell), lmax_shear, use_nonlimber, mask.ctypes.data_as(_ip), _p(dv))
        return dv

    def limber_tables(self):
        assert self.which == "orc"
        pss, pgs, pgg = self.npairs
        ne = self.cfg.n_ell
        ss = np.zeros(2 * pss * ne)
        gs = np.zeros(pgs * ne + 1)
        gg = np.zeros(pgg * ne + 1)
        self.lib.orc_limber_tables(_p(ss), _p(gs), _p(gg))
        return ss.reshape(2, pss, ne), gs[:-1].reshape(pgs, ne), gg[:-1].reshape(pgg, ne)

    def ell_nodes(self, which):
        out = np.zeros(self.cfg.n_ell)
        self.lib.orc_ell_nodes(which, _p(out))
        return out

    def legendre_filters(self):
        nt, L = self.cfg.ntheta, self.cfg.lmax
        out = np.zeros(4 * nt * L)
        self.lib.orc_legendre_filters(_p(out))
        return out.reshape(4, nt, L)

    def fpt_bias(self):
        n = C.c_int(0)
        f = getattr(self.lib, self.which + "_fpt_bias")
        f(None, C.byref(n))
        out = np.zeros(8 * n.value)
        f(_p(out), C.byref(n))
        return out.reshape(8, n.value)

    def set_d1d3_table(self, tab, lnkmin, lnkmax):
        """The P_d1p3 table the oracle interpolates in ln k (the reference
        embeds one; the default is none, i.e. zero)."""
        t = np.ascontiguousarray(tab, dtype=np.float64)
        self._keep.append(t)
        f = getattr(self.lib, self.which + "_set_d1d3_table")
        f.argtypes = [_dp, C.c_int, C.c_double, C.c_double]
        return f(_p(t), len(t), lnkmin, lnkmax)

    def set_baryon_ratio(self, log10k, a, log10r):
        """The baryon P(k) ratio applied to p_nonlin (PkRatio_baryons): log10
        ratio [len(a)][len(log10k)] on log10 k (h/Mpc) x a; empty: off."""
        lk = np.ascontiguousarray(log10k, dtype=np.float64)
        av = np.ascontiguousarray(a, dtype=np.float64)
        lr = np.ascontiguousarray(log10r, dtype=np.float64)
        self._keep += [lk, av, lr]
        f = getattr(self.lib, self.which + "_set_baryon_ratio")
        f.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp]
        return f(len(lk), _p(lk), len(av), _p(av), _p(lr))

    def dC_ss_dlnk(self, k, l, ni, nj, EE=1):
        """dC_ss_dlnk_tomo_limber_nointerp (the point must be set)."""
        f = getattr(self.lib, self.which + "_dC_ss_dlnk_nointerp")
        f.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int]
        f.restype = C.c_double
        return f(float(k), float(l), int(ni), int(nj), int(EE))

    def RF_C_ss(self, kmax, l, ni, nj, EE=1):
        """RF_C_ss_tomo_limber_nointerp with the nointerp dlnC/dlnk at every l."""
        f = getattr(self.lib, self.which + "_RF_C_ss_nointerp")
        f.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int]
        f.restype = C.c_double
        return f(float(kmax), float(l), int(ni), int(nj), int(EE))

    def C_cmb(self, which, l, ni=0):
        """CMB-lensing C_l (C_gk_tomo_limber_nointerp / C_ks / C_kk): which in
        'gk', 'ks', 'kk'."""
        f = getattr(self.lib, "%s_C_%s_nointerp" % (self.which, which))
        f.restype = C.c_double
        if which == "kk":
            f.argtypes = [C.c_double]
            return f(float(l))
        f.argtypes = [C.c_double, C.c_int]
        return f(float(l), int(ni))

    def set_cmb(self, lmin, lmax, fwhm_arcmin, healpixwin=None):
        """The CMB map filter of w_gk / w_ks (init_cmb_cross_correlation):
        beam fwhm in arcmin, l range, optional HEALPix window per l."""
        win = None if healpixwin is None else np.ascontiguousarray(healpixwin, dtype=np.float64)
        f = getattr(self.lib, self.which + "_set_cmb")
        f.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, _dp]
        self._cmbwin = win
        st = f(int(lmin), int(lmax), float(fwhm_arcmin) * 2.90888208665721580e-4,
               0 if win is None else len(win), None if win is None else _p(win))
        if st != 0:
            raise RuntimeError(f"set_cmb failed: {st}")

    def w_cmb(self, which):
        """Real-space CMB-lensing cross-correlations w_gk [n_lens][ntheta]
        or w_ks [n_source][ntheta] (which: 'gk', 'ks')."""
        nb = self.cfg.n_lens if which == "gk" else self.cfg.n_source
        out = np.zeros((nb, self.cfg.ntheta))
        f = getattr(self.lib, "%s_w_%s" % (self.which, which))
        f.argtypes = [_dp]
        st = f(_p(out))
        if st != 0:
            raise RuntimeError(f"w_{which} failed: {st}")
        return out

    def set_dlnk_grid(self, nlnk=190, kmin=1e-5, kmax=1e2):
        """The ln k grid of the dC/dlnk tables (Ntable.dCX_dlnk_*); the
        point must be set (the reference builds its tables on demand)."""
        f = getattr(self.lib, self.which + "_set_dlnk_grid")
        f.argtypes = [C.c_int, C.c_double, C.c_double]
        if f(int(nlnk), float(kmin), float(kmax)) != 0:
            raise RuntimeError("set_dlnk_grid failed")

    def dlnxi_table(self, nlnk, kmin, kmax):
        """dlnxi+-/dlnk [2][pss][ntheta][nlnk] on the nlnk ln k nodes of
        [kmin, kmax] (dlnxi_dlnk_pm_tomo); also the table RF_xi reads."""
        npair = self.npairs[0]
        out = np.zeros((2, npair, self.cfg.ntheta, nlnk))
        f = getattr(self.lib, self.which + "_dlnxi_table")
        f.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        if f(int(nlnk), float(kmin), float(kmax), _p(out)) != 0:
            raise RuntimeError("dlnxi_table failed")
        return out

    def RF_xi(self, kmax, p, i, q):
        """RF_xi_tomo_limber_nointerp for xi+ (p 0) or xi- (p 1), theta bin
        i, shear pair q, on the last dlnxi_table grid."""
        f = getattr(self.lib, self.which + "_RF_xi")
        f.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int]
        f.restype = C.c_double
        return f(float(kmax), int(p), int(i), int(q))

    def C_kk_dv(self, ell):
        """C_kk at ell by the 6x2pt data vector's rule (nointerp at
        l <= lmin_tab, the ln l table above)."""
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        out = np.zeros(len(ell))
        f = getattr(self.lib, self.which + "_C_kk_dv")
        f.argtypes = [C.c_int, _dp, _dp]
        if f(len(ell), _p(ell), _p(out)) != 0:
            raise RuntimeError("C_kk_dv failed")
        return out

    def kk_bandpower(self, lminbp, lmaxbp, binmat, offset):
        """kk bandpowers: binmat [nbp][lmaxbp - lminbp + 1], offset [nbp]."""
        bm = np.ascontiguousarray(binmat, dtype=np.float64)
        off = np.ascontiguousarray(offset, dtype=np.float64)
        out = np.zeros(bm.shape[0])
        f = getattr(self.lib, self.which + "_kk_bandpower")
        f.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        if f(bm.shape[0], int(lminbp), int(lmaxbp), _p(bm), _p(off), _p(out)) != 0:
            raise RuntimeError("kk_bandpower failed")
        return out

    def set_direct_conv_size(self, n):
        """Transform length of the TATT direct convolutions (0: the reference's)."""
        self.lib.orc_set_direct_conv_size.argtypes = [C.c_long]
        self.lib.orc_set_direct_conv_size(int(n))

    def fpt_ia(self):
        n = C.c_int(0)
        f = getattr(self.lib, self.which + "_fpt_ia")
        f(None, C.byref(n))
        out = np.zeros(12 * n.value)
        f(_p(out), C.byref(n))
        return out.reshape(12, n.value)

    def fpt_ia_spectrum(self, k, P):
        """get_FPT_IA's [12][N0] table for spectrum P on log grid k (oracle only)."""
        k = np.ascontiguousarray(k, dtype=np.float64)
        P = np.ascontiguousarray(P, dtype=np.float64)
        out = np.zeros(12 * len(k))
        self.lib.orc_fpt_ia_spectrum.argtypes = [_dp, _dp, C.c_long, _dp]
        self.lib.orc_fpt_ia_spectrum(_p(k), _p(P), len(k), _p(out))
        return out.reshape(12, len(k))

    def ia_jrows(self):
        """(rows [n][5] = alpha, beta, J1, J2, Jk; coeff [n]; start [9]; tab_row [8])."""
        cap = 512
        rows = np.zeros((cap, 5), dtype=np.int32)
        coeff = np.zeros(cap)
        start = np.zeros(9, dtype=np.int32)
        trow = np.zeros(8, dtype=np.int32)
        n = self.lib.orc_ia_jrows(cap, rows.ctypes.data_as(_ip), _p(coeff),
                                  start.ctypes.data_as(_ip), trow.ctypes.data_as(_ip))
        return rows[:n], coeff[:n], start, trow

    def J_abJ1J2Jk(self, x, fx, alpha, beta, J1, J2, Jk, c_window=0.65, npad=1500, nlow=500,
                   nhigh=500):
        x = np.ascontiguousarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(fx, dtype=np.float64)
        ia = lambda v: np.ascontiguousarray(v, dtype=np.int32)
        a, b, j1, j2, jk = ia(alpha), ia(beta), ia(J1), ia(J2), ia(Jk)
        Fy = np.zeros(len(a) * len(x))
        f = getattr(self.lib, self.which + "_J_abJ1J2Jk")
        f.argtypes = [_dp, _dp, C.c_long, _ip, _ip, _ip, _ip, _ip, C.c_int, C.c_double,
                      C.c_double, C.c_long, C.c_long, C.c_long, _dp]
        f(_p(x), _p(fx), len(x), *(v.ctypes.data_as(_ip) for v in (a, b, j1, j2, jk)), len(a),
          0.0, c_window, npad, nlow, nhigh, _p(Fy))
        return Fy.reshape(len(a), len(x))

    def J_abl(self, x, fx, alpha, beta, ell, nu=-2.0, c_window=0.65, npad=1500,
              nlow=500, nhigh=500):
        x = np.ascontiguousarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(fx, dtype=np.float64)
        ia = lambda v: np.ascontiguousarray(v, dtype=np.int32)
        a, b, l = ia(alpha), ia(beta), ia(ell)
        Fy = np.zeros(len(a) * len(x))
        f = getattr(self.lib, self.which + "_J_abl")
        f.argtypes = [_dp, _dp, C.c_long, _ip, _ip, _ip, C.c_int, C.c_double, C.c_double,
                      C.c_long, C.c_long, C.c_long, _dp]
        f(_p(x), _p(fx), len(x), a.ctypes.data_as(_ip), b.ctypes.data_as(_ip),
          l.ctypes.data_as(_ip), len(a), nu, c_window, npad, nlow, nhigh, _p(Fy))
        return Fy.reshape(len(a), len(x))
