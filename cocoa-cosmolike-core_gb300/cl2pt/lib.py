"""ctypes binding of libcl2pt.so (the C ABI in include/cl2pt.h).

The library is the only compute path: if it is missing or fails to load,
every entry point raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcl2pt.so")

PREC_MIXED, PREC_FP64 = 0, 1
# Legendre contraction of a mixed plan (CL2PT_CONTRACT_*)
CONTRACT_FP32, CONTRACT_TF32X3, CONTRACT_BF16X3, CONTRACT_BF16X6 = 0, 1, 2, 3
FFTLOG_STATE_AUTO, FFTLOG_STATE_GLOBAL, FFTLOG_STATE_SHARED = 0, 1, 2
# kernel ids of cl2pt_kernel_times (CL2PT_K_* in include/cl2pt.h)
KERNELS = ["k_gtab", "k_nodes", "k_limber_ss", "k_limber_gs", "k_limber_gg", "k_limber_ggl",
           "k_nonlimber", "k_contract", "k_assemble", "k_vjp"]
HOST, DEVICE = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Grid(C.Structure):
    _fields_ = [
        ("chi_nz", C.c_int), ("chi_z", _dp), ("G_nz", C.c_int), ("G_z", _dp),
        ("pk_nk", C.c_int), ("pk_nz", C.c_int), ("pk_log10k", _dp), ("pk_z", _dp),
        ("pkl_nk", C.c_int), ("pkl_nz", C.c_int), ("pkl_log10k", _dp), ("pkl_z", _dp),
    ]


class Batch(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("where", C.c_int), ("omega_m", _dp), ("h0", _dp), ("chi", _dp),
        ("G", _dp), ("lnP", _dp), ("lnPL", _dp), ("nuisance", C.POINTER(abi.Nuisance)),
    ]


class FastPTConfig(C.Structure):
    """cl2pt_fastpt_config (the reference's fastpt_config)."""
    _fields_ = [("nu", C.c_double), ("c_window_width", C.c_double), ("N_pad", C.c_long),
                ("N_extrap_low", C.c_long), ("N_extrap_high", C.c_long)]


class CL2PTError(RuntimeError):
    pass


_lib = None


def load(path: str = LIB_PATH):
    """Load libcl2pt.so once (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CL2PTError(f"{path} is missing: build it with cl2pt.build.build()")
    lib = C.CDLL(path)
    lib.cl2pt_plan_create.argtypes = [C.POINTER(abi.Config), C.POINTER(abi.NZ), C.POINTER(abi.NZ),
                                      C.POINTER(Grid), C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    lib.cl2pt_plan_destroy.argtypes = [C.c_void_p]
    lib.cl2pt_plan_set_contraction.argtypes = [C.c_void_p, C.c_int]
    lib.cl2pt_plan_set_d1p3.argtypes = [C.c_void_p, _dp, C.c_int]
    lib.cl2pt_plan_get_contraction.argtypes = [C.c_void_p, _ip]
    lib.cl2pt_real_sizes.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip]
    lib.cl2pt_eval_real.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p]
    lib.cl2pt_check_errors.argtypes = [C.c_void_p, C.c_void_p]
    lib.cl2pt_vjp_real.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]
    lib.cl2pt_like_create.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, C.POINTER(C.c_void_p)]
    lib.cl2pt_plan_set_lens_photoz_grad.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
    lib.cl2pt_baryon_pcas.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(Batch), C.c_int, C.c_int, _dp, C.c_int, _dp,
                                      _dp, C.c_void_p, C.c_void_p]
    lib.cl2pt_like_destroy.argtypes = [C.c_void_p]
    lib.cl2pt_loglike_real.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.cl2pt_cl_nonlimber.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_void_p, C.c_void_p]
    lib.cl2pt_vjp_fourier.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, C.c_double, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
    lib.cl2pt_jacobian_real.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_void_p, C.c_int,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
    lib.cl2pt_eval_fourier.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, C.c_double,
                                       C.c_void_p, C.c_void_p, C.c_void_p]
    lib.cl2pt_fourier_sizes.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, _ip]
    lib.cl2pt_eval_fourier_ragged.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, C.c_double,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.cl2pt_fourier_graph_create.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, C.c_double,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.POINTER(C.c_void_p)]
    lib.cl2pt_plan_set_fftlog_state.argtypes = [C.c_void_p, C.c_int]
    lib.cl2pt_scut_ss_dlnk.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, C.c_int, _dp, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    lib.cl2pt_scut_ss_rf.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, _dp, C.c_void_p, C.c_void_p]
    lib.cl2pt_scut_ss_rf_grid.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, C.c_double, C.c_double, C.c_int,
                                          _dp, _dp, C.c_void_p, C.c_void_p]
    lib.cl2pt_scut_xi_dlnk.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, C.c_double, C.c_double, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    lib.cl2pt_scut_xi_rf.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, C.c_double, C.c_double, C.c_int, _dp,
                                     C.c_void_p, C.c_void_p]
    lib.cl2pt_cmb_cl.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p]
    lib.cl2pt_plan_set_cmb.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, _dp]
    lib.cl2pt_cmb_kk.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, _dp, C.c_void_p, C.c_void_p]
    lib.cl2pt_cmb_kk_bandpower.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_int, C.c_int, C.c_int, _dp, _dp,
                                           C.c_void_p, C.c_void_p]
    lib.cl2pt_cmb_real.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_void_p, C.c_void_p]
    lib.cl2pt_plan_set_baryon_ratio.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _dp, _dp]
    lib.cl2pt_plan_autotune.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_int, _ip, _ip,
                                        C.POINTER(C.c_double)]
    lib.cl2pt_real_graph_create.argtypes = [C.c_void_p, C.POINTER(Batch), C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.POINTER(C.c_void_p)]
    lib.cl2pt_graph_launch.argtypes = [C.c_void_p, C.c_void_p]
    lib.cl2pt_graph_launch_count.argtypes = [C.c_void_p]
    lib.cl2pt_graph_destroy.argtypes = [C.c_void_p]
    lib.cl2pt_debug_limber_tables.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
    lib.cl2pt_debug_nonlimber.argtypes = [C.c_void_p, C.c_int, _dp, _ip]
    lib.cl2pt_debug_g_tables.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.cl2pt_debug_limber_bb.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.cl2pt_last_launch_count.argtypes = [C.c_void_p]
    lib.cl2pt_set_timing.argtypes = [C.c_void_p, C.c_int]
    lib.cl2pt_kernel_times.argtypes = [C.c_void_p, _dp, _ip]
    lib.cl2pt_status_string.restype = C.c_char_p
    lib.cl2pt_fastpt_plan_create.argtypes = [_dp, C.c_long, _ip, _ip, _ip, C.c_int,
                                             C.POINTER(FastPTConfig), C.c_int,
                                             C.POINTER(C.c_void_p)]
    lib.cl2pt_fastpt_plan_destroy.argtypes = [C.c_void_p]
    lib.cl2pt_fastpt_J_abl.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                       C.c_void_p]
    lib.cl2pt_fastpt_bias.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                      C.c_void_p]
    lib.cl2pt_fastpt_check_errors.argtypes = [C.c_void_p]
    for name in ("cl2pt_fastpt_J_abl_vjp", "cl2pt_fastpt_bias_vjp", "cl2pt_fastpt_ia_vjp"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p]
    lib.cl2pt_fastpt_bias_terms.argtypes = [_ip, _ip, _ip, _ip, _dp]
    lib.cl2pt_J_abl.argtypes = [_dp, _dp, C.c_long, _ip, _ip, _ip, _ip, C.c_int,
                                C.POINTER(FastPTConfig), C.POINTER(_dp)]
    lib.cl2pt_fastpt_jk_plan_create.argtypes = [_dp, C.c_long, _ip, _ip, _ip, _ip, _ip, C.c_int,
                                                C.POINTER(FastPTConfig), C.c_int,
                                                C.POINTER(C.c_void_p)]
    lib.cl2pt_fastpt_ia_plan_create.argtypes = [_dp, C.c_long, C.POINTER(FastPTConfig), C.c_int,
                                                C.POINTER(C.c_void_p)]
    lib.cl2pt_fastpt_J_abJ1J2Jk.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                            C.c_void_p]
    lib.cl2pt_fastpt_ia.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                    C.c_void_p]
    lib.cl2pt_fastpt_ia_terms.argtypes = [C.c_int, _ip, _ip, _ip, _ip, _ip, _ip, _dp]
    lib.cl2pt_J_abJ1J2Jk.argtypes = [_dp, _dp, C.c_long, _ip, _ip, _ip, _ip, _ip, C.c_int,
                                     C.POINTER(FastPTConfig), C.POINTER(_dp)]
    _lib = lib
    return lib


def check(st: int, what: str = "cl2pt"):
    if st != 0:
        msg = load().cl2pt_status_string(st).decode()
        raise CL2PTError(f"{what}: status {st} ({msg})")


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class Plan:
    """A cl2pt plan: geometry, redshift samples, shared axes and workspace."""

    def __init__(self, cfg: abi.Config, src_table, lens_table, tables, precision=PREC_MIXED,
                 max_batch=1, linear_table=False):
        """linear_table: host batches may carry a separate linear P(k, z)
        table (lnPL) on the same axes as lnP."""
        lib = load()
        self.cfg = cfg
        self._src = abi.make_nz(src_table)
        self._lens = abi.make_nz(lens_table)
        ax = [np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in
              (tables.chi_z, tables.G_z, tables.log10k, tables.pk_z)]
        self._axes = ax
        g = Grid()
        g.chi_nz, g.chi_z = len(ax[0]), _p(ax[0])
        g.G_nz, g.G_z = len(ax[1]), _p(ax[1])
        g.pk_nk, g.pk_nz, g.pk_log10k, g.pk_z = len(ax[2]), len(ax[3]), _p(ax[2]), _p(ax[3])
        g.pkl_nk = 0
        if linear_table:
            g.pkl_nk, g.pkl_nz, g.pkl_log10k, g.pkl_z = len(ax[2]), len(ax[3]), _p(ax[2]), _p(ax[3])
        self.grid = g
        self.shapes = dict(chi=len(ax[0]), G=len(ax[1]), nk=len(ax[2]), nz=len(ax[3]))
        h = C.c_void_p()
        check(lib.cl2pt_plan_create(C.byref(cfg), C.byref(self._src.struct),
                                    C.byref(self._lens.struct), C.byref(g), precision, max_batch,
                                    C.byref(h)), "cl2pt_plan_create")
        self.h = h
        self.max_batch = max_batch
        sz = [C.c_int() for _ in range(4)]
        check(lib.cl2pt_real_sizes(h, *[C.byref(s) for s in sz]))
        self.n_xi, self.n_gammat, self.n_w, self.n_total = (s.value for s in sz)
        ns = cfg.n_source
        self.pss = ns * (ns + 1) // 2  # shear pairs (N_shear order)

    def set_contraction(self, mode: int):
        """CONTRACT_FP32 (CUDA cores) or a tensor-core form (CONTRACT_TF32X3,
        CONTRACT_BF16X3, CONTRACT_BF16X6) for the Legendre contraction."""
        check(load().cl2pt_plan_set_contraction(self.h, mode), "cl2pt_plan_set_contraction")

    def set_lens_photoz_grad(self, on=True, h_dz=0.0, h_stretch=0.0):
        """Lens photo-z shift / stretch gradients in the adjoint by central
        differences of the forward (cl2pt_plan_set_lens_photoz_grad)."""
        check(load().cl2pt_plan_set_lens_photoz_grad(self.h, int(bool(on)), float(h_dz), float(h_stretch)),
              "cl2pt_plan_set_lens_photoz_grad")

    def set_d1p3(self, p_d1p3):
        """P_d1p3 on the plan's FAST-PT grid (1100 values, the reference's
        FPTbias row 5) for the one-loop b3 terms."""
        a = np.ascontiguousarray(p_d1p3, dtype=np.float64)
        check(load().cl2pt_plan_set_d1p3(self.h, _p(a), len(a)), "cl2pt_plan_set_d1p3")

    def contraction(self) -> int:
        m = C.c_int()
        check(load().cl2pt_plan_get_contraction(self.h, C.byref(m)))
        return m.value

    def close(self):
        if getattr(self, "h", None):
            load().cl2pt_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- host
    def _host_batch(self, omega_m, h0, chi, G, lnP, nuisance, lnPL=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (omega_m, h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        n = arrs[0].shape[0]
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        return b, (arrs, lpl, nus)

    def scut_ss_dlnk(self, omega_m, h0, chi, G, lnP, nuisance, k, l, lnPL=None):
        """Scale-cut diagnostics of C_ss (cl2pt_scut_ss_dlnk): dC/dlnk and
        dlnC/dlnk [n][2][pss][len(k)][len(l)], k in h/Mpc."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        k = np.ascontiguousarray(k, dtype=np.float64)
        l = np.ascontiguousarray(l, dtype=np.float64)
        n = b.n
        dC = np.zeros((n, 2, self.pss, len(k), len(l)))
        dlnC = np.zeros_like(dC)
        check(load().cl2pt_scut_ss_dlnk(self.h, C.byref(b), len(k), _p(k), len(l), _p(l), dC.ctypes.data,
                                        dlnC.ctypes.data, None), "cl2pt_scut_ss_dlnk")
        return dC, dlnC

    def scut_ss_rf(self, omega_m, h0, chi, G, lnP, nuisance, kmax, l, lnPL=None, grid=None):
        """RF_C_ss at the requests (kmax[i], l[i]) (cl2pt_scut_ss_rf, or
        cl2pt_scut_ss_rf_grid with grid = (nlnk, kmin, kmax) for the dlnC
        table above lmin_tab): [n][2][pss][len(kmax)]."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        kmax = np.ascontiguousarray(kmax, dtype=np.float64)
        l = np.ascontiguousarray(l, dtype=np.float64)
        assert len(kmax) == len(l)
        rf = np.zeros((b.n, 2, self.pss, len(kmax)))
        if grid is None:
            check(load().cl2pt_scut_ss_rf(self.h, C.byref(b), len(kmax), _p(kmax), _p(l), rf.ctypes.data, None),
                  "cl2pt_scut_ss_rf")
        else:
            check(load().cl2pt_scut_ss_rf_grid(self.h, C.byref(b), int(grid[0]), float(grid[1]), float(grid[2]),
                                               len(kmax), _p(kmax), _p(l), rf.ctypes.data, None),
                  "cl2pt_scut_ss_rf_grid")
        return rf

    def scut_xi_dlnk(self, omega_m, h0, chi, G, lnP, nuisance, nlnk=190, kmin=1e-5, kmax=1e2, lnPL=None):
        """Real-space scale-cut diagnostics (cl2pt_scut_xi_dlnk): dxi/dlnk
        and the dlnxi/dlnk table [n][2][pss][ntheta][nlnk]."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        dxi = np.zeros((b.n, 2, self.pss, self.cfg.ntheta, nlnk))
        dln = np.zeros_like(dxi)
        check(load().cl2pt_scut_xi_dlnk(self.h, C.byref(b), nlnk, kmin, kmax, dxi.ctypes.data, dln.ctypes.data,
                                        None), "cl2pt_scut_xi_dlnk")
        return dxi, dln

    def scut_xi_rf(self, omega_m, h0, chi, G, lnP, nuisance, kmax_req, nlnk=190, kmin=1e-5, kmax=1e2, lnPL=None):
        """RF_xi at kmax_req (cl2pt_scut_xi_rf): [n][2][pss][ntheta][nreq]."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        kr = np.ascontiguousarray(kmax_req, dtype=np.float64)
        rf = np.zeros((b.n, 2, self.pss, self.cfg.ntheta, len(kr)))
        check(load().cl2pt_scut_xi_rf(self.h, C.byref(b), nlnk, kmin, kmax, len(kr), _p(kr), rf.ctypes.data, None),
              "cl2pt_scut_xi_rf")
        return rf

    def cmb_cl(self, omega_m, h0, chi, G, lnP, nuisance, ell, lnPL=None):
        """CMB-lensing spectra of the 6x2pt probes (cl2pt_cmb_cl) at the
        multipoles ell: C_gk [n][n_lens][nell], C_ks [n][n_source][nell],
        C_kk [n][nell]."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        n, ne = b.n, len(ell)
        gk = np.zeros((n, self.cfg.n_lens, ne))
        ks = np.zeros((n, self.cfg.n_source, ne))
        kk = np.zeros((n, ne))
        check(load().cl2pt_cmb_cl(self.h, C.byref(b), ne, _p(ell), gk.ctypes.data, ks.ctypes.data,
                                  kk.ctypes.data, None), "cl2pt_cmb_cl")
        return gk, ks, kk

    def cmb_kk(self, omega_m, h0, chi, G, lnP, nuisance, ell, lnPL=None):
        """C_kk [n][nell] by the 6x2pt data vector's rule (cl2pt_cmb_kk)."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        out = np.zeros((b.n, len(ell)))
        check(load().cl2pt_cmb_kk(self.h, C.byref(b), len(ell), _p(ell), out.ctypes.data, None), "cl2pt_cmb_kk")
        return out

    def cmb_kk_bandpower(self, omega_m, h0, chi, G, lnP, nuisance, lminbp, lmaxbp, binmat, offset, lnPL=None):
        """kk bandpowers [n][nbp] (cl2pt_cmb_kk_bandpower); binmat
        [nbp][lmaxbp - lminbp + 1]."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        bm = np.ascontiguousarray(binmat, dtype=np.float64)
        off = np.ascontiguousarray(offset, dtype=np.float64)
        out = np.zeros((b.n, bm.shape[0]))
        check(load().cl2pt_cmb_kk_bandpower(self.h, C.byref(b), bm.shape[0], int(lminbp), int(lmaxbp), _p(bm),
                                            _p(off), out.ctypes.data, None), "cl2pt_cmb_kk_bandpower")
        return out

    def set_cmb(self, lmin, lmax, fwhm_arcmin, healpixwin=None):
        """The CMB map filter of w_gk / w_ks (cl2pt_plan_set_cmb): beam fwhm
        in arcmin on lmin <= l <= lmax, optional HEALPix window per l."""
        win = None if healpixwin is None else np.ascontiguousarray(healpixwin, dtype=np.float64)
        check(load().cl2pt_plan_set_cmb(self.h, int(lmin), int(lmax), float(fwhm_arcmin),
                                        0 if win is None else len(win), None if win is None else _p(win)),
              "cl2pt_plan_set_cmb")

    def cmb_real(self, omega_m, h0, chi, G, lnP, nuisance, lnPL=None):
        """Real-space CMB-lensing cross-correlations (cl2pt_cmb_real):
        w_gk [n][n_lens][ntheta], w_ks [n][n_source][ntheta]."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        nt = self.cfg.ntheta
        wgk = np.zeros((b.n, self.cfg.n_lens, nt))
        wks = np.zeros((b.n, self.cfg.n_source, nt))
        check(load().cl2pt_cmb_real(self.h, C.byref(b), wgk.ctypes.data, wks.ctypes.data, None),
              "cl2pt_cmb_real")
        return wgk, wks

    def eval_real(self, omega_m, h0, chi, G, lnP, nuisance, mask=None, pm=None, lnPL=None, out=None):
        """Host arrays in, host data vectors out ([n][n_total]); out: an
        optional C-contiguous float64 host array of that shape (e.g. pinned)
        to write into."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64)
        n = om.shape[0]
        hh = np.ascontiguousarray(h0, dtype=np.float64)
        ch = np.ascontiguousarray(chi, dtype=np.float64)
        gg = np.ascontiguousarray(G, dtype=np.float64)
        lp = np.ascontiguousarray(lnP, dtype=np.float64)
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), _p(hh), _p(ch), _p(gg), _p(lp)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        if out is None:
            out = np.zeros((n, self.n_total))
        elif out.shape != (n, self.n_total) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape (n, n_total)")
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        pmm = None if pm is None else np.ascontiguousarray(pm, dtype=np.float64)
        check(load().cl2pt_eval_real(self.h, C.byref(b),
                                     mk.ctypes.data if mk is not None else None,
                                     pmm.ctypes.data if pmm is not None else None,
                                     out.ctypes.data, None), "cl2pt_eval_real")
        return out

    def eval_fourier(self, omega_m, h0, chi, G, lnP, nuisance, ell, lmax_shear=1e30, mask=None,
                     lnPL=None):
        """Fourier 3x2pt at multipoles ell: host arrays in, [n][nell (pss + pgs + n_lens)] out."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64)
        n = om.shape[0]
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), *(_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        nt = C.c_int()
        check(load().cl2pt_fourier_sizes(self.h, len(ell), None, None, None, C.byref(nt)))
        out = np.zeros((n, nt.value))
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        check(load().cl2pt_eval_fourier(self.h, C.byref(b), len(ell), _p(ell), float(lmax_shear),
                                        mk.ctypes.data if mk is not None else None,
                                        out.ctypes.data, None), "cl2pt_eval_fourier")
        return out

    def vjp_real(self, omega_m, h0, chi, G, lnP, nuisance, cot, mask=None, pm=None, lnPL=None):
        """Value and vector-Jacobian product on host arrays: returns
        (dv [n][n_total], lnP_bar [n][nk*nz], nu_bar [n][13*MAX_BINS] in the
        flat cl2pt_nuisance layout), plus lnPL_bar when lnPL is given."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64)
        n = om.shape[0]
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), *(_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        cv = np.ascontiguousarray(np.broadcast_to(cot, (n, self.n_total)), dtype=np.float64)
        dv = np.zeros((n, self.n_total))
        lbar = np.zeros((n, arrs[3].size // n))
        lbarl = None if lpl is None else np.zeros((n, lpl.size // n))
        nbar = (abi.Nuisance * n)()
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        pmm = None if pm is None else np.ascontiguousarray(pm, dtype=np.float64)
        check(load().cl2pt_vjp_real(self.h, C.byref(b),
                                    mk.ctypes.data if mk is not None else None,
                                    pmm.ctypes.data if pmm is not None else None,
                                    cv.ctypes.data, dv.ctypes.data, lbar.ctypes.data,
                                    None if lbarl is None else lbarl.ctypes.data,
                                    C.addressof(nbar), None), "cl2pt_vjp_real")
        nb = np.frombuffer(bytes(nbar), dtype=np.float64).reshape(n, -1).copy()
        if lbarl is not None:
            return dv, lbar, nb, lbarl
        return dv, lbar, nb

    def likelihood(self, data, inv_cov, mask=None):
        """A cl2pt_like over this plan's real-space vector."""
        d = np.ascontiguousarray(data, dtype=np.float64)
        ic = np.ascontiguousarray(inv_cov, dtype=np.float64)
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        h = C.c_void_p()
        check(load().cl2pt_like_create(self.h, mk.ctypes.data if mk is not None else None, _p(d), _p(ic),
                                       C.byref(h)), "cl2pt_like_create")
        return Likelihood(h, self)

    def baryon_pcas(self, like, omega_m, h0, chi, G, lnP, nuisance, log10k, a, log10r, lnPL=None):
        """Baryon PCs [nscen][n_total] of one point (cl2pt_baryon_pcas);
        log10r [nscen][len(a)][len(log10k)]."""
        b, keep = self._host_batch(omega_m, h0, chi, G, lnP, nuisance, lnPL)
        lk = np.ascontiguousarray(log10k, dtype=np.float64)
        av = np.ascontiguousarray(a, dtype=np.float64)
        lr = np.ascontiguousarray(log10r, dtype=np.float64)
        R = np.zeros((lr.shape[0], self.n_total))
        check(load().cl2pt_baryon_pcas(self.h, like.h, C.byref(b), lr.shape[0], len(lk), _p(lk), len(av), _p(av),
                                       _p(lr), R.ctypes.data, None), "cl2pt_baryon_pcas")
        return R

    def loglike_real(self, like, omega_m, h0, chi, G, lnP, nuisance, pm=None, grad=False, lnPL=None):
        """chi2 [n] (host arrays); with grad also (lnP_bar, nu_bar) of
        ln L = -chi2/2."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64)
        n = om.shape[0]
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), *(_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        chi2 = np.zeros(n)
        lbar = np.zeros((n, arrs[3].size // n)) if grad else None
        lbarl = np.zeros((n, lpl.size // n)) if (grad and lpl is not None) else None
        nbar = (abi.Nuisance * n)() if grad else None
        pmm = None if pm is None else np.ascontiguousarray(pm, dtype=np.float64)
        check(load().cl2pt_loglike_real(self.h, like.h, C.byref(b),
                                        pmm.ctypes.data if pmm is not None else None, chi2.ctypes.data,
                                        lbar.ctypes.data if grad else None,
                                        lbarl.ctypes.data if lbarl is not None else None,
                                        C.addressof(nbar) if grad else None, None), "cl2pt_loglike_real")
        if not grad:
            return chi2
        nb = np.frombuffer(bytes(nbar), dtype=np.float64).reshape(n, -1).copy()
        return chi2, lbar, nb

    def cl_nonlimber(self, omega_m, h0, chi, G, lnP, nuisance, lnPL=None):
        """Batched non-Limber C_l: (cl [n][n_lens][lmax_nolimber], conv_l [n][n_lens])."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64)
        n = om.shape[0]
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), *(_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        nl, L = self.cfg.n_lens, self.cfg.lmax_nolimber
        cl = np.zeros((n, nl, L))
        conv = np.zeros((n, nl), dtype=np.int32)
        check(load().cl2pt_cl_nonlimber(self.h, C.byref(b), cl.ctypes.data, conv.ctypes.data, None),
              "cl2pt_cl_nonlimber")
        return cl, conv

    def vjp_fourier(self, omega_m, h0, chi, G, lnP, nuisance, ell, cot, lmax_shear=1e30, mask=None,
                    lnPL=None):
        """Value and VJP of the Fourier vector on host arrays: (dv, lnP_bar,
        nu_bar[, lnPL_bar]) as vjp_real."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64)
        n = om.shape[0]
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), *(_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        nt = C.c_int()
        check(load().cl2pt_fourier_sizes(self.h, len(ell), None, None, None, C.byref(nt)))
        cv = np.ascontiguousarray(np.broadcast_to(cot, (n, nt.value)), dtype=np.float64)
        dv = np.zeros((n, nt.value))
        lbar = np.zeros((n, arrs[3].size // n))
        lbarl = None if lpl is None else np.zeros((n, lpl.size // n))
        nbar = (abi.Nuisance * n)()
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        check(load().cl2pt_vjp_fourier(self.h, C.byref(b), len(ell), _p(ell), float(lmax_shear),
                                       mk.ctypes.data if mk is not None else None, cv.ctypes.data,
                                       dv.ctypes.data, lbar.ctypes.data,
                                       None if lbarl is None else lbarl.ctypes.data,
                                       C.addressof(nbar), None), "cl2pt_vjp_fourier")
        nb = np.frombuffer(bytes(nbar), dtype=np.float64).reshape(n, -1).copy()
        if lbarl is not None:
            return dv, lbar, nb, lbarl
        return dv, lbar, nb

    def fourier_n_total(self, nell) -> int:
        """Length of the Fourier vector at nell multipoles."""
        nt = C.c_int()
        check(load().cl2pt_fourier_sizes(self.h, int(nell), None, None, None, C.byref(nt)))
        return nt.value

    def eval_fourier_device(self, omega_m, h0, chi, G, lnP, nuisance, ell, out, lmax_shear=1e30, mask=None,
                            lnPL=None, stream=None):
        """Device form of eval_fourier: torch CUDA tensors in and out as in
        eval_real_device (out [n][fourier_n_total(len(ell))]); ell a host
        array."""
        b = Batch()
        b.n, b.where = int(omega_m.shape[0]), DEVICE
        cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), _dp)
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (cast(t) for t in (omega_m, h0, chi, G, lnP))
        b.lnPL = cast(lnPL) if lnPL is not None else None
        b.nuisance = C.cast(C.c_void_p(nuisance.data_ptr()), C.POINTER(abi.Nuisance))
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        st = load().cl2pt_eval_fourier(self.h, C.byref(b), len(ell), _p(ell), float(lmax_shear),
                                       None if mask is None else mask.data_ptr(), out.data_ptr(), stream)
        check(st, "cl2pt_eval_fourier")

    def vjp_fourier_device(self, omega_m, h0, chi, G, lnP, nuisance, ell, cot, dv, lnP_bar, nu_bar,
                           lmax_shear=1e30, mask=None, lnPL=None, lnPL_bar=None, stream=None):
        """Device form of vjp_fourier (CUDA tensors as in vjp_real_device)."""
        b = Batch()
        b.n, b.where = int(omega_m.shape[0]), DEVICE
        cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), _dp)
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (cast(t) for t in (omega_m, h0, chi, G, lnP))
        b.lnPL = cast(lnPL) if lnPL is not None else None
        b.nuisance = C.cast(C.c_void_p(nuisance.data_ptr()), C.POINTER(abi.Nuisance))
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        st = load().cl2pt_vjp_fourier(self.h, C.byref(b), len(ell), _p(ell), float(lmax_shear),
                                      None if mask is None else mask.data_ptr(), cot.data_ptr(),
                                      None if dv is None else dv.data_ptr(), lnP_bar.data_ptr(),
                                      None if lnPL_bar is None else lnPL_bar.data_ptr(),
                                      nu_bar.data_ptr(), stream)
        check(st, "cl2pt_vjp_fourier")

    def jacobian_real(self, omega_m, h0, chi, G, lnP, nuisance, rows=None, mask=None, pm=None,
                      lnPL=None):
        """Jacobian of one point's data vector (host arrays, n = 1): returns
        (dv [n_total], J_lnP [nrows][nk*nz], J_nu [nrows][13*MAX_BINS]) and
        J_lnPL when lnPL is given."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64).reshape(1)
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        nus = (abi.Nuisance * 1)(*nuisance)
        b = Batch()
        b.n, b.where = 1, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), *(_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        rw = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
        nr = self.n_total if rw is None else len(rw)
        dv = np.zeros(self.n_total)
        jl = np.zeros((nr, arrs[3].size))
        jll = None if lpl is None else np.zeros((nr, lpl.size))
        jn = (abi.Nuisance * nr)()
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        pmm = None if pm is None else np.ascontiguousarray(pm, dtype=np.float64)
        check(load().cl2pt_jacobian_real(self.h, C.byref(b),
                                         mk.ctypes.data if mk is not None else None,
                                         pmm.ctypes.data if pmm is not None else None, nr,
                                         rw.ctypes.data if rw is not None else None,
                                         dv.ctypes.data, jl.ctypes.data,
                                         None if jll is None else jll.ctypes.data,
                                         C.addressof(jn), None), "cl2pt_jacobian_real")
        jnu = np.frombuffer(bytes(jn), dtype=np.float64).reshape(nr, -1).copy()
        if jll is not None:
            return dv, jl, jnu, jll
        return dv, jl, jnu

    def vjp_real_device(self, omega_m, h0, chi, G, lnP, nuisance, cot, dv, lnP_bar, nu_bar,
                        mask=None, pm=None, lnPL=None, lnPL_bar=None, stream=None):
        """Device form of vjp_real: float64 CUDA tensors; nuisance and nu_bar
        hold n packed cl2pt_nuisance structs (any dtype, contiguous); dv may
        be None; lnPL_bar is needed with lnPL."""
        b = Batch()
        b.n, b.where = int(omega_m.shape[0]), DEVICE
        cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), _dp)
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (cast(t) for t in (omega_m, h0, chi, G, lnP))
        b.lnPL = cast(lnPL) if lnPL is not None else None
        b.nuisance = C.cast(C.c_void_p(nuisance.data_ptr()), C.POINTER(abi.Nuisance))
        st = load().cl2pt_vjp_real(self.h, C.byref(b),
                                   None if mask is None else mask.data_ptr(),
                                   None if pm is None else pm.data_ptr(),
                                   cot.data_ptr(), None if dv is None else dv.data_ptr(),
                                   lnP_bar.data_ptr(),
                                   None if lnPL_bar is None else lnPL_bar.data_ptr(),
                                   nu_bar.data_ptr(), stream)
        check(st, "cl2pt_vjp_real")

    def eval_fourier_ragged(self, omega_m, h0, chi, G, lnP, nuisance, ell, row_ptr, idx,
                            lmax_shear=1e30, lnPL=None):
        """Ragged Fourier vectors on host arrays: point i keeps idx[row_ptr[i]:
        row_ptr[i+1]]; returns the compacted values [row_ptr[-1]]."""
        om = np.ascontiguousarray(omega_m, dtype=np.float64)
        n = om.shape[0]
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (h0, chi, G, lnP)]
        lpl = None if lnPL is None else np.ascontiguousarray(lnPL, dtype=np.float64)
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        nus = (abi.Nuisance * n)(*nuisance)
        b = Batch()
        b.n, b.where = n, HOST
        b.omega_m, b.h0, b.chi, b.G, b.lnP = _p(om), *(_p(a) for a in arrs)
        b.lnPL = _p(lpl) if lpl is not None else None
        b.nuisance = nus
        rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
        ix = np.ascontiguousarray(idx, dtype=np.int32)
        out = np.zeros(max(int(rp[-1]), 1))
        check(load().cl2pt_eval_fourier_ragged(self.h, C.byref(b), len(ell), _p(ell), float(lmax_shear),
                                               rp.ctypes.data, ix.ctypes.data, out.ctypes.data, None),
              "cl2pt_eval_fourier_ragged")
        return out[:int(rp[-1])]

    def fourier_graph(self, omega_m, h0, chi, G, lnP, nuisance, ell, out, lmax_shear=1e30,
                      mask=None, row_ptr=None, idx=None, lnPL=None, stream=None):
        """Capture a Fourier evaluation over these CUDA tensors as a graph
        (see cl2pt_fourier_graph_create); returns a Graph."""
        b = Batch()
        b.n, b.where = int(omega_m.shape[0]), DEVICE
        cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), _dp)
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (cast(t) for t in (omega_m, h0, chi, G, lnP))
        b.lnPL = cast(lnPL) if lnPL is not None else None
        b.nuisance = C.cast(C.c_void_p(nuisance.data_ptr()), C.POINTER(abi.Nuisance))
        ell = np.ascontiguousarray(ell, dtype=np.float64)
        g = C.c_void_p()
        ptr = lambda t: None if t is None else t.data_ptr()
        check(load().cl2pt_fourier_graph_create(self.h, C.byref(b), len(ell), _p(ell), float(lmax_shear),
                                                ptr(mask), ptr(row_ptr), ptr(idx), out.data_ptr(), stream,
                                                C.byref(g)), "cl2pt_fourier_graph_create")
        # keep the tensors the graph reads alive with it
        return Graph(g, (omega_m, h0, chi, G, lnP, nuisance, out, mask, row_ptr, idx, lnPL, self))

    def set_baryon_ratio(self, log10k, a, log10r):
        """p_nonlin x 10^(log10r interpolated on (log10 k [h/Mpc], a))
        (cl2pt_plan_set_baryon_ratio); log10r is [len(a)][len(log10k)];
        an empty log10k turns it off."""
        lk = np.ascontiguousarray(log10k, dtype=np.float64)
        av = np.ascontiguousarray(a, dtype=np.float64)
        lr = np.ascontiguousarray(log10r, dtype=np.float64)
        if len(lk) == 0:
            check(load().cl2pt_plan_set_baryon_ratio(self.h, 0, None, 0, None, None), "cl2pt_plan_set_baryon_ratio")
            return
        assert lr.shape == (len(av), len(lk))
        check(load().cl2pt_plan_set_baryon_ratio(self.h, len(lk), _p(lk), len(av), _p(av), _p(lr)),
              "cl2pt_plan_set_baryon_ratio")

    def set_fftlog_state(self, mode):
        """Where the FFTLog loop keeps its spectra and state (FFTLOG_STATE_*)."""
        check(load().cl2pt_plan_set_fftlog_state(self.h, int(mode)), "cl2pt_plan_set_fftlog_state")

    def autotune(self, omega_m, h0, chi, G, lnP, nuisance, reps=3, lnPL=None, stream=None):
        """Time the candidate configurations on these CUDA tensors, keep the
        fastest (cl2pt_plan_autotune); returns (contraction, fftlog_state, ms)."""
        b = Batch()
        b.n, b.where = int(omega_m.shape[0]), DEVICE
        cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), _dp)
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (cast(t) for t in (omega_m, h0, chi, G, lnP))
        b.lnPL = cast(lnPL) if lnPL is not None else None
        b.nuisance = C.cast(C.c_void_p(nuisance.data_ptr()), C.POINTER(abi.Nuisance))
        c, st, ms = C.c_int(), C.c_int(), C.c_double()
        check(load().cl2pt_plan_autotune(self.h, C.byref(b), stream, int(reps), C.byref(c), C.byref(st),
                                         C.byref(ms)), "cl2pt_plan_autotune")
        return c.value, st.value, ms.value

    def real_graph(self, omega_m, h0, chi, G, lnP, nuisance, out, mask=None, pm=None, lnPL=None,
                   stream=None):
        """Capture a real-space evaluation over these CUDA tensors as a graph
        (see cl2pt_real_graph_create); returns a Graph."""
        b = Batch()
        b.n, b.where = int(omega_m.shape[0]), DEVICE
        cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), _dp)
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (cast(t) for t in (omega_m, h0, chi, G, lnP))
        b.lnPL = cast(lnPL) if lnPL is not None else None
        b.nuisance = C.cast(C.c_void_p(nuisance.data_ptr()), C.POINTER(abi.Nuisance))
        g = C.c_void_p()
        ptr = lambda t: None if t is None else t.data_ptr()
        check(load().cl2pt_real_graph_create(self.h, C.byref(b), ptr(mask), ptr(pm), out.data_ptr(), stream,
                                             C.byref(g)), "cl2pt_real_graph_create")
        return Graph(g, (omega_m, h0, chi, G, lnP, nuisance, out, mask, pm, lnPL, self))

    # ------------------------------------------------------------ device
    def eval_real_device(self, omega_m, h0, chi, G, lnP, nuisance, out, mask=None, pm=None,
                         lnPL=None, stream=None):
        """torch CUDA tensors in and out (float64, contiguous); nuisance is
        a uint8 CUDA tensor holding n packed cl2pt_nuisance structs."""
        b = Batch()
        b.n, b.where = int(omega_m.shape[0]), DEVICE
        cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), _dp)
        b.omega_m, b.h0, b.chi, b.G, b.lnP = (cast(t) for t in (omega_m, h0, chi, G, lnP))
        b.lnPL = cast(lnPL) if lnPL is not None else None
        b.nuisance = C.cast(C.c_void_p(nuisance.data_ptr()), C.POINTER(abi.Nuisance))
        st = load().cl2pt_eval_real(self.h, C.byref(b),
                                    None if mask is None else mask.data_ptr(),
                                    None if pm is None else pm.data_ptr(),
                                    out.data_ptr(), stream)
        check(st, "cl2pt_eval_real")

    def check_errors(self, stream=None):
        check(load().cl2pt_check_errors(self.h, stream), "device check")

    def set_timing(self, on: bool):
        check(load().cl2pt_set_timing(self.h, 1 if on else 0))

    def kernel_times(self):
        """(ms per kernel id, launches per kernel id) since the last call."""
        ms = np.zeros(len(KERNELS))
        n = np.zeros(len(KERNELS), dtype=np.int32)
        check(load().cl2pt_kernel_times(self.h, _p(ms), n.ctypes.data_as(_ip)))
        return dict(zip(KERNELS, ms)), dict(zip(KERNELS, n.tolist()))

    def launches(self) -> int:
        return load().cl2pt_last_launch_count(self.h)

    # ------------------------------------------------------------- debug
    def limber_tables(self, point=0):
        pss, pgs, pgg = abi.n_pairs(self.cfg)
        nn = self.cfg.lmin_tab - 1 + self.cfg.n_ell
        ss = np.zeros(pss * nn)
        gs = np.zeros(max(pgs, 1) * nn)
        gg = np.zeros(pgg * nn)
        check(load().cl2pt_debug_limber_tables(self.h, point, _p(ss), _p(gs), _p(gg)))
        return ss.reshape(pss, nn), gs[: pgs * nn].reshape(pgs, nn), gg.reshape(pgg, nn)

    def limber_bb(self, point=0):
        """C_ss BB on the C_l nodes [pss][nnode] (TATT plans)."""
        pss, _, _ = abi.n_pairs(self.cfg)
        nn = self.cfg.lmin_tab - 1 + self.cfg.n_ell
        bb = np.zeros(pss * nn)
        check(load().cl2pt_debug_limber_bb(self.h, point, _p(bb)))
        return bb.reshape(pss, nn)

    def nonlimber(self, point=0):
        nl, L = self.cfg.n_lens, self.cfg.lmax_nolimber
        cl = np.zeros(nl * L)
        conv = np.zeros(nl, dtype=np.int32)
        check(load().cl2pt_debug_nonlimber(self.h, point, _p(cl), conv.ctypes.data_as(_ip)))
        return cl.reshape(nl, L), conv

    def g_tables(self, point=0):
        out = np.zeros(self.cfg.n_source * self.cfg.n_a)
        check(load().cl2pt_debug_g_tables(self.h, point, _p(out)))
        return out.reshape(self.cfg.n_source, self.cfg.n_a)


# ------------------------------------------------------------------ FAST-PT
class Likelihood:
    """A cl2pt_like (mask, data, inverse covariance on the device)."""

    def __init__(self, h, plan):
        self.h = h
        self._plan = plan

    def close(self):
        if getattr(self, "h", None):
            load().cl2pt_like_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Graph:
    """A captured evaluation (cl2pt_graph: Fourier or real space)."""

    def __init__(self, h, keep):
        self.h = h
        self._keep = keep

    def launch(self, stream=None):
        check(load().cl2pt_graph_launch(self.h, stream), "cl2pt_graph_launch")

    def launches(self) -> int:
        return load().cl2pt_graph_launch_count(self.h)

    def close(self):
        if getattr(self, "h", None):
            load().cl2pt_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ints(v):
    return np.ascontiguousarray(v, dtype=np.int32)


def fastpt_config(nu=-2.0, c_window=0.65, npad=1500, nlow=500, nhigh=500) -> FastPTConfig:
    """Defaults: the settings get_FPT_bias passes (pt_cfastpt.c:130-135)."""
    c = FastPTConfig()
    c.nu, c.c_window_width, c.N_pad, c.N_extrap_low, c.N_extrap_high = nu, c_window, npad, nlow, nhigh
    return c


def bias_terms():
    """(alpha, beta, ell, output index, coefficient) of the 13 bias terms."""
    a, b, l, o = (np.zeros(13, dtype=np.int32) for _ in range(4))
    c = np.zeros(13)
    n = load().cl2pt_fastpt_bias_terms(*(v.ctypes.data_as(_ip) for v in (a, b, l, o)), _p(c))
    assert n == 13
    return a, b, l, o, c


def ia_terms():
    """(alpha, beta, J1, J2, Jk, output row, coefficient) of the 184 TATT J-rows."""
    cols = [np.zeros(512, dtype=np.int32) for _ in range(6)]
    c = np.zeros(512)
    n = load().cl2pt_fastpt_ia_terms(512, *(v.ctypes.data_as(_ip) for v in cols), _p(c))
    return tuple(v[:n] for v in cols) + (c[:n],)


class FastPT:
    """Batched FAST-PT over spectra on one log-spaced grid x.

    FastPT(x, alpha, beta, ell)            J_abl terms (bias list: .bias())
    FastPT.jk(x, alpha, beta, J1, J2, Jk)  J_abJ1J2Jk terms
    FastPT.for_ia(x)                       get_FPT_IA tables (.ia())
    """

    def __init__(self, x, alpha=None, beta=None, ell=None, cfg: FastPTConfig | None = None,
                 max_spec=1, _kind="jabl", _jk=None):
        lib = load()
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.cfg = cfg if cfg is not None else fastpt_config()
        self.max_spec = max_spec
        self.kind = _kind
        h = C.c_void_p()
        if _kind == "jabl":
            self.alpha, self.beta, self.ell = _ints(alpha), _ints(beta), _ints(ell)
            self.nterms = len(self.alpha)
            st = lib.cl2pt_fastpt_plan_create(_p(self.x), len(self.x), self.alpha.ctypes.data_as(_ip),
                                              self.beta.ctypes.data_as(_ip),
                                              self.ell.ctypes.data_as(_ip), self.nterms,
                                              C.byref(self.cfg), max_spec, C.byref(h))
        elif _kind == "jk":
            self._cols = [_ints(v) for v in _jk]
            self.nterms = len(self._cols[0])
            st = lib.cl2pt_fastpt_jk_plan_create(_p(self.x), len(self.x),
                                                 *(v.ctypes.data_as(_ip) for v in self._cols),
                                                 self.nterms, C.byref(self.cfg), max_spec, C.byref(h))
        else:
            self.nterms = len(ia_terms()[0])
            st = lib.cl2pt_fastpt_ia_plan_create(_p(self.x), len(self.x), C.byref(self.cfg), max_spec,
                                                 C.byref(h))
        check(st, "FAST-PT plan")
        self.h = h

    @classmethod
    def for_bias(cls, x, max_spec=1, cfg: FastPTConfig | None = None):
        a, b, l, _, _ = bias_terms()
        return cls(x, a, b, l, cfg, max_spec)

    @classmethod
    def jk(cls, x, alpha, beta, J1, J2, Jk, max_spec=1, cfg: FastPTConfig | None = None):
        return cls(x, cfg=cfg, max_spec=max_spec, _kind="jk", _jk=(alpha, beta, J1, J2, Jk))

    @classmethod
    def for_ia(cls, x, max_spec=1, cfg: FastPTConfig | None = None):
        return cls(x, cfg=cfg, max_spec=max_spec, _kind="ia")

    def close(self):
        if getattr(self, "h", None):
            load().cl2pt_fastpt_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _run(self, fn, fx, nout):
        fx = np.ascontiguousarray(np.atleast_2d(fx), dtype=np.float64)
        out = np.zeros((fx.shape[0], nout, len(self.x)))
        check(fn(self.h, fx.ctypes.data, fx.shape[0], out.ctypes.data, HOST, None), "fastpt")
        return out

    def J_abl(self, fx):
        """fx [n][N0] (host) -> [n][nterms][N0]."""
        return self._run(load().cl2pt_fastpt_J_abl, fx, self.nterms)

    def _vjp(self, fn, fx, obar, nout):
        fx = np.ascontiguousarray(np.atleast_2d(fx), dtype=np.float64)
        ob = np.ascontiguousarray(obar, dtype=np.float64).reshape(fx.shape[0], nout, len(self.x))
        g = np.zeros_like(fx)
        check(fn(self.h, fx.ctypes.data, fx.shape[0], ob.ctypes.data, g.ctypes.data, HOST, None), "fastpt vjp")
        return g

    def J_vjp(self, fx, obar):
        """Gradient [n][N0] of <obar, J(fx)> for the per-term outputs
        (J_abl and J_abJ1J2Jk plans; obar [n][nterms][N0])."""
        return self._vjp(load().cl2pt_fastpt_J_abl_vjp, fx, obar, self.nterms)

    def bias_vjp(self, fx, obar):
        """Gradient [n][N0] of <obar, bias(fx)>, obar [n][5][N0]."""
        return self._vjp(load().cl2pt_fastpt_bias_vjp, fx, obar, 5)

    def ia_vjp(self, fx, obar):
        """Gradient [n][N0] of <obar, ia(fx)>, obar [n][10][N0]."""
        return self._vjp(load().cl2pt_fastpt_ia_vjp, fx, obar, 10)

    def bias(self, fx):
        """fx [n][N0] (host) -> [n][5][N0]: P_d1d2, P_d2d2, P_d1s2, P_d2s2, P_s2s2."""
        return self._run(load().cl2pt_fastpt_bias, fx, 5)

    def J_abJ1J2Jk(self, fx):
        """fx [n][N0] (host) -> [n][nterms][N0] (jk and ia plans)."""
        return self._run(load().cl2pt_fastpt_J_abJ1J2Jk, fx, self.nterms)

    def ia(self, fx):
        """fx [n][N0] (host) -> [n][10][N0]: the get_FPT_IA table rows 0-9."""
        return self._run(load().cl2pt_fastpt_ia, fx, 10)

    def ia_device(self, fx, out, stream=None):
        """torch CUDA float64 tensors fx [n][N0], out [n][10][N0]."""
        check(load().cl2pt_fastpt_ia(self.h, fx.data_ptr(), int(fx.shape[0]), out.data_ptr(),
                                     DEVICE, stream), "fastpt")

    def J_abl_device(self, fx, out, stream=None):
        """torch CUDA float64 tensors fx [n][N0], out [n][nterms][N0]."""
        check(load().cl2pt_fastpt_J_abl(self.h, fx.data_ptr(), int(fx.shape[0]), out.data_ptr(),
                                        DEVICE, stream), "fastpt")

    def bias_device(self, fx, out, stream=None):
        """torch CUDA float64 tensors fx [n][N0], out [n][5][N0]."""
        check(load().cl2pt_fastpt_bias(self.h, fx.data_ptr(), int(fx.shape[0]), out.data_ptr(),
                                       DEVICE, stream), "fastpt")

    def check_errors(self):
        check(load().cl2pt_fastpt_check_errors(self.h), "fastpt device check")


def J_abl(x, fx, alpha, beta, ell, cfg: FastPTConfig | None = None):
    """The reference-shaped entry point cl2pt_J_abl (one spectrum, host
    arrays, Fy as an array of row pointers)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    fx = np.ascontiguousarray(fx, dtype=np.float64)
    a, b, l = _ints(alpha), _ints(beta), _ints(ell)
    cfg = cfg if cfg is not None else fastpt_config()
    out = np.zeros((len(a), len(x)))
    rows = (_dp * len(a))(*[out[t].ctypes.data_as(_dp) for t in range(len(a))])
    check(load().cl2pt_J_abl(_p(x), _p(fx), len(x), a.ctypes.data_as(_ip), b.ctypes.data_as(_ip),
                             l.ctypes.data_as(_ip), None, len(a), C.byref(cfg), rows), "cl2pt_J_abl")
    return out


def J_abJ1J2Jk(x, fx, alpha, beta, J1, J2, Jk, cfg: FastPTConfig | None = None):
    """The reference-shaped entry point cl2pt_J_abJ1J2Jk (one spectrum)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    fx = np.ascontiguousarray(fx, dtype=np.float64)
    cols = [_ints(v) for v in (alpha, beta, J1, J2, Jk)]
    cfg = cfg if cfg is not None else fastpt_config()
    n = len(cols[0])
    out = np.zeros((n, len(x)))
    rows = (_dp * n)(*[out[t].ctypes.data_as(_dp) for t in range(n)])
    check(load().cl2pt_J_abJ1J2Jk(_p(x), _p(fx), len(x), *(v.ctypes.data_as(_ip) for v in cols), n,
                                  C.byref(cfg), rows), "cl2pt_J_abJ1J2Jk")
    return out
