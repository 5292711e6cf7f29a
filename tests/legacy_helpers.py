"""ctypes set-up of libcl2pt_legacy.so for the tests."""
import ctypes as C

import numpy as np

from cl2pt import abi, build

_dp = C.POINTER(C.c_double)


class FPT(C.Structure):
    _fields_ = [("N", C.c_int), ("k_min", C.c_double), ("k_max", C.c_double),
                ("k_cutoff", C.c_double), ("sigma4", C.c_double), ("tab", C.POINTER(_dp))]


def load():
    build.build()
    lib = C.CDLL(build.LEGACY)
    lib.cl2pt_legacy_set_config.argtypes = [C.POINTER(abi.Config), C.c_int]
    lib.cl2pt_legacy_set_samples.argtypes = [C.POINTER(abi.NZ), C.POINTER(abi.NZ)]
    lib.cl2pt_legacy_set_cosmology.argtypes = [C.POINTER(abi.Cosmo)]
    lib.cl2pt_legacy_set_nuisance.argtypes = [C.POINTER(abi.Nuisance)]
    for f in ("xi_pm_tomo",):
        getattr(lib, f).argtypes = [C.c_int] * 5
        getattr(lib, f).restype = C.c_double
    for f in ("w_gammat_tomo", "w_gg_tomo"):
        getattr(lib, f).argtypes = [C.c_int] * 4
        getattr(lib, f).restype = C.c_double
    lib.C_ss_tomo_limber.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int]
    lib.C_ss_tomo_limber.restype = C.c_double
    for f in ("C_gs_tomo_limber", "C_gg_tomo_limber"):
        getattr(lib, f).argtypes = [C.c_double, C.c_int, C.c_int]
        getattr(lib, f).restype = C.c_double
    lib.C_ss_tomo_limber_nointerp.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.C_ss_tomo_limber_nointerp.restype = C.c_double
    for f in ("C_gs_tomo_limber_nointerp", "C_gg_tomo_limber_nointerp"):
        getattr(lib, f).argtypes = [C.c_double, C.c_int, C.c_int, C.c_int]
        getattr(lib, f).restype = C.c_double
    lib.C_cl_tomo.argtypes = [C.POINTER(_dp), C.c_double]
    return lib


def set_state(lib, w, table, nu, prec):
    keep = []
    cfg = w.cfg
    assert lib.cl2pt_legacy_set_config(C.byref(cfg), prec) == 0
    src, lens = abi.make_nz(w.src), abi.make_nz(w.lens)
    keep += [src, lens]
    assert lib.cl2pt_legacy_set_samples(C.byref(src.struct), C.byref(lens.struct)) == 0
    cosmo = abi.make_cosmo(table)
    # one table: the linear spectrum is the nonlinear one
    cosmo.struct.lnPL = None
    cosmo.struct.pkl_nk = 0
    keep.append(cosmo)
    assert lib.cl2pt_legacy_set_cosmology(C.byref(cosmo.struct)) == 0
    assert lib.cl2pt_legacy_set_nuisance(C.byref(nu)) == 0
    return keep


def fpt_table(lib, name, rows):
    f = FPT.in_dll(lib, name)
    return np.array([[f.tab[r][i] for i in range(f.N)] for r in range(rows)]), f
