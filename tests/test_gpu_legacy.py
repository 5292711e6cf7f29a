"""The reference-named entry points of libcl2pt_legacy.so (cosmo2D.h,
pt_cfastpt.h, cfastpt.h signatures) on one parameter point, against the
FP64 oracle (1e-4 relative, the data-vector bar) and against the batched
plan they sit on."""
import ctypes as C

import numpy as np
import pytest

import legacy_helpers as L
from cl2pt import abi, lib, workloads
from test_gpu_fastpt import ia_check
from test_gpu_real import REL, rel_err, rel_err_spectra


@pytest.fixture(scope="module")
def legacy_case(gpu_lib, oracle_built):
    import oracle as O
    w = workloads.make("real_3x2pt_small")
    # the legacy setters take one table: both spectra are the linear one
    tabs, nus = workloads.points(w, 1, seed=17)
    tabs = workloads.one_table(tabs)
    lg = L.load()
    keep = L.set_state(lg, w, tabs[0], nus[0], lib.PREC_MIXED)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    o.set_point(tabs[0], nus[0])
    return w, tabs, nus, lg, o, keep


@pytest.mark.gpu
def test_legacy_real_space(legacy_case):
    w, tabs, nus, lg, o, _ = legacy_case
    ns, nl, nt = w.cfg.n_source, w.cfg.n_lens, w.cfg.ntheta
    pairs = abi.shear_pairs(ns)
    xp = np.array([[lg.xi_pm_tomo(1, t, a, b, 1) for t in range(nt)] for a, b in pairs])
    xm = np.array([[lg.xi_pm_tomo(-1, t, b, a, 1) for t in range(nt)] for a, b in pairs])
    oxp, oxm = o.xi_pm()
    assert rel_err_spectra(xp, oxp, nt) <= REL
    assert rel_err_spectra(xm, oxm, nt) <= REL
    ggl = [(zl, zs) for zl in range(nl) for zs in range(ns)]
    gt = np.array([[lg.w_gammat_tomo(t, zl, zs, 1) for t in range(nt)] for zl, zs in ggl])
    assert rel_err_spectra(gt, o.w_gammat(), nt) <= REL
    wg = np.array([[lg.w_gg_tomo(t, i, i, 0) for t in range(nt)] for i in range(nl)])
    assert rel_err_spectra(wg, o.w_gg(), nt) <= REL
    # the same values as the batched plan without shear calibration
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=1)
    nu0 = abi.make_nuisance()
    C.memmove(C.addressof(nu0), C.addressof(nus[0]), C.sizeof(nu0))
    for i in range(abi.MAX_BINS):
        nu0.shear_m[i] = 0.0
    om, h0, chi, G, lnP = workloads.stack(tabs)
    dv = plan.eval_real(om, h0, chi, G, lnP, [nu0])[0]
    a = plan.n_xi // 2
    assert np.array_equal(xp.reshape(-1), dv[:a])
    assert np.array_equal(gt.reshape(-1), dv[2 * a:2 * a + plan.n_gammat])


@pytest.mark.gpu
def test_legacy_limber_tables_and_nonlimber(legacy_case):
    w, tabs, nus, lg, o, _ = legacy_case
    ns, nl = w.cfg.n_source, w.cfg.n_lens
    oss, ogs, ogg = o.limber_tables()
    ells = o.ell_nodes(0)
    pairs = abi.shear_pairs(ns)
    for k in (3, 40, 150):
        l = float(ells[k])
        got = np.array([lg.C_ss_tomo_limber(l, a, b, 1) for a, b in pairs])
        assert rel_err(got, oss[0][:, k]) <= REL
    ellg = o.ell_nodes(1)
    for k in (5, 90):
        l = float(ellg[k])
        got = np.array([lg.C_gs_tomo_limber(l, zl, zs) for zl in range(nl) for zs in range(ns)])
        assert rel_err(got, ogs[:, k]) <= REL
        got = np.array([lg.C_gg_tomo_limber(l, i, i) for i in range(nl)])
        assert rel_err(got, ogg[:, k]) <= REL
        # the direct quadrature at a node multipole equals the node value
        got_ni = np.array([lg.C_gg_tomo_limber_nointerp(l, i, i, 0) for i in range(nl)])
        assert rel_err(got_ni, ogg[:, k]) <= REL
        got_ni = np.array([lg.C_ss_tomo_limber_nointerp(l, a, b, 1, 0) for a, b in pairs])
        assert rel_err(got_ni, np.array([lg.C_ss_tomo_limber(l, a, b, 1) for a, b in pairs])) <= REL
    Lnl = w.cfg.lmax_nolimber
    cl = np.zeros((nl, Lnl))
    rows = (C.POINTER(C.c_double) * nl)(*[cl[i].ctypes.data_as(C.POINTER(C.c_double)) for i in range(nl)])
    lg.C_cl_tomo(rows, 0.01)
    ocl, _ = o.C_cl_tomo()
    assert rel_err(cl[:, 1:], ocl[:, 1:]) <= REL


@pytest.mark.gpu
def test_legacy_fastpt_globals(legacy_case):
    w, tabs, nus, lg, o, _ = legacy_case
    lg.get_FPT_bias()
    tb, f = L.fpt_table(lg, "FPTbias", 8)
    ob = o.fpt_bias()
    assert f.N == ob.shape[1] == 1100
    np.testing.assert_allclose(tb[6], ob[6], rtol=1e-14)
    np.testing.assert_allclose(tb[7], ob[7], rtol=1e-12)
    for r in range(5):
        assert rel_err(tb[r], ob[r], floor=1e-6) <= REL, r
    assert abs(f.sigma4 - tb[1][0] / 2) == 0.0
    lg.get_FPT_IA()
    ti, _ = L.fpt_table(lg, "FPTIA", 12)
    oi = o.fpt_ia()
    # rows 3 and 7 (delta E2, mix B) are direct FP64 convolutions whose
    # high-k tail is rounding-limited in the reference itself: held to 2e-5
    # of the row's peak in absolute terms, as in the FAST-PT tests
    err, rows = ia_check(ti[:10], oi[:10])
    assert err <= REL, rows
    # J_abl forwards to the drop-in
    k = tb[6]
    P = tb[7]
    a, b, l, _, _ = lib.bias_terms()
    cfg = lib.fastpt_config()
    n = len(a)
    Fy = np.zeros((n, len(k)))
    rows = (C.POINTER(C.c_double) * n)(*[Fy[i].ctypes.data_as(C.POINTER(C.c_double)) for i in range(n)])
    ia = lambda v: np.ascontiguousarray(v, dtype=np.int32).ctypes.data_as(C.POINTER(C.c_int))
    aa, bb, ll = (np.ascontiguousarray(v, dtype=np.int32) for v in (a, b, l))
    iso = np.zeros(n, dtype=np.int32)
    lg.J_abl.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_long] + [C.POINTER(C.c_int)] * 4 + \
        [C.c_int, C.c_void_p, C.POINTER(C.POINTER(C.c_double))]
    kk, PP = np.ascontiguousarray(k), np.ascontiguousarray(P)
    lg.J_abl(kk.ctypes.data_as(C.POINTER(C.c_double)), PP.ctypes.data_as(C.POINTER(C.c_double)), len(k),
             aa.ctypes.data_as(C.POINTER(C.c_int)), bb.ctypes.data_as(C.POINTER(C.c_int)),
             ll.ctypes.data_as(C.POINTER(C.c_int)), iso.ctypes.data_as(C.POINTER(C.c_int)), n,
             C.addressof(cfg), rows)
    ref = lib.J_abl(k, P, a, b, l)
    np.testing.assert_array_equal(Fy, ref)
