"""CMB-lensing spectra of the 6x2pt probes (cl2pt_cmb_cl): C_gk, C_ks and
C_kk against the golden fixtures made by the reference's own code
(C_gk_tomo_limber_nointerp, C_ks_tomo_limber_nointerp, C_kk_limber_nointerp)
and against the FP64 oracle for magnification and the linear run mode.
The spectra are computed in FP64 in both plans."""
import os

import numpy as np
import pytest

from cl2pt import lib, workloads

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-10  # relative to each spectrum's peak: the kernel is FP64 throughout


def _plan(w, prec, n, **kw):
    return lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=n, **kw)


def _close(got, ref, what):
    scale = np.abs(ref).max(axis=-1, keepdims=True)
    err = float(np.max(np.abs(got - ref) / scale))
    assert err <= TOL, (what, err)
    return err


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cmb_lensing_small", "cmb_lensing_tatt_small"])
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_cmb_vs_reference_golden(gpu_lib, case, prec):
    w = workloads.make(case)
    tabs, nus = workloads.points(w, 2, seed=11)
    plan = _plan(w, prec, 2, linear_table=True)
    # the one-loop bias tables come from the linear P(k)
    gk, ks, kk = plan.cmb_cl(*workloads.stack(tabs), nus, w.ell, lnPL=workloads.stack_lin(tabs))
    g = dict(np.load(os.path.join(GOLD, case + ".npz")))
    for i in range(2):
        _close(gk[i], g[f"Cgk_{i}"], "gk")
        _close(ks[i], g[f"Cks_{i}"], "ks")
        _close(kk[i][None], g[f"Ckk_{i}"][None], "kk")
    assert np.all(kk > 0)


@pytest.mark.gpu
def test_cmb_magnification_and_linear_mode(gpu_lib, oracle_built):
    """W_mag enters C_gk with l(l+1)/(l+1/2)^2; the linear run mode reads
    the linear table."""
    import oracle as O
    for linear in (False, True):
        w = workloads.make("cmb_lensing_small")
        if linear:
            w.cfg.linear_pk = 1
        tabs, nus = workloads.points(w, 2, seed=5, bmag=True)
        plan = _plan(w, lib.PREC_MIXED, 2, linear_table=True)
        gk, ks, kk = plan.cmb_cl(*workloads.stack(tabs), nus, w.ell, lnPL=workloads.stack_lin(tabs))
        o = O.Oracle("orc")
        o.setup(w.cfg, w.src, w.lens)
        for i in range(2):
            o.set_point(tabs[i], nus[i])
            ref = np.array([[o.C_cmb("gk", l, q) for l in w.ell] for q in range(w.cfg.n_lens)])
            _close(gk[i], ref, "gk")
            ref = np.array([o.C_cmb("kk", l) for l in w.ell])
            _close(kk[i][None], ref[None], "kk")


@pytest.mark.gpu
def test_cmb_batch_waves_and_null_outputs(gpu_lib):
    """More points than one wave of the plan (512 points), and outputs left
    out, give the same spectra as one point at a time."""
    n = 514
    w = workloads.make("cmb_lensing_small")
    tabs, nus = workloads.points(w, n, seed=9)
    plan = _plan(w, lib.PREC_MIXED, n)
    gk, ks, kk = plan.cmb_cl(*workloads.stack(tabs), nus, w.ell)
    for i in (0, 511, 512, 513):
        g1, k1, kk1 = plan.cmb_cl(*workloads.stack(tabs[i:i + 1]), nus[i:i + 1], w.ell)
        assert np.array_equal(g1[0], gk[i]) and np.array_equal(k1[0], ks[i]) and np.array_equal(kk1[0], kk[i])
    om, h0, chi, G, lnP = workloads.stack(tabs)
    b, keep = plan._host_batch(om, h0, chi, G, lnP, nus, None)
    ell = np.ascontiguousarray(w.ell)
    only = np.zeros((n, len(ell)))
    lib.check(lib.load().cl2pt_cmb_cl(plan.h, lib.C.byref(b), len(ell), lib._p(ell), None, None,
                                      only.ctypes.data, None), "cl2pt_cmb_cl")
    assert np.array_equal(only, kk)


@pytest.mark.gpu
def test_cmb_needs_last_scattering_in_table(gpu_lib):
    """A distance table that stops short of z = 1090 is refused."""
    w = workloads.make("real_3x2pt_small")
    tabs, nus = workloads.points(w, 1, seed=2)
    plan = _plan(w, lib.PREC_MIXED, 1)
    with pytest.raises(lib.CL2PTError):
        plan.cmb_cl(*workloads.stack(tabs), nus, [10.0, 100.0])
    w = workloads.make("cmb_lensing_small")
    tabs, nus = workloads.points(w, 1, seed=2)
    plan = _plan(w, lib.PREC_MIXED, 1)
    with pytest.raises(lib.CL2PTError):
        plan.cmb_cl(*workloads.stack(tabs), nus, [10.0, np.nan])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cmb_lensing_small", "cmb_lensing_tatt_small"])
def test_cmb_real_vs_reference_golden(gpu_lib, case):
    """w_gk and w_ks with the beam and pixel window (w_gk_tomo / w_ks_tomo,
    limber = 1) against the reference's own outputs; FP64 throughout, the
    map filter folded into the node filters on the host."""
    w = workloads.make(case)
    tabs, nus = workloads.points(w, 2, seed=11)
    plan = _plan(w, lib.PREC_MIXED, 2, linear_table=True)
    args = (*workloads.stack(tabs), nus)
    with pytest.raises(lib.CL2PTError):  # no map filter yet
        plan.cmb_real(*args, lnPL=workloads.stack_lin(tabs))
    f = workloads.cmb_map_filter()
    plan.set_cmb(f["lmin"], f["lmax"], f["fwhm_arcmin"], f["healpixwin"])
    wgk, wks = plan.cmb_real(*args, lnPL=workloads.stack_lin(tabs))
    g = dict(np.load(os.path.join(GOLD, case + ".npz")))
    worst = 0.0
    for i in range(2):
        for got, ref in ((wgk[i], g[f"wgk_{i}"]), (wks[i], g[f"wks_{i}"])):
            scale = np.abs(ref).max(axis=-1, keepdims=True)
            worst = max(worst, float(np.max(np.abs(got - ref) / scale)))
    print("w_gk / w_ks max error / peak", worst)
    assert worst <= 1e-9
    # no pixel window and a wider beam: a different filter, and the sums follow
    plan.set_cmb(f["lmin"], f["lmax"], 10.0)
    wgk2, _ = plan.cmb_real(*args, lnPL=workloads.stack_lin(tabs))
    assert not np.allclose(wgk2, wgk)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cmb_lensing_small", "cmb_lensing_tatt_small"])
def test_cmb_kk_dv_and_bandpowers(gpu_lib, case):
    """C_kk by the 6x2pt data vector's rule (nointerp at l <= lmin_tab, the
    ln l table above, its end value beyond l_max) and the kk bandpowers,
    against the reference's own outputs."""
    w = workloads.make(case)
    tabs, nus = workloads.points(w, 2, seed=11)
    plan = _plan(w, lib.PREC_MIXED, 2, linear_table=True)
    args = (*workloads.stack(tabs), nus)
    lnPL = workloads.stack_lin(tabs)
    kl = np.concatenate([w.ell, [float(w.cfg.lmin_tab), w.cfg.lmin_tab + 0.5, 7000.0]])
    kk = plan.cmb_kk(*args, kl, lnPL=lnPL)
    bp = plan.cmb_kk_bandpower(*args, *workloads.cmb_kk_bandpowers(), lnPL=lnPL)
    g = dict(np.load(os.path.join(GOLD, case + ".npz")))
    for i in range(2):
        _close(kk[i][None], g[f"Ckk_dv_{i}"][None], "kk_dv")
        _close(bp[i][None], g[f"kk_bp_{i}"][None], "kk_bp")
    assert kk[0, -1] == kk[0, -1] and np.all(bp != 0)
