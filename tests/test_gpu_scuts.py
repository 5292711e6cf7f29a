"""Scale-cut diagnostics of the cosmic-shear C_l (cosmolike/cosmo2D_scuts.c):
dC_ss/dlnk and dlnC_ss/dlnk on a (k, l) grid and the response fraction RF
against the FP64 oracle's restatement (dC_ss_dlnk_tomo_limber_nointerp,
the nointerp dlnC of int_RF_C_ss, RF_C_ss_tomo_limber_nointerp), both plans
(the diagnostics run in FP64 in both)."""
import numpy as np
import pytest

from cl2pt import abi, lib, workloads


def case(prec, seed=41):
    w = workloads.make("real_3x2pt_small_nla")
    tabs, nus = workloads.points(w, 2, seed=seed)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=2, linear_table=True)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    return w, tabs, nus, plan, (om, h0, chi, G, lnP), workloads.stack_lin(tabs)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_dlnk_vs_oracle(gpu_lib, oracle_built, prec):
    import oracle as O
    w, tabs, nus, plan, args, lnPL = case(prec)
    k = np.exp(np.linspace(np.log(1e-3), np.log(30.0), 23))
    l = np.array([2.0, 10.0, 37.5, 150.0, 800.0, 4000.0])
    dC, dlnC = plan.scut_ss_dlnk(*args, nus, k, l, lnPL=lnPL)
    assert np.all(dC[:, 1] == 0.0)  # no B modes without TATT
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    ns = w.cfg.n_source
    pairs = [(i, j) for i in range(ns) for j in range(i, ns)]
    worst = 0.0
    for pt in range(2):
        o.set_point(tabs[pt], nus[pt])
        for p, (i, j) in enumerate(pairs):
            C = np.array([o.C_ss_nointerp(lv, i, j, 1) for lv in l])
            ref = np.array([[o.dC_ss_dlnk(kv, lv, i, j) for lv in l] for kv in k])
            g = dC[pt, 0, p]
            scale = np.abs(ref).max()
            worst = max(worst, float(np.max(np.abs(g - ref)) / scale))
            refl = np.where(np.abs(C)[None, :] > 1e-30, ref / np.where(np.abs(ref) > 1e-30, C[None, :], 1.0), 0.0)
            assert np.allclose(dlnC[pt, 0, p], refl, rtol=1e-9, atol=1e-12 * np.abs(refl).max())
    print("dC/dlnk max error / peak", worst)
    assert worst <= 1e-9


@pytest.mark.gpu
def test_rf_vs_oracle(gpu_lib, oracle_built):
    import oracle as O
    w, tabs, nus, plan, args, lnPL = case(lib.PREC_FP64, seed=42)
    kmax = np.array([0.05, 0.3, 1.0, 5.0])
    l = np.array([30.0, 200.0, 1000.0, 300.0])
    rf = plan.scut_ss_rf(*args, nus, kmax, l, lnPL=lnPL)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    ns = w.cfg.n_source
    pairs = [(i, j) for i in range(ns) for j in range(i, ns)]
    o.set_point(tabs[1], nus[1])
    for p in (0, len(pairs) - 1):
        i, j = pairs[p]
        ref = np.array([o.RF_C_ss(km, lv, i, j) for km, lv in zip(kmax, l)])
        assert np.allclose(rf[1, 0, p], ref, rtol=1e-9, atol=1e-12), (p, rf[1, 0, p], ref)
        assert np.all(ref > 0)
    # RF grows with kmax at fixed l
    r2 = plan.scut_ss_rf(*args, nus, [0.1, 0.5, 2.0], [300.0] * 3, lnPL=lnPL)
    assert np.all(np.diff(r2[0, 0, 0]) > 0)


@pytest.mark.gpu
@pytest.mark.parametrize("gold", ["scale_cuts_small", "scale_cuts_tatt_small"])
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_scuts_vs_reference_golden(gpu_lib, prec, gold):
    """dC_ss/dlnk, RF_C_ss above lmin_tab, the real-space dlnxi/dlnk table
    and RF_xi against the reference's own outputs (tests/golden/<gold>.npz;
    the _tatt case with TATT intrinsic alignments: B modes, and the TATT
    terms of the E-mode integrand from the FAST-PT IA tables)."""
    import os
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", gold + ".npz")))
    tatt = "tatt" in gold
    w = workloads.make("real_3x2pt_tatt_small" if tatt else "real_3x2pt_small_nla")
    tabs, nus = workloads.points(w, 2, seed=41)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=2, linear_table=True)
    args = workloads.stack(tabs)
    lnPL = workloads.stack_lin(tabs)
    sc = workloads.scale_cut_requests()
    ns = w.cfg.n_source
    pairs = [(i, j) for i in range(ns) for j in range(i, ns)]
    dC, _ = plan.scut_ss_dlnk(*args, nus, sc["k"], sc["l"], lnPL=lnPL)
    dxi, dln = plan.scut_xi_dlnk(*args, nus, sc["nlnk"], sc["kmin"], sc["kmax"], lnPL=lnPL)
    rf = plan.scut_xi_rf(*args, nus, sc["xi_kmax"], sc["nlnk"], sc["kmin"], sc["kmax"], lnPL=lnPL)
    rfc = plan.scut_ss_rf(*args, nus, sc["rf_kmax"], sc["rf_l"], lnPL=lnPL,
                          grid=(sc["nlnk"], sc["kmin"], sc["kmax"]))
    assert np.all(dxi[:, :, :, :, 0] == 0.0)  # k = 1e-5: no source at chi = (l + 1/2) / k
    worst = {}
    for pt in range(2):
        for e, tag in ((0, ""), (1, "B")) if tatt else ((0, ""),):
            ref = g[f"dC{tag}_{pt}"]
            got = np.array([dC[pt, e, pairs.index(pq)] for pq in sc["pairs"]])
            worst["dC" + tag] = max(worst.get("dC" + tag, 0.0), float(np.max(np.abs(got - ref)) / np.abs(ref).max()))
            ref = g[f"rf{tag}_{pt}"]
            got = np.array([rfc[pt, e, pairs.index(pq)] for pq in sc["pairs"]])
            worst["rf_C" + tag] = max(worst.get("rf_C" + tag, 0.0), float(np.max(np.abs(got - ref))))
        ref = g[f"dlnxi_{pt}"]
        # the divisor of each slot (xi- for the xi+ slot and vice versa)
        xdiv = g[f"xi_{pt}"][::-1][:, :, :, None]
        # dxi/dlnk undivided (well conditioned everywhere)
        rd = ref * xdiv
        scale = np.abs(rd).max(axis=-1, keepdims=True) + 1e-300
        worst["dxi"] = max(worst.get("dxi", 0.0), float(np.max(np.abs(dxi[pt] - rd) / scale)))
        # the ratio where the divisor is not at a zero crossing of xi(theta)
        ok = np.abs(xdiv) > 1e-2 * np.abs(xdiv).max(axis=2, keepdims=True)
        scale = np.abs(ref).max(axis=-1, keepdims=True) + 1e-300
        worst["dlnxi"] = max(worst.get("dlnxi", 0.0), float(np.max(np.where(ok, np.abs(dln[pt] - ref) / scale, 0.0))))
        ref = g[f"rfxi_{pt}"]
        worst["rf"] = max(worst.get("rf", 0.0), float(np.max(np.abs(rf[pt] - ref))))
    print(gold, "scale cuts vs reference", worst)
    # TATT: the FAST-PT IA rows are the GPU's own (2e-7 of the reference's,
    # the rows' FP64 conditioning), so the TATT terms carry that error
    tol = 1e-6 if tatt else 1e-9
    for k, v in worst.items():
        assert v <= (100 * tol if k in ("dxi", "dlnxi", "rf") else tol), (k, v, worst)
