"""Baryon PCA (cl2pt_baryon_pcas) against compute_baryon_pcas_Mx2pt_N's
algorithm (generic_interface.hpp:1168-1225) restated in numpy on the FP64
oracle's data vectors: Cholesky of the masked covariance, SVD of
L^-1 (dv_scenario - dv_dm), PCs L U_i expanded to the full vector.  PCs are
compared up to sign (singular vectors are defined up to sign)."""
import numpy as np
import pytest

from cl2pt import lib, workloads


def reference_pcas(dvs, mask, cov):
    """compute_baryon_pcas_Mx2pt_N's linear algebra on the data vectors dvs
    (no baryons first, then one per scenario)."""
    keep = mask == 1
    dvs = [d[keep] for d in dvs]
    D = np.stack([d - dvs[0] for d in dvs[1:]], axis=1)
    L = np.linalg.cholesky(cov[np.ix_(keep, keep)])
    U, S, Vt = np.linalg.svd(np.linalg.solve(L, D), full_matrices=False)
    PC = L @ U
    R = np.zeros((D.shape[1], len(mask)))
    R[:, keep] = PC.T
    return R, S


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_MIXED])
def test_baryon_pcas_vs_reference_algorithm(gpu_lib, oracle_built, prec):
    import oracle as O
    w = workloads.make("real_3x2pt_small")
    tabs, nus = workloads.points(w, 1, seed=61)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=1, linear_table=True)
    args = (*workloads.stack(tabs), nus)
    lnPL = workloads.stack_lin(tabs)
    rng = np.random.default_rng(5)
    dv0 = plan.eval_real(*args, lnPL=lnPL)[0]
    n = plan.n_total
    mask = (rng.uniform(size=n) < 0.85).astype(np.int32)
    sig = 0.05 * np.abs(dv0) + 1e-3 * np.abs(dv0).max()
    U = rng.normal(size=(n, 5)) * sig[:, None] * 0.3
    cov = np.diag(sig ** 2) + U @ U.T
    keep = mask == 1
    inv = np.zeros((n, n))
    inv[np.ix_(keep, keep)] = np.linalg.inv(cov[np.ix_(keep, keep)])
    like = plan.likelihood(dv0, inv, mask)
    lk, a, lr = workloads.baryon_scenarios(4)
    # the plan's own baryon ratio survives the call
    plan.set_baryon_ratio(lk, a, lr[1])
    before = plan.eval_real(*args, lnPL=lnPL)
    R = plan.baryon_pcas(like, *args, lk, a, lr, lnPL=lnPL)
    assert np.array_equal(plan.eval_real(*args, lnPL=lnPL), before)
    assert np.all(R[:, ~keep] == 0.0)

    def pc_errors(ref):
        return [min(np.abs(R[i] - ref[i]).max(), np.abs(R[i] + ref[i]).max()) / np.abs(ref[i]).max()
                for i in range(len(ref))]

    # (1) the PCA itself: the reference's algorithm on this plan's own data
    # vectors (the FP64 Gram product and Jacobi solve against numpy's
    # Cholesky and SVD)
    dvs = []
    for i in range(-1, lr.shape[0]):
        if i < 0:
            plan.set_baryon_ratio([], [], [])
        else:
            plan.set_baryon_ratio(lk, a, lr[i])
        dvs.append(plan.eval_real(*args, mask=mask, lnPL=lnPL)[0])
    ref, S = reference_pcas(dvs, mask, cov)
    e1 = pc_errors(ref)
    # (2) the chain: the oracle's data vectors, which apply each ratio per
    # evaluation as the reference does (the plan folds ln R into its table:
    # a second-order difference, a few 1e-5 of the data vector)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    odv = []
    for i in range(-1, lr.shape[0]):
        o.set_baryon_ratio(*(([], [], []) if i < 0 else (lk, a, lr[i])))
        o.set_point(tabs[0], nus[0])
        odv.append(o.data_vector_real(mask=mask))
    o.set_baryon_ratio([], [], [])
    ref2, S2 = reference_pcas(odv, mask, cov)
    e2 = pc_errors(ref2)
    print(prec, "singular values", S, "PCA errors / peak", e1, "vs oracle chain", e2)
    assert max(e1) <= 1e-8, e1
    assert max(e2) <= 2e-3, e2
