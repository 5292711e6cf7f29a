"""Likelihood epilogue (cl2pt_loglike_real): chi2 against numpy on the same
GPU data vectors (the split-FP32 product with FP64 chunk sums: 1e-7
relative, i.e. ~1e-4 absolute on chi2 ~ 1e3, far below what a sampler
resolves), and the gradient of ln L = -chi2/2 against central differences
and against cl2pt_vjp_real with the cotangent -C^-1 (dv - data)."""
import numpy as np
import pytest

from cl2pt import abi, lib, workloads
from test_gpu_vjp import GRAD_REL, H, clone, flat_index, nu_get, nu_set, param_list, setup_case


def make_like(plan, dv_ref, rng):
    n = plan.n_total
    mask = (rng.uniform(size=n) < 0.8).astype(np.int32)
    # a positive-definite covariance: diagonal errors of 5 % plus a
    # low-rank correlated part
    sig = 0.05 * np.abs(dv_ref) + 1e-3 * np.abs(dv_ref).max()
    U = rng.normal(size=(n, 6)) * sig[:, None] * 0.3
    cov = np.diag(sig ** 2) + U @ U.T
    keep = mask == 1
    inv = np.zeros((n, n))
    inv[np.ix_(keep, keep)] = np.linalg.inv(cov[np.ix_(keep, keep)])
    data = dv_ref + rng.normal(size=n) * sig
    return mask, data, inv


@pytest.mark.gpu
def test_chi2_and_gradient(gpu_lib):
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, npts=3, seed=71, name="real_3x2pt_small")
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(3)
    dv_ref = plan.eval_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1], nus[:1])[0]
    mask, data, inv = make_like(plan, dv_ref, rng)
    like = plan.likelihood(data, inv, mask)
    chi2 = plan.loglike_real(like, om, h0, chi, G, lnP, nus)
    dv = plan.eval_real(om, h0, chi, G, lnP, nus, mask=mask)
    d = np.where(mask == 1, dv - data, 0.0)
    ref = np.einsum("pi,ij,pj->p", d, inv, d)
    np.testing.assert_allclose(chi2, ref, rtol=1e-7)
    # gradient of ln L
    c2, lbar, nbar = plan.loglike_real(like, om, h0, chi, G, lnP, nus, grad=True)
    np.testing.assert_allclose(c2, chi2, rtol=1e-12)
    cot = -(d @ inv) * (mask == 1)
    _, l2, n2 = plan.vjp_real(om, h0, chi, G, lnP, nus, cot, mask=mask)
    np.testing.assert_allclose(lbar, l2, rtol=1e-7, atol=1e-7 * np.abs(l2).max())
    np.testing.assert_allclose(nbar, n2, rtol=1e-7, atol=1e-7 * np.abs(n2).max())
    for pt in range(2):
        sl = slice(pt, pt + 1)
        for field, i, j in param_list(w, abi.IA_REDSHIFT_EVOLUTION)[::3]:
            x0 = nu_get(nus[pt], field, i, j)
            h = H * max(abs(x0), 0.1)
            f = []
            for s in (1, -1):
                nu = clone(nus[pt])
                nu_set(nu, field, i, j, x0 + s * h)
                # ln L in FP64 on the host from the FP64 plan's vector (smooth
                # in the parameter, unlike the split-FP32 product's rounding)
                dvp = plan.eval_real(om[sl], h0[sl], chi[sl], G[sl], lnP[sl], [nu], mask=mask)[0]
                dd = np.where(mask == 1, dvp - data, 0.0)
                f.append(-0.5 * dd @ inv @ dd)
            fd = (f[0] - f[1]) / (2 * h)
            an = nbar[pt, flat_index(field, i, j)]
            assert abs(an - fd) <= 1e-5 * max(abs(fd), 1e-9 * abs(f[0]) / h), (field, i, j, an, fd)
    like.close()


@pytest.mark.gpu
def test_loglike_lens_photoz_gradient(gpu_lib):
    """With the lens photo-z gradients on, the likelihood's gradient carries
    them too, equal to the adjoint's with the cotangent -C^-1 (dv - data)."""
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, npts=2, seed=72, name="real_3x2pt_small")
    tabs = workloads.one_table(tabs)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(4)
    dv_ref = plan.eval_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1], nus[:1])[0]
    mask, data, inv = make_like(plan, dv_ref, rng)
    like = plan.likelihood(data, inv, mask)
    plan.set_lens_photoz_grad(True)
    c2, lbar, nbar = plan.loglike_real(like, om, h0, chi, G, lnP, nus, grad=True)
    dv = plan.eval_real(om, h0, chi, G, lnP, nus, mask=mask)
    d = np.where(mask == 1, dv - data, 0.0)
    cot = -(d @ inv) * (mask == 1)
    _, _, n2 = plan.vjp_real(om, h0, chi, G, lnP, nus, cot, mask=mask)
    idx = [flat_index(f, q) for f in ("lens_dz", "lens_stretch") for q in range(w.cfg.n_lens)]
    assert np.all(nbar[:, idx] != 0.0)
    np.testing.assert_allclose(nbar[:, idx], n2[:, idx], rtol=1e-6, atol=1e-9 * np.abs(n2[:, idx]).max())
