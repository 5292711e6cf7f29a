"""Adjoint of the Fourier-space vector (cl2pt_vjp_fourier) against central
differences of the FP64 forward: the Limber passes at the caller's
multipoles, and below LMAX_NOLIMBER the FFTLog clustering with its Limber
hand-over.  Same conventions as tests/test_gpu_vjp.py."""
import numpy as np
import pytest

from cl2pt import abi, lib, workloads
from test_gpu_vjp import GRAD_REL, H, clone, fd_step, flat_index, nu_get, nu_set, set_bk


def case(name, prec, seed, ia_mode=abi.IA_REDSHIFT_EVOLUTION, npts=2, ell=None, linear_table=False, bmag=False):
    w = workloads.make(name)
    if w.cfg.ia_model == abi.IA_NLA:
        w.cfg.ia_mode = ia_mode
    tabs, nus = workloads.points(w, npts, seed=seed, bmag=bmag)
    rng = np.random.default_rng(seed)
    if w.cfg.ia_model == abi.IA_NLA and ia_mode == abi.IA_REDSHIFT_EVOLUTION:
        for nu in nus:
            nu.ia[0][0] = rng.uniform(0.3, 1.0)
            nu.ia[0][1] = rng.uniform(-1.5, 1.5)
    p64 = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64, max_batch=npts, linear_table=linear_table)
    plan = p64 if prec == lib.PREC_FP64 else lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=npts,
                                                      linear_table=linear_table)
    ell = w.ell if ell is None else ell
    return w, tabs, nus, p64, plan, ell


def params(w, mag=False):
    ps = [("shear_m", s, None) for s in range(w.cfg.n_source)]
    ps += [("src_dz", s, None) for s in range(w.cfg.n_source)]
    ps += [("gb", 0, q) for q in range(w.cfg.n_lens)]
    if mag:
        ps += [("gb", 4, q) for q in range(w.cfg.n_lens)]
    if w.cfg.ia_model == abi.IA_TATT:
        ps += [("gb", k, q) for k in (1, 2, 5) for q in range(w.cfg.n_lens)]
        ps += [("ia", 0, 0), ("ia", 0, 1), ("ia", 1, 0), ("ia", 1, 1), ("ia", 2, 0)]
    else:
        ps += [("ia", 0, 0), ("ia", 0, 1)]
    return ps


def check(w, tabs, nus, p64, plan, ell, tol, lmax_shear=1e30, separate_linear=False, mag=False):
    """separate_linear: pass the linear table on its own (TATT / one-loop:
    the FAST-PT tables read it and their dependence is not differentiated, so
    the lnP direction is checked on the nonlinear table alone)."""
    om, h0, chi, G, lnP = workloads.stack(tabs)
    lnPL = np.stack([t.lnPL.reshape(-1) for t in tabs]) if separate_linear else None
    n = len(tabs)
    rng = np.random.default_rng(77)
    dv0 = p64.eval_fourier(om, h0, chi, G, lnP, nus, ell, lmax_shear=lmax_shear, lnPL=lnPL)
    v = rng.normal(size=dv0.shape)
    out = plan.vjp_fourier(om, h0, chi, G, lnP, nus, ell, v, lmax_shear=lmax_shear, lnPL=lnPL)
    dv, lbar, nbar = out[:3]
    worst = 0.0
    for pt in range(n):
        sl = slice(pt, pt + 1)
        lpl = None if lnPL is None else lnPL[sl]
        f = lambda nu, lp=lnP[sl]: float(v[pt] @ p64.eval_fourier(om[sl], h0[sl], chi[sl], G[sl], lp, [nu], ell,
                                                                  lmax_shear=lmax_shear, lnPL=lpl)[0])
        for field, i, j in params(w, mag):
            x0 = nu_get(nus[pt], field, i, j)
            h = fd_step(field, i, x0)
            fs = []
            for sgn in (1, -1):
                nu = clone(nus[pt])
                nu_set(nu, field, i, j, x0 + sgn * h)
                fs.append(f(nu))
            fd = (fs[0] - fs[1]) / (2 * h)
            an = nbar[pt, flat_index(field, i, j)]
            # floor: the round-off of the difference quotient, ~eps |f| / h
            err = abs(an - fd) / max(abs(fd), 1e-9 * abs(fs[0]) / h)
            worst = max(worst, err)
            assert err <= tol, (field, i, j, an, fd)
        f0 = abs(f(nus[pt]))
        floor = 1e-9 * f0 / H  # round-off of the difference quotient
        for u in (rng.normal(size=lnP.shape[1]),):
            fs = [f(nus[pt], lnP[sl] + s * H * u) for s in (1, -1)]
            fd = (fs[0] - fs[1]) / (2 * H)
            assert abs(lbar[pt] @ u - fd) <= tol * max(abs(fd), floor), (lbar[pt] @ u, fd)
        # the z = 0 columns (FFTLog P_lin slice and low-z Limber nodes)
        nk, nz = p64.shapes["nk"], p64.shapes["nz"]
        u0 = np.zeros((nk, nz))
        u0[:, :2] = rng.normal(size=(nk, 2))
        u0 = u0.reshape(-1)
        fs = [f(nus[pt], lnP[sl] + s * H * u0) for s in (1, -1)]
        fd = (fs[0] - fs[1]) / (2 * H)
        assert abs(lbar[pt] @ u0 - fd) <= tol * max(abs(fd), floor), (lbar[pt] @ u0, fd)
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_MIXED])
def test_vjp_fourier_nonlimber(gpu_lib, prec):
    """The serving layout at reduced size: 4 + 3 bins, 12 log l bins in
    20-15000, five of them below LMAX_NOLIMBER = 200 (FFTLog clustering)."""
    w, tabs, nus, p64, plan, ell = case("fourier_serving_small", prec, seed=61)
    worst = check(w, tabs, nus, p64, plan, ell, GRAD_REL if prec == lib.PREC_FP64 else 2e-5,
                  lmax_shear=0.7 * w.ell[-1])
    print("Fourier non-Limber max rel gradient error", worst)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_MIXED])
def test_vjp_fourier_magnification(gpu_lib, prec):
    """bmag != 0 in every lens bin on the serving layout at reduced size
    (Limber W_mag terms at the caller's multipoles, the FFTLog
    magnification kernel below LMAX_NOLIMBER)."""
    w, tabs, nus, p64, plan, ell = case("fourier_serving_small", prec, seed=65, bmag=True)
    worst = check(w, tabs, nus, p64, plan, ell, GRAD_REL if prec == lib.PREC_FP64 else 2e-5,
                  lmax_shear=0.7 * w.ell[-1], mag=True)
    print("Fourier magnification max rel gradient error", worst)


@pytest.mark.gpu
def test_vjp_fourier_tatt(gpu_lib):
    """TATT + one-loop bias (bK set on the second point) and magnification
    on the Fourier vector (FP64)."""
    ell = np.exp(np.log(20.0) + (np.arange(10) + 0.5) * (np.log(3000.0) - np.log(20.0)) / 10)
    w, tabs, nus, p64, plan, ell = case("real_3x2pt_tatt_small", lib.PREC_FP64, seed=63, ell=ell,
                                        linear_table=True, bmag=True)
    set_bk(nus, w, 63)
    worst = check(w, tabs, nus, p64, plan, ell, GRAD_REL, separate_linear=True, mag=True)
    print("Fourier TATT max rel gradient error", worst)


@pytest.mark.gpu
def test_vjp_fourier_lens_photoz(gpu_lib):
    """Lens photo-z shift and stretch gradients of the Fourier vector
    (cl2pt_plan_set_lens_photoz_grad) against central differences of the
    FP64 forward with the same step."""
    w, tabs, nus, p64, plan, ell = case("fourier_serving_small", lib.PREC_FP64, seed=67)
    rng = np.random.default_rng(9)
    for q in range(w.cfg.n_lens):
        nus[0].lens_stretch[q] = float(rng.uniform(0.9, 1.1))
    om, h0, chi, G, lnP = workloads.stack(tabs)
    lm = 0.7 * w.ell[-1]
    dv0 = p64.eval_fourier(om, h0, chi, G, lnP, nus, ell, lmax_shear=lm)
    v = rng.normal(size=dv0.shape)
    plan.set_lens_photoz_grad(True, 1e-4, 1e-4)
    nbar = plan.vjp_fourier(om, h0, chi, G, lnP, nus, ell, v, lmax_shear=lm)[2]
    worst = 0.0
    for pt in range(len(tabs)):
        sl = slice(pt, pt + 1)
        for field in ("lens_dz", "lens_stretch"):
            for q in range(w.cfg.n_lens):
                fs = []
                for s in (1, -1):
                    nu = clone(nus[pt])
                    getattr(nu, field)[q] += s * 1e-4
                    fs.append(float(v[pt] @ p64.eval_fourier(om[sl], h0[sl], chi[sl], G[sl], lnP[sl], [nu], ell,
                                                             lmax_shear=lm)[0]))
                fd = (fs[0] - fs[1]) / 2e-4
                an = nbar[pt, flat_index(field, q)]
                worst = max(worst, abs(an - fd) / abs(fd))
                assert abs(an - fd) <= 1e-9 * abs(fd), (pt, field, q, an, fd)
    print("Fourier lens photo-z gradient max rel err vs the forward's differences", worst)


@pytest.mark.gpu
def test_vjp_fourier_torch_autograd(gpu_lib):
    """torch.autograd.Function of the Fourier vector: the forward equals
    eval_fourier and the backward of sum(v * dv) equals vjp_fourier on the
    same host inputs (mixed plan, serving layout at reduced size)."""
    import torch
    from cl2pt import autograd as AG
    w, tabs, nus, p64, plan, ell = case("fourier_serving_small", lib.PREC_MIXED, seed=69)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    lm = 0.7 * w.ell[-1]
    ref = plan.eval_fourier(om, h0, chi, G, lnP, nus, ell, lmax_shear=lm)
    v = np.random.default_rng(13).normal(size=ref.shape)
    _, lbar, nbar = plan.vjp_fourier(om, h0, chi, G, lnP, nus, ell, v, lmax_shear=lm)
    dev = torch.device("cuda:0")
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    nu_t = T(np.stack([abi.nuisance_to_array(n) for n in nus])).requires_grad_(True)
    lnP_t = T(lnP).requires_grad_(True)
    dv = AG.fourier_data_vector(plan, T(om), T(h0), T(chi), T(G), lnP_t, nu_t, ell, lmax_shear=lm)
    assert dv.shape == ref.shape == (len(tabs), plan.fourier_n_total(len(ell)))
    np.testing.assert_allclose(dv.detach().cpu().numpy(), ref, rtol=1e-12, atol=1e-15 * np.abs(ref).max())
    (dv * T(v)).sum().backward()
    torch.cuda.synchronize()
    # two runs of the mixed plan's adjoint: its atomic scatters sum in
    # run-dependent order (measured: a few of the 80000 lnP entries differ,
    # by at most 5.7e-14 against a largest entry of 5.4e-6); a wrong routing
    # would differ at order one
    np.testing.assert_allclose(lnP_t.grad.cpu().numpy(), lbar, rtol=1e-5, atol=1e-6 * np.abs(lbar).max())
    np.testing.assert_allclose(nu_t.grad.cpu().numpy(), nbar, rtol=1e-5, atol=1e-6 * np.abs(nbar).max())
