"""Adjoint of the real-space 3x2pt data vector (cl2pt_vjp_real) against
central finite differences.

For a seeded cotangent v, the scalar f = v . dv is differentiated
  * on the GPU: central differences of the FP64 plan's forward,
  * on the CPU: central differences of the FP64 oracle (the restatement of
    the reference C path),
with respect to the shear m-bias, the source photo-z shifts, b1, the NLA
amplitude and its redshift power, and the P(k, z) table (a dense random direction and single entries).
Step: 1e-4 relative (1e-4 absolute in lnP).  Every quantity here is smooth
in the parameters (the bilinear table walk is linear in the table values;
b1 and A1 enter polynomially), so the analytic gradient must match the
GPU differences to GRAD_REL and the oracle differences to the data-vector
bar of 1e-4.
"""
import numpy as np
import pytest

from cl2pt import abi, lib, workloads

GRAD_REL = 1e-6   # analytic vs FD of the same FP64 forward
ORACLE_REL = 1e-4  # analytic vs FD of the oracle
H = 1e-4


def setup_case(ia_mode=abi.IA_REDSHIFT_EVOLUTION, npts=2, seed=21, prec=lib.PREC_FP64, name="real_3x2pt_small_limber",
               bmag=False):
    w = workloads.make(name)
    w.cfg.ia_mode = ia_mode
    tabs, nus = workloads.points(w, npts, seed=seed, bmag=bmag)
    rng = np.random.default_rng(seed)
    for nu in nus:
        if ia_mode == abi.IA_REDSHIFT_EVOLUTION:
            nu.ia[0][0] = rng.uniform(0.3, 1.0)
            nu.ia[0][1] = rng.uniform(-1.5, 1.5)
        elif ia_mode == abi.IA_REDSHIFT_BINNING:
            for s in range(w.cfg.n_source):
                nu.ia[0][s] = rng.uniform(-1.0, 1.0)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=npts)
    return w, tabs, nus, plan


def nu_get(nu, field, i, j=None):
    a = getattr(nu, field)
    return a[i] if j is None else a[i][j]


def nu_set(nu, field, i, j, v):
    a = getattr(nu, field)
    if j is None:
        a[i] = v
    else:
        a[i][j] = v


def flat_index(field, i, j=None):
    """Index of a cl2pt_nuisance field in the flat float64 layout."""
    off = {"src_dz": 0, "lens_dz": 1, "lens_stretch": 2, "shear_m": 3, "gb": 4, "ia": 10}[field]
    if j is None:
        return off * abi.MAX_BINS + i
    return (off + i) * abi.MAX_BINS + j


def param_list(w, ia_mode, mag=False):
    """mag: also bmag (gb[4]), for points with bmag != 0 in every lens bin."""
    ps = [("shear_m", s, None) for s in range(w.cfg.n_source)]
    ps += [("src_dz", s, None) for s in range(w.cfg.n_source)]
    ps += [("gb", 0, q) for q in range(w.cfg.n_lens)]
    if mag:
        ps += [("gb", 4, q) for q in range(w.cfg.n_lens)]
    if ia_mode == abi.IA_REDSHIFT_EVOLUTION:
        ps += [("ia", 0, 0), ("ia", 0, 1)]
    elif ia_mode == abi.IA_REDSHIFT_BINNING:
        ps += [("ia", 0, s) for s in range(w.cfg.n_source)]
    return ps


def clone(nu):
    c = abi.Nuisance()
    C = __import__("ctypes")
    C.memmove(C.addressof(c), C.addressof(nu), C.sizeof(nu))
    return c


def check_nuisance_fd(plan, w, tabs, nus, v, nbar, ia_mode, point, mask=None, pm=None):
    om, h0, chi, G, lnP = workloads.stack(tabs)
    sl = slice(point, point + 1)
    worst = 0.0
    for field, i, j in param_list(w, ia_mode):
        x0 = nu_get(nus[point], field, i, j)
        h = H * max(abs(x0), 0.1)
        f = []
        for sgn in (1, -1):
            nu = clone(nus[point])
            nu_set(nu, field, i, j, x0 + sgn * h)
            dv = plan.eval_real(om[sl], h0[sl], chi[sl], G[sl], lnP[sl], [nu], mask=mask,
                                pm=None if pm is None else pm[sl])[0]
            f.append(float(v[point] @ dv))
        fd = (f[0] - f[1]) / (2 * h)
        an = nbar[point, flat_index(field, i, j)]
        # floor: the round-off of the difference quotient, ~eps |f| / h
        scale = max(abs(fd), 1e-9 * max(abs(f[0]), 1e-300) / h)
        err = abs(an - fd) / scale
        worst = max(worst, err)
        assert err <= GRAD_REL, (field, i, j, an, fd, err)
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("ia_mode", [abi.IA_REDSHIFT_EVOLUTION, abi.IA_REDSHIFT_BINNING, abi.NO_IA])
def test_vjp_nuisance_vs_gpu_fd(gpu_lib, ia_mode):
    w, tabs, nus, plan = setup_case(ia_mode)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(5)
    v = rng.normal(size=(len(tabs), plan.n_total))
    dv, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    # the value equals the forward
    assert np.array_equal(dv, plan.eval_real(om, h0, chi, G, lnP, nus))
    for pt in range(len(tabs)):
        worst = check_nuisance_fd(plan, w, tabs, nus, v, nbar, ia_mode, pt)
        print("nuisance max rel err vs GPU FD", worst)
    # fields the adjoint does not cover stay zero
    covered = {flat_index(*p) for p in param_list(w, ia_mode)}
    other = [k for k in range(nbar.shape[1]) if k not in covered]
    assert np.all(nbar[:, other] == 0.0)


@pytest.mark.gpu
def test_vjp_lnP_vs_gpu_fd(gpu_lib):
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(6)
    v = rng.normal(size=(len(tabs), plan.n_total))
    _, lbar, _ = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    assert np.all(np.isfinite(lbar)) and np.any(lbar != 0)
    for pt in range(len(tabs)):
        sl = slice(pt, pt + 1)
        # dense random direction
        u = rng.normal(size=lnP.shape[1])
        f = [float(v[pt] @ plan.eval_real(om[sl], h0[sl], chi[sl], G[sl], lnP[sl] + s * H * u, nus[sl])[0])
             for s in (1, -1)]
        fd = (f[0] - f[1]) / (2 * H)
        an = float(lbar[pt] @ u)
        assert abs(an - fd) <= GRAD_REL * abs(fd), (an, fd)
        # single entries: the largest gradients and random touched ones
        top = np.argsort(-np.abs(lbar[pt]))[:4]
        nz = np.flatnonzero(lbar[pt])
        pick = np.concatenate([top, rng.choice(nz, 4, replace=False)])
        for k in pick:
            e = np.zeros(lnP.shape[1])
            e[k] = H
            f = [float(v[pt] @ plan.eval_real(om[sl], h0[sl], chi[sl], G[sl], lnP[sl] + s * e, nus[sl])[0])
                 for s in (1, -1)]
            fd = (f[0] - f[1]) / (2 * H)
            assert abs(lbar[pt, k] - fd) <= GRAD_REL * np.max(np.abs(lbar[pt])), (k, lbar[pt, k], fd)
        # untouched entries have zero gradient: a step there changes nothing
        zero = np.flatnonzero(lbar[pt] == 0)
        k = rng.choice(zero)
        e = np.zeros(lnP.shape[1])
        e[k] = 1.0
        d0 = plan.eval_real(om[sl], h0[sl], chi[sl], G[sl], lnP[sl], nus[sl])
        d1 = plan.eval_real(om[sl], h0[sl], chi[sl], G[sl], lnP[sl] + e, nus[sl])
        assert np.array_equal(d0, d1)


@pytest.mark.gpu
def test_vjp_mask_point_mass(gpu_lib):
    """Masked entries carry no gradient; the point-mass term enters the
    m-bias gradient of gamma_t."""
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, npts=1, seed=4)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(8)
    mask = (rng.uniform(size=plan.n_total) < 0.6).astype(np.int32)
    pm = rng.uniform(0.0, 3.0, size=(1, w.cfg.n_lens))
    v = rng.normal(size=(1, plan.n_total))
    dv, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v, mask=mask, pm=pm)
    check_nuisance_fd(plan, w, tabs, nus, v, nbar, abi.IA_REDSHIFT_EVOLUTION, 0, mask=mask, pm=pm)
    v2 = np.where(mask == 1, v, rng.normal(size=v.shape))  # masked cotangents are ignored
    _, lbar2, nbar2 = plan.vjp_real(om, h0, chi, G, lnP, nus, v2, mask=mask, pm=pm)
    np.testing.assert_allclose(lbar2, lbar, rtol=1e-12, atol=1e-12 * np.abs(lbar).max())
    np.testing.assert_allclose(nbar2, nbar, rtol=1e-12, atol=1e-12 * np.abs(nbar).max())


@pytest.mark.gpu
def test_vjp_mixed_plan_matches_fp64(gpu_lib):
    """The mixed plan's adjoint (FP32 per-(l, node) arithmetic, FP64
    accumulators) against the FP64 plan's: 1e-5 of the largest entry for the
    table gradient, 1e-5 relative for the nuisance gradient."""
    w, tabs, nus, p64 = setup_case(abi.IA_REDSHIFT_EVOLUTION)
    pmx = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=len(tabs))
    om, h0, chi, G, lnP = workloads.stack(tabs)
    v = np.random.default_rng(9).normal(size=(len(tabs), p64.n_total))
    _, l64, n64 = p64.vjp_real(om, h0, chi, G, lnP, nus, v)
    _, lmx, nmx = pmx.vjp_real(om, h0, chi, G, lnP, nus, v)
    err_l = np.max(np.abs(lmx - l64)) / np.max(np.abs(l64))
    keep = n64 != 0
    err_n = np.max(np.abs(nmx[keep] - n64[keep]) / np.abs(n64[keep]))
    print("mixed vs FP64 adjoint:", err_l, err_n)
    assert err_l <= 1e-5 and err_n <= 1e-5
    assert np.all(nmx[~keep] == 0)


@pytest.mark.gpu
def test_vjp_vs_oracle_fd(gpu_lib, oracle_built):
    """Central differences of the FP64 oracle (the reference C path
    restated) against the analytic gradient: m, b1, A1, eta and a lnP
    direction of one point."""
    import oracle as O
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, npts=1, seed=13)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(10)
    v = rng.normal(size=(1, plan.n_total))
    _, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    import dataclasses
    worst = 0.0
    for field, i, j in [("shear_m", 0, None), ("shear_m", 3, None), ("src_dz", 1, None), ("src_dz", 3, None),
                        ("gb", 0, 1), ("ia", 0, 0), ("ia", 0, 1)]:
        x0 = nu_get(nus[0], field, i, j)
        h = H * max(abs(x0), 0.1)
        f = []
        for s in (1, -1):
            nu = clone(nus[0])
            nu_set(nu, field, i, j, x0 + s * h)
            o.set_point(tabs[0], nu)
            f.append(float(v[0] @ o.data_vector_real()))
        fd = (f[0] - f[1]) / (2 * h)
        an = nbar[0, flat_index(field, i, j)]
        err = abs(an - fd) / abs(fd)
        worst = max(worst, err)
        assert err <= ORACLE_REL, (field, i, j, an, fd)
    u = rng.normal(size=lnP.shape[1])
    f = []
    for s in (1, -1):
        t = dataclasses.replace(tabs[0], lnP=np.ascontiguousarray(
            (tabs[0].lnP.reshape(-1) + s * H * u).reshape(tabs[0].lnP.shape)))
        o.set_point(t, nus[0])
        f.append(float(v[0] @ o.data_vector_real()))
    fd = (f[0] - f[1]) / (2 * H)
    an = float(lbar[0] @ u)
    worst = max(worst, abs(an - fd) / abs(fd))
    print("max rel gradient error vs oracle FD", worst)
    assert abs(an - fd) <= ORACLE_REL * abs(fd), (an, fd)


@pytest.mark.gpu
def test_vjp_torch_autograd(gpu_lib):
    """torch.autograd.Function: backward of sum(v * dv) equals the VJP, and
    the fused value_and_vjp agrees."""
    import torch
    from cl2pt import autograd as AG
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    v = np.random.default_rng(11).normal(size=(len(tabs), plan.n_total))
    _, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    dev = torch.device("cuda:0")
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    nu_t = T(np.stack([abi.nuisance_to_array(n) for n in nus]))
    lnP_t = T(lnP).requires_grad_(True)
    nu_t.requires_grad_(True)
    dv = AG.real_data_vector(plan, T(om), T(h0), T(chi), T(G), lnP_t, nu_t)
    (dv * T(v)).sum().backward()
    torch.cuda.synchronize()
    np.testing.assert_allclose(lnP_t.grad.cpu().numpy(), lbar, rtol=1e-12, atol=1e-14 * np.abs(lbar).max())
    np.testing.assert_allclose(nu_t.grad.cpu().numpy(), nbar, rtol=1e-12, atol=1e-14 * np.abs(nbar).max())
    dv2, l2, n2 = AG.value_and_vjp(plan, T(om), T(h0), T(chi), T(G), T(lnP), nu_t.detach(), T(v))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dv2.cpu().numpy(), dv.detach().cpu().numpy())
    np.testing.assert_allclose(l2.cpu().numpy(), lbar, rtol=1e-12, atol=1e-14 * np.abs(lbar).max())


def lnp_direction_fd(plan, tabs, nus, v, pt, u, lnPL=None, which="lnP", step=None):
    """Central difference of v . dv along u in lnP (or in lnPL).  The
    non-Limber hand-over multipole is a discrete choice the gradient holds
    fixed: with non-Limber w(theta) the step shrinks until it is the same at
    both ends."""
    om, h0, chi, G, lnP = workloads.stack(tabs)
    sl = slice(pt, pt + 1)

    def tables(s, h):
        a, b = lnP[sl], None if lnPL is None else lnPL[sl]
        if which == "lnP":
            a = a + s * h * u
        else:
            b = b + s * h * u
        return a, b

    h = H if step is None else step
    for _ in range(4):
        try:
            conv = []
            for s in (1, -1):
                a, b = tables(s, h)
                conv.append(plan.cl_nonlimber(om[sl], h0[sl], chi[sl], G[sl], a, nus[sl], lnPL=b)[1])
        except lib.CL2PTError:
            break  # Limber-only plan: no hand-over
        if np.array_equal(conv[0], conv[1]):
            break
        h /= 4
    f = []
    for s in (1, -1):
        a, b = tables(s, h)
        f.append(float(v[pt] @ plan.eval_real(om[sl], h0[sl], chi[sl], G[sl], a, nus[sl], lnPL=b)[0]))
    return (f[0] - f[1]) / (2 * h)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_MIXED])
def test_vjp_nonlimber_vs_gpu_fd(gpu_lib, prec):
    """Non-Limber w(theta): the adjoint runs through the FFTLog C_l (b1 and
    the z = 0 slice of the linear table), the integer-l Limber spectra and
    the hand-over; checked against differences of the FP64 forward.  The
    mixed plan's FFTLog adjoint runs in FP32: 1e-5 against the FP64 one."""
    w, tabs, nus, p64 = setup_case(abi.IA_REDSHIFT_EVOLUTION, name="real_3x2pt_small", seed=31)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(12)
    v = rng.normal(size=(len(tabs), p64.n_total))
    plan = p64 if prec == lib.PREC_FP64 else lib.Plan(w.cfg, w.src, w.lens, w.base, prec,
                                                      max_batch=len(tabs))
    dv, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    tol = GRAD_REL if prec == lib.PREC_FP64 else 1e-5
    for pt in range(len(tabs)):
        for field, i, j in param_list(w, abi.IA_REDSHIFT_EVOLUTION):
            x0 = nu_get(nus[pt], field, i, j)
            h = H * max(abs(x0), 0.1)
            f = []
            for sgn in (1, -1):
                nu = clone(nus[pt])
                nu_set(nu, field, i, j, x0 + sgn * h)
                f.append(float(v[pt] @ p64.eval_real(om[pt:pt + 1], h0[pt:pt + 1], chi[pt:pt + 1],
                                                     G[pt:pt + 1], lnP[pt:pt + 1], [nu])[0]))
            fd = (f[0] - f[1]) / (2 * h)
            an = nbar[pt, flat_index(field, i, j)]
            assert abs(an - fd) <= tol * abs(fd), (field, i, j, an, fd)
        u = rng.normal(size=lnP.shape[1])
        fd = lnp_direction_fd(p64, tabs, nus, v, pt, u)
        assert abs(lbar[pt] @ u - fd) <= tol * abs(fd), (lbar[pt] @ u, fd)
        # a direction confined to the z = 0 columns (the FFTLog's P_lin slice)
        nk, nz = p64.shapes["nk"], p64.shapes["nz"]
        u0 = np.zeros((nk, nz))
        u0[:, :2] = rng.normal(size=(nk, 2))
        fd = lnp_direction_fd(p64, tabs, nus, v, pt, u0.reshape(-1))
        assert abs(lbar[pt] @ u0.reshape(-1) - fd) <= tol * abs(fd)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_MIXED])
def test_vjp_magnification(gpu_lib, prec):
    """Magnification bias bmag != 0 in every lens bin, non-Limber w(theta):
    d/dbmag through the gs and gg Limber weights W_mag bmag and the FFTLog
    magnification kernel, with every other gradient, against differences of
    the FP64 forward."""
    w, tabs, nus, p64 = setup_case(abi.IA_REDSHIFT_EVOLUTION, name="real_3x2pt_small", seed=35, bmag=True)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(18)
    v = rng.normal(size=(len(tabs), p64.n_total))
    plan = p64 if prec == lib.PREC_FP64 else lib.Plan(w.cfg, w.src, w.lens, w.base, prec,
                                                      max_batch=len(tabs))
    dv, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    tol = GRAD_REL if prec == lib.PREC_FP64 else 1e-5
    for pt in range(len(tabs)):
        for field, i, j in param_list(w, abi.IA_REDSHIFT_EVOLUTION, mag=True):
            x0 = nu_get(nus[pt], field, i, j)
            h = H * max(abs(x0), 0.1)
            f = []
            for sgn in (1, -1):
                nu = clone(nus[pt])
                nu_set(nu, field, i, j, x0 + sgn * h)
                f.append(float(v[pt] @ p64.eval_real(om[pt:pt + 1], h0[pt:pt + 1], chi[pt:pt + 1],
                                                     G[pt:pt + 1], lnP[pt:pt + 1], [nu])[0]))
            fd = (f[0] - f[1]) / (2 * h)
            an = nbar[pt, flat_index(field, i, j)]
            assert abs(an - fd) <= tol * abs(fd), (field, i, j, an, fd)
        u = rng.normal(size=lnP.shape[1])
        fd = lnp_direction_fd(p64, tabs, nus, v, pt, u)
        assert abs(lbar[pt] @ u - fd) <= tol * abs(fd), (lbar[pt] @ u, fd)


@pytest.mark.gpu
def test_vjp_bmag_zero_is_zero(gpu_lib):
    """At bmag = 0 the lens integration range differs from the one of any
    bmag != 0 (redshift_spline.c:50-79): the data vector jumps there and its
    bmag gradient entry is 0."""
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, name="real_3x2pt_small", seed=35, npts=1)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    v = np.random.default_rng(3).normal(size=(1, plan.n_total))
    _, _, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    assert all(nbar[0, flat_index("gb", 4, q)] == 0.0 for q in range(w.cfg.n_lens))


@pytest.mark.gpu
def test_vjp_separate_linear_table(gpu_lib):
    """With a separate linear table the linear-table terms go to lnPL_bar;
    with identical tables lnP_bar + lnPL_bar equals the single-table
    gradient."""
    w, tabs, nus, _ = setup_case(abi.IA_REDSHIFT_EVOLUTION, name="real_3x2pt_small", seed=33)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64, max_batch=len(tabs), linear_table=True)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(14)
    v = rng.normal(size=(len(tabs), plan.n_total))
    _, l1, n1 = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    _, l2, n2, l2l = plan.vjp_real(om, h0, chi, G, lnP, nus, v, lnPL=lnP.copy())
    scale = np.abs(l1).max()
    assert np.max(np.abs(l2 + l2l - l1)) <= 1e-12 * scale
    assert np.max(np.abs(n2 - n1)) <= 1e-12 * np.abs(n1).max()
    assert np.any(l2l != 0) and np.any(l2 != 0)
    lnPL = lnP + 0.01 * rng.normal(size=lnP.shape)
    _, l3, _, l3l = plan.vjp_real(om, h0, chi, G, lnP, nus, v, lnPL=lnPL)
    for pt in range(len(tabs)):
        u = rng.normal(size=lnP.shape[1])
        fd = lnp_direction_fd(plan, tabs, nus, v, pt, u, lnPL=lnPL, which="lnPL")
        assert abs(l3l[pt] @ u - fd) <= GRAD_REL * abs(fd), (l3l[pt] @ u, fd)
        fd = lnp_direction_fd(plan, tabs, nus, v, pt, u, lnPL=lnPL, which="lnP")
        assert abs(l3[pt] @ u - fd) <= GRAD_REL * abs(fd), (l3[pt] @ u, fd)


@pytest.mark.gpu
def test_vjp_nonlimber_vs_oracle_fd(gpu_lib, oracle_built):
    """Non-Limber plan against central differences of the FP64 oracle: b1 of
    every lens bin and a lnP direction (both tables moved together)."""
    import dataclasses
    import oracle as O
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, npts=1, name="real_3x2pt_small", seed=35)
    tabs = workloads.one_table(tabs)  # the plan is given one table
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rng = np.random.default_rng(15)
    v = rng.normal(size=(1, plan.n_total))
    _, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    worst = 0.0
    for q in range(w.cfg.n_lens):
        x0 = nus[0].gb[0][q]
        h = H * max(abs(x0), 0.1)
        f = []
        for s in (1, -1):
            nu = clone(nus[0])
            nu.gb[0][q] = x0 + s * h
            o.set_point(tabs[0], nu)
            f.append(float(v[0] @ o.data_vector_real()))
        fd = (f[0] - f[1]) / (2 * h)
        an = nbar[0, flat_index("gb", 0, q)]
        worst = max(worst, abs(an - fd) / abs(fd))
        assert abs(an - fd) <= ORACLE_REL * abs(fd), (q, an, fd)
    u = rng.normal(size=lnP.shape[1])
    f = []
    for s in (1, -1):
        t = tabs[0]
        lp = np.ascontiguousarray((t.lnP.reshape(-1) + s * H * u).reshape(t.lnP.shape))
        o.set_point(dataclasses.replace(t, lnP=lp, lnPL=lp.copy()), nus[0])
        f.append(float(v[0] @ o.data_vector_real()))
    fd = (f[0] - f[1]) / (2 * H)
    an = float(lbar[0] @ u)
    worst = max(worst, abs(an - fd) / abs(fd))
    print("non-Limber: max rel gradient error vs oracle FD", worst)
    assert abs(an - fd) <= ORACLE_REL * abs(fd), (an, fd)


def tatt_params(w):
    ps = [("shear_m", s, None) for s in range(w.cfg.n_source)]
    ps += [("src_dz", s, None) for s in range(w.cfg.n_source)]
    ps += [("gb", k, q) for k in (0, 1, 2, 4, 5) for q in range(w.cfg.n_lens)]
    ps += [("ia", 0, 0), ("ia", 0, 1), ("ia", 1, 0), ("ia", 1, 1), ("ia", 2, 0)]
    return ps


def fd_step(field, i, x0):
    """Central-difference step: bK (gb[5]) is ~1e-8 in c/H0 units."""
    return H * max(abs(x0), 1e-8 if (field, i) == ("gb", 5) else 0.1)


def set_bk(nus, w, seed):
    """bK ~ U(0, 2e-8) on every point but the first (whose bK stays 0: with
    the one-loop gate on, its bK gradient is still nonzero)."""
    rng = np.random.default_rng(seed)
    for nu in nus[1:]:
        for q in range(w.cfg.n_lens):
            nu.gb[5][q] = float(rng.uniform(0.0, 2e-8))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_MIXED])
def test_vjp_tatt_one_loop(gpu_lib, prec):
    """TATT intrinsic alignments (A1, eta_1, A2, eta_2, b_TA) and one-loop
    bias (b2, bs2, bK) and magnification (bmag) with non-Limber w(theta):
    every nuisance gradient and a direction in each of the nonlinear and
    the separate linear table (the latter through the FAST-PT adjoint as
    well) against differences of the FP64 forward."""
    w = workloads.make("real_3x2pt_tatt_small")
    tabs, nus = workloads.points(w, 2, seed=41, bmag=True)
    set_bk(nus, w, 41)
    p64 = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64, max_batch=2, linear_table=True)
    plan = p64 if prec == lib.PREC_FP64 else lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=2,
                                                      linear_table=True)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    lnPL = np.stack([t.lnPL.reshape(-1) for t in tabs])
    rng = np.random.default_rng(16)
    v = rng.normal(size=(2, plan.n_total))
    dv, lbar, nbar, lplbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v, lnPL=lnPL)
    tol = GRAD_REL if prec == lib.PREC_FP64 else 2e-5
    worst = 0.0
    for pt in range(2):
        sl = slice(pt, pt + 1)
        for field, i, j in tatt_params(w):
            x0 = nu_get(nus[pt], field, i, j)
            h = fd_step(field, i, x0)
            f = []
            for sgn in (1, -1):
                nu = clone(nus[pt])
                nu_set(nu, field, i, j, x0 + sgn * h)
                f.append(float(v[pt] @ p64.eval_real(om[sl], h0[sl], chi[sl], G[sl], lnP[sl], [nu],
                                                     lnPL=lnPL[sl])[0]))
            fd = (f[0] - f[1]) / (2 * h)
            an = nbar[pt, flat_index(field, i, j)]
            err = abs(an - fd) / max(abs(fd), 1e-9 * abs(f[0]))
            worst = max(worst, err)
            assert err <= tol, (field, i, j, an, fd)
        u = rng.normal(size=lnP.shape[1])
        fd = lnp_direction_fd(p64, tabs, nus, v, pt, u, lnPL=lnPL, which="lnP")
        assert abs(lbar[pt] @ u - fd) <= tol * abs(fd), (lbar[pt] @ u, fd)
        # the linear table: FFTLog P_lin slice, Limber_lin hand-over and,
        # through p_lin(k, z = 0), every FAST-PT table.  The TATT delta-E2
        # and mix-B tables are direct FP64 convolutions whose rounding (the
        # reference algorithm's own) puts ~1e-9 relative noise on the data
        # vector, so the difference needs a step of 4e-4 and a smooth
        # direction (a random one also jitters the slopes of the FAST-PT
        # log-extrapolation, which acts through 500 extrapolated points);
        # it is then good to ~1e-5
        nk, nz = tabs[pt].lnP.shape
        us = (np.sin(7 * np.linspace(0, 1, nk)[:, None] + 1.0) * np.cos(3 * np.linspace(0, 1, nz)[None, :]))
        fd = lnp_direction_fd(p64, tabs, nus, v, pt, us.reshape(-1), lnPL=lnPL, which="lnPL", step=4 * H)
        an = float(lplbar[pt] @ us.reshape(-1))
        worst = max(worst, abs(an - fd) / abs(fd))
        assert abs(an - fd) <= max(tol, 5e-5) * abs(fd), (an, fd)
    print("TATT/one-loop max rel gradient error", worst)


@pytest.mark.gpu
@pytest.mark.parametrize("tables", ["one", "two"])
def test_vjp_tatt_one_loop_vs_oracle_fd(gpu_lib, oracle_built, tables):
    """TATT and one-loop bias against central differences of the FP64
    oracle (the reference's algorithm): A1, eta_1, A2, eta_2, b_TA, b2 and
    bs2, shear m and source dz, and lnP directions -- with one table (lnP
    is also the linear spectrum: the Limber walks, the FFTLog slice and the
    FAST-PT tables all move) and with a separate linear table (lnP and lnPL
    differentiated separately)."""
    import dataclasses
    import oracle as O
    w = workloads.make("real_3x2pt_tatt_small")
    tabs, nus = workloads.points(w, 1, seed=57)
    two = tables == "two"
    if not two:
        tabs = workloads.one_table(tabs)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64, max_batch=1, linear_table=two)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    lnPL = np.stack([t.lnPL.reshape(-1) for t in tabs]) if two else None
    rng = np.random.default_rng(58)
    v = rng.normal(size=(1, plan.n_total))
    res = plan.vjp_real(om, h0, chi, G, lnP, nus, v, lnPL=lnPL)
    lbar, nbar = res[1], res[2]
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    worst = 0.0
    params = [("ia", 0, 0), ("ia", 0, 1), ("ia", 1, 0), ("ia", 1, 1), ("ia", 2, 0),
              ("gb", 1, 0), ("gb", 1, 2), ("gb", 2, 1), ("gb", 0, 1), ("shear_m", 1, None), ("src_dz", 2, None)]
    for field, i, j in params:
        x0 = nu_get(nus[0], field, i, j)
        h = H * max(abs(x0), 0.1)
        f = []
        for sg in (1, -1):
            nu = clone(nus[0])
            nu_set(nu, field, i, j, x0 + sg * h)
            o.set_point(tabs[0], nu)
            f.append(float(v[0] @ o.data_vector_real()))
        fd = (f[0] - f[1]) / (2 * h)
        an = nbar[0, flat_index(field, i, j)]
        err = abs(an - fd) / abs(fd)
        print(field, i, j, an, fd, err)
        worst = max(worst, err)
        assert err <= ORACLE_REL, (field, i, j, an, fd)
    # lnP directions: smooth in k so the oracle's rounding stays out of
    # the difference; the step is held where the non-Limber hand-over
    # multipoles do not move (lnp_direction_fd's rule, checked on the GPU)
    nk, nz = tabs[0].lnP.shape
    kk = np.linspace(0.0, 1.0, nk)[:, None]
    zz = np.linspace(0.0, 1.0, nz)[None, :]
    u = (np.sin(7 * kk + 1.0) * np.cos(3 * zz) + 0.3 * rng.normal(size=(nk, nz))).reshape(-1)
    which = ["lnP", "lnPL"] if two else ["lnP"]
    for wh in which:
        hstep = H
        for _ in range(4):
            conv = []
            for sg in (1, -1):
                a = lnP + (sg * hstep * u if wh == "lnP" else 0.0)
                b = None if not two else lnPL + (sg * hstep * u if wh == "lnPL" else 0.0)
                conv.append(plan.cl_nonlimber(om, h0, chi, G, a, nus, lnPL=b)[1])
            if np.array_equal(conv[0], conv[1]):
                break
            hstep /= 4
        f = []
        for sg in (1, -1):
            t = tabs[0]
            lp = t.lnP.reshape(-1) + (sg * hstep * u if wh == "lnP" else 0.0)
            if two:
                ll = t.lnPL.reshape(-1) + (sg * hstep * u if wh == "lnPL" else 0.0)
            else:
                ll = lp
            t2 = dataclasses.replace(t, lnP=np.ascontiguousarray(lp.reshape(t.lnP.shape)),
                                     lnPL=np.ascontiguousarray(ll.reshape(t.lnP.shape)))
            o.set_point(t2, nus[0])
            f.append(float(v[0] @ o.data_vector_real()))
        fd = (f[0] - f[1]) / (2 * hstep)
        an = float((lbar if wh == "lnP" else res[3])[0] @ u)
        err = abs(an - fd) / abs(fd)
        print(wh, an, fd, err)
        worst = max(worst, err)
        assert err <= ORACLE_REL, (wh, an, fd)
    print(f"TATT/one-loop ({tables} table): max rel gradient error vs oracle FD {worst:.2e}")


@pytest.mark.gpu
def test_vjp_b3(gpu_lib, oracle_built):
    """The one-loop b3 terms with the reference's P_d1p3: the b3 and b1
    gradients against differences of the FP64 forward (1e-6) and the b3
    gradient against differences of the oracle (1e-4)."""
    import os
    import oracle as O
    here = os.path.dirname(os.path.abspath(__file__))
    tab = np.load(os.path.join(here, "golden", "fastpt_bias.npz"))["fpt_bias"][5]
    w = workloads.make("real_3x2pt_tatt_small")
    tabs, nus = workloads.points(w, 1, seed=61)
    rng = np.random.default_rng(62)
    for q in range(w.cfg.n_lens):
        nus[0].gb[3][q] = float(rng.uniform(-1.0, 1.0))
    p64 = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64, max_batch=1)
    p64.set_d1p3(tab)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    v = rng.normal(size=(1, p64.n_total))
    _, lbar, nbar = p64.vjp_real(om, h0, chi, G, lnP, nus, v)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    o.set_d1d3_table(tab, np.log(0.05), np.log(1e6))
    worst = 0.0
    for field, i, j in [("gb", 3, q) for q in range(w.cfg.n_lens)] + [("gb", 0, 1), ("gb", 0, 3)]:
        x0 = nu_get(nus[0], field, i, j)
        # the data vector is linear in b3 and quadratic in b1, so a central
        # difference is exact at any step: a large one keeps the forward's
        # rounding out of it
        h = 0.05 * max(abs(x0), 0.5)
        f, fo = [], []
        for sg in (1, -1):
            nu = clone(nus[0])
            nu_set(nu, field, i, j, x0 + sg * h)
            f.append(float(v[0] @ p64.eval_real(om, h0, chi, G, lnP, [nu])[0]))
            if i == 3 and j < 2:
                o.set_point(tabs[0], nu)
                fo.append(float(v[0] @ o.data_vector_real()))
        fd = (f[0] - f[1]) / (2 * h)
        an = nbar[0, flat_index(field, i, j)]
        err = abs(an - fd) / max(abs(fd), 1e-9 * abs(f[0]))
        worst = max(worst, err)
        assert err <= GRAD_REL, (field, i, j, an, fd)
        if fo:
            fdo = (fo[0] - fo[1]) / (2 * h)
            assert abs(an - fdo) <= ORACLE_REL * abs(fdo), (field, i, j, an, fdo)
    o.set_d1d3_table(np.zeros(0), 0.0, 0.0)
    print("b3 max rel gradient error", worst)


@pytest.mark.gpu
def test_jacobian_rows(gpu_lib):
    """cl2pt_jacobian_real: rows of the Jacobian equal the VJP of the one-hot
    cotangent, the value equals the forward, a chunked pass (max_batch
    smaller than the row count) matches, and a table-entry column matches
    a central difference."""
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, npts=3, name="real_3x2pt_small", seed=51)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    rows = np.array([0, 7, plan.n_xi // 2 + 3, plan.n_xi + 5, plan.n_total - 1], dtype=np.int32)
    dv, J, Jn = plan.jacobian_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1], nus[:1], rows=rows)
    assert np.array_equal(dv, plan.eval_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1], nus[:1])[0])
    for k, r in enumerate(rows):
        e = np.zeros((1, plan.n_total))
        e[0, r] = 1.0
        _, lb, nb = plan.vjp_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1], nus[:1], e)
        np.testing.assert_allclose(J[k], lb[0], rtol=1e-12, atol=1e-14 * np.abs(lb).max())
        np.testing.assert_allclose(Jn[k], nb[0], rtol=1e-12, atol=1e-14 * max(np.abs(nb).max(), 1e-300))
    # max_batch 3 < 5 rows: two passes
    _, J2, Jn2 = plan.jacobian_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1], nus[:1], rows=rows)
    np.testing.assert_allclose(J2, J, rtol=1e-12, atol=1e-14 * np.abs(J).max())
    k = int(np.argmax(np.abs(J[1])))
    d = np.zeros(lnP.shape[1])
    d[k] = H
    fp = plan.eval_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1] + d, nus[:1])[0][rows[1]]
    fm = plan.eval_real(om[:1], h0[:1], chi[:1], G[:1], lnP[:1] - d, nus[:1])[0][rows[1]]
    fd = (fp - fm) / (2 * H)
    assert abs(J[1, k] - fd) <= GRAD_REL * abs(fd), (J[1, k], fd)


@pytest.mark.gpu
def test_vjp_unsupported_plan(gpu_lib):
    """Plans with b2/bs2 derived from b1 (bias models 1, 2) report
    CL2PT_ERR_UNSUPPORTED."""
    for name in ("real_3x2pt_tatt_small",):
        w = workloads.make(name)
        w.cfg.bias_model[1] = 1
        tabs, nus = workloads.points(w, 1, seed=1)
        plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64, max_batch=1)
        om, h0, chi, G, lnP = workloads.stack(tabs)
        with pytest.raises(lib.CL2PTError, match="-4"):
            plan.vjp_real(om, h0, chi, G, lnP, nus, np.ones(plan.n_total))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_MIXED])
def test_vjp_lens_photoz_vs_oracle_fd(gpu_lib, oracle_built, prec):
    """Lens photo-z shift and stretch gradients (cl2pt_plan_set_lens_photoz_grad:
    central differences of the plan's forward inside the adjoint) against
    central differences of the FP64 oracle with the same steps, on the
    non-Limber geometry (the FFTLog n(z) samples move as well as the
    Limber nodes); off, those entries stay 0."""
    import oracle as O
    w, tabs, nus, plan = setup_case(abi.IA_REDSHIFT_EVOLUTION, npts=2, name="real_3x2pt_small", seed=37, prec=prec)
    tabs = workloads.one_table(tabs)
    rng = np.random.default_rng(17)
    for q in range(w.cfg.n_lens):
        nus[1].lens_stretch[q] = float(rng.uniform(0.9, 1.1))
    om, h0, chi, G, lnP = workloads.stack(tabs)
    v = rng.normal(size=(2, plan.n_total))
    _, _, nb0 = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    assert np.all(nb0[:, [flat_index(f, q) for f in ("lens_dz", "lens_stretch") for q in range(w.cfg.n_lens)]] == 0)
    plan.set_lens_photoz_grad(True)
    _, lbar, nbar = plan.vjp_real(om, h0, chi, G, lnP, nus, v)
    h = 1e-4 if prec == lib.PREC_FP64 else 2e-3
    tol = ORACLE_REL if prec == lib.PREC_FP64 else 5e-3
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    worst = 0.0
    for pt in range(2):
        for field in ("lens_dz", "lens_stretch"):
            for q in range(w.cfg.n_lens):
                x0 = getattr(nus[pt], field)[q]
                f = []
                for s in (1, -1):
                    nu = clone(nus[pt])
                    getattr(nu, field)[q] = x0 + s * h
                    o.set_point(tabs[pt], nu)
                    f.append(float(v[pt] @ o.data_vector_real()))
                fd = (f[0] - f[1]) / (2 * h)
                an = nbar[pt, flat_index(field, q)]
                err = abs(an - fd) / abs(fd)
                worst = max(worst, err)
                assert err <= tol, (pt, field, q, an, fd, err)
    # the other gradients are those of the plain adjoint (up to the order of
    # its atomic sums)
    l2 = plan.vjp_real(om, h0, chi, G, lnP, nus, v)[1]
    np.testing.assert_allclose(lbar, l2, rtol=1e-9 if prec == lib.PREC_FP64 else 1e-6, atol=1e-12 * np.abs(l2).max())
    print(prec, "lens photo-z gradient max rel err vs oracle FD", worst)
