"""GPU adjoint of the FAST-PT convolutions (cl2pt_fastpt_*_vjp) against
central finite differences of the FP64 oracle (the reference's J_abl /
J_abJ1J2Jk / get_FPT_IA algorithm restated in C).

For a cotangent obar of the outputs, <fx_bar, d> must equal the directional
derivative (<obar, out(fx + e d)> - <obar, out(fx - e d)>) / 2e of the
oracle.  The outputs are quadratic in the padded spectrum, so central
differences are exact but for rounding and the log-extrapolation, and a
large step (1e-3 relative) keeps the oracle's own rounding out of the
difference.  The cotangents are scaled by 1 / max(|out|, 1e-3 of the row's
peak) so that most k carry weight without the far tails' rounding
dominating.  Directions: random relative noise on the interior points, a
smooth bump, and a smooth tilt that also moves the first and last two
points (which steer the extrapolation; random noise there would change its
slope by O(1) over the 500 extrapolated points).  Tolerance: 1e-5 relative.
"""
import numpy as np
import pytest

from cl2pt import lib, workloads

REL = 1e-5
STEP = 1e-3


def directions(P, rng):
    n = len(P)
    x = np.linspace(0.0, 1.0, n)
    noise = rng.normal(size=n)
    noise[:2] = noise[-2:] = 0.0
    return [P * noise,
            P * np.exp(-0.5 * ((x - 0.3) / 0.05) ** 2),
            P * (1.0 + x)]  # moves the end points too


def fd_check(forward, P, obar, grad, rng, tag):
    worst = 0.0
    for d in directions(P, rng):
        fp = forward(P + STEP * d)
        fm = forward(P - STEP * d)
        fd = float(np.sum(obar * (fp - fm))) / (2 * STEP)
        an = float(np.dot(grad, d))
        err = abs(fd - an) / max(abs(fd), 1e-300)
        print(f"{tag}: FD {fd:.10e} adjoint {an:.10e} rel {err:.2e}")
        assert np.isfinite(fd) and np.isfinite(an), (fd, an)
        worst = max(worst, err)
    return worst


def plan_grid_spectrum():
    """The k grid of the 3x2pt plans' FAST-PT tables (the reference's:
    1100 points over 0.05..1e6 in units of H0/c, i.e. k c/H0 with k in
    h/Mpc) and the Eisenstein-Hu linear spectrum there in the same units.
    (A spectrum without the k^-3 fall-off makes the biased FFTLog inputs
    of the alpha != beta terms grow at high k, where neither this code nor
    the reference is well conditioned.)"""
    from cl2pt import synthetic
    ch = 2997.92458
    k = np.exp(np.log(0.05) + np.arange(1100) * (np.log(1e6) - np.log(0.05)) / 1100)
    return k, (synthetic.plin_z0(k / ch, synthetic.Cosmo()) / ch ** 3)[None, :]


def cotangent(out, rng):
    peak = np.abs(out).max(axis=-1, keepdims=True)
    return rng.normal(size=out.shape) / np.maximum(np.abs(out), 1e-3 * peak + 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("grid", ["plan", "batched"])
def test_bias_vjp_vs_oracle_fd(gpu_lib, oracle_built, grid):
    """get_FPT_bias's five spectra: on the k grid the TATT / one-loop plans
    use (1100 points in 0.05..1e6 in units of c/H0 as the reference) and on
    the batched workload's grid (2048 points in 1e-5..1e3 h/Mpc)."""
    import oracle as O
    o = O.Oracle("orc")
    rng = np.random.default_rng(5)
    if grid == "plan":
        k, P = plan_grid_spectrum()
    else:
        k, P, _ = workloads.fastpt_spectra(2, seed=7)
    plan = lib.FastPT.for_bias(k, max_spec=len(P))
    a, b, l, oi, c = lib.bias_terms()

    def forward(f):
        J = o.J_abl(k, f, a, b, l)
        res = np.zeros((5, len(k)))
        for t in range(13):
            res[oi[t]] += c[t] * J[t]
        return res

    out = plan.bias(P)
    obar = cotangent(out, rng)
    g = plan.bias_vjp(P, obar)
    worst = 0.0
    for s in range(len(P)):
        worst = max(worst, fd_check(forward, P[s], obar[s], g[s], rng, f"bias {grid} {s}"))
    assert worst <= REL, worst


@pytest.mark.gpu
def test_J_abl_vjp_per_term(gpu_lib, oracle_built):
    """The drop-in J_abl plan's per-term outputs (a term list outside the
    bias decomposition: mixed alpha, beta and ell)."""
    import oracle as O
    o = O.Oracle("orc")
    rng = np.random.default_rng(6)
    k, P, _ = workloads.fastpt_spectra(1, seed=8)
    a, b, l = [0, 1, 0, 1], [0, -1, 0, -1], [0, 1, 3, 3]
    plan = lib.FastPT(k, a, b, l, max_spec=1)
    out = plan.J_abl(P)
    obar = cotangent(out, rng)
    g = plan.J_vjp(P, obar)
    worst = fd_check(lambda f: o.J_abl(k, f, a, b, l), P[0], obar[0], g[0], rng, "J_abl")
    assert worst <= REL, worst


@pytest.mark.gpu
def test_ia_vjp_vs_oracle_fd(gpu_lib, oracle_built):
    """get_FPT_IA's ten rows (184 J_abJ1J2Jk terms and the two direct
    convolutions) on the plans' k grid."""
    import oracle as O
    o = O.Oracle("orc")
    rng = np.random.default_rng(9)
    k, P = plan_grid_spectrum()
    plan = lib.FastPT.for_ia(k, max_spec=1)
    out = plan.ia(P)
    obar = cotangent(out, rng)
    # rows 3 and 7 (delta-E2, mix-B) are direct FP64 convolutions whose
    # high-k values carry rounding of ~1e-6 relative and more in the oracle
    # itself, which the differences would amplify: their cotangent is kept
    # below k index 600
    obar[:, 3, 600:] = 0.0
    obar[:, 7, 600:] = 0.0
    g = plan.ia_vjp(P, obar)
    worst = fd_check(lambda f: o.fpt_ia_spectrum(k, f)[:10], P[0], obar[0], g[0], rng, "ia")
    assert worst <= REL, worst
