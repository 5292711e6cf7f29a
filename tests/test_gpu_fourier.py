"""GPU parity of the Fourier-space 3x2pt path (cl2pt_eval_fourier).

Cosmic shear at 20 log-spaced l in 20-3000 against the reference's own
C_ss_tomo_limber_nointerp (tests/golden/cosmic_shear_fourier.npz), and the
full Fourier 3x2pt with the non-Limber C_gg below LMAX_NOLIMBER against the
oracle.  Tolerance: 1e-4 relative per entry, entries below 1e-4 of their
spectrum's peak held to that floor; TATT runs use the measured envelope of
tests/test_gpu_real.py.
"""
import os

import numpy as np
import pytest

from cl2pt import abi, lib, workloads
from test_gpu_real import DIRECT_ALT, PAIR_FLOOR, REL, rel_err_env

HERE = os.path.dirname(os.path.abspath(__file__))


def fourier_ells(n, lmin, lmax):
    # init_binning_fourier's bin centres (generic_interface.cpp:448-456)
    logdl = (np.log(lmax) - np.log(lmin)) / n
    return np.exp(np.log(lmin) + (np.arange(n) + 0.5) * logdl)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_cosmic_shear_fourier_vs_reference(gpu_lib, prec):
    gold = np.load(os.path.join(HERE, "golden", "cosmic_shear_fourier.npz"))
    w = workloads.make("cosmic_shear_fourier")
    tabs, nus = workloads.points(w, 2, seed=11)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=2)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    dv = plan.eval_fourier(om, h0, chi, G, lnP, nus, w.ell)
    pairs = abi.shear_pairs(w.cfg.n_source)
    nell = len(w.ell)
    for i in range(2):
        m = np.array([(1 + nus[i].shear_m[a]) * (1 + nus[i].shear_m[b]) for a, b in pairs])
        ref = gold[f"Css_EE_{i}"] * m[:, None]
        got = dv[i][: len(pairs) * nell].reshape(len(pairs), nell)  # the shear block
        assert np.all(dv[i][len(pairs) * nell:] == 0.0)  # probes: shear only
        err = rel_err_env(got, ref, None, floor=PAIR_FLOOR, ntheta=nell)
        print(prec, i, err)
        assert err <= REL, (i, err)


def fourier_case(name, npts, prec, ell, seed=3, bmag=False):
    import oracle as O
    w = workloads.make(name)
    tabs, nus = workloads.points(w, npts, seed=seed, bmag=bmag)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, prec, max_batch=npts, linear_table=True)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    lmax_shear = 0.7 * np.max(ell)
    dv = plan.eval_fourier(om, h0, chi, G, lnP, nus, ell, lmax_shear=lmax_shear,
                           lnPL=workloads.stack_lin(tabs))
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    tatt = w.cfg.ia_model == abi.IA_TATT
    worst = 0.0
    nell = len(ell)
    for i in range(npts):
        alt = None
        if tatt:
            alt = []
            for n_alt in DIRECT_ALT:
                o.set_direct_conv_size(n_alt)
                o.set_point(tabs[i], nus[i])
                alt.append(o.data_vector_fourier(ell, lmax_shear=lmax_shear))
            o.set_direct_conv_size(0)
        o.set_point(tabs[i], nus[i])
        ref = o.data_vector_fourier(ell, lmax_shear=lmax_shear)
        worst = max(worst, rel_err_env(dv[i], ref, alt, floor=PAIR_FLOOR, ntheta=nell))
    return worst, dv


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_fourier_3x2pt_nonlimber(gpu_lib, oracle_built, prec):
    """26 log-spaced l in 20-5000 (10 of them below LMAX_NOLIMBER = 150:
    clustering from the FFTLog C_l), shear cut at 0.7 l_max."""
    ell = fourier_ells(26, 20.0, 5000.0)
    worst, _ = fourier_case("real_3x2pt_small", 2, prec, ell)
    print(prec, worst)
    assert worst <= REL, worst


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_fourier_magnification(gpu_lib, oracle_built, prec):
    """Magnification bias bmag ~ U(-1, 3) per lens bin: the W_mag terms of
    C_gs and C_gg (Limber), the FFTLog magnification kernel below
    LMAX_NOLIMBER, and the lens integration ranges that open to the
    sources' z_min when bmag != 0 (redshift_spline.c:50-79)."""
    ell = fourier_ells(26, 20.0, 5000.0)
    worst, _ = fourier_case("real_3x2pt_small", 2, prec, ell, bmag=True)
    print(prec, worst)
    assert worst <= REL, worst


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_fourier_nla_stretch_bias_model(gpu_lib, oracle_built, prec):
    """NLA (redshift evolution), lens stretch and bias model 1 on the
    Fourier vector."""
    ell = fourier_ells(26, 20.0, 5000.0)
    worst, _ = fourier_case("real_3x2pt_small_nla", 2, prec, ell)
    print(prec, worst)
    assert worst <= REL, worst


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
@pytest.mark.parametrize("name", ["real_3x2pt_small_hdi", "real_3x2pt_small_lin", "real_3x2pt_small_nlabin"])
def test_fourier_config_variants(gpu_lib, oracle_built, prec, name):
    """high_def_integration = 1 with ggl exclusions, the linear run mode, and
    NLA per-bin amplitudes with bias model 2, on the Fourier vector."""
    ell = fourier_ells(26, 20.0, 5000.0)
    worst, _ = fourier_case(name, 2, prec, ell)
    print(prec, name, worst)
    assert worst <= REL, worst


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [lib.PREC_MIXED, lib.PREC_FP64])
def test_fourier_unsorted_ells(gpu_lib, oracle_built, prec):
    """Caller multipoles in any order, down to l = 3 where the chi(a_min)
    cut of C_gg removes nodes (the mixed plan's cut falls back from a
    first-kept index to its threshold form): the shuffled list against the
    oracle, and entry for entry against the ascending list."""
    ell = fourier_ells(26, 3.0, 5000.0)
    perm = np.random.default_rng(5).permutation(len(ell))
    worst, dv = fourier_case("real_3x2pt_small", 2, prec, ell[perm])
    print(prec, worst)
    assert worst <= REL, worst
    _, dv_sorted = fourier_case("real_3x2pt_small", 2, prec, ell)
    nell = len(ell)
    a = dv.reshape(2, -1, nell)
    b = dv_sorted.reshape(2, -1, nell)[:, :, perm]
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14 * np.abs(b).max())


@pytest.mark.gpu
def test_fourier_tatt_one_loop(gpu_lib, oracle_built):
    ell = fourier_ells(20, 20.0, 4000.0)
    worst, _ = fourier_case("real_3x2pt_tatt_small", 2, lib.PREC_MIXED, ell, seed=11)
    print(worst)
    assert worst <= REL, worst


@pytest.mark.gpu
def test_fourier_mask(gpu_lib):
    w = workloads.make("real_3x2pt_small")
    tabs, nus = workloads.points(w, 1, seed=5)
    ell = fourier_ells(12, 30.0, 3000.0)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=1)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    full = plan.eval_fourier(om, h0, chi, G, lnP, nus, ell)[0]
    mask = (np.random.default_rng(1).uniform(size=full.size) < 0.5).astype(np.int32)
    masked = plan.eval_fourier(om, h0, chi, G, lnP, nus, ell, mask=mask)[0]
    assert np.all(masked[mask == 0] == 0.0)
    assert np.array_equal(masked[mask == 1], full[mask == 1])
