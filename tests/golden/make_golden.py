"""Generate the golden fixtures from the reference's own code.

Runs each case in its own process against oracle/_ref/libcosmolike_ref.so
(the reference's hot-path sources compiled unchanged against this
project's GSL/FFTW stand-ins; built by `make -C oracle ref`, which needs
the reference source tree) on the seeded synthetic inputs of
cl2pt.workloads, and writes tests/golden/<case>.npz.

    python tests/golden/make_golden.py [case ...]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cocoa-cosmolike-core_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CASES = ["cosmic_shear_fourier", "real_3x2pt_small", "real_3x2pt_small_limber", "real_3x2pt",
         "fastpt_bias", "fastpt_ia", "real_3x2pt_tatt_small", "real_3x2pt_small_mag",
         "real_3x2pt_small_nla", "real_3x2pt_small_nlabin", "real_3x2pt_small_hdi",
         "real_3x2pt_small_lin", "cmb_lensing_small", "cmb_lensing_tatt_small", "scale_cuts_small",
         "scale_cuts_tatt_small"]

# J_abJ1J2Jk rows {alpha, beta, J1, J2, Jk} checked on the batched FAST-PT grid
JK_ROWS = [[0, 0, 0, 0, 0], [1, -1, 2, 1, 1], [-1, 1, 1, 3, 2], [0, 0, 4, 2, 2]]


def run_case(case, which="ref"):
    """Outputs of one case from the 'ref' or 'orc' library (dict of arrays)."""
    import oracle as O
    from cl2pt import abi, workloads
    o = O.Oracle(which)
    out = {}
    if case == "fastpt_bias":
        w = workloads.make("real_3x2pt_small")
        o.setup(w.cfg, w.src, w.lens)
        o.set_point(w.base, abi.make_nuisance())
        out["fpt_bias"] = o.fpt_bias()
        return out
    if case == "fastpt_ia":
        w = workloads.make("real_3x2pt_small")
        o.setup(w.cfg, w.src, w.lens)
        o.set_point(w.base, abi.make_nuisance())
        out["fpt_ia"] = o.fpt_ia()
        k, P, _ = workloads.fastpt_spectra(1, seed=1)
        r = np.array(JK_ROWS)
        out["J_abJ1J2Jk"] = o.J_abJ1J2Jk(k, P[0], r[:, 0], r[:, 1], r[:, 2], r[:, 3], r[:, 4])
        return out
    if case in ("scale_cuts_small", "scale_cuts_tatt_small"):
        # cosmo2D_scuts.c on real_3x2pt_small_nla's points: dC_ss/dlnk on a
        # (k, l) grid, RF_C_ss at l > lmin_tab (from its dlnC table), and the
        # real-space dlnxi/dlnk table and RF_xi.  (The reference's RF_C_ss
        # exits at l <= lmin_tab: its quadrature nodes near t = 1e-5
        # underflow k to 0, which dC_ss_dlnk rejects.)
        # (the _tatt case: real_3x2pt_tatt_small's points, B modes as well)
        tatt = "tatt" in case
        w = workloads.make("real_3x2pt_tatt_small" if tatt else "real_3x2pt_small_nla")
        o.setup(w.cfg, w.src, w.lens)
        tabs, nus = workloads.points(w, 2, seed=41)
        sc = workloads.scale_cut_requests()
        for i in range(2):
            o.set_point(tabs[i], nus[i])
            for e, tag in ((1, ""), (0, "B")) if tatt else ((1, ""),):
                out[f"dC{tag}_{i}"] = np.array([[[o.dC_ss_dlnk(k, l, a, b, e) for l in sc["l"]] for k in sc["k"]]
                                                for a, b in sc["pairs"]])
            o.set_dlnk_grid(sc["nlnk"], sc["kmin"], sc["kmax"])
            for e, tag in ((1, ""), (0, "B")) if tatt else ((1, ""),):
                out[f"rf{tag}_{i}"] = np.array([[o.RF_C_ss(km, l, a, b, e)
                                                 for km, l in zip(sc["rf_kmax"], sc["rf_l"])]
                                                for a, b in sc["pairs"]])
            out[f"dlnxi_{i}"] = o.dlnxi_table(sc["nlnk"], sc["kmin"], sc["kmax"])
            out[f"xi_{i}"] = np.stack(o.xi_pm())  # [2][pss][ntheta], the divisors
            out[f"rfxi_{i}"] = np.array([[[[o.RF_xi(km, p, t, q) for km in sc["xi_kmax"]]
                                           for t in range(w.cfg.ntheta)] for q in range(o.npairs[0])]
                                         for p in range(2)])
        return out
    if case.startswith("cmb_lensing"):
        w = workloads.make(case)
        o.setup(w.cfg, w.src, w.lens)
        f = workloads.cmb_map_filter()
        o.set_cmb(f["lmin"], f["lmax"], f["fwhm_arcmin"], f["healpixwin"])
        tabs, nus = workloads.points(w, 2, seed=11)
        for i in range(2):
            o.set_point(tabs[i], nus[i])
            out[f"wgk_{i}"] = o.w_cmb("gk")
            out[f"wks_{i}"] = o.w_cmb("ks")
            kl = np.concatenate([w.ell, [float(w.cfg.lmin_tab), w.cfg.lmin_tab + 0.5, 7000.0]])
            out[f"Ckk_dv_{i}"] = o.C_kk_dv(kl)
            out[f"kk_bp_{i}"] = o.kk_bandpower(*workloads.cmb_kk_bandpowers())
            out[f"Cgk_{i}"] = np.array([[o.C_cmb("gk", l, n) for l in w.ell] for n in range(w.cfg.n_lens)])
            out[f"Cks_{i}"] = np.array([[o.C_cmb("ks", l, n) for l in w.ell] for n in range(w.cfg.n_source)])
            out[f"Ckk_{i}"] = np.array([o.C_cmb("kk", l) for l in w.ell])
        return out
    # <workload>_mag: the workload's points with magnification bias
    mag = case.endswith("_mag")
    w = workloads.make(case[:-4] if mag else case)
    o.setup(w.cfg, w.src, w.lens)
    tabs, nus = workloads.points(w, 2, seed=11, bmag=mag)
    for i in range(2):
        o.set_point(tabs[i], nus[i])
        if case == "cosmic_shear_fourier":
            pairs = abi.shear_pairs(w.cfg.n_source)
            out[f"Css_EE_{i}"] = np.array([[o.C_ss_nointerp(l, a, b, 1) for l in w.ell] for a, b in pairs])
            out[f"Css_EE_tab_{i}"] = np.array([[o.C_ss_limber(l, a, b, 1) for l in w.ell] for a, b in pairs])
        else:
            out[f"dv_{i}"] = o.data_vector_real()
            if not w.cfg.adopt_limber_gg:
                out[f"cl_nonlimber_{i}"] = o.C_cl_tomo()[0]
            if case == "real_3x2pt_small" and i == 0:
                out["Cgs_l"] = np.array([o.C_gs_nointerp(l, 1, 2) for l in (3.0, 30.0, 300.0)])
                out["Cgg_l"] = np.array([o.C_gg_nointerp(l, 1, 0) for l in (3.0, 30.0, 300.0)])
                out["Cgg_lin_l"] = np.array([o.C_gg_nointerp(l, 1, 1) for l in (3.0, 30.0, 300.0)])
        if case == "real_3x2pt":
            break
    return out


def main(cases):
    for c in cases:
        if os.environ.get("CL2PT_GOLDEN_CHILD") == c:
            np.savez_compressed(os.path.join(HERE, f"{c}.npz"), **run_case(c))
            return
    for c in cases:
        env = dict(os.environ, CL2PT_GOLDEN_CHILD=c)
        subprocess.run([sys.executable, __file__, c], check=True, env=env)
        print("wrote", c)


if __name__ == "__main__":
    main(sys.argv[1:] or CASES)
