"""CPU checks of the oracle's scale-cut diagnostics: RF grows with kmax from
0 (below the k range the sources see at that l) towards 1, and dC/dlnk
vanishes outside the sources' redshift range."""
import numpy as np
import pytest

from cl2pt import workloads


def test_rf_monotone_and_range(oracle_built):
    import oracle as O
    w = workloads.make("real_3x2pt_small_nla")
    tabs, nus = workloads.points(w, 1, seed=6)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    o.set_point(tabs[0], nus[0])
    # (the two integrals use different maps of ln k onto the same rule, so
    # RF is a fraction only up to that quadrature: kmax far above the
    # sources' k range reads above 1, as in the reference)
    r = [o.RF_C_ss(km, 300.0, 0, 1) for km in (1e-3, 0.05, 0.5, 5.0)]
    assert r[0] == 0.0 and r[-1] > 0.9
    assert np.all(np.diff(r) >= 0) and r[2] > 0
    # chi(a) = (l + 1/2)/k beyond the farthest source (tiny k) or nearer
    # than the nearest (huge k): no contribution
    assert o.dC_ss_dlnk(1e-7, 300.0, 0, 1) == 0.0 and o.dC_ss_dlnk(1e7, 300.0, 0, 1) == 0.0
    assert o.dC_ss_dlnk(0.3, 300.0, 0, 1) != 0.0
