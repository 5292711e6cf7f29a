"""FAST-PT term tables of the library (host code, no GPU): the TATT J_table
expansion and the bias decomposition equal the oracle's."""
import numpy as np


def test_ia_jrows_match_oracle(oracle_built):
    from cl2pt import build, lib
    import oracle as O
    build.build()
    a, b, j1, j2, jk, slot, c = lib.ia_terms()
    rows, coeff, start, trow = O.Oracle("orc").ia_jrows()
    assert len(a) == len(rows) == 184
    assert np.array_equal(np.stack([a, b, j1, j2, jk], axis=1), rows)
    gslot = np.concatenate([np.full(start[g + 1] - start[g], trow[g]) for g in range(8)])
    assert np.array_equal(slot, gslot)
    assert np.allclose(c, coeff, rtol=1e-13, atol=0)


def test_bias_terms():
    from cl2pt import build, lib
    build.build()
    a, b, l, o, c = lib.bias_terms()
    assert len(a) == 13 and set(o) == {0, 1, 2, 3, 4}
    assert np.all(a + b == 0)
