"""cl2pt_J_abl_noalloc -- J_abl with its workspace in a static device array
-- against the allocating entry point cl2pt_J_abl, through the C ABI.

Two calls in a row on different spectra (and a third with another term
list), so contents the shared array keeps from the previous call cannot
leak into the next result; the first result is also checked against the
CPU oracle (the reference's J_abl restated in C).  Tolerance: the FAST-PT
bar (1e-6 relative per entry, entries below 1e-4 of a spectrum's peak held
to that floor).
"""
import ctypes as C

import numpy as np
import pytest

from cl2pt import lib, workloads

REL = 1e-6
FLOOR = 1e-4


def rel_rows(got, ref):
    g = np.asarray(got, dtype=np.float64).reshape(-1, np.shape(ref)[-1])
    r = np.asarray(ref, dtype=np.float64).reshape(-1, np.shape(ref)[-1])
    peak = np.max(np.abs(r), axis=1, keepdims=True)
    return float(np.max(np.abs(g - r) / np.maximum(np.abs(r), FLOOR * peak + 1e-300)))


def noalloc(x, fx_dev, alpha, beta, ell, out_dev, cfg, stream):
    f = lib.load().cl2pt_J_abl_noalloc
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    f.argtypes = [dp, C.c_void_p, C.c_long, ip, ip, ip, C.c_int, C.POINTER(lib.FastPTConfig),
                  C.c_void_p, C.c_void_p]
    x = np.ascontiguousarray(x, dtype=np.float64)
    a, b, l = (np.ascontiguousarray(v, dtype=np.int32) for v in (alpha, beta, ell))
    return f(x.ctypes.data_as(dp), fx_dev, len(x), a.ctypes.data_as(ip), b.ctypes.data_as(ip),
             l.ctypes.data_as(ip), len(a), C.byref(cfg), out_dev, stream)


@pytest.mark.gpu
def test_J_abl_noalloc_matches_J_abl(gpu_lib, oracle_built):
    import torch
    import oracle as O
    k, P, _ = workloads.fastpt_spectra(3, seed=21)
    a, b, l, _, _ = lib.bias_terms()
    cfg = lib.fastpt_config()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(P[0], a, b, l), (P[1], a, b, l), (P[2], [0, 1, 2], [0, -1, 0], [2, 1, 0])]
    for i, (fx, aa, bb, ll) in enumerate(cases):
        ref = lib.J_abl(k, fx, aa, bb, ll, cfg)  # the allocating entry point
        fx_d = torch.tensor(fx, device="cuda")
        out = torch.full((len(aa), len(k)), float("nan"), dtype=torch.float64, device="cuda")
        st = noalloc(k, fx_d.data_ptr(), aa, bb, ll, out.data_ptr(), cfg, stream)
        assert st == 0, st
        err = rel_rows(out.cpu().numpy(), ref)
        print("noalloc vs J_abl", err)
        assert err <= REL, err
        if i == 0:
            orc = O.Oracle("orc").J_abl(k, fx, aa, bb, ll)
            err_o = rel_rows(out.cpu().numpy(), orc)
            print("noalloc vs oracle", err_o)
            assert err_o <= REL, err_o


@pytest.mark.gpu
def test_J_abl_noalloc_rejects_oversize(gpu_lib):
    import torch
    k, P, _ = workloads.fastpt_spectra(1, seed=22)
    cfg = lib.fastpt_config()
    fx_d = torch.tensor(P[0], device="cuda")
    out = torch.zeros((17, len(k)), dtype=torch.float64, device="cuda")
    z = np.zeros(17, dtype=np.int32)
    assert noalloc(k, fx_d.data_ptr(), z, z, z, out.data_ptr(), cfg, None) == -1  # > 16 terms
    # padded size N = N0 + 2 N_pad + N_extrap_low + N_extrap_high must stay
    # within FPT_NOALLOC_MAX_N = 7231 (Ntot >= 2N + 1 <= 14464 points)
    big = lib.fastpt_config(npad=2093)  # N = 2048 + 4186 + 1000 = 7234 > 7231
    assert noalloc(k, fx_d.data_ptr(), z[:1], z[:1], z[:1], out.data_ptr(), big, None) == -1


@pytest.mark.gpu
def test_J_abl_noalloc_at_the_limit(gpu_lib):
    """npad = 2076 gives N = 7200 (7-smooth), Ntot = 14406: just inside the
    static array's bound, so it is accepted and matches cl2pt_J_abl."""
    import torch
    k, P, _ = workloads.fastpt_spectra(1, seed=23)
    a, b, l, _, _ = lib.bias_terms()
    cfg = lib.fastpt_config(npad=2076)
    ref = lib.J_abl(k, P[0], a, b, l, cfg)
    fx_d = torch.tensor(P[0], device="cuda")
    out = torch.full((len(a), len(k)), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert noalloc(k, fx_d.data_ptr(), a, b, l, out.data_ptr(), cfg, stream) == 0
    err = rel_rows(out.cpu().numpy(), ref)
    print("noalloc at the limit vs J_abl", err)
    assert err <= REL, err
