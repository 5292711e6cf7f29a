"""Batched serving path: ragged (per-point scale cut) Fourier vectors and
the CUDA-graph replay.

* cl2pt_eval_fourier_ragged returns exactly the kept entries of the full
  vectors of cl2pt_eval_fourier (same kernels, then a gather);
* a captured graph replays bit-identically to the eager call, and picks up
  new inputs written into the same device buffers;
* the full-size serving layout (10 + 10 bins, 26 l bins, FFTLog on 2048
  log-chi points below l = 200) against the FP64 oracle at 1e-4.
"""
import numpy as np
import pytest

from cl2pt import lib, workloads
from test_gpu_real import PAIR_FLOOR, REL, rel_err_env


def device_batch(data, dev):
    import torch
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    om, h0, chi, G, lnP = (T(a) for a in data[:5])
    nub = np.frombuffer(b"".join(bytes(n) for n in data[5]), dtype=np.uint8).copy()
    return om, h0, chi, G, lnP, T(nub)


@pytest.mark.gpu
def test_ragged_matches_full(gpu_lib):
    w = workloads.make("fourier_serving_small")
    tabs, nus = workloads.points(w, 5, seed=2)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=5)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    full = plan.eval_fourier(om, h0, chi, G, lnP, nus, w.ell)
    ptr, idx = workloads.scale_cuts(w, 5, seed=1)
    rag = plan.eval_fourier_ragged(om, h0, chi, G, lnP, nus, w.ell, ptr, idx)
    ref = np.concatenate([full[i][idx[ptr[i]:ptr[i + 1]]] for i in range(5)])
    assert np.array_equal(rag, ref)
    sizes = np.diff(ptr)
    assert sizes.min() < sizes.max()  # ragged
    bad = idx.copy()
    bad[3] = full.shape[1]
    with pytest.raises(lib.CL2PTError):
        plan.eval_fourier_ragged(om, h0, chi, G, lnP, nus, w.ell, ptr, bad)


@pytest.mark.gpu
def test_graph_replay(gpu_lib):
    import torch
    dev = torch.device("cuda:0")
    w = workloads.make("fourier_serving_small")
    n = 6
    tabs, nus = workloads.points(w, n, seed=4)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=n)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    d = device_batch((om, h0, chi, G, lnP, nus), dev)
    ptr, idx = workloads.scale_cuts(w, n, seed=2)
    dptr, didx = torch.from_numpy(ptr).to(dev), torch.from_numpy(idx).to(dev)
    out = torch.zeros(int(ptr[-1]), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        g = plan.fourier_graph(*d, w.ell, out, row_ptr=dptr, idx=didx, stream=stream.cuda_stream)
        out.zero_()
        g.launch(stream.cuda_stream)
    stream.synchronize()
    assert g.launches() > 0
    ref = plan.eval_fourier_ragged(om, h0, chi, G, lnP, nus, w.ell, ptr, idx)
    assert np.array_equal(out.cpu().numpy(), ref)
    # new walkers written into the same buffers
    tabs2, nus2 = workloads.points(w, n, seed=9)
    om2, h02, chi2, G2, lnP2 = workloads.stack(tabs2)
    d2 = device_batch((om2, h02, chi2, G2, lnP2, nus2), dev)
    with torch.cuda.stream(stream):
        for a, b in zip(d, d2):
            a.copy_(b)
        g.launch(stream.cuda_stream)
    stream.synchronize()
    ref2 = plan.eval_fourier_ragged(om2, h02, chi2, G2, lnP2, nus2, w.ell, ptr, idx)
    assert np.array_equal(out.cpu().numpy(), ref2)
    assert not np.array_equal(ref, ref2)
    g.close()


@pytest.mark.gpu
def test_serving_layout_vs_oracle(gpu_lib, oracle_built):
    """The full serving layout at two points against the FP64 oracle."""
    import oracle as O
    w = workloads.make("fourier_serving")
    tabs, nus = workloads.points(w, 2, seed=6)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=2)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    dv = plan.eval_fourier(om, h0, chi, G, lnP, nus, w.ell)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    nell = len(w.ell)
    worst = 0.0
    for i in range(2):
        o.set_point(tabs[i], nus[i])
        ref = o.data_vector_fourier(w.ell)
        worst = max(worst, rel_err_env(dv[i], ref, None, floor=PAIR_FLOOR, ntheta=nell))
    print("serving layout max rel err", worst)
    assert worst <= REL
