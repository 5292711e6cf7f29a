"""The real-space evaluation captured as a CUDA graph, and the plan's
autotuner.

* cl2pt_real_graph_create: a replay equals the eager cl2pt_eval_real on the
  same device buffers bit for bit (the same kernels in the same order), and
  picks up new points written into those buffers;
* cl2pt_plan_autotune: returns one of its candidates, leaves the plan in
  that configuration, and the tuned plan's data vectors stay within the
  1e-4 bar of the FP64 oracle.
"""
import numpy as np
import pytest

from cl2pt import lib, workloads
from test_gpu_serving import device_batch


@pytest.mark.gpu
def test_real_graph_replay(gpu_lib):
    import torch
    dev = torch.device("cuda:0")
    w = workloads.make("real_3x2pt_small")
    n = 5
    tabs, nus = workloads.points(w, n, seed=21)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=n)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    d = device_batch((om, h0, chi, G, lnP, nus), dev)
    out = torch.zeros((n, plan.n_total), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        g = plan.real_graph(*d, out, stream=stream.cuda_stream)
        out.zero_()
        g.launch(stream.cuda_stream)
    stream.synchronize()
    assert g.launches() > 0
    ref = plan.eval_real(om, h0, chi, G, lnP, nus)
    assert np.array_equal(out.cpu().numpy(), ref)
    tabs2, nus2 = workloads.points(w, n, seed=22)
    om2, h02, chi2, G2, lnP2 = workloads.stack(tabs2)
    d2 = device_batch((om2, h02, chi2, G2, lnP2, nus2), dev)
    with torch.cuda.stream(stream):
        for a, b in zip(d, d2):
            a.copy_(b)
        g.launch(stream.cuda_stream)
    stream.synchronize()
    ref2 = plan.eval_real(om2, h02, chi2, G2, lnP2, nus2)
    assert np.array_equal(out.cpu().numpy(), ref2)
    assert not np.array_equal(ref, ref2)
    g.close()


@pytest.mark.gpu
def test_autotune(gpu_lib, oracle_built):
    import torch
    import oracle as O
    from test_gpu_real import plain_and_floored, REL
    dev = torch.device("cuda:0")
    w = workloads.make("real_3x2pt")
    n = 2
    tabs, nus = workloads.points(w, n, seed=23)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=n)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    d = device_batch((om, h0, chi, G, lnP, nus), dev)
    c, st, ms = plan.autotune(*d, reps=2)
    print("autotune:", c, st, ms)
    assert c in (lib.CONTRACT_TF32X3, lib.CONTRACT_BF16X6, lib.CONTRACT_FP32)
    assert st in (lib.FFTLOG_STATE_SHARED, lib.FFTLOG_STATE_GLOBAL)
    assert plan.contraction() == c and ms > 0
    dv = plan.eval_real(om, h0, chi, G, lnP, nus)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    for i in range(n):
        o.set_point(tabs[i], nus[i])
        ref = o.data_vector_real()
        _, worst_f, _ = plain_and_floored(plan, dv[i], ref, w.cfg.ntheta)
        assert worst_f <= REL, (i, worst_f)
    # the global-state form of the loop gives the same vectors to rounding
    plan.set_fftlog_state(lib.FFTLOG_STATE_GLOBAL)
    dv_g = plan.eval_real(om, h0, chi, G, lnP, nus)
    plan.set_fftlog_state(lib.FFTLOG_STATE_SHARED)
    dv_s = plan.eval_real(om, h0, chi, G, lnP, nus)
    assert np.allclose(dv_g, dv_s, rtol=1e-6, atol=1e-6 * np.abs(dv_s).max())
