"""Benchmark: batched real-space 3x2pt data vectors per second on GB300.

Workload (the real_3x2pt configuration): 10 source + 5 lens bins, 55 xi+/xi-
+ 50 gamma_t + 5 w(theta) spectra on 20 log theta bins in 2.5-250 arcmin,
Legendre sums to l = 50000 from 1000 log-spaced C_l nodes, 600 x 200
P(k, z) table per point, non-Limber w(theta) (the reference default), one
step = one batch of `--batch` distinct parameter points (each with its own
P(k,z), distances, growth and nuisances), synthetic inputs.

`value`: data vectors/s with inputs resident in HBM (torch CUDA tensors,
one CUDA-event-timed region over --steps batches); the inputs of one batch
(~1 MB of FP64 P(k,z) per point) exceed the 129 MB L2, so no flush is
needed.  `e2e`: the same metric through the public C-ABI call with host
(pinned) buffers, host->device copies of every input and device->host of
the data vectors inside the timed region.  Per-kernel durations come from
CUDA events the library records around each launch during the timed steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cocoa-cosmolike-core_gb300"))

METRIC = "3x2pt data vectors/s (real-space, <=1e-4 rel err vs FP64)"
# Legendre contraction forms of the mixed plan (cl2pt.h CL2PT_CONTRACT_*)
CONTRACTS = {"fp32": 0, "tf32x3": 1, "bf16x3": 2, "bf16x6": 3}
UNIT = "data vectors/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def max_over_ranks(x: float, device=None) -> float:
    """The largest x over the ranks of the default process group (the job's
    time is its slowest rank's); x itself without one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def walker_seed(base: int, rank: int) -> int:
    """Replicas: every rank evaluates its own walkers."""
    return base + rank


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling in the background during the timed region."""

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def make_batch(w, B, seed):
    from cl2pt import abi, workloads
    tabs, nus = workloads.points(w, B, seed=seed)
    om, h0, chi, G, lnP = workloads.stack(tabs)
    nub = np.frombuffer(b"".join(bytes(n) for n in nus), dtype=np.uint8).copy()
    return dict(om=om, h0=h0, chi=chi, G=G, lnP=lnP, nus=nus, nub=nub, tabs=tabs)


def cpu_sample(w, data, budget_s=12.0, min_pts=2, threads=None):
    """Time the oracle port (the reference algorithm restated in C, OpenMP
    over all host cores) on consecutive points of the same batch."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    n, t0 = 0, time.perf_counter()
    while True:
        o.set_point(data["tabs"][n % len(data["tabs"])], data["nus"][n % len(data["nus"])])
        o.data_vector_real()
        n += 1
        el = time.perf_counter() - t0
        if (el >= budget_s and n >= min_pts) or n >= 200:
            break
    return n, el


def parity_spot(w, data, dv, idxs, n_xi, n_gt, nt):
    """Spot check of the timed batch's data vectors against the FP64 oracle:
    the largest relative error per entry (plain, and with entries below
    1e-4 of their spectrum's peak held to that floor, the zero-crossing
    rule) and the number of entries above 1e-4 plain."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    o = O.Oracle("orc")
    o.setup(w.cfg, w.src, w.lens)
    worst_f = worst_p = 0.0
    above = total = 0
    for i in idxs:
        o.set_point(data["tabs"][i], data["nus"][i])
        ref = o.data_vector_real()
        a = n_xi // 2
        for lo, hi in ((0, a), (a, n_xi), (n_xi, n_xi + n_gt), (n_xi + n_gt, len(ref))):
            if hi <= lo:
                continue
            r = ref[lo:hi].reshape(-1, nt)
            g = dv[i, lo:hi].reshape(-1, nt)
            err = np.abs(g - r)
            peak = np.abs(r).max(axis=1, keepdims=True)
            plain = err / np.maximum(np.abs(r), 1e-300)
            floored = err / np.maximum(np.abs(r), 1e-4 * peak + 1e-300)
            worst_f = max(worst_f, float(floored.max()))
            worst_p = max(worst_p, float(plain.max()))
            above += int(np.count_nonzero(plain > 1e-4))
            total += plain.size
    return {"points": [int(i) for i in idxs], "entries": total,
            "max_rel_err_floored": worst_f, "max_rel_err_plain": worst_p,
            "entries_above_1e-4_plain": above,
            "rule": "floored: entries below 1e-4 of their spectrum's peak are held to 1e-4 of the peak"}


def run_reference(args):
    """--impl reference: the reference algorithm on the host cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(ref=False)
    from cl2pt import workloads
    w = workloads.make(args.workload)
    data = make_batch(w, 8, seed=1)
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)
    for _ in range(args.warmup):
        cpu_sample(w, data, budget_s=0.0, min_pts=1)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        n, t = cpu_sample(w, data, budget_s=2.0, min_pts=2)
        tot_n += n
        tot_t += t
    v = tot_n / tot_t
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (EH no-wiggle P(k,z), LCDM chi/D, seeded n(z) and nuisances)",
        "config": {"workload": args.workload, "points_per_step": tot_n / args.steps},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{tot_n} points over {args.steps} steps"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def value_grad(plan, w, data, d_om, d_h0, d_chi, d_G, d_lnP, d_nu, out, stream, args, p64=None):
    if out is None:
        import torch
        out = torch.empty((d_om.shape[0], plan.n_total), dtype=torch.float64, device=d_om.device)
    """value+grad/s: cl2pt_vjp_real with a fixed cotangent on device-resident
    inputs, CUDA-event timed over --steps batches (mixed plan, then the FP64
    plan as the plain-FP64 GPU form)."""
    import torch
    from cl2pt import abi
    B = d_om.shape[0]
    dev = d_om.device
    cot = torch.from_numpy(np.random.default_rng(7).normal(size=(B, plan.n_total))).to(dev)
    lbar = torch.empty_like(d_lnP)
    nbar = torch.empty_like(d_nu)
    sptr = stream.cuda_stream

    def run(p, n):
        for _ in range(n):
            p.vjp_real_device(d_om, d_h0, d_chi, d_G, d_lnP, d_nu, cot, out, lbar, nbar, stream=sptr)

    run(plan, args.warmup)
    plan.check_errors(sptr)
    torch.cuda.synchronize()
    plan.set_timing(True)
    plan.kernel_times()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run(plan, args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kms, _ = plan.kernel_times()
    plan.set_timing(False)
    plan.check_errors(sptr)
    nb = nbar.cpu().numpy().view(np.float64).reshape(B, -1)
    n_nu = int(np.count_nonzero(np.any(nb != 0.0, axis=0)))
    tatt = w.cfg.ia_model == 1
    what = "shear m, source dz, b1" + (", b2, bs2, A1, eta1, A2, eta2, b_TA" if tatt else
                                      (", A1" if w.cfg.ia_mode else ""))
    paths = "Limber table walks, FFTLog z=0 slice, non-Limber hand-over"
    if tatt or w.cfg.one_loop_bias:
        paths += ", and the FAST-PT one-loop/TATT tables through p_lin(k, z=0)"
    res = {"value": B * args.steps / (ms / 1e3), "unit": "value+gradient evaluations/s",
           "ms_per_step": ms / args.steps, "workload": w.name, "points_per_step": B,
           "grad_wrt": f"lnP table ({plan.shapes['nk']}x{plan.shapes['nz']}; {paths}) and {n_nu} nuisance "
                       f"parameters ({what})",
           "n_nuisance": n_nu, "launches_per_step": plan.launches(),
           "kernel_ms_per_step": {k: v / args.steps for k, v in kms.items() if v > 0}}
    if p64 is not None:
        run(p64, 3)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n64 = max(2, args.steps // 2)
        a.record(stream)
        run(p64, n64)
        b.record(stream)
        torch.cuda.synchronize()
        res["fp64_plain_gpu"] = B * n64 / (a.elapsed_time(b) / 1e3)
        p64.close()
    return res


def run_serving(args):
    """--workload serving: batched sampler serving.  One step = one batch of
    --batch (default 4096) parameter points through the CUDA-graph-captured
    Fourier evaluation (10 + 10 bins, 26 l bins in 20-15000, non-Limber
    clustering below l = 200 with the FFTLog on 2048 log-chi points) with
    per-point ragged scale cuts; reports data vectors/s and the per-batch
    latency distribution."""
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cl2pt import lib, workloads
    from cl2pt import build as cbuild
    cbuild.build()
    w = workloads.make("fourier_serving")
    B = args.batch if args.batch != 512 else 4096
    data = make_batch(w, B, seed=walker_seed(300, rank))
    ptr, idx = workloads.scale_cuts(w, B, seed=rank)
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=B)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d = [T(data[k]) for k in ("om", "h0", "chi", "G", "lnP")] + [T(data["nub"])]
    dptr, didx = T(ptr), T(idx)
    out = torch.zeros(int(ptr[-1]), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    # per-kernel breakdown from one eager, event-timed evaluation
    plan.set_timing(True)
    plan.kernel_times()
    with torch.cuda.stream(stream):
        g = plan.fourier_graph(*d, w.ell, out, row_ptr=dptr, idx=didx, stream=sptr)
    stream.synchronize()
    kms, kl = plan.kernel_times()
    plan.set_timing(False)
    for _ in range(args.warmup):
        g.launch(sptr)
    stream.synchronize()
    plan.check_errors(sptr)
    if world > 1:
        torch.distributed.barrier()
    clk = Clocks(local)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for k in range(args.steps):
        g.launch(sptr)
        evs[k + 1].record(stream)
    stream.synchronize()
    clocks = clk.stop()
    plan.check_errors(sptr)
    lat = np.array([evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)])
    ms = float(lat.sum())
    ms = max_over_ranks(ms, dev)
    value = world * B * args.steps / (ms / 1e3)
    # e2e: host arrays (pinned) through the public ragged call
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h = {k: pin(data[k]) for k in ("om", "h0", "chi", "G", "lnP")}
    plan.eval_fourier_ragged(h["om"], h["h0"], h["chi"], h["G"], h["lnP"], data["nus"], w.ell, ptr, idx)
    n_e = max(2, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(n_e):
        rag = plan.eval_fourier_ragged(h["om"], h["h0"], h["chi"], h["G"], h["lnP"], data["nus"], w.ell,
                                       ptr, idx)
    te = time.perf_counter() - t0
    e2e = world * B * n_e / te
    h2d = sum(h[k].nbytes for k in h) + B * 13 * 20 * 8 + ptr.nbytes + idx.nbytes
    # value + gradient: cl2pt_vjp_fourier on the same device batch, with a
    # cotangent that is zero outside each point's kept entries
    vg = None
    if not args.no_grad:
        nfull = plan_fourier_size(plan, len(w.ell))
        cot_h = np.zeros((B, nfull))
        rng = np.random.default_rng(5)
        for i in range(B):
            sel = idx[ptr[i]:ptr[i + 1]]
            cot_h[i, sel] = rng.normal(size=len(sel))
        cot = T(cot_h)
        dvf = torch.empty((B, nfull), dtype=torch.float64, device=dev)
        lbar = torch.empty_like(d[4])
        nbar = torch.empty_like(d[5])

        def vjp():
            plan.vjp_fourier_device(*d, w.ell, cot, dvf, lbar, nbar, stream=sptr)

        with torch.cuda.stream(stream):
            for _ in range(2):
                vjp()
        stream.synchronize()
        n_g = max(2, args.steps // 4)
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record(stream)
        with torch.cuda.stream(stream):
            for _ in range(n_g):
                vjp()
        b_.record(stream)
        stream.synchronize()
        plan.check_errors(sptr)
        msg = a_.elapsed_time(b_) / n_g
        vg = {"value": world * B / (msg / 1e3), "unit": "value+gradient evaluations/s", "ms_per_batch": msg,
              "grad_wrt": "lnP table (600x200) and the nuisances (shear m, source dz, b1)"}
    hbm, src = peaks()
    top = max(kms, key=lambda k: kms[k])
    line = {
        "metric": "Fourier 3x2pt data vectors/s, batched serving (CUDA-graph replay, ragged scale cuts)",
        "value": value, "unit": "data vectors/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (EH no-wiggle P(k,z) per point, seeded photo-z shifts and nuisances)",
        "config": {"workload": "fourier_serving", "points_per_step_per_gpu": B, "n_source": 10,
                   "n_lens": 10, "nell": len(w.ell), "ell_range": [20, 15000], "lmax_nolimber": 200,
                   "nl_nchi": 2048, "n_data_full": plan_fourier_size(plan, len(w.ell)),
                   "kept_fraction_mean": float(np.diff(ptr).mean() / plan_fourier_size(plan, len(w.ell))),
                   "l2": "inputs > L2 (no flush)"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "min": float(lat.min()), "max": float(lat.max()), "batches": int(len(lat))},
        "e2e": {"value": e2e, "unit": "data vectors/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(rag.nbytes)},
        "gpu_launches": int(g.launches() * args.steps),
        "value_grad": vg,
        "kernel_ms_per_batch": {k: v for k, v in kms.items() if v > 0},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": None, "peak": hbm, "unit": "GB/s",
                     "frac": None, "traffic": None, "peak_source": src,
                     "note": "FFTLog multipole loop dominates: FP32-pipe / barrier bound (profiles/)"},
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        o = O.Oracle("orc")
        o.setup(w.cfg, w.src, w.lens)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < 12.0 or n < 2:
            o.set_point(data["tabs"][n % B], data["nus"][n % B])
            o.data_vector_fourier(w.ell)
            n += 1
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n / t, "unit": "data vectors/s", "cores": os.cpu_count(),
                                "kind": "port", "sample": f"{n} points of the same batch, {t:.1f} s"}
    if rank == 0:
        print(json.dumps(line))
    g.close()
    plan.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def plan_fourier_size(plan, nell):
    import ctypes as C
    from cl2pt import lib
    nt = C.c_int()
    lib.check(lib.load().cl2pt_fourier_sizes(plan.h, nell, None, None, None, C.byref(nt)))
    return nt.value


def run_fastpt(args):
    """--workload fastpt: the batched FAST-PT workload -- for each linear
    spectrum (2048 log-k in 1e-5..1e3 h/Mpc) get_FPT_bias's five one-loop
    bias spectra and get_FPT_IA's ten TATT rows."""
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cl2pt import lib, workloads
    from cl2pt import build as cbuild
    cbuild.build()
    B = args.batch
    k, P, _ = workloads.fastpt_spectra(B, seed=walker_seed(100, rank))
    pb = lib.FastPT.for_bias(k, max_spec=B)
    pi = lib.FastPT.for_ia(k, max_spec=B)
    fx = torch.from_numpy(P).to(dev)
    ob = torch.empty((B, 5, len(k)), dtype=torch.float64, device=dev)
    oi = torch.empty((B, 10, len(k)), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step():
        pb.bias_device(fx, ob, sptr)
        pi.ia_device(fx, oi, sptr)

    for _ in range(args.warmup):
        step()
    pb.check_errors()
    pi.check_errors()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = Clocks(local)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(stream)
    for _ in range(args.steps):
        pb.bias_device(fx, ob, sptr)
    ev[1].record(stream)
    for _ in range(args.steps):
        pi.ia_device(fx, oi, sptr)
    ev[2].record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    pb.check_errors()
    pi.check_errors()
    ms_b, ms_i = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    ms = ms_b + ms_i
    ms = max_over_ranks(ms, dev)
    value = world * B * args.steps / (ms / 1e3)
    waves_b, waves_i = -(-B // 512), -(-B // 256)
    launches = (3 * waves_b + 4 * waves_i + 1) * args.steps
    # e2e: host (pinned) spectra in, both tables out, through the C ABI
    Ph = torch.from_numpy(P).pin_memory().numpy()
    for _ in range(2):
        rb, ri = pb.bias(Ph), pi.ia(Ph)
    n_e = max(2, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(n_e):
        rb, ri = pb.bias(Ph), pi.ia(Ph)
    te = time.perf_counter() - t0
    e2e = world * B * n_e / te
    N0 = len(k)
    hbm, src = peaks()
    alg_bytes = 8 * N0 * (1 + 5) * B
    achieved = alg_bytes / (ms_b / args.steps / 1e3) / 1e9
    line = {
        "metric": "FAST-PT spectra/s (one-loop bias + TATT IA tables per input spectrum, FP64)",
        "value": value, "unit": "input spectra/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (EH no-wiggle P(k), per-spectrum Om, h, ns, sigma8 ~ U)",
        "config": {"workload": "fastpt", "spectra_per_step_per_gpu": B, "nk": N0,
                   "bias": {"N": 6048, "Ntot": 12150, "nu": -2.0, "terms": 13},
                   "ia": {"N": 6048, "Ntot": 12150, "terms": 184, "direct_conv": 6144},
                   "c_window": 0.65, "N_pad": 1500, "N_extrap": [500, 500],
                   "l2": "per-spectrum workspace > 1 MB x batch > L2"},
        "split_ms_per_step": {"bias": ms_b / args.steps, "ia": ms_i / args.steps},
        "e2e": {"value": e2e, "unit": "input spectra/s", "h2d_bytes_per_step": int(2 * P.nbytes),
                "d2h_bytes_per_step": int(rb.nbytes + ri.nbytes)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_fpt_* (bias pass)", "achieved": achieved,
                     "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                     "peak_source": src,
                     "note": "FP64-pipe bound (ncu: FP64 pipe 81-84% active); see profiles"},
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        o = O.Oracle("orc")
        a, b, l, _, _ = lib.bias_terms()
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < 15.0 or n < 2:
            o.J_abl(k, P[n % B], a, b, l)
            o.fpt_ia_spectrum(k, P[n % B])
            n += 1
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n / t, "unit": "input spectra/s", "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": f"{n} spectra of the same batch (13 J_abl + 184 J_abJ1J2Jk "
                                          f"terms + 2 direct convolutions each), {t:.1f} s"}
    if rank == 0:
        print(json.dumps(line))
    pb.close()
    pi.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--workload", default="real_3x2pt")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--contract", default="tf32x3", choices=sorted(CONTRACTS),
                    help="Legendre contraction of the mixed plan")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "fastpt":
        return run_fastpt(args)
    if args.workload == "serving":
        return run_serving(args)

    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cl2pt import lib, workloads
    from cl2pt import build as cbuild
    cbuild.build()
    w = workloads.make(args.workload)
    B = args.batch
    data = make_batch(w, B, seed=walker_seed(100, rank))
    plan = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_MIXED, max_batch=B)
    plan.set_contraction(CONTRACTS[args.contract])
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_om, d_h0, d_chi, d_G, d_lnP = (T(data[k]) for k in ("om", "h0", "chi", "G", "lnP"))
    d_nu = T(data["nub"])
    out = torch.empty((B, plan.n_total), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step(p=plan, o=out):
        p.eval_real_device(d_om, d_h0, d_chi, d_G, d_lnP, d_nu, o, stream=sptr)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    plan.check_errors(sptr)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    plan.set_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    kms, kl = plan.kernel_times()
    plan.set_timing(False)
    plan.check_errors(sptr)
    launches = plan.launches() * args.steps
    ms = max_over_ranks(ms, dev)
    value = world * B * args.steps / (ms / 1e3)
    dv_timed = out.cpu().numpy()  # the last timed step's data vectors

    # ---- e2e through the C ABI with pinned host buffers
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h = {k: pin(data[k]) for k in ("om", "h0", "chi", "G", "lnP")}
    dv_host = pin(np.zeros((B, plan.n_total)))
    for _ in range(2):
        plan.eval_real(h["om"], h["h0"], h["chi"], h["G"], h["lnP"], data["nus"], out=dv_host)
    torch.cuda.synchronize()
    barrier()
    # as many calls as the device-timed steps: a wall-clock number over a
    # few calls is sensitive to other work on the host
    e2e_steps = max(5, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.eval_real(h["om"], h["h0"], h["chi"], h["G"], h["lnP"], data["nus"], out=dv_host)
    te = time.perf_counter() - t0
    te = max_over_ranks(te, dev)
    e2e = world * B * e2e_steps / te
    h2d = sum(h[k].nbytes for k in h) + B * 13 * 20 * 8
    d2h = dv_host.nbytes

    # ---- plain FP64 GPU form of the same pipeline
    fp64 = None
    if not args.no_fp64:
        p64 = lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64, max_batch=B)
        o64 = torch.empty_like(out)
        for _ in range(3):
            step(p64, o64)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n64 = max(2, args.steps // 2)
        a.record(stream)
        for _ in range(n64):
            step(p64, o64)
        b.record(stream)
        torch.cuda.synchronize()
        fp64 = B * n64 / (a.elapsed_time(b) / 1e3)
        p64.close()

    # ---- value + gradient: cl2pt_vjp_real on the same batch (forward and
    # hand-written adjoint in one call; gradient w.r.t. the P(k, z) table and
    # every nuisance parameter the data vector depends on)
    vg = None
    if not args.no_grad:
        vg = value_grad(plan, w, data, d_om, d_h0, d_chi, d_G, d_lnP, d_nu, out, stream, args,
                        None if args.no_fp64 else lib.Plan(w.cfg, w.src, w.lens, w.base, lib.PREC_FP64,
                                                           max_batch=B))

    # ---- value + gradient of the differentiable layout: TATT intrinsic
    # alignments, one-loop bias, photo-z shifts and m-bias on the same
    # geometry (real_3x2pt_tatt)
    vg4 = None
    if not args.no_grad:
        w4 = workloads.make("real_3x2pt_tatt")
        B4 = min(B, 256)
        data4 = make_batch(w4, B4, seed=walker_seed(200, rank))
        plan4 = lib.Plan(w4.cfg, w4.src, w4.lens, w4.base, lib.PREC_MIXED, max_batch=B4)
        t4 = [T(data4[k]) for k in ("om", "h0", "chi", "G", "lnP")]
        vg4 = value_grad(plan4, w4, data4, *t4, T(data4["nub"]), None, stream, args)
        plan4.close()

    # ---- roofline of the dominant kernel group.  The library records one
    # event pair per launch group per wave (and, for the FFTLog stage, one
    # for its second-stream transforms as well), so the per-step group time
    # is the figure to divide by: achieved = algorithmic bytes per point x
    # the points of one step / that group's event time per step.
    hbm, src = peaks()
    top = max(kms, key=lambda k: kms[k])
    step_ms = kms[top] / args.steps
    # the plan evaluates a batch in waves of up to 512 points
    wave = min(B, 512)
    waves = -(-B // wave)
    nk, nz = plan.shapes["nk"], plan.shapes["nz"]
    pss, pgs, pgg = plan.n_xi // (2 * w.cfg.ntheta), plan.n_gammat // w.cfg.ntheta, w.cfg.n_lens
    nnode = w.cfg.lmin_tab - 1 + w.cfg.n_ell
    nt = w.cfg.ntheta
    # algorithmic bytes per point of each kernel group (the counting rules:
    # compulsory P(k,z) table read + node-table write for the Limber
    # kernels, the C_l tables read + observables written for the
    # contraction, the radial kernels + C_l for the FFTLog stage)
    per_point = {
        "k_limber_ss": 8 * nk * nz + 8 * pss * nnode,
        "k_limber_gs": 8 * nk * nz + 8 * pgs * nnode,
        "k_limber_gg": 8 * nk * nz + 8 * pgg * nnode,
        "k_limber_ggl": 8 * nk * nz + 16 * pgg * w.cfg.lmax_nolimber,
        "k_nonlimber": 8 * w.cfg.nl_nchi * 3 * pgg + 8 * pgg * w.cfg.lmax_nolimber,
        "k_contract": 8 * (pss + pgs + pgg) * nnode + 8 * pgg * w.cfg.lmax_nolimber + 8 * plan.n_total,
        "k_gtab": 8 * plan.shapes["chi"] + 8 * w.cfg.n_source * w.cfg.n_a,
        "k_nodes": 8 * (plan.shapes["chi"] + plan.shapes["G"]),
        "k_assemble": 16 * plan.n_total,
    }
    alg_step = per_point.get(top, 0) * B
    achieved = alg_step / (step_ms / 1e3) / 1e9 if step_ms > 0 else None
    # arithmetic of the same group by the counting rules (integrand
    # evaluations x a fixed cost for the Limber kernels, 2 K per output for
    # the contraction, 2.5 N log2 N per real transform + 10 N_chi per
    # multipole and radial kernel for the FFTLog loop), against the nominal
    # FP32 rate (SMs x 128 lanes x 2 x the sampled SM clock)
    conv = np.concatenate([plan.nonlimber(i)[1] for i in range(min(wave, B))]) \
        if top == "k_nonlimber" else None
    nl_n = [900, 1500, 1500] if w.cfg.nl_nchi == 500 else None
    flops_pt = {
        "k_limber_ss": 12.0 * nnode * pss * 64,
        "k_limber_gs": 20.0 * nnode * pgs * 64,
        "k_limber_gg": 30.0 * nnode * pgg * 96,
        "k_contract": 2.0 * nnode * nt * (2 * pss + pgs + pgg),
    }
    if conv is not None and nl_n is not None:
        per_l = sum(2.5 * n * np.log2(n) + 10 * w.cfg.nl_nchi for n in nl_n[:2])
        flops_pt["k_nonlimber"] = float(conv.mean()) * pgg * per_l
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    pipe = None
    if top in flops_pt and step_ms > 0:
        tf = flops_pt[top] * B / (step_ms / 1e3) / 1e12
        pipe = {"unit": "TFLOP/s", "achieved": tf, "peak": fp32_peak, "frac": tf / fp32_peak,
                "peak_source": f"nominal FP32: {sms} SMs x 128 lanes x 2 x {mhz:.0f} MHz",
                "flops_per_point": flops_pt[top]}
        if conv is not None:
            pipe["mean_handover_multipole"] = float(conv.mean())
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (EH no-wiggle P(k,z) per point, LCDM chi/D, seeded n(z) and nuisances)",
        "config": {"workload": args.workload, "points_per_step_per_gpu": B, "contraction": args.contract,
                   "n_data": plan.n_total, "lmax": w.cfg.lmax, "n_ell": w.cfg.n_ell,
                   "pk_table": [nk, nz], "l2": "inputs > L2 (no flush)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm if achieved else None, "traffic": None,
                     "algorithmic_bytes_per_point": per_point.get(top),
                     "algorithmic_bytes_per_launch": per_point.get(top, 0) * wave,
                     "launches_per_step": waves, "group_ms_per_step": step_ms,
                     "peak_source": src, "pipe": pipe},
        "kernel_ms_per_step": {k: v / args.steps for k, v in kms.items()},
        "clocks": clocks,
        "fp64_plain_gpu": {"value": fp64, "unit": UNIT,
                           "speedup_of_mixed": (value / world) / fp64 if fp64 else None},
    }
    if vg is not None:
        vg["value"] *= world
        line["value_grad"] = vg
    if vg4 is not None:
        vg4["value"] *= world
        line["value_grad_tatt"] = vg4
    if rank == 0 and not args.no_cpu:
        line["parity"] = parity_spot(w, data, dv_timed, [0, B // 3, (2 * B) // 3, B - 1], plan.n_xi,
                                     plan.n_gammat, w.cfg.ntheta)
    if rank == 0 and world == 1 and not args.no_cpu:
        n, t = cpu_sample(w, data, budget_s=12.0)
        line["cpu_baseline"] = {"value": n / t, "unit": UNIT, "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": f"{n} points of the same batch, {t:.1f} s"}
        if vg is not None:
            # central differences on the CPU: 2 evaluations per parameter + 1
            npar = vg["n_nuisance"]
            vg["cpu_fd"] = {"value": (n / t) / (2 * npar + 1), "unit": "value+gradient/s",
                            "kind": "port", "cores": os.cpu_count(),
                            "note": f"nuisance gradient only ({npar} parameters) by central "
                                    f"differences; the {nk}x{nz} table gradient would take "
                                    f"{2 * nk * nz} more evaluations"}
    if rank == 0:
        print(json.dumps(line))
    plan.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
