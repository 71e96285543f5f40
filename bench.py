"""Benchmark: objective + gradient evaluations per second on one GB300.

A step is one ObjectiveFunction::calcFunction + calcGradient pair (chi2 with
entropy and TSV priors active, DChi2 direct-sum gradient) over the whole
synthetic data set, i.e. one "chi2+grad evaluation" of the headline metric.
Default workload: 2048 x 2048 image, 8 channels 225-235 GHz, 50 antennas in a
2 km disk, 4 h at 4 s, Briggs robust 0 (35.28M visibilities), seeded
synthetic data.

  value   device-timed evaluations/s with every input resident in HBM;
  e2e     the same through the public API (gpuvmem_gb300.Problem), the image
          copied in from pinned host memory and the gradient and objective
          read back every step;
  roofline  the dominant kernel (tcgen05 DChi2, timed inside the timed
          loop as the gradient call) as TFLOP/s against the measured
          sustained dense BF16 peak / 3 (three FP16 products per
          algorithmic multiply-add; the gradient runs about a second per
          launch inside a long loop);
  reference_cuda  the reference's own CUDA kernels (compiled from its
          sources, launched with its launch shapes and host sequence by the
          harness in oracle/ref_harness) timed on the same GPU: chi2() in
          full, dchi2() over a band of rows scaled to the image;
  converge  the first half of the headline metric: wall time to an
          objective within 1e-4 of the plain solver's converged value, from
          the learned warm start (network forward pass and start policy
          included) against the plain start, on held-out 256^2 skies;
  cpu_baseline  the CPU oracle (FP64 restatement of the reference's
          algorithm) on a bounded sample, scaled to evaluations/s.

--impl reference times the reference's CPU implementation of this path.  The
reference has none (its objective and gradient exist only as CUDA kernels),
so the arm runs the oracle port with all host threads; each step is a bounded
sample (the full chi2 and DChi2 at a few pixels), scaled to one evaluation.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from gpuvmem_gb300 import synth  # noqa: E402

METRIC = "chi2+grad evals/s"
L2_BYTES = 129 * 2 ** 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3])
    ap.add_argument("--engine", type=int, default=0)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--case", default=None, help="run a profiling case instead of the bench")
    ap.add_argument("--autotune", action="store_true",
                    help="measure and keep the fastest launch shapes before timing")
    ap.add_argument("--converge-skies", type=int, default=200,
                    help="held-out skies of the warm-start measurement (0: skip)")
    ap.add_argument("--ref-band-rows", type=int, default=16,
                    help="image rows of the reference DChi2 band (configuration 1)")
    ap.add_argument("--no-reference-cuda", action="store_true")
    return ap.parse_args()


def workload(cfg_id):
    cfg = {0: synth.CONFIG0, 1: synth.CONFIG1, 2: synth.CONFIG2}[cfg_id]
    terms = [("Chi2", 1.0), ("Entropy", 0.01), ("TotalSquaredVariation", 1e-4)]
    return cfg, terms


def config_desc(cfg, data):
    return {"workload": f"{cfg.name}: {cfg.n}x{cfg.n} image, {len(cfg.freqs_hz)} channels, "
                        f"{data.nvis} visibilities, {cfg.weighting} weights",
            "image": cfg.n, "channels": len(cfg.freqs_hz), "visibilities": int(data.nvis),
            "objective": "chi2 + entropy + TSV", "step": "objective + gradient",
            "l2": "inputs larger than L2" if data.nvis * 56 > L2_BYTES
                  else "L2 flushed between timed steps"}


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            # a sample before the region starts (short regions end before the
            # next 200 ms sample)
            t0 = time.time()
            while not self.rows and time.time() - t0 < 3.0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            # and one after it ends
            n0, t0 = len(self.rows), time.time()
            while len(self.rows) == n0 and time.time() - t0 < 1.0:
                time.sleep(0.01)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, device=0):
        rows = [r for r in self.rows if len(r) >= 9 and r[0] == str(device)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# DRAM bytes per visibility of one DChi2 launch (dram__bytes_read.sum +
# dram__bytes_write.sum of k_dchi2_tc in an ncu capture of the one-channel
# 2048^2 case, `bench.py --case dchi2_2048_1ch`, divided by its
# visibilities).  The traffic of the full launch is this times its
# visibilities: the operands are generated on chip, so the traffic is the
# visibility constants re-read per output tile plus the partial images.
DCHI2_DRAM_BYTES_PER_VIS = 168.48
DCHI2_TRAFFIC_SOURCE = ("ncu capture of k_dchi2_tc, one channel of 2048^2 (bench.py --case "
                        "dchi2_2048_1ch), scaled by the visibility count")


def cpu_baseline(data, terms, sample_s, impl_kind="port"):
    """The FP64 CPU oracle on a bounded sample: the full objective of the
    first channel and the DChi2 sum at a few pixels, scaled to one full
    objective + gradient evaluation over all channels and mask pixels."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    kinds = {"Chi2": O.FI_CHI2, "Entropy": O.FI_ENTROPY, "TotalSquaredVariation": O.FI_TSV}
    oterms = [(kinds[k], lam, 0, 0, 0.001, -1.0, 1e-12) for k, lam in terms]
    orc = O.Oracle(data, oterms)
    img = orc.initial_image()
    C = len(data.freqs)
    t0 = time.time()
    # objective: all channels in full (FFT + degrid + chi2)
    chi0 = time.time()
    orc.chi2(img.copy())
    t_obj = time.time() - chi0
    # gradient: DChi2 at a few mask pixels of channel 0 until the budget
    mask_idx = np.flatnonzero(orc.mask.ravel())
    rng = np.random.default_rng(0)
    npix, t_grad = 0, 0.0
    while t_grad < sample_s and npix < mask_idx.size:
        pix = rng.choice(mask_idx, size=1)
        tg = time.time()
        orc.dchi2_pixels(0, pix)
        t_grad += time.time() - tg
        npix += 1
    per_eval = t_obj + t_grad / npix * mask_idx.size * C
    return {"value": 1.0 / per_eval, "unit": METRIC, "cores": O.lib().or_num_threads(),
            "kind": impl_kind,
            "sample": f"FP64 oracle: full chi2 of all {C} channels ({t_obj:.1f} s) + DChi2 at "
                      f"{npix} of {mask_idx.size} mask pixels of channel 0 over all its "
                      f"visibilities ({t_grad:.1f} s), scaled to the full gradient",
            "seconds": time.time() - t0}


def run_reference(args):
    """The FP64 oracle port on the host cores (the reference has no CPU
    implementation of this path).  Each step is one bounded sample -- the
    full chi2 of every channel and DChi2 at mask pixels of channel 0 for a
    fixed time -- scaled to one full evaluation; ms_per_step is the
    sample's own wall time, ms_per_eval the scaled figure."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.config == 3:
        raise SystemExit("--impl reference covers configurations 0-2")
    cfg, terms = workload(args.config)
    data = synth.generate(cfg, device=None if args.config == 0 else _gen_device())
    per_eval, walls = [], []
    base = None
    for s in range(args.warmup + args.steps):
        t0 = time.time()
        b = cpu_baseline(data, terms, max(2.0, args.cpu_sample_s / max(1, args.steps)))
        if s >= args.warmup:
            per_eval.append(1.0 / b["value"])
            walls.append(time.time() - t0)
            base = b
    v = args.steps / sum(per_eval)
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(walls) / args.steps,
            "ms_per_eval": 1e3 * sum(per_eval) / args.steps,
            "step": "one bounded sample (full chi2 + DChi2 at a few mask pixels), scaled to "
                    "one evaluation for value",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (FP64 oracle port; the reference computes this path in FP32 on the GPU)",
            "data": "synthetic", "config": config_desc(cfg, data), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": base["cores"],
                             "kind": "port", "sample": base["sample"]},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cufft_inverse_2d(C, n, stream, reps=5):
    """Device time of cuFFT's unnormalised inverse 2-D C2C transform of C
    grids of n x n complex64 (the comparison the FFT passes stand against)."""
    import torch
    x = torch.randn(C, n, n, dtype=torch.complex64, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(2):
            torch.fft.ifft2(x, norm="forward")
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(reps)]
        for a, b in ev:
            a.record(stream)
            torch.fft.ifft2(x, norm="forward")
            b.record(stream)
    torch.cuda.synchronize()
    return statistics.median(a.elapsed_time(b) for a, b in ev) / 1e3


def reference_cuda(data, img, band_rows):
    """The reference's own kernels on this GPU (oracle/ref_harness): device
    time of chi2() (src/functions.cu:4323-4454) and of dchi2()
    (:4456-4558); dchi2 over a band of rows at the image centre, scaled by
    N / rows when the band is not the whole image (every row of the
    benchmark images lies inside the mask, so rows cost alike)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import refrun
    except Exception as e:  # pragma: no cover
        return {"unavailable": f"harness import failed: {e}"}
    if not refrun.available():
        return {"unavailable": "reference kernels (oracle/_ref/ref_kernels.cubin) or the "
                               "harness library are not built"}
    rows = max(16, min(data.N, band_rows) // 16 * 16)
    ref = refrun.RefHarness(data)
    try:
        ms_chi2, ms_band = ref.time(img, reps=3 if rows == data.N else 1, band_rows=rows)
    finally:
        ref.close()
    ms_dchi2 = ms_band * data.N / rows
    return {"evals_per_s": 1e3 / (ms_chi2 + ms_dchi2), "chi2_ms": ms_chi2, "dchi2_ms": ms_dchi2,
            "dchi2_band_rows": rows, "dchi2_scaled_from_band": rows < data.N,
            "build": "reference kernels compiled unmodified from src/functions.cu for sm_103a, "
                     "launch shapes -X 16 -Y 16 -V 256, cuFFT, the reference's host sequence"}


def converge_measure(n_skies):
    """Time to converge, learned warm start against the plain start, on
    held-out skies (seeds 900000...) of the 256^2 configuration-0 array:
    wall time until a line search reaches f <= f* (1 + 1e-4), f* the plain
    solver's converged objective; the warm time includes the network's
    forward pass and the start policy."""
    from gpuvmem_gb300 import warmstart as W
    path = W.NETWORK_PATH
    if not os.path.exists(path):
        return {"unavailable": f"no trained network at {os.path.relpath(path, ROOT)}"}
    net, meta = W.load_network(path)
    t0 = time.time()
    with Clocks() as clk:
        rows = W.evaluate(net, range(900000, 900000 + n_skies), iterations=300)
    summ = W.summarize(rows)
    pol = [r["t_policy"] for r in rows]
    out = {"skies": n_skies, "seeds": f"900000-{900000 + n_skies - 1} (held out)",
           "rel": 1e-4, "solver": "CG-FRPRMN (line search on the GPU), chi2 + entropy 0.01",
           "network": {k: meta[k] for k in ("levels", "base_channels", "train_skies", "epochs")
                       if k in meta},
           "policy_ms_median": 1e3 * statistics.median(pol) if pol else None,
           "seconds": time.time() - t0, "clocks": clk.summary(0)}
    out.update(summ)
    return out


def max_over_ranks(t, dist, device):
    """The slowest rank's time (every rank gets it).  Ranks are independent
    replicas of the problem, so this is the whole job's time."""
    import torch
    tt = torch.tensor([float(t)], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_throughput(world, steps, t):
    """Whole-job evaluations per second of `world` replicas that each did
    `steps` evaluations in (at most) t seconds."""
    return world * steps / t


def _gen_device():
    import torch
    return "cuda" if torch.cuda.is_available() else None


def run_ours(args):
    import torch
    import gpuvmem_gb300 as gv

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cfg, terms = workload(args.config)
    data = synth.generate(cfg, device="cuda")
    prob = gv.Problem(data, [gv.term(k, lam) for k, lam in terms], engine=args.engine)
    stream = torch.cuda.current_stream()
    prob.set_stream(stream.cuda_stream)
    tune = None
    if args.autotune:
        r = prob.autotune()
        tune = {f: getattr(r, f) for f, _ in r._fields_}
    info = prob.info
    img = prob.initial_image()
    xi = torch.zeros_like(img)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    small = data.nvis * 56 <= L2_BYTES

    # the gradient (DChi2 plus the prior gradients) is bracketed by events
    # inside the timed step: its launches' average duration is the
    # roofline's
    evg = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]

    def step(s=None):
        f, _ = prob.objective(img)
        if s is not None:
            evg[s][0].record(stream)
        prob.gradient(img, 1, xi=xi)
        if s is not None:
            evg[s][1].record(stream)
        return f

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = gv.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks() as clk:
        for s in range(args.steps):
            if small:
                flush.zero_()
            ev[s][0].record(stream)
            step(s)
            ev[s][1].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = (gv.launch_count() - launches0) // args.steps
    t = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    if dist:
        t = max_over_ranks(t, dist, "cuda")
    value = replica_throughput(world, args.steps, t)

    t_grad = sum(a.elapsed_time(b) for a, b in evg) / 1e3 / args.steps

    # DChi2 alone (gv_dchi2 = tcgen05 kernel + split-K reduce), a few
    # launches after the timed loop
    prob.chi2(img)
    evk = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(3)]
    for a, b in evk:
        a.record(stream)
        prob.dchi2(img, out=xi)
        b.record(stream)
    torch.cuda.synchronize()
    t_dchi2 = statistics.median(a.elapsed_time(b) for a, b in evk) / 1e3

    # objective alone (clip + I_nu + beam staging, FFTs, degridding with the
    # residuals stored, chi2 and prior sums): degridded visibilities per
    # second and the HBM roofline of the objective path
    evo = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(5)]
    for a, b in evo:
        if small:
            flush.zero_()
        a.record(stream)
        prob.objective(img)
        b.record(stream)
    torch.cuda.synchronize()
    t_obj_call = statistics.median(a.elapsed_time(b) for a, b in evo) / 1e3
    # the objective as the optimisers evaluate it: per evaluation inside
    # linmin (bracket + Brent along -gradient from the current image; the
    # search's set-up and read-back included, L2 warm from one evaluation to
    # the next as in a solve)
    p_ls, d_ls = torch.empty_like(img), torch.empty_like(img)
    ls = []
    for _ in range(3):
        p_ls.copy_(img)
        torch.neg(xi, out=d_ls)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, n_ls = prob.linmin(p_ls, d_ls)
        ls.append(((time.perf_counter() - t0), n_ls))
    t_obj = statistics.median(t / max(k, 1) for t, k in ls)
    t_cufft = cufft_inverse_2d(len(data.freqs), cfg.n, stream)

    # end to end through the public API with host buffers
    h_img = torch.empty(img.shape, dtype=torch.float32).pin_memory()
    h_img.copy_(img.cpu())
    h_xi = torch.empty(img.shape, dtype=torch.float32).pin_memory()
    d_img = torch.empty_like(img)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        d_img.copy_(h_img, non_blocking=True)
        f, _ = prob.objective(d_img)
        prob.gradient(d_img, 1, xi=xi)
        h_xi.copy_(xi, non_blocking=True)
        torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    e2e = world * args.steps / t_e2e

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks, src = measured_peaks()
    # about a second per launch, inside a loop of several seconds: the
    # sustained (power-capped) peak; the burst figure is reported beside it
    peak = peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"]) / 3.0
    peak_burst = peaks["bf16_tflops"] / 3.0
    V = info.nvis_in_grid
    flops = 4.0 * cfg.n * cfg.n * V
    achieved = flops / t_grad / 1e12
    traffic = DCHI2_DRAM_BYTES_PER_VIS * V if info.dchi2_engine == 2 else None
    # objective algorithmic bytes of a line-search evaluation: both image
    # planes read once (8 MN), per channel a grid written by the row FFTs and
    # read + written by the column FFTs (16 MN), 20 B per visibility in
    # (u, v, Vo, w); the line search stores no residuals
    MN = cfg.n * cfg.n
    obj_bytes = 8.0 * MN + 16.0 * MN * len(data.freqs) + 20.0 * data.nvis
    obj = {"ms": 1e3 * t_obj,
           "ms_note": "per objective evaluation inside gv_linmin (wall time of the whole "
                      "search over its evaluation count)",
           "linmin_evaluations": [k for _, k in ls], "ms_single_call": 1e3 * t_obj_call,
           "ms_single_call_note": "one gv_objective call on its own, CUDA events around the "
                                  "call (its host round trip included)",
           "degridded_vis_per_s": data.nvis / t_obj,
           "algorithmic_bytes": obj_bytes, "achieved_gbs": obj_bytes / t_obj / 1e9,
           "hbm_peak_gbs": peaks["hbm_gbs"], "frac": obj_bytes / t_obj / 1e9 / peaks["hbm_gbs"],
           "note": "8 MN + 16 MN per channel + 20 B per visibility",
           "cufft_inverse_2d_ms": 1e3 * t_cufft,
           "cufft_note": "cuFFT (torch.fft.ifft2, unnormalised) of the same C x N x N complex64 "
                         "grids, for comparison with the two FFT passes of the objective (which "
                         "also stage the image and apply the phase rotation); not on the "
                         "product path"}
    cpu = cpu_baseline(data, terms, args.cpu_sample_s)
    refc = None
    if not args.no_reference_cuda:
        try:
            refc = reference_cuda(data, img.cpu().numpy(),
                                  args.ref_band_rows if cfg.n > 512 else cfg.n)
            if "evals_per_s" in refc:
                refc["speedup_value"] = value / refc["evals_per_s"]
                refc["speedup_e2e"] = e2e / refc["evals_per_s"]
        except Exception as e:  # the harness is test infrastructure: report, go on
            refc = {"unavailable": f"{type(e).__name__}: {e}"}
    conv = converge_measure(args.converge_skies) if args.converge_skies > 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (DChi2: fp16 hi/lo x3, fp32 acc)",
        "data": "synthetic (seeded; no public data set)", "config": config_desc(cfg, data),
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": int(img.numel() * 4),
                "d2h_bytes_per_step": int(xi.numel() * 4 + 8 * (1 + len(terms)))},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": DCHI2_TRAFFIC_SOURCE,
                     "kernel": "k_dchi2_tc + k_reduce_partials (+ prior gradients): the "
                               "gradient call, timed inside the timed loop",
                     "peak_source": f"{src} dense bf16 sustained "
                                    f"{peaks.get('bf16_tflops_sustained')} TFLOP/s / 3",
                     "frac_of_burst": achieved / peak_burst,
                     "gradient_ms": 1e3 * t_grad, "dchi2_alone_ms": 1e3 * t_dchi2,
                     "algorithmic_flop": flops},
        "objective": obj,
        "reference_cuda": refc,
        "converge": conv,
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "clocks": clk.summary(local),
        "gpu_launches": int(launches),
        "engine": info.dchi2_engine,
    }
    if tune is not None:
        line["autotune"] = tune
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_batch(args):
    """Configuration 3: 64 independent problems (sides 128-512, 20k-500k
    visibilities each); a step is one objective + gradient evaluation of
    every problem, all of them in one CUDA-graph launch (gv_batch)."""
    import torch
    import gpuvmem_gb300 as gv
    rank = int(os.environ.get("RANK", "0"))
    cfgs, lams = synth.config3_problems()
    probs, imgs, xis = [], [], []
    flops, nvis = 0.0, 0
    for c, lam in zip(cfgs, lams):
        d = synth.generate(c, device="cuda")
        p = gv.Problem(d, [gv.term("Chi2", 1.0), gv.term("Entropy", lam)])
        probs.append(p)
        img = p.initial_image()
        imgs.append(img)
        xis.append(torch.zeros_like(img))
        flops += 4.0 * c.n * c.n * p.info.nvis_in_grid
        nvis += d.nvis
    batch = gv.Batch(probs)
    n = len(probs)

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / steps

    launches0 = gv.launch_count()
    with Clocks() as clk:
        t_graph = timed(lambda: batch.evaluate(imgs, xis, 1), args.steps)
    launches = (gv.launch_count() - launches0) // (args.steps + args.warmup)
    batch.set_graphs(False)
    t_streams = timed(lambda: batch.evaluate(imgs, xis, 1), args.steps)
    batch.set_graphs(True)

    def one_by_one():
        for p, i_, x_ in zip(probs, imgs, xis):
            p.objective(i_)
            p.gradient(i_, 1, xi=x_)
    t_seq = timed(one_by_one, max(1, args.steps // 2))
    # end to end: every image in from pinned host memory, every gradient out
    h_imgs = [torch.empty(i_.shape, dtype=torch.float32).pin_memory() for i_ in imgs]
    h_xis = [torch.empty(i_.shape, dtype=torch.float32).pin_memory() for i_ in imgs]
    for h, i_ in zip(h_imgs, imgs):
        h.copy_(i_.cpu())

    def e2e_step():
        for h, i_ in zip(h_imgs, imgs):
            i_.copy_(h, non_blocking=True)
        batch.evaluate(imgs, xis, 1)
        for h, x_ in zip(h_xis, xis):
            h.copy_(x_, non_blocking=True)
    t_e2e = timed(e2e_step, args.steps)
    if rank != 0:
        return
    peaks, src = measured_peaks()
    peak = peaks["bf16_tflops"] / 3.0
    bytes_img = sum(i_.numel() * 4 for i_ in imgs)
    line = {
        "metric": METRIC, "value": n / t_graph, "unit": "problem " + METRIC, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_graph,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (DChi2: fp16 hi/lo x3, fp32 acc)", "data": "synthetic (seeded)",
        "config": {"workload": f"batch of {n} independent problems (sides 128/256/512, "
                               f"{nvis} visibilities in total), one graph launch per step",
                   "problems": n, "visibilities": int(nvis), "step": "objective + gradient of every problem"},
        "e2e": {"value": n / t_e2e, "unit": "problem " + METRIC,
                "h2d_bytes_per_step": int(bytes_img), "d2h_bytes_per_step": int(bytes_img)},
        "roofline": {"bound": "tensor", "achieved": flops / t_graph / 1e12, "peak": peak,
                     "unit": "TFLOP/s", "frac": flops / t_graph / 1e12 / peak, "traffic": None,
                     "kernel": "whole batch step (DChi2 FLOP over the step time)",
                     "peak_source": f"{src} dense bf16 burst / 3"},
        "batch_ms": {"one_graph": 1e3 * t_graph, "streams_no_graph": 1e3 * t_streams,
                     "one_problem_after_another": 1e3 * t_seq},
        "clocks": clk.summary(0), "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)


def weighting_inputs(cfg):
    """uvw (metres) and natural weights of a configuration's visibilities,
    channel by channel (no sky needed for the weighting schemes)."""
    rng = np.random.default_rng([cfg.seed, 1])
    base = synth.baseline_uvw(cfg, rng)
    C = len(cfg.freqs_hz)
    uvw = np.concatenate([base] * C, axis=0)
    off = np.arange(C + 1, dtype=np.int64) * base.shape[0]
    w = np.full(uvw.shape[0], np.float32(1.0 / cfg.sigma_jy ** 2), dtype=np.float32)
    freqs = np.array(cfg.freqs_hz, dtype=np.float32)
    return uvw, w, freqs, off


def run_case(name, reps):
    """Small fixed workloads for profiling one kernel (used by the commands
    recorded in profiles/): `dchi2_2048_1ch` (configuration 1 reduced to one
    channel at 230 GHz, natural weights, 16 s integrations), `cfg0`, and
    `weighting` (Uniform and Briggs weighting of configuration 1's 35.28M
    visibilities on a 2048^2 grid), `gridding` (the same visibilities
    gridded with the PillBox2D and 7 x 7 PSWF kernels), `objective_cfg1`
    (two objective evaluations of configuration 1),
    `objective_lbfgs_cfg1` (the same, then two L-BFGS iterations) and
    `objective_2048_4ch` (two objective evaluations of configuration 1
    reduced to four channels)."""
    import dataclasses
    import torch
    import gpuvmem_gb300 as gv
    if name == "weighting":
        cfg = synth.CONFIG1
        uvw, w, freqs, off = weighting_inputs(cfg)
        dx = -cfg.cell_arcsec / 3600.0
        out = {}
        for scheme, robust in (("uniform", 0.0), ("briggs", 0.0)):
            gv.apply_weighting(scheme, robust, cfg.n, cfg.n, dx, -dx, freqs, off, uvw, w)
            t = []
            for _ in range(max(1, reps)):
                t0 = time.perf_counter()
                gv.apply_weighting(scheme, robust, cfg.n, cfg.n, dx, -dx, freqs, off, uvw, w)
                t.append(time.perf_counter() - t0)
            out[scheme] = 1e3 * min(t)
        print(json.dumps({"case": name, "visibilities": int(off[-1]), "grid": cfg.n,
                          "ms_including_host_copies": out}))
        return
    if name == "gridding":
        cfg = synth.CONFIG1
        uvw, w, freqs, off = weighting_inputs(cfg)
        rng = np.random.default_rng([cfg.seed, 2])
        vo = rng.normal(0.0, 1.0, (uvw.shape[0], 2)).astype(np.float32)
        dx = -cfg.cell_arcsec / 3600.0
        out = {}
        for kind in ("PillBox2D", "PSWF"):
            table, sup, _ = gv.ckernel_build(kind, cfg.n, cfg.n, dx, -dx)
            res = gv.grid_visibilities(table, sup, cfg.n, cfg.n, dx, -dx, freqs, off, uvw, vo, w)
            t = []
            for _ in range(max(1, reps)):
                t0 = time.perf_counter()
                gv.grid_visibilities(table, sup, cfg.n, cfg.n, dx, -dx, freqs, off, uvw, vo, w)
                t.append(time.perf_counter() - t0)
            out[kind] = {"ms_including_host_copies": 1e3 * min(t), "taps": int(table.size),
                         "gridded_visibilities": int(res[0][-1])}
        print(json.dumps({"case": name, "visibilities": int(off[-1]), "grid": cfg.n,
                          "channels": len(freqs), "kernels": out}))
        return
    if name in ("objective_cfg1", "objective_lbfgs_cfg1", "objective_2048_4ch"):
        # configuration 1 with chi2 + entropy + TSV: two objective evaluations
        # (priors on), then (second case) two L-BFGS iterations; the third
        # case is configuration 1 reduced to four channels at natural weights
        # and 16 s integrations (4.41M visibilities, grids of 134 MB: above
        # the L2), for single-kernel profiles
        cfg = synth.CONFIG1
        if name == "objective_2048_4ch":
            cfg = dataclasses.replace(cfg, freqs_hz=list(np.linspace(225e9, 235e9, 4)),
                                      weighting="natural", dt_s=16.0)
        data = synth.generate(cfg, device="cuda")
        prob = gv.Problem(data, [gv.term("Chi2", 1.0), gv.term("Entropy", 0.01),
                                 gv.term("TotalSquaredVariation", 1e-4)])
        img = prob.initial_image()
        prob.set_iteration(1)
        for _ in range(2):
            prob.objective(img)
        rep = None
        if name == "objective_lbfgs_cfg1":
            prob.set_iteration(0)
            rep = prob.optimize(img, "CG-LBFGS", iterations=2)
        torch.cuda.synchronize()
        print(json.dumps({"case": name, "visibilities": int(data.nvis),
                          "lbfgs_objective_evaluations": None if rep is None else int(rep.n_objective)}))
        return
    if name == "dchi2_2048_1ch":
        cfg = dataclasses.replace(synth.CONFIG1, freqs_hz=[230e9], weighting="natural", dt_s=16.0)
    elif name == "cfg0":
        cfg = synth.CONFIG0
    else:
        raise SystemExit(f"unknown case {name}")
    data = synth.generate(cfg, device="cuda")
    prob = gv.Problem(data, [gv.term("Chi2", 1.0), gv.term("Entropy", 0.01)])
    img = prob.initial_image()
    prob.chi2(img)
    xi = torch.zeros_like(img)
    for _ in range(reps):
        prob.objective(img)
        prob.dchi2(img, out=xi)
    torch.cuda.synchronize()
    print(json.dumps({"case": name, "visibilities": int(data.nvis), "reps": reps,
                      "engine": prob.info.dchi2_engine}))


def main():
    args = parse()
    if args.case:
        run_case(args.case, args.steps)
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.config == 3:
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
