"""Learned warm start for the imaging objective path (no counterpart in the
reference).

  1. Training pairs: seeded skies observed with a fixed array (configuration
     0's array, beam and noise; 5-50 sources per sky), each solved to
     convergence by the plain solver (frprmn).  Stored: the network input
     (dirty image and PSF), the converged image, the converged objective.
  2. Network: gv_unet (5 levels, 16-256 channels, BF16 tensor-core
     convolutions), trained with Adam on the mean squared error with a
     cosine learning-rate decay.
  3. Policy: the network's image, floored at the positivity floor, is
     scaled about the floor by the best of a few factors, scored by the
     solver's own objective with the priors active, and compared with the
     plain start; the better of the two is the start.  The plain solver then
     always iterates from it to convergence.
  4. Evaluation: on held-out skies, the wall time until the objective is
     within `rel` of the plain solver's converged value, warm vs plain.

Scaling of the data: the dirty image and PSF are divided by sum(w) (the PSF
peak), the dirty image further by its own peak d; the target is the
converged plane-0 image times fg_scale / d, so the map is linear in flux.
"""

from __future__ import annotations

import argparse
import dataclasses
import json
import os
import time
from typing import List, Optional, Sequence

import numpy as np

from . import Problem, synth, term
from .unet import UNet

CONFIG4 = dataclasses.replace(synth.CONFIG0, name="learned-256", array_seed=synth.CONFIG0.seed)
# the trained network shipped with the package (written by `main --save`)
NETWORK_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                            "warmstart_unet.npz")
TERMS = (("Chi2", 1.0), ("Entropy", 0.01))


def sky_config(seed: int, base: synth.SynthConfig = CONFIG4, n_min=5, n_max=50):
    rng = np.random.default_rng([seed, 11])
    return dataclasses.replace(base, seed=int(seed), n_sources=int(rng.integers(n_min, n_max + 1)))


@dataclasses.dataclass
class Sky:
    seed: int
    prob: Problem
    x: object          # torch [2, H, W]: dirty / (sum w * d), PSF / sum w
    scale: float       # d
    fg_scale: float
    floor: float       # positivity floor of plane 0


def load_sky(seed: int, base: synth.SynthConfig = CONFIG4, device="cuda") -> Sky:
    import torch
    data = synth.generate(sky_config(seed, base), device=device)
    prob = Problem(data, [term(k, lam) for k, lam in TERMS])
    dirty = prob.dirty_image()
    psf = prob.psf_image()
    s = float(psf.max())
    dn = dirty / s
    d = float(dn.abs().max()) or 1.0
    x = torch.stack([dn / d, psf / s]).contiguous()
    info = prob.info
    return Sky(seed, prob, x, d, float(info.fg_scale), float(info.minpix))


# restarts of frprmn after a stall (see solve)
RESTARTS = 3


def solve(sky: Sky, img, iterations: int, ftol=1e-12, f_target=-np.inf,
          priors_from_start=False, restarts=RESTARTS):
    """frprmn from img (in place) to convergence, as the solver of both the
    plain and the warm runs.  frprmn ends on ftol when a line search finds
    no decrease at all; with an inexact float line search and the
    positivity floor a conjugate direction can lose descent that way well
    above the optimum.  After such a stop the solver is restarted from where
    it stopped (steepest descent, the priors active), at most `restarts`
    times; a restart that cannot move ends it.  Stops early once
    f <= f_target.  Returns (report of the last leg, iterations in all,
    restarts used)."""
    total, k, rep = 0, 0, None
    while True:
        sky.prob.set_iteration(1 if (priors_from_start or k > 0) else 0)
        rep = sky.prob.optimize_until(img, f_target, "CG-FRPRMN", iterations=iterations - total,
                                      ftol=ftol, priors_from_start=priors_from_start or k > 0)
        total += rep.iterations
        if rep.exit_reason != 1 or total >= iterations or k >= restarts:
            break
        if k > 0 and rep.iterations <= 1:
            break
        k += 1
    return rep, total, k


def plain_solve(sky: Sky, iterations: int, ftol: float):
    img = sky.prob.initial_image()
    rep, _, _ = solve(sky, img, iterations, ftol=ftol)
    return img, rep


def network_target(sky: Sky, img):
    return (img[0] * (sky.fg_scale / sky.scale)).contiguous()


def make_pairs(seeds: Sequence[int], iterations=150, ftol=1e-9, base=CONFIG4, log=None):
    """(X [n,2,H,W], Y [n,1,H,W], converged objective values)."""
    import torch
    X, Y, F = [], [], []
    t0 = time.time()
    for i, s in enumerate(seeds):
        sky = load_sky(s, base)
        img, rep = plain_solve(sky, iterations, ftol)
        X.append(sky.x)
        Y.append(network_target(sky, img))
        F.append(rep.f_final)
        del sky
        if log and (i + 1) % 32 == 0:
            log(f"pairs {i + 1}/{len(seeds)} ({time.time() - t0:.1f} s)")
    return torch.stack(X), torch.stack(Y)[:, None].contiguous(), np.array(F)


def train(X, Y, epochs=80, batch=8, lr=1e-3, lr_min=1e-5, base_channels=16, levels=5, seed=0,
          log=None):
    """Adam on the mean squared error with a cosine learning-rate decay from
    lr to lr_min; returns (net, per-epoch mean loss)."""
    n, _, H, _ = X.shape
    net = UNet(H, in_channels=X.shape[1], base_channels=base_channels, levels=levels,
               max_batch=batch, seed=seed)
    rng = np.random.default_rng(seed)
    hist = []
    steps = max(1, epochs * (n // batch))
    k = 0
    for ep in range(epochs):
        perm = rng.permutation(n)
        tot, cnt = 0.0, 0
        for a in range(0, n - batch + 1, batch):
            idx = perm[a:a + batch].tolist()
            lr_k = lr_min + 0.5 * (lr - lr_min) * (1.0 + np.cos(np.pi * k / steps))
            tot += net.train_step(X[idx], Y[idx], lr_k)
            cnt += 1
            k += 1
        hist.append(tot / max(1, cnt))
        if log:
            log(f"epoch {ep + 1}/{epochs} loss {hist[-1]:.4e}")
    return net, hist


def param_layout(in_channels: int, base_channels: int, levels: int):
    """gv_unet's parameter vector, layer by layer: (weight offset, weight
    count, bias offset, bias count).  Encoder: two 3x3 convolutions per
    level (channels base * 2^l); decoder: two 3x3 convolutions per level on
    the upsampled deeper level concatenated with the skip connection; a
    final 1x1 convolution to one channel.  Each layer stores its weights
    [out][in][ky][kx], then its biases."""
    ch = [base_channels << l for l in range(levels)]
    layers = []
    for l in range(levels):
        layers.append((in_channels if l == 0 else ch[l - 1], ch[l], 3))
        layers.append((ch[l], ch[l], 3))
    for l in range(levels - 2, -1, -1):
        layers.append((ch[l + 1] + ch[l], ch[l], 3))
        layers.append((ch[l], ch[l], 3))
    layers.append((ch[0], 1, 1))
    out, off = [], 0
    for ci, co, ks in layers:
        nw = co * ci * ks * ks
        out.append((off, nw, off + nw, co))
        off += nw + co
    return out, off


def _bf16_bits(x):
    """float32 -> bfloat16 bit patterns, round to nearest even (the rounding
    the convolution kernels apply to their operands)."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return b.astype(np.uint16)


def save_network(net: UNet, path: str, meta: dict):
    """Writes the network's parameters: convolution weights as bfloat16 (the
    kernels round weights to BF16 before every product, so nothing is lost
    for the forward pass), biases as float32, and `meta` (shape and training
    record) as JSON."""
    lay, n = param_layout(net.desc.in_channels, net.desc.base_channels, net.desc.levels)
    assert n == net.nparams, (n, net.nparams)
    theta = net.params().cpu().numpy()
    w = np.concatenate([theta[o:o + k] for o, k, _, _ in lay])
    b = np.concatenate([theta[o:o + k] for _, _, o, k in lay])
    m = dict(meta, height=net.H, in_channels=net.desc.in_channels,
             base_channels=net.desc.base_channels, levels=net.desc.levels)
    np.savez_compressed(path, weights_bf16=_bf16_bits(w), biases=b.astype(np.float32),
                        meta=np.frombuffer(json.dumps(m).encode(), dtype=np.uint8))


def load_network(path: str, max_batch: int = 1):
    """(UNet with the saved parameters, meta dict)."""
    import torch
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    net = UNet(meta["height"], in_channels=meta["in_channels"],
               base_channels=meta["base_channels"], levels=meta["levels"], max_batch=max_batch,
               seed=0)
    lay, n = param_layout(meta["in_channels"], meta["base_channels"], meta["levels"])
    assert n == net.nparams, (n, net.nparams)
    w = (z["weights_bf16"].astype(np.uint32) << 16).view(np.float32)
    b = z["biases"].astype(np.float32)
    theta = np.empty(n, np.float32)
    wi = bi = 0
    for wo, wk, bo, bk in lay:
        theta[wo:wo + wk] = w[wi:wi + wk]
        theta[bo:bo + bk] = b[bi:bi + bk]
        wi += wk
        bi += bk
    net.set_params(torch.from_numpy(theta).cuda())
    return net, meta


def warm_image(sky: Sky, net: UNet):
    import torch
    pred = net.forward(sky.x[None])[0, 0]
    img = sky.prob.initial_image()
    img[0] = torch.clamp(pred * (sky.scale / sky.fg_scale), min=sky.floor)
    return img


SCALES = (0.7, 0.85, 1.0, 1.15)
CUTS = (0.0, 1e-3, 1e-2)


def choose_start(sky: Sky, net: UNet, scales=SCALES, cuts=CUTS):
    """The warm image, scaled about the positivity floor and with the
    pixels below a fraction of its peak set to the floor (the factor and the
    fraction the objective prefers), if the objective, priors active, scores
    it at least as well as the plain start; else the plain start."""
    import torch
    warm = warm_image(sky, net)
    plain = sky.prob.initial_image()
    sky.prob.set_iteration(1)
    ex = warm[0] - sky.floor
    # every (cut, scale) candidate in one tensor, cut-major
    cut_t = torch.tensor(cuts, dtype=ex.dtype, device=ex.device).view(-1, 1, 1)
    kept = ex[None] * (ex[None] > cut_t * ex.max())                    # [cuts, H, W]
    sc = torch.tensor(scales, dtype=ex.dtype, device=ex.device).view(1, -1, 1, 1)
    cands = warm[None, None].repeat(len(cuts), len(scales), 1, 1, 1)    # [cuts, scales, 2, H, W]
    cands[:, :, 0] = sky.floor + sc * kept[:, None]
    flat = cands.view(-1, *warm.shape)
    # the candidates and the plain start scored with one synchronisation
    # (each evaluated in the problem's scratch image, so none is clipped)
    scores = sky.prob.objective_many(list(flat) + [plain])
    fs, fp = scores[:-1], scores[-1]
    i_best = min(range(len(fs)), key=lambda i: (fs[i] if fs[i] == fs[i] else float("inf"), i))
    best, fw = flat[i_best].clone(), fs[i_best]
    sky.prob.set_iteration(0)
    return (best, "warm", fw, fp) if fw <= fp else (plain, "plain", fw, fp)


def time_to_target(sky: Sky, start, f_target: float, max_iter: int, priors_from_start=False):
    """Wall time of solve() from `start` until f <= f_target; returns (time,
    report with .iterations the total over restarts, reached, restarts)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rep, total, k = solve(sky, start, max_iter, f_target=f_target,
                          priors_from_start=priors_from_start)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    rep.iterations = total
    return t, rep, bool(rep.exit_reason == 4 or rep.f_final <= f_target), k


def evaluate(net: UNet, seeds: Sequence[int], iterations=300, ftol=1e-9, rel=1e-4,
             base=CONFIG4, log=None) -> List[dict]:
    import torch
    rows = []
    # first calls of the network's and the policy's kernels (module loading)
    # outside the timing
    warm_sky = load_sky(int(seeds[0]) + 7777777, base)
    choose_start(warm_sky, net)
    del warm_sky
    torch.cuda.synchronize()
    for s in seeds:
        sky = load_sky(s, base)
        _, rep = plain_solve(sky, iterations, ftol)
        f_star = float(rep.f_final)
        target = f_star + rel * abs(f_star)
        tp, rp, okp, kp = time_to_target(sky, sky.prob.initial_image(), target, iterations)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        start, which, fw, fpl = choose_start(sky, net)
        torch.cuda.synchronize()
        t_policy = time.perf_counter() - t0
        # the plain solver from the chosen start, in the reference's order
        # (priors off during the first line search) ...
        tw, rw, okw, kw = time_to_target(sky, start.clone(), target, iterations)
        # ... and, for comparison, with the priors counting from the start
        tw1, rw1, okw1, _ = time_to_target(sky, start.clone(), target, iterations,
                                           priors_from_start=True)
        row = dict(seed=int(s), f_plain_converged=f_star, plain_iterations=int(rep.iterations),
                   t_plain=tp, it_plain=int(rp.iterations), reached_plain=okp,
                   t_warm=t_policy + tw, t_policy=t_policy, it_warm=int(rw.iterations),
                   reached_warm=okw, start=which, f_start_warm=float(fw),
                   f_start_plain=float(fpl), f_warm_final=float(rw.f_final),
                   t_warm_priors_first=t_policy + tw1, it_warm_priors_first=int(rw1.iterations),
                   reached_warm_priors_first=okw1, restarts_plain=kp, restarts_warm=kw,
                   exit_plain=int(rp.exit_reason), exit_warm=int(rw.exit_reason))
        rows.append(row)
        if log:
            log(json.dumps(row))
        del sky
    return rows


def summarize(rows: List[dict]) -> dict:
    ok = [r for r in rows if r["reached_plain"] and r["reached_warm"]]
    tp = np.array([r["t_plain"] for r in ok])
    tw = np.array([r["t_warm"] for r in ok])
    ok1 = [r for r in rows if r["reached_plain"] and r.get("reached_warm_priors_first")]
    sp1 = [r["t_plain"] / r["t_warm_priors_first"] for r in ok1]
    tp1 = sum(r["t_plain"] for r in ok1)
    tw1 = sum(r["t_warm_priors_first"] for r in ok1)
    return {"skies": len(rows), "both_reached": len(ok),
            "speedup_median_priors_first": float(np.median(sp1)) if ok1 else None,
            "speedup_total_priors_first": float(tp1 / tw1) if ok1 else None,
            "both_reached_priors_first": len(ok1),
            "warm_chosen": sum(r["start"] == "warm" for r in rows),
            "t_plain_median_s": float(np.median(tp)) if ok else None,
            "t_warm_median_s": float(np.median(tw)) if ok else None,
            "speedup_median": float(np.median(tp / tw)) if ok else None,
            "speedup_total": float(tp.sum() / tw.sum()) if ok else None,
            "it_plain_median": float(np.median([r["it_plain"] for r in ok])) if ok else None,
            "it_warm_median": float(np.median([r["it_warm"] for r in ok])) if ok else None}


def main(argv: Optional[Sequence[str]] = None):
    """Trains and evaluates the warm start.  The network shipped in
    gpuvmem_gb300/data/warmstart_unet.npz was made by

        python -m gpuvmem_gb300.warmstart --train 2000 --eval 200 --epochs 80 \
            --shapes 5x16 --pair-iterations 300 \
            --save unet_{shape}_p300e80.npz --out ws_p300e80.json

    (pairs from the plain solver on seeds 1000-2999, each solved for up to
    300 iterations as the evaluation's plain runs are; the held-out skies
    are seeds 900000-900199).  The 5-level shape was chosen over the planned
    4 x 32 by an earlier run of both shapes on the same pairs
    (`--shapes 4x32,5x16`), which kept the larger summed-time speed-up."""
    ap = argparse.ArgumentParser(description="train and evaluate the learned warm start")
    ap.add_argument("--train", type=int, default=512)
    ap.add_argument("--eval", type=int, default=32)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-min", type=float, default=1e-5)
    ap.add_argument("--levels", type=int, default=5)
    ap.add_argument("--base-channels", type=int, default=16)
    ap.add_argument("--shapes", default=None,
                    help="comma-separated LEVELSxBASE shapes trained on the same pairs "
                         "(overrides --levels / --base-channels)")
    ap.add_argument("--pair-iterations", type=int, default=150)
    ap.add_argument("--eval-iterations", type=int, default=300)
    ap.add_argument("--out", default=None, help="write the summary JSON here")
    ap.add_argument("--save", default=None,
                    help="write the trained network here (.npz; {shape} is replaced by "
                         "LEVELSxBASE)")
    ap.add_argument("--train-seed0", type=int, default=1000)
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)  # noqa: E731
    shapes = ([tuple(int(v) for v in sh.split("x")) for sh in a.shapes.split(",")]
              if a.shapes else [(a.levels, a.base_channels)])
    t0 = time.time()
    X, Y, _ = make_pairs(range(a.train_seed0, a.train_seed0 + a.train), a.pair_iterations,
                         log=log)
    t_pairs = time.time() - t0
    log(f"targets: mean {float(Y.mean()):.3e} max {float(Y.max()):.3e} "
        f"mean square {float((Y * Y).mean()):.3e}")
    Xv, Yv, _ = make_pairs(range(900000, 900000 + min(a.eval, 16)), a.pair_iterations)
    results = {}
    for levels, base in shapes:
        tag = f"{levels}x{base}"
        t1 = time.time()
        net, hist = train(X, Y, a.epochs, a.batch, a.lr, a.lr_min, base, levels, log=log)
        t_train = time.time() - t1
        val = float(np.mean([((net.forward(Xv[i:i + 1]) - Yv[i:i + 1]) ** 2).mean().item()
                             for i in range(Xv.shape[0])]))
        log(f"{tag}: held-out mse {val:.4e} (target mean square {float((Yv * Yv).mean()):.4e})")
        if a.save:
            save_network(net, a.save.replace("{shape}", tag),
                         {"train_skies": a.train, "train_seed0": a.train_seed0,
                          "epochs": a.epochs, "batch": a.batch, "lr": a.lr, "lr_min": a.lr_min,
                          "pair_iterations": a.pair_iterations, "final_train_loss": hist[-1],
                          "heldout_mse": val})
        rows = evaluate(net, range(900000, 900000 + a.eval), a.eval_iterations, log=log)
        summ = summarize(rows)
        summ.update({"train_skies": a.train, "epochs": a.epochs, "levels": levels,
                     "base_channels": base, "final_train_loss": hist[-1], "heldout_mse": val,
                     "pair_generation_s": t_pairs, "training_s": t_train})
        print(json.dumps(summ), flush=True)
        results[tag] = {"summary": summ, "rows": rows, "loss_history": hist}
        del net
    if a.out:
        with open(a.out, "w") as f:
            json.dump(results, f, indent=1)
    return results


if __name__ == "__main__":
    main()
