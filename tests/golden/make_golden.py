"""Generates the golden fixtures of tests/golden/ from the reference's own
kernels.

Runs on a GPU: the reference harness (oracle/refrun.py) executes the
reference's CUDA kernels, compiled from the reference sources into
oracle/_ref/ref_kernels.cubin, with the reference's launch sequence
(MFS::setDevice, chi2(), dchi2(), the prior kernels and deviceReduce).
Each fixture stores the inputs (so the CPU tests need no generator) and the
reference's outputs.  Usage: python tests/golden/make_golden.py [outdir]
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refrun  # noqa: E402
from gpuvmem_gb300 import synth  # noqa: E402

CASES = {
    "ref_small64_2ch": dict(cfg=synth.small_config(n=64, nchan=2, seed=3)),
    "ref_small128_1ch": dict(cfg=synth.small_config(n=128, n_ant=10, n_times=60, nchan=1, seed=5)),
    "ref_briggs64_3ch": dict(cfg=synth.small_config(n=64, nchan=3, seed=11, weighting="briggs")),
}
PRIORS = [(1, 0.01, 0.001, -1.0, 0.0), (2, 1e-4, 0.0, 0.0, 0.0), (3, 1e-4, 0.0, 0.0, 1e-12),
          (4, 1e-3, 0.0, 0.0, 1e-12), (5, 1e-5, 0.0, 0.0, 0.0)]


def rand_image(minpix, shape, seed, alpha=False):
    rng = np.random.default_rng(seed)
    img = np.zeros((2,) + shape, dtype=np.float32)
    img[0] = minpix
    img[0] += ((rng.uniform(0, 1, shape) < 0.2) * np.abs(rng.normal(0, 2000.0, shape))).astype(np.float32)
    if alpha:
        img[1] = rng.uniform(-1, 3, shape).astype(np.float32)
    return img


def make(name, cfg, outdir=HERE):
    d = synth.generate(cfg)
    r = refrun.RefHarness(d)
    out = dict(M=d.M, N=d.N, DELTAX=d.DELTAX, DELTAY=d.DELTAY, xobs=d.xobs, yobs=d.yobs,
               nu_0=d.nu_0, antenna_diameter=d.antenna_diameter, pb_factor=d.pb_factor,
               pb_cutoff=d.pb_cutoff, primary_beam=d.primary_beam, freqs=d.freqs,
               chan_off=d.chan_off, uvw_m=d.uvw_m, vo=d.vo, weight=d.weight,
               fg_scale=r.fg_scale, noise_cut=r.noise_cut, noise=r.noise)
    img0 = r.initial_image()
    out["chi2_init"], _ = r.chi2(img0)
    img = rand_image(r.minpix, (d.N, d.M), 7)
    out["img_rand"] = img
    out["chi2_rand"], out["img_rand_clipped"] = r.chi2(img)
    out["res_rand"] = r.residuals()
    out["dchi2_rand"] = r.dchi2(out["img_rand_clipped"])
    imga = rand_image(r.minpix, (d.N, d.M), 13, alpha=True)
    out["img_alpha"] = imga
    out["chi2_alpha"], out["img_alpha_clipped"] = r.chi2(imga, flag_opt=1)
    out["dchi2_alpha"] = r.dchi2(out["img_alpha_clipped"], flag_opt=1)
    for kind, lam, G, eta, eps in PRIORS:
        v, g = r.prior(kind, lam, out["img_rand_clipped"], G=G, eta=eta, eps=eps)
        out[f"prior{kind}_value"] = v
        out[f"prior{kind}_grad"] = g
    r.close()
    path = os.path.join(outdir, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    outdir = sys.argv[1] if len(sys.argv) > 1 else HERE
    os.makedirs(outdir, exist_ok=True)
    for n, c in CASES.items():
        make(n, c["cfg"], outdir)
