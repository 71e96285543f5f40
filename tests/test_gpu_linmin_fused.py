"""A whole line search in one cluster launch (k_linmin_cluster: the bracket
+ Brent state machine stepped by CTA 0 after each evaluation, the grid kept
in the cluster's shared memory, the sums replaying the separate kernels'
reductions) against the CUDA-graph WHILE loop of separate launches
(GV_LS_FUSED=0) and the host search (GV_DEVICE_LS=0): iterations,
evaluation counts, the final objective and the image agree bit for bit,
with clusters of 16 and of 8 CTAs, including the plain-MEM 256^2
configuration (104,400 visibilities) solved for 100 frprmn iterations.
Problems the cluster does not take (several channels, images above 256)
fall back to the graph loop."""

import os

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

TERMS = [("Chi2", 1.0), ("Entropy", 0.01), ("TotalSquaredVariation", 1e-5)]


def _solve(mode, cfg, method, iterations, terms=TERMS):
    """mode: 'host', 'graph' (WHILE loop of separate launches), 'cluster16',
    'cluster8' (one launch, clusters of 16 / 8 CTAs)."""
    import torch
    import gpuvmem_gb300 as gv
    env = {"host": {"GV_DEVICE_LS": "0"}, "graph": {"GV_LS_FUSED": "0"},
           "cluster16": {"GV_LS_FUSED": "1", "GV_LS_CTAS": "16"},
           "cluster8": {"GV_LS_FUSED": "1", "GV_LS_CTAS": "8"}}[mode]
    os.environ.update(env)
    try:
        data = synth.generate(cfg, device="cuda")
        prob = gv.Problem(data, [gv.term(k, lam) for k, lam in terms])
    finally:
        for k in env:
            os.environ.pop(k, None)
    img = prob.initial_image()
    rep = prob.optimize(img, method, iterations=iterations)
    torch.cuda.synchronize()
    out = (rep, img.cpu().numpy())
    prob.close()
    return out


def _same(a, b):
    (ra, ia), (rb, ib) = a, b
    assert ra.iterations == rb.iterations and ra.exit_reason == rb.exit_reason
    assert ra.n_objective == rb.n_objective and ra.n_gradient == rb.n_gradient
    assert np.float32(ra.f_final).tobytes() == np.float32(rb.f_final).tobytes()
    np.testing.assert_array_equal(ia.view(np.uint32), ib.view(np.uint32))


@pytest.mark.parametrize("method,iterations,n,nchan,n_ant", [
    ("CG-FRPRMN", 15, 64, 1, 12),
    ("CG-LBFGS", 10, 64, 1, 12),
    ("CG-FRPRMN", 8, 128, 1, 12),
    ("CG-LBFGS", 6, 256, 1, 12),
    ("CG-FRPRMN", 6, 256, 1, 40),    # more visibilities than virtual threads
    ("CG-FRPRMN", 6, 64, 2, 12),     # two channels: the graph loop
    ("CG-FRPRMN", 3, 512, 1, 12),    # 512^2: the graph loop
])
def test_single_launch_line_search_matches(method, iterations, n, nchan, n_ant):
    cfg = synth.small_config(n=n, n_ant=n_ant, n_times=40 if n_ant < 40 else 400, nchan=nchan,
                             seed=70 + n + nchan + n_ant)
    ref = _solve("graph", cfg, method, iterations)
    _same(_solve("cluster16", cfg, method, iterations), ref)
    _same(_solve("cluster8", cfg, method, iterations), ref)
    _same(_solve("host", cfg, method, iterations), ref)


def test_single_launch_line_search_four_priors():
    terms = TERMS + [("L1-Norm", 1e-4), ("TotalVariation", 1e-5)]
    cfg = synth.small_config(n=128, nchan=1, seed=21)
    ref = _solve("graph", cfg, "CG-FRPRMN", 10, terms)
    _same(_solve("cluster16", cfg, "CG-FRPRMN", 10, terms), ref)
    _same(_solve("cluster8", cfg, "CG-FRPRMN", 10, terms), ref)


def test_single_launch_plain256_frprmn_trajectory():
    """The plain-MEM 256^2 configuration (chi2 + entropy 0.01), frprmn for
    100 iterations: the same trajectory bit for bit from the single-launch
    line search and from the graph loop; prints both solve times."""
    terms = [("Chi2", 1.0), ("Entropy", 0.01)]
    a = _solve("cluster16", synth.CONFIG0, "CG-FRPRMN", 100, terms)
    b = _solve("graph", synth.CONFIG0, "CG-FRPRMN", 100, terms)
    print(f"\nplain 256^2 frprmn: {a[0].iterations} iterations, {a[0].n_objective} objective "
          f"evaluations, f = {a[0].f_final!r}; single-launch line search "
          f"{a[0].seconds * 1e3:.1f} ms, graph loop {b[0].seconds * 1e3:.1f} ms")
    _same(a, b)
