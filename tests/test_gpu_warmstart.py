"""Learned warm start end to end: the training pipeline on a small geometry
(64 x 64, a fixed 10-antenna array: pairs from the plain solver, a short
training run, the policy), and what the network shipped with the package
gains over the plain start on held-out skies of its own 256 x 256
geometry."""

import dataclasses

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu


def test_warm_start_pipeline_64():
    """Training pairs from the plain solver, a short training run of the
    network and the start policy on a 64 x 64 geometry."""
    from gpuvmem_gb300 import warmstart as W
    base = dataclasses.replace(synth.small_config(n=64, n_ant=10, n_times=48, seed=0),
                               name="learned-64", array_seed=0, n_sources=6)
    X, Y, F = W.make_pairs(range(100, 228), iterations=80, base=base)
    assert X.shape == (128, 2, 64, 64) and Y.shape == (128, 1, 64, 64) and np.all(np.isfinite(F))
    net, hist = W.train(X, Y, epochs=40, batch=8, base_channels=16, levels=4, seed=1)
    assert hist[-1] < 0.2 * hist[0]
    rows = W.evaluate(net, range(5000, 5008), iterations=200, base=base)
    info = [(r["start"], r["f_start_warm"], r["f_start_plain"], r["it_plain"], r["it_warm"],
             r["reached_plain"], r["reached_warm"]) for r in rows]
    warm = [r for r in rows if r["start"] == "warm"]
    # the policy never starts from something the objective scores worse
    assert all(r["f_start_warm"] <= r["f_start_plain"] or r["start"] == "plain" for r in rows)
    # the trained network's start is far better than the plain start
    assert len(warm) >= 6, info
    assert np.median([r["f_start_warm"] / r["f_start_plain"] for r in rows]) < 0.5, info


def test_shipped_network_gains_over_plain_start():
    """What the trained network shipped with the package gains on its own
    geometry (the 256^2 configuration-0 array), on 8 of the held-out skies
    the bench's converge key uses: fewer iterations and less wall time to
    f* (1 + 1e-4) of the plain solver's converged objective, in the
    reference's order (priors off for the first line search)."""
    import os
    from gpuvmem_gb300 import warmstart as W
    if not os.path.exists(W.NETWORK_PATH):
        pytest.fail(f"no trained network at {W.NETWORK_PATH}")
    net, _ = W.load_network(W.NETWORK_PATH)
    rows = W.evaluate(net, range(900000, 900008), iterations=300)
    both = [r for r in rows if r["reached_plain"] and r["reached_warm"]]
    info = [(r["start"], r["it_plain"], r["it_warm"], round(r["t_plain"], 4), round(r["t_warm"], 4))
            for r in rows]
    assert len(both) >= 6, info
    assert all(r["start"] == "warm" for r in rows), info
    assert np.median([r["it_warm"] for r in both]) < 0.5 * np.median([r["it_plain"] for r in both]), info
    assert np.median([r["t_plain"] / r["t_warm"] for r in both]) > 1.5, info
