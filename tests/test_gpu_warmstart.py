"""Learned warm start end to end on a small geometry (64 x 64, a fixed
10-antenna array): training pairs from the plain solver, a short training
run of the network, the policy, and what the trained network gains over the
plain start on held-out skies."""

import dataclasses

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu


def test_warm_start_gains_over_plain_start():
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
    # and the solver, with the priors counting from its first line search,
    # needs fewer iterations from it to the plain solver's converged objective
    # (in the reference's order -- priors off for the first line search --
    # that first search fits chi2 alone and walks away from the regularised
    # start; on this 64^2 geometry that variant is decided by rounding)
    both = [r for r in rows if r["reached_plain"] and r["reached_warm_priors_first"]]
    assert len(both) >= 4, info
    assert (np.median([r["it_warm_priors_first"] for r in both])
            < np.median([r["it_plain"] for r in both])), info
