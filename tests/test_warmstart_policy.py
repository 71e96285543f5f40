"""The warm-start policy's host logic on the CPU, with a stand-in problem and
network: how the candidate starts are built from the network's image (a
scale about the positivity floor, faint pixels cut to the floor), which one
the objective picks, and the fallback to the plain start."""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gpuvmem_gb300 import warmstart as W  # noqa: E402

H = 8
FLOOR = 0.25


class FakeProblem:
    """Scores images with a given function; records what it was asked."""

    def __init__(self, score):
        self.score = score
        self.iterations = []
        self.seen = []

    def initial_image(self):
        img = torch.zeros(2, H, H)
        img[0] = FLOOR
        img[1] = 0.125  # a plane 1 the candidates must carry over unchanged
        return img

    def set_iteration(self, it):
        self.iterations.append(it)

    def objective_many(self, imgs):
        self.seen = [i.clone() for i in imgs]
        return [self.score(i) for i in imgs]


class FakeNet:
    def __init__(self, pred):
        self.pred = pred

    def forward(self, x):
        assert x.shape[0] == 1
        return self.pred[None, None].clone()


def _pred():
    rng = np.random.default_rng(3)
    p = rng.uniform(0.0, 2.0, (H, H)).astype(np.float32)
    p[0, :4] = [10.0, 0.005, 0.05, 0.3]  # a peak, and pixels around the cut levels
    return torch.from_numpy(p)


def _sky(score):
    x = torch.zeros(2, H, H)
    return W.Sky(seed=0, prob=FakeProblem(score), x=x, scale=2.0, fg_scale=4.0, floor=FLOOR)


def _expected_candidates(pred):
    warm0 = torch.clamp(pred * (2.0 / 4.0), min=FLOOR)
    ex = warm0 - FLOOR
    out = []
    for cut in W.CUTS:
        kept = ex * (ex > cut * ex.max())
        for s in W.SCALES:
            c = torch.empty(2, H, H)
            c[0] = FLOOR + s * kept
            c[1] = 0.125
            out.append(c)
    return out


def test_candidates_are_scaled_and_cut_about_the_floor():
    pred = _pred()
    sky = _sky(lambda img: float(img[0].sum()))
    W.choose_start(sky, FakeNet(pred))
    seen = sky.prob.seen
    exp = _expected_candidates(pred)
    assert len(seen) == len(W.CUTS) * len(W.SCALES) + 1  # candidates, then the plain start
    for got, want in zip(seen[:-1], exp):
        torch.testing.assert_close(got, want, rtol=0, atol=1e-6)
    torch.testing.assert_close(seen[-1], sky.prob.initial_image(), rtol=0, atol=0)
    # scored with the priors active, then the gating restored
    assert sky.prob.iterations == [1, 0]


def test_the_candidate_the_objective_prefers_is_the_start():
    pred = _pred()
    exp = _expected_candidates(pred)
    k_best = 7  # cut index 1, scale index 3 in cut-major order
    target = float(exp[k_best][0].sum())
    sky = _sky(lambda img: abs(float(img[0].sum()) - target) + (1e9 if img[1, 0, 0] != 0.125 else 0))
    # the plain start scores worse than every candidate
    start, which, fw, fp = W.choose_start(sky, FakeNet(pred))
    assert which == "warm"
    torch.testing.assert_close(start, exp[k_best], rtol=0, atol=1e-6)
    assert fw <= fp


def test_plain_start_when_it_scores_better():
    pred = _pred()
    sky = _sky(lambda img: 0.0 if float(img[0].sum()) == FLOOR * H * H else 1.0)
    start, which, fw, fp = W.choose_start(sky, FakeNet(pred))
    assert which == "plain" and fp < fw
    torch.testing.assert_close(start, sky.prob.initial_image(), rtol=0, atol=0)


def test_nan_scores_never_win():
    pred = _pred()
    exp = _expected_candidates(pred)
    calls = {"n": 0}

    def score(img):
        k = calls["n"]
        calls["n"] += 1
        if k < len(exp) - 1:
            return math.nan  # every candidate but the last fails to score
        return 5.0 if k == len(exp) - 1 else 6.0  # last candidate 5, plain start 6

    sky = _sky(score)
    start, which, fw, fp = W.choose_start(sky, FakeNet(pred))
    assert which == "warm" and fw == 5.0 and fp == 6.0
    torch.testing.assert_close(start, exp[-1], rtol=0, atol=1e-6)


def test_summary_counts_only_skies_that_reach_the_target_in_both_runs():
    rows = [
        dict(t_plain=0.06, t_warm=0.02, reached_plain=True, reached_warm=True, start="warm",
             it_plain=60, it_warm=20, t_warm_priors_first=0.015, reached_warm_priors_first=True),
        dict(t_plain=0.04, t_warm=0.01, reached_plain=True, reached_warm=True, start="warm",
             it_plain=40, it_warm=10, t_warm_priors_first=0.02, reached_warm_priors_first=True),
        dict(t_plain=0.05, t_warm=0.05, reached_plain=True, reached_warm=True, start="plain",
             it_plain=50, it_warm=50, t_warm_priors_first=0.05, reached_warm_priors_first=False),
        # the warm run did not reach the target: left out of the warm statistics
        dict(t_plain=0.30, t_warm=0.001, reached_plain=True, reached_warm=False, start="warm",
             it_plain=300, it_warm=1, t_warm_priors_first=0.001, reached_warm_priors_first=True),
    ]
    s = W.summarize(rows)
    assert s["skies"] == 4 and s["both_reached"] == 3 and s["warm_chosen"] == 3
    assert s["speedup_median"] == pytest.approx(3.0)   # ratios 3, 4, 1
    assert s["speedup_total"] == pytest.approx(0.15 / 0.08)
    assert s["t_plain_median_s"] == pytest.approx(0.05)
    assert s["it_plain_median"] == 50 and s["it_warm_median"] == 20
    # priors-first: skies 1, 2 and 4 reach it (ratios 4, 2, 300)
    assert s["speedup_median_priors_first"] == pytest.approx(4.0)
    assert s["both_reached_priors_first"] == 3
    assert s["speedup_total_priors_first"] == pytest.approx((0.06 + 0.04 + 0.30) / (0.015 + 0.02 + 0.001))
