"""Synthetic configurations: the batched and MFS workloads' generators."""

from gpuvmem_gb300 import synth


def test_config3_generator():
    cfgs, lams = synth.config3_problems(count=64)
    assert len(cfgs) == 64 and len(lams) == 64
    assert {c.n for c in cfgs} <= {128, 256, 512}
    assert all(1e-3 <= l <= 1e-1 for l in lams)
    nvis = [c.n_ant * (c.n_ant - 1) // 2 * round((c.ha_stop_h - c.ha_start_h) * 3600 / c.dt_s)
            for c in cfgs]
    assert 15e3 <= min(nvis) and max(nvis) <= 600e3


def test_config2_shape():
    c = synth.CONFIG2
    assert c.n == 1024 and len(c.freqs_hz) == 64 and c.alpha_range == (-1.0, 3.0)
    assert c.flag_fraction_range == (0.0, 0.4)
