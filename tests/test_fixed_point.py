"""fixedPointOpt (src/fixedpoint.cu:32-57) in the Python and C++ mirrors:
a contraction toward 0.2 per entry, with the reference's iteration order (x0
advances only from the third call) checked step by step."""

import numpy as np

import gpuvmem_gb300 as gv


def test_fixed_point_contraction_and_call_order():
    calls = []

    def optf(x):
        calls.append(list(x))
        return [0.5 * v + 0.1 for v in x]

    out = gv.fixed_point_opt([0.9, 0.9, 0.6], optf, 1e-3, 50)
    # the first two calls see the start point; later ones the previous result
    assert calls[0] == calls[1] == [0.9, 0.9, 0.6]
    assert calls[2] == out if len(calls) == 3 else calls[2] != calls[0]
    np.testing.assert_allclose(out[1:], [0.2, 0.2], atol=2e-3)


def test_fixed_point_stops_at_one_and_limit():
    n = []
    out = gv.fixed_point_opt([0.1, 0.3], lambda x: (n.append(1), [x[0], 2.0 * x[1]])[1], 1e-9, 10)
    # 0.3 -> 0.6, again 0.3 -> 0.6 (x0 not yet advanced), then 0.6 -> 1.2: stop
    assert len(n) == 3 and abs(out[1] - 1.2) < 1e-6
    m = []
    gv.fixed_point_opt([0.1, 0.5], lambda x: (m.append(1), [x[0], 0.5 * x[1]])[1], 0.0, 4)
    assert len(m) == 4
