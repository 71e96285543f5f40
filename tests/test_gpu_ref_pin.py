"""The CUDA path against the reference's own kernels run live on the GPU
(reference harness), on the same seeded inputs: the parity gates proper,
with each side's error against the FP64 oracle."""

import numpy as np
import pytest

import oracle as O
import refrun
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0), (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0)]


def rand_image(minpix, shape, seed):
    rng = np.random.default_rng(seed)
    img = np.zeros((2,) + shape, dtype=np.float32)
    img[0] = minpix
    img[0] += ((rng.uniform(0, 1, shape) < 0.2) * np.abs(rng.normal(0, 2000.0, shape))).astype(np.float32)
    return img


@pytest.mark.skipif(not refrun.available(), reason="reference kernels cubin not built")
@pytest.mark.parametrize("n,nchan,engine", [(64, 2, 1), (128, 1, 2), (256, 2, 2)])
def test_ours_vs_reference_kernels(n, nchan, engine):
    import torch
    import gpuvmem_gb300 as gv
    cfg = synth.small_config(n=n, n_ant=10, n_times=48, nchan=nchan, seed=21 + n)
    d = synth.generate(cfg)
    ref = refrun.RefHarness(d)
    orc = O.Oracle(d, TERMS)
    prob = gv.Problem(d, TERMS, engine=engine)
    assert abs(prob.info.fg_scale - ref.fg_scale) <= 2e-6 * ref.fg_scale
    img = rand_image(ref.minpix, (n, n), 3)
    c_ref, img_ref = ref.chi2(img)
    c_orc, img_orc = orc.chi2(img.copy())
    t = torch.from_numpy(img.copy()).cuda()
    c_ours = prob.chi2(t)
    np.testing.assert_array_equal(t.cpu().numpy(), img_ref)
    assert abs(c_ours - c_ref) <= 1e-5 * abs(c_ref), (c_ours, c_ref)
    g_ref = ref.dchi2(img_ref)
    g_orc = orc.dchi2(img_orc)
    g_ours = prob.dchi2(t).cpu().numpy()
    scale = np.abs(g_ref[0]).max()
    err = np.abs(g_ours - g_ref).max() / scale
    err_ref_oracle = np.abs(g_ref - g_orc).max() / scale
    err_ours_oracle = np.abs(g_ours - g_orc).max() / scale
    print(f"n={n}: chi2 rel ours-ref {abs(c_ours-c_ref)/c_ref:.2e}, ref-oracle "
          f"{abs(c_ref-c_orc)/c_orc:.2e}; grad ours-ref {err:.2e}, ref-oracle {err_ref_oracle:.2e}, "
          f"ours-oracle {err_ours_oracle:.2e}")
    assert err <= 1e-5
    ref.close()
