"""Warm-start network kernels on the GPU against the FP64 oracle
(oracle/cnn_oracle.py): single convolution passes with BF16-exact inputs
(so only the FP32 accumulation differs), the whole U-Net's loss and
parameter gradients, and a few training steps."""

import numpy as np
import pytest

import cnn_oracle as CO

pytestmark = pytest.mark.gpu


def _bf16_exact(rng, shape, scale=1.0):
    return CO.bf16(rng.normal(0, scale, shape).astype(np.float32)).astype(np.float32)


@pytest.mark.parametrize("B,Cin,Cout,H,ks,relu", [(2, 2, 32, 16, 3, True), (1, 96, 32, 12, 3, False),
                                                  (2, 32, 1, 16, 1, False), (1, 64, 128, 8, 3, True),
                                                  (1, 256, 256, 8, 3, True), (3, 8, 64, 5, 3, False),
                                                  (1, 384, 128, 8, 3, True), (1, 24, 320, 6, 3, False)])
def test_conv_forward_and_backward_match_oracle(B, Cin, Cout, H, ks, relu):
    import torch
    from gpuvmem_gb300 import unet
    rng = np.random.default_rng(B * 1000 + Cin + Cout + H)
    x = _bf16_exact(rng, (B, Cin, H, H))
    w = _bf16_exact(rng, (Cout, Cin, ks, ks), 0.2)
    b = rng.normal(0, 0.1, Cout).astype(np.float32)
    dz = _bf16_exact(rng, (B, Cout, H, H))
    tx, tw, tb, tz = (torch.from_numpy(a).cuda() for a in (x, w, b, dz))
    y = unet.conv2d_forward(tx, tw, tb, ks, relu).cpu().numpy()
    yr = CO.conv_forward(x, w, b, ks, relu)
    assert np.abs(y - yr).max() <= 1e-5 * max(1.0, np.abs(yr).max())
    dx, dw, db = (t.cpu().numpy() for t in unet.conv2d_backward(tx, tw, tz, ks))
    dxr, dwr, dbr = CO.conv_backward(x, w, dz, ks)
    for got, ref in ((dx, dxr), (dw, dwr), (db, dbr)):
        assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def test_unet_loss_and_gradients_match_oracle():
    import torch
    from gpuvmem_gb300 import unet
    net = unet.UNet(16, in_channels=2, base_channels=8, levels=3, max_batch=2, seed=3)
    ref = CO.UNet(16, 2, 8, 3)
    assert net.nparams == ref.nparams
    rng = np.random.default_rng(1)
    x = rng.normal(0, 1, (2, 2, 16, 16)).astype(np.float32)
    t = rng.normal(0, 1, (2, 1, 16, 16)).astype(np.float32)
    theta = net.params().cpu().numpy().astype(np.float64)
    loss_ref, g_ref, out_ref = ref.loss_grad(theta, x, t)
    tx, tt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    out = net.forward(tx).cpu().numpy()
    loss = net.loss_grad(tx, tt)
    g = net.grads().cpu().numpy()
    # intermediate activations are FP32 on the GPU and FP64 in the oracle, so
    # a few BF16 roundings of operands land on the other side of a tie
    assert np.abs(out - out_ref).max() <= 1e-2 * np.abs(out_ref).max()
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert rel <= 1e-2, rel


def test_unet_training_reduces_loss():
    import torch
    from gpuvmem_gb300 import unet
    net = unet.UNet(32, in_channels=2, base_channels=8, levels=3, max_batch=4, seed=5)
    rng = np.random.default_rng(2)
    x = rng.normal(0, 1, (4, 2, 32, 32)).astype(np.float32)
    t = (0.5 * x[:, :1] - 0.25 * x[:, 1:]).astype(np.float32)  # a linear map to learn
    tx, tt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = net.train_step(tx, tt, 1e-3)
    for _ in range(60):
        last = net.train_step(tx, tt, 1e-3)
    assert last < 0.2 * first, (first, last)
