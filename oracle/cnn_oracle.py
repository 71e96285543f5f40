"""FP64 CPU oracle of the warm-start network (test infrastructure only).

Restates, in numpy, the convolution passes and the U-Net of
gpuvmem_gb300/csrc/cnn.cu: every GEMM operand is rounded to BF16 (round to
nearest even) exactly where the GPU rounds it when it stages a tile, and the
products are summed in FP64.  Biases, pooling, upsampling, ReLU masks, the
loss and the bias gradients are FP64 on FP32 inputs.  The network has no
counterpart in the reference; the oracle pins the GPU kernels.
"""

from __future__ import annotations

import numpy as np


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(x, dy, dx):
    """x[..., y + dy, x + dx] with zeros outside."""
    B, C, H, W = x.shape
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ys < ye and xs < xe:
        out[:, :, ys:ye, xs:xe] = x[:, :, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv_forward(x, w, b, ks, relu):
    """y = act(sum_taps W x(shifted) + b); x (B,Cin,H,W), w (Cout,Cin,ks,ks)."""
    xr, wr = bf16(x), bf16(w)
    p = ks // 2
    y = np.zeros((x.shape[0], w.shape[0]) + x.shape[2:])
    for ky in range(ks):
        for kx in range(ks):
            xs = _shift(xr, ky - p, kx - p)
            y += np.einsum("bchw,oc->bohw", xs, wr[:, :, ky, kx])
    y += np.asarray(b, np.float64)[None, :, None, None]
    return np.maximum(y, 0.0) if relu else y


def conv_backward(x, w, dz, ks):
    """dx, dw, db of conv_forward (dz is the gradient at the pre-activation)."""
    xr, wr, zr = bf16(x), bf16(w), bf16(dz)
    p = ks // 2
    dx = np.zeros(x.shape)
    dw = np.zeros(w.shape)
    for ky in range(ks):
        for kx in range(ks):
            # forward used x[y + ky - p, x + kx - p]
            dx += np.einsum("bohw,oc->bchw", _shift(zr, p - ky, p - kx), wr[:, :, ky, kx])
            dw[:, :, ky, kx] = np.einsum("bohw,bchw->oc", zr, _shift(xr, ky - p, kx - p))
    db = np.asarray(dz, np.float64).sum(axis=(0, 2, 3))
    return dx, dw, db


def pool2(x):
    B, C, H, W = x.shape
    return x.reshape(B, C, H // 2, 2, W // 2, 2).mean(axis=(3, 5))


def pool2_bwd(dy):
    return 0.25 * np.repeat(np.repeat(dy, 2, axis=2), 2, axis=3)


def up2(x):
    return np.repeat(np.repeat(x, 2, axis=2), 2, axis=3)


def up2_bwd(dy):
    B, C, H, W = dy.shape
    return dy.reshape(B, C, H // 2, 2, W // 2, 2).sum(axis=(3, 5))


class UNet:
    """Same layer order and parameter layout as gv_unet."""

    def __init__(self, height, in_channels, base_channels, levels):
        self.H, self.cin, self.c0, self.L = height, in_channels, base_channels, levels
        C = self.C
        layers = []
        for l in range(levels):
            layers.append((in_channels if l == 0 else C(l - 1), C(l), 3, True))
            layers.append((C(l), C(l), 3, True))
        for l in range(levels - 2, -1, -1):
            layers.append((C(l + 1) + C(l), C(l), 3, True))
            layers.append((C(l), C(l), 3, True))
        layers.append((C(0), 1, 1, False))
        self.layers = layers
        self.offsets = []
        off = 0
        for ci, co, ks, _ in layers:
            self.offsets.append((off, off + co * ci * ks * ks))
            off += co * ci * ks * ks + co
        self.nparams = off

    def C(self, l):
        return self.c0 << l

    def unpack(self, theta):
        out = []
        for (ci, co, ks, _), (w0, b0) in zip(self.layers, self.offsets):
            out.append((theta[w0:b0].reshape(co, ci, ks, ks), theta[b0:b0 + co]))
        return out

    def forward(self, theta, x):
        P = self.unpack(np.asarray(theta, np.float64))
        L = self.L
        cache = {"in": [None] * L, "a": [None] * L, "enc": [None] * L, "cat": [None] * L,
                 "b": [None] * L, "dec": [None] * L}
        h = np.asarray(x, np.float64)
        k = 0
        for l in range(L):
            cache["in"][l] = h
            a = conv_forward(h, *P[k], 3, True)
            e = conv_forward(a, *P[k + 1], 3, True)
            k += 2
            cache["a"][l], cache["enc"][l] = a, e
            if l + 1 < L:
                h = pool2(e)
        cache["dec"][L - 1] = cache["enc"][L - 1]
        for l in range(L - 2, -1, -1):
            cat = np.concatenate([up2(cache["dec"][l + 1]), cache["enc"][l]], axis=1)
            bb = conv_forward(cat, *P[k], 3, True)
            d = conv_forward(bb, *P[k + 1], 3, True)
            k += 2
            cache["cat"][l], cache["b"][l], cache["dec"][l] = cat, bb, d
        out = conv_forward(cache["dec"][0], *P[k], 1, False)
        return out, cache

    def loss_grad(self, theta, x, t):
        """MSE loss and its gradient with respect to theta."""
        out, c = self.forward(theta, x)
        n = out.size
        d = out - t
        loss = float((d * d).sum() / n)
        dout = 2.0 * d / n
        P = self.unpack(np.asarray(theta, np.float64))
        grads = [None] * len(P)
        L = self.L
        ko = len(P) - 1
        dx, dw, db = conv_backward(c["dec"][0], P[ko][0], dout, 1)
        grads[ko] = (dw, db)
        ddec = [None] * L
        ddec[0] = dx
        denc = [None] * L
        for l in range(0, L - 1):
            k = 2 * L + 2 * (L - 2 - l)
            g = ddec[l] * (c["dec"][l] > 0)
            dbb, dw2, db2 = conv_backward(c["b"][l], P[k + 1][0], g, 3)
            grads[k + 1] = (dw2, db2)
            g = dbb * (c["b"][l] > 0)
            dcat, dw1, db1 = conv_backward(c["cat"][l], P[k][0], g, 3)
            grads[k] = (dw1, db1)
            cu = self.C(l + 1)
            ddec[l + 1] = up2_bwd(dcat[:, :cu])
            denc[l] = dcat[:, cu:]
        denc[L - 1] = ddec[L - 1]
        din = [None] * (L + 1)
        for l in range(L - 1, -1, -1):
            k = 2 * l
            g = denc[l]
            if l + 1 < L:
                g = g + pool2_bwd(din[l + 1])
            g = g * (c["enc"][l] > 0)
            da, dw2, db2 = conv_backward(c["a"][l], P[k + 1][0], g, 3)
            grads[k + 1] = (dw2, db2)
            g = da * (c["a"][l] > 0)
            dinl, dw1, db1 = conv_backward(c["in"][l], P[k][0], g, 3)
            grads[k] = (dw1, db1)
            din[l] = dinl
        flat = np.zeros(self.nparams)
        for (w0, b0), (dw, db) in zip(self.offsets, grads):
            flat[w0:b0] = dw.ravel()
            flat[b0:b0 + db.size] = db
        return loss, flat, out
