"""Python view of the warm-start network's C ABI (gv_unet_*, gv_conv2d_*).

The network, its training step and every convolution run in the in-tree
CUDA library; torch tensors only hold the device buffers.
"""

from __future__ import annotations

import ctypes as C

from . import _ptr, check, lib


class UNetDesc(C.Structure):
    _fields_ = [("height", C.c_int32), ("width", C.c_int32), ("in_channels", C.c_int32),
                ("base_channels", C.c_int32), ("levels", C.c_int32), ("max_batch", C.c_int32),
                ("seed", C.c_uint64)]


_SIGS = None


def _lib():
    global _SIGS
    L = lib()
    if _SIGS is None:
        vp, i32, f32 = C.c_void_p, C.c_int32, C.c_float
        f64p = C.POINTER(C.c_double)
        sig = {
            "gv_unet_create": [C.POINTER(UNetDesc), C.POINTER(vp)],
            "gv_unet_destroy": [vp],
            "gv_unet_set_stream": [vp, vp],
            "gv_unet_num_params": [vp, C.POINTER(C.c_int64)],
            "gv_unet_get_params": [vp, vp],
            "gv_unet_set_params": [vp, vp],
            "gv_unet_get_grads": [vp, vp],
            "gv_unet_forward": [vp, vp, i32, vp],
            "gv_unet_loss_grad": [vp, vp, vp, i32, f64p],
            "gv_unet_train_step": [vp, vp, vp, i32, f32, f64p],
            "gv_conv2d_forward": [vp, vp, vp, vp, i32, i32, i32, i32, i32, i32, i32, vp],
            "gv_conv2d_backward": [vp, vp, vp, vp, vp, vp, i32, i32, i32, i32, i32, i32, vp],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _SIGS = sig
    return L


class UNet:
    """gv_unet: encoder-decoder CNN, BF16 tensor-core convolutions."""

    def __init__(self, height, in_channels=2, base_channels=32, levels=4, max_batch=8, seed=0):
        self.desc = UNetDesc(height, height, in_channels, base_channels, levels, max_batch, seed)
        h = C.c_void_p()
        check(_lib().gv_unet_create(C.byref(self.desc), C.byref(h)))
        self.h = h
        n = C.c_int64()
        check(_lib().gv_unet_num_params(self.h, C.byref(n)))
        self.nparams = int(n.value)
        self.H = height

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            try:
                _lib().gv_unet_destroy(h)
            except Exception:
                pass
            self.h = None

    def set_stream(self, stream):
        check(_lib().gv_unet_set_stream(self.h, C.c_void_p(stream)))

    def params(self):
        import torch
        out = torch.empty(self.nparams, dtype=torch.float32, device="cuda")
        check(_lib().gv_unet_get_params(self.h, _ptr(out)))
        return out

    def set_params(self, theta):
        check(_lib().gv_unet_set_params(self.h, _ptr(theta.contiguous())))

    def grads(self):
        import torch
        out = torch.empty(self.nparams, dtype=torch.float32, device="cuda")
        check(_lib().gv_unet_get_grads(self.h, _ptr(out)))
        return out

    def forward(self, x):
        import torch
        B = x.shape[0]
        out = torch.empty((B, 1, self.H, self.H), dtype=torch.float32, device="cuda")
        check(_lib().gv_unet_forward(self.h, _ptr(x.contiguous()), B, _ptr(out)))
        return out

    def loss_grad(self, x, t):
        loss = C.c_double()
        check(_lib().gv_unet_loss_grad(self.h, _ptr(x.contiguous()), _ptr(t.contiguous()),
                                       x.shape[0], C.byref(loss)))
        return loss.value

    def train_step(self, x, t, lr):
        loss = C.c_double()
        check(_lib().gv_unet_train_step(self.h, _ptr(x.contiguous()), _ptr(t.contiguous()),
                                        x.shape[0], float(lr), C.byref(loss)))
        return loss.value


def conv2d_forward(x, w, b, ks, relu=False):
    import torch
    B, Cin, H, W = x.shape
    Cout = w.shape[0]
    y = torch.empty((B, Cout, H, W), dtype=torch.float32, device="cuda")
    check(_lib().gv_conv2d_forward(_ptr(x.contiguous()), _ptr(w.contiguous()),
                                   _ptr(b.contiguous()), _ptr(y), B, Cin, Cout, H, W, ks,
                                   int(relu), None))
    return y


def conv2d_backward(x, w, dz, ks):
    import torch
    B, Cin, H, W = x.shape
    Cout = w.shape[0]
    dx = torch.empty_like(x)
    dw = torch.empty_like(w)
    db = torch.empty(Cout, dtype=torch.float32, device="cuda")
    check(_lib().gv_conv2d_backward(_ptr(x.contiguous()), _ptr(w.contiguous()),
                                    _ptr(dz.contiguous()), _ptr(dx), _ptr(dw), _ptr(db), B, Cin,
                                    Cout, H, W, ks, None))
    return dx, dw, db
