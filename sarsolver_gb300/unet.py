"""The learned warm start's network: a bf16 4-level U-Net run and trained by the library's own
tensor-core kernels (``sar_unet_*`` in include/sargpu.h).

``UNet`` owns one native network object: FP32 master parameters, Adam moments, gradients, bf16
filter copies and the activations of the last forward call.  Images are complex64 ``[B, H, W]``;
the network sees two channels (re, im) times ``in_scale`` and returns a complex64 image.
``UNetFunction`` makes it a ``torch.autograd.Function`` (backward = the native backward pass,
which accumulates parameter gradients inside the object; the gradient with respect to the input
is not formed, the input being data).
"""
from __future__ import annotations

import ctypes
import math
from typing import List, Optional

import numpy as np
import torch

from . import _lib

LAYER_NAMES = ["enc0a", "enc0b", "enc1a", "enc1b", "enc2a", "enc2b", "bot_a", "bot_b",
               "dec2a", "dec2b", "dec1a", "dec1b", "dec0a", "dec0b", "out"]


class UNet:
    def __init__(self, base_channels: int = 32, device: Optional[torch.device] = None, seed: int = 0,
                 zero_output: bool = False):
        if not torch.cuda.is_available():
            raise RuntimeError("UNet needs a CUDA device")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.current_stream(self.device)
            _lib.check(self._lib.sar_unet_create(int(base_channels), self.device.index, ctypes.byref(h)),
                       "sar_unet_create")
        self._handle = h
        self.base_channels = int(base_channels)
        n = ctypes.c_size_t()
        layers = (_lib.SarUnetLayer * _lib.SAR_UNET_LAYERS)()
        _lib.check(self._lib.sar_unet_info(h, ctypes.byref(n), layers), "sar_unet_info")
        self.num_params = int(n.value)
        self.layers: List[dict] = [
            dict(name=LAYER_NAMES[i], weight_offset=int(l.weight_offset), bias_offset=int(l.bias_offset),
                 cin0=int(l.cin0), cin1=int(l.cin1), cout=int(l.cout), taps=int(l.taps), relu=bool(l.relu),
                 level=int(l.level))
            for i, l in enumerate(layers)]
        self.step_count = 0
        self.set_params(self.initial_params(seed, zero_output))

    # ------------------------------------------------------------------ parameters
    def initial_params(self, seed: int, zero_output: bool = False) -> torch.Tensor:
        """He-normal filters (the output layer scaled by 0.1, only its two used outputs non-zero, or
        all zero with ``zero_output`` so that the untrained network outputs zero), zero biases."""
        g = torch.Generator(device="cpu")
        g.manual_seed(seed)
        p = torch.zeros(self.num_params, dtype=torch.float32)
        for l in self.layers:
            cin = l["cin0"] + l["cin1"]
            fan_in = l["taps"] * cin
            nw = l["cout"] * fan_in
            w = torch.randn(nw, generator=g) * math.sqrt(2.0 / fan_in)
            if l["name"] == "enc0a":   # only input channels 0, 1 carry data
                w = w.view(l["cout"], l["taps"], cin)
                w[:, :, 2:] = 0.0
                w = w * math.sqrt(cin / 2.0)
                w = w.reshape(-1)
            if l["name"] == "out":
                w = w.view(l["cout"], fan_in) * (0.0 if zero_output else 0.1)
                w[2:] = 0.0
                w = w.reshape(-1)
            p[l["weight_offset"]:l["weight_offset"] + nw] = w
        return p.to(self.device)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def set_params(self, params: torch.Tensor) -> None:
        p = torch.as_tensor(params).to(device=self.device, dtype=torch.float32).contiguous()
        if p.numel() != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.numel()}")
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_unet_set_params(self._handle, ctypes.c_void_p(p.data_ptr()), self._stream()),
                       "sar_unet_set_params")
        self._keep = p
        self.step_count = 0

    def params(self) -> torch.Tensor:
        out = torch.empty(self.num_params, dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_unet_get_params(self._handle, ctypes.c_void_p(out.data_ptr()), self._stream()),
                       "sar_unet_get_params")
        return out

    def grads(self) -> torch.Tensor:
        out = torch.empty(self.num_params, dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_unet_get_grads(self._handle, ctypes.c_void_p(out.data_ptr()), self._stream()),
                       "sar_unet_get_grads")
        return out

    def zero_grad(self) -> None:
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_unet_zero_grad(self._handle, self._stream()), "sar_unet_zero_grad")

    def adam_step(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step_count += 1
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_unet_adam_step(self._handle, float(lr), float(beta1), float(beta2), float(eps),
                                                    self.step_count, self._stream()), "sar_unet_adam_step")

    # ------------------------------------------------------------------ passes
    def forward(self, x: torch.Tensor, in_scale: float = 1.0) -> torch.Tensor:
        """``U(in_scale * x)`` for complex64 ``x`` of shape ``[B, H, W]`` (or ``[H, W]``)."""
        squeeze = x.dim() == 2
        xx = x.reshape(1, *x.shape) if squeeze else x
        xx = xx.to(device=self.device, dtype=torch.complex64).resolve_conj().resolve_neg().contiguous()
        B, H, W = xx.shape
        out = torch.empty_like(xx)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_unet_forward(self._handle, ctypes.c_void_p(xx.data_ptr()), float(in_scale), B, H, W,
                                                  ctypes.c_void_p(out.data_ptr()), self._stream()), "sar_unet_forward")
        self._last_shape = xx.shape
        return out.reshape(x.shape)

    def backward(self, grad_out: torch.Tensor) -> None:
        """Accumulate parameter gradients for ``grad_out`` of the last forward call."""
        g = grad_out.to(device=self.device, dtype=torch.complex64).resolve_conj().resolve_neg().contiguous()
        if g.numel() != int(np.prod(self._last_shape)):
            raise ValueError("grad_out does not match the last forward call")
        with torch.cuda.device(self.device):
            _lib.check(self._lib.sar_unet_backward(self._handle, ctypes.c_void_p(g.data_ptr()), self._stream()),
                       "sar_unet_backward")

    def flags(self) -> int:
        f = ctypes.c_uint(0)
        _lib.check(self._lib.sar_unet_flags(self._handle, ctypes.byref(f)), "sar_unet_flags")
        return int(f.value)

    # ------------------------------------------------------------------ persistence
    def state_dict(self) -> dict:
        return {"base_channels": self.base_channels, "params": self.params().cpu()}

    def load_state_dict(self, state: dict) -> None:
        if int(state["base_channels"]) != self.base_channels:
            raise ValueError("checkpoint has a different width")
        self.set_params(state["params"])

    def close(self) -> None:
        if getattr(self, "_handle", None):
            torch.cuda.synchronize(self.device)
            self._lib.sar_unet_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class UNetFunction(torch.autograd.Function):
    """``U(in_scale * x)``; backward adds parameter gradients inside ``net`` and returns no input
    gradient.  The backward must follow its own forward before the next forward call."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, net: UNet, in_scale: float) -> torch.Tensor:
        ctx.net = net
        return net.forward(x, in_scale)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        ctx.net.backward(grad_out)
        return None, None, None
