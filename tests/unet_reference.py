"""Plain PyTorch FP32 restatement of the U-Net (the numerics reference for its CUDA kernels).

Same layer table and parameter layout as the native network: for each layer a filter
[cout][taps][cin0 + cin1] (tap = 3 * ky + kx) followed by a bias [cout]; input channels
(re, im) * in_scale padded with zeros to 32; 2x2 average pooling, nearest 2x upsampling,
concatenation (upsampled, skip); ReLU after every 3x3 convolution; output channels 0, 1.
"""
import torch
import torch.nn.functional as F


def conv(params, layer, x):
    cin = layer["cin0"] + layer["cin1"]
    k = 3 if layer["taps"] == 9 else 1
    wo, bo, co = layer["weight_offset"], layer["bias_offset"], layer["cout"]
    w = params[wo:wo + co * layer["taps"] * cin].view(co, layer["taps"], cin).permute(0, 2, 1).reshape(co, cin, k, k)
    y = F.conv2d(x, w, params[bo:bo + co], padding=k // 2)
    return torch.relu(y) if layer["relu"] else y


def unet_forward(params, layers, x, in_scale=1.0):
    """x complex [B, H, W] -> complex [B, H, W] in FP32."""
    B, H, W = x.shape
    inp = torch.zeros(B, 32, H, W, dtype=torch.float32, device=x.device)
    inp[:, 0] = x.real.float() * in_scale
    inp[:, 1] = x.imag.float() * in_scale
    L = layers
    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")
    a0 = conv(params, L[0], inp)
    a1 = conv(params, L[1], a0)
    a2 = conv(params, L[2], F.avg_pool2d(a1, 2))
    a3 = conv(params, L[3], a2)
    a4 = conv(params, L[4], F.avg_pool2d(a3, 2))
    a5 = conv(params, L[5], a4)
    a6 = conv(params, L[6], F.avg_pool2d(a5, 2))
    a7 = conv(params, L[7], a6)
    a8 = conv(params, L[8], torch.cat([up(a7), a5], 1))
    a9 = conv(params, L[9], a8)
    a10 = conv(params, L[10], torch.cat([up(a9), a3], 1))
    a11 = conv(params, L[11], a10)
    a12 = conv(params, L[12], torch.cat([up(a11), a1], 1))
    a13 = conv(params, L[13], a12)
    out = conv(params, L[14], a13)
    return torch.complex(out[:, 0], out[:, 1])
