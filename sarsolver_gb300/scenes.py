"""Synthetic scenes and collection geometries of the benchmark configurations.

All generation is seeded and runs on the GPU (torch), so training data for the learned solver
and benchmark inputs are produced by the operator itself:
  * circular-spotlight apertures (monostatic, scene centre at the origin, fc 10 GHz,
    200 MHz sampled bandwidth, 10 km ground radius, 5 km altitude);
  * square image grids in the z = 0 plane centred on the origin;
  * reflectivity = point scatterers with complex-Gaussian amplitudes at uniform random pixels
    + a smooth extended field (real Gaussian noise low-passed by a Gaussian of sigma pixels,
    normalised to unit RMS) times complex-Gaussian speckle;
  * complex white noise at a given SNR relative to the mean |Ax|^2.
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np
import torch

from .geometry import GridSarScene, NumpySimpleSarAperture

C = 299792458.0


def spotlight_positions(num_pulses: int, aperture_deg: float, radius: float = 10.0e3, altitude: float = 5.0e3,
                        centre_az_deg: float = 0.0) -> np.ndarray:
    az = np.deg2rad(centre_az_deg + np.linspace(-0.5, 0.5, num_pulses) * aperture_deg)
    return np.stack([radius * np.cos(az), radius * np.sin(az), np.full(num_pulses, altitude)], axis=-1)


def spotlight_aperture(num_pulses: int, num_freqs: int, aperture_deg: float, radius: float = 10.0e3,
                       altitude: float = 5.0e3, centre_frequency: float = 10.0e9, bandwidth: float = 200.0e6,
                       centre_az_deg: float = 0.0) -> NumpySimpleSarAperture:
    tx = spotlight_positions(num_pulses, aperture_deg, radius, altitude, centre_az_deg)
    return NumpySimpleSarAperture(tx, tx.copy(), np.zeros((num_pulses, 3)), centre_frequency, bandwidth,
                                  num_freqs=num_freqs)


def grid_scene(n: int, spacing: float) -> GridSarScene:
    side = spacing * (n - 1)
    return GridSarScene([1, n, n], [0.0, side, side])


def _crandn(shape, gen: torch.Generator, device) -> torch.Tensor:
    re = torch.randn(shape, generator=gen, device=device, dtype=torch.float32)
    im = torch.randn(shape, generator=gen, device=device, dtype=torch.float32)
    return torch.complex(re, im) * (1.0 / math.sqrt(2.0))


def gaussian_smooth(field: torch.Tensor, sigma_px: float) -> torch.Tensor:
    """Periodic Gaussian low-pass of a real [n, n] field by FFT."""
    n0, n1 = field.shape
    f0 = torch.fft.fftfreq(n0, device=field.device)
    f1 = torch.fft.rfftfreq(n1, device=field.device)
    h = torch.exp(-2.0 * (math.pi * sigma_px) ** 2 * (f0[:, None] ** 2 + f1[None, :] ** 2))
    return torch.fft.irfft2(torch.fft.rfft2(field) * h, s=(n0, n1))


def reflectivity(n: int, num_points: int, sigma_px: float, seed: int, device="cuda",
                 clutter_level: float = 0.3, gen: Optional[torch.Generator] = None) -> torch.Tensor:
    """Complex64 image [n*n]: point scatterers + speckled smooth clutter."""
    if gen is None:
        gen = torch.Generator(device=device)
        gen.manual_seed(seed)
    field = gaussian_smooth(torch.randn((n, n), generator=gen, device=device), sigma_px)
    field = field / field.pow(2).mean().sqrt().clamp_min(1e-30)
    x = (clutter_level * field.abs()).to(torch.complex64) * _crandn((n, n), gen, device)
    x = x.reshape(-1)
    if num_points:
        idx = torch.randperm(n * n, generator=gen, device=device)[:num_points]
        x[idx] += _crandn((num_points,), gen, device)
    return x


def add_noise(y: torch.Tensor, snr_db: float, seed: int, gen: Optional[torch.Generator] = None) -> torch.Tensor:
    """y + complex white noise with power mean|y|^2 / 10^(snr/10)."""
    if gen is None:
        gen = torch.Generator(device=y.device)
        gen.manual_seed(seed)
    p = y.abs().pow(2).mean()
    sigma = torch.sqrt(p / (10.0 ** (snr_db / 10.0)))
    return y + sigma * _crandn(y.shape, gen, y.device)


def config_workload(name: str):
    """(aperture, scene, upsample, description) of the benchmark configurations."""
    if name == "config1":
        return (spotlight_aperture(128, 512, 3.0), grid_scene(256, 0.5), 8.0,
                "128 pulses x 512 samples, U=8, 256^2 at 0.5 m, 3 deg")
    if name == "config2":
        return (spotlight_aperture(4096, 4096, 5.0), grid_scene(2048, 0.25), 8.0,
                "4096 pulses x 4096 samples, U=8, 2048^2 at 0.25 m, 5 deg")
    if name == "config2_quarter":
        return (spotlight_aperture(4096, 4096, 5.0), grid_scene(1024, 0.25), 8.0,
                "4096 pulses x 4096 samples, U=8, 1024^2 at 0.25 m, 5 deg")
    if name == "config2_turned":
        return (spotlight_aperture(4096, 4096, 5.0, centre_az_deg=90.0), grid_scene(2048, 0.25), 8.0,
                "4096 pulses x 4096 samples, U=8, 2048^2 at 0.25 m, 5 deg, looking along y")
    if name == "config2_quarter_turned":
        return (spotlight_aperture(4096, 4096, 5.0, centre_az_deg=90.0), grid_scene(1024, 0.25), 8.0,
                "4096 pulses x 4096 samples, U=8, 1024^2 at 0.25 m, 5 deg, looking along y")
    if name == "config2_slice256":
        return (spotlight_aperture(256, 4096, 5.0 * 256 / 4096), grid_scene(2048, 0.25), 8.0,
                "256 of 4096 pulses x 4096 samples (the same pulse spacing), U=8, 2048^2 at 0.25 m")
    if name == "config2_quarter_diagonal":
        return (spotlight_aperture(4096, 4096, 5.0, centre_az_deg=45.0), grid_scene(1024, 0.25), 8.0,
                "4096 pulses x 4096 samples, U=8, 1024^2 at 0.25 m, 5 deg, looking along the grid diagonal")
    if name == "config2_diagonal":
        return (spotlight_aperture(4096, 4096, 5.0, centre_az_deg=45.0), grid_scene(2048, 0.25), 8.0,
                "4096 pulses x 4096 samples, U=8, 2048^2 at 0.25 m, 5 deg, looking along the grid diagonal")
    if name == "config2_steep":
        return (spotlight_aperture(4096, 4096, 5.0, centre_az_deg=63.43), grid_scene(2048, 0.25), 8.0,
                "4096 pulses x 4096 samples, U=8, 2048^2 at 0.25 m, 5 deg, looking at 63.4 deg to x (tan 2)")
    if name == "config3":
        return (spotlight_aperture(2048, 2048, 3.0), grid_scene(1024, 0.25), 8.0,
                "2048 pulses x 2048 samples, U=8, 1024^2 at 0.25 m")
    if name == "config5":
        return (spotlight_aperture(16384, 8192, 5.0), grid_scene(8192, 0.125), 8.0,
                "16384 pulses x 8192 samples, U=8, 8192^2 at 0.125 m, 5 deg")
    raise ValueError(name)
