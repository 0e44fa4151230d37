"""Shared test cases: golden fixtures and seeded synthetic geometries.

Geometry of the synthetic cases follows the benchmark configurations: circular spotlight at
10 km ground radius and 5 km altitude, fc = 10 GHz, 200 MHz sampled bandwidth, monostatic,
scene centred on the stabilisation reference point at the origin.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

import oracle
from sarsolver_gb300.geometry import GridSarScene, NumpySimpleSarAperture, SimpleSarScene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
C = 299792458.0


@dataclass
class Case:
    scene: object
    aperture: NumpySimpleSarAperture
    upsample_ratio: float
    data: dict

    def problem(self) -> oracle.Problem:
        ap = self.aperture
        return oracle.Problem(
            tx=ap.transmitter_positions, rx=ap.receiver_positions, srp=ap.stab_ref_posns,
            positions=self.scene.positions, centre_frequency=ap.centre_frequency,
            sample_frequency=ap.sample_bandwidth, num_freqs=ap.num_freqs, waveform_fft=ap.waveform_fft,
            slow_time_weighting=ap.slow_time_weighting, c_eff=ap.c_eff, sign_multiplier=ap.sign_multiplier,
            upsample_ratio=self.upsample_ratio)


def load_golden(name: str) -> Case:
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    ap = NumpySimpleSarAperture(d["tx"], d["rx"], d["srp"], float(d["centre_frequency"]),
                                float(d["sample_frequency"]), waveform_fft=d["waveform_fft"],
                                slow_time_weighting=d["slow_time_weighting"],
                                sign_multiplier=float(d["sign_multiplier"]), c_eff=float(d["c_eff"]))
    if "positions" in d:
        scene = SimpleSarScene(d["positions"])
    else:
        scene = GridSarScene(d["grid_shape"].tolist(), d["grid_dimensions"].tolist(), d["grid_centre"],
                             d["rotation_matrix"])
    return Case(scene, ap, float(d["upsample_ratio"]), d)


def spotlight(num_pulses: int, aperture_deg: float, radius: float = 10.0e3, altitude: float = 5.0e3,
              centre_az_deg: float = 0.0) -> np.ndarray:
    az = np.deg2rad(centre_az_deg + np.linspace(-0.5, 0.5, num_pulses) * aperture_deg)
    return np.stack([radius * np.cos(az), radius * np.sin(az), np.full(num_pulses, altitude)], axis=-1)


def spotlight_case(num_pulses: int, num_freqs: int, n: int, spacing: float, aperture_deg: float,
                   upsample: float = 8.0, bandwidth: float = 200.0e6, fc: float = 10.0e9,
                   bistatic: bool = False, weights=None) -> Case:
    tx = spotlight(num_pulses, aperture_deg)
    rx = tx.copy() if not bistatic else spotlight(num_pulses, aperture_deg * 0.5, 8.0e3, 3.0e3, 20.0)
    ap = NumpySimpleSarAperture(tx, rx, np.zeros((num_pulses, 3)), fc, bandwidth, num_freqs=num_freqs,
                                slow_time_weighting=weights)
    side = spacing * (n - 1)
    scene = GridSarScene([1, n, n], [0.0, side, side])
    return Case(scene, ap, upsample, {})


def point_scene(rng, n: int, num: int) -> np.ndarray:
    """Complex-Gaussian point scatterers at uniform pixels of an n x n image."""
    x = np.zeros(n * n, np.complex128)
    idx = rng.choice(n * n, num, replace=False)
    x[idx] = (rng.standard_normal(num) + 1j * rng.standard_normal(num)) / np.sqrt(2.0)
    return x


def crandn(rng, *shape) -> np.ndarray:
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0)


def rel_l2(a, b) -> float:
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
