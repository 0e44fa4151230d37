"""Scene and aperture descriptions (host-side metadata of the operator).

These mirror the reference's concrete classes so code written against sarsolver keeps working:
  GridSarScene, SimpleSarScene     src/sarsolver/numpy/hypothesis.py:10-267
  NumpySimpleSarAperture           src/sarsolver/numpy/measurement.py:13-241
  NumpySimpleSarDataset            src/sarsolver/numpy/measurement.py:244-290
The operator also accepts the reference's own objects (duck typing on the same attributes).
Grid sizing from k-space (``GridSarScene.from_aperture``, ``scene_params_classic_sar``) is host-side
geometry here too; dataset resampling lives in ``sarsolver_gb300.resample``.
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

C = 299792458.0


# ------------------------------------------------------------------ k-space geometry (host, FP64)
WGS84_A = 6378137.0
WGS84_F = 1.0 / 298.257223563


def wgs84_up(p_ecef: np.ndarray) -> np.ndarray:
    """Unit normal of the WGS84 ellipsoid at the geodetic position of an ECEF point (the local
    'up' the reference takes from pymap3d's enu2ecef at the point's geodetic coordinates)."""
    x, y, z = (float(v) for v in p_ecef)
    e2 = WGS84_F * (2.0 - WGS84_F)
    lon = np.arctan2(y, x)
    r = np.hypot(x, y)
    lat = np.arctan2(z, r * (1.0 - e2))
    for _ in range(8):   # fixed-point iteration on the geodetic latitude
        n = WGS84_A / np.sqrt(1.0 - e2 * np.sin(lat) ** 2)
        h = r / np.cos(lat) - n if abs(np.cos(lat)) > 1e-12 else abs(z) - n * (1.0 - e2)
        lat = np.arctan2(z, r * (1.0 - e2 * n / (n + h)))
    return np.array([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)])


def kspace_box(points: np.ndarray):
    """Box around the finite rows of ``points`` aligned with their principal axes
    (utils/k_space.py:9-80).  Returns (basis, spans, range_index, cross_range_index,
    out_of_plane_index): range is the axis along which the box centre lies furthest, cross range
    the widest other axis (the middle one when range is the widest)."""
    x = points[np.isfinite(points).all(axis=1)]
    z = x - x.mean(axis=0, keepdims=True)
    _, basis = np.linalg.eigh(z.T @ z)
    if np.linalg.det(basis) < 0.0:
        basis = -basis
    y = (basis.T @ x.T).T
    lo, hi = y.min(axis=0), y.max(axis=0)
    spans = np.abs(hi - lo)
    r = int(np.argmax(np.abs(0.5 * (lo + hi))))
    cr = int(np.argmax(spans)) if spans[r] < spans.max() else int(np.argsort(spans)[1])
    oop = [i for i in range(3) if i not in (r, cr)][0]
    return basis, spans, r, cr, oop


def scene_params_classic_sar(scene_centre_ecef: np.ndarray, aperture, tol: float = 1.0e-6):
    """(rotation matrix with columns range / cross range / out of plane, Nyquist sample rates in
    1/m per box axis, ground cosines) for a scene at ``scene_centre_ecef`` (utils/geodesy.py:124-172)."""
    c = np.asarray(scene_centre_ecef, np.float64)
    up = wgs84_up(c) if np.linalg.norm(c) > tol else np.array([0.0, 0.0, 1.0])
    up = up / np.linalg.norm(up)
    basis, spans, r, cr, oop = kspace_box(aperture.edge_k_vecs())
    unit = lambda v: v / np.linalg.norm(v)
    rng, crs, out = unit(basis.T[r]), unit(basis.T[cr]), unit(basis.T[oop])
    if np.dot(out, up) < 0.0:
        out, crs = -out, -crs
    rot = np.stack([rng, crs, out], axis=0)
    cosines = np.array([np.sqrt(1.0 - np.dot(rng, up) ** 2), np.sqrt(1.0 - np.dot(crs, up) ** 2),
                        np.dot(out, up)]) / (2.0 * np.pi)
    return rot.T, spans / (2.0 * np.pi), cosines


class SimpleSarScene:
    """Point scatterers at arbitrary positions [P, 3] (numpy/hypothesis.py:10-70)."""

    def __init__(self, scatterer_positions: np.ndarray):
        self._scatterer_positions = np.asarray(scatterer_positions)
        self._num_scatterers = self._scatterer_positions.shape[0]

    @property
    def positions(self) -> np.ndarray:
        return self._scatterer_positions

    @property
    def num_scatterers(self) -> int:
        return self._num_scatterers

    def to_blocks(self, num_blocks: int = 1) -> List["SimpleSarScene"]:
        if num_blocks == 1:
            return [self]
        n = self.num_scatterers // num_blocks
        out = []
        for b in range(num_blocks):
            hi = self.num_scatterers if b == num_blocks - 1 else (b + 1) * n
            out.append(SimpleSarScene(self.positions[b * n:hi, :]))
        return out


class GridSarScene:
    """Regular grid of scatterers (numpy/hypothesis.py:73-206).

    grid_shape and grid_dimensions are in (z, y, x) order; pixel (k, j, i) sits at
    ``rotation_matrix @ (x_i, y_j, z_k) + grid_centre`` with x_i = linspace(-lx/2, lx/2, nx)[i];
    the flattened index is (k*ny + j)*nx + i.
    """

    def __init__(self, grid_shape: Sequence[int], grid_dimensions: Sequence[float],
                 grid_centre: Optional[np.ndarray] = None, rotation_matrix: Optional[np.ndarray] = None):
        self._grid_centre = np.zeros(3) if grid_centre is None else np.asarray(grid_centre, dtype=np.float64)
        self._rotation_matrix = np.identity(3) if rotation_matrix is None else np.asarray(rotation_matrix, np.float64)
        self._grid_shape = [int(v) for v in grid_shape]
        self._grid_dimensions = [float(v) for v in grid_dimensions]

    @staticmethod
    def from_aperture(aperture, scene_centre_ecef: np.ndarray, grid_dimensions: Sequence[float],
                      grid_shape: Optional[Sequence[int]] = None, safety_factor: float = 1.2) -> "GridSarScene":
        """Grid aligned with the aperture's range / cross-range / out-of-plane axes at the scene
        centre; without ``grid_shape`` the point counts follow the Nyquist sample rates of the
        aperture's k-space support times ``safety_factor`` (numpy/hypothesis.py:236-267)."""
        rot, rates, _ = scene_params_classic_sar(scene_centre_ecef, aperture)
        if grid_shape is None:
            grid_shape = np.rint(np.clip(np.asarray(grid_dimensions, np.float64) * rates * safety_factor, 1.0, None))
            grid_shape = grid_shape.astype(int).tolist()
        return GridSarScene(grid_shape, grid_dimensions, scene_centre_ecef, rot)

    @property
    def num_scatterers(self) -> int:
        return int(np.prod(np.array(self.grid_shape)))

    @property
    def rotation_matrix(self) -> np.ndarray:
        return self._rotation_matrix

    @property
    def grid_centre(self) -> np.ndarray:
        return self._grid_centre

    @property
    def grid_dimensions(self) -> Sequence[float]:
        return self._grid_dimensions

    @property
    def grid_shape(self) -> Sequence[int]:
        return self._grid_shape

    @property
    def positions(self) -> np.ndarray:
        xs = np.linspace(-0.5 * self.grid_dimensions[2], 0.5 * self.grid_dimensions[2], self.grid_shape[2])
        ys = np.linspace(-0.5 * self.grid_dimensions[1], 0.5 * self.grid_dimensions[1], self.grid_shape[1])
        zs = np.linspace(-0.5 * self.grid_dimensions[0], 0.5 * self.grid_dimensions[0], self.grid_shape[0])
        zz, yy, xx = np.meshgrid(zs, ys, xs, indexing="ij")
        base = np.stack([xx.reshape(-1), yy.reshape(-1), zz.reshape(-1)], axis=-1)
        return (self.rotation_matrix @ base.T).T + self.grid_centre[None, :]

    def to_blocks(self, num_blocks: int = 1) -> List:
        if num_blocks == 1:
            return [self]
        return SimpleSarScene(self.positions).to_blocks(num_blocks)


def grid_axes(scene) -> Optional[Tuple[Tuple[int, int, int], np.ndarray, np.ndarray, np.ndarray, np.ndarray]]:
    """(shape (nz, ny, nx), origin, step_x, step_y, step_z) of a regular-grid scene, else None.

    Works on any object with the GridSarScene attributes, including the reference's own.
    """
    needed = ("grid_shape", "grid_dimensions", "grid_centre", "rotation_matrix")
    if not all(hasattr(scene, a) for a in needed):
        return None
    shape = tuple(int(v) for v in scene.grid_shape)
    dims = [float(v) for v in scene.grid_dimensions]
    rot = np.asarray(scene.rotation_matrix, dtype=np.float64)
    centre = np.asarray(scene.grid_centre, dtype=np.float64).reshape(3)
    nz, ny, nx = shape
    first = np.array([-0.5 * dims[2], -0.5 * dims[1], -0.5 * dims[0]])
    step = np.array([dims[2] / (nx - 1) if nx > 1 else 0.0,
                     dims[1] / (ny - 1) if ny > 1 else 0.0,
                     dims[0] / (nz - 1) if nz > 1 else 0.0])
    origin = rot @ first + centre
    return shape, origin, rot[:, 0] * step[0], rot[:, 1] * step[1], rot[:, 2] * step[2]


class NumpySimpleSarAperture:
    """Bistatic scalar SAR collection (numpy/measurement.py:13-241)."""

    def __init__(self, trans_posns: np.ndarray, rec_posns: np.ndarray, srps: np.ndarray, centre_freq: float,
                 sample_freq: float, waveform_fft: Optional[np.ndarray] = None,
                 slow_time_weighting: Optional[np.ndarray] = None, num_freqs: Optional[int] = None,
                 sign_multiplier: float = 1.0, c_eff: float = C):
        self._transmitter_positions = np.asarray(trans_posns)
        self._receiver_positions = np.asarray(rec_posns)
        self._stab_ref_posns = np.asarray(srps)
        self._centre_freq = centre_freq
        self._sample_bandwidth = sample_freq
        self._sign_multiplier = sign_multiplier
        self._c_eff = c_eff
        if waveform_fft is None:
            if num_freqs is None:
                raise ValueError("Number of frequencies needs to be set somehow")
            waveform_fft = np.ones(num_freqs, dtype=np.complex128)
        self._waveform_fft = np.asarray(waveform_fft)
        self._num_freqs = self._waveform_fft.shape[0]
        self._num_slow_times = self._transmitter_positions.shape[0]
        if slow_time_weighting is None:
            slow_time_weighting = np.ones(self._num_slow_times, dtype=np.complex128)
        self._slow_time_weighting = np.asarray(slow_time_weighting)

    @property
    def num_slow_times(self) -> int:
        return self._num_slow_times

    @property
    def num_freqs(self) -> int:
        return self._num_freqs

    @property
    def centre_frequency(self) -> float:
        return self._centre_freq

    @property
    def sample_bandwidth(self) -> float:
        return self._sample_bandwidth

    @property
    def freqs(self) -> np.ndarray:
        return self.centre_frequency + np.fft.fftshift(np.fft.fftfreq(self.num_freqs, 1.0 / self.sample_bandwidth))

    @property
    def transmitter_positions(self) -> np.ndarray:
        return self._transmitter_positions

    @property
    def receiver_positions(self) -> np.ndarray:
        return self._receiver_positions

    @property
    def stab_ref_posns(self) -> np.ndarray:
        return self._stab_ref_posns

    @property
    def waveform_fft(self) -> np.ndarray:
        return self._waveform_fft

    @property
    def slow_time_weighting(self) -> np.ndarray:
        return self._slow_time_weighting

    @property
    def sign_multiplier(self) -> float:
        return self._sign_multiplier

    @property
    def c_eff(self) -> float:
        return self._c_eff

    def edge_k_vecs(self, real_space_origin: Optional[np.ndarray] = None) -> np.ndarray:
        """Band-edge k-vectors of every pulse at ``real_space_origin`` (each pulse's SRP when None):
        bistatic direction (unit vector towards the receiver minus unit vector from the transmitter)
        times the lowest, then the highest wavenumber, [2S, 3] (base/measurement.py:250-321)."""
        o = self.stab_ref_posns if real_space_origin is None else np.asarray(real_space_origin)[None, :]
        unit = lambda v: v / np.linalg.norm(v, axis=-1, keepdims=True)
        with np.errstate(invalid="ignore", divide="ignore"):
            d = unit(self.receiver_positions - o) - unit(o - self.transmitter_positions)
        k = 2.0 * np.pi / self.c_eff
        return np.concatenate([d * k * (self.centre_frequency - 0.5 * self.sample_bandwidth),
                               d * k * (self.centre_frequency + 0.5 * self.sample_bandwidth)], axis=0)

    @property
    def bad_slow_times(self) -> List[int]:
        """Slow times with a non-finite position (base/measurement.py:325-339)."""
        bad = set()
        for arr in (self.transmitter_positions, self.receiver_positions, self.stab_ref_posns):
            bad.update(np.argwhere(~np.isfinite(arr).all(axis=-1))[:, 0].tolist())
        return sorted(bad)

    def get_subset(self, item: slice = None) -> "NumpySimpleSarAperture":
        return NumpySimpleSarAperture(self.transmitter_positions[item, :], self.receiver_positions[item, :],
                                      self.stab_ref_posns[item, :], self.centre_frequency, self.sample_bandwidth,
                                      self.waveform_fft, self.slow_time_weighting[item],
                                      sign_multiplier=self.sign_multiplier, c_eff=self.c_eff)

    def to_blocks(self, num_blocks: int = 1) -> List["NumpySimpleSarAperture"]:
        if num_blocks == 1:
            return [self.get_subset(slice(None))]
        n = self.num_slow_times // num_blocks
        return [self.get_subset(slice(b * n, self.num_slow_times if b == num_blocks - 1 else (b + 1) * n))
                for b in range(num_blocks)]


class NumpySimpleSarDataset:
    """An aperture plus its phase history [S, N] (numpy/measurement.py:244-290)."""

    def __init__(self, aperture, phase_history: np.ndarray):
        self._aperture = aperture
        self._phase_history = phase_history

    @property
    def aperture(self):
        return self._aperture

    def phase_history(self, item: slice = slice(None)) -> Optional[np.ndarray]:
        return None if self._phase_history is None else self._phase_history[item, :]

    def get_subset(self, item: slice = None) -> "NumpySimpleSarDataset":
        return NumpySimpleSarDataset(self.aperture.get_subset(item), self.phase_history(item))

    @staticmethod
    def from_scratch(trans_posns: np.ndarray, rec_posns: np.ndarray, srps: np.ndarray, centre_freq: float,
                     sample_freq: float, phase_history: Optional[np.ndarray] = None,
                     waveform_fft: Optional[np.ndarray] = None, slow_time_weighting: Optional[np.ndarray] = None,
                     num_freqs: Optional[int] = None, sign_multiplier: float = 1.0,
                     c_eff: float = C) -> "NumpySimpleSarDataset":
        """Aperture and dataset from the aperture's arguments (numpy/measurement.py:258-304)."""
        ap = NumpySimpleSarAperture(trans_posns, rec_posns, srps, centre_freq, sample_freq, waveform_fft=waveform_fft,
                                    slow_time_weighting=slow_time_weighting, num_freqs=num_freqs,
                                    sign_multiplier=sign_multiplier, c_eff=c_eff)
        return NumpySimpleSarDataset(ap, phase_history)

    @staticmethod
    def from_resampling(original_dataset, range_amb: Optional[float] = None, cross_range_amb: Optional[float] = None,
                        fast_downsample_factor: float = 1.0, slow_downsample_factor: int = 1,
                        new_srp: Optional[np.ndarray] = None, safety_factor: float = 1.2,
                        num_threads: Optional[int] = None, device=None,
                        keep_on_device: bool = False) -> "NumpySimpleSarDataset":
        """Resampled dataset (numpy/measurement.py:342-458), computed on the GPU by
        ``resample.resample_dataset``; ``num_threads`` is accepted for the reference's signature and
        unused (there is no host worker pool).  A dataset that can hand over its phase history on
        the device (``phase_history_device``, e.g. a CPHD file) is read straight to the device."""
        from .resample import resample_dataset
        return resample_dataset(original_dataset, fast_downsample_factor, slow_downsample_factor, new_srp=new_srp,
                                safety_factor=safety_factor, device=device, keep_on_device=keep_on_device,
                                range_amb=range_amb, cross_range_amb=cross_range_amb)

    @staticmethod
    def from_datasets(datasets: Sequence) -> "NumpySimpleSarDataset":
        """Pulse-wise concatenation of datasets sharing the band (numpy/measurement.py:463-504)."""
        import torch

        aps = [d.aperture for d in datasets]
        ap0 = aps[0]
        cat = lambda name: np.concatenate([np.asarray(getattr(a, name)) for a in aps], axis=0)
        parts = [d.phase_history(slice(None)) for d in datasets]
        if all(p is None for p in parts):
            ph = None
        elif any(isinstance(p, torch.Tensor) for p in parts):
            dev = next(p.device for p in parts if isinstance(p, torch.Tensor))
            ph = torch.cat([p.to(dev) if isinstance(p, torch.Tensor) else torch.as_tensor(p, device=dev) for p in parts])
        else:
            ph = np.concatenate(parts, axis=0)
        return NumpySimpleSarDataset.from_scratch(cat("transmitter_positions"), cat("receiver_positions"),
                                                  cat("stab_ref_posns"), ap0.centre_frequency, ap0.sample_bandwidth,
                                                  phase_history=ph, waveform_fft=ap0.waveform_fft,
                                                  slow_time_weighting=cat("slow_time_weighting"),
                                                  sign_multiplier=ap0.sign_multiplier, c_eff=ap0.c_eff)
