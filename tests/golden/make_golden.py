"""Generate the golden fixtures in this directory by running the reference implementation.

Run in a container that holds the reference checkout (default /root/reference) after
``make -C oracle`` has built ``oracle/_ref/libsarsolver_ref.so`` from the reference's own
``sarsolver_cxx.cpp``:

    python tests/golden/make_golden.py [--reference /root/reference]

The reference's Python package is copied to a temporary directory (its source tree is
read-only and its ctypes loader looks for ``sarsolver_cxx*.so`` in the package root,
src/sarsolver/cxx_binding/sarsolver_cxx.py:34-46), the shim-built kernel is placed there,
and a stub ``pymap3d`` module is put on the path (src/sarsolver/utils/geodesy.py:4 imports
it; none of the cases here needs geodesy).  Each fixture stores the geometry, the inputs and
the outputs of the reference's public ``NumpySimpleSarOperator.matvec`` / ``rmatvec``
(src/sarsolver/numpy/operator.py:44-56).

Fixtures written:
  little.npz         -- the reference's own "little" test case (tests/conftest.py:46-117):
                        249 pulses x 251 samples, grid [1, 244, 241] from
                        GridSarScene.from_aperture(safety_factor=3), upsample 128.  Input is
                        tests/artifacts/little_noisy_meas.npy, output the reference adjoint,
                        checked on generation against tests/artifacts/little_backproj.npy.
  spot_small.npz     -- circular spotlight (10 km ground radius, 5 km altitude, 3 deg),
                        32 pulses x 64 samples, upsample 8, 32 x 32 grid at 0.5 m.
  bistatic_odd.npz   -- bistatic, odd N = 63, complex weights, a waveform, sign -1,
                        rotated 2-plane grid off the SRP, upsample 8.
  points.npz         -- unstructured scatterer positions (SimpleSarScene), upsample 4.
  little_pdhg.npz    -- the reference's PDHG artifact tests/artifacts/little_soln.npy (CIL PDHG with
                        f = L2NormSquared(b = little_noisy_meas), g = ZeroFunction, from zero, the
                        operator norm pinned to 756.6231381576064 by tests/conftest.py:93-96, then
                        run(3), tests/test_cil.py:25-37), with that norm.  Checked on generation:
                        two PDHG updates in CIL's order (sigma = tau = 1 / norm, theta = 1) on the
                        oracle's nearest-bin operator (bit-identical to the reference kernel)
                        reproduce it to 1e-12; three updates are 4.6 % away, so that run(3) applied
                        two updates (its run loop counts the set-up step as iteration 0).
                        ``--only little_pdhg`` writes just this file.
"""
from __future__ import annotations

import argparse
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

PYMAP3D_STUB = '''
"""Stub: the golden cases place every scene at the origin and never call geodesy."""
def _unavailable(*args, **kwargs):
    raise NotImplementedError("pymap3d is not installed")
ecef2geodetic = geodetic2ecef = enu2ecef = _unavailable
'''


def import_reference(ref_root: str, workdir: str):
    pkg_src = os.path.join(ref_root, "src", "sarsolver")
    pkg_dst = os.path.join(workdir, "sarsolver")
    shutil.copytree(pkg_src, pkg_dst)
    so = os.path.join(REPO, "oracle", "_ref", "libsarsolver_ref.so")
    if not os.path.exists(so):
        raise SystemExit("build oracle/_ref first: make -C oracle")
    shutil.copy(so, os.path.join(pkg_dst, "sarsolver_cxx.so"))
    with open(os.path.join(workdir, "pymap3d.py"), "w") as f:
        f.write(PYMAP3D_STUB)
    sys.path.insert(0, workdir)
    os.environ["PYTHONPATH"] = workdir + os.pathsep + os.environ.get("PYTHONPATH", "")
    import sarsolver.numpy as sn  # noqa: E402
    return sn


def grid_fields(scene):
    return dict(
        grid_shape=np.asarray(scene.grid_shape, dtype=np.int64),
        grid_dimensions=np.asarray(scene.grid_dimensions, dtype=np.float64),
        grid_centre=np.asarray(scene.grid_centre, dtype=np.float64),
        rotation_matrix=np.asarray(scene.rotation_matrix, dtype=np.float64),
    )


def aperture_fields(ap):
    return dict(
        tx=np.asarray(ap.transmitter_positions, np.float64),
        rx=np.asarray(ap.receiver_positions, np.float64),
        srp=np.asarray(ap.stab_ref_posns, np.float64),
        centre_frequency=np.float64(ap.centre_frequency),
        sample_frequency=np.float64(ap.sample_bandwidth),
        waveform_fft=np.asarray(ap.waveform_fft, np.complex128),
        slow_time_weighting=np.asarray(ap.slow_time_weighting, np.complex128),
        sign_multiplier=np.float64(ap.sign_multiplier),
        c_eff=np.float64(ap.c_eff),
    )


def spotlight(S, radius, altitude, aperture_deg, centre_az_deg=0.0):
    az = np.deg2rad(centre_az_deg + np.linspace(-0.5, 0.5, S) * aperture_deg)
    return np.stack([radius * np.cos(az), radius * np.sin(az), np.full(S, altitude)], -1)


def run_case(sn, scene, ap, x, y, upsample, threads):
    op = sn.NumpySimpleSarOperator(scene, ap, num_threads=threads, upsample_ratio=upsample)
    fwd = op.matvec(x.reshape(-1)).reshape(ap.num_slow_times, ap.num_freqs)
    adj = op.rmatvec(y.reshape(-1))
    return fwd, adj


def little_pdhg(ref_root: str):
    """little_pdhg.npz from the reference's artifact, checked against two oracle PDHG updates."""
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.dirname(HERE))
    import oracle
    from cases import load_golden

    arts = os.path.join(ref_root, "tests", "artifacts")
    soln = np.load(os.path.join(arts, "little_soln.npy"))
    norm = 756.6231381576064                      # tests/conftest.py:95
    case = load_golden("little")
    prob, b = case.problem(), case.data["y"]
    th = oracle.default_threads()
    fwd = lambda v: oracle.forward(prob, v, "nearest_ref", threads=th)
    adj = lambda v: oracle.adjoint(prob, v, "nearest_ref", threads=th)
    sigma = tau = 1.0 / norm
    x_prev = x = np.zeros(prob.num_scatterers, np.complex128)
    yd = np.zeros_like(b)
    errs = []
    for _ in range(3):
        xbar = 2.0 * x - x_prev
        yd = (yd + sigma * fwd(xbar) - sigma * b) / (1.0 + sigma / 2.0)
        x_prev, x = x, x - tau * adj(yd)
        errs.append(np.linalg.norm(x - soln.reshape(-1)) / np.linalg.norm(soln))
    print("little_pdhg: rel L2 of 1, 2, 3 updates vs little_soln.npy:", ", ".join(f"{e:.3e}" for e in errs))
    assert errs[1] < 1e-12, errs
    np.savez(os.path.join(HERE, "little_pdhg.npz"), soln=soln.reshape(-1), operator_norm=np.float64(norm),
             updates=np.int64(2))


def main():
    ap_ = argparse.ArgumentParser()
    ap_.add_argument("--reference", default="/root/reference")
    ap_.add_argument("--threads", type=int, default=4)
    ap_.add_argument("--only", choices=["little_pdhg"], default=None)
    args = ap_.parse_args()
    little_pdhg(args.reference)
    if args.only:
        return
    work = tempfile.mkdtemp(prefix="sar_golden_")
    try:
        sn = import_reference(args.reference, work)
        arts = os.path.join(args.reference, "tests", "artifacts")
        rng = np.random.Generator(np.random.PCG64(20261203))

        # ---- little: the reference's own fixture parameters (tests/conftest.py:47-72)
        S, N = 249, 251
        track = np.linspace(np.array([2000.0, -30.0, 0.0]), np.array([2000.0, 30.0, 0.0]), S)
        ap = sn.NumpySimpleSarAperture(trans_posns=track, rec_posns=track.copy(),
                                       srps=np.zeros((S, 3)), centre_freq=10.0e9,
                                       sample_freq=300.0e6, num_freqs=N)
        scene = sn.GridSarScene.from_aperture(ap, np.array([0.0, 0.0, 0.0]),
                                              np.array([0.0, 40.0, 40.0]), safety_factor=3.0)
        y = np.load(os.path.join(arts, "little_noisy_meas.npy"))
        bp_ref = np.load(os.path.join(arts, "little_backproj.npy"))
        op = sn.NumpySimpleSarOperator(scene, ap, num_threads=args.threads)
        bp = op.rmatvec(y.reshape(-1)).reshape(bp_ref.shape)
        rel = np.linalg.norm(bp - bp_ref) / np.linalg.norm(bp_ref)
        print(f"little: grid {list(scene.grid_shape)}, rel L2 vs little_backproj.npy = {rel:.3e}")
        assert rel < 1e-12, rel
        np.savez(os.path.join(HERE, "little.npz"), **grid_fields(scene), **aperture_fields(ap),
                 upsample_ratio=np.float64(128.0), y=y, adjoint=bp_ref.reshape(-1))

        # ---- spot_small: config-1 geometry at reduced size
        S, N, U = 32, 64, 8.0
        tx = spotlight(S, 10000.0, 5000.0, 3.0)
        ap = sn.NumpySimpleSarAperture(trans_posns=tx, rec_posns=tx.copy(), srps=np.zeros((S, 3)),
                                       centre_freq=10.0e9, sample_freq=200.0e6, num_freqs=N)
        scene = sn.GridSarScene([1, 32, 32], [0.0, 15.5, 15.5])
        x = np.zeros(scene.num_scatterers, np.complex128)
        idx = rng.choice(scene.num_scatterers, 20, replace=False)
        x[idx] = (rng.standard_normal(20) + 1j * rng.standard_normal(20)) / np.sqrt(2)
        y = (rng.standard_normal((S, N)) + 1j * rng.standard_normal((S, N))) / np.sqrt(2)
        fwd, adj = run_case(sn, scene, ap, x, y, U, args.threads)
        np.savez(os.path.join(HERE, "spot_small.npz"), **grid_fields(scene), **aperture_fields(ap),
                 upsample_ratio=np.float64(U), x=x, y=y, forward=fwd, adjoint=adj)
        print("spot_small written")

        # ---- bistatic_odd: every optional input exercised
        S, N, U = 24, 63, 8.0
        tx = spotlight(S, 9000.0, 4000.0, 4.0, centre_az_deg=10.0)
        rx = spotlight(S, 7000.0, 3000.0, 2.0, centre_az_deg=-25.0)
        srp = np.tile(np.array([[3.0, -2.0, 0.5]]), (S, 1))
        wf = np.fft.fftshift(np.hanning(N + 2)[1:-1]) * np.exp(1j * rng.uniform(-0.3, 0.3, N))
        wt = (1.0 + 0.2 * rng.standard_normal(S)) * np.exp(1j * rng.uniform(-np.pi, np.pi, S))
        ap = sn.NumpySimpleSarAperture(trans_posns=tx, rec_posns=rx, srps=srp,
                                       centre_freq=9.6e9, sample_freq=150.0e6,
                                       waveform_fft=wf, slow_time_weighting=wt,
                                       sign_multiplier=-1.0, c_eff=299700000.0)
        th = np.deg2rad(17.0)
        rot = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
        scene = sn.GridSarScene([2, 20, 24], [1.0, 9.5, 11.5], grid_centre=np.array([1.0, 0.5, 0.25]),
                                rotation_matrix=rot)
        x = (rng.standard_normal(scene.num_scatterers) + 1j * rng.standard_normal(scene.num_scatterers))
        y = (rng.standard_normal((S, N)) + 1j * rng.standard_normal((S, N)))
        # The operator path (numpy/operator.py -> multi_*_evaluate) rebuilds the aperture in
        # NumpySimpleSarAperture.to_blocks without c_eff (numpy/measurement.py:78-85), so it
        # computes with vacuum c; single_*_evaluate passes measurements.c_eff through
        # (cxx_binding/forward.py:30-32).  The golden outputs honour c_eff; the operator's
        # vacuum-c outputs are stored alongside as a record of that behaviour.
        from sarsolver.cxx_binding import single_adjoint_evaluate, single_forward_evaluate
        fwd = single_forward_evaluate(scene, ap, x.reshape(-1), upsample_ratio=U)
        adj = single_adjoint_evaluate(scene, ap, y, upsample_ratio=U)
        fwd_op, adj_op = run_case(sn, scene, ap, x, y, U, args.threads)
        np.savez(os.path.join(HERE, "bistatic_odd.npz"), **grid_fields(scene), **aperture_fields(ap),
                 upsample_ratio=np.float64(U), x=x, y=y, forward=fwd, adjoint=adj,
                 forward_operator_vacuum_c=fwd_op, adjoint_operator_vacuum_c=adj_op)
        print("bistatic_odd written")

        # ---- points: unstructured positions
        S, N, U = 20, 48, 4.0
        tx = spotlight(S, 5000.0, 2000.0, 5.0, centre_az_deg=40.0)
        ap = sn.NumpySimpleSarAperture(trans_posns=tx, rec_posns=tx.copy(), srps=np.zeros((S, 3)),
                                       centre_freq=5.0e9, sample_freq=100.0e6, num_freqs=N)
        pos = np.stack([rng.uniform(-15, 15, 300), rng.uniform(-15, 15, 300), rng.uniform(-1, 1, 300)], -1)
        scene = sn.SimpleSarScene(pos)
        x = (rng.standard_normal(300) + 1j * rng.standard_normal(300))
        y = (rng.standard_normal((S, N)) + 1j * rng.standard_normal((S, N)))
        fwd, adj = run_case(sn, scene, ap, x, y, U, args.threads)
        np.savez(os.path.join(HERE, "points.npz"), positions=pos, **aperture_fields(ap),
                 upsample_ratio=np.float64(U), x=x, y=y, forward=fwd, adjoint=adj)
        print("points written")
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
