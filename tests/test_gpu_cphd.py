"""CPHD signal arrays decoded on the GPU (sar_cphd_decode through the C ABI, and the streaming
reader) against the CPU decode oracle, bit for bit: every format, AmpSF scaling, unaligned
buffers and ragged tails, all integer extremes, row selections, multi-block streaming; then a
collection written to a CPHD file, read back and backprojected, and resampled straight from the
file (the reference's real-data flow, tests/conftest.py:25-34)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle.cphd import decode_signal
from sarsolver_gb300 import _lib
from sarsolver_gb300.cphd import FORMATS, Cphd101Dataset, Cphd03Dataset, write_cphd
from sarsolver_gb300.geometry import NumpySimpleSarAperture, NumpySimpleSarDataset

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _decode_dev(raw: np.ndarray, fmt: str, V: int, N: int, amp=None, raw_shift=0, out_shift=0):
    """Decode through the C ABI with the raw bytes at byte offset raw_shift and the output at
    complex64 offset out_shift inside larger device buffers (alignment paths)."""
    lib = _lib.load()
    code = FORMATS[fmt][0]
    rd = torch.zeros(raw.size + 16, dtype=torch.uint8, device="cuda")
    rd[raw_shift:raw_shift + raw.size] = torch.from_numpy(raw.reshape(-1)).cuda()
    od = torch.full((V * N + 2,), complex(7, 7), dtype=torch.complex64, device="cuda")
    ad = None if amp is None else torch.from_numpy(np.asarray(amp, np.float32)).cuda()
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.sar_cphd_decode(ctypes.c_void_p(rd.data_ptr() + raw_shift), code, V, N,
                                   ctypes.c_void_p(None if ad is None else ad.data_ptr()),
                                   ctypes.c_void_p(od.data_ptr() + 8 * out_shift), ctypes.c_void_p(st)),
               "sar_cphd_decode")
    out = od.cpu().numpy()
    # nothing outside the output span is touched
    assert np.all(out[:out_shift] == complex(7, 7)) and np.all(out[out_shift + V * N:] == complex(7, 7))
    return out[out_shift:out_shift + V * N].reshape(V, N)


def _bits(a):
    return np.asarray(a, np.complex64).view(np.uint32)


@pytest.mark.parametrize("fmt", ["CI2", "CI4", "CF8"])
@pytest.mark.parametrize("shape", [(64, 256), (3, 37), (1, 1), (5, 1), (129, 33)])
@pytest.mark.parametrize("shifts", [(0, 0), (1, 0), (0, 1), (3, 1)])
def test_decode_bit_exact(fmt, shape, shifts):
    V, N = shape
    rng = np.random.default_rng(V * 1000 + N)
    nbytes = V * N * FORMATS[fmt][1]
    if fmt == "CF8":
        raw = rng.normal(scale=1e3, size=2 * V * N).astype(">f4").view(np.uint8)
    else:
        raw = rng.integers(0, 256, size=nbytes, dtype=np.uint8)
    amp = rng.uniform(1e-3, 10.0, size=V)
    for a in (None, amp):
        got = _decode_dev(raw, fmt, V, N, a, *shifts)
        np.testing.assert_array_equal(_bits(got), _bits(decode_signal(raw, fmt, V, N, a)))


def test_decode_every_integer_value():
    # CI2: all 65536 (I, Q) byte pairs; CI4: every 16-bit value as I and as Q
    pairs = np.arange(65536, dtype=np.uint16)
    raw2 = np.stack([(pairs >> 8).astype(np.uint8), (pairs & 0xff).astype(np.uint8)], axis=-1).reshape(-1)
    got = _decode_dev(raw2, "CI2", 256, 256)
    np.testing.assert_array_equal(_bits(got), _bits(decode_signal(raw2, "CI2", 256, 256)))
    v = np.arange(-32768, 32768, dtype=np.int64)
    comp = np.stack([v, v[::-1]], axis=-1).astype(">i2").view(np.uint8).reshape(-1)
    got = _decode_dev(comp, "CI4", 256, 256)
    ref = decode_signal(comp, "CI4", 256, 256)
    np.testing.assert_array_equal(_bits(got), _bits(ref))
    assert ref.reshape(-1)[0] == complex(-32768, 32767)


def test_decode_nan_and_inf_patterns_pass_through():
    raw = np.array([0x7f800000, 0xff800000, 0x7fc00001, 0x00000001, 0x80000000, 0x3f800000],
                   dtype=np.uint32).astype(">u4").view(np.uint8)
    got = _decode_dev(raw, "CF8", 1, 3)
    np.testing.assert_array_equal(_bits(got), _bits(decode_signal(raw, "CF8", 1, 3)))


def test_decode_rejects_bad_arguments():
    lib = _lib.load()
    assert lib.sar_cphd_decode(None, 9, 1, 1, None, None, None) == 1   # unknown format
    assert lib.sar_cphd_decode(None, 1, 1, 1, None, None, None) == 1   # null buffers
    assert lib.sar_cphd_decode(None, 1, 0, 5, None, None, None) == 0   # nothing to do


def _ch(S, N, seed, scale=2000.0):
    rng = np.random.default_rng(seed)
    az = np.linspace(-0.05, 0.05, S)
    tx = np.stack([10e3 * np.cos(az), 10e3 * np.sin(az), np.full(S, 5e3)], axis=-1)
    ph = (rng.normal(size=(S, N)) + 1j * rng.normal(size=(S, N))) * scale
    return dict(phase_history=ph, trans_posns=tx, rec_posns=tx, srps=np.zeros((S, 3)), centre_freq=10e9,
                sample_bandwidth=200e6)


@pytest.mark.parametrize("version,cls", [("1.0.1", Cphd101Dataset), ("0.3", Cphd03Dataset)])
@pytest.mark.parametrize("fmt,amp", [("CI2", True), ("CI4", True), ("CI4", False), ("CF8", False)])
def test_reader_streams_match_oracle(tmp_path, version, cls, fmt, amp):
    chs = [_ch(70, 48, 1), _ch(45, 40, 2)]
    path = tmp_path / "s.cphd"
    write_cphd(path, chs, version=version, signal_format=fmt, amp_sf=amp)
    for ci, (S, N) in enumerate([(70, 48), (45, 40)]):
        ds = cls(str(path), channel_index=ci)
        r = ds.reader
        a = r.amp_sf(ci) if amp else None
        want = decode_signal(r.read_raw(slice(None), ci), fmt, S, N, a)
        # tiny blocks: many blocks through both buffers, ragged last block
        for blk in (64 << 20, 3 * N * FORMATS[fmt][1] + 1):
            got = r.read_device(slice(None), ci, block_bytes=blk).cpu().numpy()
            np.testing.assert_array_equal(_bits(got), _bits(want))
        np.testing.assert_array_equal(_bits(ds.phase_history(slice(5, 33))), _bits(want[5:33]))
        np.testing.assert_array_equal(_bits(ds.phase_history(slice(1, None, 7))), _bits(want[1::7]))
        idx = [9, 2, 2, S - 1, 0]
        np.testing.assert_array_equal(_bits(r.read(idx, ci)), _bits(want[idx]))
        np.testing.assert_array_equal(_bits(r.read(-1, ci)), _bits(want[-1:]))
        if amp:
            raw_only = r.read(slice(None), ci, apply_amp_sf=False)
            np.testing.assert_array_equal(_bits(raw_only), _bits(decode_signal(r.read_raw(slice(None), ci), fmt, S, N)))
        sub = ds.get_subset(slice(10, 20))
        np.testing.assert_array_equal(_bits(sub.phase_history()), _bits(want[10:20]))
        assert sub.aperture.num_slow_times == 10


def test_file_to_backprojection_and_resampling(tmp_path):
    """A simulated collection written as CPHD (CF8, exact), read back through Cphd101Dataset:
    backprojection equals that of the in-memory data; from_resampling straight from the file
    equals resampling the in-memory dataset."""
    from sarsolver_gb300 import GridSarScene, NumpySimpleSarOperator

    S, N = 256, 200
    az = np.deg2rad(np.linspace(-1.5, 1.5, S))
    tx = np.stack([10e3 * np.cos(az), 10e3 * np.sin(az), np.full(S, 5e3)], axis=-1)
    ap = NumpySimpleSarAperture(tx, tx, np.zeros((S, 3)), 10e9, 200e6, num_freqs=N, sign_multiplier=-1.0)
    scene = GridSarScene([1, 64, 64], [0.0, 32.0, 32.0])
    op = NumpySimpleSarOperator(scene, ap, upsample_ratio=8)
    rng = np.random.default_rng(4)
    x = np.zeros(64 * 64, np.complex128)
    x[rng.integers(0, x.size, 20)] = rng.normal(size=20) + 1j * rng.normal(size=20)
    y = (op.matvec(x)).reshape(S, N).astype(np.complex64)
    path = tmp_path / "sim.cphd"
    write_cphd(path, [dict(phase_history=y, trans_posns=tx, rec_posns=tx, srps=np.zeros((S, 3)), centre_freq=10e9,
                           sample_bandwidth=200e6)], signal_format="CF8", sign=-1)
    ds = Cphd101Dataset(str(path))
    assert ds.sign_multiplier == -1.0
    ph = ds.phase_history()
    np.testing.assert_array_equal(ph, y)
    op2 = NumpySimpleSarOperator(scene, ds.aperture, upsample_ratio=8)
    np.testing.assert_allclose(op2.rmatvec(ph.reshape(-1)), op.rmatvec(y.reshape(-1).astype(np.complex128)),
                               rtol=0, atol=1e-6 * np.abs(op.rmatvec(y.reshape(-1))).max())
    mem = NumpySimpleSarDataset(ds.aperture, y)
    a = NumpySimpleSarDataset.from_resampling(ds, fast_downsample_factor=2.0, slow_downsample_factor=2,
                                              new_srp=np.array([3.0, -2.0, 0.0]))
    b = NumpySimpleSarDataset.from_resampling(mem, fast_downsample_factor=2.0, slow_downsample_factor=2,
                                              new_srp=np.array([3.0, -2.0, 0.0]))
    np.testing.assert_array_equal(a.phase_history(), b.phase_history())
    np.testing.assert_array_equal(a.aperture.transmitter_positions, b.aperture.transmitter_positions)
