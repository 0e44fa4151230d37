"""CPHD files on the host: layout parsing (1.0.1 and 0.3), per-vector parameters, the dataset
properties the reference derives from them (src/sarsolver/io/cphd101.py, io/cphd03.py), and the
CPU decode oracle.  No GPU: signal arrays are checked as stored bytes through the oracle."""
import pickle
import struct

import numpy as np
import pytest

from oracle.cphd import decode_signal, decode_signal_bytewise
from sarsolver_gb300.cphd import (Cphd03Dataset, Cphd101Dataset, CphdReader, open_phase_history, read_header,
                                  write_cphd)


def _collection(S=37, N=29, seed=0, fc=9.6e9, bw=150e6, scale=1000.0):
    rng = np.random.default_rng(seed)
    az = np.linspace(-0.03, 0.03, S)
    tx = np.stack([8e3 * np.cos(az), 8e3 * np.sin(az), np.full(S, 3e3)], axis=-1)
    rx = tx + rng.normal(size=(S, 3))
    srp = rng.normal(size=(S, 3))
    ph = (rng.normal(size=(S, N)) + 1j * rng.normal(size=(S, N))) * scale
    return dict(phase_history=ph, trans_posns=tx, rec_posns=rx, srps=srp, centre_freq=fc, sample_bandwidth=bw)


@pytest.mark.parametrize("version,cls", [("1.0.1", Cphd101Dataset), ("0.3", Cphd03Dataset)])
@pytest.mark.parametrize("fmt", ["CI2", "CI4", "CF8"])
def test_roundtrip_metadata_and_samples(tmp_path, version, cls, fmt):
    ch = _collection(scale=30.0 if fmt == "CI2" else 1000.0)
    path = tmp_path / f"c_{version}_{fmt}.cphd"
    write_cphd(path, [ch], version=version, signal_format=fmt, sign=-1, amp_sf=False)
    ds = cls(str(path))
    S, N = ch["phase_history"].shape
    assert ds.num_slow_times == S and ds.num_freqs == N
    assert ds.sign_multiplier == -1.0
    np.testing.assert_array_equal(ds.transmitter_positions, ch["trans_posns"])
    np.testing.assert_array_equal(ds.receiver_positions, ch["rec_posns"])
    np.testing.assert_array_equal(ds.stab_ref_posns, ch["srps"])
    # the reference's band: first-sample frequency + N * spacing / 2, and N * spacing
    assert ds.centre_frequency == pytest.approx(ch["centre_freq"], rel=1e-15)
    assert ds.sample_bandwidth == pytest.approx(ch["sample_bandwidth"], rel=1e-15)
    ap = ds.aperture
    assert ap.num_slow_times == S and ap.num_freqs == N and ap.sign_multiplier == -1.0
    np.testing.assert_array_equal(ap.waveform_fft, np.ones(N))
    np.testing.assert_array_equal(ap.slow_time_weighting, np.ones(S))
    r = ds.reader
    raw = r.read_raw(slice(None))
    got = decode_signal(raw, r.signal_format, S, N)
    ref = ch["phase_history"]
    if fmt == "CF8":
        np.testing.assert_array_equal(got, ref.astype(np.complex64))
    else:
        top = 127 if fmt == "CI2" else 32767
        want = np.clip(np.rint(ref.real), -top, top) + 1j * np.clip(np.rint(ref.imag), -top, top)
        np.testing.assert_array_equal(got, want.astype(np.complex64))


def test_version_dispatch_and_mismatch(tmp_path):
    ch = _collection()
    p1, p3 = tmp_path / "a.cphd", tmp_path / "b.cphd"
    write_cphd(p1, [ch], version="1.0.1")
    write_cphd(p3, [ch], version="0.3")
    assert isinstance(open_phase_history(str(p1)), Cphd101Dataset)
    assert isinstance(open_phase_history(str(p3)), Cphd03Dataset)
    with pytest.raises(ValueError):
        Cphd03Dataset(str(p1))
    with pytest.raises(ValueError):
        Cphd101Dataset(str(p3))
    bad = tmp_path / "bad.cphd"
    bad.write_bytes(b"NITF02.10" + b"\0" * 100)
    with pytest.raises(ValueError):
        CphdReader(str(bad))
    with open(p1, "rb") as f:
        version, keys = read_header(f)
    assert version == "1.0.1"
    assert {"XML_BLOCK_SIZE", "PVP_BLOCK_BYTE_OFFSET", "SIGNAL_BLOCK_SIZE", "CLASSIFICATION"} <= set(keys)


@pytest.mark.parametrize("version", ["1.0.1", "0.3"])
def test_channels_and_amp_sf(tmp_path, version):
    a, b = _collection(S=11, N=17, seed=1), _collection(S=23, N=9, seed=2, fc=5.3e9, bw=80e6)
    path = tmp_path / "two.cphd"
    write_cphd(path, [a, b], version=version, signal_format="CI4", sign=1, amp_sf=True)
    ds = (Cphd101Dataset if version.startswith("1.") else Cphd03Dataset)(str(path), channel_index=1)
    assert (ds.num_slow_times, ds.num_freqs) == (23, 9)
    assert ds.sign_multiplier == 1.0
    assert ds.centre_frequency == pytest.approx(5.3e9, rel=1e-15)
    np.testing.assert_array_equal(ds.transmitter_positions, b["trans_posns"])
    r = ds.reader
    amp = r.amp_sf(1)
    assert amp.shape == (23,) and np.all(amp > 0)
    got = decode_signal(r.read_raw(slice(None), 1), "CI4", 23, 9, amp)
    # integer quantisation with the largest component at 32767: error <= AmpSF / 2 per component
    err = np.abs(got.astype(np.complex128) - b["phase_history"])
    assert np.all(err <= np.sqrt(2) * 0.5 * amp[:, None] * (1 + 1e-6))
    with pytest.raises(IndexError):
        Cphd101Dataset(str(path), channel_index=2) if version.startswith("1.") else Cphd03Dataset(str(path), 2)


def test_pvp_variable_ranges_and_added_pvp(tmp_path):
    ch = _collection(S=15, N=8)
    extra = {"BeamGain": np.linspace(0.5, 1.5, 15)}
    path = tmp_path / "added.cphd"
    write_cphd(path, [ch], added_pvp=extra)
    r = CphdReader(str(path))
    assert r.read_pvp_variable("NoSuchThing") is None
    np.testing.assert_array_equal(r.read_pvp_variable("BeamGain"), extra["BeamGain"])
    np.testing.assert_array_equal(r.read_pvp_variable("TxPos", 0, slice(3, 7)), ch["trans_posns"][3:7])
    one = r.read_pvp_variable("TxPos", 0, 4)
    assert one.shape == (1, 3)
    np.testing.assert_array_equal(one[0], ch["trans_posns"][4])
    sc0 = r.read_pvp_variable("SC0", 0, 0)[0]   # the reference's call form
    assert sc0 == pytest.approx(ch["centre_freq"] - 0.5 * ch["sample_bandwidth"], rel=1e-15)


def test_to_blocks_and_pickle(tmp_path):
    ch = _collection(S=10, N=6)
    path = tmp_path / "blocks.cphd"
    write_cphd(path, [ch])
    ds = Cphd101Dataset(str(path), slow_time_weighting=np.arange(10) + 1j)
    blocks = ds.to_blocks(3)
    assert [b.aperture.num_slow_times for b in blocks] == [3, 3, 4]   # remainder in the last block
    assert all(b.phase_history() is None for b in blocks)
    np.testing.assert_array_equal(blocks[2].aperture.slow_time_weighting, np.arange(6, 10) + 1j)
    np.testing.assert_array_equal(blocks[1].aperture.transmitter_positions, ch["trans_posns"][3:6])
    assert len(ds.to_blocks(1)) == 1 and ds.to_blocks(1)[0].aperture.num_slow_times == 10
    ds2 = pickle.loads(pickle.dumps(ds))
    assert ds2.num_slow_times == 10 and ds2.centre_frequency == ds.centre_frequency


@pytest.mark.parametrize("fmt", ["CI2", "CI4", "CF8"])
def test_oracle_restatements_agree(fmt):
    rng = np.random.default_rng(3)
    V, N = 5, 7
    if fmt == "CF8":
        comp = rng.normal(size=2 * V * N).astype(">f4")
        raw = comp.tobytes()
    else:
        code = ">b" if fmt == "CI2" else ">h"
        lo, hi = (-128, 127) if fmt == "CI2" else (-32768, 32767)
        vals = rng.integers(lo, hi + 1, size=2 * V * N)
        vals[:4] = [lo, hi, -1, 0]
        raw = b"".join(struct.pack(code, int(v)) for v in vals)
    amp = rng.uniform(0.1, 3.0, size=V)
    for a in (None, amp):
        np.testing.assert_array_equal(decode_signal(np.frombuffer(raw, np.uint8), fmt, V, N, a),
                                      decode_signal_bytewise(raw, fmt, V, N, a))
    if fmt != "CF8":
        d = decode_signal(np.frombuffer(raw, np.uint8), fmt, V, N)
        assert d[0, 0] == complex(lo, hi) and d[0, 1] == complex(-1, 0)
